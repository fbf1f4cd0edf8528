// Device-side structures and arithmetic shared by the FEC kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fec_consts.h"

namespace cusat {

// One LDPC code as laid out for the decoder (all pointers device memory).
struct DevCode {
    int N, K, R, q;
    int n_steps;
    int cmax;        // circulant slots per layer (= kernel CMAX)
    int fast_lim;    // |LLR| bound under which no int16 saturation can occur
    int msg_row;     // bytes of one check row of messages (16 or 32)
    int n_items;     // shared-group items over all steps
    const uint4* tab;          // [q * cmax] slot descriptors (fec_consts.h)
    const int16_t* sched;      // [n_steps * 2] layer per lane, -1 idle
    const uint8_t* step_conf;  // [n_steps] 0, kConfDefer or kConfMid
    const uint16_t* item_off;  // [n_steps + 1] group items of step s
    const uint2* items;        // [n_items]
    // learned min-sum weights [max_trials][32][2] = {beta, alpha in 64ths}
    // per (iteration, check degree); nullptr = plain offset min-sum
    const int16_t* weights;
};

// Demapper parameters of one MODCOD (points live in device memory).
struct DevDemap {
    int kind;             // 0 QPSK formula, 1 8PSK formula, 2 log-MAP over the points
    int n_mod, n_points;
    int xfec, interleaved_len, fec_len;
    uint32_t col[8];      // deinterleave column offsets
    const float2* points; // [n_points] by label (kind 2)
};

__device__ __forceinline__ int16_t llr_round(float v)
{
    v = rintf(v);
    v = fminf(fmaxf(v, -32768.0f), 32767.0f);
    return (int16_t)v;
}

// e^-x for 0 <= x < 88: 2^-n e^u with n = rint(x log2 e), u = -(x log2 e - n) ln 2,
// e^u by its degree-7 Taylor polynomial (Horner, fused multiply-adds).
__device__ __forceinline__ float dm_exp_neg(float x)
{
    const float t = __fmul_rn(x, 1.44269504088896341f);
    const float n = rintf(t);
    const float f = __fsub_rn(t, n);
    const float u = -__fmul_rn(f, 0.693147180559945309f);
    float p = 1.98412698412698413e-4f;
    p = __fmaf_rn(p, u, 1.38888888888888889e-3f);
    p = __fmaf_rn(p, u, 8.33333333333333333e-3f);
    p = __fmaf_rn(p, u, 4.16666666666666667e-2f);
    p = __fmaf_rn(p, u, 1.66666666666666667e-1f);
    p = __fmaf_rn(p, u, 0.5f);
    p = __fmaf_rn(p, u, 1.0f);
    p = __fmaf_rn(p, u, 1.0f);
    return __fmul_rn(p, __uint_as_float((uint32_t)(127 - (int)n) << 23));
}

// ln x for normal x > 0: x = m 2^e with m in [sqrt(1/2), sqrt 2), ln m =
// 2 atanh(s), s = (m - 1)/(m + 1), odd series to s^9.
__device__ __forceinline__ float dm_log(float x)
{
    uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xff) - 127;
    float m = __uint_as_float((b & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356237309505f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(s, s);
    float p = 0.111111111111111111f;
    p = __fmaf_rn(p, s2, 0.142857142857142857f);
    p = __fmaf_rn(p, s2, 0.2f);
    p = __fmaf_rn(p, s2, 0.333333333333333333f);
    p = __fmaf_rn(p, s2, 1.0f);
    const float l = __fmul_rn(__fmul_rn(2.0f, s), p);
    return __fmaf_rn((float)e, 0.693147180559945309f, l);
}

// LLRs of symbol j, written to their deinterleaved positions (pos >= the
// frame length is dropped).  Reference: cuda/demapper_kernel.cu:53-183.
//
// QPSK: 2 LLRs at 2j, 2j+1 (no interleaver).
__device__ __forceinline__ void demap_qpsk(const DevDemap& d, float re, float im, int j, float noise_var,
                                           int16_t* out)
{
    const float scalar = __fdiv_rn(2.0f * 1.4142135623730951f, noise_var);
    if (2 * j + 1 >= d.fec_len)
        return;  // both dropped together, like the reference
    out[2 * j] = llr_round(__fmul_rn(re, scalar));
    out[2 * j + 1] = llr_round(__fmul_rn(im, scalar));
}

// 8PSK: formula after the -pi/8 rotation.
__device__ __forceinline__ void demap_8psk(const DevDemap& d, float re, float im, int j, float llr_gain,
                                           int16_t* out)
{
    const float C8 = 0.92387953251128676f, S8 = 0.38268343236508977f;
    const float R2 = 0.70710678118654752f;
    const float DIST = 2.0f * 0.38268343236508977f;
    const float cr = __fmaf_rn(re, C8, __fmul_rn(im, S8));
    const float ci = __fmaf_rn(-re, S8, __fmul_rn(im, C8));
    const float scale = __fmul_rn(DIST, llr_gain);
    const int16_t l[3] = {llr_round(__fmul_rn(__fmul_rn(R2, __fsub_rn(fabsf(cr), fabsf(ci))), scale)),
                          llr_round(__fmul_rn(cr, scale)), llr_round(__fmul_rn(ci, scale))};
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int p = (int)d.col[b] + j;
        if (p < d.fec_len)
            out[p] = l[b];
    }
}

// Points per unrolled step of the log-MAP loops: the label bits below
// log2 of it are compile-time constants, but every unrolled point carries
// its bits' exps inline, and past a few KB of loop body the warps wait on
// instruction fetch (ncu, 256APSK unrolled by 16: 9.9 of 15.9 cycles per
// issue stalled on no instruction).  Measured best on GB300 (demap of 256
// normal frames): 16 points for up to 16 points, 8 for 32, 4 for 64 to 256
// (256APSK 4.25 -> 2.73 ms, 128APSK 2.08 -> 1.41 ms; with the grouped first
// pass and the point skip, 2 and 8 lose at 128-256 points and 4 gains 1 %
// at 64).
__host__ __device__ constexpr int logmap_unroll(int nm) { return nm == 0 ? 1 : nm <= 4 ? 16 : nm <= 5 ? 8 : 4; }

// APSK: log-MAP over the points (pts in shared memory), NM bits per symbol
// (0: d.n_mod at run time; a compile-time NM resolves every label-bit test
// and bit loop, same arithmetic; the point loops are then unrolled by
// logmap_unroll(NM)).
// VOTE: a term's exp is evaluated only when some lane of the warp has that
// (point, bit) inside its cutoff, and each lane adds only its own terms (the
// same terms in the same order, so the LLRs are those without VOTE); all 32
// lanes must call it, `valid` false for a lane without a symbol (it adds
// nothing and stores nothing).
template <int NM, bool VOTE = false>
__device__ __forceinline__ void demap_logmap(const DevDemap& d, const float2* pts, float re, float im, int j,
                                             float llr_gain, int16_t* out, bool valid = true)
{
    constexpr int MB = NM ? NM : 8;
    const int nm = NM ? NM : d.n_mod;
    // a specialised call has exactly 2^NM points (checked by its launcher)
    const int np = NM ? (1 << NM) : d.n_points;
    float mn0[MB], mn1[MB], s0[MB], s1[MB];
#pragma unroll
    for (int b = 0; b < MB; b++) {
        mn0[b] = 1e30f;
        mn1[b] = 1e30f;
        s0[b] = 0.0f;
        s1[b] = 0.0f;
    }
    if constexpr (NM >= 5) {
        // groups of 16 points: the 4 low label bits are known at compile
        // time (one min each), the high bits are constant over a group (one
        // min of the group's minimum each).  The same minima as point by
        // point.
#pragma unroll 1
        for (int h = 0; h < (1 << (NM - 4)); h++) {
            float mg = 1e30f;
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const float2 p = pts[(h << 4) | u];
                const float dr = __fsub_rn(re, p.x), di = __fsub_rn(im, p.y);
                const float dd = __fmaf_rn(dr, dr, __fmul_rn(di, di));
#pragma unroll
                for (int b = NM - 4; b < NM; b++) {
                    if (u & (1 << (NM - 1 - b)))
                        mn1[b] = fminf(mn1[b], dd);
                    else
                        mn0[b] = fminf(mn0[b], dd);
                }
                mg = fminf(mg, dd);
            }
#pragma unroll
            for (int b = 0; b < NM - 4; b++) {
                if (h & (1 << (NM - 5 - b)))
                    mn1[b] = fminf(mn1[b], mg);
                else
                    mn0[b] = fminf(mn0[b], mg);
            }
        }
    } else {
#pragma unroll (logmap_unroll(NM))
        for (int i = 0; i < np; i++) {
            const float2 p = pts[i];
            const float dr = __fsub_rn(re, p.x), di = __fsub_rn(im, p.y);
            const float dd = __fmaf_rn(dr, dr, __fmul_rn(di, di));
#pragma unroll
            for (int b = 0; b < MB; b++) {
                if (NM || b < nm) {
                    if (i & (1 << (nm - 1 - b))) {
                        if (dd < mn1[b]) mn1[b] = dd;
                    } else {
                        if (dd < mn0[b]) mn0[b] = dd;
                    }
                }
            }
        }
    }
    const float scale = __fmul_rn(llr_gain, 0.25f);
    // A point whose (dd - M) * scale is at least 16, M the largest of the
    // per-bit minima, has every per-bit delta (dd - mn) * scale >= 16 --
    // subtraction and multiplication by a positive scale are monotone under
    // round-to-nearest and mn <= M -- so none of its terms enters a sum:
    // it is skipped with one test instead of one per bit (same sums).
    // From 32 points up (measured: 256APSK 3.35 -> 2.79 ms per 256 normal
    // frames; 16 points and fewer were faster without the test).
    float M = 0.0f;
#pragma unroll
    for (int b = 0; b < MB; b++)
        if (NM || b < nm)
            M = fmaxf(M, fmaxf(mn0[b], mn1[b]));
#pragma unroll (logmap_unroll(NM))
    for (int i = 0; i < np; i++) {
        const float2 p = pts[i];
        const float dr = __fsub_rn(re, p.x), di = __fsub_rn(im, p.y);
        const float dd = __fmaf_rn(dr, dr, __fmul_rn(di, di));
        if (NM == 0 || NM >= 5) {
            const bool near = valid && __fmul_rn(__fsub_rn(dd, M), scale) < 16.0f;
            if (VOTE ? !__any_sync(0xffffffffu, near) : !near)
                continue;
        }
#pragma unroll
        for (int b = 0; b < MB; b++) {
            if (NM || b < nm) {
                const bool one = i & (1 << (nm - 1 - b));
                const float delta = __fmul_rn(__fsub_rn(dd, one ? mn1[b] : mn0[b]), scale);
                if (VOTE) {
                    const bool in = valid && delta < 16.0f;
                    if (__any_sync(0xffffffffu, in)) {
                        const float e = dm_exp_neg(delta);
                        if (in && one) s1[b] = __fadd_rn(s1[b], e);
                        if (in && !one) s0[b] = __fadd_rn(s0[b], e);
                    }
                } else if (delta < 16.0f) {
                    if (one)
                        s1[b] = __fadd_rn(s1[b], dm_exp_neg(delta));
                    else
                        s0[b] = __fadd_rn(s0[b], dm_exp_neg(delta));
                }
            }
        }
    }
    if (!valid)
        return;
    const float half_gain = __fmul_rn(llr_gain, 0.5f);
#pragma unroll
    for (int b = 0; b < MB; b++) {
        if (NM || b < nm) {
            const float corr = __fmul_rn(2.0f, __fsub_rn(dm_log(fmaxf(s0[b], 1e-30f)),
                                                         dm_log(fmaxf(s1[b], 1e-30f))));
            const int p = (int)d.col[b] + j;
            if (p < d.fec_len)
                out[p] = llr_round(__fmaf_rn(__fsub_rn(mn1[b], mn0[b]), half_gain, corr));
        }
    }
}

// Demaps the symbols j0, j0 + step, ... (U of them, those inside the frame)
// of one frame: all U loads first (memory parallelism for the formula
// kinds), then each symbol.  KIND 0 QPSK, 1 8PSK, 2 log-MAP with NM bits.
template <int KIND, int NM, int U>
__device__ __forceinline__ void demap_span(const DevDemap& d, const float2* pts, const float2* sym, int16_t* out,
                                           int j0, int step, float noise_var, float llr_gain)
{
    float2 s[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int j = j0 + u * step;
        s[u] = j < d.interleaved_len ? __ldcs(sym + j) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int j = j0 + u * step;
        if (j >= d.interleaved_len)
            break;
        if (KIND == 0)
            demap_qpsk(d, s[u].x, s[u].y, j, noise_var, out);
        else if (KIND == 1)
            demap_8psk(d, s[u].x, s[u].y, j, llr_gain, out);
        else
            demap_logmap<NM>(d, pts, s[u].x, s[u].y, j, llr_gain, out);
    }
}

}  // namespace cusat
