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

// LLRs of symbol j.  QPSK: 2 LLRs at positions 2j, 2j+1 (no interleaver);
// 8PSK: formula after the -pi/8 rotation; APSK: log-MAP over the points
// (pts in shared memory).  Writes n_mod (pos, llr) pairs; pos >= fec_len is
// dropped by the caller.  Reference: cuda/demapper_kernel.cu:53-183.
__device__ __forceinline__ int demap_symbol(const DevDemap& d, const float2* pts, float re, float im,
                                            int j, float noise_var, float llr_gain, int* pos,
                                            int16_t* llr)
{
    if (d.kind == 0) {
        const float scalar = __fdiv_rn(2.0f * 1.4142135623730951f, noise_var);
        pos[0] = 2 * j;
        pos[1] = 2 * j + 1;
        llr[0] = llr_round(__fmul_rn(re, scalar));
        llr[1] = llr_round(__fmul_rn(im, scalar));
        if (2 * j + 1 >= d.fec_len)
            pos[0] = pos[1] = d.fec_len;  // dropped together, like the reference
        return 2;
    }
    if (d.kind == 1) {
        const float C8 = 0.92387953251128676f, S8 = 0.38268343236508977f;
        const float R2 = 0.70710678118654752f;
        const float DIST = 2.0f * 0.38268343236508977f;
        const float cr = __fmaf_rn(re, C8, __fmul_rn(im, S8));
        const float ci = __fmaf_rn(-re, S8, __fmul_rn(im, C8));
        const float scale = __fmul_rn(DIST, llr_gain);
        llr[0] = llr_round(__fmul_rn(__fmul_rn(R2, __fsub_rn(fabsf(cr), fabsf(ci))), scale));
        llr[1] = llr_round(__fmul_rn(cr, scale));
        llr[2] = llr_round(__fmul_rn(ci, scale));
        pos[0] = (int)d.col[0] + j;
        pos[1] = (int)d.col[1] + j;
        pos[2] = (int)d.col[2] + j;
        return 3;
    }
    const int nm = d.n_mod;
    float mn0[8], mn1[8], s0[8], s1[8];
#pragma unroll
    for (int b = 0; b < 8; b++) {
        mn0[b] = 1e30f;
        mn1[b] = 1e30f;
        s0[b] = 0.0f;
        s1[b] = 0.0f;
    }
    for (int i = 0; i < d.n_points; i++) {
        const float2 p = pts[i];
        const float dr = __fsub_rn(re, p.x), di = __fsub_rn(im, p.y);
        const float dd = __fmaf_rn(dr, dr, __fmul_rn(di, di));
#pragma unroll
        for (int b = 0; b < 8; b++) {
            if (b < nm) {
                if (i & (1 << (nm - 1 - b))) {
                    if (dd < mn1[b]) mn1[b] = dd;
                } else {
                    if (dd < mn0[b]) mn0[b] = dd;
                }
            }
        }
    }
    const float scale = __fmul_rn(llr_gain, 0.25f);
    for (int i = 0; i < d.n_points; i++) {
        const float2 p = pts[i];
        const float dr = __fsub_rn(re, p.x), di = __fsub_rn(im, p.y);
        const float dd = __fmaf_rn(dr, dr, __fmul_rn(di, di));
#pragma unroll
        for (int b = 0; b < 8; b++) {
            if (b < nm) {
                if (i & (1 << (nm - 1 - b))) {
                    const float delta = __fmul_rn(__fsub_rn(dd, mn1[b]), scale);
                    if (delta < 16.0f) s1[b] = __fadd_rn(s1[b], dm_exp_neg(delta));
                } else {
                    const float delta = __fmul_rn(__fsub_rn(dd, mn0[b]), scale);
                    if (delta < 16.0f) s0[b] = __fadd_rn(s0[b], dm_exp_neg(delta));
                }
            }
        }
    }
    const float half_gain = __fmul_rn(llr_gain, 0.5f);
#pragma unroll
    for (int b = 0; b < 8; b++) {
        if (b < nm) {
            const float corr = __fmul_rn(2.0f, __fsub_rn(dm_log(fmaxf(s0[b], 1e-30f)),
                                                         dm_log(fmaxf(s1[b], 1e-30f))));
            llr[b] = llr_round(__fmaf_rn(__fsub_rn(mn1[b], mn0[b]), half_gain, corr));
            pos[b] = (int)d.col[b] + j;
        }
    }
    return nm;
}

}  // namespace cusat
