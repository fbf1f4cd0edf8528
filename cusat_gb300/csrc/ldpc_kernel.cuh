// Layered offset min-sum LDPC decoder for sm_103a.
//
// One CTA decodes one frame at a time and pulls frames from a queue
// (persistent).  Each lane of 384 threads (12 warps) processes one layer of
// the schedule step, thread j owning check row j (j < 360) of that layer;
// LANES = 2 runs the paired layers of the reference's schedule side by side
// (reference lib/cusat_dsp/cuda/ldpc_decode_kernel.cu:947-963).
//
// Frame state in shared memory: the int16 APP of the N bits, information
// bits in natural order then the parity bits transposed to
// [layer][check] (slot i*360 + j holds parity bit q*j + i).  Check j of
// layer i reads information bit base + (j - shift) mod 360 of each
// circulant: consecutive threads read consecutive halfwords, so every
// gather and scatter is a conflict-free shared-memory access.  Check-to-bit
// messages (int8) live in this CTA's global scratch, one 16- or 32-byte row
// per check (two parity edges first, then the circulants), loaded with
// 128-bit loads one step ahead of use.
//
// Arithmetic.  The reference semantics (qsat16 extrinsic, offset min-sum
// with beta 1, int8 clamp, saturating APP updates) are computed exactly.
// When every channel LLR of the frame is within DevCode::fast_lim, no
// intermediate can leave int16 (|APP| <= |llr| + 127 (deg + 1)), and the
// kernel takes the SAT = false path that drops the clamps; otherwise the
// SAT = true path evaluates every saturation.  Magnitudes are compared
// before the offset: offset-then-clamp is monotone, so min1/min2 and the
// "is this edge the minimum" test give the same messages as the
// reference's finalp_oms_i16 (:242-275), ties included.
//
// Checks of one step that share a variable node (a table row with two
// accumulator addresses in one layer, or in both paired layers) are a data
// race in the reference (:793-802).  Here they are resolved
// deterministically, step-Jacobi: the first circulant on the node (owner)
// keeps its updated value in a register, the others (guests) write their
// message delta to a stage row, and after a CTA barrier the owner stores
// sat16(APP + all deltas).
#pragma once

#include "fec_device.cuh"

namespace cusat {

struct DecodeArgs {
    DevCode code;
    DevDemap dm;             // fused demap when sym != nullptr
    const int16_t* llr;      // [n_frames][N] int16 LLRs (unfused)
    const float* sym;        // [n_frames][xfec][2] symbols (fused)
    float noise_var, llr_gain;
    int n_frames, max_trials;
    uint8_t* hard;           // [n_frames][K/8]
    int32_t* trials;         // [n_frames]
    uint4* msg;              // [gridDim.x][R * msg_row / 16] scratch
    unsigned int* queue;     // frame counter, zero at launch
    const int16_t* weights;  // learned min-sum weights or nullptr (plain)
    // shared-memory carve-up (bytes)
    int sm_stage, sm_circ, sm_sched, sm_cnt, sm_conf, sm_pts, sm_misc, sm_total;
};

__device__ __forceinline__ int sat16(int v) { return max(-32768, min(32767, v)); }

// signed byte b (0..3) of w
__device__ __forceinline__ int sbyte(uint32_t w, int b)
{
    // prmt with the sign-replicate bit set on the three upper selectors
    int r;
    asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(w), "r"((unsigned)((0x8 | b) * 0x1110 + b)));
    return r;
}

__device__ __forceinline__ uint32_t word_of(const uint4& v, int k)
{
    return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

template <int RW>
__device__ __forceinline__ void load_row(uint4 (&dst)[RW], const uint4* src, bool pred)
{
#pragma unroll
    for (int w = 0; w < RW; w++)
        dst[w] = pred ? __ldcg(src + w) : make_uint4(0, 0, 0, 0);
}

// Syndrome of the current hard decisions: true iff every check is
// satisfied.  Steps are voted in groups of 4 (one barrier per group), so a
// failing frame pays about one group.  Reference :693-745.
template <int CMAX, int LANES>
__device__ bool syndrome_ok(const int16_t* app, const uint32_t* s_circ, const int16_t* s_sched,
                            const uint8_t* s_cnt, int K, int q, int n_steps, int lane, int j,
                            bool active)
{
    const int16_t* pty = app + K;
    for (int s0 = 0; s0 < n_steps; s0 += 4) {
        int bad = 0;
        if (active) {
            const int s1 = min(s0 + 4, n_steps);
            for (int s = s0; s < s1; s++) {
                const int i = s_sched[2 * s + lane];
                if (i < 0)
                    continue;
                const int cnt = s_cnt[i];
                int x = pty[i * kM + j];
                if (i > 0)
                    x ^= pty[(i - 1) * kM + j];
                else if (j > 0)
                    x ^= pty[(q - 1) * kM + j - 1];
                const uint32_t* ci = s_circ + i * CMAX;
#pragma unroll
                for (int e = 0; e < CMAX; e++) {
                    if (e < cnt) {
                        const uint32_t w = ci[e];
                        int m = j - (int)((w >> 16) & 0x1ff);
                        m += (m >> 31) & kM;
                        x ^= app[(int)(w & 0xffff) + m];
                    }
                }
                bad |= x;
            }
        }
        if (__syncthreads_or(bad < 0))
            return false;
    }
    return true;
}

// Packs APP[0..K) < 0 MSB-first into K/8 bytes.
__device__ __forceinline__ void pack_hard(const int16_t* app, int K, uint8_t* out)
{
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int base = warp * 32; base < K; base += nw * 32) {
        const int v = base + l;
        const bool neg = v < K && app[v] < 0;
        const unsigned m = __ballot_sync(0xffffffffu, neg);
        const unsigned r = __byte_perm(__brev(m), 0, 0x0123);
        if (l < 4 && base + 8 * l < K)
            out[(base >> 3) + l] = (uint8_t)(r >> (8 * l));
    }
}

// Learned weights: offset beta and scale alpha/64 for (iteration, degree);
// nullptr = beta 1, alpha off (the reference's plain decoder).
__device__ __forceinline__ int scaled_mag(int r, int beta, int alpha)
{
    int m = max(r - beta, 0);
    if (alpha > 0)
        m = (min(m, 32767) * alpha + 32) >> 6;
    return min(m, 127);
}

template <int CMAX, int LANES, bool SAT>
__device__ void decode_frame(const DecodeArgs& a, int16_t* app, int16_t* stage, const uint32_t* s_circ,
                             const int16_t* s_sched, const uint8_t* s_cnt, const uint8_t* s_conf, int f)
{
    constexpr int NE = CMAX + 2;
    constexpr int RW = (NE + 15) / 16;
    const DevCode& c = a.code;
    const int tid = threadIdx.x;
    const int lane = (LANES == 2 && tid >= kLaneThreads) ? 1 : 0;
    const int j = tid - lane * kLaneThreads;
    const bool active = j < kM;
    const int K = c.K, q = c.q, T = a.max_trials, n_steps = c.n_steps;
    uint4* msg_cta = a.msg + (size_t)blockIdx.x * ((size_t)c.R * RW);
    int result = -1;

    for (int trial = 0;; trial++) {
        if (syndrome_ok<CMAX, LANES>(app, s_circ, s_sched, s_cnt, K, q, n_steps, lane, j, active)) {
            result = T - trial;
            break;
        }
        if (trial == T)
            break;
        const bool load = trial > 0;
        uint4 cur[RW];
        {
            const int i0 = s_sched[lane];
            load_row<RW>(cur, msg_cta + ((size_t)max(i0, 0) * kM + j) * RW, load && active && i0 >= 0);
        }
        for (int s = 0; s < n_steps; s++) {
            const int i = s_sched[2 * s + lane];
            uint4 nxt[RW];
            {
                const int i_n = s + 1 < n_steps ? s_sched[2 * (s + 1) + lane] : -1;
                load_row<RW>(nxt, msg_cta + ((size_t)max(i_n, 0) * kM + j) * RW,
                             load && active && i_n >= 0);
            }
            const bool work = active && i >= 0;
            // keep the bit indices of the circulants in registers when they fit
            constexpr bool KEEP_VN = CMAX <= 14;
            int dd[NE];
            int vn[KEEP_VN ? CMAX : 1];
            int cnt = 0;
            const uint32_t* ci = s_circ + max(i, 0) * CMAX;
            if (work) {
                cnt = s_cnt[i];
                // gather: two parity edges, then the circulants
                const int ps0 = K + i * kM + j;
                const int ps1 = i > 0 ? ps0 - kM : (j > 0 ? K + (q - 1) * kM + j - 1 : -1);
                {
                    const int a0 = app[ps0] - sbyte(cur[0].x, 0);
                    dd[0] = SAT ? sat16(a0) : a0;
                    if (ps1 >= 0) {
                        const int a1 = app[ps1] - sbyte(cur[0].x, 1);
                        dd[1] = SAT ? sat16(a1) : a1;
                    } else {
                        dd[1] = kBig;
                    }
                }
#pragma unroll
                for (int e = 0; e < CMAX; e++) {
                    if (e < cnt) {
                        const uint32_t w = ci[e];
                        int m = j - (int)((w >> 16) & 0x1ff);
                        m += (m >> 31) & kM;
                        const int v = (int)(w & 0xffff) + m;
                        if (KEEP_VN)
                            vn[KEEP_VN ? e : 0] = v;
                        const int x = app[v] - sbyte(word_of(cur[(e + 2) >> 4], ((e + 2) >> 2) & 3), (e + 2) & 3);
                        dd[2 + e] = SAT ? sat16(x) : x;
                    } else {
                        dd[2 + e] = kBig;
                    }
                }
                // check node: min1/min2 of |extrinsic|, sign product
                int r1 = kBig, r2 = kBig, sx = 0;
#pragma unroll
                for (int e = 0; e < NE; e++) {
                    const int r = abs(dd[e]);
                    r2 = min(r2, max(r1, r));
                    r1 = min(r1, r);
                    sx ^= dd[e];
                }
                int m1, m2;
                if (a.weights) {
                    const int deg = cnt + (ps1 >= 0 ? 2 : 1);
                    const int16_t* w = a.weights + ((size_t)trial * 32 + deg) * 2;
                    m1 = scaled_mag(r1, w[0], w[1]);
                    m2 = scaled_mag(r2, w[0], w[1]);
                } else {
                    m1 = min(max(r1 - 1, 0), 127);
                    m2 = min(max(r2 - 1, 0), 127);
                }
                // messages, scatter, and the new message row
                uint32_t wv[RW * 4];
#pragma unroll
                for (int k = 0; k < RW * 4; k++)
                    wv[k] = 0;
#pragma unroll
                for (int e = 0; e < NE; e++) {
                    const int oth = (abs(dd[e]) == r1) ? m2 : m1;
                    const int mg = ((sx ^ dd[e]) < 0) ? -oth : oth;
                    wv[e >> 2] = __byte_perm(wv[e >> 2], (uint32_t)mg,
                                             (e & 3) == 0 ? 0x3214 : (e & 3) == 1 ? 0x3240
                                                                   : (e & 3) == 2 ? 0x3410 : 0x4210);
                    if (e == 0) {
                        app[ps0] = (int16_t)(SAT ? sat16(dd[0] + mg) : dd[0] + mg);
                    } else if (e == 1) {
                        if (ps1 >= 0)
                            app[ps1] = (int16_t)(SAT ? sat16(dd[1] + mg) : dd[1] + mg);
                    } else if (e - 2 < cnt) {
                        const uint32_t w = ci[e - 2];
                        int v;
                        if (KEEP_VN) {
                            v = vn[KEEP_VN ? e - 2 : 0];
                        } else {
                            int m = j - (int)((w >> 16) & 0x1ff);
                            m += (m >> 31) & kM;
                            v = (int)(w & 0xffff) + m;
                        }
                        const int delta = mg - sbyte(word_of(cur[e >> 4], (e >> 2) & 3), e & 3);
                        // SAT: re-read the APP (unchanged: no other check of
                        // the step writes this bit) and saturate once
                        const int nv = SAT ? app[v] + delta : dd[e] + mg;
                        const uint32_t role = (w >> 25) & 3;
                        if (role == kRolePlain)
                            app[v] = (int16_t)(SAT ? sat16(nv) : nv);
                        else if (role == kRoleGuest)
                            stage[((w >> 27) & 7) * kM + (v - (int)(w & 0xffff))] = (int16_t)delta;
                        else
                            dd[e] = nv;  // owner: completed after the barrier
                    }
                }
                uint4* dst = msg_cta + ((size_t)i * kM + j) * RW;
#pragma unroll
                for (int w = 0; w < RW; w++)
                    __stcg(dst + w, make_uint4(wv[4 * w], wv[4 * w + 1], wv[4 * w + 2], wv[4 * w + 3]));
            }
            if (s_conf[s]) {
                __syncthreads();
                if (work) {
#pragma unroll
                    for (int e = 0; e < CMAX; e++) {
                        const uint32_t w = ci[e];
                        if (e < cnt && ((w >> 25) & 3) == kRoleOwner) {
                            const int k0 = (w >> 27) & 7, ng = (int)(w >> 30) + 1;
                            int m = j - (int)((w >> 16) & 0x1ff);
                            m += (m >> 31) & kM;
                            int sum = dd[2 + e];
                            for (int g = 0; g < ng; g++)
                                sum += stage[(k0 + g) * kM + m];
                            app[(int)(w & 0xffff) + m] = (int16_t)(SAT ? sat16(sum) : sum);
                        }
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int w = 0; w < RW; w++)
                cur[w] = nxt[w];
        }
    }
    pack_hard(app, K, a.hard + (size_t)f * (K / 8));
    if (threadIdx.x == 0)
        a.trials[f] = result;
}

// Channel LLRs of frame f into shared memory; returns nonzero if one is
// outside the saturation-free range.  Reference init :655-670 (clamp to
// +-32767, parity transpose).
__device__ __forceinline__ int load_llr(const DecodeArgs& a, int16_t* app, int f)
{
    const DevCode& c = a.code;
    const int K = c.K, R = c.R, q = c.q, lim = c.fast_lim;
    const int16_t* src = a.llr + (size_t)f * c.N;
    int over = 0;
    const bool vec = ((reinterpret_cast<uintptr_t>(a.llr) & 15) == 0);
    if (vec) {
        for (int v = threadIdx.x * 8; v < K; v += blockDim.x * 8) {
            const uint4 w = __ldcs(reinterpret_cast<const uint4*>(src + v));
            uint32_t o[4];
            const uint32_t in[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                int lo = (int)(int16_t)(in[k] & 0xffff), hi = (int)(int16_t)(in[k] >> 16);
                lo = max(lo, -32767);
                hi = max(hi, -32767);
                over |= (abs(lo) > lim) | (abs(hi) > lim);
                o[k] = (uint32_t)(lo & 0xffff) | ((uint32_t)hi << 16);
            }
            *reinterpret_cast<uint4*>(app + v) = make_uint4(o[0], o[1], o[2], o[3]);
        }
        for (int p = threadIdx.x * 8; p < R; p += blockDim.x * 8) {
            const uint4 w = __ldcs(reinterpret_cast<const uint4*>(src + K + p));
            const uint32_t in[4] = {w.x, w.y, w.z, w.w};
            int li = p % q, lj = p / q;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                int x = (int)(int16_t)(in[k >> 1] >> (16 * (k & 1)));
                x = max(x, -32767);
                over |= abs(x) > lim;
                app[K + li * kM + lj] = (int16_t)x;
                if (++li == q) {
                    li = 0;
                    lj++;
                }
            }
        }
    } else {
        for (int v = threadIdx.x; v < c.N; v += blockDim.x) {
            int x = max((int)src[v], -32767);
            over |= abs(x) > lim;
            if (v < K)
                app[v] = (int16_t)x;
            else
                app[K + ((v - K) % q) * kM + (v - K) / q] = (int16_t)x;
        }
    }
    return over;
}

// Fused demap + deinterleave of frame f's symbols straight into the APP.
__device__ __forceinline__ int demap_into(const DecodeArgs& a, int16_t* app, const float2* pts, int f)
{
    const DevCode& c = a.code;
    const DevDemap& d = a.dm;
    const int K = c.K, q = c.q, lim = c.fast_lim, N = c.N;
    const float2* src = reinterpret_cast<const float2*>(a.sym) + (size_t)f * d.xfec;
    int over = 0;
    for (int jj = threadIdx.x; jj < d.interleaved_len; jj += blockDim.x) {
        const float2 s = __ldcs(src + jj);
        int pos[8];
        int16_t l[8];
        const int nb = demap_symbol(d, pts, s.x, s.y, jj, a.noise_var, a.llr_gain, pos, l);
#pragma unroll
        for (int b = 0; b < 8; b++) {
            if (b < nb && pos[b] < N) {
                const int x = max((int)l[b], -32767);
                over |= abs(x) > lim;
                const int p = pos[b];
                if (p < K)
                    app[p] = (int16_t)x;
                else
                    app[K + ((p - K) % q) * kM + (p - K) / q] = (int16_t)x;
            }
        }
    }
    return over;
}

template <int CMAX, int LANES, bool FUSED>
__global__ void __launch_bounds__(LANES * kLaneThreads, LANES == 2 ? 1 : 2) ldpc_layered_kernel(DecodeArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    int16_t* app = reinterpret_cast<int16_t*>(smem);
    int16_t* stage = reinterpret_cast<int16_t*>(smem + a.sm_stage);
    uint32_t* s_circ = reinterpret_cast<uint32_t*>(smem + a.sm_circ);
    int16_t* s_sched = reinterpret_cast<int16_t*>(smem + a.sm_sched);
    uint8_t* s_cnt = smem + a.sm_cnt;
    uint8_t* s_conf = smem + a.sm_conf;
    float2* pts = reinterpret_cast<float2*>(smem + a.sm_pts);
    int* s_misc = reinterpret_cast<int*>(smem + a.sm_misc);
    const DevCode& c = a.code;

    for (int k = threadIdx.x; k < c.q * CMAX; k += blockDim.x)
        s_circ[k] = c.circ[k];
    for (int k = threadIdx.x; k < 2 * c.n_steps; k += blockDim.x)
        s_sched[k] = c.sched[k];
    for (int k = threadIdx.x; k < c.q; k += blockDim.x)
        s_cnt[k] = c.cnt[k];
    for (int k = threadIdx.x; k < c.n_steps; k += blockDim.x)
        s_conf[k] = c.step_conf[k];
    if (FUSED && a.dm.kind == 2)
        for (int k = threadIdx.x; k < a.dm.n_points; k += blockDim.x)
            pts[k] = a.dm.points[k];

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0)
            s_misc[0] = (int)atomicAdd(a.queue, 1u);
        __syncthreads();
        const int f = s_misc[0];
        if (f >= a.n_frames)
            break;
        const int over = FUSED ? demap_into(a, app, pts, f) : load_llr(a, app, f);
        if (__syncthreads_or(over))
            decode_frame<CMAX, LANES, true>(a, app, stage, s_circ, s_sched, s_cnt, s_conf, f);
        else
            decode_frame<CMAX, LANES, false>(a, app, stage, s_circ, s_sched, s_cnt, s_conf, f);
    }
}

}  // namespace cusat
