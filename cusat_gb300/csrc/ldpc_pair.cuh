// Two short frames per CTA: the layered decoder with the frame state of two
// frames interleaved as int16 halves of 32-bit words.
//
// For codes decoded one layer per step (short frames), a CTA holds two
// frames A and B: APP word v = (A's APP of bit v, B's APP of bit v), the
// same layout as the one-frame kernel otherwise (information bits, then the
// parity bits transposed to [layer][check]).  Thread j still owns check row
// j of the step's layer, now for both frames: one slot descriptor load, one
// address computation, one 32-bit gather and one 32-bit scatter per edge
// serve the two frames, and the check arithmetic of process_check_packed
// (complemented magnitudes, one-DPX message magnitude, sign by LOP3) runs on
// the two halves -- each half is one frame's check, so nothing is merged
// across halves.  Message rows hold two bytes per edge (A's, then B's
// negated message).
//
// The two slots run independently: each has its own iteration count and
// syndrome vote (a check before every iteration, as in the one-frame
// kernel), and a slot whose frame has converged or reached the iteration
// cap takes the next frame of the launch's queue while the other slot goes
// on; a fresh frame's first iteration reads zero messages (its bytes of
// the loaded rows are masked).  Only frames whose channel LLRs are all
// within DevCode::fast_lim are decoded here (no int16 intermediate can
// overflow); a frame with a larger LLR is appended to DecodeArgs::list
// and decoded by a following launch of the one-frame kernel, which
// evaluates every saturation.  Single-code launches of the plain decoder
// only: learned weights and mixed batches use the one-frame kernel.
#pragma once

#include "ldpc_kernel.cuh"

namespace cusat {

// Slot state of a two-frame CTA (shared memory; written by thread 0 between
// barriers).
struct PairState {
    int f[2];       // frame index of the slot, -1 = empty
    int trial[2];   // iterations done on the slot's frame
    int cand;       // frame drawn from the queue
    int exhausted;  // the queue is drained
};

__device__ __forceinline__ uint32_t lds32(const unsigned char* smem, int off)
{
    return *reinterpret_cast<const uint32_t*>(smem + off);
}

__device__ __forceinline__ void sts32(unsigned char* smem, int off, uint32_t v)
{
    *reinterpret_cast<uint32_t*>(smem + off) = v;
}

// One check row of one layer for both frames.
template <int CMAX, int RW2>
__device__ __forceinline__ void process_check_pair(unsigned char* smem, const uint4* tb, int j, int ps0, int ps1r,
                                                   int ps1w, const uint4 (&cur)[RW2], uint4* dst)
{
    constexpr int NE = CMAX + 2;
    constexpr bool kKeepAddr = CMAX <= 14;
    const int one = c_pipe_one, neg = -one, two = one + one;
    const int j2 = j + j;
    uint32_t x[NE];
    int sa[kKeepAddr ? CMAX : 1];
    // gather: x = APP + (-m_old) for both frames; row bytes 2e, 2e + 1
    x[0] = vadd2(lds32(smem, ps0), prmt(cur[0].x, 0, pair_sel(0, false)));
    x[1] = vadd2(lds32(smem, ps1r), prmt(cur[0].x, 0, pair_sel(2, false)));
#pragma unroll
    for (int c = 0; c < CMAX; c++) {
        const int e = c + 2;
        const uint4 w = tb[c];
        const int ad = madd(rot720(j2, w.y, one), two, (int)w.x);
        if (kKeepAddr)
            sa[c] = madd((int)w.z, one, ad);
        const uint32_t rw = word_of(cur[e >> 3], (e >> 1) & 3);
        x[e] = vadd2(lds32(smem, ad), prmt(rw, 0, pair_sel((e & 1) * 2, false)));
    }
    // check node per half: max of ~|x| and the runner-up, sign parity
    uint32_t nr[NE];
    uint32_t N1 = 0x80008000u, N2 = 0x80008000u, SX = 0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
        nr[e] = __viaddmin_s16x2(x[e], 0xffffffffu, (uint32_t)madd((int)x[e], neg, neg));  // ~|x|
        const uint32_t t = vmin2(N1, nr[e]);
        N2 = vmax2(N2, t);
        N1 = vmax2(N1, nr[e]);
        SX ^= x[e];
    }
    const uint32_t R1c = vmin2((uint32_t)madd((int)N1, neg, neg), 0x00800080u);  // min(r1, 128) per frame
    const uint32_t R2c = vmin2((uint32_t)madd((int)N2, neg, neg), 0x00800080u);
    const uint32_t A = vadd2(R1c, R2c);
    const uint32_t B = __viaddmax_s16x2_relu(R1c, 0xffffffffu, 0u);  // max(r1c - 1, 0)
    // sign bits of x ^ Z flag a message >= 0: Z has a half's sign bit set
    // iff that frame's sign parity is even
    const uint32_t Z = lop3<0x0c>(SX, 0x80008000u, 0);  // ~SX & 0x80008000
    uint32_t nm[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
        const uint32_t mag = __viaddmax_s16x2_relu(A, nr[e], B);
        const uint32_t ns = prmt(x[e] ^ Z, 0, 0xbb99);
        const uint32_t P = vadd2(x[e], mag), Q = vadd2((uint32_t)madd((int)x[e], neg, neg), mag);
        const uint32_t app = lop3<0xb1>(P, Q, ns);  // ns ? x + mag : x - mag
        nm[e] = vadd2(mag, ns) ^ ns;                // -message
        int at;
        if (e == 0) {
            at = ps0;
        } else if (e == 1) {
            at = ps1w;
        } else if (kKeepAddr) {
            at = sa[e - 2];
        } else {
            const uint4 w = tb[e - 2];
            at = madd((int)w.z, one, madd(rot720(j2, w.y, one), two, (int)w.x));
        }
        sts32(smem, at, app);
    }
    uint32_t wv[RW2 * 4];
#pragma unroll
    for (int q = 0; q < RW2 * 4; q++)
        wv[q] = 2 * q < NE ? prmt(nm[2 * q], 2 * q + 1 < NE ? nm[2 * q + 1] : 0u, 0x6420) : 0u;
#pragma unroll
    for (int q = 0; q < RW2; q++)
        __stcg(dst + q, make_uint4(wv[4 * q], wv[4 * q + 1], wv[4 * q + 2], wv[4 * q + 3]));
}

// Completion of step s's shared groups for both frames: APP + sum(row - APP)
// per half (row0 + row1 - APP for the common two-writer group).
__device__ __forceinline__ void complete_groups_pair(unsigned char* smem, const uint32_t* stage, const SmemCode& t,
                                                     int s, int max_stage, int j)
{
    const int o0 = t.item_off[s], o1 = t.item_off[s + 1];
    const uint32_t* st = stage + (size_t)(s & 1) * max_stage * kM;
    const int neg = -c_pipe_one;
    for (int k = o0; k < o1; k++) {
        const uint2 it = t.items[k];
        const int r0 = (int)(it.y & 0xff), nr = (int)(it.y >> 8);
        uint32_t* app = reinterpret_cast<uint32_t*>(smem + it.x) + j;
        const uint32_t* rows = st + r0 * kM + j;
        const uint32_t na = vadd2((uint32_t)madd((int)*app, neg, neg), 0x00010001u);  // -APP
        uint32_t sum = rows[0];
        for (int g = 1; g < nr; g++)
            sum = vadd2(vadd2(sum, rows[g * kM]), na);
        *app = sum;
    }
}

// Syndrome of both frames' hard decisions.  Returns the halves (bit 0: A,
// bit 1: B) with an unsatisfied check; votes after the first step, then
// every 4 steps, stopping once every half in `want` has failed.
template <int CMAX>
__device__ int syndrome_pair(const unsigned char* smem, const SmemCode& t, int K, int q, int n_steps, int j,
                             bool active, int want)
{
    const int pty = 4 * K;
    const int one = c_pipe_one, two = one + one;
    int failed = 0;
    for (int s0 = 0, g = 1; s0 < n_steps; s0 += g, g = 4) {
        uint32_t bad = 0;
        if (active) {
            const int s1 = min(s0 + g, n_steps);
            for (int s = s0; s < s1; s++) {
                const int i = t.sched[2 * s];
                if (i < 0)
                    continue;
                uint32_t x = lds32(smem, pty + 4 * (i * kM + j));
                if (i > 0)
                    x ^= lds32(smem, pty + 4 * ((i - 1) * kM + j));
                else if (j > 0)
                    x ^= lds32(smem, pty + 4 * ((q - 1) * kM + j - 1));
                const uint4* tb = t.tab + i * CMAX;
#pragma unroll
                for (int e = 0; e < CMAX; e++) {
                    const uint4 w = tb[e];
                    x ^= lds32(smem, madd(rot720(2 * j, w.y, one), two, (int)w.x));
                }
                bad |= x;
            }
        }
        if (__syncthreads_or((bad >> 15) & 1))
            failed |= 1;
        if (__syncthreads_or(bad >> 31))
            failed |= 2;
        if ((failed & want) == want)
            break;
    }
    return failed;
}

// Packs the hard decisions of frame `half` (APP < 0 of its int16 half),
// MSB-first, K/8 bytes.
__device__ __forceinline__ void pack_hard_pair(const uint32_t* app, int K, int half, uint8_t* out)
{
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int base = warp * 32; base < K; base += nw * 32) {
        const int v = base + l;
        const bool neg = v < K && ((app[v] >> (15 + 16 * half)) & 1);
        const unsigned m = __ballot_sync(0xffffffffu, neg);
        const unsigned r = __byte_perm(__brev(m), 0, 0x0123);
        if (l < 4 && base + 8 * l < K)
            out[(base >> 3) + l] = (uint8_t)(r >> (8 * l));
    }
}

// Channel LLRs of one frame into half `half` of the APP words (the
// one-frame load with the -32768 clamp and the parity transpose); returns
// nonzero if one is outside the saturation-free range.
__device__ __forceinline__ int load_llr_pair(const DevCode& c, int16_t* app16, int half, const int16_t* src)
{
    const int K = c.K, R = c.R, q = c.q, lim = c.fast_lim;
    int over = 0;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        for (int v = threadIdx.x * 8; v < K; v += blockDim.x * 8) {
            const uint4 w = __ldcs(reinterpret_cast<const uint4*>(src + v));
            const uint32_t in[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int x = max((int)(int16_t)(in[k >> 1] >> (16 * (k & 1))), -32767);
                over |= abs(x) > lim;
                app16[2 * (v + k) + half] = (int16_t)x;
            }
        }
        // plain order: the rotated stores of the one-frame load cost this
        // kernel registers (57 -> 80) and measured slower here
        for (int p = threadIdx.x * 8; p < R; p += blockDim.x * 8) {
            const uint4 w = __ldcs(reinterpret_cast<const uint4*>(src + K + p));
            const uint32_t in[4] = {w.x, w.y, w.z, w.w};
            int li = p % q, lj = p / q;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int x = max((int)(int16_t)(in[k >> 1] >> (16 * (k & 1))), -32767);
                over |= abs(x) > lim;
                app16[2 * (K + li * kM + lj) + half] = (int16_t)x;
                if (++li == q) {
                    li = 0;
                    lj++;
                }
            }
        }
    } else {
        for (int v = threadIdx.x; v < c.N; v += blockDim.x) {
            const int x = max((int)src[v], -32767);
            over |= abs(x) > lim;
            const int at = v < K ? v : K + ((v - K) % q) * kM + (v - K) / q;
            app16[2 * at + half] = (int16_t)x;
        }
    }
    return over;
}

// The code's tables into shared memory, the slot descriptors rebased onto
// the two-frame layout: APP offsets doubled, stage rows of 360 words in
// sets of DecodeArgs::max_stage rows, the dummy/junk regions of this
// kernel.
template <int CMAX>
__device__ void load_code_pair(const DecodeArgs& a, unsigned char* smem, const DevCode& gc)
{
    DevCode* s_code = reinterpret_cast<DevCode*>(smem + a.sm_code);
    uint4* s_tab = reinterpret_cast<uint4*>(smem + a.sm_tab);
    int16_t* s_sched = reinterpret_cast<int16_t*>(smem + a.sm_sched);
    uint8_t* s_conf = smem + a.sm_conf;
    uint16_t* s_item_off = reinterpret_cast<uint16_t*>(smem + a.sm_item_off);
    uint2* s_items = reinterpret_cast<uint2*>(smem + a.sm_items);
    if (threadIdx.x == 0)
        *s_code = gc;
    for (int k = threadIdx.x; k < gc.q * CMAX; k += blockDim.x) {
        const uint4 w = gc.tab[k];
        uint4 o;
        o.y = 2 * w.y;
        o.w = 0;
        if (w.w == kSlotAbsent) {
            o.x = (uint32_t)a.sm_dummy;
            o.z = 4 * kM;  // the junk region follows the dummy region
        } else {
            o.x = 2 * w.x;
            if (w.w == kSlotStaged) {
                // the stage entry's row among the one-frame layout's sets of
                // kMaxStage rows -> this kernel's sets of max_stage rows
                const uint32_t rel = w.z + w.x;  // byte offset in the one-frame stage region
                const int set_row = (int)(rel / (2 * kM));
                const int set = set_row / kMaxStage, row = set_row % kMaxStage;
                o.z = (uint32_t)(a.sm_stage + (set * a.max_stage + row) * 4 * kM) - o.x;
            } else {
                o.z = 0;
            }
        }
        s_tab[k] = o;
    }
    for (int k = threadIdx.x; k < 2 * gc.n_steps; k += blockDim.x)
        s_sched[k] = gc.sched[k];
    for (int k = threadIdx.x; k < gc.n_steps; k += blockDim.x)
        s_conf[k] = gc.step_conf[k];
    for (int k = threadIdx.x; k <= gc.n_steps; k += blockDim.x)
        s_item_off[k] = gc.item_off[k];
    for (int k = threadIdx.x; k < gc.n_items; k += blockDim.x) {
        const uint2 it = gc.items[k];
        s_items[k] = make_uint2(2 * it.x, it.y);
    }
}

// One iteration (all steps of the schedule) on both frames; `keep` masks
// the loaded message rows (0x00ff00ff keeps frame A's bytes, 0xff00ff00
// B's; a frame in its first iteration reads zero messages).
template <int CMAX>
__device__ void iterate_pair(const DecodeArgs& a, const DevCode& c, unsigned char* smem, const uint32_t* stage,
                             const SmemCode& t, uint32_t keep)
{
    constexpr int NE = CMAX + 2;
    constexpr int RW2 = (2 * NE + 15) / 16;
    const int j = threadIdx.x;
    const bool active = j < kM;
    const int K = c.K, q = c.q, n_steps = c.n_steps;
    const int pty = 4 * K;
    uint4* msg_cta = a.msg + (size_t)blockIdx.x * (size_t)a.msg_stride;
    const bool load = keep != 0;
    uint4 cur[RW2];
    {
        const int i0 = t.sched[0];
        load_row<RW2>(cur, msg_cta + ((size_t)max(i0, 0) * kM + j) * RW2, load && active && i0 >= 0);
    }
    for (int s = 0; s < n_steps; s++) {
        const int i = t.sched[2 * s];
        uint4 nxt[RW2];
        {
            const int i_n = s + 1 < n_steps ? t.sched[2 * (s + 1)] : -1;
            load_row<RW2>(nxt, msg_cta + ((size_t)max(i_n, 0) * kM + j) * RW2, load && active && i_n >= 0);
        }
#pragma unroll
        for (int w = 0; w < RW2; w++) {
            cur[w].x &= keep;
            cur[w].y &= keep;
            cur[w].z &= keep;
            cur[w].w &= keep;
        }
        if (active) {
            if (s > 0 && t.conf[s - 1] == kConfDefer)
                complete_groups_pair(smem, stage, t, s - 1, a.max_stage, j);
            if (i >= 0) {
                const int ps0 = pty + 4 * (i * kM + j);
                const bool absent = (i == 0 && j == 0);
                // the absent edge reads the +32640 region and writes the junk region
                const int ps1r = i > 0 ? ps0 - 4 * kM : (absent ? a.sm_dummy : pty + 4 * ((q - 1) * kM + j - 1));
                const int ps1w = absent ? a.sm_dummy + 4 * kM : ps1r;
                process_check_pair<CMAX, RW2>(smem, t.tab + i * CMAX, j, ps0, ps1r, ps1w, cur,
                                              msg_cta + ((size_t)i * kM + j) * RW2);
            }
        }
        if (t.conf[s] == kConfMid) {
            __syncthreads();
            if (active)
                complete_groups_pair(smem, stage, t, s, a.max_stage, j);
        }
        __syncthreads();
#pragma unroll
        for (int w = 0; w < RW2; w++)
            cur[w] = nxt[w];
    }
}

template <int CMAX>
__global__ void __launch_bounds__(lane_threads(1), 2) ldpc_pair_kernel(DecodeArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* app = reinterpret_cast<uint32_t*>(smem);
    int16_t* app16 = reinterpret_cast<int16_t*>(smem);
    uint32_t* dummy = reinterpret_cast<uint32_t*>(smem + a.sm_dummy);
    const uint32_t* stage = reinterpret_cast<const uint32_t*>(smem + a.sm_stage);
    const DevCode& c = *reinterpret_cast<const DevCode*>(smem + a.sm_code);
    PairState* ps = reinterpret_cast<PairState*>(smem + a.sm_misc);
    const SmemCode t = {reinterpret_cast<const uint4*>(smem + a.sm_tab), smem + a.sm_cnt,
                        reinterpret_cast<const int16_t*>(smem + a.sm_sched), smem + a.sm_conf,
                        reinterpret_cast<const uint16_t*>(smem + a.sm_item_off),
                        reinterpret_cast<const uint2*>(smem + a.sm_items)};
    for (int k = threadIdx.x; k < kM; k += blockDim.x)
        dummy[k] = 0x7f807f80u;  // +32640 in both halves (see the one-frame kernel)
    load_code_pair<CMAX>(a, smem, a.code);
    if (threadIdx.x == 0) {
        ps->f[0] = ps->f[1] = -1;
        ps->trial[0] = ps->trial[1] = 0;
        ps->exhausted = 0;
    }
    __syncthreads();
    const int T = a.max_trials, K = c.K, q = c.q, n_steps = c.n_steps;
    const int period = a.syn_period > 1 ? a.syn_period : 1;
    const bool active = threadIdx.x < kM;
    for (;;) {
        // fill empty slots from the queue; frames that need the saturating
        // arithmetic go to the list of the following one-frame launch
        for (int h = 0; h < 2; h++) {
            while (ps->f[h] < 0 && !ps->exhausted) {
                if (threadIdx.x == 0)
                    ps->cand = (int)atomicAdd(a.queue, 1u);
                __syncthreads();
                const int f = ps->cand;
                if (f >= a.n_frames) {
                    __syncthreads();
                    if (threadIdx.x == 0)
                        ps->exhausted = 1;
                    __syncthreads();
                    break;
                }
                const int over = load_llr_pair(c, app16, h, a.llr + (size_t)f * c.N);
                if (__syncthreads_or(over)) {
                    if (threadIdx.x == 0) {
                        // the list holds n_frames entries; the one-frame
                        // launch after this one zeroes the count
                        const unsigned k = atomicAdd(a.list_count, 1u);
                        if (k < (unsigned)a.n_frames)
                            a.list[k] = f;
                    }
                } else if (threadIdx.x == 0) {
                    ps->f[h] = f;
                    ps->trial[h] = 0;
                }
                __syncthreads();
            }
        }
        const int f0 = ps->f[0], f1 = ps->f[1], t0 = ps->trial[0], t1 = ps->trial[1];
        if (f0 < 0 && f1 < 0)
            break;
        // syndrome before the iteration (and at the cap) of each slot
        int want = 0;
        if (f0 >= 0 && (period == 1 || t0 % period == 0 || t0 == T))
            want |= 1;
        if (f1 >= 0 && (period == 1 || t1 % period == 0 || t1 == T))
            want |= 2;
        const int failed = want ? syndrome_pair<CMAX>(smem, t, K, q, n_steps, threadIdx.x, active, want) : 3;
        int retired = 0;
        for (int h = 0; h < 2; h++) {
            const int f = h ? f1 : f0, tr = h ? t1 : t0;
            if (f < 0)
                continue;
            const bool conv = ((want >> h) & 1) && !((failed >> h) & 1);
            if (conv || tr == T) {
                pack_hard_pair(app, K, h, a.hard + (size_t)f * (K / 8));
                if (threadIdx.x == 0)
                    a.trials[f] = conv ? T - tr : -1;
                retired |= 1 << h;
            }
        }
        __syncthreads();
        if (retired) {
            if (threadIdx.x == 0) {
                if (retired & 1)
                    ps->f[0] = -1;
                if (retired & 2)
                    ps->f[1] = -1;
            }
            __syncthreads();
            continue;
        }
        const uint32_t keep = (f0 >= 0 && t0 > 0 ? 0x00ff00ffu : 0u) | (f1 >= 0 && t1 > 0 ? 0xff00ff00u : 0u);
        iterate_pair<CMAX>(a, c, smem, stage, t, keep);
        if (threadIdx.x == 0) {
            if (f0 >= 0)
                ps->trial[0] = t0 + 1;
            if (f1 >= 0)
                ps->trial[1] = t1 + 1;
        }
        __syncthreads();
    }
    // the last CTA out rearms the frame counters (as the one-frame kernel)
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(a.queue + 1, 1u) == gridDim.x - 1) {
            atomicExch(a.queue, 0u);
            atomicExch(a.queue + 1, 0u);
        }
    }
}

}  // namespace cusat
