// Layered offset min-sum LDPC decoder for sm_103a.
//
// One CTA decodes one frame at a time and pulls frames from a queue
// (persistent).  Each lane processes one layer of the schedule step, thread
// j owning check row j (j < 360) of that layer (with two lanes, 360 threads
// each, lane 1 starts mid-warp);
// LANES = 2 runs the paired layers of the reference's schedule side by side
// (reference lib/cusat_dsp/cuda/ldpc_decode_kernel.cu:947-963).
//
// Frame state in shared memory: the int16 APP of the N bits, information
// bits in natural order then the parity bits transposed to
// [layer][check] (slot i*360 + j holds parity bit q*j + i).  Check j of
// layer i reads bit (j + r) mod 360 of each circulant's group, found with
// one add and one unsigned DPX min (viaddmin): consecutive threads read
// consecutive halfwords, so gathers and scatters are conflict-free
// shared-memory accesses.  Check-to-bit messages (int8) live in this CTA's
// global scratch, one row of 4, 8, 16 or 32 bytes per check (the two parity
// edges, then the circulants; row_words), loaded one step ahead of use.
//
// Arithmetic.  The reference semantics (qsat16 extrinsic, offset min-sum
// with beta 1, int8 clamp, saturating APP updates) are computed exactly.
// When every channel LLR of the frame is within DevCode::fast_lim no
// intermediate can leave int16 (|APP| <= |llr| + 127 dv) and the kernel
// runs the packed path: two edges of a check row per 32-bit register as
// int16 lanes (process_check_packed).  Otherwise one edge per instruction
// with every saturation evaluated (process_check, SAT).  Magnitudes are
// compared before the offset: offset-then-clamp is monotone, so min1/min2
// and the "is this edge the minimum" test give the messages of the
// reference's finalp_oms_i16 (:242-275), ties included.
//
// Checks of one step that share a variable node (a table row with two
// accumulator addresses in one layer, or in both paired layers) are a data
// race in the reference (:793-802).  They are resolved deterministically,
// step-Jacobi: the circulants of a shared group store their updates to
// their own stage rows instead of the APP (every slot stores to its bit's
// address plus a per-slot offset, so the body has no per-slot branch), and
// a group item stores sat16(APP + all deltas) -- at the start of the next
// step when that step does not touch the group, else after a barrier.
//
// Syndrome.  The check before each iteration (reference :693-745) votes
// after the first step's checks and then every 4 steps, stopping at the
// first failing group.  DecodeArgs::syn_period > 1 checks only before every
// syn_period-th iteration and at the cap (the reference's
// CUSAT_LDPC_SYN_PERIOD, :1237-1241).
#pragma once

#include "fec_device.cuh"

namespace cusat {

// One frame of a mixed batch (device memory).
struct FrameDesc {
    int code;                // index into DecodeArgs::codes
    int pad[3];
    const int16_t* llr;      // [N] channel LLRs
    uint8_t* hard;           // [K/8]
    int32_t* trials;         // [1]
};

struct DecodeArgs {
    DevCode code;            // single-code launch (codes == nullptr)
    const DevCode* codes;    // mixed batch: per-code tables, frames[f].code indexes them
    const FrameDesc* frames;
    const int16_t* llr;      // single code: [n_frames][N] int16 LLRs
    int n_frames, max_trials;
    int syn_period;          // syndrome before iterations t with t % syn_period == 0 (and at the cap); <= 1: every one
    uint8_t* hard;           // single code: [n_frames][K/8]
    int32_t* trials;         // single code: [n_frames]
    uint4* msg;              // [gridDim.x][msg_stride] scratch
    int msg_stride;          // uint4 per CTA: max over the launch's codes of R * row bytes / 16
    unsigned int* queue;     // [0] frame counter, [1] CTAs done: zero at launch, zeroed again by the last CTA
    // Frame lists between the frame-pair kernel and the one-frame kernel
    // (single code): the pair kernel appends the frames that need the
    // saturating arithmetic to list; a one-frame launch with list non-null
    // decodes list[0..*list_count) only, and its last CTA out zeroes
    // *list_count.  nullptr otherwise.
    int* list;
    unsigned int* list_count;
    int max_stage;           // frame-pair kernel: stage rows per set (the plan's busiest step)
    // shared-memory carve-up (bytes)
    int sm_dummy, sm_stage, sm_tab, sm_cnt, sm_sched, sm_conf, sm_item_off, sm_items, sm_code, sm_misc, sm_msgbuf,
        sm_total;
};

// Where one frame comes from and goes to.
struct Job {
    const int16_t* llr;
    uint8_t* hard;
    int32_t* trials;
};

// Shared-memory views of the code tables.
struct SmemCode {
    const uint4* tab;  // per slot: x = byte base, y = 2 r, z = store offset
    const uint8_t* cnt;
    const int16_t* sched;
    const uint8_t* conf;
    const uint16_t* item_off;
    const uint2* items;
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

// old message of edge e of a row held in registers
template <int RW>
__device__ __forceinline__ int row_byte(const uint4 (&row)[RW], int e)
{
    return sbyte(word_of(row[e >> 4], (e >> 2) & 3), e & 3);
}

template <int RW>
__device__ __forceinline__ void load_row(uint4 (&dst)[RW], const uint4* src, bool pred)
{
#pragma unroll
    for (int w = 0; w < RW; w++)
        dst[w] = pred ? __ldcg(src + w) : make_uint4(0, 0, 0, 0);
}

// Message rows of the one-frame kernel: W 32-bit words per check row
// (row_words: 4, 8, 16 or 32 bytes, the edge count rounded up), moved with
// one load or store of that width (two 128-bit ones for 32 bytes).
template <int W>
__device__ __forceinline__ int row_byte_w(const uint32_t (&row)[W], int e)
{
    return sbyte(row[e >> 2], e & 3);
}

template <int W>
__device__ __forceinline__ void load_row_w(uint32_t (&dst)[W], const uint32_t* src, bool pred)
{
    if constexpr (W == 1 || W == 3) {
#pragma unroll
        for (int k = 0; k < W; k++)
            dst[k] = pred ? __ldcg(src + k) : 0u;
    } else if constexpr (W == 2) {
        const uint2 v = pred ? __ldcg(reinterpret_cast<const uint2*>(src)) : make_uint2(0, 0);
        dst[0] = v.x;
        dst[1] = v.y;
    } else {
#pragma unroll
        for (int k = 0; k < W / 4; k++) {
            const uint4 v = pred ? __ldcg(reinterpret_cast<const uint4*>(src) + k) : make_uint4(0, 0, 0, 0);
            dst[4 * k] = v.x;
            dst[4 * k + 1] = v.y;
            dst[4 * k + 2] = v.z;
            dst[4 * k + 3] = v.w;
        }
    }
}

template <int W>
__device__ __forceinline__ void store_row_w(uint32_t* dst, const uint32_t (&v)[W])
{
    if constexpr (W == 1 || W == 3) {
#pragma unroll
        for (int k = 0; k < W; k++)
            __stcg(dst + k, v[k]);
    } else if constexpr (W == 2) {
        __stcg(reinterpret_cast<uint2*>(dst), make_uint2(v[0], v[1]));
    } else {
#pragma unroll
        for (int k = 0; k < W / 4; k++)
            __stcg(reinterpret_cast<uint4*>(dst) + k, make_uint4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
    }
}

// Message rows of the next step are staged in shared memory by per-thread
// asynchronous copies (cp.async, 16 bytes each, bypassing L1): a thread
// copies and later reads only its own row, so it waits for its own copies
// and no barrier is involved.  One commit group per step, empty when the
// thread has nothing to copy.
template <int RW>
__device__ __forceinline__ void stage_row_async(uint4* dst, const uint4* src, bool pred)
{
    if (pred) {
        const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
#pragma unroll
        for (int w = 0; w < RW; w++)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16 * w), "l"(src + w) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// all of this thread's copies but the most recent group have landed
__device__ __forceinline__ void wait_staged_but_last() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void wait_staged_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Integer adds of the check loop issue as multiply-adds: the kernel is bound
// by the integer ALU pipe while the multiply-add pipe idles, and x * k + y
// with k read from constant memory (value 1 or -1, unknown to the compiler)
// becomes one IMAD on that pipe.  Same results as x + y.
static __constant__ int c_pipe_one = 1;

__device__ __forceinline__ int madd(int x, int k, int y) { return x * k + y; }

// 2 ((j + r) mod 360) from j2 = 2 j and r2 = 2 r, j, r in [0, 360)
__device__ __forceinline__ int rot720(int j2, uint32_t r2, int one)
{
    const unsigned u = (unsigned)madd((int)r2, one, j2);
    return (int)__viaddmin_u32(u, (unsigned)(-2 * kM), u);
}

__device__ __forceinline__ int lds16(const unsigned char* smem, int off)
{
    return *reinterpret_cast<const int16_t*>(smem + off);
}

__device__ __forceinline__ void sts16(unsigned char* smem, int off, int v)
{
    *reinterpret_cast<int16_t*>(smem + off) = (int16_t)v;
}

// Syndrome of the current hard decisions: true iff every check is
// satisfied.  The first vote (one barrier) follows the first step's checks,
// the next ones groups of 4 steps, so a failing frame -- nearly every
// iteration of every frame -- pays for about one step of gathers.
template <int CMAX>
__device__ bool syndrome_ok(const unsigned char* smem, const SmemCode& t, int K, int q, int n_steps, int lane,
                            int j, bool active)
{
    const int pty = 2 * K;
    for (int s0 = 0, g = 1; s0 < n_steps; s0 += g, g = 4) {
        int bad = 0;
        if (active) {
            const int s1 = min(s0 + g, n_steps);
            for (int s = s0; s < s1; s++) {
                const int i = t.sched[2 * s + lane];
                if (i < 0)
                    continue;
                int x = lds16(smem, pty + 2 * (i * kM + j));
                if (i > 0)
                    x ^= lds16(smem, pty + 2 * ((i - 1) * kM + j));
                else if (j > 0)
                    x ^= lds16(smem, pty + 2 * ((q - 1) * kM + j - 1));
                const uint4* tb = t.tab + i * CMAX;
#pragma unroll
                for (int e = 0; e < CMAX; e++) {
                    const uint4 w = tb[e];
                    x ^= lds16(smem, (int)w.x + rot720(2 * j, w.y, 1));
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
    // full warps only (the block may end in a partial warp)
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (warp >= nw)
        return;
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

// One check row of one layer: gather, offset min-sum, scatter, new message
// row; straight-line code for every layer (plain, staged and absent slots
// differ only in their descriptors).
template <int CMAX, int W, bool SAT>
__device__ __forceinline__ void process_check(const int16_t* wts, unsigned char* smem, const uint4* tb, int cnt,
                                              int j, int ps0, int ps1, bool absent, const uint32_t (&cur)[W],
                                              uint32_t* dst, int trial)
{
    constexpr int NE = CMAX + 2;
    // Wide rows would not fit the register budget with every slot's store
    // address held from the gather to the scatter: they recompute it there.
    constexpr bool kKeepAddr = CMAX <= 14;
    const int one = c_pipe_one, neg = -one;
    const int j2 = j + j;
    int d[NE];
    int sa[kKeepAddr ? CMAX : 1];  // where each slot's update is stored (its APP slot, or stage/junk)
    // gather: two parity edges (the second absent for check 0 of layer 0,
    // which then reads and writes a scratch slot), then the circulants
    const int a0 = lds16(smem, ps0);
    const int a1 = lds16(smem, ps1);
    {
        const int x0 = madd(row_byte_w(cur, 0), neg, a0);
        const int x1 = madd(row_byte_w(cur, 1), neg, a1);
        d[0] = SAT ? sat16(x0) : x0;
        d[1] = absent ? kBig : (SAT ? sat16(x1) : x1);
    }
#pragma unroll
    for (int e = 0; e < CMAX; e++) {
        const uint4 w = tb[e];
        const int ad = madd(rot720(j2, w.y, one), one, (int)w.x);
        if (kKeepAddr)
            sa[e] = madd((int)w.z, one, ad);
        const int x = madd(row_byte_w(cur, e + 2), neg, lds16(smem, ad));
        d[2 + e] = SAT ? sat16(x) : x;
    }
    // check node: min1/min2 of |extrinsic|, sign product
    int r1 = kBig, r2 = kBig, sx = 0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
        const int r = abs(d[e]);
        r2 = min(r2, max(r1, r));
        r1 = min(r1, r);
        sx ^= d[e];
    }
    int m1, m2;
    if (wts) {
        const int deg = cnt + (absent ? 1 : 2);
        const int16_t* w = wts + ((size_t)trial * 32 + deg) * 2;
        m1 = scaled_mag(r1, w[0], w[1]);
        m2 = scaled_mag(r2, w[0], w[1]);
    } else {
        m1 = min(max(r1 - 1, 0), 127);
        m2 = min(max(r2 - 1, 0), 127);
    }
    // each message carries the sign product of the other edges.  Per edge,
    // in multiply-add form (FMA pipe; the ALU pipe is the busier one):
    // s = sign of the extrinsic (+1 / -1), t = 0 iff |d| is the minimum,
    // message = s * (t ? p1 : p2)
    const int sg = sx >> 31;
    const int p1 = madd(sg, neg, m1 ^ sg), p2 = madd(sg, neg, m2 ^ sg);
    const int dp = p1 - p2, nr1 = -r1, two = one + one;
    uint32_t wv[W];
#pragma unroll
    for (int k = 0; k < W; k++)
        wv[k] = 0;
#pragma unroll
    for (int e = 0; e < NE; e++) {
        const int s = madd(d[e] >> 31, two, one);
        const int t = min(madd(d[e], s, nr1), one);
        const int mg = madd(madd(t, dp, p2), s, 0);
        wv[e >> 2] = __byte_perm(wv[e >> 2], (uint32_t)mg,
                                 (e & 3) == 0 ? 0x3214 : (e & 3) == 1 ? 0x3240 : (e & 3) == 2 ? 0x3410 : 0x4210);
        if (e < 2) {
            // parity: APP = sat16(extrinsic + message)
            sts16(smem, e == 0 ? ps0 : ps1, SAT ? sat16(d[e] + mg) : madd(mg, one, d[e]));
        } else {
            int at;
            if (kKeepAddr) {
                at = sa[e - 2];
            } else {
                const uint4 w = tb[e - 2];
                at = madd((int)w.z, one, madd(rot720(j2, w.y, one), one, (int)w.x));
            }
            int v;
            if (SAT) {
                // re-read the APP (unchanged: no other check of the step
                // writes this bit); a staged slot stores its delta, the
                // completion saturates the sum once
                const int delta = mg - row_byte_w(cur, e);
                v = tb[e - 2].z == 0 ? sat16(lds16(smem, at) + delta) : delta;
            } else {
                v = madd(mg, one, d[e]);
            }
            sts16(smem, at, v);
        }
    }
    store_row_w<W>(dst, wv);
}

// ---------------------------------------------------------------------------
// Packed 16-bit check rows (the saturation-free path).
//
// Two edges of a check row share one 32-bit register as a pair of int16
// lanes (edge 2k in the low half, 2k + 1 in the high half): the extrinsic
// values, the running min1/min2 and the message magnitudes and signs are
// computed two edges per instruction with the packed 16-bit adds (FMA pipe)
// and min/max/DPX ops (ALU pipe) of sm_90+, the work split about evenly
// between the two pipes.  Exact: in this path every value is within int16
// (|extrinsic| <= fast_lim + 127 (dv - 1), DevCode::fast_lim), so a packed
// add never wraps where the result is used.
//
// Magnitudes are tracked bitwise complemented, nr = ~|x| = -|x| - 1 =
// min(x - 1, ~x) (one DPX op given ~x), so min |x| is max nr.  With
// r1 <= r2 the two smallest magnitudes clamped to 128 (a message is at most
// 127: offset min-sum m = min(max(r - 1, 0), 127)), the message magnitude of
// edge e is max(r1c + r2c + nr_e, r1c - 1, 0) -- r2c - 1 when |x_e| = r1
// (the minimum edge; r1c - 1 as well when r1 = r2) and r1c - 1 when
// |x_e| >= r2 -- one DPX op per pair.  With learned weights the two
// magnitudes m1 <= m2 are computed per check and edge e takes m2 iff
// |x_e| < r2.  The message sign is the sign of x_e times the product of all
// signs (0 counts as +), as in the reference's finalp_oms_i16 (:242-275).
// Message rows hold the negated messages -m, so that the extrinsic of the
// next iteration is one packed add: x = APP + (-m).
static __constant__ int c_pipe_k16 = 65536;  // IMAD operands the compiler cannot fold
static __constant__ int c_pipe_k128 = 128;

__device__ __forceinline__ uint32_t vadd2(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("add.s16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

__device__ __forceinline__ uint32_t vmin2(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("min.s16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

__device__ __forceinline__ uint32_t vmax2(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("max.s16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

// prmt with sign replication (bit 3 of a selector nibble)
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}

template <uint32_t F>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t r;
    asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(r) : "r"(a), "r"(b), "r"(c), "n"(F));
    return r;
}

// Selector taking bytes s and s + 1 of a row word sign-extended into the two
// int16 halves (s even); pad: the high half is 0.
__host__ __device__ constexpr uint32_t pair_sel(int s, bool pad)
{
    return pad ? (uint32_t)(s | ((8 | s) << 4) | (4 << 8) | (4 << 12))
               : (uint32_t)(s | ((8 | s) << 4) | ((s + 1) << 8) | ((8 | (s + 1)) << 12));
}

__device__ __forceinline__ int ldu16(const unsigned char* smem, int off)
{
    return *reinterpret_cast<const uint16_t*>(smem + off);
}

template <int CMAX, int W, bool WTS>
__device__ __forceinline__ void process_check_packed(const int16_t* wts, unsigned char* smem, const uint4* tb, int cnt,
                                                     int j, int ps0, int ps1r, int ps1w, bool absent,
                                                     const uint32_t (&cur)[W], uint32_t* dst, int trial)
{
    constexpr int NE = CMAX + 2;
    constexpr int NP = (NE + 1) / 2;
    constexpr bool kKeepAddr = CMAX <= 14;
    const int one = c_pipe_one, neg = -one, k16 = c_pipe_k16;
    const int j2 = j + j;
    uint32_t x[NP];
    int sa[kKeepAddr ? CMAX : 1];
    // gather: x = APP + (-m_old) two edges at a time
    {
        const int a0 = ldu16(smem, ps0), a1 = ldu16(smem, ps1r);
        x[0] = vadd2((uint32_t)madd(a1, k16, a0), prmt(cur[0], 0, pair_sel(0, false)));
    }
    int lo = 0;
#pragma unroll
    for (int c = 0; c < CMAX; c++) {
        const int e = c + 2;
        const uint4 w = tb[c];
        const int ad = madd(rot720(j2, w.y, one), one, (int)w.x);
        if (kKeepAddr)
            sa[c] = madd((int)w.z, one, ad);
        const int a = ldu16(smem, ad);
        const uint32_t rw = cur[e >> 2];
        if ((e & 1) == 0) {
            lo = a;
            if (e == NE - 1)  // odd edge count: the high half is a pad that never wins a minimum
                x[e >> 1] = vadd2((uint32_t)madd(32767, k16, lo), prmt(rw, 0, pair_sel(e & 3, true)));
        } else {
            x[e >> 1] = vadd2((uint32_t)madd(a, k16, lo), prmt(rw, 0, pair_sel((e - 1) & 3, false)));
        }
    }
    // check node: max of ~|x| (= ~min |x|) and the runner-up, sign parity
    uint32_t nr[NP];
    uint32_t N1 = 0x80008000u, N2 = 0x80008000u, SX = 0;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        nr[k] = __viaddmin_s16x2(x[k], 0xffffffffu, (uint32_t)madd((int)x[k], neg, neg));  // min(x - 1, ~x) = ~|x|
        const uint32_t t = vmin2(N1, nr[k]);
        N2 = vmax2(N2, t);
        N1 = vmax2(N1, nr[k]);
        SX ^= x[k];
    }
    // both halves' results merged, replicated into both halves
    const uint32_t N1s = prmt(N1, N1, 0x1032), N2s = prmt(N2, N2, 0x1032);
    const uint32_t M1 = vmax2(N1, N1s);                              // ~r1
    const uint32_t M2 = vmax2(vmin2(N1, N1s), vmax2(N2, N2s));        // ~r2
    // message >= 0 iff sign(x_e) equals the parity of all signs T: Z has the
    // sign bits set iff T = 0, so the sign bits of x ^ Z flag a message >= 0
    const uint32_t w = SX ^ (uint32_t)madd((int)SX, k16, 0);
    const uint32_t Z = lop3<0x0c>(prmt(w, 0, 0xbbbb), 0x80008000u, 0);   // ~a & b
    uint32_t A, B, C;  // per-check constants of the magnitude rule
    if (WTS) {
        const int r1 = (int)(~M1 & 0xffffu), r2 = (int)(~M2 & 0xffffu);
        const int deg = cnt + (absent ? 1 : 2);
        const int16_t* wt = wts + ((size_t)trial * 32 + deg) * 2;
        const int m1 = scaled_mag(r1, wt[0], wt[1]), m2 = scaled_mag(r2, wt[0], wt[1]);
        A = (uint32_t)madd(m1, 0x10001, 0);
        B = (uint32_t)madd(m2, 0x10001, 0);
        C = vadd2((uint32_t)madd((int)M2, neg, neg), 0x00010001u);  // r2 + 1
    } else {
        const uint32_t R1c = vmin2((uint32_t)madd((int)M1, neg, neg), 0x00800080u);  // min(r1, 128)
        const uint32_t R2c = vmin2((uint32_t)madd((int)M2, neg, neg), 0x00800080u);
        A = vadd2(R1c, R2c);
        B = __viaddmax_s16x2_relu(R1c, 0xffffffffu, 0u);  // max(r1c - 1, 0)
        C = 0;
    }
    uint32_t nm[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) {
        uint32_t mag;
        if (WTS) {
            const uint32_t lt = __viaddmin_s16x2_relu(C, nr[k], 0x00010001u);  // |x| < r2
            mag = __viaddmin_s16x2(A, (uint32_t)madd((int)lt, c_pipe_k128, 0), B);
        } else {
            mag = __viaddmax_s16x2_relu(A, nr[k], B);
        }
        const uint32_t ns = prmt(x[k] ^ Z, 0, 0xbb99);  // 0xffff where the message is >= 0
        const uint32_t P = vadd2(x[k], mag), Q = vadd2((uint32_t)madd((int)x[k], neg, neg), mag);
        const uint32_t app = lop3<0xb1>(P, Q, ns);   // ns ? x + mag : ~(~x + mag) = x - mag
        nm[k] = vadd2(mag, ns) ^ ns;                 // -message
        const int lo_at = k == 0 ? ps0 : (kKeepAddr ? sa[2 * k - 2]
                                                     : madd((int)tb[2 * k - 2].z, one,
                                                            madd(rot720(j2, tb[2 * k - 2].y, one), one, (int)tb[2 * k - 2].x)));
        sts16(smem, lo_at, (int)app);
        if (2 * k + 1 < NE) {
            const int hi_at = k == 0 ? ps1w : (kKeepAddr ? sa[2 * k - 1]
                                                          : madd((int)tb[2 * k - 1].z, one,
                                                                 madd(rot720(j2, tb[2 * k - 1].y, one), one, (int)tb[2 * k - 1].x)));
            sts16(smem, hi_at, (int)__umulhi(app, (unsigned)k16));
        }
    }
    // new message row: byte e = -message of edge e
    uint32_t wv[W];
#pragma unroll
    for (int q = 0; q < W; q++)
        wv[q] = 2 * q < NP ? prmt(nm[2 * q], 2 * q + 1 < NP ? nm[2 * q + 1] : 0u, 0x6420) : 0u;
    store_row_w<W>(dst, wv);
}

// Completion of step s's shared groups: thread j of each lane takes bit j of
// the lane's items.  Plain path: APP + sum(row - APP); saturating path: the
// rows hold deltas, sat16(APP + sum).
template <int LANES, bool SAT>
__device__ __forceinline__ void complete_groups(unsigned char* smem, const int16_t* stage, const SmemCode& t,
                                                int s, int lane, int j)
{
    const int o0 = t.item_off[s], o1 = t.item_off[s + 1];
    const int16_t* st = stage + (s & 1) * kMaxStage * kM;
    for (int k = o0 + lane; k < o1; k += LANES) {
        const uint2 it = t.items[k];
        const int r0 = (int)(it.y & 0xff), nr = (int)(it.y >> 8);
        const int app = lds16(smem, (int)it.x + 2 * j);
        const int16_t* rows = st + r0 * kM + j;
        int sum;
        if (!SAT && nr == 2) {
            // the common group of two writers: row0 + row1 - APP
            sum = (int)rows[0] + (int)rows[kM] - app;
        } else {
            sum = app;
            for (int g = 0; g < nr; g++)
                sum += SAT ? (int)rows[g * kM] : (int)rows[g * kM] - app;
        }
        sts16(smem, (int)it.x + 2 * j, SAT ? sat16(sum) : sum);
    }
}

// MODE 0: saturating arithmetic, one edge per instruction (frames with a
// channel LLR beyond fast_lim); 1: packed pairs, plain offset min-sum;
// 2: packed pairs with learned weights.
template <int CMAX, int LANES, int MODE>
__device__ void decode_frame(const DecodeArgs& a, const DevCode& c, unsigned char* smem, const int16_t* stage,
                             const SmemCode& t, const Job& job)
{
    constexpr bool SAT = MODE == 0;
    constexpr int W = row_words(CMAX, LANES);
    const int tid = threadIdx.x;
    constexpr int LT = lane_threads(LANES);
    const int lane = (LANES == 2 && tid >= LT) ? 1 : 0;
    const int j = tid - lane * LT;
    const bool active = j < kM;
    const int K = c.K, q = c.q, T = a.max_trials, n_steps = c.n_steps;
    const int period = a.syn_period > 1 ? a.syn_period : 1;
    const int pty = 2 * K;         // byte offset of the parity APP
    const int spare = 2 * c.N;     // scratch slot for the absent parity edge
    uint32_t* msg_cta = reinterpret_cast<uint32_t*>(a.msg + (size_t)blockIdx.x * (size_t)a.msg_stride);
    constexpr bool kSmemRows = stage_rows_in_smem(CMAX, LANES);
    static_assert(!kSmemRows || W == 4, "rows staged in shared memory are 16 bytes");
    // staged rows (kSmemRows): set s & 1 holds this thread's row of step s
    uint4* mrow = reinterpret_cast<uint4*>(smem + a.sm_msgbuf) + tid;
    const int mset = (int)blockDim.x;
    int result = -1;

    for (int trial = 0;; trial++) {
        // step 0's rows are requested before the syndrome pass so that their
        // latency hides behind it (left unread when the frame converged)
        const bool load = trial > 0 && trial < T;
        uint32_t cur[W];
        {
            const int i0 = t.sched[lane];
            const uint32_t* src = msg_cta + ((size_t)max(i0, 0) * kM + j) * W;
            if (kSmemRows)
                stage_row_async<1>(mrow, reinterpret_cast<const uint4*>(src), load && active && i0 >= 0);
            else
                load_row_w<W>(cur, src, load && active && i0 >= 0);
        }
        // periodic + final check (reference ldpc_decode_kernel.cu:693-694)
        if ((period == 1 || trial % period == 0 || trial == T) &&
            syndrome_ok<CMAX>(smem, t, K, q, n_steps, lane, j, active)) {
            result = T - trial;
            break;
        }
        if (trial == T)
            break;
        for (int s = 0; s < n_steps; s++) {
            const int i = t.sched[2 * s + lane];
            uint32_t nxt[W];
            {
                const int i_n = s + 1 < n_steps ? t.sched[2 * (s + 1) + lane] : -1;
                const uint32_t* src = msg_cta + ((size_t)max(i_n, 0) * kM + j) * W;
                if (kSmemRows)
                    stage_row_async<1>(mrow + ((s + 1) & 1) * mset, reinterpret_cast<const uint4*>(src),
                                       load && active && i_n >= 0);
                else
                    load_row_w<W>(nxt, src, load && active && i_n >= 0);
            }
            if (kSmemRows) {
                wait_staged_but_last();
                const uint4 m = (load && active && i >= 0) ? mrow[(s & 1) * mset] : make_uint4(0, 0, 0, 0);
                const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
                for (int w = 0; w < W; w++)
                    cur[w] = mw[w & 3];
            }
            if (active) {
                // groups of the previous step whose completion was deferred
                if (s > 0 && t.conf[s - 1] == kConfDefer)
                    complete_groups<LANES, SAT>(smem, stage, t, s - 1, lane, j);
                if (i >= 0) {
                    const int ps0 = pty + 2 * (i * kM + j);
                    const bool absent = (i == 0 && j == 0);
                    uint32_t* dst = msg_cta + ((size_t)i * kM + j) * W;
                    if constexpr (SAT) {
                        const int ps1 = i > 0 ? ps0 - 2 * kM : (absent ? spare : pty + 2 * ((q - 1) * kM + j - 1));
                        process_check<CMAX, W, true>(c.weights, smem, t.tab + i * CMAX, t.cnt[i], j, ps0, ps1, absent,
                                                      cur, dst, trial);
                    } else {
                        // the absent edge reads the +32640 region and writes the junk region
                        const int ps1r = i > 0 ? ps0 - 2 * kM : (absent ? a.sm_dummy : pty + 2 * ((q - 1) * kM + j - 1));
                        const int ps1w = absent ? a.sm_dummy + 2 * kM : ps1r;
                        process_check_packed<CMAX, W, MODE == 2>(c.weights, smem, t.tab + i * CMAX, t.cnt[i], j, ps0,
                                                                  ps1r, ps1w, absent, cur, dst, trial);
                    }
                }
            }
            if (t.conf[s] == kConfMid) {
                __syncthreads();
                if (active)
                    complete_groups<LANES, SAT>(smem, stage, t, s, lane, j);
            }
            __syncthreads();
            if (!kSmemRows) {
#pragma unroll
                for (int w = 0; w < W; w++)
                    cur[w] = nxt[w];
            }
        }
    }
    if (kSmemRows)
        wait_staged_all();
    pack_hard(reinterpret_cast<const int16_t*>(smem), K, job.hard);
    if (threadIdx.x == 0)
        *job.trials = result;
}

// Channel LLRs of frame f into shared memory; returns nonzero if one is
// outside the saturation-free range.  Reference init :655-670 (clamp to
// +-32767, parity transpose).
__device__ __forceinline__ int load_llr(const DevCode& c, int16_t* app, const int16_t* src)
{
    const int K = c.K, R = c.R, q = c.q, lim = c.fast_lim;
    int over = 0;
    const bool vec = ((reinterpret_cast<uintptr_t>(src) & 15) == 0);
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
        // Parity bits p and p + 8 land 8 layers apart, in one shared-memory
        // bank: the threads of a warp store their 8 values in rotated order
        // (thread t starts at value t mod 8), so one store instruction of
        // the warp spreads over the banks instead of hitting one 32 times.
        const int rot = threadIdx.x & 7;
        for (int p = threadIdx.x * 8; p < R; p += blockDim.x * 8) {
            const uint4 w = __ldcs(reinterpret_cast<const uint4*>(src + K + p));
            const int li0 = p % q, lj0 = p / q;
#pragma unroll
            for (int s = 0; s < 8; s++) {
                const int k = (s + rot) & 7;
                const uint32_t wd = k < 2 ? w.x : k < 4 ? w.y : k < 6 ? w.z : w.w;
                int x = (int)(int16_t)(wd >> (16 * (k & 1)));
                x = max(x, -32767);
                over |= abs(x) > lim;
                int li = li0 + k, lj = lj0;  // q >= 5: at most two wraps
                if (li >= q) {
                    li -= q;
                    lj++;
                }
                if (li >= q) {
                    li -= q;
                    lj++;
                }
                app[K + li * kM + lj] = (int16_t)x;
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

// Copies one code's tables into shared memory; the slot descriptors are
// rebased onto this kernel's stage and dummy regions.
template <int CMAX>
__device__ void load_code(const DecodeArgs& a, unsigned char* smem, const DevCode& gc)
{
    DevCode* s_code = reinterpret_cast<DevCode*>(smem + a.sm_code);
    uint4* s_tab = reinterpret_cast<uint4*>(smem + a.sm_tab);
    uint8_t* s_cnt = smem + a.sm_cnt;
    int16_t* s_sched = reinterpret_cast<int16_t*>(smem + a.sm_sched);
    uint8_t* s_conf = smem + a.sm_conf;
    uint16_t* s_item_off = reinterpret_cast<uint16_t*>(smem + a.sm_item_off);
    uint2* s_items = reinterpret_cast<uint2*>(smem + a.sm_items);
    if (threadIdx.x == 0)
        *s_code = gc;
    for (int k = threadIdx.x; k < gc.q * CMAX; k += blockDim.x) {
        uint4 w = gc.tab[k];
        if (w.w == kSlotStaged)
            w.z += (uint32_t)a.sm_stage;
        else if (w.w == kSlotAbsent)
            w.x = (uint32_t)a.sm_dummy;
        s_tab[k] = make_uint4(w.x, 2 * w.y, w.z, 0);
    }
    for (int k = threadIdx.x; k < gc.q; k += blockDim.x) {
        int n = 0;
        for (int e = 0; e < CMAX; e++)
            n += gc.tab[k * CMAX + e].w != kSlotAbsent;
        s_cnt[k] = (uint8_t)n;
    }
    for (int k = threadIdx.x; k < 2 * gc.n_steps; k += blockDim.x)
        s_sched[k] = gc.sched[k];
    for (int k = threadIdx.x; k < gc.n_steps; k += blockDim.x)
        s_conf[k] = gc.step_conf[k];
    for (int k = threadIdx.x; k <= gc.n_steps; k += blockDim.x)
        s_item_off[k] = gc.item_off[k];
    for (int k = threadIdx.x; k < gc.n_items; k += blockDim.x)
        s_items[k] = gc.items[k];
}

// Resident CTAs per SM the register budget is cut for: a two-lane CTA holds
// a normal frame (one per SM); one-lane CTAs of narrow rows (short frames)
// fit three per SM in 55 registers without spilling, wider rows two.
constexpr int min_ctas_per_sm(int cmax, int lanes) { return lanes == 2 ? 1 : (cmax <= 5 ? 3 : 2); }

template <int CMAX, int LANES>
__global__ void __launch_bounds__(LANES * lane_threads(LANES), min_ctas_per_sm(CMAX, LANES)) ldpc_layered_kernel(DecodeArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    int16_t* app = reinterpret_cast<int16_t*>(smem);
    int16_t* dummy = reinterpret_cast<int16_t*>(smem + a.sm_dummy);
    const int16_t* stage = reinterpret_cast<const int16_t*>(smem + a.sm_stage);
    const DevCode& c = *reinterpret_cast<const DevCode*>(smem + a.sm_code);
    int* s_misc = reinterpret_cast<int*>(smem + a.sm_misc);
    const SmemCode t = {reinterpret_cast<const uint4*>(smem + a.sm_tab), smem + a.sm_cnt,
                        reinterpret_cast<const int16_t*>(smem + a.sm_sched), smem + a.sm_conf,
                        reinterpret_cast<const uint16_t*>(smem + a.sm_item_off),
                        reinterpret_cast<const uint2*>(smem + a.sm_items)};

    for (int k = threadIdx.x; k < kM; k += blockDim.x)
        // absent edges read +32640: with a message of at most 127 subtracted
        // their extrinsic stays in [32513, 32767] -- positive, above every
        // real magnitude of the saturation-free path (<= fast_lim + 127 (dv - 1)
        // = 32386) and above 127, so it never changes a message
        dummy[k] = 32640;
    int loaded = -1;
    // the list is complete when this launch starts (stream order); every CTA
    // reads its length before its exit count, so before the reset below
    const int n_frames = a.list ? min((int)*a.list_count, a.n_frames) : a.n_frames;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0)
            s_misc[0] = (int)atomicAdd(a.queue, 1u);
        __syncthreads();
        const int ticket = s_misc[0];
        if (ticket >= n_frames)
            break;
        const int f = a.list ? a.list[ticket] : ticket;
        Job job;
        int code_id = 0;
        if (a.frames) {
            const FrameDesc fd = a.frames[f];
            code_id = fd.code;
            job = {fd.llr, fd.hard, fd.trials};
        }
        if (code_id != loaded) {
            load_code<CMAX>(a, smem, a.codes ? a.codes[code_id] : a.code);
            loaded = code_id;
            __syncthreads();
        }
        if (!a.frames) {
            job.llr = a.llr + (size_t)f * c.N;
            job.hard = a.hard + (size_t)f * (c.K / 8);
            job.trials = a.trials + f;
        }
        const int over = load_llr(c, app, job.llr);
        if (__syncthreads_or(over))
            decode_frame<CMAX, LANES, 0>(a, c, smem, stage, t, job);
        else if (c.weights)
            decode_frame<CMAX, LANES, 2>(a, c, smem, stage, t, job);
        else
            decode_frame<CMAX, LANES, 1>(a, c, smem, stage, t, job);
    }
    // The last CTA out rearms the counters for the next launch (no memset
    // before each launch or graph replay): every CTA has drawn its final
    // ticket before its fenced exit count, so none reads the counter after
    // the reset.
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(a.queue + 1, 1u) == gridDim.x - 1) {
            atomicExch(a.queue, 0u);
            atomicExch(a.queue + 1, 0u);
            if (a.list)
                atomicExch(a.list_count, 0u);
        }
    }
}

}  // namespace cusat
