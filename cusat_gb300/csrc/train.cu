// Training kernels of the learned min-sum weights: the unrolled FP32 layered
// min-sum forward (T iterations, per-iteration x per-check-degree
// {beta, alpha}) and its hand-written backward, on the GPU.
//
// Model (no counterpart in the reference; the decoder structure is the
// reference's layered min-sum, ldpc_decode_kernel.cu:583-945, with the
// offset/scale of its normalised-min-sum hook nms_scale, :75-90, made
// learnable):
//   L = channel LLRs.  Per iteration t, per step of the paired-layer
//   schedule, per check c of the step's layers:
//     x_e = L[v_e] - m_old(c, e)
//     m(c, e) = sgn_e * min(alpha * max(r_e - beta, 0), 127)
//       r_e = smallest |x| of the other edges, sgn_e = sign product of the
//       other edges, (beta, alpha) = theta[t][deg(c)]
//   then every touched L[v] += m - m_old (additive within a step, like the
//   integer decoder's shared groups).
//   loss = sum_t w_t (1/N) sum_v softplus(-y_v L_v after iteration t), w_t
//   the per-iteration loss weights (1/T each by default).
//
// L and dL/dL are updated with atomics (L2) and read back with L1-bypassing
// loads after each barrier.
//
// Layout: one CTA per frame (lanes x 384 threads; thread j of lane l owns
// check j of the step's l-th layer).  The frame's L, dL/dL, the per-edge
// message adjoints and the per-(iteration, check) states live in global
// memory slices of this CTA.  The forward stores, per iteration and check,
// min1, min2, the two argmin edges and the sign bits (16 bytes); every
// message is recomputed from them, so the backward needs nothing else.  It
// replays the steps in reverse, rebuilding L before each step (L -= m -
// m_old) for the per-iteration loss terms.  Gradients of the weights are
// reduced per warp, then per CTA in shared memory, then added to the global
// gradient.
#include <algorithm>

#include "engine.h"
#include "fec_consts.h"

using namespace cusat_internal;
using cusat::kM;

namespace {

constexpr int kTrainLane = 384;
constexpr int kMaxIter = 64;

struct TrainCode {
    int N, K, R, q, n_steps, ew, lanes;
    const int16_t* sched;  // [n_steps * 2] layer per lane, -1 idle
    const uint8_t* cnt;    // [q] information circulants per layer
    const uint32_t* ent;   // [q * ew] group bit base | shift << 17
};

struct TrainArgs {
    TrainCode c;
    int T, B;
    const int16_t* llr;  // [B][N]
    const uint8_t* cw;   // [B][N/8] transmitted codewords, MSB first
    const float* theta;  // [T][32][2] {beta, alpha}
    const float* iter_w; // [T] loss weight per iteration, or nullptr (1/T)
    float* grad;         // [T][32][2] accumulated, or nullptr (forward only)
    float* loss;         // [1] accumulated
    float* L;            // [grid][N]
    float* gL;           // [grid][N]
    float* G;            // [grid][R * ew]
    uint4* st;           // [grid][T * R]
};

struct CState {
    float min1, min2;
    uint32_t signs;
    int i1, i2;
};

__device__ __forceinline__ uint4 pack_state(const CState& s)
{
    return make_uint4(__float_as_uint(s.min1), __float_as_uint(s.min2), s.signs,
                      (uint32_t)(s.i1 & 0xff) | ((uint32_t)(s.i2 & 0xff) << 8));
}

__device__ __forceinline__ CState unpack_state(uint4 u)
{
    CState s;
    s.min1 = __uint_as_float(u.x);
    s.min2 = __uint_as_float(u.y);
    s.signs = u.z;
    s.i1 = (int)(u.w & 0xff);
    s.i2 = (int)((u.w >> 8) & 0xff);
    return s;
}

// message of edge e from a check state (explicit roundings: no contraction)
__device__ __forceinline__ float msg_of(const CState& s, int e, float beta, float alpha)
{
    const float r = e == s.i1 ? s.min2 : s.min1;
    const float u = r > beta ? __fsub_rn(r, beta) : 0.0f;
    const float mag = fminf(__fmul_rn(alpha, u), 127.0f);
    return ((__popc(s.signs) ^ (int)(s.signs >> e)) & 1) ? -mag : mag;
}

__device__ __forceinline__ int var_of(const TrainCode& c, int i, int j, int e)
{
    if (e == 0)
        return c.K + c.q * j + i;
    if (e == 1)
        return c.K + c.q * j + i - 1;
    const uint32_t en = __ldg(c.ent + i * c.ew + e - 2);
    int d = j - (int)(en >> 17);
    d += d < 0 ? kM : 0;
    return (int)(en & 0x1ffff) + d;
}

__device__ __forceinline__ int code_bit(const uint8_t* cw, int v) { return (cw[v >> 3] >> (7 - (v & 7))) & 1; }

__device__ __forceinline__ float softplus_of(float z) { return z > 0.0f ? z + log1pf(expf(-z)) : log1pf(expf(z)); }

// d/dL softplus(-y L) = -y / (1 + exp(y L))
__device__ __forceinline__ float dsoftplus_of(float L, int bit)
{
    const float y = bit ? -1.0f : 1.0f;
    return -y / (1.0f + expf(y * L));
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(2 * kTrainLane, 1) nms_train_kernel(TrainArgs a)
{
    const TrainCode& c = a.c;
    __shared__ float s_g[64];     // gradient of one iteration's weights
    __shared__ float s_red[32];
    const int tid = threadIdx.x;
    const int lane = tid / kTrainLane;
    const int j = tid - lane * kTrainLane;
    const int N = c.N, R = c.R, EW = c.ew, T = a.T;
    const float inv_n = 1.0f / (float)N;
    auto wt = [&](int t) { return (a.iter_w ? a.iter_w[t] : 1.0f / (float)T) * inv_n; };
    float* L = a.L + (size_t)blockIdx.x * N;
    float* gL = a.gL + (size_t)blockIdx.x * N;
    float* G = a.G + (size_t)blockIdx.x * R * EW;
    uint4* st = a.st + (size_t)blockIdx.x * T * R;
    if (tid < 64)
        s_g[tid] = 0.0f;

    for (int f = blockIdx.x; f < a.B; f += gridDim.x) {
        const int16_t* llr = a.llr + (size_t)f * N;
        const uint8_t* cw = a.cw + (size_t)f * (N / 8);
        float loss = 0.0f;
        for (int v = tid; v < N; v += blockDim.x)
            L[v] = (float)llr[v];
        __syncthreads();

        // ---------------- forward ----------------
        for (int t = 0; t < T; t++) {
            const float* th = a.theta + (size_t)t * 64;
            const float* thp = a.theta + (size_t)(t > 0 ? t - 1 : 0) * 64;
            for (int s = 0; s < c.n_steps; s++) {
                const int i = c.sched[2 * s + lane];
                const bool active = j < kM && i >= 0;
                CState n{1e30f, 1e30f, 0u, -1, -1}, p{};
                int ne = 0, deg = 0;
                bool absent = false;
                float bp = 0.0f, ap = 0.0f;
                if (active) {
                    ne = c.cnt[i] + 2;
                    absent = i == 0 && j == 0;
                    deg = ne - (absent ? 1 : 0);
                    const int ch = i * kM + j;
                    if (t > 0) {
                        p = unpack_state(st[(size_t)(t - 1) * R + ch]);
                        bp = thp[2 * deg];
                        ap = thp[2 * deg + 1];
                    }
                    for (int e = 0; e < ne; e++) {
                        if (e == 1 && absent)
                            continue;
                        const int v = var_of(c, i, j, e);
                        const float mo = t > 0 ? msg_of(p, e, bp, ap) : 0.0f;
                        const float x = __fsub_rn(__ldcg(&L[v]), mo);
                        const float ax = fabsf(x);
                        if (x < 0.0f)
                            n.signs |= 1u << e;
                        if (ax < n.min1) {
                            n.min2 = n.min1;
                            n.i2 = n.i1;
                            n.min1 = ax;
                            n.i1 = e;
                        } else if (ax < n.min2) {
                            n.min2 = ax;
                            n.i2 = e;
                        }
                    }
                    st[(size_t)t * R + ch] = pack_state(n);
                }
                __syncthreads();
                if (active) {
                    const float b = th[2 * deg], al = th[2 * deg + 1];
                    for (int e = 0; e < ne; e++) {
                        if (e == 1 && absent)
                            continue;
                        const float mo = t > 0 ? msg_of(p, e, bp, ap) : 0.0f;
                        atomicAdd(&L[var_of(c, i, j, e)], __fsub_rn(msg_of(n, e, b, al), mo));
                    }
                }
                __syncthreads();
            }
            float lt = 0.0f;
            for (int v = tid; v < N; v += blockDim.x) {
                const float l = __ldcg(&L[v]);
                lt += softplus_of(code_bit(cw, v) ? l : -l);
            }
            loss += wt(t) * lt;
        }
        loss = warp_sum(loss);
        if ((tid & 31) == 0)
            s_red[tid >> 5] = loss;
        __syncthreads();
        if (tid == 0) {
            float sum = 0.0f;
            for (int k = 0; k < (int)(blockDim.x >> 5); k++)
                sum += s_red[k];
            atomicAdd(a.loss, sum);
        }
        if (!a.grad) {
            __syncthreads();
            continue;
        }

        // ---------------- backward ----------------
        for (int v = tid; v < N; v += blockDim.x)
            gL[v] = wt(T - 1) * dsoftplus_of(__ldcg(&L[v]), code_bit(cw, v));
        for (int k = tid; k < R * EW; k += blockDim.x)
            G[k] = 0.0f;
        __syncthreads();
        for (int t = T - 1; t >= 0; t--) {
            const float* th = a.theta + (size_t)t * 64;
            const float* thp = a.theta + (size_t)(t > 0 ? t - 1 : 0) * 64;
            for (int s = c.n_steps - 1; s >= 0; s--) {
                const int i = c.sched[2 * s + lane];
                const bool active = j < kM && i >= 0;
                CState n{}, p{};
                int ne = 0, deg = 0, ch = 0;
                bool absent = false;
                float gx1 = 0.0f, gx2 = 0.0f, ga = 0.0f, gb = 0.0f;
                float beta = 0.0f, alpha = 0.0f, bp = 0.0f, ap = 0.0f;
                if (active) {
                    ne = c.cnt[i] + 2;
                    absent = i == 0 && j == 0;
                    deg = ne - (absent ? 1 : 0);
                    ch = i * kM + j;
                    n = unpack_state(st[(size_t)t * R + ch]);
                    if (t > 0) {
                        p = unpack_state(st[(size_t)(t - 1) * R + ch]);
                        bp = thp[2 * deg];
                        ap = thp[2 * deg + 1];
                    }
                    beta = th[2 * deg];
                    alpha = th[2 * deg + 1];
                    const int S = __popc(n.signs) & 1;
                    for (int e = 0; e < ne; e++) {
                        if (e == 1 && absent)
                            continue;
                        const int v = var_of(c, i, j, e);
                        const float gm = __fadd_rn(G[(size_t)ch * EW + e], __ldcg(&gL[v]));
                        const float r = e == n.i1 ? n.min2 : n.min1;
                        const float u = __fsub_rn(r, beta);
                        if (u > 0.0f && __fmul_rn(alpha, u) < 127.0f) {
                            const float gs = ((S ^ (int)(n.signs >> e)) & 1) ? -gm : gm;
                            ga = __fadd_rn(ga, __fmul_rn(gs, u));
                            gb = __fsub_rn(gb, __fmul_rn(gs, alpha));
                            const float gr = __fmul_rn(gs, alpha);
                            if (e == n.i1)
                                gx2 = __fadd_rn(gx2, ((n.signs >> n.i2) & 1) ? -gr : gr);
                            else
                                gx1 = __fadd_rn(gx1, ((n.signs >> n.i1) & 1) ? -gr : gr);
                        }
                    }
                    for (int e = 0; e < ne; e++) {
                        if (e == 1 && absent)
                            continue;
                        const float gxe = e == n.i1 ? gx1 : (e == n.i2 ? gx2 : 0.0f);
                        G[(size_t)ch * EW + e] = __fsub_rn(-gxe, __ldcg(&gL[var_of(c, i, j, e)]));
                    }
                }
                // weight gradients: one sum per warp (a warp covers one layer;
                // the degree-reduced check 0 of layer 0 adds its own)
                {
                    const bool mine = active && !absent;
                    const float sa = warp_sum(mine ? ga : 0.0f);
                    const float sb = warp_sum(mine ? gb : 0.0f);
                    if ((tid & 31) == 0 && active) {
                        atomicAdd(&s_g[2 * (c.cnt[i] + 2)], sb);
                        atomicAdd(&s_g[2 * (c.cnt[i] + 2) + 1], sa);
                    }
                    if (active && absent) {
                        atomicAdd(&s_g[2 * deg], gb);
                        atomicAdd(&s_g[2 * deg + 1], ga);
                    }
                }
                __syncthreads();
                if (active) {
                    if (gx1 != 0.0f)
                        atomicAdd(&gL[var_of(c, i, j, n.i1)], gx1);
                    if (gx2 != 0.0f)
                        atomicAdd(&gL[var_of(c, i, j, n.i2)], gx2);
                    for (int e = 0; e < ne; e++) {
                        if (e == 1 && absent)
                            continue;
                        const float mo = t > 0 ? msg_of(p, e, bp, ap) : 0.0f;
                        atomicAdd(&L[var_of(c, i, j, e)], -__fsub_rn(msg_of(n, e, beta, alpha), mo));
                    }
                }
                __syncthreads();
            }
            if (t > 0)
                for (int v = tid; v < N; v += blockDim.x)
                    gL[v] = __ldcg(&gL[v]) + wt(t - 1) * dsoftplus_of(__ldcg(&L[v]), code_bit(cw, v));
            if (tid < 64) {
                const float g = s_g[tid];
                if (g != 0.0f)
                    atomicAdd(&a.grad[(size_t)t * 64 + tid], g);
                s_g[tid] = 0.0f;
            }
            __syncthreads();
        }
    }
}

}  // namespace

struct cusat_nms_trainer {
    const cusat::CodePlan* plan = nullptr;
    int T = 0, max_batch = 0, grid = 0, deg_lo = 0, deg_hi = 0;
    int deg_count[32] = {0};  // checks of each degree
    TrainArgs proto{};
    void* blob = nullptr;  // code tables
    float* bufs = nullptr; // L, gL, G
    uint4* st = nullptr;
};

namespace {

void release(cusat_nms_trainer* t)
{
    if (!t)
        return;
    if (t->blob)
        cudaFree(t->blob);
    if (t->bufs)
        cudaFree(t->bufs);
    if (t->st)
        cudaFree(t->st);
    delete t;
}

}  // namespace

extern "C" {

int cusat_nms_trainer_create(int framesize, int rate, int n_iter, int max_batch, cusat_nms_trainer** out)
{
    if (!out || n_iter <= 0 || n_iter > kMaxIter || max_batch <= 0)
        return fail(CUSAT_ERR_ARG, "invalid trainer arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    const int q = p->q, ew = p->cnt_max + 2;
    // information circulants of each layer in table order (row, then entry)
    std::vector<uint32_t> ent((size_t)q * ew, 0);
    std::vector<int> fill(q, 0);
    for (int r = 0, o = 0; r < p->n_rows; r++)
        for (int d = 0; d < p->row_deg[r]; d++, o++) {
            const int a = p->addr[o], i = a % q;
            ent[(size_t)i * ew + fill[i]++] = (uint32_t)(r * kM) | ((uint32_t)(a / q) << 17);
        }
    cusat_nms_trainer* t = new cusat_nms_trainer();
    t->plan = p;
    t->T = n_iter;
    t->max_batch = max_batch;
    t->deg_lo = 64;
    for (int i = 0; i < q; i++) {
        t->deg_lo = std::min(t->deg_lo, (int)p->cnt[i] + (i == 0 ? 1 : 2));
        t->deg_hi = std::max(t->deg_hi, (int)p->cnt[i] + 2);
        t->deg_count[p->cnt[i] + 2] += i == 0 ? kM - 1 : kM;
    }
    t->deg_count[p->cnt[0] + 1] += 1;  // check 0 of layer 0 has no wrap edge
    const size_t o_sched = 0, n_sched = p->sched.size() * 2;
    const size_t o_cnt = (o_sched + n_sched + 255) / 256 * 256, n_cnt = p->cnt.size();
    const size_t o_ent = (o_cnt + n_cnt + 255) / 256 * 256, n_ent = ent.size() * 4;
    std::vector<unsigned char> host(o_ent + n_ent);
    memcpy(host.data() + o_sched, p->sched.data(), n_sched);
    memcpy(host.data() + o_cnt, p->cnt.data(), n_cnt);
    memcpy(host.data() + o_ent, ent.data(), n_ent);
    int sms = 0, per_sm = 0;
    const int threads = p->lanes * kTrainLane;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nms_train_kernel, threads, 0);
    t->grid = std::max(1, std::min(max_batch, per_sm * sms));
    if (e == cudaSuccess)
        e = cudaMalloc(&t->blob, host.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(t->blob, host.data(), host.size(), cudaMemcpyHostToDevice);
    const size_t per_cta = (size_t)2 * p->N + (size_t)p->R * ew;
    if (e == cudaSuccess)
        e = cudaMalloc(&t->bufs, per_cta * t->grid * sizeof(float));
    if (e == cudaSuccess)
        e = cudaMalloc(&t->st, (size_t)t->grid * n_iter * p->R * sizeof(uint4));
    if (e != cudaSuccess) {
        release(t);
        return cuda_fail(e, "trainer set-up");
    }
    const unsigned char* b = (const unsigned char*)t->blob;
    TrainCode& c = t->proto.c;
    c.N = p->N;
    c.K = p->K;
    c.R = p->R;
    c.q = q;
    c.n_steps = p->n_steps;
    c.ew = ew;
    c.lanes = p->lanes;
    c.sched = (const int16_t*)(b + o_sched);
    c.cnt = (const uint8_t*)(b + o_cnt);
    c.ent = (const uint32_t*)(b + o_ent);
    t->proto.T = n_iter;
    t->proto.L = t->bufs;
    t->proto.gL = t->bufs + (size_t)t->grid * p->N;
    t->proto.G = t->bufs + (size_t)2 * t->grid * p->N;
    t->proto.st = t->st;
    *out = t;
    return CUSAT_OK;
}

void cusat_nms_trainer_destroy(cusat_nms_trainer* t) { release(t); }

int cusat_nms_trainer_info(const cusat_nms_trainer* t, int32_t* out)
{
    if (!t || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = t->plan->N;
    out[1] = t->plan->K;
    out[2] = t->T;
    out[3] = t->max_batch;
    out[4] = t->deg_lo;
    out[5] = t->deg_hi;
    return CUSAT_OK;
}

int cusat_nms_trainer_degree_counts(const cusat_nms_trainer* t, int32_t* counts)
{
    if (!t || !counts)
        return fail(CUSAT_ERR_ARG, "null argument");
    for (int d = 0; d < 32; d++)
        counts[d] = t->deg_count[d];
    return CUSAT_OK;
}

int cusat_nms_train_step(cusat_nms_trainer* t, const int16_t* llr_dev, const uint8_t* cw_dev, int batch,
                         const float* theta_dev, const float* iter_w_dev, float* grad_dev, float* loss_dev,
                         void* stream)
{
    if (!t || !llr_dev || !cw_dev || !theta_dev || !loss_dev || batch <= 0 || batch > t->max_batch)
        return fail(CUSAT_ERR_ARG, "invalid training step arguments");
    TrainArgs a = t->proto;
    a.B = batch;
    a.llr = llr_dev;
    a.cw = cw_dev;
    a.theta = theta_dev;
    a.iter_w = iter_w_dev;
    a.grad = grad_dev;
    a.loss = loss_dev;
    const int grid = std::min(batch, t->grid);
    nms_train_kernel<<<grid, t->plan->lanes * kTrainLane, 0, (cudaStream_t)stream>>>(a);
    CU(cudaGetLastError(), "training kernel launch");
    return CUSAT_OK;
}

}  // extern "C"
