// Traffic generation on the GPU: systematic BCH encode, IRA LDPC encode and
// constellation mapping of a batch of messages (what the transmitter does;
// used to make training and benchmark frames without a host round trip).
// Reference: ldpc_encode.cc:6-13 and cuda/ldpc_encode_kernel.cu (IRA
// accumulate), fec/bch_code.cc:99-144 and cuda/bch_common.cuh (systematic BCH
// through a byte LUT), cuda/mapper_kernel.cu:22-51 (label = the frame bits at
// the interleaver's column offsets, MSB first).  The results equal this
// library's host encoder and mapper bit for bit.
#include <algorithm>

#include "engine.h"
#include "fec_consts.h"

using namespace cusat_internal;
using cusat::kM;

namespace {

constexpr int kEncThreads = 512;

// BCH parity of each frame's message: the remainder m(x) x^p mod g(x), one
// warp per frame, byte-LUT LFSR per lane chunk and the five-level shuffle
// combine of the check kernel (tables built for the message length).
template <int W>
__global__ void __launch_bounds__(128) bch_encode_kernel(cusat::BchDev t, const uint8_t* __restrict__ msg,
                                                         uint8_t* __restrict__ cw, int cw_bytes, int batch)
{
    __shared__ uint64_t lut[256 * W];
    for (int k = threadIdx.x; k < 256 * W; k += blockDim.x)
        lut[k] = t.lut[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (f >= batch)
        return;
    const int p = t.p;
    const uint64_t top_mask = (p % 64) ? ((1ull << (p % 64)) - 1) : ~0ull;
    const uint8_t* src = msg + (size_t)f * t.n_bytes;
    uint8_t* out = cw + (size_t)f * cw_bytes;
    for (int v = lane; v < (int)t.n_bytes; v += 32)
        out[v] = src[v];
    uint64_t r[W];
#pragma unroll
    for (int w = 0; w < W; w++)
        r[w] = 0;
    const int v0 = lane * t.chunk, v1 = v0 + t.chunk;
    for (int v = max(v0, (int)t.lead); v < v1; v++) {
        const unsigned b = src[v - t.lead];
        const int lo = p - 8;
        const unsigned idx = b ^ (unsigned)((r[lo >> 6] >> (lo & 63)) & 255);
#pragma unroll
        for (int w = W - 1; w >= 0; w--)
            r[w] = (r[w] << 8) | (w ? r[w - 1] >> 56 : 0);
        r[W - 1] &= top_mask;
#pragma unroll
        for (int w = 0; w < W; w++)
            r[w] ^= lut[idx * W + w];
    }
    const int nb = p / 8;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        uint64_t o[W], a[W], acc[W];
#pragma unroll
        for (int w = 0; w < W; w++) {
            o[w] = __shfl_xor_sync(0xffffffffu, r[w], 1 << k);
            a[w] = (lane & (1 << k)) ? o[w] : r[w];
            acc[w] = (lane & (1 << k)) ? r[w] : o[w];
        }
        const uint64_t* tk = t.tree + (size_t)k * nb * 256 * W;
        for (int jb = 0; jb < nb; jb++) {
            const unsigned byte = (unsigned)((a[jb >> 3] >> ((jb & 7) * 8)) & 255);
            const uint64_t* e = tk + ((size_t)jb * 256 + byte) * W;
#pragma unroll
            for (int w = 0; w < W; w++)
                acc[w] ^= __ldg(e + w);
        }
#pragma unroll
        for (int w = 0; w < W; w++)
            r[w] = acc[w];
    }
    for (int jb = lane; jb < nb; jb += 32) {
        const int lo = p - 8 * (jb + 1);
        out[t.n_bytes + jb] = (uint8_t)(r[lo >> 6] >> (lo & 63));
    }
}

struct LdpcEnc {
    int K, R, q, n_rows;
    const uint16_t* addr;     // accumulator addresses of the table rows, concatenated
    const int32_t* row_off;   // [n_rows + 1]
};

// IRA encode of one frame per CTA, in place: the information bits (the BCH
// codeword) are read from cw, the parity bits written after them.  Each set
// information bit m of row r toggles accumulators (a + (m mod 360) q) mod R for
// the row's addresses a (atomic XOR into a shared-memory bitset, bit i of the
// accumulators at word i / 32, bit 31 - i % 32); parity bit i is then the XOR
// of accumulators 0..i: a prefix XOR inside each word (shifts), and across
// words the parity of all earlier words (block scan).
__global__ void __launch_bounds__(kEncThreads) ldpc_encode_kernel(LdpcEnc e, uint8_t* __restrict__ cw, int cw_bytes,
                                                                   int batch)
{
    extern __shared__ uint32_t acc[];  // [ceil(R / 32)]
    __shared__ uint32_t s_par[kEncThreads / 32];
    const int nw = (e.R + 31) / 32;
    for (int f = blockIdx.x; f < batch; f += gridDim.x) {
        uint8_t* out = cw + (size_t)f * cw_bytes;
        for (int w = threadIdx.x; w < nw; w += blockDim.x)
            acc[w] = 0;
        __syncthreads();
        for (int v = threadIdx.x; v < e.K; v += blockDim.x) {
            if (!((out[v >> 3] >> (7 - (v & 7))) & 1))
                continue;
            const int r = v / kM, m = v - r * kM;
            const int mq = m * e.q;
            for (int k = e.row_off[r]; k < e.row_off[r + 1]; k++) {
                int a = (int)e.addr[k] + mq;
                a -= a >= e.R ? e.R : 0;
                atomicXor(&acc[a >> 5], 1u << (31 - (a & 31)));
            }
        }
        __syncthreads();
        // prefix XOR: each thread takes a contiguous run of words
        const int per = (nw + blockDim.x - 1) / blockDim.x;
        const int w0 = min(nw, (int)threadIdx.x * per), w1 = min(nw, w0 + per);
        uint32_t run = 0;  // parity of this thread's words
        for (int w = w0; w < w1; w++)
            run ^= __popc(acc[w]) & 1;
        // exclusive XOR scan of the runs over the block
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl ^= y;
        }
        if (lane == 31)
            s_par[warp] = incl;
        __syncthreads();
        uint32_t before = incl ^ run;
        for (int k = 0; k < warp; k++)
            before ^= s_par[k];
        for (int w = w0; w < w1; w++) {
            uint32_t x = acc[w];
            x ^= x >> 1;
            x ^= x >> 2;
            x ^= x >> 4;
            x ^= x >> 8;
            x ^= x >> 16;
            const uint32_t y = before ? ~x : x;
            before ^= __popc(acc[w]) & 1;
            acc[w] = y;  // this thread alone reads and writes word w
        }
        __syncthreads();
        const int kb = e.K / 8;
        for (int y = threadIdx.x; y < e.R / 8; y += blockDim.x)
            out[kb + y] = (uint8_t)(acc[y >> 2] >> (24 - 8 * (y & 3)));
        __syncthreads();
    }
}

struct MapArgs {
    int n_mod, xfec, stride;  // QPSK: bits 2j, 2j+1; otherwise column offsets, stride 1
    int interleaved_len;      // symbols that carry frame bits (128APSK: xfec - 12)
    int fec_bits;             // positions at or past it are stuffing bits (0)
    uint32_t col[8];
    const float2* points;     // by label
};

// Mapper: one thread per symbol; label bit b (MSB first) is frame bit
// col[b] + j * stride, 0 past the FECFRAME; padding symbols (128APSK) carry
// the all-ones label (reference mapper.cc:42-62).
__global__ void map_kernel(const uint8_t* __restrict__ cw, int cw_bytes, MapArgs m, float2* __restrict__ sym,
                           int batch)
{
    const size_t n = (size_t)batch * m.xfec;
    for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (size_t)gridDim.x * blockDim.x) {
        const int f = (int)(g / m.xfec), j = (int)(g - (size_t)f * m.xfec);
        const uint8_t* in = cw + (size_t)f * cw_bytes;
        int label = (1 << m.n_mod) - 1;
        if (j < m.interleaved_len) {
            label = 0;
            for (int b = 0; b < m.n_mod; b++) {
                const int pos = (int)m.col[b] + j * m.stride;
                if (pos < m.fec_bits)
                    label |= ((in[pos >> 3] >> (7 - (pos & 7))) & 1) << (m.n_mod - 1 - b);
            }
        }
        sym[g] = __ldg(m.points + label);
    }
}

}  // namespace

struct cusat_generator {
    const cusat::CodePlan* plan = nullptr;
    DevBch bch;
    DevDemapObj dm;
    LdpcEnc enc{};
    void* blob = nullptr;
    int max_batch = 0, sms = 0;
};

extern "C" {

int cusat_generator_create(int modulation, int rate, int framesize, int max_batch, cusat_generator** out)
{
    if (!out || max_batch <= 0)
        return fail(CUSAT_ERR_ARG, "invalid generator arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    if (p->p % 8 || p->k_bch % 8)
        return fail(CUSAT_ERR_UNSUPPORTED, "BCH geometry not byte aligned");
    cusat_generator* g = new cusat_generator();
    g->plan = p;
    g->max_batch = max_batch;
    cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, dev);
    rc = g->bch.init(p->gen, p->p, (unsigned)(p->k_bch / 8));
    if (rc == CUSAT_OK)
        rc = g->dm.init(modulation, rate, framesize);
    if (rc == CUSAT_OK && g->dm.m.fec_len != p->N)
        rc = fail(CUSAT_ERR_UNSUPPORTED, "MODCOD and code do not match");
    if (rc == CUSAT_OK) {
        int n_addr = 0;
        for (int r = 0; r < p->n_rows; r++)
            n_addr += p->row_deg[r];
        std::vector<int32_t> off(p->n_rows + 1, 0);
        for (int r = 0; r < p->n_rows; r++)
            off[r + 1] = off[r] + p->row_deg[r];
        const size_t o_off = ((size_t)n_addr * 2 + 255) / 256 * 256;
        cudaError_t e = cudaMalloc(&g->blob, o_off + off.size() * 4);
        if (e == cudaSuccess)
            e = cudaMemcpy(g->blob, p->addr, (size_t)n_addr * 2, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy((char*)g->blob + o_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "generator tables");
        g->enc = LdpcEnc{p->K, p->R, p->q, p->n_rows, (const uint16_t*)g->blob,
                         (const int32_t*)((char*)g->blob + o_off)};
    }
    if (rc == CUSAT_OK && p->K != p->n_bch)
        rc = fail(CUSAT_ERR_UNSUPPORTED, "BCH codeword length differs from the LDPC information length");
    if (rc) {
        cusat_generator_destroy(g);
        return rc;
    }
    *out = g;
    return CUSAT_OK;
}

void cusat_generator_destroy(cusat_generator* g)
{
    if (!g)
        return;
    g->bch.release();
    g->dm.release();
    if (g->blob)
        cudaFree(g->blob);
    delete g;
}

int cusat_generator_info(const cusat_generator* g, int32_t* out)
{
    if (!g || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = g->plan->k_bch / 8;
    out[1] = g->plan->N / 8;
    out[2] = g->dm.m.xfec;
    out[3] = g->max_batch;
    return CUSAT_OK;
}

int cusat_generate(cusat_generator* g, const uint8_t* msg_dev, int batch, uint8_t* cw_dev, float* sym_dev,
                   void* stream)
{
    if (!g || !msg_dev || !cw_dev || batch <= 0 || batch > g->max_batch)
        return fail(CUSAT_ERR_ARG, "invalid generation arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const cusat::CodePlan& p = *g->plan;
    const int cw_bytes = p.N / 8;
    const int blocks = (batch + 3) / 4;
    const cusat::BchDev& t = g->bch.d;
    if (t.words == 1)
        bch_encode_kernel<1><<<blocks, 128, 0, s>>>(t, msg_dev, cw_dev, cw_bytes, batch);
    else if (t.words == 2)
        bch_encode_kernel<2><<<blocks, 128, 0, s>>>(t, msg_dev, cw_dev, cw_bytes, batch);
    else if (t.words == 3)
        bch_encode_kernel<3><<<blocks, 128, 0, s>>>(t, msg_dev, cw_dev, cw_bytes, batch);
    else
        bch_encode_kernel<4><<<blocks, 128, 0, s>>>(t, msg_dev, cw_dev, cw_bytes, batch);
    CU(cudaGetLastError(), "BCH encode launch");
    const int smem = ((p.R + 31) / 32) * 4;
    ldpc_encode_kernel<<<std::min(batch, 4 * std::max(g->sms, 1)), kEncThreads, smem, s>>>(g->enc, cw_dev, cw_bytes,
                                                                                         batch);
    CU(cudaGetLastError(), "LDPC encode launch");
    if (sym_dev) {
        const cusat::DevDemap& d = g->dm.d;
        MapArgs m{};
        m.n_mod = d.n_mod;
        m.xfec = d.xfec;
        m.interleaved_len = d.interleaved_len;
        m.fec_bits = d.fec_len;
        m.stride = d.kind == 0 ? 2 : 1;
        for (int b = 0; b < 8; b++)
            m.col[b] = d.kind == 0 ? (uint32_t)b : d.col[b];
        m.points = d.points;
        const size_t n = (size_t)batch * d.xfec;
        const int mb = (int)std::min<size_t>((n + 255) / 256, (size_t)std::max(g->sms, 1) * 16);
        map_kernel<<<mb, 256, 0, s>>>(cw_dev, cw_bytes, m, reinterpret_cast<float2*>(sym_dev), batch);
        CU(cudaGetLastError(), "map launch");
    }
    return CUSAT_OK;
}

}  // extern "C"
