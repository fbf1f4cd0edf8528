// Post-FEC baseband stage on the device: for a batch of decoded frames, drop
// those whose LDPC decode failed or whose BCH check failed, descramble the
// rest (EN 302 307-1 clause 5.2.2), check their BBHEADER and pack the data
// fields of generic-packetized (GSE) streams back to back.  Replaces the RX
// chain's host loop (reference rx_fec_chain.cc:604-626, bb_scrambler.cc,
// bbframe_parser.cc:14-56): the hard bits of dropped or foreign frames never
// leave the GPU, and the caller copies one packed buffer.
#include <algorithm>

#include "engine.h"

using namespace cusat_internal;

namespace {

constexpr int kHeaderBytes = 10;      // BBHEADER
constexpr int kMaxBbframe = 7274;     // largest K_bch / 8

__device__ __forceinline__ uint8_t crc8_bb(const uint8_t* d, int n)
{
    uint8_t reg = 0;
    for (int i = 0; i < n; i++) {
        reg ^= d[i];
        for (int b = 0; b < 8; b++)
            reg = (reg & 0x80) ? (uint8_t)((reg << 1) ^ 0xD5) : (uint8_t)(reg << 1);
    }
    return reg;
}

// One thread per frame: the data-field length the frame contributes (0 when
// it is dropped): converged, BCH valid, header CRC zero, DFL <= 8 kbch - 80
// and a multiple of 8, TS/GS generic packetized.  kbch_f: per-frame K_bch/8
// (frames of different codes), or nullptr for kbch everywhere.
__global__ void bb_header_kernel(const uint8_t* __restrict__ hard, int stride, int kbch_all,
                                 const int32_t* __restrict__ kbch_f, const int32_t* __restrict__ trials,
                                 const int32_t* __restrict__ valid, const uint8_t* __restrict__ prbs, int batch,
                                 int32_t* __restrict__ lengths)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < batch; f += gridDim.x * blockDim.x) {
        int n = 0;
        const int kbch = kbch_f ? kbch_f[f] : kbch_all;
        if (trials[f] >= 0 && valid[f]) {
            uint8_t h[kHeaderBytes];
            const uint8_t* src = hard + (size_t)f * stride;
#pragma unroll
            for (int i = 0; i < kHeaderBytes; i++)
                h[i] = src[i] ^ prbs[i];
            const int dfl = (h[4] << 8) | h[5];
            if (crc8_bb(h, kHeaderBytes) == 0 && dfl <= 8 * kbch - 80 && dfl % 8 == 0 && (h[0] >> 6) == 0)
                n = dfl / 8;
        }
        lengths[f] = n;
    }
}

// Output placement in frame order: a frame whose data field does not fit the
// room left yields nothing (the chain's rule), later frames may still fit.
// Sequential by nature; one thread walks the batch.
__global__ void bb_place_kernel(int batch, int max_out, int32_t* __restrict__ lengths,
                                int32_t* __restrict__ offsets)
{
    if (blockIdx.x != 0 || threadIdx.x != 0)
        return;
    int used = 0;
    for (int f = 0; f < batch; f++) {
        int n = lengths[f];
        if (n > max_out - used)
            n = 0;
        offsets[f] = used;
        lengths[f] = n;
        used += n;
    }
    offsets[batch] = used;
}

// One CTA per frame: descrambled data-field bytes to their place.
__global__ void bb_copy_kernel(const uint8_t* __restrict__ hard, int stride, const uint8_t* __restrict__ prbs,
                               int batch, const int32_t* __restrict__ lengths, const int32_t* __restrict__ offsets,
                               uint8_t* __restrict__ out)
{
    for (int f = blockIdx.x; f < batch; f += gridDim.x) {
        const int n = lengths[f];
        const uint8_t* src = hard + (size_t)f * stride + kHeaderBytes;
        uint8_t* dst = out + offsets[f];
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            dst[i] = src[i] ^ prbs[kHeaderBytes + i];
    }
}

}  // namespace

struct cusat_bb_extractor {
    int kbch = 0, sms = 0;
    uint8_t* prbs = nullptr;  // the scrambler sequence, kbch bytes (a prefix serves shorter codes)
};

namespace {

int extract(cusat_bb_extractor* x, const uint8_t* hard_dev, int hard_stride, const int32_t* kbch_dev,
            const int32_t* trials_dev, const int32_t* bch_valid_dev, int batch, uint8_t* out_dev, int max_out,
            int32_t* lengths_dev, int32_t* offsets_dev, cudaStream_t s)
{
    bb_header_kernel<<<(batch + 255) / 256, 256, 0, s>>>(hard_dev, hard_stride, x->kbch, kbch_dev, trials_dev,
                                                         bch_valid_dev, x->prbs, batch, lengths_dev);
    CU(cudaGetLastError(), "BBHEADER launch");
    bb_place_kernel<<<1, 32, 0, s>>>(batch, max_out, lengths_dev, offsets_dev);
    CU(cudaGetLastError(), "placement launch");
    bb_copy_kernel<<<std::min(batch, std::max(x->sms, 1) * 8), 256, 0, s>>>(hard_dev, hard_stride, x->prbs, batch,
                                                                         lengths_dev, offsets_dev, out_dev);
    CU(cudaGetLastError(), "data-field launch");
    return CUSAT_OK;
}

}  // namespace

extern "C" {

int cusat_bb_extractor_create(int framesize, int rate, cusat_bb_extractor** out)
{
    if (!out)
        return fail(CUSAT_ERR_ARG, "null argument");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    if (p->k_bch % 8 || p->k_bch / 8 > kMaxBbframe)
        return fail(CUSAT_ERR_UNSUPPORTED, "BBFRAME not byte aligned");
    // BB scrambler PRBS: 1 + X^14 + X^15 loaded with 100101010000000 (stage 1
    // first) at every BBFRAME, output bits MSB first
    std::vector<uint8_t> seq(p->k_bch / 8);
    unsigned reg = 0;
    const char* init = "100101010000000";
    for (int s = 0; s < 15; s++)
        if (init[s] == '1')
            reg |= 1u << s;
    for (auto& byte : seq) {
        byte = 0;
        for (int b = 0; b < 8; b++) {
            const unsigned o = ((reg >> 13) ^ (reg >> 14)) & 1u;
            reg = ((reg << 1) | o) & 0x7fffu;
            byte = (uint8_t)((byte << 1) | o);
        }
    }
    cusat_bb_extractor* x = new cusat_bb_extractor();
    x->kbch = p->k_bch / 8;
    cudaDeviceGetAttribute(&x->sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaMalloc(&x->prbs, seq.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(x->prbs, seq.data(), seq.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cusat_bb_extractor_destroy(x);
        return cuda_fail(e, "BB scrambler sequence");
    }
    *out = x;
    return CUSAT_OK;
}

void cusat_bb_extractor_destroy(cusat_bb_extractor* x)
{
    if (!x)
        return;
    if (x->prbs)
        cudaFree(x->prbs);
    delete x;
}

int cusat_bb_extract(cusat_bb_extractor* x, const uint8_t* hard_dev, int hard_stride, const int32_t* trials_dev,
                     const int32_t* bch_valid_dev, int batch, uint8_t* out_dev, int max_out, int32_t* lengths_dev,
                     int32_t* offsets_dev, void* stream)
{
    if (!x || !hard_dev || !trials_dev || !bch_valid_dev || !lengths_dev || !offsets_dev || batch <= 0 ||
        hard_stride < x->kbch || max_out < 0 || (max_out > 0 && !out_dev))
        return fail(CUSAT_ERR_ARG, "invalid extraction arguments");
    return extract(x, hard_dev, hard_stride, nullptr, trials_dev, bch_valid_dev, batch, out_dev, max_out, lengths_dev,
                   offsets_dev, (cudaStream_t)stream);
}

int cusat_bb_extract_frames(cusat_bb_extractor* x, const uint8_t* hard_dev, int hard_stride, const int32_t* kbch_dev,
                            const int32_t* trials_dev, const int32_t* bch_valid_dev, int batch, uint8_t* out_dev,
                            int max_out, int32_t* lengths_dev, int32_t* offsets_dev, void* stream)
{
    if (!x || !hard_dev || !kbch_dev || !trials_dev || !bch_valid_dev || !lengths_dev || !offsets_dev || batch <= 0 ||
        max_out < 0 || (max_out > 0 && !out_dev))
        return fail(CUSAT_ERR_ARG, "invalid extraction arguments");
    // every frame's kbch_dev[f] must be <= the extractor's code's and <= hard_stride
    return extract(x, hard_dev, hard_stride, kbch_dev, trials_dev, bch_valid_dev, batch, out_dev, max_out, lengths_dev,
                   offsets_dev, (cudaStream_t)stream);
}

}  // extern "C"
