// Standalone soft demapper and BCH syndrome-check kernels.
#include "fec_device.cuh"
#include "kernels.h"

namespace cusat {

constexpr int kDemapThreads = 256, kDemapSpan = 4;  // symbols per thread per pass
// Symbols a thread loads before demapping them: four for the load-bound
// formula kinds, one for the compute-bound log-MAP (fewer registers, more
// blocks: 64APSK normal, 256 frames, 1.8 -> 1.06 ms).
__host__ __device__ constexpr int span_of(int kind) { return kind == 2 ? 1 : kDemapSpan; }

// One MODCOD: grid.y = frame, each thread span_of(KIND) symbols spaced a
// block apart, points staged in shared memory.  Reference
// cuda/demapper_kernel.cu:31-184.
template <int KIND, int NM>
__global__ void __launch_bounds__(kDemapThreads) demap_kernel(DevDemap d, const float2* __restrict__ sym,
                                                             int16_t* __restrict__ out, float noise_var,
                                                             float llr_gain)
{
    __shared__ float2 pts[256];
    if (KIND == 2) {
        for (int k = threadIdx.x; k < d.n_points; k += blockDim.x)
            pts[k] = d.points[k];
        __syncthreads();
    }
    const int f = blockIdx.y;
    demap_span<KIND, NM, span_of(KIND)>(d, pts, sym + (size_t)f * d.xfec, out + (size_t)f * d.fec_len,
                                        blockIdx.x * kDemapThreads * span_of(KIND) + threadIdx.x, kDemapThreads,
                                        noise_var, llr_gain);
}

template <int KIND, int NM>
void launch_demap_kind(const DevDemap& d, const float2* sym, int batch, float noise_var, float llr_gain,
                       int16_t* out, cudaStream_t stream)
{
    const int per_block = kDemapThreads * span_of(KIND);
    for (int f0 = 0; f0 < batch; f0 += 65535) {
        dim3 grid((d.interleaved_len + per_block - 1) / per_block, batch - f0 < 65535 ? batch - f0 : 65535);
        demap_kernel<KIND, NM><<<grid, kDemapThreads, 0, stream>>>(d, sym + (size_t)f0 * d.xfec,
                                                                  out + (size_t)f0 * d.fec_len, noise_var,
                                                                  llr_gain);
    }
}

// Log-MAP with 32 to 256 points on symbols grouped by position.  The lanes
// of a warp that demap 32 unrelated symbols between them need nearly every
// (point, bit) exp; lanes whose symbols lie close together need the same
// few.  A block takes a chunk of kSortChunk symbols of one frame, counting-
// sorts them in shared memory by their cell of a kSortGrid x kSortGrid grid
// over [-kSortR, kSortR]^2 (clamped at the edges), and demaps them in that
// order with the vote variant of demap_logmap: per symbol the same terms in
// the same order, so the LLRs do not depend on the grouping.  Reference
// cuda/demapper_kernel.cu:108-183 (the APSK branch).
constexpr int kSortThreads = 256, kSortChunk = 1024, kSortGrid = 16;
constexpr float kSortR = 1.8f;  // unit-energy APSK: outer rings up to 1.70 (256APSK 31/45)

static_assert(kSortThreads == kDemapThreads, "the grouped chunk routine serves both demap kernels");

// Sorts the n <= CH symbols fs[0..n) of a chunk of one frame (frame positions
// c0..c0+n) by grid cell and demaps them in that order; all kSortThreads
// threads of the block call it, and it leaves cell / order / key free for
// the next chunk.
template <int NM, int CH>
__device__ __forceinline__ void demap_chunk_grouped(const DevDemap& d, const float2* pts, const float2* fs, int n,
                                                    int c0, float llr_gain, int16_t* o, int* cell, uint16_t* order,
                                                    uint8_t* key)
{
    const int tid = threadIdx.x;
    for (int k = tid; k < kSortGrid * kSortGrid; k += kSortThreads)
        cell[k] = 0;
    __syncthreads();
    const float gs = kSortGrid / (2.0f * kSortR);
    for (int p = tid; p < n; p += kSortThreads) {
        const float2 v = fs[p];
        // fminf/fmaxf map NaN to the edge cell
        const int cx = (int)fminf(fmaxf((v.x + kSortR) * gs, 0.0f), kSortGrid - 1.0f);
        const int cy = (int)fminf(fmaxf((v.y + kSortR) * gs, 0.0f), kSortGrid - 1.0f);
        key[p] = (uint8_t)(cy * kSortGrid + cx);
        atomicAdd(&cell[cy * kSortGrid + cx], 1);
    }
    __syncthreads();
    if (tid < 32) {  // exclusive scan of the 256 cell counts: 8 per lane
        int v[8], sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = cell[tid * 8 + k];
            sum += v[k];
        }
        int inc = sum;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, off);
            if (tid >= off)
                inc += y;
        }
        int run = inc - sum;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            cell[tid * 8 + k] = run;
            run += v[k];
        }
    }
    __syncthreads();
    for (int p = tid; p < n; p += kSortThreads)
        order[atomicAdd(&cell[key[p]], 1)] = (uint16_t)p;
    __syncthreads();
    for (int r = 0; r < CH / kSortThreads; r++) {
        const int slot = r * kSortThreads + tid;
        if (r * kSortThreads + (tid & ~31) >= n)
            break;  // the whole warp is past the chunk's symbols
        const bool valid = slot < n;
        const int p = valid ? order[slot] : 0;
        const float2 v = valid ? fs[p] : make_float2(0.0f, 0.0f);
        demap_logmap<NM, true>(d, pts, v.x, v.y, c0 + p, llr_gain, o, valid);
    }
    __syncthreads();
}

template <int NM>
__global__ void __launch_bounds__(kSortThreads) demap_sorted_kernel(DevDemap d, const float2* __restrict__ sym,
                                                                   int16_t* __restrict__ out, float llr_gain)
{
    __shared__ float2 pts[1 << NM];
    __shared__ int cell[kSortGrid * kSortGrid];
    __shared__ uint16_t order[kSortChunk];
    __shared__ uint8_t key[kSortChunk];
    for (int k = threadIdx.x; k < (1 << NM); k += kSortThreads)
        pts[k] = d.points[k];
    __syncthreads();
    const int c0 = blockIdx.x * kSortChunk;
    demap_chunk_grouped<NM, kSortChunk>(d, pts, sym + (size_t)blockIdx.y * d.xfec + c0,
                                        min(kSortChunk, d.interleaved_len - c0), c0, llr_gain,
                                        out + (size_t)blockIdx.y * d.fec_len, cell, order, key);
}

template <int NM>
void launch_demap_sorted(const DevDemap& d, const float2* sym, int batch, float llr_gain, int16_t* out,
                         cudaStream_t stream)
{
    for (int f0 = 0; f0 < batch; f0 += 65535) {
        dim3 grid((d.interleaved_len + kSortChunk - 1) / kSortChunk, batch - f0 < 65535 ? batch - f0 : 65535);
        demap_sorted_kernel<NM><<<grid, kSortThreads, 0, stream>>>(d, sym + (size_t)f0 * d.xfec,
                                                                  out + (size_t)f0 * d.fec_len, llr_gain);
    }
}

int launch_demap(const DevDemap& d, const float* sym, int batch, float noise_var, float llr_gain,
                 int16_t* out, cudaStream_t stream)
{
    const float2* s = reinterpret_cast<const float2*>(sym);
    if (d.kind == 0)
        launch_demap_kind<0, 0>(d, s, batch, noise_var, llr_gain, out, stream);
    else if (d.kind == 1)
        launch_demap_kind<1, 0>(d, s, batch, noise_var, llr_gain, out, stream);
    else if (d.n_points != 1 << d.n_mod)
        launch_demap_kind<2, 0>(d, s, batch, noise_var, llr_gain, out, stream);
    else if (d.n_mod == 3)
        launch_demap_kind<2, 3>(d, s, batch, noise_var, llr_gain, out, stream);
    else if (d.n_mod == 4)
        launch_demap_kind<2, 4>(d, s, batch, noise_var, llr_gain, out, stream);
    else if (d.n_mod == 5)
        launch_demap_sorted<5>(d, s, batch, llr_gain, out, stream);
    else if (d.n_mod == 6)
        launch_demap_sorted<6>(d, s, batch, llr_gain, out, stream);
    else if (d.n_mod == 7)
        launch_demap_sorted<7>(d, s, batch, llr_gain, out, stream);
    else if (d.n_mod == 8)
        launch_demap_sorted<8>(d, s, batch, llr_gain, out, stream);
    else
        launch_demap_kind<2, 0>(d, s, batch, noise_var, llr_gain, out, stream);
    return (int)cudaGetLastError();
}

// Mixed batch: grid.y = frame, each frame's MODCOD parameters (and points)
// staged in shared memory, blocks stride over the frame's symbols; the
// frame's kind and bit count are uniform over the block.
__global__ void __launch_bounds__(kDemapThreads) demap_mixed_kernel(const DevDemap* __restrict__ demaps,
                                                                   const DemapFrame* __restrict__ frames)
{
    __shared__ float2 pts[256];
    __shared__ DevDemap d;
    __shared__ int cell[kSortGrid * kSortGrid];
    __shared__ uint16_t order[kDemapThreads * kDemapSpan];
    __shared__ uint8_t key[kDemapThreads * kDemapSpan];
    const DemapFrame fr = frames[blockIdx.y];
    if (threadIdx.x == 0)
        d = demaps[fr.modcod];
    __syncthreads();
    if (d.kind == 2)
        for (int k = threadIdx.x; k < d.n_points; k += blockDim.x)
            pts[k] = d.points[k];
    __syncthreads();
    const bool full = d.n_points == 1 << d.n_mod;  // 2^n_mod points: the specialised log-MAP applies
    const int sel = d.kind == 2 ? 2 * 16 + (full && d.n_mod >= 4 && d.n_mod <= 8 ? d.n_mod : 0) : d.kind * 16;
    const int per_block = kDemapThreads * kDemapSpan;
    if (sel >= 37 && sel <= 40) {
        // 32 to 256 points: the block's chunks grouped by position, as in
        // demap_sorted_kernel
        for (int base = blockIdx.x * per_block; base < d.interleaved_len; base += gridDim.x * per_block) {
            const int n = min(per_block, d.interleaved_len - base);
            switch (sel) {
            case 37: demap_chunk_grouped<5, kDemapThreads * kDemapSpan>(d, pts, fr.sym + base, n, base, fr.llr_gain, fr.out, cell, order, key); break;
            case 38: demap_chunk_grouped<6, kDemapThreads * kDemapSpan>(d, pts, fr.sym + base, n, base, fr.llr_gain, fr.out, cell, order, key); break;
            case 39: demap_chunk_grouped<7, kDemapThreads * kDemapSpan>(d, pts, fr.sym + base, n, base, fr.llr_gain, fr.out, cell, order, key); break;
            default: demap_chunk_grouped<8, kDemapThreads * kDemapSpan>(d, pts, fr.sym + base, n, base, fr.llr_gain, fr.out, cell, order, key); break;
            }
        }
        return;
    }
    for (int j0 = blockIdx.x * per_block + threadIdx.x; j0 - (int)threadIdx.x < d.interleaved_len;
         j0 += gridDim.x * per_block) {
        switch (sel) {
        case 0: demap_span<0, 0, kDemapSpan>(d, pts, fr.sym, fr.out, j0, kDemapThreads, fr.noise_var, fr.llr_gain); break;
        case 16: demap_span<1, 0, kDemapSpan>(d, pts, fr.sym, fr.out, j0, kDemapThreads, fr.noise_var, fr.llr_gain); break;
        default:
            // log-MAP: one symbol at a time (compute-bound)
            for (int u = 0; u < kDemapSpan; u++) {
                const int j = j0 + u * kDemapThreads;
                switch (sel) {
                case 36: demap_span<2, 4, 1>(d, pts, fr.sym, fr.out, j, kDemapThreads, fr.noise_var, fr.llr_gain); break;
                default: demap_span<2, 0, 1>(d, pts, fr.sym, fr.out, j, kDemapThreads, fr.noise_var, fr.llr_gain); break;
                }
            }
            break;
        }
    }
}

int launch_demap_mixed(const DevDemap* demaps, const DemapFrame* frames, int n, int max_len, cudaStream_t stream)
{

    const int per_block = kDemapThreads * kDemapSpan;
    for (int f0 = 0; f0 < n; f0 += 65535) {
        dim3 grid((max_len + per_block - 1) / per_block, n - f0 < 65535 ? n - f0 : 65535);
        demap_mixed_kernel<<<grid, kDemapThreads, 0, stream>>>(demaps, frames + f0);
    }
    return (int)cudaGetLastError();
}

// BCH check: one warp per frame.  Lane l runs the byte-LUT LFSR
// r <- (r x^8 + b x^p) mod g over bytes [l chunk, (l+1) chunk) of the frame
// front-padded with zero bytes to 32 chunks (leading zeros leave the
// remainder unchanged).  The 32 lane remainders are then combined in five
// shuffle levels: at level k the earlier block A and the later block B of
// each pair give A x^(8 chunk 2^k) + B mod g, the multiplication being a
// XOR of per-byte tables.  The result is c(x) x^p mod g(x), which is zero iff
// c is a codeword.  Reference cuda/bch_common.cuh:91-158.
template <int W>
__global__ void __launch_bounds__(128) bch_check_kernel(BchDev t, const uint8_t* __restrict__ cw,
                                                        int32_t* __restrict__ valid,
                                                        uint8_t* __restrict__ rem, int batch)
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
    const uint8_t* src = cw + (size_t)f * t.n_bytes;
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
    if (lane == 0) {
        uint64_t any = 0;
#pragma unroll
        for (int w = 0; w < W; w++)
            any |= r[w];
        if (valid)
            valid[f] = any == 0;
        if (rem)
            for (int jb = 0; jb < nb; jb++) {
                const int lo = p - 8 * (jb + 1);
                rem[(size_t)f * nb + jb] = (uint8_t)(r[lo >> 6] >> (lo & 63));
            }
    }
}

// Mixed batches: one warp per frame, each frame with its own code's tables
// (LUT read through L1 instead of staged in shared memory).
template <int W>
__device__ void bch_frame(const BchDev& t, const uint8_t* __restrict__ src, int32_t* valid, int lane)
{
    const int p = t.p;
    const uint64_t top_mask = (p % 64) ? ((1ull << (p % 64)) - 1) : ~0ull;
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
            r[w] ^= __ldg(t.lut + idx * W + w);
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
    if (lane == 0) {
        uint64_t any = 0;
#pragma unroll
        for (int w = 0; w < W; w++)
            any |= r[w];
        *valid = any == 0;
    }
}

__global__ void __launch_bounds__(128) bch_check_mixed_kernel(const BchDev* __restrict__ codes,
                                                              const BchFrame* __restrict__ frames, int n)
{
    const int lane = threadIdx.x & 31;
    const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (f >= n)
        return;
    const BchFrame fr = frames[f];
    if (!fr.valid)
        return;
    const BchDev t = codes[fr.code];
    if (t.words == 2)
        bch_frame<2>(t, fr.cw, fr.valid, lane);
    else if (t.words == 3)
        bch_frame<3>(t, fr.cw, fr.valid, lane);
    else if (t.words == 4)
        bch_frame<4>(t, fr.cw, fr.valid, lane);
    else
        bch_frame<1>(t, fr.cw, fr.valid, lane);
}

int launch_bch_check_mixed(const BchDev* codes, const BchFrame* frames, int n, cudaStream_t stream)
{
    if (n <= 0)
        return 0;
    bch_check_mixed_kernel<<<(n + 3) / 4, 128, 0, stream>>>(codes, frames, n);
    return (int)cudaGetLastError();
}

int launch_bch_check(const BchDev& t, const uint8_t* cw, int32_t* valid, uint8_t* rem, int batch,
                     cudaStream_t stream)
{
    const int blocks = (batch + 3) / 4;
    if (t.words == 1)
        bch_check_kernel<1><<<blocks, 128, 0, stream>>>(t, cw, valid, rem, batch);
    else if (t.words == 2)
        bch_check_kernel<2><<<blocks, 128, 0, stream>>>(t, cw, valid, rem, batch);
    else if (t.words == 3)
        bch_check_kernel<3><<<blocks, 128, 0, stream>>>(t, cw, valid, rem, batch);
    else
        bch_check_kernel<4><<<blocks, 128, 0, stream>>>(t, cw, valid, rem, batch);
    return (int)cudaGetLastError();
}

}  // namespace cusat
