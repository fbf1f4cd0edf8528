// Launchers of the FEC kernels (host-callable, defined in the .cu files).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "fec_device.cuh"

namespace cusat {

struct DecodeArgs;

// BCH check tables in device memory (host.h BchTables layout).
struct BchDev {
    int p, words;
    unsigned n_bytes, chunk, lead;
    const uint64_t* lut;   // [256 * words]
    const uint64_t* tree;  // [5][p/8][256][words]
};

// One frame of a mixed BCH check.
struct BchFrame {
    int code, pad;
    const uint8_t* cw;
    int32_t* valid;  // nullptr: frame not checked
};

// Shared-memory layout and limits of one decoder kernel instantiation.
struct DecoderKernelInfo {
    const void* fn;
    int threads;
    int blocks_per_sm;
};

// Largest code dimensions a decoder launch must hold in shared memory.
struct SmemDims {
    int N, q, n_steps, n_items, cmax, lanes;
};

// The kernel instantiation for (cmax, lanes), or nullptr.
const void* select_decoder_kernel(int cmax, int lanes);
// Fills the shared-memory carve-up of a for codes up to d.
void decoder_smem_layout(DecodeArgs* a, const SmemDims& d);
SmemDims smem_dims_of(const DevCode& c, int lanes);
int decoder_threads(int lanes);
// Syndrome-check period of every decoder launch: CUSAT_LDPC_SYN_PERIOD when
// it is a positive integer, else 1; read once per process, like the
// reference (cuda/ldpc_decode_kernel.cu:1237-1241).
int syndrome_period();
int launch_decoder(const void* fn, const DecodeArgs& a, int grid, int threads, cudaStream_t stream);
// The frame-pair kernel (two frames per CTA, single-code launches of codes
// decoded one layer per step) for cmax, or nullptr; its threads per CTA;
// its shared-memory carve-up for codes up to d with max_stage stage rows per
// set (also sets a->max_stage).
const void* select_pair_kernel(int cmax);
constexpr int kPairThreads = 384;
void pair_smem_layout(DecodeArgs* a, const SmemDims& d, int max_stage);
// Bytes of one check row of messages in the frame-pair kernel (two frames'
// bytes per edge, whole 16-byte words).
int pair_msg_row(int cmax);

int launch_demap(const DevDemap& d, const float* sym, int batch, float noise_var, float llr_gain,
                 int16_t* out, cudaStream_t stream);
// One frame of a mixed demap launch (device memory).
struct DemapFrame {
    int modcod;              // index into the launch's DevDemap array
    float noise_var, llr_gain;
    int pad;
    const float2* sym;       // [xfec] symbols
    int16_t* out;            // [fec_len] LLRs
};
// Demaps n frames of any of the given MODCODs; max_len = the largest
// interleaved length among them.
int launch_demap_mixed(const DevDemap* demaps, const DemapFrame* frames, int n, int max_len, cudaStream_t stream);
// Sets the message returned by cusat_last_error() on this thread.
void set_last_error(const std::string& msg);

int launch_bch_check_mixed(const BchDev* codes, const BchFrame* frames, int n, cudaStream_t stream);
int launch_bch_check(const BchDev& t, const uint8_t* cw, int32_t* valid, uint8_t* rem, int batch,
                     cudaStream_t stream);

}  // namespace cusat
