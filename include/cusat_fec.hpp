// cusat_fec.hpp -- header-only C++ shims with the reference's class names and
// signatures, over the C ABI of cusat_fec.h.  A translation unit of the
// reference's RX chain that includes this header instead of
//   lib/cusat_dsp/cuda/ldpc_decode_kernel.cuh   (cuda::ldpc_decode_cuda)
//   lib/cusat_dsp/ldpc_decode.h                 (ldpc_decode)
//   lib/cusat_dsp/cuda/demapper_kernel.cuh      (cuda::demapper_cuda)
//   lib/cusat_dsp/cuda/bch_check_kernel.cuh     (cuda::bch_check_cuda)
//   lib/cusat_dsp/rx_fec_chain.h                (rx_fec_chain, gpu_decode_budget)
//   lib/cusat_dsp/rx_fec_pool.h                 (rx_fec_pool: declared when this
//                                                header is included after the
//                                                reference's acm_config.h)
// compiles unchanged and links against libcusat_fec.so.
//
// Error behaviour mirrors the reference: a batch size outside 1..max_batch is
// a silent no-op (ldpc_decode_kernel.cu:1291-1292, demapper_kernel.cu:305-306),
// a CUDA failure aborts (cuda_util.cu:23-44), the BCH checker throws
// std::invalid_argument on a bad geometry, negative batch or null buffer
// (bch_check_kernel.cu:17-18,28-33), and construction without a GPU aborts
// (ldpc_decode.cc:33-40).
#ifndef CUSAT_FEC_HPP
#define CUSAT_FEC_HPP

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <chrono>
#include <complex>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "cusat_fec.h"

#ifndef INCLUDED_CUSAT_DSP_MODCOD_TYPES_H
// Standalone use: the enumerations of the reference's modcod_types.h with
// the same numeric values (cusat_data.h lists all of them).
namespace cusat_dsp {
enum code_rate_t : int {
    RATE_1_4, RATE_1_3, RATE_2_5, RATE_1_2, RATE_3_5, RATE_2_3, RATE_3_4, RATE_4_5, RATE_5_6, RATE_8_9,
    RATE_9_10, RATE_11_45, RATE_4_15, RATE_13_45, RATE_14_45, RATE_9_20, RATE_7_15, RATE_90_180,
    RATE_8_15, RATE_96_180, RATE_11_20, RATE_100_180, RATE_26_45, RATE_104_180, RATE_18_30,
    RATE_28_45, RATE_23_36, RATE_116_180, RATE_20_30, RATE_124_180, RATE_25_36, RATE_32_45,
    RATE_128_180, RATE_13_18, RATE_22_30, RATE_132_180, RATE_135_180, RATE_7_9, RATE_140_180,
    RATE_154_180,
};
enum fecframe_size_t : int { FECFRAME_NORMAL, FECFRAME_SHORT, FECFRAME_MEDIUM };
enum modulation_t : int { MOD_QPSK, MOD_8PSK, MOD_8APSK, MOD_16APSK, MOD_32APSK, MOD_64APSK, MOD_128APSK,
                          MOD_256APSK };
// Flat table descriptor (reference ldpc_tables/ldpc_code.h:25-39); only n
// is read here, to recover the frame size.
struct ldpc_code {
    int n, k, m, links_total, links_max_cn, n_rows;
    const uint8_t* row_deg;
    const uint32_t* row_off;
    const uint16_t* addr;
};
}  // namespace cusat_dsp
#endif

namespace cusat_dsp {
namespace cusat_shim {

inline void die(int rc, const char* what)
{
    fprintf(stderr, "cusat_fec: %s failed (%d): %s\n", what, rc, cusat_last_error());
    abort();
}

inline int framesize_of(int n_bits)
{
    return n_bits == 64800 ? FECFRAME_NORMAL : n_bits == 16200 ? FECFRAME_SHORT : FECFRAME_MEDIUM;
}

}  // namespace cusat_shim

namespace cuda {

// Reference lib/cusat_dsp/cuda/ldpc_decode_kernel.cuh:22-107.
class ldpc_decode_cuda
{
  public:
    ldpc_decode_cuda(const ldpc_code* code, code_rate_t rate, int max_trials = 25, int max_batch = 64)
    {
        const int rc = cusat_ldpc_decoder_create(cusat_shim::framesize_of(code->n), (int)rate, max_trials,
                                                 max_batch, &d_);
        if (rc)
            cusat_shim::die(rc, "ldpc_decode_cuda");
        int32_t info[8];
        cusat_ldpc_decoder_info(d_, info);
        n_ = info[0];
        k_ = info[1];
        max_batch_ = max_batch;
    }
    ~ldpc_decode_cuda() { cusat_ldpc_decoder_destroy(d_); }
    ldpc_decode_cuda(const ldpc_decode_cuda&) = delete;
    ldpc_decode_cuda& operator=(const ldpc_decode_cuda&) = delete;

    void decode_batch(const int16_t* soft_in, uint8_t* hard_out, int* trials_out, int batch_size,
                      cudaStream_t stream)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_ldpc_decode_batch(d_, soft_in, hard_out, (int32_t*)trials_out, batch_size, stream);
        if (rc)
            cusat_shim::die(rc, "decode_batch");
    }

    void decode_batch_d2h(const int16_t* soft_in_dev, uint8_t* hard_out_host, int* trials_out_host,
                          int batch_size, cudaStream_t stream)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_ldpc_decode_batch_d2h(d_, soft_in_dev, hard_out_host, (int32_t*)trials_out_host,
                                                   batch_size, stream);
        if (rc)
            cusat_shim::die(rc, "decode_batch_d2h");
    }

    void decode_launch_async(const int16_t* soft_in, int batch_size, cudaStream_t stream,
                             uint8_t* hard_out = nullptr, int* result_out = nullptr)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_ldpc_decode_launch(d_, soft_in, batch_size, stream, hard_out, (int32_t*)result_out);
        if (rc)
            cusat_shim::die(rc, "decode_launch_async");
    }

    int n_bits() const { return n_; }
    int k_bits() const { return k_; }
    int k_bytes() const { return k_ / 8; }

  private:
    cusat_ldpc_decoder* d_ = nullptr;
    int n_ = 0, k_ = 0, max_batch_ = 0;
};

// Reference lib/cusat_dsp/cuda/demapper_kernel.cuh:23-89.
class demapper_cuda
{
  public:
    demapper_cuda(modulation_t constellation, code_rate_t rate, fecframe_size_t framesize, int max_batch = 64)
    {
        const int rc = cusat_demapper_create((int)constellation, (int)rate, (int)framesize, max_batch, &d_);
        if (rc)
            cusat_shim::die(rc, "demapper_cuda");
        cusat_demapper_info(d_, info_);
        max_batch_ = max_batch;
    }
    ~demapper_cuda() { cusat_demapper_destroy(d_); }
    demapper_cuda(const demapper_cuda&) = delete;
    demapper_cuda& operator=(const demapper_cuda&) = delete;

    void demap_batch(const float* sym_in_host, int batch_size, float noise_var, float llr_gain)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_demap_batch(d_, sym_in_host, batch_size, noise_var, llr_gain);
        if (rc)
            cusat_shim::die(rc, "demap_batch");
    }

    void demap_batch_async(const float* sym_in_host, int batch_size, float noise_var, float llr_gain,
                           cudaStream_t stream)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_demap_batch_async(d_, sym_in_host, batch_size, noise_var, llr_gain, stream);
        if (rc)
            cusat_shim::die(rc, "demap_batch_async");
    }

    float capped_llr_gain(float llr_gain) const { return cusat_demapper_capped_llr_gain(d_, llr_gain); }
    int16_t* soft_out_dev() const { return cusat_demapper_soft_out_dev(d_); }
    int fecframe_len() const { return info_[0]; }
    int xfecframe_len() const { return info_[1]; }
    int n_mod() const { return info_[2]; }

  private:
    cusat_demapper* d_ = nullptr;
    int32_t info_[4] = {0, 0, 0, 0};
    int max_batch_ = 0;
};

// Reference lib/cusat_dsp/cuda/bch_check_kernel.cuh:9-24.
class bch_check_cuda
{
  public:
    bch_check_cuda(const uint64_t* flat_lut, const uint64_t* gen_poly, int gen_degree, unsigned int n_bytes)
    {
        const int rc = cusat_bch_checker_create(flat_lut, gen_poly, gen_degree, n_bytes, &c_);
        if (rc == CUSAT_ERR_ARG)
            throw std::invalid_argument(cusat_last_error());
        if (rc)
            cusat_shim::die(rc, "bch_check_cuda");
    }
    ~bch_check_cuda() { cusat_bch_checker_destroy(c_); }
    bch_check_cuda(const bch_check_cuda&) = delete;
    bch_check_cuda& operator=(const bch_check_cuda&) = delete;

    void check_async(const uint8_t* codewords_dev, int* valid_out_dev, int batch_size, cudaStream_t stream)
    {
        if (batch_size < 0)
            throw std::invalid_argument("negative BCH batch");
        if (!batch_size)
            return;
        if (!codewords_dev || !valid_out_dev)
            throw std::invalid_argument("null BCH checker buffer");
        const int rc = cusat_bch_check_launch(c_, codewords_dev, (int32_t*)valid_out_dev, nullptr, batch_size,
                                              stream);
        if (rc)
            cusat_shim::die(rc, "check_async");
    }
    unsigned int n_bytes() const { return cusat_bch_checker_n_bytes(c_); }

  private:
    cusat_bch_checker* c_ = nullptr;
};

}  // namespace cuda

// Reference lib/cusat_dsp/ldpc_decode.h:22-69: owns its stream.
class ldpc_decode
{
  public:
    ldpc_decode(fecframe_size_t framesize, code_rate_t rate, int max_trials = 25, int cuda_max_batch = 64)
    {
        const int rc = cusat_ldpc_decoder_create((int)framesize, (int)rate, max_trials, cuda_max_batch, &d_);
        if (rc)
            cusat_shim::die(rc, "ldpc_decode");
        int32_t info[8];
        cusat_ldpc_decoder_info(d_, info);
        n_ = (unsigned)info[0];
        k_ = (unsigned)info[1];
        max_batch_ = cuda_max_batch;
        if (cudaStreamCreate(&stream_) != cudaSuccess)
            cusat_shim::die(CUSAT_ERR_CUDA, "cudaStreamCreate");
    }
    ~ldpc_decode()
    {
        cusat_ldpc_decoder_destroy(d_);
        if (stream_)
            cudaStreamDestroy(stream_);
    }
    ldpc_decode(const ldpc_decode&) = delete;
    ldpc_decode& operator=(const ldpc_decode&) = delete;

    void decode_batch_cuda(const int16_t* soft_in, uint8_t* hard_out, int* trials_out, int batch_size)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_ldpc_decode_batch(d_, soft_in, hard_out, (int32_t*)trials_out, batch_size, stream_);
        if (rc)
            cusat_shim::die(rc, "decode_batch_cuda");
    }

    void decode_batch_cuda_d2h(const int16_t* soft_in_dev, uint8_t* hard_out, int* trials_out, int batch_size)
    {
        if (batch_size <= 0 || batch_size > max_batch_)
            return;
        const int rc = cusat_ldpc_decode_batch_d2h(d_, soft_in_dev, hard_out, (int32_t*)trials_out, batch_size,
                                                   stream_);
        if (rc)
            cusat_shim::die(rc, "decode_batch_cuda_d2h");
    }

    CUstream_st* cuda_stream() const { return stream_; }
    unsigned int n_bits() const { return n_; }
    unsigned int k_bits() const { return k_; }
    unsigned int n_bytes() const { return n_ / 8; }
    unsigned int k_bytes() const { return k_ / 8; }

  private:
    cusat_ldpc_decoder* d_ = nullptr;
    cudaStream_t stream_ = nullptr;
    unsigned n_ = 0, k_ = 0;
    int max_batch_ = 0;
};

// Reference lib/cusat_dsp/ldpc_encode.h:18-84 (the systematic IRA encoder,
// for the reference's transmit-side and test callers; not on the receive
// path).  The codewords are computed on the host (cusat_ldpc_encode); the
// *_to_device variants copy them on the caller's stream, the D2D variant
// reads the info bits back first.
class ldpc_encode
{
  public:
    ldpc_encode(fecframe_size_t framesize, code_rate_t rate) : fs_((int)framesize), rate_((int)rate)
    {
        int32_t info[12];
        const int rc = cusat_code_info(fs_, rate_, info);
        if (rc)
            cusat_shim::die(rc, "ldpc_encode");
        n_ = (unsigned)info[0];
        k_ = (unsigned)info[1];
    }
    ldpc_encode(const ldpc_encode&) = delete;
    ldpc_encode& operator=(const ldpc_encode&) = delete;

    void encode(const uint8_t* info_in, uint8_t* codeword_out)
    {
        const int rc = cusat_ldpc_encode(fs_, rate_, info_in, codeword_out, 1);
        if (rc)
            cusat_shim::die(rc, "ldpc_encode::encode");
    }
    void encode_to_device(const uint8_t* info_packed_host, uint8_t* fecframe_device, void* cuda_stream)
    {
        encode_batch_to_device(info_packed_host, fecframe_device, 1, cuda_stream);
    }
    void encode_batch_to_device(const uint8_t* info_packed_host, uint8_t* fecframes_device, int batch_size,
                                void* cuda_stream)
    {
        if (batch_size <= 0)
            return;
        buf_.resize((size_t)batch_size * n_bytes());
        const int rc = cusat_ldpc_encode(fs_, rate_, info_packed_host, buf_.data(), batch_size);
        if (rc)
            cusat_shim::die(rc, "ldpc_encode::encode_batch_to_device");
        // a pageable source is staged before the call returns
        if (cudaMemcpyAsync(fecframes_device, buf_.data(), buf_.size(), cudaMemcpyHostToDevice,
                            (cudaStream_t)cuda_stream) != cudaSuccess)
            cusat_shim::die(CUSAT_ERR_CUDA, "ldpc_encode copy");
    }
    void encode_batch_d2d(const uint8_t* info_packed_device, uint8_t* fecframes_device, int batch_size,
                          void* cuda_stream)
    {
        if (batch_size <= 0)
            return;
        std::vector<uint8_t> info((size_t)batch_size * k_bytes());
        if (cudaMemcpyAsync(info.data(), info_packed_device, info.size(), cudaMemcpyDeviceToHost,
                            (cudaStream_t)cuda_stream) != cudaSuccess ||
            cudaStreamSynchronize((cudaStream_t)cuda_stream) != cudaSuccess)
            cusat_shim::die(CUSAT_ERR_CUDA, "ldpc_encode read-back");
        encode_batch_to_device(info.data(), fecframes_device, batch_size, cuda_stream);
    }
    unsigned int n_bits() const { return n_; }
    unsigned int k_bits() const { return k_; }
    unsigned int n_bytes() const { return n_ / 8; }
    unsigned int k_bytes() const { return k_ / 8; }

  private:
    int fs_, rate_;
    unsigned n_ = 0, k_ = 0;
    std::vector<uint8_t> buf_;
};


// Reference lib/cusat_dsp/rx_fec_chain.h:52-59.  The cap lives in the
// library; chains share it through set_decode_budget.
struct gpu_decode_budget {
    cusat_decode_budget* h = nullptr;
    explicit gpu_decode_budget(int cap_frames = -1)
    {
        const int rc = cusat_decode_budget_create(cap_frames, &h);
        if (rc)
            cusat_shim::die(rc, "gpu_decode_budget");
    }
    ~gpu_decode_budget() { cusat_decode_budget_destroy(h); }
    gpu_decode_budget(const gpu_decode_budget&) = delete;
    gpu_decode_budget& operator=(const gpu_decode_budget&) = delete;
    static std::shared_ptr<gpu_decode_budget> make_default() { return std::make_shared<gpu_decode_budget>(-1); }
    int cap() const
    {
        int32_t v[2];
        cusat_decode_budget_info(h, v);
        return v[0];
    }
    int in_flight() const
    {
        int32_t v[2];
        cusat_decode_budget_info(h, v);
        return v[1];
    }
};

// Reference lib/cusat_dsp/rx_fec_chain.h:61-297 (the diagnostic flags are
// accepted and ignored: they write files under /tmp in the reference).
class rx_fec_chain
{
  public:
    typedef std::complex<float> sym_t;

    rx_fec_chain(fecframe_size_t framesize, code_rate_t rate, modulation_t constellation, int max_trials = 25,
                 int cuda_max_batch = 64, int n_gpu_streams = 8, int micro_batch = 4)
    {
        const int rc = cusat_rx_chain_create((int)framesize, (int)rate, (int)constellation, max_trials,
                                             cuda_max_batch, n_gpu_streams, micro_batch, &c_);
        if (rc)
            cusat_shim::die(rc, "rx_fec_chain");
        owned_ = true;
        init();
    }
    explicit rx_fec_chain(cusat_rx_chain* borrowed) : c_(borrowed) { init(); }
    ~rx_fec_chain()
    {
        if (owned_)
            cusat_rx_chain_destroy(c_);
    }
    rx_fec_chain(const rx_fec_chain&) = delete;
    rx_fec_chain& operator=(const rx_fec_chain&) = delete;

    bool submit_xfecframe(const sym_t* symbols, int n_symbols)
    {
        return ok(cusat_rx_chain_submit_xfecframe(c_, reinterpret_cast<const float*>(symbols), n_symbols),
                  "submit_xfecframe") > 0;
    }
    int get_gse_output(uint8_t* out, int max_bytes)
    {
        const int n = ok(cusat_rx_chain_get_gse_output(c_, out, max_bytes), "get_gse_output");
        const int k = cusat_rx_chain_gse_dfl_sizes(c_, nullptr, 0);
        sizes_.resize((size_t)k);
        cusat_rx_chain_gse_dfl_sizes(c_, sizes_.data(), k);
        return n;
    }
    const std::vector<int>& gse_dfl_sizes() const { return sizes_; }
    void reset() { ok(cusat_rx_chain_reset(c_), "reset"); }
    void flush() { ok(cusat_rx_chain_flush(c_), "flush"); }
    bool drain_completed() { return ok(cusat_rx_chain_drain_completed(c_), "drain_completed") > 0; }
    void launch_partial() { ok(cusat_rx_chain_launch_partial(c_), "launch_partial"); }
    void warmup() { ok(cusat_rx_chain_warmup(c_), "warmup"); }
    void update_snr(float snr_db) { cusat_rx_chain_update_snr(c_, snr_db); }
    void set_block_when_full(bool on) { cusat_rx_chain_set_block_when_full(c_, on ? 1 : 0); }
    // extension (not in the reference): frame copies split across helper threads
    void set_copy_threads(int helpers) { ok(cusat_rx_chain_set_copy_threads(c_, helpers), "set_copy_threads"); }
    void set_diag_fec_bench(bool) {}
    void set_diag_llr_histogram(bool) {}
    void set_diag_ldpc_convergence(bool) {}
    void set_cuda_mutex(std::mutex* mtx)
    {
        if (mtx)
            cusat_rx_chain_set_launch_lock(c_, &lock_mutex, &unlock_mutex, mtx);
        else
            cusat_rx_chain_set_launch_lock(c_, nullptr, nullptr, nullptr);
    }
    void set_decode_budget(std::shared_ptr<gpu_decode_budget> b)
    {
        if (b) {
            cusat_rx_chain_set_decode_budget(c_, b->h);
            budget_ = std::move(b);
        }
    }
    static bool frame_passes_fec_checks(int ldpc_trials_remaining, bool bch_valid)
    {
        return ldpc_trials_remaining >= 0 && bch_valid;
    }

    float snr_db() const { return (float)stat(7); }
    float data_snr_db() const { return (float)stat(7); }
    float precision() const { return (float)stat(8); }
    uint64_t frame_count() const { return (uint64_t)stat(0); }
    uint64_t frame_error_count() const { return (uint64_t)stat(1); }
    uint64_t gpu_drop_count() const { return (uint64_t)stat(2); }
    int gpu_inflight() const { return (int)stat(3); }
    int gpu_pending_launch() const { return (int)stat(4); }
    uint64_t force_drain_count() const { return (uint64_t)stat(5); }
    int pending_count() const { return (int)stat(6); }
    int batch_size() const { return info_[2]; }
    int max_output_bytes() const { return info_[3]; }
    std::chrono::steady_clock::time_point batch_start_time() const
    {
        return std::chrono::steady_clock::now() -
               std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                   std::chrono::duration<double>(stat(10)));
    }

  private:
    void init() { cusat_rx_chain_info(c_, info_); }
    double stat(int i) const
    {
        double v[12];
        cusat_rx_chain_stats(c_, v);
        return v[i];
    }
    static int ok(int rc, const char* what)
    {
        if (rc < 0)
            cusat_shim::die(rc, what);
        return rc;
    }
    static void lock_mutex(void* m) { static_cast<std::mutex*>(m)->lock(); }
    static void unlock_mutex(void* m) { static_cast<std::mutex*>(m)->unlock(); }

    cusat_rx_chain* c_ = nullptr;
    bool owned_ = false;
    int32_t info_[6] = {0, 0, 0, 0, 0, 0};
    std::vector<int> sizes_;
    std::shared_ptr<gpu_decode_budget> budget_;
};

}  // namespace cusat_dsp
#endif  // CUSAT_FEC_HPP

// The pool needs the reference's find_modcod (acm_config.h): it is declared
// by whichever inclusion of this header follows acm_config.h.
#if defined(INCLUDED_CUSAT_DSP_ACM_CONFIG_H) && !defined(CUSAT_FEC_HPP_POOL)
#define CUSAT_FEC_HPP_POOL
namespace cusat_dsp {

// Reference lib/cusat_dsp/rx_fec_pool.h:25-140; MODCODs resolved with the
// reference's find_modcod.  submit takes any layout type with a modcod
// member (the reference's pl_layout).
class rx_fec_pool
{
  public:
    typedef std::complex<float> sym_t;

    // mixed: every MODCOD in one slot ring of slot_frames-frame launches
    // (cusat_rx_pool_create_mixed); the reference's arguments keep their meaning
    rx_fec_pool(fecframe_size_t framesize, const std::vector<uint8_t>& enabled_modcods, int max_trials = 25,
                int cuda_max_batch = 64, int n_gpu_streams = 8, int micro_batch = 4, bool mixed = false,
                int slot_frames = 64)
    {
        std::vector<int32_t> triples;
        for (uint8_t idx : enabled_modcods) {
            const modcod_def_t* def = find_modcod(idx);
            if (!def)
                throw std::invalid_argument("Unknown modcod_idx: " + std::to_string(idx));
            triples.push_back(idx);
            triples.push_back((int32_t)def->constellation);
            triples.push_back((int32_t)def->code_rate);
        }
        const int rc = mixed ? cusat_rx_pool_create_mixed((int)framesize, triples.data(), (int)enabled_modcods.size(),
                                                          max_trials, n_gpu_streams, micro_batch, slot_frames, &p_)
                             : cusat_rx_pool_create((int)framesize, triples.data(), (int)enabled_modcods.size(),
                                                    max_trials, cuda_max_batch, n_gpu_streams, micro_batch, &p_);
        if (rc)
            cusat_shim::die(rc, "rx_fec_pool");
    }
    ~rx_fec_pool() { cusat_rx_pool_destroy(p_); }
    rx_fec_pool(const rx_fec_pool&) = delete;
    rx_fec_pool& operator=(const rx_fec_pool&) = delete;

    template <class Layout>
    bool submit(const sym_t* symbols, int n_symbols, const Layout& pls)
    {
        return ok(cusat_rx_pool_submit(p_, reinterpret_cast<const float*>(symbols), n_symbols, (int)pls.modcod),
                  "submit") > 0;
    }
    int get_gse_output(uint8_t* out, int max_bytes)
    {
        const int n = ok(cusat_rx_pool_get_gse_output(p_, out, max_bytes), "get_gse_output");
        const int k = cusat_rx_pool_gse_dfl_sizes(p_, nullptr, 0);
        sizes_.resize((size_t)k);
        cusat_rx_pool_gse_dfl_sizes(p_, sizes_.data(), k);
        return n;
    }
    const std::vector<int>& gse_dfl_sizes() const { return sizes_; }
    void reset_all() { ok(cusat_rx_pool_reset_all(p_), "reset_all"); }
    void warmup_all() { ok(cusat_rx_pool_warmup_all(p_), "warmup_all"); }
    bool launch_stale(std::chrono::milliseconds max_age)
    {
        return ok(cusat_rx_pool_launch_stale(p_, (double)max_age.count()), "launch_stale") > 0;
    }
    bool drain_all_completed() { return ok(cusat_rx_pool_drain_all_completed(p_), "drain_all_completed") > 0; }
    void finish_all_pending() { ok(cusat_rx_pool_finish_all_pending(p_), "finish_all_pending"); }
    void set_diag_fec_bench(bool) {}
    void set_diag_llr_histogram(bool) {}
    void set_diag_ldpc_convergence(bool) {}
    void set_cuda_mutex(std::mutex* mtx)
    {
        if (mtx)
            cusat_rx_pool_set_launch_lock(p_, &lock_mutex, &unlock_mutex, mtx);
        else
            cusat_rx_pool_set_launch_lock(p_, nullptr, nullptr, nullptr);
    }
    void update_snr(uint8_t modcod, float snr_db) { cusat_rx_pool_update_snr(p_, modcod, snr_db); }
    void set_copy_threads(int helpers) { ok(cusat_rx_pool_set_copy_threads(p_, helpers), "set_copy_threads"); }
    int max_output_bytes() const { return (int)stat(3); }
    uint64_t total_frame_count() const { return (uint64_t)stat(0); }
    uint64_t total_error_count() const { return (uint64_t)stat(1); }
    bool modcod_counters(uint8_t modcod, uint64_t& frames, uint64_t& errors) const
    {
        return cusat_rx_pool_modcod_counters(p_, modcod, &frames, &errors) == 1;
    }
    uint64_t total_gpu_drop_count() const { return (uint64_t)stat(2); }
    float data_snr_db() const { return (float)stat(4); }

  private:
    double stat(int i) const
    {
        double v[5];
        cusat_rx_pool_stats(p_, v);
        return v[i];
    }
    static int ok(int rc, const char* what)
    {
        if (rc < 0)
            cusat_shim::die(rc, what);
        return rc;
    }
    static void lock_mutex(void* m) { static_cast<std::mutex*>(m)->lock(); }
    static void unlock_mutex(void* m) { static_cast<std::mutex*>(m)->unlock(); }

    cusat_rx_pool* p_ = nullptr;
    std::vector<int> sizes_;
};

}  // namespace cusat_dsp
#endif  // pool
