// C ABI (include/cusat_fec.h) over the FEC kernels.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/cusat_fec.h"
#include "engine.h"

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace cusat {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace cusat

using namespace cusat_internal;

namespace {

// Decoder engine shared by the plain decoder and the receive chain.
struct Engine {
    const cusat::CodePlan* plan = nullptr;
    DevPlan dp;
    int max_trials = 0, max_batch = 0, device = 0;
    const void* fn = nullptr;
    int threads = 0, grid_max = 0;
    cusat::DecodeArgs proto{};
    uint4* msg = nullptr;
    unsigned int* queue = nullptr;
    DevWeights weights;
    int max_ctas = 0;                 // test hook: cap on the persistent grid (0 = none)
    cudaEvent_t last = nullptr;       // recorded after every launch
    bool launched = false;
    // Two frames per CTA (codes decoded one layer per step whose frame pair
    // fits twice per SM: the short frames): pair_fn decodes the frames of
    // the saturation-free path, then the one-frame kernel the frames it
    // listed.  nullptr: one-frame kernel only.
    const void* pair_fn = nullptr;
    cusat::DecodeArgs pair_layout{};  // its shared-memory carve-up and message stride
    int pair_grid_max = 0;
    int* list = nullptr;              // [max_batch] frames left to the one-frame kernel
    int pair_mode = 0;                // 0 by batch size, 1 one frame per CTA, 2 pairs when the code allows
    int sms = 0;

    int set_weights(const int16_t* w, int n_iter)
    {
        if (!w) {
            proto.code.weights = nullptr;
            return CUSAT_OK;
        }
        // a launch of this object still running reads the old table
        int rc = wait_last_launch(last, launched);
        if (rc)
            return rc;
        rc = weights.set(w, n_iter, max_trials);
        if (rc)
            return rc;
        proto.code.weights = weights.d;
        return CUSAT_OK;
    }

    int init(const cusat::CodePlan* p, int trials, int batch)
    {
        plan = p;
        max_trials = trials;
        max_batch = batch;
        int rc = require_device(&device);
        if (rc)
            return rc;
        rc = upload_plan(*p, &dp);
        if (rc)
            return rc;
        fn = cusat::select_decoder_kernel(p->cmax, p->lanes);
        if (!fn)
            return fail(CUSAT_ERR_UNSUPPORTED, "no decoder kernel for this check degree");
        threads = cusat::decoder_threads(p->lanes);
        memset(&proto, 0, sizeof(proto));
        proto.code = dp.code;
        proto.max_trials = max_trials;
        proto.syn_period = cusat::syndrome_period();
        cusat::decoder_smem_layout(&proto, cusat::smem_dims_of(proto.code, p->lanes));
        int optin = 0;
        CU(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "attr");
        CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attr");
        if (proto.sm_total > optin)
            return fail(CUSAT_ERR_UNSUPPORTED, "frame state does not fit in shared memory");
        CU(allow_full_smem(fn), "cudaFuncSetAttribute");
        int per_sm = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, proto.sm_total),
           "occupancy");
        if (per_sm < 1)
            return fail(CUSAT_ERR_UNSUPPORTED, "decoder kernel cannot be resident");
        // no launch runs more CTAs than frames: message scratch for at most
        // max_batch of them
        grid_max = per_sm * sms < batch ? per_sm * sms : batch;
        size_t msg_bytes = (size_t)grid_max * p->R * p->msg_row;
        if (p->lanes == 1) {
            const void* pf = cusat::select_pair_kernel(p->cmax);
            cusat::DecodeArgs pl{};
            cusat::pair_smem_layout(&pl, cusat::smem_dims_of(proto.code, 1), p->max_stage);
            int pair_per_sm = 0;
            if (pf && pl.sm_total <= optin) {
                CU(allow_full_smem(pf), "cudaFuncSetAttribute");
                CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pair_per_sm, pf, cusat::kPairThreads, pl.sm_total),
                   "occupancy");
            }
            // a frame pair pays when two of them are resident per SM
            if (pair_per_sm >= 2) {
                pair_fn = pf;
                pair_layout = pl;
                pair_layout.msg_stride = p->R * cusat::pair_msg_row(p->cmax) / 16;
                const int pairs = (batch + 1) / 2;
                pair_grid_max = pair_per_sm * sms < pairs ? pair_per_sm * sms : pairs;
                const size_t pair_bytes = (size_t)pair_grid_max * pair_layout.msg_stride * 16;
                if (pair_bytes > msg_bytes)
                    msg_bytes = pair_bytes;
                CU(cudaMalloc(&list, (size_t)batch * sizeof(int)), "cudaMalloc(frame list)");
            }
        }
        CU(cudaMalloc(&msg, msg_bytes), "cudaMalloc(messages)");
        CU(cudaMalloc(&queue, 256), "cudaMalloc(queue)");
        CU(cudaEventCreateWithFlags(&last, cudaEventDisableTiming), "cudaEventCreate");
        // frame/exit counters and the list length: the kernels rearm them
        CU(cudaMemset(queue, 0, 256), "cudaMemset(queue)");
        proto.msg = msg;
        proto.msg_stride = p->R * p->msg_row / 16;
        proto.queue = queue;
        return CUSAT_OK;
    }

    // Frames per CTA of a launch of `batch` frames.  By default pairs run
    // where they were measured faster on GB300: codes of at most 5
    // circulant slots per layer (16-43 % more throughput once the SMs are
    // busy), in launches whose pairs occupy at least three quarters of the
    // SMs (a smaller launch would leave SMs idle that single frames fill).
    // The wider short codes gain at most 13 % at four frames per SM and
    // lose up to 35 % elsewhere: one frame per CTA unless asked.
    int frames_per_cta(int batch) const
    {
        if (!pair_fn || proto.code.weights || pair_mode == 1)
            return 1;
        if (pair_mode == 2)
            return 2;
        return plan->cmax <= 5 && 4 * ((batch + 1) / 2) >= 3 * sms ? 2 : 1;
    }

    int launch(cusat::DecodeArgs a, int batch, cudaStream_t stream)
    {
        a.n_frames = batch;
        if (frames_per_cta(batch) == 2) {
            // frame pairs, then the one-frame kernel over the frames they
            // listed (usually none: its CTAs exit at once)
            cusat::DecodeArgs b = a;
            const cusat::DecodeArgs& l = pair_layout;
            b.sm_dummy = l.sm_dummy;
            b.sm_stage = l.sm_stage;
            b.sm_tab = l.sm_tab;
            b.sm_cnt = l.sm_cnt;
            b.sm_sched = l.sm_sched;
            b.sm_conf = l.sm_conf;
            b.sm_item_off = l.sm_item_off;
            b.sm_items = l.sm_items;
            b.sm_code = l.sm_code;
            b.sm_misc = l.sm_misc;
            b.sm_msgbuf = l.sm_msgbuf;
            b.sm_total = l.sm_total;
            b.max_stage = l.max_stage;
            b.msg_stride = l.msg_stride;
            b.list = list;
            b.list_count = queue + 4;
            int pgrid = (batch + 1) / 2 < pair_grid_max ? (batch + 1) / 2 : pair_grid_max;
            if (max_ctas > 0 && pgrid > max_ctas)
                pgrid = max_ctas;
            const int rc = cusat::launch_decoder(pair_fn, b, pgrid, cusat::kPairThreads, stream);
            if (rc != 0)
                return cuda_fail((cudaError_t)rc, "decoder launch (frame pairs)");
            a.list = list;
            a.list_count = queue + 4;
        }
        int grid = batch < grid_max ? batch : grid_max;
        if (max_ctas > 0 && grid > max_ctas)
            grid = max_ctas;
        const int rc = cusat::launch_decoder(fn, a, grid, threads, stream);
        if (rc != 0)
            return cuda_fail((cudaError_t)rc, "decoder launch");
        CU(cudaEventRecord(last, stream), "cudaEventRecord(last launch)");
        launched = true;
        return CUSAT_OK;
    }

    void release()
    {
        if (dp.blob)
            cudaFree(dp.blob);
        if (msg)
            cudaFree(msg);
        if (queue)
            cudaFree(queue);
        if (list)
            cudaFree(list);
        list = nullptr;
        weights.release();
        if (last)
            cudaEventDestroy(last);
        last = nullptr;
        dp.blob = nullptr;
        msg = nullptr;
        queue = nullptr;
    }
};

}  // namespace

struct cusat_ldpc_decoder {
    Engine eng;
    int16_t* soft_dev = nullptr;
    uint8_t* hard_pinned = nullptr;
    int32_t* trials_pinned = nullptr;
};

struct cusat_demapper {
    DevDemapObj dm;
    int max_batch = 0;
    float* sym_dev = nullptr;
    int16_t* soft_dev = nullptr;
    cudaStream_t stream = nullptr;
};

struct cusat_bch_checker {
    DevBch bch;
};

struct cusat_rx_fec {
    Engine eng;
    DevDemapObj dm;
    DevBch bch;
    int16_t* llr = nullptr;  // [max_batch][N] demapped LLRs
};

extern "C" {

const char* cusat_last_error(void) { return g_last_error.c_str(); }

// --------------------------------------------------------------------------
// LDPC decoder
// --------------------------------------------------------------------------

int cusat_ldpc_decoder_create(int framesize, int rate, int max_trials, int max_batch,
                              cusat_ldpc_decoder** out)
{
    if (!out || max_trials < 0 || max_trials > 1000 || max_batch <= 0)
        return fail(CUSAT_ERR_ARG, "invalid decoder arguments");
    *out = nullptr;
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    cusat_ldpc_decoder* d = new cusat_ldpc_decoder();
    int rc = d->eng.init(p, max_trials, max_batch);
    if (rc == CUSAT_OK) {
        cudaError_t e = cudaMalloc(&d->soft_dev, (size_t)max_batch * p->N * 2);
        if (e == cudaSuccess)
            e = cudaMallocHost(&d->hard_pinned, (size_t)max_batch * (p->K / 8));
        if (e == cudaSuccess)
            e = cudaMallocHost(&d->trials_pinned, (size_t)max_batch * 4);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "decoder buffers");
    }
    if (rc != CUSAT_OK) {
        cusat_ldpc_decoder_destroy(d);
        return rc;
    }
    *out = d;
    return CUSAT_OK;
}

void cusat_ldpc_decoder_destroy(cusat_ldpc_decoder* d)
{
    if (!d)
        return;
    d->eng.release();
    if (d->soft_dev)
        cudaFree(d->soft_dev);
    if (d->hard_pinned)
        cudaFreeHost(d->hard_pinned);
    if (d->trials_pinned)
        cudaFreeHost(d->trials_pinned);
    delete d;
}

int cusat_ldpc_decoder_set_weights(cusat_ldpc_decoder* d, const int16_t* weights, int n_iter)
{
    if (!d)
        return fail(CUSAT_ERR_ARG, "null decoder");
    return d->eng.set_weights(weights, n_iter);
}

int cusat_ldpc_decoder_set_max_ctas(cusat_ldpc_decoder* d, int max_ctas)
{
    if (!d || max_ctas < 0)
        return fail(CUSAT_ERR_ARG, "null decoder or negative CTA cap");
    d->eng.max_ctas = max_ctas;
    return CUSAT_OK;
}

int cusat_ldpc_decoder_set_frames_per_cta(cusat_ldpc_decoder* d, int n)
{
    if (!d || n < 0 || n > 2)
        return fail(CUSAT_ERR_ARG, "null decoder or frames per CTA outside 0..2");
    d->eng.pair_mode = n;
    return CUSAT_OK;
}

int cusat_ldpc_decoder_frames_per_cta(const cusat_ldpc_decoder* d, int batch)
{
    if (!d || batch <= 0)
        return fail(CUSAT_ERR_ARG, "null decoder or empty batch");
    return d->eng.frames_per_cta(batch);
}

int cusat_ldpc_decoder_info(const cusat_ldpc_decoder* d, int32_t* out)
{
    if (!d || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    const cusat::CodePlan* p = d->eng.plan;
    out[0] = p->N;
    out[1] = p->K;
    out[2] = p->K / 8;
    out[3] = p->q;
    out[4] = p->n_steps;
    out[5] = d->eng.max_trials;
    out[6] = d->eng.max_batch;
    out[7] = p->lanes;
    return CUSAT_OK;
}

int cusat_ldpc_decode_launch(cusat_ldpc_decoder* d, const int16_t* soft_dev, int batch, void* stream,
                             uint8_t* hard_out, int32_t* trials_out)
{
    if (!d || !soft_dev)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (batch <= 0 || batch > d->eng.max_batch)
        return fail(CUSAT_ERR_ARG, "batch outside 1..max_batch");
    cusat::DecodeArgs a = d->eng.proto;
    a.llr = soft_dev;
    a.hard = hard_out ? hard_out : d->hard_pinned;
    a.trials = trials_out ? trials_out : d->trials_pinned;
    return d->eng.launch(a, batch, (cudaStream_t)stream);
}

int cusat_ldpc_decode_batch(cusat_ldpc_decoder* d, const int16_t* soft_host, uint8_t* hard_host,
                            int32_t* trials_host, int batch, void* stream)
{
    if (!d || !soft_host || !hard_host || !trials_host)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (batch <= 0 || batch > d->eng.max_batch)
        return fail(CUSAT_ERR_ARG, "batch outside 1..max_batch");
    cudaStream_t s = (cudaStream_t)stream;
    const cusat::CodePlan* p = d->eng.plan;
    CU(cudaMemcpyAsync(d->soft_dev, soft_host, (size_t)batch * p->N * 2, cudaMemcpyHostToDevice, s),
       "cudaMemcpyAsync(llr)");
    int rc = cusat_ldpc_decode_launch(d, d->soft_dev, batch, stream, nullptr, nullptr);
    if (rc)
        return rc;
    CU(cudaStreamSynchronize(s), "decode");
    memcpy(hard_host, d->hard_pinned, (size_t)batch * (p->K / 8));
    memcpy(trials_host, d->trials_pinned, (size_t)batch * 4);
    return CUSAT_OK;
}

int cusat_ldpc_decode_batch_d2h(cusat_ldpc_decoder* d, const int16_t* soft_dev, uint8_t* hard_host,
                                int32_t* trials_host, int batch, void* stream)
{
    if (!d || !hard_host || !trials_host)
        return fail(CUSAT_ERR_ARG, "null argument");
    int rc = cusat_ldpc_decode_launch(d, soft_dev, batch, stream, nullptr, nullptr);
    if (rc)
        return rc;
    CU(cudaStreamSynchronize((cudaStream_t)stream), "decode");
    const cusat::CodePlan* p = d->eng.plan;
    memcpy(hard_host, d->hard_pinned, (size_t)batch * (p->K / 8));
    memcpy(trials_host, d->trials_pinned, (size_t)batch * 4);
    return CUSAT_OK;
}

int cusat_ldpc_decoder_results(const cusat_ldpc_decoder* d, uint8_t* hard_host, int32_t* trials_host,
                               int batch)
{
    if (!d || batch <= 0 || batch > d->eng.max_batch)
        return fail(CUSAT_ERR_ARG, "invalid arguments");
    const cusat::CodePlan* p = d->eng.plan;
    if (hard_host)
        memcpy(hard_host, d->hard_pinned, (size_t)batch * (p->K / 8));
    if (trials_host)
        memcpy(trials_host, d->trials_pinned, (size_t)batch * 4);
    return CUSAT_OK;
}

// --------------------------------------------------------------------------
// Demapper
// --------------------------------------------------------------------------

int cusat_demapper_create(int modulation, int rate, int framesize, int max_batch, cusat_demapper** out)
{
    if (!out || max_batch <= 0)
        return fail(CUSAT_ERR_ARG, "invalid demapper arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_demapper* d = new cusat_demapper();
    d->max_batch = max_batch;
    rc = d->dm.init(modulation, rate, framesize);
    if (rc == CUSAT_OK) {
        cudaError_t e = cudaMalloc(&d->sym_dev, (size_t)max_batch * d->dm.m.xfec * 8);
        if (e == cudaSuccess)
            e = cudaMalloc(&d->soft_dev, (size_t)max_batch * d->dm.m.fec_len * 2);
        if (e == cudaSuccess)
            e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "demapper buffers");
    }
    if (rc != CUSAT_OK) {
        cusat_demapper_destroy(d);
        return rc;
    }
    *out = d;
    return CUSAT_OK;
}

void cusat_demapper_destroy(cusat_demapper* d)
{
    if (!d)
        return;
    d->dm.release();
    if (d->sym_dev)
        cudaFree(d->sym_dev);
    if (d->soft_dev)
        cudaFree(d->soft_dev);
    if (d->stream)
        cudaStreamDestroy(d->stream);
    delete d;
}

int cusat_demapper_info(const cusat_demapper* d, int32_t* out)
{
    if (!d || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = d->dm.m.fec_len;
    out[1] = d->dm.m.xfec;
    out[2] = d->dm.m.n_mod;
    out[3] = d->dm.m.interleaved_len;
    return CUSAT_OK;
}

float cusat_demapper_capped_llr_gain(const cusat_demapper* d, float llr_gain)
{
    return d ? cusat::capped_llr_gain(d->dm.m, llr_gain) : llr_gain;
}

int16_t* cusat_demapper_soft_out_dev(const cusat_demapper* d) { return d ? d->soft_dev : nullptr; }

int cusat_demap_launch(cusat_demapper* d, const float* sym_dev, int batch, float noise_var, float llr_gain,
                       int16_t* soft_out_dev, void* stream)
{
    if (!d || !sym_dev)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (batch <= 0 || batch > d->max_batch)
        return fail(CUSAT_ERR_ARG, "batch outside 1..max_batch");
    const int rc = cusat::launch_demap(d->dm.d, sym_dev, batch, noise_var, llr_gain,
                                       soft_out_dev ? soft_out_dev : d->soft_dev, (cudaStream_t)stream);
    if (rc)
        return cuda_fail((cudaError_t)rc, "demap launch");
    return CUSAT_OK;
}

int cusat_demap_batch_async(cusat_demapper* d, const float* sym_host, int batch, float noise_var,
                            float llr_gain, void* stream)
{
    if (!d || !sym_host)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (batch <= 0 || batch > d->max_batch)
        return fail(CUSAT_ERR_ARG, "batch outside 1..max_batch");
    llr_gain = cusat::capped_llr_gain(d->dm.m, llr_gain);
    CU(cudaMemcpyAsync(d->sym_dev, sym_host, (size_t)batch * d->dm.m.xfec * 8, cudaMemcpyHostToDevice,
                       (cudaStream_t)stream),
       "cudaMemcpyAsync(symbols)");
    return cusat_demap_launch(d, d->sym_dev, batch, noise_var, llr_gain, nullptr, stream);
}

int cusat_demap_batch(cusat_demapper* d, const float* sym_host, int batch, float noise_var, float llr_gain)
{
    if (!d)
        return fail(CUSAT_ERR_ARG, "null argument");
    const int rc = cusat_demap_batch_async(d, sym_host, batch, noise_var, llr_gain, d->stream);
    if (rc)
        return rc;
    CU(cudaStreamSynchronize(d->stream), "demap");
    return CUSAT_OK;
}

// --------------------------------------------------------------------------
// BCH check
// --------------------------------------------------------------------------

int cusat_bch_checker_create(const uint64_t* flat_lut, const uint64_t* gen_poly, int gen_degree,
                             unsigned int n_bytes, cusat_bch_checker** out)
{
    if (!out || !flat_lut || !gen_poly)
        return fail(CUSAT_ERR_ARG, "null argument");
    *out = nullptr;
    if (gen_degree < 8 || gen_degree > 248 || (gen_degree & 7) || n_bytes <= (unsigned)(gen_degree / 8))
        return fail(CUSAT_ERR_ARG, "invalid BCH checker geometry");
    // the LUT must be the encoder table of this generator
    uint64_t lut[256 * 4];
    cusat::bch_encoder_lut(gen_poly, gen_degree, lut);
    for (int b = 0; b < 256; b++)
        for (int w = 0; w < (gen_degree + 63) / 64; w++)
            if (lut[b * 4 + w] != flat_lut[b * 4 + w])
                return fail(CUSAT_ERR_ARG, "BCH LUT does not match the generator");
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_bch_checker* c = new cusat_bch_checker();
    rc = c->bch.init(gen_poly, gen_degree, n_bytes);
    if (rc) {
        cusat_bch_checker_destroy(c);
        return rc;
    }
    *out = c;
    return CUSAT_OK;
}

int cusat_bch_checker_create_for_code(int framesize, int rate, cusat_bch_checker** out)
{
    if (!out)
        return fail(CUSAT_ERR_ARG, "null argument");
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    uint64_t lut[256 * 4];
    cusat::bch_encoder_lut(p->gen, p->p, lut);
    return cusat_bch_checker_create(lut, p->gen, p->p, (unsigned)(p->n_bch / 8), out);
}

void cusat_bch_checker_destroy(cusat_bch_checker* c)
{
    if (!c)
        return;
    c->bch.release();
    delete c;
}

unsigned int cusat_bch_checker_n_bytes(const cusat_bch_checker* c) { return c ? c->bch.t.n_bytes : 0; }

int cusat_bch_check_launch(cusat_bch_checker* c, const uint8_t* codewords_dev, int32_t* valid_out,
                           uint8_t* rem_out, int batch, void* stream)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (batch < 0)
        return fail(CUSAT_ERR_ARG, "negative BCH batch");
    if (batch == 0)
        return CUSAT_OK;
    if (!codewords_dev || (!valid_out && !rem_out))
        return fail(CUSAT_ERR_ARG, "null BCH checker buffer");
    const int rc = cusat::launch_bch_check(c->bch.d, codewords_dev, valid_out, rem_out, batch,
                                           (cudaStream_t)stream);
    if (rc)
        return cuda_fail((cudaError_t)rc, "BCH launch");
    return CUSAT_OK;
}

// --------------------------------------------------------------------------
// Receive chain: demap -> decode -> BCH
// --------------------------------------------------------------------------

int cusat_rx_fec_create(int modulation, int rate, int framesize, int max_trials, int max_batch,
                        cusat_rx_fec** out)
{
    if (!out || max_trials < 0 || max_trials > 1000 || max_batch <= 0)
        return fail(CUSAT_ERR_ARG, "invalid arguments");
    *out = nullptr;
    int dev;
    int rc0 = require_device(&dev);
    if (rc0)
        return rc0;
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    cusat_rx_fec* r = new cusat_rx_fec();
    int rc = r->dm.init(modulation, rate, framesize);
    if (rc == CUSAT_OK)
        rc = r->eng.init(p, max_trials, max_batch);
    if (rc == CUSAT_OK)
        rc = r->bch.init(p->gen, p->p, (unsigned)(p->n_bch / 8));
    if (rc == CUSAT_OK) {
        const cudaError_t e = cudaMalloc(&r->llr, (size_t)max_batch * p->N * sizeof(int16_t));
        if (e != cudaSuccess)
            rc = cuda_fail(e, "cudaMalloc(LLRs)");
    }
    if (rc != CUSAT_OK) {
        cusat_rx_fec_destroy(r);
        return rc;
    }
    *out = r;
    return CUSAT_OK;
}

void cusat_rx_fec_destroy(cusat_rx_fec* r)
{
    if (!r)
        return;
    r->eng.release();
    r->dm.release();
    r->bch.release();
    if (r->llr)
        cudaFree(r->llr);
    delete r;
}

int cusat_rx_fec_set_weights(cusat_rx_fec* r, const int16_t* weights, int n_iter)
{
    if (!r)
        return fail(CUSAT_ERR_ARG, "null chain");
    return r->eng.set_weights(weights, n_iter);
}

int cusat_rx_fec_set_frames_per_cta(cusat_rx_fec* r, int n)
{
    if (!r || n < 0 || n > 2)
        return fail(CUSAT_ERR_ARG, "null chain or frames per CTA outside 0..2");
    r->eng.pair_mode = n;
    return CUSAT_OK;
}

int cusat_rx_fec_info(const cusat_rx_fec* r, int32_t* out)
{
    if (!r || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    const cusat::CodePlan* p = r->eng.plan;
    out[0] = r->dm.m.xfec;
    out[1] = p->N;
    out[2] = p->K;
    out[3] = p->K / 8;
    out[4] = p->k_bch;
    out[5] = r->dm.m.n_mod;
    return CUSAT_OK;
}

float cusat_rx_fec_capped_llr_gain(const cusat_rx_fec* r, float llr_gain)
{
    return r ? cusat::capped_llr_gain(r->dm.m, llr_gain) : llr_gain;
}

int cusat_rx_fec_launch(cusat_rx_fec* r, const float* sym_dev, int batch, float noise_var, float llr_gain,
                        uint8_t* hard_out, int32_t* trials_out, int32_t* bch_valid_out, void* stream)
{
    if (!r || !sym_dev || !hard_out || !trials_out)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (batch <= 0 || batch > r->eng.max_batch)
        return fail(CUSAT_ERR_ARG, "batch outside 1..max_batch");
    // demap + deinterleave over the whole grid into HBM, then decode: the
    // decoder holds one frame per SM, and a demap inside it would run at one
    // CTA's memory parallelism
    const int e = cusat::launch_demap(r->dm.d, sym_dev, batch, noise_var, cusat::capped_llr_gain(r->dm.m, llr_gain),
                                      r->llr, (cudaStream_t)stream);
    if (e)
        return cuda_fail((cudaError_t)e, "demap launch");
    cusat::DecodeArgs a = r->eng.proto;
    a.llr = r->llr;
    a.hard = hard_out;
    a.trials = trials_out;
    int rc = r->eng.launch(a, batch, (cudaStream_t)stream);
    if (rc)
        return rc;
    if (bch_valid_out) {
        const int e = cusat::launch_bch_check(r->bch.d, hard_out, bch_valid_out, nullptr, batch,
                                              (cudaStream_t)stream);
        if (e)
            return cuda_fail((cudaError_t)e, "BCH launch");
    }
    return CUSAT_OK;
}

// --------------------------------------------------------------------------
// Code description and traffic generation (host side, not on the receive path)
// --------------------------------------------------------------------------

int cusat_code_info(int framesize, int rate, int32_t* out)
{
    if (!out)
        return fail(CUSAT_ERR_ARG, "null argument");
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    out[0] = p->N;
    out[1] = p->K;
    out[2] = p->k_bch;
    out[3] = p->n_bch;
    out[4] = p->t;
    out[5] = p->p;
    out[6] = p->q;
    out[7] = p->n_steps;
    out[8] = p->lanes;
    out[9] = p->cmax;
    out[10] = p->links_total;
    out[11] = p->cnt_max;
    return CUSAT_OK;
}

int cusat_gen_encode(int framesize, int rate, const uint8_t* msg, uint8_t* cw, int batch)
{
    if (!msg || !cw || batch < 0)
        return fail(CUSAT_ERR_ARG, "invalid arguments");
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    std::vector<uint8_t> bch((size_t)p->n_bch / 8);
    for (int f = 0; f < batch; f++) {
        cusat::bch_encode_frames(*p, msg + (size_t)f * (p->k_bch / 8), bch.data(), 1);
        cusat::ldpc_encode_frames(*p, bch.data(), cw + (size_t)f * (p->N / 8), 1);
    }
    return CUSAT_OK;
}

int cusat_ldpc_encode(int framesize, int rate, const uint8_t* info, uint8_t* cw, int batch)
{
    if (!info || !cw || batch < 0)
        return fail(CUSAT_ERR_ARG, "invalid arguments");
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    cusat::ldpc_encode_frames(*p, info, cw, batch);
    return CUSAT_OK;
}

int cusat_gen_map(int modulation, int rate, int framesize, const uint8_t* cw, int batch, float* sym)
{
    if (!cw || !sym || batch < 0)
        return fail(CUSAT_ERR_ARG, "invalid arguments");
    cusat::ModcodDemap m;
    std::string err;
    if (!cusat::build_modcod_demap(modulation, rate, framesize, &m, &err))
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    cusat::map_frames(m, cw, batch, sym);
    return CUSAT_OK;
}

int cusat_modcod_info(int modulation, int rate, int framesize, float* points, uint32_t* col, int32_t* out)
{
    cusat::ModcodDemap m;
    std::string err;
    if (!cusat::build_modcod_demap(modulation, rate, framesize, &m, &err))
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    if (points)
        memcpy(points, m.pts.data(), m.pts.size() * 4);
    if (col)
        memcpy(col, m.col, sizeof(m.col));
    if (out) {
        out[0] = m.n_mod;
        out[1] = m.n_points;
        out[2] = m.fec_len;
        out[3] = m.xfec;
        out[4] = m.interleaved_len;
        out[5] = m.kind;
    }
    return CUSAT_OK;
}

float cusat_modcod_capped_llr_gain(int modulation, int rate, int framesize, float llr_gain)
{
    cusat::ModcodDemap m;
    std::string err;
    if (!cusat::build_modcod_demap(modulation, rate, framesize, &m, &err))
        return llr_gain;
    return cusat::capped_llr_gain(m, llr_gain);
}

}  // extern "C"
