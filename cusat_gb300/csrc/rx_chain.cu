// Frame-at-a-time receive chain and its per-MODCOD pool: the reference's
// rx_fec_chain (lib/cusat_dsp/rx_fec_chain.cc:41-627) and rx_fec_pool
// (lib/cusat_dsp/rx_fec_pool.cc:15-270) with the same submit / drain / output
// semantics, over the receive-chain kernels of this library.
//
// Where the reference launches demap, LDPC and BCH per micro-batch on one of
// n streams, copies every frame's hard bits to pinned memory and descrambles
// and parses each BBFRAME on the host, a slot here is one H2D copy of its
// symbols, the demap and decode launches, the BCH check and the device-side
// BB stage, which writes only the packed GSE data fields, their lengths and
// the per-frame verdicts into the slot's pinned memory.  The host's drain is
// a counter update and one memcpy per slot.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/cusat_fec.h"
#include "copy_crew.h"
#include "engine.h"

using namespace cusat_internal;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kFlight = 128;     // flight ring slots (rx_fec_chain.h N_FLIGHT)
constexpr int kSnrPeriod = 32;   // frames between decision-directed SNR updates

struct BudgetState {
    std::atomic<int> in_flight{0};  // frames launched and not yet drained
    int cap = 0;                    // 0: unlimited
};

// One decode block per SM, CUSAT_LDPC_INFLIGHT_CAP overrides (0: no cap);
// gpu_decode_budget::make_default, rx_fec_chain.cc:21-39.
std::shared_ptr<BudgetState> default_budget()
{
    auto b = std::make_shared<BudgetState>();
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 0;
    b->cap = sms;
    if (const char* e = getenv("CUSAT_LDPC_INFLIGHT_CAP"))
        b->cap = atoi(e);
    return b;
}

using cusat_internal::CopyCrew;

void copy_frame(const std::shared_ptr<CopyCrew>& crew, void* dst, const void* src, size_t bytes)
{
    if (crew)
        crew->copy(dst, src, bytes);
    else
        memcpy(dst, src, bytes);
}

// Pinned per-slot state; the device writes results straight into it.
struct Slot {
    float* sym = nullptr;      // [micro_batch][xfec][2]
    int32_t* res = nullptr;    // trials[mb], bch_valid[mb], lengths[mb], offsets[mb + 1]
    uint8_t* out = nullptr;    // packed data fields, micro_batch * kbch bytes
    cudaEvent_t done = nullptr;
    bool in_flight = false;
    int stream = -1, n_frames = 0;
};

// One stream with its own receive chain and device buffers.
struct Lane {
    cusat_rx_fec* rx = nullptr;
    cudaStream_t stream = nullptr;
    float* sym_dev = nullptr;
    uint8_t* hard_dev = nullptr;
};

}  // namespace

struct cusat_decode_budget {
    std::shared_ptr<BudgetState> s;
};

struct cusat_rx_chain {
    int modulation = 0, rate = 0, framesize = 0;
    int micro_batch = 0, n_streams = 0;
    int xfec = 0, k_bytes = 0, kbch_bytes = 0, bits_per_sym = 0;
    std::vector<float> pts;  // constellation, for the SNR estimate
    cusat_bb_extractor* bb = nullptr;
    std::vector<Slot> flight;
    std::vector<Lane> lanes;
    int submit_idx = 0, launch_idx = 0, drain_idx = 0, next_stream = 0, batch_idx = 0;
    std::vector<uint8_t> output;
    int output_len = 0;
    std::vector<int32_t> dfl_sizes;
    float snr_db = 0.0f, pilot_snr_db = 0.0f, noise_var = 1.0f, llr_gain = 4.0f;
    uint64_t frames = 0, errors = 0, drops = 0, force_drains = 0;
    int snr_skip = 0;
    bool block_when_full = false;
    Clock::time_point batch_start{};
    std::shared_ptr<BudgetState> budget;
    void (*lock_fn)(void*) = nullptr;
    void (*unlock_fn)(void*) = nullptr;
    void* lock_ctx = nullptr;
    std::shared_ptr<CopyCrew> crew;  // frame copies split across helper threads, or none
    int failed = 0;  // first CUDA failure; the chain refuses work afterwards

    Slot& slot(int idx) { return flight[idx % kFlight]; }
    int32_t* trials(Slot& s) const { return s.res; }
    int32_t* valid(Slot& s) const { return s.res + micro_batch; }
    int32_t* lengths(Slot& s) const { return s.res + 2 * micro_batch; }
    int32_t* offsets(Slot& s) const { return s.res + 3 * micro_batch; }
};

namespace {

int chain_fail(cusat_rx_chain* c, int rc)
{
    if (!c->failed)
        c->failed = rc;
    return rc;
}

void release_budget(cusat_rx_chain* c, int n)
{
    if (c->budget)
        c->budget->in_flight.fetch_sub(n, std::memory_order_relaxed);
}

// rx_fec_chain::launch_slot_gpu (rx_fec_chain.cc:361-505): symbols up,
// demap + decode, BCH, BB stage, completion event; the noise variance and
// gain are the chain's at launch time.
int launch_slot(cusat_rx_chain* c, Slot& s)
{
    const int li = c->next_stream++ % c->n_streams;
    Lane& L = c->lanes[li];
    const int n = s.n_frames;
    if (c->lock_fn)
        c->lock_fn(c->lock_ctx);
    int rc = CUSAT_OK;
    cudaError_t e = cudaMemcpyAsync(L.sym_dev, s.sym, (size_t)n * c->xfec * 2 * sizeof(float),
                                    cudaMemcpyHostToDevice, L.stream);
    if (e != cudaSuccess)
        rc = cuda_fail(e, "symbol copy");
    if (rc == CUSAT_OK)
        rc = cusat_rx_fec_launch(L.rx, L.sym_dev, n, c->noise_var, c->llr_gain, L.hard_dev, c->trials(s),
                                 c->valid(s), L.stream);
    if (rc == CUSAT_OK)
        rc = cusat_bb_extract(c->bb, L.hard_dev, c->k_bytes, c->trials(s), c->valid(s), n, s.out,
                              n * c->kbch_bytes, c->lengths(s), c->offsets(s), L.stream);
    if (rc == CUSAT_OK) {
        e = cudaEventRecord(s.done, L.stream);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "event record");
    }
    if (c->unlock_fn)
        c->unlock_fn(c->lock_ctx);
    if (rc)
        return chain_fail(c, rc);
    s.in_flight = true;
    s.stream = li;
    return CUSAT_OK;
}

// pump_launches (rx_fec_chain.cc:507-525): launch ready slots in order while
// the shared budget allows; an empty GPU always admits one.
int pump(cusat_rx_chain* c, bool bypass_cap)
{
    while (c->launch_idx < c->submit_idx) {
        Slot& s = c->slot(c->launch_idx);
        BudgetState* b = c->budget.get();
        if (!bypass_cap && b && b->cap > 0) {
            const int cur = b->in_flight.load(std::memory_order_relaxed);
            if (cur > 0 && cur + s.n_frames > b->cap)
                break;
        }
        if (b)
            b->in_flight.fetch_add(s.n_frames, std::memory_order_relaxed);
        const int rc = launch_slot(c, s);
        if (rc) {
            release_budget(c, s.n_frames);
            return rc;
        }
        c->launch_idx++;
    }
    return CUSAT_OK;
}

// post_process_slot (rx_fec_chain.cc:574-625): count the frames, keep the
// data fields of those that converged and passed BCH (the device already
// dropped the rest and packed the survivors in frame order).
void post_process(cusat_rx_chain* c, Slot& s)
{
    const int n = s.n_frames;
    const int32_t* tr = c->trials(s);
    const int32_t* va = c->valid(s);
    const int32_t* len = c->lengths(s);
    for (int i = 0; i < n; i++) {
        c->frames++;
        if (!(tr[i] >= 0 && va[i])) {
            c->errors++;
            continue;
        }
        if (len[i] > 0)
            c->dfl_sizes.push_back(len[i]);
    }
    const int bytes = c->offsets(s)[n];
    if (bytes > 0) {
        memcpy(c->output.data() + c->output_len, s.out, (size_t)bytes);
        c->output_len += bytes;
    }
}

void retire(cusat_rx_chain* c, Slot& s)
{
    post_process(c, s);
    s.in_flight = false;
    release_budget(c, s.n_frames);
    c->drain_idx++;
}

// drain_completed without clearing the output (rx_fec_chain.cc:237-260):
// completed slots in order, stopping at the first one still running.
int drain(cusat_rx_chain* c)
{
    int any = 0;
    while (c->drain_idx < c->launch_idx) {
        Slot& s = c->slot(c->drain_idx);
        if (!s.in_flight) {
            c->drain_idx++;
            continue;
        }
        const cudaError_t e = cudaEventQuery(s.done);
        if (e == cudaErrorNotReady)
            break;
        if (e != cudaSuccess)
            return chain_fail(c, cuda_fail(e, "decode slot"));
        retire(c, s);
        any = 1;
    }
    const int rc = pump(c, false);
    return rc ? rc : any;
}

// force_drain_oldest (rx_fec_chain.cc:532-572): launch the oldest slot even
// past the budget if it is still waiting, then wait for it.
int force_drain_oldest(cusat_rx_chain* c)
{
    if (c->drain_idx >= c->launch_idx && c->drain_idx < c->submit_idx) {
        const int rc = pump(c, true);
        if (rc)
            return rc;
    }
    Slot& s = c->slot(c->drain_idx);
    if (!s.in_flight) {
        c->drain_idx++;
        return CUSAT_OK;
    }
    c->force_drains++;
    const cudaError_t e = cudaEventSynchronize(s.done);
    if (e != cudaSuccess)
        return chain_fail(c, cuda_fail(e, "decode slot"));
    retire(c, s);
    return CUSAT_OK;
}

int launch_partial(cusat_rx_chain* c)
{
    if (c->batch_idx > 0) {
        c->slot(c->submit_idx).n_frames = c->batch_idx;
        c->submit_idx++;
        c->batch_idx = 0;
    }
    return pump(c, false);
}

int flush(cusat_rx_chain* c)
{
    c->output_len = 0;
    c->dfl_sizes.clear();
    int rc = launch_partial(c);
    while (rc == CUSAT_OK && c->drain_idx < c->submit_idx)
        rc = force_drain_oldest(c);
    return rc;
}

// The SNR the demapper scales by, every kSnrPeriod submitted frames
// (rx_fec_chain.cc:322-342): pilot SNR for 128-point and larger
// constellations when one is known, else decision-directed on this frame.
void estimate_snr(cusat_rx_chain* c, const float* sym, int n_sym)
{
    float lin;
    if (c->bits_per_sym >= 7 && c->pilot_snr_db > 5.0f)
        lin = std::pow(10.0f, c->pilot_snr_db / 10.0f);
    else if (c->modulation == 0)
        lin = cusat::dd_snr_qpsk(sym, n_sym);
    else
        lin = cusat::dd_snr_points(c->pts, sym, n_sym, 8);
    if (lin > 1.0f) {
        c->snr_db = 10.0f * std::log10(lin);
        c->noise_var = 1.0f / lin;
        c->llr_gain = std::min(4.0f / c->noise_var, 1000.0f);
    }
}

void chain_free(cusat_rx_chain* c)
{
    for (Lane& L : c->lanes) {
        if (L.stream)
            cudaStreamSynchronize(L.stream);
        cusat_rx_fec_destroy(L.rx);
        if (L.sym_dev)
            cudaFree(L.sym_dev);
        if (L.hard_dev)
            cudaFree(L.hard_dev);
        if (L.stream)
            cudaStreamDestroy(L.stream);
    }
    for (Slot& s : c->flight) {
        if (s.sym)
            cudaFreeHost(s.sym);
        if (s.res)
            cudaFreeHost(s.res);
        if (s.out)
            cudaFreeHost(s.out);
        if (s.done)
            cudaEventDestroy(s.done);
    }
    cusat_bb_extractor_destroy(c->bb);
    delete c;
}

}  // namespace

extern "C" {

int cusat_dd_snr(int modulation, int rate, int framesize, const float* sym, int n_sym, int stride, float* out)
{
    if (!sym || !out || n_sym < 0 || stride <= 0)
        return fail(CUSAT_ERR_ARG, "invalid arguments");
    if (modulation == 0) {
        *out = cusat::dd_snr_qpsk(sym, n_sym);
        return CUSAT_OK;
    }
    std::vector<float> pts;
    if (cusat::make_constellation(modulation, rate, framesize, &pts) <= 0)
        return fail(CUSAT_ERR_UNSUPPORTED, "constellation");
    *out = cusat::dd_snr_points(pts, sym, n_sym, stride);
    return CUSAT_OK;
}

int cusat_decode_budget_create(int cap, cusat_decode_budget** out)
{
    if (!out)
        return fail(CUSAT_ERR_ARG, "null argument");
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_decode_budget* b = new cusat_decode_budget();
    if (cap < 0) {
        b->s = default_budget();
    } else {
        b->s = std::make_shared<BudgetState>();
        b->s->cap = cap;
    }
    *out = b;
    return CUSAT_OK;
}

void cusat_decode_budget_destroy(cusat_decode_budget* b) { delete b; }

int cusat_decode_budget_info(const cusat_decode_budget* b, int32_t* out)
{
    if (!b || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = b->s->cap;
    out[1] = b->s->in_flight.load(std::memory_order_relaxed);
    return CUSAT_OK;
}

int cusat_rx_chain_create(int framesize, int rate, int modulation, int max_trials, int cuda_max_batch,
                          int n_gpu_streams, int micro_batch, cusat_rx_chain** out)
{
    (void)cuda_max_batch;  // the reference's per-chain decoder sizing; slots size by micro_batch
    if (!out || max_trials < 0 || max_trials > 1000 || n_gpu_streams <= 0 || n_gpu_streams > 64 ||
        micro_batch <= 0 || micro_batch > 4096)
        return fail(CUSAT_ERR_ARG, "invalid chain arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_rx_chain* c = new cusat_rx_chain();
    c->modulation = modulation;
    c->rate = rate;
    c->framesize = framesize;
    c->micro_batch = micro_batch;
    // Launches on one stream run one after another, so n_gpu_streams
    // micro-batches of micro_batch frames bound the frames in flight (32 at
    // the reference's defaults, against 152 SMs).  The in-flight budget is
    // what bounds residency: enough streams to fill the default budget (one
    // frame per SM), never fewer than asked for.
    {
        const int cap = default_budget()->cap;
        const int fill = cap > 0 ? (cap + micro_batch - 1) / micro_batch : n_gpu_streams;
        c->n_streams = std::min(64, std::max(n_gpu_streams, fill));
    }
    c->lanes.resize(c->n_streams);
    c->flight.resize(kFlight);
    int32_t info[6];
    for (Lane& L : c->lanes) {
        rc = cusat_rx_fec_create(modulation, rate, framesize, max_trials, micro_batch, &L.rx);
        if (rc)
            break;
    }
    if (rc == CUSAT_OK)
        rc = cusat_rx_fec_info(c->lanes[0].rx, info);
    if (rc == CUSAT_OK)
        rc = cusat_bb_extractor_create(framesize, rate, &c->bb);
    if (rc == CUSAT_OK) {
        c->xfec = info[0];
        c->k_bytes = info[3];
        c->kbch_bytes = info[4] / 8;
        c->bits_per_sym = cusat::make_constellation(modulation, rate, framesize, &c->pts);
        if (c->bits_per_sym <= 0)
            rc = fail(CUSAT_ERR_UNSUPPORTED, "constellation");
    }
    int lo = 0, hi = 0;
    if (rc == CUSAT_OK && cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess)
        lo = 0;
    const size_t sym_bytes = (size_t)micro_batch * c->xfec * 2 * sizeof(float);
    for (size_t i = 0; rc == CUSAT_OK && i < c->lanes.size(); i++) {
        Lane& L = c->lanes[i];
        cudaError_t e = cudaStreamCreateWithPriority(&L.stream, cudaStreamNonBlocking, lo);
        if (e == cudaSuccess)
            e = cudaMalloc(&L.sym_dev, sym_bytes);
        if (e == cudaSuccess)
            e = cudaMalloc(&L.hard_dev, (size_t)micro_batch * c->k_bytes);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "chain stream buffers");
    }
    for (size_t i = 0; rc == CUSAT_OK && i < c->flight.size(); i++) {
        Slot& s = c->flight[i];
        cudaError_t e = cudaMallocHost(&s.sym, sym_bytes);
        if (e == cudaSuccess)
            e = cudaMallocHost(&s.res, (size_t)(4 * micro_batch + 1) * sizeof(int32_t));
        if (e == cudaSuccess)
            e = cudaMallocHost(&s.out, (size_t)micro_batch * c->kbch_bytes);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "flight slot");
    }
    if (rc != CUSAT_OK) {
        chain_free(c);
        return rc;
    }
    c->budget = default_budget();
    c->output.resize((size_t)c->kbch_bytes * kFlight * micro_batch);
    *out = c;
    return CUSAT_OK;
}

void cusat_rx_chain_destroy(cusat_rx_chain* c)
{
    if (!c)
        return;
    // frames in flight are abandoned; give back their budget
    for (int i = c->drain_idx; i < c->launch_idx; i++)
        if (c->slot(i).in_flight)
            release_budget(c, c->slot(i).n_frames);
    chain_free(c);
}

int cusat_rx_chain_info(const cusat_rx_chain* c, int32_t* out)
{
    if (!c || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = c->xfec;
    out[1] = c->kbch_bytes;
    out[2] = c->micro_batch * kFlight;                  // batch_size()
    out[3] = c->kbch_bytes * c->micro_batch * kFlight;  // max_output_bytes()
    out[4] = c->micro_batch;
    out[5] = c->n_streams;
    return CUSAT_OK;
}

int cusat_rx_chain_set_weights(cusat_rx_chain* c, const int16_t* weights, int n_iter)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    for (Lane& L : c->lanes) {
        const int rc = cusat_rx_fec_set_weights(L.rx, weights, n_iter);
        if (rc)
            return rc;
    }
    return CUSAT_OK;
}

int cusat_rx_chain_set_decode_budget(cusat_rx_chain* c, const cusat_decode_budget* b)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    if (b)
        c->budget = b->s;
    return CUSAT_OK;
}

int cusat_rx_chain_set_launch_lock(cusat_rx_chain* c, void (*lock)(void*), void (*unlock)(void*), void* ctx)
{
    if (!c || (!lock) != (!unlock))
        return fail(CUSAT_ERR_ARG, "lock and unlock go together");
    c->lock_fn = lock;
    c->unlock_fn = unlock;
    c->lock_ctx = ctx;
    return CUSAT_OK;
}

int cusat_rx_chain_set_copy_threads(cusat_rx_chain* c, int helpers)
{
    if (!c || helpers < 0 || helpers > 32)
        return fail(CUSAT_ERR_ARG, "invalid copy thread count");
    c->crew = helpers ? std::make_shared<CopyCrew>(helpers) : nullptr;
    return CUSAT_OK;
}

void cusat_rx_chain_set_block_when_full(cusat_rx_chain* c, int on)
{
    if (c)
        c->block_when_full = on != 0;
}

void cusat_rx_chain_update_snr(cusat_rx_chain* c, float snr_db)
{
    if (!c || !(snr_db > 0.0f))
        return;
    const float lin = std::pow(10.0f, snr_db / 10.0f);
    c->pilot_snr_db = snr_db;
    c->snr_db = snr_db;
    c->noise_var = 1.0f / lin;
    c->llr_gain = std::min(4.0f / c->noise_var, 1000.0f);
}

// rx_fec_chain::submit_gpu (rx_fec_chain.cc:268-359)
int cusat_rx_chain_submit_xfecframe(cusat_rx_chain* c, const float* symbols, int n_symbols)
{
    if (!c || (!symbols && n_symbols > 0))
        return fail(CUSAT_ERR_ARG, "null argument");
    if (c->failed)
        return c->failed;
    int ready = 0;
    if (c->batch_idx == 0 || c->submit_idx - c->drain_idx >= kFlight / 2) {
        c->output_len = 0;
        c->dfl_sizes.clear();
        const int rc = drain(c);
        if (rc < 0)
            return rc;
        ready = rc;
    }
    while (c->block_when_full && c->submit_idx - c->drain_idx >= kFlight - 2) {
        const int rc = force_drain_oldest(c);
        if (rc)
            return rc;
        ready = 1;
    }
    if (c->submit_idx - c->drain_idx >= kFlight - 2 || n_symbols != c->xfec) {
        // ring full (real-time drop) or a frame of the wrong length
        c->drops++;
        c->frames++;
        c->errors++;
        return ready;
    }
    Slot& s = c->slot(c->submit_idx);
    float* dest = s.sym + (size_t)c->batch_idx * c->xfec * 2;
    copy_frame(c->crew, dest, symbols, (size_t)n_symbols * 2 * sizeof(float));
    if (++c->snr_skip >= kSnrPeriod) {
        c->snr_skip = 0;
        estimate_snr(c, dest, n_symbols);
    }
    if (c->batch_idx == 0)
        c->batch_start = Clock::now();
    if (++c->batch_idx >= c->micro_batch) {
        s.n_frames = c->batch_idx;
        c->submit_idx++;
        c->batch_idx = 0;
        const int rc = pump(c, false);
        if (rc)
            return rc;
    }
    return ready;
}

int cusat_rx_chain_drain_completed(cusat_rx_chain* c)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    if (c->failed)
        return c->failed;
    c->output_len = 0;
    c->dfl_sizes.clear();
    return drain(c);
}

int cusat_rx_chain_get_gse_output(cusat_rx_chain* c, uint8_t* out, int max_bytes)
{
    if (!c || (!out && max_bytes > 0) || max_bytes < 0)
        return fail(CUSAT_ERR_ARG, "invalid output buffer");
    const int n = std::min(c->output_len, max_bytes);
    if (n > 0)
        memcpy(out, c->output.data(), (size_t)n);
    c->output_len = 0;
    return n;
}

int cusat_rx_chain_gse_dfl_sizes(const cusat_rx_chain* c, int32_t* out, int max)
{
    if (!c || (!out && max > 0))
        return fail(CUSAT_ERR_ARG, "null argument");
    const int n = (int)c->dfl_sizes.size();
    if (out)
        memcpy(out, c->dfl_sizes.data(), sizeof(int32_t) * (size_t)std::min(n, max));
    return n;
}

int cusat_rx_chain_launch_partial(cusat_rx_chain* c)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    if (c->failed)
        return c->failed;
    return launch_partial(c);
}

int cusat_rx_chain_flush(cusat_rx_chain* c)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    if (c->failed)
        return c->failed;
    return flush(c);
}

// rx_fec_chain::reset (rx_fec_chain.cc:175-206)
int cusat_rx_chain_reset(cusat_rx_chain* c)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    int rc = CUSAT_OK;
    if (c->lock_fn)
        c->lock_fn(c->lock_ctx);
    while (c->drain_idx < c->submit_idx) {
        Slot& s = c->slot(c->drain_idx);
        if (s.in_flight) {
            const cudaError_t e = cudaEventSynchronize(s.done);
            if (e != cudaSuccess && rc == CUSAT_OK)
                rc = cuda_fail(e, "decode slot");
            release_budget(c, s.n_frames);
        }
        s.in_flight = false;
        s.stream = -1;
        s.n_frames = 0;
        c->drain_idx++;
    }
    if (c->unlock_fn)
        c->unlock_fn(c->lock_ctx);
    c->submit_idx = c->launch_idx = c->drain_idx = 0;
    c->next_stream = 0;
    c->batch_idx = 0;
    c->output_len = 0;
    c->snr_db = 0.0f;
    c->noise_var = 1.0f;
    c->llr_gain = 4.0f;
    c->frames = 0;
    c->errors = 0;
    c->dfl_sizes.clear();
    return rc ? chain_fail(c, rc) : CUSAT_OK;
}

// rx_fec_chain::warmup (rx_fec_chain.cc:218-232): one all-zero frame through
// the whole path, then a clean state.
int cusat_rx_chain_warmup(cusat_rx_chain* c)
{
    if (!c)
        return fail(CUSAT_ERR_ARG, "null chain");
    std::vector<float> zeros((size_t)c->xfec * 2, 0.0f);
    int rc = cusat_rx_chain_submit_xfecframe(c, zeros.data(), c->xfec);
    if (rc >= 0)
        rc = cusat_rx_chain_launch_partial(c);
    if (rc >= 0)
        rc = cusat_rx_chain_flush(c);
    if (rc >= 0)
        rc = cusat_rx_chain_reset(c);
    c->force_drains = 0;
    c->drops = 0;
    return rc < 0 ? rc : CUSAT_OK;
}

int cusat_rx_chain_stats(const cusat_rx_chain* c, double* out)
{
    if (!c || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = (double)c->frames;
    out[1] = (double)c->errors;
    out[2] = (double)c->drops;
    out[3] = (double)(c->launch_idx - c->drain_idx);  // gpu_inflight (slots)
    out[4] = (double)(c->submit_idx - c->launch_idx);  // gpu_pending_launch
    out[5] = (double)c->force_drains;
    out[6] = (double)c->batch_idx;                     // pending_count
    out[7] = (double)c->snr_db;
    out[8] = (double)c->llr_gain;                      // precision()
    out[9] = (double)c->noise_var;
    out[10] = c->batch_idx > 0
                  ? std::chrono::duration<double>(Clock::now() - c->batch_start).count()
                  : 0.0;                               // age of the partial micro-batch, s
    out[11] = (double)c->output_len;
    return CUSAT_OK;
}

}  // extern "C"

// --------------------------------------------------------------------------
// Pool: one chain per MODCOD (rx_fec_pool.cc)
// --------------------------------------------------------------------------

namespace {

struct PoolEntry {
    int modcod = 0;
    cusat_rx_chain* chain = nullptr;
};

struct Block {
    std::vector<uint8_t> bytes;
    std::vector<int32_t> dfl;
    int modcod = 0;
};

}  // namespace

// Mixed pool: one slot ring for every MODCOD, each slot one multi-MODCOD
// launch (cusat_batch) -- no flush at a MODCOD change.  The reference's
// per-MODCOD micro-batches survive as "virtual" ones: they decide when a
// frame's LLR gain is fixed (the MODCOD's gain when its micro-batch closes:
// full, MODCOD change, stale, flush), which is the gain the reference's chain
// launches it with; a slot launches once all its frames' gains are fixed.
namespace {

struct MixModcod {
    int idx = 0, mod = 0, rate = 0;
    int xfec = 0, k_bytes = 0, kbch_bytes = 0, bits_per_sym = 0;
    std::vector<float> pts;
    float snr_db = 0.0f, pilot_snr_db = 0.0f, noise_var = 1.0f, llr_gain = 4.0f;
    int snr_skip = 0;
    uint64_t frames = 0, errors = 0, drops = 0;
};

struct MixSlot {
    float* sym = nullptr;    // pinned [slot_frames][max_xfec][2]
    int32_t* res = nullptr;  // pinned: trials, valid, lengths, kbch [slot_frames each], offsets [slot_frames + 1]
    uint8_t* out = nullptr;  // pinned: packed data fields
    cudaEvent_t done = nullptr;
    std::vector<int> modcod;  // per frame: index into MixPool::mc
    std::vector<float> noise_var, llr_gain;
    int n_frames = 0, open = 0;  // frames; frames whose gain is not fixed yet
    bool in_flight = false;
};

struct MixLane {
    cusat_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;  // the lane's last launch (its batch staging is reusable after it)
    bool used = false;
    float* sym_dev = nullptr;
    uint8_t* hard_dev = nullptr;
    std::vector<cusat_frame> frames;
};

struct MixPool {
    std::vector<MixModcod> mc;
    int slot_frames = 0, micro_batch = 0, max_xfec = 0, max_kbytes = 0, max_kbch = 0;
    cusat_bb_extractor* bb = nullptr;
    std::vector<MixSlot> flight;
    std::vector<MixLane> lanes;
    int submit_idx = 0, launch_idx = 0, drain_idx = 0, next_lane = 0, fill = 0;
    int open_mc = -1;                          // MODCOD of the open virtual micro-batch
    std::vector<std::pair<int, int>> open_at;  // its frames: (slot submit index, frame)
    Clock::time_point open_start{};            // its first frame's submission
    Clock::time_point slot_start{};            // the current slot's first frame's submission
    std::shared_ptr<BudgetState> budget;
    void (*lock_fn)(void*) = nullptr;
    void (*unlock_fn)(void*) = nullptr;
    void* lock_ctx = nullptr;
    std::shared_ptr<CopyCrew> crew;
    int failed = 0;

    MixSlot& slot(int i) { return flight[i % kFlight]; }
    int32_t* trials(MixSlot& t) const { return t.res; }
    int32_t* valid(MixSlot& t) const { return t.res + slot_frames; }
    int32_t* lengths(MixSlot& t) const { return t.res + 2 * slot_frames; }
    int32_t* kbch(MixSlot& t) const { return t.res + 3 * slot_frames; }
    int32_t* offsets(MixSlot& t) const { return t.res + 4 * slot_frames; }
    int find(int modcod) const
    {
        for (size_t i = 0; i < mc.size(); i++)
            if (mc[i].idx == modcod)
                return (int)i;
        return -1;
    }
};

}  // namespace

struct cusat_rx_pool {
    std::unique_ptr<MixPool> mix;   // mixed mode, else one chain per MODCOD
    std::vector<PoolEntry> chains;  // creation order: drains and flushes visit them in it
    int last_decoded = 0, last_submitted = 0;
    bool has_prev = false;
    int max_output_bytes = 0;
    std::deque<Block> ready;
    std::vector<Block> spare;
    std::vector<int32_t> last_sizes;
    cusat_decode_budget budget;

    cusat_rx_chain* find(int modcod)
    {
        for (PoolEntry& e : chains)
            if (e.modcod == modcod)
                return e.chain;
        return nullptr;
    }
};

namespace {

// harvest_output (rx_fec_pool.cc:120-146): move one chain's output into the
// pool's FIFO right away, before another poll of it clears it.
int harvest(cusat_rx_pool* p, int modcod)
{
    cusat_rx_chain* c = p->find(modcod);
    if (!c || c->output_len <= 0) {
        if (c)
            c->output_len = 0;
        return 0;
    }
    Block b;
    if (!p->spare.empty()) {
        b = std::move(p->spare.back());
        p->spare.pop_back();
    }
    b.bytes.assign(c->output.begin(), c->output.begin() + c->output_len);
    b.dfl = c->dfl_sizes;
    b.modcod = modcod;
    c->output_len = 0;
    p->ready.push_back(std::move(b));
    return 1;
}

void clear_ready(cusat_rx_pool* p)
{
    while (!p->ready.empty()) {
        Block b = std::move(p->ready.front());
        p->ready.pop_front();
        b.bytes.clear();
        b.dfl.clear();
        p->spare.push_back(std::move(b));
    }
    p->last_sizes.clear();
}


// ---- mixed pool ----

int mix_fail(MixPool& x, int rc)
{
    if (!x.failed)
        x.failed = rc;
    return rc;
}

// Fixes the gain of the open virtual micro-batch's frames: its MODCOD's
// current N0 and gain (what the reference's chain launches it with).
void mix_close(MixPool& x)
{
    if (x.open_mc >= 0) {
        const MixModcod& m = x.mc[x.open_mc];
        for (const auto& at : x.open_at) {
            MixSlot& t = x.slot(at.first);
            t.noise_var[at.second] = m.noise_var;
            t.llr_gain[at.second] = m.llr_gain;
            t.open--;
        }
    }
    x.open_at.clear();
    x.open_mc = -1;
}

void mix_estimate_snr(MixModcod& m, const float* sym, int n_sym)
{
    float lin;
    if (m.bits_per_sym >= 7 && m.pilot_snr_db > 5.0f)
        lin = std::pow(10.0f, m.pilot_snr_db / 10.0f);
    else if (m.mod == 0)
        lin = cusat::dd_snr_qpsk(sym, n_sym);
    else
        lin = cusat::dd_snr_points(m.pts, sym, n_sym, 8);
    if (lin > 1.0f) {
        m.snr_db = 10.0f * std::log10(lin);
        m.noise_var = 1.0f / lin;
        m.llr_gain = std::min(4.0f / m.noise_var, 1000.0f);
    }
}

// One slot: symbols up, the multi-MODCOD launch (demap -> per-class
// decoders -> BCH), the per-frame-code BB stage into the slot's pinned
// memory, completion event.
int mix_launch(MixPool& x, MixSlot& t)
{
    const int li = x.next_lane++ % (int)x.lanes.size();
    MixLane& L = x.lanes[li];
    const int n = t.n_frames;
    if (x.lock_fn)
        x.lock_fn(x.lock_ctx);
    int rc = CUSAT_OK;
    cudaError_t e = cudaSuccess;
    if (L.used)
        e = cudaEventSynchronize(L.done);  // the lane's batch descriptors are staged again below
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(L.sym_dev, t.sym, (size_t)n * x.max_xfec * 2 * sizeof(float), cudaMemcpyHostToDevice,
                            L.stream);
    if (e != cudaSuccess)
        rc = cuda_fail(e, "symbol copy");
    for (int k = 0; rc == CUSAT_OK && k < n; k++) {
        const MixModcod& m = x.mc[t.modcod[k]];
        x.kbch(t)[k] = m.kbch_bytes;
        cusat_frame& f = L.frames[k];
        f.modcod = t.modcod[k];
        f.noise_var = t.noise_var[k];
        f.llr_gain = t.llr_gain[k];
        f.reserved = 0;
        f.sym = L.sym_dev + (size_t)k * x.max_xfec * 2;
        f.hard = L.hard_dev + (size_t)k * x.max_kbytes;
        f.trials = x.trials(t) + k;
        f.bch_valid = x.valid(t) + k;
    }
    if (rc == CUSAT_OK)
        rc = batch_launch_ready(L.batch, L.frames.data(), n, L.stream);
    if (rc == CUSAT_OK)
        rc = cusat_bb_extract_frames(x.bb, L.hard_dev, x.max_kbytes, x.kbch(t), x.trials(t), x.valid(t), n, t.out,
                                     n * x.max_kbch, x.lengths(t), x.offsets(t), L.stream);
    if (rc == CUSAT_OK) {
        e = cudaEventRecord(t.done, L.stream);
        if (e == cudaSuccess)
            e = cudaEventRecord(L.done, L.stream);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "event record");
    }
    if (x.unlock_fn)
        x.unlock_fn(x.lock_ctx);
    if (rc)
        return mix_fail(x, rc);
    L.used = true;
    t.in_flight = true;
    return CUSAT_OK;
}

// Launches ready slots in order: full (or flushed), every gain fixed, and
// within the in-flight budget (an empty GPU always admits one).
int mix_pump(MixPool& x, bool bypass_cap)
{
    while (x.launch_idx < x.submit_idx) {
        MixSlot& t = x.slot(x.launch_idx);
        if (t.open > 0)
            break;
        BudgetState* b = x.budget.get();
        if (!bypass_cap && b && b->cap > 0) {
            const int cur = b->in_flight.load(std::memory_order_relaxed);
            if (cur > 0 && cur + t.n_frames > b->cap)
                break;
        }
        if (b)
            b->in_flight.fetch_add(t.n_frames, std::memory_order_relaxed);
        const int rc = mix_launch(x, t);
        if (rc) {
            if (b)
                b->in_flight.fetch_sub(t.n_frames, std::memory_order_relaxed);
            return rc;
        }
        x.launch_idx++;
    }
    return CUSAT_OK;
}

// Counts a completed slot's frames per MODCOD and moves its output into the
// FIFO as one block per run of same-MODCOD frames (a block belongs to one
// MODCOD, as the reference pool's blocks do).
void mix_retire(cusat_rx_pool* p, MixSlot& t)
{
    MixPool& x = *p->mix;
    const int n = t.n_frames;
    const int32_t* tr = x.trials(t);
    const int32_t* va = x.valid(t);
    const int32_t* len = x.lengths(t);
    const int32_t* off = x.offsets(t);
    for (int k0 = 0; k0 < n;) {
        int k1 = k0;
        while (k1 < n && t.modcod[k1] == t.modcod[k0])
            k1++;
        MixModcod& m = x.mc[t.modcod[k0]];
        Block b;
        if (!p->spare.empty()) {
            b = std::move(p->spare.back());
            p->spare.pop_back();
        }
        b.bytes.clear();
        b.dfl.clear();
        for (int k = k0; k < k1; k++) {
            m.frames++;
            if (!(tr[k] >= 0 && va[k])) {
                m.errors++;
                continue;
            }
            if (len[k] > 0)
                b.dfl.push_back(len[k]);
        }
        const int bytes = off[k1] - off[k0];
        if (bytes > 0) {
            b.bytes.assign(t.out + off[k0], t.out + off[k1]);
            b.modcod = m.idx;
            p->last_decoded = m.idx;
            p->ready.push_back(std::move(b));
        } else {
            p->spare.push_back(std::move(b));
        }
        k0 = k1;
    }
    t.in_flight = false;
    if (x.budget)
        x.budget->in_flight.fetch_sub(n, std::memory_order_relaxed);
    x.drain_idx++;
}

int mix_drain(cusat_rx_pool* p)
{
    MixPool& x = *p->mix;
    while (x.drain_idx < x.launch_idx) {
        MixSlot& t = x.slot(x.drain_idx);
        if (!t.in_flight) {
            x.drain_idx++;
            continue;
        }
        const cudaError_t e = cudaEventQuery(t.done);
        if (e == cudaErrorNotReady)
            break;
        if (e != cudaSuccess)
            return mix_fail(x, cuda_fail(e, "decode slot"));
        mix_retire(p, t);
    }
    return mix_pump(x, false);
}

// Closes the open micro-batch and submits the partial slot.
void mix_seal(MixPool& x)
{
    mix_close(x);
    if (x.fill > 0) {
        x.submit_idx++;
        x.fill = 0;
    }
}

// Submits the current slot without the open micro-batch's frames at its end,
// which move to the start of the next slot (symbols copied, references
// updated); returns 1 if frames were submitted.
int mix_split(MixPool& x)
{
    int first = x.fill;
    for (const auto& at : x.open_at)
        if (at.first == x.submit_idx)
            first = std::min(first, at.second);
    if (first == 0 || x.submit_idx + 1 - x.drain_idx >= kFlight - 2)
        return 0;  // nothing closed to launch, or no free slot
    MixSlot& cur = x.slot(x.submit_idx);
    MixSlot& nxt = x.slot(x.submit_idx + 1);
    const int n_move = x.fill - first;
    for (int k = 0; k < n_move; k++) {
        memcpy(nxt.sym + (size_t)k * x.max_xfec * 2, cur.sym + (size_t)(first + k) * x.max_xfec * 2,
               (size_t)x.mc[cur.modcod[first + k]].xfec * 2 * sizeof(float));
        nxt.modcod[k] = cur.modcod[first + k];
    }
    cur.n_frames = first;
    cur.open -= n_move;
    nxt.n_frames = n_move;
    nxt.open = n_move;
    nxt.in_flight = false;
    for (auto& at : x.open_at)
        if (at.first == x.submit_idx) {
            at.first++;
            at.second -= first;
        }
    x.submit_idx++;
    x.fill = n_move;
    x.slot_start = x.open_start;
    return 1;
}

int mix_finish(cusat_rx_pool* p)
{
    MixPool& x = *p->mix;
    mix_seal(x);
    int rc = mix_pump(x, true);
    while (rc == CUSAT_OK && x.drain_idx < x.submit_idx) {
        if (x.drain_idx >= x.launch_idx) {
            rc = mix_pump(x, true);
            if (rc)
                break;
        }
        MixSlot& t = x.slot(x.drain_idx);
        if (!t.in_flight) {
            x.drain_idx++;
            continue;
        }
        const cudaError_t e = cudaEventSynchronize(t.done);
        if (e != cudaSuccess)
            return mix_fail(x, cuda_fail(e, "decode slot"));
        mix_retire(p, t);
    }
    return rc;
}

// rx_fec_pool::submit for the mixed pool (rx_fec_pool.cc:48-87 semantics:
// frames in submission order; the flush at a MODCOD change becomes the close
// of that MODCOD's micro-batch, without waiting).
int mix_submit(cusat_rx_pool* p, const float* symbols, int n_symbols, int modcod)
{
    MixPool& x = *p->mix;
    const int mi = x.find(modcod);
    if (mi < 0)
        return 0;  // MODCOD not enabled: skipped
    if (x.failed)
        return x.failed;
    if (x.fill == 0 || x.submit_idx - x.drain_idx >= kFlight / 2) {
        const int rc = mix_drain(p);
        if (rc)
            return rc;
    }
    MixModcod& m = x.mc[mi];
    // a MODCOD change closes the previous MODCOD's micro-batch even when this
    // frame is then dropped (the reference flushes that chain first)
    if (x.open_mc >= 0 && x.open_mc != mi)
        mix_close(x);
    if (x.submit_idx - x.drain_idx >= kFlight - 2 || n_symbols != m.xfec) {
        m.drops++;
        m.frames++;
        m.errors++;
        const int rc = mix_pump(x, false);  // the closed frames may complete a slot
        if (rc)
            return rc;
        return p->ready.empty() ? 0 : 1;
    }
    MixSlot& t = x.slot(x.submit_idx);
    const int k = x.fill;
    float* dest = t.sym + (size_t)k * x.max_xfec * 2;
    copy_frame(x.crew, dest, symbols, (size_t)n_symbols * 2 * sizeof(float));
    if (++m.snr_skip >= kSnrPeriod) {
        m.snr_skip = 0;
        mix_estimate_snr(m, dest, n_symbols);
    }
    t.modcod[k] = mi;
    t.open++;
    if (k == 0)
        x.slot_start = Clock::now();
    if (x.open_at.empty())
        x.open_start = Clock::now();
    x.open_mc = mi;
    x.open_at.push_back(std::make_pair(x.submit_idx, k));
    t.n_frames = ++x.fill;
    if ((int)x.open_at.size() >= x.micro_batch)
        mix_close(x);
    if (x.fill >= x.slot_frames) {
        x.submit_idx++;
        x.fill = 0;
    }
    const int rc = mix_pump(x, false);
    if (rc)
        return rc;
    return p->ready.empty() ? 0 : 1;
}

int mix_reset(cusat_rx_pool* p)
{
    MixPool& x = *p->mix;
    int rc = CUSAT_OK;
    if (x.lock_fn)
        x.lock_fn(x.lock_ctx);
    for (int i = x.drain_idx; i < x.submit_idx; i++) {
        MixSlot& t = x.slot(i);
        if (t.in_flight) {
            const cudaError_t e = cudaEventSynchronize(t.done);
            if (e != cudaSuccess && rc == CUSAT_OK)
                rc = cuda_fail(e, "decode slot");
            if (x.budget)
                x.budget->in_flight.fetch_sub(t.n_frames, std::memory_order_relaxed);
        }
        t.in_flight = false;
        t.n_frames = t.open = 0;
    }
    if (x.fill > 0) {
        MixSlot& t = x.slot(x.submit_idx);
        t.n_frames = t.open = 0;
    }
    if (x.unlock_fn)
        x.unlock_fn(x.lock_ctx);
    x.submit_idx = x.launch_idx = x.drain_idx = x.next_lane = x.fill = 0;
    x.open_at.clear();
    x.open_mc = -1;
    for (MixModcod& m : x.mc) {
        // rx_fec_chain::reset: SNR state and counters, not the drop count nor
        // the frames-since-estimate counter
        m.snr_db = 0.0f;
        m.noise_var = 1.0f;
        m.llr_gain = 4.0f;
        m.frames = m.errors = 0;
    }
    return rc ? mix_fail(x, rc) : CUSAT_OK;
}

void mix_free(MixPool* x)
{
    if (!x)
        return;
    for (MixLane& L : x->lanes) {
        if (L.stream)
            cudaStreamSynchronize(L.stream);
        cusat_batch_destroy(L.batch);
        if (L.sym_dev)
            cudaFree(L.sym_dev);
        if (L.hard_dev)
            cudaFree(L.hard_dev);
        if (L.done)
            cudaEventDestroy(L.done);
        if (L.stream)
            cudaStreamDestroy(L.stream);
    }
    for (MixSlot& t : x->flight) {
        if (t.sym)
            cudaFreeHost(t.sym);
        if (t.res)
            cudaFreeHost(t.res);
        if (t.out)
            cudaFreeHost(t.out);
        if (t.done)
            cudaEventDestroy(t.done);
    }
    cusat_bb_extractor_destroy(x->bb);
    delete x;
}

int mix_create(int framesize, const int32_t* modcods, int n_modcods, int max_trials, int n_streams, int micro_batch,
               int slot_frames, MixPool** out)
{
    *out = nullptr;
    MixPool* x = new MixPool();
    x->slot_frames = slot_frames;
    x->micro_batch = micro_batch;
    int rc = CUSAT_OK;
    std::vector<int32_t> triples;
    int longest = -1;
    for (int i = 0; i < n_modcods && rc == CUSAT_OK; i++) {
        MixModcod m;
        m.idx = modcods[3 * i];
        m.mod = modcods[3 * i + 1];
        m.rate = modcods[3 * i + 2];
        if (x->find(m.idx) >= 0) {
            rc = fail(CUSAT_ERR_ARG, "MODCOD listed twice");
            break;
        }
        int32_t mi[6];
        std::vector<float> pts(512);
        uint32_t col[8];
        rc = cusat_modcod_info(m.mod, m.rate, framesize, pts.data(), col, mi);
        if (rc)
            break;
        int32_t ci[12];
        rc = cusat_code_info(framesize, m.rate, ci);
        if (rc)
            break;
        m.xfec = mi[3];
        m.k_bytes = ci[1] / 8;
        m.kbch_bytes = ci[2] / 8;
        m.bits_per_sym = cusat::make_constellation(m.mod, m.rate, framesize, &m.pts);
        if (m.bits_per_sym <= 0) {
            rc = fail(CUSAT_ERR_UNSUPPORTED, "constellation");
            break;
        }
        x->max_xfec = std::max(x->max_xfec, m.xfec);
        x->max_kbytes = std::max(x->max_kbytes, m.k_bytes);
        if (m.kbch_bytes > x->max_kbch) {
            x->max_kbch = m.kbch_bytes;
            longest = m.rate;
        }
        triples.push_back(m.mod);
        triples.push_back(m.rate);
        triples.push_back(framesize);
        x->mc.push_back(m);
    }
    if (rc == CUSAT_OK)
        rc = cusat_bb_extractor_create(framesize, longest, &x->bb);
    x->lanes.resize(n_streams);
    x->flight.resize(kFlight);
    const size_t sym_bytes = (size_t)slot_frames * x->max_xfec * 2 * sizeof(float);
    for (MixLane& L : x->lanes) {
        if (rc)
            break;
        rc = cusat_batch_create(triples.data(), n_modcods, max_trials, slot_frames, &L.batch);
        if (rc)
            break;
        L.frames.resize(slot_frames);
        cudaError_t e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaMalloc(&L.sym_dev, sym_bytes);
        if (e == cudaSuccess)
            e = cudaMalloc(&L.hard_dev, (size_t)slot_frames * x->max_kbytes);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "mixed pool stream buffers");
    }
    for (size_t i = 0; rc == CUSAT_OK && i < x->flight.size(); i++) {
        MixSlot& t = x->flight[i];
        t.modcod.assign(slot_frames, 0);
        t.noise_var.assign(slot_frames, 1.0f);
        t.llr_gain.assign(slot_frames, 4.0f);
        cudaError_t e = cudaMallocHost(&t.sym, sym_bytes);
        if (e == cudaSuccess)
            e = cudaMallocHost(&t.res, (size_t)(5 * slot_frames + 1) * sizeof(int32_t));
        if (e == cudaSuccess)
            e = cudaMallocHost(&t.out, (size_t)slot_frames * x->max_kbch);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&t.done, cudaEventDisableTiming);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "mixed pool slot");
    }
    if (rc) {
        mix_free(x);
        return rc;
    }
    x->budget = default_budget();
    *out = x;
    return CUSAT_OK;
}

}  // namespace

extern "C" {

int cusat_rx_pool_create(int framesize, const int32_t* modcods, int n_modcods, int max_trials, int cuda_max_batch,
                         int n_gpu_streams, int micro_batch, cusat_rx_pool** out)
{
    if (!out || !modcods || n_modcods <= 0 || n_modcods > 256)
        return fail(CUSAT_ERR_ARG, "invalid pool arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_rx_pool* p = new cusat_rx_pool();
    p->budget.s = default_budget();
    for (int i = 0; i < n_modcods && rc == CUSAT_OK; i++) {
        const int idx = modcods[3 * i], mod = modcods[3 * i + 1], rate = modcods[3 * i + 2];
        if (p->find(idx)) {
            rc = fail(CUSAT_ERR_ARG, "MODCOD listed twice");
            break;
        }
        PoolEntry e;
        e.modcod = idx;
        rc = cusat_rx_chain_create(framesize, rate, mod, max_trials, cuda_max_batch, n_gpu_streams, micro_batch,
                                   &e.chain);
        if (rc)
            break;
        e.chain->budget = p->budget.s;
        p->max_output_bytes = std::max(p->max_output_bytes, e.chain->kbch_bytes * e.chain->micro_batch * kFlight);
        p->chains.push_back(e);
    }
    if (rc) {
        cusat_rx_pool_destroy(p);
        return rc;
    }
    *out = p;
    return CUSAT_OK;
}

int cusat_rx_pool_create_mixed(int framesize, const int32_t* modcods, int n_modcods, int max_trials,
                               int n_gpu_streams, int micro_batch, int slot_frames, cusat_rx_pool** out)
{
    if (!out || !modcods || n_modcods <= 0 || n_modcods > 256 || max_trials < 0 || max_trials > 1000 ||
        n_gpu_streams <= 0 || n_gpu_streams > 64 || micro_batch <= 0 || slot_frames <= 0 || slot_frames > 4096)
        return fail(CUSAT_ERR_ARG, "invalid pool arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_rx_pool* p = new cusat_rx_pool();
    MixPool* x = nullptr;
    rc = mix_create(framesize, modcods, n_modcods, max_trials, n_gpu_streams, micro_batch, slot_frames, &x);
    if (rc) {
        delete p;
        return rc;
    }
    p->mix.reset(x);
    p->budget.s = x->budget;
    // a block holds at most one slot's frames
    p->max_output_bytes = x->max_kbch * std::max(micro_batch * kFlight, slot_frames);
    *out = p;
    return CUSAT_OK;
}

void cusat_rx_pool_destroy(cusat_rx_pool* p)
{
    if (!p)
        return;
    for (PoolEntry& e : p->chains)
        cusat_rx_chain_destroy(e.chain);
    if (p->mix) {
        MixPool* x = p->mix.release();
        for (int i = x->drain_idx; i < x->launch_idx; i++)
            if (x->slot(i).in_flight && x->budget)
                x->budget->in_flight.fetch_sub(x->slot(i).n_frames, std::memory_order_relaxed);
        mix_free(x);
    }
    delete p;
}

cusat_rx_chain* cusat_rx_pool_chain(cusat_rx_pool* p, int modcod) { return p ? p->find(modcod) : nullptr; }

// rx_fec_pool::submit (rx_fec_pool.cc:48-87): a MODCOD change finishes the
// previous MODCOD's chain first, so output stays in submission order.
int cusat_rx_pool_submit(cusat_rx_pool* p, const float* symbols, int n_symbols, int modcod)
{
    if (!p)
        return fail(CUSAT_ERR_ARG, "null pool");
    if (p->mix)
        return mix_submit(p, symbols, n_symbols, modcod);
    cusat_rx_chain* c = p->find(modcod);
    if (!c)
        return 0;  // MODCOD not enabled: skipped
    int ready = 0;
    if (p->has_prev && modcod != p->last_submitted) {
        cusat_rx_chain* prev = p->find(p->last_submitted);
        if (prev && (prev->batch_idx > 0 || prev->launch_idx - prev->drain_idx > 0 ||
                     prev->submit_idx - prev->launch_idx > 0)) {
            const int rc = cusat_rx_chain_flush(prev);
            if (rc)
                return rc;
            p->last_decoded = p->last_submitted;
            ready |= harvest(p, p->last_submitted);
        }
    }
    p->last_submitted = modcod;
    p->has_prev = true;
    const int rc = cusat_rx_chain_submit_xfecframe(c, symbols, n_symbols);
    if (rc < 0)
        return rc;
    if (rc > 0) {
        p->last_decoded = modcod;
        ready |= harvest(p, modcod);
    }
    return (ready || !p->ready.empty()) ? 1 : 0;
}

int cusat_rx_pool_get_gse_output(cusat_rx_pool* p, uint8_t* out, int max_bytes)
{
    if (!p || (!out && max_bytes > 0) || max_bytes < 0)
        return fail(CUSAT_ERR_ARG, "invalid output buffer");
    p->last_sizes.clear();
    if (p->ready.empty())
        return 0;
    Block b = std::move(p->ready.front());
    p->ready.pop_front();
    const int n = std::min((int)b.bytes.size(), max_bytes);
    if (n > 0)
        memcpy(out, b.bytes.data(), (size_t)n);
    p->last_decoded = b.modcod;
    p->last_sizes = std::move(b.dfl);
    b.bytes.clear();
    b.dfl.clear();
    p->spare.push_back(std::move(b));
    return n;
}

int cusat_rx_pool_gse_dfl_sizes(const cusat_rx_pool* p, int32_t* out, int max)
{
    if (!p || (!out && max > 0))
        return fail(CUSAT_ERR_ARG, "null argument");
    const int n = (int)p->last_sizes.size();
    if (out)
        memcpy(out, p->last_sizes.data(), sizeof(int32_t) * (size_t)std::min(n, max));
    return n;
}

int cusat_rx_pool_drain_all_completed(cusat_rx_pool* p)
{
    if (!p)
        return fail(CUSAT_ERR_ARG, "null pool");
    if (p->mix) {
        if (p->mix->failed)
            return p->mix->failed;
        const int rc = mix_drain(p);
        return rc ? rc : (p->ready.empty() ? 0 : 1);
    }
    int any = 0;
    for (PoolEntry& e : p->chains) {
        const int rc = cusat_rx_chain_drain_completed(e.chain);
        if (rc < 0)
            return rc;
        if (rc > 0) {
            p->last_decoded = e.modcod;
            any |= harvest(p, e.modcod);
        }
    }
    return (any || !p->ready.empty()) ? 1 : 0;
}

int cusat_rx_pool_finish_all_pending(cusat_rx_pool* p)
{
    if (!p)
        return fail(CUSAT_ERR_ARG, "null pool");
    if (p->mix)
        return p->mix->failed ? p->mix->failed : mix_finish(p);
    for (PoolEntry& e : p->chains) {
        const int rc = cusat_rx_chain_flush(e.chain);
        if (rc)
            return rc;
        harvest(p, e.modcod);
    }
    return CUSAT_OK;
}

// launch_stale (rx_fec_pool.cc:190-207): launch partial micro-batches older
// than max_age_ms without waiting for them.
int cusat_rx_pool_launch_stale(cusat_rx_pool* p, double max_age_ms)
{
    if (!p)
        return fail(CUSAT_ERR_ARG, "null pool");
    const Clock::time_point now = Clock::now();
    int launched = 0;
    if (p->mix) {
        MixPool& x = *p->mix;
        if (x.failed)
            return x.failed;
        auto age_ms = [&](Clock::time_point t0) { return std::chrono::duration<double, std::milli>(now - t0).count(); };
        if (!x.open_at.empty() && age_ms(x.open_start) >= max_age_ms) {
            // the open micro-batch is stale (the reference launches it): close
            // it and launch the partial slot
            mix_seal(x);
            launched = 1;
        } else if (x.fill > 0 && age_ms(x.slot_start) >= max_age_ms) {
            // frames of earlier micro-batches wait in the partial slot (the
            // reference launched them at their MODCOD change or when full):
            // launch them, the open micro-batch moves on to a new slot
            launched = mix_split(x);
        }
        const int rc = mix_pump(x, false);
        if (rc)
            return rc;
        return launched;
    }
    for (PoolEntry& e : p->chains) {
        cusat_rx_chain* c = e.chain;
        if (c->batch_idx > 0 &&
            std::chrono::duration<double, std::milli>(now - c->batch_start).count() >= max_age_ms) {
            const int rc = cusat_rx_chain_launch_partial(c);
            if (rc)
                return rc;
            launched = 1;
        }
    }
    return launched;
}

int cusat_rx_pool_reset_all(cusat_rx_pool* p)
{
    if (!p)
        return fail(CUSAT_ERR_ARG, "null pool");
    int rc = p->mix ? mix_reset(p) : CUSAT_OK;
    for (PoolEntry& e : p->chains) {
        const int r = cusat_rx_chain_reset(e.chain);
        if (r && rc == CUSAT_OK)
            rc = r;
    }
    p->last_decoded = p->last_submitted = 0;
    p->has_prev = false;
    clear_ready(p);
    return rc;
}

int cusat_rx_pool_warmup_all(cusat_rx_pool* p)
{
    if (!p)
        return fail(CUSAT_ERR_ARG, "null pool");
    if (p->mix) {
        // rx_fec_chain::warmup per MODCOD: one all-zero frame through the
        // path, then a clean state (each MODCOD's frames-since-estimate
        // counter keeps the one frame, as the reference's chains do)
        MixPool& x = *p->mix;
        std::vector<float> zeros((size_t)x.max_xfec * 2, 0.0f);
        int rc = CUSAT_OK;
        for (const MixModcod& m : x.mc) {
            rc = mix_submit(p, zeros.data(), m.xfec, m.idx);
            if (rc < 0)
                return rc;
        }
        rc = mix_finish(p);
        if (rc == CUSAT_OK)
            rc = mix_reset(p);
        for (MixModcod& m : x.mc)
            m.drops = 0;
        p->last_decoded = p->last_submitted = 0;
        p->has_prev = false;
        clear_ready(p);
        return rc;
    }
    for (PoolEntry& e : p->chains) {
        const int rc = cusat_rx_chain_warmup(e.chain);
        if (rc)
            return rc;
    }
    p->last_decoded = p->last_submitted = 0;
    p->has_prev = false;
    clear_ready(p);
    return CUSAT_OK;
}

int cusat_rx_pool_set_copy_threads(cusat_rx_pool* p, int helpers)
{
    if (!p || helpers < 0 || helpers > 32)
        return fail(CUSAT_ERR_ARG, "invalid copy thread count");
    std::shared_ptr<CopyCrew> crew = helpers ? std::make_shared<CopyCrew>(helpers) : nullptr;
    if (p->mix)
        p->mix->crew = crew;
    for (PoolEntry& e : p->chains)
        e.chain->crew = crew;  // one crew: the pool submits to one chain at a time
    return CUSAT_OK;
}

void cusat_rx_pool_update_snr(cusat_rx_pool* p, int modcod, float snr_db)
{
    if (!p)
        return;
    if (p->mix) {
        const int mi = p->mix->find(modcod);
        if (mi < 0 || !(snr_db > 0.0f))
            return;
        MixModcod& m = p->mix->mc[mi];
        const float lin = std::pow(10.0f, snr_db / 10.0f);
        m.pilot_snr_db = snr_db;
        m.snr_db = snr_db;
        m.noise_var = 1.0f / lin;
        m.llr_gain = std::min(4.0f / m.noise_var, 1000.0f);
        return;
    }
    cusat_rx_chain_update_snr(p->find(modcod), snr_db);
}

int cusat_rx_pool_set_launch_lock(cusat_rx_pool* p, void (*lock)(void*), void (*unlock)(void*), void* ctx)
{
    if (!p || (!lock) != (!unlock))
        return fail(CUSAT_ERR_ARG, "lock and unlock go together");
    if (p->mix) {
        p->mix->lock_fn = lock;
        p->mix->unlock_fn = unlock;
        p->mix->lock_ctx = ctx;
        return CUSAT_OK;
    }
    for (PoolEntry& e : p->chains) {
        const int rc = cusat_rx_chain_set_launch_lock(e.chain, lock, unlock, ctx);
        if (rc)
            return rc;
    }
    return CUSAT_OK;
}

// out[0..4] = total frames, total errors, total GPU drops, max_output_bytes,
// data SNR (dB) of the last decoded MODCOD
int cusat_rx_pool_stats(const cusat_rx_pool* p, double* out)
{
    if (!p || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    double f = 0, e = 0, d = 0, snr = 0;
    if (p->mix)
        for (const MixModcod& m : p->mix->mc) {
            f += (double)m.frames;
            e += (double)m.errors;
            d += (double)m.drops;
            if (m.idx == p->last_decoded)
                snr = m.snr_db;
        }
    for (const PoolEntry& c : p->chains) {
        f += (double)c.chain->frames;
        e += (double)c.chain->errors;
        d += (double)c.chain->drops;
        if (c.modcod == p->last_decoded)
            snr = c.chain->snr_db;
    }
    out[0] = f;
    out[1] = e;
    out[2] = d;
    out[3] = p->max_output_bytes;
    out[4] = snr;
    return CUSAT_OK;
}

int cusat_rx_pool_modcod_counters(const cusat_rx_pool* p, int modcod, uint64_t* frames, uint64_t* errors)
{
    if (!p || !frames || !errors)
        return fail(CUSAT_ERR_ARG, "null argument");
    if (p->mix) {
        const int mi = p->mix->find(modcod);
        if (mi < 0)
            return 0;
        *frames = p->mix->mc[mi].frames;
        *errors = p->mix->mc[mi].errors;
        return 1;
    }
    for (const PoolEntry& c : p->chains)
        if (c.modcod == modcod) {
            *frames = c.chain->frames;
            *errors = c.chain->errors;
            return 1;
        }
    return 0;
}

}  // extern "C"
