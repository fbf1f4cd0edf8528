// Serving loop: continuous batching of frame requests of mixed MODCODs.
//
// Requests carry an arrival time.  A scheduler thread admits arrived
// requests into an HBM arena of a fixed budget (each batch takes one block
// for its frames' symbols and results), launches a mixed-MODCOD batch on a
// free slot (each slot: its own batch object, stream and pinned result
// staging), and reaps completed slots while others run: batches on
// different slots overlap on the device, and requests that arrive while
// the GPU is busy join the next batch as soon as a slot and memory are
// free.  Each frame is decoded by one CTA from its own symbols, so its
// result does not depend on what it was batched with.
//
// The reference's serving counterpart is the RX chain pool: a flight ring
// of 128 slots over 8 streams per MODCOD chain, flushed on MODCOD change
// (lib/cusat_dsp/rx_fec_chain.cc:281-627, rx_fec_pool.cc:48-87).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

#include "arena.h"
#include "engine.h"

using namespace cusat_internal;

namespace {

struct CopyDesc {
    const float2* src;
    float2* dst;
    int n;  // symbols
    int pad;
};

// Copies each admitted frame's symbols into its arena slice (one CTA per
// frame at a time, coalesced 8-byte loads).
__global__ void gather_frames_kernel(const CopyDesc* __restrict__ d, int n)
{
    for (int f = blockIdx.x; f < n; f += gridDim.x) {
        const CopyDesc c = d[f];
        for (int i = threadIdx.x; i < c.n; i += blockDim.x)
            c.dst[i] = __ldcs(c.src + i);
    }
}

struct Geo {
    int xfec = 0, k_bytes = 0;
    size_t sym_bytes = 0;
};

struct Pending {
    cusat_request req;
    double admit_s = 0;
};

struct Slot {
    cusat_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<Pending> frames;
    std::vector<cusat_frame> desc;
    size_t off = 0, bytes = 0;          // arena block
    size_t hard_off = 0, res_off = 0;   // within the block
    std::vector<size_t> hard_at;        // per frame, within the hard region
    unsigned char* h_out = nullptr;     // pinned: hard bits, trials, flags
    size_t h_cap = 0;
    CopyDesc* h_copy = nullptr;         // pinned
    CopyDesc* d_copy = nullptr;
};

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct cusat_server {
    int device = 0, max_batch = 0, max_trials = 0;
    std::vector<Geo> geo;
    std::vector<Slot> slots;
    Arena arena;
    unsigned char* d_arena = nullptr;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Pending> pending;       // submission order
    std::deque<cusat_result> done;
    std::thread thread;
    std::atomic<bool> stop{false};
    int error = 0;
    std::string error_msg;
    // statistics (written by the scheduler, read by cusat_server_stats)
    std::atomic<uint64_t> n_batches{0}, n_frames{0}, max_batch_seen{0}, peak_bytes{0};
    std::atomic<int> inflight{0}, max_inflight_batches{0};
};

namespace {

size_t frame_bytes(const cusat_server* s, int m)
{
    return s->arena.round(s->geo[m].sym_bytes) + (size_t)(s->geo[m].k_bytes + 15) / 16 * 16 + 8;
}

void set_error(cusat_server* s, int rc)
{
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->error) {
        s->error = rc;
        s->error_msg = cusat_last_error();
    }
    s->cv.notify_all();
}

// Completes a finished slot: results to the done queue, block back to the arena.
void reap(cusat_server* s, Slot& sl)
{
    const double t = seconds_since(s->t0);
    const int n = (int)sl.frames.size();
    const size_t hard_bytes = sl.res_off - sl.hard_off;
    const int32_t* trials = (const int32_t*)(sl.h_out + hard_bytes);
    const int32_t* valid = trials + n;
    std::vector<cusat_result> out(n);
    for (int k = 0; k < n; k++) {
        const cusat_request& r = sl.frames[k].req;
        if (r.hard_host)
            memcpy(r.hard_host, sl.h_out + sl.hard_at[k], s->geo[r.modcod].k_bytes);
        cusat_result& o = out[k];
        o.tag = r.tag;
        o.modcod = r.modcod;
        o.trials = trials[k];
        o.bch_valid = valid[k];
        o.reserved = 0;
        o.arrival_s = r.arrival_s;
        o.admit_s = sl.frames[k].admit_s;
        o.done_s = t;
    }
    s->arena.release(sl.off, sl.bytes);
    sl.busy = false;
    sl.frames.clear();
    s->inflight--;
    std::lock_guard<std::mutex> g(s->mu);
    for (auto& o : out)
        s->done.push_back(o);
    s->cv.notify_all();
}

// Launches the frames in sl.frames (arena block already taken).
int launch(cusat_server* s, Slot& sl)
{
    const int n = (int)sl.frames.size();
    unsigned char* base = s->d_arena + sl.off;
    size_t o = 0;
    sl.desc.resize(n);
    sl.hard_at.resize(n);
    int n_dev = 0;
    for (int k = 0; k < n; k++) {
        const cusat_request& r = sl.frames[k].req;
        const Geo& g = s->geo[r.modcod];
        float* dst = (float*)(base + o);
        if (r.flags & CUSAT_REQ_HOST_SYMBOLS) {
            CU(cudaMemcpyAsync(dst, r.sym, g.sym_bytes, cudaMemcpyHostToDevice, sl.stream), "cudaMemcpyAsync(symbols)");
        } else {
            sl.h_copy[n_dev++] = CopyDesc{(const float2*)r.sym, (float2*)dst, g.xfec, 0};
        }
        cusat_frame& d = sl.desc[k];
        d.modcod = r.modcod;
        d.noise_var = r.noise_var;
        d.llr_gain = r.llr_gain;
        d.reserved = 0;
        d.sym = dst;
        o += s->arena.round(g.sym_bytes);
    }
    sl.hard_off = o;
    size_t h = 0;
    for (int k = 0; k < n; k++) {
        sl.hard_at[k] = h;
        sl.desc[k].hard = base + o + h;
        h += (size_t)(s->geo[sl.frames[k].req.modcod].k_bytes + 15) / 16 * 16;
    }
    sl.res_off = o + h;
    int32_t* trials = (int32_t*)(base + sl.res_off);
    for (int k = 0; k < n; k++) {
        sl.desc[k].trials = trials + k;
        sl.desc[k].bch_valid = trials + n + k;
    }
    if (n_dev) {
        CU(cudaMemcpyAsync(sl.d_copy, sl.h_copy, n_dev * sizeof(CopyDesc), cudaMemcpyHostToDevice, sl.stream),
           "cudaMemcpyAsync(copy list)");
        gather_frames_kernel<<<std::min(n_dev, 1024), 256, 0, sl.stream>>>(sl.d_copy, n_dev);
        CU(cudaGetLastError(), "gather launch");
    }
    int rc = batch_launch_ready(sl.batch, sl.desc.data(), n, sl.stream);
    if (rc)
        return rc;
    const size_t out_bytes = h + 8 * (size_t)n;
    CU(cudaMemcpyAsync(sl.h_out, base + o, out_bytes, cudaMemcpyDeviceToHost, sl.stream), "cudaMemcpyAsync(results)");
    CU(cudaEventRecord(sl.done, sl.stream), "cudaEventRecord");
    sl.busy = true;
    return CUSAT_OK;
}

void scheduler(cusat_server* s)
{
    cudaSetDevice(s->device);
    while (!s->stop.load()) {
        bool progress = false;
        int busy = 0;
        for (auto& sl : s->slots) {
            if (!sl.busy)
                continue;
            const cudaError_t e = cudaEventQuery(sl.done);
            if (e == cudaSuccess) {
                reap(s, sl);
                progress = true;
            } else if (e != cudaErrorNotReady) {
                set_error(s, cuda_fail(e, "batch execution"));
                return;
            } else {
                busy++;
            }
        }
        double next_arrival = -1;
        for (auto& sl : s->slots) {
            if (sl.busy)
                continue;
            // take arrived requests in order while they fit one arena block
            const double now = seconds_since(s->t0);
            const size_t room = s->arena.largest();
            size_t need = 0;
            {
                std::lock_guard<std::mutex> g(s->mu);
                while (!s->pending.empty() && (int)sl.frames.size() < s->max_batch) {
                    const Pending& p = s->pending.front();
                    if (p.req.arrival_s > now) {
                        next_arrival = p.req.arrival_s;
                        break;
                    }
                    const size_t b = frame_bytes(s, p.req.modcod);
                    if (need + b > room)
                        break;
                    need += b;
                    sl.frames.push_back(p);
                    sl.frames.back().admit_s = now;
                    s->pending.pop_front();
                }
            }
            if (sl.frames.empty())
                break;
            if (!s->arena.alloc(need, &sl.off)) {
                set_error(s, fail(CUSAT_ERR_CUDA, "arena accounting"));
                return;
            }
            sl.bytes = need;
            const int rc = launch(s, sl);
            if (rc) {
                set_error(s, rc);
                return;
            }
            s->n_batches++;
            s->n_frames += sl.frames.size();
            if (sl.frames.size() > s->max_batch_seen.load())
                s->max_batch_seen = sl.frames.size();
            s->peak_bytes = s->arena.peak();
            busy++;
            s->inflight++;
            if (busy > s->max_inflight_batches.load())
                s->max_inflight_batches = busy;
            progress = true;
        }
        if (progress)
            continue;
        if (busy) {
            std::this_thread::yield();
            continue;
        }
        // idle: wait for a submission or the next arrival time
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->stop.load())
            break;
        if (s->pending.empty()) {
            s->cv.wait_for(lk, std::chrono::milliseconds(2));
        } else if (next_arrival > 0) {
            const double dt = next_arrival - seconds_since(s->t0);
            if (dt > 200e-6)
                s->cv.wait_for(lk, std::chrono::microseconds((long)(dt * 1e6) - 100));
        }
    }
}

void release(cusat_server* s)
{
    if (!s)
        return;
    if (s->thread.joinable()) {
        s->stop.store(true);
        s->cv.notify_all();
        s->thread.join();
    }
    cudaDeviceSynchronize();
    for (auto& sl : s->slots) {
        if (sl.batch) cusat_batch_destroy(sl.batch);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.h_out) cudaFreeHost(sl.h_out);
        if (sl.h_copy) cudaFreeHost(sl.h_copy);
        if (sl.d_copy) cudaFree(sl.d_copy);
    }
    if (s->d_arena)
        cudaFree(s->d_arena);
    delete s;
}

}  // namespace

extern "C" {

int cusat_server_create(const int32_t* modcods, int n_modcods, int max_trials, size_t hbm_budget, int slots,
                        int max_batch, cusat_server** out)
{
    if (!out || !modcods || n_modcods <= 0 || slots <= 0 || slots > 64 || max_batch <= 0 || hbm_budget == 0)
        return fail(CUSAT_ERR_ARG, "invalid server arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_server* s = new cusat_server();
    s->device = dev;
    s->max_batch = max_batch;
    s->max_trials = max_trials;
    s->arena = Arena(hbm_budget);
    size_t largest = 0, max_k = 0;
    for (int i = 0; i < n_modcods && rc == CUSAT_OK; i++) {
        std::string err;
        cusat::ModcodDemap dm;
        const cusat::CodePlan* p = cusat::get_code_plan(modcods[3 * i + 2], modcods[3 * i + 1], &err);
        if (!p || !cusat::build_modcod_demap(modcods[3 * i], modcods[3 * i + 1], modcods[3 * i + 2], &dm, &err)) {
            rc = fail(CUSAT_ERR_UNSUPPORTED, err);
            break;
        }
        Geo g;
        g.xfec = dm.xfec;
        g.k_bytes = p->K / 8;
        g.sym_bytes = (size_t)dm.xfec * 8;
        s->geo.push_back(g);
        largest = std::max(largest, frame_bytes(s, i));
        max_k = std::max(max_k, (size_t)(g.k_bytes + 15) / 16 * 16);
    }
    if (rc == CUSAT_OK && largest > hbm_budget)
        rc = fail(CUSAT_ERR_ARG, "HBM budget smaller than one frame");
    if (rc == CUSAT_OK) {
        cudaError_t e = cudaMalloc(&s->d_arena, hbm_budget);
        s->slots.resize(slots);
        for (auto& sl : s->slots) {
            if (e != cudaSuccess)
                break;
            rc = cusat_batch_create(modcods, n_modcods, max_trials, max_batch, &sl.batch);
            if (rc)
                break;
            sl.h_cap = (size_t)max_batch * (max_k + 8);
            e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
            if (e == cudaSuccess)
                e = cudaMallocHost(&sl.h_out, sl.h_cap);
            if (e == cudaSuccess)
                e = cudaMallocHost(&sl.h_copy, (size_t)max_batch * sizeof(CopyDesc));
            if (e == cudaSuccess)
                e = cudaMalloc(&sl.d_copy, (size_t)max_batch * sizeof(CopyDesc));
        }
        if (rc == CUSAT_OK && e != cudaSuccess)
            rc = cuda_fail(e, "server set-up");
    }
    if (rc) {
        release(s);
        return rc;
    }
    s->t0 = std::chrono::steady_clock::now();
    s->thread = std::thread(scheduler, s);
    *out = s;
    return CUSAT_OK;
}

void cusat_server_destroy(cusat_server* s) { release(s); }

double cusat_server_now(const cusat_server* s) { return s ? seconds_since(s->t0) : 0.0; }

int cusat_server_set_weights(cusat_server* s, int modcod, const int16_t* weights, int n_iter)
{
    if (!s)
        return fail(CUSAT_ERR_ARG, "null server");
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (!s->pending.empty() || s->inflight.load())
            return fail(CUSAT_ERR_ARG, "weights change while requests are pending or in flight");
    }
    for (auto& sl : s->slots) {
        const int rc = cusat_batch_set_weights(sl.batch, modcod, weights, n_iter);
        if (rc)
            return rc;
    }
    return CUSAT_OK;
}

int cusat_server_submit(cusat_server* s, const cusat_request* reqs, int n)
{
    if (!s || (!reqs && n) || n < 0)
        return fail(CUSAT_ERR_ARG, "invalid submission");
    const double now = seconds_since(s->t0);
    std::lock_guard<std::mutex> g(s->mu);
    if (s->error)
        return fail(s->error, s->error_msg);
    for (int i = 0; i < n; i++) {
        const cusat_request& r = reqs[i];
        if (r.modcod < 0 || r.modcod >= (int)s->geo.size() || !r.sym)
            return fail(CUSAT_ERR_ARG, "request with an unknown MODCOD or no symbols");
    }
    for (int i = 0; i < n; i++) {
        Pending p;
        p.req = reqs[i];
        if (p.req.arrival_s < 0)
            p.req.arrival_s = now;
        s->pending.push_back(p);
    }
    s->cv.notify_all();
    return CUSAT_OK;
}

int cusat_server_poll(cusat_server* s, cusat_result* out, int max, int wait_ms)
{
    if (!s || !out || max <= 0)
        return fail(CUSAT_ERR_ARG, "invalid poll");
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && wait_ms > 0 && !s->error)
        s->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty() || s->error; });
    int k = 0;
    while (k < max && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    if (!k && s->error)
        return fail(s->error, s->error_msg);
    return k;
}

int cusat_server_stats(cusat_server* s, double* out)
{
    if (!s || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> g(s->mu);
    out[0] = (double)s->pending.size();
    out[1] = (double)s->n_batches.load();
    out[2] = (double)s->n_frames.load();
    out[3] = (double)s->max_batch_seen.load();
    out[4] = (double)s->max_inflight_batches.load();
    out[5] = (double)s->peak_bytes.load();
    out[6] = (double)s->arena.size();
    out[7] = (double)s->inflight.load();
    return CUSAT_OK;
}

}  // extern "C"
