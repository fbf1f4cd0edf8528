// Mixed-MODCOD batches: one launch decodes frames of many MODCODs and frame
// sizes (symbols in; hard decisions, iteration counts, BCH flags out).
//
// The MODCODs of a batch fall into kernel classes (circulant slots per layer
// x lanes); each class runs one persistent decoder kernel over its frames,
// reloading a code's tables into shared memory when consecutive frames of a
// CTA change code.  The class kernels run concurrently on forked streams and
// one mixed-code BCH kernel follows; the whole sequence can be captured once
// into a CUDA graph and replayed.  A measurement-driven tuner picks each
// class's grid (number of persistent CTAs) and the class launch order.
// The reference decodes one MODCOD per chain and launches per
// (chain, micro-batch, stream) (lib/cusat_dsp/rx_fec_chain.cc:361-505,
// rx_fec_pool.cc:48-87).
#include <algorithm>
#include <map>
#include <memory>

#include "engine.h"

using namespace cusat_internal;

namespace {

struct ModcodObj {
    int mod = 0, rate = 0, fs = 0;
    const cusat::CodePlan* plan = nullptr;
    DevPlan dp;
    DevDemapObj dm;
    DevBch bch;
    DevWeights weights;
    int cls = -1;       // kernel class
    int code_in_class = 0;
};

struct KernelClass {
    int cmax = 0, lanes = 0;
    const void* fn = nullptr;
    int threads = 0, per_sm = 0, grid_max = 0;
    cusat::DecodeArgs proto{};
    std::vector<int> modcods;  // modcod indices, position = code index in the class
    cusat::DevCode* d_codes = nullptr;
    cusat::FrameDesc* d_frames = nullptr;
    uint4* msg = nullptr;
    unsigned int* queue = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    // tuned launch: persistent CTAs of this class's decoder (0 = every
    // resident slot), i.e. about count / grid frames per CTA
    int grid = 0;
    float tuned_ms = 0.0f;  // the class's decoder alone on its full grid, at the last tuning
};

}  // namespace

struct cusat_batch {
    std::vector<std::unique_ptr<ModcodObj>> modcods;
    std::vector<KernelClass> classes;
    std::vector<int> order;  // class launch order
    int max_trials = 0, max_frames = 0, sms = 0;
    // staging (pinned) and device descriptors
    cusat::FrameDesc* h_frames = nullptr;   // [max_frames], grouped by class
    cusat::BchFrame* h_bch = nullptr;       // [max_frames]
    cusat::DemapFrame* h_demap = nullptr;   // [max_frames]
    cusat::FrameDesc* d_frames = nullptr;
    cusat::BchFrame* d_bch = nullptr;
    cusat::DemapFrame* d_demap = nullptr;
    cusat::BchDev* d_bch_codes = nullptr;
    cusat::DevDemap* d_demap_params = nullptr;  // [modcods]
    int16_t* llr = nullptr;                     // [max_frames][max_n] demapped LLRs
    int max_n = 0, max_len = 0;                 // largest code length, largest interleaved length
    std::vector<int> class_count, class_off;
    cudaEvent_t fork = nullptr;
    cudaEvent_t last = nullptr;  // recorded after every launch and replay
    bool launched = false;
    int max_ctas = 0;            // test hook: cap on every class's persistent grid (0 = none)
    // captured sequence: its own device descriptors (written once at capture),
    // so that later launches with other frames leave it intact
    cudaGraphExec_t graph = nullptr;
    cusat::FrameDesc* g_frames = nullptr;
    cusat::BchFrame* g_bch = nullptr;
    cusat::DemapFrame* g_demap = nullptr;
    int graph_frames = 0;
};

namespace {

void release(cusat_batch* b)
{
    if (!b)
        return;
    if (b->graph)
        cudaGraphExecDestroy(b->graph);
    for (auto& c : b->classes) {
        if (c.d_codes) cudaFree(c.d_codes);
        if (c.msg) cudaFree(c.msg);
        if (c.queue) cudaFree(c.queue);
        if (c.stream) cudaStreamDestroy(c.stream);
        if (c.done) cudaEventDestroy(c.done);
    }
    for (auto& m : b->modcods) {
        m->dp.blob ? (void)cudaFree(m->dp.blob) : (void)0;
        m->dm.release();
        m->bch.release();
        m->weights.release();
    }
    if (b->h_frames) cudaFreeHost(b->h_frames);
    if (b->h_bch) cudaFreeHost(b->h_bch);
    if (b->h_demap) cudaFreeHost(b->h_demap);
    if (b->d_frames) cudaFree(b->d_frames);
    if (b->d_bch) cudaFree(b->d_bch);
    if (b->d_demap) cudaFree(b->d_demap);
    if (b->d_bch_codes) cudaFree(b->d_bch_codes);
    if (b->d_demap_params) cudaFree(b->d_demap_params);
    if (b->llr) cudaFree(b->llr);
    if (b->g_frames) cudaFree(b->g_frames);
    if (b->g_bch) cudaFree(b->g_bch);
    if (b->g_demap) cudaFree(b->g_demap);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->last) cudaEventDestroy(b->last);
    delete b;
}

// Writes the staged descriptors of frames[0..n) grouped by class.
int stage(cusat_batch* b, const cusat_frame* frames, int n)
{
    const int nc = (int)b->classes.size();
    b->class_count.assign(nc, 0);
    for (int i = 0; i < n; i++) {
        const int m = frames[i].modcod;
        if (m < 0 || m >= (int)b->modcods.size())
            return fail(CUSAT_ERR_ARG, "frame refers to an unknown MODCOD index");
        if (!frames[i].sym || !frames[i].hard || !frames[i].trials)
            return fail(CUSAT_ERR_ARG, "null frame buffer");
        b->class_count[b->modcods[m]->cls]++;
    }
    b->class_off.assign(nc + 1, 0);
    for (int k = 0; k < nc; k++)
        b->class_off[k + 1] = b->class_off[k] + b->class_count[k];
    // within a class, frames ordered by code so that CTAs rarely reload tables
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++)
        idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) {
        const ModcodObj& a = *b->modcods[frames[x].modcod];
        const ModcodObj& c = *b->modcods[frames[y].modcod];
        return a.cls != c.cls ? a.cls < c.cls : a.code_in_class < c.code_in_class;
    });
    for (int k = 0; k < n; k++) {
        const cusat_frame& fr = frames[idx[k]];
        const ModcodObj& m = *b->modcods[fr.modcod];
        int16_t* llr = b->llr + (size_t)k * b->max_n;
        cusat::DemapFrame& q = b->h_demap[k];
        q.modcod = fr.modcod;
        q.noise_var = fr.noise_var;
        q.llr_gain = cusat::capped_llr_gain(m.dm.m, fr.llr_gain);
        q.pad = 0;
        q.sym = reinterpret_cast<const float2*>(fr.sym);
        q.out = llr;
        cusat::FrameDesc& d = b->h_frames[k];
        d.code = m.code_in_class;
        d.pad[0] = d.pad[1] = d.pad[2] = 0;
        d.llr = llr;
        d.hard = fr.hard;
        d.trials = fr.trials;
        cusat::BchFrame& c = b->h_bch[k];
        c.code = fr.modcod;
        c.pad = 0;
        c.cw = fr.hard;
        c.valid = fr.bch_valid;
    }
    return CUSAT_OK;
}

// Launch sequence for n staged frames whose descriptors are (or, with
// `copy`, are first copied from the pinned staging arrays) at
// d_frames/d_bch/d_demap: the demap of every frame in one launch (per-class
// demap launches on the class streams measured slower: their overlap with
// decoding does not pay for eleven smaller grids), then one decoder launch
// per kernel class on its own stream, then the BCH check of every frame.
int enqueue(cusat_batch* b, int n, cudaStream_t s, cusat::FrameDesc* d_frames, cusat::BchFrame* d_bch,
            cusat::DemapFrame* d_demap, bool copy)
{
    if (copy) {
        CU(cudaMemcpyAsync(d_frames, b->h_frames, (size_t)n * sizeof(cusat::FrameDesc), cudaMemcpyHostToDevice, s),
           "cudaMemcpyAsync(frames)");
        CU(cudaMemcpyAsync(d_bch, b->h_bch, (size_t)n * sizeof(cusat::BchFrame), cudaMemcpyHostToDevice, s),
           "cudaMemcpyAsync(bch frames)");
        CU(cudaMemcpyAsync(d_demap, b->h_demap, (size_t)n * sizeof(cusat::DemapFrame), cudaMemcpyHostToDevice, s),
           "cudaMemcpyAsync(demap frames)");
    }
    const int dr = cusat::launch_demap_mixed(b->d_demap_params, d_demap, n, b->max_len, s);
    if (dr)
        return cuda_fail((cudaError_t)dr, "demap launch");
    CU(cudaEventRecord(b->fork, s), "cudaEventRecord");
    for (int k : b->order) {
        KernelClass& c = b->classes[k];
        const int cnt = b->class_count[k];
        if (!cnt)
            continue;
        CU(cudaStreamWaitEvent(c.stream, b->fork, 0), "cudaStreamWaitEvent");
        cusat::DecodeArgs a = c.proto;
        a.frames = d_frames + b->class_off[k];
        a.n_frames = cnt;
        int grid = c.grid > 0 ? c.grid : c.grid_max;
        grid = std::min(grid, std::min(cnt, c.grid_max));
        if (b->max_ctas > 0)
            grid = std::min(grid, b->max_ctas);
        const int rc = cusat::launch_decoder(c.fn, a, grid, c.threads, c.stream);
        if (rc)
            return cuda_fail((cudaError_t)rc, "decoder launch");
        CU(cudaEventRecord(c.done, c.stream), "cudaEventRecord");
        CU(cudaStreamWaitEvent(s, c.done, 0), "cudaStreamWaitEvent");
    }
    const int rc = cusat::launch_bch_check_mixed(b->d_bch_codes, d_bch, n, s);
    if (rc)
        return cuda_fail((cudaError_t)rc, "BCH launch");
    CU(cudaEventRecord(b->last, s), "cudaEventRecord(last launch)");
    b->launched = true;
    return CUSAT_OK;
}

}  // namespace

extern "C" {

int cusat_batch_create(const int32_t* modcods, int n_modcods, int max_trials, int max_frames, cusat_batch** out)
{
    if (!out || !modcods || n_modcods <= 0 || n_modcods > 256 || max_frames <= 0 || max_trials < 0 ||
        max_trials > 1000)
        return fail(CUSAT_ERR_ARG, "invalid batch arguments");
    *out = nullptr;
    int dev;
    int rc = require_device(&dev);
    if (rc)
        return rc;
    cusat_batch* b = new cusat_batch();
    b->max_trials = max_trials;
    b->max_frames = max_frames;
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    std::map<std::pair<int, int>, int> class_of;
    for (int i = 0; i < n_modcods && rc == CUSAT_OK; i++) {
        auto m = std::make_unique<ModcodObj>();
        m->mod = modcods[3 * i];
        m->rate = modcods[3 * i + 1];
        m->fs = modcods[3 * i + 2];
        std::string err;
        m->plan = cusat::get_code_plan(m->fs, m->rate, &err);
        if (!m->plan) {
            rc = fail(CUSAT_ERR_UNSUPPORTED, err);
            break;
        }
        rc = upload_plan(*m->plan, &m->dp);
        if (rc == CUSAT_OK)
            rc = m->dm.init(m->mod, m->rate, m->fs);
        if (rc == CUSAT_OK)
            rc = m->bch.init(m->plan->gen, m->plan->p, (unsigned)(m->plan->n_bch / 8));
        if (rc)
            break;
        const auto key = std::make_pair(m->plan->cmax, m->plan->lanes);
        if (!class_of.count(key)) {
            class_of[key] = (int)b->classes.size();
            KernelClass c;
            c.cmax = key.first;
            c.lanes = key.second;
            b->classes.push_back(c);
        }
        m->cls = class_of[key];
        m->code_in_class = (int)b->classes[m->cls].modcods.size();
        b->classes[m->cls].modcods.push_back(i);
        b->modcods.push_back(std::move(m));
    }
    // per class: kernel, shared-memory layout for its largest code, tables,
    // message scratch for every resident CTA, stream
    for (size_t k = 0; k < b->classes.size() && rc == CUSAT_OK; k++) {
        KernelClass& c = b->classes[k];
        cusat::SmemDims dims{0, 0, 0, 0, c.cmax, c.lanes};
        size_t msg_cta = 0;
        std::vector<cusat::DevCode> codes;
        for (int mi : c.modcods) {
            const ModcodObj& m = *b->modcods[mi];
            const cusat::DevCode& dc = m.dp.code;
            dims.N = std::max(dims.N, dc.N);
            dims.q = std::max(dims.q, dc.q);
            dims.n_steps = std::max(dims.n_steps, dc.n_steps);
            dims.n_items = std::max(dims.n_items, dc.n_items);
            msg_cta = std::max(msg_cta, (size_t)dc.R * dc.msg_row);
            codes.push_back(dc);
        }
        c.fn = cusat::select_decoder_kernel(c.cmax, c.lanes);
        c.threads = cusat::decoder_threads(c.lanes);
        memset(&c.proto, 0, sizeof(c.proto));
        c.proto.max_trials = max_trials;
        c.proto.syn_period = cusat::syndrome_period();
        cusat::decoder_smem_layout(&c.proto, dims);
        if (!c.fn || c.proto.sm_total > optin) {
            rc = fail(CUSAT_ERR_UNSUPPORTED, "no decoder kernel fits this MODCOD");
            break;
        }
        cudaError_t e = allow_full_smem(c.fn);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_sm, c.fn, c.threads, c.proto.sm_total);
        // no launch runs more CTAs than frames: message scratch for at most max_frames
        c.grid_max = std::min(c.per_sm * b->sms, max_frames);
        if (e == cudaSuccess)
            e = cudaMalloc(&c.d_codes, codes.size() * sizeof(cusat::DevCode));
        if (e == cudaSuccess)
            e = cudaMemcpy(c.d_codes, codes.data(), codes.size() * sizeof(cusat::DevCode), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMalloc(&c.msg, (size_t)c.grid_max * msg_cta);
        if (e == cudaSuccess)
            e = cudaMalloc(&c.queue, 256);
        if (e == cudaSuccess)
            e = cudaMemset(c.queue, 0, 256);  // the decoder rearms it after each launch
        if (e == cudaSuccess)
            e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "batch class set-up");
            break;
        }
        c.proto.codes = c.d_codes;
        c.proto.msg = c.msg;
        c.proto.msg_stride = (int)(msg_cta / 16);
        c.proto.queue = c.queue;
        b->order.push_back((int)k);
    }
    if (rc == CUSAT_OK) {
        std::vector<cusat::BchDev> bch;
        std::vector<cusat::DevDemap> demaps;
        for (auto& m : b->modcods) {
            bch.push_back(m->bch.d);
            demaps.push_back(m->dm.d);
            b->max_n = std::max(b->max_n, m->plan->N);
            b->max_len = std::max(b->max_len, m->dm.m.interleaved_len);
        }
        b->max_n = (b->max_n + 7) & ~7;  // 16-byte aligned LLR rows
        cudaError_t e = cudaMallocHost(&b->h_frames, (size_t)max_frames * sizeof(cusat::FrameDesc));
        if (e == cudaSuccess)
            e = cudaMallocHost(&b->h_demap, (size_t)max_frames * sizeof(cusat::DemapFrame));
        if (e == cudaSuccess)
            e = cudaMalloc(&b->d_demap, (size_t)max_frames * sizeof(cusat::DemapFrame));
        if (e == cudaSuccess)
            e = cudaMalloc(&b->d_demap_params, demaps.size() * sizeof(cusat::DevDemap));
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_demap_params, demaps.data(), demaps.size() * sizeof(cusat::DevDemap),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMalloc(&b->llr, (size_t)max_frames * b->max_n * sizeof(int16_t));
        if (e == cudaSuccess)
            e = cudaMallocHost(&b->h_bch, (size_t)max_frames * sizeof(cusat::BchFrame));
        if (e == cudaSuccess)
            e = cudaMalloc(&b->d_frames, (size_t)max_frames * sizeof(cusat::FrameDesc));
        if (e == cudaSuccess)
            e = cudaMalloc(&b->d_bch, (size_t)max_frames * sizeof(cusat::BchFrame));
        if (e == cudaSuccess)
            e = cudaMalloc(&b->d_bch_codes, bch.size() * sizeof(cusat::BchDev));
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_bch_codes, bch.data(), bch.size() * sizeof(cusat::BchDev), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&b->last, cudaEventDisableTiming);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "batch buffers");
    }
    if (rc != CUSAT_OK) {
        release(b);
        return rc;
    }
    *out = b;
    return CUSAT_OK;
}

void cusat_batch_destroy(cusat_batch* b) { release(b); }

int cusat_batch_info(const cusat_batch* b, int32_t* out)
{
    if (!b || !out)
        return fail(CUSAT_ERR_ARG, "null argument");
    out[0] = (int32_t)b->modcods.size();
    out[1] = (int32_t)b->classes.size();
    out[2] = b->max_frames;
    out[3] = b->max_trials;
    return CUSAT_OK;
}

int cusat_batch_set_weights(cusat_batch* b, int modcod, const int16_t* weights, int n_iter)
{
    if (!b || modcod < 0 || modcod >= (int)b->modcods.size())
        return fail(CUSAT_ERR_ARG, "unknown MODCOD index");
    ModcodObj& m = *b->modcods[modcod];
    cusat::DevCode dc = m.dp.code;
    // this batch's last launch or replay still reads the tables; other
    // streams of the application are not waited for
    int rc = wait_last_launch(b->last, b->launched);
    if (rc)
        return rc;
    if (weights) {
        rc = m.weights.set(weights, n_iter, b->max_trials);
        if (rc)
            return rc;
        dc.weights = m.weights.d;
    }
    KernelClass& c = b->classes[m.cls];
    return m.weights.upload(c.d_codes + m.code_in_class, &dc, sizeof(dc));
}

}  // extern "C"

namespace cusat_internal {

// Launch for callers that know the object's previous launch has completed
// (its staging buffers are free): no stream synchronisation.
int batch_launch_ready(cusat_batch* b, const cusat_frame* frames, int n, cudaStream_t stream)
{
    if (!b || !frames || n <= 0 || n > b->max_frames)
        return fail(CUSAT_ERR_ARG, "frames outside 1..max_frames");
    const int rc = stage(b, frames, n);
    if (rc)
        return rc;
    return enqueue(b, n, stream, b->d_frames, b->d_bch, b->d_demap, true);
}

}  // namespace cusat_internal

extern "C" {

int cusat_batch_launch(cusat_batch* b, const cusat_frame* frames, int n, void* stream)
{
    if (!b || !frames || n <= 0 || n > b->max_frames)
        return fail(CUSAT_ERR_ARG, "frames outside 1..max_frames");
    // the staging buffers are read by the copies of the previous launch
    CU(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
    int rc = stage(b, frames, n);
    if (rc)
        return rc;
    return enqueue(b, n, (cudaStream_t)stream, b->d_frames, b->d_bch, b->d_demap, true);
}

int cusat_batch_capture(cusat_batch* b, const cusat_frame* frames, int n, void* stream)
{
    if (!b || !frames || n <= 0 || n > b->max_frames)
        return fail(CUSAT_ERR_ARG, "frames outside 1..max_frames");
    cudaStream_t s = (cudaStream_t)stream;
    if (!s)
        return fail(CUSAT_ERR_ARG, "graph capture needs a created stream");
    CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    int rc = stage(b, frames, n);
    if (rc)
        return rc;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->g_frames) {
        CU(cudaMalloc(&b->g_frames, (size_t)b->max_frames * sizeof(cusat::FrameDesc)), "cudaMalloc(graph frames)");
        CU(cudaMalloc(&b->g_bch, (size_t)b->max_frames * sizeof(cusat::BchFrame)), "cudaMalloc(graph frames)");
        CU(cudaMalloc(&b->g_demap, (size_t)b->max_frames * sizeof(cusat::DemapFrame)), "cudaMalloc(graph frames)");
    }
    CU(cudaMemcpy(b->g_frames, b->h_frames, (size_t)n * sizeof(cusat::FrameDesc), cudaMemcpyHostToDevice),
       "cudaMemcpy(graph frames)");
    CU(cudaMemcpy(b->g_bch, b->h_bch, (size_t)n * sizeof(cusat::BchFrame), cudaMemcpyHostToDevice),
       "cudaMemcpy(graph frames)");
    CU(cudaMemcpy(b->g_demap, b->h_demap, (size_t)n * sizeof(cusat::DemapFrame), cudaMemcpyHostToDevice),
       "cudaMemcpy(graph frames)");
    CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    rc = enqueue(b, n, s, b->g_frames, b->g_bch, b->g_demap, false);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc)
        return rc;
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t e2 = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess)
        return cuda_fail(e2, "cudaGraphInstantiate");
    b->graph_frames = n;
    return CUSAT_OK;
}

int cusat_batch_replay(cusat_batch* b, void* stream)
{
    if (!b || !b->graph)
        return fail(CUSAT_ERR_ARG, "no captured batch");
    CU(cudaGraphLaunch(b->graph, (cudaStream_t)stream), "cudaGraphLaunch");
    CU(cudaEventRecord(b->last, (cudaStream_t)stream), "cudaEventRecord(last launch)");
    b->launched = true;
    return CUSAT_OK;
}

int cusat_batch_set_max_ctas(cusat_batch* b, int max_ctas)
{
    if (!b || max_ctas < 0)
        return fail(CUSAT_ERR_ARG, "null batch or negative CTA cap");
    b->max_ctas = max_ctas;
    return CUSAT_OK;
}

int cusat_batch_tune(cusat_batch* b, const cusat_frame* frames, int n, int reps, void* stream, float* best_ms)
{
    if (!b || !frames || n <= 0 || n > b->max_frames || reps <= 0)
        return fail(CUSAT_ERR_ARG, "invalid tuning arguments");
    cudaStream_t s = (cudaStream_t)stream;
    CU(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    int rc = stage(b, frames, n);
    if (rc)
        return rc;
    const int nc = (int)b->classes.size();
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0), "cudaEventCreate");
    CU(cudaEventCreate(&e1), "cudaEventCreate");
    // mean time of reps launch sequences (one untimed first: caches, clocks)
    auto time_seq = [&](float* ms_out) -> int {
        float sum = 0;
        for (int r = 0; r <= reps; r++) {
            CU(cudaEventRecord(e0, s), "cudaEventRecord");
            const int rc2 = enqueue(b, n, s, b->d_frames, b->d_bch, b->d_demap, true);
            if (rc2)
                return rc2;
            CU(cudaEventRecord(e1, s), "cudaEventRecord");
            CU(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0;
            CU(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            if (r > 0)
                sum += ms;
        }
        *ms_out = sum / reps;
        return CUSAT_OK;
    };
    std::vector<int> saved_grid(nc);
    for (int k = 0; k < nc; k++)
        saved_grid[k] = b->classes[k].grid;
    // 1. each class's decoder alone on its full grid (its LLRs are in place
    // after one full sequence): the measured cost that orders the classes
    std::vector<float> solo(nc, 0.0f);
    float ms0 = 0;
    rc = time_seq(&ms0);
    for (int k = 0; k < nc && rc == CUSAT_OK; k++) {
        KernelClass& c = b->classes[k];
        const int cnt = b->class_count[k];
        if (!cnt)
            continue;
        cusat::DecodeArgs a = c.proto;
        a.frames = b->d_frames + b->class_off[k];
        a.n_frames = cnt;
        const int grid = std::min(cnt, c.grid_max);
        float sum = 0;
        for (int r = 0; r <= reps; r++) {
            cudaEventRecord(e0, s);
            const int lr = cusat::launch_decoder(c.fn, a, grid, c.threads, s);
            if (lr) {
                rc = cuda_fail((cudaError_t)lr, "decoder launch");
                break;
            }
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0)
                sum += ms;
        }
        solo[k] = sum / reps;
    }
    // 2. candidates: class order x grid rule.  Rules 0-3 make each persistent
    // CTA decode f = 1, 2, 3, 4 frames of its class (grid = count / f, at
    // most the resident slots); rule 4 shares the SMs in proportion to the
    // classes' measured cost
    std::vector<int> by_cost(nc), by_cost_rev;
    for (int k = 0; k < nc; k++)
        by_cost[k] = k;
    std::sort(by_cost.begin(), by_cost.end(), [&](int x, int y) { return solo[x] > solo[y]; });
    by_cost_rev.assign(by_cost.rbegin(), by_cost.rend());
    double total = 0;
    for (float v : solo)
        total += v;
    auto frames_per_cta = [&](int k, int f) {
        const int cnt = b->class_count[k];
        return std::max(1, std::min(b->classes[k].grid_max, (cnt + f - 1) / f));
    };
    auto set_rule = [&](int rule) {
        for (int k = 0; k < nc; k++) {
            KernelClass& c = b->classes[k];
            if (rule <= 3) {
                c.grid = frames_per_cta(k, rule + 1);
            } else {
                const double share = total > 0 ? solo[k] / total : 1.0;
                c.grid = std::max(1, (int)(share * c.grid_max + 0.5));
            }
        }
    };
    float best = 1e30f;
    std::vector<int> best_order = by_cost, best_grid(nc, 0);
    const std::vector<int>* orders[] = {&by_cost, &by_cost_rev};
    for (int oi = 0; oi < 2 && rc == CUSAT_OK; oi++) {
        for (int rule = 0; rule < 5 && rc == CUSAT_OK; rule++) {
            b->order = *orders[oi];
            set_rule(rule);
            float ms = 0;
            if ((rc = time_seq(&ms)) != CUSAT_OK)
                break;
            if (ms < best) {
                best = ms;
                best_order = b->order;
                for (int k = 0; k < nc; k++)
                    best_grid[k] = b->classes[k].grid;
            }
        }
    }
    // 3. per class, costliest first: frames per CTA in {1, 2, 3, 4, 6, 8}
    // with the others fixed, kept when it gains at least 0.5 %
    b->order = best_order;
    for (int k = 0; k < nc; k++)
        b->classes[k].grid = best_grid[k];
    for (int oi = 0; oi < nc && rc == CUSAT_OK; oi++) {
        const int k = by_cost[oi];
        if (!b->class_count[k])
            continue;
        const int keep = b->classes[k].grid;
        int best_g = keep;
        for (int f : {1, 2, 3, 4, 6, 8}) {
            const int g = frames_per_cta(k, f);
            if (g == keep)
                continue;
            b->classes[k].grid = g;
            float ms = 0;
            if ((rc = time_seq(&ms)) != CUSAT_OK)
                break;
            if (ms < best * 0.995f) {
                best = ms;
                best_g = g;
            }
        }
        b->classes[k].grid = best_g;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        for (int k = 0; k < nc; k++)
            b->classes[k].grid = saved_grid[k];
        return rc;
    }
    for (int k = 0; k < nc; k++)
        b->classes[k].tuned_ms = solo[k];
    if (best_ms)
        *best_ms = best;
    return CUSAT_OK;
}

int cusat_batch_tuned(const cusat_batch* b, int32_t* out, float* solo_ms, int max_classes)
{
    if (!b || !out || max_classes < 0)
        return fail(CUSAT_ERR_ARG, "null argument");
    const int nc = (int)b->classes.size();
    for (int k = 0; k < nc && k < max_classes; k++) {
        const KernelClass& c = b->classes[k];
        int pos = -1;
        for (int o = 0; o < (int)b->order.size(); o++)
            if (b->order[o] == k)
                pos = o;
        out[5 * k + 0] = c.cmax;
        out[5 * k + 1] = c.lanes;
        const int cnt = k < (int)b->class_count.size() ? b->class_count[k] : 0;
        const int grid = std::min(c.grid > 0 ? c.grid : c.grid_max, c.grid_max);
        out[5 * k + 2] = cnt;
        out[5 * k + 3] = cnt > 0 ? std::min(grid, cnt) : grid;  // what a launch of these frames uses
        out[5 * k + 4] = pos;
        if (solo_ms)
            solo_ms[k] = c.tuned_ms;
    }
    return nc;
}

}  // extern "C"
