// LDPC decode entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a real-time receive thread that runs
// under a no-allocation rule once the link is up, a process whose device
// memory pool is owned by another runtime, or a host application that manages
// every device allocation itself and forbids libraries to allocate behind its
// back.  cusat_ldpc_decode_noalloc serves
// them: the caller passes the LLRs and the output buffers, and everything the
// decoder needs besides -- the code's decoding tables, the check-to-bit
// message rows of every CTA, the frame counter -- lives in the file-scope
// device arrays below, which exist on every GPU that loads the library for as
// long as the process lives.
//
// Limits: the message area holds kNoallocMsgBytes; the number of CTAs is
// bounded by it (for normal-frame rate 3/5, 24 MiB holds 60 CTAs' message
// rows), so the decoder may use fewer SMs than the allocating path.  The
// table area holds kNoallocPlanBytes, enough for every DVB-S2/S2X code.
//
// All calls on a device share that device's copy of these arrays: two calls
// whose kernels overlap on the GPU (for instance on two streams) race on
// them.  Every call looks up the arrays' device addresses on the current
// device (cheap, and still right after cudaDeviceReset has reloaded the
// module) and copies its code's tables into the table area ahead of the
// decode, on the caller's stream: at most 64 KiB from a static host buffer,
// a copy and not an allocation.  No host-side record says which code the
// table area holds, so calls for different codes in a row on one stream are
// always decoded with their own tables.  A call on a stream that is being
// captured into a CUDA graph is refused (CUSAT_ERR_UNSUPPORTED) and enqueues
// nothing: a recorded table copy would read the static host buffer when the
// graph runs, by which time another call may have refilled it.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>
#include <string>

#include "../../include/cusat_fec.h"
#include "host.h"
#include "kernels.h"
#include "ldpc_kernel.cuh"

namespace {

constexpr size_t kNoallocMsgBytes = 24u << 20;
constexpr size_t kNoallocPlanBytes = 64u << 10;

static __device__ __align__(256) unsigned char g_noalloc_msg[kNoallocMsgBytes];
static __device__ __align__(256) unsigned char g_noalloc_plan[kNoallocPlanBytes];
static __device__ __align__(256) unsigned int g_noalloc_queue[64];

// Host staging of the tables of the call in progress (guarded by g_mu).
static unsigned char g_plan_host[kNoallocPlanBytes];

struct DeviceState {
    unsigned char* msg = nullptr;    // device address of g_noalloc_msg on this device
    unsigned char* plan = nullptr;   // ... of g_noalloc_plan
    unsigned int* queue = nullptr;   // ... of g_noalloc_queue
    int sms = 0, optin = 0;
};

std::mutex g_mu;

// errors are reported through cusat_last_error(), like every entry point
int fail(int code, const std::string& msg)
{
    cusat::set_last_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    cusat::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return CUSAT_ERR_CUDA;
}

// With the device current: the arrays' device addresses and its limits
// (looked up on every call).
int setup_device(int dev, DeviceState* st)
{
    cudaError_t e = cudaGetSymbolAddress((void**)&st->msg, g_noalloc_msg);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetSymbolAddress(message area)");
    e = cudaGetSymbolAddress((void**)&st->plan, g_noalloc_plan);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetSymbolAddress(table area)");
    e = cudaGetSymbolAddress((void**)&st->queue, g_noalloc_queue);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetSymbolAddress(frame counter)");
    e = cudaDeviceGetAttribute(&st->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&st->optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaDeviceGetAttribute");
    return CUSAT_OK;
}

}  // namespace

extern "C" {

int cusat_ldpc_decode_noalloc(int framesize, int rate, int max_trials, const int16_t* soft_dev, int batch,
                              uint8_t* hard_out, int32_t* trials_out, void* stream)
{
    if (!soft_dev || !hard_out || !trials_out)
        return fail(CUSAT_ERR_ARG, "null buffer");
    if (batch <= 0 || max_trials < 0 || max_trials > 1000)
        return fail(CUSAT_ERR_ARG, "batch must be >= 1 and max_trials 0..1000");
    std::string err;
    const cusat::CodePlan* p = cusat::get_code_plan(framesize, rate, &err);
    if (!p)
        return fail(CUSAT_ERR_UNSUPPORTED, err);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaStreamIsCapturing");
    if (cap != cudaStreamCaptureStatusNone)
        return fail(CUSAT_ERR_UNSUPPORTED, "cusat_ldpc_decode_noalloc cannot be recorded into a CUDA graph");

    std::lock_guard<std::mutex> lock(g_mu);
    DeviceState st;
    {
        const int rc = setup_device(dev, &st);
        if (rc)
            return rc;
    }

    // tables of the code, laid out like the allocating path's
    struct Part { const void* src; size_t n; size_t off; };
    Part parts[] = {
        {p->tab.data(), p->tab.size() * 4, 0},           {p->sched.data(), p->sched.size() * 2, 0},
        {p->step_conf.data(), p->step_conf.size(), 0},   {p->item_off.data(), p->item_off.size() * 2, 0},
        {p->items.data(), p->items.size() * 4, 0},
    };
    size_t total = 0;
    for (auto& pt : parts) {
        pt.off = total;
        total += (pt.n + 255) & ~(size_t)255;
    }
    if (total > kNoallocPlanBytes)
        return fail(CUSAT_ERR_ARG, "decoding tables exceed the 64 KiB table area");
    const size_t per_cta = (size_t)p->R * p->msg_row;
    if (per_cta > kNoallocMsgBytes)
        return fail(CUSAT_ERR_ARG, "message rows of one frame exceed the 24 MiB message area");
    memset(g_plan_host, 0, total);
    for (auto& pt : parts)
        if (pt.n)
            memcpy(&g_plan_host[pt.off], pt.src, pt.n);
    // pageable source: the driver has staged the bytes when the call returns,
    // so the next call may refill g_plan_host
    e = cudaMemcpyAsync(st.plan, g_plan_host, total, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemcpyAsync(tables)");

    cusat::DecodeArgs a;
    memset(&a, 0, sizeof(a));
    cusat::DevCode& c = a.code;
    c.N = p->N;
    c.K = p->K;
    c.R = p->R;
    c.q = p->q;
    c.n_steps = p->n_steps;
    c.cmax = p->cmax;
    c.fast_lim = p->fast_lim;
    c.msg_row = p->msg_row;
    c.n_items = (int)(p->items.size() / 2);
    c.tab = (const uint4*)(st.plan + parts[0].off);
    c.sched = (const int16_t*)(st.plan + parts[1].off);
    c.step_conf = st.plan + parts[2].off;
    c.item_off = (const uint16_t*)(st.plan + parts[3].off);
    c.items = (const uint2*)(st.plan + parts[4].off);
    a.llr = soft_dev;
    a.n_frames = batch;
    a.max_trials = max_trials;
    a.syn_period = cusat::syndrome_period();
    a.hard = hard_out;
    a.trials = trials_out;
    a.msg = (uint4*)st.msg;
    a.msg_stride = p->R * p->msg_row / 16;
    a.queue = st.queue;
    cusat::decoder_smem_layout(&a, cusat::smem_dims_of(a.code, p->lanes));
    if (a.sm_total > st.optin)
        return fail(CUSAT_ERR_UNSUPPORTED, "frame state does not fit in shared memory");
    const void* fn = cusat::select_decoder_kernel(p->cmax, p->lanes);
    if (!fn)
        return fail(CUSAT_ERR_UNSUPPORTED, "no decoder kernel for this check degree");
    // the cap is shared by every object launching this kernel: raise it to
    // the device limit, never lower it
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, st.optin);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaFuncSetAttribute");
    int per_sm = 0;
    const int threads = cusat::decoder_threads(p->lanes);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, a.sm_total);
    if (e != cudaSuccess)
        return cuda_fail(e, "occupancy");
    int grid = per_sm * st.sms;
    const int fit = (int)(kNoallocMsgBytes / per_cta);
    if (grid > fit)
        grid = fit;
    if (grid > batch)
        grid = batch;
    if (grid < 1)
        return fail(CUSAT_ERR_UNSUPPORTED, "decoder kernel cannot be resident");
    // frame and exit counters start at zero (the kernel also rearms them on
    // exit; zeroed here as well since nothing else owns these arrays)
    e = cudaMemsetAsync(st.queue, 0, 2 * sizeof(unsigned int), s);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemsetAsync(frame counter)");
    const int rc = cusat::launch_decoder(fn, a, grid, threads, s);
    if (rc != 0)
        return cuda_fail((cudaError_t)rc, "decoder launch");
    return CUSAT_OK;
}

}  // extern "C"
