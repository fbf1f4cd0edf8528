// Device-side objects shared by the C ABI entry points (internal).
#pragma once

#include <cuda_runtime.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/cusat_fec.h"
#include "host.h"
#include "kernels.h"
#include "ldpc_kernel.cuh"

namespace cusat_internal {

inline int fail(int code, const std::string& msg)
{
    cusat::set_last_error(msg);
    return code;
}

inline int cuda_fail(cudaError_t e, const char* what)
{
    cusat::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return CUSAT_ERR_CUDA;
}

#define CU(call, what)                          \
    do {                                        \
        cudaError_t e_ = (call);                \
        if (e_ != cudaSuccess)                  \
            return cuda_fail(e_, what);         \
    } while (0)

inline int require_device(int* dev)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(CUSAT_ERR_NO_DEVICE, "no CUDA device");
    e = cudaGetDevice(dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    return CUSAT_OK;
}

// The dynamic shared-memory cap is a property of the kernel function shared
// by every object that launches it: objects raise it to the device's opt-in
// limit and never lower it, so one object's setting cannot make another's
// larger launch invalid.
inline cudaError_t allow_full_smem(const void* fn)
{
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    return e;
}

// Learned min-sum weights: validates n_iter rows of [32][2] {beta, alpha in
// 64ths} and expands them to `rows` rows (later rows repeat the last one).
inline int weight_table(const int16_t* w, int n_iter, int rows, std::vector<int16_t>* out)
{
    if (!w || n_iter <= 0)
        return fail(CUSAT_ERR_ARG, "weights need at least one iteration row");
    for (int i = 0; i < n_iter * 32; i++)
        if (w[2 * i] < 0 || w[2 * i] > 127 || w[2 * i + 1] < 0 || w[2 * i + 1] > 255)
            return fail(CUSAT_ERR_ARG, "weight outside beta 0..127, alpha 0..255");
    rows = rows < 1 ? 1 : rows;
    out->resize((size_t)rows * 64);
    for (int t = 0; t < rows; t++)
        memcpy(out->data() + (size_t)t * 64, w + (size_t)(t < n_iter ? t : n_iter - 1) * 64, 64 * sizeof(int16_t));
    return CUSAT_OK;
}

// Waits for the work an event marks, if it was ever recorded: replacing a
// table waits for the owning object's last launch, not for the device.
inline int wait_last_launch(cudaEvent_t ev, bool recorded)
{
    if (ev && recorded)
        CU(cudaEventSynchronize(ev), "cudaEventSynchronize(last launch)");
    return CUSAT_OK;
}

// Device weight table of one code ([max(1, max_trials)][32][2] int16, one
// allocation made on the first set); set() replaces its contents.  Callers
// first wait for their own last launch that reads it (wait_last_launch); the
// copy runs on a private non-blocking stream, so other streams of the
// application are not stalled.
struct DevWeights {
    int16_t* d = nullptr;
    int rows = 0;
    cudaStream_t up = nullptr;

    int set(const int16_t* w, int n_iter, int max_trials)
    {
        std::vector<int16_t> tab;
        int rc = weight_table(w, n_iter, max_trials, &tab);
        if (rc)
            return rc;
        if (!d) {
            CU(cudaMalloc(&d, tab.size() * sizeof(int16_t)), "cudaMalloc(weights)");
            rows = (int)tab.size() / 64;
        }
        if (!up)
            CU(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking), "cudaStreamCreate(weights)");
        CU(cudaMemcpyAsync(d, tab.data(), tab.size() * sizeof(int16_t), cudaMemcpyHostToDevice, up),
           "cudaMemcpyAsync(weights)");
        CU(cudaStreamSynchronize(up), "cudaStreamSynchronize(weights)");
        return CUSAT_OK;
    }
    // copies one host object to device memory on the private stream
    int upload(void* dst, const void* src, size_t n)
    {
        if (!up)
            CU(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking), "cudaStreamCreate(weights)");
        CU(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, up), "cudaMemcpyAsync(code)");
        CU(cudaStreamSynchronize(up), "cudaStreamSynchronize(code)");
        return CUSAT_OK;
    }
    void release()
    {
        if (d)
            cudaFree(d);
        if (up)
            cudaStreamDestroy(up);
        d = nullptr;
        up = nullptr;
        rows = 0;
    }
};

// Device copy of a code plan (one allocation).
struct DevPlan {
    void* blob = nullptr;
    cusat::DevCode code{};
};

inline int upload_plan(const cusat::CodePlan& p, DevPlan* d)
{
    struct Part { const void* src; size_t n; size_t off; };
    Part parts[] = {
        {p.tab.data(), p.tab.size() * 4, 0},           {p.sched.data(), p.sched.size() * 2, 0},
        {p.step_conf.data(), p.step_conf.size(), 0},   {p.item_off.data(), p.item_off.size() * 2, 0},
        {p.items.data(), p.items.size() * 4, 0},
    };
    size_t total = 0;
    for (auto& pt : parts) {
        pt.off = total;
        total += (pt.n + 255) & ~(size_t)255;
    }
    std::vector<unsigned char> h(total + 256, 0);
    for (auto& pt : parts)
        if (pt.n)
            memcpy(&h[pt.off], pt.src, pt.n);
    CU(cudaMalloc(&d->blob, total + 256), "cudaMalloc(plan)");
    CU(cudaMemcpy(d->blob, h.data(), total + 256, cudaMemcpyHostToDevice), "cudaMemcpy(plan)");
    unsigned char* b = (unsigned char*)d->blob;
    cusat::DevCode& c = d->code;
    c.N = p.N;
    c.K = p.K;
    c.R = p.R;
    c.q = p.q;
    c.n_steps = p.n_steps;
    c.cmax = p.cmax;
    c.fast_lim = p.fast_lim;
    c.msg_row = p.msg_row;
    c.n_items = (int)(p.items.size() / 2);
    c.tab = (const uint4*)(b + parts[0].off);
    c.sched = (const int16_t*)(b + parts[1].off);
    c.step_conf = b + parts[2].off;
    c.item_off = (const uint16_t*)(b + parts[3].off);
    c.items = (const uint2*)(b + parts[4].off);
    return CUSAT_OK;
}

struct DevBch {
    cusat::BchTables t;
    void* blob = nullptr;
    cusat::BchDev d{};

    int init(const uint64_t* gen, int p, unsigned n_bytes)
    {
        std::string err;
        if (!cusat::build_bch_tables(gen, p, n_bytes, &t, &err))
            return fail(CUSAT_ERR_ARG, err);
        const size_t nl = t.lut.size() * 8, nt = t.tree.size() * 8;
        CU(cudaMalloc(&blob, nl + nt), "cudaMalloc(bch)");
        CU(cudaMemcpy(blob, t.lut.data(), nl, cudaMemcpyHostToDevice), "cudaMemcpy(bch)");
        CU(cudaMemcpy((char*)blob + nl, t.tree.data(), nt, cudaMemcpyHostToDevice), "cudaMemcpy(bch)");
        d.p = t.p;
        d.words = t.words;
        d.n_bytes = t.n_bytes;
        d.chunk = t.chunk;
        d.lead = t.lead;
        d.lut = (const uint64_t*)blob;
        d.tree = (const uint64_t*)((char*)blob + nl);
        return CUSAT_OK;
    }
    void release()
    {
        if (blob)
            cudaFree(blob);
        blob = nullptr;
    }
};

struct DevDemapObj {
    cusat::ModcodDemap m;
    float2* pts = nullptr;
    cusat::DevDemap d{};

    int init(int mod, int rate, int fs)
    {
        std::string err;
        if (!cusat::build_modcod_demap(mod, rate, fs, &m, &err))
            return fail(CUSAT_ERR_UNSUPPORTED, err);
        CU(cudaMalloc(&pts, m.pts.size() * 4), "cudaMalloc(points)");
        CU(cudaMemcpy(pts, m.pts.data(), m.pts.size() * 4, cudaMemcpyHostToDevice), "cudaMemcpy(points)");
        d.kind = m.kind;
        d.n_mod = m.n_mod;
        d.n_points = m.n_points;
        d.xfec = m.xfec;
        d.interleaved_len = m.interleaved_len;
        d.fec_len = m.fec_len;
        for (int b = 0; b < 8; b++)
            d.col[b] = m.col[b];
        d.points = pts;
        return CUSAT_OK;
    }
    void release()
    {
        if (pts)
            cudaFree(pts);
        pts = nullptr;
    }
};

// Mixed-MODCOD batch launch without the stream synchronisation of
// cusat_batch_launch (batch.cu); the caller guarantees that the object's
// previous launch has completed.
int batch_launch_ready(cusat_batch* b, const cusat_frame* frames, int n, cudaStream_t stream);

}  // namespace cusat_internal
