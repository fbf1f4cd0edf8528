/*
 * The reference's own GPU kernels on this GPU -- TEST INFRASTRUCTURE ONLY.
 *
 * oracle/build.py compiles the reference's demapper and layered decoder
 * sources unchanged (lib/cusat_dsp/cuda/demapper_kernel.cu,
 * lib/cusat_dsp/cuda/ldpc_decode_kernel.cu) into cubins under oracle/_ref/
 * with the reference's Release flags for sm_103, where the reference tree is
 * present.  This file loads those cubins through the CUDA driver API and
 * launches the kernels the way the reference's host classes do:
 *
 *   - decoder: the tables of ldpc_decode_cuda's constructor
 *     (ldpc_decode_kernel.cu:991-1063: pos[] per check, transposed
 *     edge-major per layer, one edge count per layer, message-block offsets
 *     M * (cnt + 2) per layer), its schedule buffer (:1115-1170: 140 x 2
 *     int16, zeroed, the table's blossom schedule when its layer count
 *     matches the code, else one layer per step) and its launch
 *     (:1198-1285: one 720-thread block per frame, (K + R) * 2 + 4 bytes of
 *     dynamic shared memory, syndrome period 1, hard decisions fused);
 *   - demapper: demapper_cuda::demap_batch's launch (demapper_kernel.cu:
 *     293-330: 256-thread blocks over the interleaved length, one grid row
 *     per frame).
 *
 * The reference's L2 access-policy window on the decoder's global APP
 * buffer (:1207-1217) is not set: the shared-memory instance never reads
 * that buffer.  Nothing in the product links or loads this file; the tests
 * and oracle/ref_gpu_compare.py use it to hold the reference's kernels
 * against the oracle and to time them beside this project's kernels.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../cusat_gb300/csrc/cusat_data.h"
#include "../cusat_gb300/csrc/gen/code_tables.inc"

#define RG_M 360
#define RG_SCHED_MAX 140

/* entry-point names as ptxas lists them for the reference's sources */
static const char* kDecName =
    "_ZN9cusat_dsp4cuda26ldpc_decode_layered_kernelILb1EEEvPsS2_PaPKtPKhPKiPiPhiiiiiiiPKsiiSD_i";
static const char* kDemapName = "_ZN9cusat_dsp4cuda25demap_deinterleave_kernelEPKfPsS2_S2_iiiiijjjjjjjjff";

static CUmodule g_dec_mod, g_demap_mod;
static CUfunction g_dec_fn, g_demap_fn;
static char g_err[512];

const char* rg_last_error(void) { return g_err; }

static int fail_cu(CUresult r, const char* what)
{
    const char* s = 0;
    cuGetErrorString(r, &s);
    snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
    return -1;
}

#define CU(call, what)                      \
    do {                                    \
        CUresult r_ = (call);               \
        if (r_ != CUDA_SUCCESS)             \
            return fail_cu(r_, what);       \
    } while (0)

/* Loads both cubins into the primary context of device 0 (the context the
 * CUDA runtime of the calling process uses). */
int rg_open(const char* dec_cubin, const char* demap_cubin)
{
    if (g_dec_fn)
        return 0;
    CUdevice dev;
    CUcontext ctx;
    CU(cuInit(0), "cuInit");
    CU(cuDeviceGet(&dev, 0), "cuDeviceGet");
    CU(cuDevicePrimaryCtxRetain(&ctx, dev), "cuDevicePrimaryCtxRetain");
    CU(cuCtxSetCurrent(ctx), "cuCtxSetCurrent");
    CU(cuModuleLoad(&g_dec_mod, dec_cubin), "cuModuleLoad(decoder)");
    CU(cuModuleGetFunction(&g_dec_fn, g_dec_mod, kDecName), "cuModuleGetFunction(decoder)");
    CU(cuModuleLoad(&g_demap_mod, demap_cubin), "cuModuleLoad(demapper)");
    CU(cuModuleGetFunction(&g_demap_fn, g_demap_mod, kDemapName), "cuModuleGetFunction(demapper)");
    return 0;
}

typedef struct {
    int N, K, R, q, cnl, lt_alloc, n_steps, max_batch, max_trials;
    CUdeviceptr pos, cnc, layer_off, sched, data, pty, bnl;
    unsigned smem;
} rg_dec;

static const cusat_table_src* find_table(int framesize, int rate)
{
    const char* name = cusat_table_name(framesize, rate);
    if (!name)
        return 0;
    for (int i = 0; i < CUSAT_N_TABLE_SRCS; i++)
        if (!strcmp(cusat_table_srcs[i].name, name))
            return &cusat_table_srcs[i];
    return 0;
}

static const cusat_sched_src* find_sched(const char* name, int q)
{
    for (int i = 0; i < CUSAT_N_SCHED_SRCS; i++)
        if (!strcmp(cusat_sched_srcs[i].name, name) && cusat_sched_srcs[i].q == q)
            return &cusat_sched_srcs[i];
    return 0;
}

void rg_dec_destroy(rg_dec* d)
{
    if (!d)
        return;
    CUdeviceptr p[] = {d->pos, d->cnc, d->layer_off, d->sched, d->data, d->pty, d->bnl};
    for (unsigned i = 0; i < sizeof(p) / sizeof(p[0]); i++)
        if (p[i])
            cuMemFree(p[i]);
    free(d);
}

/* The decoder of one (framesize, rate) for up to max_batch frames; NULL on
 * error (rg_last_error). */
rg_dec* rg_dec_create(int framesize, int rate, int max_trials, int max_batch)
{
    const cusat_table_src* t = find_table(framesize, rate);
    if (!t || !g_dec_fn || max_batch <= 0) {
        snprintf(g_err, sizeof(g_err), "rg_dec_create: no table, no module or bad batch");
        return 0;
    }
    rg_dec* d = (rg_dec*)calloc(1, sizeof(rg_dec));
    d->N = t->n;
    d->K = t->k;
    d->R = d->N - d->K;
    d->q = d->R / RG_M;
    d->cnl = t->links_max_cn - 2;
    d->max_batch = max_batch;
    d->max_trials = max_trials;
    const int R = d->R, q = d->q, cnl = d->cnl;
    /* pos[] and edge counts per check: info bit j = row * M + jj meets
     * check (addr + jj * q) % R of each address of its row */
    uint16_t* pos_raw = (uint16_t*)calloc((size_t)R * cnl, sizeof(uint16_t));
    uint8_t* cnc_raw = (uint8_t*)calloc(R, 1);
    for (int row = 0, o = 0; row < t->n_rows; o += t->row_deg[row], row++)
        for (int jj = 0; jj < RG_M; jj++)
            for (int n = 0; n < t->row_deg[row]; n++) {
                const int i = ((int)t->addr[o + n] + jj * q) % R;
                pos_raw[cnl * i + cnc_raw[i]++] = (uint16_t)(row * RG_M + jj);
            }
    /* edge-major per layer: pos_t[(i * cnl + c) * M + j] = pos_raw[cnl * (q * j + i) + c] */
    uint16_t* pos_t = (uint16_t*)calloc((size_t)R * cnl, sizeof(uint16_t));
    for (int i = 0; i < q; i++)
        for (int j = 0; j < RG_M; j++)
            for (int c = 0; c < cnl; c++)
                pos_t[((size_t)i * cnl + c) * RG_M + j] = pos_raw[(size_t)cnl * (q * j + i) + c];
    uint8_t* cnc_layer = (uint8_t*)malloc(q);
    int* off = (int*)malloc((q + 1) * sizeof(int));
    off[0] = 0;
    for (int i = 0; i < q; i++) {
        cnc_layer[i] = cnc_raw[i];
        off[i + 1] = off[i] + RG_M * (cnc_layer[i] + 2);
    }
    d->lt_alloc = off[q];
    int16_t sched[RG_SCHED_MAX * 2];
    memset(sched, 0, sizeof(sched));
    const cusat_sched_src* ss = find_sched(t->name, q);
    if (ss) {
        d->n_steps = ss->n_steps;
        memcpy(sched, ss->pairs, 2 * ss->n_steps * sizeof(int16_t));
    } else {
        d->n_steps = q;
        for (int i = 0; i < q; i++) {
            sched[2 * i] = (int16_t)i;
            sched[2 * i + 1] = -1;
        }
    }
    d->smem = (unsigned)(((size_t)d->K + R) * sizeof(int16_t) + sizeof(int));
    CUresult r = CUDA_SUCCESS;
#define TRY(x)                        \
    if (r == CUDA_SUCCESS)            \
        r = (x);
    TRY(cuMemAlloc(&d->pos, (size_t)R * cnl * 2));
    TRY(cuMemcpyHtoD(d->pos, pos_t, (size_t)R * cnl * 2));
    TRY(cuMemAlloc(&d->cnc, q));
    TRY(cuMemcpyHtoD(d->cnc, cnc_layer, q));
    TRY(cuMemAlloc(&d->layer_off, (q + 1) * sizeof(int)));
    TRY(cuMemcpyHtoD(d->layer_off, off, (q + 1) * sizeof(int)));
    TRY(cuMemAlloc(&d->sched, sizeof(sched)));
    TRY(cuMemcpyHtoD(d->sched, sched, sizeof(sched)));
    TRY(cuMemAlloc(&d->data, (size_t)max_batch * d->K * 2));
    TRY(cuMemAlloc(&d->pty, (size_t)max_batch * R * 2));
    TRY(cuMemAlloc(&d->bnl, (size_t)max_batch * d->lt_alloc));
#undef TRY
    free(pos_raw);
    free(cnc_raw);
    free(pos_t);
    free(cnc_layer);
    free(off);
    if (r != CUDA_SUCCESS) {
        fail_cu(r, "rg_dec_create");
        rg_dec_destroy(d);
        return 0;
    }
    return d;
}

/* info[0..7] = N, K, R, q, cnl, lt_alloc, n_steps, smem bytes */
int rg_dec_info(const rg_dec* d, int32_t* info)
{
    const int32_t v[8] = {d->N, d->K, d->R, d->q, d->cnl, d->lt_alloc, d->n_steps, (int32_t)d->smem};
    memcpy(info, v, sizeof(v));
    return 0;
}

/* Decodes B frames of N int16 LLRs (device) into hard (B * K/8 bytes) and
 * result (B ints: max_trials - iterations, or -1), on stream s. */
int rg_dec_launch(rg_dec* d, CUdeviceptr llr, int B, CUdeviceptr hard, CUdeviceptr result, CUstream s)
{
    if (!d || B <= 0 || B > d->max_batch) {
        snprintf(g_err, sizeof(g_err), "rg_dec_launch: bad batch");
        return -1;
    }
    int K = d->K, R = d->R, M = RG_M, q = d->q, CNL = d->cnl, LT = d->lt_alloc, T = d->max_trials;
    int N = d->N, syn = 1, steps = d->n_steps;
    void* args[] = {&d->data, &d->pty, &d->bnl, &d->pos, &d->cnc, &d->layer_off, &result, &hard,
                    &K, &R, &M, &q, &CNL, &LT, &T, &llr, &N, &syn, &d->sched, &steps};
    /* this code's shared-memory opt-in (decoders of other codes may have set another) */
    CU(cuFuncSetAttribute(g_dec_fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)d->smem),
       "decoder shared-memory opt-in");
    CU(cuLaunchKernel(g_dec_fn, (unsigned)B, 1, 1, 2 * RG_M, 1, 1, d->smem, s, args, 0), "decoder launch");
    return 0;
}

/* demap_deinterleave_kernel over B frames (all pointers device). */
int rg_demap_launch(CUdeviceptr sym, CUdeviceptr out, CUdeviceptr pts_re, CUdeviceptr pts_im, int xfec,
                    int interleaved_len, int fec_len, int n_mod, int n_points, const uint32_t* col8,
                    float noise_var, float llr_gain, int B, CUstream s)
{
    unsigned ra[8];
    for (int i = 0; i < 8; i++)
        ra[i] = col8[i];
    void* args[] = {&sym, &out, &pts_re, &pts_im, &xfec, &interleaved_len, &fec_len, &n_mod, &n_points,
                    &ra[0], &ra[1], &ra[2], &ra[3], &ra[4], &ra[5], &ra[6], &ra[7], &noise_var, &llr_gain};
    const unsigned threads = 256, gx = ((unsigned)interleaved_len + threads - 1) / threads;
    CU(cuLaunchKernel(g_demap_fn, gx, (unsigned)B, 1, threads, 1, 1, 0, s, args, 0), "demap launch");
    return 0;
}
