// Instantiations and launch helpers of the layered decoder kernel (one
// frame per CTA).
#include <stdlib.h>

#include "kernels.h"
#include "ldpc_kernel.cuh"

namespace cusat {

namespace {

template <int CMAX>
const void* pick(int lanes)
{
    return lanes == 2 ? (const void*)ldpc_layered_kernel<CMAX, 2> : (const void*)ldpc_layered_kernel<CMAX, 1>;
}

int align16(int x) { return (x + 15) & ~15; }

}  // namespace

const void* select_decoder_kernel(int cmax, int lanes)
{
    switch (cmax) {
    case 2: return pick<2>(lanes);
    case 3: return pick<3>(lanes);
    case 4: return pick<4>(lanes);
    case 5: return pick<5>(lanes);
    case 6: return pick<6>(lanes);
    case 8: return pick<8>(lanes);
    case 9: return pick<9>(lanes);
    case 10: return pick<10>(lanes);
    case 12: return pick<12>(lanes);
    case 14: return pick<14>(lanes);
    case 16: return pick<16>(lanes);
    case 18: return pick<18>(lanes);
    case 20: return pick<20>(lanes);
    case 26: return pick<26>(lanes);
    case 28: return pick<28>(lanes);
    default: return nullptr;
    }
}

int decoder_threads(int lanes) { return lanes * lane_threads(lanes); }

int syndrome_period()
{
    static const int period = [] {
        const char* e = getenv("CUSAT_LDPC_SYN_PERIOD");
        return (e && atoi(e) > 0) ? atoi(e) : 1;
    }();
    return period;
}

void decoder_smem_layout(DecodeArgs* a, const SmemDims& d)
{
    int off = align16(d.N * 2 + 2);  // APP + the absent-edge scratch slot
    auto take = [&](int* field, int bytes) {
        *field = off;
        off = align16(off + bytes);
    };
    take(&a->sm_dummy, 2 * kM * 2);  // +32640 region, then the junk region
    take(&a->sm_stage, kStageSets * kMaxStage * kM * 2);
    take(&a->sm_tab, d.q * d.cmax * 16);
    take(&a->sm_cnt, d.q);
    take(&a->sm_sched, d.n_steps * 4);
    take(&a->sm_conf, d.n_steps);
    take(&a->sm_item_off, (d.n_steps + 1) * 2);
    take(&a->sm_items, d.n_items * 8);
    take(&a->sm_code, (int)sizeof(DevCode));
    take(&a->sm_misc, 16);
    // message rows staged for the next step: two sets x threads x row words
    // (one 16-byte slot per thread and set: staged rows are 16 bytes)
    take(&a->sm_msgbuf, stage_rows_in_smem(d.cmax, d.lanes) ? 2 * d.lanes * lane_threads(d.lanes) * 16 : 0);
    a->sm_total = off;
}

SmemDims smem_dims_of(const DevCode& c, int lanes)
{
    return SmemDims{c.N, c.q, c.n_steps, c.n_items, c.cmax, lanes};
}

int launch_decoder(const void* fn, const DecodeArgs& a, int grid, int threads, cudaStream_t stream)
{
    void* args[] = {const_cast<DecodeArgs*>(&a)};
    return (int)cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, (size_t)a.sm_total, stream);
}

}  // namespace cusat
