// Instantiations and launch helpers of the frame-pair decoder kernel (two
// short frames per CTA).
#include "kernels.h"
#include "ldpc_pair.cuh"

namespace cusat {

namespace {

int align16(int x) { return (x + 15) & ~15; }

}  // namespace

static_assert(kPairThreads == lane_threads(1), "the frame-pair kernel runs one lane");

const void* select_pair_kernel(int cmax)
{
    switch (cmax) {
    case 2: return (const void*)ldpc_pair_kernel<2>;
    case 3: return (const void*)ldpc_pair_kernel<3>;
    case 4: return (const void*)ldpc_pair_kernel<4>;
    case 5: return (const void*)ldpc_pair_kernel<5>;
    case 6: return (const void*)ldpc_pair_kernel<6>;
    case 8: return (const void*)ldpc_pair_kernel<8>;
    case 9: return (const void*)ldpc_pair_kernel<9>;
    case 10: return (const void*)ldpc_pair_kernel<10>;
    case 12: return (const void*)ldpc_pair_kernel<12>;
    case 14: return (const void*)ldpc_pair_kernel<14>;
    case 16: return (const void*)ldpc_pair_kernel<16>;
    case 18: return (const void*)ldpc_pair_kernel<18>;
    case 20: return (const void*)ldpc_pair_kernel<20>;
    case 26: return (const void*)ldpc_pair_kernel<26>;
    case 28: return (const void*)ldpc_pair_kernel<28>;
    default: return nullptr;
    }
}

int pair_msg_row(int cmax) { return (2 * (cmax + 2) + 15) / 16 * 16; }

void pair_smem_layout(DecodeArgs* a, const SmemDims& d, int max_stage)
{
    int off = align16(d.N * 4);  // APP words: frame A's int16 in the low half, B's in the high half
    auto take = [&](int* field, int bytes) {
        *field = off;
        off = align16(off + bytes);
    };
    take(&a->sm_dummy, 2 * kM * 4);  // +32640 region, then the junk region
    take(&a->sm_stage, kStageSets * max_stage * kM * 4);
    take(&a->sm_tab, d.q * d.cmax * 16);
    take(&a->sm_cnt, d.q);
    take(&a->sm_sched, d.n_steps * 4);
    take(&a->sm_conf, d.n_steps);
    take(&a->sm_item_off, (d.n_steps + 1) * 2);
    take(&a->sm_items, d.n_items * 8);
    take(&a->sm_code, (int)sizeof(DevCode));
    take(&a->sm_misc, (int)sizeof(PairState));
    take(&a->sm_msgbuf, 0);
    a->sm_total = off;
    a->max_stage = max_stage;
}

}  // namespace cusat
