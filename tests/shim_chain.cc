// The rx_fec_chain / rx_fec_pool C++ shims of include/cusat_fec.hpp, used
// the way the reference's receiver uses them (lib/cusat_dsp/rx_fec_pool.cc
// callers): GSE BBFRAMEs (built by the oracle) -> BCH + LDPC encode -> map
// -> pool.submit with a PL layout per frame, MODCOD runs alternating ->
// every payload comes back, in submission order, with its data-field size.
// Then the same through a standalone chain under a launch mutex.  Prints
// "OK" and exits 0 on success.
#include <complex>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "cusat_fec.hpp"

// Stand-in for the reference's acm_config.h (two of its MODCOD rows); the
// second inclusion of the shim header then declares the pool, as in the
// reference's tree where rx_fec_pool.h includes acm_config.h.
#define INCLUDED_CUSAT_DSP_ACM_CONFIG_H
namespace cusat_dsp {
struct modcod_def_t {
    uint8_t modcod_idx;
    modulation_t constellation;
    code_rate_t code_rate;
};
inline const modcod_def_t* find_modcod(uint8_t idx)
{
    static const modcod_def_t rows[] = {{4, MOD_QPSK, RATE_1_2}, {12, MOD_8PSK, RATE_3_5}};
    for (const auto& r : rows)
        if (r.modcod_idx == idx)
            return &r;
    return nullptr;
}
}  // namespace cusat_dsp
#include "cusat_fec.hpp"

extern "C" {
#include "fec_oracle.h"
}

using namespace cusat_dsp;

struct pl_layout {
    uint8_t modcod = 0;
};

static int fail(const char* what)
{
    fprintf(stderr, "FAIL %s\n", what);
    return 1;
}

struct Frame {
    std::vector<std::complex<float>> sym;
    std::vector<uint8_t> payload;
    uint8_t modcod;
};

static Frame make_frame(uint8_t modcod, std::mt19937& gen)
{
    const modcod_def_t* m = find_modcod(modcod);
    int32_t ci[12];
    cusat_code_info(FECFRAME_SHORT, m->code_rate, ci);
    const int N = ci[0], kbch = ci[2];
    Frame f;
    f.modcod = modcod;
    f.payload.resize(1 + gen() % (kbch / 8 - 11));
    for (auto& b : f.payload)
        b = (uint8_t)(gen() & 0xff);
    std::vector<uint8_t> bb(kbch / 8), cw(N / 8);
    orc_bb_build(f.payload.data(), (int)f.payload.size(), kbch / 8, 0, bb.data());
    cusat_gen_encode(FECFRAME_SHORT, m->code_rate, bb.data(), cw.data(), 1);
    const int bits = m->constellation == MOD_QPSK ? 2 : 3;
    f.sym.resize(N / bits);
    cusat_gen_map(m->constellation, m->code_rate, FECFRAME_SHORT, cw.data(), 1,
                  reinterpret_cast<float*>(f.sym.data()));
    return f;
}

static void collect(rx_fec_pool& pool, std::vector<uint8_t>& out, std::vector<int>& sizes)
{
    std::vector<uint8_t> buf((size_t)pool.max_output_bytes());
    for (;;) {
        const int n = pool.get_gse_output(buf.data(), (int)buf.size());
        if (n <= 0)
            break;
        out.insert(out.end(), buf.begin(), buf.begin() + n);
        sizes.insert(sizes.end(), pool.gse_dfl_sizes().begin(), pool.gse_dfl_sizes().end());
    }
}

int main()
{
    std::mt19937 gen(7);
    std::vector<Frame> frames;
    const uint8_t runs[][2] = {{4, 5}, {12, 5}, {4, 6}, {12, 3}, {4, 2}};
    for (const auto& r : runs)
        for (int k = 0; k < r[1]; k++)
            frames.push_back(make_frame(r[0], gen));

    rx_fec_pool pool(FECFRAME_SHORT, {4, 12}, 25, 64, 2, 4);
    pool.warmup_all();
    std::vector<uint8_t> out;
    std::vector<int> sizes;
    for (const Frame& f : frames) {
        pl_layout pls;
        pls.modcod = f.modcod;
        if (pool.submit(f.sym.data(), (int)f.sym.size(), pls))
            collect(pool, out, sizes);
    }
    pool.finish_all_pending();
    collect(pool, out, sizes);

    std::vector<uint8_t> want;
    std::vector<int> want_sizes;
    for (const Frame& f : frames) {
        want.insert(want.end(), f.payload.begin(), f.payload.end());
        want_sizes.push_back((int)f.payload.size());
    }
    if (out != want || sizes != want_sizes)
        return fail("pool output");
    uint64_t fr = 0, er = 0;
    if (pool.total_frame_count() != frames.size() || pool.total_error_count() != 0)
        return fail("pool counters");
    if (!pool.modcod_counters(12, fr, er) || fr != 8 || er != 0 || pool.modcod_counters(99, fr, er))
        return fail("modcod counters");

    std::mutex mtx;
    rx_fec_chain chain(FECFRAME_SHORT, RATE_1_2, MOD_QPSK, 25, 64, 3, 2);
    chain.set_cuda_mutex(&mtx);
    chain.set_decode_budget(gpu_decode_budget::make_default());
    std::vector<uint8_t> cout;
    std::vector<uint8_t> buf((size_t)chain.max_output_bytes());
    std::vector<uint8_t> cwant;
    for (const Frame& f : frames) {
        if (f.modcod != 4)
            continue;
        cwant.insert(cwant.end(), f.payload.begin(), f.payload.end());
        if (chain.submit_xfecframe(f.sym.data(), (int)f.sym.size())) {
            const int n = chain.get_gse_output(buf.data(), (int)buf.size());
            cout.insert(cout.end(), buf.begin(), buf.begin() + n);
        }
    }
    chain.flush();
    const int n = chain.get_gse_output(buf.data(), (int)buf.size());
    cout.insert(cout.end(), buf.begin(), buf.begin() + n);
    if (cout != cwant || chain.frame_count() != 13 || chain.frame_error_count() != 0 || chain.gpu_inflight() != 0)
        return fail("chain output");
    printf("OK\n");
    return 0;
}
