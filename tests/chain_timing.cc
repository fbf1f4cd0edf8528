// Times the rx_fec_chain C++ shim (include/cusat_fec.hpp) the way the
// reference's receiver drives it: XFECFRAMEs submitted one by one from host
// memory, output collected when reported, a final flush.  Used by
// `bench.py --workload chain` for the C++ rows.
//   chain_timing <frames> <micro_batch> <streams> <budget: -1 default, 0 none> <copy helpers> <esn0_db> [connections]
// Prints one JSON object: frames, seconds, info Gbit/s, frame errors.
#include <stdio.h>
#include <stdlib.h>

#include <chrono>
#include <complex>
#include <random>
#include <vector>

#include "cusat_fec.hpp"

using namespace cusat_dsp;

int main(int argc, char** argv)
{
    if (argc < 7)
        return 2;
    // launches of many streams share CUDA_DEVICE_MAX_CONNECTIONS hardware
    // queues (8 unless set before the first CUDA call): a receiver that runs
    // small micro-batches on many streams raises it first
    if (argc > 7)
        setenv("CUDA_DEVICE_MAX_CONNECTIONS", argv[7], 1);
    const int n = atoi(argv[1]), mb = atoi(argv[2]), streams = atoi(argv[3]), cap = atoi(argv[4]),
              helpers = atoi(argv[5]);
    const float esn0 = (float)atof(argv[6]);
    const modulation_t mod = MOD_8PSK;
    const code_rate_t rate = RATE_3_5;
    int32_t ci[12], mi[6];
    cusat_code_info(FECFRAME_NORMAL, rate, ci);
    std::vector<float> pts(512);
    uint32_t col[8];
    cusat_modcod_info(mod, rate, FECFRAME_NORMAL, pts.data(), col, mi);
    const int N = ci[0], K = ci[1], kbch = ci[2], xfec = mi[3];
    // 64 distinct noisy frames (BCH + LDPC encoded, 8PSK, unit Es, AWGN), cycled
    const int distinct = 64;
    std::mt19937 gen(2024);
    std::normal_distribution<float> awgn(0.0f, std::sqrt(0.5f / std::pow(10.0f, esn0 / 10.0f)));
    std::vector<std::vector<std::complex<float>>> frames(distinct);
    std::vector<uint8_t> msg(kbch / 8), cw(N / 8);
    for (auto& f : frames) {
        for (auto& b : msg)
            b = (uint8_t)(gen() & 0xff);
        cusat_gen_encode(FECFRAME_NORMAL, rate, msg.data(), cw.data(), 1);
        f.resize(xfec);
        cusat_gen_map(mod, rate, FECFRAME_NORMAL, cw.data(), 1, reinterpret_cast<float*>(f.data()));
        for (auto& s : f)
            s += std::complex<float>(awgn(gen), awgn(gen));
    }
    rx_fec_chain chain(FECFRAME_NORMAL, rate, mod, 50, 64, streams, mb);
    chain.set_decode_budget(std::make_shared<gpu_decode_budget>(cap));
    chain.set_block_when_full(true);
    chain.set_copy_threads(helpers);
    chain.warmup();
    chain.update_snr(esn0);
    std::vector<uint8_t> out((size_t)chain.max_output_bytes());
    auto run = [&](int count) {
        for (int i = 0; i < count; i++)
            if (chain.submit_xfecframe(frames[i % distinct].data(), xfec))
                chain.get_gse_output(out.data(), (int)out.size());
        chain.flush();
        chain.get_gse_output(out.data(), (int)out.size());
    };
    run(std::min(n, 256));  // warm-up
    const uint64_t errors0 = chain.frame_error_count();
    const auto t0 = std::chrono::steady_clock::now();
    run(n);
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("{\"frames\": %d, \"seconds\": %.6f, \"gbit_s\": %.4f, \"us_per_frame\": %.3f, \"frame_errors\": %llu}\n", n, s,
           (double)n * K / s / 1e9, s / n * 1e6, (unsigned long long)(chain.frame_error_count() - errors0));
    return 0;
}
