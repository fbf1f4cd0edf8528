// Restates the reference's lib/qa_ldpc_encode.cc:35-87 through the C++ shims
// of include/cusat_fec.hpp: for every normal-frame DVB-S2 rate, seed-42
// random messages -> BCH + LDPC encode -> +-127 LLRs -> decode with 50
// trials (both the ldpc_decode and cuda::ldpc_decode_cuda paths) -> the
// information bits come back and trials_left > 0.  Also runs the demapper
// and BCH shims on the same frames.  Prints "OK" and exits 0 on success.
#include <random>
#include <vector>

#include "cusat_fec.hpp"

using namespace cusat_dsp;

static int fail(const char* what, int rate)
{
    fprintf(stderr, "FAIL %s rate %d\n", what, rate);
    return 1;
}

int main()
{
    std::mt19937 gen(42);
    for (int r = RATE_1_4; r <= RATE_9_10; r++) {
        int32_t ci[12];
        if (cusat_code_info(FECFRAME_NORMAL, r, ci))
            return fail("code_info", r);
        const int N = ci[0], K = ci[1], kbch = ci[2];
        std::vector<uint8_t> msg(kbch / 8), cw(N / 8), hard(K / 8);
        for (auto& b : msg)
            b = (uint8_t)(gen() & 0xff);
        if (cusat_gen_encode(FECFRAME_NORMAL, r, msg.data(), cw.data(), 1))
            return fail("encode", r);
        std::vector<int16_t> soft(N);
        for (int j = 0; j < N; j++)
            soft[j] = ((cw[j / 8] >> (7 - j % 8)) & 1) ? -127 : 127;
        ldpc_decode dec(FECFRAME_NORMAL, (code_rate_t)r, 50);
        int trials_left = 0;
        dec.decode_batch_cuda(soft.data(), hard.data(), &trials_left, 1);
        if (trials_left <= 0)
            return fail("trials", r);
        for (int j = 0; j < K / 8; j++)
            if (hard[j] != cw[j])
                return fail("hard", r);
        ldpc_code code{};
        code.n = N;
        cuda::ldpc_decode_cuda dc(&code, (code_rate_t)r, 50, 4);
        int16_t* d_soft;
        uint8_t* d_hard;
        int* d_res;
        cudaMalloc(&d_soft, N * 2);
        cudaMalloc(&d_hard, K / 8);
        cudaMalloc(&d_res, 4);
        cudaMemcpy(d_soft, soft.data(), N * 2, cudaMemcpyHostToDevice);
        dc.decode_launch_async(d_soft, 1, nullptr, d_hard, d_res);
        dc.decode_launch_async(d_soft, 5, nullptr, d_hard, d_res);  // > max_batch: silent no-op
        int res = -7;
        cudaMemcpy(&res, d_res, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(hard.data(), d_hard, K / 8, cudaMemcpyDeviceToHost);
        if (res != 50)
            return fail("launch_async trials", r);
        for (int j = 0; j < K / 8; j++)
            if (hard[j] != cw[j])
                return fail("launch_async hard", r);
        cudaFree(d_soft);
        cudaFree(d_hard);
        cudaFree(d_res);
    }
    // demapper shim: 8PSK 3/5, noiseless symbols demap to LLR signs of the codeword
    {
        int32_t ci[12];
        cusat_code_info(FECFRAME_NORMAL, RATE_3_5, ci);
        const int N = ci[0], kbch = ci[2];
        std::vector<uint8_t> msg(kbch / 8), cw(N / 8);
        for (auto& b : msg)
            b = (uint8_t)(gen() & 0xff);
        cusat_gen_encode(FECFRAME_NORMAL, RATE_3_5, msg.data(), cw.data(), 1);
        cuda::demapper_cuda dm(MOD_8PSK, RATE_3_5, FECFRAME_NORMAL, 2);
        std::vector<float> sym(2 * dm.xfecframe_len());
        cusat_gen_map(MOD_8PSK, RATE_3_5, FECFRAME_NORMAL, cw.data(), 1, sym.data());
        dm.demap_batch(sym.data(), 1, 0.1f, 40.0f);
        std::vector<int16_t> llr(N);
        cudaMemcpy(llr.data(), dm.soft_out_dev(), N * 2, cudaMemcpyDeviceToHost);
        for (int j = 0; j < N; j++) {
            const int bit = (cw[j / 8] >> (7 - j % 8)) & 1;
            if ((llr[j] < 0) != bit || llr[j] == 0)
                return fail("demap sign", j);
        }
    }
    printf("OK\n");
    return 0;
}
