/*
 * CPU oracle for the receive-side FEC path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithms that tests/ and
 * __graft_entry__.smoke() compare the CUDA kernels against, and that bench.py
 * times as the CPU baseline.  Nothing in the product (cusat_gb300/) links, loads or calls it.
 *
 * Decoder semantics (reference lib/cusat_dsp/cuda/ldpc_decode_kernel.cu):
 *   - APP init with the -32768 -> -32767 clamp and the parity transpose
 *     pty[M*i + j] = llr[K + q*j + i]                          (:635-684)
 *   - syndrome before every iteration, trials = T - t on success, -1 after
 *     T iterations                                          (:689-749, :943)
 *   - layer update: x = qsat16(APP - old), offset min-sum finalp with
 *     beta = 1, message = clamp8, info APP += msg - old (saturating),
 *     parity APP = sat16(x + msg)                       (:242-275, :761-837)
 *   - the reference leaves checks of one schedule step that share a variable
 *     node to a data race (:793-802); the oracle resolves it as step-Jacobi:
 *     every check of a step gathers from the APP state at the start of the
 *     step and a shared variable node receives sat16(APP + sum of deltas).
 * Parity pinned by: the message clamp/delta known answers of
 * lib/qa_ldpc_message_update.cc:10-27, the BCH tests of lib/qa_bch_code.cc
 * and apps/bench_bch_gpu.cc:52-104, the table manifest
 * lib/cusat_dsp/ldpc_tables/checksums.txt, the noiseless round trips of
 * lib/qa_ldpc_encode.cc:35-87 and, where the reference tree is present, the
 * reference's own host code compiled into oracle/_ref.  The reference has no
 * CPU decoder and no decoder golden vector, so iteration-level decoder
 * behaviour on noisy input is pinned only through these round trips.
 */
#ifndef FEC_ORACLE_H
#define FEC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out[0..9] = N, K, q, n_steps, k_bch, n_bch, t, bch_degree, links_total, cnl */
int orc_code_info(int framesize, int rate, int32_t* out);

/* Decodes B frames of N int16 LLRs. hard: B*K/8 bytes MSB-first;
 * trials: T - iterations used, or -1. weights (may be NULL): per iteration t
 * (0..T-1) and check degree d (0..31) an int16 pair {beta, alpha64} at
 * weights[(t*32 + d)*2]; NULL = offset min-sum beta 1, no scaling. */
int orc_ldpc_decode(int framesize, int rate, const int16_t* llr, int B, int max_trials,
                    const int16_t* weights, uint8_t* hard, int32_t* trials, int nthreads);

/* Same, with the syndrome checked only before iterations t with
 * t % syn_period == 0 and at t == max_trials (the reference's
 * CUSAT_LDPC_SYN_PERIOD, ldpc_decode_kernel.cu:693-694,1237-1241). */
int orc_ldpc_decode_period(int framesize, int rate, const int16_t* llr, int B, int max_trials, int syn_period,
                           const int16_t* weights, uint8_t* hard, int32_t* trials, int nthreads);

/* Syndrome of hard decisions from APP signs (test helper): 1 if every
 * parity check of the int16 LLR vector (< 0 = bit 1) is satisfied. */
int orc_syndrome_ok(int framesize, int rate, const int16_t* llr);

/* IRA encode: info K/8 bytes -> codeword N/8 bytes (info then parity). */
int orc_ldpc_encode(int framesize, int rate, const uint8_t* info, uint8_t* cw, int B);

/* BCH generator (bit i of word i/64 = coeff of x^i), returns its degree. */
int orc_bch_generator(int framesize, int rate, uint64_t gen[4]);
/* Systematic BCH encode: k_bch/8 bytes -> n_bch/8 bytes. */
int orc_bch_encode(int framesize, int rate, const uint8_t* msg, uint8_t* cw, int B);
/* Bit-serial remainder of n_bch/8-byte words mod g: rem (p/8 bytes, the
 * coefficient of x^(p-1) first) and valid = (rem == 0). */
int orc_bch_check(int framesize, int rate, const uint8_t* cw, uint8_t* rem, int32_t* valid,
                  int B);

/* Soft demap + deinterleave (reference cuda/demapper_kernel.cu:31-184).
 * kind 0 = QPSK formula, 1 = 8PSK formula, 2 = log-MAP over the points. */
int orc_demap(const float* sym, int B, int xfec, int interleaved_len, int fec_len, int n_mod,
              int kind, const float* pts_re, const float* pts_im, int n_points,
              const uint32_t* col_offset, float noise_var, float llr_gain, int16_t* out);

/* Demapper gain cap (reference cuda/demapper_kernel.cu:216-239, 283-291).
 * dmax: "loudest bit" squared distance -- 2 for QPSK (kind 0), 4 for 8PSK
 * (kind 1), else the largest over (point, bit) of the squared distance to
 * the nearest point whose label differs in that bit.  The capped gain is
 * min(llr_gain, 2 llr_target / dmax); llr_target <= 0 or dmax <= 0 leave
 * llr_gain unchanged (the reference's target is 320 unless
 * CUSAT_DEMAP_LLR_TARGET sets it). */
float orc_demap_dmax(int kind, const float* pts_re, const float* pts_im, int n_points, int n_mod);
float orc_capped_llr_gain(float dmax, float llr_target, float llr_gain);

/* Mapper: codeword N/8 bytes -> xfec complex symbols (re, im pairs).
 * Symbols j < interleaved_len take label bits at col_offset[b] + j * stride,
 * 0 at positions >= fec_len (stuffing); the rest (128APSK padding) carry
 * the all-ones label (reference mapper.cc:28-62). */
int orc_map(const uint8_t* cw, int B, int cw_bytes, int xfec, int interleaved_len, int fec_len, int n_mod,
            const uint32_t* col_offset, int stride, const float* pts_re, const float* pts_im, float* sym);

/* Known-answer hook: reference ldpc_make_bnl_update (message clamp, delta). */
int orc_bnl_update(int raw_new, int old, int32_t* delta);

/* The exp/log used by the log-MAP demapper (shared with the CUDA kernel's
 * algorithm, exposed for accuracy tests). */
float orc_exp_neg(float x);
float orc_log(float x);

/* Post-FEC baseband stage: the BB scrambler PRBS (n_bytes <= 7274), the
 * RX chain's descramble + BBHEADER check + data-field extraction of a batch
 * (hard bits of frame f at hard + f * stride, kbch bytes), and a scrambled
 * GSE BBFRAME builder for test traffic. */
void orc_bb_prbs(uint8_t* seq, int n_bytes);
int orc_bb_extract(const uint8_t* hard, int stride, int kbch, const int32_t* trials, const int32_t* valid, int B,
                   uint8_t* out, int max_out, int32_t* lengths, int32_t* offsets);
int orc_bb_build(const uint8_t* data, int len, int kbch, int matype_ts_gs, uint8_t* out);

/* Decision-directed SNR (linear) of n_sym symbols (re, im): QPSK by the
 * signs of I and Q (qpsk != 0), otherwise the nearest of n_points points on
 * every stride-th symbol.  Reference modulation/dd_snr.cc:12-47. */
float orc_dd_snr(const float* sym, int n_sym, const float* pts, int n_points, int stride, int qpsk);

/* PL receiver tail (EN 302 307-1 clause 5.5.4; reference
 * framing/pl_scrambler.cc, plrx/pl_receiver.cc:1694-1741): the
 * descrambling rotation index R_n(i) (factor e^{-j R pi/2}) of gold code n
 * for i < len, and the data symbols of one located PLFRAME's payload
 * (descramble, drop the pilot blocks, counter-rotate each slot by
 * rot * step^i; slot_rot may be NULL). */
int orc_pl_rotation(int gold, uint8_t* r, int len);
int orc_pl_extract(const float* payload, int slots, int pilots, const uint8_t* r, const float* slot_rot, float* out);

/* Unrolled learned min-sum (training model; nms_model.inc): loss and its
 * gradient with respect to theta[T][32][2] = {beta, alpha} per iteration and
 * check degree, summed over B frames of int16 LLRs and packed codewords
 * (N/8 bytes, MSB first).  iter_w: per-iteration loss weights or NULL
 * (uniform).  grad (may be NULL) and loss are accumulated into.  float and
 * double copies of the same code. */
int orc_nms_train_f32(int framesize, int rate, const int16_t* llr, const uint8_t* cw, int B, int T,
                      const float* theta, const float* iter_w, float* grad, float* loss, int nthreads);
int orc_nms_train_f64(int framesize, int rate, const int16_t* llr, const uint8_t* cw, int B, int T,
                      const double* theta, const double* iter_w, double* grad, double* loss, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
