/*
 * cusat_fec.h -- C ABI of the GB300 receive-side FEC path.
 *
 * Soft demapping with deinterleave, layered offset min-sum LDPC decoding of
 * the DVB-S2/S2X codes on int16 LLRs with a syndrome early exit, and the BCH
 * syndrome check, as hand-written sm_103a CUDA kernels behind plain C entry
 * points (pointers, sizes, ints; no CUDA or C++ types).  `stream` arguments
 * are cudaStream_t values passed as void*; NULL is the legacy default stream.
 * Device pointers are device (or mapped pinned) memory; "host" pointers are
 * ordinary host memory.
 *
 * Enumerations (frame size, code rate, modulation) use the numeric values of
 * the reference's lib/cusat_dsp/include/cusat_dsp/modcod_types.h:14-95, so a
 * caller of the reference passes its own enum values unchanged.
 *
 * Every entry point returns CUSAT_OK (0) or a negative CUSAT_ERR_* code;
 * cusat_last_error() returns a one-line description of the last failure on
 * the calling thread.  Objects are not thread-safe (like the reference's
 * classes); distinct objects may be used from distinct threads.
 *
 * Results follow the reference conventions: trials[f] = max_trials -
 * iterations used when the syndrome is satisfied, -1 after max_trials
 * iterations without convergence; hard decisions are the k_ldpc information
 * bits, packed MSB-first (k_ldpc/8 bytes per frame); bch_valid[f] = 1 when
 * the hard decisions are a BCH codeword.
 */
#ifndef CUSAT_FEC_H
#define CUSAT_FEC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUSAT_OK 0
#define CUSAT_ERR_ARG (-1)          /* invalid argument (batch, pointer, size) */
#define CUSAT_ERR_UNSUPPORTED (-2)  /* frame size / rate / modulation not supported */
#define CUSAT_ERR_CUDA (-3)         /* CUDA runtime error (message in cusat_last_error) */
#define CUSAT_ERR_NO_DEVICE (-4)    /* no CUDA device */

const char* cusat_last_error(void);

/* ---------------------------------------------------------------------- */
/* LDPC decoder                                                            */
/* ---------------------------------------------------------------------- */

typedef struct cusat_ldpc_decoder cusat_ldpc_decoder;

/* Replaces cusat_dsp::cuda::ldpc_decode_cuda::ldpc_decode_cuda
 * (reference lib/cusat_dsp/cuda/ldpc_decode_kernel.cuh:22-35, .cu:990-1181)
 * and cusat_dsp::ldpc_decode::ldpc_decode (lib/cusat_dsp/ldpc_decode.h:22-33):
 * builds the code's decoding plan on the current device and reserves
 * buffers for up to max_batch frames. */
int cusat_ldpc_decoder_create(int framesize, int rate, int max_trials, int max_batch,
                              cusat_ldpc_decoder** out);
void cusat_ldpc_decoder_destroy(cusat_ldpc_decoder* dec);

/* out[0..7] = n_bits, k_bits, k_bytes, q, n_steps, max_trials, max_batch,
 * lanes (2 = paired-layer schedule) */
int cusat_ldpc_decoder_info(const cusat_ldpc_decoder* dec, int32_t* out);

/* Frames per CTA.  Codes decoded one layer per step whose frame pair fits
 * twice per SM (the short frames) can run two frames per CTA when no
 * learned weights are set; frames with channel LLRs beyond the
 * saturation-free range then go to a one-frame launch.  n = 0 (default):
 * pairs for codes of at most 5 circulants per layer (short rates 1/4 to
 * 1/2) in launches whose pairs occupy three quarters of the SMs or more;
 * 1: one frame per CTA; 2: pairs whenever the code allows -- for smaller
 * launches of those codes that overlap others on several streams (the
 * wider short codes measured slower as pairs).  Results do not depend on
 * it.  cusat_ldpc_decoder_frames_per_cta returns what a launch of `batch`
 * frames runs (1 or 2). */
int cusat_ldpc_decoder_set_frames_per_cta(cusat_ldpc_decoder* dec, int n);
int cusat_ldpc_decoder_frames_per_cta(const cusat_ldpc_decoder* dec, int batch);

/* Learned min-sum weights (no counterpart in the reference, whose
 * normalised-min-sum hook nms_scale, ldpc_decode_kernel.cu:75-90, is never
 * enabled).  weights[(t * 32 + d) * 2 + {0, 1}] = {beta, alpha} for
 * iteration t < n_iter and check degree d: the check-to-bit magnitude
 * becomes min(((max(m - beta, 0) * alpha + 32) >> 6), 127) instead of
 * min(max(m - 1, 0), 127), with m the smallest |extrinsic| of the other edges
 * and alpha in 64ths (0 = no scaling); iterations past n_iter reuse the last
 * row.  beta in 0..127, alpha in 0..255.  weights == NULL returns to the
 * plain decoder.  Waits for this decoder's last launch to finish (not for
 * the device) before replacing the table, then copies it on a private
 * non-blocking stream; launches captured in a CUDA graph are not waited
 * for. */
int cusat_ldpc_decoder_set_weights(cusat_ldpc_decoder* dec, const int16_t* weights, int n_iter);

/* No counterpart in the reference, which launches one CTA per frame
 * (ldpc_decode_kernel.cu:1198-1285).  Caps the CTAs of this decoder's
 * persistent launches (0 = one per resident slot, at most one per frame).
 * With fewer CTAs than frames each CTA decodes several frames in turn --
 * the path every batch larger than the resident slots takes -- so small
 * tests can hold that path against the oracle. */
int cusat_ldpc_decoder_set_max_ctas(cusat_ldpc_decoder* dec, int max_ctas);

/* Replaces ldpc_decode_cuda::decode_launch_async (ldpc_decode_kernel.cuh:51-64,
 * .cu:1324-1336): decodes `batch` frames of n_bits int16 LLRs read from
 * device memory, asynchronously on `stream`.  hard_out (batch*k_bytes) and
 * trials_out (batch) are device or mapped pinned pointers; NULL selects the
 * decoder's internal pinned buffers (read them with _results after a sync).
 * One launch at a time per decoder object (its message scratch), as with
 * the reference's instances. */
int cusat_ldpc_decode_launch(cusat_ldpc_decoder* dec, const int16_t* soft_dev, int batch,
                             void* stream, uint8_t* hard_out, int32_t* trials_out);

/* Replaces ldpc_decode_cuda::decode_batch (ldpc_decode_kernel.cuh:37-49,
 * .cu:1287-1305) and ldpc_decode::decode_batch_cuda (ldpc_decode.h:35-44):
 * host LLRs in, host results out, synchronous on `stream`. */
int cusat_ldpc_decode_batch(cusat_ldpc_decoder* dec, const int16_t* soft_host, uint8_t* hard_host,
                            int32_t* trials_host, int batch, void* stream);

/* Replaces ldpc_decode_cuda::decode_batch_d2h (ldpc_decode_kernel.cuh:44-49,
 * .cu:1307-1322) and ldpc_decode::decode_batch_cuda_d2h (ldpc_decode.h:46-53):
 * device LLRs in, host results out, synchronous on `stream`. */
int cusat_ldpc_decode_batch_d2h(cusat_ldpc_decoder* dec, const int16_t* soft_dev,
                                uint8_t* hard_host, int32_t* trials_host, int batch, void* stream);

/* Copies the internal result buffers of the last launch that used them. */
int cusat_ldpc_decoder_results(const cusat_ldpc_decoder* dec, uint8_t* hard_host,
                               int32_t* trials_host, int batch);

/* ---------------------------------------------------------------------- */
/* Soft demapper + deinterleaver                                           */
/* ---------------------------------------------------------------------- */

typedef struct cusat_demapper cusat_demapper;

/* Replaces cusat_dsp::cuda::demapper_cuda::demapper_cuda
 * (lib/cusat_dsp/cuda/demapper_kernel.cuh:23-38, .cu:188-281). */
int cusat_demapper_create(int modulation, int rate, int framesize, int max_batch,
                          cusat_demapper** out);
void cusat_demapper_destroy(cusat_demapper* dm);

/* out[0..3] = fecframe_len, xfecframe_len, n_mod, interleaved_len */
int cusat_demapper_info(const cusat_demapper* dm, int32_t* out);

/* Replaces demapper_cuda::capped_llr_gain (demapper_kernel.cuh:68-70,
 * .cu:283-291). */
float cusat_demapper_capped_llr_gain(const cusat_demapper* dm, float llr_gain);

/* Device pointer of the internal LLR buffer [max_batch * fecframe_len]
 * (replaces demapper_cuda::soft_out_dev, demapper_kernel.cuh:72-73). */
int16_t* cusat_demapper_soft_out_dev(const cusat_demapper* dm);

/* Demaps symbols already on the device (batch * xfecframe_len complex
 * float pairs) into soft_out_dev (NULL = internal buffer), async. */
int cusat_demap_launch(cusat_demapper* dm, const float* sym_dev, int batch, float noise_var,
                       float llr_gain, int16_t* soft_out_dev, void* stream);

/* Replaces demapper_cuda::demap_batch_async (demapper_kernel.cuh:53-66,
 * .cu:335-362): copies host symbols to the device and demaps into the
 * internal buffer, asynchronously on `stream` (llr_gain is capped first). */
int cusat_demap_batch_async(cusat_demapper* dm, const float* sym_host, int batch,
                            float noise_var, float llr_gain, void* stream);

/* Replaces demapper_cuda::demap_batch (demapper_kernel.cuh:40-51,
 * .cu:302-333): as _async, then synchronizes. */
int cusat_demap_batch(cusat_demapper* dm, const float* sym_host, int batch, float noise_var,
                      float llr_gain);

/* ---------------------------------------------------------------------- */
/* BCH syndrome check                                                      */
/* ---------------------------------------------------------------------- */

typedef struct cusat_bch_checker cusat_bch_checker;

/* Replaces cusat_dsp::cuda::bch_check_cuda::bch_check_cuda
 * (lib/cusat_dsp/cuda/bch_check_kernel.cuh:9-24, .cu:13-23): flat_lut is
 * the reference's 256 x 4 uint64 encoder LUT (bch_code_t::encoder_lut),
 * gen_poly the 4-word generator, n_bytes the codeword length in bytes. */
int cusat_bch_checker_create(const uint64_t* flat_lut, const uint64_t* gen_poly, int gen_degree,
                             unsigned int n_bytes, cusat_bch_checker** out);
/* Same checker built from the standard code of (framesize, rate). */
int cusat_bch_checker_create_for_code(int framesize, int rate, cusat_bch_checker** out);
void cusat_bch_checker_destroy(cusat_bch_checker* bc);
unsigned int cusat_bch_checker_n_bytes(const cusat_bch_checker* bc);

/* Replaces bch_check_cuda::check_async (bch_check_kernel.cu:26-36):
 * valid_out[f] = 1 iff codeword f (n_bytes, device) is a BCH codeword.
 * rem_out (NULL or batch * degree/8 bytes) receives c(x) x^p mod g(x),
 * coefficient of x^(p-1) first. */
int cusat_bch_check_launch(cusat_bch_checker* bc, const uint8_t* codewords_dev,
                           int32_t* valid_out, uint8_t* rem_out, int batch, void* stream);

/* ---------------------------------------------------------------------- */
/* Receive chain for one MODCOD                                            */
/* ---------------------------------------------------------------------- */

typedef struct cusat_rx_fec cusat_rx_fec;

/* One MODCOD's demap + deinterleave -> LDPC decode -> BCH check as one
 * launch sequence on one stream: the demap over the whole grid into the
 * object's LLR scratch in device memory, the persistent decoder, the BCH
 * check.  Replaces the
 * per-slot launch sequence of rx_fec_chain::launch_slot_gpu
 * (lib/cusat_dsp/rx_fec_chain.cc:361-505). */
int cusat_rx_fec_create(int modulation, int rate, int framesize, int max_trials, int max_batch,
                        cusat_rx_fec** out);
void cusat_rx_fec_destroy(cusat_rx_fec* rx);
/* out[0..5] = xfecframe_len, n_bits, k_bits, k_bytes, k_bch, n_mod */
int cusat_rx_fec_info(const cusat_rx_fec* rx, int32_t* out);
/* Learned weights for the chain's decoder (see cusat_ldpc_decoder_set_weights). */
int cusat_rx_fec_set_weights(cusat_rx_fec* rx, const int16_t* weights, int n_iter);
/* The decoder's frames per CTA, as cusat_ldpc_decoder_set_frames_per_cta. */
int cusat_rx_fec_set_frames_per_cta(cusat_rx_fec* rx, int n);
float cusat_rx_fec_capped_llr_gain(const cusat_rx_fec* rx, float llr_gain);
/* Symbols on the device in, results to device or mapped pinned memory;
 * llr_gain is capped like demap_batch does (demapper_kernel.cu:283-291).
 * The object's LLR and message scratch serve one launch at a time: launches
 * of one object on different streams must not overlap (one object per
 * stream, as the reference's chain keeps one instance per stream). */
int cusat_rx_fec_launch(cusat_rx_fec* rx, const float* sym_dev, int batch, float noise_var,
                        float llr_gain, uint8_t* hard_out, int32_t* trials_out,
                        int32_t* bch_valid_out, void* stream);

/* ---------------------------------------------------------------------- */
/* Mixed-MODCOD batches                                                    */
/* ---------------------------------------------------------------------- */

typedef struct cusat_batch cusat_batch;

/* One frame of a mixed batch. */
typedef struct {
    int32_t modcod;       /* index into the MODCOD list given at creation */
    float noise_var;      /* N0 of this frame (QPSK LLR scale) */
    float llr_gain;       /* gain for 8PSK/APSK, capped like demap_batch */
    int32_t reserved;
    const float* sym;     /* device: xfecframe_len complex symbols (re, im) */
    uint8_t* hard;        /* device or mapped pinned: k_ldpc/8 bytes */
    int32_t* trials;      /* device or mapped pinned: one int */
    int32_t* bch_valid;   /* device or mapped pinned: one int, or NULL */
} cusat_frame;

/* No counterpart in the reference, which builds one chain per MODCOD and
 * flushes on every MODCOD change (lib/cusat_dsp/rx_fec_pool.cc:48-87).  A
 * batch decodes frames of any of the given MODCODs (modcods: n triples
 * modulation, rate, frame size) in one launch sequence: demap ->
 * decode -> BCH; each frame's results equal those of a single-MODCOD
 * cusat_rx_fec launch on the same symbols. */
int cusat_batch_create(const int32_t* modcods, int n_modcods, int max_trials, int max_frames,
                       cusat_batch** out);
void cusat_batch_destroy(cusat_batch* b);
/* out[0..3] = MODCODs, kernel classes, max_frames, max_trials */
int cusat_batch_info(const cusat_batch* b, int32_t* out);
/* Learned weights for one MODCOD of the batch (NULL: plain); takes effect
 * for later launches and for replays of an existing capture.  Waits for
 * this batch's last launch or replay (not for the device) first. */
int cusat_batch_set_weights(cusat_batch* b, int modcod, const int16_t* weights, int n_iter);
/* Caps every kernel class's persistent grid at max_ctas CTAs (0 = no cap),
 * so that CTAs decode several frames in turn and switch between the codes
 * of their class -- what a large mixed batch does -- at sizes the oracle
 * checks quickly.  Takes effect for later launches and captures. */
int cusat_batch_set_max_ctas(cusat_batch* b, int max_ctas);
/* Decodes n frames on `stream` (waits for the previous launch's descriptor
 * copies first; the frames' buffers must stay valid until completion).  One
 * launch (or replay) at a time per batch object: they share its LLR and
 * message scratch. */
int cusat_batch_launch(cusat_batch* b, const cusat_frame* frames, int n, void* stream);
/* Tunes the launch sequence on this frame list (reps timed launches per
 * candidate) and keeps the fastest for later launches and captures: times
 * each kernel class's decoder alone; tries class orders (costliest first,
 * or last) x grid rules (each persistent CTA decoding f = 1, 2, 3 or 4
 * frames of its class, or CTAs in proportion to the classes' measured
 * cost); then refines each class's frames per CTA over {1, 2, 3, 4, 6, 8}.
 * best_ms: the chosen sequence's time. */
int cusat_batch_tune(cusat_batch* b, const cusat_frame* frames, int n, int reps, void* stream,
                     float* best_ms);
/* The tuned configuration, per kernel class k < max_classes:
 * out[5k..5k+4] = circulant slots per layer, lanes, frames of the last
 * staged list, persistent CTAs, position in the launch order; solo_ms[k]
 * (may be NULL) = the class's decoder alone at the last tuning.  Returns
 * the number of classes. */
int cusat_batch_tuned(const cusat_batch* b, int32_t* out, float* solo_ms, int max_classes);
/* Captures the launch sequence for this frame list into a CUDA graph
 * (stream must not be the legacy default stream); cusat_batch_replay
 * relaunches it: same frames, same buffers, whatever they hold now. */
int cusat_batch_capture(cusat_batch* b, const cusat_frame* frames, int n, void* stream);
int cusat_batch_replay(cusat_batch* b, void* stream);

/* ---------------------------------------------------------------------- */
/* Serving loop                                                            */
/* ---------------------------------------------------------------------- */

typedef struct cusat_server cusat_server;

#define CUSAT_REQ_HOST_SYMBOLS 1  /* request flag: sym is host memory */

/* One frame request. */
typedef struct {
    int32_t modcod;       /* index into the server's MODCOD list */
    float noise_var;
    float llr_gain;       /* capped like demap_batch */
    int32_t flags;        /* CUSAT_REQ_* */
    const float* sym;     /* xfecframe_len complex symbols, device (default) or
                             host; read when the frame is admitted, must stay
                             valid until its result is returned */
    uint8_t* hard_host;   /* k_ldpc/8 bytes of host memory for the hard
                             decisions, or NULL */
    uint64_t tag;         /* returned with the result */
    double arrival_s;     /* server clock (cusat_server_now); the frame is
                             not admitted before; < 0: now */
} cusat_request;

typedef struct {
    uint64_t tag;
    int32_t modcod, trials, bch_valid, reserved;
    double arrival_s, admit_s, done_s;  /* server clock, seconds */
} cusat_result;

/* No counterpart in the reference (its RX chain pool runs a fixed flight
 * ring per MODCOD chain, lib/cusat_dsp/rx_fec_chain.cc:281-627).  A
 * scheduler thread admits arrived requests, in order, into an arena of
 * hbm_budget device bytes (per frame: its symbols, hard decisions, two
 * counters) and launches them as mixed-MODCOD batches of at most max_batch
 * frames on `slots` streams; batches overlap on the device and requests
 * that arrive meanwhile join the next batch when a slot and memory free up.
 * Each frame's results equal those of a single-MODCOD cusat_rx_fec launch on
 * its symbols, whatever it was batched with. */
int cusat_server_create(const int32_t* modcods, int n_modcods, int max_trials, size_t hbm_budget, int slots,
                        int max_batch, cusat_server** out);
/* Stops the scheduler (requests not yet completed are dropped). */
void cusat_server_destroy(cusat_server* srv);
double cusat_server_now(const cusat_server* srv);
/* Learned weights (NULL: plain) for one MODCOD; only while nothing is
 * pending or in flight. */
int cusat_server_set_weights(cusat_server* srv, int modcod, const int16_t* weights, int n_iter);
/* Queues n requests (thread-safe); admitted in submission order once their
 * arrival time has passed. */
int cusat_server_submit(cusat_server* srv, const cusat_request* reqs, int n);
/* Up to max completed results, waiting up to wait_ms for the first; returns
 * the count or a negative error (a failed launch stops the server). */
int cusat_server_poll(cusat_server* srv, cusat_result* out, int max, int wait_ms);
/* out[0..7] = pending, batches launched, frames launched, largest batch,
 * most batches in flight, peak arena bytes, arena bytes, batches in flight */
int cusat_server_stats(cusat_server* srv, double* out);

/* ---------------------------------------------------------------------- */
/* Training the learned min-sum weights                                    */
/* ---------------------------------------------------------------------- */

typedef struct cusat_nms_trainer cusat_nms_trainer;

/* No counterpart in the reference.  The unrolled FP32 model of the layered
 * decoder with learnable {beta, alpha} per iteration (n_iter <= 64) and
 * check degree: per check, m_e = sign product of the other edges *
 * min(alpha * max(r_e - beta, 0), 127), r_e the smallest |extrinsic| of the
 * other edges; the reference's paired-layer schedule; loss = sum over
 * iterations t of w_t times the mean over bits of softplus(-y L) (y = +1 for
 * a 0 bit, L the APP after iteration t).  Forward and backward run on the GPU, one CTA per frame. */
int cusat_nms_trainer_create(int framesize, int rate, int n_iter, int max_batch, cusat_nms_trainer** out);
void cusat_nms_trainer_destroy(cusat_nms_trainer* tr);
/* out[0..5] = n_ldpc, k_ldpc, n_iter, max_batch, smallest and largest check degree */
int cusat_nms_trainer_info(const cusat_nms_trainer* tr, int32_t* out);
/* counts[d], d < 32: number of checks of degree d in the code */
int cusat_nms_trainer_degree_counts(const cusat_nms_trainer* tr, int32_t* counts);
/* batch frames of int16 LLRs (device, n_ldpc each, as the decoder takes them)
 * and their transmitted codewords (device, n_ldpc/8 bytes, MSB first);
 * theta_dev [n_iter][32][2] = {beta, alpha} (float, device); iter_w_dev
 * [n_iter] loss weight of each iteration's APP (device, or NULL: 1/n_iter
 * each).  Adds the sum
 * over frames of the loss to *loss_dev and, unless grad_dev is NULL, of its
 * gradient to grad_dev [n_iter][32][2].  Asynchronous on `stream`. */
int cusat_nms_train_step(cusat_nms_trainer* tr, const int16_t* llr_dev, const uint8_t* cw_dev, int batch,
                         const float* theta_dev, const float* iter_w_dev, float* grad_dev, float* loss_dev,
                         void* stream);

/* ---------------------------------------------------------------------- */
/* Decoding without device allocation                                      */
/* ---------------------------------------------------------------------- */

/* No counterpart in the reference.  For callers that may not allocate
 * device memory (a real-time thread under a no-allocation rule, a host
 * application whose memory pool owns every device allocation): decodes like
 * cusat_ldpc_decode_launch -- same kernel,
 * same results -- but every buffer besides the caller's LLRs (soft_dev,
 * batch * n_ldpc int16, device) and outputs (hard_out batch * k_ldpc/8
 * bytes, trials_out batch int32, device or mapped pinned) is a fixed array
 * inside the library: 24 MiB of message rows (which bounds the CTAs used:
 * 60 for normal rate 3/5), 64 KiB of code tables, a frame counter.  They
 * exist on every device that loads the library until the process exits.
 * Every call looks up their addresses on the current device and copies its
 * code's tables (at most 64 KiB, from a static host buffer) into the table
 * area on `stream` ahead of the decode.  All calls on a device share its
 * arrays: calls whose kernels overlap on the GPU race.  A call on a stream
 * that is capturing a CUDA graph returns CUSAT_ERR_UNSUPPORTED and enqueues
 * nothing.  Returns CUSAT_ERR_ARG when a code's tables or one frame's
 * message rows exceed the arrays (no DVB-S2/S2X code does). */
int cusat_ldpc_decode_noalloc(int framesize, int rate, int max_trials, const int16_t* soft_dev, int batch,
                              uint8_t* hard_out, int32_t* trials_out, void* stream);

/* ---------------------------------------------------------------------- */
/* PL receiver tail: located PLFRAMEs -> XFECFRAMEs                         */
/* ---------------------------------------------------------------------- */

typedef struct cusat_pl_extractor cusat_pl_extractor;

/* One located PLFRAME of a cusat_pl_extract call. */
typedef struct cusat_pl_frame {
    const float* payload;   /* device: the symbols after the 90-symbol PLHEADER (re, im), 8-byte aligned */
    float* data;            /* device: 90 S data symbols out (re, im), 8-byte aligned */
    const float* slot_rot;  /* device: per slot {rot re, rot im, step re, step im}, 16-byte aligned; NULL = 1 */
    int32_t pls_code;       /* 8-bit PLS code of the PLHEADER: sets the slots S and the pilot blocks */
    int32_t gold;           /* PL scrambling (Gold) code n, one of the extractor's */
} cusat_pl_frame;

/* Replaces pl_layout_from_code (lib/cusat_dsp/framing/plframe.h:66-73,
 * plframe.cc:221): out[0..10] = slots S, pilots, pilot blocks, data symbols
 * (90 S), payload symbols (data + 36 per pilot block), MODCOD index, frame
 * size, bits per symbol, dummy, deliverable (carries an XFECFRAME of a
 * supported MODCOD and frame size), reserved. */
int cusat_pl_layout(int pls_code, int32_t* out);

/* The scrambling rotation index R_n(i) (0..3, descrambling factor
 * e^{-j R pi/2}) of Gold code n for i < len: the sequence the reference's
 * pl_descrambling_sequence (lib/cusat_dsp/framing/pl_scrambler.h:17-18,
 * pl_scrambler.cc:47-71) turns into complex factors.  Host only. */
int cusat_pl_rotation_index(int gold, uint8_t* r, int len);

/* Replaces the data step of pl_receiver::process_payload
 * (lib/cusat_dsp/plrx/pl_receiver.cc:1694-1741, rotate_slot :1217-1282) for
 * a batch of frames the host-side synchroniser has located: each frame's
 * payload is descrambled, its pilot blocks (36 symbols after every 16 slots
 * when the PLS code signals pilots) are dropped, and slot s is
 * counter-rotated by slot_rot[s] (rot * step^i for its symbol i, the
 * reference's arithmetic, non-finite results set to 0) into data.  The
 * extractor holds the descrambling tables of the given Gold codes.
 * Asynchronous on `stream`; waits for the previous call's descriptor copy.
 * Errors: CUSAT_ERR_UNSUPPORTED for a PLS code without a decodable
 * XFECFRAME (dummy, reserved, unsupported MODCOD or frame size). */
int cusat_pl_extractor_create(const int32_t* gold_codes, int n_codes, int max_frames, cusat_pl_extractor** out);
void cusat_pl_extractor_destroy(cusat_pl_extractor* x);
int cusat_pl_extract(cusat_pl_extractor* x, const cusat_pl_frame* frames, int n, void* stream);

/* ---------------------------------------------------------------------- */
/* Post-FEC baseband stage                                                 */
/* ---------------------------------------------------------------------- */

typedef struct cusat_bb_extractor cusat_bb_extractor;

/* Replaces the RX chain's host post-processing (reference
 * rx_fec_chain.cc:604-626 with bb_scrambler.cc and bbframe_parser.cc): frames
 * whose LDPC decode failed (trials < 0) or whose BCH check failed are dropped,
 * the others descrambled (EN 302 307-1 5.2.2) and their BBHEADER checked
 * (CRC-8, DFL <= 8 K_bch - 80 and a multiple of 8, TS/GS generic packetized);
 * the DFL/8 data-field bytes of each accepted frame are packed into out_dev in
 * frame order, a frame whose field does not fit the room left yielding
 * nothing.  All pointers are device memory; hard_dev holds frame f's decoded
 * bits at f * hard_stride (>= K_bch/8, e.g. the decoder's k_ldpc/8);
 * lengths_dev[f] = bytes of frame f, offsets_dev[f] = where they start,
 * offsets_dev[batch] = total.  Asynchronous on `stream`. */
int cusat_bb_extractor_create(int framesize, int rate, cusat_bb_extractor** out);
void cusat_bb_extractor_destroy(cusat_bb_extractor* x);
int cusat_bb_extract(cusat_bb_extractor* x, const uint8_t* hard_dev, int hard_stride, const int32_t* trials_dev,
                     const int32_t* bch_valid_dev, int batch, uint8_t* out_dev, int max_out, int32_t* lengths_dev,
                     int32_t* offsets_dev, void* stream);
/* The same over frames of different codes: kbch_dev[f] = K_bch/8 of frame f
 * (device or mapped pinned memory), each at most the extractor's code's
 * (create it for the longest code of the batch) and at most hard_stride. */
int cusat_bb_extract_frames(cusat_bb_extractor* x, const uint8_t* hard_dev, int hard_stride, const int32_t* kbch_dev,
                            const int32_t* trials_dev, const int32_t* bch_valid_dev, int batch, uint8_t* out_dev,
                            int max_out, int32_t* lengths_dev, int32_t* offsets_dev, void* stream);

/* ---------------------------------------------------------------------- */
/* Frame-at-a-time receive chain and per-MODCOD pool                       */
/* ---------------------------------------------------------------------- */

/* Shared in-flight budget of decode blocks (frames), replacing
 * cusat_dsp::gpu_decode_budget (lib/cusat_dsp/rx_fec_chain.h:52-59).
 * cap < 0: the default, one frame per SM, overridden by the environment
 * variable CUSAT_LDPC_INFLIGHT_CAP; cap 0: unlimited.  Chains keep their
 * share alive after the handle is destroyed.  info: out[0] = cap,
 * out[1] = frames in flight. */
typedef struct cusat_decode_budget cusat_decode_budget;
int cusat_decode_budget_create(int cap, cusat_decode_budget** out);
void cusat_decode_budget_destroy(cusat_decode_budget* b);
int cusat_decode_budget_info(const cusat_decode_budget* b, int32_t* out);

/* Decision-directed SNR (linear) of n_sym symbols (re, im): QPSK by the
 * signs, other constellations by the nearest point on every stride-th
 * symbol.  Replaces qpsk_snr_dd / constellation_snr_dd
 * (lib/cusat_dsp/modulation/dd_snr.h:17-21). */
int cusat_dd_snr(int modulation, int rate, int framesize, const float* sym, int n_sym, int stride, float* out);

/* One MODCOD's frame-at-a-time receive chain, replacing cusat_dsp::rx_fec_chain
 * (lib/cusat_dsp/rx_fec_chain.h:61-297) call for call: frames accumulate
 * into micro-batches in a 128-slot flight ring, each full micro-batch is
 * launched at once (within the decode budget) on the next of the chain's
 * streams (n_gpu_streams, or more when that many micro-batches cannot fill
 * the default in-flight budget: launches on one stream run one after
 * another), completed slots are drained in submission order into GSE output
 * (the data fields of frames that converged, passed BCH and carry a valid
 * GSE BBHEADER) and per-frame data-field sizes.  Every 32nd submitted frame
 * re-estimates the SNR (decision-directed; pilot SNR for >= 128 points).
 * Return conventions: submit / drain return 1 when output is available,
 * 0 when not, < 0 on error (the reference aborts); a frame of the wrong
 * length or one that finds the ring full is counted as dropped and as a
 * frame error, as in the reference.  Not thread-safe (like the reference);
 * the launch lock (rx_fec_chain::set_cuda_mutex) serialises the chain's CUDA
 * launches with the caller's. */
typedef struct cusat_rx_chain cusat_rx_chain;
int cusat_rx_chain_create(int framesize, int rate, int modulation, int max_trials, int cuda_max_batch,
                          int n_gpu_streams, int micro_batch, cusat_rx_chain** out);
void cusat_rx_chain_destroy(cusat_rx_chain* c);
/* out[0..5] = xfecframe_len, kbch_bytes, batch_size(), max_output_bytes(),
 * micro_batch, streams in use (at least n_gpu_streams; enough to fill the
 * default in-flight budget) */
int cusat_rx_chain_info(const cusat_rx_chain* c, int32_t* out);
int cusat_rx_chain_set_weights(cusat_rx_chain* c, const int16_t* weights, int n_iter);
int cusat_rx_chain_set_decode_budget(cusat_rx_chain* c, const cusat_decode_budget* b);
int cusat_rx_chain_set_launch_lock(cusat_rx_chain* c, void (*lock)(void*), void (*unlock)(void*), void* ctx);
void cusat_rx_chain_set_block_when_full(cusat_rx_chain* c, int on);
/* No counterpart in the reference (opt-in; 0, the default, copies on the
 * submitting thread as the reference does): split each frame's copy into the
 * pinned ring across `helpers` extra threads, which spin while frames keep
 * coming and sleep after 0.5 ms without one. */
int cusat_rx_chain_set_copy_threads(cusat_rx_chain* c, int helpers);
void cusat_rx_chain_update_snr(cusat_rx_chain* c, float snr_db);
/* symbols: n_symbols complex (re, im) host values; copied before return */
int cusat_rx_chain_submit_xfecframe(cusat_rx_chain* c, const float* symbols, int n_symbols);
int cusat_rx_chain_drain_completed(cusat_rx_chain* c);
int cusat_rx_chain_get_gse_output(cusat_rx_chain* c, uint8_t* out, int max_bytes);
/* returns the number of sizes; copies up to max of them */
int cusat_rx_chain_gse_dfl_sizes(const cusat_rx_chain* c, int32_t* out, int max);
int cusat_rx_chain_launch_partial(cusat_rx_chain* c);
int cusat_rx_chain_flush(cusat_rx_chain* c);
int cusat_rx_chain_reset(cusat_rx_chain* c);
int cusat_rx_chain_warmup(cusat_rx_chain* c);
/* out[0..11] = frame_count, frame_error_count, gpu_drop_count, gpu_inflight
 * (slots), gpu_pending_launch, force_drain_count, pending_count, snr_db,
 * precision (LLR gain), noise variance, age of the partial micro-batch (s),
 * output bytes waiting */
int cusat_rx_chain_stats(const cusat_rx_chain* c, double* out);

/* One chain per enabled MODCOD behind one decode budget, replacing
 * cusat_dsp::rx_fec_pool (lib/cusat_dsp/rx_fec_pool.h:25-140).  modcods:
 * n triples (modcod_idx, modulation, rate), the caller's find_modcod()
 * lookup.  A MODCOD change flushes the previous MODCOD's chain before the new
 * frame is admitted, so output blocks come out in submission order;
 * submit of a MODCOD not enabled is skipped (returns 0).  Chains are visited
 * in creation order. */
typedef struct cusat_rx_pool cusat_rx_pool;
int cusat_rx_pool_create(int framesize, const int32_t* modcods, int n_modcods, int max_trials, int cuda_max_batch,
                         int n_gpu_streams, int micro_batch, cusat_rx_pool** out);
/* The same pool with every MODCOD in one slot ring (no counterpart in the
 * reference, which runs one chain per MODCOD and waits for the previous
 * MODCOD's chain at every MODCOD change): frames of any MODCOD fill slots of
 * slot_frames frames, each slot one multi-MODCOD launch (cusat_batch) with the
 * BB stage per frame code, drained in submission order; no wait at a MODCOD
 * change.  micro_batch keeps the reference's per-MODCOD micro-batches as the
 * points where a frame's LLR gain is fixed (its MODCOD's gain when that
 * micro-batch fills, the MODCOD changes, it goes stale or the pool is
 * flushed: the gain the reference's chain launches it with), so the output
 * equals the per-MODCOD pool's whenever that pool's launches are not deferred
 * by the in-flight budget.  Output blocks hold one run of same-MODCOD frames.
 * cusat_rx_pool_chain returns NULL for this pool. */
int cusat_rx_pool_create_mixed(int framesize, const int32_t* modcods, int n_modcods, int max_trials,
                               int n_gpu_streams, int micro_batch, int slot_frames, cusat_rx_pool** out);
void cusat_rx_pool_destroy(cusat_rx_pool* p);
/* the pool's chain of one MODCOD (owned by the pool), or NULL */
cusat_rx_chain* cusat_rx_pool_chain(cusat_rx_pool* p, int modcod);
int cusat_rx_pool_submit(cusat_rx_pool* p, const float* symbols, int n_symbols, int modcod);
int cusat_rx_pool_get_gse_output(cusat_rx_pool* p, uint8_t* out, int max_bytes);
int cusat_rx_pool_gse_dfl_sizes(const cusat_rx_pool* p, int32_t* out, int max);
int cusat_rx_pool_drain_all_completed(cusat_rx_pool* p);
int cusat_rx_pool_finish_all_pending(cusat_rx_pool* p);
int cusat_rx_pool_launch_stale(cusat_rx_pool* p, double max_age_ms);
int cusat_rx_pool_reset_all(cusat_rx_pool* p);
int cusat_rx_pool_warmup_all(cusat_rx_pool* p);
void cusat_rx_pool_update_snr(cusat_rx_pool* p, int modcod, float snr_db);
/* As cusat_rx_chain_set_copy_threads, for every chain of the pool. */
int cusat_rx_pool_set_copy_threads(cusat_rx_pool* p, int helpers);
int cusat_rx_pool_set_launch_lock(cusat_rx_pool* p, void (*lock)(void*), void (*unlock)(void*), void* ctx);
/* out[0..4] = total frames, total errors, total GPU drops, max_output_bytes,
 * data SNR (dB) of the last decoded MODCOD */
int cusat_rx_pool_stats(const cusat_rx_pool* p, double* out);
/* 1 and the counters if the MODCOD is enabled, else 0 */
int cusat_rx_pool_modcod_counters(const cusat_rx_pool* p, int modcod, uint64_t* frames, uint64_t* errors);

/* ---------------------------------------------------------------------- */
/* Traffic generation on the GPU                                           */
/* ---------------------------------------------------------------------- */

typedef struct cusat_generator cusat_generator;

/* The transmitter side on the device, for generating training and benchmark
 * traffic (reference ldpc_encode.cc, cuda/ldpc_encode_kernel.cu,
 * cuda/bch_common.cuh with Encode = true, cuda/mapper_kernel.cu):
 * systematic BCH encode, IRA LDPC encode and constellation mapping of a batch
 * of messages; equal bit for bit to cusat_gen_encode and cusat_gen_map. */
int cusat_generator_create(int modulation, int rate, int framesize, int max_batch, cusat_generator** out);
void cusat_generator_destroy(cusat_generator* g);
/* out[0..3] = message bytes (k_bch/8), codeword bytes (n_ldpc/8), xfecframe_len, max_batch */
int cusat_generator_info(const cusat_generator* g, int32_t* out);
/* msg_dev: batch x k_bch/8 bytes; cw_dev: batch x n_ldpc/8 bytes (out);
 * sym_dev: batch x xfecframe_len complex symbols (out, or NULL); all
 * device memory; asynchronous on `stream`. */
int cusat_generate(cusat_generator* g, const uint8_t* msg_dev, int batch, uint8_t* cw_dev, float* sym_dev,
                   void* stream);

/* ---------------------------------------------------------------------- */
/* Code description and traffic generation (host side; used to generate     */
/* test and benchmark traffic, not part of the receive path)               */
/* ---------------------------------------------------------------------- */

/* out[0..11] = n_ldpc, k_ldpc, k_bch, n_bch, t, bch_degree, q, n_steps,
 * lanes, kernel slot bucket, Tanner edges, largest circulants per layer.
 * Reference get_fec_params (lib/cusat_dsp/fec/code_params.cc:102-108) and
 * create_ldpc_table (lib/cusat_dsp/ldpc_table_factory.cc:97-102). */
int cusat_code_info(int framesize, int rate, int32_t* out);
/* Replaces ldpc_encode::encode (lib/cusat_dsp/ldpc_encode.h:31, the
 * systematic IRA encoder of EN 302 307 Annex C): batch codewords, k_ldpc/8
 * info bytes in (the BCH codeword), n_ldpc/8 bytes out (info then parity,
 * MSB first).  Host code; test traffic and the reference's encode callers. */
int cusat_ldpc_encode(int framesize, int rate, const uint8_t* info, uint8_t* cw, int batch);

/* BCH + LDPC encode: msg k_bch/8 bytes -> codeword n_ldpc/8 bytes per frame
 * (reference bch_encode fec/bch_code.cc:124-144, IRA encoder
 * ldpc_encode.cc:6-13). */
int cusat_gen_encode(int framesize, int rate, const uint8_t* msg, uint8_t* cw, int batch);
/* Interleave + map codewords to xfecframe_len symbols (re, im) per frame
 * (reference mapper.cc:75-86, cuda/mapper_kernel.cu:22-51); 128APSK: 6
 * stuffing bits of 0 ahead of the interleaver and 12 padding symbols on the
 * all-ones label after it (mapper.cc:28-62). */
int cusat_gen_map(int modulation, int rate, int framesize, const uint8_t* cw, int batch, float* sym);
/* Constellation points (2 * n_points floats, by label), interleaver column
 * offsets (8) and out[0..5] = n_mod, n_points, fecframe_len, xfecframe_len,
 * interleaved_len, demap kind (0 QPSK, 1 8PSK, 2 log-MAP).  Reference
 * make_constellation (modulation/constellation.cc:461) and
 * make_bit_interleaver (modulation/bit_interleaver.cc:76-96). */
int cusat_modcod_info(int modulation, int rate, int framesize, float* points, uint32_t* col,
                      int32_t* out);
float cusat_modcod_capped_llr_gain(int modulation, int rate, int framesize, float llr_gain);

#ifdef __cplusplus
}
#endif
#endif /* CUSAT_FEC_H */
