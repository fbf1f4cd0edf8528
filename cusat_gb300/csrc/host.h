// Host-side construction of everything the FEC kernels consume: decoding
// plans of the LDPC codes, BCH tables, constellations and interleavers.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace cusat {

// Kernel instantiations: circulant slots per layer (CMAX) buckets.
int cmax_bucket(int cnt_max);

struct CodePlan {
    int framesize = 0, rate = 0;
    std::string name;
    int N = 0, K = 0, R = 0, q = 0;
    int n_steps = 0;
    int cnt_max = 0;   // largest number of circulants of a layer
    int cmax = 0;      // kernel bucket >= cnt_max
    int lanes = 1;     // 2 when the schedule pairs layers
    int msg_row = 16;  // bytes per check row of messages
    int dv_max = 0;    // largest information-bit degree
    int fast_lim = 0;  // |LLR| bound of the saturation-free path
    int max_stage = 0; // stage rows used by the busiest step
    int links_total = 0;
    std::vector<uint32_t> tab;      // [q * cmax * 4] slot descriptors (fec_consts.h)
    std::vector<uint8_t> cnt;       // [q] circulants per layer
    std::vector<int16_t> sched;     // [n_steps * 2]
    std::vector<uint8_t> step_conf; // [n_steps] 0, kConfDefer or kConfMid
    std::vector<uint16_t> item_off; // [n_steps + 1]
    std::vector<uint32_t> items;    // [n_items * 2] shared-group items
    // BCH outer code
    int k_bch = 0, n_bch = 0, t = 0, p = 0;
    uint64_t gen[4] = {0, 0, 0, 0};
    // raw ETSI rows (for the encoder)
    const uint8_t* row_deg = nullptr;
    const uint16_t* addr = nullptr;
    int n_rows = 0;
};

// Cached, thread-safe; nullptr (and a message) for an unsupported code.
const CodePlan* get_code_plan(int framesize, int rate, std::string* err);

// BCH tables for a generator of degree p (multiple of 8, <= 256) and a
// codeword of n_bytes bytes, in the layout of the check kernel.
struct BchTables {
    int p = 0, words = 0, bytes = 0;  // degree, 64-bit words, remainder bytes
    unsigned n_bytes = 0, chunk = 0, lead = 0;
    std::vector<uint64_t> lut;    // [256 * words]: b(x) x^p mod g
    std::vector<uint64_t> tree;   // [5][bytes][256][words]: (b x^(8j)) x^(8 chunk 2^k) mod g
};
// gen: 4 words, bit i of word i/64 = coefficient of x^i (monic, degree p).
bool build_bch_tables(const uint64_t* gen, int p, unsigned n_bytes, BchTables* out, std::string* err);
// Encoder LUT of the reference layout (256 x 4 words): T[b] = b(x) x^p mod g.
void bch_encoder_lut(const uint64_t* gen, int p, uint64_t* lut256x4);

struct ModcodDemap {
    int modulation = 0, rate = 0, framesize = 0;
    int n_mod = 0, n_points = 0;
    int fec_len = 0, xfec = 0, interleaved_len = 0;
    int kind = 0;            // 0 QPSK formula, 1 8PSK formula, 2 log-MAP
    uint32_t col[8] = {0};   // deinterleave column offsets (QPSK: 0)
    float dmax = 0.0f;       // loudest-bit squared distance
    float llr_target = 320.0f;
    std::vector<float> pts;  // [2 * n_points] (re, im) by label
};
bool build_modcod_demap(int modulation, int rate, int framesize, ModcodDemap* out, std::string* err);
float capped_llr_gain(const ModcodDemap& d, float llr_gain);

// Constellation points by label (first bit = MSB), unit average energy for
// APSK; returns bits per symbol or -1.
int make_constellation(int modulation, int rate, int framesize, std::vector<float>* pts);
// Interleaver: column offsets; returns the number of columns (0 = none).
int make_interleaver(int modulation, int rate, int framesize, uint32_t col[8], uint32_t* rows);

// Decision-directed SNR estimates (linear) of received symbols (re, im):
// QPSK by the signs, any constellation by its nearest point on every
// stride-th symbol.
float dd_snr_qpsk(const float* sym, int n_sym);
float dd_snr_points(const std::vector<float>& pts, const float* sym, int n_sym, int stride);

// Product-side encoders used to generate test traffic (bench, training).
void bch_encode_frames(const CodePlan& c, const uint8_t* msg, uint8_t* cw, int B);
void ldpc_encode_frames(const CodePlan& c, const uint8_t* info, uint8_t* cw, int B);
// Maps N/8-byte codewords to xfec symbols (re, im) with interleaving.
void map_frames(const ModcodDemap& d, const uint8_t* cw, int B, float* sym);

}  // namespace cusat
