// extern "C" accessors over the reference's own host code (test
// infrastructure only; compiled into oracle/_ref with the reference sources
// by oracle/build.py, never shipped).  Each accessor returns what the named
// reference function returns, flattened into plain arrays.
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "fec/bch_code.h"
#include "fec/code_params.h"
#include "ldpc_table_factory.h"
#include "modulation/bit_interleaver.h"
#include "modulation/constellation.h"
#include "modulation/dd_snr.h"
#include "cuda/ldpc_message_update.h"
#include "bb_header.h"
#include "bb_scrambler.h"
#include "bbframe_parser.h"
#include "framing/pl_scrambler.h"
#include "framing/plframe.h"

using namespace cusat_dsp;

extern "C" {

// get_fec_params (fec/code_params.cc:102-108): out = k_bch, n_bch, t, k_ldpc, n_ldpc
int ref_fec_params(int fs, int rate, uint32_t* out)
{
    try {
        fec_params_t p = get_fec_params((fecframe_size_t)fs, (code_rate_t)rate);
        out[0] = p.k_bch; out[1] = p.n_bch; out[2] = p.t_bch; out[3] = p.k_ldpc; out[4] = p.n_ldpc;
        return 0;
    } catch (...) {
        return -1;
    }
}

// make_bch_code (fec/bch_code.cc:99-122): generator words and degree
int ref_bch_generator(int fs, int n_bits, int t, uint64_t* gen4)
{
    bch_code_t c = make_bch_code((fecframe_size_t)fs, n_bits, t);
    for (int w = 0; w < 4; w++) gen4[w] = c.generator[w];
    return c.parity_bits;
}

// bch_encode (fec/bch_code.cc:124-144)
int ref_bch_encode(int fs, int n_bits, int t, const uint8_t* msg, uint8_t* cw)
{
    bch_code_t c = make_bch_code((fecframe_size_t)fs, n_bits, t);
    bch_encode(c, msg, cw);
    return 0;
}

// make_bit_interleaver (modulation/bit_interleaver.cc:76-96)
int ref_interleaver(int mod, int rate, int fs, uint32_t* col8, uint32_t* rows)
{
    try {
        bit_interleaver_t il = make_bit_interleaver((modulation_t)mod, (code_rate_t)rate, (fecframe_size_t)fs);
        for (int i = 0; i < 8; i++) col8[i] = il.col_offset[i];
        *rows = il.rows;
        return il.n_cols;
    } catch (...) {
        return -1;
    }
}

// qpsk_snr_dd / constellation_snr_dd (modulation/dd_snr.cc:23-47)
float ref_dd_snr(int mod, int rate, int fs, const float* sym, int n_sym, int stride, int qpsk)
{
    const complexf* z = reinterpret_cast<const complexf*>(sym);
    if (qpsk)
        return qpsk_snr_dd(z, n_sym);
    constellation_t c = make_constellation((modulation_t)mod, (code_rate_t)rate, (fecframe_size_t)fs);
    return constellation_snr_dd(c, z, n_sym, stride);
}

// make_constellation (modulation/constellation.cc:461-496): points by label
int ref_constellation(int mod, int rate, int fs, float* re, float* im)
{
    try {
        constellation_t c = make_constellation((modulation_t)mod, (code_rate_t)rate, (fecframe_size_t)fs);
        for (int i = 0; i < c.n_points; i++) { re[i] = c.points[i].real(); im[i] = c.points[i].imag(); }
        return c.bits_per_sym;
    } catch (...) {
        return -1;
    }
}

// create_ldpc_table (ldpc_table_factory.cc:97-102): n, k, n_rows, links_total,
// links_max_cn and the flat address rows.
int ref_ldpc_table(int fs, int rate, int32_t* info, uint8_t* deg, uint16_t* addr, int addr_cap)
{
    ldpc_code* c = create_ldpc_table((fecframe_size_t)fs, (code_rate_t)rate);
    if (!c) return -1;
    info[0] = c->n; info[1] = c->k; info[2] = c->n_rows; info[3] = c->links_total; info[4] = c->links_max_cn;
    int total = (int)c->row_off[c->n_rows];
    if (total <= addr_cap) {
        memcpy(deg, c->row_deg, c->n_rows);
        memcpy(addr, c->addr, total * sizeof(uint16_t));
    }
    delete c;
    return total;
}

// ldpc_make_bnl_update (cuda/ldpc_message_update.h:25-35)
int ref_bnl_update(int raw, int old, int32_t* delta)
{
    cuda::ldpc_bnl_update_t u = cuda::ldpc_make_bnl_update(raw, old);
    *delta = u.delta;
    return u.message;
}
// bb_scrambler_sequence (bb_scrambler.cc:43-49): the first n PRBS bytes
int ref_bb_prbs(uint8_t* out, int n)
{
    if (n < 0 || (size_t)n > BB_SCRAMBLER_MAX_BYTES)
        return -1;
    memcpy(out, bb_scrambler_sequence(), (size_t)n);
    return 0;
}

// bb_scramble (bb_scrambler.cc:53-67)
int ref_bb_scramble(const uint8_t* in, uint8_t* out, int n)
{
    try {
        bb_scramble(in, out, (size_t)n);
        return 0;
    } catch (...) {
        return -1;
    }
}

// extract_gse_datafield (bbframe_parser.cc:44-56) on an already descrambled BBFRAME
int ref_extract_datafield(const uint8_t* bbframe, int kbch, uint8_t* out, int max_out)
{
    return extract_gse_datafield(bbframe, (size_t)kbch, out, max_out);
}

// bb_header::build_gse_bbframe (bb_header.cc): an unscrambled GSE BBFRAME
int ref_build_bbframe(int fs, int rate, const uint8_t* data, int len, uint8_t* out)
{
    try {
        bb_header h((fecframe_size_t)fs, (code_rate_t)rate);
        return (int)h.build_gse_bbframe(data, (unsigned)len, out);
    } catch (...) {
        return -1;
    }
}

}

extern "C" {

// pl_layout_from_code (framing/plframe.cc:221): out = slots, pilots, pilot
// blocks, data symbols, payload symbols, MODCOD index, frame size, bits per
// symbol, dummy, deliverable, reserved
int ref_pl_layout(int code, int32_t* out)
{
    const pl_layout l = pl_layout_from_code((uint8_t)code);
    out[0] = l.slots; out[1] = l.pilots; out[2] = l.pilot_block_count(); out[3] = l.data_symbols();
    out[4] = l.payload_symbols(); out[5] = l.modcod; out[6] = (int)l.fec_size; out[7] = l.bits_per_symbol;
    out[8] = l.dummy; out[9] = l.deliverable(); out[10] = l.reserved;
    return 0;
}

// pl_descrambling_sequence (framing/pl_scrambler.cc:47-71): the factors as
// (re, im) float pairs
int ref_pl_descrambling(int gold, float* seq, int len)
{
    try {
        std::vector<complexf> v(len);
        pl_descrambling_sequence(gold, v.data(), len);
        for (int i = 0; i < len; i++) {
            seq[2 * i] = v[i].real();
            seq[2 * i + 1] = v[i].imag();
        }
        return 0;
    } catch (...) {
        return -1;
    }
}

}  // extern "C"
