/*
 * Standard data shared by the CUDA library and by the CPU oracle.
 *
 * Everything here is a table of ETSI EN 302 307-1 (DVB-S2) / EN 302 307-2
 * (DVB-S2X) or an enumeration whose numeric order must equal the reference
 * library's, so that a caller of the reference can pass its own enum values
 * through the C ABI unchanged:
 *   - code rates, frame sizes, modulations: reference
 *     lib/cusat_dsp/include/cusat_dsp/modcod_types.h:14-95;
 *   - BCH/LDPC dimensions (EN 302 307-1 Tables 5a/5b, -2 Tables 4a-4c):
 *     reference lib/cusat_dsp/fec/code_params.cc:17-78;
 *   - BCH minimal polynomials g1..g12 (EN 302 307-1 Tables 6a/6b):
 *     reference lib/cusat_dsp/fec/bch_code.cc:14-19;
 *   - (frame size, rate) -> parity-check table: reference
 *     lib/cusat_dsp/ldpc_table_factory.cc:17-95.
 * Plain C so that the oracle (C99) and the CUDA/C++ library include the same
 * numbers; no algorithm lives here.
 */
#ifndef CUSAT_DATA_H
#define CUSAT_DATA_H

#include <stdint.h>

enum {
    CUSAT_RATE_1_4, CUSAT_RATE_1_3, CUSAT_RATE_2_5, CUSAT_RATE_1_2, CUSAT_RATE_3_5,
    CUSAT_RATE_2_3, CUSAT_RATE_3_4, CUSAT_RATE_4_5, CUSAT_RATE_5_6, CUSAT_RATE_8_9,
    CUSAT_RATE_9_10,
    CUSAT_RATE_11_45, CUSAT_RATE_4_15, CUSAT_RATE_13_45, CUSAT_RATE_14_45, CUSAT_RATE_9_20,
    CUSAT_RATE_7_15, CUSAT_RATE_90_180, CUSAT_RATE_8_15, CUSAT_RATE_96_180, CUSAT_RATE_11_20,
    CUSAT_RATE_100_180, CUSAT_RATE_26_45, CUSAT_RATE_104_180, CUSAT_RATE_18_30,
    CUSAT_RATE_28_45, CUSAT_RATE_23_36, CUSAT_RATE_116_180, CUSAT_RATE_20_30,
    CUSAT_RATE_124_180, CUSAT_RATE_25_36, CUSAT_RATE_32_45, CUSAT_RATE_128_180,
    CUSAT_RATE_13_18, CUSAT_RATE_22_30, CUSAT_RATE_132_180, CUSAT_RATE_135_180,
    CUSAT_RATE_7_9, CUSAT_RATE_140_180, CUSAT_RATE_154_180,
    CUSAT_RATE_VLSNR_SET1_QPSK_2_9, CUSAT_RATE_VLSNR_SET1_BPSK_1_5,
    CUSAT_RATE_VLSNR_SET1_BPSK_11_45, CUSAT_RATE_VLSNR_SET1_BPSK_1_3,
    CUSAT_RATE_VLSNR_SET1_BPSKS_1_5, CUSAT_RATE_VLSNR_SET1_BPSKS_11_45,
    CUSAT_RATE_VLSNR_SET2_BPSK_1_5, CUSAT_RATE_VLSNR_SET2_BPSK_4_15,
    CUSAT_RATE_VLSNR_SET2_BPSK_1_3,
    CUSAT_RATE_COUNT
};

enum { CUSAT_FECFRAME_NORMAL, CUSAT_FECFRAME_SHORT, CUSAT_FECFRAME_MEDIUM };

enum {
    CUSAT_MOD_QPSK, CUSAT_MOD_8PSK, CUSAT_MOD_8APSK, CUSAT_MOD_16APSK, CUSAT_MOD_32APSK,
    CUSAT_MOD_64APSK, CUSAT_MOD_128APSK, CUSAT_MOD_256APSK
};

static inline int cusat_fecframe_bits(int framesize)
{
    return framesize == CUSAT_FECFRAME_NORMAL ? 64800
         : framesize == CUSAT_FECFRAME_SHORT ? 16200 : 32400;
}

/* One row of the BCH/LDPC dimension tables. */
typedef struct { int rate; uint32_t k_bch, n_bch, t; } cusat_bch_row;

static const cusat_bch_row cusat_bch_rows_normal[] = {
    {CUSAT_RATE_1_4, 16008, 16200, 12}, {CUSAT_RATE_1_3, 21408, 21600, 12},
    {CUSAT_RATE_2_5, 25728, 25920, 12}, {CUSAT_RATE_1_2, 32208, 32400, 12},
    {CUSAT_RATE_3_5, 38688, 38880, 12}, {CUSAT_RATE_2_3, 43040, 43200, 10},
    {CUSAT_RATE_3_4, 48408, 48600, 12}, {CUSAT_RATE_4_5, 51648, 51840, 12},
    {CUSAT_RATE_5_6, 53840, 54000, 10}, {CUSAT_RATE_8_9, 57472, 57600, 8},
    {CUSAT_RATE_9_10, 58192, 58320, 8},
    {CUSAT_RATE_VLSNR_SET1_QPSK_2_9, 14208, 14400, 12}, {CUSAT_RATE_13_45, 18528, 18720, 12},
    {CUSAT_RATE_9_20, 28968, 29160, 12}, {CUSAT_RATE_90_180, 32208, 32400, 12},
    {CUSAT_RATE_96_180, 34368, 34560, 12}, {CUSAT_RATE_11_20, 35448, 35640, 12},
    {CUSAT_RATE_100_180, 35808, 36000, 12}, {CUSAT_RATE_104_180, 37248, 37440, 12},
    {CUSAT_RATE_26_45, 37248, 37440, 12}, {CUSAT_RATE_18_30, 38688, 38880, 12},
    {CUSAT_RATE_28_45, 40128, 40320, 12}, {CUSAT_RATE_23_36, 41208, 41400, 12},
    {CUSAT_RATE_116_180, 41568, 41760, 12}, {CUSAT_RATE_20_30, 43008, 43200, 12},
    {CUSAT_RATE_124_180, 44448, 44640, 12}, {CUSAT_RATE_25_36, 44808, 45000, 12},
    {CUSAT_RATE_128_180, 45888, 46080, 12}, {CUSAT_RATE_13_18, 46608, 46800, 12},
    {CUSAT_RATE_132_180, 47328, 47520, 12}, {CUSAT_RATE_22_30, 47328, 47520, 12},
    {CUSAT_RATE_135_180, 48408, 48600, 12}, {CUSAT_RATE_140_180, 50208, 50400, 12},
    {CUSAT_RATE_7_9, 50208, 50400, 12}, {CUSAT_RATE_154_180, 55248, 55440, 12},
};

static const cusat_bch_row cusat_bch_rows_short[] = {
    {CUSAT_RATE_1_4, 3072, 3240, 12}, {CUSAT_RATE_1_3, 5232, 5400, 12},
    {CUSAT_RATE_2_5, 6312, 6480, 12}, {CUSAT_RATE_1_2, 7032, 7200, 12},
    {CUSAT_RATE_3_5, 9552, 9720, 12}, {CUSAT_RATE_2_3, 10632, 10800, 12},
    {CUSAT_RATE_3_4, 11712, 11880, 12}, {CUSAT_RATE_4_5, 12432, 12600, 12},
    {CUSAT_RATE_5_6, 13152, 13320, 12}, {CUSAT_RATE_8_9, 14232, 14400, 12},
    {CUSAT_RATE_11_45, 3792, 3960, 12}, {CUSAT_RATE_4_15, 4152, 4320, 12},
    {CUSAT_RATE_14_45, 4872, 5040, 12}, {CUSAT_RATE_7_15, 7392, 7560, 12},
    {CUSAT_RATE_8_15, 8472, 8640, 12}, {CUSAT_RATE_26_45, 9192, 9360, 12},
    {CUSAT_RATE_32_45, 11352, 11520, 12},
    {CUSAT_RATE_VLSNR_SET1_BPSKS_1_5, 2512, 2680, 12},
    {CUSAT_RATE_VLSNR_SET1_BPSKS_11_45, 3792, 3960, 12},
    {CUSAT_RATE_VLSNR_SET2_BPSK_1_5, 3072, 3240, 12},
    {CUSAT_RATE_VLSNR_SET2_BPSK_4_15, 4152, 4320, 12},
    {CUSAT_RATE_VLSNR_SET2_BPSK_1_3, 5232, 5400, 12},
};

static const cusat_bch_row cusat_bch_rows_medium[] = {
    {CUSAT_RATE_VLSNR_SET1_BPSK_1_5, 5660, 5840, 12},
    {CUSAT_RATE_VLSNR_SET1_BPSK_11_45, 7740, 7920, 12},
    {CUSAT_RATE_VLSNR_SET1_BPSK_1_3, 10620, 10800, 12},
};

/* Looks up (k_bch, n_bch, t) for a frame size and rate; NULL if undefined. */
static inline const cusat_bch_row* cusat_find_bch_row(int framesize, int rate)
{
    const cusat_bch_row* rows;
    int n;
    if (framesize == CUSAT_FECFRAME_NORMAL) {
        rows = cusat_bch_rows_normal;
        n = (int)(sizeof(cusat_bch_rows_normal) / sizeof(rows[0]));
    } else if (framesize == CUSAT_FECFRAME_SHORT) {
        rows = cusat_bch_rows_short;
        n = (int)(sizeof(cusat_bch_rows_short) / sizeof(rows[0]));
    } else if (framesize == CUSAT_FECFRAME_MEDIUM) {
        rows = cusat_bch_rows_medium;
        n = (int)(sizeof(cusat_bch_rows_medium) / sizeof(rows[0]));
    } else {
        return 0;
    }
    for (int i = 0; i < n; i++)
        if (rows[i].rate == rate)
            return &rows[i];
    return 0;
}

/* BCH minimal polynomials g1..g12 (bit i = coefficient of x^i) over
 * GF(2^16) (normal), GF(2^14) (short), GF(2^15) (medium). */
static const uint32_t cusat_bch_minpoly[3][12] = {
    {0x1002D, 0x10173, 0x10FBD, 0x15A55, 0x11F2F, 0x1F7B5,
     0x1AF65, 0x17367, 0x10EA1, 0x175A7, 0x13A2D, 0x11AE3},
    {0x402B, 0x4941, 0x4647, 0x5591, 0x6B55, 0x6389,
     0x6CE5, 0x4F21, 0x460F, 0x5A49, 0x5811, 0x65EF},
    {0x802D, 0x8C93, 0xB555, 0x8D6D, 0x94D7, 0xB0D1,
     0xD8B5, 0xCB55, 0xBAB7, 0xBC9F, 0x8A17, 0xED15},
};

/* (frame size, rate) -> name of the ETSI parity-check table, or NULL. */
static inline const char* cusat_table_name(int framesize, int rate)
{
    if (framesize == CUSAT_FECFRAME_NORMAL) {
        switch (rate) {
        case CUSAT_RATE_1_4: return "s2_b1";
        case CUSAT_RATE_1_3: return "s2_b2";
        case CUSAT_RATE_2_5: return "s2_b3";
        case CUSAT_RATE_1_2: return "s2_b4";
        case CUSAT_RATE_3_5: return "s2_b5";
        case CUSAT_RATE_2_3: return "s2_b6";
        case CUSAT_RATE_3_4: return "s2_b7";
        case CUSAT_RATE_4_5: return "s2_b8";
        case CUSAT_RATE_5_6: return "s2_b9";
        case CUSAT_RATE_8_9: return "s2_b10";
        case CUSAT_RATE_9_10: return "s2_b11";
        case CUSAT_RATE_VLSNR_SET1_QPSK_2_9: return "s2x_b1";
        case CUSAT_RATE_13_45: return "s2x_b2";
        case CUSAT_RATE_9_20: return "s2x_b3";
        case CUSAT_RATE_90_180: return "s2x_b11";
        case CUSAT_RATE_96_180: return "s2x_b12";
        case CUSAT_RATE_11_20: return "s2x_b4";
        case CUSAT_RATE_100_180: return "s2x_b13";
        case CUSAT_RATE_104_180: return "s2x_b14";
        case CUSAT_RATE_26_45: return "s2x_b5";
        case CUSAT_RATE_18_30: return "s2x_b22";
        case CUSAT_RATE_28_45: return "s2x_b6";
        case CUSAT_RATE_23_36: return "s2x_b7";
        case CUSAT_RATE_116_180: return "s2x_b15";
        case CUSAT_RATE_20_30: return "s2x_b23";
        case CUSAT_RATE_124_180: return "s2x_b16";
        case CUSAT_RATE_25_36: return "s2x_b8";
        case CUSAT_RATE_128_180: return "s2x_b17";
        case CUSAT_RATE_13_18: return "s2x_b9";
        case CUSAT_RATE_132_180: return "s2x_b18";
        case CUSAT_RATE_22_30: return "s2x_b24";
        case CUSAT_RATE_135_180: return "s2x_b19";
        case CUSAT_RATE_140_180: return "s2x_b20";
        case CUSAT_RATE_7_9: return "s2x_b10";
        case CUSAT_RATE_154_180: return "s2x_b21";
        default: return 0;
        }
    } else if (framesize == CUSAT_FECFRAME_SHORT) {
        switch (rate) {
        case CUSAT_RATE_1_4: return "s2_c1";
        case CUSAT_RATE_1_3: return "s2_c2";
        case CUSAT_RATE_2_5: return "s2_c3";
        case CUSAT_RATE_1_2: return "s2_c4";
        case CUSAT_RATE_3_5: return "s2_c5";
        case CUSAT_RATE_2_3: return "s2_c6";
        case CUSAT_RATE_3_4: return "s2_c7";
        case CUSAT_RATE_4_5: return "s2_c8";
        case CUSAT_RATE_5_6: return "s2_c9";
        case CUSAT_RATE_8_9: return "s2_c10";
        case CUSAT_RATE_11_45: return "s2x_c1";
        case CUSAT_RATE_4_15: return "s2x_c2";
        case CUSAT_RATE_14_45: return "s2x_c3";
        case CUSAT_RATE_7_15: return "s2x_c4";
        case CUSAT_RATE_8_15: return "s2x_c5";
        case CUSAT_RATE_26_45: return "s2x_c6";
        case CUSAT_RATE_32_45: return "s2x_c7";
        case CUSAT_RATE_VLSNR_SET1_BPSKS_1_5: return "s2_c1";
        case CUSAT_RATE_VLSNR_SET1_BPSKS_11_45: return "s2x_c1";
        case CUSAT_RATE_VLSNR_SET2_BPSK_1_5: return "s2_c1";
        case CUSAT_RATE_VLSNR_SET2_BPSK_4_15: return "s2x_c2";
        case CUSAT_RATE_VLSNR_SET2_BPSK_1_3: return "s2_c2";
        default: return 0;
        }
    } else if (framesize == CUSAT_FECFRAME_MEDIUM) {
        switch (rate) {
        case CUSAT_RATE_VLSNR_SET1_BPSK_1_5: return "s2x_c8";
        case CUSAT_RATE_VLSNR_SET1_BPSK_11_45: return "s2x_c9";
        case CUSAT_RATE_VLSNR_SET1_BPSK_1_3: return "s2x_c10";
        default: return 0;
        }
    }
    return 0;
}

/* Source records of the generated tables (code_tables.inc). */
typedef struct {
    const char* name;
    int n, k, n_rows, links_total, links_max_cn;
    const uint8_t* row_deg;  /* [n_rows] addresses per 360-bit row */
    const uint16_t* addr;    /* row-major accumulator addresses */
} cusat_table_src;

typedef struct {
    const char* name;  /* table the schedule was built for */
    int q, n_steps;
    const int16_t* pairs; /* [n_steps][2] layer ids, -1 = lane idle */
} cusat_sched_src;

#endif /* CUSAT_DATA_H */
