"""Frame sizes, code rates, modulations and the MODCOD table.

Numeric values equal the reference's enums
(lib/cusat_dsp/include/cusat_dsp/modcod_types.h:14-95) so that values pass
through the C ABI unchanged.  MODCODS restates the reference's MODCOD table
(lib/cusat_dsp/acm_config.h:53-121): index, modulation, rate, name and the
Es/N0 at which the reference measured post-BCH FER <= 1e-5 with normal
frames, 25 iterations and AWGN.
"""

FECFRAME_NORMAL, FECFRAME_SHORT, FECFRAME_MEDIUM = 0, 1, 2

_RATES = [
    "1_4", "1_3", "2_5", "1_2", "3_5", "2_3", "3_4", "4_5", "5_6", "8_9", "9_10",
    "11_45", "4_15", "13_45", "14_45", "9_20", "7_15", "90_180", "8_15", "96_180", "11_20",
    "100_180", "26_45", "104_180", "18_30", "28_45", "23_36", "116_180", "20_30", "124_180",
    "25_36", "32_45", "128_180", "13_18", "22_30", "132_180", "135_180", "7_9", "140_180",
    "154_180",
    "VLSNR_SET1_QPSK_2_9", "VLSNR_SET1_BPSK_1_5", "VLSNR_SET1_BPSK_11_45", "VLSNR_SET1_BPSK_1_3",
    "VLSNR_SET1_BPSKS_1_5", "VLSNR_SET1_BPSKS_11_45", "VLSNR_SET2_BPSK_1_5", "VLSNR_SET2_BPSK_4_15",
    "VLSNR_SET2_BPSK_1_3",
]
for _i, _r in enumerate(_RATES):
    globals()["RATE_" + _r] = _i
RATE_COUNT = len(_RATES)

MOD_QPSK, MOD_8PSK, MOD_8APSK, MOD_16APSK, MOD_32APSK, MOD_64APSK, MOD_128APSK, MOD_256APSK = range(8)
BITS_PER_SYMBOL = {MOD_QPSK: 2, MOD_8PSK: 3, MOD_8APSK: 3, MOD_16APSK: 4, MOD_32APSK: 5, MOD_64APSK: 6,
                   MOD_128APSK: 7, MOD_256APSK: 8}


def rate_index(name):
    """'3/5' or '3_5' -> code_rate_t value."""
    return _RATES.index(name.replace("/", "_"))


# (modcod_idx, modulation, rate, name, spectral efficiency, min Es/N0 dB)
MODCODS = [
    (1, MOD_QPSK, 0, "qpsk1/4", 0.49, -0.05), (33, MOD_QPSK, 13, "qpsk13/45", 0.57, 0.07),
    (2, MOD_QPSK, 1, "qpsk1/3", 0.66, 0.56), (3, MOD_QPSK, 2, "qpsk2/5", 0.79, 1.00),
    (43, MOD_QPSK, 15, "qpsk9/20", 0.89, 1.42), (4, MOD_QPSK, 3, "qpsk1/2", 0.99, 1.80),
    (44, MOD_QPSK, 20, "qpsk11/20", 1.09, 2.25), (5, MOD_QPSK, 4, "qpsk3/5", 1.19, 2.73),
    (6, MOD_QPSK, 5, "qpsk2/3", 1.32, 3.50), (7, MOD_QPSK, 6, "qpsk3/4", 1.49, 4.43),
    (8, MOD_QPSK, 7, "qpsk4/5", 1.59, 5.08), (9, MOD_QPSK, 8, "qpsk5/6", 1.65, 5.48),
    (10, MOD_QPSK, 9, "qpsk8/9", 1.77, 6.50), (11, MOD_QPSK, 10, "qpsk9/10", 1.79, 6.72),
    (56, MOD_8APSK, 21, "8apsk5/9", 1.65, 4.93), (57, MOD_8APSK, 23, "8apsk26/45", 1.71, 5.33),
    (12, MOD_8PSK, 4, "8psk3/5", 1.78, 5.80), (45, MOD_8PSK, 26, "8psk23/36", 1.90, 7.22),
    (13, MOD_8PSK, 5, "8psk2/3", 1.98, 6.92), (46, MOD_8PSK, 30, "8psk25/36", 2.06, 7.22),
    (47, MOD_8PSK, 33, "8psk13/18", 2.15, 7.69), (14, MOD_8PSK, 6, "8psk3/4", 2.23, 8.11),
    (15, MOD_8PSK, 8, "8psk5/6", 2.48, 9.55), (16, MOD_8PSK, 9, "8psk8/9", 2.65, 10.79),
    (17, MOD_8PSK, 10, "8psk9/10", 2.68, 11.08),
    (58, MOD_16APSK, 17, "16apsk1/2l", 1.97, 6.27), (59, MOD_16APSK, 19, "16apsk8/15l", 2.10, 6.85),
    (60, MOD_16APSK, 21, "16apsk5/9l", 2.19, 7.04), (61, MOD_16APSK, 24, "16apsk3/5l", 2.37, 7.71),
    (62, MOD_16APSK, 28, "16apsk2/3l", 2.64, 8.73),
    (48, MOD_16APSK, 22, "16apsk26/45", 2.28, 7.81), (49, MOD_16APSK, 4, "16apsk3/5", 2.37, 8.10),
    (50, MOD_16APSK, 25, "16apsk28/45", 2.46, 8.30), (51, MOD_16APSK, 26, "16apsk23/36", 2.52, 8.58),
    (18, MOD_16APSK, 5, "16apsk2/3", 2.64, 9.17), (52, MOD_16APSK, 30, "16apsk25/36", 2.75, 9.47),
    (53, MOD_16APSK, 33, "16apsk13/18", 2.86, 9.91), (19, MOD_16APSK, 6, "16apsk3/4", 2.97, 10.41),
    (54, MOD_16APSK, 38, "16apsk7/9", 3.08, 10.85), (20, MOD_16APSK, 7, "16apsk4/5", 3.17, 11.13),
    (21, MOD_16APSK, 8, "16apsk5/6", 3.30, 11.71), (55, MOD_16APSK, 39, "16apsk77/90", 3.39, 12.19),
    (22, MOD_16APSK, 9, "16apsk8/9", 3.52, 12.99), (23, MOD_16APSK, 10, "16apsk9/10", 3.57, 13.23),
    (63, MOD_32APSK, 5, "32apsk2/3l", 3.29, 11.30), (64, MOD_32APSK, 32, "32apsk32/45", 3.51, 12.05),
    (65, MOD_32APSK, 35, "32apsk11/15", 3.62, 12.47), (24, MOD_32APSK, 6, "32apsk3/4", 3.70, 12.93),
    (66, MOD_32APSK, 38, "32apsk7/9", 3.84, 13.35), (25, MOD_32APSK, 7, "32apsk4/5", 3.95, 13.84),
    (26, MOD_32APSK, 8, "32apsk5/6", 4.12, 14.48), (27, MOD_32APSK, 9, "32apsk8/9", 4.40, 15.79),
    (28, MOD_32APSK, 10, "32apsk9/10", 4.47, 16.05),
    (29, MOD_64APSK, 35, "64apsk11/15", 4.40, 15.00), (30, MOD_64APSK, 37, "64apsk7/9", 4.67, 15.60),
    (31, MOD_64APSK, 7, "64apsk4/5", 4.80, 16.10), (35, MOD_64APSK, 8, "64apsk5/6", 4.98, 17.23),
    (36, MOD_64APSK, 32, "64apsk32/45", 4.27, 14.18),
    (32, MOD_128APSK, 36, "128apsk3/4", 5.25, 18.00), (34, MOD_128APSK, 38, "128apsk7/9", 5.44, 18.89),
    (37, MOD_256APSK, 36, "256apsk3/4", 6.00, 23.34), (38, MOD_256APSK, 32, "256apsk32/45", 5.69, 22.40),
    (39, MOD_256APSK, 27, "256apsk29/45", 5.16, 20.20), (40, MOD_256APSK, 29, "256apsk31/45", 5.51, 21.50),
    (41, MOD_256APSK, 28, "256apsk2/3", 5.06, 18.10), (42, MOD_256APSK, 34, "256apsk11/15", 5.50, 19.80),
]


def find_modcod(name):
    for m in MODCODS:
        if m[3] == name:
            return m
    raise KeyError(name)


def modcod_by_index(idx):
    """The MODCOD table row of a modcod_idx (acm_config.h find_modcod)."""
    for m in MODCODS:
        if m[0] == idx:
            return m
    raise KeyError(idx)
