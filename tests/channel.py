"""Seeded AWGN traffic for the tests (numpy; independent of the oracle)."""
import numpy as np

import cusat_gb300 as cs


def es_normalised(sym):
    """Scales symbols to unit average energy (reference
    apps/bench_coded_modulation.cc:287-308)."""
    s = sym.astype(np.float64)
    es = np.mean(s[..., 0::2] ** 2 + s[..., 1::2] ** 2)
    return (sym * np.float32(1.0 / np.sqrt(es))).astype(np.float32)


def awgn(sym, esn0_db, rng):
    """N0 = 1/SNR, sigma = sqrt(N0/2) per component (bench_coded_modulation.cc:373-391)."""
    n0 = np.float32(1.0 / 10 ** (esn0_db / 10.0))
    sigma = np.float32(np.sqrt(n0 / np.float32(2.0)))
    noisy = sym + sigma * rng.standard_normal(sym.shape, dtype=np.float32)
    return noisy.astype(np.float32), float(n0)


def frames(mod, rate, fs, B, esn0_db, seed):
    """Returns (msg bytes, codeword bytes, noisy symbols, N0, llr_gain)."""
    rng = np.random.default_rng(seed)
    ci = cs.code_info(fs, rate)
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    cw = cs.encode_frames(fs, rate, msg)
    sym = es_normalised(cs.map_frames(mod, rate, fs, cw))
    noisy, n0 = awgn(sym, esn0_db, rng)
    gain = min(4.0 / n0, 1000.0)
    return msg, cw, noisy, n0, gain
