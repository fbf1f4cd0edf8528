"""Seeded synthetic DVB-S2/S2X traffic for benchmarks, training and serving.

Frames are built with this package's own BCH + LDPC encoder and mapper
(cusat_gen_encode / cusat_gen_map) and an AWGN channel: unit average symbol
energy, N0 = 1/SNR, sigma = sqrt(N0/2) per component, LLR gain
min(4/N0, 1000) -- the conventions of the reference's
apps/bench_coded_modulation.cc:287-308,373-391.
"""
import numpy as np

from . import code_info, encode_frames, map_frames, modcod_info
from .enums import FECFRAME_NORMAL, FECFRAME_SHORT, find_modcod

# The ten MODCODs of the mixed-batch workload.  "S2X 64APSK 2/3" is not a
# MODCOD of the reference's table; 64APSK 32/45 (the nearest rate) stands in.
MIXED_MODCODS = ["qpsk1/4", "qpsk1/2", "qpsk3/4", "8psk3/5", "8psk9/10", "16apsk2/3", "16apsk5/6",
                 "32apsk3/4", "32apsk9/10", "64apsk32/45"]
# Short FECFRAMEs exist only for these (DVB-S2 base MODCODs with short codes).
SHORT_CAPABLE = ["qpsk1/4", "qpsk1/2", "qpsk3/4", "8psk3/5", "16apsk2/3", "16apsk5/6", "32apsk3/4"]


def unit_energy(sym):
    s = sym.astype(np.float64)
    es = np.mean(s[..., 0::2] ** 2 + s[..., 1::2] ** 2)
    return (sym * np.float32(1.0 / np.sqrt(es))).astype(np.float32)


def awgn(sym, esn0_db, rng):
    n0 = np.float32(1.0 / 10 ** (esn0_db / 10.0))
    sigma = np.float32(np.sqrt(n0 / np.float32(2.0)))
    return (sym + sigma * rng.standard_normal(sym.shape, dtype=np.float32)).astype(np.float32), float(n0)


class _PackageGen:
    """Encoder and mapper of this package (the default generator)."""

    @staticmethod
    def code_info(fs, rate):
        return code_info(fs, rate)

    @staticmethod
    def encode(fs, rate, msg):
        return encode_frames(fs, rate, msg)

    @staticmethod
    def map(mod, rate, fs, cw):
        return map_frames(mod, rate, fs, cw)

    @staticmethod
    def modcod_info(mod, rate, fs):
        return modcod_info(mod, rate, fs)


def modcod_frames(name, fs, n, esn0_db, rng, gen=None):
    """n frames of one MODCOD: (messages, symbols [n, 2 xfec], N0, gain).
    gen: an object with code_info/encode/map (default: this package's)."""
    gen = gen or _PackageGen
    _, mod, rate, _, _, _ = find_modcod(name)
    ci = gen.code_info(fs, rate)
    msg = rng.integers(0, 256, (n, ci["k_bch"] // 8), dtype=np.uint8)
    sym = unit_energy(gen.map(mod, rate, fs, gen.encode(fs, rate, msg)))
    noisy, n0 = awgn(sym, esn0_db, rng)
    return msg, noisy, n0, min(4.0 / n0, 1000.0)


def mixed_traffic(n_frames, seed, modcods=MIXED_MODCODS, short_share=0.3, margin_db=0.5, gen=None):
    """Frames drawn uniformly over `modcods`, a share of them short (drawn
    among the short-capable ones), each at its threshold + margin (the
    reference's normal-frame thresholds, acm_config.h:54-115, also used for
    short frames).  Returns (table, frames): table lists the distinct
    (name, modulation, rate, frame size); frames is a list of dicts with the
    table index, symbols, N0, gain and message."""
    rng = np.random.default_rng(seed)
    short_ok = [m for m in modcods if m in SHORT_CAPABLE]
    picks = []
    for _ in range(n_frames):
        if short_ok and rng.random() < short_share:
            picks.append((short_ok[rng.integers(len(short_ok))], FECFRAME_SHORT))
        else:
            picks.append((modcods[rng.integers(len(modcods))], FECFRAME_NORMAL))
    table = sorted(set(picks), key=lambda x: (modcods.index(x[0]), x[1]))
    index = {t: i for i, t in enumerate(table)}
    frames = [None] * n_frames
    for key in table:
        ids = [i for i, p in enumerate(picks) if p == key]
        thr = find_modcod(key[0])[5]
        msg, noisy, n0, gain = modcod_frames(key[0], key[1], len(ids), thr + margin_db, rng, gen)
        for k, i in enumerate(ids):
            frames[i] = {"modcod": index[key], "sym": noisy[k], "n0": n0, "gain": gain, "msg": msg[k]}
    out = [(name, find_modcod(name)[1], find_modcod(name)[2], fs) for name, fs in table]
    return out, frames


def geometry(table, gen=None):
    """Per table entry: xfecframe_len, k_ldpc, k_bch."""
    gen = gen or _PackageGen
    geo = []
    for _, mod, rate, fs in table:
        mi = gen.modcod_info(mod, rate, fs)
        ci = gen.code_info(fs, rate)
        geo.append((mi["xfecframe_len"], ci["k_ldpc"], ci["k_bch"]))
    return geo
