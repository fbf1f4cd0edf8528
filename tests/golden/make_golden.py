"""Writes tests/golden/reference_host.json: answers of the reference's own
host code (compiled into oracle/_ref from the reference tree by
oracle/build.py), so that the oracle and this project's host code stay pinned
on machines without the reference tree.

    python tests/golden/make_golden.py

Contents: FEC dimensions and BCH generators of every supported (frame size,
rate); BCH codewords of seeded messages; interleaver column offsets and
constellation points (as float32 bit patterns) of every MODCOD; the BB
scrambler PRBS; PLFRAME layouts of all 256 PLS codes and PL scrambling
sequences; the demapper's loudest-bit distance (dmax, which sets the
LLR gain cap) of every MODCOD's reference points; GSE BBFRAMEs built by the reference and its data-field
extraction of them; decision-directed SNR estimates of seeded symbols."""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle_lib as O  # noqa: E402
from cusat_gb300 import enums as E  # noqa: E402


def p(a):
    return ctypes.c_void_p(a.ctypes.data)


# (modulation, rate, frame size, stride, seed) of the SNR-estimate vectors
DD_CASES = [(0, 3, 1, 1, 21), (1, 4, 0, 8, 22), (1, 4, 0, 1, 23), (3, 6, 0, 8, 24), (4, 6, 0, 8, 25),
            (3, 6, 0, 1, 26)]


def dd_symbols(seed, n=2000):
    """Seeded symbols for the SNR vectors: uniform over [-1.3, 1.3)^2, and for
    seed 0 exact QPSK points (zero decision error)."""
    if seed == 0:
        a = np.float32(np.sqrt(0.5))
        s = np.random.default_rng(7).integers(0, 2, 2 * n) * 2 - 1
        return (s * a).astype(np.float32)
    return np.random.default_rng(seed).uniform(-1.3, 1.3, 2 * n).astype(np.float32)


PL_GOLDS = [0, 1, 5, 77777, 262141]
PL_LEN = 33192  # the longest PLFRAME payload (QPSK normal frame with pilots)


def pl_index(seq):
    """Rotation index R (factor e^{-j R pi/2}) from (re, im) factor pairs."""
    re, im = seq[0::2], seq[1::2]
    r = np.full(re.size, 255, np.uint8)
    r[(re == 1) & (im == 0)] = 0
    r[(re == 0) & (im == -1)] = 1
    r[(re == -1) & (im == 0)] = 2
    r[(re == 0) & (im == 1)] = 3
    assert (r != 255).all()
    return r


def main():
    ref = O.ref()
    if ref is None:
        raise SystemExit("the reference tree is needed to generate the fixtures")
    doc = {"codes": [], "bch_words": [], "modcods": [], "bbframes": []}
    for fs in (0, 1):
        for r in range(E.RATE_COUNT):
            out = np.zeros(5, np.uint32)
            if ref.ref_fec_params(fs, r, p(out)) != 0:
                continue
            k_bch, n_bch, t, k_ldpc, n_ldpc = (int(v) for v in out)
            gen = np.zeros(4, np.uint64)
            deg = ref.ref_bch_generator(fs, n_bch, t, p(gen))
            doc["codes"].append({"fs": fs, "rate": r, "k_bch": k_bch, "n_bch": n_bch, "t": t, "k_ldpc": k_ldpc,
                                 "n_ldpc": n_ldpc, "bch_degree": deg, "bch_gen": [str(int(g)) for g in gen]})
    for fs, r in [(0, E.RATE_3_5), (0, E.RATE_1_4), (0, E.RATE_9_10), (1, E.RATE_1_2), (1, E.RATE_8_9)]:
        c = next(c for c in doc["codes"] if (c["fs"], c["rate"]) == (fs, r))
        rng = np.random.default_rng(1000 + 10 * fs + r)
        msg = rng.integers(0, 256, c["k_bch"] // 8, dtype=np.uint8)
        cw = np.zeros(c["n_bch"] // 8, np.uint8)
        ref.ref_bch_encode(fs, c["n_bch"], c["t"], p(msg), p(cw))
        doc["bch_words"].append({"fs": fs, "rate": r, "msg_seed": 1000 + 10 * fs + r, "parity": cw[len(msg):].tobytes().hex()})
    for m in E.MODCODS:
        for fs in (0, 1):
            re = np.zeros(256, np.float32)
            im = np.zeros(256, np.float32)
            bits = ref.ref_constellation(m[1], m[2], fs, p(re), p(im))
            if bits <= 0:
                continue
            col = np.zeros(8, np.uint32)
            rows = np.zeros(1, np.uint32)
            ncol = ref.ref_interleaver(m[1], m[2], fs, p(col), p(rows))
            n = 1 << bits
            # loudest-bit distance of the reference's points (the oracle's
            # restatement of demapper_kernel.cu:216-237, float32 bits)
            kind = 0 if m[1] == E.MOD_QPSK else 1 if m[1] == E.MOD_8PSK else 2
            dmax = np.float32(O.lib().orc_demap_dmax(kind, p(re), p(im), n, bits))
            doc["modcods"].append({"name": m[3], "fs": fs, "bits": bits, "n_cols": int(ncol),
                                   "col": [int(v) for v in col], "re": re[:n].view(np.uint32).tolist(),
                                   "im": im[:n].view(np.uint32).tolist(),
                                   "dmax": int(dmax.view(np.uint32))})
    prbs = np.zeros(7274, np.uint8)
    ref.ref_bb_prbs(p(prbs), 7274)
    doc["prbs_head"] = prbs[:64].tobytes().hex()
    doc["prbs_sha256"] = hashlib.sha256(prbs.tobytes()).hexdigest()
    for fs, r, n, seed in [(0, E.RATE_3_5, 100, 1), (1, E.RATE_1_2, 0, 2), (1, E.RATE_1_2, 869, 3)]:
        c = next(c for c in doc["codes"] if (c["fs"], c["rate"]) == (fs, r))
        kbch = c["k_bch"] // 8
        data = np.random.default_rng(seed).integers(0, 256, n, dtype=np.uint8)
        plain = np.zeros(kbch, np.uint8)
        ref.ref_build_bbframe(fs, r, p(data), n, p(plain))
        outb = np.zeros(kbch, np.uint8)
        got = ref.ref_extract_datafield(p(plain), kbch, p(outb), kbch)
        doc["bbframes"].append({"fs": fs, "rate": r, "payload_seed": seed, "len": n,
                                "header": plain[:10].tobytes().hex(), "extracted": int(got)})
    doc["dd_snr"] = []
    for mod, rate, fs, stride, seed in DD_CASES + [(0, 3, 1, 1, 0)]:
        sym = dd_symbols(seed)
        v = ref.ref_dd_snr(mod, rate, fs, p(sym), len(sym) // 2, stride, 1 if mod == 0 else 0)
        doc["dd_snr"].append({"mod": mod, "rate": rate, "fs": fs, "stride": stride, "seed": seed,
                              "value": int(np.float32(v).view(np.uint32))})
    # PLFRAME layouts of every PLS code and scrambling sequences (rotation
    # index R per symbol, from the reference's descrambling factors)
    doc["pl_layouts"] = []
    for code in range(256):
        out = np.zeros(11, np.int32)
        ref.ref_pl_layout(code, p(out))
        doc["pl_layouts"].append([int(v) for v in out])
    doc["pl_rotation"] = []
    for gold in PL_GOLDS:
        seq = np.zeros(2 * PL_LEN, np.float32)
        assert ref.ref_pl_descrambling(gold, p(seq), PL_LEN) == 0
        r = pl_index(seq)
        doc["pl_rotation"].append({"gold": gold, "len": PL_LEN, "head": "".join(str(int(v)) for v in r[:96]),
                                   "sha256": hashlib.sha256(r.tobytes()).hexdigest()})
    path = os.path.join(HERE, "reference_host.json")
    with open(path, "w") as f:
        json.dump(doc, f, separators=(",", ":"))
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
