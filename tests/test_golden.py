"""The oracle and this project's host code against golden answers of the
reference's own host code (tests/golden/reference_host.json, written by
tests/golden/make_golden.py from the reference compiled into oracle/_ref).
Runs without the reference tree."""
import hashlib
import json
import os

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_host.json")))


def test_fec_dimensions_and_bch_generators(built_lib):
    assert len(GOLD["codes"]) >= 50
    built = 0
    for c in GOLD["codes"]:
        g, deg = O.bch_generator(c["fs"], c["rate"])
        try:
            ci = cs.code_info(c["fs"], c["rate"])
        except cs.CusatError:
            # shortened VL-SNR codes: table keys only in the reference, not built
            assert deg < 0 and c["rate"] >= E.rate_index("VLSNR_SET1_QPSK_2_9")
            continue
        built += 1
        assert deg == c["bch_degree"] and [str(int(v)) for v in g] == c["bch_gen"]
        assert (ci["k_bch"], ci["n_bch"], ci["t"], ci["k_ldpc"], ci["n_ldpc"]) == \
            (c["k_bch"], c["n_bch"], c["t"], c["k_ldpc"], c["n_ldpc"])
    assert built >= 50


def test_bch_codewords(built_lib):
    for w in GOLD["bch_words"]:
        ci = cs.code_info(w["fs"], w["rate"])
        msg = np.random.default_rng(w["msg_seed"]).integers(0, 256, ci["k_bch"] // 8, dtype=np.uint8)
        cw = O.bch_encode(w["fs"], w["rate"], msg)[0]
        assert cw[len(msg):].tobytes().hex() == w["parity"]
        full = cs.encode_frames(w["fs"], w["rate"], msg[None])[0]      # product encoder: BCH part
        assert full[:ci["n_bch"] // 8].tobytes() == cw.tobytes()


def test_constellations_and_interleavers(built_lib):
    assert len(GOLD["modcods"]) >= 80
    for m in GOLD["modcods"]:
        _, mod, rate, _, _, _ = E.find_modcod(m["name"])
        mi = cs.modcod_info(mod, rate, m["fs"])
        assert mi["n_mod"] == m["bits"]
        pts = mi["points"]
        assert pts.real.astype(np.float32).view(np.uint32).tolist() == m["re"]
        assert pts.imag.astype(np.float32).view(np.uint32).tolist() == m["im"]
        if mod != E.MOD_QPSK:
            assert mi["col_offset"].tolist() == m["col"]


def test_llr_gain_cap_every_modcod(built_lib):
    """The demapper's gain cap min(g, 2 * 320 / dmax) (reference
    demapper_kernel.cu:216-239, 283-291): the oracle's dmax of the
    reference's points equals the recorded one, and the product's cap equals
    the oracle's for every MODCOD and frame size, bit for bit, over a range
    of requested gains."""
    for m in GOLD["modcods"]:
        _, mod, rate, _, _, _ = E.find_modcod(m["name"])
        mi = O.modcod(mod, rate, m["fs"])
        assert np.float32(mi["dmax"]).view(np.uint32) == m["dmax"], m["name"]
        for g in (1e9, 1000.0, 160.5, 15.92, 4.0, 0.5, 0.0):
            want = O.capped_llr_gain(mi, g)
            got = cs.capped_llr_gain(mod, rate, m["fs"], g)
            assert np.float32(got).view(np.uint32) == np.float32(want).view(np.uint32), (m["name"], g, got, want)
        if mod == E.MOD_8PSK:
            assert O.capped_llr_gain(mi, 1e9) == 160.0  # 2 * 320 / 4


def test_llr_target_knob(built_lib, monkeypatch):
    """CUSAT_DEMAP_LLR_TARGET moves the cap as in the reference
    (demapper_kernel.cu:238-239; <= 0 disables it)."""
    mod, rate = E.MOD_16APSK, E.RATE_3_4
    for tgt in ("100", "0"):
        monkeypatch.setenv("CUSAT_DEMAP_LLR_TARGET", tgt)
        mi = O.modcod(mod, rate, 0, llr_target=float(tgt))
        want = O.capped_llr_gain(mi, 1e9)
        assert cs.capped_llr_gain(mod, rate, 0, 1e9) == want
    monkeypatch.delenv("CUSAT_DEMAP_LLR_TARGET")
    assert cs.capped_llr_gain(mod, rate, 0, 1e9) == O.capped_llr_gain(O.modcod(mod, rate, 0), 1e9)


def test_bb_scrambler_and_bbframes():
    prbs = O.bb_prbs(7274)
    assert prbs[:64].tobytes().hex() == GOLD["prbs_head"]
    assert hashlib.sha256(prbs.tobytes()).hexdigest() == GOLD["prbs_sha256"]
    for b in GOLD["bbframes"]:
        kbch = cs.code_info(b["fs"], b["rate"])["k_bch"] // 8
        data = np.random.default_rng(b["payload_seed"]).integers(0, 256, b["len"], dtype=np.uint8)
        scr = O.bb_build(data, kbch)
        plain = scr ^ prbs[:kbch]
        assert plain[:10].tobytes().hex() == b["header"]
        out, lengths, _ = O.bb_extract(scr[None], kbch, [3], [1], kbch)
        assert lengths[0] == b["extracted"] == len(data) and (out == data).all()


def _dd_symbols(seed, n=2000):
    # same draw as tests/golden/make_golden.py:dd_symbols
    if seed == 0:
        a = np.float32(np.sqrt(0.5))
        s = np.random.default_rng(7).integers(0, 2, 2 * n) * 2 - 1
        return (s * a).astype(np.float32)
    return np.random.default_rng(seed).uniform(-1.3, 1.3, 2 * n).astype(np.float32)


def test_dd_snr_estimates(built_lib):
    """The RX chain's decision-directed SNR (product and oracle) bit-exact
    with the reference's qpsk_snr_dd / constellation_snr_dd."""
    assert len(GOLD["dd_snr"]) >= 7
    for c in GOLD["dd_snr"]:
        sym = _dd_symbols(c["seed"])
        want = np.uint32(c["value"]).view(np.float32)
        got = cs.dd_snr(c["mod"], c["rate"], c["fs"], sym, stride=c["stride"])
        pts = cs.modcod_info(c["mod"], c["rate"], c["fs"])["points"].view(np.float32)
        orc = O.dd_snr(sym, pts, c["stride"], qpsk=c["mod"] == E.MOD_QPSK)
        assert np.float32(got).view(np.uint32) == c["value"], (c, got, want)
        assert np.float32(orc).view(np.uint32) == c["value"], (c, orc, want)
