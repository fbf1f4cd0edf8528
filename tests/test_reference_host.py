"""This project's host-side data against the reference's own host code.

oracle/_ref is compiled from the reference sources where they lie (only in
the build container; skipped where the reference tree is absent).  Compared:
FEC dimensions, BCH generator/encoder, interleaver column offsets,
constellation points (bit-exact), parity-check tables.
"""
import ctypes

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E

ref = O.ref()
pytestmark = pytest.mark.skipif(ref is None, reason="reference tree not present")


def _p(a):
    return a.ctypes.data


ALL_CODES = [(fs, r) for fs in (0, 1, 2) for r in range(E.RATE_COUNT)]


def _ref_params(fs, r):
    out = np.zeros(5, np.uint32)
    rc = ref.ref_fec_params(fs, r, ctypes.c_void_p(_p(out)))
    return None if rc != 0 else [int(v) for v in out]


@pytest.mark.parametrize("fs,r", ALL_CODES)
def test_fec_params_and_tables(fs, r, built_lib):
    rp = _ref_params(fs, r)
    try:
        ci = cs.code_info(fs, r)
    except cs.CusatError:
        ci = None
    if rp is None:
        assert ci is None
        return
    k_bch, n_bch, t, k_ldpc, n_ldpc = rp
    info = np.zeros(5, np.int32)
    deg = np.zeros(256, np.uint8)
    addr = np.zeros(4096, np.uint16)
    total = ref.ref_ldpc_table(fs, r, ctypes.c_void_p(_p(info)), ctypes.c_void_p(_p(deg)),
                               ctypes.c_void_p(_p(addr)), 4096)
    if ci is None:
        # shortened VL-SNR codes (n_bch below the table's K): table keys only in
        # the reference, which never receives them; not built here either
        assert r >= E.rate_index("VLSNR_SET1_QPSK_2_9") and info[1] != n_bch
        return
    assert (ci["k_bch"], ci["n_bch"], ci["t"], ci["k_ldpc"], ci["n_ldpc"]) == (k_bch, n_bch, t, k_ldpc, n_ldpc)
    assert total > 0 and info[0] == n_ldpc and info[1] == k_ldpc
    assert ci["edges"] == info[3] and ci["cnt_max"] + 2 == info[4]
    oi = O.code_info(fs, r)
    assert oi["links_total"] == info[3] and oi["cnl"] == info[4] - 2


@pytest.mark.parametrize("fs,r", [(0, 0), (0, 4), (0, 5), (0, 9), (0, 10), (0, 32), (1, 3), (1, 9), (2, 42)])
def test_bch_generator_and_encoder(fs, r):
    rp = _ref_params(fs, r)
    gen = np.zeros(4, np.uint64)
    p_ref = ref.ref_bch_generator(fs, rp[1], rp[2], ctypes.c_void_p(_p(gen)))
    g, p = O.bch_generator(fs, r)
    assert p == p_ref and (g == gen).all()
    if p % 8:
        return  # medium VL-SNR codes: not byte-aligned, no byte-wise encoder
    rng = np.random.default_rng(r)
    msg = rng.integers(0, 256, rp[0] // 8, dtype=np.uint8)
    cw_ref = np.zeros(rp[1] // 8, np.uint8)
    ref.ref_bch_encode(fs, rp[1], rp[2], ctypes.c_void_p(_p(msg)), ctypes.c_void_p(_p(cw_ref)))
    assert (O.bch_encode(fs, r, msg)[0] == cw_ref).all()


MODS = [(m[1], m[2]) for m in E.MODCODS]


@pytest.mark.parametrize("mod,r", MODS)
@pytest.mark.parametrize("fs", [0, 1])
def test_constellation_and_interleaver_bit_exact(mod, r, fs, built_lib):
    re = np.zeros(256, np.float32)
    im = np.zeros(256, np.float32)
    bits = ref.ref_constellation(mod, r, fs, ctypes.c_void_p(_p(re)), ctypes.c_void_p(_p(im)))
    col = np.zeros(8, np.uint32)
    rows = np.zeros(1, np.uint32)
    ncol = ref.ref_interleaver(mod, r, fs, ctypes.c_void_p(_p(col)), ctypes.c_void_p(_p(rows)))
    mi = cs.modcod_info(mod, r, fs)
    assert mi["n_mod"] == bits
    n = 1 << bits
    assert (mi["points"].real == re[:n]).all() and (mi["points"].imag == im[:n]).all()
    if mod != E.MOD_QPSK:
        assert ncol == bits and (mi["col_offset"] == col).all()


def test_message_update_against_reference():
    for raw in range(-400, 401, 7):
        for old in (-127, -5, 0, 42, 127):
            d = np.zeros(1, np.int32)
            m = ref.ref_bnl_update(raw, old, ctypes.c_void_p(_p(d)))
            assert (m, int(d[0])) == O.bnl_update(raw, old)


@pytest.mark.parametrize("mod,rate,fs", [(E.MOD_QPSK, E.RATE_1_2, 1), (E.MOD_8PSK, E.RATE_3_5, 0),
                                         (E.MOD_16APSK, E.RATE_3_4, 0), (E.MOD_32APSK, E.RATE_3_4, 0),
                                         (E.MOD_64APSK, E.RATE_4_5, 0), (E.MOD_128APSK, E.RATE_135_180, 0),
                                         (E.MOD_256APSK, E.RATE_20_30, 0), (E.MOD_256APSK, E.RATE_116_180, 0)])
def test_dd_snr_matches_reference(mod, rate, fs, built_lib):
    """Decision-directed SNR: product and oracle bit-exact with the
    reference's dd_snr.cc on noisy constellation points, every stride."""
    mi = cs.modcod_info(mod, rate, fs)
    pts = mi["points"]
    rng = np.random.default_rng(mod * 100 + rate)
    for sigma in (0.0, 0.05, 0.3, 1.0):
        lab = rng.integers(0, len(pts), 3000)
        z = pts[lab] + sigma * (rng.standard_normal(3000) + 1j * rng.standard_normal(3000))
        sym = z.astype(np.complex64).view(np.float32)
        for stride in (1, 8):
            want = ref.ref_dd_snr(mod, rate, fs, ctypes.c_void_p(_p(sym)), 3000, stride,
                                  1 if mod == E.MOD_QPSK else 0)
            got = cs.dd_snr(mod, rate, fs, sym, stride=stride)
            orc = O.dd_snr(sym, pts.view(np.float32), stride, qpsk=mod == E.MOD_QPSK)
            assert np.float32(got) == np.float32(want) and np.float32(orc) == np.float32(want), (sigma, stride)
    bad = np.full(20, np.nan, np.float32)
    assert cs.dd_snr(mod, rate, fs, bad) == 0.0 == ref.ref_dd_snr(mod, rate, fs, ctypes.c_void_p(_p(bad)), 10, 1,
                                                                 1 if mod == E.MOD_QPSK else 0)


def test_apsk256_coordinate_tables_regenerate(tmp_path):
    """csrc/gen/apsk256_points.inc is exactly what tables/gen_apsk256.py makes
    from the reference's modulation/apsk256_points.h (its checks included)."""
    import importlib.util
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(root, "oracle", "build.py"))
    build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(build)
    out = tmp_path / "apsk256_points.inc"
    subprocess.run([sys.executable, os.path.join(root, "cusat_gb300", "tables", "gen_apsk256.py"),
                    "--ref", build.REF, "--out", str(out)], check=True, capture_output=True)
    committed = os.path.join(root, "cusat_gb300", "csrc", "gen", "apsk256_points.inc")
    assert out.read_bytes() == open(committed, "rb").read()
