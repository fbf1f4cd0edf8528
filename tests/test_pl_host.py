"""The PL receiver tail's host side against the reference (no GPU): PLFRAME
layouts of every PLS code, the PL scrambling sequence, and the oracle's
slot descrambling/de-rotation -- against golden answers of the reference's
framing/plframe.cc and framing/pl_scrambler.cc (tests/golden/reference_host.json),
and, where the reference tree is present, against its code compiled into
oracle/_ref (including plrx/pl_receiver.cc's rotate_slot)."""
import ctypes
import hashlib

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O

GOLD = O.golden()
KEYS = cs._PL_KEYS if hasattr(cs, "_PL_KEYS") else None


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def test_layout_of_every_pls_code(built_lib):
    assert len(GOLD["pl_layouts"]) == 256
    for code, want in enumerate(GOLD["pl_layouts"]):
        got = cs.pl_layout(code)
        assert [got[k] for k in cs._PL_KEYS] == want, (code, got, want)
    # the headline frame: 8PSK 3/5 normal with pilots, 240 slots, 14 pilot blocks
    l = cs.pl_layout((12 << 2) | 1)
    assert (l["slots"], l["pilot_blocks"], l["payload_symbols"], l["deliverable"]) == (240, 14, 22104, 1)


def test_scrambling_sequence(built_lib):
    for g in GOLD["pl_rotation"]:
        r = cs.pl_rotation_index(g["gold"], g["len"])
        assert "".join(str(int(v)) for v in r[:96]) == g["head"]
        assert hashlib.sha256(r.tobytes()).hexdigest() == g["sha256"], g["gold"]
        ro = np.zeros(g["len"], np.uint8)
        assert O.lib().orc_pl_rotation(g["gold"], _p(ro), g["len"]) == 0
        assert (ro == r).all()
    with pytest.raises(cs.CusatError):
        cs.pl_rotation_index(262142, 4)  # 2^18 - 2 codes: 0 .. 262141


def test_against_reference_tree(built_lib):
    ref = O.ref()
    if ref is None:
        pytest.skip("reference tree absent")
    rng = np.random.default_rng(9)
    for gold in rng.integers(0, 262142, 6):
        n = 4000
        seq = np.zeros(2 * n, np.float32)
        assert ref.ref_pl_descrambling(int(gold), _p(seq), n) == 0
        r = cs.pl_rotation_index(int(gold), n)
        assert (np.array([1, 0, -1, 0], np.float32)[r] == seq[0::2]).all()
        assert (np.array([0, -1, 0, 1], np.float32)[r] == seq[1::2]).all()
    # the oracle's slot descrambling + de-rotation equals the reference's
    # rotate_slot bit for bit, including gains, tiny and large steps and
    # non-finite inputs
    for trial in range(40):
        pay = rng.standard_normal(180).astype(np.float32) * np.float32(rng.uniform(0.1, 10))
        if trial % 10 == 3:
            pay[7] = np.inf
            pay[50] = np.nan
        r = rng.integers(0, 4, 90).astype(np.uint8)
        ang, stp, g = rng.uniform(-3.2, 3.2), rng.uniform(-0.05, 0.05) * (trial % 3), rng.uniform(0.3, 3)
        rot = np.array([g * np.cos(ang), g * np.sin(ang), np.cos(stp), np.sin(stp)], np.float32)
        out = np.zeros(180, np.float32)
        assert O.lib().orc_pl_extract(_p(pay), 1, 0, _p(r), _p(rot), _p(out)) == 0
        d = np.zeros(180, np.float32)
        d[0::2] = np.array([1, 0, -1, 0], np.float32)[r]
        d[1::2] = np.array([0, -1, 0, 1], np.float32)[r]
        want = np.zeros(180, np.float32)
        ref.ref_rotate_slot(_p(pay), _p(d), ctypes.c_float(rot[0]), ctypes.c_float(rot[1]), ctypes.c_float(rot[2]),
                            ctypes.c_float(rot[3]), _p(want))
        assert (out.view(np.uint32) == want.view(np.uint32)).all(), trial


def test_pilot_removal_layout():
    """Slot s of the payload starts at 90 s + 36 min(s / 16, blocks): the
    oracle extracts exactly the data symbols around the pilot blocks."""
    slots, blocks = 240, 14
    payload_len = 90 * slots + 36 * blocks
    pay = np.zeros((payload_len, 2), np.float32)
    pay[:, 0] = np.arange(payload_len)  # symbol index in the real part
    r = np.zeros(payload_len, np.uint8)  # no scrambling
    out = np.zeros((90 * slots, 2), np.float32)
    assert O.lib().orc_pl_extract(_p(pay), slots, 1, _p(r), None, _p(out)) == 0
    idx = out[:, 0].astype(np.int64)
    is_pilot = np.zeros(payload_len, bool)
    for b in range(blocks):
        is_pilot[90 * 16 * (b + 1) + 36 * b: 90 * 16 * (b + 1) + 36 * (b + 1)] = True
    assert (idx == np.nonzero(~is_pilot)[0]).all()
