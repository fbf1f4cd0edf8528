"""The oracle's post-FEC baseband stage against the reference's own host code
(bb_scrambler.cc, bbframe_parser.cc, bb_header.cc compiled into oracle/_ref):
the PRBS, the BBFRAME builder, and frame-by-frame data-field extraction on
valid, corrupted and foreign frames."""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from cusat_gb300 import enums as E

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT


def _ref():
    r = O.ref()
    if r is None:
        pytest.skip("reference tree not available")
    return r


def test_prbs_matches_reference():
    r = _ref()
    ref = np.zeros(7274, np.uint8)
    assert r.ref_bb_prbs(ref.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), 7274) == 0
    assert (O.bb_prbs(7274) == ref).all()


@pytest.mark.parametrize("fs,rate", [(NORMAL, E.RATE_3_5), (SHORT, E.RATE_1_2), (NORMAL, E.RATE_9_10)])
def test_builder_and_extraction_match_reference(fs, rate):
    r = _ref()
    import cusat_gb300 as cs
    kbch = cs.code_info(fs, rate)["k_bch"] // 8
    rng = np.random.default_rng(rate)
    u8 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    frames, lens = [], []
    for k in range(12):
        n = [0, 1, kbch - 10, int(rng.integers(1, kbch - 10))][k % 4]
        data = rng.integers(0, 256, n, dtype=np.uint8)
        plain = np.zeros(kbch, np.uint8)
        assert r.ref_build_bbframe(fs, rate, u8(data), n, u8(plain)) == n
        scr = np.zeros(kbch, np.uint8)
        assert r.ref_bb_scramble(u8(plain), u8(scr), kbch) == 0
        assert (O.bb_build(data, kbch) == scr).all()
        frames.append(scr)
        lens.append(n)
    hard = np.stack(frames)
    hard[5, 3] ^= 0x10                      # header corrupted: CRC fails
    hard[6] = O.bb_build(rng.integers(0, 256, 40, dtype=np.uint8), kbch, ts_gs=3)  # not generic packetized
    trials = np.full(len(frames), 5, np.int32)
    valid = np.ones(len(frames), np.int32)
    trials[7] = -1                          # LDPC failure
    valid[8] = 0                            # BCH failure
    out, lengths, offsets = O.bb_extract(hard, kbch, trials, valid, 10**6)
    for f in range(len(frames)):
        plain = np.zeros(kbch, np.uint8)
        assert r.ref_bb_scramble(u8(np.ascontiguousarray(hard[f])), u8(plain), kbch) == 0
        buf = np.zeros(kbch, np.uint8)
        n = r.ref_extract_datafield(u8(plain), kbch, u8(buf), kbch) if trials[f] >= 0 and valid[f] else 0
        assert lengths[f] == n, f
        assert (out[offsets[f]:offsets[f] + n] == buf[:n]).all()
    assert lengths[5] == lengths[6] == lengths[7] == lengths[8] == 0
    # output room: a frame that does not fit the room left yields nothing,
    # later smaller ones still go in (the chain's per-frame rule)
    room = int(lengths[0] + lengths[1] + lengths[3] // 2)
    _, l2, o2 = O.bb_extract(hard, kbch, trials, valid, room)
    used = 0
    for f in range(len(frames)):
        expect = lengths[f] if lengths[f] <= room - used else 0
        assert l2[f] == expect and o2[f] == used
        used += expect
