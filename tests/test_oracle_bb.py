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


# ---- known answers of the reference's own tests, without the reference tree ----

def crc8_dvbs2(data):
    """CRC-8/DVB-S2: polynomial 0xD5, init 0, no reflection (EN 302 307-1 5.1.6)."""
    reg = 0
    for b in bytes(data):
        reg ^= b
        for _ in range(8):
            reg = ((reg << 1) ^ 0xD5) & 0xFF if reg & 0x80 else (reg << 1) & 0xFF
    return reg


def bbframe(kbch, dfl_bits, ts_gs=0, rng=None, payload=None):
    """A scrambled BBFRAME with the given header fields (MATYPE-1 = TS/GS in
    its top bits, SIS, CCM, RO 0.35; CRC-8 over the first 9 bytes) and random
    or given data field (reference lib/qa_bbframe_parser.cc:27-43)."""
    rng = rng or np.random.default_rng(0)
    f = rng.integers(0, 256, kbch, dtype=np.uint8)
    f[0] = (ts_gs << 6) | (1 << 5) | (1 << 4)
    f[1] = 0
    f[2:4] = 0
    f[4], f[5] = (dfl_bits >> 8) & 0xFF, dfl_bits & 0xFF
    f[6:9] = 0
    f[9] = crc8_dvbs2(f[:9])
    if payload is not None:
        f[10:10 + len(payload)] = payload
    return f ^ O.bb_prbs(kbch)


def test_crc8_and_prbs_known_answers():
    # lib/qa_crc8.cc:13-19, lib/qa_bb_scrambler.cc:40-46
    assert crc8_dvbs2(b"123456789") == 0xBC and crc8_dvbs2(b"") == 0
    assert O.bb_prbs(8)[0] == 0x03
    # figure 5's register, bit-serial: stage 14 xor stage 15 fed back to stage 1
    st = [0] + [int(c) for c in "100101010000000"]
    bits = []
    for _ in range(8 * 64):
        b = st[14] ^ st[15]
        st = [0, b] + st[1:15]
        bits.append(b)
    ref = np.packbits(np.array(bits, np.uint8))
    assert (O.bb_prbs(64) == ref).all()


def header_cases(kbch, rng):
    """(frame, expected data-field bytes) pairs of the reference's parser
    tests (lib/qa_bbframe_parser.cc:47-139): a valid field, the largest legal
    DFL, an empty field, every single-bit header error, DFL one byte too large,
    DFL not a byte multiple, TS/GS other than generic packetized."""
    cases = []
    data = rng.integers(0, 256, 100, dtype=np.uint8)
    cases.append((bbframe(kbch, 800, payload=data, rng=rng), 100))
    cases.append((bbframe(kbch, 8 * kbch - 80, rng=rng), kbch - 10))
    cases.append((bbframe(kbch, 0, rng=rng), 0))
    for bit in range(80):
        f = bbframe(kbch, 800, rng=rng)
        f[bit // 8] ^= 0x80 >> (bit % 8)
        cases.append((f, 0))
    cases.append((bbframe(kbch, 8 * kbch - 80 + 8, rng=rng), 0))
    cases.append((bbframe(kbch, 803, rng=rng), 0))
    for ts in (1, 2, 3):
        cases.append((bbframe(kbch, 800, ts_gs=ts, rng=rng), 0))
    return cases


@pytest.mark.parametrize("fs,rate", [(NORMAL, E.RATE_1_2), (SHORT, E.RATE_1_2)])
def test_parser_rejections_known_answers(fs, rate):
    import cusat_gb300 as cs
    kbch = cs.code_info(fs, rate)["k_bch"] // 8
    cases = header_cases(kbch, np.random.default_rng(2))
    hard = np.stack([c[0] for c in cases])
    want = np.array([c[1] for c in cases])
    ones = np.ones(len(cases), np.int32)
    out, lengths, _ = O.bb_extract(hard, kbch, ones * 5, ones, len(cases) * kbch)
    assert (lengths == want).all()
    # the valid field comes back descrambled, byte for byte
    plain = cases[0][0] ^ O.bb_prbs(kbch)
    assert (out[:100] == plain[10:110]).all()


def test_frame_acceptance_rule():
    # lib/qa_rx_fec_chain.cc:9-17: usable iff LDPC converged and BCH valid
    import cusat_gb300 as cs
    ok = cs.rx_fec_chain.frame_passes_fec_checks
    assert ok(25, True) and ok(0, True)
    assert not ok(-1, True) and not ok(3, False) and not ok(-1, False)
