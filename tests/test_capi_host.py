"""C ABI without a GPU: the library loads, exports every declared entry point,
rejects bad arguments, and its host-side encoders/mapper agree with the
oracle's independent restatements."""
import os
import re

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import _capi
from cusat_gb300 import enums as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    hdr = open(os.path.join(ROOT, "include", "cusat_fec.h")).read()
    return sorted(set(re.findall(r"\b(cusat_\w+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = _capi.lib()
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_capi.exported_symbols())


def test_no_device_is_a_loud_error(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cs.CusatError) as e:
        cs.ldpc_decode_cuda(E.FECFRAME_SHORT, E.RATE_1_2, 50, 4)
    assert e.value.code == -4
    # every object that needs the GPU refuses the same way
    from cusat_gb300 import learned
    makers = [lambda: cs.rx_fec(E.MOD_QPSK, E.RATE_1_2, E.FECFRAME_SHORT, 20, 4),
              lambda: cs.demapper_cuda(E.MOD_8PSK, E.RATE_3_5, E.FECFRAME_NORMAL, 4),
              lambda: cs.bch_check_cuda.for_code(E.FECFRAME_NORMAL, E.RATE_3_5),
              lambda: cs.batch([(E.MOD_QPSK, E.RATE_1_2, E.FECFRAME_SHORT)], 20, 8),
              lambda: cs.server([(E.MOD_QPSK, E.RATE_1_2, E.FECFRAME_SHORT)], 20, 64 << 20, 1, 8),
              lambda: learned.nms_trainer(E.FECFRAME_SHORT, E.RATE_1_2, 5, 4),
              lambda: cs.rx_fec_chain(E.FECFRAME_SHORT, E.RATE_1_2, E.MOD_QPSK, 20, 64, 2, 4),
              lambda: cs.rx_fec_pool(E.FECFRAME_SHORT, [4, 12], 20, 64, 2, 4),
              lambda: cs.gpu_decode_budget.make_default(),
              lambda: cs.bb_extractor(E.FECFRAME_SHORT, E.RATE_1_2)]
    for make in makers:
        with pytest.raises(cs.CusatError) as e:
            make()
        assert e.value.code == -4


def test_invalid_arguments(built_lib):
    with pytest.raises(cs.CusatError):
        cs.code_info(E.FECFRAME_SHORT, E.RATE_9_10)  # no short 9/10 code
    with pytest.raises(cs.CusatError):
        cs.code_info(7, 0)
    with pytest.raises(cs.CusatError):
        cs.modcod_info(8, E.RATE_135_180, E.FECFRAME_NORMAL)


@pytest.mark.parametrize("fs,r", [(0, 4), (0, 0), (0, 10), (0, 32), (1, 3), (1, 8), (0, 5)])
def test_product_encoder_matches_oracle(fs, r, built_lib):
    ci = cs.code_info(fs, r)
    rng = np.random.default_rng(fs * 100 + r)
    msg = rng.integers(0, 256, (3, ci["k_bch"] // 8), dtype=np.uint8)
    cw = cs.encode_frames(fs, r, msg)
    ref_cw = O.ldpc_encode(fs, r, O.bch_encode(fs, r, msg))
    assert (cw == ref_cw).all()
    llr = np.where(np.unpackbits(cw, axis=1) == 1, -9, 9).astype(np.int16)
    assert all(O.syndrome_ok(fs, r, l) for l in llr)


@pytest.mark.parametrize("name", ["qpsk1/2", "8psk3/5", "16apsk2/3", "32apsk3/4", "64apsk32/45", "8apsk5/9",
                                  "128apsk3/4", "256apsk3/4", "256apsk2/3"])
def test_product_mapper_matches_oracle(name, built_lib):
    _, mod, r, *_ = E.find_modcod(name)
    fs = 0
    ci = cs.code_info(fs, r)
    mi = cs.modcod_info(mod, r, fs)
    rng = np.random.default_rng(5)
    cw = cs.encode_frames(fs, r, rng.integers(0, 256, (2, ci["k_bch"] // 8), dtype=np.uint8))
    sym = cs.map_frames(mod, r, fs, cw)
    col = mi["col_offset"] if mod != E.MOD_QPSK else np.array([0, 1, 0, 0, 0, 0, 0, 0], np.uint32)
    stride = 2 if mod == E.MOD_QPSK else 1
    ref_sym = O.map_symbols(cw, mi["xfecframe_len"], mi["n_mod"], col, stride, mi["points"],
                            mi["interleaved_len"], mi["fecframe_len"])
    assert (sym == ref_sym).all()
    if mod == E.MOD_128APSK:
        # 6 stuffing bits, 12 padding symbols on the all-ones label (mapper.cc:28-62)
        assert mi["interleaved_len"] == 9258 and mi["xfecframe_len"] == 9270
        pad = sym[:, 2 * 9258:].reshape(2, 12, 2)
        assert (pad[..., 0] == mi["points"][127].real).all() and (pad[..., 1] == mi["points"][127].imag).all()


def test_interleaver_known_answers(built_lib):
    # lib/qa_bit_interleaver.cc:23-66
    def order(mod, r, fs=0):
        mi = cs.modcod_info(mod, r, fs)
        rows = mi["fecframe_len"] // mi["n_mod"]
        return [int(c) // rows for c in mi["col_offset"][:mi["n_mod"]]], rows
    assert cs.modcod_info(E.MOD_QPSK, E.RATE_1_2, 0)["col_offset"].sum() == 0
    o, rows = order(E.MOD_8PSK, E.RATE_2_3)
    assert rows == 64800 // 3 and o == [0, 1, 2]
    assert order(E.MOD_8PSK, E.RATE_3_5)[0] == [2, 1, 0]
    assert order(E.MOD_32APSK, E.RATE_3_4, 1)[1] == 16200 // 5
    assert order(E.MOD_32APSK, E.RATE_2_3)[0] == [2, 1, 4, 3, 0]
    assert order(E.MOD_64APSK, E.RATE_4_5)[0] == [1, 2, 4, 0, 5, 3]
    for m in E.MODCODS:
        if m[1] == E.MOD_QPSK:
            continue
        o, _ = order(m[1], m[2])
        assert sorted(o) == list(range(len(o))), m[3]


def test_constellation_known_answers(built_lib):
    # lib/qa_constellation.cc:18-140
    a = np.float32(np.sqrt(0.5))
    q = cs.modcod_info(E.MOD_QPSK, E.RATE_1_2, 0)["points"]
    assert list(q) == [complex(a, a), complex(a, -a), complex(-a, a), complex(-a, -a)]
    p8 = cs.modcod_info(E.MOD_8PSK, E.RATE_3_5, 0)["points"]
    phase = [1, 0, 4, -3, 2, -1, 3, -2]
    assert np.max(np.abs(p8 - np.exp(1j * np.array(phase) * np.pi / 4))) < 1e-6
    for m in E.MODCODS:
        pts = cs.modcod_info(m[1], m[2], 0)["points"].astype(np.complex128)
        assert abs(np.mean(np.abs(pts) ** 2) - 1.0) < 1e-3, m[3]
        assert len({(round(z.real * 1e5), round(z.imag * 1e5)) for z in pts}) == len(pts)
    def rings(mod, r):
        return len({round(abs(z) * 1e4) for z in cs.modcod_info(mod, r, 0)["points"].astype(np.complex128)})
    assert rings(E.MOD_16APSK, E.RATE_3_4) == 2 and rings(E.MOD_16APSK, E.RATE_90_180) == 2
    assert rings(E.MOD_32APSK, E.RATE_3_4) == 3 and rings(E.MOD_32APSK, E.RATE_128_180) == 4
    assert rings(E.MOD_64APSK, E.RATE_132_180) == 4
    assert rings(E.MOD_128APSK, E.RATE_135_180) == 6 and rings(E.MOD_256APSK, E.RATE_135_180) == 8
    c = cs.modcod_info(E.MOD_16APSK, E.RATE_3_4, 0)["points"]
    assert abs(abs(c[0]) / abs(c[12]) - 2.85) < 1e-5
    for r, g1, g2 in [(6, 2.84, 5.27), (7, 2.72, 4.87), (8, 2.64, 4.64), (9, 2.54, 4.33), (10, 2.53, 4.30)]:
        c = cs.modcod_info(E.MOD_32APSK, r, 0)["points"].astype(np.complex128)
        r1, r2, r3 = abs(c[17]), abs(c[0]), abs(c[8])
        assert abs(r2 / r1 - g1) < 1e-6 * g1 * 10 and abs(r3 / r1 - g2) < 1e-6 * g2 * 10


def test_slot_buckets_waste_at_most_one_half(built_lib):
    """Every code's kernel class (circulant-slot bucket) holds its largest
    layer, and its check rows of cmax + 2 slots take as many packed edge
    pairs as the real edges need: at most one half of a pair is an absent
    slot or the pad."""
    import cusat_gb300 as cs
    from cusat_gb300 import enums as E
    n = 0
    for fs in (E.FECFRAME_NORMAL, E.FECFRAME_SHORT, E.FECFRAME_MEDIUM):
        for r in range(E.RATE_COUNT):
            try:
                ci = cs.code_info(fs, r)
            except Exception:
                continue
            n += 1
            assert ci["cmax"] >= ci["cnt_max"], (fs, r)
            assert (ci["cmax"] + 3) // 2 == (ci["cnt_max"] + 3) // 2, (fs, r, ci["cmax"], ci["cnt_max"])
    assert n >= 56
