"""CUDA kernels against the CPU oracle (bit-exact), through the C ABI.

Decoder: hard decisions and iteration counts identical to the oracle on the
same int16 LLRs; demapper: identical int16 LLRs; BCH: identical flags and
remainders.  The oracle side takes its demap parameters (points,
interleaver columns, gain cap) from its own restatement and the reference's
recorded host answers, never from the product.  The benchmark workloads at
their full sizes, and CTAs that decode several frames in turn, are checked
in test_gpu_bench_parity.py.
"""
import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from channel import frames
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT


def oracle_llr(mod, rate, fs, noisy, n0, gain):
    return O.demap_modcod(noisy, O.modcod(mod, rate, fs), n0, gain)


def gpu_decode(torch, fs, rate, llr, T, max_batch=None):
    B = llr.shape[0]
    dec = cs.ldpc_decode_cuda(fs, rate, T, max_batch or B)
    d_llr = torch.from_numpy(np.ascontiguousarray(llr)).cuda()
    hard = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), hard, trials)
    torch.cuda.synchronize()
    return hard.cpu().numpy(), trials.cpu().numpy()


def assert_same(h1, t1, h2, t2):
    bad = np.nonzero((t1 != t2) | (h1 != h2).any(axis=1))[0]
    assert len(bad) == 0, f"frames {bad[:8]} differ: trials gpu {t1[bad[:8]]} oracle {t2[bad[:8]]}"


def test_c1_short_half_qpsk(cuda):
    # short 1/2 (s2_c4), QPSK, Es/N0 1.5 dB, 64 frames, 50 iterations
    mod, rate = E.MOD_QPSK, E.RATE_1_2
    msg, cw, noisy, n0, gain = frames(mod, rate, SHORT, 64, 1.5, seed=11)
    llr = oracle_llr(mod, rate, SHORT, noisy, n0, gain)
    hg, tg = gpu_decode(cuda, SHORT, rate, llr, 50)
    ho, to = O.ldpc_decode(SHORT, rate, llr, 50)
    assert_same(hg, tg, ho, to)
    assert (to >= 0).sum() > 32  # the workload actually decodes


def test_c2_normal_35_8psk(cuda):
    # normal 3/5 (s2_b5), 8PSK, Es/N0 6.0 dB, 50 iterations (32 of the 256 frames)
    mod, rate = E.MOD_8PSK, E.RATE_3_5
    msg, cw, noisy, n0, gain = frames(mod, rate, NORMAL, 32, 6.0, seed=12)
    llr = oracle_llr(mod, rate, NORMAL, noisy, n0, gain)
    hg, tg = gpu_decode(cuda, NORMAL, rate, llr, 50)
    ho, to = O.ldpc_decode(NORMAL, rate, llr, 50, nthreads=16)
    assert_same(hg, tg, ho, to)
    assert (to > 0).sum() > 16


QPSK_SNR = {0: -2.0, 1: -1.0, 2: -0.2, 3: 0.9, 4: 1.9, 5: 2.8, 6: 3.7, 7: 4.4, 8: 4.9, 9: 6.0, 10: 6.3}


def _all_codes():
    out = []
    for fs in (NORMAL, SHORT):
        for r in range(E.RATE_COUNT):
            try:
                cs.code_info(fs, r)
            except Exception:
                continue
            out.append((fs, r))
    return out


@pytest.mark.parametrize("fs,rate", _all_codes())
def test_every_code_matches_oracle(cuda, fs, rate):
    # noisy BPSK-like LLRs near each code's waterfall: many iterations, some failures
    ci = cs.code_info(fs, rate)
    rng = np.random.default_rng(1000 * fs + rate)
    B = 6
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    cw = cs.encode_frames(fs, rate, msg)
    bits = np.unpackbits(cw, axis=1).astype(np.float32)
    R = ci["k_ldpc"] / ci["n_ldpc"]
    ebn0 = 10 ** ((1.2 - 1.0 * (R < 0.5) + 1.5 * (R > 0.85)) / 10)
    sigma = np.sqrt(1 / (2 * R * ebn0))
    y = (1 - 2 * bits) + sigma * rng.standard_normal(bits.shape).astype(np.float32)
    llr = np.clip(np.rint(y * 2 / sigma ** 2 * 4), -32768, 32767).astype(np.int16)
    T = 30
    hg, tg = gpu_decode(cuda, fs, rate, llr, T)
    ho, to = O.ldpc_decode(fs, rate, llr, T, nthreads=8)
    assert_same(hg, tg, ho, to)


@pytest.mark.parametrize("fs,rate", [(SHORT, E.RATE_1_2), (NORMAL, E.RATE_3_5), (NORMAL, E.RATE_5_6),
                                     (NORMAL, E.RATE_9_10)])
def test_saturating_path(cuda, fs, rate):
    # channel LLRs at the int16 rails force the saturating arithmetic path
    ci = cs.code_info(fs, rate)
    rng = np.random.default_rng(77 + rate)
    B = 4
    cw = cs.encode_frames(fs, rate, rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8))
    sgn = 1 - 2 * np.unpackbits(cw, axis=1).astype(np.int32)
    mag = rng.integers(0, 32768, sgn.shape)
    mag[:, ::7] = rng.integers(32600, 32768, mag[:, ::7].shape)
    flip = rng.random(sgn.shape) < 0.08
    llr = np.clip(np.where(flip, -sgn, sgn) * mag, -32768, 32767).astype(np.int16)
    llr[:, 5] = -32768
    hg, tg = gpu_decode(cuda, fs, rate, llr, 20)
    ho, to = O.ldpc_decode(fs, rate, llr, 20)
    assert_same(hg, tg, ho, to)


@pytest.mark.parametrize("T", [0, 1, 2])
def test_tiny_iteration_caps(cuda, T):
    mod, rate = E.MOD_QPSK, E.RATE_1_2
    _, _, noisy, n0, gain = frames(mod, rate, SHORT, 8, 2.5, seed=5)
    llr = oracle_llr(mod, rate, SHORT, noisy, n0, gain)
    llr[0] = np.abs(llr[0])  # the all-zero codeword: converges at trial 0
    hg, tg = gpu_decode(cuda, SHORT, rate, llr, T)
    ho, to = O.ldpc_decode(SHORT, rate, llr, T)
    assert_same(hg, tg, ho, to)
    assert tg[0] == T


def test_batch_edges_and_errors(cuda):
    torch = cuda
    mod, rate = E.MOD_QPSK, E.RATE_1_2
    _, _, noisy, n0, gain = frames(mod, rate, SHORT, 9, 2.0, seed=6)
    llr = oracle_llr(mod, rate, SHORT, noisy, n0, gain)
    ho, to = O.ldpc_decode(SHORT, rate, llr, 25)
    dec = cs.ldpc_decode_cuda(SHORT, rate, 25, 9)
    # synchronous host path and max_batch
    h, t = dec.decode_batch(llr)
    assert_same(h, t, ho, to)
    # batch 1
    h, t = dec.decode_batch(llr[3:4])
    assert_same(h, t, ho[3:4], to[3:4])
    # device input, host output; misaligned device pointer (scalar load path)
    buf = torch.zeros(9 * llr.shape[1] + 8, dtype=torch.int16, device="cuda")
    buf[1:1 + llr.size] = torch.from_numpy(llr.reshape(-1)).cuda()
    h, t = dec.decode_batch_d2h(buf.data_ptr() + 2, 9, torch.cuda.current_stream())
    assert_same(h, t, ho, to)
    # internal pinned results after an async launch
    d = torch.from_numpy(llr).cuda()
    dec.decode_launch_async(d, 9, torch.cuda.current_stream())
    torch.cuda.synchronize()
    h, t = dec.results(9)
    assert_same(h, t, ho, to)
    for bad in (0, 10, -1):
        with pytest.raises(cs.CusatError):
            dec.decode_launch_async(d, bad, None)


MODCOD_CASES = ["qpsk1/2", "qpsk3/4", "8psk3/5", "8psk9/10", "16apsk2/3", "16apsk5/6", "32apsk3/4",
                "32apsk9/10", "64apsk32/45", "16apsk1/2l", "32apsk2/3l", "8apsk5/9", "128apsk3/4", "128apsk7/9",
                "256apsk3/4", "256apsk2/3", "256apsk11/15"]


@pytest.mark.parametrize("name", MODCOD_CASES)
@pytest.mark.parametrize("fs", [NORMAL, SHORT])
def test_demapper_bit_exact(cuda, name, fs):
    torch = cuda
    _, mod, rate, _, _, thr = E.find_modcod(name)
    try:
        cs.code_info(fs, rate)
    except cs.CusatError:
        pytest.skip("no such frame")
    _, _, noisy, n0, gain = frames(mod, rate, fs, 3, thr + 0.5, seed=21)
    dm = cs.demapper_cuda(mod, rate, fs, 3)
    g = dm.capped_llr_gain(gain)
    d_sym = torch.from_numpy(noisy).cuda()
    out = torch.zeros((3, dm.fecframe_len()), dtype=torch.int16, device="cuda")
    dm.demap_launch(d_sym, 3, n0, g, out, torch.cuda.current_stream())
    torch.cuda.synchronize()
    ref = oracle_llr(mod, rate, fs, noisy, n0, gain)
    got = out.cpu().numpy()
    assert (got == ref).all(), f"{np.count_nonzero(got != ref)} LLRs differ"
    # host path (reference demap_batch, caps the gain itself): its internal
    # buffer feeds the decoder, which must then match the oracle's decode
    dm.demap_batch(noisy, 3, n0, gain)
    dec = cs.ldpc_decode_cuda(fs, rate, 20, 3)
    h, t = dec.decode_batch_d2h(dm.soft_out_dev(), 3, torch.cuda.current_stream())
    ho, to = O.ldpc_decode(fs, rate, ref, 20)
    assert_same(h, t, ho, to)


@pytest.mark.parametrize("name,fs", [("qpsk1/2", SHORT), ("8psk3/5", NORMAL), ("16apsk2/3", NORMAL),
                                     ("32apsk3/4", SHORT), ("64apsk32/45", NORMAL), ("128apsk7/9", NORMAL),
                                     ("256apsk32/45", NORMAL)])
def test_fused_chain_matches_separate_and_oracle(cuda, name, fs):
    torch = cuda
    _, mod, rate, _, _, thr = E.find_modcod(name)
    B = 8
    msg, cw, noisy, n0, gain = frames(mod, rate, fs, B, thr + 0.3, seed=31)
    rx = cs.rx_fec(mod, rate, fs, 50, B)
    d_sym = torch.from_numpy(noisy).cuda()
    hard = torch.zeros((B, rx.k_bytes), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(B, dtype=torch.int32, device="cuda")
    valid = torch.zeros(B, dtype=torch.int32, device="cuda")
    rx.launch(d_sym, B, n0, gain, hard, trials, valid, torch.cuda.current_stream())
    torch.cuda.synchronize()
    llr = oracle_llr(mod, rate, fs, noisy, n0, gain)
    ho, to = O.ldpc_decode(fs, rate, llr, 50, nthreads=16)
    assert_same(hard.cpu().numpy(), trials.cpu().numpy(), ho, to)
    _, vo = O.bch_check(fs, rate, ho)
    assert (valid.cpu().numpy() == vo).all()


@pytest.mark.parametrize("fs,rate", [(NORMAL, E.RATE_3_5), (NORMAL, E.RATE_2_3), (NORMAL, E.RATE_9_10),
                                     (SHORT, E.RATE_1_2), (SHORT, E.RATE_1_4)])
@pytest.mark.parametrize("B", [1, 2, 3, 4, 7, 16, 31, 32, 64, 129])
def test_bch_check_matches_oracle(cuda, fs, rate, B):
    # apps/bench_bch_gpu.cc:52-104 geometry and corruption pattern
    torch = cuda
    ci = cs.code_info(fs, rate)
    k, n = ci["k_bch"] // 8, ci["n_bch"] // 8
    rng = np.random.default_rng(B + 100 * rate)
    cw = O.bch_encode(fs, rate, rng.integers(0, 256, (B, k), dtype=np.uint8))
    chk = cs.bch_check_cuda.for_code(fs, rate)
    assert chk.n_bytes() == n
    pos = [0, k - 1, k, n - 1][B % 4]
    bad = cw.copy()
    for f in range(B):
        if f % 3 != 1:
            bad[f, pos] ^= 1 << (f % 8)
    for words in (cw, bad):
        d = torch.from_numpy(words).cuda()
        valid = torch.zeros(B, dtype=torch.int32, device="cuda")
        rem = torch.zeros((B, ci["bch_degree"] // 8), dtype=torch.uint8, device="cuda")
        chk.check_async(d, valid, B, torch.cuda.current_stream(), rem)
        torch.cuda.synchronize()
        ro, vo = O.bch_check(fs, rate, words)
        assert (valid.cpu().numpy() == vo).all()
        assert (rem.cpu().numpy() == ro).all()


@pytest.mark.parametrize("name", ["64apsk32/45", "128apsk3/4", "256apsk3/4", "256apsk2/3"])
@pytest.mark.parametrize("offset_db,gain", [(-12.0, None), (12.0, None), (0.0, 0.0), (0.0, 1e-30), (0.0, 3e38),
                                            (0.0, 1e5)])
def test_demapper_cutoff_extremes(cuda, name, offset_db, gain):
    """The 64- to 256-point log-MAP demapper at the edges of its cutoff (a
    term counts when (d - min) * gain / 4 < 16): far below threshold (most
    terms inside), far above (almost none), and gains of 0, 1e-30, 3e38 and
    1e5 all give the oracle's LLRs."""
    torch = cuda
    _, mod, rate, _, _, thr = E.find_modcod(name)
    _, _, noisy, n0, g0 = frames(mod, rate, NORMAL, 2, thr + offset_db, seed=23)
    g = g0 if gain is None else gain
    dm = cs.demapper_cuda(mod, rate, NORMAL, 2)
    d_sym = torch.from_numpy(noisy).cuda()
    out = torch.zeros((2, dm.fecframe_len()), dtype=torch.int16, device="cuda")
    dm.demap_launch(d_sym, 2, n0, g, out, torch.cuda.current_stream())
    torch.cuda.synchronize()
    mi = O.modcod(mod, rate, NORMAL)
    ref = O.demap(noisy, mi["xfecframe_len"], mi["interleaved_len"], mi["fecframe_len"], mi["n_mod"], mi["kind"],
                  mi["points"], mi["col_offset"], n0, g)
    got = out.cpu().numpy()
    assert (got == ref).all(), f"{np.count_nonzero(got != ref)} LLRs differ"
