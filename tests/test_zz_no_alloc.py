"""The decode entry point that allocates no device memory.

cusat_ldpc_decode_noalloc exists for callers that must not allocate device
memory (a real-time thread under a no-allocation rule, a host whose memory
pool owns every device allocation).  It keeps its message rows, code tables
and frame counter in fixed arrays inside the library.  This file is collected
last so that a failure here never hides the other tests; it passes alone in
a fresh process and after the rest of the suite.
"""
import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from channel import frames
from cusat_gb300 import _capi
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

SHORT_HALF = (E.MOD_QPSK, E.RATE_1_2, E.FECFRAME_SHORT, 1.5, 64)
NORMAL_35 = (E.MOD_8PSK, E.RATE_3_5, E.FECFRAME_NORMAL, 6.0, 96)


def _call(torch, fs, rate, T, d_llr, B):
    hard = torch.zeros((B, cs.code_info(fs, rate)["k_ldpc"] // 8), dtype=torch.uint8, device="cuda")
    trials = torch.full((B,), -7, dtype=torch.int32, device="cuda")
    rc = _capi.lib().cusat_ldpc_decode_noalloc(fs, rate, T, d_llr.data_ptr(), B, hard.data_ptr(), trials.data_ptr(),
                                               torch.cuda.current_stream().cuda_stream)
    return rc, hard, trials


def _noalloc(torch, fs, rate, T, d_llr, B):
    rc, hard, trials = _call(torch, fs, rate, T, d_llr, B)
    _capi.check(rc)
    torch.cuda.synchronize()
    return hard.cpu().numpy(), trials.cpu().numpy()


def _llr(mod, rate, fs, B, esn0, seed):
    # demapped by the oracle with its own gain cap and the reference's points
    _, _, noisy, n0, gain = frames(mod, rate, fs, B, esn0, seed)
    return O.demap_modcod(noisy, O.modcod(mod, rate, fs), n0, gain)


def _assert_same(h, t, ho, to):
    bad = np.nonzero((t != to) | (h != ho).any(axis=1))[0]
    assert len(bad) == 0, f"frames {bad[:8]} differ: trials {t[bad[:8]]} vs {to[bad[:8]]}"


@pytest.mark.parametrize("mod,rate,fs,esn0,B", [SHORT_HALF, NORMAL_35])
def test_noalloc_matches_allocating_decoder_and_oracle_twice(cuda, mod, rate, fs, esn0, B):
    # 96 normal frames on the <= 60 CTAs the 24 MiB message area holds: CTAs
    # decode several frames each
    torch = cuda
    llr = _llr(mod, rate, fs, B, esn0, seed=41)
    ho, to = O.ldpc_decode(fs, rate, llr, 50, nthreads=16)
    d_llr = torch.from_numpy(llr).cuda()
    # the existing entry point
    dec = cs.ldpc_decode_cuda(fs, rate, 50, B)
    ref_h = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    ref_t = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), ref_h, ref_t)
    torch.cuda.synchronize()
    ref_h, ref_t = ref_h.cpu().numpy(), ref_t.cpu().numpy()
    _assert_same(ref_h, ref_t, ho, to)
    # two calls in a row share the fixed arrays and must both agree
    for _ in range(2):
        h, t = _noalloc(torch, fs, rate, 50, d_llr, B)
        _assert_same(h, t, ref_h, ref_t)
        _assert_same(h, t, ho, to)
    assert (to >= 0).sum() > B // 2


def test_noalloc_switches_codes_back_and_forth(cuda):
    # short 1/2 -> normal 3/5 -> short 1/2 on one stream: each call decodes
    # with its own code's tables
    torch = cuda
    cases = []
    for mod, rate, fs, esn0, _ in (SHORT_HALF, NORMAL_35):
        llr = _llr(mod, rate, fs, 24, esn0, seed=43 + rate)
        cases.append((fs, rate, torch.from_numpy(llr).cuda(), O.ldpc_decode(fs, rate, llr, 50, nthreads=16)))
    for k in (0, 1, 0, 1, 0):
        fs, rate, d_llr, (ho, to) = cases[k]
        h, t = _noalloc(torch, fs, rate, 50, d_llr, 24)
        _assert_same(h, t, ho, to)


def _all_codes():
    out = []
    for fs in (E.FECFRAME_NORMAL, E.FECFRAME_SHORT):
        for r in range(E.RATE_COUNT):
            try:
                cs.code_info(fs, r)
            except Exception:
                continue
            out.append((fs, r))
    return out


def test_noalloc_every_code_fits(cuda):
    # every supported code's tables and message rows fit the fixed arrays:
    # one noiseless frame each (+-127 LLRs of a codeword) decodes at trial 0
    torch = cuda
    codes = _all_codes()
    assert len(codes) >= 50
    rng = np.random.default_rng(5)
    for fs, rate in codes:
        ci = cs.code_info(fs, rate)
        msg = rng.integers(0, 256, (1, ci["k_bch"] // 8), dtype=np.uint8)
        cw = cs.encode_frames(fs, rate, msg)
        llr = (127 - 254 * np.unpackbits(cw, axis=1).astype(np.int16)).astype(np.int16)
        d_llr = torch.from_numpy(llr).cuda()
        rc, hard, trials = _call(torch, fs, rate, 10, d_llr, 1)
        assert rc == 0, (fs, rate, _capi.lib().cusat_last_error())
        torch.cuda.synchronize()
        assert trials.item() == 10, (fs, rate)
        assert (hard.cpu().numpy()[0] == cw[0, :ci["k_ldpc"] // 8]).all(), (fs, rate)


def test_noalloc_refuses_graph_capture(cuda):
    torch = cuda
    llr = torch.zeros((1, 16200), dtype=torch.int16, device="cuda")
    hard = torch.zeros((1, 900), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(1, dtype=torch.int32, device="cuda")
    _noalloc(torch, E.FECFRAME_SHORT, E.RATE_1_2, 5, llr, 1)  # loads the module outside the capture
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin(capture_error_mode="relaxed")
        try:
            rc = _capi.lib().cusat_ldpc_decode_noalloc(E.FECFRAME_SHORT, E.RATE_1_2, 5, llr.data_ptr(), 1,
                                                       hard.data_ptr(), trials.data_ptr(), s.cuda_stream)
        finally:
            g.capture_end()
    assert rc == -2  # CUSAT_ERR_UNSUPPORTED, nothing enqueued
    assert b"CUDA graph" in _capi.lib().cusat_last_error()
    torch.cuda.synchronize()


def test_noalloc_rejects_bad_arguments(cuda):
    torch = cuda
    d = torch.zeros(16200, dtype=torch.int16, device="cuda")
    out = torch.zeros(1024, dtype=torch.uint8, device="cuda")
    tr = torch.zeros(4, dtype=torch.int32, device="cuda")
    L = _capi.lib()
    assert L.cusat_ldpc_decode_noalloc(E.FECFRAME_SHORT, E.RATE_1_2, 50, d.data_ptr(), 0, out.data_ptr(),
                                       tr.data_ptr(), None) == -1
    assert L.cusat_ldpc_decode_noalloc(E.FECFRAME_SHORT, E.RATE_9_10, 50, d.data_ptr(), 1, out.data_ptr(),
                                       tr.data_ptr(), None) == -2
    assert b"" != L.cusat_last_error()
