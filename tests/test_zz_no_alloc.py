"""The decode entry point that allocates no device memory.

cusat_ldpc_decode_noalloc exists for callers that must not allocate device
memory (a real-time thread under a no-allocation rule, a host whose memory
pool owns every device allocation).  It keeps its message rows, code tables
and frame counter in fixed arrays inside the library.  This file is collected
last so that a failure here never hides the other tests; it passes alone in
a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from channel import frames
from cusat_gb300 import _capi
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu


def _noalloc(torch, fs, rate, T, d_llr, B):
    hard = torch.zeros((B, cs.code_info(fs, rate)["k_ldpc"] // 8), dtype=torch.uint8, device="cuda")
    trials = torch.full((B,), -7, dtype=torch.int32, device="cuda")
    _capi.check(_capi.lib().cusat_ldpc_decode_noalloc(fs, rate, T, d_llr.data_ptr(), B, hard.data_ptr(),
                                                      trials.data_ptr(), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return hard.cpu().numpy(), trials.cpu().numpy()


def _llr(mod, rate, fs, B, esn0, seed):
    _, _, noisy, n0, gain = frames(mod, rate, fs, B, esn0, seed)
    mi = cs.modcod_info(mod, rate, fs)
    return O.demap(noisy, mi["xfecframe_len"], mi["interleaved_len"], mi["fecframe_len"], mi["n_mod"],
                   mi["kind"], mi["points"], mi["col_offset"], n0, cs.capped_llr_gain(mod, rate, fs, gain))


@pytest.mark.parametrize("mod,rate,fs,esn0,B", [(E.MOD_QPSK, E.RATE_1_2, E.FECFRAME_SHORT, 1.5, 64),
                                               (E.MOD_8PSK, E.RATE_3_5, E.FECFRAME_NORMAL, 6.0, 96)])
def test_noalloc_matches_allocating_decoder_twice(cuda, mod, rate, fs, esn0, B):
    torch = cuda
    llr = _llr(mod, rate, fs, B, esn0, seed=41)
    d_llr = torch.from_numpy(llr).cuda()
    # the existing entry point
    dec = cs.ldpc_decode_cuda(fs, rate, 50, B)
    ref_h = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    ref_t = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), ref_h, ref_t)
    torch.cuda.synchronize()
    ref_h, ref_t = ref_h.cpu().numpy(), ref_t.cpu().numpy()
    # two calls in a row share the fixed arrays and must both agree
    for _ in range(2):
        h, t = _noalloc(torch, fs, rate, 50, d_llr, B)
        assert (t == ref_t).all() and (h == ref_h).all()


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
