"""The reference's own GPU kernels against the oracle and this project's kernels.

The reference's demapper and layered decoder sources
(lib/cusat_dsp/cuda/demapper_kernel.cu, lib/cusat_dsp/cuda/ldpc_decode_kernel.cu)
are compiled unchanged into cubins where the reference tree is present
(oracle/build.py; the cubins travel with the other built files) and launched
through oracle/ref_gpu.c the way the reference's host classes launch them.

- Demapper: the reference kernel's int16 LLRs equal the oracle's and this
  project's, every LLR, for every MODCOD of the ACM table and frame size
  (QPSK, the 8PSK formula and the log-MAP families 8APSK to 256APSK).
- Decoder: checks of one schedule step that share a bit race in the
  reference kernel (ldpc_decode_kernel.cu:793-802), so its iteration counts
  vary from run to run; the oracle resolves the race deterministically.  The
  reference's hard decisions equal the oracle's on every frame where both
  converge, for every code; on the benchmark workloads both converge on the
  same frames.
"""
import os

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

DEMAP_CASES = [("qpsk1/2", 1), ("qpsk3/4", 0), ("8psk3/5", 0), ("8psk8/9", 1), ("8apsk5/9", 0),
               ("16apsk2/3", 0), ("16apsk5/6", 1), ("32apsk3/4", 0), ("64apsk32/45", 0), ("128apsk3/4", 0),
               ("256apsk3/4", 0), ("256apsk32/45", 0)]
# (MODCOD, frame size, frames, Es/N0 dB or None = threshold + 0.5, seed)
DECODE_CASES = [("8psk3/5", 0, 256, 6.0, 2024), ("qpsk1/2", 1, 64, 1.5, 2025), ("8psk9/10", 0, 64, None, 32),
                ("qpsk1/4", 0, 32, None, 31)]


def _modcod_cases():
    out = []
    for m in E.MODCODS:
        for fs in (0, 1):
            try:
                cs.code_info(fs, m[2])
            except cs.CusatError:
                continue
            out.append((m[3], fs))
    return out


def _codes():
    out = []
    for fs in (0, 1):
        for r in range(E.RATE_COUNT):
            try:
                cs.code_info(fs, r)
            except cs.CusatError:
                continue
            out.append((fs, r))
    return out


@pytest.fixture(scope="module")
def rg(cuda):
    try:
        return O.RefGpu()
    except FileNotFoundError as e:
        pytest.skip(f"reference kernels not built here: {e}")


def traffic(name, fs, B, esn0, seed):
    _, mod, rate, _, _, thr = E.find_modcod(name)
    esn0 = thr + 0.5 if esn0 is None else esn0
    rng = np.random.default_rng(seed)
    ci = cs.code_info(fs, rate)
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    sym = cs.map_frames(mod, rate, fs, cs.encode_frames(fs, rate, msg))
    sym = (sym / np.float32(np.sqrt(float(np.mean(sym.astype(np.float64) ** 2) * 2)))).astype(np.float32)
    n0 = np.float32(1.0 / 10 ** (esn0 / 10.0))
    noisy = (sym + np.float32(np.sqrt(n0 / np.float32(2.0))) * rng.standard_normal(sym.shape, dtype=np.float32))
    mi = O.modcod(mod, rate, fs)
    return mod, rate, noisy.astype(np.float32), float(n0), O.capped_llr_gain(mi, min(4.0 / float(n0), 1000.0)), mi


@pytest.mark.parametrize("name,fs", _modcod_cases())
def test_reference_demapper_bit_exact(cuda, rg, name, fs):
    # every MODCOD of the ACM table, both frame sizes where the code exists
    torch = cuda
    B = 2 if (name, fs) not in DEMAP_CASES else 4
    mod, rate, sym, n0, gain, mi = traffic(name, fs, B, None, 41)
    s = torch.cuda.current_stream()
    d_sym = torch.from_numpy(sym).cuda()
    pts = mi["points"]
    d_re = torch.from_numpy(np.ascontiguousarray(pts.real, np.float32)).cuda()
    d_im = torch.from_numpy(np.ascontiguousarray(pts.imag, np.float32)).cuda()
    d_ref = torch.zeros((B, mi["fecframe_len"]), dtype=torch.int16, device="cuda")
    d_ours = torch.zeros_like(d_ref)
    rg.demap(d_sym, d_ref, d_re, d_im, mi, n0, gain, B, s)
    dm = cs.demapper_cuda(mod, rate, fs, B)
    dm.demap_launch(d_sym, B, n0, gain, d_ours, s)
    torch.cuda.synchronize()
    want = O.demap_modcod(sym, mi, n0, gain)
    ref, ours = d_ref.cpu().numpy(), d_ours.cpu().numpy()
    assert (ref == want).all(), f"reference kernel vs oracle: {np.count_nonzero(ref != want)} LLRs differ"
    assert (ours == ref).all(), f"this project vs reference kernel: {np.count_nonzero(ours != ref)} LLRs differ"


@pytest.mark.parametrize("name,fs,B,esn0,seed", DECODE_CASES)
def test_reference_decoder_agrees_with_oracle(cuda, rg, name, fs, B, esn0, seed):
    torch = cuda
    mod, rate, sym, n0, gain, mi = traffic(name, fs, B, esn0, seed)
    llr = O.demap_modcod(sym, mi, n0, gain)
    ho, to = O.ldpc_decode(fs, rate, llr, 50, nthreads=os.cpu_count() or 8)
    kb = O.code_info(fs, rate)["K"] // 8
    s = torch.cuda.current_stream()
    d_llr = torch.from_numpy(llr).cuda()
    h = torch.zeros((B, kb), dtype=torch.uint8, device="cuda")
    t = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec = rg.decoder(fs, rate, 50, B)
    try:
        dec.launch(d_llr, B, h, t, s)
        torch.cuda.synchronize()
    finally:
        dec.close()
    hr, tr = h.cpu().numpy(), t.cpu().numpy()
    assert ((tr >= 0) == (to >= 0)).all(), "the reference kernel and the oracle converge on different frames"
    conv = (tr >= 0) & (to >= 0)
    bad = np.nonzero(conv & (hr != ho).any(axis=1))[0]
    assert len(bad) == 0, f"converged frames {bad[:8]} decode to different bits"
    assert conv.sum() >= B // 2  # the workload actually decodes
    print(f"{name}: trials identical on {(tr == to).sum()} of {B} frames")


@pytest.mark.parametrize("fs,rate", _codes())
def test_reference_decoder_every_code(cuda, rg, fs, rate):
    # every code, noisy BPSK-like LLRs a little above its waterfall (Eb/N0
    # rising with the rate; about 9 iterations on average, nearly every
    # frame converging): where both converge, the reference kernel's hard
    # bits are the oracle's
    torch = cuda
    ci = cs.code_info(fs, rate)
    rng = np.random.default_rng(1000 * fs + rate)
    B = 16
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    bits = np.unpackbits(cs.encode_frames(fs, rate, msg), axis=1).astype(np.float32)
    R = ci["k_ldpc"] / ci["n_ldpc"]
    ebn0 = 10 ** ((2.0 + 5.0 * (R - 0.5)) / 10)
    sigma = np.sqrt(1 / (2 * R * ebn0))
    y = (1 - 2 * bits) + sigma * rng.standard_normal(bits.shape).astype(np.float32)
    llr = np.clip(np.rint(y * 2 / sigma ** 2 * 4), -32768, 32767).astype(np.int16)
    T = 30
    ho, to = O.ldpc_decode(fs, rate, llr, T, nthreads=os.cpu_count() or 8)
    assert (to >= 0).sum() >= B // 2  # the recipe decodes
    s = torch.cuda.current_stream()
    h = torch.zeros((B, ci["k_ldpc"] // 8), dtype=torch.uint8, device="cuda")
    t = torch.zeros(B, dtype=torch.int32, device="cuda")
    dec = rg.decoder(fs, rate, T, B)
    try:
        dec.launch(torch.from_numpy(llr).cuda(), B, h, t, s)
        torch.cuda.synchronize()
    finally:
        dec.close()
    hr, tr = h.cpu().numpy(), t.cpu().numpy()
    conv = (tr >= 0) & (to >= 0)
    bad = np.nonzero(conv & (hr != ho).any(axis=1))[0]
    assert len(bad) == 0, f"converged frames {bad[:8]} decode to different bits"
    assert conv.sum() >= B // 4
    print(f"fs {fs} rate {rate}: converged ref {(tr >= 0).sum()} oracle {(to >= 0).sum()} both {conv.sum()}, "
          f"trials identical {(tr == to).sum()} of {B}")
