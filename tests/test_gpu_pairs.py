"""The frame-pair decoder kernel (two short frames per CTA, one per int16
half of the APP words) against the oracle, bit for bit.

Short frames of every decoder kernel class run through cusat_ldpc_decoder
and the receive chain as pairs; frames whose channel LLRs leave the
saturation-free range are listed by the pair kernel and decoded by the
one-frame kernel.  Covered: odd batches (a CTA with one empty slot), slots
refilled from the queue while the other slot keeps decoding (a capped grid),
batches where every frame or no frame takes the saturating path, repeated
launches (the rearmed counters and list), the syndrome period knob, and
learned weights (which keep the one-frame kernel)."""
import os
import subprocess
import sys

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

SHORT = E.FECFRAME_SHORT
THREADS = os.cpu_count() or 8
HERE = os.path.dirname(os.path.abspath(__file__))

# one short code per kernel class (circulant slots per layer)
SHORT_CODES = [E.RATE_1_4, E.RATE_1_2, E.RATE_3_5, E.RATE_3_4, E.RATE_5_6, E.RATE_8_9]


def _llr(fs, rate, B, seed, db=None):
    """Noisy BPSK LLRs of B random codewords, each frame at its own Es/N0
    within [-1.5, +0.5] dB of a point near the code's waterfall (frames that
    converge early, late and never)."""
    ci = cs.code_info(fs, rate)
    rng = np.random.default_rng(seed)
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    cw = cs.encode_frames(fs, rate, msg)
    bits = np.unpackbits(cw, axis=1).astype(np.float32)
    R = ci["k_ldpc"] / ci["n_ldpc"]
    if db is None:
        db = 1.0 + (R >= 0.5) + 1.5 * (R > 0.7) + 1.0 * (R > 0.85)
    db = db + rng.uniform(-1.5, 0.5, (B, 1))
    sigma = np.sqrt(1 / (2 * R * 10 ** (db / 10)))
    y = (1 - 2 * bits) + sigma * rng.standard_normal(bits.shape).astype(np.float32)
    return np.clip(np.rint(y * 2 / sigma ** 2 * 4), -32768, 32767).astype(np.int16)


def _decode(torch, dec, llr, T):
    B = llr.shape[0]
    d_llr = torch.from_numpy(llr).cuda()
    hard = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    trials = torch.full((B,), -9, dtype=torch.int32, device="cuda")
    dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), hard, trials)
    torch.cuda.synchronize()
    return hard.cpu().numpy(), trials.cpu().numpy()


def _same(tag, h, t, ho, to):
    bad = np.nonzero((t != to) | (h != ho).any(axis=1))[0]
    assert len(bad) == 0, f"{tag}: frames {bad[:8]} differ: trials gpu {t[bad[:8]]} oracle {to[bad[:8]]}"


@pytest.mark.parametrize("rate", SHORT_CODES)
def test_pairs_match_oracle_every_class(cuda, rate):
    torch = cuda
    T = 30
    dec = cs.ldpc_decode_cuda(SHORT, rate, T, 96)
    dec.set_frames_per_cta(2)
    assert dec.frames_per_cta(1) == 2
    llr = _llr(SHORT, rate, 96, seed=700 + rate)
    ho, to = O.ldpc_decode(SHORT, rate, llr, T, nthreads=THREADS)
    # odd and even batches: a CTA of an odd batch keeps one slot empty
    for B in (1, 2, 7, 96):
        h, t = _decode(torch, dec, llr[:B], T)
        _same(f"B={B}", h, t, ho[:B], to[:B])
    assert (to >= 0).sum() >= 24 and (to < 0).any()


@pytest.mark.parametrize("rate", [E.RATE_1_2, E.RATE_3_4])
def test_pairs_refill_and_saturating_list(cuda, rate):
    """Three CTAs for 61 frames: each slot refills from the queue as its
    frame retires.  Every fourth frame has LLRs at the rails and goes to the
    one-frame kernel through the list; two launches in a row reuse the
    counters and the list."""
    torch = cuda
    T = 40
    B = 61
    llr = _llr(SHORT, rate, B, seed=900 + rate)
    llr[1::4, ::13] = np.where(llr[1::4, ::13] < 0, -32768, 32767)
    ho, to = O.ldpc_decode(SHORT, rate, llr, T, nthreads=THREADS)
    dec = cs.ldpc_decode_cuda(SHORT, rate, T, B)
    dec.set_frames_per_cta(2)
    dec.set_max_ctas(3)
    for rep in range(2):
        h, t = _decode(torch, dec, llr, T)
        _same(f"launch {rep}", h, t, ho, to)
    # every frame saturating, then none: the list holds all frames, then none
    sat = llr.copy()
    sat[:, ::7] = np.where(sat[:, ::7] < 0, -32768, 32767)
    hs, ts = O.ldpc_decode(SHORT, rate, sat, T, nthreads=THREADS)
    plain = np.clip(llr, -2000, 2000)
    hp, tp = O.ldpc_decode(SHORT, rate, plain, T, nthreads=THREADS)
    dec.set_max_ctas(0)
    for rep in range(2):
        h, t = _decode(torch, dec, sat, T)
        _same(f"all saturating {rep}", h, t, hs, ts)
        h, t = _decode(torch, dec, plain, T)
        _same(f"none saturating {rep}", h, t, hp, tp)


def test_pairs_trial_cap_edges(cuda):
    """max_trials 0 and 1: frames retire at the first syndrome or after one
    iteration; noiseless frames converge at trial 0 in both slots."""
    torch = cuda
    rate = E.RATE_2_3
    ci = cs.code_info(SHORT, rate)
    llr = _llr(SHORT, rate, 9, seed=5)
    rng = np.random.default_rng(6)
    msg = rng.integers(0, 256, (4, ci["k_bch"] // 8), dtype=np.uint8)
    clean = (127 - 254 * np.unpackbits(cs.encode_frames(SHORT, rate, msg), axis=1).astype(np.int16)).astype(np.int16)
    both = np.concatenate([llr, clean])
    for T in (0, 1, 2):
        dec = cs.ldpc_decode_cuda(SHORT, rate, T, len(both))
        dec.set_frames_per_cta(2)
        ho, to = O.ldpc_decode(SHORT, rate, both, T, nthreads=THREADS)
        h, t = _decode(torch, dec, both, T)
        _same(f"T={T}", h, t, ho, to)
        assert (to[-4:] == T).all()


def test_learned_weights_keep_one_frame_kernel(cuda):
    torch = cuda
    rate = E.RATE_1_2
    T = 20
    dec = cs.ldpc_decode_cuda(SHORT, rate, T, 32)
    dec.set_frames_per_cta(2)
    assert dec.frames_per_cta(32) == 2
    w = np.zeros((T, 32, 2), np.int16)
    w[:, :, 0] = 1
    w[:, :, 1] = 48  # beta 1, alpha 0.75
    dec.set_weights(w)
    assert dec.frames_per_cta(32) == 1
    llr = _llr(SHORT, rate, 32, seed=77)
    ho, to = O.ldpc_decode(SHORT, rate, llr, T, weights=w, nthreads=THREADS)
    h, t = _decode(torch, dec, llr, T)
    _same("weighted", h, t, ho, to)
    dec.set_weights(None)
    assert dec.frames_per_cta(32) == 2
    ho, to = O.ldpc_decode(SHORT, rate, llr, T, nthreads=THREADS)
    h, t = _decode(torch, dec, llr, T)
    _same("plain again", h, t, ho, to)


def test_frames_per_cta_choice(cuda):
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for fs, rate in ((E.FECFRAME_NORMAL, E.RATE_3_5), (E.FECFRAME_NORMAL, E.RATE_22_30)):
        dec = cs.ldpc_decode_cuda(fs, rate, 10, 8)
        dec.set_frames_per_cta(2)
        assert dec.frames_per_cta(8) == 1  # normal frames: no pair fits
    dec = cs.ldpc_decode_cuda(SHORT, E.RATE_1_2, 10, 4 * sms)
    lo = -(-3 * sms // 4) * 2  # the smallest batch whose pairs cover 3/4 of the SMs
    assert dec.frames_per_cta(lo - 2) == 1 and dec.frames_per_cta(lo) == 2
    wide = cs.ldpc_decode_cuda(SHORT, E.RATE_8_9, 10, 4 * sms)
    assert wide.frames_per_cta(4 * sms) == 1  # 28 slots: one frame per CTA by default
    wide.set_frames_per_cta(2)
    assert wide.frames_per_cta(1) == 2
    dec.set_frames_per_cta(1)
    assert dec.frames_per_cta(4 * sms) == 1
    dec.set_frames_per_cta(2)
    assert dec.frames_per_cta(1) == 2
    with pytest.raises(cs.CusatError):
        dec.set_frames_per_cta(3)


def test_pairs_by_batch_size_match_oracle(cuda):
    """Default choice: a small batch runs one frame per CTA, a batch whose
    pairs cover the SMs frame pairs -- same results."""
    torch = cuda
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rate, T = E.RATE_1_2, 25
    B = 2 * sms + 3
    llr = _llr(SHORT, rate, B, seed=4242)
    ho, to = O.ldpc_decode(SHORT, rate, llr, T, nthreads=THREADS)
    dec = cs.ldpc_decode_cuda(SHORT, rate, T, B)
    assert dec.frames_per_cta(B) == 2 and dec.frames_per_cta(40) == 1
    for n in (B, 40):
        h, t = _decode(torch, dec, llr[:n], T)
        _same(f"B={n} ({dec.frames_per_cta(n)} per CTA)", h, t, ho[:n], to[:n])


_PERIOD_CHILD = r"""
import os, sys
sys.path[:0] = [os.path.dirname({here!r}), {here!r}]
import numpy as np, torch
import oracle_lib as O
from cusat_gb300 import enums as E
import cusat_gb300 as cs
from test_gpu_pairs import _llr, _decode, _same
for fs, rate in ((E.FECFRAME_SHORT, E.RATE_1_2), (E.FECFRAME_SHORT, E.RATE_5_6), (E.FECFRAME_NORMAL, E.RATE_3_5)):
    llr = _llr(fs, rate, 24, seed=31 + rate)
    ho, to = O.ldpc_decode(fs, rate, llr, 25, nthreads=8, syn_period=3)
    dec = cs.ldpc_decode_cuda(fs, rate, 25, 24)
    dec.set_frames_per_cta(2)
    h, t = _decode(torch, dec, llr, 25)
    _same(f"period 3 fs {{fs}} rate {{rate}}", h, t, ho, to)
print("ok")
"""


def test_syndrome_period_knob(cuda):
    """CUSAT_LDPC_SYN_PERIOD=3 (read once per process): both kernels check
    the syndrome before every third iteration and at the cap, as the oracle
    does."""
    env = dict(os.environ, CUSAT_LDPC_SYN_PERIOD="3")
    r = subprocess.run([sys.executable, "-c", _PERIOD_CHILD.format(here=HERE)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
