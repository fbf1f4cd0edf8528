"""The benchmark workloads at their full sizes against the oracle (bit-exact).

- Normal 3/5 8PSK: every frame of every input batch bench.py cycles through
  (4 x 256 frames, built by bench.make_traffic with its seed), through the
  receive chain the bench times (demap -> decode -> BCH), compared frame by
  frame with the oracle's demap -> decode -> BCH check: LLRs, hard decisions,
  iteration counts, BCH flags.
- Short 1/2 QPSK: the same for the short workload's batches.
- Mixed batch: the 1024 frames of bench.py's mixed workload (10 MODCODs,
  normal and short), launched, tuned, captured and replayed as the bench
  does, against the oracle frame by frame.
- CTAs that decode several frames in turn: a capped grid (a handful of CTAs
  for dozens of frames) for one code of every decoder kernel class, with
  saturating and non-saturating frames interleaved, and a mixed batch whose
  CTAs switch codes.  This is the path every batch larger than the resident
  CTA slots takes.

The oracle side derives its demap parameters (points, interleaver columns,
gain cap) from its own restatement, not from the product.
"""
import os

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT
THREADS = os.cpu_count() or 8


def _bench():
    import bench
    return bench


def _oracle_chain(mod, rate, fs, sym, n0, gain, T):
    mi = O.modcod(mod, rate, fs)
    llr = O.demap_modcod(sym, mi, n0, gain)
    hard, trials = O.ldpc_decode(fs, rate, llr, T, nthreads=THREADS)
    _, valid = O.bch_check(fs, rate, hard)
    return llr, hard, trials, valid


def _assert_frames(tag, h, t, v, ho, to, vo):
    bad = np.nonzero((t != to) | (h != ho).any(axis=1) | ((v != 0) != (vo != 0)))[0]
    assert len(bad) == 0, f"{tag}: frames {bad[:8]} differ: trials gpu {t[bad[:8]]} oracle {to[bad[:8]]}"


@pytest.mark.parametrize("which", ["single", "short"])
def test_bench_batches_match_oracle(cuda, which):
    torch = cuda
    bench = _bench()
    wl = dict(bench.WORKLOAD if which == "single" else bench.WORKLOAD_SHORT)
    nb = bench.n_bufs_for(wl, bench.ProductGen())
    ci, msg, bufs, n0, gain = bench.make_traffic(wl, nb)
    B, T = wl["frames"], wl["max_trials"]
    mod, rate, fs = wl["mod"], wl["rate"], wl["fs"]
    rx = cs.rx_fec(mod, rate, fs, T, B)
    # frames per CTA as the bench chooses them (frame pairs for the short
    # workload's eight chains)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    pipe = min(8, max(bench.PIPE, -(-bench.RESIDENT_CTAS // B)))
    rx.set_frames_per_cta(bench.frames_per_cta_for(cs.code_info(fs, rate), pipe, B, sms))
    dm = cs.demapper_cuda(mod, rate, fs, B)
    st = torch.cuda.current_stream()
    hard = torch.zeros((B, ci["k_ldpc"] // 8), dtype=torch.uint8, device="cuda")
    trials = torch.zeros(B, dtype=torch.int32, device="cuda")
    valid = torch.zeros(B, dtype=torch.int32, device="cuda")
    soft = torch.zeros((B, ci["n_ldpc"]), dtype=torch.int16, device="cuda")
    converged = 0
    for k, sym in enumerate(bufs):
        d_sym = torch.from_numpy(sym).cuda()
        rx.launch(d_sym, B, n0, gain, hard, trials, valid, st)
        dm.demap_launch(d_sym, B, n0, dm.capped_llr_gain(gain), soft, st)
        torch.cuda.synchronize()
        llr, ho, to, vo = _oracle_chain(mod, rate, fs, sym, n0, gain, T)
        assert (soft.cpu().numpy() == llr).all(), f"batch {k}: LLRs differ"
        _assert_frames(f"batch {k}", hard.cpu().numpy(), trials.cpu().numpy(), valid.cpu().numpy(), ho, to, vo)
        converged += int((to >= 0).sum())
    assert converged > len(bufs) * B // 2


def test_bench_mixed_batch_matches_oracle(cuda):
    torch = cuda
    bench = _bench()
    T = bench.MIXED["max_trials"]
    mt = bench.MixedTraffic(cs, bench.MIXED["frames"], bench.MIXED["seed"])
    n = len(mt.frames)
    # oracle, one call per MODCOD
    ho = [None] * n
    to = np.zeros(n, np.int32)
    vo = np.zeros(n, np.int32)
    groups = {}
    for f, fr in enumerate(mt.frames):
        groups.setdefault(fr["modcod"], []).append(f)
    for m, ids in groups.items():
        _, mod, rate, fs = mt.table[m]
        fr0 = mt.frames[ids[0]]
        sym = np.stack([mt.frames[f]["sym"] for f in ids])
        _, h, t, v = _oracle_chain(mod, rate, fs, sym, fr0["n0"], fr0["gain"], T)
        for k, f in enumerate(ids):
            ho[f], to[f], vo[f] = h[k], t[k], v[k]

    st = torch.cuda.Stream()
    d_sym = torch.from_numpy(mt.sym).cuda()
    d_hard = torch.zeros(mt.hard_bytes, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros((2, n), dtype=torch.int32, device="cuda")
    b = cs.batch(mt.modcods, max_trials=T, max_frames=n)
    fr = mt.descriptors(cs, d_sym, d_hard, d_res[0], d_res[1])

    def check(tag):
        hard = d_hard.cpu().numpy()
        res = d_res.cpu().numpy()
        bad = []
        for f in range(n):
            kb = mt.geo[mt.frames[f]["modcod"]][1] // 8
            h = hard[mt.hard_off[f]:mt.hard_off[f] + kb]
            if res[0, f] != to[f] or (res[1, f] != 0) != (vo[f] != 0) or not (h == ho[f]).all():
                bad.append(f)
        assert not bad, f"{tag}: frames {bad[:8]} differ (trials gpu {res[0, bad[:8]]} oracle {to[bad[:8]]})"

    torch.cuda.synchronize()
    b.launch(fr, st)
    st.synchronize()
    check("launch")
    # as the bench runs it: tuned, captured, replayed
    d_hard.zero_()
    d_res.fill_(-9)
    torch.cuda.synchronize()
    b.tune(fr, reps=1, stream=st)
    b.capture(fr, st)
    d_hard.zero_()
    d_res.fill_(-9)
    torch.cuda.synchronize()
    b.replay(st)
    st.synchronize()
    check("replay")
    # three CTAs per kernel class: each CTA decodes many frames and switches
    # between the codes of its class
    b2 = cs.batch(mt.modcods, max_trials=T, max_frames=n)
    b2.set_max_ctas(3)
    d_hard.zero_()
    d_res.fill_(-9)
    torch.cuda.synchronize()
    b2.launch(fr, st)
    st.synchronize()
    check("3 CTAs per class")
    assert (to >= 0).sum() > n * 0.9


# one code per decoder kernel class (circulant slots per layer, lanes)
CLASS_CODES = [
    (NORMAL, E.RATE_1_4), (SHORT, E.RATE_1_4),          # 2 slots
    (NORMAL, E.RATE_1_3), (SHORT, E.RATE_1_3),          # 3
    (NORMAL, E.RATE_2_5), (SHORT, E.RATE_2_5),          # 4
    (NORMAL, E.RATE_1_2), (SHORT, E.RATE_1_2),          # 5
    (NORMAL, E.RATE_90_180),                            # 6
    (NORMAL, E.RATE_2_3), (SHORT, E.RATE_2_3),          # 8
    (NORMAL, E.RATE_3_5), (SHORT, E.RATE_3_5),          # 9
    (NORMAL, E.RATE_116_180),                           # 10
    (NORMAL, E.RATE_3_4), (SHORT, E.RATE_3_4),          # 12
    (NORMAL, E.RATE_128_180),                           # 14
    (NORMAL, E.RATE_4_5), (NORMAL, E.RATE_22_30),       # 16, two lanes and one lane (sequential schedule)
    (NORMAL, E.RATE_140_180), (SHORT, E.RATE_5_6),      # 18
    (NORMAL, E.RATE_5_6),                               # 20
    (NORMAL, E.RATE_8_9), (SHORT, E.RATE_8_9),          # 26
    (NORMAL, E.RATE_9_10),                              # 28
]


@pytest.mark.parametrize("fs,rate", CLASS_CODES)
def test_few_ctas_decode_many_frames(cuda, fs, rate):
    torch = cuda
    ci = cs.code_info(fs, rate)
    rng = np.random.default_rng(300 + 50 * fs + rate)
    B = 40
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    cw = cs.encode_frames(fs, rate, msg)
    bits = np.unpackbits(cw, axis=1).astype(np.float32)
    R = ci["k_ldpc"] / ci["n_ldpc"]
    # past each code's waterfall (about 13-23 mean iterations) for the
    # non-rail frames
    ebn0 = 10 ** ((1.0 + (R >= 0.5) + 1.5 * (R > 0.7) + 1.0 * (R > 0.85)) / 10)
    sigma = np.sqrt(1 / (2 * R * ebn0))
    y = (1 - 2 * bits) + sigma * rng.standard_normal(bits.shape).astype(np.float32)
    llr = np.clip(np.rint(y * 2 / sigma ** 2 * 4), -32768, 32767).astype(np.int16)
    # every third frame carries LLRs at the rails: the saturating arithmetic
    # path, chosen again for each frame a CTA picks up
    llr[::3, ::11] = np.where(llr[::3, ::11] < 0, -32768, 32767)
    T = 30
    dec = cs.ldpc_decode_cuda(fs, rate, T, B)
    dec.set_max_ctas(3)
    d_llr = torch.from_numpy(llr).cuda()
    hard = torch.zeros((B, dec.k_bytes()), dtype=torch.uint8, device="cuda")
    trials = torch.full((B,), -9, dtype=torch.int32, device="cuda")
    for rep in range(2):  # the second launch reuses message rows and the rearmed frame counter
        dec.decode_launch_async(d_llr, B, torch.cuda.current_stream(), hard, trials)
        torch.cuda.synchronize()
        ho, to = O.ldpc_decode(fs, rate, llr, T, nthreads=THREADS)
        h, t = hard.cpu().numpy(), trials.cpu().numpy()
        bad = np.nonzero((t != to) | (h != ho).any(axis=1))[0]
        assert len(bad) == 0, f"launch {rep}: frames {bad[:8]} differ: trials gpu {t[bad[:8]]} oracle {to[bad[:8]]}"
    assert (to >= 0).sum() >= B // 2 and (to < 0).any()
