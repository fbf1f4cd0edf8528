"""Mixed-MODCOD batches: every frame's hard decisions, iteration count and BCH
flag equal those of a single-MODCOD rx_fec launch on the same symbols (which
the parity tests hold equal to the oracle); graph replay and the tuner do not
change results."""
import numpy as np
import pytest

import cusat_gb300 as cs
from cusat_gb300 import enums as E
from cusat_gb300 import traffic

import oracle_lib as O

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT
# six kernel classes (slots per layer x lanes); two pairs of MODCODs share a code
MIX = [("qpsk1/4", NORMAL, 5), ("qpsk1/2", SHORT, 9), ("8psk3/5", NORMAL, 7), ("8psk9/10", NORMAL, 4),
       ("16apsk2/3", NORMAL, 3), ("32apsk3/4", SHORT, 6), ("32apsk9/10", NORMAL, 2), ("64apsk32/45", NORMAL, 3),
       ("qpsk3/4", SHORT, 1)]


def _workload(seed=5):
    rng = np.random.default_rng(seed)
    per = []
    for name, fs, cnt in MIX:
        thr = E.find_modcod(name)[5]
        # the last frame of each MODCOD sits 3 dB below threshold (mostly fails)
        msg, sym, n0, gain = traffic.modcod_frames(name, fs, cnt, thr + 0.3, rng)
        if cnt > 1:
            _, low, n0l, gl = traffic.modcod_frames(name, fs, 1, thr - 3.0, rng)
            sym[-1] = low[0]
            n0s, gains = [n0] * (cnt - 1) + [n0l], [gain] * (cnt - 1) + [gl]
        else:
            n0s, gains = [n0], [gain]
        per.append((name, fs, sym, n0s, gains))
    return per


def _single(per, T, torch):
    out = []
    for name, fs, sym, n0s, gains in per:
        _, mod, rate, _, _, _ = E.find_modcod(name)
        rx = cs.rx_fec(mod, rate, fs, T, len(sym))
        hs, ts, vs = [], [], []
        for i in range(len(sym)):  # one launch per frame: per-frame N0 and gain
            d = torch.from_numpy(sym[i:i + 1]).cuda()
            h = torch.zeros((1, rx.k_bytes), dtype=torch.uint8, device="cuda")
            t = torch.zeros(1, dtype=torch.int32, device="cuda")
            v = torch.zeros(1, dtype=torch.int32, device="cuda")
            rx.launch(d, 1, n0s[i], gains[i], h, t, v, torch.cuda.current_stream())
            hs.append(h)
            ts.append(t)
            vs.append(v)
        torch.cuda.synchronize()
        out.append((torch.cat(hs).cpu().numpy(), torch.cat(ts).cpu().numpy(), torch.cat(vs).cpu().numpy()))
    return out


def _buffers(per, order, torch):
    """Device buffers per MODCOD and the frame list in `order` (pairs of
    MODCOD index, frame index)."""
    bufs = []
    for name, fs, sym, n0s, gains in per:
        _, mod, rate, _, _, _ = E.find_modcod(name)
        kb = cs.code_info(fs, rate)["k_ldpc"] // 8
        bufs.append((torch.from_numpy(sym).cuda(), torch.zeros((len(sym), kb), dtype=torch.uint8, device="cuda"),
                     torch.full((len(sym),), -7, dtype=torch.int32, device="cuda"),
                     torch.full((len(sym),), -7, dtype=torch.int32, device="cuda")))
    cols = [[] for _ in range(7)]
    for m, i in order:
        d, h, t, v = bufs[m]
        cols[0].append(m)
        cols[1].append(per[m][3][i])
        cols[2].append(per[m][4][i])
        cols[3].append(d[i].data_ptr())
        cols[4].append(h[i].data_ptr())
        cols[5].append(t[i].data_ptr())
        cols[6].append(v[i].data_ptr())
    torch.cuda.synchronize()
    return bufs, cs.batch.frames(*cols)


def _check(bufs, ref):
    for (d, h, t, v), (hr, tr, vr) in zip(bufs, ref):
        assert (t.cpu().numpy() == tr).all()
        assert (h.cpu().numpy() == hr).all()
        assert (v.cpu().numpy() == vr).all()


def _modcod_triples(per):
    out = []
    for name, fs, *_ in per:
        _, mod, rate, _, _, _ = E.find_modcod(name)
        out.append((mod, rate, fs))
    return out


@pytest.fixture(scope="module")
def mixed(cuda):
    torch = cuda
    per = _workload()
    T = 30
    ref = _single(per, T, torch)
    rng = np.random.default_rng(9)
    order = [(m, i) for m, p in enumerate(per) for i in range(len(p[2]))]
    order = [order[k] for k in rng.permutation(len(order))]
    return torch, per, T, ref, order


def test_reference_results_are_oracle_results(mixed):
    """The single-MODCOD results used as reference agree with the oracle for
    one MODCOD of each frame size (the parity suite covers the rest)."""
    torch, per, T, ref, _ = mixed
    from test_gpu_parity import oracle_llr
    for k in (1, 2):
        name, fs, sym, n0s, gains = per[k]
        _, mod, rate, _, _, _ = E.find_modcod(name)
        llr = np.concatenate([oracle_llr(mod, rate, fs, sym[i:i + 1], n0s[i], gains[i])
                              for i in range(len(sym))])
        ho, to = O.ldpc_decode(fs, rate, llr, T, nthreads=16)
        assert (ref[k][1] == to).all() and (ref[k][0] == ho).all()
        assert (ref[k][2] == O.bch_check(fs, rate, ho)[1]).all()
        assert (to == -1).any() and (to > 0).any()


def test_mixed_batch_equals_single_modcod(mixed):
    torch, per, T, ref, order = mixed
    b = cs.batch(_modcod_triples(per), max_trials=T, max_frames=64)
    n_modcods, n_classes, max_frames, max_trials = b.info()
    assert (n_modcods, max_frames, max_trials) == (len(per), 64, T)
    # one class per kernel instantiation (circulant-slot bucket, lanes)
    assert n_classes == len({(cs.code_info(fs, rate)["cmax"], cs.code_info(fs, rate)["lanes"])
                             for _, rate, fs in _modcod_triples(per)})
    bufs, frames = _buffers(per, order, torch)
    b.launch(frames, torch.cuda.current_stream())
    torch.cuda.synchronize()
    _check(bufs, ref)


def test_mixed_batch_repeat_and_subsets(mixed):
    """Two launches in a row on the same object, then a one-frame batch and a
    batch of a single MODCOD."""
    torch, per, T, ref, order = mixed
    b = cs.batch(_modcod_triples(per), max_trials=T, max_frames=64)
    for _ in range(2):
        bufs, frames = _buffers(per, order, torch)
        b.launch(frames, torch.cuda.current_stream())
        torch.cuda.synchronize()
        _check(bufs, ref)
    bufs, frames = _buffers(per, [(4, 0)], torch)
    b.launch(frames, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert (bufs[4][2][0].item(), bufs[4][3][0].item()) == (ref[4][1][0], ref[4][2][0])
    assert (bufs[4][1][0].cpu().numpy() == ref[4][0][0]).all()
    bufs, frames = _buffers(per, [(2, i) for i in range(len(per[2][2]))], torch)
    b.launch(frames, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert (bufs[2][2].cpu().numpy() == ref[2][1]).all()
    assert (bufs[2][1].cpu().numpy() == ref[2][0]).all()


def test_graph_replay_and_tuner(mixed):
    torch, per, T, ref, order = mixed
    b = cs.batch(_modcod_triples(per), max_trials=T, max_frames=64)
    s = torch.cuda.Stream()
    bufs, frames = _buffers(per, order, torch)
    best = b.tune(frames, reps=2, stream=s)
    assert best > 0
    torch.cuda.synchronize()
    _check(bufs, ref)
    # the tuned configuration: every class with frames has a grid of 1 ..
    # frames CTAs, a launch position, and a measured solo time
    tuned = b.tuned()
    assert len(tuned) == b.info()[1]
    used = [c for c in tuned if c["frames"] > 0]
    assert used and all(1 <= c["ctas"] <= c["frames"] and c["solo_ms"] > 0 for c in used)
    assert sorted(c["order"] for c in tuned) == list(range(len(tuned)))
    bufs, frames = _buffers(per, order, torch)
    b.capture(frames, s)
    # a launch with other frames between capture and replay leaves the graph intact
    other, oframes = _buffers(per, [(0, 0), (5, 1)], torch)
    b.launch(oframes, s)
    for _ in range(2):
        for d, h, t, v in bufs:
            h.zero_()
            t.fill_(-7)
            v.fill_(-7)
        torch.cuda.synchronize()
        b.replay(s)
        s.synchronize()
        _check(bufs, ref)
    assert other[0][2][0].item() == ref[0][1][0] and other[5][2][1].item() == ref[5][1][1]


def test_batch_rejects_bad_frames(mixed):
    torch, per, T, ref, order = mixed
    b = cs.batch(_modcod_triples(per)[:2], max_trials=T, max_frames=4)
    bufs, frames = _buffers(per, order[:5], torch)
    with pytest.raises(cs.CusatError):
        b.launch(frames)  # five frames, max_frames 4
    _, frames = _buffers(per, [(3, 0)], torch)
    with pytest.raises(cs.CusatError):
        b.launch(frames)  # MODCOD index 3 not in this batch
    with pytest.raises(cs.CusatError):
        b.replay(torch.cuda.current_stream())  # nothing captured
    with pytest.raises(cs.CusatError):
        cs.batch([(E.MOD_QPSK, E.RATE_1_2, 7)])


def test_single_code_objects_created_later_leave_the_batch_launchable(mixed):
    """A single-MODCOD object of the same kernel class needs less shared
    memory than the batch; creating one after the batch must not lower what
    the batch may launch with."""
    torch, per, T, ref, order = mixed
    b = cs.batch(_modcod_triples(per), max_trials=T, max_frames=64)
    keep = [cs.rx_fec(mod, rate, fs, T, 1) for mod, rate, fs in _modcod_triples(per)]
    keep += [cs.ldpc_decode_cuda(fs, rate, T, 1) for _, rate, fs in _modcod_triples(per)]
    bufs, frames = _buffers(per, order, torch)
    b.launch(frames, torch.cuda.current_stream())
    torch.cuda.synchronize()
    _check(bufs, ref)


def test_mixed_batch_with_128_and_256_points(cuda):
    """128APSK (9258 of 9270 symbols carry bits, 6 stuffing bits) and the
    ring and coordinate 256APSK constellations in one mixed batch with 8PSK:
    per frame the same results as single-MODCOD launches."""
    torch = cuda
    rng = np.random.default_rng(17)
    per = []
    for name, cnt in [("128apsk3/4", 3), ("256apsk32/45", 2), ("256apsk2/3", 2), ("8psk3/5", 2)]:
        thr = E.find_modcod(name)[5]
        msg, sym, n0, gain = traffic.modcod_frames(name, NORMAL, cnt, thr + 0.5, rng)
        per.append((name, NORMAL, sym, [n0] * cnt, [gain] * cnt))
    T = 30
    ref = _single(per, T, torch)
    assert all((r[1] >= 0).any() for r in ref)
    order = [(m, i) for m, p in enumerate(per) for i in range(len(p[2]))]
    order = [order[k] for k in rng.permutation(len(order))]
    b = cs.batch(_modcod_triples(per), max_trials=T, max_frames=16)
    bufs, frames = _buffers(per, order, torch)
    b.launch(frames, torch.cuda.current_stream())
    torch.cuda.synchronize()
    _check(bufs, ref)
