"""Serving loop: every frame's hard decisions, iteration count and BCH flag
are identical whether it is decoded alone (a one-frame rx_fec launch) or
admitted into mixed batches next to other requests, and equal to the
oracle's demap -> decode -> BCH check of that frame; the HBM budget bounds
the in-flight bytes; per-MODCOD learned weights apply."""
import ctypes

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from cusat_gb300 import enums as E
from cusat_gb300 import serving

pytestmark = pytest.mark.gpu

NAMES = ["qpsk1/4", "qpsk1/2", "8psk3/5", "16apsk2/3", "32apsk3/4", "64apsk32/45"]


@pytest.fixture(scope="module")
def pool(cuda):
    return serving.TracePool(NAMES, seed=12, per_entry=3, torch=cuda)


def alone(torch, pool, e, f, T, weights=None):
    mod, rate, fs = pool.modcods[e]
    ent = pool.entries[e]
    rx = cs.rx_fec(mod, rate, fs, T, 1)
    rx.set_weights(weights)
    h = torch.zeros((1, rx.k_bytes), dtype=torch.uint8, device="cuda")
    t = torch.zeros(1, dtype=torch.int32, device="cuda")
    v = torch.zeros(1, dtype=torch.int32, device="cuda")
    rx.launch(ent["sym"][f:f + 1], 1, ent["n0"], ent["gain"], h, t, v, torch.cuda.current_stream())
    torch.cuda.synchronize()
    return h.cpu().numpy()[0], int(t.item()), int(v.item())


def oracle(pool, e, f, T):
    """The oracle's chain on frame f of entry e (its own demap parameters)."""
    mod, rate, fs = pool.modcods[e]
    ent = pool.entries[e]
    sym = ent["sym"][f:f + 1].cpu().numpy()
    llr = O.demap_modcod(sym, O.modcod(mod, rate, fs), ent["n0"], ent["gain"])
    hard, trials = O.ldpc_decode(fs, rate, llr, T)
    _, valid = O.bch_check(fs, rate, hard)
    return hard[0], int(trials[0]), int(valid[0] != 0)


def run(srv, pool, trace, lead_s=0.02):
    hard = [np.zeros(pool.entries[e]["k_ldpc"] // 8, np.uint8) for _, e, _ in trace]
    t0 = srv.now() + lead_s
    cols = ([], [], [], [], [], [])
    for k, (t, e, f) in enumerate(trace):
        ent = pool.entries[e]
        for c, v in zip(cols, [e, ent["n0"], ent["gain"], ent["sym"][f].data_ptr(), k, t0 + t]):
            c.append(v)
    srv.submit(srv.requests(*cols, hard_host=[h.ctypes.data for h in hard]))
    got = []
    while len(got) < len(trace):
        got += srv.poll(wait_ms=50)
    got.sort(key=lambda r: r.tag)
    return got, hard


def test_results_identical_alone_and_in_mix(cuda, pool):
    torch = cuda
    T = 30
    srv = cs.server(pool.modcods, max_trials=T, hbm_budget=256 << 20, slots=3, max_batch=48)
    # a burst far above capacity: frames queue and are batched together
    trace = serving.make_trace(pool, rate_sym_s=50e9, duration_s=0.0004, seed=3, stay=0.5)
    assert len(trace) > 60
    got, hard = run(srv, pool, trace)
    st = srv.stats()
    assert st["frames"] == len(trace) and st["largest_batch"] > 1 and st["batches"] < len(trace)
    assert st["max_inflight_batches"] >= 2
    ref = {}
    for r, (t, e, f), h in zip(got, trace, hard):
        assert r.arrival_s <= r.admit_s <= r.done_s
        if (e, f) not in ref:
            ref[(e, f)] = alone(torch, pool, e, f, T)
        hr, tr, vr = ref[(e, f)]
        assert (r.trials, r.bch_valid) == (tr, vr)
        assert (h == hr).all()
    # spread arrivals (light load): same results
    trace2 = serving.make_trace(pool, rate_sym_s=0.2e9, duration_s=0.01, seed=4)
    got2, hard2 = run(srv, pool, trace2)
    for r, (t, e, f), h in zip(got2, trace2, hard2):
        if (e, f) not in ref:
            ref[(e, f)] = alone(torch, pool, e, f, T)
        hr, tr, vr = ref[(e, f)]
        assert (r.trials, r.bch_valid) == (tr, vr) and (h == hr).all()
    # and each distinct frame as the oracle decodes it
    for (e, f), (hr, tr, vr) in ref.items():
        ho, to, vo = oracle(pool, e, f, T)
        assert (tr, int(vr != 0)) == (to, vo) and (hr == ho).all(), f"entry {e} frame {f} differs from the oracle"
    srv.close()


def test_budget_bounds_inflight_bytes(cuda, pool):
    # room for about two normal QPSK frames (symbols 259 KB each + results)
    budget = 600 << 10
    srv = cs.server(pool.modcods, max_trials=20, hbm_budget=budget, slots=4, max_batch=64)
    trace = serving.make_trace(pool, rate_sym_s=50e9, duration_s=0.0003, seed=5)
    got, _ = run(srv, pool, trace)
    st = srv.stats()
    assert len(got) == len(trace)
    assert 0 < st["peak_bytes"] <= budget
    srv.close()


def test_rejections(cuda, pool):
    with pytest.raises(cs.CusatError):
        cs.server(pool.modcods, hbm_budget=100 << 10)  # smaller than one normal frame
    srv = cs.server(pool.modcods, hbm_budget=64 << 20, slots=1, max_batch=8)
    bad = srv.requests([len(pool.modcods)], [1.0], [1.0], [pool.entries[0]["sym"][0].data_ptr()], [0])
    with pytest.raises(cs.CusatError):
        srv.submit(bad)
    srv.close()


def test_learned_weights_per_modcod(cuda, pool):
    torch = cuda
    T = 20
    rng = np.random.default_rng(2)
    w = np.zeros((T, 32, 2), np.int16)
    w[:, :, 0] = rng.integers(0, 3, (T, 32))
    w[:, :, 1] = rng.integers(48, 80, (T, 32))
    srv = cs.server(pool.modcods, max_trials=T, hbm_budget=128 << 20, slots=2, max_batch=32)
    learned_entry = pool.index[("8psk3/5", E.FECFRAME_NORMAL)]
    srv.set_weights(learned_entry, w)  # 8PSK 3/5 normal learned, the rest plain
    trace = serving.make_trace(pool, rate_sym_s=30e9, duration_s=0.0004, seed=6, stay=0.3)
    got, hard = run(srv, pool, trace)
    ref = {}
    for r, (t, e, f), h in zip(got, trace, hard):
        if (e, f) not in ref:
            ref[(e, f)] = alone(torch, pool, e, f, T, w if e == learned_entry else None)
        hr, tr, vr = ref[(e, f)]
        assert (r.trials, r.bch_valid) == (tr, vr) and (h == hr).all()
    assert any(e == learned_entry for e, _ in ref)
    srv.close()


def test_host_symbols(cuda, pool):
    """Requests whose symbols are in host memory (CUSAT_REQ_HOST_SYMBOLS) are
    copied in at admission and decode like device-resident ones."""
    torch = cuda
    T = 25
    srv = cs.server(pool.modcods, max_trials=T, hbm_budget=64 << 20, slots=2, max_batch=16)
    picks = [(e, f) for e in range(len(pool.modcods)) for f in range(2)]
    host = [np.ascontiguousarray(pool.entries[e]["sym"][f].cpu().numpy()) for e, f in picks]
    hard = [np.zeros(pool.entries[e]["k_ldpc"] // 8, np.uint8) for e, _ in picks]
    reqs = srv.requests([e for e, _ in picks], [pool.entries[e]["n0"] for e, _ in picks],
                        [pool.entries[e]["gain"] for e, _ in picks], [h.ctypes.data for h in host],
                        list(range(len(picks))), hard_host=[h.ctypes.data for h in hard], flags=cs.server.HOST_SYMBOLS)
    srv.submit(reqs)
    got = []
    while len(got) < len(picks):
        got += srv.poll(wait_ms=50)
    got.sort(key=lambda r: r.tag)
    for r, (e, f), h in zip(got, picks, hard):
        hr, tr, vr = alone(torch, pool, e, f, T)
        assert (r.trials, r.bch_valid) == (tr, vr) and (h == hr).all()
    srv.close()


def test_concurrent_submitters(cuda, pool):
    """Three host threads submit interleaved traces at once; every request
    comes back exactly once with the result it has alone."""
    import threading
    torch = cuda
    T = 25
    srv = cs.server(pool.modcods, max_trials=T, hbm_budget=128 << 20, slots=3, max_batch=32)
    traces = [serving.make_trace(pool, 20e9, 0.0002, seed=40 + k) for k in range(3)]
    errors = []

    def submit(k):
        try:
            rec = serving.request_records(pool, traces[k], tag0=100000 * k)
            serving.submit_records(srv, rec, lead_s=0.005)
        except Exception as e:  # reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=submit, args=(k,)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    total = sum(len(t) for t in traces)
    got = []
    while len(got) < total:
        got += srv.poll(wait_ms=50)
    assert len({r.tag for r in got}) == total
    ref = {}
    for r in got:
        k, i = divmod(r.tag, 100000)
        _, e, f = traces[k][i]
        if (e, f) not in ref:
            ref[(e, f)] = alone(torch, pool, e, f, T)
        assert (r.trials, r.bch_valid) == ref[(e, f)][1:]
    srv.close()


def test_destroy_with_work_in_flight(cuda, pool):
    """Closing a server with requests queued and batches on the GPU returns
    promptly and leaves the device usable."""
    import time
    torch = cuda
    srv = cs.server(pool.modcods, max_trials=50, hbm_budget=64 << 20, slots=2, max_batch=64)
    serving.submit_records(srv, serving.request_records(pool, serving.make_trace(pool, 50e9, 0.002, seed=9)),
                           lead_s=0.0)
    time.sleep(0.005)
    t0 = time.time()
    srv.close()
    assert time.time() - t0 < 10.0
    x = torch.ones(4, device="cuda")
    assert float((x * 2).sum().item()) == 8.0
