"""Frame-at-a-time receive chain and pool (rx_fec_chain / rx_fec_pool
semantics) against a model of the reference's chain built from the oracle:
the same micro-batches, the same decision-directed SNR updates every 32
frames, the oracle's demap -> decode -> BCH -> BB stage per micro-batch.
Output bytes, data-field sizes and frame/error counts must be identical."""
import ctypes

import numpy as np
import pytest

import cusat_gb300 as cs
import oracle_lib as O
from channel import awgn, es_normalised
from cusat_gb300 import enums as E

pytestmark = pytest.mark.gpu

NORMAL, SHORT = E.FECFRAME_NORMAL, E.FECFRAME_SHORT


def traffic(mod, rate, fs, n, esn0_db, seed):
    """n XFECFRAMEs of GSE BBFRAMEs: mostly good frames, every 7th sent 4 dB
    below esn0_db (LDPC failures), every 9th carrying a TS stream (no GSE
    output), every 11th with a broken BBHEADER."""
    rng = np.random.default_rng(seed)
    ci = cs.code_info(fs, rate)
    kbch = ci["k_bch"] // 8
    bb = np.zeros((n, kbch), np.uint8)
    for f in range(n):
        size = [1, kbch - 10, int(rng.integers(1, kbch - 10))][f % 3]
        bb[f] = O.bb_build(rng.integers(0, 256, size, dtype=np.uint8), kbch, ts_gs=3 if f % 9 == 4 else 0)
    bb[5::11, 3] ^= 0x40
    sym = es_normalised(cs.map_frames(mod, rate, fs, cs.encode_frames(fs, rate, bb)))
    out = np.zeros_like(sym)
    for f in range(n):
        out[f], _ = awgn(sym[f], esn0_db - (4.0 if f % 7 == 2 else 0.0), rng)
    return out


class OracleChain:
    """The reference's chain with an unlimited budget: frames accumulate into
    micro-batches, every 32nd submitted frame re-estimates the SNR, a full
    micro-batch is decoded with the chain's current noise variance and gain."""

    def __init__(self, mod, rate, fs, micro_batch, T):
        self.mod, self.rate, self.fs, self.mb, self.T = mod, rate, fs, micro_batch, T
        self.mi = O.modcod(mod, rate, fs)
        self.kbch = cs.code_info(fs, rate)["k_bch"] // 8
        self.noise_var, self.llr_gain = np.float32(1.0), np.float32(4.0)
        self.skip, self.pending, self.pilot = 0, [], 0.0
        self.out, self.dfl, self.frames, self.errors = [], [], 0, 0

    def start_from(self, chain, snr_db, skip=0):
        """The chain's SNR after update_snr(snr_db) (a pilot estimate) and its
        frame count since the last SNR update (warmup submits one frame)."""
        chain.update_snr(snr_db)
        self.noise_var, self.llr_gain = np.float32(chain.noise_var()), np.float32(chain.precision())
        self.skip = skip
        self.pilot = snr_db

    def submit(self, sym):
        self.skip += 1
        # 128 points and more with a pilot SNR above 5 dB take the pilot SNR
        # again (rx_fec_chain.cc:327-330): what update_snr already set
        pilot = self.mi["n_mod"] >= 7 and self.pilot > 5.0
        if self.skip >= 32:
            self.skip = 0
            lin = np.float32(0.0) if pilot else np.float32(
                O.dd_snr(sym, self.mi["points"].view(np.float32), 8, qpsk=self.mod == E.MOD_QPSK))
            if lin > 1:
                self.noise_var = np.float32(1.0) / lin
                self.llr_gain = min(np.float32(4.0) / self.noise_var, np.float32(1000.0))
        self.pending.append(sym)
        if len(self.pending) == self.mb:
            self.run()

    def run(self):
        if not self.pending:
            return
        noisy = np.stack(self.pending)
        self.pending = []
        mi = self.mi
        g = O.capped_llr_gain(mi, float(self.llr_gain))
        llr = O.demap(noisy, mi["xfecframe_len"], mi["interleaved_len"], mi["fecframe_len"], mi["n_mod"],
                      mi["kind"], mi["points"], mi["col_offset"], float(self.noise_var), g)
        hard, trials = O.ldpc_decode(self.fs, self.rate, llr, self.T)
        _, valid = O.bch_check(self.fs, self.rate, hard)
        out, lengths, _ = O.bb_extract(hard, self.kbch, trials, valid, len(noisy) * self.kbch)
        ok = (trials >= 0) & (valid != 0)
        self.frames += len(noisy)
        self.errors += int((~ok).sum())
        self.dfl += [int(v) for v, g in zip(lengths, ok) if g and v > 0]
        self.out.append(out)

    def output(self):
        return np.concatenate(self.out) if self.out else np.zeros(0, np.uint8)


def run_chain(chain, frames):
    """Submits every frame, collecting output whenever it is reported, then
    flushes; returns (bytes, data-field sizes)."""
    out, dfl = [], []
    for f in frames:
        if chain.submit_xfecframe(f):
            out.append(chain.get_gse_output())
            dfl += chain.gse_dfl_sizes()
    chain.flush()
    out.append(chain.get_gse_output())
    dfl += chain.gse_dfl_sizes()
    return np.concatenate(out), dfl


@pytest.mark.parametrize("name,fs,n,mb,streams,helpers", [("qpsk1/2", SHORT, 45, 4, 2, 0),
                                                          ("qpsk1/2", SHORT, 45, 4, 2, 2),
                                                          ("8psk3/5", SHORT, 40, 8, 3, 0),
                                                          ("8psk3/5", NORMAL, 36, 5, 4, 3),
                                                          ("16apsk2/3", SHORT, 40, 8, 2, 1),
                                                          ("128apsk3/4", NORMAL, 34, 6, 3, 1)])
def test_chain_matches_oracle(cuda, name, fs, n, mb, streams, helpers):
    _, mod, rate, _, _, thr = E.find_modcod(name)
    frames = traffic(mod, rate, fs, n, thr + 0.8, seed=n + mb)
    chain = cs.rx_fec_chain(fs, rate, mod, 50, 64, streams, mb)
    chain.set_decode_budget(cs.gpu_decode_budget(0))
    chain.set_copy_threads(helpers)           # frame copies split across helper threads (or not)
    ref = OracleChain(mod, rate, fs, mb, 50)
    ref.start_from(chain, thr + 0.8)
    out, dfl = run_chain(chain, frames)
    for f in frames:
        ref.submit(f)
    ref.run()
    assert chain.frame_count() == ref.frames == n
    assert chain.frame_error_count() == ref.errors and ref.errors >= n // 7
    assert dfl == ref.dfl and len(dfl) > n // 2
    assert out.size == ref.output().size and (out == ref.output()).all()
    assert chain.noise_var() == float(ref.noise_var) != 1.0   # one SNR update happened (128APSK: the pilot's)
    assert chain.gpu_inflight() == 0 and chain.pending_count() == 0 and chain.gpu_drop_count() == 0


def test_budget_defers_launches_and_keeps_order(cuda):
    """A budget of one micro-batch: launches wait for drains (or are forced
    by flush), the output is still the oracle's, the budget returns to 0."""
    _, mod, rate, _, _, thr = E.find_modcod("qpsk1/2")
    frames = traffic(mod, rate, SHORT, 30, thr + 0.8, seed=5)
    budget = cs.gpu_decode_budget(4)
    chain = cs.rx_fec_chain(SHORT, rate, mod, 50, 64, 4, 4)
    chain.set_decode_budget(budget)
    chain.set_block_when_full(True)
    ref = OracleChain(mod, rate, SHORT, 4, 50)
    ref.start_from(chain, thr + 0.8)
    out, dfl = run_chain(chain, frames)
    for f in frames:
        ref.submit(f)
    ref.run()
    assert (out == ref.output()).all() and dfl == ref.dfl
    assert budget.in_flight == 0 and budget.cap == 4
    assert chain.force_drain_count() > 0


def test_launch_lock_wraps_every_launch(cuda):
    _, mod, rate, _, _, thr = E.find_modcod("qpsk1/2")
    frames = traffic(mod, rate, SHORT, 10, thr + 1.0, seed=6)
    chain = cs.rx_fec_chain(SHORT, rate, mod, 50, 64, 2, 3)
    calls = {"lock": 0, "unlock": 0}
    CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p)
    lock = CB(lambda _: calls.__setitem__("lock", calls["lock"] + 1))
    unlock = CB(lambda _: calls.__setitem__("unlock", calls["unlock"] + 1))
    assert cs._capi.lib().cusat_rx_chain_set_launch_lock(chain._h, ctypes.cast(lock, ctypes.c_void_p),
                                                         ctypes.cast(unlock, ctypes.c_void_p), None) == 0
    run_chain(chain, frames)
    assert calls["lock"] == calls["unlock"] == 4        # ceil(10 / 3) micro-batches
    assert chain.frame_count() == 10


def test_drops_warmup_reset_and_snr(cuda):
    _, mod, rate, _, _, thr = E.find_modcod("8psk3/5")
    chain = cs.rx_fec_chain(SHORT, rate, mod, 50, 64, 2, 4)
    chain.warmup()
    assert chain.frame_count() == 0 and chain.gpu_drop_count() == 0 and chain.force_drain_count() == 0
    xfec = chain.xfecframe_len
    assert chain.submit_xfecframe(np.zeros(2 * (xfec - 1), np.float32)) is False   # wrong length: dropped
    assert (chain.frame_count(), chain.frame_error_count(), chain.gpu_drop_count()) == (1, 1, 1)
    chain.update_snr(10.0)
    assert abs(chain.noise_var() - 0.1) < 1e-6 and abs(chain.precision() - 40.0) < 1e-3
    assert chain.snr_db() == 10.0
    chain.update_snr(-3.0)                                  # ignored, like the reference
    assert chain.snr_db() == 10.0
    frames = traffic(mod, rate, SHORT, 6, thr + 1.0, seed=7)
    for f in frames:
        chain.submit_xfecframe(f)
    assert chain.pending_count() == 2
    chain.reset()
    assert (chain.frame_count(), chain.frame_error_count(), chain.pending_count(), chain.gpu_inflight()) == \
        (0, 0, 0, 0)
    assert chain.noise_var() == 1.0 and chain.precision() == 4.0


def test_pool_output_in_submission_order(cuda):
    """Two MODCODs in runs: each change flushes the previous chain, so the
    pool's output blocks, concatenated, are the oracle's in submission order;
    per-MODCOD counters follow."""
    A, B = 4, 12                                        # qpsk1/2, 8psk3/5
    pool = cs.rx_fec_pool(SHORT, [A, B], 50, 64, 2, 4)
    pool.warmup_all()
    models, frames = {}, {}
    for idx in (A, B):
        m = E.modcod_by_index(idx)
        frames[idx] = list(traffic(m[1], m[2], SHORT, 22, m[5] + 0.8, seed=idx))
        models[idx] = OracleChain(m[1], m[2], SHORT, 4, 50)
        models[idx].start_from(pool.chain(idx), m[5] + 0.8, skip=1)
    runs = [(A, 6), (B, 5), (A, 3), (B, 9), (A, 13), (B, 8)]
    out, dfl, expect_out, expect_dfl = [], [], [], []
    last = None
    for idx, k in runs:
        if last is not None and last != idx:
            models[last].run()
            expect_out.append(models[last].output())
            expect_dfl += models[last].dfl
            models[last].out, models[last].dfl = [], []
        for _ in range(k):
            f = frames[idx].pop(0)
            models[idx].submit(f)
            if pool.submit(f, idx):
                while True:
                    o = pool.get_gse_output()
                    if o.size == 0:
                        break
                    out.append(o)
                    dfl += pool.gse_dfl_sizes()
        last = idx
    pool.finish_all_pending()
    while True:
        o = pool.get_gse_output()
        if o.size == 0:
            break
        out.append(o)
        dfl += pool.gse_dfl_sizes()
    models[last].run()
    expect_out.append(models[last].output())
    expect_dfl += models[last].dfl
    got, want = np.concatenate(out), np.concatenate(expect_out)
    assert got.size == want.size and (got == want).all() and dfl == expect_dfl
    for idx in (A, B):
        assert pool.modcod_counters(idx) == (models[idx].frames, models[idx].errors)
    assert pool.modcod_counters(99) is None
    assert pool.total_frame_count() == 44
    assert pool.submit(np.zeros(2 * pool.chain(A).xfecframe_len, np.float32), 99) is False   # not enabled
    pool.reset_all()
    assert pool.total_frame_count() == 0


def _drain_pool(pool, out, dfl):
    while True:
        o = pool.get_gse_output()
        if o.size == 0:
            return
        out.append(o)
        dfl += pool.gse_dfl_sizes()


def _run_pool(pool, seq, warm=True):
    """Submits (frame, modcod) in order, collecting output as reported, then
    finishes; returns (bytes, data-field sizes)."""
    if warm:
        pool.warmup_all()
    out, dfl = [], []
    for f, m in seq:
        if pool.submit(f, m):
            _drain_pool(pool, out, dfl)
    pool.finish_all_pending()
    _drain_pool(pool, out, dfl)
    return (np.concatenate(out) if out else np.zeros(0, np.uint8)), dfl


@pytest.mark.parametrize("pattern", ["runs", "random"])
def test_mixed_pool_equals_per_modcod_pool(cuda, monkeypatch, pattern):
    """The mixed pool (one slot ring, multi-MODCOD launches, no wait at a
    MODCOD change) returns exactly the per-MODCOD pool's bytes, data-field
    sizes and counters -- SNR re-estimates included -- when the per-MODCOD
    pool's launches are not deferred by the in-flight cap."""
    monkeypatch.setenv("CUSAT_LDPC_INFLIGHT_CAP", "0")
    mods = [4, 12, 18]                                  # qpsk1/2, 8psk3/5, 16apsk2/3 (short)
    pools = {}
    frames = {}
    for idx in mods:
        mm = E.modcod_by_index(idx)
        frames[idx] = list(traffic(mm[1], mm[2], SHORT, 44, mm[5] + 0.8, seed=100 + idx))
    rng = np.random.default_rng(9)
    if pattern == "runs":
        order = [4] * 7 + [12] * 5 + [18] * 9 + [4] * 3 + [12] * 17 + [18] * 30 + [4] * 34 + [12] * 22 + [18] * 5
    else:
        order = list(rng.permutation([m for m in mods for _ in range(40)]))
    used = {m: 0 for m in mods}
    seq = []
    for m in order:
        seq.append((frames[m][used[m] % 44], int(m)))
        used[m] += 1
    per = cs.rx_fec_pool(SHORT, mods, 50, 64, 2, 4)
    mix = cs.rx_fec_pool(SHORT, mods, 50, 64, 2, 4, mixed=True, slot_frames=16)
    mix.set_copy_threads(2)
    for p in (per, mix):
        p.warmup_all()
        for idx in mods:
            p.update_snr(idx, E.modcod_by_index(idx)[5] + 0.8)
    out_p, dfl_p = _run_pool(per, seq, warm=False)
    out_m, dfl_m = _run_pool(mix, seq, warm=False)
    assert len(dfl_p) > len(seq) // 2
    assert out_m.size == out_p.size and (out_m == out_p).all() and dfl_m == dfl_p
    for idx in mods:
        assert mix.modcod_counters(idx) == per.modcod_counters(idx)
    assert mix.total_frame_count() == per.total_frame_count() == len(seq)
    assert mix.total_error_count() == per.total_error_count() > 0


def test_mixed_pool_with_128_and_256_points(cuda, monkeypatch):
    """Normal frames of 8PSK 3/5, 128APSK 3/4 (9270-symbol XFECFRAMEs, pilot
    SNR) and 256APSK 2/3 (coordinate-defined points) in random order: the
    mixed pool returns the per-MODCOD pool's bytes, sizes and counters."""
    monkeypatch.setenv("CUSAT_LDPC_INFLIGHT_CAP", "0")
    mods = [12, 32, 41]
    frames = {}
    for idx in mods:
        mm = E.modcod_by_index(idx)
        frames[idx] = list(traffic(mm[1], mm[2], NORMAL, 20, mm[5] + 0.8, seed=200 + idx))
    rng = np.random.default_rng(11)
    order = list(rng.permutation([m for m in mods for _ in range(20)]))
    used = {m: 0 for m in mods}
    seq = []
    for m in order:
        seq.append((frames[m][used[m]], int(m)))
        used[m] += 1
    per = cs.rx_fec_pool(NORMAL, mods, 50, 32, 2, 4)
    mix = cs.rx_fec_pool(NORMAL, mods, 50, 32, 2, 4, mixed=True, slot_frames=8)
    assert per.chain(32).xfecframe_len == 9270
    for p in (per, mix):
        p.warmup_all()
        for idx in mods:
            p.update_snr(idx, E.modcod_by_index(idx)[5] + 0.8)
    out_p, dfl_p = _run_pool(per, seq, warm=False)
    out_m, dfl_m = _run_pool(mix, seq, warm=False)
    assert len(dfl_p) > len(seq) // 2
    assert out_m.size == out_p.size and (out_m == out_p).all() and dfl_m == dfl_p
    for idx in mods:
        assert mix.modcod_counters(idx) == per.modcod_counters(idx)
    assert mix.total_error_count() == per.total_error_count() > 0


def test_mixed_pool_stale_launch_and_reset(cuda):
    pool = cs.rx_fec_pool(SHORT, [4, 12], 50, 64, 2, 4, mixed=True, slot_frames=32)
    pool.warmup_all()
    mm = E.modcod_by_index(4)
    pool.update_snr(4, mm[5] + 1.0)
    fr = traffic(mm[1], mm[2], SHORT, 3, mm[5] + 1.0, seed=3)   # frame 2 is sent 4 dB lower
    for f in fr:
        pool.submit(f, 4)
    assert pool.launch_stale(0.0) is True           # the open micro-batch and partial slot go
    import time
    for _ in range(2000):
        if pool.drain_all_completed():
            break
        time.sleep(0.001)
    assert pool.modcod_counters(4) == (3, 1)
    assert pool.chain(4) is None
    pool.reset_all()
    assert pool.total_frame_count() == 0


def test_mixed_pool_stale_slot_split(cuda):
    """A partial slot whose frames are stale but whose open micro-batch is
    fresh: launch_stale launches the closed frames now (the reference
    launched them at their MODCOD change or when full) and carries the open
    micro-batch into the next slot."""
    import time
    pool = cs.rx_fec_pool(SHORT, [4], 50, 64, 2, 4, mixed=True, slot_frames=64)
    pool.warmup_all()
    mm = E.modcod_by_index(4)
    pool.update_snr(4, mm[5] + 1.0)
    fr = traffic(mm[1], mm[2], SHORT, 6, mm[5] + 1.0, seed=8)   # frame 2 is sent 4 dB lower
    for f in fr[:4]:
        pool.submit(f, 4)                     # one full (closed) micro-batch in the partial slot
    time.sleep(0.3)
    pool.submit(fr[4], 4)                     # a new micro-batch opens
    assert pool.launch_stale(150.0) is True   # slot 300 ms old, open micro-batch fresh
    for _ in range(2000):
        pool.drain_all_completed()
        if pool.modcod_counters(4)[0] == 4:
            break
        time.sleep(0.001)
    assert pool.modcod_counters(4) == (4, 1)  # the closed four decoded, frame 4 still held
    pool.submit(fr[5], 4)
    pool.finish_all_pending()
    assert pool.modcod_counters(4) == (6, 1)
