"""Seeded serving traffic and trace replay for the serving loop.

A trace is a list of frame requests with arrival times: Poisson arrivals at
an aggregate symbol rate, each frame's MODCOD from a seeded ACM schedule
over a MODCOD set (a Markov chain: the link keeps its MODCOD with
probability `stay`, else moves to a random one), normal or short FECFRAMEs
(short only for short-capable MODCODs), each at its threshold + margin in
AWGN.  A frame occupies plframe_symbols = 90 + 90 S + 36 floor((S - 1) / 16)
symbols on the air with pilots, S = XFECFRAME symbols / 90 (the reference's
framing/plframe.cc:209-226).  The noisy symbols come from a pool generated
once per (MODCOD, frame size) and kept on the device; LLRs are produced on
the device by the batch's demap kernel.
"""
import numpy as np

from . import modcod_info, code_info, traffic
from .enums import FECFRAME_NORMAL, FECFRAME_SHORT, find_modcod


def plframe_symbols(xfec):
    s = xfec // 90
    return 90 + 90 * s + 36 * ((s - 1) // 16)


class TracePool:
    """Device-resident noisy frames for every (MODCOD, frame size) of a set."""

    def __init__(self, names, seed, per_entry, torch, short_share=0.3, margin_db=0.5):
        self.names = list(names)
        rng = np.random.default_rng(seed)
        self.table = []
        for name in self.names:
            self.table.append((name, FECFRAME_NORMAL))
            if short_share > 0 and name in traffic.SHORT_CAPABLE:
                self.table.append((name, FECFRAME_SHORT))
        self.short_share = short_share
        self.modcods, self.entries = [], []
        for name, fs in self.table:
            _, mod, rate, _, _, thr = find_modcod(name)
            msg, sym, n0, gain = traffic.modcod_frames(name, fs, per_entry, thr + margin_db, rng)
            mi = modcod_info(mod, rate, fs)
            ci = code_info(fs, rate)
            self.modcods.append((mod, rate, fs))
            self.entries.append({"sym": torch.from_numpy(sym).cuda(), "n0": n0, "gain": gain,
                                 "xfec": mi["xfecframe_len"], "k_ldpc": ci["k_ldpc"],
                                 "plsym": plframe_symbols(mi["xfecframe_len"])})
        self.index = {key: i for i, key in enumerate(self.table)}


def make_trace(pool, rate_sym_s, duration_s, seed, stay=0.9):
    """Arrival offsets (s), pool entry and pool frame of each request."""
    rng = np.random.default_rng(seed)
    names = pool.names
    cur = names[rng.integers(len(names))]
    t, out = 0.0, []
    while True:
        if rng.random() > stay:
            cur = names[rng.integers(len(names))]
        fs = FECFRAME_NORMAL
        if cur in traffic.SHORT_CAPABLE and rng.random() < pool.short_share:
            fs = FECFRAME_SHORT
        e = pool.index[(cur, fs)]
        # exponential gap with mean = this frame's air time at the aggregate rate
        t += rng.exponential(pool.entries[e]["plsym"] / rate_sym_s)
        if t > duration_s:
            break
        out.append((t, e, int(rng.integers(pool.entries[e]["sym"].shape[0]))))
    return out


# cusat_request as a numpy record (same layout as the C struct: 48 bytes)
REQUEST = np.dtype([("modcod", "<i4"), ("noise_var", "<f4"), ("llr_gain", "<f4"), ("flags", "<i4"),
                    ("sym", "<u8"), ("hard_host", "<u8"), ("tag", "<u8"), ("arrival_s", "<f8")])


def request_records(pool, trace, tag0=0, hard_host=None):
    """Records of a trace with arrival offsets (add the start time later)."""
    n = len(trace)
    rec = np.zeros(n, REQUEST)
    e = np.array([x[1] for x in trace], np.int64)
    f = np.array([x[2] for x in trace], np.int64)
    rec["modcod"] = e
    rec["noise_var"] = np.array([pool.entries[i]["n0"] for i in range(len(pool.entries))], np.float32)[e]
    rec["llr_gain"] = np.array([pool.entries[i]["gain"] for i in range(len(pool.entries))], np.float32)[e]
    base = np.array([pool.entries[i]["sym"].data_ptr() for i in range(len(pool.entries))], np.uint64)
    row = np.array([pool.entries[i]["sym"].shape[1] * 4 for i in range(len(pool.entries))], np.uint64)
    rec["sym"] = base[e] + row[e] * f.astype(np.uint64)
    if hard_host is not None:
        rec["hard_host"] = np.asarray(hard_host, np.uint64)
    rec["tag"] = tag0 + np.arange(n, dtype=np.uint64)
    rec["arrival_s"] = np.array([x[0] for x in trace], np.float64)
    return rec


def submit_records(srv, rec, lead_s):
    """Shifts the offsets to start lead_s from now (server clock) and submits."""
    import ctypes
    from . import _capi
    rec = rec.copy()
    rec["arrival_s"] += srv.now() + lead_s
    arr = (_capi.Request * len(rec)).from_buffer(rec)
    srv.submit(arr)
    return rec


def replay(srv, pool, trace, lead_s=0.02, timeout_s=120.0, hard_host=None):
    """Submits the whole trace (arrivals from now + lead_s) and collects the
    results.  Returns (results sorted by tag, stats)."""
    import time
    rec = request_records(pool, trace, hard_host=hard_host)
    keep = submit_records(srv, rec, lead_s)
    got = []
    deadline = time.time() + timeout_s
    while len(got) < len(trace):
        got += srv.poll(max_results=65536, wait_ms=20)
        if time.time() > deadline:
            raise TimeoutError(f"{len(got)} of {len(trace)} results after {timeout_s} s")
    del keep
    got.sort(key=lambda r: r.tag)
    return got, srv.stats()


def summarize(pool, trace, results):
    """Latency percentiles (ms), info throughput, iteration counts."""
    lat = np.array([r.done_s - r.arrival_s for r in results]) * 1e3
    wait = np.array([r.admit_s - r.arrival_s for r in results]) * 1e3
    bits = sum(pool.entries[e]["k_ldpc"] for _, e, _ in trace)
    span = max(r.done_s for r in results) - min(r.arrival_s for r in results)
    sym = sum(pool.entries[e]["plsym"] for _, e, _ in trace)
    return {"frames": len(results), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()), "queue_p99_ms": float(np.percentile(wait, 99)),
            "info_gbit_s": bits / span / 1e9, "offered_gsym_s": sym / trace[-1][0] / 1e9 if trace else 0.0,
            "failed": int(sum(r.trials < 0 for r in results)), "bch_bad": int(sum(r.bch_valid == 0 for r in results))}
