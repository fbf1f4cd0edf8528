"""Benchmark of the receive-side FEC path on GB300.

Workload (headline): normal FECFRAME 3/5 (s2_b5), 8PSK with interleave
"210", 256 frames per step at Es/N0 6.0 dB (seeded synthetic traffic from
this project's BCH/LDPC encoder, mapper and AWGN channel), soft demap
+ deinterleave -> layered min-sum LDPC decode (max 50 iterations, syndrome
early exit) -> BCH syndrome check.  One step = one batch through the chain.

  value     decoded information Gbit/s (frames x k_ldpc / time), symbols
            already in HBM; inputs cycle over 4 batches (> L2) so no step
            reads its symbols from L2
  e2e       the same through the public API with the step's symbols copied
            from pinned host memory and hard bits, iteration counts and BCH
            flags copied back inside the timed region
  roofline  HBM bytes of the chain (symbols in, hard bits + counters out)
            per launch / launch time, against the measured copy bandwidth
  cpu_baseline  the oracle (C restatement of the reference's algorithm;
            the reference has no CPU decoder) on the host cores, on a
            sample of the same frames

--impl reference times that CPU implementation alone on all host cores
(rank 0 only) and prints the same JSON line with "impl": "reference".

--workload mixed: 1024 frames per step drawn by seed from 10 MODCODs (70%
normal, 30% short FECFRAMEs, each at its threshold + 0.5 dB), decoded by the
mixed-MODCOD batch API as one tuned CUDA graph replay per step; the JSON line
adds per-MODCOD iteration and failure counts and the replay latency.

Multi-GPU: frames are independent and nothing is exchanged; N ranks run N
replicas of the workload on their own GPU and `value` is the frames of all
ranks over the slowest rank's time (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# The mixed batch and the serving loop launch every decoder class on its own
# stream (up to 4 slots x 14 classes in flight); with CUDA's default 8
# hardware queues those streams share queues and serialise (serving p99 at
# 5 Gsym/s: 4.2 ms with 8 queues, 2.9 ms with 32).  Takes effect only before
# the CUDA context exists; a value already set is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "LDPC decode info Gbit/s at equal FER (plain vs learned MS); p99 frame latency"
WORKLOAD = {"name": "normal 3/5 8PSK", "code": "s2_b5", "mod_name": "8PSK", "fs": 0, "rate": 4, "mod": 1,
            "frames": 256, "esn0_db": 6.0, "max_trials": 50, "seed": 2024}
# short FECFRAME 1/2 QPSK, 64 frames at 1.5 dB (the reference's CPU-runnable case)
WORKLOAD_SHORT = {"name": "short 1/2 QPSK", "code": "s2_c4", "mod_name": "QPSK", "fs": 1, "rate": 3, "mod": 0,
                  "frames": 64, "esn0_db": 1.5, "max_trials": 50, "seed": 2025}
N_BUFS = 4          # input batches cycled through (at least; more when a batch is small)
L2_BYTES = 160e6    # cycled inputs exceed this (GB300 L2: 129 MB)
PIPE = 2            # chains (streams) whose consecutive batches overlap, at least
RESIDENT_CTAS = 456 # resident decoder CTAs on a GB300 (152 SMs x 3 for short QPSK 1/2 frames)


class ProductGen:
    """Traffic generation with this project's encoder and mapper (GPU arm)."""

    def __init__(self):
        import cusat_gb300 as cs
        self.cs = cs

    def code_info(self, fs, rate):
        return self.cs.code_info(fs, rate)

    def encode(self, fs, rate, msg):
        return self.cs.encode_frames(fs, rate, msg)

    def map(self, mod, rate, fs, cw):
        return self.cs.map_frames(mod, rate, fs, cw)

    def modcod_info(self, mod, rate, fs):
        return self.cs.modcod_info(mod, rate, fs)


class OracleGen:
    """The same traffic from the oracle's BCH/LDPC encoder and mapper (the
    reference arm loads no library of this project); bit-identical to
    ProductGen's output (tests/test_bench_host.py)."""

    def __init__(self):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib as O
        self.O = O

    def code_info(self, fs, rate):
        ci = self.O.code_info(fs, rate)
        return {"k_bch": ci["k_bch"], "n_bch": ci["n_bch"], "k_ldpc": ci["K"], "n_ldpc": ci["N"],
                "edges": ci["links_total"]}

    def encode(self, fs, rate, msg):
        return self.O.ldpc_encode(fs, rate, self.O.bch_encode(fs, rate, msg))

    def map(self, mod, rate, fs, cw):
        mi = self.O.modcod(mod, rate, fs)
        qpsk = mi["kind"] == 0
        col = np.arange(8, dtype=np.uint32) if qpsk else mi["col_offset"]
        return self.O.map_symbols(cw, mi["xfecframe_len"], mi["n_mod"], col, 2 if qpsk else 1, mi["points"],
                                  mi["interleaved_len"], mi["fecframe_len"])

    def modcod_info(self, mod, rate, fs):
        return self.O.modcod(mod, rate, fs)


def n_bufs_for(wl, gen):
    """Batches to cycle through so that the inputs exceed the L2."""
    mi = gen.modcod_info(wl["mod"], wl["rate"], wl["fs"])
    batch_bytes = wl["frames"] * mi["xfecframe_len"] * 8
    return max(N_BUFS, int(np.ceil(L2_BYTES / batch_bytes)))


def frames_per_cta_for(ci, pipe, B, sms):
    """Frames per CTA for `pipe` chains of B-frame batches: the library's
    default looks at one launch; with the chains' batches in flight the
    short codes of at most 5 slots take frame pairs once the frames in
    flight give every SM two."""
    return 2 if ci["cmax"] <= 5 and pipe * B >= 2 * sms else 0


def single_config(wl, nb, batch_bytes):
    """The workload's config dict, the same in both arms (nothing measured)."""
    return {"workload": f"{wl['name']} ({wl['code']}), {wl['frames']} frames, Es/N0 {wl['esn0_db']} dB: demap + "
                        f"deinterleave -> layered min-sum LDPC (max {wl['max_trials']} it) -> BCH check",
            "frames": wl["frames"], "max_trials": wl["max_trials"], "esn0_db": wl["esn0_db"], "seed": wl["seed"],
            "decoder": "plain offset min-sum",
            "l2": f"inputs cycled over {nb} batches ({nb * batch_bytes / 1e6:.0f} MB > L2)"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-sample", type=int, default=0, help="frames in the CPU sample (0 = auto)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="wall time of the CPU baseline sample")
    ap.add_argument("--workload", choices=["single", "short", "mixed", "serve", "learned", "codes", "chain", "acm",
                                           "pl"],
                    default="single",
                    help="single: the headline 8PSK 3/5 batch; short: 64 short QPSK 1/2 frames; mixed: 1024 frames of 10 MODCODs in a CUDA graph; "
                         "serve: Poisson arrivals through the serving loop; learned: plain (max 50 it) vs "
                         "learned (max 20 it) min-sum on normal QPSK 1/3 at its threshold")
    ap.add_argument("--rates", default="0.5,1,2,3,4,5", help="serve: aggregate Gsym/s to sweep")
    ap.add_argument("--duration", type=float, default=0.25, help="serve: seconds of traffic per rate")
    ap.add_argument("--pipe", type=int, default=0,
                    help="single/short: chains whose consecutive batches overlap (0 = enough to fill the resident CTA slots, at least 2)")
    ap.add_argument("--demap-modcods", default="",
                    help="codes: comma-separated MODCOD names for the demapper table (default: one per family)")
    ap.add_argument("--learned", action="store_true",
                    help="mixed/serve: decode each MODCOD with its adopted learned weights where one exists")
    ap.add_argument("--no-extra", dest="extra", action="store_false",
                    help="single, N=1: skip the other configurations' runs summarised under \"workloads\"")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def make_traffic(wl, n_bufs, gen=None):
    """n_bufs noisy batches of the workload (same codewords, fresh noise),
    encoded and mapped by gen (ProductGen by default)."""
    gen = gen or ProductGen()
    rng = np.random.default_rng(wl["seed"])
    ci = gen.code_info(wl["fs"], wl["rate"])
    msg = rng.integers(0, 256, (wl["frames"], ci["k_bch"] // 8), dtype=np.uint8)
    cw = gen.encode(wl["fs"], wl["rate"], msg)
    sym = gen.map(wl["mod"], wl["rate"], wl["fs"], cw)
    es = float(np.mean(sym.astype(np.float64) ** 2) * 2)
    sym = (sym / np.float32(np.sqrt(es))).astype(np.float32)
    n0 = np.float32(1.0 / 10 ** (wl["esn0_db"] / 10.0))
    sigma = np.float32(np.sqrt(n0 / np.float32(2.0)))
    bufs = [(sym + sigma * rng.standard_normal(sym.shape, dtype=np.float32)).astype(np.float32)
            for _ in range(n_bufs)]
    return ci, msg, bufs, float(n0), min(4.0 / float(n0), 1000.0)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_chain(wl, bufs, n0, gain, n_frames, threads):
    """Oracle demap + decode + BCH check of the first n_frames of batch 0
    (demap parameters and gain cap from the oracle's own restatement)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    mi = O.modcod(wl["mod"], wl["rate"], wl["fs"])
    sym = bufs[0][:n_frames]
    t0 = time.perf_counter()
    llr = O.demap_modcod(sym, mi, n0, gain)
    hard, trials = O.ldpc_decode(wl["fs"], wl["rate"], llr, wl["max_trials"], nthreads=threads)
    O.bch_check(wl["fs"], wl["rate"], hard)
    return time.perf_counter() - t0, trials


def cpu_sample(wl, bufs, n0, gain, threads, seconds):
    """Oracle chain over the workload's batches (cycled) until `seconds` of
    wall time have passed; returns (seconds, frames)."""
    total, frames, k = 0.0, 0, 0
    while total < seconds:
        dt, _ = cpu_chain(wl, [bufs[k % len(bufs)]], n0, gain, wl["frames"], threads)
        total += dt
        frames += wl["frames"]
        k += 1
    return total, frames


def reference_arm(args, wl):
    """The reference's algorithm on the host cores: the oracle (the reference
    ships no CPU decoder), fed by the oracle's own encoder and mapper -- no
    library of this project is loaded in this arm."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    gen = OracleGen()
    nb = n_bufs_for(wl, gen)
    ci, msg, bufs, n0, gain = make_traffic(wl, 1, gen)
    threads = os.cpu_count() or 1
    n = args.cpu_sample or wl["frames"]
    for _ in range(args.warmup):
        cpu_chain(wl, bufs, n0, gain, min(n, 4), threads)
    total = 0.0
    for _ in range(args.steps):
        dt, _ = cpu_chain(wl, bufs, n0, gain, n, threads)
        total += dt
    value = args.steps * n * ci["k_ldpc"] / total / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gbit/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
            "data": f"synthetic (seeded BCH/LDPC-encoded {wl['mod_name']} frames, AWGN at Es/N0 {wl['esn0_db']} dB)",
            "config": single_config(wl, nb, bufs[0].nbytes),
            "cpu_baseline": {"value": value, "unit": "Gbit/s", "cores": threads, "kind": "port",
                             "sample": f"{n} frames of the workload's first batch per step, demap + decode + BCH "
                                       f"(the reference ships no CPU decoder: C restatement of its algorithm)"},
            "e2e": {"value": value, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if wl is WORKLOAD or wl["name"] == WORKLOAD["name"]:
        line["reference_gpu_kernels"] = reference_gpu_leg(args, wl, gen, nb)
    print(json.dumps(line), flush=True)


def reference_gpu_leg(args, wl, gen, nb):
    """The reference's own demap and decoder kernels (compiled unchanged into
    oracle/_ref cubins, launched by oracle/ref_gpu.c as its host classes launch
    them) on the workload's batches from the oracle's encoder and mapper: one
    demap + decode per batch on one stream, inputs cycled over batches larger
    than the L2, CUDA events.  Loads no library of this project.  Reported
    beside the CPU line, not as its value; {"unavailable": why} where the
    cubins or a GPU are missing."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device"}
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib as O
        rg = O.RefGpu()
        mi = O.modcod(wl["mod"], wl["rate"], wl["fs"])
        ci, _, bufs, n0, gain = make_traffic(wl, nb, gen)
        B, T = wl["frames"], wl["max_trials"]
        g = O.capped_llr_gain(mi, gain)
        pts = mi["points"]
        d_re = torch.from_numpy(np.ascontiguousarray(pts.real, np.float32)).cuda()
        d_im = torch.from_numpy(np.ascontiguousarray(pts.imag, np.float32)).cuda()
        d_sym = [torch.from_numpy(b).cuda() for b in bufs]
        llr = torch.zeros((B, mi["fecframe_len"]), dtype=torch.int16, device="cuda")
        hard = torch.zeros((B, ci["k_ldpc"] // 8), dtype=torch.uint8, device="cuda")
        res = torch.zeros(B, dtype=torch.int32, device="cuda")
        dec = rg.decoder(wl["fs"], wl["rate"], T, B)
        s = torch.cuda.current_stream()

        def step(i):
            rg.demap(d_sym[i % nb], llr, d_re, d_im, mi, n0, g, B, s)
            dec.launch(llr, B, hard, res, s)

        for i in range(args.warmup):
            step(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for i in range(args.steps):
            step(i)
        e1.record(s)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        tr = res.cpu().numpy()
        dec.close()
        return {"value": B * ci["k_ldpc"] / (ms * 1e6), "unit": "Gbit/s", "ms_per_step": ms,
                "frames_failed": int((tr < 0).sum()), "steps": args.steps, "warmup": args.warmup,
                "kind": "the reference's demapper_kernel.cu and ldpc_decode_kernel.cu compiled unchanged "
                        "(sm_103 cubins), one demap + decode launch per batch on one stream, no BCH"}
    except Exception as e:  # the CPU line stands without it
        return {"unavailable": f"{type(e).__name__}: {e}"[:300]}


# The other configurations, run after the headline's timed region as
# separate processes of this script (each with its own warm-up, CUDA-event
# timing and clock record) and summarised in the headline line, so that one
# default run records every configuration.
EXTRA_WORKLOADS = [
    ("C1", ["--workload", "short"]),
    ("C3", ["--workload", "mixed"]),
    ("C4", ["--workload", "learned"]),
    ("C5", ["--workload", "serve", "--rates", "3,4", "--duration", "0.25"]),
]


def extra_workloads(args):
    out = {}
    for key, extra in EXTRA_WORKLOADS:
        cmd = [sys.executable, os.path.abspath(__file__), "--steps", str(args.steps), "--warmup", str(args.warmup),
               "--cpu-seconds", "3", *extra]
        t0 = time.time()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
            line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
        except Exception as e:  # a failed extra run is recorded, not fatal to the headline
            out[key] = {"error": f"{type(e).__name__}: {e}"[:300]}
            continue
        summ = {"cmd": "python bench.py " + " ".join(cmd[2:]), "workload": line["config"].get("workload"),
                "value": line.get("value"), "unit": line.get("unit"), "ms_per_step": line.get("ms_per_step"),
                "wall_s": round(time.time() - t0, 1)}
        for k in ("e2e", "cpu_baseline", "clocks", "gpu_launches"):
            if k in line:
                summ[k] = {kk: vv for kk, vv in line[k].items() if kk != "path"} if isinstance(line[k], dict) \
                    else line[k]
        st = line.get("stats", {})
        for k in ("batch_latency_ms", "mean_iterations", "frames_failed", "frames_per_cta"):
            if k in st:
                summ[k] = st[k]
        cfg = line["config"]
        if key == "C4":
            summ.update({k: cfg[k] for k in ("learned", "plain", "speedup")})
        if key == "C5":
            summ.update({"rates": [{k: r_.get(k) for k in ("rate_gsym_s", "offered_gsym_s", "info_gbit_s", "p50_ms", "p99_ms", "failed")
                                    if k in r_} for r_ in cfg["rates"]]})
        out[key] = summ
    return out


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def main():
    args = parse()
    wl = dict(WORKLOAD_SHORT if args.workload == "short" else WORKLOAD)
    if args.impl == "reference":
        if args.workload == "mixed":
            mixed_reference_arm(args)
        else:
            reference_arm(args, wl)
        return
    if args.workload in ("chain", "acm"):
        # many streams of small launches: more hardware work queues than the
        # default 8 (process setting, must precede CUDA initialisation)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import torch
    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    import cusat_gb300 as cs
    from cusat_gb300 import build as lib_build
    lib_build.build()
    if args.workload in ("mixed", "serve", "learned", "codes", "chain", "acm", "pl"):
        {"mixed": mixed_main, "serve": serve_main, "learned": learned_main, "codes": codes_main, "pl": pl_main,
         "chain": chain_main, "acm": acm_main}[args.workload](
            args, torch, cs, rank, local_rank, world)
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    gen = ProductGen()
    nb = n_bufs_for(wl, gen)
    ci, msg, bufs, n0, gain = make_traffic(wl, nb, gen)
    B, T = wl["frames"], wl["max_trials"]
    mod, rate, fs = wl["mod"], wl["rate"], wl["fs"]
    # chains on their own streams: consecutive batches overlap, so the SMs
    # that finish one batch's last frames start on the next batch; enough
    # chains in flight that small batches (64 short frames) fill the
    # resident CTA slots
    pipe = args.pipe or min(8, max(PIPE, -(-RESIDENT_CTAS // B)))
    streams = [torch.cuda.Stream() for _ in range(pipe)]
    # value: symbols already in HBM, one rx_fec launch (demap -> decode ->
    # BCH) per batch into device outputs
    rxs = [cs.rx_fec(mod, rate, fs, T, B) for _ in range(pipe)]
    d_sym = [torch.from_numpy(b).cuda() for b in bufs]
    k_bytes = rxs[0].k_bytes
    outs = [(torch.zeros((B, k_bytes), dtype=torch.uint8, device="cuda"),
             torch.zeros(B, dtype=torch.int32, device="cuda"),
             torch.zeros(B, dtype=torch.int32, device="cuda")) for _ in range(pipe)]
    # e2e: the reference's per-slot launch sequence (rx_fec_chain.cc:361-505)
    # through the library's host-buffer entry points -- demap_batch_async
    # from pinned host symbols (copy into the demapper + demap),
    # decode_launch_async from the demapper's LLRs into mapped pinned
    # outputs, check_async of those outputs into a mapped pinned flag
    h_sym = [torch.from_numpy(b).pin_memory() for b in bufs]
    dms = [cs.demapper_cuda(mod, rate, fs, B) for _ in range(pipe)]
    decs = [cs.ldpc_decode_cuda(fs, rate, T, B) for _ in range(pipe)]
    bcs = [cs.bch_check_cuda.for_code(fs, rate) for _ in range(pipe)]
    h_out = [(torch.zeros((B, k_bytes), dtype=torch.uint8).pin_memory(),
              torch.zeros(B, dtype=torch.int32).pin_memory(),
              torch.zeros(B, dtype=torch.int32).pin_memory()) for _ in range(pipe)]
    sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
    fpc = frames_per_cta_for(ci, pipe, B, sms)
    for o in rxs + decs:
        o.set_frames_per_cta(fpc)
    fpc_used = decs[0].frames_per_cta(B)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step(i, e2e):
        k = i % pipe
        st = streams[k]
        if e2e:
            hard, trials, valid = h_out[k]
            dms[k].demap_batch_async(h_sym[i % nb].numpy(), B, n0, gain, st)
            decs[k].decode_launch_async(dms[k].soft_out_dev(), B, st, hard, trials)
            bcs[k].check_async(hard, valid, B, st)
        else:
            hard, trials, valid = outs[k]
            rxs[k].launch(d_sym[i % nb], B, n0, gain, hard, trials, valid, st)

    def timed(e2e):
        for i in range(args.warmup):
            step(i, e2e)
        barrier()
        start = torch.cuda.Event(enable_timing=True)
        start.record(streams[0])
        for st in streams[1:]:
            st.wait_event(start)
        for i in range(args.steps):
            step(i, e2e)
        for st in streams[1:]:
            ev = torch.cuda.Event()
            ev.record(st)
            streams[0].wait_event(ev)
        end = torch.cuda.Event(enable_timing=True)
        end.record(streams[0])
        barrier()
        return start.elapsed_time(end)

    clocks = Clocks(local_rank)
    clocks.start()
    t_wall = time.perf_counter()
    dev_ms = timed(False)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    e2e_ms = timed(True)

    # one batch at a time: launch duration of the chain (roofline), and the
    # iteration statistics of each input batch
    st = streams[0]
    hard, trials, valid = outs[0]
    launch = []
    iters = []
    for i in range(N_BUFS):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        rxs[0].launch(d_sym[i], B, n0, gain, hard, trials, valid, st)
        b.record(st)
        st.synchronize()
        launch.append(a.elapsed_time(b))
        tr = trials.cpu().numpy()
        iters.append(np.where(tr >= 0, T - tr, T))
    it = np.concatenate(iters)
    launch_ms = float(np.mean(launch))
    # the chain's kernels one at a time (the same kernels rx_fec launches):
    # demap into an LLR buffer, then the decoder, each bracketed by events
    dmp = cs.demapper_cuda(wl["mod"], wl["rate"], wl["fs"], B)
    dec = cs.ldpc_decode_cuda(wl["fs"], wl["rate"], T, B)
    soft = torch.empty((B, ci["n_ldpc"]), dtype=torch.int16, device="cuda")
    g_cap = cs.capped_llr_gain(wl["mod"], wl["rate"], wl["fs"], gain)
    demap_t, dec_t = [], []
    for i in range(N_BUFS + 1):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        dmp.demap_launch(d_sym[i % N_BUFS], B, n0, g_cap, soft, st)
        e1.record(st)
        dec.decode_launch_async(soft, B, st, hard, trials)
        e2.record(st)
        st.synchronize()
        if i:  # first round warms the two objects up
            demap_t.append(e0.elapsed_time(e1))
            dec_t.append(e1.elapsed_time(e2))
    demap_ms, dec_ms = float(np.mean(demap_t)), float(np.mean(dec_t))

    # max over ranks
    from cusat_gb300 import replicas
    dev_ms, e2e_ms = replicas.reduce_timing([dev_ms, e2e_ms], device="cuda")
    bits = args.steps * B * ci["k_ldpc"] * world
    value = bits / (dev_ms * 1e-3) / 1e9
    e2e = bits / (e2e_ms * 1e-3) / 1e9

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    mi = cs.modcod_info(wl["mod"], wl["rate"], wl["fs"])
    # algorithmic HBM bytes: the chain reads symbols (8 B each) and writes
    # hard bits, iteration counts and BCH flags; the decoder reads the LLRs
    # (2 B per bit) and writes hard bits and counts; the demap reads symbols
    # and writes LLRs
    per_launch_bytes = B * (mi["xfecframe_len"] * 8 + ci["k_ldpc"] // 8 + 12)
    dec_bytes = B * (2 * ci["n_ldpc"] + ci["k_ldpc"] // 8 + 4)
    demap_bytes = B * (mi["xfecframe_len"] * 8 + 2 * ci["n_ldpc"])
    launch_s = launch_ms * 1e-3
    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = dec_bytes / (dec_ms * 1e-3) / 1e9
    traffic, prof = None, {}
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "dram_traffic.json"))).get(args.workload, {})
        traffic = prof["dram_read_bytes"] + prof["dram_write_bytes"]
    except (OSError, KeyError, ValueError):
        pass
    edge_iters = float(np.mean(it)) * ci["edges"] * B
    issue_frac = None
    if prof.get("warp_instructions") and clk.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
        issue_frac = prof["warp_instructions"] / (dec_ms * 1e-3) / (sms * 4 * clk["sm_mhz"] * 1e6)
    threads = os.cpu_count() or 1
    cpu_s, n_cpu = cpu_sample(wl, bufs, n0, gain, threads, args.cpu_seconds)
    cpu_value = n_cpu * ci["k_ldpc"] / cpu_s / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": f"synthetic (seeded BCH/LDPC-encoded {wl['mod_name']} frames, AWGN at Es/N0 {wl['esn0_db']} dB)",
        "config": single_config(wl, nb, bufs[0].nbytes),
        "stats": {"parallelism": f"replicas x{world}; {pipe} chains on {pipe} streams, consecutive batches overlap",
                  "frames_per_cta": fpc_used,
                  "launch_ms": launch_ms, "mean_iterations": float(np.mean(it)),
                  "p99_iterations": float(np.percentile(it, 99)), "frames_failed": int(np.sum(it >= T))},
        "e2e": {"value": e2e, "unit": "Gbit/s", "h2d_bytes_per_step": int(bufs[0].nbytes),
                "d2h_bytes_per_step": int(B * (k_bytes + 8)),
                "path": "per batch: demapper_cuda.demap_batch_async from pinned host symbols (H2D copy + demap), "
                        "ldpc_decode_cuda.decode_launch_async into mapped pinned hard bits and counts, "
                        "bch_check_cuda.check_async of them into a mapped pinned flag -- the reference's "
                        "launch_slot_gpu sequence; results written to host memory inside the timed region"},
        "roofline": {"bound": "hbm", "kernel": "ldpc_layered_kernel (decoder)", "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                     "algorithmic_bytes": dec_bytes, "launch_ms": dec_ms,
                     "note": "dominant kernel = the decoder: algorithmic HBM bytes per launch (2 B per LLR in, "
                             "k/8 + 4 B per frame out) over its launch time (CUDA events on its stream), peak "
                             "= measured copy bandwidth (of measured); traffic = DRAM bytes of one decoder "
                             "launch from the ncu capture in profiles/ (null when none was taken for this "
                             "workload); the decoder is bound by integer issue (onchip), not HBM",
                     "kernels": {
                         "demap": {"launch_ms": demap_ms, "algorithmic_bytes": demap_bytes,
                                   "achieved_gbs": demap_bytes / (demap_ms * 1e-3) / 1e9,
                                   "frac": demap_bytes / (demap_ms * 1e-3) / 1e9 / hbm_peak},
                         "decoder": {"launch_ms": dec_ms, "algorithmic_bytes": dec_bytes},
                         "chain": {"launch_ms": launch_ms, "algorithmic_bytes": per_launch_bytes,
                                   "achieved_gbs": per_launch_bytes / launch_s / 1e9}}},
        "onchip": {"edge_iterations_per_s": edge_iters / (dec_ms * 1e-3),
                   "issue_frac": issue_frac,
                   "issue_note": "warp instructions of one decoder launch (ncu capture in profiles/) over its "
                                 "live launch time, divided by the issue peak (SMs x 4 schedulers x median "
                                 "SM clock): the decoder's binding roofline",
                   "alu_pipe_pct_ncu": prof.get("alu_pipe_pct"), "issue_active_pct_ncu": prof.get("issue_active_pct"),
                   "smem_app_bytes_per_s": 4.0 * edge_iters / (dec_ms * 1e-3),
                   "note": "mean iterations x Tanner edges x frames per launch; 4 B of shared-memory APP "
                           "traffic per edge-iteration (gather + scatter), messages 2 B in L2"},
        "cpu_baseline": {"value": cpu_value, "unit": "Gbit/s", "cores": threads, "kind": "port",
                         "sample": f"{n_cpu} frames of the workload ({n_cpu // B} batches) through the C oracle "
                                   f"(demap + decode + BCH), {cpu_s:.1f} s on {threads} threads"},
        "clocks": clk,
        "gpu_launches": 3 * args.steps,  # demap, decoder, BCH check per step
        "wall_s": wall,
    }
    if args.workload == "single" and world == 1 and args.extra:
        line["workloads"] = extra_workloads(args)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


MIXED = {"frames": 1024, "seed": 2025, "max_trials": 50, "sets": 2, "short_share": 0.3, "margin_db": 0.5}


class MixedTraffic:
    """The mixed workload packed into flat buffers: per frame a symbol slice,
    a hard-decision slice, an iteration counter and a BCH flag."""

    def __init__(self, cs, n_frames, seed, gen=None):
        from cusat_gb300 import traffic
        self.table, self.frames = traffic.mixed_traffic(n_frames, seed, short_share=MIXED["short_share"],
                                                        margin_db=MIXED["margin_db"], gen=gen)
        self.geo = traffic.geometry(self.table, gen)
        self.modcods = [(mod, rate, fs) for _, mod, rate, fs in self.table]
        self.sym_off, self.hard_off = [], []
        so = ho = 0
        for fr in self.frames:
            xfec, k_ldpc, _ = self.geo[fr["modcod"]]
            self.sym_off.append(so)
            self.hard_off.append(ho)
            so += (2 * xfec + 63) // 64 * 64          # floats; 256-byte aligned slices
            ho += (k_ldpc // 8 + 15) // 16 * 16
        self.sym = np.zeros(so, np.float32)
        for fr, o in zip(self.frames, self.sym_off):
            self.sym[o:o + fr["sym"].size] = fr["sym"].ravel()
        self.hard_bytes = ho
        self.info_bits = sum(self.geo[fr["modcod"]][1] for fr in self.frames)

    def descriptors(self, cs, d_sym, d_hard, d_trials, d_valid):
        n = len(self.frames)
        sb, hb = d_sym.data_ptr(), d_hard.data_ptr()
        tb, vb = d_trials.data_ptr(), d_valid.data_ptr()
        return cs.batch.frames([f["modcod"] for f in self.frames], [f["n0"] for f in self.frames],
                               [f["gain"] for f in self.frames], [sb + 4 * o for o in self.sym_off],
                               [hb + o for o in self.hard_off], [tb + 4 * i for i in range(n)],
                               [vb + 4 * i for i in range(n)])


def cpu_mixed(mt, n_sample, threads, max_trials):
    """Oracle demap + decode + BCH of the first n_sample frames, one oracle
    call per MODCOD (the oracle spreads a call's frames over the threads);
    returns (seconds, information bits)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    groups = {}
    for fr in mt.frames[:n_sample]:
        groups.setdefault(fr["modcod"], []).append(fr)
    t0 = time.perf_counter()
    bits = 0
    for m, frs in groups.items():
        _, mod, rate, fs = mt.table[m]
        sym = np.stack([fr["sym"] for fr in frs])
        llr = O.demap_modcod(sym, O.modcod(mod, rate, fs), frs[0]["n0"], frs[0]["gain"])
        hard, _ = O.ldpc_decode(fs, rate, llr, max_trials, nthreads=threads)
        O.bch_check(fs, rate, hard)
        bits += mt.geo[m][1] * len(frs)
    return time.perf_counter() - t0, bits


def mixed_config(n, learned, sets, sym_bytes):
    """The mixed workload's config dict, the same in both arms."""
    return {"workload": "mixed: 1024 frames of 10 MODCODs (64APSK 32/45 for S2X 64APSK 2/3), 70% normal "
                        "/ 30% short, demap -> decode (max 50 it) -> BCH, one CUDA graph replay "
                        "per step (tuned grid and class order)",
            "frames": n, "max_trials": MIXED["max_trials"], "seed": MIXED["seed"], "learned_weights": bool(learned),
            "l2": f"inputs alternate over {sets} sets ({sets * sym_bytes / 1e6:.0f} MB > L2)"}


def mixed_reference_arm(args):
    rank, _, _ = dist_env()
    if rank != 0:
        return
    mt = MixedTraffic(None, MIXED["frames"], MIXED["seed"], OracleGen())
    threads = os.cpu_count() or 1
    n = args.cpu_sample or 128
    cpu_mixed(mt, 2, threads, MIXED["max_trials"])
    total, bits = 0.0, 0
    for _ in range(args.steps):
        dt, b = cpu_mixed(mt, n, threads, MIXED["max_trials"])
        total += dt
        bits += b
    value = bits / total / 1e9
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gbit/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic (seeded mixed-MODCOD frames from the oracle's encoder and mapper, AWGN at each "
                "MODCOD's threshold + 0.5 dB)",
        "config": mixed_config(len(mt.frames), args.learned, MIXED["sets"], mt.sym.nbytes),
        "cpu_baseline": {"value": value, "unit": "Gbit/s", "cores": threads, "kind": "port",
                         "sample": f"first {n} frames of the 1024-frame mixed batch per step, demap + decode + "
                                   f"BCH through the C oracle (plain decoder)"},
        "e2e": {"value": value, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
        flush=True)


def mixed_main(args, torch, cs, rank, local_rank, world):
    """1024 frames of 10 MODCODs (70% normal, 30% short, each at its
    threshold + 0.5 dB) per step: one CUDA graph replay of the tuned batch
    launch sequence.  Two input sets on two streams (> L2 in total)."""
    T = MIXED["max_trials"]
    mt = MixedTraffic(cs, MIXED["frames"], MIXED["seed"] + rank)
    n = len(mt.frames)
    S = MIXED["sets"]
    streams = [torch.cuda.Stream() for _ in range(S)]
    h_sym = torch.from_numpy(mt.sym).pin_memory()
    sets = []
    for k in range(S):
        d_sym = torch.from_numpy(mt.sym).cuda()
        d_hard = torch.zeros(mt.hard_bytes, dtype=torch.uint8, device="cuda")
        d_res = torch.zeros((2, n), dtype=torch.int32, device="cuda")
        h_hard = torch.empty(mt.hard_bytes, dtype=torch.uint8).pin_memory()
        h_res = torch.empty((2, n), dtype=torch.int32).pin_memory()
        b = cs.batch(mt.modcods, max_trials=T, max_frames=n)
        if args.learned:
            from cusat_gb300 import learned
            for e, (name, _, _, fs) in enumerate(mt.table):
                w = learned.load_weights(name, fs)
                if w is not None:
                    b.set_weights(e, w)
        fr = mt.descriptors(cs, d_sym, d_hard, d_res[0], d_res[1])
        torch.cuda.synchronize()
        tune_ms = b.tune(fr, reps=3, stream=streams[k])
        b.capture(fr, streams[k])
        sets.append({"b": b, "fr": fr, "d_sym": d_sym, "d_hard": d_hard, "d_res": d_res, "h_hard": h_hard,
                     "h_res": h_res, "tune_ms": tune_ms})
    n_classes = sets[0]["b"].info()[1]

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step(i, e2e):
        k = i % S
        st, z = streams[k], sets[k]
        with torch.cuda.stream(st):
            if e2e:
                z["d_sym"].copy_(h_sym, non_blocking=True)
            z["b"].replay(st)
            if e2e:
                z["h_hard"].copy_(z["d_hard"], non_blocking=True)
                z["h_res"].copy_(z["d_res"], non_blocking=True)

    def timed(e2e):
        for i in range(args.warmup):
            step(i, e2e)
        barrier()
        start = torch.cuda.Event(enable_timing=True)
        start.record(streams[0])
        for st in streams[1:]:
            st.wait_event(start)
        for i in range(args.steps):
            step(i, e2e)
        for st in streams[1:]:
            ev = torch.cuda.Event()
            ev.record(st)
            streams[0].wait_event(ev)
        end = torch.cuda.Event(enable_timing=True)
        end.record(streams[0])
        barrier()
        return start.elapsed_time(end)

    clocks = Clocks(local_rank)
    clocks.start()
    dev_ms = timed(False)
    clk = clocks.stop()
    e2e_ms = timed(True)

    # one replay at a time: batch latency distribution and decode statistics
    st = streams[0]
    lat = []
    for i in range(max(args.steps, 8)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        sets[0]["b"].replay(st)
        b.record(st)
        st.synchronize()
        lat.append(a.elapsed_time(b))
    res = sets[0]["d_res"].cpu().numpy()
    trials, valid = res[0], res[1]
    it = np.where(trials >= 0, T - trials, T)

    from cusat_gb300 import replicas
    dev_ms, e2e_ms = replicas.reduce_timing([dev_ms, e2e_ms], device="cuda")
    bits = args.steps * mt.info_bits * world
    value = bits / (dev_ms * 1e-3) / 1e9
    e2e = bits / (e2e_ms * 1e-3) / 1e9
    if rank != 0:
        return

    per = {}
    for f, fr in enumerate(mt.frames):
        name, _, _, fs = mt.table[fr["modcod"]]
        key = f"{name}{'s' if fs == 1 else 'n'}"
        d = per.setdefault(key, {"frames": 0, "iters": 0, "failed": 0, "bch_bad": 0})
        d["frames"] += 1
        d["iters"] += int(it[f])
        d["failed"] += int(trials[f] < 0)
        d["bch_bad"] += int(valid[f] == 0)
    for d in per.values():
        d["mean_iterations"] = d.pop("iters") / d["frames"]
    lat_ms = float(np.median(lat))
    in_bytes = sum(2 * 4 * mt.geo[fr["modcod"]][0] for fr in mt.frames)
    out_bytes = sum(mt.geo[fr["modcod"]][1] // 8 + 12 for fr in mt.frames)
    hbm_peak = load_peaks().get("hbm_gbs", 6800.0)
    achieved = (in_bytes + out_bytes) / (lat_ms * 1e-3) / 1e9
    threads = os.cpu_count() or 1
    n_cpu = args.cpu_sample or n
    cpu_s, cpu_bits, reps = 0.0, 0, 0
    while cpu_s < args.cpu_seconds:
        dt, b = cpu_mixed(mt, n_cpu, threads, T)
        cpu_s += dt
        cpu_bits += b
        reps += 1
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic (seeded mixed-MODCOD frames from this project's encoder and mapper, AWGN at each "
                "MODCOD's threshold + 0.5 dB)",
        "config": mixed_config(n, args.learned, S, mt.sym.nbytes),
        "stats": {"kernel_classes": n_classes,
                  "parallelism": f"replicas x{world}; {S} graphs on {S} streams, consecutive batches overlap",
                  "batch_latency_ms": {"p50": lat_ms, "p99": float(np.percentile(lat, 99))},
                  "tune_ms": [z["tune_ms"] for z in sets],
                  "tuned": sets[0]["b"].tuned(),
                  "mean_iterations": float(np.mean(it)), "frames_failed": int(np.sum(trials < 0)),
                  "per_modcod": per},
        "e2e": {"value": e2e, "unit": "Gbit/s", "h2d_bytes_per_step": int(mt.sym.nbytes),
                "d2h_bytes_per_step": int(mt.hard_bytes + 8 * n)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None,
                     "note": "algorithmic bytes (symbols in, hard bits + counters out) per replay over the "
                             "replay time; the decoders are bound by the integer ALU pipe"},
        "cpu_baseline": {"value": cpu_bits / cpu_s / 1e9, "unit": "Gbit/s", "cores": threads, "kind": "port",
                         "sample": f"{reps} x the first {n_cpu} frames through the C oracle, {cpu_s:.1f} s on "
                                   f"{threads} threads"},
        "clocks": clk,
        "gpu_launches": args.steps * (n_classes + 2),  # demap, one decoder per class, BCH
    }), flush=True)


def pl_frames(cs, sym, pls_code, gold):
    """PLFRAME payloads (the symbols after the PLHEADER) of XFECFRAMEs: a
    36-symbol pilot block ((1 + j)/sqrt 2) after every 16 slots when the PLS
    code signals pilots, then scrambling by e^{+j R pi/2} (EN 302 307-1
    clauses 5.5.3, 5.5.4) -- test traffic for the PL receiver tail."""
    lay = cs.pl_layout(pls_code)
    S, nb = lay["slots"], lay["pilot_blocks"]
    r = cs.pl_rotation_index(gold, lay["payload_symbols"])
    B = sym.shape[0]
    d = sym.reshape(B, S, 90, 2)
    a = np.float32(np.sqrt(0.5))
    parts = []
    for s in range(S):
        parts.append(d[:, s])
        if s % 16 == 15 and (s + 1) // 16 <= nb:
            parts.append(np.full((B, 36, 2), a, np.float32))
    pay = np.concatenate(parts, axis=1)
    re, im = pay[..., 0], pay[..., 1]
    out = np.empty_like(pay)
    out[..., 0] = np.select([r == 0, r == 1, r == 2, r == 3], [re, -im, -re, im])
    out[..., 1] = np.select([r == 0, r == 1, r == 2, r == 3], [im, re, -im, -re])
    return out.reshape(B, -1), lay


def pl_main(args, torch, cs, rank, local_rank, world):
    """The PL receiver tail alone: 256 located PLFRAMEs of the headline
    MODCOD (8PSK 3/5 normal, pilots on) per step through cusat_pl_extract
    (descramble, drop 14 pilot blocks, counter-rotate 240 slots); inputs
    cycled over 4 batches (> L2).  HBM-bound: 8 B read per payload symbol + 1 B
    scrambling index, 8 B written per data symbol."""
    wl = dict(WORKLOAD)
    gen = ProductGen()
    ci, msg, bufs, n0, gain = make_traffic(wl, 1, gen)
    code, gold = (12 << 2) | 1, 0
    pay, lay = pl_frames(cs, bufs[0], code, gold)
    B = pay.shape[0]
    rng = np.random.default_rng(3)
    rot = np.zeros((B, lay["slots"], 4), np.float32)
    ang = rng.uniform(-3.1, 3.1, (B, lay["slots"]))
    rot[..., 0], rot[..., 1] = np.cos(ang), np.sin(ang)
    rot[..., 2], rot[..., 3] = np.float32(np.cos(1e-3)), np.float32(np.sin(1e-3))
    d_pay = [torch.from_numpy(pay).cuda() for _ in range(N_BUFS)]
    d_rot = torch.from_numpy(rot).cuda()
    d_out = torch.zeros((B, 2 * lay["data_symbols"]), dtype=torch.float32, device="cuda")
    x = cs.pl_extractor([gold], max_frames=B)
    frs = [x.frames([p[f] for f in range(B)], [d_out[f] for f in range(B)], [code] * B, [gold] * B,
                    [d_rot[f] for f in range(B)]) for p in d_pay]
    st = torch.cuda.current_stream()
    for i in range(args.warmup):
        x.extract(frs[i % N_BUFS], st)
    torch.cuda.synchronize()
    clocks = Clocks(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for i in range(args.steps):
        x.extract(frs[i % N_BUFS], st)
    e1.record(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    bytes_step = B * (lay["payload_symbols"] * 9 + lay["data_symbols"] * 8 + lay["slots"] * 16)
    peak = load_peaks().get("hbm_gbs", 6800.0)
    gbs = bytes_step / (ms * 1e-3) / 1e9
    print(json.dumps({
        "metric": "PL receiver tail: located PLFRAMEs -> XFECFRAMEs (info Gbit/s of the frames carried)",
        "value": B * ci["k_ldpc"] / (ms * 1e-3) / 1e9, "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 8PSK 3/5 XFECFRAMEs with pilot blocks, scrambled with Gold code 0, random per-slot rotations)",
        "config": {"workload": f"{B} PLFRAMEs (PLS code {code}: {lay['slots']} slots, {lay['pilot_blocks']} pilot "
                               f"blocks) per step through cusat_pl_extract", "frames": B,
                   "l2": f"inputs cycled over {N_BUFS} batches ({N_BUFS * pay.nbytes / 1e6:.0f} MB > L2)"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "traffic": None, "algorithmic_bytes": bytes_step,
                     "note": "per frame: payload 8 B and scrambling index 1 B per payload symbol read, 16 B of "
                             "rotation per slot read, 8 B per data symbol written; peak = measured copy "
                             "bandwidth (of measured)"},
        "clocks": clk, "gpu_launches": args.steps}), flush=True)


def serve_main(args, torch, cs, rank, local_rank, world):
    """Serving loop under Poisson arrivals (seeded ACM schedule over the 10
    MODCODs, 70% normal / 30% short, threshold + 0.5 dB) at each aggregate
    symbol rate: p50/p99 frame latency (arrival -> results on the host) and
    info Gbit/s.  One line; value = info Gbit/s at the highest rate."""
    from cusat_gb300 import serving, traffic
    pool = serving.TracePool(traffic.MIXED_MODCODS, seed=2026 + rank, per_entry=16, torch=torch)
    learned_entries = {}
    if args.learned:
        from cusat_gb300 import learned
        for e, (name, fs) in enumerate(pool.table):
            w = learned.load_weights(name, fs)
            if w is not None:
                learned_entries[e] = w

    def new_server():
        srv = cs.server(pool.modcods, max_trials=50, hbm_budget=4 << 30, slots=4, max_batch=512)
        for e, w in learned_entries.items():
            srv.set_weights(e, w)
        return srv

    srv = new_server()
    serving.replay(srv, pool, serving.make_trace(pool, 1e9, 0.02, seed=1))  # warm-up
    clocks = Clocks(local_rank)
    clocks.start()
    rows = []
    for k, r in enumerate(float(x) for x in args.rates.split(",")):
        trace = serving.make_trace(pool, r * 1e9, args.duration, seed=100 + k)
        res, st = serving.replay(srv, pool, trace)
        row = serving.summarize(pool, trace, res)
        row.update({"rate_gsym_s": r, "batches": int(st["batches"]), "largest_batch": int(st["largest_batch"]),
                    "peak_arena_mb": st["peak_bytes"] / 1e6})
        rows.append(row)
        srv.close()
        srv = new_server()
    clk = clocks.stop()
    srv.close()
    if rank != 0:
        return
    top = rows[-1]
    print(json.dumps({
        "metric": METRIC, "value": top["info_gbit_s"], "unit": "Gbit/s", "n_gpus": world,
        "steps": len(rows), "warmup": 1, "ms_per_step": args.duration * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic (seeded ACM trace over 10 MODCODs, device-resident noisy frames at threshold + 0.5 dB)",
        "config": {"workload": "serving loop: Poisson arrivals, HBM-budget admission (4 GiB), continuous "
                               "batching on 4 slots (max 512 frames per batch), max 50 iterations",
                   "learned_weights": sorted(f"{pool.table[e][0]} {'short' if pool.table[e][1] else 'normal'}"
                                             for e in learned_entries),
                   "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"], "rates": rows},
        "clocks": clk,
    }), flush=True)


LEARNED = {"name": "normal 1/3 QPSK", "modcod": "qpsk1/3", "fs": 0, "rate": 1, "mod": 0, "frames": 256,
           "esn0_db": 0.56, "seed": 2027}


def learned_main(args, torch, cs, rank, local_rank, world):
    """Plain offset min-sum capped at 50 iterations against the learned
    weights capped at 20, same frames, same timing as the headline (two
    chains on two streams, inputs cycled over 4 batches); value = learned
    info Gbit/s.  Frame errors are counted against the sent codewords."""
    from cusat_gb300 import learned, replicas
    wl = dict(LEARNED)
    from cusat_gb300.enums import find_modcod
    _, wl["mod"], wl["rate"], _, _, _ = find_modcod(wl["modcod"])
    w = learned.load_weights(wl["modcod"], wl["fs"])
    if w is None:
        raise RuntimeError("no adopted weight file for " + wl["modcod"])
    nb = n_bufs_for(wl, ProductGen())
    ci, msg, bufs, n0, gain = make_traffic(wl, nb)
    B = wl["frames"]
    sent = [torch.from_numpy(cs.encode_frames(wl["fs"], wl["rate"], msg)[:, :ci["k_ldpc"] // 8]).cuda()]
    d_sym = [torch.from_numpy(b).cuda() for b in bufs]
    streams = [torch.cuda.Stream() for _ in range(PIPE)]
    res = {}
    for label, T, wt in (("plain50", 50, None), ("learned20", 20, w)):
        rxs = [cs.rx_fec(wl["mod"], wl["rate"], wl["fs"], T, B) for _ in range(PIPE)]
        for rx in rxs:
            rx.set_weights(wt)
        outs = [(torch.zeros((B, rxs[0].k_bytes), dtype=torch.uint8, device="cuda"),
                 torch.zeros(B, dtype=torch.int32, device="cuda")) for _ in range(PIPE)]

        def step(i):
            k = i % PIPE
            with torch.cuda.stream(streams[k]):
                rxs[k].launch(d_sym[i % nb], B, n0, gain, outs[k][0], outs[k][1], None, streams[k])

        for i in range(args.warmup):
            step(i)
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        start.record(streams[0])
        for st in streams[1:]:
            st.wait_event(start)
        for i in range(args.steps):
            step(i)
        for st in streams[1:]:
            ev = torch.cuda.Event()
            ev.record(st)
            streams[0].wait_event(ev)
        end = torch.cuda.Event(enable_timing=True)
        end.record(streams[0])
        torch.cuda.synchronize()
        ms = replicas.reduce_timing([start.elapsed_time(end)], device="cuda")[0]
        errors = frames = iters = 0
        for i in range(N_BUFS):
            rxs[0].launch(d_sym[i], B, n0, gain, outs[0][0], outs[0][1], None, streams[0])
            streams[0].synchronize()
            errors += int((outs[0][0] != sent[0]).any(dim=1).sum().item())
            tr = outs[0][1].cpu().numpy()
            iters += float(np.sum(np.where(tr >= 0, T - tr, T)))
            frames += B
        res[label] = {"gbit_s": args.steps * B * ci["k_ldpc"] * world / (ms * 1e-3) / 1e9,
                      "ms_per_step": ms / args.steps, "frame_errors": errors, "frames": frames,
                      "mean_iterations": iters / frames}
    if rank != 0:
        return
    print(json.dumps({
        "metric": METRIC, "value": res["learned20"]["gbit_s"], "unit": "Gbit/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["learned20"]["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic (seeded BCH/LDPC-encoded QPSK frames, AWGN at Es/N0 0.56 dB)",
        "config": {"workload": "normal 1/3 QPSK (s2_b2), 256 frames at its threshold 0.56 dB: demap -> "
                               "learned min-sum (max 20 it) vs plain (max 50 it) -> BCH",
                   "learned": res["learned20"], "plain": res["plain50"],
                   "speedup": res["learned20"]["gbit_s"] / res["plain50"]["gbit_s"]},
    }), flush=True)


CODES = [("qpsk1/4", 0), ("qpsk1/2", 1), ("qpsk1/2", 0), ("8psk3/5", 1), ("8psk3/5", 0), ("16apsk3/4", 1),
         ("qpsk3/4", 0), ("16apsk5/6", 1), ("8psk5/6", 0), ("8psk8/9", 1), ("8psk9/10", 0)]

DEMAP_MODCODS = ["qpsk1/2", "8psk3/5", "8apsk5/9", "16apsk2/3", "32apsk3/4", "64apsk32/45", "128apsk3/4",
                 "256apsk3/4", "256apsk2/3"]


def codes_main(args, torch, cs, rank, local_rank, world):
    """One MODCOD per kernel class (circulant slots per layer x lanes): 256
    frames at threshold + 0.5 dB through the receive chain, median of `steps`
    single launches (CUDA events) after `warmup`; value = the headline
    class's Gbit/s, the others in config.codes."""
    from cusat_gb300 import traffic
    from cusat_gb300.enums import find_modcod
    B, rows = 256, {}
    st = torch.cuda.current_stream()
    clocks = Clocks(local_rank)
    clocks.start()
    for name, fs in CODES:
        _, mod, rate, _, _, thr = find_modcod(name)
        _, sym, n0, gain = traffic.modcod_frames(name, fs, B, thr + 0.5, np.random.default_rng(5))
        ci = cs.code_info(fs, rate)
        rx = cs.rx_fec(mod, rate, fs, 50, B)
        d = torch.from_numpy(sym).cuda()
        h = torch.zeros((B, rx.k_bytes), dtype=torch.uint8, device="cuda")
        t = torch.zeros(B, dtype=torch.int32, device="cuda")
        for _ in range(args.warmup):
            rx.launch(d, B, n0, gain, h, t, None, st)
        ts = []
        for _ in range(max(args.steps, 3)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            rx.launch(d, B, n0, gain, h, t, None, st)
            b.record(st)
            st.synchronize()
            ts.append(a.elapsed_time(b))
        ms = float(np.median(ts))
        tr = t.cpu().numpy()
        it = float(np.mean(np.where(tr >= 0, 50 - tr, 50)))
        rows[f"{name} {'short' if fs else 'normal'}"] = {
            "slots": ci["cmax"], "lanes": ci["lanes"], "launch_ms": ms, "gbit_s": B * ci["k_ldpc"] / ms / 1e6,
            "mean_iterations": it, "edge_iterations_per_ns": B * it * ci["edges"] / ms / 1e6}
    # the demapper per constellation family, normal frames: the demap launch
    # alone and the whole receive launch (demap + decode + BCH) on the same
    # 256 frames, so the demap's share of the path shows
    demap = {}
    for name in (args.demap_modcods.split(",") if args.demap_modcods else DEMAP_MODCODS):
        _, mod, rate, _, _, thr = find_modcod(name)
        _, sym, n0, gain = traffic.modcod_frames(name, 0, B, thr + 0.5, np.random.default_rng(6))
        ci = cs.code_info(0, rate)
        dm = cs.demapper_cuda(mod, rate, 0, B)
        rx = cs.rx_fec(mod, rate, 0, 50, B)
        d = torch.from_numpy(sym).cuda()
        llr = torch.zeros((B, dm.fecframe_len()), dtype=torch.int16, device="cuda")
        h = torch.zeros((B, rx.k_bytes), dtype=torch.uint8, device="cuda")
        t = torch.zeros(B, dtype=torch.int32, device="cuda")
        g = dm.capped_llr_gain(gain)

        def timed(fn):
            for _ in range(args.warmup):
                fn()
            ts = []
            for _ in range(max(args.steps, 3)):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(st)
                fn()
                b.record(st)
                st.synchronize()
                ts.append(a.elapsed_time(b))
            return float(np.median(ts))
        dms = timed(lambda: dm.demap_launch(d, B, n0, g, llr, st))
        rms = timed(lambda: rx.launch(d, B, n0, gain, h, t, None, st))
        demap[name] = {"bits_per_symbol": dm.n_mod(), "symbols_per_frame": dm.xfecframe_len(), "demap_ms": dms,
                       "msym_s": B * dm.xfecframe_len() / dms / 1e3, "receive_ms": rms,
                       "receive_gbit_s": B * ci["k_ldpc"] / rms / 1e6, "demap_share": dms / rms}
    clk = clocks.stop()
    if rank != 0:
        return
    head = rows["8psk3/5 normal"]
    print(json.dumps({
        "metric": METRIC, "value": head["gbit_s"], "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["launch_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16", "data": "synthetic (seeded frames at threshold + 0.5 dB)",
        "config": {"workload": "one MODCOD per decoder kernel class, 256 frames, single launches (inputs in "
                               "L2 for the short codes)", "codes": rows, "demap": demap}, "clocks": clk}), flush=True)


# (micro_batch, streams, decode budget: -1 = one frame per SM, 0 = unlimited,
# copy helper threads); (4, 8, -1, 0) is the reference's default
CHAIN_SETTINGS = [(4, 8, -1, 0), (16, 8, -1, 0), (64, 4, -1, 0), (64, 4, 0, 0), (128, 4, 0, 0), (128, 4, 0, 3),
                  (128, 4, -1, 3)]


def chain_cpp_rows(cs, n, esn0):
    """Builds tests/chain_timing.cc against the library and runs it for a few
    chain settings; {} if no C++ compiler is available."""
    exe = os.path.join(ROOT, "cusat_gb300", "_build", "chain_timing")
    lib = cs.library_path()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "chain_timing.cc"), "-o", exe, lib,
           "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "targets", "sbsa-linux", "lib"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib)]
    try:
        subprocess.run(cmd, check=True, capture_output=True, timeout=300)
    except (OSError, subprocess.SubprocessError):
        return {}
    rows = {}
    for mb, streams, cap, helpers, conn in [(4, 8, -1, 0, 8), (4, 8, -1, 0, 32), (4, 8, -1, 3, 32),
                                            (128, 4, 0, 0, 32), (128, 4, 0, 3, 32), (128, 4, -1, 3, 32)]:
        r = subprocess.run([exe, str(n), str(mb), str(streams), str(cap), str(helpers), str(esn0), str(conn)],
                           capture_output=True, text=True, timeout=300)
        try:
            rows[f"micro_batch {mb}, {streams} streams, budget {'default' if cap < 0 else 'unlimited'}, "
                 f"copy helpers {helpers}, {conn} hardware queues"] = json.loads(r.stdout.strip().splitlines()[-1])
        except (ValueError, IndexError):
            rows[f"micro_batch {mb}, {streams} streams"] = {"error": r.stderr[-200:]}
    return rows


def chain_main(args, torch, cs, rank, local_rank, world):
    """The frame-at-a-time receive chain (rx_fec_chain API) on the headline
    MODCOD: host XFECFRAMEs submitted one by one, micro-batched, launched on
    the chain's streams within the default decode budget (one frame per SM),
    drained in order; offline mode (block when the flight ring is full).  One
    step = 256 frames; wall time from the first submit to the end of the final
    flush.  value = the best setting's info Gbit/s."""
    wl = dict(WORKLOAD)
    _, _, bufs, n0, _ = make_traffic(wl, n_bufs_for(wl, ProductGen()))
    frames = [f for b in bufs for f in b]
    ci = cs.code_info(wl["fs"], wl["rate"])
    rows = {}
    clocks = Clocks(local_rank)
    clocks.start()
    for mb, streams, cap, helpers in CHAIN_SETTINGS:
        chain = cs.rx_fec_chain(wl["fs"], wl["rate"], wl["mod"], wl["max_trials"], 64, streams, mb)
        budget = cs.gpu_decode_budget(cap)
        chain.set_decode_budget(budget)
        chain.set_copy_threads(helpers)
        chain.set_block_when_full(True)
        chain.warmup()
        chain.update_snr(wl["esn0_db"])
        k = 0
        for _ in range(args.warmup * wl["frames"]):
            chain.submit_xfecframe(frames[k % len(frames)])
            k += 1
        chain.flush()
        n = args.steps * wl["frames"]
        t_submit = 0.0
        t0 = time.perf_counter()
        for _ in range(n):
            ta = time.perf_counter()
            chain.submit_xfecframe(frames[k % len(frames)])
            t_submit += time.perf_counter() - ta
            k += 1
        chain.flush()
        dt = time.perf_counter() - t0
        rows[f"micro_batch {mb}, {streams} streams, budget {budget.cap or 'unlimited'}, copy helpers {helpers}"] = {
            "gbit_s": n * ci["k_ldpc"] / dt / 1e9, "ms_per_step": dt * 1e3 / args.steps,
            "frames_per_s": n / dt, "host_us_per_submit": t_submit / n * 1e6,
            "force_drains": chain.force_drain_count(), "errors": chain.frame_error_count()}
        chain.close()
        budget.close()
    # the same chain driven from C++ through the rx_fec_chain shim
    # (include/cusat_fec.hpp; tests/chain_timing.cc), no Python in the loop
    cpp_rows = chain_cpp_rows(cs, args.steps * wl["frames"], wl["esn0_db"])
    clk = clocks.stop()
    # where a submit's host time goes: copying one frame into a pinned buffer
    # (numpy), and the ctypes round trip of a trivial call
    pinned = torch.empty(frames[0].size, dtype=torch.float32).pin_memory().numpy()
    reps = 2000
    t0 = time.perf_counter()
    for i in range(reps):
        np.copyto(pinned, frames[i % len(frames)].reshape(-1))
    copy_us = (time.perf_counter() - t0) / reps * 1e6
    probe = cs.rx_fec_chain(wl["fs"], wl["rate"], wl["mod"], wl["max_trials"], 64, 1, 4)
    t0 = time.perf_counter()
    for _ in range(reps):
        probe.pending_count()
    call_us = (time.perf_counter() - t0) / reps * 1e6
    probe.close()
    if rank != 0:
        return
    best = max(rows.values(), key=lambda r: r["gbit_s"])
    print(json.dumps({
        "metric": METRIC, "value": best["gbit_s"], "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": best["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16", "data": "synthetic (seeded 8PSK 3/5 normal frames at 6 dB, host "
                                                       "memory, random payloads)",
        "config": {"workload": "rx_fec_chain: frames submitted one at a time from host memory, 256 per step, "
                               "max 50 iterations", "settings": rows,
                   "e2e_note": "host symbols in, per-frame verdicts and GSE data fields out (pinned)",
                   "host_frame_copy_us": copy_us, "host_ctypes_call_us": call_us, "cpp": cpp_rows,
                   "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS")},
        "clocks": clk}), flush=True)


def acm_main(args, torch, cs, rank, local_rank, world):
    """The receive pool under ACM traffic: the 10-MODCOD mix in normal
    frames at threshold + 0.5 dB, submitted one by one from host memory with
    the MODCOD drawn per frame (rx_fec_pool::submit), through the per-MODCOD
    pool (the reference's design: one chain per MODCOD, wait at every MODCOD
    change) and the mixed pool (one slot ring, multi-MODCOD launches).  Wall
    time from the first submit to the end of finish_all_pending; value = the
    mixed pool's info Gbit/s."""
    from cusat_gb300 import traffic
    from cusat_gb300.enums import find_modcod
    table, frames = traffic.mixed_traffic(512, 2031, short_share=0.0)
    idx = [find_modcod(name)[0] for name, _, _, _ in table]
    kbits = [cs.code_info(fs, rate)["k_ldpc"] for _, _, rate, fs in table]
    thr = [find_modcod(name)[5] + 0.5 for name, _, _, _ in table]
    rows = {}

    def run(pool, n):
        pool.warmup_all()
        for m, t in zip(idx, thr):
            pool.update_snr(m, t)
        bits = 0
        t0 = time.perf_counter()
        for f in frames[:n]:
            if pool.submit(f["sym"], idx[f["modcod"]]):
                while pool.get_gse_output().size:
                    pass
            bits += kbits[f["modcod"]]
        pool.finish_all_pending()
        dt = time.perf_counter() - t0
        return {"frames": n, "gbit_s": bits / dt / 1e9, "ms": dt * 1e3, "frame_errors": pool.total_error_count()}

    clocks = Clocks(local_rank)
    clocks.start()
    per = cs.rx_fec_pool(0, idx, 50, 64, 8, 4)
    rows["per-MODCOD pool (reference design), micro-batch 4, 8 streams"] = run(per, 128)
    per.close()
    for sf, helpers in ((32, 0), (64, 0), (128, 0), (128, 3)):
        mix = cs.rx_fec_pool(0, idx, 50, 64, 4, 4, mixed=True, slot_frames=sf)
        mix.set_copy_threads(helpers)
        run(mix, 64)  # warm-up
        rows[f"mixed pool, {sf}-frame slots, 4 streams, copy helpers {helpers}"] = run(mix, len(frames))
        mix.close()
    clk = clocks.stop()
    if rank != 0:
        return
    best = max((v for k, v in rows.items() if k.startswith("mixed")), key=lambda r: r["gbit_s"])
    changes = sum(1 for a, b in zip(frames, frames[1:]) if a["modcod"] != b["modcod"])
    print(json.dumps({
        "metric": METRIC, "value": best["gbit_s"], "unit": "Gbit/s", "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": best["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int16", "data": "synthetic (seeded 10-MODCOD normal-frame ACM sequence at threshold + 0.5 dB, "
                                  "host memory)",
        "config": {"workload": f"rx_fec_pool under ACM: {len(frames)} frames, MODCOD changes at {changes} of "
                               f"{len(frames) - 1} frame boundaries, submitted one by one, max 50 iterations",
                   "pools": rows}, "clocks": clk}), flush=True)


if __name__ == "__main__":
    main()
