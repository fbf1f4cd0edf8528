"""The reference's own GPU kernels beside this project's, on one GPU.

TEST INFRASTRUCTURE: runs the reference's demapper and layered decoder
(compiled unchanged into oracle/_ref/*.cubin by oracle/build.py, launched
by oracle/ref_gpu.c) on the same inputs as this project's kernels and the
oracle, and prints one JSON object:

  demap    per MODCOD: the reference kernel's int16 LLRs against the
           oracle's (count equal, largest difference)
  decode   per workload: the reference decoder's (hard bits, trials) per
           frame against the oracle's (identical, same hard bits, both
           converged), and against a second run of itself
  timing   per workload: CUDA-event time per launch of the reference
           decoder and of this project's decoder on the same LLR batches,
           one launch after another on one stream, inputs cycled over
           batches larger than the L2 together; the same for the demappers
  mixed    the bench's 1024-frame mixed batch: this project's graph replay
           against the reference's demap + decoder per MODCOD entry on
           concurrent streams, one round at a time
  fer      frame error rates of both decoders on the same fresh GPU-made
           LLRs near the waterfall of C1's and C2's codes

Usage (on a GPU host, after __graft_entry__.build()):
    python oracle/ref_gpu_compare.py [--out FILE] [--steps K] [--warmup W] [--no-fer]
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
# the mixed section runs many streams on both sides: 32 hardware queues, as
# bench.py sets them (must precede CUDA initialisation)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
sys.path.insert(0, os.path.join(ROOT, "tests"))

# (name, MODCOD, frame size, frames, Es/N0 dB, seed)
DECODE_CASES = [
    ("C2 normal 3/5 8PSK", "8psk3/5", 0, 256, 6.0, 2024),
    ("C1 short 1/2 QPSK", "qpsk1/2", 1, 64, 1.5, 2025),
    ("normal 1/4 QPSK", "qpsk1/4", 0, 256, None, 31),
    ("normal 9/10 8PSK", "8psk9/10", 0, 256, None, 32),
    ("short 5/6 16APSK", "16apsk5/6", 1, 256, None, 33),
]
DEMAP_CASES = [("qpsk1/2", 1), ("qpsk3/4", 0), ("8psk3/5", 0), ("8psk8/9", 1), ("8apsk5/9", 0),
               ("16apsk2/3", 0), ("16apsk5/6", 1), ("32apsk3/4", 0), ("64apsk32/45", 0), ("128apsk3/4", 0),
               ("256apsk3/4", 0), ("256apsk32/45", 0)]
L2_BYTES = 160e6


def traffic(cs, E, O, name, fs, B, esn0, seed, n_bufs=1):
    """Noisy symbols (the bench's recipe: one set of codewords, fresh noise
    per buffer), N0, the capped gain and the MODCOD description."""
    _, mod, rate, _, _, thr = E.find_modcod(name)
    esn0 = thr + 0.5 if esn0 is None else esn0
    rng = np.random.default_rng(seed)
    ci = cs.code_info(fs, rate)
    msg = rng.integers(0, 256, (B, ci["k_bch"] // 8), dtype=np.uint8)
    sym = cs.map_frames(mod, rate, fs, cs.encode_frames(fs, rate, msg))
    es = float(np.mean(sym.astype(np.float64) ** 2) * 2)
    sym = (sym / np.float32(np.sqrt(es))).astype(np.float32)
    n0 = np.float32(1.0 / 10 ** (esn0 / 10.0))
    sigma = np.float32(np.sqrt(n0 / np.float32(2.0)))
    bufs = [(sym + sigma * rng.standard_normal(sym.shape, dtype=np.float32)).astype(np.float32)
            for _ in range(n_bufs)]
    mi = O.modcod(mod, rate, fs)
    gain = O.capped_llr_gain(mi, min(4.0 / float(n0), 1000.0))
    return mod, rate, esn0, bufs, float(n0), gain, mi


def time_launches(torch, launch, n_inputs, steps, warmup):
    """ms per launch: warmup untimed launches, then steps launches timed
    with CUDA events on the current stream, inputs cycled."""
    s = torch.cuda.current_stream()
    for i in range(warmup):
        launch(i % n_inputs)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for i in range(steps):
        launch(i % n_inputs)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def demap_section(torch, cs, E, O, rg):
    out = []
    s = torch.cuda.current_stream()
    for name, fs in DEMAP_CASES:
        mod, rate, esn0, bufs, n0, gain, mi = traffic(cs, E, O, name, fs, 8, None, 41)
        sym = bufs[0]
        ref = O.demap_modcod(sym, mi, n0, gain)
        pts = mi["points"]
        d_re = torch.from_numpy(np.ascontiguousarray(pts.real, np.float32)).cuda()
        d_im = torch.from_numpy(np.ascontiguousarray(pts.imag, np.float32)).cuda()
        d_sym = torch.from_numpy(sym).cuda()
        d_out = torch.zeros((8, mi["fecframe_len"]), dtype=torch.int16, device="cuda")
        rg.demap(d_sym, d_out, d_re, d_im, mi, n0, gain, 8, s)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().astype(np.int32)
        diff = np.abs(got - ref.astype(np.int32))
        out.append({"modcod": name, "fs": fs, "esn0_db": round(esn0, 2), "llrs": int(diff.size),
                    "equal": int((diff == 0).sum()), "max_abs_diff": int(diff.max()),
                    "diff_hist": {str(int(k)): int(v) for k, v in zip(*np.unique(diff, return_counts=True))}})
    return out


def decode_section(torch, cs, E, O, rg, steps, warmup):
    out = []
    s = torch.cuda.current_stream()
    for label, name, fs, B, esn0, seed in DECODE_CASES:
        _, mod, rate, _, _, _ = E.find_modcod(name)
        mi0 = O.modcod(mod, rate, fs)
        batch_bytes = B * mi0["fecframe_len"] * 2
        nb = max(4, int(np.ceil(L2_BYTES / batch_bytes)))
        mod, rate, esn0, bufs, n0, gain, mi = traffic(cs, E, O, name, fs, B, esn0, seed, nb)
        llr0 = O.demap_modcod(bufs[0], mi, n0, gain)
        ho, to = O.ldpc_decode(fs, rate, llr0, 50, nthreads=os.cpu_count() or 8)
        # LLR batches on the device (this project's demapper, bit-exact with
        # the oracle's; checked on the first batch)
        dm = cs.demapper_cuda(mod, rate, fs, B)
        llrs = []
        for b in bufs:
            d = torch.zeros((B, mi["fecframe_len"]), dtype=torch.int16, device="cuda")
            dm.demap_launch(torch.from_numpy(b).cuda(), B, n0, gain, d, s)
            llrs.append(d)
        torch.cuda.synchronize()
        assert (llrs[0].cpu().numpy() == llr0).all(), "device LLRs differ from the oracle's"
        kb = O.code_info(fs, rate)["K"] // 8
        rdec = rg.decoder(fs, rate, 50, B)
        ours = cs.ldpc_decode_cuda(fs, rate, 50, B)
        rh = torch.zeros((B, kb), dtype=torch.uint8, device="cuda")
        rt = torch.zeros(B, dtype=torch.int32, device="cuda")
        oh = torch.zeros((B, kb), dtype=torch.uint8, device="cuda")
        ot = torch.zeros(B, dtype=torch.int32, device="cuda")
        runs = []
        for _ in range(2):
            rdec.launch(llrs[0], B, rh, rt, s)
            torch.cuda.synchronize()
            runs.append((rh.cpu().numpy().copy(), rt.cpu().numpy().copy()))
        ours.decode_launch_async(llrs[0], B, s, oh, ot)
        torch.cuda.synchronize()
        hg, tg = oh.cpu().numpy(), ot.cpu().numpy()
        (h1, t1), (h2, t2) = runs
        same_hard = ~(h1 != ho).any(axis=1)
        conv = (t1 >= 0) & (to >= 0)
        rec = {"workload": label, "modcod": name, "fs": fs, "frames": B, "esn0_db": round(esn0, 2),
               "ref_schedule_steps": rdec.n_steps,
               "oracle_failed": int((to < 0).sum()), "ref_failed": int((t1 < 0).sum()),
               "oracle_mean_iterations": float(np.mean(np.where(to >= 0, 50 - to, 50))),
               "ref_mean_iterations": float(np.mean(np.where(t1 >= 0, 50 - t1, 50))),
               "ref_vs_oracle_identical": int((same_hard & (t1 == to)).sum()),
               "ref_vs_oracle_same_hard": int(same_hard.sum()),
               "both_converged": int(conv.sum()),
               "both_converged_same_hard": int((conv & same_hard).sum()),
               "ref_run_to_run_identical": int((~(h1 != h2).any(axis=1) & (t1 == t2)).sum()),
               "ours_vs_oracle_identical": int((~(hg != ho).any(axis=1) & (tg == to)).sum())}
        # timing: the same LLR batches, one launch after another on one stream
        k_info = O.code_info(fs, rate)["K"]
        ms_ref = time_launches(torch, lambda i: rdec.launch(llrs[i], B, rh, rt, s), nb, steps, warmup)
        ms_ours = time_launches(torch, lambda i: ours.decode_launch_async(llrs[i], B, s, oh, ot), nb, steps,
                                warmup)
        rec["timing"] = {"batches_cycled": nb, "steps": steps, "warmup": warmup,
                         "ref_ms_per_launch": ms_ref, "ours_ms_per_launch": ms_ours,
                         "ref_info_gbps": B * k_info / (ms_ref * 1e6),
                         "ours_info_gbps": B * k_info / (ms_ours * 1e6),
                         "speedup": ms_ref / ms_ours}
        rdec.close()
        ours.close()
        out.append(rec)
        print(json.dumps(rec), file=sys.stderr)
    return out


def demap_timing(torch, cs, E, O, rg, steps, warmup):
    """Both demappers on the headline batch (256 normal 8PSK 3/5 frames)."""
    s = torch.cuda.current_stream()
    out = []
    for name, fs, B in [("8psk3/5", 0, 256), ("32apsk3/4", 0, 256), ("256apsk32/45", 0, 256)]:
        mod, rate, esn0, _, n0, gain, mi = traffic(cs, E, O, name, fs, B, None, 51)
        sym_bytes = B * mi["xfecframe_len"] * 8
        nb = max(4, int(np.ceil(L2_BYTES / sym_bytes)))
        _, _, _, bufs, _, _, _ = traffic(cs, E, O, name, fs, B, None, 51, nb)
        d_syms = [torch.from_numpy(b).cuda() for b in bufs]
        pts = mi["points"]
        d_re = torch.from_numpy(np.ascontiguousarray(pts.real, np.float32)).cuda()
        d_im = torch.from_numpy(np.ascontiguousarray(pts.imag, np.float32)).cuda()
        d_out = torch.zeros((B, mi["fecframe_len"]), dtype=torch.int16, device="cuda")
        dm = cs.demapper_cuda(mod, rate, fs, B)
        ms_ref = time_launches(torch, lambda i: rg.demap(d_syms[i], d_out, d_re, d_im, mi, n0, gain, B, s), nb,
                               steps, warmup)
        ms_ours = time_launches(torch, lambda i: dm.demap_launch(d_syms[i], B, n0, gain, d_out, s), nb, steps,
                                warmup)
        out.append({"modcod": name, "fs": fs, "frames": B, "batches_cycled": nb, "ref_ms_per_launch": ms_ref,
                    "ours_ms_per_launch": ms_ours, "speedup": ms_ref / ms_ours})
    return out


def mixed_section(torch, cs, O, rg, steps, warmup):
    """The bench's 1024-frame mixed batch (10 MODCODs, normal and short
    frames, seed 2025): this project's tuned graph replay (demap -> per-class
    decoders -> BCH) against the reference's kernels as its receive pool
    would run them -- one demap + decoder pair per MODCOD entry, each entry
    on its own stream, all entries concurrently -- one round at a time."""
    import bench
    T = 50
    mt = bench.MixedTraffic(cs, bench.MIXED["frames"], bench.MIXED["seed"])
    n = len(mt.frames)
    s0 = torch.cuda.Stream()  # graph capture needs a created stream
    # this project: one graph replay per round
    d_sym = torch.from_numpy(mt.sym).cuda()
    d_hard = torch.zeros(mt.hard_bytes, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros((2, n), dtype=torch.int32, device="cuda")
    b = cs.batch(mt.modcods, max_trials=T, max_frames=n)
    fr = mt.descriptors(cs, d_sym, d_hard, d_res[0], d_res[1])
    torch.cuda.synchronize()
    b.tune(fr, reps=3, stream=s0)
    b.capture(fr, s0)
    with torch.cuda.stream(s0):
        ms_ours = time_launches(torch, lambda i: b.replay(s0), 1, steps, warmup)
    ours_trials = d_res[0].cpu().numpy()
    hard_np = d_hard.cpu().numpy()
    # the reference: per MODCOD entry, its frames' symbols, demap and decoder
    groups = {}
    for f, frm in enumerate(mt.frames):
        groups.setdefault(frm["modcod"], []).append(f)
    ents = []
    for m, fids in groups.items():
        _, mod, rate, fs = mt.table[m]
        mi = O.modcod(mod, rate, fs)
        B = len(fids)
        sym = np.stack([mt.frames[f]["sym"].ravel() for f in fids]).astype(np.float32)
        pts = mi["points"]
        ent = {"fids": fids, "B": B, "mi": mi, "stream": torch.cuda.Stream(),
               "sym": torch.from_numpy(sym).cuda(),
               "re": torch.from_numpy(np.ascontiguousarray(pts.real, np.float32)).cuda(),
               "im": torch.from_numpy(np.ascontiguousarray(pts.imag, np.float32)).cuda(),
               "llr": torch.zeros((B, mi["fecframe_len"]), dtype=torch.int16, device="cuda"),
               "hard": torch.zeros((B, O.code_info(fs, rate)["K"] // 8), dtype=torch.uint8, device="cuda"),
               "res": torch.zeros(B, dtype=torch.int32, device="cuda"),
               "dec": rg.decoder(fs, rate, T, B), "n0": mt.frames[fids[0]]["n0"],
               "gain": O.capped_llr_gain(mi, mt.frames[fids[0]]["gain"])}
        ents.append(ent)
    torch.cuda.synchronize()

    def round_ref(_):
        start = torch.cuda.Event()
        start.record(s0)
        for e in ents:
            st = e["stream"]
            st.wait_event(start)
            rg.demap(e["sym"], e["llr"], e["re"], e["im"], e["mi"], e["n0"], e["gain"], e["B"], st)
            e["dec"].launch(e["llr"], e["B"], e["hard"], e["res"], st)
            done = torch.cuda.Event()
            done.record(st)
            s0.wait_event(done)

    with torch.cuda.stream(s0):
        ms_ref = time_launches(torch, round_ref, 1, steps, warmup)
    # agreement with this project's results (equal to the oracle's by the tests)
    same_hard = converged = 0
    for e in ents:
        rt = e["res"].cpu().numpy()
        rh = e["hard"].cpu().numpy()
        for k, f in enumerate(e["fids"]):
            kb = rh.shape[1]
            oh = hard_np[mt.hard_off[f]:mt.hard_off[f] + kb]
            converged += int(rt[k] >= 0 and ours_trials[f] >= 0)
            same_hard += int((rh[k] == oh).all())
    for e in ents:
        e["dec"].close()
    return {"frames": n, "modcod_entries": len(ents), "info_bits": int(mt.info_bits),
            "ours_ms_per_round": ms_ours, "ref_ms_per_round": ms_ref,
            "ours_info_gbps": mt.info_bits / (ms_ours * 1e6), "ref_info_gbps": mt.info_bits / (ms_ref * 1e6),
            "speedup": ms_ref / ms_ours, "both_converged": converged, "same_hard_bits": same_hard,
            "note": "one round at a time; ours = demap + decoders + BCH in one graph replay, ref = demap + "
                    "decoder per MODCOD entry on concurrent streams (no BCH)"}


# (MODCOD, frame size, Es/N0 dB, frames): near the waterfall of C1's and C2's codes
FER_POINTS = [("qpsk1/2", 1, 1.25, 51200), ("qpsk1/2", 1, 1.5, 51200), ("8psk3/5", 0, 5.5, 25600),
              ("8psk3/5", 0, 5.6, 25600), ("8psk3/5", 0, 5.7, 25600)]


def fer_section(torch, cs, rg, points=FER_POINTS, batch=256, seed=7):
    """Frame error rates of the reference decoder kernel and this project's
    decoder on the same LLRs: fresh random messages encoded, mapped and
    demapped on the GPU by this library (learned.ChannelPool), AWGN per
    frame, max 50 iterations; a frame error is any information bit wrong."""
    from cusat_gb300 import learned
    out = []
    s = torch.cuda.current_stream()
    for name, fs, esn0, n_frames in points:
        pool = learned.ChannelPool(name, fs, 0, seed, batch, torch)
        rate = pool.rate
        kb = cs.code_info(fs, rate)["k_ldpc"] // 8
        rdec = rg.decoder(fs, rate, 50, batch)
        ours = cs.ldpc_decode_cuda(fs, rate, 50, batch)
        rh = torch.zeros((batch, kb), dtype=torch.uint8, device="cuda")
        rt = torch.zeros(batch, dtype=torch.int32, device="cuda")
        oh = torch.zeros_like(rh)
        ot = torch.zeros_like(rt)
        err_ref = err_ours = fail_ref = fail_ours = it_ref = it_ours = 0
        for _ in range(n_frames // batch):
            _, llr, cw, _, _ = pool.draw(batch, esn0, s)
            rdec.launch(llr, batch, rh, rt, s)
            ours.decode_launch_async(llr, batch, s, oh, ot)
            info = cw[:, :kb]
            err_ref += int((rh != info).any(dim=1).sum())
            err_ours += int((oh != info).any(dim=1).sum())
            fail_ref += int((rt < 0).sum())
            fail_ours += int((ot < 0).sum())
            it_ref += int(torch.where(rt >= 0, 50 - rt, 50).sum())
            it_ours += int(torch.where(ot >= 0, 50 - ot, 50).sum())
        n = (n_frames // batch) * batch
        rdec.close()
        ours.close()
        rec = {"modcod": name, "fs": fs, "esn0_db": esn0, "frames": n,
               "ref_frame_errors": err_ref, "ours_frame_errors": err_ours,
               "ref_fer": err_ref / n, "ours_fer": err_ours / n,
               "ref_not_converged": fail_ref, "ours_not_converged": fail_ours,
               "ref_mean_iterations": it_ref / n, "ours_mean_iterations": it_ours / n}
        out.append(rec)
        print(json.dumps(rec), file=sys.stderr)
    return out


def profile_case(torch, cs, E, O, rg):
    """The headline batch (256 normal 3/5 8PSK frames at 6.0 dB): two
    launches of the reference decoder kernel, then two of this project's,
    on the same LLRs, one after another."""
    label, name, fs, B, esn0, seed = DECODE_CASES[0]
    mod, rate, esn0, bufs, n0, gain, mi = traffic(cs, E, O, name, fs, B, esn0, seed)
    s = torch.cuda.current_stream()
    dm = cs.demapper_cuda(mod, rate, fs, B)
    llr = torch.zeros((B, mi["fecframe_len"]), dtype=torch.int16, device="cuda")
    dm.demap_launch(torch.from_numpy(bufs[0]).cuda(), B, n0, gain, llr, s)
    kb = O.code_info(fs, rate)["K"] // 8
    h = torch.zeros((B, kb), dtype=torch.uint8, device="cuda")
    t = torch.zeros(B, dtype=torch.int32, device="cuda")
    rdec = rg.decoder(fs, rate, 50, B)
    ours = cs.ldpc_decode_cuda(fs, rate, 50, B)
    for _ in range(2):
        rdec.launch(llr, B, h, t, s)
    for _ in range(2):
        ours.decode_launch_async(llr, B, s, h, t)
    torch.cuda.synchronize()
    it = np.where(t.cpu().numpy() >= 0, 50 - t.cpu().numpy(), 50)
    print(json.dumps({"case": label, "frames": B, "mean_iterations": float(it.mean()),
                      "edges": int(cs.code_info(fs, rate)["edges"])}))
    rdec.close()
    ours.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--no-fer", action="store_true", help="skip the frame-error-rate comparison")
    ap.add_argument("--fer-only", action="store_true", help="run the frame-error-rate comparison alone")
    ap.add_argument("--fer-points", default="",
                    help="frame-error-rate points as MODCOD:framesize:EsN0:frames, comma-separated (default: "
                         "near the waterfall of C1's and C2's codes)")
    ap.add_argument("--profile-case", action="store_true",
                    help="only two launches of each decoder on the headline batch (for an ncu capture)")
    args = ap.parse_args()
    import torch

    import cusat_gb300 as cs
    import oracle_lib as O
    from cusat_gb300 import enums as E

    torch.cuda.set_device(0)
    rg = O.RefGpu()
    if args.profile_case:
        profile_case(torch, cs, E, O, rg)
        return
    points = FER_POINTS
    if args.fer_points:
        points = [(m, int(f), float(e), int(n)) for m, f, e, n in (x.split(":") for x in args.fer_points.split(","))]
    if args.fer_only:
        line = json.dumps({"gpu": torch.cuda.get_device_name(0), "fer": fer_section(torch, cs, rg, points)})
        print(line)
        if args.out:
            with open(args.out, "w") as f:
                f.write(line + "\n")
        return
    res = {"gpu": torch.cuda.get_device_name(0), "demap": demap_section(torch, cs, E, O, rg)}
    print(json.dumps(res["demap"]), file=sys.stderr)
    res["decode"] = decode_section(torch, cs, E, O, rg, args.steps, args.warmup)
    res["demap_timing"] = demap_timing(torch, cs, E, O, rg, args.steps, args.warmup)
    res["mixed"] = mixed_section(torch, cs, O, rg, args.steps, args.warmup)
    print(json.dumps(res["mixed"]), file=sys.stderr)
    if not args.no_fer:
        res["fer"] = fer_section(torch, cs, rg, points)
    line = json.dumps(res)
    print(line)
    if args.out:
        with open(args.out, "w") as f:
            f.write(line + "\n")


if __name__ == "__main__":
    main()
