"""bench.py's host side, without a GPU: both arms build the same traffic and
print the same config, and the reference arm (the oracle on the host cores)
loads no library of this project."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_traffic_equals_product_traffic(built_lib):
    import bench
    for wl in (bench.WORKLOAD, bench.WORKLOAD_SHORT):
        a = bench.make_traffic(dict(wl, frames=8), 2, bench.ProductGen())
        b = bench.make_traffic(dict(wl, frames=8), 2, bench.OracleGen())
        assert (a[1] == b[1]).all()
        for x, y in zip(a[2], b[2]):
            assert x.dtype == y.dtype == np.float32 and (x.view(np.uint32) == y.view(np.uint32)).all()
        assert a[3] == b[3] and a[4] == b[4]
        assert bench.n_bufs_for(wl, bench.ProductGen()) == bench.n_bufs_for(wl, bench.OracleGen())


def test_oracle_mixed_traffic_equals_product_traffic(built_lib):
    import bench
    import cusat_gb300 as cs
    a = bench.MixedTraffic(cs, 48, 7)
    b = bench.MixedTraffic(None, 48, 7, bench.OracleGen())
    assert a.table == b.table and a.geo == b.geo
    assert (a.sym.view(np.uint32) == b.sym.view(np.uint32)).all()


def test_reference_arm_loads_only_the_oracle():
    code = (
        "import sys, json, types; sys.argv = ['bench.py']; import bench\n"
        "args = types.SimpleNamespace(gpus=1, steps=1, warmup=0, cpu_sample=2, learned=False)\n"
        "bench.reference_arm(args, dict(bench.WORKLOAD))\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'so': 'libcusat_fec' in maps, 'oracle': 'libfec_oracle' in maps}))\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(ln) for ln in out.stdout.splitlines() if ln.startswith("{")]
    line, maps = lines[0], lines[-1]
    assert maps == {"so": False, "oracle": True}
    assert line["impl"] == "reference" and line["value"] > 0
    import bench
    wl = dict(bench.WORKLOAD)
    nb = bench.n_bufs_for(wl, bench.OracleGen())
    sym_bytes = wl["frames"] * bench.OracleGen().modcod_info(wl["mod"], wl["rate"], wl["fs"])["xfecframe_len"] * 8
    assert line["config"] == bench.single_config(wl, nb, sym_bytes)


def test_pl_workload_traffic(built_lib):
    """bench.py's PLFRAME builder (pilots + scrambling) equals the oracle's,
    and the oracle's receiver tail recovers the XFECFRAMEs exactly."""
    import bench
    import cusat_gb300 as cs
    import oracle_lib as O
    ci, msg, bufs, n0, gain = bench.make_traffic(dict(bench.WORKLOAD, frames=3), 1)
    pay, lay = bench.pl_frames(cs, bufs[0], (12 << 2) | 1, 0)
    r = O.pl_rotation(0, lay["payload_symbols"])
    for f in range(3):
        assert np.array_equal(pay[f], O.pl_frame_payload(bufs[0][f], lay["slots"], 1, r))
        assert np.array_equal(O.pl_extract(pay[f], lay["slots"], 1, r), bufs[0][f])
