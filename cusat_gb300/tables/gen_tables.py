#!/usr/bin/env python3
"""Regenerate ``cusat_gb300/csrc/gen/code_tables.inc`` from the reference tree.

The DVB-S2/S2X LDPC codes are defined by the accumulator-address tables of
ETSI EN 302 307-1 Annex B/C and EN 302 307-2 Annex B/C.  The reference keeps
them as constexpr C++ arrays (``lib/cusat_dsp/ldpc_tables/dvb_s2_tables.h``,
``dvb_s2x_tables.h``) with a sha256 manifest (``ldpc_tables/checksums.txt``),
and the parallel-layer schedules of its decoder as generated headers
(``lib/cusat_dsp/cuda/ldpc_schedules/*.h``).  Both are data that a drop-in
decoder must reproduce exactly, so this script parses them and re-emits the
numbers in this project's own flat C layout (one ``cusat_table_src`` per code,
one ``cusat_sched_src`` per scheduled code).

Checks performed before anything is written:
  * every table's canonical content hashes to the manifest entry
    (the manifest rule of ``scripts/check_ldpc_tables.py``: a first line
    ``"<name> N=<n> K=<k> M=<m>"`` then one line of addresses per row);
  * the structural invariants (R divisible by 360, addresses < R,
    links_total = 360*sum(deg) + 2R - 1, links_max_cn);
  * every schedule covers each layer once and never pairs parity-chain
    neighbours (|a-b| <= 1 mod q);
  * the rate -> schedule registry (``ldpc_schedule_registry.h``) and the
    rate -> table factory (``ldpc_table_factory.cc``) agree on the table.

Usage:  python3 cusat_gb300/tables/gen_tables.py --ref REFERENCE_TREE (or CUSAT_REFERENCE_TREE set)
"""
import argparse
import hashlib
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "csrc", "gen", "code_tables.inc")
M = 360


def parse_tables(path):
    text = open(path).read()
    arrays = {}
    for mm in re.finditer(r"inline constexpr (?:uint8_t|uint16_t|uint32_t) (\w+)\[\] = \{(.*?)\};",
                          text, re.S):
        arrays[mm.group(1)] = [int(x) for x in mm.group(2).replace(",", " ").split()]
    codes = []
    for mm in re.finditer(r"inline constexpr ldpc_code (\w+) = \{\s*(\d+), (\d+), (\d+), (\d+), (\d+), (\d+),",
                          text):
        name = mm.group(1)
        n, k, m, lt, lmc, n_rows = (int(mm.group(i)) for i in range(2, 8))
        deg, off, addr = arrays[name + "_deg"], arrays[name + "_off"], arrays[name + "_addr"]
        assert len(deg) == n_rows and len(off) == n_rows + 1 and off[-1] == len(addr)
        rows = [addr[off[r]:off[r + 1]] for r in range(n_rows)]
        assert [len(r) for r in rows] == deg
        codes.append(dict(name=name, n=n, k=k, m=m, lt=lt, lmc=lmc, rows=rows))
    return codes


def canonical(c):
    parts = [f"{c['name']} N={c['n']} K={c['k']} M={c['m']}"]
    for row in c["rows"]:
        parts.append(" ".join(str(a) for a in row))
    return "\n".join(parts) + "\n"


def check_code(c):
    n, k, m = c["n"], c["k"], c["m"]
    r = n - k
    assert m == M and r % M == 0 and k == len(c["rows"]) * M, c["name"]
    q = r // M
    for row in c["rows"]:
        assert 0 < len(row) < 256
        for a in row:
            assert 0 <= a < r
    assert c["lt"] == M * sum(len(x) for x in c["rows"]) + 2 * r - 1, c["name"]
    cnc = [0] * r
    for row in c["rows"]:
        for j in range(M):
            for a in row:
                cnc[(a + j * q) % r] += 1
    assert c["lmc"] == max(cnc) + 2, c["name"]


def parse_schedule(path):
    t = open(path).read()
    name = os.path.basename(path)[len("ldpc_schedule_"):-2]
    steps = int(re.search(r"_STEPS = (\d+);", t).group(1))
    q = int(re.search(r"_Q\s*= (\d+);", t).group(1))
    body = t[t.index("] = {") + 5:]
    body = body[:body.index("};")]
    nums = [int(x) for x in re.findall(r"-?\d+", body)]
    pairs = list(zip(nums[0::2], nums[1::2]))
    assert len(pairs) == steps
    return name, q, pairs


def check_schedule(q, pairs):
    seen = sorted(x for p in pairs for x in p if x >= 0)
    assert seen == list(range(q))
    for a, b in pairs:
        assert a >= 0
        if b >= 0:
            d = abs(a - b)
            assert not (d <= 1 or d >= q - 1), (a, b)


def rate_maps(ref):
    fac = open(os.path.join(ref, "lib/cusat_dsp/ldpc_table_factory.cc")).read()
    normal = fac[fac.index("FECFRAME_NORMAL"):fac.index("FECFRAME_SHORT")]
    fac_map = dict(re.findall(r"case (RATE_\w+):\s*return &(\w+);", normal))
    reg = open(os.path.join(ref, "lib/cusat_dsp/cuda/ldpc_schedules/ldpc_schedule_registry.h")).read()
    reg_map = {r: s.lower() for r, s in re.findall(r"case (RATE_\w+): return \{ (\w+), ", reg)}
    return fac_map, reg_map


def wrap(vals, per=20):
    return "\n".join("    " + ", ".join(str(v) for v in vals[i:i + per]) + ","
                     for i in range(0, len(vals), per))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CUSAT_REFERENCE_TREE"), required="CUSAT_REFERENCE_TREE" not in os.environ,
                    help="root of the reference source tree")
    ap.add_argument("--out", default=OUT)
    a = ap.parse_args()
    tdir = os.path.join(a.ref, "lib/cusat_dsp/ldpc_tables")
    codes = parse_tables(os.path.join(tdir, "dvb_s2_tables.h")) + \
        parse_tables(os.path.join(tdir, "dvb_s2x_tables.h"))
    manifest = {}
    for line in open(os.path.join(tdir, "checksums.txt")):
        if line.startswith("#") or not line.strip():
            continue
        h, name = line.split()
        manifest[name] = h
    for c in codes:
        check_code(c)
        got = hashlib.sha256(canonical(c).encode()).hexdigest()
        assert got == manifest[c["name"]], f"{c['name']}: checksum mismatch"
    assert len(codes) == len(manifest)

    sdir = os.path.join(a.ref, "lib/cusat_dsp/cuda/ldpc_schedules")
    scheds = {}
    for f in sorted(os.listdir(sdir)):
        if f.startswith("ldpc_schedule_s2"):
            name, q, pairs = parse_schedule(os.path.join(sdir, f))
            check_schedule(q, pairs)
            scheds[name] = (q, pairs)
    fac_map, reg_map = rate_maps(a.ref)
    for rate, sched in reg_map.items():
        assert fac_map[rate] == sched, (rate, fac_map[rate], sched)
    by_name = {c["name"]: c for c in codes}
    for name, (q, _) in scheds.items():
        c = by_name[name]
        assert (c["n"] - c["k"]) // M == q

    out = ["/* Generated by cusat_gb300/tables/gen_tables.py -- do not edit.",
           " *",
           " * DVB-S2 / DVB-S2X LDPC accumulator-address tables (ETSI EN 302 307-1",
           " * Annex B/C, EN 302 307-2 Annex B/C) and the paired-layer decoding",
           " * schedules of the reference decoder, re-emitted as flat C data.",
           " * Row r of a table lists the accumulator addresses of information bits",
           " * r*360 .. r*360+359 (bit r*360+j updates parity (a + j*q) mod (N-K)).",
           " * Every table was checked against the reference sha256 manifest.",
           " */", ""]
    for c in codes:
        nm = c["name"]
        deg = [len(r) for r in c["rows"]]
        addr = [x for r in c["rows"] for x in r]
        out += [f"static const uint8_t cusat_tab_{nm}_deg[{len(deg)}] = {{", wrap(deg), "};",
                f"static const uint16_t cusat_tab_{nm}_addr[{len(addr)}] = {{", wrap(addr, 16), "};"]
    for nm, (q, pairs) in scheds.items():
        flat = [x for p in pairs for x in p]
        out += [f"static const int16_t cusat_sched_{nm}[{len(flat)}] = {{", wrap(flat), "};"]
    out += ["", "static const cusat_table_src cusat_table_srcs[] = {"]
    for c in codes:
        nm = c["name"]
        out.append(f'    {{"{nm}", {c["n"]}, {c["k"]}, {len(c["rows"])}, {c["lt"]}, {c["lmc"]}, '
                   f"cusat_tab_{nm}_deg, cusat_tab_{nm}_addr}},")
    out += ["};", f"#define CUSAT_N_TABLE_SRCS {len(codes)}", "",
            "static const cusat_sched_src cusat_sched_srcs[] = {"]
    for nm, (q, pairs) in scheds.items():
        out.append(f'    {{"{nm}", {q}, {len(pairs)}, cusat_sched_{nm}}},')
    out += ["};", f"#define CUSAT_N_SCHED_SRCS {len(scheds)}", ""]
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    with open(a.out, "w") as f:
        f.write("\n".join(out))
    print(f"OK: {len(codes)} tables match the manifest, {len(scheds)} schedules -> {a.out}")


if __name__ == "__main__":
    sys.exit(main())
