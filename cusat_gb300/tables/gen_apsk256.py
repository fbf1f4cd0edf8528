#!/usr/bin/env python3
"""Regenerate ``cusat_gb300/csrc/gen/apsk256_points.inc`` from the reference tree.

DVB-S2X defines the 256APSK constellations of code rates 2/3 (20/30) and
11/15-L (22/30) by explicit coordinates (ETSI EN 302 307-2 Table 15d), not
by rings.  The reference keeps the standard's printed values as two float
arrays (``lib/cusat_dsp/modulation/apsk256_points.h``, one ``{I, Q}`` row
per 8-bit label).  A drop-in demapper must use the very same points, so this
script parses those arrays and re-emits them as flat C data (I, Q
interleaved, label order) with the same decimal literals, hence the same
float values.

Checks performed before anything is written:
  * both tables have 256 rows and every row's comment is its own label in
    binary (the label order is the standard's);
  * every value has at most four decimals, as printed in the standard;
  * the mean energy per point of each table is within 1e-3 of 1 (the
    printed values are unit energy up to their four decimals; the product
    still renormalises them, as the reference does).

Usage:  python3 cusat_gb300/tables/gen_apsk256.py --ref REFERENCE_TREE (or CUSAT_REFERENCE_TREE set) [--out FILE]
"""
import argparse
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "csrc", "gen", "apsk256_points.inc")
TABLES = [("APSK256_POINTS_20_30", "cusat_apsk256_20_30"), ("APSK256_POINTS_22_30", "cusat_apsk256_22_30")]


def parse(text, name):
    i = text.index(name + "[256][2] = {")
    j = text.index("};", i)
    rows = re.findall(r"\{\s*(-?\d+\.\d+)f,\s*(-?\d+\.\d+)f\s*\},\s*//\s*([01]{8})", text[i:j])
    assert len(rows) == 256, (name, len(rows))
    for label, (re_s, im_s, bits) in enumerate(rows):
        assert int(bits, 2) == label, (name, label, bits)
        assert len(re_s.split(".")[1]) <= 4 and len(im_s.split(".")[1]) <= 4, (name, label)
    e = sum(float(a) ** 2 + float(b) ** 2 for a, b, _ in rows) / 256
    assert abs(e - 1.0) < 1e-3, (name, e)
    return [(a, b) for a, b, _ in rows]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CUSAT_REFERENCE_TREE"), required="CUSAT_REFERENCE_TREE" not in os.environ,
                    help="root of the reference source tree")
    ap.add_argument("--out", default=OUT)
    args = ap.parse_args()
    text = open(os.path.join(args.ref, "lib/cusat_dsp/modulation/apsk256_points.h")).read()
    out = ["/* Generated by cusat_gb300/tables/gen_apsk256.py -- do not edit.",
           " *",
           " * DVB-S2X 256APSK explicit-coordinate constellations (ETSI EN 302 307-2",
           " * Table 15d) for code rates 20/30 and 22/30, as printed in the standard",
           " * (four decimals, unit energy up to rounding): I, Q of label 0, then",
           " * label 1, ... label 255.",
           " */", ""]
    for src, dst in TABLES:
        pts = parse(text, src)
        out.append(f"static const float {dst}[512] = {{")
        for k in range(0, 256, 4):
            out.append("    " + " ".join(f"{a}f, {b}f," for a, b in pts[k:k + 4]))
        out.append("};")
        out.append("")
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    with open(args.out, "w") as f:
        f.write("\n".join(out))
    print("wrote", os.path.normpath(args.out))


if __name__ == "__main__":
    main()
