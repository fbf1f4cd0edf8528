"""The launcher of the reference's own GPU kernels (oracle/ref_gpu.c) builds
and exports its entry points; where the reference tree is present, its
decoder and demapper sources compile into the cubins the launcher loads.
No GPU is used here (tests/test_gpu_reference_kernels.py runs the kernels)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build as oracle_build  # noqa: E402  (oracle/build.py)

sys.path.pop(0)

ENTRY_POINTS = ["rg_open", "rg_last_error", "rg_dec_create", "rg_dec_destroy", "rg_dec_info", "rg_dec_launch",
                "rg_demap_launch"]


def test_launcher_exports_its_entry_points():
    so = oracle_build.build_ref_gpu()
    if so is None:
        pytest.skip("cuda.h not available")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    names = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in ENTRY_POINTS if n not in names]
    assert not missing, f"missing exports: {missing}"


def test_reference_cubins_build_where_the_tree_is():
    outs = oracle_build.build_ref_cubins()
    if outs is None:
        pytest.skip("reference tree or nvcc not present")
    for path in outs.values():
        with open(path, "rb") as f:
            assert f.read(4) == b"\x7fELF", f"{path} is not a cubin"
