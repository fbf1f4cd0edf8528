"""The serving loop's arena allocator (header-only C++), compiled alone and
run on the host: randomised allocations and releases never overlap, stay in
range, account exactly and coalesce back to one block."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_arena_allocator(tmp_path):
    exe = str(tmp_path / "arena_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "cusat_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "arena_check.cc"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_copy_crew(tmp_path):
    """The receive chain's split frame copy (copy_crew.h), compiled alone:
    byte-exact copies of every size, crews used before their helper threads
    start, many consecutive jobs, wake-up after sleeping, clean shutdown."""
    exe = str(tmp_path / "copy_crew_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "cusat_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "copy_crew_check.cc"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
