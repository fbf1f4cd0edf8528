"""The header-only C++ shims (include/cusat_fec.hpp) compile against the
reference's signatures, link against the library, and (on a GPU) reproduce
the reference's lib/qa_ldpc_encode.cc round trip."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path, lib):
    exe = str(tmp_path / "shim_roundtrip")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "shim_roundtrip.cc"), "-o", exe, lib, "-L", os.path.join(CUDA, "lib64"),
           "-L", os.path.join(CUDA, "targets", "sbsa-linux", "lib"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(built_lib, tmp_path):
    assert os.path.exists(_build(tmp_path, built_lib))


@pytest.mark.gpu
def test_shim_roundtrip_on_gpu(cuda, built_lib, tmp_path):
    exe = _build(tmp_path, built_lib)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stderr + r.stdout


def _build_chain(tmp_path, lib):
    import oracle_lib as O
    O.lib()  # builds the oracle library
    orc = os.path.join(ROOT, "oracle", "_build")
    exe = str(tmp_path / "shim_chain")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           "-I", os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "shim_chain.cc"), "-o", exe, lib,
           os.path.join(orc, "libfec_oracle.so"), "-L", os.path.join(CUDA, "lib64"),
           "-L", os.path.join(CUDA, "targets", "sbsa-linux", "lib"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib) + ":" + orc]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_chain_and_pool_shims_compile(built_lib, tmp_path):
    assert os.path.exists(_build_chain(tmp_path, built_lib))


@pytest.mark.gpu
def test_chain_and_pool_shims_on_gpu(cuda, built_lib, tmp_path):
    """GSE payloads through the C++ pool (MODCOD runs) and chain shims come
    back in submission order."""
    exe = _build_chain(tmp_path, built_lib)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stderr + r.stdout
