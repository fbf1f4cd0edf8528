"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/_build/libfec_oracle.so`` -- the C restatement in fec_oracle.c.
* ``oracle/_ref/libcusat_ref_host.so`` -- when the reference tree is present
  (never on the GPU host), the reference's own host-side code for this path
  (code parameters, BCH generator/encoder, bit interleaver, constellations,
  table factory, message clamp) compiled unchanged from where it lies,
  together with ``ref_shim.cc`` (this project's extern "C" accessors), so
  that tests can compare the restatement with the reference itself.

Usage: python3 oracle/build.py   (also run by __graft_entry__.build()).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("CUSAT_REFERENCE_TREE", "/root/reference")
REF_SOURCES = [
    "lib/cusat_dsp/fec/code_params.cc",
    "lib/cusat_dsp/fec/bch_code.cc",
    "lib/cusat_dsp/modulation/bit_interleaver.cc",
    "lib/cusat_dsp/modulation/constellation.cc",
    "lib/cusat_dsp/ldpc_table_factory.cc",
    "lib/cusat_dsp/bb_scrambler.cc",
    "lib/cusat_dsp/bbframe_parser.cc",
    "lib/cusat_dsp/bb_header.cc",
    "lib/cusat_dsp/modulation/dd_snr.cc",
    "lib/cusat_dsp/framing/plframe.cc",
    "lib/cusat_dsp/framing/pl_scrambler.cc",
    "lib/cusat_dsp/framing/plheader.cc",
]


def _newer(out, deps):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_oracle(verbose=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libfec_oracle.so")
    deps = [os.path.join(HERE, "fec_oracle.c"), os.path.join(HERE, "fec_oracle.h"),
            os.path.join(HERE, "nms_model.inc"),
            os.path.join(HERE, "..", "cusat_gb300", "csrc", "cusat_data.h"),
            os.path.join(HERE, "..", "cusat_gb300", "csrc", "gen", "code_tables.inc")]
    if _newer(out, deps):
        return out
    cmd = ["gcc", "-std=c99", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", out + ".tmp", os.path.join(HERE, "fec_oracle.c"), "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build_ref(verbose=False):
    """Compile the reference's host code; returns the path or None if absent."""
    if not os.path.isdir(os.path.join(REF, "lib", "cusat_dsp")):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libcusat_ref_host.so")
    srcs = [os.path.join(REF, s) for s in REF_SOURCES]
    shim = os.path.join(HERE, "ref_shim.cc")
    # compiles plrx/pl_receiver.cc in place (its slot de-rotation is file-local)
    plrx_shim = os.path.join(HERE, "ref_plrx_shim.cc")
    if _newer(out, srcs + [shim, plrx_shim, os.path.join(REF, "lib", "cusat_dsp", "plrx", "pl_receiver.cc")]):
        return out
    inc = ["-I" + os.path.join(REF, "lib", "cusat_dsp"),
           "-I" + os.path.join(REF, "lib", "cusat_dsp", "include")]
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", *inc,
           "-o", out + ".tmp", shim, plrx_shim, *srcs]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


REF_KERNELS = {
    "ref_ldpc_decode.sm_103.cubin": "lib/cusat_dsp/cuda/ldpc_decode_kernel.cu",
    "ref_demap.sm_103.cubin": "lib/cusat_dsp/cuda/demapper_kernel.cu",
}
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def ref_cubin_paths():
    return {k: os.path.join(HERE, "_ref", k) for k in REF_KERNELS}


def build_ref_cubins(verbose=False):
    """Compile the reference's decoder and demapper kernels into cubins;
    returns the paths, or None when the reference tree or nvcc is absent."""
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.isdir(os.path.join(REF, "lib", "cusat_dsp")) or not os.path.exists(nvcc):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    inc = ["-I" + os.path.join(REF, "lib", "cusat_dsp", "include"), "-I" + os.path.join(REF, "lib", "cusat_dsp")]
    outs = ref_cubin_paths()
    for name, src in REF_KERNELS.items():
        out, src = outs[name], os.path.join(REF, src)
        if _newer(out, [src]):
            continue
        # CMake Release flags of the reference (-O3 -DNDEBUG, C++17) for
        # CMAKE_CUDA_ARCHITECTURES=103
        cmd = [nvcc, "-O3", "-DNDEBUG", "-std=c++17", "-gencode", "arch=compute_103,code=sm_103", "-cubin",
               *inc, "-o", out + ".tmp", src]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        os.replace(out + ".tmp", out)
    return outs


def build_ref_gpu(verbose=False):
    """Compile ref_gpu.c (driver-API launcher of the reference cubins);
    returns the path, or None without the CUDA headers."""
    cuda_h = os.path.join(CUDA_HOME, "include", "cuda.h")
    if not os.path.exists(cuda_h):
        return None
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libref_gpu.so")
    src = os.path.join(HERE, "ref_gpu.c")
    deps = [src, os.path.join(HERE, "..", "cusat_gb300", "csrc", "cusat_data.h"),
            os.path.join(HERE, "..", "cusat_gb300", "csrc", "gen", "code_tables.inc")]
    if _newer(out, deps):
        return out
    libdirs = [os.path.join(CUDA_HOME, "lib64", "stubs"), os.path.join(CUDA_HOME, "lib64")]
    cmd = ["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-I" + os.path.join(CUDA_HOME, "include"),
           "-o", out + ".tmp", src, *["-L" + d for d in libdirs], "-lcuda"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(verbose=True))
    print(build_ref_cubins(verbose=True))
    print(build_ref_gpu(verbose=True))
    sys.exit(0)
