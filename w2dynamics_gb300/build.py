"""Build the GB300 CT-HYB engine (in-tree shared library, sm_103a only).

    python -m w2dynamics_gb300.build

produces w2dynamics_gb300/_build/libcthyb_gpu.so from csrc/engine.cu and
csrc/model.cpp with `nvcc -gencode arch=compute_103a,code=sm_103a`.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcthyb_gpu.so")
SOURCES = ("engine.cu", "engine.cuh", "model.cpp", "model.h")
HEADER = os.path.join(os.path.dirname(HERE), "include", "cthyb_gpu.h")


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + [HEADER]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, out=None, defines=()):
    """Compile the engine; `out`/`defines` build a variant (e.g. another
    SWEEP_MIN_BLOCKS register budget) next to the default library."""
    lib = out or LIB
    if out is None and not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = lib + ".tmp"
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
           "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", tmp,
           *[f"-D{d}" for d in defines],
           os.path.join(CSRC, "engine.cu"), os.path.join(CSRC, "model.cpp")]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
