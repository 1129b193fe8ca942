"""Build recipe for the oracle (test infrastructure only).

Compiles
  * oracle/cthyb_oracle.cpp  -> oracle/_build/libcthyb_oracle.so (the CPU
    restatement of the w2dynamics pair-move loop, used only by tests/, the
    smoke check and bench.py's CPU-baseline leg), and
  * when the w2dynamics sources are present (their root directory from
    --reference-root, else the environment variable W2DYNAMICS_SRC, else
    /root/reference):
    src/mtrng/random.cc -> oracle/_ref/librandom_ref.so, the reference's own
    random-number wrapper compiled unchanged from where it lies, used to pin
    the oracle's proposal stream.

Run: python oracle/build_oracle.py [--reference-root DIR]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF_ROOT = "/root/reference"


def reference_root(arg=None):
    """Root directory of the w2dynamics sources (may not exist)."""
    return arg or os.environ.get("W2DYNAMICS_SRC") or DEFAULT_REF_ROOT


def _compile(src, out, extra=()):
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", out, src, *extra]
    subprocess.check_call(cmd)
    return out


def build(verbose=False, ref_root=None):
    lib = _compile(os.path.join(HERE, "cthyb_oracle.cpp"),
                   os.path.join(HERE, "_build", "libcthyb_oracle.so"))
    ref = None
    ref_random = os.path.join(reference_root(ref_root), "src", "mtrng", "random.cc")
    if os.path.exists(ref_random):
        ref = _compile(ref_random, os.path.join(HERE, "_ref", "librandom_ref.so"),
                       extra=("-std=c++11",))
    if verbose:
        print(lib, ref)
    return lib, ref


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=None, help="root of the w2dynamics sources")
    build(verbose=True, ref_root=ap.parse_args().reference_root)
    sys.exit(0)
