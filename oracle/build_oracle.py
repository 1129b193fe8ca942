"""Build recipe for the oracle (test infrastructure only).

Compiles
  * oracle/cthyb_oracle.cpp  -> oracle/_build/libcthyb_oracle.so (the CPU
    restatement of the w2dynamics pair-move loop, used only by tests/, the
    smoke check and bench.py's CPU-baseline leg), and
  * when the w2dynamics sources are present at /root/reference:
    src/mtrng/random.cc -> oracle/_ref/librandom_ref.so, the reference's own
    random-number wrapper compiled unchanged from where it lies, used to pin
    the oracle's proposal stream.

Run: python oracle/build_oracle.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_RANDOM = "/root/reference/src/mtrng/random.cc"


def _compile(src, out, extra=()):
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", out, src, *extra]
    subprocess.check_call(cmd)
    return out


def build(verbose=False):
    lib = _compile(os.path.join(HERE, "cthyb_oracle.cpp"),
                   os.path.join(HERE, "_build", "libcthyb_oracle.so"))
    ref = None
    if os.path.exists(REF_RANDOM):
        ref = _compile(REF_RANDOM, os.path.join(HERE, "_ref", "librandom_ref.so"),
                       extra=("-std=c++11",))
    if verbose:
        print(lib, ref)
    return lib, ref


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
