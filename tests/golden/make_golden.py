"""Generate the golden fixtures in tests/golden/ from the w2dynamics reference.

Run where the reference sources are present (they are not needed
afterwards); their root directory comes from --reference-root, else the
environment variable W2DYNAMICS_SRC, else /root/reference:

    python oracle/build_oracle.py [--reference-root DIR]    # oracle/_ref/librandom_ref.so
    python tests/golden/make_golden.py [--reference-root DIR]

Writes
  * umatrices.npz: U matrices produced by the reference's own
    w2dyn/dmft/interaction.py (Density and Kanamori) for the benchmark
    problems and a few small ones;
  * rng_streams.npz: uniform reals and bounded integers drawn through the
    reference's src/mtrng/random.cc (compiled unchanged from the reference
    sources into oracle/_ref/) for several seeds and ranges, including an
    interleaved sequence shaped like the draws of one pair proposal;
  * bath_legendre.npz: F(tau) of the discrete baths of the exact-
    diagonalisation tests from the reference's
    w2dyn/auxiliaries/transform.py (hybr_from_sites), and its Legendre-to-tau
    matrix (leg2tau), which fixes the G_l normalisation.
"""
import ctypes as C
import os
import sys

import numpy as np

REF = os.environ.get("W2DYNAMICS_SRC") or "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def umatrices():
    sys.path.insert(0, REF)
    import w2dyn.dmft.interaction as I  # reference code, used only here
    out = {}
    cases = {
        "density_1_2.0_2.0_0.0": ("Density", 1, 2.0, 2.0, 0.0),
        "density_2_3.0_2.0_0.5": ("Density", 2, 3.0, 2.0, 0.5),
        "density_3_4.0_2.8_0.6": ("Density", 3, 4.0, 2.8, 0.6),
        "kanamori_2_3.0_1.6_0.7": ("Kanamori", 2, 3.0, 1.6, 0.7),
        "kanamori_3_4.0_2.8_0.6": ("Kanamori", 3, 4.0, 2.8, 0.6),
        "kanamori_5_3.0_1.6_0.7": ("Kanamori", 5, 3.0, 1.6, 0.7),
    }
    for key, (kind, nd, u, v, j) in cases.items():
        cls = getattr(I, kind)
        obj = cls(nd, u, v, j)
        out[key] = obj.convert_u_matrix()
        out[key + "_autoqn"] = np.array(" ".join(obj.auto_quantum_numbers))
    return out


def rng_streams():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "librandom_ref.so"))
    lib.new_random.restype = C.c_void_p
    lib.seed_random.argtypes = [C.c_void_p, C.c_uint]
    lib.get_random.argtypes = [C.c_void_p]
    lib.get_random.restype = C.c_double
    lib.get_randint.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.get_randint.restype = C.c_int
    lib.delete_random.argtypes = [C.c_void_p]
    out = {}
    for seed in (0, 1, 42, 4095):
        r = lib.new_random()
        lib.seed_random(r, seed)
        out[f"reals_{seed}"] = np.array([lib.get_random(r) for _ in range(1000)])
        lib.delete_random(r)
        for lo, hi in ((1, 1), (1, 2), (1, 3), (1, 5), (8, 16), (1, 1000), (1, 123457)):
            r = lib.new_random()
            lib.seed_random(r, seed)
            out[f"ints_{seed}_{lo}_{hi}"] = np.array([lib.get_randint(r, lo, hi) for _ in range(400)],
                                                     dtype=np.int32)
            lib.delete_random(r)
        # interleaved: move draws, pair draws, accept, removal index
        r = lib.new_random()
        lib.seed_random(r, seed)
        seq = []
        for i in range(400):
            seq.append(lib.get_random(r))
            seq.append(lib.get_random(r))
            seq.append(lib.get_random(r))
            seq.append(float(lib.get_randint(r, 1, 3)))
            seq.append(float(lib.get_randint(r, 1, 2)))
            seq.append(lib.get_random(r))
            seq.append(float(lib.get_randint(r, 1, 7 + (i % 50))))
        out[f"mixed_{seed}"] = np.array(seq)
        lib.delete_random(r)
    return out


def bath_legendre():
    sys.path.insert(0, REF)
    import w2dyn.auxiliaries.transform as T  # reference code, used only here
    beta, ntau = 4.0, 201
    tau = np.linspace(0.0, beta, ntau)
    iw = T.matfreq(beta, "fermi", 10)
    eps = np.array([-0.6, 0.9])
    out = {}
    # one orbital, both spins coupled with V_b to every level (rows: levels)
    out["single"] = T.hybr_from_sites(eps, np.array([[0.6], [0.8]]), iw, tau, beta)[1]
    # spinless levels with spin-dependent amplitudes V_{b s}
    out["offdiag"] = T.hybr_from_sites(eps, np.array([[0.6, 0.3], [0.5, -0.4]]), iw, tau, beta)[1]
    # two orbitals, spinful levels eps_b: mode (b, s) couples to flavour
    # 2 o + s with V_{b o}
    eps2, v2 = np.array([-0.5, 0.7]), [[0.6, 0.3], [0.4, -0.5]]
    vki = np.zeros((4, 4))
    for b in range(2):
        for s in range(2):
            for o in range(2):
                vki[2 * b + s, 2 * o + s] = v2[b][o]
    out["spinful"] = T.hybr_from_sites(np.repeat(eps2, 2), vki, iw, tau, beta)[1]
    out["leg2tau"] = T.leg2tau(beta, 40, np.linspace(0.0, beta, 41))
    out["beta"] = np.array(beta)
    return out


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=None, help="root of the w2dynamics sources")
    a = ap.parse_args()
    if a.reference_root:
        REF = a.reference_root
    np.savez_compressed(os.path.join(HERE, "umatrices.npz"), **umatrices())
    np.savez_compressed(os.path.join(HERE, "rng_streams.npz"), **rng_streams())
    np.savez_compressed(os.path.join(HERE, "bath_legendre.npz"), **bath_legendre())
    print("written")
