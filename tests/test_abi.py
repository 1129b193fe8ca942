"""C-ABI boundary and host logic of the GPU library (no GPU needed).

* the shared library builds for sm_103a, loads, and exports every function
  include/cthyb_gpu.h declares;
* the host-side model (superstates, Connect table, eigenvalues, monomial
  detection) agrees with the oracle's restatement of init_solver.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    return E.load(build_if_missing=True)


def test_exports_every_declared_symbol(lib):
    hdr = open(os.path.join(ROOT, "include", "cthyb_gpu.h")).read()
    declared = set(re.findall(r"\b(cthyb_[a-z_0-9]+)\s*\(", hdr))
    assert declared, "no declarations found"
    assert declared == set(E.EXPORTS)
    raw = C.CDLL(E.library_path())
    for name in declared:
        assert hasattr(raw, name), name


@pytest.mark.parametrize("name,qns", [
    ("anderson1", None), ("dd3", None), ("dd3", "Nt"), ("kanamori5", None),
    ("dd3", "All"), ("dd3", "Nt All"), ("kanamori5", "Nt All"),
])
def test_host_model_matches_oracle(lib, name, qns):
    pr = P.config_problem(name, beta=5.0)
    q = qns or pr["quantum_numbers"]
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    assert mg.nsst == mo.nsst and mg.nstates == mo.nstates and mg.nsmax == mo.nsmax
    assert np.array_equal(mg.sst_size, mo.sst_size)
    assert np.array_equal(mg.sst_offset, mo.sst_offset)
    assert np.allclose(mg.evals, mo.evals, rtol=0, atol=1e-11)
    assert abs(mg.egs - mo.egs) < 1e-11
    for sst in range(mg.nsst):
        for b in range(pr["nd"]):
            for s in range(2):
                for ca in range(2):
                    assert mg.connect(sst, b + 1, s + 1, ca + 1) == mo.connect(sst, b, s, ca)
    expect_mono = name != "kanamori5"
    assert bool(mg.monomial) == expect_mono


def test_model_rejects_bad_input(lib):
    with pytest.raises(E.EngineError):
        E.Model(9, np.zeros((18,) * 4), np.zeros((9, 2, 9, 2)), "Nt")


def _hopping_model(t):
    """Two orbitals, density-density U = 2, mu = 1, inter-orbital hopping t
    of either spin (muimp off the orbital diagonal)."""
    nd = 2
    um = P.flat_umatrix(P.umatrix_density(nd, 2.0, 2.0, 0.0))
    mu = P.muimp_solver(nd, 1.0).copy()
    for s in range(2):
        mu[0, s, 1, s] = mu[1, s, 0, s] = t
    return nd, um, mu


def _blocks(m):
    """Superstates as sets of Fock states (occupation-basis order)."""
    fk, _ = m.basis()
    return [frozenset(int(x) for x in fk[o:o + n]) for o, n in zip(m.sst_offset, m.sst_size)]


def test_automatic_partitioning_known_answers(lib):
    """QuantumNumbers "All" (analyze_hamiltonian, Operator.F90:303-442):
    * a density-density model has a diagonal Hamiltonian, so every Fock
      state is its own block;
    * with inter-orbital hopping, "Nt All" gives the (N_up, N_dn) sectors
      (numbered by the nets found inside each Nt superstate) and the
      eigenvalues of the "Nt Szt" model;
    * a hopping below EPSBLOCK (relative to the largest entry of muimp and
      U) is ignored, and a smaller EPSBLOCK token keeps it;
    * "All" alone starts from one superstate, which no operator may
      connect to itself, so its Hamiltonian is empty and every state is its
      own block (as in the reference, whose Hamiltonian is built from the
      superstate connections);
    * engine and oracle agree on every partition."""
    pr = P.config_problem("dd3", beta=5.0)
    for q in ("All", "Nt All"):
        m = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
        assert m.nsst == 64 and m.nsmax == 1
    nd, um, mu = _hopping_model(-0.3)
    ma = E.Model(nd, um, mu, "Nt All")
    mq = E.Model(nd, um, mu, "Nt Szt")
    assert set(_blocks(ma)) == set(_blocks(mq)) and ma.nsst == 9
    assert [len(b) for b in _blocks(ma)] == [1, 2, 2, 1, 4, 1, 2, 2, 1]
    assert np.allclose(np.sort(ma.evals), np.sort(mq.evals), rtol=0, atol=1e-12)
    assert E.Model(nd, um, mu, "All").nsst == 16
    nd, um, mu = _hopping_model(-3e-14)  # 1.5e-14 of the largest entry
    assert E.Model(nd, um, mu, "Nt All").nsst == 16
    assert set(_blocks(E.Model(nd, um, mu, "Nt All EPSBLOCK=1e-15"))) == set(_blocks(mq))
    for t, q in ((-0.3, "All"), (-0.3, "Nt All"), (-3e-14, "Nt All"), (-3e-14, "Nt All EPSBLOCK=1e-15")):
        nd, um, mu = _hopping_model(t)
        mg, mo = E.Model(nd, um, mu, q), O.Model(nd, um, mu, q)
        assert mg.nsst == mo.nsst and np.array_equal(mg.sst_size, mo.sst_size), (t, q)
        assert np.allclose(mg.evals, mo.evals, rtol=0, atol=1e-11)


def test_automatic_partitioning_refines_the_given_quantum_numbers(lib):
    """"Nt All" for the 5-orbital Kanamori model: every block lies inside
    one "Nt Szt" block (the Hamiltonian conserves Sz), the blocks close
    under every creator and annihilator (a connection table exists), and
    the Hamiltonian has no entry between blocks (the eigenvalues of the
    blocks are those of the "Nt Szt" blocks they refine)."""
    pr = P.config_problem("kanamori5", beta=5.0)
    ma = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], "Nt All")
    mq = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], "Nt Szt")
    coarse = _blocks(mq)
    for blk in _blocks(ma):
        assert any(blk <= c for c in coarse)
    assert ma.nsst >= mq.nsst
    assert np.allclose(np.sort(ma.evals), np.sort(mq.evals), rtol=0, atol=1e-10)


def test_error_message_api(lib):
    lib.cthyb_batch_sync.argtypes = [C.c_void_p]
    rc = lib.cthyb_batch_sync(None)
    assert rc == -1
    assert b"null" in lib.cthyb_last_error()
