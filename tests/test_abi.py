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
        E.Model(1, np.zeros((2, 2, 2, 2)), np.zeros((1, 2, 1, 2)), "All")
    with pytest.raises(E.EngineError):
        E.Model(9, np.zeros((18,) * 4), np.zeros((9, 2, 9, 2)), "Nt")


def test_error_message_api(lib):
    lib.cthyb_batch_sync.argtypes = [C.c_void_p]
    rc = lib.cthyb_batch_sync(None)
    assert rc == -1
    assert b"null" in lib.cthyb_last_error()
