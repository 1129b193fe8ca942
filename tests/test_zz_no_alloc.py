"""Allocation-free inverse hybridisation matrix (cthyb_minv_rebuild_noalloc).

For callers that cannot call cudaMalloc themselves -- e.g. a solver whose
device memory was sized at start-up -- the library offers one entry point
whose work space is a static device array.  It is checked here, through the
C ABI, against the matrices the regular entry point (set_mc_config followed
by cthyb_batch_minv) produces for the same operator times, on two calls in a
row that share the static array.  Tolerance as in the parity tests: 1e-9
relative on M, 1e-10 on log|det|.
"""
import ctypes as C

import numpy as np
import pytest

from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import problems as P


def _reference(pr, beta, taus_c, taus_a, b, s):
    """M and log|det| from the regular entry points (one flavour only)."""
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    k = len(taus_c)
    batch = E.Batch(mg, [E.Group(beta, pr["ftau"], 20, nchains=1, seed0=1, taudiff_max=beta,
                                 kcap=max(64, k + 4), opcap=max(512, 2 * k + 8))])
    taus = np.concatenate([taus_c, taus_a])
    orbs = np.full(2 * k, b + 1)
    spins = np.full(2 * k, s + 1)
    cas = np.concatenate([np.ones(k, int), np.full(k, 2)])
    batch.set_config(0, taus, orbs, spins, cas, 0)
    M = batch.minv(0, 2 * b + s)
    st = batch.state(0)
    return M, st["det_log"], st["det_sign"]


def _noalloc(torch, lib, beta, taus_c, taus_a, F):
    dev = torch.device("cuda:0")
    k = len(taus_c)
    tc = torch.tensor(np.sort(taus_c), dtype=torch.float64, device=dev)
    ta = torch.tensor(np.sort(taus_a), dtype=torch.float64, device=dev)
    f = torch.tensor(F, dtype=torch.float64, device=dev)
    minv = torch.empty(max(k * k, 1), dtype=torch.float64, device=dev)
    logdet = torch.empty(2, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.cthyb_minv_rebuild_noalloc(k, C.c_void_p(tc.data_ptr()), C.c_void_p(ta.data_ptr()),
                                        C.c_void_p(f.data_ptr()), len(F), beta,
                                        C.c_void_p(minv.data_ptr()), C.c_void_p(logdet.data_ptr()),
                                        None)
    assert rc == 0, lib.cthyb_last_error()
    torch.cuda.synchronize()
    return minv[:k * k].cpu().numpy().reshape((k, k), order="F"), logdet.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    lib = E.load(build_if_missing=True)
    beta = 10.0
    pr = P.config_problem("dd3", beta=beta)
    rng = np.random.default_rng(7)
    for k, (b, s) in ((6, (1, 0)), (17, (2, 1))):  # two calls in a row, different sizes
        taus = np.sort(rng.uniform(0.0, beta, 2 * k))
        rng.shuffle(taus)
        taus_c, taus_a = np.sort(taus[:k]), np.sort(taus[k:])
        M_ref, dlog_ref, dsign_ref = _reference(pr, beta, taus_c, taus_a, b, s)
        M, ld = _noalloc(torch, lib, beta, taus_c, taus_a, pr["ftau"][b, s])
        assert np.allclose(M, M_ref, rtol=1e-9, atol=1e-9 * np.abs(M_ref).max())
        assert abs(ld[0] - dlog_ref) <= 1e-10 * max(1.0, abs(dlog_ref))
        assert ld[1] == dsign_ref


def test_noalloc_rejects_oversized_k():
    """Host-side argument check only (no kernel is launched), so it runs
    without a GPU as well."""
    lib = E.load(build_if_missing=True)
    rc = lib.cthyb_minv_rebuild_noalloc(257, None, None, None, 10, 1.0, None, None, None)
    assert rc == -3
    assert b"static scratch limit of 256" in lib.cthyb_last_error()
