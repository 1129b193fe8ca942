"""Drift control of the fast updates (periodic full rebuild of M).

The reference rebuilds the inverse hybridisation matrices exactly only in
global moves and set_mc_config (Trace.F90:2279-2336, MatrixUpdate.F90:41-99);
between those the Sherman-Morrison updates of StepAdd/StepRem accumulate
rounding.  The engine rebuilds every chain's matrices by Gauss-Jordan
elimination after every `refresh_every` accepted pair updates, records the
largest deviation of the fast-updated matrices and log-determinant from the
rebuilt ones, and continues with the rebuilt ones.  The rebuild draws no
random numbers, so the proposal stream stays the oracle's.
"""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import problems as P

from test_gpu_parity import _diag_of, _offdiag_problem, compare_logs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return E.load(build_if_missing=True)


def test_drift_bounded_at_beta_100_over_1e5_updates(lib):
    """3-orbital density-density model at beta = 100 (the largest expansion
    orders of the batched configuration), 8 chains x 1e5 proposals with a
    rebuild every 1000 accepted updates: every rebuild finds the fast-updated
    M within 1e-9 of the exact inverse (absolute, for entries of order 1-100)
    and log|det| within 1e-9, with no sign disagreement; after the run the
    installed matrices still agree with a fresh rebuild."""
    pr = P.config_problem("dd3", beta=100.0)
    m = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(m, [E.Group(100.0, pr["ftau"], 50, nchains=8, seed0=100, taudiff_max=5.0,
                            kcap=64, opcap=1024, refresh_every=1000)])
    b.warmup(100000)
    b.sync()
    d = b.drift()
    st = [b.state(c) for c in range(8)]
    acc = sum(b.results(c)["counters"]["acc_add"] + b.results(c)["counters"]["acc_rem"] for c in range(8))
    assert d["refreshes"] >= acc // 1000 - 8
    assert d["refreshes"] > 20, d
    assert d["sign_errors"] == 0, d
    assert d["max_dev_m"] < 1e-9, d
    assert d["max_dev_logdet"] < 1e-9, d
    assert min(s["noper"] for s in st) > 40  # expansion orders of beta = 100
    assert b.refresh_minv(replace=False) < 1e-9
    print(f"\ndrift at beta=100: {d}, mean operators {np.mean([s['noper'] for s in st]):.1f}")
    d2 = b.drift(reset=True)
    assert d2["refreshes"] == d["refreshes"]
    assert b.drift()["refreshes"] == 0


def test_frequent_rebuilds_keep_the_proposal_stream(lib):
    """A rebuild after every 20 accepted updates: the proposal stream,
    decisions and weights still match the oracle (which never rebuilds)
    proposal by proposal."""
    pr = P.config_problem("dd3", beta=25.0)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    co = O.Chain(mo, 25.0, pr["ftau"], 50, seed=21, taudiff_max=5.0, p_outer=0.1)
    co.start_log(6000)
    co.warmup(6000)
    ref = co.log()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(25.0, pr["ftau"], 50, nchains=1, seed0=21, taudiff_max=5.0, p_outer=0.1,
                             kcap=64, opcap=512, refresh_every=20)])
    b.set_log(6000)
    b.warmup(6000)
    b.sync()
    compare_logs(ref, b.log(0), pr["ftau"][0, 0], 25.0)
    d = b.drift()
    assert d["refreshes"] > 10 and d["sign_errors"] == 0 and d["max_dev_m"] < 1e-10, d


def test_offdiag_rebuilds_keep_the_proposal_stream(lib):
    """Off-diagonal hybridisation: the full matrix over all flavours is
    rebuilt in block order after every 10 accepted updates; the stream
    matches the oracle and the deviations stay at rounding level."""
    nd, beta, um, muimp, ff, qns = _offdiag_problem("orbital")
    mo = O.Model(nd, um, muimp, qns)
    co = O.Chain(mo, beta, ff, 10, seed=31, taudiff_max=-1.0, p_outer=0.1, ncorr=20, maxhisto=30)
    co.start_log(4000)
    co.warmup(4000)
    ref = co.log()
    mg = E.Model(nd, um, muimp, qns)
    b = E.Batch(mg, [E.Group(beta, _diag_of(ff), 10, nchains=1, seed0=31, taudiff_max=-1.0, p_outer=0.1,
                             ncorr=20, maxhisto=30, kcap=64, opcap=256, ftau_full=ff, refresh_every=10)])
    b.set_log(4000)
    b.warmup(4000)
    b.sync()
    compare_logs(ref, b.log(0))
    d = b.drift()
    assert d["refreshes"] > 5 and d["sign_errors"] == 0 and d["max_dev_m"] < 1e-10, d
    mo_, mg_ = co.minv_full(), b.minv_full(0)
    if mo_.size:
        assert np.allclose(mg_, mo_, rtol=1e-9, atol=1e-9 * np.abs(mo_).max())


def test_rebuilds_can_be_switched_off(lib):
    pr = P.config_problem("dd3", beta=10.0)
    m = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(m, [E.Group(10.0, pr["ftau"], 20, nchains=2, seed0=3, taudiff_max=5.0, refresh_every=-1)])
    b.warmup(20000)
    b.sync()
    assert b.drift()["refreshes"] == 0
