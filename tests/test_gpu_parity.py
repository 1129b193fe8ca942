"""Proposal-by-proposal parity of the GPU engine with the oracle.

The GPU chain and the oracle chain start from the same seed, so they draw the
same proposals (the device generator reproduces std::mt19937 and the
standard-library distributions of src/mtrng/random.cc).  For every proposal
the move type, flavour, times, FPos, NPairs, outcome and superstate must be
bit-identical; the determinant ratio and the new trace must agree to 1e-10
relative (|delta log| <= 1e-10), the acceptance probability to 1e-10.
"""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import problems as P

pytestmark = pytest.mark.gpu

EXACT = ("move", "outcome", "orb", "spin", "change_outer", "fpos_c", "fpos_a", "npairs",
         "outer_sst", "k_total", "tau_c", "tau_a", "rand")
RTOL = 1e-10


@pytest.fixture(scope="module")
def lib():
    return E.load(build_if_missing=True)


def run_pair(name, beta, tdm, p_outer, nprop, seed, dense=False, qns=None, ntau=50):
    pr = P.config_problem(name, beta=beta)
    q = qns or pr["quantum_numbers"]
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    co = O.Chain(mo, beta, pr["ftau"], ntau, seed=seed, taudiff_max=tdm, p_outer=p_outer)
    co.start_log(nprop)
    co.warmup(nprop)
    ref = co.log()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    grp = E.Group(beta, pr["ftau"], ntau, nchains=1, seed0=seed, taudiff_max=tdm,
                  p_outer=p_outer, dense=dense, kcap=64, opcap=512)
    b = E.Batch(mg, [grp])
    b.set_log(nprop)
    b.warmup(nprop)
    b.sync()
    got = b.log(0)
    return ref, got, co, b


def compare_logs(ref, got):
    assert len(got) == len(ref)
    for key in EXACT:
        bad = np.nonzero(ref[key] != got[key])[0]
        assert len(bad) == 0, (key, bad[:5], ref[bad[:3]], got[bad[:3]])
    evald = ref["outcome"] >= 3
    for key in ("det_log", "tr_log"):
        d = np.abs(ref[key][evald] - got[key][evald])
        scale = np.maximum(1.0, np.abs(ref[key][evald])) if key == "tr_log" else 1.0
        assert np.all(d <= RTOL * scale), (key, d.max())
    for key in ("det_sign", "tr_sign"):
        assert np.array_equal(ref[key][evald], got[key][evald])
    p = evald & (ref["prob"] > 0)
    assert np.all(np.abs(got["prob"][p] / ref["prob"][p] - 1.0) <= 1e-9)


CASES = [
    ("anderson1", 10.0, 10.0, 0.0, 20000, 0, False, None),
    ("anderson1", 10.0, 3.0, 0.2, 20000, 7, False, None),
    ("dd3", 10.0, 10.0, 0.0, 8000, 1, False, None),
    ("dd3", 25.0, 5.0, 0.1, 8000, 3, False, None),
    ("dd3", 10.0, 4.0, 0.1, 3000, 2, True, None),
    ("dd3", 8.0, 8.0, 0.0, 3000, 5, False, "Nt"),
    ("kanamori5", 2.0, 2.0, 0.0, 300, 4, False, None),
]


@pytest.mark.parametrize("name,beta,tdm,pout,nprop,seed,dense,qns", CASES)
def test_proposal_stream_parity(lib, name, beta, tdm, pout, nprop, seed, dense, qns):
    ref, got, co, b = run_pair(name, beta, tdm, pout, nprop, seed, dense=dense, qns=qns)
    compare_logs(ref, got)
    # final configuration and inverse matrices
    so, sg = co.state(), b.state(0)
    assert so["noper"] == sg["noper"] and so["outer_sst"] == sg["outer_sst"]
    assert so["npairs"] == sg["npairs"] and so["cfgsign"] == sg["cfgsign"]
    assert abs(so["det_log"] - sg["det_log"]) < 1e-8
    t_o, *_ = co.get_config()
    t_g, *_ = b.get_config(0)
    assert np.array_equal(t_o, t_g)
    nf = 2 * co.model.nd
    for f in range(nf):
        mo_, mg_ = co.minv(f), b.minv(0, f)
        assert mo_.shape == mg_.shape
        if mo_.size:
            assert np.allclose(mg_, mo_, rtol=1e-9, atol=1e-9 * np.abs(mo_).max())


def test_measurement_parity(lib):
    """G(tau), sign, histogram and density matrix of one chain equal the
    oracle's to rounding (identical proposal streams)."""
    pr = P.config_problem("dd3", beta=10.0)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    co = O.Chain(mo, 10.0, pr["ftau"], 40, seed=9, taudiff_max=5.0, p_outer=0.1, ncorr=50)
    co.warmup(2000)
    co.measure(300)
    ro = co.results()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 40, nchains=1, seed0=9, taudiff_max=5.0,
                             p_outer=0.1, ncorr=50, kcap=64, opcap=512)])
    b.warmup(2000)
    b.measure(300)
    b.sync()
    rg = b.results(0)
    assert rg["mean_sign"] == ro["mean_sign"]
    go = ro["gtau"]  # [f][tau], f = 2b+s
    gg = np.stack([rg["gtau"][f // 2, f % 2] for f in range(6)])
    assert np.allclose(gg, go, rtol=1e-9, atol=1e-12)
    assert np.allclose(np.diag(rg["densitymatrix"]), np.diag(ro["densitymatrix"]), rtol=1e-9, atol=1e-12)
    ho = ro["histo"]
    hg = np.stack([rg["histo"][f // 2, f % 2] for f in range(6)])
    assert np.array_equal(hg[:, :ho.shape[1]], ho)


def test_batched_chains_match_oracle_per_seed(lib):
    """Every chain of a batch is the reference chain of its own seed."""
    pr = P.config_problem("dd3", beta=10.0)
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    n = 64
    b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 20, nchains=n, seed0=100, taudiff_max=5.0,
                             kcap=64, opcap=512)])
    b.warmup(3000)
    b.sync()
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    for c in (0, 17, 63):
        co = O.Chain(mo, 10.0, pr["ftau"], 20, seed=100 + c, taudiff_max=5.0)
        co.warmup(3000)
        t_o, *_ = co.get_config()
        t_g, *_ = b.get_config(c)
        assert np.array_equal(t_o, t_g), c


def test_set_config_and_refresh(lib):
    """set_mc_config: trace and determinant of a fixed configuration equal
    the oracle's; the LU refresh of fast-updated M shows only rounding drift."""
    pr = P.config_problem("dd3", beta=10.0)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    co = O.Chain(mo, 10.0, pr["ftau"], 20, seed=21, taudiff_max=10.0)
    co.warmup(4000)
    t, o, s, c = co.get_config()
    outer = int(co.state()["outer_sst"])
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 20, nchains=1, seed0=21, taudiff_max=10.0,
                             kcap=64, opcap=512)])
    b.set_config(0, t, o, s, c, outer)
    sg = b.state(0)
    ft = co.full_trace()
    fd = co.full_det()
    assert abs(sg["trace_log"] - ft[0]) < 1e-10 * max(1, abs(ft[0]))
    assert sg["trace_sign"] == ft[1]
    assert abs(sg["det_log"] - fd[0]) < 1e-10 * max(1, abs(fd[0]))
    assert sg["det_sign"] == fd[1]
    b.warmup(5000)
    dev = b.refresh_minv(replace=False)
    assert dev < 1e-9
