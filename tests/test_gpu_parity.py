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


def run_pair(name, beta, tdm, p_outer, nprop, seed, dense=False, qns=None, ntau=50, p_global=0.0,
             p_shift=0.0, symmoves=None, p_4op=0.0, tree_levels=0):
    pr = P.config_problem(name, beta=beta)
    q = qns or pr["quantum_numbers"]
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    co = O.Chain(mo, beta, pr["ftau"], ntau, seed=seed, taudiff_max=tdm, p_outer=p_outer,
                 p_global=p_global, p_shift=p_shift, symmoves=symmoves, p_4op=p_4op)
    co.start_log(nprop)
    co.warmup(nprop)
    ref = co.log()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    grp = E.Group(beta, pr["ftau"], ntau, nchains=1, seed0=seed, taudiff_max=tdm,
                  p_outer=p_outer, dense=dense, kcap=64, opcap=512, p_global=p_global,
                  p_shift=p_shift, symmoves=symmoves, p_4op=p_4op, tree_levels=tree_levels)
    b = E.Batch(mg, [grp])
    b.set_log(nprop)
    b.warmup(nprop)
    b.sync()
    got = b.log(0)
    return ref, got, co, b


def hybrf(F, beta, tau):
    """get_HybrF (Trace.F90:1014-1033) in numpy, vectorised over tau."""
    tau = np.asarray(tau, np.float64)
    sig = np.where(tau < 0, -1.0, 1.0)
    t = np.where(tau < 0, tau + beta, tau)
    n = t / beta * (len(F) - 1)
    i = np.minimum(n.astype(np.int64), len(F) - 2)
    return sig * (F[i] + (n - np.floor(n)) * (F[i + 1] - F[i]))


def cancellation(ref, F, beta):
    """|S| / |ratio| for insertions (S = Delta(tau_a - tau_c)), 1 otherwise.

    The ratio S - R.M.Q loses about log10(C) digits to cancellation in any
    floating-point evaluation, the reference's included."""
    S = np.abs(hybrf(F, beta, ref["tau_a"] - ref["tau_c"]))
    C = S / np.exp(ref["det_log"])
    return np.where(ref["move"] == 0, np.maximum(C, 1.0), 1.0)


def compare_logs(ref, got, F=None, beta=None):
    assert len(got) == len(ref)
    for key in EXACT:
        bad = np.nonzero(ref[key] != got[key])[0]
        assert len(bad) == 0, (key, bad[:5], ref[bad[:3]], got[bad[:3]])
    evald = ref["outcome"] >= 3
    C = cancellation(ref, F, beta)[evald] if F is not None else 1.0
    # ratios: 1e-10 relative, widened by the cancellation factor C of the
    # proposal (2e-14 * C: unit rounding times a few accumulated updates)
    d = np.abs(ref["det_log"][evald] - got["det_log"][evald])
    assert np.all(d <= RTOL + 2e-14 * C), ("det_log", d.max())
    d = np.abs(ref["tr_log"][evald] - got["tr_log"][evald])
    assert np.all(d <= RTOL * np.maximum(1.0, np.abs(ref["tr_log"][evald]))), ("tr_log", d.max())
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


GLOBAL_CASES = [
    ("anderson1", 10.0, 3.0, 0.1, 20000, 12, False, None),
    ("dd3", 10.0, 4.0, 0.1, 8000, 13, False, None),
    ("dd3", 25.0, 5.0, 0.0, 6000, 14, False, None),
    ("dd3", 10.0, 4.0, 0.1, 2000, 15, True, None),
    ("dd3", 8.0, 8.0, 0.0, 3000, 16, False, "Nt"),
]


@pytest.mark.parametrize("name,beta,levels,dense,nprop,moves", [
    ("dd3", 10.0, -1, False, 6000, dict(p_global=0.05, p_shift=0.05)),
    ("dd3", 25.0, -1, False, 6000, dict(p_4op=0.1)),
    ("dd3", 10.0, -1, True, 2000, dict(p_global=0.05, p_shift=0.05)),
    ("dd3", 50.0, 4, False, 8000, dict(p_global=0.02, p_shift=0.02)),
    ("kanamori5", 2.0, -1, False, 300, {}),
])
def test_tree_depth_keeps_the_proposal_stream(lib, name, beta, levels, dense, nprop, moves):
    """The time-bin tree's depth is a schedule choice: a single leaf (every
    proposal walks all operators, no combine steps) and a deep tree leave
    the proposal stream equal to the oracle's, global, tau-shift and
    4-operator moves included (one-chain batches also run with their chain
    state in shared memory)."""
    ref, got, co, b = run_pair(name, beta, 4.0 if beta <= 25 else 5.0, 0.1, nprop, 31, dense=dense,
                               tree_levels=levels, **moves)
    F = P.config_problem(name, beta=beta)["ftau"][0, 0]
    compare_logs(ref, got, F, beta)
    assert (ref["outcome"] == 4).sum() > 20
    so, sg = co.state(), b.state(0)
    assert so["noper"] == sg["noper"] and so["outer_sst"] == sg["outer_sst"]
    assert abs(so["trace_log"] - sg["trace_log"]) <= 1e-9 * max(1.0, abs(so["trace_log"]))


def test_automatic_partition_proposal_stream(lib):
    """QuantumNumbers "Nt All" (automatic block partitioning) for two
    orbitals with inter-orbital hopping in H_loc (dense blocks): the
    superstates of the engine and the oracle agree and the proposal stream
    with outer-superstate, global and tau-shift moves matches proposal by
    proposal."""
    nd, beta, ntau = 2, 8.0, 20
    um = P.flat_umatrix(P.umatrix_density(nd, 2.0, 2.0, 0.0))
    mu = P.muimp_solver(nd, 1.0).copy()
    for sp in range(2):
        mu[0, sp, 1, sp] = mu[1, sp, 0, sp] = -0.3
    ff = P.semicircle_ftau(nd, beta, 1.0, 1000)
    moves = dict(p_outer=0.1, p_global=0.02, p_shift=0.02)
    mo = O.Model(nd, um, mu, "Nt All")
    co = O.Chain(mo, beta, ff, ntau, seed=41, taudiff_max=4.0, **moves)
    co.start_log(4000)
    co.warmup(4000)
    ref = co.log()
    mg = E.Model(nd, um, mu, "Nt All")
    assert mg.nsst == mo.nsst == 9 and np.array_equal(mg.sst_size, mo.sst_size)
    b = E.Batch(mg, [E.Group(beta, ff, ntau, nchains=1, seed0=41, taudiff_max=4.0, kcap=64, opcap=512, **moves)])
    b.set_log(4000)
    b.warmup(4000)
    b.sync()
    compare_logs(ref, b.log(0), ff[0, 0], beta)
    assert (ref["outcome"] == 4).sum() > 100


@pytest.mark.parametrize("name,beta,tdm,pout,nprop,seed,dense,qns", GLOBAL_CASES)
def test_global_and_shift_move_parity(lib, name, beta, tdm, pout, nprop, seed, dense, qns):
    """Global moves (StepGlob) and tau-shift moves (StepShiftTau) at 5 %
    each, proposal by proposal; the final state and inverse matrices."""
    # user symmetry moves for the 3-orbital model: a cyclic orbital permutation
    sym = [[2, 3, 1, 5, 6, 4], [2, 1, 3, 5, 4, 6]] if name == "dd3" else None
    ref, got, co, b = run_pair(name, beta, tdm, pout, nprop, seed, dense=dense, qns=qns,
                               p_global=0.05, p_shift=0.05, symmoves=sym)
    F = P.config_problem(name, beta=beta)["ftau"][0, 0]
    compare_logs(ref, got, F, beta)
    for mv in (2, 3):
        assert np.sum((ref["move"] == mv) & (ref["outcome"] == 4)) > 0, mv
    if sym is not None:
        assert np.sum((ref["move"] == 2) & (ref["orb"] == 2)) > 0  # user symmetry moves drawn
    mc = b.move_counters(0)
    oc = co.counters()
    for key in ("try_glob", "acc_glob", "qn_glob", "try_shift", "acc_shift"):
        assert mc[key] == oc[key], key
    so, sg = co.state(), b.state(0)
    assert so["noper"] == sg["noper"] and so["outer_sst"] == sg["outer_sst"]
    assert so["cfgsign"] == sg["cfgsign"] and so["det_sign"] == sg["det_sign"]
    assert abs(so["det_log"] - sg["det_log"]) < 1e-8
    assert so["window_position"] == sg["window_position"]
    t_o, *_ = co.get_config()
    t_g, *_ = b.get_config(0)
    assert np.array_equal(t_o, t_g)
    for f in range(2 * co.model.nd):
        mo_, mg_ = co.minv(f), b.minv(0, f)
        assert mo_.shape == mg_.shape
        if mo_.size:
            assert np.allclose(mg_, mo_, rtol=1e-9, atol=1e-9 * np.abs(mo_).max())


FOUR_CASES = [
    ("anderson1", 10.0, 3.0, 0.1, 20000, 31, False),
    ("dd3", 10.0, 4.0, 0.1, 6000, 32, False),
    ("dd3", 25.0, 5.0, 0.0, 4000, 33, False),
    ("dd3", 10.0, 4.0, 0.1, 2000, 34, True),
    ("kanamori5", 2.0, 2.0, 0.0, 400, 35, False),
]


@pytest.mark.parametrize("name,beta,tdm,pout,nprop,seed,dense", FOUR_CASES)
def test_four_operator_move_parity(lib, name, beta, tdm, pout, nprop, seed, dense):
    """4-operator moves (StepAdd4 / StepRem4) at 30 % of the insertions and
    removals, with global and tau-shift moves at 2 % each, proposal by
    proposal (the first pair's times, both flavours, the removable-pair
    counts of each proposal, outcome, ratios); the final configuration,
    state, move counters and inverse matrices."""
    ref, got, co, b = run_pair(name, beta, tdm, pout, nprop, seed, dense=dense,
                               p_global=0.02, p_shift=0.02, p_4op=0.3)
    F = P.config_problem(name, beta=beta)["ftau"][0, 0]
    compare_logs(ref, got, F, beta)
    for mv in (5, 6):
        assert np.sum((ref["move"] == mv) & (ref["outcome"] == 4)) > 0, mv
    mc = b.move_counters(0)
    oc = co.counters()
    for key in ("try_add4", "acc_add4", "try_rem4", "acc_rem4", "try_glob", "acc_glob"):
        assert mc[key] == oc[key], key
    so, sg = co.state(), b.state(0)
    assert so["noper"] == sg["noper"] and so["outer_sst"] == sg["outer_sst"]
    assert so["cfgsign"] == sg["cfgsign"] and so["det_sign"] == sg["det_sign"]
    assert so["npairs"] == sg["npairs"] or so["npairs"] == -1 or sg["npairs"] == -1
    assert abs(so["det_log"] - sg["det_log"]) < 1e-8
    t_o, *_ = co.get_config()
    t_g, *_ = b.get_config(0)
    assert np.array_equal(t_o, t_g)
    for f in range(2 * co.model.nd):
        mo_, mg_ = co.minv(f), b.minv(0, f)
        assert mo_.shape == mg_.shape
        if mo_.size:
            assert np.allclose(mg_, mo_, rtol=1e-9, atol=1e-9 * np.abs(mo_).max())


@pytest.mark.parametrize("name,beta,tdm,pout,nprop,seed,dense,qns", CASES)
def test_proposal_stream_parity(lib, name, beta, tdm, pout, nprop, seed, dense, qns):
    ref, got, co, b = run_pair(name, beta, tdm, pout, nprop, seed, dense=dense, qns=qns)
    F = P.config_problem(name, beta=beta)["ftau"][0, 0]
    compare_logs(ref, got, F, beta)
    C = cancellation(ref, F, beta)[ref["outcome"] >= 3]
    # the plain 1e-10 bound holds for every well-conditioned proposal
    assert np.mean(C < 5e3) > 0.98
    # final configuration and inverse matrices
    so, sg = co.state(), b.state(0)
    assert so["noper"] == sg["noper"] and so["outer_sst"] == sg["outer_sst"]
    # NPairs is -1 ("recount before use") right after a window shift
    assert sg["npairs"] == -1 or so["npairs"] == sg["npairs"]
    assert so["cfgsign"] == sg["cfgsign"]
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
    """G(tau), sign, histogram, density matrix, Legendre G_l and the outer
    superstate/state histograms of one chain (global and tau-shift moves at
    1 % each) equal the oracle's to rounding (identical proposal streams)."""
    pr = P.config_problem("dd3", beta=10.0)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    co = O.Chain(mo, 10.0, pr["ftau"], 40, seed=9, taudiff_max=5.0, p_outer=0.1, ncorr=50,
                 p_global=0.01, p_shift=0.01, nleg=12)
    co.warmup(2000)
    co.measure(300)
    ro = co.results()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 40, nchains=1, seed0=9, taudiff_max=5.0,
                             p_outer=0.1, ncorr=50, kcap=64, opcap=512, p_global=0.01,
                             p_shift=0.01, nleg=12)])
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
    # Legendre coefficients and outer-state histograms
    xo, xg = co.results_extra(), b.results_extra(0)
    gl = np.stack([xg["gleg"][f // 2, f % 2] for f in range(6)])
    assert np.allclose(gl, xo["gleg"], rtol=1e-9, atol=1e-12 * np.abs(xo["gleg"]).max())
    for key in ("outer_sst_histo", "outer_state_histo"):
        assert np.array_equal(xg[key], xo[key]), key
    for key in ("sign_sst", "sign_state"):
        assert np.allclose(xg[key], xo[key], rtol=1e-12, atol=1e-12, equal_nan=True), key
    for key in ("contrib_sst", "contrib_state"):
        assert np.allclose(xg[key], xo[key], rtol=1e-9, atol=1e-300), key


@pytest.mark.parametrize("name,beta,dense,nprop", [("dd3", 10.0, True, 1500), ("kanamori5", 2.0, False, 200)])
def test_dense_block_trace_and_density_matrix(lib, name, beta, dense, nprop):
    """Dense-block models (block products with bin-edge checkpoints): the
    proposal stream, G(tau) and the full density matrix (superstate blocks,
    compared in the occupation basis) equal the oracle's."""
    pr = P.config_problem(name, beta=beta)
    q = pr["quantum_numbers"]
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    co = O.Chain(mo, beta, pr["ftau"], 30, seed=31, taudiff_max=beta / 2, ncorr=20, p_outer=0.1,
                 p_global=0.02, p_shift=0.02)
    co.start_log(nprop + 20 * 30)
    co.warmup(nprop)
    co.measure(30)
    ref = co.log()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], 30, nchains=1, seed0=31, taudiff_max=beta / 2, ncorr=20,
                             p_outer=0.1, dense=dense, kcap=64, opcap=512, p_global=0.02,
                             p_shift=0.02, tree_levels=3)])
    b.set_log(nprop + 20 * 30)
    b.warmup(nprop)
    b.measure(30)
    b.sync()
    got = b.log(0)
    F = pr["ftau"][0, 0]
    compare_logs(ref, got, F, beta)
    ro, rg = co.results(), b.results(0)
    nf = 2 * pr["nd"]
    gg = np.stack([rg["gtau"][f // 2, f % 2] for f in range(nf)])
    assert np.allclose(gg, ro["gtau"], rtol=1e-9, atol=1e-12 * max(1.0, np.abs(ro["gtau"]).max()))
    fk, ev_g = mg.basis()
    ev_o = np.zeros_like(ev_g)
    for s in range(len(mo.sst_size)):
        o, n = mo.sst_offset[s], mo.sst_size[s]
        ev_o[o:o + n, o:o + n] = mo.evec(s)
    dm_g = ev_g @ rg["densitymatrix"] @ ev_g.T
    dm_o = ev_o @ ro["densitymatrix"] @ ev_o.T
    assert np.allclose(dm_g, dm_o, rtol=1e-8, atol=1e-10)
    assert abs(np.trace(dm_g) - 1.0) < 1e-9


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


@pytest.mark.parametrize("warps", [-1, 7, 32])
def test_phase_synchronous_schedule_matches_oracle(lib, warps):
    """The phase-synchronous schedule (blocks of `warps` chains, a partial
    last block; global and tau-shift moves at 2 % each, 4-operator moves at
    10 % of the insertions and removals) runs every chain as the reference
    chain of its own seed, and
    its measurements equal the independent-warp schedule's: histogram and
    sign exactly, G(tau) and the density matrix to 1e-12 relative (G(tau)
    bins are summed with atomics, whose order is not fixed)."""
    pr = P.config_problem("dd3", beta=10.0)
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    n = 45
    runs = []
    for sched in (0, warps):
        b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 20, nchains=n, seed0=300, taudiff_max=5.0,
                                 kcap=64, opcap=512, ncorr=50, p_global=0.02, p_shift=0.02,
                                 p_4op=0.1)])
        b.set_schedule(sched)
        b.warmup(2000)
        b.measure(20)
        b.sync()
        runs.append(b)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    for c in (0, 6, 7, 44):
        co = O.Chain(mo, 10.0, pr["ftau"], 20, seed=300 + c, taudiff_max=5.0, ncorr=50,
                     p_global=0.02, p_shift=0.02, p_4op=0.1)
        co.warmup(2000)
        co.measure(20)
        t_o, *_ = co.get_config()
        t_g, *_ = runs[1].get_config(c)
        assert np.array_equal(t_o, t_g), c
    for c in range(n):
        r0, r1 = runs[0].results(c), runs[1].results(c)
        scale = np.abs(r0["gtau"]).max()
        assert np.allclose(r0["gtau"], r1["gtau"], rtol=1e-12, atol=1e-12 * scale), c
        assert r0["mean_sign"] == r1["mean_sign"]
        assert np.array_equal(r0["histo"], r1["histo"])
        assert np.allclose(r0["densitymatrix"], r1["densitymatrix"], rtol=1e-12, atol=1e-14)
        assert r0["counters"] == r1["counters"]


def test_graph_replay_and_autotune_keep_the_chains():
    """Warmup/measure through captured CUDA graphs give the same chains and
    measurements as direct launches; the schedule autotuner's proposals are
    ordinary warmup steps (the chains stay the oracle chains of their seeds)."""
    pr = P.config_problem("dd3", beta=10.0)
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    runs = []
    for graphs in (False, True):
        b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 20, nchains=40, seed0=500, taudiff_max=5.0,
                                 kcap=64, opcap=512, ncorr=50, p_global=0.02, p_shift=0.02,
                                 p_4op=0.1)])
        b.use_graphs(graphs)
        for _ in range(2):
            b.warmup(300)
            b.measure(4)
        b.sync()
        runs.append(b)
    for c in range(40):
        assert np.array_equal(runs[0].get_config(c)[0], runs[1].get_config(c)[0])
        r0, r1 = runs[0].results(c), runs[1].results(c)
        assert r0["counters"] == r1["counters"]
        assert np.allclose(r0["gtau"], r1["gtau"], rtol=1e-12, atol=1e-12 * np.abs(r0["gtau"]).max())
    b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 20, nchains=40, seed0=600, taudiff_max=5.0,
                             kcap=64, opcap=512)])
    best = b.autotune(50)
    assert best in (0, 4, 8, 12, 14, 16, 20, 24, 28, 32)
    b.sync()
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    for c in (0, 39):
        co = O.Chain(mo, 10.0, pr["ftau"], 20, seed=600 + c, taudiff_max=5.0)
        for _ in range(10):  # one warmup call per candidate schedule
            co.warmup(50)
        assert np.array_equal(co.get_config()[0], b.get_config(c)[0])


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


def test_bulk_configs_warm_start(lib):
    """cthyb_batch_get_configs / cthyb_batch_set_configs (the mc_config_inout
    warm start for a whole batch): the bulk read equals the per-chain
    get_mc_config; configurations moved into a fresh batch of two groups
    (a range across the group boundary) carry the trace and determinant of
    the oracle's full rebuild; an invalid chain in the middle of a bulk
    write is rejected before any chain is written; the warm-started chains
    keep running with only rounding drift in M."""
    betas = (10.0, 25.0)
    pr = {b: P.config_problem("dd3", beta=b) for b in betas}
    q = pr[10.0]["quantum_numbers"]
    mg = E.Model(3, pr[10.0]["umatrix"], pr[10.0]["muimp"], q)

    def batch(seed0):
        return E.Batch(mg, [E.Group(b, pr[b]["ftau"], 20, nchains=6, seed0=seed0 + 100 * i,
                                    taudiff_max=5.0, kcap=64, opcap=512, p_outer=0.1)
                            for i, b in enumerate(betas)])

    a = batch(1)
    a.warmup(3000)
    a.sync()
    offs, t, o, s, c, outer = a.get_configs()
    assert len(offs) == 13 and offs[-1] > 0
    for ch in range(12):
        tg, og, sg_, cg, outg = a.get_config(ch)
        sl = slice(offs[ch], offs[ch + 1])
        assert np.array_equal(tg, t[sl]) and np.array_equal(og, o[sl])
        assert np.array_equal(sg_, s[sl]) and np.array_equal(cg, c[sl]) and outg == outer[ch]
    b = batch(7)
    b.set_configs(offs, t, o, s, c, outer)
    o2 = b.get_configs()
    for x, y in zip(o2, (offs, t, o, s, c, outer)):
        assert np.array_equal(x, y)
    mo = O.Model(3, pr[10.0]["umatrix"], pr[10.0]["muimp"], q)
    for ch in range(12):
        beta = betas[ch // 6]
        co = O.Chain(mo, beta, pr[beta]["ftau"], 20, seed=0, taudiff_max=5.0)
        sl = slice(offs[ch], offs[ch + 1])
        co.set_config(t[sl], o[sl], s[sl], c[sl], int(outer[ch]))
        ft, fd = co.full_trace(), co.full_det()
        st = b.state(ch)
        assert abs(st["trace_log"] - ft[0]) < 1e-10 * max(1, abs(ft[0])) and st["trace_sign"] == ft[1]
        assert abs(st["det_log"] - fd[0]) < 1e-10 * max(1, abs(fd[0])) and st["det_sign"] == fd[1]
        sa = a.state(ch)
        assert st["cfgsign"] == sa["cfgsign"] and st["noper"] == sa["noper"]
    # chains 4..9 (groups 0 and 1) with chain 7's configuration made invalid
    sub = slice(offs[4], offs[10])
    t_bad = t[sub].copy()
    k7 = offs[7] - offs[4]
    n7 = offs[8] - offs[7]
    before = b.get_configs()
    if n7 >= 2:
        t_bad[k7 + 1] = t_bad[k7]  # two operators at one time
    else:
        t_bad[k7] = betas[1] + 1.0  # beyond beta
    with pytest.raises(E.EngineError):
        b.set_configs(offs[4:11] - offs[4], t_bad, o[sub], s[sub], c[sub], outer[4:10], chain0=4)
    after = b.get_configs()
    for x, y in zip(after, before):
        assert np.array_equal(x, y)
    # the same range, valid: written across the group boundary in one call
    b.set_configs(offs[4:11] - offs[4], t[sub], o[sub], s[sub], c[sub], outer[4:10], chain0=4)
    for x, y in zip(b.get_configs(), (offs, t, o, s, c, outer)):
        assert np.array_equal(x, y)
    b.warmup(2000)
    b.sync()
    assert b.refresh_minv(replace=False) < 1e-9


def test_ratios_against_dense_lu(lib):
    """Every determinant ratio of a GPU run against det(H_new)/det(H_old)
    from dense LU (numpy.linalg.slogdet) of the rebuilt hybridisation
    matrices: |error| <= 1e-10 + 2e-14 * cancellation factor."""
    name, beta, tdm, pout, nprop, seed = "dd3", 25.0, 5.0, 0.1, 4000, 3
    ref, got, co, b = run_pair(name, beta, tdm, pout, nprop, seed)
    F = P.config_problem(name, beta=beta)["ftau"][0, 0]
    cfg = {f: ([], []) for f in range(6)}
    C = cancellation(got, F, beta)
    worst = 0.0
    for i, r in enumerate(got):
        if r["outcome"] < 3:
            continue
        f = 2 * (r["orb"] - 1) + (r["spin"] - 1)
        tc, ta = cfg[f]
        if r["move"] == 0:
            tc2, ta2 = sorted(tc + [r["tau_c"]]), sorted(ta + [r["tau_a"]])
        else:
            tc2 = [t for t in tc if t != r["tau_c"]]
            ta2 = [t for t in ta if t != r["tau_a"]]

        def H(a_, c_):
            return hybrf(F, beta, np.subtract.outer(np.array(a_), np.array(c_)))

        ln = np.linalg.slogdet(H(ta2, tc2))[1] if tc2 else 0.0
        lo = np.linalg.slogdet(H(ta, tc))[1] if tc else 0.0
        err = abs(r["det_log"] - (ln - lo))
        assert err <= 1e-10 + 2e-14 * C[i], (i, err, C[i])
        worst = max(worst, err / (1e-10 + 2e-14 * C[i]))
        if r["outcome"] == 4:
            cfg[f] = (tc2, ta2)


def test_capacity_limit_and_invalid_configurations(lib):
    """Edge cases: a chain that outgrows kcap stops with CTHYB_ERR_CAPACITY
    reported by sync (no fault, the other chains' results stay readable);
    set_mc_config rejects unbalanced, out-of-range, colliding (equal-time)
    and over-capacity configurations with an error code; the empty
    configuration is accepted."""
    pr = P.config_problem("dd3", beta=50.0)
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(50.0, pr["ftau"], 20, nchains=8, seed0=1, taudiff_max=5.0, kcap=4,
                             opcap=64)])
    b.warmup(5000)
    with pytest.raises(E.EngineError, match="capacity"):
        b.sync()
    r = b.results(0)
    assert r["gtau"].shape == (3, 2, 20)
    b2 = E.Batch(mg, [E.Group(10.0, P.config_problem("dd3", beta=10.0)["ftau"], 20, nchains=1, seed0=1,
                              taudiff_max=10.0, kcap=16, opcap=64)])
    bad = [
        ([1.0, 2.0], [1, 1], [1, 1], [1, 1], 0),          # unbalanced (two creators)
        ([1.0, 12.0], [1, 1], [1, 1], [1, 2], 0),         # time beyond beta
        ([1.0, 1.0], [1, 1], [1, 1], [1, 2], 0),          # equal times
        ([1.0, 2.0], [4, 4], [1, 1], [1, 2], 0),          # orbital out of range
        (list(np.arange(1, 35) * 0.25), [1] * 34, [1] * 34, [1, 2] * 17, 0),  # 17 pairs > kcap 16
    ]
    for taus, orbs, spins, cas, outer in bad:
        with pytest.raises(E.EngineError):
            b2.set_config(0, taus, orbs, spins, cas, outer)
    b2.set_config(0, [], [], [], [], 0)
    assert b2.state(0)["noper"] == 0
    b2.warmup(100)
    b2.sync()


def _offdiag_problem(kind):
    """One orbital with a spin-mixing bath ("Nt"), or two orbitals with
    inter-orbital hopping (dense H_loc) and an orbital-mixing bath."""
    import exact_bath as XB
    if kind == "spin":
        beta = 4.0
        um = P.flat_umatrix(P.umatrix_density(1, 2.0, 2.0, 0.0))
        muimp = P.muimp_solver(1, 1.3)
        ff = XB.ftau_full_bath(beta, [-0.6, 0.9], [[0.6, 0.3], [0.5, -0.4]], 2000)
        return 1, beta, um, muimp, ff, "Nt"
    nd, beta = 2, 3.0
    um = P.flat_umatrix(P.umatrix_density(nd, 2.0, 2.0, 0.0))
    muimp = P.muimp_solver(nd, 1.0).copy()
    for s in range(2):
        muimp[0, s, 1, s] = muimp[1, s, 0, s] = -0.3
    ff = XB.ftau_full_spinful(nd, beta, [-0.5, 0.7], [[0.6, 0.3], [0.4, -0.5]], 2000)
    return nd, beta, um, muimp, ff, "Nt Szt"


def _diag_of(ff):
    nd = ff.shape[0]
    return np.stack([np.stack([ff[b, s, b, s] for s in range(2)]) for b in range(nd)])


@pytest.mark.parametrize("kind,tdm,pout,nprop,seed,prare,p4", [("spin", 1.5, 0.1, 20000, 5, 0.0, 0.0),
                                                               ("spin", -1.0, 0.0, 10000, 9, 0.0, 0.0),
                                                               ("orbital", -1.0, 0.1, 6000, 6, 0.0, 0.0),
                                                               ("orbital", 1.0, 0.1, 6000, 8, 0.0, 0.0),
                                                               ("spin", 1.5, 0.1, 12000, 11, 0.05, 0.0),
                                                               ("orbital", -1.0, 0.1, 6000, 12, 0.05, 0.0),
                                                               ("spin", 1.5, 0.1, 12000, 21, 0.02, 0.3),
                                                               ("orbital", -1.0, 0.1, 6000, 22, 0.02, 0.3)])
def test_offdiag_proposal_stream_and_measurement_parity(lib, kind, tdm, pout, nprop, seed, prare, p4):
    """Off-diagonal hybridisation (offdiag = 1): the GPU chain proposes,
    decides and updates like the oracle chain of the same seed, proposal by
    proposal (flavours, block positions, pair counts, outcomes bit-exact;
    ratios to 1e-10), with global and tau-shift moves at prare each where
    given and 4-operator moves at p4; then the measured G for every flavour
    pair and its Legendre
    coefficients (GLeg_full), the order histogram and the sign agree, and
    so do the final configuration and the inverse matrix over all
    flavours."""
    nd, beta, um, muimp, ff, qns = _offdiag_problem(kind)
    ntau = 10
    mo = O.Model(nd, um, muimp, qns)
    co = O.Chain(mo, beta, ff, ntau, seed=seed, taudiff_max=tdm, p_outer=pout, ncorr=20, maxhisto=30,
                 p_global=prare, p_shift=prare, nleg=6, p_4op=p4)
    co.start_log(nprop)
    co.warmup(nprop)
    ref = co.log()
    mg = E.Model(nd, um, muimp, qns)
    b = E.Batch(mg, [E.Group(beta, _diag_of(ff), ntau, nchains=1, seed0=seed, taudiff_max=tdm,
                             p_outer=pout, ncorr=20, maxhisto=30, kcap=64, opcap=256,
                             ftau_full=ff, p_global=prare, p_shift=prare, nleg=6, p_4op=p4)])
    b.set_log(nprop)
    b.warmup(nprop)
    b.sync()
    got = b.log(0)
    compare_logs(ref, got)
    assert np.sum((ref["outcome"] == 4) & (ref["move"] == 0)) > 20
    if prare > 0:
        for mv in (2, 3):
            assert np.sum((ref["outcome"] == 4) & (ref["move"] == mv)) > 5
    if p4 > 0:  # 4-operator moves with off-diagonal F (CTQMC.F90:3647-3651, 3822-3827, 4352-4357)
        for mv in (5, 6):
            assert np.sum((ref["outcome"] == 4) & (ref["move"] == mv)) > 5, mv
    co.measure(300)
    b.measure(300)
    b.sync()
    ro, rg = co.results(), b.results(0)
    assert ro["mean_sign"] == rg["mean_sign"]
    nf = 2 * nd
    assert np.array_equal(ro["histo"], np.stack([rg["histo"][f // 2, f % 2] for f in range(nf)]))
    go, gg = co.results_full(), b.results_full(0)
    assert np.allclose(gg, go, rtol=1e-9, atol=1e-12 * np.abs(go).max())
    lo, lg = co.gleg_full(), b.results_gleg_full(0)  # GLeg_full, CTQMC.F90:2533-2555
    assert np.allclose(lg, lo, rtol=1e-9, atol=1e-12 * np.abs(lo).max())
    assert not np.any(b.results_extra(0)["gleg"])
    t_o, *_ = co.get_config()
    t_g, *_ = b.get_config(0)
    assert np.array_equal(t_o, t_g)
    mo_, mg_ = co.minv_full(), b.minv_full(0)
    assert mo_.shape == mg_.shape
    if mo_.size:
        assert np.allclose(mg_, mo_, rtol=1e-9, atol=1e-9 * np.abs(mo_).max())
    so, sg = co.state(), b.state(0)
    assert so["cfgsign"] == sg["cfgsign"] and so["det_sign"] == sg["det_sign"]
    assert abs(so["det_log"] - sg["det_log"]) < 1e-8


def test_accepted_pair_histogram(lib):
    """AccPair of the measurement loop (CTQMC.F90:3579-3582, 4112-4122):
    the device histogram of accepted pair moves by flavour and time
    difference equals the one built from the oracle's proposal records of
    the same run (bin min(Ntau, floor(dtau / beta * Ntau) + 1))."""
    beta, ntau, nprop = 10.0, 40, 6000
    pr = P.config_problem("dd3", beta=beta)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    co = O.Chain(mo, beta, pr["ftau"], ntau, seed=31, taudiff_max=5.0, ncorr=50)
    co.start_log(nprop)
    co.warmup(nprop)
    ref = co.log()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], ntau, nchains=1, seed0=31, taudiff_max=5.0, ncorr=50,
                             kcap=64, opcap=512, measure_accpair=True)])
    b.warmup(nprop)
    b.sync()
    got = b.results_accpair(0)
    acc = ref[(ref["outcome"] == 4) & (ref["move"] <= 1)]
    want = np.zeros((3, 2, ntau))
    for r in acc:
        dt = abs(r["tau_a"] - r["tau_c"])
        k = min(ntau, int(np.floor(dt / beta * ntau)) + 1)
        want[r["orb"] - 1, r["spin"] - 1, k - 1] += 1
    assert want.sum() > 500
    assert np.array_equal(got, want)
    b.reset_measurements()
    assert not np.any(b.results_accpair(0))
