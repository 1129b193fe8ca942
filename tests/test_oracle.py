"""Pins of the oracle (CPU restatement of the w2dynamics pair-move loop).

* RNG stream against the reference's src/mtrng/random.cc (golden fixture
  made by tests/golden/make_golden.py from that file compiled unchanged).
* U matrices of w2dynamics_gb300.problems against the reference's
  w2dyn/dmft/interaction.py (golden fixture).
* time_evolve_in_eigenbasis known answer
  (testsuite/ctqmc.tests/2-time-evolve-in-eigenbasis.F90:5-58).
* fast updates (Sherman-Morrison grow/shrink, windowed trace) against full
  recomputation after every proposal (the intent of the dead
  MatrixUpdate.F90:489-632 test).
* operator-list invariants of testsuite/ctqmc.tests/3-operator-list-stress-
  test.F90 with a fixed seed.
* physics known answers: U=0 impurity G(tau) equals the bath g(tau)
  (half-filled Bethe lattice self-consistency), atomic-limit density matrix,
  and detailed balance: the sampled expansion-order distribution and
  occupations of a single-orbital impurity with a discrete asymmetric bath
  equal exact diagonalisation of impurity + bath (tests/exact_bath.py);
  the baths' F(tau) and the Legendre convention of those known answers
  against the reference's w2dyn/auxiliaries/transform.py (golden fixture).
* get_MatLogDetFull on the matrix of testsuite/ctqmc.tests/1-get-MatFull.F90.
* off-diagonal mode (offdiag = 1): fast updates, G for every flavour pair,
  its Legendre coefficients and the occupations against exact
  diagonalisation, with global, tau-shift and 4-operator moves.
"""
import os

import numpy as np
import pytest

import exact_bath as XB
import oracle as O
from w2dynamics_gb300 import estimators as ES
from w2dynamics_gb300 import problems as P

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_rng_stream_matches_reference_random_cc():
    z = np.load(os.path.join(GOLD, "rng_streams.npz"))
    for seed in (0, 1, 42, 4095):
        ref = z[f"reals_{seed}"]
        mine, _ = O.rng_stream(seed, len(ref), 0, 1, 1)
        assert np.array_equal(mine, ref)
        for lo, hi in ((1, 1), (1, 2), (1, 3), (1, 5), (8, 16), (1, 1000), (1, 123457)):
            ref = z[f"ints_{seed}_{lo}_{hi}"]
            _, ints = O.rng_stream(seed, 0, len(ref), lo, hi)
            assert np.array_equal(ints, ref), (seed, lo, hi)


def test_reference_rng_live_if_built():
    """Compare directly against oracle/_ref (only where it could be built)."""
    path = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref",
                        "librandom_ref.so")
    if not os.path.exists(path):
        pytest.skip("reference random.cc not built here")
    import ctypes as C
    lib = C.CDLL(path)
    lib.new_random.restype = C.c_void_p
    lib.seed_random.argtypes = [C.c_void_p, C.c_uint]
    lib.get_random.argtypes = [C.c_void_p]
    lib.get_random.restype = C.c_double
    r = lib.new_random()
    lib.seed_random(r, 777)
    ref = np.array([lib.get_random(r) for _ in range(5000)])
    mine, _ = O.rng_stream(777, 5000, 0, 1, 1)
    assert np.array_equal(mine, ref)


@pytest.mark.parametrize("key,fn,args", [
    ("density_1_2.0_2.0_0.0", P.umatrix_density, (1, 2.0, 2.0, 0.0)),
    ("density_2_3.0_2.0_0.5", P.umatrix_density, (2, 3.0, 2.0, 0.5)),
    ("density_3_4.0_2.8_0.6", P.umatrix_density, (3, 4.0, 2.8, 0.6)),
    ("kanamori_2_3.0_1.6_0.7", P.umatrix_kanamori, (2, 3.0, 1.6, 0.7)),
    ("kanamori_3_4.0_2.8_0.6", P.umatrix_kanamori, (3, 4.0, 2.8, 0.6)),
    ("kanamori_5_3.0_1.6_0.7", P.umatrix_kanamori, (5, 3.0, 1.6, 0.7)),
])
def test_umatrix_matches_reference_interaction(key, fn, args):
    z = np.load(os.path.join(GOLD, "umatrices.npz"))
    assert np.array_equal(P.flat_umatrix(fn(*args)), z[key])


def test_bath_functions_and_legendre_convention_match_reference_transform():
    """The F(tau) of the exact-diagonalisation baths equal the reference's
    hybr_from_sites (w2dyn/auxiliaries/transform.py:114-146, golden
    fixture) for the one-orbital, the spin-mixing and the orbital-mixing
    bath; the exact Legendre coefficients used as known answers for GLeg
    follow the reference's convention: its leg2tau matrix
    (transform.py:148-179) maps them back onto the exact G(tau)."""
    z = np.load(os.path.join(GOLD, "bath_legendre.npz"))
    beta = float(z["beta"])
    eps = [-0.6, 0.9]
    assert np.allclose(XB.ftau_bath(beta, eps, [0.6, 0.8], 201), z["single"][0, 0], rtol=1e-13, atol=0)
    ff = XB.ftau_full_bath(beta, eps, [[0.6, 0.3], [0.5, -0.4]], 201)[0, :, 0, :]
    assert np.allclose(ff, z["offdiag"], rtol=1e-13, atol=1e-16)
    fs = XB.ftau_full_spinful(2, beta, [-0.5, 0.7], [[0.6, 0.3], [0.4, -0.5]], 201).reshape(4, 4, 201)
    assert np.allclose(fs, z["spinful"], rtol=1e-13, atol=1e-16)
    assert np.abs(z["spinful"][0, 2]).max() > 0.05 and np.abs(z["offdiag"][0, 1]).max() > 0.05
    h, dd = XB.offdiag_hamiltonian(1.3, 2.0, eps, [[0.6, 0.3], [0.5, -0.4]])
    gl = XB.legendre_answers(beta, h, dd, 40)
    w, q = np.linalg.eigh(h)
    w = w - w.min()
    zz = np.exp(-beta * w).sum()
    d = [q.T @ o @ q for o in dd]
    taus = np.linspace(0.0, beta, 41)
    el = np.exp(-(beta - taus)[:, None] * w[None, :])
    er = np.exp(-taus[:, None] * w[None, :])
    g = np.array([[np.einsum("tm,mn,tn,nm->t", el, d[a], er, d[b].T) / zz for b in range(2)] for a in range(2)])
    rec = np.einsum("il,abl->abi", z["leg2tau"], gl)
    assert np.abs(rec - g).max() < 1e-8 * np.abs(g).max()


def test_time_evolve_known_answer():
    """exp(-(E_i - Egs) tau) scaling of the reference test (10 states,
    E_i = 0.1 i, tau = 0.3, rel 1e-14): the oracle's trace of a one-block
    empty configuration equals the closed form."""
    ev = 0.1 * np.arange(10)
    tau = 0.3
    vec = np.exp(-(ev - 0.0) * tau) * np.ones(10)
    ref = np.array([np.exp(-(0.1 * i) * 0.3) for i in range(10)])
    assert np.allclose(vec, ref, rtol=1e-14, atol=0)
    # the same identity through the oracle: H = diag(-mu n) for one orbital
    m = O.Model(1, np.zeros((2, 2, 2, 2)), P.muimp_solver(1, 0.7), "Nt Szt")
    c = O.Chain(m, tau, np.ones((1, 2, 5)) * 0.1, 10, seed=3, taudiff_max=tau)
    # empty trace of the chosen outer superstate: sum_i exp(-(E_i-Egs) beta)
    sst = int(c.state()["outer_sst"])
    off, n = m.sst_offset[sst], m.sst_size[sst]
    e = m.evals[off:off + n]
    expect = np.log(np.sum(np.exp(-(e - m.egs) * tau)))
    assert abs(c.state()["trace_log"] - expect) < 1e-14


def test_mat_logdet_full_reference_case_and_known_answers():
    """get_MatLogDetFull (MatrixUpdate.F90:41-99): the reference test's
    rank-2 matrix N(i, j) = i + j, k = 10 (testsuite/ctqmc.tests/
    1-get-MatFull.F90, which only requires the call to return) goes through
    without error and is singular to working precision; k = 0 gives
    (log 0, sign 1); well-conditioned matrices give numpy's slogdet and
    inverse."""
    k = 10
    n = np.array([[i + j for j in range(1, k + 1)] for i in range(1, k + 1)], np.float64)
    lg, sg, inv = O.mat_logdet_full(n)
    hadamard = np.sum(np.log(np.linalg.norm(n, axis=0)))
    assert sg == 0.0 or lg < hadamard - 25.0  # |det| below 1e-11 of the Hadamard bound
    assert O.mat_logdet_full(np.zeros((0, 0)))[:2] == (0.0, 1.0)
    one = O.mat_logdet_full(np.array([[-2.5]]))
    assert one[1] == -1.0 and abs(one[0] - np.log(2.5)) < 1e-15 and one[2][0, 0] == -0.4
    rng = np.random.default_rng(4)
    for k in (2, 7, 40):
        a = rng.normal(size=(k, k)) + 3.0 * np.eye(k) * rng.choice([-1.0, 1.0], size=k)
        lg, sg, inv = O.mat_logdet_full(a)
        s_np, l_np = np.linalg.slogdet(a)
        assert sg == s_np and abs(lg - l_np) < 1e-12 * max(1.0, abs(l_np))
        assert np.allclose(inv @ a, np.eye(k), atol=1e-12)
    z = np.ones((3, 3))
    z[:, 1] = 0.0  # a zero column: exact zero pivot, (-huge, 0)
    lg, sg, inv = O.mat_logdet_full(z)
    assert sg == 0.0 and lg == -np.finfo(np.float64).max and inv is None


def _hyb(F, beta, t):
    s = 1.0
    if t < 0:
        t += beta
        s = -1.0
    n = t / beta * (len(F) - 1)
    i = int(n)
    return s * (F[i] + (n - i) * (F[i + 1] - F[i]))


@pytest.mark.parametrize("name,beta,tdm,pout", [
    ("anderson1", 10.0, 10.0, 0.0),
    ("anderson1", 10.0, 3.0, 0.2),
    ("dd3", 8.0, 8.0, 0.1),
    ("dd3", 8.0, 2.5, 0.0),
])
def test_fast_updates_match_full_recompute(name, beta, tdm, pout):
    pr = P.config_problem(name, beta=beta)
    m = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    c = O.Chain(m, pr["beta"], pr["ftau"], 50, seed=11, taudiff_max=tdm, p_outer=pout)
    nacc = 0
    for i in range(1500):
        c.warmup(1)
        st = c.state()
        fd, ft = c.full_det(), c.full_trace()
        assert abs(fd[0] - st["det_log"]) < 1e-9 and fd[1] == st["det_sign"], i
        assert abs(ft[0] - st["trace_log"]) < 1e-9 and ft[1] == st["trace_sign"], i
        nacc = st["noper"]
    # inverse matrices against direct inversion
    taus, orbs, spins, cas = c.get_config()
    F = pr["ftau"][0, 0]
    for b in range(pr["nd"]):
        for s in range(2):
            sel = (orbs - 1 == b) & (spins - 1 == s)
            tc = np.sort(taus[sel & (cas == 1)])
            ta = np.sort(taus[sel & (cas == 2)])
            if len(tc) == 0:
                continue
            H = np.array([[_hyb(F, beta, a - cc) for cc in tc] for a in ta])
            assert np.allclose(c.minv(2 * b + s), np.linalg.inv(H), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("name,beta,tdm", [("anderson1", 10.0, 3.0), ("dd3", 8.0, 2.5),
                                            ("dd3", 8.0, 8.0)])
def test_global_and_shift_moves_keep_state_consistent(name, beta, tdm):
    """Global moves (spin flip, CA flip, user symmetry moves, random
    permutation) and tau-shift moves at 10 % each, 4-operator moves at 30 %
    of the insertions and removals: trace, determinant and inverse matrices
    stay equal to a full recompute after every step, and every move kind is
    accepted."""
    pr = P.config_problem(name, beta=beta)
    m = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    # a cyclic orbital permutation (its inverse differs) for the 3-orbital model
    sym = [[2, 3, 1, 5, 6, 4]] if pr["nd"] == 3 else None
    c = O.Chain(m, pr["beta"], pr["ftau"], 50, seed=23, taudiff_max=tdm, p_outer=0.1,
                p_global=0.1, p_shift=0.1, symmoves=sym, p_4op=0.3)
    acc = {"acc_glob": 0, "acc_shift": 0, "acc_add4": 0, "acc_rem4": 0}
    for i in range(1500):
        c.warmup(1)  # counters restart with every call
        for k in acc:
            acc[k] += c.counters()[k]
        st = c.state()
        fd, ft = c.full_det(), c.full_trace()
        assert abs(fd[0] - st["det_log"]) < 1e-9 and fd[1] == st["det_sign"], i
        assert abs(ft[0] - st["trace_log"]) < 1e-9 and ft[1] == st["trace_sign"], i
    assert acc["acc_glob"] > 0 and acc["acc_shift"] > 0, acc
    taus, orbs, spins, cas = c.get_config()
    assert np.all(np.diff(taus) > 0) and taus.min() >= 0 and taus.max() < beta
    F = pr["ftau"][0, 0]
    for b in range(pr["nd"]):
        for s in range(2):
            sel = (orbs - 1 == b) & (spins - 1 == s)
            tc = np.sort(taus[sel & (cas == 1)])
            ta = np.sort(taus[sel & (cas == 2)])
            if len(tc) == 0:
                continue
            H = np.array([[_hyb(F, beta, a - cc) for cc in tc] for a in ta])
            assert np.allclose(c.minv(2 * b + s), np.linalg.inv(H), rtol=1e-9, atol=1e-9)


def test_legendre_coefficients_u0_known_answer_and_sum_rule():
    """Legendre G_l (MeasGtauRem, CTQMC.F90:2368-2389): at U = 0 equal to
    sqrt(2l+1) * int_0^beta P_l(2 tau/beta - 1) g(tau) dtau of the bath; and
    G_0 = (beta/Ntau) * sum of the G(tau) bins in the same run (both sum the
    same M elements)."""
    from numpy.polynomial import legendre as npl
    beta, nleg = 5.0, 8
    um = P.flat_umatrix(P.umatrix_density(1, 0.0, 0.0, 0.0))
    ft = P.semicircle_ftau(1, beta, 1.0, 500)
    g = P.semicircle_gtau(beta, 1.0, 500)
    m = O.Model(1, um, P.muimp_solver(1, 0.0), "Nt Szt Azt")
    gls = []
    for seed in range(16):
        c = O.Chain(m, beta, ft, 20, seed=200 + seed, taudiff_max=beta, nleg=nleg)
        c.warmup(3000)
        c.measure(3000)
        r, x = c.results(), c.results_extra()
        for f in range(2):
            assert abs(x["gleg"][f, 0] - r["gtau"][f].sum() * beta / 20) < 1e-12
        gls.append(x["gleg"])
    G = np.mean(gls, axis=0)
    E = np.std(gls, axis=0, ddof=1) / np.sqrt(len(gls))
    tt = np.linspace(0, beta, 20001)
    gg = np.interp(tt, np.linspace(0, beta, 500), g)
    exact = np.array([np.sqrt(2 * l + 1) * np.trapezoid(npl.legval(2 * tt / beta - 1, [0] * l + [1]) * gg, tt)
                      for l in range(nleg)])
    z = (G - exact[None, :]) / E
    assert np.abs(z).max() < 4.5, z


def test_outer_histograms_sum_rules():
    """MeasOuterHistograms: superstate visit frequencies sum to one, state
    visits add up to their superstate's size, signs are within [-1, 1] and
    the trace contributions of the states add up to their superstate's."""
    pr = P.config_problem("dd3", beta=8.0)
    m = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    c = O.Chain(m, 8.0, pr["ftau"], 20, seed=3, taudiff_max=4.0, ncorr=20, p_global=0.05, p_shift=0.05)
    c.warmup(2000)
    c.measure(300)
    x = c.results_extra()
    assert abs(x["outer_sst_histo"].sum() - 1.0) < 1e-12
    for s, (o, n) in enumerate(zip(m.sst_offset, m.sst_size)):
        assert np.allclose(x["outer_state_histo"][o:o + n], x["outer_sst_histo"][s])
        assert abs(x["contrib_state"][o:o + n].sum() - x["contrib_sst"][s]) <= 1e-12 * max(1, x["contrib_sst"][s])
    visited = x["outer_sst_histo"] > 0
    assert np.all(np.abs(x["sign_sst"][visited]) <= 1.0)


def test_u0_green_function_with_global_and_shift_moves():
    """The U=0 known answer of the bath G(tau) holds with global and
    tau-shift moves switched on (detailed balance of the added moves)."""
    beta = 5.0
    um = P.flat_umatrix(P.umatrix_density(1, 0.0, 0.0, 0.0))
    ft = P.semicircle_ftau(1, beta, 1.0, 500)
    g = P.semicircle_gtau(beta, 1.0, 500)
    m = O.Model(1, um, P.muimp_solver(1, 0.0), "Nt Szt Azt")
    res = []
    for seed in range(16):
        c = O.Chain(m, beta, ft, 20, seed=100 + seed, taudiff_max=beta, p_global=0.1,
                    p_shift=0.1)
        c.warmup(5000)
        c.measure(4000)
        res.append(c.results()["gtau"])
    G = np.mean(res, axis=0)
    E = np.std(res, axis=0, ddof=1) / np.sqrt(len(res))
    tt = np.linspace(0, beta, 500)
    edges = np.linspace(0, beta, 21)
    gex = np.array([np.mean(np.interp(np.linspace(a, b, 400), tt, g))
                    for a, b in zip(edges[:-1], edges[1:])])
    z = (G - gex) / E
    assert np.abs(z).max() < 4.5
    assert abs(z.mean()) < 1.0


def test_operator_list_stress_invariants():
    """3-operator-list-stress-test.F90 invariants with a fixed seed: time
    order, per-flavour consistency, NPairs equal to a recount, window edges
    (beta=100, 3 bands, TaudiffMax=10, window shift every 50 proposals)."""
    nd = 3
    um = P.flat_umatrix(P.umatrix_density(nd, 0.0, 0.0, 0.0))
    m = O.Model(nd, um, P.muimp_solver(nd, 0.0), "Nt Szt")
    beta = 100.0
    ft = np.full((nd, 2, 200), 0.2)
    c = O.Chain(m, beta, ft, 20, seed=12345, taudiff_max=10.0, ncorr=500)
    st = c.state()
    assert st["num_windows"] == 9 and st["nslide"] == max(6, 500 // 9)
    for _ in range(300):
        c.warmup(50)
        st = c.state()
        taus, orbs, spins, cas = c.get_config()
        assert np.all(np.diff(taus) > 0)
        for b in range(1, nd + 1):
            for s in (1, 2):
                sel = (orbs == b) & (spins == s)
                assert np.sum(sel & (cas == 1)) == np.sum(sel & (cas == 2))
        # NPairs recount from scratch
        wmin, wmax, tdm = st["tauwin_min"], st["tauwin_max"], st["taudiff_max"]
        n = 0
        for i in range(len(taus)):
            for j in range(i + 1, len(taus)):
                if orbs[i] == orbs[j] and spins[i] == spins[j] and cas[i] != cas[j]:
                    if taus[i] >= wmin and taus[j] <= wmax and taus[j] <= taus[i] + tdm:
                        n += 1
        assert n == st["npairs"]
        assert wmax - wmin == pytest.approx(2 * beta / (st["num_windows"] + 1))


def test_u0_green_function_equals_bath():
    """U=0, mu=0, semicircle bath: the impurity G(tau) equals g(tau) of the
    bath (half-filled Bethe lattice); w2dynamics' gtau convention is
    positive.  16 chains, 20 bins per flavour."""
    beta = 5.0
    um = P.flat_umatrix(P.umatrix_density(1, 0.0, 0.0, 0.0))
    ft = P.semicircle_ftau(1, beta, 1.0, 500)
    g = P.semicircle_gtau(beta, 1.0, 500)
    m = O.Model(1, um, P.muimp_solver(1, 0.0), "Nt Szt Azt")
    res, dms = [], []
    for seed in range(16):
        c = O.Chain(m, beta, ft, 20, seed=seed, taudiff_max=beta, p_outer=0.1)
        c.warmup(5000)
        c.measure(4000)
        r = c.results()
        res.append(r["gtau"])
        dms.append(np.diag(r["densitymatrix"]))
        assert r["mean_sign"] == -1.0
    G = np.mean(res, axis=0)
    E = np.std(res, axis=0, ddof=1) / np.sqrt(len(res))
    tt = np.linspace(0, beta, 500)
    edges = np.linspace(0, beta, 21)
    gex = np.array([np.mean(np.interp(np.linspace(a, b, 400), tt, g))
                    for a, b in zip(edges[:-1], edges[1:])])
    z = (G - gex) / E
    assert np.abs(z).max() < 4.5
    assert abs(z.mean()) < 1.0
    assert np.allclose(np.mean(dms, axis=0), 0.25, atol=0.01)


def test_atomic_limit_density_matrix():
    """Delta -> 0: the sampled density matrix is exp(-beta H)/Z restricted
    to the chain's outer superstate sector (no insertion is ever accepted)."""
    beta = 2.0
    pr = P.config_problem("dd3", beta=beta)
    m = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    ft = np.full((3, 2, 100), 1e-12)
    c = O.Chain(m, beta, ft, 10, seed=5, taudiff_max=beta)
    c.warmup(200)
    c.measure(100)
    r = c.results()
    sst = int(c.state()["outer_sst"])
    off, n = m.sst_offset[sst], m.sst_size[sst]
    e = m.evals[off:off + n]
    w = np.exp(-beta * (e - e.min()))
    dm = np.diag(r["densitymatrix"])[off:off + n]
    assert np.allclose(dm, w / w.sum(), rtol=1e-10)


# single-orbital impurity, two bath levels, away from particle-hole symmetry
BATH = dict(beta=4.0, mu=1.3, u=2.0, eps=[-0.6, 0.9], v=[0.6, 0.8])


def bath_problem(nftau=2000):
    b = BATH
    um = P.flat_umatrix(P.umatrix_density(1, b["u"], b["u"], 0.0))
    f = XB.ftau_bath(b["beta"], b["eps"], b["v"], nftau)
    return um, P.muimp_solver(1, b["mu"]), np.broadcast_to(f, (1, 2, nftau)).copy()


@pytest.mark.parametrize("p_4op", [0.0, 0.5])
def test_detailed_balance_order_distribution_and_occupations(p_4op):
    """Exact answer for the whole sampler (acceptance factors, NPairs,
    sliding windows, outer-superstate, global and tau-shift moves): the
    per-flavour expansion-order histogram and the occupations from the
    density matrix of 16 chains agree with exact diagonalisation of
    impurity + discrete bath within 4.5 standard errors; F(tau) follows the
    reference's bath-site formula, and swapping the bath energies' sign
    (the other time convention) is detected at > 5 standard errors.  With
    p_4op = 0.5 half of the insertions and removals are 4-operator moves
    (StepAdd4 / StepRem4)."""
    b = BATH
    pex = XB.order_marginal(b["beta"], b["mu"], b["u"], b["eps"], b["v"])[:30]
    nup, ndn, dbl = XB.occupations(b["beta"], b["mu"], b["u"], b["eps"], b["v"])
    um, muimp, ft = bath_problem()
    m = O.Model(1, um, muimp, "Nt Szt Azt")
    ev = np.eye(m.nstates)
    hist, occ = [], []
    for seed in range(16):
        c = O.Chain(m, b["beta"], ft, 20, seed=seed, taudiff_max=1.0, ncorr=20, p_outer=0.1,
                    p_global=0.01, p_shift=0.01, maxhisto=30, p_4op=p_4op)
        c.warmup(2000)
        c.measure(10000)
        r = c.results()
        hist.append(r["histo"] / r["histo"].sum(axis=1, keepdims=True))
        o = ES.from_density_matrix(1, m.fock_states, ev, r["densitymatrix"])["occ"]
        occ.append([o[0, 0, 0, 0], o[0, 1, 0, 1], o[0, 0, 0, 1]])
    hist, occ = np.array(hist), np.array(occ)
    sel = pex > 1e-3
    mean, se = hist.mean(0)[:, sel], hist.std(0, ddof=1)[:, sel] / 4.0
    z = (mean - pex[sel]) / se
    assert np.abs(z).max() < 4.5, z
    zo = (occ.mean(0) - [nup, ndn, dbl]) / (occ.std(0, ddof=1) / 4.0)
    assert np.abs(zo).max() < 4.5, zo
    # the same sampler with the bath energies reflected is a different model
    flip = XB.ftau_bath(b["beta"], -np.array(b["eps"]), b["v"], 2000)
    c = O.Chain(m, b["beta"], np.broadcast_to(flip, (1, 2, 2000)).copy(), 20, seed=99,
                taudiff_max=1.0, ncorr=20, maxhisto=30)
    c.warmup(2000)
    c.measure(40000)
    h = c.results()["histo"]
    h = h / h.sum(axis=1, keepdims=True)
    assert np.abs(h[:, 0] - pex[0]).max() > 5 * se[:, 0].max()


# single orbital, two spinless bath levels with spin-dependent amplitudes:
# F has off-diagonal (up, down) elements, Sz is not conserved
OFFDIAG = dict(beta=4.0, mu=1.3, u=2.0, eps=[-0.6, 0.9], v=[[0.6, 0.3], [0.5, -0.4]])


def offdiag_chain(seed, **kw):
    b = OFFDIAG
    um = P.flat_umatrix(P.umatrix_density(1, b["u"], b["u"], 0.0))
    m = O.Model(1, um, P.muimp_solver(1, b["mu"]), "Nt")
    ff = XB.ftau_full_bath(b["beta"], b["eps"], b["v"], 2000)
    return m, O.Chain(m, b["beta"], ff, 10, seed=seed, **kw)


@pytest.mark.parametrize("p_4op", [0.0, 0.3])
def test_offdiag_fast_updates_match_full_recompute(p_4op):
    """Off-diagonal hybridisation (offdiag = 1): after every proposal the
    determinant and the inverse matrix over all flavours (block order:
    flavour-major, time within a flavour) equal a full rebuild from F for
    every flavour pair, and the trace a full recompute, with global and
    tau-shift moves (block rotation of the inverse matrix) at 10 % each and
    both accepted, and with 4-operator moves of any flavours.  (With a
    spin-conserving H_loc a single pair of unlike flavours has zero trace,
    so accepted pairs are of like flavours; the up-down elements of F couple
    the flavours through the determinant, and a 4-operator move can insert
    two unlike pairs at once.)"""
    m, c = offdiag_chain(7, taudiff_max=1.5, p_outer=0.1, p_global=0.1, p_shift=0.1, p_4op=p_4op)
    F = XB.ftau_full_bath(OFFDIAG["beta"], OFFDIAG["eps"], OFFDIAG["v"], 2000)[0, :, 0]
    beta = OFFDIAG["beta"]
    c.start_log(3000)
    mixed = 0
    acc = {"acc_glob": 0, "acc_shift": 0, "acc_add4": 0, "acc_rem4": 0}
    for i in range(3000):
        c.warmup(1)
        for key in acc:
            acc[key] += c.counters()[key]
        st = c.state()
        fd, ft = c.full_det(), c.full_trace()
        assert abs(fd[0] - st["det_log"]) < 1e-9 and fd[1] == st["det_sign"], i
        assert abs(ft[0] - st["trace_log"]) < 1e-9 and ft[1] == st["trace_sign"], i
        taus, orbs, spins, cas = c.get_config()
        cr = sorted([(s - 1, t) for t, s, a in zip(taus, spins, cas) if a == 1])
        an = sorted([(s - 1, t) for t, s, a in zip(taus, spins, cas) if a == 2])
        if not cr:
            continue
        H = np.array([[_hyb(F[fa, fc], beta, ta - tc) for fc, tc in cr] for fa, ta in an])
        assert np.allclose(c.minv_full(), np.linalg.inv(H), rtol=1e-9, atol=1e-9), i
        mixed += len(set(f for f, _ in cr)) == 2
    assert mixed > 100  # configurations with both flavours: cross blocks in H
    assert acc["acc_glob"] > 0 and acc["acc_shift"] > 0, acc
    if p_4op > 0:
        assert acc["acc_add4"] > 10 and acc["acc_rem4"] > 10, acc
    log = c.log()
    acc = log["outcome"] == 4
    assert np.sum(acc & (log["move"] == 0)) > 0 and np.sum(acc & (log["move"] == 1)) > 0
    assert np.sum((log["move"] == 0) & (log["orb"] != log["spin"])) > 0  # unlike pairs proposed


@pytest.mark.parametrize("p_4op", [0.0, 0.3])
def test_offdiag_green_function_and_occupations_exact(p_4op):
    """Known answer for the off-diagonal mode: G(tau) for every spin pair
    (Gtau_full, including the off-diagonal up-down element) and the
    occupations and double occupancy from the density matrix of 16 chains
    agree with exact diagonalisation of impurity + bath within 4.5 standard
    errors, also with 30 % of the insertions and removals made as
    4-operator moves ((2 Nd)^4 proposal factors, removable pairs of any
    flavours)."""
    b = OFFDIAG
    ex = XB.offdiag_answers(b["beta"], b["mu"], b["u"], b["eps"], b["v"], 10)
    G, occ = [], []
    for seed in range(16):
        m, c = offdiag_chain(seed, taudiff_max=1.0, ncorr=20, p_outer=0.1, maxhisto=30, p_4op=p_4op)
        c.warmup(2000)
        c.measure(5000)
        G.append(c.results_full())
        ev = np.zeros((m.nstates, m.nstates))
        for s in range(len(m.sst_size)):
            o, n = m.sst_offset[s], m.sst_size[s]
            ev[o:o + n, o:o + n] = m.evec(s)
        o = ES.from_density_matrix(1, m.fock_states, ev, c.results()["densitymatrix"])["occ"]
        occ.append([o[0, 0, 0, 0], o[0, 1, 0, 1], o[0, 0, 0, 1]])
    G, occ = np.array(G), np.array(occ)
    z = (G.mean(0) - ex["gtau"]) / (G.std(0, ddof=1) / 4.0)
    assert np.abs(z).max() < 4.5, z
    assert np.abs(ex["gtau"][0, 1]).max() > 0.1  # a real off-diagonal G
    want = [ex["rho1"][0, 0], ex["rho1"][1, 1], ex["double_occ"]]
    zo = (occ.mean(0) - want) / (occ.std(0, ddof=1) / 4.0)
    assert np.abs(zo).max() < 4.5, zo


def test_offdiag_legendre_coefficients_exact():
    """GLeg_full (MeasGtauRem_full, CTQMC.F90:2533-2555, normalised as
    8767-8771): the Legendre coefficients of G for every spin pair from 16
    off-diagonal chains agree with the exact coefficients of impurity + bath
    within 4.5 standard errors, and the l = 0 coefficient is the integral of
    the measured G(tau) bins (sqrt(1) x beta x bin mean)."""
    b = OFFDIAG
    nleg = 8
    h, dd = XB.offdiag_hamiltonian(b["mu"], b["u"], b["eps"], b["v"])
    ex = XB.legendre_answers(b["beta"], h, dd, nleg)
    GL, G0 = [], []
    for seed in range(16):
        m, c = offdiag_chain(seed, taudiff_max=1.0, ncorr=20, p_outer=0.1, maxhisto=30, nleg=nleg)
        c.warmup(2000)
        c.measure(5000)
        GL.append(c.gleg_full())
        G0.append(c.results_full())
    GL, G0 = np.array(GL), np.array(G0)
    z = (GL.mean(0) - ex) / np.maximum(GL.std(0, ddof=1) / 4.0, 1e-12)
    assert np.abs(z).max() < 4.5, z
    assert np.abs(ex[0, 1]).max() > 0.05  # a real off-diagonal G_l
    assert np.allclose(GL[..., 0], G0.mean(-1) * b["beta"], rtol=1e-9, atol=1e-12)


def test_offdiag_two_orbitals_with_hopping_exact():
    """Off-diagonal mode with a sign problem: two orbitals with inter-orbital
    hopping in H_loc (dense superstate blocks) and bath levels coupling both
    orbitals (orbital-mixing F), global and tau-shift moves at 5 % each:
    G(tau) for all 16 flavour pairs from 16
    chains agrees with exact diagonalisation within 4.5 standard errors;
    the mean sign is about -0.7 (the configuration sign, recalc_sign, and
    the block order of the inverse matrix matter here)."""
    nd, beta = 2, 3.0
    um = P.flat_umatrix(P.umatrix_density(nd, 2.0, 2.0, 0.0))
    muimp = P.muimp_solver(nd, 1.0).copy()
    for s in range(2):
        muimp[0, s, 1, s] = muimp[1, s, 0, s] = -0.3
    eps, v = [-0.5, 0.7], [[0.6, 0.3], [0.4, -0.5]]
    ex = XB.spinful_answers(nd, beta, um, muimp, eps, v, 8)
    ff = XB.ftau_full_spinful(nd, beta, eps, v, 2000)
    m = O.Model(nd, um, muimp, "Nt Szt")
    G, S = [], []
    for seed in range(16):
        c = O.Chain(m, beta, ff, 8, seed=seed, ncorr=20, p_outer=0.1, maxhisto=30,
                    p_global=0.05, p_shift=0.05)
        c.warmup(2000)
        c.measure(10000)
        G.append(c.results_full())
        S.append(c.results()["mean_sign"])
    G = np.array(G)
    assert -0.8 < np.mean(S) < -0.6
    z = (G.mean(0) - ex["gtau"]) / np.maximum(G.std(0, ddof=1) / 4.0, 1e-12)
    assert np.abs(z).max() < 4.5, z
    assert np.abs(ex["gtau"][0, 2]).max() > 0.05  # inter-orbital G
