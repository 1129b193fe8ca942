"""The mctqmc drop-in module: parameter-string rules (Parameters.F90:281-320,
77-160) and rejection of unsupported modes on the CPU; a full solve through
the module's entry points against the oracle on the GPU."""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import estimators as ES
from w2dynamics_gb300 import mctqmc as ctqmc
from w2dynamics_gb300 import problems as P


def pstring(d):
    # the driver's config_to_pstring (cthyb_solver.py:765-767)
    return "".join("%s = %s #\n" % (k, v) for k, v in sorted(d.items()))


BASE = {"beta": 10.0, "Nd": 3, "Ntau": 40, "NCorr": 50, "Nmeas": 60, "Nwarmups": 2000,
        "MaxHisto": 60, "TaudiffMax": 5.0, "QuantumNumbers": "Nt Szt",
        "PercentageGlobalMove": 0.005, "PercentageTauShiftMove": 0.005,
        "Percentage4OperatorMove": 0.1, "PercentageOuterMove": 0.1,
        "PercentageWormInsert": 0.0, "segment": 0, "offdiag": 0, "statesampling": 0,
        "MeasDensityMatrix": 1, "MeasSsquare": 1, "Eigenbasis": 1, "NLegMax": 10,
        "NSymMove": 1, "SymMove01": "2 3 1 5 6 4"}


def test_parameter_string_rules():
    ctqmc.init_paras("# comment line\nNCorr = 1e2 # trailing\nbeta=\t25.5\nNd = 3\n"
                     "QuantumNumbers = Nt Szt #\nSymMove01 = 1,2\n")
    assert ctqmc._int("NCorr") == 100          # integer given in scientific notation
    assert ctqmc._real("beta") == 25.5         # tabs are blanks
    assert ctqmc._str("QuantumNumbers") == "Nt Szt"
    assert ctqmc._raw("SymMove01") == "1 2"     # commas are blanks
    assert ctqmc._int("N") == 100               # prefix match: first name starting with "N"
    with pytest.raises(KeyError):
        ctqmc._int("Nmeas")
    with pytest.raises(ValueError):
        ctqmc.init_paras("NCorr = 1.5\n")
        ctqmc._int("NCorr")
    ctqmc.dest_paras()


@pytest.mark.parametrize("key,val", [("flavourchange_moves", 1), ("segment", 1),
                                     ("PercentageWormInsert", 0.1), ("statesampling", 1)])
def test_unsupported_modes_are_rejected(key, val):
    ctqmc.init_paras(pstring(dict(BASE, **{key: val})))
    with pytest.raises(NotImplementedError, match=key):
        ctqmc._check_supported()
    ctqmc.dest_paras()


def test_supported_configuration_passes_the_check():
    ctqmc.init_paras(pstring(BASE))
    ctqmc._check_supported()
    ctqmc.dest_paras()
    # automatic block partitioning (the driver's choice for custom U
    # matrices and for off-diagonal H_loc) is supported
    ctqmc.init_paras(pstring(dict(BASE, QuantumNumbers="Nt All", EPSBLOCK=1e-12)))
    ctqmc._check_supported()
    ctqmc.dest_paras()


def test_offdiag_with_global_shift_and_four_operator_moves_passes_the_check():
    ctqmc.init_paras(pstring(dict(BASE, offdiag=1, Percentage4OperatorMove=0.1)))
    ctqmc._check_supported()
    ctqmc.dest_paras()


class _OracleBatch:
    """The batch calls of ctqmc_calibrate served by oracle chains."""

    def __init__(self, chains):
        self.chains = chains
        self.logcap = None

    def set_log(self, cap):
        self.logcap = cap
        for c in self.chains:
            c.start_log(cap)

    def warmup(self, n):
        for c in self.chains:
            c.warmup(n)

    def sync(self):
        pass

    def log(self, i):
        return self.chains[i].log()

    def set_taudiffmax(self, group, tdm):
        for c in self.chains:
            c.set_taudiffmax(tdm)


def _calibration_chains(offdiag, n, seed0):
    if offdiag:
        import exact_bath as XB
        beta, nd = 4.0, 1
        ff = XB.ftau_full_bath(beta, [-0.6, 0.9], [[0.6, 0.3], [0.5, -0.4]], 2000)
        m = O.Model(1, P.flat_umatrix(P.umatrix_density(1, 2.0, 2.0, 0.0)), P.muimp_solver(1, 1.3), "Nt")
        return beta, nd, [O.Chain(m, beta, ff, 10, seed=seed0 + i, p_outer=0.1) for i in range(n)]
    pr = P.config_problem("dd3", beta=10.0)
    m = O.Model(3, pr["umatrix"], pr["muimp"], "Nt Szt")
    return 10.0, 3, [O.Chain(m, 10.0, pr["ftau"], 20, seed=seed0 + i, p_outer=0.1, p_global=0.01,
                             p_shift=0.01) for i in range(n)]


def _first_accepted_dtau(chain, n, nprop):
    chain.start_log(nprop)
    chain.warmup(nprop)
    r = chain.log()
    r = r[(r["outcome"] == 4) & ((r["move"] == 0) | (r["move"] == 1))]
    return np.abs(r["tau_a"] - r["tau_c"])[:n]


@pytest.mark.parametrize("offdiag", [0, 1])
def test_window_calibration_on_oracle_chains(monkeypatch, offdiag):
    """ctqmc_calibrate as cthyb_solver.calibrate_taudiff_max calls it
    (cthyb_solver.py:899-922), run on oracle chains behind the batch calls:
    phase 1 gives the time differences of the first accepted pair moves of
    the chains in turn (the same as one long run of identical chains);
    phase 2 fills the per-flavour histogram over [0, taudiff_max) until
    every flavour has phase2pairnum entries; a calibration that cannot
    finish raises; the proposal records are switched off afterwards."""
    beta, nd, chains = _calibration_chains(offdiag, 3, 40)
    fake = _OracleBatch(chains)
    monkeypatch.setattr(ctqmc, "_batch", fake)
    monkeypatch.setattr(ctqmc, "_nchains", 3)
    monkeypatch.setattr(ctqmc, "_nd", nd)
    monkeypatch.setattr(ctqmc, "_beta", beta)
    monkeypatch.setattr(ctqmc, "_taudiffmax", beta)
    ctqmc.init_paras(pstring(dict(BASE, offdiag=offdiag)))
    ctqmc.ctqmc_calibrate(True, 500, 20, 300, 100000, chunk=400)
    assert fake.logcap == 0
    want = np.concatenate([_first_accepted_dtau(c, 167, 20000)
                           for c in _calibration_chains(offdiag, 3, 40)[2]])[:500]
    assert ctqmc.accpairtau.shape == (500,)
    assert np.array_equal(ctqmc.accpairtau, want)
    tdm = float(np.sort(ctqmc.accpairtau)[int(0.995 * 500)])
    assert 0.0 < tdm <= beta
    ctqmc.set_taudiffmax(tdm)
    assert ctqmc._taudiffmax == tdm
    ctqmc.ctqmc_calibrate(False, 500, 10, 200, 100000, chunk=400)
    assert ctqmc.accpair.shape == (nd, 2, 10)
    assert ctqmc.accpair.reshape(2 * nd, 10).sum(axis=1).min() >= 200
    assert ctqmc.accpair[..., 0].sum() > ctqmc.accpair[..., -1].sum()  # acceptance falls with the distance
    with pytest.raises(RuntimeError, match="calibration"):
        ctqmc.ctqmc_calibrate(False, 500, 10, 10 ** 9, 100000, chunk=50, max_chunks=2)
    assert fake.logcap == 0
    ctqmc.dest_paras()


class _OracleSolveBatch(_OracleBatch):
    """The batch calls of ctqmc_warmup / ctqmc_measure and the result
    collection, served by oracle chains (results in the engine's layout)."""

    class _G:
        ftau_full = None

    def __init__(self, chains, nd, ftau_full=None):
        super().__init__(chains)
        self.nd = nd
        self.groups = [self._G()]
        self.groups[0].ftau_full = ftau_full

    def results_full(self, i):
        return self.chains[i].results_full()

    def measure(self, n):
        for c in self.chains:
            c.measure(n)

    def reset_measurements(self):
        pass

    def results(self, i):
        r = self.chains[i].results()
        cnt = self.chains[i].counters()
        return dict(gtau=r["gtau"].reshape(self.nd, 2, -1), mean_sign=r["mean_sign"],
                    densitymatrix=r["densitymatrix"], histo=r["histo"].reshape(self.nd, 2, -1),
                    counters={k: cnt[k] for k in ("try_add", "acc_add", "try_rem", "acc_rem")})

    def results_extra(self, i):
        x = self.chains[i].results_extra()
        x["gleg"] = x["gleg"].reshape(self.nd, 2, -1)
        if self.groups[0].ftau_full is not None:
            x["gleg"] = np.zeros_like(x["gleg"])  # offdiag = 1: GLeg stays zero
        return x

    def results_gleg_full(self, i):
        return self.chains[i].gleg_full()

    def move_counters(self, i):
        cnt = self.chains[i].counters()
        return {k: cnt[k] for k in ("try_glob", "acc_glob", "try_shift", "acc_shift", "try_add4",
                                    "acc_add4", "try_rem4", "acc_rem4")}


# module variables cthyb_solver.get_resultset reads in every Z-space run
# (cthyb_solver.py:946-977); it copies each with .copy() (1028-1030)
RESULTSET = ["gtau", "gtau_full", "rhisto", "lhisto", "histo", "statessuperstates",
             "eigenstatesenergies", "occbasismapping", "outersuperstatehisto", "outerstatehisto",
             "signhistosuperstates", "signhistostates", "tracecontribsuperstates",
             "tracecontribstates", "occ", "gleg", "gleg_full", "accadd", "accadd4", "accrem",
             "accrem4", "accpair", "accglob", "accshift", "accflavc", "mean_sign", "time_warmup",
             "time_sim", "time_sim_steps", "ssquare_operator", "densitymatrix", "rho2", "rho1",
             "ssquare"]


def test_module_results_on_oracle_chains(monkeypatch):
    """ctqmc_warmup / ctqmc_measure and the result collection of the module
    with two oracle chains behind the batch calls (the host model set-up is
    the engine's own, which needs no GPU): every module variable the
    driver's get_resultset reads exists and copies like an f2py variable,
    with the driver's shapes, and G(tau), the sign and the histogram are the
    sign-weighted combination of the chains."""
    from w2dynamics_gb300 import engine as E
    pr = P.config_problem("dd3", beta=10.0)
    nd, ntau = 3, BASE["Ntau"]
    par = dict(BASE, Nmeas=40, GPUChains=2)
    ctqmc.init_paras(pstring(par))
    mo = O.Model(nd, pr["umatrix"], pr["muimp"], "Nt Szt")
    chains = [O.Chain(mo, 10.0, pr["ftau"], ntau, seed=11 + i, taudiff_max=5.0, ncorr=BASE["NCorr"],
                      p_outer=0.1, maxhisto=BASE["MaxHisto"] + 1, p_global=0.005, p_shift=0.005,
                      nleg=BASE["NLegMax"], symmoves=[[2, 3, 1, 5, 6, 4]], p_4op=0.1)
              for i in range(2)]
    fake = _OracleSolveBatch(chains, nd)
    model = E.Model(nd, pr["umatrix"], pr["muimp"], "Nt Szt")
    for key, val in (("_batch", fake), ("_model", model), ("_nd", nd), ("_nchains", 2), ("_beta", 10.0)):
        monkeypatch.setattr(ctqmc, key, val)
    ctqmc._model_tables()
    ctqmc.ctqmc_warmup(500)
    ctqmc.ctqmc_measure(1, 1)
    for name in RESULTSET:
        v = getattr(ctqmc, name)
        assert isinstance(v, np.ndarray), name
        v.copy()
    assert ctqmc.gtau.shape == (nd, 2, ntau) and ctqmc.gtau_full.shape == (nd, 2, nd, 2, ntau)
    assert ctqmc.gleg_full.shape == (nd, 2, nd, 2, BASE["NLegMax"])
    assert ctqmc.accpair.shape == (nd, 2, ntau)
    assert ctqmc.rho1.size == (2 * nd) ** 2 and ctqmc.rho2.size == (2 * nd) ** 4
    rs = [c.results() for c in chains]
    s = np.array([r["mean_sign"] for r in rs])
    want = sum(r["gtau"] * w for r, w in zip(rs, s)) / s.sum()
    assert np.allclose(ctqmc.gtau.reshape(2 * nd, ntau), want, rtol=1e-13, atol=0)
    assert ctqmc.mean_sign == s.mean()
    assert np.array_equal(ctqmc.histo.reshape(2 * nd, -1), sum(r["histo"] for r in rs) / 2)
    assert 0.0 < float(ctqmc.accadd4) < 1.0
    ctqmc.dest_paras()


def test_offdiag_module_results_on_oracle_chains(monkeypatch):
    """offdiag = 1 through the module's result collection with two oracle
    chains: gtau_full[b, s, b', s'] is the sign-weighted Gtau_full of the
    chains at (flavour 2b + s, flavour 2b' + s'), including the spin-mixing
    element."""
    import exact_bath as XB
    from w2dynamics_gb300 import engine as E
    beta, ntau = 4.0, 10
    ff = XB.ftau_full_bath(beta, [-0.6, 0.9], [[0.6, 0.3], [0.5, -0.4]], 2000)
    um = P.flat_umatrix(P.umatrix_density(1, 2.0, 2.0, 0.0))
    muimp = P.muimp_solver(1, 1.3)
    par = dict(BASE, beta=beta, Nd=1, Ntau=ntau, QuantumNumbers="Nt", offdiag=1, Nmeas=300, NCorr=20,
               PercentageGlobalMove=0.05, PercentageTauShiftMove=0.05, Percentage4OperatorMove=0.0,
               NSymMove=0, MeasSsquare=0, NLegMax=8)
    ctqmc.init_paras(pstring(par))
    ctqmc._check_supported()
    mo = O.Model(1, um, muimp, "Nt")
    chains = [O.Chain(mo, beta, ff, ntau, seed=3 + i, taudiff_max=1.5, ncorr=20, p_outer=0.1,
                      maxhisto=BASE["MaxHisto"] + 1, p_global=0.05, p_shift=0.05, nleg=8) for i in range(2)]
    fake = _OracleSolveBatch(chains, 1, ftau_full=ff)
    model = E.Model(1, um, muimp, "Nt")
    for key, val in (("_batch", fake), ("_model", model), ("_nd", 1), ("_nchains", 2), ("_beta", beta)):
        monkeypatch.setattr(ctqmc, key, val)
    ctqmc._model_tables()
    ctqmc.ctqmc_warmup(2000)
    ctqmc.ctqmc_measure(1, 1)
    s = np.array([c.results()["mean_sign"] for c in chains])
    want = sum(c.results_full() * w for c, w in zip(chains, s)) / s.sum()
    got = np.array([[ctqmc.gtau_full[fa // 2, fa % 2, fc // 2, fc % 2] for fc in range(2)] for fa in range(2)])
    assert np.allclose(got, want, rtol=1e-13, atol=0)
    assert np.abs(got[0, 1]).max() > 0.01
    # GLeg_full of every flavour pair, GLeg zero (MeasGtauRem_full only)
    wl = sum(c.gleg_full() * w for c, w in zip(chains, s)) / s.sum()
    gl = np.array([[ctqmc.gleg_full[fa // 2, fa % 2, fc // 2, fc % 2] for fc in range(2)] for fa in range(2)])
    assert gl.shape == (2, 2, 8) and np.allclose(gl, wl, rtol=1e-13, atol=0)
    assert np.abs(gl[0, 1]).max() > 0.0 and not np.any(ctqmc.gleg)
    for name in RESULTSET:
        if name not in ("ssquare", "ssquare_operator"):
            getattr(ctqmc, name).copy()
    ctqmc.dest_paras()


@pytest.mark.gpu
def test_solve_through_the_module_matches_the_oracle():
    """init_rnd/init_paras/init_solver/set_taudiffmax/ctqmc_warmup/
    ctqmc_measure as cthyb_solver.py calls them, with the default global and
    tau-shift move percentages; the results equal the oracle chain of the
    same seed (identical proposal streams)."""
    pr = P.config_problem("dd3", beta=10.0)
    nd, ntau = 3, BASE["Ntau"]
    ftau = pr["ftau"]
    ftau_full = np.zeros((nd, 2, nd, 2, ftau.shape[-1]))
    for b in range(nd):
        for s in range(2):
            ftau_full[b, s, b, s] = ftau[b, s]
    umat = np.asarray(pr["umatrix"]).reshape((2 * nd,) * 4)
    ctqmc.init_rnd(11)
    ctqmc.init_paras(pstring(BASE))
    ctqmc.init_solver(umat, ftau_full, pr["muimp"], np.zeros_like(ftau_full), 1)
    ctqmc.set_taudiffmax(BASE["TaudiffMax"])
    ctqmc.ctqmc_warmup(BASE["Nwarmups"])
    ctqmc.ctqmc_measure(1, 1)
    mo = O.Model(nd, pr["umatrix"], pr["muimp"], "Nt Szt")
    co = O.Chain(mo, 10.0, ftau, ntau, seed=11, taudiff_max=5.0, ncorr=BASE["NCorr"],
                 p_outer=0.1, maxhisto=BASE["MaxHisto"] + 1, p_global=0.005, p_shift=0.005,
                 nleg=BASE["NLegMax"], symmoves=[[2, 3, 1, 5, 6, 4]], p_4op=0.1)
    co.set_taudiffmax(5.0)
    co.warmup(BASE["Nwarmups"])
    co.measure(BASE["Nmeas"])
    ro = co.results()
    assert ctqmc.mean_sign == ro["mean_sign"]
    gg = np.stack([ctqmc.gtau[f // 2, f % 2] for f in range(2 * nd)])
    assert np.allclose(gg, ro["gtau"], rtol=1e-9, atol=1e-12)
    hg = np.stack([ctqmc.histo[f // 2, f % 2] for f in range(2 * nd)])
    assert np.array_equal(hg, ro["histo"])
    evec = np.zeros((mo.nstates, mo.nstates))
    for s in range(len(mo.sst_size)):
        o, n = mo.sst_offset[s], mo.sst_size[s]
        evec[o:o + n, o:o + n] = mo.evec(s)
    ref = ES.from_density_matrix(nd, mo.fock_states, evec, ro["densitymatrix"])
    assert np.allclose(ctqmc.densitymatrix, ref["densitymatrix"], atol=1e-10)
    assert np.allclose(ctqmc.occ, ref["occ"], atol=1e-10)
    assert np.allclose(ctqmc.rho1, ref["rho1"], atol=1e-10)
    ssq, _ = ES.spin_square(nd, mo.fock_states, mo.sst_size, mo.sst_offset, ref["densitymatrix"])
    assert np.allclose(ctqmc.ssquare, ssq, atol=1e-10)
    assert ctqmc.ssquare_operator.shape == (mo.nstates, mo.nstates)
    assert ctqmc.gtau_full.shape == (nd, 2, nd, 2, ntau)
    xo = co.results_extra()
    gl = np.stack([ctqmc.gleg[f // 2, f % 2] for f in range(2 * nd)])
    assert np.allclose(gl, xo["gleg"], rtol=1e-9, atol=1e-12 * np.abs(xo["gleg"]).max())
    assert np.array_equal(ctqmc.outersuperstatehisto, xo["outer_sst_histo"])
    assert np.allclose(ctqmc.signhistosuperstates, xo["sign_sst"], equal_nan=True)
    assert ctqmc.occbasismapping.shape == (mo.nstates, nd, 2)
    cnt = co.counters()
    assert ctqmc.accadd[0] == cnt["acc_add"] / cnt["try_add"]
    assert ctqmc.accadd4 == cnt["acc_add4"] / cnt["try_add4"] and cnt["acc_add4"] > 0
    n, outer, _ = ctqmc.get_mc_config_scalars()
    taus, orbs, spins, cas, hashybs, outer2, _ = ctqmc.get_mc_config(n)
    t_o, *_ = co.get_config()
    assert np.array_equal(taus, t_o) and outer2 == outer
    ctqmc.dest_ctqmc()
    ctqmc.dest_paras()


@pytest.mark.gpu
def test_warm_start_files_for_all_chains(tmp_path):
    """save_mc_configs / load_mc_configs keep each of GPUChains = 6 chains'
    configuration across solves; a one-configuration file in the driver's
    CtHybConfig npz layout (cthyb_solver.py:78-87) goes to every chain; the
    warm-started chains keep running."""
    pr = P.config_problem("dd3", beta=10.0)
    nd = 3
    ftau = pr["ftau"]
    ftau_full = np.zeros((nd, 2, nd, 2, ftau.shape[-1]))
    for b in range(nd):
        for s in range(2):
            ftau_full[b, s, b, s] = ftau[b, s]
    umat = np.asarray(pr["umatrix"]).reshape((2 * nd,) * 4)
    par = dict(BASE, GPUChains=6, Nmeas=5)

    def solver():
        ctqmc.init_rnd(3)
        ctqmc.init_paras(pstring(par))
        ctqmc.init_solver(umat, ftau_full, pr["muimp"], np.zeros_like(ftau_full), 1)
        ctqmc.set_taudiffmax(BASE["TaudiffMax"])

    solver()
    ctqmc.ctqmc_warmup(1500)
    before = ctqmc.get_mc_configs()
    assert len(before["offsets"]) == 7 and before["offsets"][-1] > 0
    ctqmc.save_mc_configs(tmp_path / "cfg.npz")
    ctqmc.dest_ctqmc()
    solver()
    ctqmc.load_mc_configs(tmp_path / "cfg.npz")
    after = ctqmc.get_mc_configs()
    for k in ("offsets", "taus", "orbs", "spins", "cas", "outer_sst"):
        assert np.array_equal(before[k], after[k]), k
    # one configuration in the driver's layout
    n = before["offsets"][1]
    np.savez(tmp_path / "one.npz", taus=before["taus"][:n], orbs=before["orbs"][:n],
             spins=before["spins"][:n], cas=before["cas"][:n], hashybs=np.ones(n, int),
             outer_sst=np.array([before["outer_sst"][0]]), outer_state=np.array([1]))
    ctqmc.load_mc_configs(tmp_path / "one.npz")
    rep = ctqmc.get_mc_configs()
    assert np.array_equal(rep["offsets"], np.arange(7) * n)
    for c in range(6):
        assert np.array_equal(rep["taus"][c * n:(c + 1) * n], before["taus"][:n])
    ctqmc.ctqmc_measure(1, 1)
    assert np.isfinite(ctqmc.gtau).all()
    ctqmc.dest_ctqmc()
    ctqmc.dest_paras()


@pytest.mark.gpu
def test_offdiag_solve_through_the_module_matches_the_oracle():
    """offdiag = 1 through the module (pair and outer-superstate moves): the
    Gtau_full of the solve equals the oracle chain of the same seed."""
    import exact_bath as XB
    beta = 4.0
    ff = XB.ftau_full_bath(beta, [-0.6, 0.9], [[0.6, 0.3], [0.5, -0.4]], 2000)
    um = P.flat_umatrix(P.umatrix_density(1, 2.0, 2.0, 0.0))
    muimp = P.muimp_solver(1, 1.3)
    par = dict(BASE, beta=beta, Nd=1, Ntau=10, QuantumNumbers="Nt", offdiag=1, Nmeas=400,
               NCorr=20, PercentageGlobalMove=0.0, PercentageTauShiftMove=0.0,
               Percentage4OperatorMove=0.0, TaudiffMax=1.5, NSymMove=0, MeasSsquare=0)
    ctqmc.init_rnd(17)
    ctqmc.init_paras(pstring(par))
    ctqmc.init_solver(np.asarray(um).reshape((2,) * 4), ff, muimp, np.zeros_like(ff), 1)
    ctqmc.set_taudiffmax(1.5)
    ctqmc.ctqmc_warmup(3000)
    ctqmc.ctqmc_measure(1, 1)
    mo = O.Model(1, um, muimp, "Nt")
    co = O.Chain(mo, beta, ff, 10, seed=17, taudiff_max=1.5, ncorr=20, p_outer=0.1,
                 maxhisto=par["MaxHisto"] + 1)
    co.set_taudiffmax(1.5)
    co.warmup(3000)
    co.measure(400)
    go = co.results_full()
    got = np.array([[ctqmc.gtau_full[fa // 2, fa % 2, fc // 2, fc % 2] for fc in range(2)] for fa in range(2)])
    assert np.allclose(got, go, rtol=1e-9, atol=1e-12 * np.abs(go).max())
    assert np.abs(go[0, 1]).max() > 0.01
    assert ctqmc.mean_sign == co.results()["mean_sign"]
    ctqmc.dest_ctqmc()
    ctqmc.dest_paras()
