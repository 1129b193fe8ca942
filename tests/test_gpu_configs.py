"""Parity and statistics at the benchmark's own configurations.

Proposal-by-proposal parity with the oracle (same seed, so the same
proposal stream; bookkeeping bit-exact, ratios to 1e-10) on
  * the single-orbital Anderson impurity (U = 2, mu = U/2, beta = 10,
    semicircular bath D = 1, Nftau = Ntau = 1000, TaudiffMax = beta, seed 0,
    pair moves only), then G(tau) on all 1000 bins after the measurement;
  * the 3-orbital density-density model (U = 4, J = 0.6, U' = U - 2J,
    "Nt Szt") at beta = 50 with Nftau = Ntau = 2000: 2e4 thermalisation
    proposals and 1e4 more, all compared, then G(tau) on 2000 bins;
  * the 5-orbital Kanamori model (U = 3, J = 0.7, crystal field +-0.2,
    beta = 40, Nftau = Ntau = 4000) with "Nt Szt" blocks (up to 100 x 100)
    at thermalised expansion order, and a short case with "Nt" blocks (up
    to 252 x 252).
Statistics (the 2-sigma criterion): G(tau), occupancies and double
occupancies of GPU chains against an oracle run with equal total samples
and different seeds, for the Anderson impurity and for the mixed-beta batch
of the 3-orbital model (beta in {10, 25, 50, 100} in one launch).

Every parity case prints the largest deviation from the oracle of each
compared quantity.
"""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import estimators as ES
from w2dynamics_gb300 import problems as P

from test_gpu_parity import EXACT, compare_logs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return E.load(build_if_missing=True)


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def _deviations(ref, got):
    ev = ref["outcome"] >= 3
    p = ev & (ref["prob"] > 0)
    out = {
        "proposals": len(ref), "accepted": int((ref["outcome"] == 4).sum()),
        "bookkeeping_mismatches": int(sum(np.sum(ref[k] != got[k]) for k in EXACT)),
        "max_dlog_detrat": float(np.abs(ref["det_log"][ev] - got["det_log"][ev]).max()) if ev.any() else 0.0,
        "max_dlog_trace": float(np.abs(ref["tr_log"][ev] - got["tr_log"][ev]).max()) if ev.any() else 0.0,
        "max_rel_prob": float(np.abs(got["prob"][p] / ref["prob"][p] - 1).max()) if p.any() else 0.0,
    }
    return out


def _pair(name, beta, qns, tdm, ntau, nwarm, nmeas, seed, ncorr=100, opcap=512, kcap=64, tree_levels=0):
    pr = P.config_problem(name, beta=beta)
    q = qns or pr["quantum_numbers"]
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    co = O.Chain(mo, beta, pr["ftau"], ntau, seed=seed, taudiff_max=tdm, ncorr=ncorr)
    ntot = nwarm + nmeas * ncorr
    co.start_log(ntot)
    co.warmup(nwarm)
    if nmeas:
        co.measure(nmeas)
    ref = co.log()
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], q)
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], ntau, nchains=1, seed0=seed, taudiff_max=tdm, ncorr=ncorr,
                             kcap=kcap, opcap=opcap, tree_levels=tree_levels)])
    b.set_log(ntot)
    b.warmup(nwarm)
    if nmeas:
        b.measure(nmeas)
    b.sync()
    return pr, mo, co, ref, mg, b, b.log(0)


def _compare_measurement(co, b, nd, label):
    ro, rg = co.results(), b.results(0)
    go = ro["gtau"]
    gg = np.stack([rg["gtau"][f // 2, f % 2] for f in range(2 * nd)])
    dev = {"max_rel_gtau": _rel(gg, go), "max_rel_dm_diag": _rel(np.diag(rg["densitymatrix"]),
                                                                  np.diag(ro["densitymatrix"])),
           "sign_equal": rg["mean_sign"] == ro["mean_sign"]}
    print(f"\n{label}: measurement deviations {dev}")
    assert dev["sign_equal"]
    assert np.allclose(gg, go, rtol=1e-9, atol=1e-12 * np.abs(go).max())
    assert np.allclose(np.diag(rg["densitymatrix"]), np.diag(ro["densitymatrix"]), rtol=1e-9, atol=1e-12)
    ho = ro["histo"]
    hg = np.stack([rg["histo"][f // 2, f % 2] for f in range(2 * nd)])
    assert np.array_equal(hg[:, :ho.shape[1]], ho)
    return dev


def test_anderson_impurity_config_parity(lib):
    """U = 2, beta = 10, Ntau = Nftau = 1000, TaudiffMax = beta, seed 0:
    1e4 thermalisation proposals and 2e4 measured proposals, then G(tau) on
    all 1000 bins."""
    pr, mo, co, ref, mg, b, got = _pair("anderson1", 10.0, None, 10.0, 1000, 10000, 200, 0)
    dev = _deviations(ref, got)
    print(f"\nanderson1 beta=10: proposal deviations {dev}")
    compare_logs(ref, got, pr["ftau"][0, 0], 10.0)
    _compare_measurement(co, b, 1, "anderson1 beta=10")


def test_three_orbital_beta50_config_parity(lib):
    """3-orbital density-density model, beta = 50, Nftau = Ntau = 2000,
    "Nt Szt", seed 0: 2e4 thermalisation proposals and 1e4 measured
    proposals at the thermalised order, then G(tau) on 2000 bins."""
    pr, mo, co, ref, mg, b, got = _pair("dd3", 50.0, None, 5.0, 2000, 20000, 100, 0)
    dev = _deviations(ref, got)
    k_late = ref["k_total"][20000:]
    print(f"\ndd3 beta=50: proposal deviations {dev}; operators in the measured part "
          f"{k_late.min()}..{k_late.max()} (mean {k_late.mean():.1f})")
    assert k_late.mean() > 60  # thermalised expansion order at beta = 50
    compare_logs(ref, got, pr["ftau"][0, 0], 50.0)
    _compare_measurement(co, b, 3, "dd3 beta=50")
    so, sg = co.state(), b.state(0)
    assert abs(so["det_log"] - sg["det_log"]) < 1e-8 and so["cfgsign"] == sg["cfgsign"]


# seeds whose initial outer superstate has 100 (seed 0), 50 (seed 7) and 5
# (seed 4) states under "Nt Szt"; 210 states (seed 4) under "Nt"
@pytest.mark.parametrize("qns,seed,nwarm,nlog", [("Nt Szt", 0, 1500, 1000), ("Nt Szt", 7, 2000, 1000),
                                                 ("Nt Szt", 4, 2000, 1000), ("Nt", 4, 150, 100)])
def test_kanamori5_config_parity(lib, qns, seed, nwarm, nlog):
    """5-orbital Kanamori model with spin-flip and pair hopping, beta = 40,
    Nftau = Ntau = 4000, one window: dense blocks of up to 100 x 100 ("Nt
    Szt") after thermalisation, or 252 x 252 ("Nt"), proposal by proposal."""
    pr, mo, co, ref, mg, b, got = _pair("kanamori5", 40.0, qns, -1.0, 4000, nwarm + nlog, 0, seed,
                                        opcap=1024, tree_levels=4)
    dev = _deviations(ref, got)
    outer = int(co.state()["outer_sst"])
    size = int(mo.sst_size[outer])
    print(f"\nkanamori5 beta=40 {qns} seed {seed}: proposal deviations {dev}; final operators "
          f"{int(ref['k_total'][-1])}, outer superstate of {size} states, largest block "
          f"{int(max(mo.sst_size))}")
    compare_logs(ref, got)
    assert (ref["outcome"][nwarm:] == 4).sum() > 10


def _occupations(nd, dm, fock, evec):
    est = ES.from_density_matrix(nd, fock, evec, dm)
    occ = est["occ"]
    n = np.array([occ[f // 2, f % 2, f // 2, f % 2] for f in range(2 * nd)])
    d = np.array([occ[b, 0, b, 1] for b in range(nd)])
    return n, d


def _oracle_evec(mo):
    ev = np.zeros((mo.nstates, mo.nstates))
    for s in range(len(mo.sst_size)):
        o, n_ = mo.sst_offset[s], mo.sst_size[s]
        ev[o:o + n_, o:o + n_] = mo.evec(s)
    return ev


def _z(a, b_):
    a, b_ = np.asarray(a), np.asarray(b_)
    se = np.sqrt(a.var(axis=0, ddof=1) / len(a) + b_.var(axis=0, ddof=1) / len(b_))
    return (a.mean(axis=0) - b_.mean(axis=0)) / se


def _check_z(z, label, frac2=0.8, zmax=3.5):
    """The 2-sigma criterion over a set of independent comparisons: at
    least `frac2` of them within 2 sigma (about 95 % expected) and none
    beyond `zmax` sigma."""
    z = np.abs(np.ravel(z))
    assert np.mean(z < 2.0) >= frac2 and z.max() < zmax, (label, z)


def _coarse(g, nbin):
    """G(tau) averaged over nbin consecutive bins (last axis)."""
    n = g.shape[-1] // nbin * nbin
    return g[..., :n].reshape(g.shape[:-1] + (-1, nbin)).mean(axis=-1)


def test_anderson_impurity_statistics_two_sigma(lib):
    """GPU: 100 chains x 1000 measurements of NCorr = 100 proposals (1e5
    measurement cycles, 1e7 proposals after thermalisation); oracle: 100
    chains x 1000 measurements with other seeds (equal total samples; as
    many independent chains on both sides, so the z-scores are close to
    normal).
    Occupancies and double occupancy, G(tau) on 1000 bins (90 % within 2
    sigma, all within 5) and G averaged over 50-bin windows, by the 2-sigma
    criterion of _check_z."""
    pr = P.config_problem("anderson1", beta=10.0)
    nd, beta, ntau = 1, 10.0, 1000
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    fk, evec = mg.basis()
    nch = 100
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], ntau, nchains=nch, seed0=100, taudiff_max=beta, ncorr=100)])
    b.warmup(10000)
    b.measure(1000)
    b.sync()
    gg, gn, gd = [], [], []
    for c in range(nch):
        r = b.results(c)
        gg.append(np.stack([r["gtau"][f // 2, f % 2] for f in range(2 * nd)]))
        n, d = _occupations(nd, r["densitymatrix"], fk, evec)
        gn.append(n)
        gd.append(d)
    mo = O.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    ev = _oracle_evec(mo)
    cg, cn, cd = [], [], []
    for c in range(nch):
        co = O.Chain(mo, beta, pr["ftau"], ntau, seed=9000 + c, taudiff_max=beta, ncorr=100)
        co.warmup(10000)
        co.measure(1000)
        r = co.results()
        cg.append(r["gtau"])
        n, d = _occupations(nd, r["densitymatrix"], mo.fock_states, ev)
        cn.append(n)
        cd.append(d)
    zg, zn, zd = _z(gg, cg), _z(gn, cn), _z(gd, cd)
    zc = _z(_coarse(np.array(gg), 50), _coarse(np.array(cg), 50))
    print(f"\nanderson1 statistics: occupancy z {zn}, double occupancy z {zd}, G within 2 sigma "
          f"{np.mean(np.abs(zg) < 2):.3f}, max |z| {np.abs(zg).max():.2f}, coarse max |z| {np.abs(zc).max():.2f}")
    _check_z(np.concatenate([zn, zd]), "occupancies", frac2=0.6)
    _check_z(zg, "G(tau)", frac2=0.9, zmax=5.0)
    _check_z(zc, "G(tau) 50-bin windows", frac2=0.8)


def test_mixed_beta_batch_statistics_two_sigma(lib):
    """The batched configuration's model with beta in {10, 25, 50, 100} in
    ONE launch (16 chains per beta) against 16 oracle chains per beta with
    the same measurements (equal total samples): occupancies and double
    occupancies of all betas, and G(tau) averaged over 100-bin windows, by
    the 2-sigma criterion of _check_z."""
    betas = (10.0, 25.0, 50.0, 100.0)
    ntau, ncorr, nch, nmeas, nwarm = 2000, 100, 16, 150, 20000
    prs = [P.config_problem("dd3", beta=bb) for bb in betas]
    nd = 3
    mg = E.Model(nd, prs[0]["umatrix"], prs[0]["muimp"], prs[0]["quantum_numbers"])
    fk, evec = mg.basis()
    moves = dict(p_outer=0.1, p_global=0.005, p_shift=0.005)
    groups = [E.Group(bb, pr["ftau"], ntau, nchains=nch, seed0=200 + 100 * i, taudiff_max=5.0, ncorr=ncorr,
                      kcap=64, opcap=1024, **moves) for i, (bb, pr) in enumerate(zip(betas, prs))]
    b = E.Batch(mg, groups)
    b.warmup(nwarm)
    b.measure(nmeas)
    b.sync()
    mo = O.Model(nd, prs[0]["umatrix"], prs[0]["muimp"], prs[0]["quantum_numbers"])
    ev = _oracle_evec(mo)
    report, zs, zcs = {}, [], []
    for i, (bb, pr) in enumerate(zip(betas, prs)):
        gg, gn, gd = [], [], []
        for c in range(i * nch, (i + 1) * nch):
            r = b.results(c)
            gg.append(np.stack([r["gtau"][f // 2, f % 2] for f in range(2 * nd)]))
            n, d = _occupations(nd, r["densitymatrix"], fk, evec)
            gn.append(n)
            gd.append(d)
        cg, cn, cd = [], [], []
        for c in range(nch):
            co = O.Chain(mo, bb, pr["ftau"], ntau, seed=7000 + 100 * i + c, taudiff_max=5.0, ncorr=ncorr,
                         **moves)
            co.warmup(nwarm)
            co.measure(nmeas)
            r = co.results()
            cg.append(r["gtau"])
            n, d = _occupations(nd, r["densitymatrix"], mo.fock_states, ev)
            cn.append(n)
            cd.append(d)
        zn, zd = _z(gn, cn), _z(gd, cd)
        zc = _z(_coarse(np.array(gg), 100), _coarse(np.array(cg), 100))
        report[bb] = (np.round(zn, 2).tolist(), np.round(zd, 2).tolist(), float(np.abs(zc).max()))
        zs.append(np.concatenate([zn, zd]))
        zcs.append(np.ravel(zc))
    print(f"\nmixed-beta batch statistics (occupancy z, double occupancy z, coarse G max |z|): {report}")
    _check_z(np.concatenate(zs), "occupancies and double occupancies", zmax=4.0)
    _check_z(np.concatenate(zcs), "G(tau) 100-bin windows")
