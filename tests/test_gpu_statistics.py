"""Statistical checks of the GPU engine.

1. G(tau), occupancies and double occupancies of a batch of GPU chains fall
   within the statistical error of an oracle (CPU) run with the same total
   number of samples but different seeds.
2. Detailed balance: the expansion-order histogram and occupations of GPU
   chains on a single-orbital impurity with a discrete asymmetric bath equal
   exact diagonalisation of impurity + bath.
3. Equal error at equal samples: the G(tau) error of a batch of n chains and
   of one chain run n times longer agree, so MC updates/s of the two forms
   compare at equal statistical error.
"""
import numpy as np
import pytest

import exact_bath as XB
import oracle as O
from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import estimators as ES
from w2dynamics_gb300 import problems as P

pytestmark = pytest.mark.gpu

BETA, NTAU, NCORR, NCH, NMEAS, NWARM = 10.0, 20, 50, 16, 400, 3000


def _occ(model_like, nd, dm, fock, evec):
    est = ES.from_density_matrix(nd, fock, evec, dm)
    return np.array([est["occ"][f // 2, f % 2, f // 2, f % 2] for f in range(2 * nd)]), est["occ"]


def test_gpu_batch_agrees_with_cpu_run_within_errors():
    pr = P.config_problem("dd3", beta=BETA)
    nd = pr["nd"]
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    fk, evec = mg.basis()
    b = E.Batch(mg, [E.Group(BETA, pr["ftau"], NTAU, nchains=NCH, seed0=1000, taudiff_max=5.0,
                             ncorr=NCORR, kcap=64, opcap=512, p_outer=0.1, p_global=0.005,
                             p_shift=0.005)])
    b.warmup(NWARM)
    b.measure(NMEAS)
    b.sync()
    gpu_g, gpu_n, gpu_d = [], [], []
    for c in range(NCH):
        r = b.results(c)
        gpu_g.append(np.stack([r["gtau"][f // 2, f % 2] for f in range(2 * nd)]))
        n, occ = _occ(mg, nd, r["densitymatrix"], fk, evec)
        gpu_n.append(n)
        gpu_d.append(occ[0, 0, 0, 1])  # double occupancy of orbital 1
    mo = O.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    ev = np.zeros((mo.nstates, mo.nstates))
    for s in range(len(mo.sst_size)):
        o, n_ = mo.sst_offset[s], mo.sst_size[s]
        ev[o:o + n_, o:o + n_] = mo.evec(s)
    cpu_g, cpu_n, cpu_d = [], [], []
    for c in range(NCH):
        co = O.Chain(mo, BETA, pr["ftau"], NTAU, seed=5000 + c, taudiff_max=5.0, ncorr=NCORR,
                     p_outer=0.1, p_global=0.005, p_shift=0.005)
        co.warmup(NWARM)
        co.measure(NMEAS)
        r = co.results()
        cpu_g.append(r["gtau"])
        n, occ = _occ(mo, nd, r["densitymatrix"], mo.fock_states, ev)
        cpu_n.append(n)
        cpu_d.append(occ[0, 0, 0, 1])

    def z(a, b_):
        a, b_ = np.asarray(a), np.asarray(b_)
        se = np.sqrt(a.var(axis=0, ddof=1) / len(a) + b_.var(axis=0, ddof=1) / len(b_))
        return (a.mean(axis=0) - b_.mean(axis=0)) / se

    zg = z(gpu_g, cpu_g)
    assert np.mean(np.abs(zg) < 2.0) > 0.85 and np.abs(zg).max() < 4.5, zg
    zn = z(gpu_n, cpu_n)
    assert np.abs(zn).max() < 4.0, zn
    assert abs(z(gpu_d, cpu_d)) < 4.0


def test_equal_error_batched_and_one_chain_forms():
    pr = P.config_problem("dd3", beta=BETA)
    nd = pr["nd"]
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    # outer-superstate, global and tau-shift moves make each chain ergodic
    # over the superstate sectors (pair moves alone keep a chain in the
    # sector it starts in)
    moves = dict(p_outer=0.1, p_global=0.005, p_shift=0.005)
    b = E.Batch(mg, [E.Group(BETA, pr["ftau"], NTAU, nchains=NCH, seed0=2000, taudiff_max=5.0,
                             ncorr=NCORR, kcap=64, opcap=512, **moves)])
    b.warmup(NWARM)
    b.measure(NMEAS)
    b.sync()
    batched = np.array([b.results(c)["gtau"] for c in range(NCH)])
    one = E.Batch(mg, [E.Group(BETA, pr["ftau"], NTAU, nchains=1, seed0=3000, taudiff_max=5.0,
                               ncorr=NCORR, kcap=64, opcap=512, **moves)])
    one.warmup(NWARM)
    blocks = []
    for _ in range(NCH):  # the same total samples, in NCH consecutive blocks
        one.reset_measurements()
        one.measure(NMEAS)
        one.sync()
        blocks.append(one.results(0)["gtau"])
    blocks = np.array(blocks)
    err_b = batched.std(axis=0, ddof=1) / np.sqrt(NCH)
    err_1 = blocks.std(axis=0, ddof=1) / np.sqrt(NCH)
    ratio = np.median(err_1 / err_b)
    assert 0.5 < ratio < 2.0, ratio
    zz = (batched.mean(axis=0) - blocks.mean(axis=0)) / np.sqrt(err_b ** 2 + err_1 ** 2)
    assert np.abs(zz).max() < 4.5


@pytest.mark.parametrize("p_4op", [0.0, 0.5])
def test_detailed_balance_against_exact_diagonalisation(p_4op):
    """64 GPU chains (sliding windows, outer-superstate, global and tau-shift
    moves, and with p_4op = 0.5 half of the insertions and removals as
    4-operator moves) of the single-orbital impurity with two bath levels:
    per-flavour order histogram and occupations within 4.5 standard errors
    of the exact values (tests/exact_bath.py)."""
    beta, mu, u, eps, v = 4.0, 1.3, 2.0, [-0.6, 0.9], [0.6, 0.8]
    pex = XB.order_marginal(beta, mu, u, eps, v)[:30]
    nup, ndn, dbl = XB.occupations(beta, mu, u, eps, v)
    um = P.flat_umatrix(P.umatrix_density(1, u, u, 0.0))
    f = XB.ftau_bath(beta, eps, v, 2000)
    mg = E.Model(1, um, P.muimp_solver(1, mu), "Nt Szt Azt")
    fk, evec = mg.basis()
    n = 64
    b = E.Batch(mg, [E.Group(beta, np.broadcast_to(f, (1, 2, 2000)).copy(), 20, nchains=n, seed0=500,
                             taudiff_max=1.0, ncorr=20, kcap=32, opcap=128, maxhisto=30, p_outer=0.1,
                             p_global=0.01, p_shift=0.01, p_4op=p_4op)])
    b.warmup(2000)
    b.measure(5000)
    b.sync()
    hist, occ = [], []
    for c in range(n):
        r = b.results(c)
        h = r["histo"].reshape(2, -1)
        hist.append(h / h.sum(axis=1, keepdims=True))
        o = ES.from_density_matrix(1, fk, evec, r["densitymatrix"])["occ"]
        occ.append([o[0, 0, 0, 0], o[0, 1, 0, 1], o[0, 0, 0, 1]])
    hist, occ = np.array(hist), np.array(occ)
    sel = pex > 1e-3
    z = (hist.mean(0)[:, sel] - pex[sel]) / (hist.std(0, ddof=1)[:, sel] / np.sqrt(n))
    assert np.abs(z).max() < 4.5, z
    zo = (occ.mean(0) - [nup, ndn, dbl]) / (occ.std(0, ddof=1) / np.sqrt(n))
    assert np.abs(zo).max() < 4.5, zo
