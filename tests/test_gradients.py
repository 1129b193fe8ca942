"""Backward pass: energy derivatives of the density-density local
Hamiltonian (CPU), and per-configuration gradients of log|w| from the GPU
kernel against central finite differences of the oracle's full LU
determinant and full trace (the dense FP64 reference) on fixed
configurations."""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import gradients as GR
from w2dynamics_gb300 import problems as P


def _dd3_umatrix(u, j):
    return P.flat_umatrix(P.umatrix_density(3, u, u - 2 * j, j))


def test_interaction_energy_matches_model_eigenvalues():
    nd, u, j = 3, 4.0, 0.6
    m = O.Model(nd, _dd3_umatrix(u, j), P.muimp_solver(nd, 0.0), "Nt Szt")
    e = GR.interaction_energy(nd, _dd3_umatrix(u, j), m.fock_states)
    for s, (o, n) in enumerate(zip(m.sst_offset, m.sst_size)):
        assert np.allclose(np.sort(e[o:o + n]), np.sort(m.evals[o:o + n]), atol=1e-12)


def test_energy_derivatives_are_exact_differences():
    nd, u, j, h = 3, 4.0, 0.6, 1e-3
    fock = np.arange(64)
    d = GR.density_density_directions(nd, fock)
    e = lambda uu, jj: GR.interaction_energy(nd, _dd3_umatrix(uu, jj), fock)
    assert np.allclose(d[2 * nd], (e(u + h, j) - e(u - h, j)) / (2 * h), atol=1e-9)
    assert np.allclose(d[2 * nd + 1], (e(u, j + h) - e(u, j - h)) / (2 * h), atol=1e-9)


def _oracle_logw(pr, umat, muimp, ftau, beta, cfg):
    """log|det| and the absolute log|trace| (energies not shifted by the
    ground-state energy, which moves with the parameters) of a fixed
    configuration, from the oracle's full LU determinant and full trace."""
    taus, orbs, spins, cas, outer = cfg
    mo = O.Model(pr["nd"], umat, muimp, pr["quantum_numbers"])
    co = O.Chain(mo, beta, ftau, 20, seed=1, taudiff_max=beta)
    co.set_config(taus, orbs, spins, cas, outer)
    return co.full_det()[0], co.full_trace()[0] - beta * mo.egs


@pytest.mark.gpu
def test_gradients_against_finite_differences():
    from w2dynamics_gb300 import engine as E
    beta, nd, u, j = 10.0, 3, 4.0, 0.6
    pr = P.config_problem("dd3", beta=beta)
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], 20, nchains=8, seed0=40, taudiff_max=5.0,
                             kcap=64, opcap=512)])
    b.warmup(3000)
    b.sync()
    dE = GR.density_density_directions(nd, mg.fock_states)
    gd, gp, lw = b.gradients(dE)
    for ch in (0, 5):
        cfg = b.get_config(ch)
        if len(cfg[0]) == 0:
            continue
        ld0, lt0 = _oracle_logw(pr, pr["umatrix"], pr["muimp"], pr["ftau"], beta, cfg)
        assert abs(lw[ch, 0] - ld0) < 1e-9 * max(1, abs(ld0))
        assert abs(lw[ch, 1] - lt0) < 1e-9 * max(1, abs(lt0))
        # d log|det| / dF on the three grid points with the largest gradient
        flat = np.abs(gd[ch]).ravel()
        for idx in np.argsort(flat)[-3:]:
            bb, ss, jj = np.unravel_index(idx, gd[ch].shape)
            h = 1e-6
            fp, fm = pr["ftau"].copy(), pr["ftau"].copy()
            fp[bb, ss, jj] += h
            fm[bb, ss, jj] -= h
            dp = _oracle_logw(pr, pr["umatrix"], pr["muimp"], fp, beta, cfg)[0]
            dm = _oracle_logw(pr, pr["umatrix"], pr["muimp"], fm, beta, cfg)[0]
            fd = (dp - dm) / (2 * h)
            assert abs(fd - gd[ch][bb, ss, jj]) < 1e-5 * max(1.0, abs(fd)), (fd, gd[ch][bb, ss, jj])
        # d log|trace| / d(eps_f, U, J)
        h = 1e-5
        for p, (du, dj, df) in enumerate([(0, 0, f) for f in range(2 * nd)] + [(1, 0, None), (0, 1, None)]):
            def tr(sig):
                uu, jj_ = u + sig * h * du, j + sig * h * dj
                mu = np.array(pr["muimp"], np.float64).reshape(nd, 2, nd, 2).copy()
                if df is not None:
                    mu[df // 2, df % 2, df // 2, df % 2] += sig * h
                return _oracle_logw(pr, _dd3_umatrix(uu, jj_), mu, pr["ftau"], beta, cfg)[1]
            fd = (tr(1) - tr(-1)) / (2 * h)
            assert abs(fd - gp[ch, p]) < 1e-5 * max(1.0, abs(fd)), (p, fd, gp[ch, p])


@pytest.mark.gpu
def test_autograd_function_applies_the_chain_rule():
    torch = pytest.importorskip("torch")
    from w2dynamics_gb300 import engine as E
    beta, nd = 10.0, 3
    pr = P.config_problem("dd3", beta=beta)
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], 20, nchains=4, seed0=70, taudiff_max=5.0,
                             kcap=64, opcap=512)])
    b.warmup(2000)
    b.sync()
    dE = GR.density_density_directions(nd, mg.fock_states)
    gd, gp, lw = b.gradients(dE)
    ftau = torch.tensor(pr["ftau"], dtype=torch.float64, requires_grad=True)
    theta = torch.zeros(dE.shape[0], dtype=torch.float64, requires_grad=True)
    logw = GR.LogWeight().apply(ftau, theta, b, dE)
    weights = torch.arange(1, 5, dtype=torch.float64)
    (logw * weights).sum().backward()
    assert np.allclose(logw.detach().numpy(), lw.sum(axis=1))
    assert np.allclose(ftau.grad.numpy(), np.tensordot(np.arange(1, 5), gd, axes=1))
    assert np.allclose(theta.grad.numpy(), np.arange(1, 5) @ gp)


@pytest.mark.gpu
def test_score_function_dG_dU_matches_finite_differences():
    """dG(tau)/dU from the score-function estimator <G g> - <G><g> (g = d
    log|trace|/dU of each measured configuration) against central
    differences of G(tau) from independent runs at U +- dU, single-orbital
    Anderson model, 2048 chains per run."""
    from w2dynamics_gb300 import engine as E
    beta, nd, u0, du, n, nt = 10.0, 1, 2.0, 0.1, 2048, 10
    ft = P.semicircle_ftau(nd, beta, 1.0, 1000)
    mu = P.muimp_solver(nd, u0 / 2)

    def run(u, seed0, score):
        um = P.flat_umatrix(P.umatrix_density(nd, u, u, 0.0))
        mg = E.Model(nd, um, mu, "Nt Szt Azt")
        dE = GR.density_density_directions(nd, mg.fock_states)[2:3] if score else None
        b = E.Batch(mg, [E.Group(beta, ft, nt, nchains=n, seed0=seed0, taudiff_max=beta, ncorr=20,
                                 p_shift=0.01, score_dE=dE)])
        b.warmup(4000)
        b.measure(400)
        b.sync()
        G = np.array([b.results(c)["gtau"][0, 0] for c in range(n)])
        dG = np.array([b.results_score(c)[0][0, 0, 0] for c in range(n)]) if score else None
        return G, dG

    _, dG = run(u0, 0, True)
    Gp, _ = run(u0 + du, 10000, False)
    Gm, _ = run(u0 - du, 20000, False)
    fd = (Gp.mean(0) - Gm.mean(0)) / (2 * du)
    efd = np.sqrt(Gp.var(0, ddof=1) / n + Gm.var(0, ddof=1) / n) / (2 * du)
    sf = dG.mean(0)
    esf = dG.std(0, ddof=1) / np.sqrt(n)
    z = (sf - fd) / np.sqrt(efd ** 2 + esf ** 2)
    assert np.abs(z).max() < 4.5, (z, sf, fd)
    assert np.mean(np.abs(z) < 2.5) >= 0.8
    assert np.abs(sf).max() > 5 * esf.max()  # the derivative is resolved


@pytest.mark.gpu
def test_device_gradients_equal_host_gradients():
    torch = pytest.importorskip("torch")
    from w2dynamics_gb300 import engine as E
    beta, nd = 10.0, 3
    pr = P.config_problem("dd3", beta=beta)
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], 20, nchains=6, seed0=90, taudiff_max=5.0,
                             kcap=64, opcap=512)])
    b.warmup(1500)
    b.sync()
    dE = GR.density_density_directions(nd, mg.fock_states)
    gd, gp, lw = b.gradients(dE)
    dev = torch.device("cuda")
    nft = pr["ftau"].shape[2]
    t_gd = torch.empty((6, 2 * nd, nft), dtype=torch.float64, device=dev)
    t_gp = torch.empty((6, dE.shape[0]), dtype=torch.float64, device=dev)
    t_lw = torch.empty((6, 2), dtype=torch.float64, device=dev)
    t_dE = torch.tensor(dE, device=dev)
    torch.cuda.synchronize()
    b.gradients_device(t_dE, t_gd, t_gp, t_lw)
    b.sync()
    g = t_gd.cpu().numpy()
    assert np.allclose(np.stack([g[:, f] for f in range(2 * nd)], 1),
                       np.stack([gd[:, f // 2, f % 2] for f in range(2 * nd)], 1))
    assert np.allclose(t_gp.cpu().numpy(), gp)
    assert np.allclose(t_lw.cpu().numpy(), lw)
