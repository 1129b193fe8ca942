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


# --------------------------------------------------------------------------
# The differentiation configuration: 3-orbital model at beta = 50.
import dense_reference as DR  # noqa: E402


def _dd3_parts(nd, u, j, muimp, occ_fock):
    """Dense H and the directions dH/d(eps_f, U, J) in the occupation basis."""
    C = DR.fock_operators(nd, occ_fock)
    H = DR.hamiltonian(nd, _dd3_umatrix(u, j), muimp, C)
    V = [C[f, 0] @ C[f, 1] for f in range(2 * nd)]
    V.append(DR.hamiltonian(nd, P.flat_umatrix(P.umatrix_density(nd, 1.0, 1.0, 0.0)), np.zeros((nd, 2, nd, 2)), C))
    V.append(DR.hamiltonian(nd, P.flat_umatrix(P.umatrix_density(nd, 0.0, -2.0, 1.0)), np.zeros((nd, 2, nd, 2)), C))
    return C, H, V


def test_dense_reference_against_oracle_weights():
    """The dense FP64 reference (full Fock-space H_loc, LU and expm) gives
    the oracle's log|det| and log|trace| of sampled configurations, its
    Hamiltonian the model's eigenvalues, and its analytic gradients equal
    its own central differences."""
    beta, nd, u, j = 10.0, 3, 4.0, 0.6
    pr = P.config_problem("dd3", beta=beta)
    mo = O.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    C, H, V = _dd3_parts(nd, u, j, pr["muimp"], mo.fock_states)
    ev = np.linalg.eigvalsh(H)
    assert np.allclose(np.sort(ev), np.sort(mo.evals), atol=1e-10)
    co = O.Chain(mo, beta, pr["ftau"], 20, seed=11, taudiff_max=5.0)
    co.warmup(2500)
    taus, orbs, spins, cas = co.get_config()
    outer = int(co.state()["outer_sst"])
    states = np.arange(mo.sst_offset[outer], mo.sst_offset[outer] + mo.sst_size[outer])
    ld, gd = DR.logdet_and_grad(pr["ftau"], beta, taus, orbs, spins, cas)
    lt, gt = DR.logtrace_and_grad(H, V, C, beta, taus, orbs, spins, cas, states)
    assert abs(ld - co.full_det()[0]) < 1e-9 * max(1, abs(ld))
    assert abs(lt - (co.full_trace()[0] - beta * mo.egs)) < 1e-9 * max(1, abs(lt))
    h = 1e-5
    for p in (0, 6, 7):
        ltp, _ = DR.logtrace_and_grad(H + h * V[p], [], C, beta, taus, orbs, spins, cas, states)
        ltm, _ = DR.logtrace_and_grad(H - h * V[p], [], C, beta, taus, orbs, spins, cas, states)
        assert abs((ltp - ltm) / (2 * h) - gt[p]) < 1e-6 * max(1, abs(gt[p]))
    b_, s_, i_ = np.unravel_index(np.argmax(np.abs(gd)), gd.shape)
    fp, fm = pr["ftau"].copy(), pr["ftau"].copy()
    fp[b_, s_, i_] += 1e-6
    fm[b_, s_, i_] -= 1e-6
    fd = (DR.logdet_and_grad(fp, beta, taus, orbs, spins, cas)[0] -
          DR.logdet_and_grad(fm, beta, taus, orbs, spins, cas)[0]) / 2e-6
    assert abs(fd - gd[b_, s_, i_]) < 1e-6 * max(1, abs(fd))


@pytest.mark.gpu
def test_gradients_100_configurations_beta50():
    """Gradient checks: 100 thermalised configurations of the 3-orbital
    model at beta = 50; the kernel's gradients against central finite
    differences (step 1e-6) of the oracle's full LU determinant and full
    trace (the two grid points of largest d log|det| and all 8 parameter
    directions per configuration), and, on 10 of them, the whole F-grid
    gradient and the parameter gradient against the dense LU / Frechet-expm
    reference."""
    from w2dynamics_gb300 import engine as E
    beta, nd, u, j, n = 50.0, 3, 4.0, 0.6, 100
    pr = P.config_problem("dd3", beta=beta)
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], 20, nchains=n, seed0=500, taudiff_max=5.0, kcap=64, opcap=512)])
    b.warmup(20000)
    b.sync()
    dE = GR.density_density_directions(nd, mg.fock_states)
    gd, gp, lw = b.gradients(dE)
    occ_fock, _ = mg.basis()
    C, H, V = _dd3_parts(nd, u, j, pr["muimp"], occ_fock)
    h = 1e-6
    worst = {"det_fd": 0.0, "trace_fd": 0.0, "det_dense": 0.0, "trace_dense": 0.0}
    for ch in range(n):
        cfg = b.get_config(ch)
        assert len(cfg[0]) > 20  # thermalised order at beta = 50
        ld0, lt0 = _oracle_logw(pr, pr["umatrix"], pr["muimp"], pr["ftau"], beta, cfg)
        assert abs(lw[ch, 0] - ld0) < 1e-9 * max(1, abs(ld0))
        assert abs(lw[ch, 1] - lt0) < 1e-9 * max(1, abs(lt0))
        flat = np.abs(gd[ch]).ravel()
        for idx in np.argsort(flat)[-2:]:
            bb, ss, jj = np.unravel_index(idx, gd[ch].shape)
            fp, fm = pr["ftau"].copy(), pr["ftau"].copy()
            fp[bb, ss, jj] += h
            fm[bb, ss, jj] -= h
            fd = (_oracle_logw(pr, pr["umatrix"], pr["muimp"], fp, beta, cfg)[0] -
                  _oracle_logw(pr, pr["umatrix"], pr["muimp"], fm, beta, cfg)[0]) / (2 * h)
            err = abs(fd - gd[ch][bb, ss, jj]) / max(1.0, abs(fd))
            worst["det_fd"] = max(worst["det_fd"], err)
            assert err < 1e-4, (ch, fd, gd[ch][bb, ss, jj])
        for p, (du, dj, df) in enumerate([(0, 0, f) for f in range(2 * nd)] + [(1, 0, None), (0, 1, None)]):
            def tr(sig):
                mu = np.array(pr["muimp"], np.float64).reshape(nd, 2, nd, 2).copy()
                if df is not None:
                    mu[df // 2, df % 2, df // 2, df % 2] += sig * h
                return _oracle_logw(pr, _dd3_umatrix(u + sig * h * du, j + sig * h * dj), mu, pr["ftau"], beta,
                                    cfg)[1]
            fd = (tr(1) - tr(-1)) / (2 * h)
            err = abs(fd - gp[ch, p]) / max(1.0, abs(fd))
            worst["trace_fd"] = max(worst["trace_fd"], err)
            assert err < 1e-4, (ch, p, fd, gp[ch, p])
        if ch < 10:
            taus, orbs, spins, cas, outer = cfg
            states = np.arange(mg.sst_offset[outer], mg.sst_offset[outer] + mg.sst_size[outer])
            ldd, gdd = DR.logdet_and_grad(pr["ftau"], beta, taus, orbs, spins, cas)
            ltd, gtd = DR.logtrace_and_grad(H, V, C, beta, taus, orbs, spins, cas, states)
            assert abs(ldd - lw[ch, 0]) < 1e-9 * max(1, abs(ldd))
            assert abs(ltd - lw[ch, 1]) < 1e-9 * max(1, abs(ltd))
            e1 = np.abs(gdd - gd[ch]).max() / max(1.0, np.abs(gdd).max())
            e2 = np.abs(gtd - gp[ch]).max() / max(1.0, np.abs(gtd).max())
            worst["det_dense"] = max(worst["det_dense"], e1)
            worst["trace_dense"] = max(worst["trace_dense"], e2)
            assert e1 < 1e-9 and e2 < 1e-9, (ch, e1, e2)
    print(f"\ngradient checks (100 configurations, beta = 50), worst relative errors: {worst}")


@pytest.mark.gpu
def test_score_function_dG_dU_three_orbital():
    """dG(tau)/dU of the 3-orbital model (beta = 50, 2048 chains) from the
    score-function estimator <G g> - <G><g> over all measurements of all
    chains (per-chain covariances alone would drop the covariance between
    the chains' means, which is large where a chain keeps its sector for a
    long time) against central differences of G(tau) from independent runs
    at U +- 0.05.  At beta = 50 the sector populations settle slowly and
    the finite differences of runs that start from U-dependent initial
    sectors carry that: 4e4 thermalisation proposals leave them 3 sigma
    above the score estimate, 1.5e5 proposals bring them within about one
    sigma, so the runs thermalise for 1.5e5 proposals."""
    from w2dynamics_gb300 import engine as E
    beta, nd, u0, j, du, n, nt = 50.0, 3, 4.0, 0.6, 0.05, 2048, 8
    pr = P.config_problem("dd3", beta=beta)
    # outer-superstate, global and tau-shift moves equilibrate the chains
    # over the superstate sectors, which the initial draw (empty-trace
    # weights, U dependent) does not
    moves = dict(p_outer=0.1, p_global=0.01, p_shift=0.01)

    def run(u, seed0, score):
        mg = E.Model(nd, _dd3_umatrix(u, j), pr["muimp"], pr["quantum_numbers"])
        dE = GR.density_density_directions(nd, mg.fock_states)[2 * nd:2 * nd + 1] if score else None
        b = E.Batch(mg, [E.Group(beta, pr["ftau"], nt, nchains=n, seed0=seed0, taudiff_max=5.0, ncorr=50,
                                 kcap=64, opcap=512, score_dE=dE, **moves)])
        b.warmup(150000)
        b.measure(400)
        b.sync()
        G = b.group_gtau(0).reshape(n, 2 * nd, nt).mean(axis=1)  # average over the degenerate flavours
        if not score:
            return G, None, None
        # per chain: the within-chain covariance <G g>_c - <G>_c <g>_c and <g>_c
        sc = [b.results_score(c) for c in range(n)]
        cov = np.array([x[0][0].reshape(2 * nd, nt).mean(axis=0) for x in sc])
        g = np.array([x[1][0] for x in sc])
        return G, cov + G * g[:, None], g  # <G g>_c

    G0, Gg, g = run(u0, 0, True)
    Gp, _, _ = run(u0 + du, 10000, False)
    Gm, _, _ = run(u0 - du, 20000, False)
    fd = (Gp.mean(0) - Gm.mean(0)) / (2 * du)
    efd = np.sqrt(Gp.var(0, ddof=1) / n + Gm.var(0, ddof=1) / n) / (2 * du)

    # the score-function estimate over all measurements of all chains (equal
    # measurement counts): <G g> - <G><g>, which keeps the between-chain
    # covariance; error by jackknife over the chains
    def est(sel):
        return Gg[sel].mean(0) - G0[sel].mean(0) * g[sel].mean()

    sf = est(np.ones(n, bool))
    jk = np.array([est(np.arange(n) != c) for c in range(n)])
    esf = np.sqrt((n - 1) / n * ((jk - jk.mean(0)) ** 2).sum(0))
    z = (sf - fd) / np.sqrt(efd ** 2 + esf ** 2)
    print(f"\ndG/dU 3-orbital: score {sf}, finite differences {fd}, z {z}")
    assert np.abs(z).max() < 4.0, (z, sf, fd)
    assert np.mean(np.abs(z) < 2.5) >= 0.75


@pytest.mark.gpu
def test_device_log_weight_function():
    """LogWeight on device tensors: forward from the chains' weights (equal
    to the kernel's log weights), backward through the device gradient
    kernel, gradients on the input tensors' device."""
    torch = pytest.importorskip("torch")
    from w2dynamics_gb300 import engine as E
    beta, nd = 50.0, 3
    pr = P.config_problem("dd3", beta=beta)
    mg = E.Model(nd, pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(mg, [E.Group(beta, pr["ftau"], 20, nchains=16, seed0=300, taudiff_max=5.0, kcap=64, opcap=512)])
    b.warmup(8000)
    b.sync()
    dE = GR.density_density_directions(nd, mg.fock_states)
    gd, gp, lw = b.gradients(dE)
    dev = torch.device("cuda")
    ftau = torch.tensor(pr["ftau"], dtype=torch.float64, device=dev, requires_grad=True)
    theta = torch.zeros(dE.shape[0], dtype=torch.float64, device=dev, requires_grad=True)
    logw = GR.LogWeight().apply(ftau, theta, b, torch.tensor(dE, device=dev))
    assert logw.is_cuda
    assert np.allclose(logw.detach().cpu().numpy(), lw.sum(axis=1), rtol=1e-12, atol=1e-9)
    wts = torch.linspace(0.5, 2.0, 16, dtype=torch.float64, device=dev)
    (logw * wts).sum().backward()
    w = wts.cpu().numpy()
    assert ftau.grad.is_cuda and theta.grad.is_cuda
    assert np.allclose(ftau.grad.cpu().numpy(), np.tensordot(w, gd, axes=1), rtol=1e-10, atol=1e-12)
    assert np.allclose(theta.grad.cpu().numpy(), w @ gp, rtol=1e-10, atol=1e-12)


def _kan3(u, j):
    return P.flat_umatrix(P.umatrix_kanamori(3, u, u - 2 * j, j))


@pytest.mark.gpu
def test_dense_block_trace_gradients_against_dense_reference():
    """Dense-block models (3-orbital Kanamori with spin flip and pair
    hopping, "Nt Szt" blocks): the adjoint trace gradient along U, J and
    one level eps_0 (directions set on the model as dU / dmuimp) equals the
    dense Frechet-expm reference on every chain, and central differences of
    the oracle's full trace on two of them."""
    from w2dynamics_gb300 import engine as E
    beta, nd, u, j = 10.0, 3, 4.0, 0.6
    muimp = P.muimp_solver(nd, 3.0)
    ft = P.semicircle_ftau(nd, beta, 1.0, 1000)
    mg = E.Model(nd, _kan3(u, j), muimp, "Nt Szt")
    assert not mg.monomial
    d_eps = np.zeros((nd, 2, nd, 2))
    d_eps[0, 0, 0, 0] = 1.0
    dirs_u = [_kan3(1.0, 0.0), _kan3(0.0, 1.0), np.zeros((6,) * 4)]
    dirs_mu = [np.zeros((nd, 2, nd, 2)), np.zeros((nd, 2, nd, 2)), d_eps]
    mg.set_directions(dirs_u, dirs_mu)
    n = 8
    b = E.Batch(mg, [E.Group(beta, ft, 20, nchains=n, seed0=60, taudiff_max=-1.0, kcap=64, opcap=512,
                             tree_levels=3)])
    b.warmup(3000)
    b.sync()
    gd, gp, lw = b.gradients()
    assert gp.shape == (n, 3)
    occ_fock, _ = mg.basis()
    C = DR.fock_operators(nd, occ_fock)
    H = DR.hamiltonian(nd, _kan3(u, j), muimp, C)
    V = [DR.hamiltonian(nd, du, dm, C) for du, dm in zip(dirs_u, dirs_mu)]
    worst = 0.0
    for ch in range(n):
        taus, orbs, spins, cas, outer = b.get_config(ch)
        states = np.arange(mg.sst_offset[outer], mg.sst_offset[outer] + mg.sst_size[outer])
        lt, gt = DR.logtrace_and_grad(H, V, C, beta, taus, orbs, spins, cas, states)
        assert abs(lt - lw[ch, 1]) < 1e-9 * max(1.0, abs(lt)), (ch, lt, lw[ch, 1])
        err = np.abs(gt - gp[ch]).max() / max(1.0, np.abs(gt).max())
        worst = max(worst, err)
        assert err < 1e-8, (ch, gt, gp[ch])
    print(f"\ndense-block trace gradients: worst relative error against the dense reference {worst:.2e}")
    h = 1e-6
    for ch in (0, 5):
        cfg = b.get_config(ch)
        for p, (du, dj) in enumerate([(1, 0), (0, 1)]):
            def tr(sig):
                mo = O.Model(nd, _kan3(u + sig * h * du, j + sig * h * dj), muimp, "Nt Szt")
                co = O.Chain(mo, beta, ft, 20, seed=1, taudiff_max=beta)
                co.set_config(*cfg[:4], cfg[4])
                return co.full_trace()[0] - beta * mo.egs
            fd = (tr(1) - tr(-1)) / (2 * h)
            assert abs(fd - gp[ch, p]) < 1e-5 * max(1.0, abs(fd)), (ch, p, fd, gp[ch, p])
