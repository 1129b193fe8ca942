"""Exact expansion-order distribution of a single-orbital impurity coupled to
discrete bath levels (test helper, numpy/scipy only).

The hybridisation expansion orders of CT-HYB are distributed as
P(k_up, k_dn) = Z_{k_up k_dn} / Z, where Z_k is the weight of all
configurations with k_s creator/annihilator pairs of spin s.  For a bath of
discrete levels the impurity + bath system is finite: with every
hybridisation amplitude of spin s scaled by sqrt(x_s),

    Z(x_up, x_dn) = Tr exp(-beta H(x)) = Z_bath * sum_k x_up^k_up x_dn^k_dn Z_k,

because each spin-s term of the expansion has as many d+c as c+d factors.
Evaluating Z on |x_s| = 1 (H then not hermitian, the amplitude enters d+c and
c+d alike) and Fourier transforming gives the Z_k; the marginal of one spin
follows with the other x fixed at 1.

The impurity Hamiltonian is the solver's: H_loc = muimp * n + U n_up n_dn with
muimp = -mu; bath levels eps_b with amplitudes V_b for both spins.  The
matching F(tau) is the reference's bath-site formula
(w2dyn/auxiliaries/transform.py:114-146):
F(tau) = sum_b V_b^2 / (exp(-tau eps_b) + exp((beta - tau) eps_b)).
"""
import numpy as np
from scipy.linalg import expm


def _fermions(n):
    """Annihilators of n modes (Jordan-Wigner), 2^n x 2^n real matrices."""
    a = np.array([[0.0, 1.0], [0.0, 0.0]])
    z = np.diag([1.0, -1.0])
    eye = np.eye(2)
    ops = []
    for j in range(n):
        m = np.array([[1.0]])
        for i in range(n):
            m = np.kron(m, z if i < j else (a if i == j else eye))
        ops.append(m)
    return ops


def ftau_bath(beta, eps, v, nftau):
    """F(tau) on tau_j = j beta / (nftau - 1) for the bath levels (eps, v)."""
    tau = np.linspace(0.0, beta, nftau)[:, None]
    eps = np.asarray(eps, np.float64)[None, :]
    v2 = np.asarray(v, np.float64)[None, :] ** 2
    return (v2 / (np.exp(-tau * eps) + np.exp((beta - tau) * eps))).sum(axis=1)


def order_marginal(beta, mu, u, eps, v, spin=0, kmax=64):
    """P(k) of the expansion order of one spin (0 = up), k = 0 .. kmax - 1."""
    nb = len(eps)
    ops = _fermions(2 + 2 * nb)  # d_up, d_dn, then c_{b,up}, c_{b,dn}
    d = ops[:2]
    c = [ops[2:][2 * b: 2 * b + 2] for b in range(nb)]
    num = [x.T @ x for x in ops]
    h0 = -mu * (num[0] + num[1]) + u * num[0] @ num[1]
    for b in range(nb):
        h0 = h0 + eps[b] * (num[2 + 2 * b] + num[3 + 2 * b])
    hyb = [sum(v[b] * (d[s].T @ c[b][s] + c[b][s].T @ d[s]) for b in range(nb)) for s in range(2)]
    zs = np.empty(kmax, complex)
    for m in range(kmax):
        x = np.exp(2j * np.pi * m / kmax)
        h = h0 + np.sqrt(x) * hyb[spin] + hyb[1 - spin]
        zs[m] = np.trace(expm(-beta * h))
    zk = np.fft.fft(zs) / kmax
    p = zk.real / zk.real.sum()
    assert np.abs(zk.imag).max() < 1e-9 * zk.real.sum()
    return p


def occupations(beta, mu, u, eps, v):
    """Exact <n_up>, <n_dn> and <n_up n_dn> of the impurity."""
    nb = len(eps)
    ops = _fermions(2 + 2 * nb)
    num = [x.T @ x for x in ops]
    h = -mu * (num[0] + num[1]) + u * num[0] @ num[1]
    for b in range(nb):
        h = h + eps[b] * (num[2 + 2 * b] + num[3 + 2 * b])
        for s in range(2):
            h = h + v[b] * (ops[s].T @ ops[2 + 2 * b + s] + ops[2 + 2 * b + s].T @ ops[s])
    w, q = np.linalg.eigh(h)
    p = np.exp(-beta * (w - w.min()))
    rho = (q * (p / p.sum())) @ q.T
    return (np.trace(rho @ num[0]), np.trace(rho @ num[1]), np.trace(rho @ num[0] @ num[1]))


def ftau_full_bath(beta, eps, v, nftau):
    """F_{s s'}(tau), shape (1, 2, 1, 2, nftau), of spinless bath levels eps_b
    coupled to impurity spin s with amplitude v[b][s] (the bath-site formula
    with V*_{b s} V_{b s'}, w2dyn/auxiliaries/transform.py:140-144)."""
    tau = np.linspace(0.0, beta, nftau)
    out = np.zeros((1, 2, 1, 2, nftau))
    for b, e in enumerate(eps):
        g = 1.0 / (np.exp(-tau * e) + np.exp((beta - tau) * e))
        for s in range(2):
            for s2 in range(2):
                out[0, s, 0, s2] += v[b][s] * v[b][s2] * g
    return out


def offdiag_answers(beta, mu, u, eps, v, ntau, nsub=64):
    """Exact <d+_s d_s'> (2 x 2), <n_up n_dn> and bin averages of
    <d_s(tau) d+_s'(0)> (2, 2, ntau) for the impurity with spinless bath
    levels of spin-dependent amplitudes v[b][s]."""
    nb = len(eps)
    ops = _fermions(2 + nb)
    num = [x.T @ x for x in ops]
    h = -mu * (num[0] + num[1]) + u * num[0] @ num[1]
    for b in range(nb):
        h = h + eps[b] * num[2 + b]
        for s in range(2):
            h = h + v[b][s] * (ops[s].T @ ops[2 + b] + ops[2 + b].T @ ops[s])
    w, q = np.linalg.eigh(h)
    w = w - w.min()
    z = np.exp(-beta * w).sum()
    rho = (q * (np.exp(-beta * w) / z)) @ q.T
    rho1 = np.array([[np.trace(rho @ ops[a].T @ ops[b]) for b in range(2)] for a in range(2)])
    dbl = np.trace(rho @ num[0] @ num[1])
    d = [q.T @ ops[s] @ q for s in range(2)]
    edges = np.linspace(0.0, beta, ntau + 1)
    g = np.zeros((2, 2, ntau))
    for i in range(ntau):
        t = edges[i] + (np.arange(nsub) + 0.5) * (edges[i + 1] - edges[i]) / nsub
        el = np.exp(-(beta - t)[:, None] * w[None, :])  # e^{-(beta - tau) w_m}
        er = np.exp(-t[:, None] * w[None, :])           # e^{-tau w_n}
        for a in range(2):
            for b in range(2):
                # Tr[e^{-(beta-tau)H} d_a e^{-tau H} d+_b] / Z
                g[a, b, i] = np.mean(np.einsum("tm,mn,tn,nm->t", el, d[a], er, d[b].T)) / z
    return dict(rho1=rho1, double_occ=dbl, gtau=g)


def impurity_hamiltonian(nd, umatrix, muimp, ops):
    """H_loc = sum_ij muimp_ij d+_i d_j + 1/2 sum_ijkl U_ijkl d+_i d+_j d_l d_k
    on the first 2 nd modes of `ops` (flavour f = 2b + s), the solver's
    convention for muimp (Nd,2,Nd,2) and the flat U matrix."""
    nf = 2 * nd
    u = np.asarray(umatrix, np.float64).reshape((nf,) * 4)
    mu = np.asarray(muimp, np.float64).reshape(nd, 2, nd, 2)
    d = ops[:nf]
    h = 0.0
    for i in range(nf):
        for j in range(nf):
            t = mu[i // 2, i % 2, j // 2, j % 2]
            if t != 0.0:
                h = h + t * d[i].T @ d[j]
    for i in range(nf):
        for j in range(nf):
            for k in range(nf):
                for l in range(nf):
                    if u[i, j, k, l] != 0.0:
                        h = h + 0.5 * u[i, j, k, l] * d[i].T @ d[j].T @ d[l] @ d[k]
    return h


def ftau_full_spinful(nd, beta, eps, v, nftau):
    """F (Nd,2,Nd,2,nftau) of spinful bath levels eps_b coupled to orbital o
    of either spin with amplitude v[b][o] (spin-diagonal, orbital-mixing)."""
    tau = np.linspace(0.0, beta, nftau)
    out = np.zeros((nd, 2, nd, 2, nftau))
    for b, e in enumerate(eps):
        g = 1.0 / (np.exp(-tau * e) + np.exp((beta - tau) * e))
        for o1 in range(nd):
            for o2 in range(nd):
                for s in range(2):
                    out[o1, s, o2, s] += v[b][o1] * v[b][o2] * g
    return out


def spinful_answers(nd, beta, umatrix, muimp, eps, v, ntau, nsub=32):
    """Exact G_ab(tau) bin averages <d_a(tau) d+_b(0)> (2nd, 2nd, ntau) and
    <n_a> for the impurity with spinful bath levels of ftau_full_spinful."""
    nf, nb = 2 * nd, len(eps)
    ops = _fermions(nf + 2 * nb)
    h = impurity_hamiltonian(nd, umatrix, muimp, ops)
    for b in range(nb):
        for s in range(2):
            cb = ops[nf + 2 * b + s]
            h = h + eps[b] * cb.T @ cb
            for o in range(nd):
                f = 2 * o + s
                h = h + v[b][o] * (ops[f].T @ cb + cb.T @ ops[f])
    w, q = np.linalg.eigh(h)
    w = w - w.min()
    z = np.exp(-beta * w).sum()
    rho = (q * (np.exp(-beta * w) / z)) @ q.T
    occ = np.array([np.trace(rho @ ops[f].T @ ops[f]) for f in range(nf)])
    d = [q.T @ ops[f] @ q for f in range(nf)]
    edges = np.linspace(0.0, beta, ntau + 1)
    g = np.zeros((nf, nf, ntau))
    for i in range(ntau):
        t = edges[i] + (np.arange(nsub) + 0.5) * (edges[i + 1] - edges[i]) / nsub
        el = np.exp(-(beta - t)[:, None] * w[None, :])
        er = np.exp(-t[:, None] * w[None, :])
        for a in range(nf):
            for b2 in range(nf):
                g[a, b2, i] = np.mean(np.einsum("tm,mn,tn,nm->t", el, d[a], er, d[b2].T)) / z
    return dict(occ=occ, gtau=g)


def legendre_answers(beta, h, ops_a, nleg, nquad=400):
    """Legendre coefficients G_l = sqrt(2l + 1) int_0^beta P_l(2 tau/beta - 1)
    <d_a(tau) d+_b(0)> dtau (the normalisation of the solver's GLeg) for the
    annihilators ops_a of a finite Hamiltonian h, by Gauss-Legendre
    quadrature; shape (n, n, nleg)."""
    w, q = np.linalg.eigh(h)
    w = w - w.min()
    z = np.exp(-beta * w).sum()
    d = [q.T @ o @ q for o in ops_a]
    x, wq = np.polynomial.legendre.leggauss(nquad)
    t = 0.5 * beta * (x + 1.0)
    el = np.exp(-(beta - t)[:, None] * w[None, :])
    er = np.exp(-t[:, None] * w[None, :])
    n = len(ops_a)
    g = np.zeros((n, n, nquad))
    for a in range(n):
        for b in range(n):
            g[a, b] = np.einsum("tm,mn,tn,nm->t", el, d[a], er, d[b].T) / z
    pl = np.stack([np.polynomial.legendre.legval(x, np.eye(nleg)[l]) for l in range(nleg)])
    gl = 0.5 * beta * np.einsum("abt,lt,t->abl", g, pl, wq)
    return gl * np.sqrt(2.0 * np.arange(nleg) + 1.0)


def offdiag_hamiltonian(mu, u, eps, v):
    """Impurity (2 spin modes) + spinless bath levels with spin-dependent
    amplitudes v[b][s]: (h, the two impurity annihilators)."""
    nb = len(eps)
    ops = _fermions(2 + nb)
    num = [x.T @ x for x in ops]
    h = -mu * (num[0] + num[1]) + u * num[0] @ num[1]
    for b in range(nb):
        h = h + eps[b] * num[2 + b]
        for s in range(2):
            h = h + v[b][s] * (ops[s].T @ ops[2 + b] + ops[2 + b].T @ ops[s])
    return h, ops[:2]
