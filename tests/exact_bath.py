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
