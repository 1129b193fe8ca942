"""Dense FP64 reference of a configuration's weight and its gradient (test
infrastructure): the hybridisation determinant by LU (numpy) with its exact
derivative with respect to the F(tau) grid, and the local trace as a
product of full Fock-space matrix exponentials (scipy) with its exact
derivative along Hamiltonian directions by the Frechet derivative of the
exponential.  Independent of the engine and of the oracle: it builds H_loc
from the U matrix and muimp as dense matrices and never uses the
eigenbasis blocks.

Conventions (as the engine's model set-up, Operator.F90:482-546,
1042-1108): flavour f = 2b + s, Fock bit b + Nd*s with the sign
(-1)^(occupied bits below); H = sum muimp[f1, f2] c+_f1 c_f2 +
1/2 sum U[i, j, k, l] c+_i c+_j c_l c_k; the trace of a configuration is
Tr_outer[e^{-(beta - tau_K) H} O_K ... O_1 e^{-tau_1 H}] over the states of
the outer superstate; Delta interpolated as get_HybrF (Trace.F90:1014-1033).
"""
import numpy as np
import scipy.linalg as sl

from w2dynamics_gb300 import estimators as ES


def fock_operators(nd, occ_fock):
    """C[f, ca] (ns x ns) in the occupation basis `occ_fock`: ca 0 = c+_f,
    ca 1 = c_f."""
    tgt, sgn = ES.ladder_tables(nd, occ_fock)
    ns = len(occ_fock)
    C = np.zeros((2 * nd, 2, ns, ns))
    for f in range(2 * nd):
        for ca in range(2):
            ok = tgt[f, ca] >= 0
            C[f, ca, tgt[f, ca][ok], np.nonzero(ok)[0]] = sgn[f, ca][ok]
    return C


def hamiltonian(nd, umatrix, muimp, C):
    nf = 2 * nd
    U = np.asarray(umatrix, np.float64).reshape((nf,) * 4)
    mu = np.asarray(muimp, np.float64).reshape(nd, 2, nd, 2)
    H = np.zeros(C.shape[2:])
    for f1 in range(nf):
        for f2 in range(nf):
            v = mu[f1 // 2, f1 % 2, f2 // 2, f2 % 2]
            if v != 0.0:
                H += v * C[f1, 0] @ C[f2, 1]
    for i, j, k, l in zip(*np.nonzero(U)):
        H += 0.5 * U[i, j, k, l] * C[i, 0] @ C[j, 0] @ C[l, 1] @ C[k, 1]
    return H


def _interp_weights(F, beta, tau):
    """value, grid index i, weights (w_i, w_i+1) and sign of get_HybrF."""
    sig = 1.0
    if tau < 0:
        tau += beta
        sig = -1.0
    n = tau / beta * (len(F) - 1)
    i = min(int(n), len(F) - 2)
    fr = n - int(n)
    return sig * (F[i] + fr * (F[i + 1] - F[i])), i, (sig * (1.0 - fr), sig * fr)


def logdet_and_grad(ftau, beta, taus, orbs, spins, cas):
    """log|det H| summed over flavours, H_f(a, c) = Delta_f(tau_a - tau_c),
    and d log|det| / dF on the grid, (Nd, 2, Nftau): M^T scattered with the
    interpolation weights."""
    nd = ftau.shape[0]
    grad = np.zeros_like(ftau, dtype=np.float64)
    total = 0.0
    f_of = 2 * (np.asarray(orbs) - 1) + (np.asarray(spins) - 1)
    for f in range(2 * nd):
        b, s = f // 2, f % 2
        tc = np.asarray(taus)[(f_of == f) & (np.asarray(cas) == 1)]
        ta = np.asarray(taus)[(f_of == f) & (np.asarray(cas) == 2)]
        k = len(tc)
        if k == 0:
            continue
        F = ftau[b, s]
        H = np.zeros((k, k))
        info = {}
        for a in range(k):
            for c in range(k):
                H[a, c], i, w = _interp_weights(F, beta, ta[a] - tc[c])
                info[a, c] = (i, w)
        sign, ld = np.linalg.slogdet(H)
        total += ld
        Minv = np.linalg.inv(H)  # d log|det H| / dH(a, c) = Minv(c, a)
        for (a, c), (i, (w0, w1)) in info.items():
            grad[b, s, i] += Minv[c, a] * w0
            grad[b, s, i + 1] += Minv[c, a] * w1
    return total, grad


def logtrace_and_grad(H, V, C, beta, taus, orbs, spins, cas, outer_states):
    """log|trace| (absolute energies) and d log|trace| / dtheta_p for
    Hamiltonian directions V[p] = dH/dtheta_p, forward mode: every segment's
    exponential and its Frechet derivative, renormalised after each operator
    (the scales cancel in the ratio)."""
    egs = np.linalg.eigvalsh(H).min()
    Hs = H - egs * np.eye(len(H))  # constant shift: same derivative
    npar = len(V)
    ns = len(H)
    P = np.zeros((ns, ns))
    P[outer_states, outer_states] = 1.0
    M = P.copy()
    dM = [np.zeros((ns, ns)) for _ in range(npar)]
    logscale = 0.0
    t = 0.0
    f_of = 2 * (np.asarray(orbs) - 1) + (np.asarray(spins) - 1)
    ops = [(tau, C[f, ca - 1]) for tau, f, ca in zip(taus, f_of, cas)] + [(beta, None)]
    for tau, O in ops:
        dt = tau - t
        A = -dt * Hs
        E = sl.expm(A)
        new_dM = []
        for p in range(npar):
            _, dE = sl.expm_frechet(A, -dt * V[p], compute_expm=True)
            new_dM.append(E @ dM[p] + dE @ M)
        M = E @ M
        dM = new_dM
        if O is not None:
            M = O @ M
            dM = [O @ d for d in dM]
        sc = np.abs(M).max()
        if sc > 0:
            M /= sc
            dM = [d / sc for d in dM]
            logscale += np.log(sc)
        t = tau
    tr = np.trace(P @ M)
    dlog = np.array([np.trace(P @ d) / tr for d in dM])
    return np.log(abs(tr)) + logscale - beta * egs, dlog
