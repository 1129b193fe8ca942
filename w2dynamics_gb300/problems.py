"""Synthetic impurity problems for the CT-HYB loop.

Builders for the inputs the w2dynamics `mctqmc.init_solver` entry takes
(src/ctqmc_fortran/CTQMC.F90:7894): the four-index interaction matrix
U[(2Nd)^4] with flavour index 2*orbital + spin (w2dyn/dmft/interaction.py
Density / Kanamori, :171-260), the one-particle term `muimp` in the solver's
sign convention (cthyb_solver.py:255: muimp_solver = -(mu - crystal field)),
and the hybridisation function F(tau) >= 0 of a semicircular bath tabulated on
Nftau equidistant points of [0, beta] (cthyb:196-197 sign convention).
"""
import numpy as np


def umatrix_density(nd, u, v, j):
    """Density-density U matrix U[b1,s1,b2,s2,b3,s3,b4,s4] (interaction.py:171-196).

    Intra-orbital U for opposite spins, V between different orbitals and
    -J for parallel spins on different orbitals (the exchange-like entry
    U[b1,s,b3,s,b3,s,b1,s] = J enters H with the annihilators swapped).
    """
    um = np.zeros((nd, 2, nd, 2, nd, 2, nd, 2))
    for b1 in range(nd):
        um[b1, 0, b1, 1, b1, 0, b1, 1] = u
        um[b1, 1, b1, 0, b1, 1, b1, 0] = u
        for b3 in range(nd):
            if b3 == b1:
                continue
            for s1 in range(2):
                for s3 in range(2):
                    um[b1, s1, b3, s3, b1, s1, b3, s3] = v
            for s in range(2):
                um[b1, s, b3, s, b3, s, b1, s] = j
    return um


def umatrix_kanamori(nd, u, v, j):
    """Kanamori U matrix: density part plus pair hopping and spin flip
    (interaction.py:217-230)."""
    um = umatrix_density(nd, u, v, j)
    for b1 in range(nd):
        for b2 in range(nd):
            if b1 == b2:
                continue
            um[b1, 0, b1, 1, b2, 0, b2, 1] = j  # pair hopping
            um[b1, 1, b1, 0, b2, 1, b2, 0] = j
            um[b1, 0, b2, 1, b2, 0, b1, 1] = j  # spin flip
            um[b1, 1, b2, 0, b2, 1, b1, 0] = j
    return um


def flat_umatrix(um):
    """(Nd,2)^4 -> (2Nd)^4 with flavour 2*b+s (interaction.convert_u_matrix)."""
    nf = um.shape[0] * 2
    return np.ascontiguousarray(um.reshape(nf, nf, nf, nf))


def muimp_solver(nd, mu, crystalfield=None):
    """One-particle term in the solver convention, shape (Nd,2,Nd,2).

    cthyb:162-164 builds muimp = mu*1 - crystalfield, and the solver negates
    it (cthyb_solver.py:255)."""
    m = mu * np.einsum("ab,st->asbt", np.eye(nd), np.eye(2))
    if crystalfield is not None:
        cf = np.asarray(crystalfield, dtype=np.float64)
        for b in range(nd):
            m[b, :, b, :] -= cf[b] * np.eye(2)
    return -m


def _gauss_legendre(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


def semicircle_gtau(beta, half_bandwidth, ntau, nquad=4000):
    """g(tau) = int rho(e) exp(-e tau) / (1 + exp(-beta e)) de on
    tau_j = j*beta/(ntau-1), rho the semicircle of half-bandwidth D.

    Substituting e = D cos(theta) gives rho de = (2/pi) sin^2(theta) dtheta;
    Gauss-Legendre quadrature in theta.  The integrand is evaluated in the
    overflow-free form exp(-e tau)/(1+exp(-beta e)) for e >= 0 and
    exp(e (beta - tau))/(1+exp(beta e)) for e < 0."""
    x, w = _gauss_legendre(nquad)
    th = 0.5 * np.pi * (x + 1.0)
    wt = 0.5 * np.pi * w * (2.0 / np.pi) * np.sin(th) ** 2
    e = half_bandwidth * np.cos(th)
    tau = np.linspace(0.0, beta, ntau)
    out = np.empty(ntau)
    pos = e >= 0
    ep, en = e[pos], e[~pos]
    dp = 1.0 / (1.0 + np.exp(-beta * ep))
    dn = 1.0 / (1.0 + np.exp(beta * en))
    for a in range(0, ntau, 256):
        t = tau[a:a + 256, None]
        out[a:a + 256] = (np.exp(-ep * t) * dp) @ wt[pos] + (np.exp(en * (beta - t)) * dn) @ wt[~pos]
    return out


def semicircle_ftau(nd, beta, half_bandwidth, ntau):
    """Diagonal F(tau) = (D/2)^2 g(tau) for every flavour, shape (Nd, 2, Ntau)."""
    g = semicircle_gtau(beta, half_bandwidth, ntau) * (half_bandwidth / 2.0) ** 2
    return np.broadcast_to(g, (nd, 2, ntau)).copy()


def ftau_full(ftau_diag):
    """(Nd,2,Ntau) diagonal -> (Nd,2,Nd,2,Ntau) as passed to init_solver."""
    nd, _, nt = ftau_diag.shape
    full = np.zeros((nd, 2, nd, 2, nt))
    for b in range(nd):
        for s in range(2):
            full[b, s, b, s, :] = ftau_diag[b, s]
    return full


# Named workloads (sizes and parameters of the benchmark configurations).
def config_problem(name, beta=None):
    """Return dict(nd, umatrix (flat), muimp, ftau (Nd,2,Nftau), beta, ntau,
    quantum_numbers) for one of the named workloads.

    'anderson1':  Nd=1 density-density U=2, mu=U/2, beta=10, D=1, Ntau=1000
    'dd3':        Nd=3 density-density U=4, J=0.6, U'=U-2J, beta=50, D=1,
                  Ntau=2000, QuantumNumbers "Nt Szt"
    'kanamori5':  Nd=5 full Kanamori U=3, J=0.7, U'=U-2J, crystal field
                  e_g +0.2 / t2g -0.2, beta=40, D=2, Ntau=4000, "Nt Szt"
    """
    if name == "anderson1":
        nd, u, j = 1, 2.0, 0.0
        b = 10.0 if beta is None else beta
        um = umatrix_density(nd, u, u, j)
        mu = u / 2.0
        return dict(nd=nd, umatrix=flat_umatrix(um), muimp=muimp_solver(nd, mu), beta=b,
                    ftau=semicircle_ftau(nd, b, 1.0, 1000), ntau=1000,
                    quantum_numbers="Nt Szt Azt")
    if name == "dd3":
        nd, u, j = 3, 4.0, 0.6
        b = 50.0 if beta is None else beta
        um = umatrix_density(nd, u, u - 2 * j, j)
        # mu for filling 2/6 of the atomic limit: between the N=1 and N=2
        # addition energies
        mu = DD3_MU
        return dict(nd=nd, umatrix=flat_umatrix(um), muimp=muimp_solver(nd, mu), beta=b,
                    ftau=semicircle_ftau(nd, b, 1.0, 2000), ntau=2000,
                    quantum_numbers="Nt Szt")
    if name == "kanamori5":
        nd, u, j = 5, 3.0, 0.7
        b = 40.0 if beta is None else beta
        um = umatrix_kanamori(nd, u, u - 2 * j, j)
        cf = np.array([-0.2, -0.2, -0.2, 0.2, 0.2])
        return dict(nd=nd, umatrix=flat_umatrix(um), muimp=muimp_solver(nd, K5_MU, cf), beta=b,
                    ftau=semicircle_ftau(nd, b, 2.0, 4000), ntau=4000,
                    quantum_numbers="Nt Szt")
    raise KeyError(name)


# Chemical potentials fixed by hand for the named fillings (the reference
# driver refuses a mu search in single-shot mode, cthyb:125-126).
DD3_MU = 3.3
K5_MU = 9.8
