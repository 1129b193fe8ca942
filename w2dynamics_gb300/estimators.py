"""Estimators derived on the host from the measured density matrix.

After the Z-space loop the reference turns the density matrix at beta/2
(eigenbasis, normalised) into
  rho1(f2, f1)          = Tr(rho c+_f2 c_f1)           Meas_rho1_from_Densitymatrix,
                                                       CTQMC.F90:3020-3060
  rho2(f4, f3, f2, f1)  = Tr(rho c+_f4 c+_f3 c_f2 c_f1) Meas_rho2_from_Densitymatrix,
                                                       CTQMC.F90:2945-3017
  occ(b1,s1,b2,s2)      = Tr(rho n_f2 n_f1)            MeasDoubleOcc_from_Densitymatrix,
                                                       CTQMC.F90:2884-2942
  ssquare(N)            = sum over superstates of N electrons of Tr(rho S^2)
                                                       MeasureS2_from_densitymatrix,
                                                       CTQMC.F90:2811-2838
and finally rotates rho to the occupation basis (Transform_DensityMatrix_EB_to_OCCB,
CTQMC.F90:3163-3179).  The reference evaluates each trace block by block in
the eigenbasis with DGEMM/DDOT; traces do not depend on the basis, so here
they are evaluated in the occupation basis, where every c/c+ is a signed
partial permutation of the basis vectors.  Flavour f = 2*(b-1) + (s-1), Fock
bit (b-1) + Nd*(s-1), sign (-1)^(occupied bits below), Operator.F90:157-168.
"""
import numpy as np


def ladder_tables(nd, occ_fock):
    """tgt[f, ca, i], sgn[f, ca, i]: c+ (ca 0) / c (ca 1) of flavour f on
    basis vector i -> sgn * basis vector tgt (tgt -1: zero)."""
    occ_fock = np.asarray(occ_fock, np.int64)
    ns, nf = len(occ_fock), 2 * nd
    index = np.full(1 << nf, -1, np.int64)
    index[occ_fock] = np.arange(ns)
    tgt = np.full((nf, 2, ns), -1, np.int64)
    sgn = np.zeros((nf, 2, ns))
    for f in range(nf):
        bit = f // 2 + nd * (f % 2)
        occupied = (occ_fock >> bit) & 1
        below = occ_fock & ((1 << bit) - 1)
        parity = np.array([bin(int(x)).count("1") & 1 for x in below])
        s = np.where(parity == 1, -1.0, 1.0)
        flipped = index[occ_fock ^ (1 << bit)]
        for ca, allowed in ((0, occupied == 0), (1, occupied == 1)):
            tgt[f, ca] = np.where(allowed, flipped, -1)
            sgn[f, ca] = np.where(allowed, s, 0.0)
    return tgt, sgn


def _trace(rho, tgt, sgn, ops):
    """Tr(rho O) for O the product of `ops` (list of (f, ca)), the last
    element acting first on the ket."""
    ns = rho.shape[0]
    cur = np.arange(ns)
    amp = np.ones(ns)
    for f, ca in reversed(ops):
        alive = cur >= 0
        c = np.where(alive, cur, 0)
        amp = np.where(alive, amp * sgn[f, ca, c], 0.0)
        cur = np.where(alive, tgt[f, ca, c], -1)
    alive = cur >= 0
    p = np.nonzero(alive)[0]
    return float(np.sum(amp[p] * rho[p, cur[p]]))


def from_density_matrix(nd, occ_fock, evec, dm_eigen):
    """densitymatrix (occupation basis), occ (Nd,2,Nd,2), rho1 (2Nd,2Nd),
    rho2 (2Nd,)*4 from the normalised eigenbasis density matrix."""
    nf = 2 * nd
    rho = evec @ dm_eigen @ evec.T
    tgt, sgn = ladder_tables(nd, occ_fock)
    n = np.zeros((nf, len(occ_fock)))
    for f in range(nf):
        bit = f // 2 + nd * (f % 2)
        n[f] = (np.asarray(occ_fock) >> bit) & 1
    diag = np.diag(rho)
    occ = np.zeros((nd, 2, nd, 2))
    for f1 in range(nf):
        for f2 in range(nf):
            occ[f1 // 2, f1 % 2, f2 // 2, f2 % 2] = float(np.sum(diag * n[f1] * n[f2]))
    rho1 = np.zeros((nf, nf))
    for f2 in range(nf):
        for f1 in range(nf):
            rho1[f2, f1] = _trace(rho, tgt, sgn, [(f2, 0), (f1, 1)])
    rho2 = np.zeros((nf,) * 4)
    for f4 in range(nf):
        for f3 in range(nf):
            for f2 in range(nf):
                for f1 in range(nf):
                    rho2[f4, f3, f2, f1] = _trace(rho, tgt, sgn, [(f4, 0), (f3, 0), (f2, 1), (f1, 1)])
    return dict(densitymatrix=rho, occ=occ, rho1=rho1, rho2=rho2)


def _apply(tgt, sgn, ops):
    """The product of `ops` ((f, ca), last acting first) on every basis
    vector: (target index or -1, amplitude)."""
    ns = tgt.shape[2]
    cur = np.arange(ns)
    amp = np.ones(ns)
    for f, ca in reversed(ops):
        alive = cur >= 0
        c = np.where(alive, cur, 0)
        amp = np.where(alive, amp * sgn[f, ca, c], 0.0)
        cur = np.where(alive, tgt[f, ca, c], -1)
    return cur, amp


def spin_square(nd, occ_fock, sst_size, sst_offset, rho):
    """(ssquare, ssquare_operator).

    ssquare_operator: S^2 = S+S-/2 + S-S+/2 + Sz^2 summed over all orbitals
    (init_S2alt2, Operator.F90:548-633), S+ = sum_b c+_{b,up} c_{b,dn}, kept on
    the superstate blocks only and in the occupation basis of the states
    (create_ssquare_full, CTQMC.F90:2769-2806).  ssquare(N), N = 0 .. 2Nd:
    Tr(rho S^2) over the blocks of the superstates with N electrons
    (MeasureS2_from_densitymatrix, CTQMC.F90:2811-2838), with `rho` the
    normalised occupation-basis density matrix (the trace of a block does
    not depend on the basis)."""
    occ_fock = np.asarray(occ_fock, np.int64)
    ns = len(occ_fock)
    tgt, sgn = ladder_tables(nd, occ_fock)
    s2 = np.zeros((ns, ns))
    cols = np.arange(ns)
    for b in range(nd):
        for b2 in range(nd):
            up, dn, up2, dn2 = 2 * b, 2 * b + 1, 2 * b2, 2 * b2 + 1
            for ops in ([(up, 0), (dn, 1), (dn2, 0), (up2, 1)],    # S+_b S-_b2
                        [(dn, 0), (up, 1), (up2, 0), (dn2, 1)]):   # S-_b S+_b2
                cur, amp = _apply(tgt, sgn, ops)
                ok = cur >= 0
                np.add.at(s2, (cur[ok], cols[ok]), 0.5 * amp[ok])
    nup = sum((occ_fock >> b) & 1 for b in range(nd))
    ndn = sum((occ_fock >> (nd + b)) & 1 for b in range(nd))
    s2[cols, cols] += (0.5 * (nup - ndn)) ** 2
    block = np.full(ns, -1)
    for i, (o, n) in enumerate(zip(sst_offset, sst_size)):
        block[o:o + n] = i
    s2 = np.where(block[:, None] == block[None, :], s2, 0.0)
    ssq = np.zeros(2 * nd + 1)
    for o, n in zip(sst_offset, sst_size):
        ne = bin(int(occ_fock[o])).count("1")
        ssq[ne] += float(np.sum(rho[o:o + n, o:o + n] * s2[o:o + n, o:o + n].T))
    return ssq, s2
