"""Host estimators from the density matrix against the reference's own block
formulas (CTQMC.F90:2884-3060, 3163-3179) evaluated with the oracle's
eigenbasis blocks, on density matrices the oracle measured."""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import estimators as ES
from w2dynamics_gb300 import problems as P


def _oracle_dm(name, beta, nmeas):
    pr = P.config_problem(name, beta=beta)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    ch = O.Chain(mo, beta, pr["ftau"], 20, seed=5, taudiff_max=5.0, ncorr=20)
    ch.warmup(1000)
    ch.measure(nmeas)
    return pr, mo, ch.results()["densitymatrix"]


def _block_formulas(nd, mo, dm):
    """The reference's loops over superstate blocks (DGEMM + DDOT per state)."""
    nf = 2 * nd
    off, size = mo.sst_offset, mo.sst_size

    def blk(s):
        return dm[off[s]:off[s] + size[s], off[s]:off[s] + size[s]]

    def conn(s, f, ca):
        return mo.connect(s, f // 2, f % 2, ca)

    def op(s, f, ca):
        return mo.psis_eb(s, f // 2, f % 2, ca)

    rho1 = np.zeros((nf, nf))
    occ = np.zeros((nd, 2, nd, 2))
    for f1 in range(nf):
        for f2 in range(nf):
            for s in range(len(size)):
                ns1 = conn(s, f1, 1)
                if ns1 < 0:
                    continue
                if conn(ns1, f2, 0) == s:
                    t = blk(s) @ op(ns1, f2, 0)
                    c1 = op(s, f1, 1)
                    rho1[f2, f1] += sum(t[i, :] @ c1[:, i] for i in range(size[s]))
                ns2 = conn(s, f2, 1)
                if ns2 < 0:
                    continue
                t1 = blk(s) @ op(ns2, f2, 0)
                t2 = t1 @ op(s, f2, 1)
                t3 = t2 @ op(ns1, f1, 0)
                c1 = op(s, f1, 1)
                occ[f1 // 2, f1 % 2, f2 // 2, f2 % 2] += sum(t3[i, :] @ c1[:, i]
                                                            for i in range(size[s]))
    evec = np.zeros_like(dm)
    for s in range(len(size)):
        evec[off[s]:off[s] + size[s], off[s]:off[s] + size[s]] = mo.evec(s)
    rho2_some = {}
    picks = ((0, 1, 1, 0), (1, 0, 1, 0), (2, 3, 3, 2), (0, 2, 2, 0))
    for (f4, f3, f2, f1) in (p for p in picks if max(p) < nf):
        acc = 0.0
        for s in range(len(size)):
            n1 = conn(s, f1, 1)
            if n1 < 0:
                continue
            n2 = conn(n1, f2, 1)
            if n2 < 0:
                continue
            n3 = conn(n2, f3, 0)
            if n3 < 0 or conn(n3, f4, 0) != s:
                continue
            t = blk(s) @ op(n3, f4, 0) @ op(n2, f3, 0) @ op(n1, f2, 1)
            c1 = op(s, f1, 1)
            acc += sum(t[i, :] @ c1[:, i] for i in range(size[s]))
        rho2_some[(f4, f3, f2, f1)] = acc
    return rho1, occ, evec @ dm @ evec.T, rho2_some, evec


@pytest.mark.parametrize("name", ["anderson1", "dd3"])
def test_estimators_match_block_formulas(name):
    pr, mo, dm = _oracle_dm(name, 10.0, 200)
    nd = pr["nd"]
    rho1, occ, dm_occ, rho2_some, evec = _block_formulas(nd, mo, dm)
    got = ES.from_density_matrix(nd, mo.fock_states, evec, dm)
    assert np.allclose(got["densitymatrix"], dm_occ, atol=1e-13)
    assert np.allclose(got["rho1"], rho1, atol=1e-13)
    assert np.allclose(got["occ"], occ, atol=1e-13)
    for key, val in rho2_some.items():
        if max(key) < 2 * nd:
            assert abs(got["rho2"][key] - val) < 1e-13, key
    # occupancies: occ(i,i) = rho1(i,i) = <n_i>, trace of rho = 1
    nf = 2 * nd
    for f in range(nf):
        assert abs(got["occ"][f // 2, f % 2, f // 2, f % 2] - got["rho1"][f, f]) < 1e-13
    assert abs(np.trace(got["densitymatrix"]) - 1.0) < 1e-12


def test_ladder_tables_anticommute():
    """c and c+ tables satisfy {c_f, c+_g} = delta_fg on the whole space."""
    nd = 2
    occ_fock = np.arange(16)
    tgt, sgn = ES.ladder_tables(nd, occ_fock)
    ns = len(occ_fock)

    def mat(f, ca):
        m = np.zeros((ns, ns))
        for i in range(ns):
            if tgt[f, ca, i] >= 0:
                m[tgt[f, ca, i], i] = sgn[f, ca, i]
        return m
    for f in range(4):
        for g in range(4):
            ac = mat(f, 1) @ mat(g, 0) + mat(g, 0) @ mat(f, 1)
            assert np.allclose(ac, np.eye(ns) * (f == g))


def _s2_block_formula(nd, mo, dm):
    """<S^2> per electron number the reference's way: S^2 = S+S-/2 + S-S+/2
    + Sz^2 built block by block from the eigenbasis ladder operators along
    the superstate connections (Operator.F90:548-633), then the trace of
    rho_block S^2_block per superstate (CTQMC.F90:2811-2838)."""
    off, size = mo.sst_offset, mo.sst_size
    ssq = np.zeros(2 * nd + 1)

    def walk(s, ops):
        """Matrix of the product `ops` ((f, ca), last first) from block s
        back to block s, or None if it leaves the block or is forbidden."""
        cur, mat = s, np.eye(size[s])
        for f, ca in reversed(ops):
            nxt = mo.connect(cur, f // 2, f % 2, ca)
            if nxt < 0:
                return None
            mat = mo.psis_eb(cur, f // 2, f % 2, ca) @ mat
            cur = nxt
        return mat if cur == s else None

    for s in range(len(size)):
        s2 = np.zeros((size[s], size[s]))
        for b in range(nd):
            for b2 in range(nd):
                up, dn, up2, dn2 = 2 * b, 2 * b + 1, 2 * b2, 2 * b2 + 1
                for ops in ([(up, 0), (dn, 1), (dn2, 0), (up2, 1)],
                            [(dn, 0), (up, 1), (up2, 0), (dn2, 1)]):
                    m = walk(s, ops)
                    if m is not None:
                        s2 += 0.5 * m
                for ops, w in (([(up, 0), (up, 1), (up2, 0), (up2, 1)], 0.25),
                               ([(dn, 0), (dn, 1), (dn2, 0), (dn2, 1)], 0.25),
                               ([(up, 0), (up, 1), (dn2, 0), (dn2, 1)], -0.25),
                               ([(dn, 0), (dn, 1), (up2, 0), (up2, 1)], -0.25)):
                    m = walk(s, ops)
                    if m is not None:
                        s2 += w * m
        ne = bin(int(mo.fock_states[off[s]])).count("1")
        blk = dm[off[s]:off[s] + size[s], off[s]:off[s] + size[s]]
        ssq[ne] += float(np.trace(blk @ s2))
    return ssq


@pytest.mark.parametrize("name", ["anderson1", "dd3"])
def test_spin_square_matches_block_formula(name):
    """ssquare from the occupation-basis density matrix equals the
    reference's eigenbasis block evaluation on an oracle-measured density
    matrix; the S^2 operator has eigenvalues S(S+1) and its infinite-
    temperature mean is 3 Nd / 8."""
    pr, mo, dm = _oracle_dm(name, 10.0, 400)
    nd = pr["nd"]
    evec = np.zeros_like(dm)
    for s in range(len(mo.sst_size)):
        o, n = mo.sst_offset[s], mo.sst_size[s]
        evec[o:o + n, o:o + n] = mo.evec(s)
    rho = evec @ dm @ evec.T
    ssq, op = ES.spin_square(nd, mo.fock_states, mo.sst_size, mo.sst_offset, rho)
    ref = _s2_block_formula(nd, mo, dm)
    assert np.allclose(ssq, ref, atol=1e-12)
    assert ssq.sum() > 0.0
    ev = np.linalg.eigvalsh(op)
    twice_s = -1.0 + np.sqrt(1.0 + 4.0 * ev)
    assert np.allclose(twice_s, np.round(twice_s), atol=1e-9)
    flat, _ = ES.spin_square(nd, mo.fock_states, mo.sst_size, mo.sst_offset,
                             np.eye(mo.nstates) / mo.nstates)
    assert abs(flat.sum() - 3.0 * nd / 8.0) < 1e-12
