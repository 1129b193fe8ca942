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
    for (f4, f3, f2, f1) in ((0, 1, 1, 0), (1, 0, 1, 0), (2, 3, 3, 2), (0, 2, 2, 0)):
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
