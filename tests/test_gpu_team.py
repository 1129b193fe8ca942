"""The team sweep and the FP64 tensor-core block products.

The team sweep (cthyb_batch_set_team) runs every chain in a block of T
warps taken from a cost-ordered queue; warp 0 runs the scalar phases with
the same functions as the other sweeps and the whole team evaluates the
dense-block trace.  The FP64 MMA path (CTHYB_FLAG_DMMA) evaluates block
products of at least 16 x 16 with m8n8k4 tensor-core MMAs.  Both must leave
each chain's proposal stream equal to the oracle's, proposal by proposal
(bookkeeping bit-exact, ratios to 1e-10), including rare moves.
"""
import numpy as np
import pytest

import oracle as O
from w2dynamics_gb300 import engine as E
from w2dynamics_gb300 import problems as P

from test_gpu_parity import compare_logs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return E.load(build_if_missing=True)


def _oracle_log(name, beta, qns, tdm, ntau, nprop, seed, moves):
    pr = P.config_problem(name, beta=beta)
    mo = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], qns or pr["quantum_numbers"])
    co = O.Chain(mo, beta, pr["ftau"], ntau, seed=seed, taudiff_max=tdm, **moves)
    co.start_log(nprop)
    co.warmup(nprop)
    return pr, co, co.log()


@pytest.mark.parametrize("name,beta,qns,tdm,nprop,seeds,team,dmma,moves", [
    ("kanamori5", 40.0, None, -1.0, 600, [0], 4, False, {}),          # 100-state outer superstate
    ("kanamori5", 40.0, None, -1.0, 600, [0], 16, False, {}),
    ("kanamori5", 40.0, None, -1.0, 600, [0], 4, True, {}),
    ("kanamori5", 40.0, None, -1.0, 600, [7, 4, 0], 2, True, {}),     # three chains, 50/5/100 states
    ("kanamori5", 40.0, None, -1.0, 600, [7], 0, True, {}),           # MMA blocks, one-warp sweep
    ("kanamori5", 10.0, None, 5.0, 1500, [3], 8, False, dict(p_outer=0.1, p_global=0.02, p_shift=0.02)),
    ("dd3", 25.0, None, 5.0, 4000, [5, 6], 2, False, dict(p_outer=0.1, p_global=0.01, p_shift=0.01)),
    ("dd3", 10.0, None, 4.0, 3000, [8], 4, False, dict(p_4op=0.1, p_global=0.02)),
])
def test_team_and_mma_keep_the_proposal_stream(lib, name, beta, qns, tdm, nprop, seeds, team, dmma, moves):
    ntau = 50
    refs = [_oracle_log(name, beta, qns, tdm, ntau, nprop, s, moves) for s in seeds]
    pr = refs[0][0]
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], qns or pr["quantum_numbers"])
    groups = [E.Group(beta, pr["ftau"], ntau, nchains=1, seed0=s, taudiff_max=tdm, kcap=64, opcap=1024,
                      tree_levels=4 if name == "kanamori5" else 0, dmma=dmma, **moves) for s in seeds]
    b = E.Batch(mg, groups)
    if team:
        b.set_team(team)
    b.set_log(nprop)
    b.warmup(nprop)
    b.sync()
    for c, (_, co, ref) in enumerate(refs):
        got = b.log(c)
        compare_logs(ref, got, pr["ftau"][0, 0], beta)
        so, sg = co.state(), b.state(c)
        assert so["noper"] == sg["noper"] and so["outer_sst"] == sg["outer_sst"]
        assert abs(so["trace_log"] - sg["trace_log"]) <= 1e-9 * max(1.0, abs(so["trace_log"]))
        assert (ref["outcome"] == 4).sum() > 10


def test_team_sweep_measurements_match_the_warp_sweep(lib):
    """Measured G(tau), sign and density matrix of a batch of dense-block
    chains run by the team sweep equal those of the phase-synchronous sweep
    (same chains, same proposals), so the queue order of the team sweep does
    not leak into results."""
    pr = P.config_problem("kanamori5", beta=10.0)
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    out = []
    for team in (0, 4):
        b = E.Batch(mg, [E.Group(10.0, pr["ftau"], 40, nchains=6, seed0=20, taudiff_max=-1.0, kcap=64,
                                 opcap=512, tree_levels=3)])
        if team:
            b.set_team(team)
        b.warmup(400)
        b.measure(4)
        b.sync()
        out.append([b.results(c) for c in range(6)])
    for ra, rb in zip(*out):
        assert ra["mean_sign"] == rb["mean_sign"]
        assert np.allclose(ra["gtau"], rb["gtau"], rtol=1e-9, atol=1e-12)
        assert np.allclose(ra["densitymatrix"], rb["densitymatrix"], rtol=1e-8, atol=1e-12)


def test_team_blocks_take_several_chains_from_the_queue(lib):
    """More chains than resident team blocks (one block per multiprocessor):
    blocks take further chains from the cost-ordered queue; every chain
    ends exactly where the phase-synchronous sweep leaves it."""
    pr = P.config_problem("kanamori5", beta=4.0)
    mg = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    n = 400
    out = []
    for team in (0, 8):
        b = E.Batch(mg, [E.Group(4.0, pr["ftau"], 20, nchains=n, seed0=1000, taudiff_max=-1.0, kcap=32,
                                 opcap=256, tree_levels=2)])
        if team:
            b.set_team(team, 1)
        b.warmup(300)
        b.measure(2)
        b.sync()
        out.append((b.get_configs(), [b.results(c)["mean_sign"] for c in range(n)],
                    b.group_gtau(0)))
        b.close()
    (ca, sa, ga), (cb, sb, gb) = out
    for x, y in zip(ca, cb):
        assert np.array_equal(x, y)
    assert sa == sb
    assert np.allclose(ga, gb, rtol=1e-9, atol=1e-12, equal_nan=True)  # NaN: chains with zero sign sum
