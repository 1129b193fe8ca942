"""Host-side pieces of the benchmark (no GPU): the off-diagonal workload's
hybridisation, the committed profile's machine-readable line and the
equal-error statistic."""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_offdiag_workload_hybridisation_is_a_valid_bath():
    """F_{bs,b's'}(tau) = delta_ss' A_bb' F(tau): spin diagonal, symmetric
    in the orbitals, positive-definite orbital matrix, the diagonal equal to
    the semicircular bath of the batched workload."""
    pr = bench.od_problem()
    ff = pr["ftau_full"]
    nd = pr["nd"]
    assert ff.shape == (nd, 2, nd, 2, pr["ntau"])
    for b in range(nd):
        for b2 in range(nd):
            assert np.all(ff[b, 0, b2, 1] == 0.0) and np.all(ff[b, 1, b2, 0] == 0.0)
            assert np.array_equal(ff[b, 0, b2, 0], ff[b2, 0, b, 0])
        assert np.array_equal(ff[b, 0, b, 0], pr["ftau"][b, 0])
    A = ff[:, 0, :, 0, pr["ntau"] // 3] / pr["ftau"][0, 0, pr["ntau"] // 3]
    assert np.all(np.linalg.eigvalsh(A) > 0)


def test_profile_keys_parse():
    """The sweep profile's bench-keys line parses and carries the DRAM bytes
    a step and the engine hash it was taken on (the bench line reports
    whether that is the present source's)."""
    k = bench.profile_keys()
    assert k is not None
    assert k["dram_bytes_per_step"] > 0
    assert len(k["engine_sha"]) == 16
    assert k["same_build"] == (k["engine_sha"] == bench.engine_sha())
    json.dumps(k)


def test_sigma2_of_mean_is_the_variance_of_the_mean():
    """sigma2_of_mean over per-chain estimates: the mean over bins of the
    sample variance divided by the number of chains."""
    rng = np.random.default_rng(3)
    x = rng.normal(size=(400, 2, 3, 5))
    got = bench.sigma2_of_mean(x)
    want = float(np.mean(np.var(x, axis=0, ddof=1) / x.shape[0]))
    assert abs(got - want) <= 1e-12 * want
