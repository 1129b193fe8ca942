"""Benchmark: MC updates/sec of the CT-HYB pair-move loop on one GB300.

Workload (the batched configuration): 4096 independent chains of the
3-orbital density-density model (U=4, J=0.6, U'=U-2J, mu=3.3 for filling
2/6, QuantumNumbers "Nt Szt"), 1024 chains at each beta in {10,25,50,100},
semicircular bath (D=1) with F(tau) on Ntau=Nftau=2000 points, seed = chain
index, TaudiffMax=5, NCorr=100, and PercentageOuterMove = 0.1: pair
insertions and removals (StepAdd/StepRem, CTQMC.F90:8428-8476), a tenth of
them also moving the outer superstate, which makes every chain ergodic over
the superstate sectors (pair moves alone keep a chain in the sector it
starts in, so the G(tau) errors of the two forms would not compare).  One
step = one measurement cycle of every chain: NCorr proposals and the
Z-space measurements (sign, order histogram, density matrix at beta/2,
G(tau)).  1 MC update = 1 proposal.  The line also times the reference's
default move mix (PercentageGlobalMove = PercentageTauShiftMove = 0.005,
configspec:81-82), whose rare global moves rebuild every inverse matrix,
the dense-block workload (1024 chains of the 5-orbital Kanamori model) and
an off-diagonal-hybridisation workload (offdiag = 1), each with its own CPU
baseline.

Footing: every chain is thermalised for THERMALIZE proposals (the GPU run
reports the mean expansion order of each beta group after every round of
THERM_ROUND proposals, so the plateau is visible), then the schedule
autotuner runs (its proposals are further warm-up), then W warm-up steps;
the timed window is the next K steps.  The CPU arms run their chains
through exactly the same proposal window and report their mean orders too.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the oracle (the C++ restatement of the reference's
Fortran loop, which cannot be built here) on all host cores.
"""
import argparse
import hashlib
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BETAS = (10.0, 25.0, 50.0, 100.0)
CHAINS_PER_BETA = 1024  # 4096 chains, 1024 at each beta
NTAU = 2000
NCORR = 100
TDM = 5.0
MOVES = dict(p_outer=0.1)  # PercentageOuterMove: pair moves that may change the outer superstate
DEFAULT_MOVES = dict(p_global=0.005, p_shift=0.005)  # the reference's default mix (configspec:81-82)
THERM_ROUND = 2000   # proposals per chain between order read-outs
THERMALIZE = 20000   # thermalisation proposals per chain (10 rounds)
TUNE = 200           # autotuner proposals per candidate (10 candidates, 2 interleaved passes)
E2E_WARMUP = 1000    # re-thermalisation proposals of the warm-started end-to-end solve
CPU_CHAINS_PER_CORE = 64  # chains per host core in the bounded CPU sample (beta cycling)
ONE_CHAIN_BLOCKS, ONE_CHAIN_MEAS = 16, 30  # one-chain form: blocks x measurement cycles per beta
# time-bin tree depth per beta (-1: one leaf; 0: the engine's default from the
# operator capacity), the measured optima at the thermalised expansion orders
# (about 14, 36, 74, 148 operators at beta 10, 25, 50, 100)
BATCH_TREE_LEVELS = {10.0: -1, 25.0: -1, 50.0: 0, 100.0: 0}
ONE_CHAIN_TREE_LEVELS = {10.0: -1, 25.0: 2, 50.0: 3, 100.0: 4}
# dense-block workload: 5-orbital Kanamori with spin-flip and pair hopping
K5_BETA, K5_CHAINS, K5_THERM, K5_STEPS, K5_TUNE = 40.0, 1024, 2000, 2, 20
K5_TUNE_PROPS = 9 * 2 * K5_TUNE  # the autotuner's dense-model candidates x 2 K5_TUNE proposals
# off-diagonal hybridisation workload: the 3-orbital model with an orbital-mixing bath
OD_BETA, OD_CHAINS, OD_THERM, OD_STEPS, OD_MIX = 25.0, 4096, 10000, 20, 0.3
OD_CPU_CHAINS_PER_CORE, OD_CPU_STEPS = 8, 100
METRIC = "MC updates/sec on 1 GB300, batched vs one-chain form, at equal G(tau) error"
PROFILE = os.path.join(ROOT, "profiles", "k_sweep_sync_bench_4096chains.md")


def workload_desc(chains_per_beta):
    return {"workload": f"{len(BETAS) * chains_per_beta} chains, 3-orbital density-density "
                        f"U=4 J=0.6 mu=3.3 (Nt Szt), beta in {list(BETAS)}, "
                        f"Ntau=Nftau={NTAU}, TaudiffMax={TDM}, NCorr={NCORR}, "
                        f"PercentageOuterMove={MOVES['p_outer']}",
            "chains": len(BETAS) * chains_per_beta, "betas": list(BETAS), "ncorr": NCORR,
            "step": "NCorr proposals per chain + measurement",
            "window": f"proposals {THERMALIZE + 10 * TUNE} + W*{NCORR} ... + K*{NCORR} of every chain",
            "l2_flush": "inputs (chain state, ~GBs) larger than L2"}


def problems():
    from w2dynamics_gb300 import problems as P
    return [P.config_problem("dd3", beta=b) for b in BETAS]


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region:
    one `nvidia-smi -lms 50` process whose lines a thread collects; entering
    waits for its first line so that sampling is live when timing starts."""

    def __init__(self, interval_ms=50):
        self.samples = []
        self.interval_ms = interval_ms
        self._proc = None
        self._t = None
        self._first = threading.Event()

    def _run(self):
        for line in self._proc.stdout:
            v = [x.strip() for x in line.strip().split(",")]
            if len(v) >= 7:
                self.samples.append(v)
                self._first.set()
        self._first.set()

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", "0", f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", f"-lms={self.interval_ms}"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._proc = None
            return self
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        self._first.wait(timeout=10)
        return self

    def __exit__(self, *a):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=10)
            except subprocess.TimeoutExpired:
                self._proc.kill()
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(sm)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback"


def engine_sha():
    h = hashlib.sha256()
    for name in ("engine.cu", "engine.cuh", "model.cpp", "model.h"):
        with open(os.path.join(ROOT, "w2dynamics_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def profile_keys():
    """The machine-readable line of the committed ncu summary of the sweep
    kernel (`bench-keys: {...}`), and whether it was taken on this build."""
    try:
        with open(PROFILE) as f:
            for line in f:
                m = re.match(r"bench-keys:\s*(\{.*\})\s*$", line.strip())
                if m:
                    d = json.loads(m.group(1))
                    d["profile"] = os.path.relpath(PROFILE, ROOT)
                    d["same_build"] = d.get("engine_sha") == engine_sha()
                    return d
    except OSError:
        pass
    return None


def mean_orders(batch, ngroups):
    return [float(batch.chain_stats(g)["noper"].mean()) for g in range(ngroups)]


def thermalise(batch, ngroups, total, rnd=THERM_ROUND):
    """`total` proposals per chain in rounds of `rnd`; the mean operator
    count of each group after every round."""
    hist = []
    for _ in range(max(1, total // rnd)):
        batch.warmup(rnd)
        batch.sync()
        hist.append([round(x, 2) for x in mean_orders(batch, ngroups)])
    return hist


def sigma2_of_mean(per_chain_g):
    """Mean over (flavour, tau) of the variance of the chain-averaged G:
    per-chain estimates are independent, so var = var_c / n_chains."""
    g = np.asarray(per_chain_g).reshape(len(per_chain_g), -1)
    return float(np.mean(g.var(axis=0, ddof=1) / len(g)))


def build_batch(E, probs, cpb, rank=0, moves=MOVES):
    """Model and `cpb` chains per beta for one GPU, from host arrays; seed =
    chain index of the whole job (rank r holds chains r*4*cpb ...)."""
    pr0 = probs[0]
    model = E.Model(pr0["nd"], pr0["umatrix"], pr0["muimp"], pr0["quantum_numbers"])
    groups = []
    for i, pr in enumerate(probs):
        groups.append(E.Group(pr["beta"], pr["ftau"], pr["ntau"], nchains=cpb,
                              seed0=(rank * len(probs) + i) * cpb, taudiff_max=TDM, ncorr=NCORR,
                              kcap=32 if pr["beta"] <= 25 else 64,
                              opcap=256 if pr["beta"] <= 25 else (512 if pr["beta"] <= 50 else 1024),
                              tree_levels=BATCH_TREE_LEVELS.get(pr["beta"], 0), **moves))
    h2d = sum(g.ftau.nbytes for g in groups) + pr0["umatrix"].nbytes + pr0["muimp"].nbytes
    return model, groups, E.Batch(model, groups), h2d


def default_mix(E, probs, cpb, steps):
    """The same batch with the reference's default move mix (0.5 % global
    and 0.5 % tau-shift moves, no outer moves): THERMALIZE proposals, then
    `steps` device-timed steps (CUDA events on the batch's stream)."""
    import torch
    model, groups, b, _ = build_batch(E, probs, cpb, moves=DEFAULT_MOVES)
    b.warmup(THERMALIZE)
    b.autotune(TUNE)
    b.measure(1)
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    b.measure(steps)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    mc = [b.move_counters(c) for c in range(0, b.nchains, 64)]
    b.close()
    return {"moves": "PercentageGlobalMove=0.005, PercentageTauShiftMove=0.005 (pair moves otherwise)",
            "value": b.nchains * NCORR * steps / (ms / 1e3), "unit": "MC updates/s", "ms_per_step": ms / steps,
            "global_accepted_over_tried": float(sum(x["acc_glob"] for x in mc) / max(1, sum(x["try_glob"] for x in mc)))}


def one_chain_forms(E, model, probs):
    """The plain drop-in form (one chain, as one Fortran process runs it) at
    each beta: thermalised like the batch, then ONE_CHAIN_BLOCKS blocks of
    ONE_CHAIN_MEAS measurement cycles; device time (CUDA events on the
    batch's stream) of the measured blocks and the variance of its G(tau)
    mean from the spread of the block averages."""
    import torch
    out = []
    for pr in probs:
        b = E.Batch(model, [E.Group(pr["beta"], pr["ftau"], NTAU, nchains=1, seed0=0, taudiff_max=TDM,
                                    ncorr=NCORR, kcap=64, opcap=1024,
                                    tree_levels=ONE_CHAIN_TREE_LEVELS.get(pr["beta"], 0), **MOVES)])
        b.warmup(THERMALIZE + 10 * TUNE)
        b.sync()
        stream = torch.cuda.ExternalStream(b.stream())
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms, blocks, k0 = 0.0, [], b.state(0)["noper"]
        for _ in range(ONE_CHAIN_BLOCKS):
            b.reset_measurements()
            ev0.record(stream)
            b.measure(ONE_CHAIN_MEAS)
            ev1.record(stream)
            ev1.synchronize()
            ms += ev0.elapsed_time(ev1)
            blocks.append(b.group_gtau(0)[0])
        props = ONE_CHAIN_BLOCKS * ONE_CHAIN_MEAS * NCORR
        out.append({"beta": pr["beta"], "value": props / (ms / 1e3), "device_s": ms / 1e3,
                    "proposals": props, "sigma2_G": sigma2_of_mean(blocks),
                    "mean_order": [k0, b.state(0)["noper"]]})
        b.close()
    return out


def measure_backward(E, model, pr, args):
    """The differentiation configuration: 2048 thermalised chains of the same
    model at beta = 50; one forward step (NCorr proposals + measurement)
    against one backward pass (d log|w| of every chain w.r.t. the F(tau)
    grid and the 2Nd + 2 parameters eps_f, U, J), both device-timed with CUDA
    events on the batch's stream."""
    import torch
    from w2dynamics_gb300 import gradients as GR
    n = 2048
    b = E.Batch(model, [E.Group(pr["beta"], pr["ftau"], pr["ntau"], nchains=n, seed0=0, taudiff_max=TDM,
                                ncorr=NCORR, kcap=64, opcap=512, **MOVES)])
    b.warmup(THERMALIZE)
    b.sync()
    dev = torch.device("cuda")
    dE = torch.tensor(GR.density_density_directions(model.nd, model.fock_states), dtype=torch.float64, device=dev)
    nf, nft = 2 * model.nd, pr["ftau"].shape[2]
    gd = torch.empty((n, nf, nft), dtype=torch.float64, device=dev)
    gp = torch.empty((n, dE.shape[0]), dtype=torch.float64, device=dev)
    lw = torch.empty((n, 2), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()  # dE copied on torch's stream before the batch's stream reads it
    stream = torch.cuda.ExternalStream(b.stream())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    reps = max(3, args.steps // 4)
    for _ in range(2):  # warm-up
        b.measure(1)
        b.gradients_device(dE, gd, gp, lw)
    b.sync()
    ev[0].record(stream)
    for _ in range(reps):
        b.measure(1)
    ev[1].record(stream)
    for _ in range(reps):
        b.gradients_device(dE, gd, gp, lw)
    ev[2].record(stream)
    ev[2].synchronize()
    fwd = ev[0].elapsed_time(ev[1]) / reps
    bwd = ev[1].elapsed_time(ev[2]) / reps
    b.close()
    return {"config": "2048 chains, beta=50, 3-orbital density-density; d log|w| w.r.t. "
                      f"F(tau) ({nf}x{nft}) and {dE.shape[0]} H_loc parameters",
            "forward_step_ms": fwd, "backward_ms": bwd, "backward_over_forward": bwd / fwd}


def run_k5(E, args, fp64_peak):
    """Dense-block workload: 1024 chains of the 5-orbital Kanamori model
    (U=3, J=0.7, crystal field +-0.2, beta=40, 1024 states in 36 (N,Sz)
    blocks up to 100x100), Ntau = Nftau = 4000, one window, NCorr = 100,
    seed = chain index, K5_THERM thermalisation proposals; K5_STEPS timed
    steps.  Roofline: FP64 flops of the trace's block products (counted at
    run time from the recomputed products) against the live DFMA peak."""
    import torch
    from w2dynamics_gb300 import problems as P
    pr = P.config_problem("kanamori5", beta=K5_BETA)
    model = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    nch = args.k5_chains
    b = E.Batch(model, [E.Group(K5_BETA, pr["ftau"], pr["ntau"], nchains=nch, seed0=0, taudiff_max=-1.0,
                                ncorr=NCORR, kcap=64, opcap=1024, tree_levels=4, dmma=args.k5_dmma)])
    b.set_team(8)
    b.warmup(K5_THERM - K5_TUNE_PROPS)
    sched = b.autotune(2 * K5_TUNE)  # its proposals are the rest of the thermalisation
    b.measure(1)
    b.sync()
    st = b.chain_stats(0)
    outer = np.array([b.state(c)["outer_sst"] for c in range(nch)], int)
    sizes = model.sst_size[outer]
    b.work_counters(reset=True)
    stream = torch.cuda.ExternalStream(b.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    b.measure(K5_STEPS)
    stop.record(stream)
    stop.synchronize()
    ms = start.elapsed_time(stop)
    wc = b.work_counters()
    k_end = float(b.chain_stats(0)["noper"].mean())
    b.close()
    value = nch * NCORR * K5_STEPS / (ms / 1e3)
    achieved = wc["trace_flops"] / (ms / 1e3) / 1e9
    return {"workload": f"{nch} chains, 5-orbital Kanamori U=3 J=0.7 crystal field +-0.2, beta={K5_BETA}, "
                        f"Ntau=Nftau=4000, Nt Szt blocks (largest 100), one window, NCorr={NCORR}, "
                        f"{K5_THERM} thermalisation proposals (the last {K5_TUNE_PROPS} of them the schedule "
                        f"autotuner's; orders still growing), {K5_STEPS} timed steps",
            "block_products": "FP64 tensor cores (mma m8n8k4)" if args.k5_dmma else "FP64 fused multiply-adds",
            "value": value, "unit": "MC updates/s", "ms_per_step": ms / K5_STEPS,
            "mean_order": [float(st["noper"].mean()), k_end],
            "schedule": {"autotuner_choice": sched,
                         "meaning": "100 + T + 1000 x blocks per SM: team sweep of T warps per chain"
                                    if sched >= 100 else "phase-synchronous warps per block"},
            "outer_superstate_sizes": {int(k): int(v) for k, v in zip(*np.unique(sizes, return_counts=True))},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "GFLOP/s",
                         "frac": achieved / fp64_peak,
                         "note": "FP64 flops of the dense block products of the trace, counted at run time, "
                                 "over the device time; peak = live DFMA probe (cthyb_probe_fp64)",
                         "trace_flops_per_proposal": wc["trace_flops"] / max(1, wc["proposals"])}}


def od_problem():
    """The batched workload's 3-orbital model at beta = OD_BETA with an
    orbital-mixing bath: F_{bs,b's'}(tau) = delta_ss' A_bb' F(tau), F the
    semicircular bath's, A = (1 - OD_MIX) 1 + OD_MIX (all ones), positive
    definite (offdiag = 1: one inverse matrix over all six flavours)."""
    from w2dynamics_gb300 import problems as P
    pr = P.config_problem("dd3", beta=OD_BETA)
    nd = pr["nd"]
    A = (1.0 - OD_MIX) * np.eye(nd) + OD_MIX * np.ones((nd, nd))
    ff = np.zeros((nd, 2, nd, 2, pr["ntau"]))
    for b in range(nd):
        for b2 in range(nd):
            for s in range(2):
                ff[b, s, b2, s] = A[b, b2] * pr["ftau"][0, 0]
    pr["ftau_full"] = ff
    return pr


def run_od(E):
    """Off-diagonal workload: OD_CHAINS chains (seed = chain index),
    TaudiffMax = TDM, NCorr = NCORR, PercentageOuterMove as the headline,
    OD_THERM thermalisation proposals, then OD_STEPS timed steps."""
    import torch
    pr = od_problem()
    model = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(model, [E.Group(OD_BETA, pr["ftau"], pr["ntau"], nchains=OD_CHAINS, seed0=0, taudiff_max=TDM,
                                ncorr=NCORR, kcap=64, opcap=256, ftau_full=pr["ftau_full"], **MOVES)])
    b.warmup(OD_THERM)
    b.measure(1)
    b.sync()
    k0 = float(b.chain_stats(0)["noper"].mean())
    stream = torch.cuda.ExternalStream(b.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    b.measure(OD_STEPS)
    stop.record(stream)
    stop.synchronize()
    ms = start.elapsed_time(stop)
    b.sync()
    st = b.chain_stats(0)
    _, ssum, cnt = b.group_sums(0)
    b.close()
    return {"workload": f"{OD_CHAINS} chains, 3-orbital density-density U=4 J=0.6 mu=3.3 (Nt Szt), beta={OD_BETA}, "
                        f"orbital-mixing bath F_bb' = (delta_bb' (1-{OD_MIX}) + {OD_MIX}) F_semicircle, offdiag=1, "
                        f"Ntau=Nftau=2000, TaudiffMax={TDM}, NCorr={NCORR}, PercentageOuterMove=0.1, "
                        f"{OD_THERM} thermalisation proposals, {OD_STEPS} timed steps",
            "value": OD_CHAINS * NCORR * OD_STEPS / (ms / 1e3), "unit": "MC updates/s", "ms_per_step": ms / OD_STEPS,
            "mean_order": [k0, float(st["noper"].mean())], "mean_sign": ssum / max(1, cnt)}


def oracle_rate_od(cores):
    """The oracle on the off-diagonal workload through the GPU run's window:
    OD_CPU_CHAINS_PER_CORE chains per host core, OD_THERM + NCORR untimed
    proposals, then OD_CPU_STEPS timed measurement cycles."""
    pr = od_problem()
    model_args = (pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    specs = [[(OD_BETA, i * OD_CPU_CHAINS_PER_CORE + j, pr["ftau_full"], TDM, MOVES)
              for j in range(OD_CPU_CHAINS_PER_CORE)] for i in range(cores)]
    pools = _spawn_pools(model_args, specs)
    try:
        k0 = sum((r.get() for r in [p.apply_async(_worker_warm, (OD_THERM + NCORR,)) for p in pools]), [])
        res = [r.get() for r in [p.apply_async(_worker_run, (OD_CPU_STEPS,)) for p in pools]]
    finally:
        for p in pools:
            p.terminate()
    tmax = max(t for t, _, _ in res)
    return {"value": sum(n for _, n, _ in res) / tmax, "unit": "MC updates/s", "cores": cores, "kind": "port",
            "sample": f"{cores * OD_CPU_CHAINS_PER_CORE} chains ({OD_CPU_CHAINS_PER_CORE} per host core), "
                      f"{OD_THERM + NCORR} untimed proposals, then {OD_CPU_STEPS} timed measurement cycles "
                      f"({tmax:.2f} s per core)",
            "mean_order_start": _per_beta(k0), "mean_order_end": _per_beta(sum((k for _, _, k in res), []))}


def run_gpu(args, rank=0, world=1):
    import torch
    from w2dynamics_gb300 import engine as E
    from w2dynamics_gb300 import shard

    cpb = args.chains_per_beta
    probs = problems()
    ng = len(probs)
    model, groups, batch, _ = build_batch(E, probs, cpb, rank)
    therm = thermalise(batch, ng, THERMALIZE)
    sched = batch.autotune(TUNE)  # after thermalisation; its proposals are more warm-up
    stream = torch.cuda.ExternalStream(batch.stream())
    for _ in range(args.warmup):
        batch.measure(1)
    batch.sync()
    batch.reset_measurements()
    batch.work_counters(reset=True)
    batch.drift(reset=True)
    order_start = mean_orders(batch, ng)
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    nchains = world * len(BETAS) * cpb  # the whole job (weak scaling: fixed chains per GPU)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    with ClockSampler() as clocks:
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            # the K steps as one measure(K) call, as ctqmc_measure(Nmeas)
            # issues them: one sweep-kernel launch per 200 cycles
            batch.measure(args.steps)
            stop.record(stream)
        stop.synchronize()
    batch.sync()
    ms = shard.max_over_ranks(start.elapsed_time(stop))
    props = nchains * NCORR * args.steps
    value = props / (ms / 1e3)
    order_end = mean_orders(batch, ng)
    wc = batch.work_counters(reset=False)
    drift = batch.drift()
    sig2_b = [sigma2_of_mean(batch.group_gtau(g)) for g in range(ng)]
    # the thermalised configurations: what one DMFT iteration hands the next
    # through mc_config_inout (cthyb_solver.py:329-345)
    cfg = batch.get_configs()
    batch.close()
    # End to end through the public API: one warm-started solver call as a
    # DMFT iteration makes it -- model and chains from host arrays (U, mu,
    # F(tau) copied to the device), the previous configurations uploaded in
    # one call, E2E_WARMUP re-thermalisation proposals per chain, then every
    # step a measurement cycle and the device->host read of every group's
    # G(tau) and sign sums, and at the end the configurations read back.  All
    # proposals of the call count as updates (all at the thermalised order).
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    model2, groups2, b2, h2d = build_batch(E, probs, cpb, rank)
    b2.set_configs(*cfg)
    h2d += sum(a.nbytes for a in cfg)
    b2.set_schedule(sched)
    b2.warmup(E2E_WARMUP)
    b2.use_graphs(True)
    d2h = 0
    for _ in range(args.steps):
        b2.measure(1)
        for gi in range(len(groups2)):
            gs, ss, cn = b2.group_sums(gi)
            d2h += gs.nbytes + 16
    cfg_out = b2.get_configs()
    d2h += sum(a.nbytes for a in cfg_out)
    b2.sync()
    t_e2e = shard.max_over_ranks(time.perf_counter() - t0)
    b2.close()
    e2e_value = nchains * (E2E_WARMUP + NCORR * args.steps) / t_e2e
    if rank != 0:
        return
    # plain one-chain drop-in form at each beta, and the equal-error ratio:
    # the one-chain form needs t1 * sigma2_1 / sigma2_b to reach the batch's
    # G(tau) error at that beta; the batch reaches all four in its K steps
    ones = one_chain_forms(E, model, probs)
    t_batch = ms / 1e3
    t_equal = [o["device_s"] * o["sigma2_G"] / s2 for o, s2 in zip(ones, sig2_b)]
    one_rate = float(np.mean([o["value"] for o in ones]))
    backward = measure_backward(E, model, probs[2], args)
    dmix = default_mix(E, probs, cpb, args.steps)
    fp64_dfma, fp64_dmma = E.probe_fp64()
    k5 = run_k5(E, args, fp64_dfma) if not args.skip_k5 else None
    od = run_od(E) if not args.skip_od else None
    cores = os.cpu_count() or 1
    cpu = oracle_rate(cores, args.steps, args.warmup)
    if k5 is not None:
        k5["cpu_baseline"] = oracle_rate_k5(cores)
    if od is not None:
        od["cpu_baseline"] = oracle_rate_od(cores)
    hbm, hbm_kind = hbm_peak()
    bytes_per_step = (wc["m_bytes"] + wc["op_bytes"]) / max(1, args.steps)
    achieved = bytes_per_step / (ms / 1e3 / args.steps) / 1e9
    fp64_achieved = wc["m_flops"] / (ms / 1e3) / 1e9
    prof = profile_keys()
    line = {
        "metric": METRIC, "value": value, "unit": "MC updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (semicircular bath, seeded chains)",
        "config": workload_desc(cpb),
        "e2e": {"value": e2e_value, "unit": "MC updates/s",
                "h2d_bytes_per_step": int(h2d) // args.steps,
                "d2h_bytes_per_step": d2h // args.steps,
                "timed": f"warm-started solve: model+batch creation from host arrays, upload of "
                         f"the thermalised configurations, {E2E_WARMUP} re-thermalisation proposals "
                         f"per chain, {args.steps} steps each with G(tau) sums read back, "
                         f"configurations read back; bytes per step = per-call bytes / steps",
                "wall_s": t_e2e},
        "footing": {"thermalisation_proposals": THERMALIZE, "autotune_proposals": 10 * TUNE,
                    "mean_order_per_round": therm, "mean_order_start": order_start,
                    "mean_order_end": order_end},
        "equal_error": {
            "sigma2_G_batched": sig2_b,
            "one_chain": ones,
            "one_chain_seconds_to_batched_error": t_equal,
            "batched_seconds": t_batch,
            "batched_over_one_chain_at_equal_error": float(sum(t_equal) / t_batch),
            "note": "sigma2_G = mean over (flavour, tau bin) of the variance of the G(tau) mean: batched from "
                    "the spread of the per-chain estimates (1024 independent chains per beta), one-chain from "
                    "the spread of block averages; the one-chain form needs t1*sigma2_1/sigma2_b to reach "
                    "the batched error at each beta, the batch reaches all four betas in batched_seconds"},
        "one_chain_form": {"value": one_rate, "unit": "MC updates/s",
                           "batched_over_one_chain": value / one_rate},
        "roofline": {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_dfma, "unit": "GFLOP/s",
                     "frac": fp64_achieved / fp64_dfma,
                     "peak_kind": "live DFMA probe (cthyb_probe_fp64) on this GPU",
                     "note": "algorithmic FP64 flops of the determinant ratios and fast updates (counted at run "
                             "time) over the device time of the K steps; the kernel is latency-bound (see "
                             "binding), so both this and the HBM fraction are small by the nature of the workload",
                     "dmma_peak": fp64_dmma,
                     "fp64_pipe_active": (prof or {}).get("fp64_pipe_active"),
                     "binding": (prof or {}).get("binding"),
                     "hbm": {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                             "traffic": (prof or {}).get("dram_bytes_per_step"), "peak_kind": hbm_kind,
                             "note": "per step (one measurement cycle, NCorr proposals a chain): algorithmic "
                                     "bytes of M and operator arrays over the device time; traffic = ncu DRAM "
                                     "bytes per step of the timed launch from the committed profile "
                                     "(see ncu.same_build)"},
                     "ncu": prof},
        "cpu_baseline": cpu,
        "backward": backward,
        "default_move_mix": dmix,
        "drift": dict(drift, refresh_every=1000),
        "dense_block": k5,
        "offdiag": od,
        "work": wc,
        "schedule": {"warps_per_block": sched, "chosen_by": "autotuner (cthyb_batch_autotune) after thermalisation",
                     "cuda_graphs": "end-to-end solve (one launch per step); the device-timed "
                                    "steps run as one measure(K) call"},
        "gpu_launches": (args.steps + 199) // 200,
        "clocks": clocks.summary(),
        "engine_sha": engine_sha(),
    }
    print(json.dumps(line))


_WORKER = {}


def _worker_init(model_args, specs):
    """The oracle chains of one host core (test infrastructure only):
    model_args = (nd, umatrix, muimp, quantum_numbers), specs one (beta,
    seed, ftau, taudiff_max, moves) per chain."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    model = O.Model(*model_args)
    chains = []
    for beta, seed, ftau, tdm, moves in specs:
        chains.append((beta, O.Chain(model, beta, ftau, ftau.shape[-1], seed=seed, taudiff_max=tdm, ncorr=NCORR,
                                     **moves)))
    _WORKER["chains"], _WORKER["model"] = chains, model


def _spawn_pools(model_args, specs_per_core):
    """One single-process pool per host core.  The children do no numpy
    linear algebra of their own (F(tau) comes from the parent), and their
    BLAS runs single-threaded so that the cores are not oversubscribed."""
    import multiprocessing as mp
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    ctx = mp.get_context("spawn")
    return [ctx.Pool(1, initializer=_worker_init, initargs=(model_args, specs)) for specs in specs_per_core]


def _worker_warm(n):
    for _, c in _WORKER["chains"]:
        c.warmup(n)
    return [(b, c.state()["noper"]) for b, c in _WORKER["chains"]]


def _worker_run(nsteps):
    """nsteps measurement cycles of every chain of this core, timed."""
    t0 = time.perf_counter()
    for _, c in _WORKER["chains"]:
        c.measure(nsteps)
    t = time.perf_counter() - t0
    return t, nsteps * NCORR * len(_WORKER["chains"]), [(b, c.state()["noper"]) for b, c in _WORKER["chains"]]


def _per_beta(pairs):
    out = {}
    for b, k in pairs:
        out.setdefault(b, []).append(k)
    return [round(float(np.mean(out[b])), 2) for b in sorted(out)]


def oracle_rate(cores, steps, warmup):
    """MC updates/s of the oracle (C++ restatement of the Fortran loop) on
    `cores` host cores with CPU_CHAINS_PER_CORE chains each (beta cycling
    over the groups, seeds = chain index), through the GPU run's proposal
    window: THERMALIZE + 10 * TUNE + warmup * NCORR untimed proposals, then
    `steps` timed measurement cycles per chain."""
    probs = {pr["beta"]: pr for pr in problems()}
    pr0 = probs[BETAS[0]]
    model_args = (pr0["nd"], pr0["umatrix"], pr0["muimp"], pr0["quantum_numbers"])
    specs = []
    for i in range(cores):
        specs.append([])
        for j in range(CPU_CHAINS_PER_CORE):
            b = BETAS[(i * CPU_CHAINS_PER_CORE + j) % len(BETAS)]
            specs[-1].append((b, i * CPU_CHAINS_PER_CORE + j, probs[b]["ftau"], TDM, MOVES))
    pools = _spawn_pools(model_args, specs)
    try:
        warm = THERMALIZE + 10 * TUNE + warmup * NCORR
        k0 = sum((r.get() for r in [p.apply_async(_worker_warm, (warm,)) for p in pools]), [])
        t0 = time.perf_counter()
        res = [r.get() for r in [p.apply_async(_worker_run, (steps,)) for p in pools]]
        wall = time.perf_counter() - t0
    finally:
        for p in pools:
            p.terminate()
    tmax = max(t for t, _, _ in res)
    nprop = sum(n for _, n, _ in res)
    k1 = sum((k for _, _, k in res), [])
    return {"value": nprop / tmax, "unit": "MC updates/s", "cores": cores, "kind": "port",
            "sample": f"{cores * CPU_CHAINS_PER_CORE} chains ({CPU_CHAINS_PER_CORE} per host core, beta cycling "
                      f"over {list(BETAS)}), {warm} untimed proposals each (the GPU run's thermalisation, "
                      f"autotuning and warm-up), then {steps} timed measurement cycles of {NCORR} proposals "
                      f"each ({tmax:.2f} s per core, {wall:.2f} s wall)",
            "mean_order_start": _per_beta(k0), "mean_order_end": _per_beta(k1)}


def oracle_rate_k5(cores):
    """The oracle on the dense-block workload through the GPU run's window:
    one chain per host core (seeds 0..cores-1), K5_THERM + NCORR untimed
    proposals, then K5_STEPS timed measurement cycles."""
    from w2dynamics_gb300 import problems as P
    pr = P.config_problem("kanamori5", beta=K5_BETA)
    model_args = (pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    pools = _spawn_pools(model_args, [[(K5_BETA, i, pr["ftau"], -1.0, {})] for i in range(cores)])
    try:
        for r in [p.apply_async(_worker_warm, (K5_THERM + NCORR,)) for p in pools]:
            r.get()
        res = [r.get() for r in [p.apply_async(_worker_run, (K5_STEPS,)) for p in pools]]
    finally:
        for p in pools:
            p.terminate()
    tmax = max(t for t, _, _ in res)
    return {"value": sum(n for _, n, _ in res) / tmax, "unit": "MC updates/s", "cores": cores, "kind": "port",
            "sample": f"{cores} chains (one per host core), {K5_THERM + NCORR} untimed proposals, then "
                      f"{K5_STEPS} timed measurement cycles ({tmax:.2f} s)"}


def run_reference(args):
    """Oracle (C++ restatement of the Fortran loop) on all host cores through
    the GPU run's proposal window (see oracle_rate)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    cpu = oracle_rate(cores, args.steps, args.warmup)
    line = {
        "metric": METRIC, "value": cpu["value"], "unit": "MC updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * CPU_CHAINS_PER_CORE * cores * NCORR / cpu["value"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (semicircular bath, seeded chains)",
        "config": workload_desc(args.chains_per_beta), "impl": "reference",
        "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": "MC updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--chains-per-beta", type=int, default=CHAINS_PER_BETA)
    ap.add_argument("--skip-k5", action="store_true", help="leave out the dense-block (5-orbital) line")
    ap.add_argument("--skip-od", action="store_true", help="leave out the off-diagonal hybridisation line")
    ap.add_argument("--k5-chains", type=int, default=K5_CHAINS, help="chains of the dense-block line")
    ap.add_argument("--k5-dmma", action="store_true",
                    help="dense-block line with the block products on the FP64 tensor cores (A/B)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        # every rank runs its own chains (seeds offset by rank); the only
        # exchange is the host-side max of the step times over a gloo group
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("gloo")
    run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
