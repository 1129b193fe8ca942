"""Benchmark: MC updates/sec of the CT-HYB pair-move loop on one GB300.

Workload (the batched configuration): 4096 independent chains of the
3-orbital density-density model (U=4, J=0.6, U'=U-2J, mu=3.3 for filling
2/6, QuantumNumbers "Nt Szt"), 1024 chains at each beta in {10,25,50,100},
semicircular bath (D=1) with F(tau) on Ntau=Nftau=2000 points, seed = chain
index, TaudiffMax=5, NCorr=100.  One step = one measurement cycle of every
chain: NCorr pair proposals (StepAdd/StepRem, CTQMC.F90:8428-8476) and the
Z-space measurements (sign, order histogram, density matrix at beta/2,
G(tau)).  1 MC update = 1 proposed pair insertion or removal.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the oracle (the C++ restatement of the reference's
Fortran loop, which cannot be built here) on the host cores, one chain per
process, on a bounded sample of the same workload.
"""
import argparse
import json
import os
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
THERMALIZE = 2000  # proposals per chain before timing (not timed)
E2E_WARMUP = 1000  # re-thermalisation proposals per chain of the warm-started end-to-end solve
TUNE = 200         # of them, per candidate schedule of the autotuner (10 candidates)
CPU_SAMPLE_MEAS = 100  # measurement cycles per host core and round of the bounded CPU sample
# dense-block workload (--workload kanamori5): 5-orbital Kanamori with
# spin-flip and pair hopping, 1024 chains, one window (TaudiffMax <= 0)
K5_BETA, K5_CHAINS, K5_THERM = 40.0, 1024, 2000
METRIC = "MC updates/sec on 1 GB300, batched vs one-chain form, at equal G(tau) error"
# From one ncu capture (--set full) of a one-cycle sweep launch of this
# workload: DRAM bytes read + written, FP64-pipe and issue utilisation.
TRAFFIC_PER_STEP = 373.3e6
NCU_FP64_PIPE = 0.372
NCU_ISSUE_ACTIVE = 0.229


def workload_desc(chains_per_beta):
    return {"workload": f"{len(BETAS) * chains_per_beta} chains, 3-orbital density-density "
                        f"U=4 J=0.6 mu=3.3 (Nt Szt), beta in {list(BETAS)}, "
                        f"Ntau=Nftau={NTAU}, TaudiffMax={TDM}, NCorr={NCORR}",
            "chains": len(BETAS) * chains_per_beta, "betas": list(BETAS), "ncorr": NCORR,
            "step": "NCorr proposals per chain + measurement",
            "l2_flush": "inputs (chain state, ~GBs) larger than L2"}


def problems():
    from w2dynamics_gb300 import problems as P
    out = []
    for b in BETAS:
        out.append(P.config_problem("dd3", beta=b))
    return out


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


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def build_batch(E, probs, cpb, rank=0):
    """Model and `cpb` chains per beta for one GPU, from host arrays; seed =
    chain index of the whole job (rank r holds chains r*4*cpb ...)."""
    pr0 = probs[0]
    model = E.Model(pr0["nd"], pr0["umatrix"], pr0["muimp"], pr0["quantum_numbers"])
    groups = []
    for i, pr in enumerate(probs):
        groups.append(E.Group(pr["beta"], pr["ftau"], pr["ntau"], nchains=cpb,
                              seed0=(rank * len(probs) + i) * cpb, taudiff_max=TDM, ncorr=NCORR,
                              kcap=32 if pr["beta"] <= 25 else 64,
                              opcap=256 if pr["beta"] <= 25 else (512 if pr["beta"] <= 50 else 1024)))
    h2d = sum(g.ftau.nbytes for g in groups) + pr0["umatrix"].nbytes + pr0["muimp"].nbytes
    return model, groups, E.Batch(model, groups), h2d


def measure_backward(E, model, pr, args):
    """The differentiation configuration: 2048 chains of the same model at
    beta = 50; one forward step (NCorr proposals + measurement) against one
    backward pass (d log|w| of every chain w.r.t. the F(tau) grid and the
    2Nd + 2 parameters eps_f, U, J), both device-timed with CUDA events on the
    batch's stream."""
    import torch
    from w2dynamics_gb300 import gradients as GR
    n = 2048
    b = E.Batch(model, [E.Group(pr["beta"], pr["ftau"], pr["ntau"], nchains=n, seed0=0, taudiff_max=TDM,
                                ncorr=NCORR, kcap=64, opcap=512)])
    b.autotune(TUNE)
    b.warmup(THERMALIZE - 10 * TUNE)
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


def run_gpu_k5(args):
    """Dense-block workload: 1024 chains of the 5-orbital Kanamori model
    (U=3, J=0.7, crystal field, beta=40, 1024 states in 36 (N,Sz) blocks up
    to 100x100), Ntau = Nftau = 4000, NCorr = 100, seed = chain index.  The
    chains are thermalised for K5_THERM proposals only (orders still
    growing); the CPU sample runs the oracle on the same footing."""
    import torch
    from w2dynamics_gb300 import engine as E
    from w2dynamics_gb300 import problems as P
    pr = P.config_problem("kanamori5", beta=K5_BETA)
    model = E.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    b = E.Batch(model, [E.Group(K5_BETA, pr["ftau"], pr["ntau"], nchains=K5_CHAINS, seed0=0, taudiff_max=-1.0,
                                ncorr=NCORR, kcap=64, opcap=1024, tree_levels=4)])
    b.warmup(K5_THERM)
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        b.measure(1)
    b.sync()
    with ClockSampler() as clocks:
        start.record(stream)
        for _ in range(args.steps):
            b.measure(1)
        stop.record(stream)
        stop.synchronize()
    ms = start.elapsed_time(stop)
    value = K5_CHAINS * NCORR * args.steps / (ms / 1e3)
    korder = float(np.mean([b.state(c)["noper"] for c in range(0, K5_CHAINS, 64)]))
    b.close()
    cores = os.cpu_count() or 1
    cpu_value, cpu_wall = oracle_rate(cores, 2, 2, 0, workload="kanamori5")
    line = {
        "metric": METRIC, "value": value, "unit": "MC updates/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (semicircular bath D=2, seeded chains)",
        "config": {"workload": f"{K5_CHAINS} chains, 5-orbital Kanamori U=3 J=0.7 crystal field +-0.2, "
                               f"beta={K5_BETA}, Ntau=Nftau=4000, Nt Szt blocks, NCorr={NCORR}, "
                               f"{K5_THERM} thermalisation proposals",
                   "mean_operators_per_chain": korder},
        "cpu_baseline": {"value": cpu_value, "unit": "MC updates/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} chains (one per host core), {K5_THERM} thermalisation "
                                   f"proposals, 2 rounds of 2 x {NCORR} proposals ({cpu_wall:.1f} s)"},
        "gpu_launches": args.steps, "clocks": clocks.summary(),
    }
    print(json.dumps(line))


def run_gpu(args, rank=0, world=1):
    import torch
    from w2dynamics_gb300 import engine as E
    from w2dynamics_gb300 import shard

    cpb = args.chains_per_beta
    probs = problems()
    model, groups, batch, _ = build_batch(E, probs, cpb, rank)
    sched = batch.autotune(TUNE)  # thermalisation doubles as schedule tuning
    batch.warmup(THERMALIZE - 10 * TUNE)
    batch.sync()
    stream = torch.cuda.ExternalStream(batch.stream())
    for _ in range(args.warmup):
        batch.measure(1)
    batch.sync()
    batch.work_counters(reset=True)
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
    wc = batch.work_counters(reset=False)
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
    b2.warmup(E2E_WARMUP)  # automatic schedule (the autotuner's choice above on this workload)
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
    # plain one-chain drop-in form on the same model (beta=50 problem)
    single = E.Batch(model, [E.Group(probs[2]["beta"], probs[2]["ftau"], NTAU, nchains=1, seed0=0,
                                     taudiff_max=TDM, ncorr=NCORR, kcap=64, opcap=512)])
    single.warmup(THERMALIZE)
    single.sync()
    s_steps = max(3, args.steps)
    s0 = time.perf_counter()
    for _ in range(s_steps):
        single.measure(1)
    single.sync()
    s_time = time.perf_counter() - s0
    single_value = s_steps * NCORR / s_time
    backward = measure_backward(E, model, probs[2], args)
    cores = os.cpu_count() or 1
    cpu_value, cpu_wall = oracle_rate(cores, CPU_SAMPLE_MEAS, 3, 1)
    hbm, peak_kind = measured_peaks()
    bytes_per_step = (wc["m_bytes"] + wc["op_bytes"]) / max(1, args.steps)
    achieved = bytes_per_step / (ms / 1e3 / args.steps) / 1e9
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
        "one_chain_form": {"value": single_value, "unit": "MC updates/s",
                           "batched_over_one_chain": value / single_value},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": TRAFFIC_PER_STEP, "peak_kind": peak_kind,
                     "note": "per step (one measurement cycle, NCorr proposals a chain): "
                             "algorithmic bytes of M and operator arrays; traffic = ncu DRAM "
                             "bytes of a one-cycle launch; the kernel is bound by barrier "
                             "waits, load latency and the FP64 pipe, not HBM",
                     "ncu": {"fp64_pipe_busy": NCU_FP64_PIPE, "issue_active": NCU_ISSUE_ACTIVE}},
        "cpu_baseline": {"value": cpu_value, "unit": "MC updates/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} chains (one per host core, beta cycling over {list(BETAS)}), "
                                   f"{THERMALIZE} thermalisation proposals, then 3 rounds of "
                                   f"{CPU_SAMPLE_MEAS} measurement cycles x {NCORR} proposals per chain "
                                   f"({cpu_wall:.1f} s wall)"},
        "backward": backward,
        "work": wc,
        "schedule": {"warps_per_block": sched, "chosen_by": "autotuner (cthyb_batch_autotune)",
                     "cuda_graphs": "end-to-end solve (one launch per step); the device-timed "
                                    "steps run as one measure(K) call"},
        "gpu_launches": (args.steps + 199) // 200,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))


_WORKER = {}


def _worker_init(name, beta, seed, ftau, therm):
    """One oracle chain per process, built and thermalised once."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from w2dynamics_gb300 import problems as P
    pr = P.config_problem(name, beta=beta)
    m = O.Model(pr["nd"], pr["umatrix"], pr["muimp"], pr["quantum_numbers"])
    tdm = TDM if name == "dd3" else -1.0
    c = O.Chain(m, beta, ftau, 100, seed=seed, taudiff_max=tdm, ncorr=NCORR)
    c.warmup(therm)
    _WORKER["chain"], _WORKER["model"] = c, m


def _worker_run(nmeas):
    c = _WORKER["chain"]
    t0 = time.perf_counter()
    c.measure(nmeas)
    return time.perf_counter() - t0, nmeas * NCORR


def oracle_rate(cores, meas, rounds, warm_rounds, workload="batched"):
    """MC updates/s of the oracle (C++ restatement of the Fortran loop) on
    `cores` host cores, one chain per core (beta cycling over the groups of
    the batched workload), each round `meas` measurement cycles per chain;
    median over rounds."""
    import multiprocessing as mp
    from w2dynamics_gb300 import problems as P
    if workload == "kanamori5":
        specs = [("kanamori5", K5_BETA, P.config_problem("kanamori5", beta=K5_BETA)["ftau"], K5_THERM)]
    else:
        specs = [("dd3", b, P.semicircle_ftau(3, b, 1.0, NTAU), THERMALIZE) for b in BETAS]
    ctx = mp.get_context("spawn")
    pools = []
    for i in range(cores):
        name, b, ft, th = specs[i % len(specs)]
        pools.append(ctx.Pool(1, initializer=_worker_init, initargs=(name, b, i, ft, th)))
    try:
        for _ in range(warm_rounds):
            for r in [p.apply_async(_worker_run, (max(1, meas // 4),)) for p in pools]:
                r.get()
        vals = []
        t0 = time.perf_counter()
        for _ in range(rounds):
            res = [r.get() for r in [p.apply_async(_worker_run, (meas,)) for p in pools]]
            vals.append(sum(n for _, n in res) / max(t for t, _ in res))
        wall = time.perf_counter() - t0
    finally:
        for p in pools:
            p.terminate()
    return float(np.median(vals)), wall


def run_reference(args):
    """Oracle (C++ restatement of the Fortran loop) on all host cores, one
    chain per core; each step runs `ref_meas` measurement cycles per chain."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    value, wall = oracle_rate(cores, args.ref_meas if args.workload == "batched" else 2, args.steps,
                              args.warmup, workload=args.workload)
    line = {
        "metric": METRIC, "value": value, "unit": "MC updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (semicircular bath, seeded chains)",
        "config": workload_desc(args.chains_per_beta), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "MC updates/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} chains (one per core, beta cycling over {list(BETAS)}), "
                                   f"{args.ref_meas} measurement cycles of {NCORR} proposals per chain "
                                   f"and step after {THERMALIZE} thermalisation proposals"},
        "e2e": {"value": value, "unit": "MC updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--chains-per-beta", type=int, default=CHAINS_PER_BETA)
    ap.add_argument("--workload", default="batched", choices=("batched", "kanamori5"),
                    help="batched: the 4096-chain benchmark; kanamori5: dense-block 5-orbital model")
    ap.add_argument("--ref-meas", type=int, default=100,
                    help="measurement cycles per chain and step of the CPU reference arm")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "kanamori5":
        run_gpu_k5(args)
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
