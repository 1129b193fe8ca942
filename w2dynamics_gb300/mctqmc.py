"""Drop-in for the f2py module ``w2dyn.auxiliaries.CTQMC.mctqmc`` on the
pair-move path.

The reference's Python driver (w2dyn/dmft/cthyb_solver.py:21,113-114,
240-241,323-345,397-398,947-1035) talks to the Fortran module only through
these procedures and module variables:

  init_rnd(Nseed)                         CTQMC.F90:9404
  init_paras(parastr) / dest_paras()      CTQMC.F90:9412 / 9420
  init_solver(u_matrix, Ftau_full, muimp_full, screening, iter_no)
                                          CTQMC.F90:7894-8086
  set_taudiffmax(x)                       CTQMC.F90:8180
  ctqmc_warmup(N)                         CTQMC.F90:8188-8263
  ctqmc_measure(iSector, iComponent)      CTQMC.F90:8355-8760
  init_counters()                         CTQMC.F90:847-899
  get_mc_config_scalars(), get_mc_config(N), set_mc_config(...),
  set_empty_mc_config(sst, state)         CTQMC.F90:9358-9392
  dest_ctqmc()                            CTQMC.F90:901
  gtau, gtau_full, histo, occ, rho1, rho2, densitymatrix, mean_sign,
  statessuperstates, eigenstatesenergies, occbasismapping, accadd, accrem,
  time_warmup, time_sim, time_sim_steps, aborted, ...

so ``import w2dynamics_gb300.mctqmc as ctqmc`` in place of the f2py import
runs the same solve on the GPU engine.  The module keeps the reference's
singleton semantics (one solver per process).  Parameters are read from the
parameter string with the reference's rules (Parameters.F90:281-320: one
``key = value`` per line, text after ``#`` ignored, commas as blanks, a key
matches the first parameter whose name starts with it).

Beyond the reference: ``GPUChains = n`` in the parameter string runs n
independent chains (seeds Nseed .. Nseed+n-1) in one batch and combines
their measurements as one longer run would (sign-weighted), the form in
which the GPU is used efficiently.  set_mc_config / set_empty_mc_config
give every chain the configuration; get_mc_configs / set_mc_configs and
save_mc_configs / load_mc_configs keep one configuration per chain across
solves (the batch form of the driver's mc_config_inout warm start and its
CtHybConfig npz files, cthyb_solver.py:24-87, 316-345).

Parameters selecting moves or modes outside the engine (worm and
flavour-change moves, segment, state sampling, retarded interactions)
raise NotImplementedError at init_solver.  With offdiag = 1 the full
Ftau_full is used and gtau_full / gleg_full hold G and its Legendre
coefficients for every flavour pair (MeasGtauRem_full).  The
trace-recomputation histograms lhisto/rhisto describe the reference's
list-walking implementation and are returned as zeros; outer trace
contributions are measured for density-density (monomial) models.  The
window calibration (ctqmc_calibrate, run by the driver for TaudiffMax <= 0)
fills accpairtau and accpair from the engine's proposal records; after a
measurement accpair holds the accepted pairs of the measurement run by
flavour and time difference (Nd, 2, Ntau), counted on the device.  Each
init_solver seeds the chains from Nseed; the reference continues one global
random stream across solves, so solves after the first draw different
(equally valid) streams.
"""
import time

import numpy as np

from . import engine as E
from . import estimators as ES

NWormSectors = 16  # CTQMC.F90:111

_seed = 0
_params = []          # (key, value) in input order
_model = None
_batch = None
_nd = 0
_beta = 0.0
_nchains = 1
_taudiffmax = 0.0     # the window's taudiff_max (beta for TaudiffMax <= 0, init_window)

# module variables read by the driver (reset by dest_ctqmc)
gtau = gtau_full = histo = occ = rho1 = rho2 = densitymatrix = None
gleg = gleg_full = None
statessuperstates = eigenstatesenergies = occbasismapping = None
outersuperstatehisto = outerstatehisto = signhistosuperstates = signhistostates = None
tracecontribsuperstates = tracecontribstates = None
lhisto = rhisto = None
ssquare = ssquare_operator = None
# scalars are 0-d arrays, as f2py exposes them (the driver copies every
# result with .copy(), cthyb_solver.py:1028-1030)
mean_sign = np.array(0.0)
accadd = np.zeros(NWormSectors)
accrem = np.zeros(NWormSectors)
accadd4, accrem4, accglob, accshift, accflavc = (np.array(0.0) for _ in range(5))
accpair = accpairtau = None
time_warmup, time_sim, time_sim_steps = (np.array(0.0) for _ in range(3))
aborted = 0
simid = 0
fancy_prog = False
fourpnt = 0


# --------------------------------------------------------------- parameters
def init_rnd(Nseed):
    """Seed of the random stream (init_rnd, CTQMC.F90:9404)."""
    global _seed
    _seed = int(Nseed)


def init_paras(parastr):
    """Parse the parameter string (read_ParameterString, Parameters.F90:281)."""
    global _params
    _params = []
    for line in str(parastr).split("\n"):
        line = line.replace("\t", " ")
        if line.startswith("#"):
            continue
        if "#" in line:
            line = line[:line.index("#")]
        if "=" not in line:
            continue
        key, val = line.split("=", 1)
        _params.append((key.strip(), val.strip().replace(",", " ")))


def dest_paras():
    global _params
    _params = []


def _raw(key):
    for k, v in _params:  # get_*_Parameter: first name that starts with key
        if k.startswith(key):
            return v
    raise KeyError(f"{key} not found in parameter list")


def _int(key, default=None):
    try:
        v = _raw(key)
    except KeyError:
        if default is None:
            raise
        return default
    try:
        return int(v.split()[0])
    except ValueError:
        r = float(v.split()[0])
        if r != int(r):
            raise ValueError(f"{key} is not an integer")
        return int(r)


def _real(key, default=None):
    try:
        return float(_raw(key).split()[0])
    except KeyError:
        if default is None:
            raise
        return default


def _str(key, default=None):
    try:
        return _raw(key)
    except KeyError:
        if default is None:
            raise
        return default


def _check_supported():
    bad = []
    if _real("PercentageWormInsert", 0.0) != 0.0:
        bad.append(f"PercentageWormInsert = {_real('PercentageWormInsert')}")
    for key in ("segment", "statesampling", "Phonon", "Screening", "Uw", "flavourchange_moves"):
        if _int(key, 0) != 0:
            bad.append(f"{key} = {_int(key)}")
    if _int("Eigenbasis", 1) == 0:
        bad.append("Eigenbasis = 0")
    if bad:
        raise NotImplementedError("outside the GPU pair-move engine: " + ", ".join(bad))


# ------------------------------------------------------------------- solver
def init_solver(u_matrix, Ftau_full, muimp_full, screening, iter_no):
    """Model and chain(s) for one solve (init_solver, CTQMC.F90:7894-8086)."""
    global _model, _batch, _nd, _beta, _nchains, _taudiffmax
    _check_supported()
    ftau_full = np.asarray(Ftau_full, np.float64)
    nd = ftau_full.shape[0]
    nftau = ftau_full.shape[-1]
    ftau = np.empty((nd, 2, nftau))
    for b in range(nd):  # Ftau(ib,is,:) = Ftau_full(ib,is,ib,is,:)
        for s in range(2):
            ftau[b, s] = ftau_full[b, s, b, s]
    mu = np.asarray(muimp_full, np.float64).reshape(nd, 2, nd, 2)
    um = np.asarray(u_matrix, np.float64).reshape((2 * nd,) * 4)
    qns = _str("QuantumNumbers", "Nt Szt")
    if "All" in qns.split():  # automatic partitioning with the EPSBLOCK threshold
        qns = f"{qns} EPSBLOCK={_real('EPSBLOCK', 1e-13)!r}"
    dest_ctqmc()
    _nd, _beta = nd, _real("beta")
    _nchains = max(1, _int("GPUChains", 1))
    _taudiffmax = _real("TaudiffMax", -1.0) if _real("TaudiffMax", -1.0) > 0.0 else _beta
    _model = E.Model(nd, um, mu, qns)
    offdiag = _int("offdiag", 0) != 0
    group = E.Group(_beta, ftau, _int("Ntau"), nchains=_nchains, seed0=_seed,
                    taudiff_max=_real("TaudiffMax", -1.0), ncorr=_int("NCorr"),
                    p_outer=_real("PercentageOuterMove", 0.0), maxhisto=_int("MaxHisto", 500) + 1,
                    measure_dm=_int("MeasDensityMatrix", 1) != 0,
                    p_global=_real("PercentageGlobalMove", 0.0),
                    p_shift=_real("PercentageTauShiftMove", 0.0),
                    nleg=_int("NLegMax", 100),
                    p_4op=_real("Percentage4OperatorMove", 0.0),
                    ftau_full=ftau_full if offdiag else None, measure_accpair=True)
    nsym = _int("NSymMove", 0)
    if nsym > 0:  # SymMove01 ... (Trace.F90:471-477)
        group.symmoves = np.array([[int(x) for x in _raw("SymMove%02d" % (i + 1)).split()]
                                   for i in range(nsym)], np.int32)
    _batch = E.Batch(_model, [group])
    _model_tables()


def _model_tables():
    """statessuperstates, eigenstatesenergies and occbasismapping of the
    present model (init_solver)."""
    global statessuperstates, eigenstatesenergies, occbasismapping
    ns, nd = _model.nstates, _nd
    statessuperstates = np.zeros(ns, np.int32)
    for s in range(_model.nsst):
        o, n = _model.sst_offset[s], _model.sst_size[s]
        statessuperstates[o:o + n] = s
    eigenstatesenergies = np.array(_model.evals)
    fk, _ = _model.basis()
    occbasismapping = np.zeros((ns, nd, 2), np.int32)
    for b in range(nd):
        for s in range(2):
            occbasismapping[:, b, s] = (fk >> (b + s * nd)) & 1


def set_taudiffmax(x):
    global _taudiffmax
    _batch.set_taudiffmax(0, float(x))
    _taudiffmax = float(x) if float(x) > 0.0 else _beta


def _accepted_pairs(rec, offdiag):
    """Flavours f = 2(b-1) + (s-1) and time differences of the accepted pair
    insertions and removals in proposal records, in proposal order: the
    entries StepAdd / StepRem add to AccPair and AccPairTau
    (CTQMC.F90:3579-3587, 4112-4127).  The flavour is that of the earlier
    operator of an inserted pair and of the creator of a removed pair; with
    diagonal hybridisation both operators have it."""
    r = rec[(rec["outcome"] == 4) & ((rec["move"] == 0) | (rec["move"] == 1))]
    dt = np.abs(r["tau_a"] - r["tau_c"])
    if not offdiag:  # orb, spin 1-based
        f = 2 * (r["orb"] - 1) + (r["spin"] - 1)
    else:  # orb = creator flavour + 1, spin = annihilator flavour + 1
        fc, fa = r["orb"] - 1, r["spin"] - 1
        f = np.where((r["move"] == 0) & (r["tau_a"] < r["tau_c"]), fa, fc)
    return f.astype(np.int64), dt


def ctqmc_calibrate(list_, phase1pairnum, phase2taugrid, phase2pairnum, nprogress=100000, chunk=1000,
                    max_chunks=10000):
    """Window calibration (ctqmc_calibrate, CTQMC.F90:8088-8175): Z-space
    proposals of every chain until, with list_, phase1pairnum accepted pair
    moves have given their time differences (accpairtau, taken from the
    chains in turn), or else until every flavour has phase2pairnum accepted
    pairs in the histogram accpair (Nd, 2, phase2taugrid) of time differences
    over [0, taudiff_max).  The proposals advance the chains like a warm-up.
    The engine's proposal records are read back after every `chunk`
    proposals of each chain; RuntimeError after max_chunks chunks (the
    reference would loop forever, e.g. for a flavour without accepted
    pairs).  nprogress only paces the reference's progress output."""
    global accpairtau, accpair
    offdiag = _int("offdiag", 0) != 0
    nf = 2 * _nd
    if list_:
        per_chain = -(-int(phase1pairnum) // _nchains)
        got = [[] for _ in range(_nchains)]
    else:
        hist = np.zeros((nf, int(phase2taugrid)), np.int64)
    try:
        for _ in range(max_chunks):
            _batch.set_log(chunk)
            _batch.warmup(chunk)
            _batch.sync()
            for c in range(_nchains):
                if list_ and len(got[c]) >= per_chain:
                    continue
                f, dt = _accepted_pairs(_batch.log(c), offdiag)
                if list_:
                    got[c].extend(dt[:per_chain - len(got[c])].tolist())
                else:
                    # min(NAccPair, floor(dtau / AccPairMax * NAccPair) + 1), 1-based
                    b = np.minimum(int(phase2taugrid), np.floor(dt / _taudiffmax * phase2taugrid).astype(np.int64) + 1)
                    np.add.at(hist, (f, b - 1), 1)
                    if hist.sum(axis=1).min() >= phase2pairnum:
                        break
            if list_ and all(len(g) >= per_chain for g in got):
                accpairtau = np.concatenate([np.asarray(g) for g in got])[:int(phase1pairnum)]
                return
            if not list_ and hist.sum(axis=1).min() >= phase2pairnum:
                accpair = hist.reshape(_nd, 2, int(phase2taugrid))
                return
        raise RuntimeError("window calibration did not complete within %d x %d proposals per chain"
                           % (max_chunks, chunk))
    finally:
        _batch.set_log(0)


def ctqmc_warmup(N):
    global time_warmup
    t0 = time.perf_counter()
    _batch.warmup(int(N))
    _batch.sync()
    time_warmup = np.array(time.perf_counter() - t0)


def init_counters():
    """Counters restart with every measurement call of the engine."""


def ctqmc_measure(iSector=1, iComponent=1):
    """Z-space loop and normalised results (CTQMC.F90:8355-8760)."""
    global time_sim, time_sim_steps
    if iSector != 1:
        raise NotImplementedError("worm sectors are outside the GPU pair-move engine")
    t0 = time.perf_counter()
    _batch.reset_measurements()
    _batch.measure(_int("Nmeas"))
    _batch.sync()
    time_sim = np.array(time.perf_counter() - t0)
    time_sim_steps = time_sim.copy()
    _collect()


def _collect():
    global gtau, gtau_full, histo, occ, rho1, rho2, densitymatrix, mean_sign, gleg, gleg_full
    global accadd, accrem, accadd4, accrem4, accglob, accshift, accpair, outersuperstatehisto, outerstatehisto, signhistosuperstates
    global signhistostates, tracecontribsuperstates, tracecontribstates, lhisto, rhisto
    global ssquare, ssquare_operator
    nd, ns, nf = _nd, _model.nstates, 2 * _nd
    res = [_batch.results(c) for c in range(_nchains)]
    signs = np.array([r["mean_sign"] for r in res])
    wsum = signs.sum()
    # the per-chain results are normalised by their own mean sign; one
    # combined run is the sign-weighted average
    gtau = sum(r["gtau"] * s for r, s in zip(res, signs)) / wsum
    dm_eigen = sum(r["densitymatrix"] * s for r, s in zip(res, signs)) / wsum
    mean_sign = np.array(signs.mean())
    histo = sum(r["histo"] for r in res) / _nchains
    cnt = {k: sum(r["counters"][k] for r in res) for k in res[0]["counters"]}
    mc = [_batch.move_counters(c) for c in range(_nchains)]
    mcnt = {k: sum(x[k] for x in mc) for k in mc[0]}
    accadd = np.zeros(NWormSectors)
    accrem = np.zeros(NWormSectors)
    accadd[0] = cnt["acc_add"] / max(cnt["try_add"], 1)
    accrem[0] = cnt["acc_rem"] / max(cnt["try_rem"], 1)
    accadd4 = np.array(mcnt["acc_add4"] / mcnt["try_add4"] if mcnt["try_add4"] else 0.0)
    accrem4 = np.array(mcnt["acc_rem4"] / mcnt["try_rem4"] if mcnt["try_rem4"] else 0.0)
    accglob = np.array(mcnt["acc_glob"] / mcnt["try_glob"] if mcnt["try_glob"] else float("nan"))
    accshift = np.array(mcnt["acc_shift"] / mcnt["try_shift"] if mcnt["try_shift"] else float("nan"))
    gtau_full = np.zeros((nd, 2, nd, 2, gtau.shape[-1]))
    if _batch.groups[0].ftau_full is not None:
        # offdiag = 1: MeasGtauRem_full fills Gtau_full, Gtau stays zero
        gf = sum(_batch.results_full(c) * s for c, s in zip(range(_nchains), signs)) / wsum
        for fa in range(nf):
            for fc in range(nf):
                gtau_full[fa // 2, fa % 2, fc // 2, fc % 2] = gf[fa, fc]
    else:
        for b in range(nd):
            for s in range(2):
                gtau_full[b, s, b, s] = gtau[b, s]
    if _int("MeasDensityMatrix", 1) != 0:
        fk, evec = _model.basis()
        est = ES.from_density_matrix(nd, fk, evec, dm_eigen)
        densitymatrix, occ, rho1, rho2 = (est["densitymatrix"], est["occ"], est["rho1"],
                                          est["rho2"])
        if _int("MeasSsquare", 0) != 0:
            ssquare, ssquare_operator = ES.spin_square(nd, fk, _model.sst_size, _model.sst_offset,
                                                       densitymatrix)
    else:
        densitymatrix = np.zeros((ns, ns))
        occ = np.zeros((nd, 2, nd, 2))
        rho1 = np.zeros((nf, nf))
        rho2 = np.zeros((nf,) * 4)
    ext = [_batch.results_extra(c) for c in range(_nchains)]
    gleg = sum(x["gleg"] * s for x, s in zip(ext, signs)) / wsum
    nleg = gleg.shape[-1]
    gleg_full = np.zeros((nd, 2, nd, 2, nleg))
    if _batch.groups[0].ftau_full is not None and nleg > 0:
        # offdiag = 1: MeasGtauRem_full fills GLeg_full, GLeg stays zero
        glf = sum(_batch.results_gleg_full(c) * s for c, s in zip(range(_nchains), signs)) / wsum
        for fa in range(nf):
            for fc in range(nf):
                gleg_full[fa // 2, fa % 2, fc // 2, fc % 2] = glf[fa, fc]
    else:
        for b in range(nd):
            for s in range(2):
                gleg_full[b, s, b, s] = gleg[b, s]
    outersuperstatehisto = sum(x["outer_sst_histo"] for x in ext) / _nchains
    outerstatehisto = sum(x["outer_state_histo"] for x in ext) / _nchains
    with np.errstate(invalid="ignore", divide="ignore"):
        # per-chain signs are normalised by their own visit counts
        signhistosuperstates = (sum(np.nan_to_num(x["sign_sst"]) * x["outer_sst_histo"] for x in ext)
                                / (outersuperstatehisto * _nchains))
        signhistostates = (sum(np.nan_to_num(x["sign_state"]) * x["outer_state_histo"] for x in ext)
                           / (outerstatehisto * _nchains))
    tracecontribsuperstates = sum(x["contrib_sst"] for x in ext) / _nchains
    tracecontribstates = sum(x["contrib_state"] for x in ext) / _nchains
    lhisto = np.zeros(1)
    rhisto = np.zeros(1)
    if hasattr(_batch, "results_accpair"):
        # AccPair of the measurement run (NAccPair = Ntau bins over [0, beta))
        accpair = sum(_batch.results_accpair(c) for c in range(_nchains)).astype(np.int64)
    else:
        accpair = np.zeros((nd, 2, _int("Ntau")), np.int64)


# ------------------------------------------------------ configuration access
def get_mc_config_scalars():
    """(number of operators, outer superstate, outer state)."""
    taus, *_ , outer = _batch.get_config(0)
    return len(taus), outer, 1


def get_mc_config(N):
    """(taus, orbs, spins, cas, hashybs, outer_sst, outer_state), 1-based
    orbital/spin/ca as in get_mc_config (CTQMC.F90:9367)."""
    taus, orbs, spins, cas, outer = _batch.get_config(0)
    n = int(N)
    return (np.array(taus[:n]), np.array(orbs[:n]), np.array(spins[:n]), np.array(cas[:n]),
            np.ones(n, np.int32), outer, 1)


def set_mc_config(N, taus, orbs, spins, cas, hashybs, outer_sst, outer_state):
    """set_mc_config (CTQMC.F90:9378): the configuration goes to every chain
    of the solver (one upload for all GPUChains chains)."""
    n = int(N)
    if np.any(np.asarray(hashybs)[:n] == 0):
        raise NotImplementedError("operators without hybridisation (worms) are not supported")
    arrs = [np.asarray(a)[:n] for a in (taus, orbs, spins, cas)]
    _replicate(arrs, int(outer_sst))


def set_empty_mc_config(outer_sst, outer_state):
    """set_empty_mc_config (CTQMC.F90:9391) for every chain."""
    _replicate([np.zeros(0), np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32)],
               int(outer_sst))


def _replicate(arrs, outer_sst):
    n = len(arrs[0])
    offs = np.arange(_nchains + 1, dtype=np.int32) * n
    _batch.set_configs(offs, *[np.tile(a, _nchains) for a in arrs], np.full(_nchains, outer_sst, np.int32))


def get_mc_configs():
    """Every chain's configuration in one read (the batch form of
    get_mc_config): dict of offsets (chain c's operators are entries
    offsets[c] .. offsets[c+1]-1), taus, orbs, spins, cas, hashybs (1-based
    as get_mc_config), outer_sst and outer_state per chain."""
    offs, t, o, s, c, outer = _batch.get_configs()
    return dict(offsets=offs, taus=t, orbs=o, spins=s, cas=c, hashybs=np.ones(len(t), np.int32),
                outer_sst=outer, outer_state=np.ones(len(outer), np.int32))


def set_mc_configs(cfg):
    """Inverse of get_mc_configs: chain c takes configuration c (one upload)."""
    offs = np.asarray(cfg["offsets"], np.int32)
    if len(offs) != _nchains + 1:
        raise ValueError(f"{len(offs) - 1} configurations for {_nchains} chains")
    if np.any(np.asarray(cfg["hashybs"]) == 0):
        raise NotImplementedError("operators without hybridisation (worms) are not supported")
    _batch.set_configs(offs, cfg["taus"], cfg["orbs"], cfg["spins"], cfg["cas"], cfg["outer_sst"])


def save_mc_configs(file):
    """All chains' configurations to an npz file with the keys of the
    driver's CtHybConfig.save_to_file (cthyb_solver.py:78-87) plus
    `offsets`; outer_sst/outer_state hold one entry per chain."""
    np.savez(file, **get_mc_configs())


def load_mc_configs(file):
    """Warm start from an npz file: a file of save_mc_configs gives chain c
    its own configuration; a file of the driver's CtHybConfig (one
    configuration, no `offsets`) goes to every chain like set_mc_config."""
    with np.load(file) as f:
        if "offsets" in f.files:
            set_mc_configs({k: f[k] for k in f.files})
        else:
            t = f["taus"]
            if t.size:
                set_mc_config(t.size, t, f["orbs"], f["spins"], f["cas"], f["hashybs"],
                              int(f["outer_sst"][0]), int(f["outer_state"][0]))
            else:
                set_empty_mc_config(int(f["outer_sst"][0]), int(f["outer_state"][0]))


def dest_ctqmc():
    """Free the solver (dest_ctqmc, CTQMC.F90:901)."""
    global _model, _batch
    if _batch is not None:
        _batch.close()
    if _model is not None:
        _model.close()
    _batch = _model = None
