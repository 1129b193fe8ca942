"""ctypes bindings of the GB300 CT-HYB engine (include/cthyb_gpu.h).

The shared library is built in-tree by w2dynamics_gb300.build; there is no
CPU fallback: if it is missing or no GPU is present, every entry point
raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

RECORD_DTYPE = np.dtype([
    ("move", "<i4"), ("outcome", "<i4"), ("orb", "<i4"), ("spin", "<i4"),
    ("change_outer", "<i4"), ("fpos_c", "<i4"), ("fpos_a", "<i4"),
    ("npairs", "<i4"), ("outer_sst", "<i4"), ("k_total", "<i4"),
    ("tau_c", "<f8"), ("tau_a", "<f8"), ("det_log", "<f8"), ("det_sign", "<f8"),
    ("tr_log", "<f8"), ("tr_sign", "<f8"), ("prob", "<f8"), ("rand", "<f8"),
])

FLAG_DENSE = 1
FLAG_NO_DM = 2
FLAG_DMMA = 4
FLAG_ACCPAIR = 8

EXPORTS = (
    "cthyb_last_error", "cthyb_model_create", "cthyb_model_destroy", "cthyb_model_info",
    "cthyb_model_states", "cthyb_model_basis", "cthyb_model_connect", "cthyb_model_set_directions", "cthyb_batch_create",
    "cthyb_batch_destroy",
    "cthyb_batch_nchains", "cthyb_batch_set_taudiffmax", "cthyb_batch_warmup",
    "cthyb_batch_measure", "cthyb_batch_reset_measurements", "cthyb_batch_sync",
    "cthyb_batch_stream", "cthyb_batch_use_graphs", "cthyb_batch_set_schedule", "cthyb_batch_set_team", "cthyb_batch_autotune", "cthyb_batch_results",
    "cthyb_batch_group_sums", "cthyb_batch_move_counters", "cthyb_batch_move_counters4", "cthyb_batch_results_full", "cthyb_batch_results_gleg_full", "cthyb_batch_results_accpair", "cthyb_batch_minv_full", "cthyb_batch_results_extra", "cthyb_batch_gradients", "cthyb_batch_gradients_device", "cthyb_batch_results_score", "cthyb_batch_state", "cthyb_batch_get_config",
    "cthyb_batch_set_config", "cthyb_batch_set_configs", "cthyb_batch_get_configs", "cthyb_batch_minv", "cthyb_batch_refresh_minv",
    "cthyb_batch_set_log", "cthyb_batch_get_log", "cthyb_batch_work_counters",
    "cthyb_batch_drift", "cthyb_batch_chain_stats", "cthyb_batch_group_gtau_raw", "cthyb_probe_fp64", "cthyb_batch_log_weights_device",
    "cthyb_minv_rebuild_noalloc",
)


class GroupDesc(C.Structure):
    _fields_ = [("beta", C.c_double), ("nftau", C.c_int32), ("ntau", C.c_int32),
                ("ftau", C.POINTER(C.c_double)), ("nchains", C.c_int32), ("seed0", C.c_int32),
                ("seeds", C.POINTER(C.c_int32)), ("taudiff_max", C.c_double),
                ("ncorr", C.c_int32), ("p_outer", C.c_double), ("kcap", C.c_int32),
                ("opcap", C.c_int32), ("tree_levels", C.c_int32), ("maxhisto", C.c_int32),
                ("flags", C.c_int32), ("p_global", C.c_double), ("p_shift", C.c_double),
                ("nleg", C.c_int32), ("nscore", C.c_int32), ("score_dE", C.POINTER(C.c_double)),
                ("nsym", C.c_int32), ("symmoves", C.POINTER(C.c_int32)), ("p_4op", C.c_double),
                ("ftau_full", C.POINTER(C.c_double)), ("refresh_every", C.c_int32)]


class EngineError(RuntimeError):
    pass


_lib = None


def library_path():
    return os.environ.get("CTHYB_GPU_LIB", _build.LIB)


def load(build_if_missing=False):
    """Load libcthyb_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_missing and path == _build.LIB:
        _build.build()
    if not os.path.exists(path):
        raise EngineError(f"{path} not built: run `python -m w2dynamics_gb300.build`")
    L = C.CDLL(path)
    vp, dp, ip, i64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int64
    L.cthyb_last_error.restype = C.c_char_p
    L.cthyb_model_create.argtypes = [C.c_int, dp, dp, C.c_char_p, C.POINTER(vp)]
    L.cthyb_model_destroy.argtypes = [vp]
    L.cthyb_model_info.argtypes = [vp, ip, ip, ip, ip, dp]
    L.cthyb_model_states.argtypes = [vp, ip, ip, ip, dp]
    L.cthyb_model_connect.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.cthyb_model_basis.argtypes = [vp, ip, dp]
    L.cthyb_model_set_directions.argtypes = [vp, C.c_int, dp, dp]
    L.cthyb_batch_create.argtypes = [vp, C.c_int, C.POINTER(GroupDesc), C.POINTER(vp)]
    L.cthyb_batch_destroy.argtypes = [vp]
    L.cthyb_batch_nchains.argtypes = [vp]
    L.cthyb_batch_set_taudiffmax.argtypes = [vp, C.c_int, C.c_double]
    L.cthyb_batch_warmup.argtypes = [vp, i64]
    L.cthyb_batch_measure.argtypes = [vp, i64]
    L.cthyb_batch_reset_measurements.argtypes = [vp]
    L.cthyb_batch_sync.argtypes = [vp]
    L.cthyb_batch_stream.argtypes = [vp, C.POINTER(vp)]
    L.cthyb_batch_use_graphs.argtypes = [vp, C.c_int]
    L.cthyb_batch_set_schedule.argtypes = [vp, C.c_int]
    L.cthyb_batch_set_team.argtypes = [vp, C.c_int, C.c_int]
    L.cthyb_batch_autotune.argtypes = [vp, i64, C.POINTER(C.c_int)]
    L.cthyb_batch_results.argtypes = [vp, C.c_int, dp, dp, dp, dp, C.POINTER(i64)]
    L.cthyb_batch_move_counters.argtypes = [vp, C.c_int, C.POINTER(i64)]
    L.cthyb_batch_move_counters4.argtypes = [vp, C.c_int, C.POINTER(i64)]
    L.cthyb_batch_results_full.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_minv_full.argtypes = [vp, C.c_int, ip, dp]
    L.cthyb_batch_results_gleg_full.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_results_accpair.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_results_extra.argtypes = [vp, C.c_int, dp, dp, dp, dp, dp, dp, dp]
    L.cthyb_batch_gradients.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    L.cthyb_batch_results_score.argtypes = [vp, C.c_int, dp, dp]
    L.cthyb_batch_gradients_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    L.cthyb_batch_group_sums.argtypes = [vp, C.c_int, dp, dp, C.POINTER(i64)]
    L.cthyb_batch_state.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_get_config.argtypes = [vp, C.c_int, ip, dp, ip, ip, ip, ip]
    L.cthyb_batch_set_config.argtypes = [vp, C.c_int, C.c_int, dp, ip, ip, ip, C.c_int]
    L.cthyb_batch_set_configs.argtypes = [vp, C.c_int, C.c_int, ip, dp, ip, ip, ip, ip]
    L.cthyb_batch_get_configs.argtypes = [vp, C.c_int, C.c_int, ip, C.c_int, dp, ip, ip, ip, ip]
    L.cthyb_batch_minv.argtypes = [vp, C.c_int, C.c_int, ip, dp]
    L.cthyb_batch_refresh_minv.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_set_log.argtypes = [vp, i64]
    L.cthyb_batch_get_log.argtypes = [vp, C.c_int, C.c_void_p, C.POINTER(i64)]
    L.cthyb_batch_work_counters.argtypes = [vp, C.POINTER(i64), C.c_int]
    L.cthyb_probe_fp64.argtypes = [dp, dp]
    L.cthyb_batch_log_weights_device.argtypes = [vp, vp, vp]
    L.cthyb_batch_chain_stats.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_group_gtau_raw.argtypes = [vp, C.c_int, dp]
    L.cthyb_batch_drift.argtypes = [vp, dp, dp, C.POINTER(i64), C.POINTER(i64), C.c_int]
    L.cthyb_minv_rebuild_noalloc.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_double, vp, vp, vp]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise EngineError(f"cthyb error {rc}: {load().cthyb_last_error().decode()}")


def probe_fp64():
    """(DFMA, DMMA) FP64 GFLOP/s of the running device."""
    a, b = C.c_double(), C.c_double()
    _check(load().cthyb_probe_fp64(C.byref(a), C.byref(b)))
    return a.value, b.value


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Model:
    """Local problem on the device (cthyb_model_create)."""

    def __init__(self, nd, umatrix, muimp, quantum_numbers):
        L = load()
        self.nd = nd
        self._u = np.asfortranarray(np.asarray(umatrix, np.float64).reshape((2 * nd,) * 4))
        self._mu = np.asfortranarray(np.asarray(muimp, np.float64).reshape(nd, 2, nd, 2))
        h = C.c_void_p()
        _check(L.cthyb_model_create(nd, _dp(self._u.ravel(order="F")),
                                    _dp(self._mu.ravel(order="F")),
                                    quantum_numbers.encode(), C.byref(h)))
        self.h = h
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        e = C.c_double()
        _check(L.cthyb_model_info(h, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(e)))
        self.nsst, self.nstates, self.nsmax, self.monomial, self.egs = (
            a.value, b.value, c.value, d.value, e.value)
        n = np.zeros(self.nsst, np.int32)
        o = np.zeros(self.nsst, np.int32)
        fk = np.zeros(self.nstates, np.int32)
        ev = np.zeros(self.nstates)
        _check(L.cthyb_model_states(h, _ip(n), _ip(o), _ip(fk), _dp(ev)))
        self.sst_size, self.sst_offset, self.fock_states, self.evals = n, o, fk, ev

    def connect(self, sst, b, s, ca):
        return load().cthyb_model_connect(self.h, sst, b, s, ca)

    def basis(self):
        """(occ_fock, evec): Fock state of each occupation-basis vector in
        superstate order and the block-diagonal eigenvector matrix."""
        fk = np.zeros(self.nstates, np.int32)
        ev = np.zeros(self.nstates * self.nstates)
        _check(load().cthyb_model_basis(self.h, _ip(fk), _dp(ev)))
        return fk, ev.reshape((self.nstates, self.nstates), order="F")

    def set_directions(self, dumatrix=None, dmuimp=None):
        """Hamiltonian directions for the trace gradients of dense-block
        models: dumatrix (nparams, 2Nd, 2Nd, 2Nd, 2Nd) and/or dmuimp
        (nparams, Nd, 2, Nd, 2), dH/dtheta_p in the operator strings of
        H_loc."""
        nd, nf = self.nd, 2 * self.nd
        n = len(dumatrix) if dumatrix is not None else len(dmuimp)
        du = None if dumatrix is None else np.concatenate(
            [np.asfortranarray(np.asarray(u, np.float64).reshape((nf,) * 4)).ravel(order="F") for u in dumatrix])
        dm = None if dmuimp is None else np.concatenate(
            [np.asfortranarray(np.asarray(x, np.float64).reshape(nd, 2, nd, 2)).ravel(order="F") for x in dmuimp])
        _check(load().cthyb_model_set_directions(self.h, n, _dp(du) if du is not None else None,
                                                 _dp(dm) if dm is not None else None))
        self.ndir = n

    def close(self):
        if getattr(self, "h", None):
            load().cthyb_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Group:
    """Parameters of one group of chains (one beta / one F(tau))."""

    def __init__(self, beta, ftau, ntau, nchains=1, seed0=0, seeds=None, taudiff_max=-1.0,
                 ncorr=100, p_outer=0.0, kcap=0, opcap=0, tree_levels=0, maxhisto=500,
                 dense=False, measure_dm=True, p_global=0.0, p_shift=0.0, nleg=0, score_dE=None,
                 symmoves=None, p_4op=0.0, ftau_full=None, refresh_every=0, dmma=False, measure_accpair=False):
        self.beta = float(beta)
        self.ftau = np.asfortranarray(np.asarray(ftau, np.float64))
        self.ntau = int(ntau)
        self.nchains = int(nchains)
        self.seed0 = int(seed0)
        self.seeds = None if seeds is None else np.ascontiguousarray(seeds, np.int32)
        self.taudiff_max = float(taudiff_max)
        self.ncorr = int(ncorr)
        self.p_outer = float(p_outer)
        self.p_global, self.p_shift = float(p_global), float(p_shift)
        self.p_4op = float(p_4op)
        # off-diagonal hybridisation: F for every flavour pair (Nd,2,Nd,2,Nftau)
        self.ftau_full = None if ftau_full is None else np.asfortranarray(np.asarray(ftau_full, np.float64))
        self.nleg = int(nleg)
        self.score_dE = None if score_dE is None else np.ascontiguousarray(score_dE, np.float64)
        # user symmetry moves: rows of 1-based target flavours in the reference's
        # flavour order (b-1) + Nd*(s-1) + 1
        self.symmoves = None if symmoves is None else np.ascontiguousarray(np.atleast_2d(symmoves), np.int32)
        self.kcap, self.opcap, self.tree_levels = int(kcap), int(opcap), int(tree_levels)
        self.maxhisto = int(maxhisto)
        self.flags = ((FLAG_DENSE if dense else 0) | (0 if measure_dm else FLAG_NO_DM) | (FLAG_DMMA if dmma else 0)
                      | (FLAG_ACCPAIR if measure_accpair else 0))
        # accepted pair updates between full rebuilds of the inverse matrices
        # (0: the library default, negative: never)
        self.refresh_every = int(refresh_every)

    def desc(self):
        d = GroupDesc()
        d.beta = self.beta
        d.nftau = self.ftau.shape[2]
        d.ntau = self.ntau
        self._fl = self.ftau.ravel(order="F")
        d.ftau = _dp(self._fl)
        d.nchains = self.nchains
        d.seed0 = self.seed0
        d.seeds = self.seeds.ctypes.data_as(C.POINTER(C.c_int32)) if self.seeds is not None else None
        d.taudiff_max = self.taudiff_max
        d.ncorr = self.ncorr
        d.p_outer = self.p_outer
        d.kcap, d.opcap, d.tree_levels = self.kcap, self.opcap, self.tree_levels
        d.maxhisto = self.maxhisto
        d.flags = self.flags
        d.p_global, d.p_shift = self.p_global, self.p_shift
        d.p_4op = self.p_4op
        if self.ftau_full is not None:
            self._ffl = self.ftau_full.ravel(order="F")
            d.ftau_full = _dp(self._ffl)
        else:
            d.ftau_full = None
        d.nleg = self.nleg
        d.nscore = 0 if self.score_dE is None else self.score_dE.shape[0]
        d.score_dE = _dp(self.score_dE) if self.score_dE is not None else None
        d.refresh_every = self.refresh_every
        d.nsym = 0 if self.symmoves is None else self.symmoves.shape[0]
        d.symmoves = self.symmoves.ctypes.data_as(C.POINTER(C.c_int32)) if self.symmoves is not None else None
        return d


class Batch:
    """A batch of independent chains (one chain = the plain drop-in form)."""

    def __init__(self, model, groups):
        L = load()
        self.model = model
        self.groups = list(groups)
        descs = (GroupDesc * len(self.groups))(*[g.desc() for g in self.groups])
        h = C.c_void_p()
        _check(L.cthyb_batch_create(model.h, len(self.groups), descs, C.byref(h)))
        self.h = h
        self.nchains = L.cthyb_batch_nchains(h)
        self._group_of = []
        for gi, g in enumerate(self.groups):
            self._group_of += [gi] * g.nchains

    # --- loop entry points
    def set_taudiffmax(self, group, tdm):
        _check(load().cthyb_batch_set_taudiffmax(self.h, group, tdm))

    def warmup(self, n):
        _check(load().cthyb_batch_warmup(self.h, int(n)))

    def measure(self, nmeas):
        _check(load().cthyb_batch_measure(self.h, int(nmeas)))

    def reset_measurements(self):
        _check(load().cthyb_batch_reset_measurements(self.h))

    def sync(self):
        _check(load().cthyb_batch_sync(self.h))

    def stream(self):
        s = C.c_void_p()
        _check(load().cthyb_batch_stream(self.h, C.byref(s)))
        return s.value

    def use_graphs(self, on=True):
        _check(load().cthyb_batch_use_graphs(self.h, 1 if on else 0))

    def set_schedule(self, warps_per_block):
        """-1: automatic; 0: independent warps; n (1..32): phase-synchronous blocks of n chains."""
        _check(load().cthyb_batch_set_schedule(self.h, int(warps_per_block)))

    def set_team(self, warps_per_chain, blocks_per_sm=0):
        """0: off; T (1..16): team sweep, blocks of T warps per chain taken
        from a cost-ordered queue (the warps share the dense-block trace);
        blocks_per_sm bounds the resident blocks (0: as many as fit)."""
        _check(load().cthyb_batch_set_team(self.h, int(warps_per_chain), int(blocks_per_sm)))

    def autotune(self, nprop):
        """Pick the fastest schedule on `nprop` warmup proposals per candidate;
        returns the chosen warps per block (0: independent warps) or
        100 + T + 1000 x blocks_per_sm for a team sweep of T warps per chain."""
        best = C.c_int()
        _check(load().cthyb_batch_autotune(self.h, int(nprop), C.byref(best)))
        return best.value

    # --- results
    def results(self, chain):
        g = self.groups[self._group_of[chain]]
        nd, ns = self.model.nd, self.model.nstates
        gt = np.zeros(nd * 2 * g.ntau)
        ms = np.zeros(1)
        dm = np.zeros(ns * ns)
        hi = np.zeros(nd * 2 * g.maxhisto)
        cnt = np.zeros(8, np.int64)
        _check(load().cthyb_batch_results(self.h, chain, _dp(gt), _dp(ms), _dp(dm), _dp(hi),
                                          cnt.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(gtau=gt.reshape((nd, 2, g.ntau), order="F"), mean_sign=float(ms[0]),
                    densitymatrix=dm.reshape((ns, ns), order="F"),
                    histo=hi.reshape((nd, 2, g.maxhisto), order="F"),
                    counters=dict(zip(("try_add", "acc_add", "try_rem", "acc_rem", "qn_add",
                                       "qn_rem", "cnt_meas", "proposals"), cnt.tolist())))

    def results_extra(self, chain):
        """Legendre G_l (Nd,2,nleg) and the outer superstate/state histograms."""
        g = self.groups[self._group_of[chain]]
        nd, ns, nss = self.model.nd, self.model.nstates, self.model.nsst
        gl = np.zeros(max(1, nd * 2 * g.nleg))
        arrs = [np.zeros(nss), np.zeros(ns), np.zeros(nss), np.zeros(ns), np.zeros(nss), np.zeros(ns)]
        _check(load().cthyb_batch_results_extra(self.h, chain, _dp(gl), *[_dp(a) for a in arrs]))
        keys = ("outer_sst_histo", "outer_state_histo", "sign_sst", "sign_state", "contrib_sst",
                "contrib_state")
        out = dict(zip(keys, arrs))
        out["gleg"] = gl[:nd * 2 * g.nleg].reshape((nd, 2, g.nleg), order="F")
        return out

    def gradients_device(self, dE_dev, grad_delta, grad_params, log_weights, stream=None):
        """Device-memory form of `gradients` (torch CUDA tensors or raw
        pointers): grad_delta (nchains, 2Nd, Nftau), grad_params (nchains,
        nparams), log_weights (nchains, 2); enqueued, not synchronised."""
        ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr() if hasattr(t, "data_ptr") else int(t))
        npar = getattr(self.model, "ndir", 0) if dE_dev is None else int(dE_dev.shape[0])
        _check(load().cthyb_batch_gradients_device(self.h, npar, ptr(dE_dev), ptr(grad_delta), ptr(grad_params),
                                                   ptr(log_weights), C.c_void_p(stream) if stream else None))

    def log_weights_device(self, out, stream=None):
        """log|det| and absolute log|trace| of every chain, (nchains, 2)
        into a device tensor (or raw pointer); enqueued, not synchronised."""
        ptr = C.c_void_p(out.data_ptr() if hasattr(out, "data_ptr") else int(out))
        _check(load().cthyb_batch_log_weights_device(self.h, ptr, C.c_void_p(stream) if stream else None))

    def results_score(self, chain):
        """Score-function dG(tau)/dtheta (nscore, Nd, 2, Ntau) and <g> (nscore)."""
        g = self.groups[self._group_of[chain]]
        nd, ns = self.model.nd, g.score_dE.shape[0]
        dg = np.zeros(ns * nd * 2 * g.ntau)
        ms = np.zeros(ns)
        _check(load().cthyb_batch_results_score(self.h, chain, _dp(dg), _dp(ms)))
        return dg.reshape((ns, g.ntau, 2, nd)).transpose(0, 3, 2, 1), ms

    def gradients(self, dE=None):
        """d log|w| of every chain's current configuration: grad_delta
        (nchains, Nd, 2, Nftau) w.r.t. the F(tau) grid, grad_params
        (nchains, nparams) along the parameter directions dE (nparams,
        nstates), log_weights (nchains, 2) = (log|det|, log|trace|)."""
        nd = self.model.nd
        nft = self.groups[0].ftau.shape[2]
        if any(g.ftau.shape[2] != nft for g in self.groups):
            raise ValueError("gradients need one Nftau for all groups")
        # dense-block models: dE None, the directions set on the model
        npar = getattr(self.model, "ndir", 0) if dE is None else int(np.asarray(dE).shape[0])
        dEc = None if dE is None else np.ascontiguousarray(dE, np.float64)
        gd = np.zeros((self.nchains, nd * 2 * nft))
        gp = np.zeros((self.nchains, max(npar, 1)))
        lw = np.zeros((self.nchains, 2))
        _check(load().cthyb_batch_gradients(self.h, npar, _dp(dEc) if dEc is not None else None, _dp(gd),
                                            _dp(gp), _dp(lw)))
        gd = gd.reshape((self.nchains, nft, 2, nd)).transpose(0, 3, 2, 1)
        return gd, gp[:, :npar], lw

    def move_counters(self, chain):
        """Global, tau-shift and 4-operator move counters since the last
        warmup/measure call."""
        out = np.zeros(5, np.int64)
        _check(load().cthyb_batch_move_counters(self.h, chain, out.ctypes.data_as(C.POINTER(C.c_int64))))
        d = dict(zip(("try_glob", "acc_glob", "qn_glob", "try_shift", "acc_shift"), out.tolist()))
        out4 = np.zeros(4, np.int64)
        _check(load().cthyb_batch_move_counters4(self.h, chain, out4.ctypes.data_as(C.POINTER(C.c_int64))))
        d.update(zip(("try_add4", "acc_add4", "try_rem4", "acc_rem4"), out4.tolist()))
        return d

    def group_sums(self, group):
        g = self.groups[group]
        nd = self.model.nd
        gs = np.zeros(nd * 2 * g.ntau)
        ss = np.zeros(1)
        cn = np.zeros(1, np.int64)
        _check(load().cthyb_batch_group_sums(self.h, group, _dp(gs), _dp(ss),
                                             cn.ctypes.data_as(C.POINTER(C.c_int64))))
        return gs.reshape((nd, 2, g.ntau), order="F"), float(ss[0]), int(cn[0])

    def state(self, chain):
        out = np.zeros(16)
        _check(load().cthyb_batch_state(self.h, chain, _dp(out)))
        keys = ("trace_log", "trace_sign", "det_log", "det_sign", "cfgsign", "npairs",
                "outer_sst", "window_position", "num_windows", "noper", "tauwin_min",
                "tauwin_max", "taudiff_max", "nslide", "status", "k0")
        return dict(zip(keys, out.tolist()))

    def get_config(self, chain):
        g = self.groups[self._group_of[chain]]
        cap = max(1, int(self.state(chain)["noper"]))
        t = np.zeros(cap)
        o = np.zeros(cap, np.int32)
        s = np.zeros(cap, np.int32)
        c = np.zeros(cap, np.int32)
        n = C.c_int()
        out = C.c_int()
        _check(load().cthyb_batch_get_config(self.h, chain, C.byref(n), _dp(t), _ip(o), _ip(s),
                                             _ip(c), C.byref(out)))
        k = n.value
        return t[:k], o[:k], s[:k], c[:k], out.value

    def set_config(self, chain, taus, orbs, spins, cas, outer_sst):
        t = np.ascontiguousarray(taus, np.float64)
        o = np.ascontiguousarray(orbs, np.int32)
        s = np.ascontiguousarray(spins, np.int32)
        c = np.ascontiguousarray(cas, np.int32)
        _check(load().cthyb_batch_set_config(self.h, chain, len(t), _dp(t), _ip(o), _ip(s),
                                             _ip(c), int(outer_sst)))

    def get_configs(self, chain0=0, n=None):
        """Configurations of chains chain0 .. chain0 + n - 1 in one call:
        (offsets, taus, orbs, spins, cas, outer_sst) with chain chain0 + i's
        operators at offsets[i] .. offsets[i + 1] - 1 (1-based orbitals,
        spins and creator/annihilator flags as get_mc_config)."""
        n = self.nchains - chain0 if n is None else int(n)
        offs = np.zeros(n + 1, np.int32)
        outer = np.zeros(max(n, 1), np.int32)
        _check(load().cthyb_batch_get_configs(self.h, chain0, n, _ip(offs), 0, None, None, None, None,
                                              _ip(outer)))
        nop = int(offs[-1])
        t = np.zeros(max(nop, 1))
        o, s, c = (np.zeros(max(nop, 1), np.int32) for _ in range(3))
        _check(load().cthyb_batch_get_configs(self.h, chain0, n, _ip(offs), len(t), _dp(t), _ip(o),
                                              _ip(s), _ip(c), _ip(outer)))
        return offs, t[:nop], o[:nop], s[:nop], c[:nop], outer[:n]

    def set_configs(self, offsets, taus, orbs, spins, cas, outer_sst, chain0=0):
        """set_mc_config of chains chain0 .. chain0 + len(outer_sst) - 1 in
        one call, in the layout get_configs returns."""
        offs = np.ascontiguousarray(offsets, np.int32)
        outer = np.ascontiguousarray(outer_sst, np.int32)
        if len(offs) != len(outer) + 1:
            raise ValueError("offsets must have one entry more than outer_sst")
        t = np.ascontiguousarray(taus, np.float64)
        o, s, c = (np.ascontiguousarray(a, np.int32) for a in (orbs, spins, cas))
        _check(load().cthyb_batch_set_configs(self.h, chain0, len(outer), _ip(offs), _dp(t), _ip(o),
                                              _ip(s), _ip(c), _ip(outer)))

    def results_full(self, chain):
        """Off-diagonal groups: G for every flavour pair, (2Nd, 2Nd, Ntau)
        indexed [f_annihilator, f_creator, bin] with f = 2b + s."""
        g = self.groups[self._group_of[chain]]
        nf = 2 * self.model.nd
        out = np.zeros(nf * nf * g.ntau)
        _check(load().cthyb_batch_results_full(self.h, chain, _dp(out)))
        return out.reshape(nf, nf, g.ntau)

    def results_accpair(self, chain):
        """Accepted pair moves by flavour and time difference, (Nd, 2, Ntau)
        (groups built with measure_accpair=True)."""
        g = self.groups[self._group_of[chain]]
        nd = self.model.nd
        out = np.zeros(nd * 2 * g.ntau)
        _check(load().cthyb_batch_results_accpair(self.h, chain, _dp(out)))
        return out.reshape((nd, 2, g.ntau), order="F")

    def results_gleg_full(self, chain):
        """Off-diagonal groups: Legendre coefficients of G for every flavour
        pair, (2Nd, 2Nd, nleg) indexed [f_annihilator, f_creator, l]."""
        g = self.groups[self._group_of[chain]]
        nf = 2 * self.model.nd
        out = np.zeros(max(1, nf * nf * g.nleg))
        _check(load().cthyb_batch_results_gleg_full(self.h, chain, _dp(out)))
        return out[:nf * nf * g.nleg].reshape(nf, nf, g.nleg)

    def minv_full(self, chain):
        """Off-diagonal groups: the inverse matrix over all flavours in block
        order (rows creators, columns annihilators)."""
        k = C.c_int()
        _check(load().cthyb_batch_minv_full(self.h, chain, C.byref(k), None))
        out = np.zeros(max(k.value, 1) ** 2)
        _check(load().cthyb_batch_minv_full(self.h, chain, C.byref(k), _dp(out)))
        return out[:k.value ** 2].reshape((k.value, k.value), order="F")

    def minv(self, chain, f):
        k = C.c_int()
        _check(load().cthyb_batch_minv(self.h, chain, f, C.byref(k), None))
        out = np.zeros(max(k.value, 1) ** 2)
        _check(load().cthyb_batch_minv(self.h, chain, f, C.byref(k), _dp(out)))
        return out[:k.value ** 2].reshape((k.value, k.value), order="F")

    def refresh_minv(self, replace=False):
        d = np.zeros(1)
        _check(load().cthyb_batch_refresh_minv(self.h, 1 if replace else 0, _dp(d)))
        return float(d[0])

    def chain_stats(self, group):
        """Per chain of a group: operators, measurements, sign sum and
        proposals since the last warmup/measure call (one copy)."""
        g = self.groups[group]
        out = np.zeros(4 * g.nchains)
        _check(load().cthyb_batch_chain_stats(self.h, group, _dp(out)))
        out = out.reshape(g.nchains, 4)
        return dict(noper=out[:, 0].astype(np.int64), cnt_meas=out[:, 1].astype(np.int64),
                    sign_sum=out[:, 2], proposals=out[:, 3].astype(np.int64))

    def group_gtau(self, group):
        """G(tau) of every chain of a group, normalised as results():
        (nchains, Nd, 2, Ntau); chains without measurements give zeros."""
        g = self.groups[group]
        nd, nt = self.model.nd, g.ntau
        raw = np.zeros(g.nchains * 2 * nd * nt)
        _check(load().cthyb_batch_group_gtau_raw(self.h, group, _dp(raw)))
        raw = raw.reshape(g.nchains, nd, 2, nt)  # f = 2b + s is (b, s) in C order
        st = self.chain_stats(group)
        cnt = st["cnt_meas"].astype(np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            ms = np.where(cnt > 0, st["sign_sum"] / cnt, 0.0)
            fac = np.where(cnt > 0, 1.0 / (cnt * ms), 0.0) * nt / (g.beta * g.beta)
        return raw * fac[:, None, None, None]

    def drift(self, reset=False):
        """Drift of the fast updates at the periodic rebuilds of M, over all
        chains: max |M_fast - M_rebuilt|, max |log|det| fast - rebuilt|,
        number of rebuilds and of determinant-sign disagreements."""
        dm, dd = np.zeros(1), np.zeros(1)
        n, se = np.zeros(1, np.int64), np.zeros(1, np.int64)
        _check(load().cthyb_batch_drift(self.h, _dp(dm), _dp(dd), n.ctypes.data_as(C.POINTER(C.c_int64)),
                                        se.ctypes.data_as(C.POINTER(C.c_int64)), 1 if reset else 0))
        return dict(max_dev_m=float(dm[0]), max_dev_logdet=float(dd[0]), refreshes=int(n[0]),
                    sign_errors=int(se[0]))

    def set_log(self, cap):
        _check(load().cthyb_batch_set_log(self.h, int(cap)))
        self._logcap = int(cap)

    def log(self, chain):
        n = C.c_int64()
        _check(load().cthyb_batch_get_log(self.h, chain, None, C.byref(n)))
        m = min(n.value, self._logcap)
        rec = np.zeros(m, RECORD_DTYPE)
        if m:
            _check(load().cthyb_batch_get_log(self.h, chain, rec.ctypes.data, C.byref(n)))
        return rec

    def work_counters(self, reset=False):
        out = np.zeros(8, np.int64)
        _check(load().cthyb_batch_work_counters(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)),
                                                1 if reset else 0))
        return dict(zip(("m_bytes", "m_flops", "op_bytes", "tree_nodes", "proposals",
                         "accepted", "trace_flops", "trace_bytes"), out.tolist()))

    def close(self):
        if getattr(self, "h", None):
            load().cthyb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
