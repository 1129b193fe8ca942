"""ctypes front-end of the oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It wraps oracle/cthyb_oracle.cpp, the CPU restatement of the
w2dynamics CT-HYB Z-space loop (src/ctqmc_fortran/CTQMC.F90 StepAdd /
StepRem / StepAdd4 / StepRem4 / StepGlob / StepShiftTau and the MTrace /
MMatrixUpdate routines they call; off-diagonal hybridisation for pair
moves).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

RECORD_DTYPE = np.dtype([
    ("move", "<i4"), ("outcome", "<i4"), ("orb", "<i4"), ("spin", "<i4"),
    ("change_outer", "<i4"), ("fpos_c", "<i4"), ("fpos_a", "<i4"),
    ("npairs", "<i4"), ("outer_sst", "<i4"), ("k_total", "<i4"),
    ("tau_c", "<f8"), ("tau_a", "<f8"), ("det_log", "<f8"), ("det_sign", "<f8"),
    ("tr_log", "<f8"), ("tr_sign", "<f8"), ("prob", "<f8"), ("rand", "<f8"),
])

OUTCOMES = {0: "equal_time", 1: "qn", 2: "no_pairs", 3: "reject", 4: "accept"}


class Params(C.Structure):
    _fields_ = [("beta", C.c_double), ("nftau", C.c_int32), ("ntau", C.c_int32),
                ("ncorr", C.c_int32), ("seed", C.c_int32), ("taudiff_max", C.c_double),
                ("p_global", C.c_double), ("p_shift", C.c_double), ("p_4op", C.c_double),
                ("p_outer", C.c_double), ("maxhisto", C.c_int32), ("meas_dm", C.c_int32),
                ("nleg", C.c_int32), ("nsym", C.c_int32), ("symmoves", C.POINTER(C.c_int32))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("build_oracle",
                                                      os.path.join(HERE, "build_oracle.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path, _ = mod.build()
        L = C.CDLL(path)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_last_error.restype = C.c_char_p
        L.orc_model_create.restype = vp
        L.orc_model_create.argtypes = [C.c_int, dp, dp, C.c_char_p]
        L.orc_model_destroy.argtypes = [vp]
        for n in ("orc_model_nsst", "orc_model_nstates", "orc_model_nsmax"):
            getattr(L, n).argtypes = [vp]
            getattr(L, n).restype = C.c_int
        L.orc_model_egs.argtypes = [vp]
        L.orc_model_egs.restype = C.c_double
        L.orc_model_sst.argtypes = [vp, ip, ip, ip, dp]
        L.orc_model_connect.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_model_psis_eb.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, dp, ip, ip]
        L.orc_model_evec.argtypes = [vp, C.c_int, dp]
        L.orc_chain_create.restype = vp
        L.orc_chain_create.argtypes = [vp, C.POINTER(Params), dp]
        L.orc_chain_create_full.restype = vp
        L.orc_chain_create_full.argtypes = [vp, C.POINTER(Params), dp]
        L.orc_chain_minv_full.argtypes = [vp, dp]
        L.orc_chain_results_full.argtypes = [vp, dp]
        L.orc_chain_gleg_full.argtypes = [vp, dp]
        L.orc_chain_destroy.argtypes = [vp]
        L.orc_chain_set_taudiffmax.argtypes = [vp, C.c_double]
        L.orc_chain_set_log.argtypes = [vp, C.c_void_p, C.c_longlong]
        L.orc_chain_log_count.argtypes = [vp]
        L.orc_chain_log_count.restype = C.c_longlong
        L.orc_chain_warmup.argtypes = [vp, C.c_longlong]
        L.orc_chain_measure.argtypes = [vp, C.c_longlong]
        L.orc_chain_results.argtypes = [vp, dp, dp, dp, dp]
        L.orc_chain_counters.argtypes = [vp, C.POINTER(C.c_longlong)]
        L.orc_chain_results_extra.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_chain_state.argtypes = [vp, dp]
        L.orc_chain_get_config.argtypes = [vp, dp, ip, ip, ip]
        L.orc_chain_set_config.argtypes = [vp, C.c_int, dp, ip, ip, ip, C.c_int]
        L.orc_chain_minv.argtypes = [vp, C.c_int, dp]
        L.orc_chain_full_trace.argtypes = [vp, dp]
        L.orc_chain_full_det.argtypes = [vp, dp]
        L.orc_rng_stream.argtypes = [C.c_uint, C.c_int, dp, C.c_int, C.c_int, C.c_int, ip]
        L.orc_mat_logdet_full.argtypes = [C.c_int, dp, dp]
        assert L.orc_record_size() == RECORD_DTYPE.itemsize
        assert L.orc_params_size() == C.sizeof(Params)
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Model:
    """Local problem: Fock space, superstates, H_loc eigenbasis, c/c+ blocks."""

    def __init__(self, nd, umatrix, muimp, quantum_numbers):
        L = lib()
        self.nd = nd
        u = np.asfortranarray(np.asarray(umatrix, dtype=np.float64).reshape((2 * nd,) * 4))
        mu = np.asfortranarray(np.asarray(muimp, dtype=np.float64).reshape(nd, 2, nd, 2))
        self._u, self._mu = u, mu
        h = L.orc_model_create(nd, _dp(u.ravel(order="F")), _dp(mu.ravel(order="F")),
                               quantum_numbers.encode())
        if not h:
            raise ValueError(L.orc_last_error().decode())
        self.h = h
        self.nsst = L.orc_model_nsst(h)
        self.nstates = L.orc_model_nstates(h)
        self.nsmax = L.orc_model_nsmax(h)
        self.egs = L.orc_model_egs(h)
        nst = np.zeros(self.nsst, np.int32)
        off = np.zeros(self.nsst, np.int32)
        states = np.zeros(self.nstates, np.int32)
        ev = np.zeros(self.nstates)
        L.orc_model_sst(h, _ip(nst), _ip(off), _ip(states), _dp(ev))
        self.sst_size, self.sst_offset, self.fock_states, self.evals = nst, off, states, ev

    def connect(self, sst, b, s, ca):
        """Target superstate of operator (b, s, ca) (0-based; ca 0=c+, 1=c)."""
        return lib().orc_model_connect(self.h, sst, b, s, ca)

    def psis_eb(self, sst, b, s, ca):
        r, c = C.c_int(), C.c_int()
        if lib().orc_model_psis_eb(self.h, sst, b, s, ca, None, C.byref(r), C.byref(c)) < 0:
            return None
        out = np.zeros(r.value * c.value)
        lib().orc_model_psis_eb(self.h, sst, b, s, ca, _dp(out), C.byref(r), C.byref(c))
        return out.reshape((r.value, c.value), order="F")

    def evec(self, sst):
        n = int(self.sst_size[sst])
        out = np.zeros(n * n)
        lib().orc_model_evec(self.h, sst, _dp(out))
        return out.reshape((n, n), order="F")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_model_destroy(self.h)
            self.h = None


class Chain:
    """One Markov chain of the restated reference loop."""

    def __init__(self, model, beta, ftau, ntau, seed, taudiff_max=-1.0, ncorr=100,
                 p_outer=0.0, maxhisto=500, meas_dm=1, p_global=0.0, p_shift=0.0, nleg=0,
                 symmoves=None, p_4op=0.0):
        """ftau: (Nd, 2, Nftau) diagonal F, or (Nd, 2, Nd, 2, Nftau) for the
        off-diagonal mode (offdiag = 1)."""
        L = lib()
        self.model = model
        nd = model.nd
        ftau = np.asarray(ftau, dtype=np.float64)
        self.offdiag = ftau.ndim == 5
        assert ftau.shape[:2] == (nd, 2) and (not self.offdiag or ftau.shape[2:4] == (nd, 2))
        self._ftau = np.asfortranarray(ftau)
        self.nftau = ftau.shape[-1]
        self.ntau = ntau
        self.maxhisto = maxhisto
        p = Params(beta=beta, nftau=self.nftau, ntau=ntau, ncorr=ncorr, seed=seed,
                   taudiff_max=taudiff_max, p_global=p_global, p_shift=p_shift, p_4op=p_4op,
                   p_outer=p_outer, maxhisto=maxhisto, meas_dm=meas_dm, nleg=nleg)
        self._sym = None
        if symmoves is not None:
            self._sym = np.ascontiguousarray(np.atleast_2d(symmoves), np.int32)
            p.nsym = self._sym.shape[0]
            p.symmoves = self._sym.ctypes.data_as(C.POINTER(C.c_int32))
        self.params = p
        create = L.orc_chain_create_full if self.offdiag else L.orc_chain_create
        self.h = create(model.h, C.byref(p), _dp(self._ftau.ravel(order="F")))
        if not self.h:
            raise RuntimeError(L.orc_last_error().decode())
        self._log = None

    def results_full(self):
        """Off-diagonal mode: G for every flavour pair, (2Nd, 2Nd, Ntau) with
        index [f_annihilator, f_creator], f = 2b + s (Gtau_full)."""
        nf = 2 * self.model.nd
        out = np.zeros(nf * nf * self.ntau)
        lib().orc_chain_results_full(self.h, _dp(out))
        return out.reshape(nf, nf, self.ntau)

    def gleg_full(self):
        """Off-diagonal mode: Legendre coefficients of G for every flavour
        pair, (2Nd, 2Nd, NLegMax), index [f_annihilator, f_creator, l]
        (GLeg_full)."""
        nf, nl = 2 * self.model.nd, self.params.nleg
        out = np.zeros(max(nf * nf * nl, 1))
        lib().orc_chain_gleg_full(self.h, _dp(out))
        return out[:nf * nf * nl].reshape(nf, nf, nl)

    def minv_full(self):
        """Off-diagonal mode: the inverse matrix over all flavours in block
        order (rows creators, columns annihilators)."""
        k = lib().orc_chain_minv_full(self.h, None)
        out = np.zeros(max(k, 1) ** 2)
        lib().orc_chain_minv_full(self.h, _dp(out))
        return out[:k * k].reshape((k, k), order="F")

    def set_taudiffmax(self, tdm):
        lib().orc_chain_set_taudiffmax(self.h, tdm)

    def start_log(self, cap):
        self._log = np.zeros(cap, RECORD_DTYPE)
        lib().orc_chain_set_log(self.h, self._log.ctypes.data, cap)

    def log(self):
        n = lib().orc_chain_log_count(self.h)
        return self._log[:min(n, len(self._log))].copy()

    def warmup(self, n):
        rc = lib().orc_chain_warmup(self.h, n)
        if rc:
            raise RuntimeError(f"oracle warmup returned {rc}")

    def measure(self, nmeas):
        rc = lib().orc_chain_measure(self.h, nmeas)
        if rc:
            raise RuntimeError(f"oracle measure returned {rc}")

    def results(self):
        nf = 2 * self.model.nd
        g = np.zeros(nf * self.ntau)
        ms = np.zeros(1)
        ns = self.model.nstates
        dm = np.zeros(ns * ns)
        hi = np.zeros(nf * self.maxhisto)
        lib().orc_chain_results(self.h, _dp(g), _dp(ms), _dp(dm), _dp(hi))
        return dict(gtau=g.reshape(nf, self.ntau), mean_sign=float(ms[0]),
                    densitymatrix=dm.reshape(ns, ns, order="F"),
                    histo=hi.reshape(nf, self.maxhisto))

    def results_extra(self):
        nf, ns, nss = 2 * self.model.nd, self.model.nstates, len(self.model.sst_size)
        nleg = self.params.nleg
        gl = np.zeros(max(1, nf * nleg))
        arrs = [np.zeros(nss), np.zeros(ns), np.zeros(nss), np.zeros(ns), np.zeros(nss), np.zeros(ns)]
        lib().orc_chain_results_extra(self.h, _dp(gl), *[_dp(a) for a in arrs])
        keys = ("outer_sst_histo", "outer_state_histo", "sign_sst", "sign_state", "contrib_sst",
                "contrib_state")
        out = dict(zip(keys, arrs))
        out["gleg"] = gl[:nf * nleg].reshape(nf, nleg)
        return out

    def counters(self):
        out = (C.c_longlong * 16)()
        lib().orc_chain_counters(self.h, out)
        return dict(zip(("try_add", "acc_add", "try_rem", "acc_rem", "qn_add", "qn_rem",
                         "cnt_meas", "try_glob", "acc_glob", "qn_glob", "try_shift",
                         "acc_shift", "try_add4", "acc_add4", "try_rem4", "acc_rem4"), list(out)))

    def state(self):
        out = np.zeros(14)
        lib().orc_chain_state(self.h, _dp(out))
        keys = ("trace_log", "trace_sign", "det_log", "det_sign", "cfgsign", "npairs",
                "outer_sst", "window_position", "num_windows", "noper", "tauwin_min",
                "tauwin_max", "taudiff_max", "nslide")
        return dict(zip(keys, out.tolist()))

    def get_config(self):
        n = int(self.state()["noper"])
        t = np.zeros(max(n, 1))
        o = np.zeros(max(n, 1), np.int32)
        s = np.zeros(max(n, 1), np.int32)
        c = np.zeros(max(n, 1), np.int32)
        lib().orc_chain_get_config(self.h, _dp(t), _ip(o), _ip(s), _ip(c))
        return t[:n], o[:n], s[:n], c[:n]

    def set_config(self, taus, orbs, spins, cas, outer_sst):
        t = np.ascontiguousarray(taus, np.float64)
        o = np.ascontiguousarray(orbs, np.int32)
        s = np.ascontiguousarray(spins, np.int32)
        c = np.ascontiguousarray(cas, np.int32)
        rc = lib().orc_chain_set_config(self.h, len(t), _dp(t), _ip(o), _ip(s), _ip(c),
                                        int(outer_sst))
        if rc:
            raise ValueError(lib().orc_last_error().decode())

    def minv(self, f):
        k = lib().orc_chain_minv(self.h, f, None)
        out = np.zeros(k * k)
        lib().orc_chain_minv(self.h, f, _dp(out))
        return out.reshape((k, k), order="F")

    def full_trace(self):
        out = np.zeros(2)
        lib().orc_chain_full_trace(self.h, _dp(out))
        return out

    def full_det(self):
        out = np.zeros(2)
        lib().orc_chain_full_det(self.h, _dp(out))
        return out

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_chain_destroy(self.h)
            self.h = None


def rng_stream(seed, n, nint, lo, hi):
    reals = np.zeros(n)
    ints = np.zeros(nint, np.int32)
    lib().orc_rng_stream(seed, n, _dp(reals), nint, lo, hi, _ip(ints))
    return reals, ints


def mat_logdet_full(mat):
    """get_MatLogDetFull: (log|det|, sign, inverse or None when singular)."""
    a = np.array(mat, np.float64, order="F", copy=True)
    k = a.shape[0]
    out = np.zeros(2)
    flat = a.ravel(order="F").copy()
    sing = lib().orc_mat_logdet_full(k, _dp(flat), _dp(out))
    inv = None if sing else flat.reshape((k, k), order="F")
    return out[0], out[1], inv
