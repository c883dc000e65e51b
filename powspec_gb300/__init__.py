"""powspec_gb300 -- GB300 (sm_103a) periodic-box P_l(k) estimator.

Python view of the C ABI in ``include/powspec_gpu.h`` (libpowspec_gpu.so),
used by the tests and the benchmark.  The estimator itself runs entirely in
the CUDA library; there is no CPU fallback: loading fails loudly when the
library is missing, and every call fails when no GPU is usable.

The two reference entry points map onto one context:

* ``genr_mesh(conf, cat)``   (src/genr_mesh.c:874) -> ``Estimator.assign``
* ``powspec(conf, cat, mesh)`` (src/multipole.c:1179) -> ``Estimator.execute``
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpowspec_gpu.so")

# status codes (include/powspec_gpu.h)
ERRORS = {
    -1: "PS_GPU_ERR_MEMORY", -2: "PS_GPU_ERR_ARG", -11: "PS_GPU_ERR_CATA",
    -13: "PS_GPU_ERR_MESH", -14: "PS_GPU_ERR_PK", -20: "PS_GPU_ERR_CUDA",
    -21: "PS_GPU_ERR_STATE", -22: "PS_GPU_ERR_RANGE",
}
ASSIGN = {"NGP": 0, "CIC": 1, "TSC": 2, "PCS": 3}

EXPORTED = [
    "ps_gpu_create", "ps_gpu_destroy", "ps_gpu_nbin", "ps_gpu_assign_aos",
    "ps_gpu_assign_soa", "ps_gpu_execute", "ps_gpu_last_error",
    "ps_gpu_last_timings", "ps_gpu_last_launches", "ps_gpu_read_mesh",
    "ps_gpu_fft_r2c_host", "ps_gpu_bin_fields_host", "ps_gpu_stream",
    "ps_gpu_set_mu_bins", "ps_gpu_read_kmu", "ps_gpu_bin_fields_noalloc",
    "ps_gpu_batch_create", "ps_gpu_batch_launch", "ps_gpu_batch_wait", "ps_gpu_batch_result",
    "ps_gpu_batch_launches", "ps_gpu_batch_destroy", "ps_gpu_autotune", "ps_gpu_set_tuning",
    "ps_gpu_execute_learned", "ps_gpu_learned_launch", "ps_gpu_learned_finish", "ps_gpu_stage_aos", "ps_gpu_assign_staged", "ps_gpu_set_survey",
    "ps_gpu_debug_fail_alloc", "ps_gpu_set_warp_fft", "ps_gpu_debug_stall_pipeline",
    "ps_gpu_ensemble_create", "ps_gpu_ensemble_launch", "ps_gpu_ensemble_wait",
    "ps_gpu_ensemble_destroy",
]


class Batch:
    """Many catalogues through one Estimator (ncat = 1): every launch of all
    their evaluations recorded once as a CUDA graph, replayed by launch().
    The device catalogues (AoS float64, 32-byte aligned) must stay alive."""

    def __init__(self, est, device_ptrs, ns):
        self.est = est
        self.ncat = len(ns)
        ptrs = (ctypes.c_void_p * self.ncat)(*[ctypes.c_void_p(int(p)) for p in device_ptrs])
        nn = (ctypes.c_size_t * self.ncat)(*[int(v) for v in ns])
        self._b = ctypes.c_void_p()
        est._check(lib().ps_gpu_batch_create(est._ctx, self.ncat, ptrs, nn, ctypes.byref(self._b)))

    def launch(self, wait=True):
        self.est._check(lib().ps_gpu_batch_launch(self._b, 1 if wait else 0))

    def wait(self):
        self.est._check(lib().ps_gpu_batch_wait(self._b))

    def result(self, i) -> "Spectrum":
        r, out = self.est._result()
        self.est._check(lib().ps_gpu_batch_result(self._b, int(i), ctypes.byref(r)))
        return self.est._spectrum(r, out)

    def launches(self):
        return lib().ps_gpu_batch_launches(self._b)

    def close(self):
        if self._b:
            lib().ps_gpu_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PowspecError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")


class Params(ctypes.Structure):
    _fields_ = [
        ("ng", ctypes.c_int),
        ("box", ctypes.c_double * 3),
        ("assign", ctypes.c_int),
        ("interlace", ctypes.c_int),
        ("ncat", ctypes.c_int),
        ("isauto", ctypes.c_int * 2),
        ("iscross", ctypes.c_int),
        ("los", ctypes.c_double * 3),
        ("kmin", ctypes.c_double),
        ("kmax", ctypes.c_double),
        ("dk", ctypes.c_double),
        ("logscale", ctypes.c_int),
        ("npole", ctypes.c_int),
        ("poles", ctypes.c_int * 7),
        ("device", ctypes.c_int),
    ]


_dp = ctypes.POINTER(ctypes.c_double)


class Result(ctypes.Structure):
    _fields_ = [
        ("nbin", ctypes.c_int),
        ("k", _dp),
        ("kedge", _dp),
        ("km", _dp),
        ("cnt", ctypes.POINTER(ctypes.c_uint64)),
        ("lcnt", _dp),
        ("pl", _dp),
        ("xpl", _dp),
        ("shot", ctypes.c_double * 2),
        ("norm", ctypes.c_double * 2),
        ("wdata", ctypes.c_double * 2),
    ]


_lib = None


def build(verbose=False):
    from . import buildlib
    return buildlib.build(verbose=verbose)


def lib():
    """Load libpowspec_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built: run powspec_gb300.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.ps_gpu_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]
        L.ps_gpu_destroy.argtypes = [ctypes.c_void_p]
        L.ps_gpu_destroy.restype = None
        L.ps_gpu_nbin.argtypes = [ctypes.c_void_p]
        L.ps_gpu_assign_aos.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_int]
        L.ps_gpu_assign_soa.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4 + [
            ctypes.c_size_t, ctypes.c_int]
        L.ps_gpu_execute.argtypes = [ctypes.c_void_p, ctypes.POINTER(Result)]
        L.ps_gpu_last_error.argtypes = [ctypes.c_void_p]
        L.ps_gpu_last_error.restype = ctypes.c_char_p
        L.ps_gpu_last_timings.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ps_gpu_last_launches.argtypes = [ctypes.c_void_p]
        L.ps_gpu_set_mu_bins.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ps_gpu_read_kmu.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ps_gpu_stream.argtypes = [ctypes.c_void_p]
        L.ps_gpu_stream.restype = ctypes.c_void_p
        L.ps_gpu_read_mesh.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.ps_gpu_fft_r2c_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.ps_gpu_bin_fields_host.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 3
        L.ps_gpu_bin_fields_noalloc.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 4
        L.ps_gpu_batch_create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
        L.ps_gpu_batch_launch.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ps_gpu_batch_wait.argtypes = [ctypes.c_void_p]
        L.ps_gpu_batch_result.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Result)]
        L.ps_gpu_batch_launches.argtypes = [ctypes.c_void_p]
        L.ps_gpu_batch_destroy.argtypes = [ctypes.c_void_p]
        L.ps_gpu_batch_destroy.restype = None
        L.ps_gpu_autotune.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                      ctypes.c_void_p]
        L.ps_gpu_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ps_gpu_set_warp_fft.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ps_gpu_debug_stall_pipeline.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ps_gpu_ensemble_create.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p)]
        L.ps_gpu_ensemble_launch.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ps_gpu_ensemble_wait.argtypes = [ctypes.c_void_p]
        L.ps_gpu_ensemble_destroy.argtypes = [ctypes.c_void_p]
        L.ps_gpu_ensemble_destroy.restype = None
        L.ps_gpu_stage_aos.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
        L.ps_gpu_assign_staged.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.ps_gpu_set_survey.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_void_p]
        _lib = L
    return _lib


@dataclass
class Spectrum:
    nbin: int
    k: np.ndarray
    kedge: np.ndarray
    km: np.ndarray
    cnt: np.ndarray
    lcnt: np.ndarray
    pl: np.ndarray    # [2, npole, nbin]
    xpl: np.ndarray   # [npole, nbin]
    shot: np.ndarray
    norm: np.ndarray
    wdata: np.ndarray


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Estimator:
    """One GPU context: settings with the meaning of the reference's CONF."""

    def __init__(self, ng, box=1000.0, assign=1, interlace=False, ncat=1,
                 poles=(0, 2, 4), los=(0.0, 0.0, 1.0), kmin=0.0, kmax=-1.0, dk=0.005,
                 logscale=False, isauto=(True, True), iscross=True, device=0):
        L = lib()
        if isinstance(assign, str):
            assign = ASSIGN[assign.upper()]
        p = Params()
        p.ng = int(ng)
        b = box if isinstance(box, (tuple, list)) else (box, box, box)
        p.box = (ctypes.c_double * 3)(*[float(x) for x in b])
        p.assign = int(assign)
        p.interlace = int(bool(interlace))
        p.ncat = int(ncat)
        p.isauto = (ctypes.c_int * 2)(*[int(bool(x)) for x in isauto])
        p.iscross = int(bool(iscross) and ncat == 2)
        p.los = (ctypes.c_double * 3)(*[float(x) for x in los])
        p.kmin, p.kmax, p.dk = float(kmin), float(kmax), float(dk)
        p.logscale = int(bool(logscale))
        poles = sorted(set(int(x) for x in poles))
        p.npole = len(poles)
        p.poles = (ctypes.c_int * 7)(*poles)
        p.device = int(device)
        self.params = p
        self.poles = poles
        self.ncat = int(ncat)
        self._ctx = ctypes.c_void_p()
        rc = L.ps_gpu_create(ctypes.byref(p), ctypes.byref(self._ctx))
        if rc:
            msg = self.last_error()
            self.close()
            raise PowspecError(rc, msg)
        self.nbin = L.ps_gpu_nbin(self._ctx)
        self._staged = [None, None]

    def last_error(self):
        if not self._ctx:
            return "context not created"
        return lib().ps_gpu_last_error(self._ctx).decode()

    def close(self):
        if self._ctx:
            lib().ps_gpu_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise PowspecError(rc, self.last_error())

    # -- gen_dens for one catalogue
    def assign(self, cat, particles=None, *, x=None, y=None, z=None, w=None, on_device=False,
               n=None):
        """AoS float64 [N,4] (host numpy or device pointer with n=...) or SoA float32."""
        L = lib()
        if particles is not None:
            if on_device:
                self._check(L.ps_gpu_assign_aos(self._ctx, cat, ctypes.c_void_p(particles), n, 1))
            else:
                a = np.ascontiguousarray(particles, dtype=np.float64)
                self._keep = a
                self._check(L.ps_gpu_assign_aos(self._ctx, cat, _ptr(a), len(a), 0))
        else:
            if on_device:
                self._check(L.ps_gpu_assign_soa(self._ctx, cat, ctypes.c_void_p(x), ctypes.c_void_p(y),
                                                ctypes.c_void_p(z),
                                                ctypes.c_void_p(w) if w else None, n, 1))
            else:
                arrs = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z)]
                wa = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
                self._keep = (arrs, wa)
                self._check(L.ps_gpu_assign_soa(self._ctx, cat, _ptr(arrs[0]), _ptr(arrs[1]),
                                                _ptr(arrs[2]), _ptr(wa), len(arrs[0]), 0))

    def _result(self):
        nb, npole = self.nbin, len(self.poles)
        out = dict(k=np.zeros(nb), kedge=np.zeros(nb + 1), km=np.zeros(nb),
                   cnt=np.zeros(nb, np.uint64), lcnt=np.zeros((npole, nb)),
                   pl=np.zeros((2, npole, nb)), xpl=np.zeros((npole, nb)))
        r = Result()
        r.k = out["k"].ctypes.data_as(_dp)
        r.kedge = out["kedge"].ctypes.data_as(_dp)
        r.km = out["km"].ctypes.data_as(_dp)
        r.cnt = out["cnt"].ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        r.lcnt = out["lcnt"].ctypes.data_as(_dp)
        r.pl = out["pl"].ctypes.data_as(_dp)
        r.xpl = out["xpl"].ctypes.data_as(_dp)
        return r, out

    @staticmethod
    def _spectrum(r, out):
        return Spectrum(nbin=r.nbin, shot=np.array(r.shot[:]), norm=np.array(r.norm[:]),
                        wdata=np.array(r.wdata[:]), **out)

    def execute(self) -> Spectrum:
        r, out = self._result()
        self._check(lib().ps_gpu_execute(self._ctx, ctypes.byref(r)))
        return self._spectrum(r, out)

    def autotune(self, device_ptr, n, reps=2):
        """Time the alternative launch configurations on one catalogue (device
        AoS float64 records) and keep the fastest; returns the choices."""
        ch = np.zeros(6, np.int32)
        self._check(lib().ps_gpu_autotune(self._ctx, ctypes.c_void_p(device_ptr), int(n), int(reps),
                                          _ptr(ch)))
        return dict(gather_threads=int(ch[0]), z_radix32=bool(ch[1]), y_radix32=bool(ch[2]),
                    pipelined_pass_c=bool(ch[3]), dense_lane_groups=bool(ch[4]),
                    region_gather=bool(ch[5]), warp_fft=self.warp_fft())

    def warp_fft(self, mask=None):
        """Warp-register transforms in use (bit 0 z, 1 y, 2 x pass); with a
        mask, sets them first (bits without a warp form are dropped)."""
        rc = lib().ps_gpu_set_warp_fft(self._ctx, -1 if mask is None else int(mask))
        if rc < 0:
            raise PowspecError(rc, self.last_error())
        return rc

    def set_tuning(self, gather_threads=None, z_radix32=None, y_radix32=None,
                   pipelined_pass_c=None, dense_lane_groups=None, region_gather=None):
        """Sets launch configurations (the autotuner's choices; None keeps one).
        region_gather: True, False, or "auto" (by particles per cell)."""
        def v(x):
            return -1 if x is None else int(x)
        rg = -1 if region_gather is None else (2 if region_gather == "auto" else int(bool(region_gather)))
        ch = np.array([v(gather_threads), v(z_radix32), v(y_radix32), v(pipelined_pass_c),
                       v(dense_lane_groups), rg], np.int32)
        self._check(lib().ps_gpu_set_tuning(self._ctx, _ptr(ch)))

    def set_survey(self, cat, shot, norm, origin=None):
        """Survey catalogue `cat`, before its assign: P_0 = (sum / cnt - shot)
        / norm; multipoles l > 0 by the spherical-harmonic decomposition
        (origin = the box corner, the observer at 0; with interlacing, over
        the c2r of the combined field).
        The catalogue holds the data (weights w) and the randoms (weights
        -alpha w), positions relative to the box corner."""
        o = None if origin is None else np.ascontiguousarray(origin, dtype=np.float64)
        self._check(lib().ps_gpu_set_survey(self._ctx, cat, float(shot), float(norm),
                                            None if o is None else _ptr(o)))

    def stage(self, slot, particles):
        """Starts copying host AoS float64 [N, 4] records (pinned memory for
        an asynchronous copy) into staging slot 0 or 1; returns at once."""
        a = np.ascontiguousarray(particles, dtype=np.float64)
        self._staged[slot] = a  # kept alive until the slot is reused
        self._check(lib().ps_gpu_stage_aos(self._ctx, slot, a.ctypes.data_as(ctypes.c_void_p), len(a)))

    def assign_staged(self, cat, slot):
        """Assigns the catalogue in a staging slot (after its copy)."""
        self._check(lib().ps_gpu_assign_staged(self._ctx, cat, slot))

    def run_stream(self, cats, execute=None):
        """Evaluates host catalogues one after another (one catalogue per
        context), the copy of each overlapping the evaluation of the one
        before through the two staging slots; yields the results."""
        execute = execute or self.execute
        it = iter(cats)
        cur = next(it, None)
        slot = 0
        if cur is None:
            return
        self.stage(slot, cur)
        while cur is not None:
            nxt = next(it, None)
            if nxt is not None:
                self.stage(1 - slot, nxt)
            self.assign_staged(0, slot)
            yield execute()
            cur, slot = nxt, 1 - slot

    def batch(self, device_ptrs, ns):
        """A CUDA-graph batch of single-catalogue evaluations (see Batch)."""
        return Batch(self, device_ptrs, ns)

    def run(self, cats):
        for i, c in enumerate(cats):
            self.assign(i, c)
        return self.execute()

    def timings(self):
        t = np.zeros(6, np.float32)
        lib().ps_gpu_last_timings(self._ctx, _ptr(t), 6)
        return t

    def launches(self):
        return lib().ps_gpu_last_launches(self._ctx)

    def set_mu_bins(self, nmu):
        self._check(lib().ps_gpu_set_mu_bins(self._ctx, int(nmu)))
        self.nmu = int(nmu)

    def read_kmu(self, nspec):
        """Raw per-(k, |mu|) sums of the last execute: [nspec, npole, nbin, nmu]."""
        out = np.zeros((nspec, len(self.poles), self.nbin, self.nmu))
        self._check(lib().ps_gpu_read_kmu(self._ctx, _ptr(out)))
        return out

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        return lib().ps_gpu_stream(self._ctx) or 0

    # -- stage-level entry points
    def read_mesh(self, cat=0, m=0):
        ng = self.params.ng
        out = np.zeros((ng, ng, ng))
        self._check(lib().ps_gpu_read_mesh(self._ctx, cat, m, _ptr(out)))
        return out

    def fft_r2c(self, real):
        ng = self.params.ng
        a = np.ascontiguousarray(real, dtype=np.float32)
        out = np.zeros((ng, ng, ng // 2 + 1), np.complex64)
        self._check(lib().ps_gpu_fft_r2c_host(self._ctx, _ptr(a), _ptr(out)))
        return out

    def bin_fields(self, f1, f2=None):
        a = np.ascontiguousarray(f1, dtype=np.complex64)
        b = a if f2 is None else np.ascontiguousarray(f2, dtype=np.complex64)
        out = np.zeros((len(self.poles), self.nbin))
        self._check(lib().ps_gpu_bin_fields_host(self._ctx, _ptr(a), _ptr(b), _ptr(out)))
        return out
