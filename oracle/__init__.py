"""The oracle: CPU checkers for the periodic-box P_l(k) path.

TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker (or the timed CPU baseline).  The GPU product never imports it.

Two CPU implementations live here:

* ``port`` -- ``oracle/port/ps_oracle.c``: the project's own FP64/OpenMP C
  restatement of the reference path (src/genr_mesh.c, src/multipole.c), built
  by ``make -C oracle port`` on any machine.
* ``ref`` -- ``oracle/_ref/libpowspec_ref.so``: the unmodified reference
  sources compiled from their read-only location by ``make -C oracle ref``
  (only where the reference tree exists), driven in memory by
  ``oracle/ref_harness.c``.

Both link the FFTW-API shim in ``oracle/fftw_shim`` (FFTW itself is absent).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libps_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpowspec_ref.so")
REF_CLI = os.path.join(HERE, "_ref", "POWSPEC")
# Where the reference tree is read from: POWSPEC_REF_DIR, else the default
# of the build recipe (oracle/Makefile, REF).
REF_SRC = os.environ.get("POWSPEC_REF_DIR", "")

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_size_p = ctypes.POINTER(ctypes.c_size_t)


class OracleParams(ctypes.Structure):
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
        ("with_c2r", ctypes.c_int),
    ]


class OracleResult(ctypes.Structure):
    _fields_ = [
        ("maxbin", ctypes.c_int),
        ("nbin", ctypes.c_int),
        ("k", _c_double_p),
        ("kedge", _c_double_p),
        ("km", _c_double_p),
        ("cnt", _c_size_p),
        ("lcnt", _c_double_p),
        ("pl", _c_double_p),
        ("xpl", _c_double_p),
        ("shot", ctypes.c_double * 2),
        ("norm", ctypes.c_double * 2),
        ("wdata", ctypes.c_double * 2),
        ("t_mesh", ctypes.c_double),
        ("t_pk", ctypes.c_double),
    ]


@dataclass
class Spec:
    """Estimator settings with the meaning of the reference's CONF fields."""

    ng: int
    box: float | tuple = 1000.0
    assign: int = 1
    interlace: bool = False
    poles: tuple = (0, 2, 4)
    los: tuple = (0.0, 0.0, 1.0)
    kmin: float = 0.0
    kmax: float = -1.0
    dk: float = 0.005
    logscale: bool = False
    isauto: tuple = (True, True)
    iscross: bool = True

    def box3(self):
        b = self.box
        return tuple(float(x) for x in (b if isinstance(b, (tuple, list)) else (b, b, b)))


@dataclass
class Result:
    nbin: int
    k: np.ndarray
    kedge: np.ndarray
    km: np.ndarray
    cnt: np.ndarray
    lcnt: np.ndarray
    pl: np.ndarray       # [2, npole, nbin]
    xpl: np.ndarray      # [npole, nbin]
    shot: np.ndarray
    norm: np.ndarray
    times: tuple = field(default=(0.0, 0.0))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def build_port(force=False):
    if force or not os.path.exists(PORT_SO):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def ref_dir():
    """The reference tree the recipe compiles: POWSPEC_REF_DIR or the
    recipe's own default."""
    if REF_SRC:
        return REF_SRC
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                       capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def build_ref():
    """Compile the reference from source (only where its tree exists)."""
    ref = ref_dir()
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True)
    return REF_SO


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        build_port()
        L = ctypes.CDLL(PORT_SO)
        L.ps_oracle_legpoly.restype = ctypes.c_double
        L.ps_oracle_alias_corr.restype = ctypes.c_double
        L.ps_oracle_alias_corr.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ps_oracle_legpoly.argtypes = [ctypes.c_int, ctypes.c_double]
        L.ps_oracle_ylm.restype = ctypes.c_double
        L.ps_oracle_ylm.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 4
        _port = L
    return _port


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference oracle not built (make -C oracle ref)")
        _ref = ctypes.CDLL(REF_SO)
    return _ref


def set_threads(n):
    port().ps_oracle_set_threads(int(n))


def get_threads():
    return int(port().ps_oracle_get_threads())


def as_aos(cat):
    """Particles as the reference DATA layout: float64 [N, 4] = x, y, z, w."""
    a = np.ascontiguousarray(cat, dtype=np.float64)
    assert a.ndim == 2 and a.shape[1] == 4
    return a


def assign(which, cat, ng, box, assign, interlace):
    """Real-space mesh(es) from the port or the reference build."""
    cat = as_aos(cat)
    b = (ctypes.c_double * 3)(*([box] * 3 if np.isscalar(box) else box))
    m0 = np.zeros((ng, ng, ng))
    m1 = np.zeros((ng, ng, ng)) if interlace else None
    if which == "port":
        rc = port().ps_oracle_assign(_ptr(cat), ctypes.c_size_t(len(cat)), ng, b,
                                     assign, int(interlace), _ptr(m0),
                                     _ptr(m1) if interlace else None)
    else:
        rc = ref().ref_mesh(_ptr(cat), ctypes.c_size_t(len(cat)), ng, b, assign,
                            int(interlace), _ptr(m0), _ptr(m1) if interlace else None)
    if rc:
        raise RuntimeError(f"{which} assign failed: {rc}")
    return (m0, m1) if interlace else m0


def _maxbin(spec):
    return int(np.ceil(np.pi * spec.ng / min(spec.box3()) / spec.dk)) + 8 if not spec.logscale else 4096


def _port_call(spec: Spec, cats, with_c2r, call) -> Result:
    """Marshal spec and the result arrays for a port entry point; call(p,
    ptrs, ns, r) runs it."""
    nc = len(cats)
    maxbin = _maxbin(spec)
    npole = len(spec.poles)
    k = np.zeros(maxbin)
    kedge = np.zeros(maxbin + 1)
    km = np.zeros(maxbin)
    cnt = np.zeros(maxbin, np.uint64)
    lcnt = np.zeros((npole, maxbin))
    pl = np.zeros((2, npole, maxbin))
    xpl = np.zeros((npole, maxbin))
    p = OracleParams()
    p.ng = spec.ng
    p.box = (ctypes.c_double * 3)(*spec.box3())
    p.assign = spec.assign
    p.interlace = int(spec.interlace)
    p.ncat = nc
    p.isauto = (ctypes.c_int * 2)(*[int(x) for x in spec.isauto])
    p.iscross = int(spec.iscross)
    p.los = (ctypes.c_double * 3)(*spec.los)
    p.kmin, p.kmax, p.dk = spec.kmin, spec.kmax, spec.dk
    p.logscale = int(spec.logscale)
    p.npole = npole
    p.poles = (ctypes.c_int * 7)(*spec.poles)
    p.with_c2r = int(with_c2r)
    r = OracleResult()
    r.maxbin = maxbin
    r.k = k.ctypes.data_as(_c_double_p)
    r.kedge = kedge.ctypes.data_as(_c_double_p)
    r.km = km.ctypes.data_as(_c_double_p)
    r.cnt = cnt.ctypes.data_as(_c_size_p)
    r.lcnt = lcnt.ctypes.data_as(_c_double_p)
    r.pl = pl.ctypes.data_as(_c_double_p)
    r.xpl = xpl.ctypes.data_as(_c_double_p)
    ptrs = (ctypes.c_void_p * 2)(*[c.ctypes.data for c in cats] + [None] * (2 - nc))
    ns = (ctypes.c_size_t * 2)(*[len(c) for c in cats] + [0] * (2 - nc))
    rc = call(ctypes.byref(p), ptrs, ns, ctypes.byref(r))
    if rc:
        raise RuntimeError(f"oracle port failed: {rc}")
    nbin = r.nbin
    return Result(nbin=nbin, k=k[:nbin].copy(), kedge=kedge[:nbin + 1].copy(),
                  km=km[:nbin].copy(), cnt=cnt[:nbin].copy(), lcnt=lcnt[:, :nbin].copy(),
                  pl=pl[:, :, :nbin].copy(), xpl=xpl[:, :nbin].copy(),
                  shot=np.array(r.shot[:nc]), norm=np.array(r.norm[:nc]),
                  times=(r.t_mesh, r.t_pk))


def run(which, spec: Spec, cats, with_c2r=True) -> Result:
    """Whole periodic-box path on one or two catalogues (float64 [N,4])."""
    cats = [as_aos(c) for c in cats]
    nc = len(cats)
    if which == "port":
        return _port_call(spec, cats, with_c2r, port().ps_oracle_run)
    maxbin = _maxbin(spec)
    npole = len(spec.poles)
    k = np.zeros(maxbin)
    kedge = np.zeros(maxbin + 1)
    km = np.zeros(maxbin)
    cnt = np.zeros(maxbin, np.uint64)
    lcnt = np.zeros((npole, maxbin))
    pl = np.zeros((2, npole, maxbin))
    xpl = np.zeros((npole, maxbin))
    box = spec.box3()
    L = ref()
    nb = ctypes.c_int(0)
    shot = np.zeros(2)
    norm = np.zeros(2)
    times = np.zeros(2)
    ptrs = (ctypes.c_void_p * 2)(*[c.ctypes.data for c in cats] + [None] * (2 - nc))
    ns = (ctypes.c_size_t * 2)(*[len(c) for c in cats] + [0] * (2 - nc))
    isauto = (ctypes.c_int * 2)(*[int(x) for x in spec.isauto])
    poles = (ctypes.c_int * 7)(*spec.poles)
    rc = L.ref_powspec(nc, ptrs, ns, spec.ng, (ctypes.c_double * 3)(*box), spec.assign,
                       int(spec.interlace), (ctypes.c_double * 3)(*spec.los), poles,
                       npole, ctypes.c_double(spec.kmin), ctypes.c_double(spec.kmax),
                       ctypes.c_double(spec.dk), int(spec.logscale), isauto,
                       int(spec.iscross), maxbin, ctypes.byref(nb), _ptr(k), _ptr(kedge),
                       _ptr(km), _ptr(cnt), _ptr(lcnt), _ptr(pl), _ptr(xpl), _ptr(shot),
                       _ptr(norm), _ptr(times), 0)
    if rc:
        raise RuntimeError(f"reference run failed: {rc}")
    nbin = nb.value
    return Result(nbin=nbin, k=k[:nbin].copy(), kedge=kedge[:nbin + 1].copy(),
                  km=km[:nbin].copy(), cnt=cnt[:nbin].copy(), lcnt=lcnt[:, :nbin].copy(),
                  pl=pl[:, :, :nbin].copy(), xpl=xpl[:, :nbin].copy(), shot=shot[:nc],
                  norm=norm[:nc], times=tuple(times))


def survey(spec: Spec, cats, origin, shot, norm) -> Result:
    """Survey path (port) on one or two catalogues, each holding its data
    (weights w) and randoms (weights -alpha w), positions relative to the
    box corner `origin`; shot and norm per catalogue.  P_0 = (sum / cnt -
    shot) / norm with the k = 0 mode binned; P_l>0 by the spherical-harmonic
    decomposition (the c2r of the combined field with interlacing)."""
    cats = [as_aos(c) for c in cats]
    o = (ctypes.c_double * 3)(*[float(x) for x in origin])
    sh = (ctypes.c_double * 2)(*(list(map(float, shot)) + [0.0] * (2 - len(shot))))
    nm = (ctypes.c_double * 2)(*(list(map(float, norm)) + [1.0] * (2 - len(norm))))
    return _port_call(spec, cats, False,
                      lambda p, ptrs, ns, r: port().ps_oracle_survey(p, o, sh, nm, ptrs, ns, r))


def ylm(ell, m, ct, st, cp, sp):
    return port().ps_oracle_ylm(ell, m, ct, st, cp, sp)


def bins(spec: Spec):
    maxbin = _maxbin(spec)
    kedge = np.zeros(maxbin + 1)
    k = np.zeros(maxbin)
    nb = ctypes.c_int(0)
    rc = port().ps_oracle_bins(spec.ng, (ctypes.c_double * 3)(*spec.box3()),
                               ctypes.c_double(spec.kmin), ctypes.c_double(spec.kmax),
                               ctypes.c_double(spec.dk), int(spec.logscale), maxbin,
                               ctypes.byref(nb), _ptr(kedge), _ptr(k))
    if rc:
        raise RuntimeError(f"bins failed: {rc}")
    return kedge[:nb.value + 1].copy(), k[:nb.value].copy()


def r2c(mesh):
    ng = mesh.shape[0]
    m = np.ascontiguousarray(mesh, dtype=np.float64).copy()
    out = np.zeros((ng, ng, ng // 2 + 1), np.complex128)
    rc = port().ps_oracle_r2c(ng, _ptr(m), _ptr(out))
    if rc:
        raise RuntimeError("r2c failed")
    return out


def precomp(spec: Spec):
    """Window table [ng][ng][ng/2+1], counts and mean k of each bin."""
    kedge, _ = bins(spec)
    nbin = len(kedge) - 1
    ng = spec.ng
    alias = np.zeros((ng, ng, ng // 2 + 1))
    cnt = np.zeros(nbin, np.uint64)
    km = np.zeros(nbin)
    rc = port().ps_oracle_precomp(ng, (ctypes.c_double * 3)(*spec.box3()), spec.assign,
                                  int(spec.interlace), int(spec.logscale), nbin, _ptr(kedge),
                                  ctypes.c_double(spec.dk), _ptr(alias), _ptr(cnt), _ptr(km))
    if rc:
        raise RuntimeError("precomp failed")
    return alias, cnt, km
