"""Learned alias/window correction for coarse meshes.

A coarse mesh (e.g. Ng = 256) is cheap but its multipoles carry residual
aliasing and window errors near its Nyquist frequency.  This module learns a
per-mode multiplicative correction c(k/k_Nyq, mu, scheme, interlace, shot
ratio) from pairs of coarse- and fine-mesh spectra produced by the plain GPU
estimator on the same catalogues, so that a coarse mesh reproduces the
fine-mesh (Ng = 1024, PCS, interlaced) P_l(k).

The correction is applied per (k bin, |mu| bin) cell of the coarse binning
(16 |mu| bins): with A_bjl the cell's raw sums / (norm cnt_b) and B_bl the
shot-noise term, P_l(b) = (2l+1) (sum_j c_bj A_bjl - B_bl).  The network
(6 -> 64 -> 64 -> 64 -> 1, GELU, BF16 tensor cores) is trained and evaluated
by the CUDA kernels of libpowspec_gpu.so (include/powspec_learned.h).  The
plain fine-mesh method stays the fallback and the judge of the error: k bins
whose held-out error exceeds the tolerance are disabled, and the fine mesh's
values replace the surrogate's there (LearnedEstimator, fallback=True).
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass, field

import numpy as np

from . import ASSIGN, Estimator, PowspecError, _ptr, lib

NMU = 16
POLES = (0, 2, 4)
FINE = dict(ng=1024, assign=3, interlace=True)
COARSE_CONFIGS = [(ng, a, il) for ng in (128, 256) for a in (1, 2, 3) for il in (False, True)]
HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "data", "learned_alias.bin")


def _mlp_lib():
    L = lib()
    if not hasattr(L, "_mlp_ready"):
        vp = ctypes.c_void_p
        L.ps_mlp_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        L.ps_mlp_destroy.argtypes = [vp]
        L.ps_mlp_destroy.restype = None
        L.ps_mlp_last_error.argtypes = [vp]
        L.ps_mlp_last_error.restype = ctypes.c_char_p
        L.ps_mlp_set_params.argtypes = [vp, vp]
        L.ps_mlp_get_params.argtypes = [vp, vp]
        L.ps_mlp_set_data.argtypes = [vp, vp, vp, vp, ctypes.c_int]
        L.ps_mlp_grad.argtypes = [vp, vp, ctypes.c_int, vp, vp]
        L.ps_mlp_train.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, vp]
        L.ps_mlp_infer.argtypes = [vp, vp, ctypes.c_int, vp]
        L.ps_mlp_save.argtypes = [vp, ctypes.c_char_p]
        L.ps_mlp_load.argtypes = [vp, ctypes.c_char_p]
        L.ps_gpu_execute_learned.argtypes = [vp, vp, vp, vp]
        L.ps_gpu_learned_launch.argtypes = [vp, vp]
        L.ps_gpu_learned_finish.argtypes = [vp, vp, vp]
        L._mlp_ready = True
    return L


class MLP:
    """The correction network on one GPU (CUDA kernels, no host compute)."""

    def __init__(self, device=0, params=None):
        L = _mlp_lib()
        self.nparam = L.ps_mlp_nparam()
        self._m = ctypes.c_void_p()
        rc = L.ps_mlp_create(device, ctypes.byref(self._m))
        if rc:
            raise PowspecError(rc, "ps_mlp_create failed")
        if params is not None:
            self.set_params(params)

    def _check(self, rc):
        if rc:
            raise PowspecError(rc, _mlp_lib().ps_mlp_last_error(self._m).decode())

    def close(self):
        if self._m:
            _mlp_lib().ps_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparam
        self._check(_mlp_lib().ps_mlp_set_params(self._m, _ptr(p)))

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        self._check(_mlp_lib().ps_mlp_get_params(self._m, _ptr(p)))
        return p

    def set_data(self, x, a, grp):
        x = np.ascontiguousarray(x, dtype=np.float32)
        a = np.ascontiguousarray(a, dtype=np.float32)
        grp = np.ascontiguousarray(grp, dtype=np.float32)
        self._data = (x, a, grp)
        self._check(_mlp_lib().ps_mlp_set_data(self._m, _ptr(x), _ptr(a), _ptr(grp), len(grp)))

    def grad(self, idx):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        g = np.zeros(self.nparam, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(_mlp_lib().ps_mlp_grad(self._m, _ptr(idx), len(idx), _ptr(g), _ptr(loss)))
        return float(loss[0]), g

    def train(self, idx, batch, lr=1e-3):
        idx = np.ascontiguousarray(idx, dtype=np.int32).ravel()
        nsteps = len(idx) // batch
        loss = np.zeros(nsteps, np.float32)
        self._check(_mlp_lib().ps_mlp_train(self._m, _ptr(idx), nsteps, batch, ctypes.c_float(lr),
                                            _ptr(loss)))
        return loss

    def infer(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        c = np.zeros(len(x), np.float32)
        self._check(_mlp_lib().ps_mlp_infer(self._m, _ptr(x), len(x), _ptr(c)))
        return c

    def save(self, path):
        self._check(_mlp_lib().ps_mlp_save(self._m, path.encode()))

    def load(self, path):
        self._check(_mlp_lib().ps_mlp_load(self._m, path.encode()))


def init_params(seed=0, nparam=9473):
    """He-style initialisation of the hidden layers, zero output layer (so
    the untrained correction is c = 1: the plain coarse method).  Layout:
    W1[16][64] (input rows 6..15 zero), b1, W2[64][64], b2, W3[64][64], b3,
    w4[64], b4."""
    rng = np.random.default_rng(seed)
    k1, h, nin = 16, 64, 6
    p = np.zeros(nparam, np.float32)
    w1 = np.zeros((k1, h))
    w1[:nin] = rng.standard_normal((nin, h)) * np.sqrt(2.0 / nin)
    p[0:k1 * h] = w1.ravel()
    o = k1 * h + h
    p[o:o + h * h] = (rng.standard_normal((h, h)) * np.sqrt(2.0 / h)).ravel()
    o += h * h + h
    p[o:o + h * h] = (rng.standard_normal((h, h)) * np.sqrt(2.0 / h)).ravel()
    return p


# ---------------------------------------------------------------- features
def features(kcen, kny, assign, interlace, shot_ratio, nmu=NMU):
    """Feature rows [nbin * nmu, 6] of the (k, |mu|) cells."""
    nb = len(kcen)
    q = np.repeat(np.asarray(kcen) / kny, nmu)
    mu = np.tile((np.arange(nmu) + 0.5) / nmu, nb)
    r = np.repeat(np.asarray(shot_ratio), nmu)
    return np.stack([q, q * q, mu * mu, np.full_like(q, assign / 3.0),
                     np.full_like(q, float(interlace)), r], axis=1).astype(np.float32)


@dataclass
class Cells:
    """One coarse measurement split into (k, |mu|) cells."""
    A: np.ndarray       # [nbin, nmu, 3] raw sums / (norm cnt)
    B: np.ndarray       # [nbin, 3] shot-noise terms
    kcen: np.ndarray
    kny: float
    shot: float
    cnt: np.ndarray
    plain: np.ndarray   # [3, nbin] the uncorrected multipoles

    def shot_ratio(self):
        raw0 = self.A[:, :, 0].sum(1)
        return np.clip(self.shot / np.maximum(raw0, 1e-30), 0.0, 1.0)

    def corrected(self, c):
        """Multipoles with cell factors c [nbin * nmu] (or [nbin, nmu])."""
        c = np.asarray(c, dtype=np.float64).reshape(self.A.shape[0], -1)
        f = np.array([1.0, 5.0, 9.0])
        return (f[:, None] * (np.einsum("bj,bjl->lb", c, self.A) - self.B.T))


def measure_cells(est: Estimator, cat) -> Cells:
    """Coarse evaluation with |mu| sub-bins (auto spectrum of one catalogue)."""
    if getattr(est, "nmu", 1) != NMU:
        est.set_mu_bins(NMU)
    r = est.run([cat])
    kmu = est.read_kmu(1)[0]  # [npole, nbin, nmu]
    norm, shot = r.norm[0], r.shot[0]
    cnt = r.cnt.astype(np.float64)
    safe = np.maximum(cnt, 1)
    A = np.transpose(kmu, (1, 2, 0)) / (norm * safe)[:, None, None]
    A[cnt == 0] = 0
    B = (shot * r.lcnt / safe).T
    B[cnt == 0] = 0
    kny = np.pi * est.params.ng / max(est.params.box)
    return Cells(A=A, B=B, kcen=r.k, kny=kny, shot=shot, cnt=cnt, plain=r.pl[0])


# ---------------------------------------------------------------- datasets
def _gen_catalogue(args):
    seed, n, box, ngen = args
    from .catalog import lognormal
    return lognormal(n, box=box, seed=seed, ngen=ngen)


def make_catalogues(seeds, n=4_000_000, box=1000.0, ngen=256, workers=None):
    """Seeded lognormal catalogues, generated in a spawn process pool (start
    it before the first GPU call).  Spawned workers import the caller's main
    module: a calling script must guard its top level with
    ``if __name__ == "__main__":``."""
    import multiprocessing as mp
    args = [(int(s), n, box, ngen) for s in seeds]
    workers = workers or min(len(args), os.cpu_count() or 1)
    if workers <= 1:
        return [_gen_catalogue(a) for a in args]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_gen_catalogue, args)


@dataclass
class Pair:
    fine: np.ndarray            # [3, nbin_fine]
    fine_shot: float
    cells: dict = field(default_factory=dict)   # config -> Cells


def measure_pairs(cats, configs=COARSE_CONFIGS, box=1000.0, dk=0.005, device=0, fine_cfg=None,
                  log=None):
    """Fine labels and coarse cells for every catalogue of the iterable
    `cats` (consumed one at a time, so only the spectra stay in memory)."""
    fc = fine_cfg or FINE
    ests = []
    try:
        fine = Estimator(ng=fc["ng"], box=box, assign=fc["assign"], interlace=fc["interlace"],
                         poles=POLES, dk=dk, device=device)
        ests.append(fine)
        coarse = {}
        for cfg in configs:
            ng, a, il = cfg
            e = Estimator(ng=ng, box=box, assign=a, interlace=il, poles=POLES, dk=dk, device=device)
            e.set_mu_bins(NMU)
            coarse[cfg] = e
            ests.append(e)
        out = []
        for i, c in enumerate(cats):
            r = fine.run([c])
            p = Pair(fine=r.pl[0], fine_shot=r.shot[0])
            for cfg, e in coarse.items():
                p.cells[cfg] = measure_cells(e, c)
            out.append(p)
            if log and (i + 1) % 32 == 0:
                log(f"measured {i + 1} catalogues")
        return out
    finally:
        for e in ests:
            e.close()


def stream_catalogues(seeds, n=4_000_000, box=1000.0, ngen=256, workers=None):
    """Seeded lognormal catalogues from a spawn process pool, yielded in seed
    order as they are ready.  Spawned workers import the caller's main
    module: a calling script must guard its top level with
    ``if __name__ == "__main__":``."""
    import multiprocessing as mp
    args = [(int(s), n, box, ngen) for s in seeds]
    workers = workers or min(len(args), os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(workers) as pool:
        for cat in pool.imap(_gen_catalogue, args, chunksize=1):
            yield cat


def kmax_frac(cells: Cells, frac=0.8):
    return cells.kcen <= frac * cells.kny


def build_groups(pairs, configs=COARSE_CONFIGS, frac=0.8):
    """Training rows/groups (see include/powspec_learned.h)."""
    xs, as_, gs, meta = [], [], [], []
    for pi, p in enumerate(pairs):
        for cfg in configs:
            cl = p.cells[cfg]
            ng, a, il = cfg
            use = kmax_frac(cl, frac) & (cl.cnt > 0)
            nb = len(cl.kcen)
            x = features(cl.kcen, cl.kny, a, il, cl.shot_ratio()).reshape(nb, NMU, 6)
            pf = p.fine[:, :nb]
            sig = pf[0] + p.fine_shot
            for b in np.nonzero(use)[0]:
                xs.append(x[b])
                as_.append(cl.A[b])
                gs.append([cl.B[b, 0], cl.B[b, 1], cl.B[b, 2], pf[0, b], pf[1, b], pf[2, b],
                           1.0 / sig[b] ** 2, 1.0])
                meta.append((pi, cfg, b))
    return (np.concatenate(xs).astype(np.float32), np.concatenate(as_).astype(np.float32),
            np.array(gs, np.float32), meta)


# ---------------------------------------------------------------- training
def train(mlp: MLP, groups, steps=20000, batch=256, lr=1e-3, seed=0, chunk=2000, log=None):
    x, a, g, _ = groups
    mlp.set_data(x, a, g)
    rng = np.random.default_rng(seed)
    losses = []
    done = 0
    while done < steps:
        n = min(chunk, steps - done)
        idx = rng.integers(0, len(g), size=(n, batch), dtype=np.int32)
        l = mlp.train(idx, batch, lr)
        losses.append(l)
        done += n
        if log:
            log(f"step {done}: loss {float(l[-200:].mean()):.4e}")
    return np.concatenate(losses)


def correct(mlp: MLP, cells: Cells, assign, interlace):
    x = features(cells.kcen, cells.kny, assign, interlace, cells.shot_ratio())
    c = mlp.infer(x)
    return cells.corrected(c)


def errors(pairs, mlp: MLP, configs=COARSE_CONFIGS, frac=0.8):
    """Per config: max over catalogues of |dP_l| / P_0^fine per k bin, for the
    plain coarse and the corrected coarse multipoles."""
    out = {}
    for cfg in configs:
        ng, a, il = cfg
        e_plain, e_corr = [], []
        for p in pairs:
            cl = p.cells[cfg]
            nb = len(cl.kcen)
            pf = p.fine[:, :nb]
            den = np.abs(pf[0])
            pc = correct(mlp, cl, a, il) if mlp is not None else cl.plain
            with np.errstate(divide="ignore", invalid="ignore"):
                e_plain.append(np.abs(cl.plain - pf) / den)
                e_corr.append(np.abs(pc - pf) / den)
        c0 = pairs[0].cells[cfg]
        # bins with modes besides DC and a positive fine monopole, up to frac k_Nyq
        use = kmax_frac(c0, frac) & (c0.cnt > 1) & np.all([p.fine[0, :len(c0.kcen)] > 0 for p in pairs], 0)
        out[cfg] = dict(plain=np.max(e_plain, 0)[:, use], corrected=np.max(e_corr, 0)[:, use],
                        k=c0.kcen[use], bins=np.nonzero(use)[0])
    return out


def disabled_bins(err, tol=0.01):
    """k-bin indices (per config) where the held-out corrected error exceeds tol."""
    return {cfg: e["bins"][e["corrected"].max(0) > tol].tolist() for cfg, e in err.items()}


def save_report(path, err, tol=0.01):
    rep = {}
    for cfg, e in err.items():
        key = f"ng{cfg[0]}_{['NGP', 'CIC', 'TSC', 'PCS'][cfg[1]]}_{'il' if cfg[2] else 'noil'}"
        rep[key] = dict(max_err_plain=float(e["plain"].max()),
                        max_err_corrected=float(e["corrected"].max()),
                        mean_err_plain=float(e["plain"].mean()),
                        mean_err_corrected=float(e["corrected"].mean()),
                        max_err_plain_by_l=[float(v) for v in e["plain"].max(1)],
                        max_err_corrected_by_l=[float(v) for v in e["corrected"].max(1)],
                        disabled_bins=[int(b) for b in e["bins"][e["corrected"].max(0) > tol]])
    with open(path, "w") as f:
        json.dump(rep, f, indent=1)
    return rep


# ------------------------------------------------------------- estimator
class LearnedEstimator:
    """Coarse-mesh P_l(k) with the learned correction applied.

    run(cat) evaluates the coarse mesh on the GPU with 16 |mu| sub-bins, runs
    the correction network on the (k, |mu|) cells (GPU kernel) and returns
    (k, P_l [3, nbin], trusted [nbin]).  `trusted` is False on k bins beyond
    the trained range (k > frac k_Nyq).

    The plain fine mesh (Ng = 1024, PCS, interlaced) is the fallback: on the
    bins where the held-out report puts the corrected error above the
    tolerance, the surrogate is disabled.  With fallback=True (default) the
    fine mesh is evaluated on the same catalogue whenever the configuration
    has such bins, and its multipoles replace the surrogate's there (its
    cost is part of the evaluation; `last_fallback` marks those bins).  With
    fallback=False those bins keep the corrected values and are reported as
    not trusted."""

    def __init__(self, ng=256, assign=3, interlace=True, box=1000.0, dk=0.005, device=0,
                 weights=DEFAULT_WEIGHTS, frac=0.8, fallback=True):
        self.cfg = (ng, assign, interlace)
        self.est = Estimator(ng=ng, box=box, assign=assign, interlace=interlace, poles=POLES,
                             dk=dk, device=device)
        self.est.set_mu_bins(NMU)
        self.mlp = MLP(device=device)
        self.mlp.load(weights)
        self.frac = frac
        self.disabled = set()
        rep = weights.replace(".bin", "_report.json")
        if os.path.exists(rep):
            with open(rep) as f:
                r = json.load(f)
            key = f"ng{ng}_{['NGP', 'CIC', 'TSC', 'PCS'][assign]}_{'il' if interlace else 'noil'}"
            self.disabled = set(r.get(key, {}).get("disabled_bins", []))
        kny = np.pi * ng / max(self.est.params.box)
        kcen = (np.arange(self.est.nbin) + 0.5) * dk + self.est.params.kmin
        # disabled bins inside the trained range: the ones the fallback replaces
        self.fallback_bins = sorted(b for b in self.disabled
                                    if b < self.est.nbin and kcen[b] <= frac * kny)
        self.fine = None
        if fallback and self.fallback_bins:
            self.fine = Estimator(ng=FINE["ng"], box=box, assign=FINE["assign"],
                                  interlace=FINE["interlace"], poles=POLES, dk=dk, device=device)
        self.last_fallback = np.zeros(self.est.nbin, bool)
        self._last = None
        self._x = None
        self._trusted = None
        self._ctor = dict(ng=ng, box=box, assign=assign, interlace=interlace, poles=POLES, dk=dk,
                          device=device)
        self._tuning = None
        self._lane2 = None  # a second context for run_many(lanes=2)

    def autotune(self, device_ptr, n):
        """The context's autotuner (Estimator.autotune), its choice kept for
        the second context of run_many(lanes=2)."""
        self._tuning = self.est.autotune(device_ptr, n)
        if self._lane2 is not None:
            self._apply_tuning(self._lane2)
        return self._tuning

    def _apply_tuning(self, e):
        t = dict(self._tuning or {})
        mask = t.pop("warp_fft", None)
        if t:
            e.set_tuning(**t)
        e.warp_fft(self.est.warp_fft() if mask is None else mask)

    def _lane(self, i):
        if i == 0:
            return self.est
        if self._lane2 is None:
            e = Estimator(**self._ctor)
            e.set_mu_bins(NMU)
            self._apply_tuning(e)
            self._lane2 = e
        return self._lane2

    def close(self):
        self.est.close()
        if self._lane2 is not None:
            self._lane2.close()
        self.mlp.close()
        if self.fine is not None:
            self.fine.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, cat=None, *, device_ptr=None, n=None):
        """One learned evaluation (ps_gpu_execute_learned: the passes, the
        cell features, the network and the corrected multipoles all on the
        GPU, one copy back), plus the fine-mesh fallback where the
        configuration needs it.  cat: host AoS float64 [N, 4]; or a device
        pointer with n."""
        if device_ptr is not None:
            self.est.assign(0, device_ptr, on_device=True, n=n)
            if self.fine is not None:
                self.fine.assign(0, device_ptr, on_device=True, n=n)
        else:
            self.est.assign(0, cat)
            if self.fine is not None:
                self.fine.assign(0, cat)
        return self._execute()

    def run_stream(self, cats, lanes=1):
        """run() over host catalogues: the copy of each next catalogue (two
        staging slots) and its assignment are enqueued before the previous
        evaluation's results are waited for, so copies, assignments and
        evaluations follow each other without the GPU idling.  lanes=2
        alternates the catalogues between two contexts (as run_many), each
        with its own staging slots.  Results come in catalogue order.  A
        configuration that needs the fine-mesh fallback evaluates them one
        at a time."""
        if self.fine is not None:
            return (self.run(c) for c in cats)
        if int(lanes) >= 2:
            return self._stream2(cats)
        return self._stream(cats)

    def _stream2(self, cats):
        ests = [self._lane(0), self._lane(1)]
        slots = [0, 0]
        it = iter(cats)
        order = []  # lanes with an evaluation in flight, oldest first

        def begin(k, c):  # copy, assign and launch on lane k
            e = ests[k]
            e.stage(slots[k], c)
            e.assign_staged(0, slots[k])
            slots[k] ^= 1
            self._launch(e)
            order.append(k)

        for k in range(2):
            c = next(it, None)
            if c is None:
                break
            begin(k, c)
        while order:
            k = order.pop(0)
            e = ests[k]
            c = next(it, None)
            if c is not None:  # the lane's next catalogue, before waiting for its results
                e.stage(slots[k], c)
                e.assign_staged(0, slots[k])
                slots[k] ^= 1
            res = self._finish(e)
            if c is not None:
                self._launch(e)
                order.append(k)
            yield res

    def _stream(self, cats):
        est = self.est
        it = iter(cats)
        cur = next(it, None)
        if cur is None:
            return
        slot = 0
        est.stage(slot, cur)
        est.assign_staged(0, slot)
        self._launch()
        while True:
            nxt = next(it, None)
            if nxt is not None:
                est.stage(1 - slot, nxt)
                est.assign_staged(0, 1 - slot)
            yield self._finish()
            if nxt is None:
                break
            self._launch()
            slot = 1 - slot

    def run_many(self, device_ptrs, n, lanes=1):
        """run() over catalogues already on the device (32-byte aligned AoS
        records, n each), back to back: each catalogue's assignment is
        enqueued before the previous evaluation's results are waited for
        (ps_gpu_learned_launch / ps_gpu_learned_finish), so the GPU does not
        idle between evaluations.  lanes=2 alternates the catalogues between
        this context and a second one (same configuration and tuning, its own
        stream and buffers), so that two evaluations are in flight and one's
        kernels fill the other's gaps and tails.  Returns one (k, pc,
        trusted) per catalogue, in order.  A configuration that needs the
        fine-mesh fallback runs them one at a time."""
        ptrs = list(device_ptrs)
        if self.fine is not None or not ptrs:
            return [self.run(device_ptr=p, n=n) for p in ptrs]
        ests = [self._lane(k) for k in range(max(1, min(2, int(lanes))))]
        L = len(ests)
        out = [None] * len(ptrs)

        def start(i):
            e = ests[i % L]
            e.assign(0, ptrs[i], on_device=True, n=n)
            self._launch(e)

        if L == 1:
            start(0)
            for i in range(len(ptrs)):
                if i + 1 < len(ptrs):
                    self.est.assign(0, ptrs[i + 1], on_device=True, n=n)
                out[i] = self._finish()
                if i + 1 < len(ptrs):
                    self._launch()
            return out
        for i in range(min(L, len(ptrs))):
            start(i)
        for i in range(len(ptrs)):
            out[i] = self._finish(ests[i % L])
            if i + L < len(ptrs):
                start(i + L)
        return out

    def _launch(self, est=None):
        est = est or self.est
        rc = _mlp_lib().ps_gpu_learned_launch(est._ctx, self.mlp._m)
        if rc:
            raise PowspecError(rc, lib().ps_gpu_last_error(est._ctx).decode())

    def _finish(self, est=None):
        est = est or self.est
        r, out = est._result()
        pc = np.zeros((len(POLES), est.nbin))
        rc = _mlp_lib().ps_gpu_learned_finish(est._ctx, ctypes.byref(r), _ptr(pc))
        if rc:
            raise PowspecError(rc, lib().ps_gpu_last_error(est._ctx).decode())
        return self._post(r, out, pc)

    def _execute(self):
        r, out = self.est._result()
        pc = np.zeros((len(POLES), self.est.nbin))
        rc = _mlp_lib().ps_gpu_execute_learned(self.est._ctx, self.mlp._m, ctypes.byref(r), _ptr(pc))
        if rc:
            raise PowspecError(rc, lib().ps_gpu_last_error(self.est._ctx).decode())
        return self._post(r, out, pc)

    def _post(self, r, out, pc):
        spec = Estimator._spectrum(r, out)
        self._last = spec
        if self._trusted is None:
            kny = np.pi * self.est.params.ng / max(self.est.params.box)
            trusted = spec.k <= self.frac * kny
            for b in self.disabled:
                if b < len(trusted):
                    trusted[b] = False
            self._trusted = trusted
        trusted = self._trusted.copy()
        self.last_fallback[:] = False
        if self.fine is not None:
            # the plain fine mesh on the bins where the surrogate is disabled
            # (the same bin edges: kmin + i dk on both meshes)
            ref = self.fine.execute()
            fb = np.asarray(self.fallback_bins, dtype=np.int64)
            pc[:, fb] = ref.pl[0][:, fb]
            trusted[fb] = True
            self.last_fallback[fb] = True
        return spec.k, pc, trusted

    @property
    def last_cells(self):
        """The (k, |mu|) cells of the last run (read back on request)."""
        return None if self._last is None else _cells_from_result(self.est, self._last)

    def run_host_correction(self, cat=None, *, device_ptr=None, n=None):
        """The same evaluation with the cells, features and correction formed
        on the host (numpy) around the network's inference kernel."""
        if device_ptr is not None:
            self.est.assign(0, device_ptr, on_device=True, n=n)
            r = self.est.execute()
            cells = _cells_from_result(self.est, r)
        else:
            cells = measure_cells(self.est, cat)
        if self._x is None or len(self._x) != len(cells.kcen) * NMU:
            self._x = features(cells.kcen, cells.kny, self.cfg[1], self.cfg[2],
                               np.zeros(len(cells.kcen)))
        self._x[:, 5] = np.repeat(cells.shot_ratio(), NMU)
        pc = cells.corrected(self.mlp.infer(self._x))
        trusted = kmax_frac(cells, self.frac)
        for b in self.disabled:
            if b < len(trusted):
                trusted[b] = False
        if self.fine is not None:
            if device_ptr is not None:
                self.fine.assign(0, device_ptr, on_device=True, n=n)
            else:
                self.fine.assign(0, cat)
            ref = self.fine.execute()
            fb = np.asarray(self.fallback_bins, dtype=np.int64)
            pc[:, fb] = ref.pl[0][:, fb]
            trusted[fb] = True
        return cells.kcen, pc, trusted


def _cells_from_result(est, r):
    kmu = est.read_kmu(1)[0]
    norm, shot = r.norm[0], r.shot[0]
    cnt = r.cnt.astype(np.float64)
    safe = np.maximum(cnt, 1)
    A = np.transpose(kmu, (1, 2, 0)) / (norm * safe)[:, None, None]
    A[cnt == 0] = 0
    B = (shot * r.lcnt / safe).T
    B[cnt == 0] = 0
    kny = np.pi * est.params.ng / max(est.params.box)
    return Cells(A=A, B=B, kcen=r.k, kny=kny, shot=shot, cnt=cnt, plain=r.pl[0])
