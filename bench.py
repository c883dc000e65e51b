"""Benchmark of the periodic-box P_l(k) path on GB300.

One step = one evaluation: a catalogue -> {P_0, P_2, P_4}(k) table.

Workloads (synthetic, seeded; no catalogue ships with the reference): a
lognormal catalogue of ~4e6 particles (spectrum A k^-1.5 exp(-(k/0.5)^2),
sigma_G^2 = 1, Zel'dovich displacement along z), L = 1000 Mpc/h, dk = 0.005
h/Mpc, l = 0, 2, 4.

* learned_ng256_vs_plain_ng1024 (default): the learned form -- Ng = 256, PCS,
  interlaced, 16 |mu| sub-bins, plus the trained correction network -- timed
  against the plain Ng = 1024 PCS interlaced evaluation of the same
  catalogue in the same run; the line reports the learned evals/s (value),
  the plain evals/s, the speed-up and the max error against plain Ng = 1024
  up to 0.8 k_Nyq(256).  The catalogue's seed is outside the training set.
* plain_pcs_il_ng{1024,512,256}_n4e6: the plain PCS interlaced evaluation at
  that mesh size (the Ng = 256 one is the small case the ncu captures use).
* ensemble_256_mixed: a mock ensemble of 256 lognormal catalogues with N
  log-uniform in [1e5, 5e6], Ng from {128, 192, 256, 384} and CIC or TSC,
  interlaced; grouped by configuration, autotuned, each group's evaluations
  recorded as one CUDA graph; reported against the same evaluations one
  catalogue at a time.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank evaluates its own catalogue on its own GPU
(replicas: the path has no exchange step); value = all evaluations / the
max time over ranks.

--impl reference times the reference's CPU implementation of the quantity
both workloads compute (plain Ng = 1024 PCS interlaced): the oracle's FP64
OpenMP C restatement of genr_mesh + powspec on all host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PART = 4_000_000
LEARNED_LANES = 2  # contexts the learned loop alternates between (run_many)
BOX = 1000.0
DK = 0.005
SEED = 1          # held out: the correction was trained on seeds >= 1000
METRIC = "P_l(k) evals/s on 1 GB300"
WORKLOADS = {
    "learned_ng256_vs_plain_ng1024": dict(learned=True, ng=256, assign=3, interlace=True),
    # a coarse configuration whose uncorrected mesh misses the 1% bar
    "learned_ng128_cic_il_vs_plain_ng1024": dict(learned=True, ng=128, assign=1, interlace=True),
    "plain_pcs_il_ng1024_n4e6": dict(learned=False, ng=1024, assign=3, interlace=True),
    "plain_pcs_il_ng512_n4e6": dict(learned=False, ng=512, assign=3, interlace=True),
    "plain_pcs_il_ng256_n4e6": dict(learned=False, ng=256, assign=3, interlace=True),
    "ensemble_256_mixed": dict(learned=False, ensemble=True, ng=0, assign=1, interlace=True),
    # large single mesh: N = 1.5e8 lognormal, FP32 SoA positions, FP32 weights
    # uniform in [0.5, 1.5], L = 2000 Mpc/h, dk = 0.002
    "large_pcs_il_ng1024_n1.5e8_f32": dict(learned=False, large=True, ng=1024, assign=3, interlace=True),
    "large_pcs_il_ng2048_n1.5e8_f32": dict(learned=False, large=True, ng=2048, assign=3, interlace=True),
    # survey: 1e6 lognormal data in a sphere of radius 500 Mpc/h centred at
    # (1500, 800, 1200) from the observer, 3e6 randoms, FKP weights, fitted
    # box (1020 Mpc/h); P_0, P_2, P_4 by the spherical-harmonic decomposition
    "survey_pcs_il_ng256_l024_n4e6": dict(learned=False, survey=True, ng=256, assign=3,
                                          interlace=True, poles=(0, 2, 4)),
}
SURVEY_ND, SURVEY_CENTRE, SURVEY_RADIUS = 1_000_000, (1500.0, 800.0, 1200.0), 500.0
LARGE_N, LARGE_BOX, LARGE_DK = 150_000_000, 2000.0, 0.002
# mock ensemble: 256 catalogues, N log-uniform in [1e5, 5e6], Ng from
# {128, 192, 256, 384}, CIC or TSC, interlaced (seeded draws)
ENS_NCAT, ENS_NMIN, ENS_NMAX = 256, 1e5, 5e6
ENS_NG, ENS_ASSIGN = (128, 192, 256, 384), (1, 2)
DEFAULT = "learned_ng256_vs_plain_ng1024"
PLAIN_REF = dict(ng=1024, assign=3, interlace=True)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_catalogue(seed):
    from powspec_gb300 import catalog
    return catalog.lognormal(N_PART, box=BOX, seed=seed, ngen=256)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [l.split(",") for l in self.f.read().strip().splitlines() if l.strip()]
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = max(smax, float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if "Active" in v and "Not" not in v:
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": smax or None, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce(world, v, op):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def algorithmic_bytes(ng, interlace, n, bp=32):
    """Per-launch algorithmic HBM bytes of each phase (FP32 path).

    assignment: N * 32 B (AoS float64 records) + 4 B * Ng^3 per mesh (the
    roofline counts both meshes against the whole assignment phase);
    z pass: 4 B * Ng^3 read + 8 B * Ncmplx written; y pass: 8 B * Ncmplx
    read + written; x pass + binning: 8 B * Ncmplx per field read.
    """
    nmesh = 2 if interlace else 1
    ntot = ng ** 3
    ncx = ng * ng * (ng // 2 + 1)
    return {
        "assign": n * bp + 4 * ntot,
        "pass_z": 4 * ntot + 8 * ncx,
        "pass_y": 16 * ncx,
        "pass_x_bin": 8 * ncx * nmesh,
        "nmesh": nmesh,
        "total": nmesh * (n * bp + 4 * ntot) + nmesh * (4 * ntot + 8 * ncx) + nmesh * 8 * ncx * 2,
    }


def roofline(phases_ms, ng, interlace, n, traffic=None, assign=3, bp=32):
    peak, peak_kind = peaks()
    ab = algorithmic_bytes(ng, interlace, n, bp)
    # assignment: the whole phase (both meshes in one pass over the particles);
    # FFT passes: per launch (one launch per mesh); x pass + binning: one launch
    kern = {"assign": (phases_ms[0], ab["nmesh"] * ab["assign"]),
            "pass_z": (phases_ms[1] / ab["nmesh"], ab["pass_z"]),
            "pass_y": (phases_ms[2] / ab["nmesh"], ab["pass_y"]),
            "pass_x_bin": (phases_ms[3], ab["pass_x_bin"])}
    dom = max(kern, key=lambda k: kern[k][0])
    ms, nbytes = kern[dom]
    achieved = nbytes / (ms * 1e-3) / 1e9
    # the assignment's real limit is shared-memory atomics: stencil node updates/s
    nodes = n * (assign + 1) ** 3 * ab["nmesh"]
    atom = {"node_updates_per_s": nodes / (phases_ms[0] * 1e-3), "per_eval": nodes}
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
            "assign_atomics": atom,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "traffic": (traffic or {}).get(f"ng{ng}", {}).get(dom),
            "per_kernel_frac": {k: (v[1] / (v[0] * 1e-3) / 1e9) / peak for k, v in kern.items()},
            "eval_algorithmic_GB": ab["total"] / 1e9,
            "eval_frac": ab["total"] / (phases_ms[5] * 1e-3) / 1e9 / peak}


def cpu_eval(cat, threads=None, ref=None):
    """One plain evaluation (default Ng = 1024 PCS interlaced) with the
    oracle's C restatement (FP64, OpenMP); returns (seconds, result)."""
    import oracle
    if threads:
        oracle.set_threads(threads)
    ref = ref or PLAIN_REF
    spec = oracle.Spec(ng=ref["ng"], box=BOX, assign=ref["assign"],
                       interlace=ref["interlace"], poles=(0, 2, 4), dk=DK,
                       isauto=(True, False), iscross=False)
    t0 = time.perf_counter()
    res = oracle.run("port", spec, [cat])
    return time.perf_counter() - t0, res


def parity(got, ref):
    """Error of a GPU evaluation against the FP64 oracle on the same
    catalogue: mode counts bit-exact?, max |dP_l| / (|P_0| + shot) over every
    bin, max |dP_l| / |P_0| over the bins where |P_0| >= shot, and over
    every bin (unbounded where P_0, shot noise subtracted, crosses 0)."""
    d = np.abs(got.pl[0] - ref.pl[0])
    p0 = np.abs(ref.pl[0][0])
    strong = p0 >= ref.shot[0]
    with np.errstate(divide="ignore", invalid="ignore"):
        every = float(np.nanmax(d / p0))
    return {"counts_exact": bool(np.array_equal(got.cnt, ref.cnt)),
            "max_dP_over_P0_plus_shot": float((d / (p0 + ref.shot[0])).max()),
            "max_dP_over_P0": float((d[:, strong] / p0[strong]).max()) if strong.any() else None,
            "bins_P0_ge_shot": int(strong.sum()), "bins": int(len(p0)),
            "max_dP_over_P0_every_bin": every, "tolerance": 1e-5,
            "oracle": "FP64 C restatement of the reference (bit-identical to it at one thread)"}


def ensemble_plan(seed):
    """Seeded (n, ng, assign) of each ensemble catalogue."""
    rng = np.random.default_rng(seed + 4242)
    n = np.exp(rng.uniform(np.log(ENS_NMIN), np.log(ENS_NMAX), ENS_NCAT)).astype(np.int64)
    ng = rng.choice(ENS_NG, ENS_NCAT)
    asg = rng.choice(ENS_ASSIGN, ENS_NCAT)
    return [(int(a), int(b_), int(c)) for a, b_, c in zip(n, ng, asg)]


def _ens_cat(args):
    from powspec_gb300 import catalog
    n, seed = args
    return catalog.lognormal(n, box=BOX, seed=seed, ngen=128)


def make_ensemble(seed):
    """The ensemble's catalogues (spawn pool: the caller has not touched the GPU)."""
    import multiprocessing as mp
    plan = ensemble_plan(seed)
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        cats = pool.map(_ens_cat, [(n, seed * 100000 + i) for i, (n, _, _) in enumerate(plan)],
                        chunksize=4)
    return plan, cats


def config_of(wl, n_actual):
    w = WORKLOADS[wl]
    if w.get("large"):
        return {"workload": wl, "ng": w["ng"], "assign": "PCS", "interlace": True,
                "n_particles": n_actual, "positions": "float32 SoA", "weights": "float32 U[0.5, 1.5]",
                "box": LARGE_BOX, "dk": LARGE_DK, "poles": [0, 2, 4], "catalogue": "lognormal (ngen 256)",
                "seed": SEED, "l2": "working set per eval >> 129 MB L2; no explicit flush"}
    if w.get("ensemble"):
        return {"workload": wl, "catalogues": ENS_NCAT, "n_particles_total": n_actual,
                "n_range": [ENS_NMIN, ENS_NMAX], "ng_choices": list(ENS_NG),
                "assign_choices": ["CIC", "TSC"], "interlace": True, "box": BOX, "dk": DK,
                "poles": [0, 2, 4], "catalogue": "lognormal (ngen 128)", "seed": SEED,
                "l2": "working set per group >> 129 MB L2; no explicit flush"}
    c = {"workload": wl, "ng": w["ng"], "assign": ["NGP", "CIC", "TSC", "PCS"][w["assign"]],
         "interlace": w["interlace"], "n_particles": n_actual, "box": BOX, "dk": DK,
         "poles": [0, 2, 4], "catalogue": "lognormal", "seed": SEED,
         "l2": "working set per eval >> 129 MB L2 (FP32 meshes 4 B/cell + 8 B/mode "
               "complex passes + 112 B/particle records); no explicit flush"}
    if w["learned"]:
        c.update({"nmu": 16, "compared_with": "plain Ng=1024 PCS interlaced, same catalogue",
                  "kmax": f"0.8 k_Nyq({w['ng']})"})
    return c


def run_reference_ensemble(args):
    """The oracle port over the ensemble's catalogues, in order, until the
    time cap: the same per-catalogue evaluations the GPU arm batches."""
    import oracle
    plan, cats = make_ensemble(SEED)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    small = oracle.Spec(ng=64, box=BOX, assign=1, interlace=True, poles=(0, 2, 4), dk=DK,
                        isauto=(True, False), iscross=False)
    for _ in range(args.warmup):
        oracle.run("port", small, [cats[0]])
    t0 = time.perf_counter()
    done = 0
    for (n, ng, a), cat in zip(plan, cats):
        spec = oracle.Spec(ng=ng, box=BOX, assign=a, interlace=True, poles=(0, 2, 4), dk=DK,
                           isauto=(True, False), iscross=False)
        oracle.run("port", spec, [cat])
        done += 1
        if time.perf_counter() - t0 > 150.0:
            break
    total = time.perf_counter() - t0
    value = done / total
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": 1, "warmup": args.warmup, "ms_per_step": 1e3 * total / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(args.workload, int(sum(len(c) for c in cats))),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"the first {done} of {len(cats)} ensemble catalogues, "
                                   "150 s cap; FFT by the project's FFTW-API shim"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def run_reference_large(args):
    """The oracle port on the large single-mesh workload: one bounded
    evaluation at Ng = 1024; Ng = 2048 does not fit the FP64 meshes in host
    memory."""
    wl = WORKLOADS[args.workload]
    if wl["ng"] > 1024:
        print(json.dumps({"impl": "reference", "unavailable": "the FP64 reference at Ng=2048 "
                          "needs about 0.3 TB of host memory for its meshes"}))
        return 0
    import oracle
    from powspec_gb300 import catalog
    x, y, z, w = catalog.lognormal(LARGE_N, box=LARGE_BOX, seed=SEED, ngen=256,
                                   weights=(0.5, 1.5), soa=True)
    cat = np.stack([x, y, z, w], axis=1).astype(np.float64)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    spec = oracle.Spec(ng=wl["ng"], box=LARGE_BOX, assign=wl["assign"], interlace=wl["interlace"],
                       poles=(0, 2, 4), dk=LARGE_DK, isauto=(True, False), iscross=False)
    t0 = time.perf_counter()
    oracle.run("port", spec, [cat])
    total = time.perf_counter() - t0
    value = 1.0 / total
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * total,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(args.workload, len(cat)),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": "one evaluation of the workload's catalogue; FFT by the "
                                   "project's FFTW-API shim"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    if WORKLOADS[args.workload].get("ensemble"):
        return run_reference_ensemble(args)
    if WORKLOADS[args.workload].get("large"):
        return run_reference_large(args)
    if WORKLOADS[args.workload].get("survey"):
        return run_reference_survey(args)
    import oracle
    cat = make_catalogue(SEED)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    small = oracle.Spec(ng=128, box=BOX, assign=3, interlace=True, poles=(0, 2, 4), dk=DK,
                        isauto=(True, False), iscross=False)
    for _ in range(args.warmup):  # warm-up: small evaluations of the same catalogue
        oracle.run("port", small, [cat])
    times = []
    wl = WORKLOADS[args.workload]
    pref = PLAIN_REF if wl["learned"] else dict(ng=wl["ng"], assign=wl["assign"],
                                                 interlace=wl["interlace"])
    for _ in range(args.steps):
        times.append(cpu_eval(cat, ref=pref)[0])
        if sum(times) > 150.0:  # bounded sample: keep the run within a few minutes
            break
    total = sum(times)
    value = len(times) / total
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": len(times), "steps_requested": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(args.workload, len(cat)),
        "reference_computes": f"plain Ng={pref['ng']} PCS interlaced (genr_mesh + powspec)",
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} full evaluation(s), 150 s cap; FFT by the "
                                   "project's FFTW-API shim, not FFTW"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def timed(stream, steps, fn, many=None):
    """Device time (CUDA events on the context stream) of `steps` calls, or
    of one call many(steps) that runs them back to back."""
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    out = None
    if many is not None:
        out = many(steps)
    else:
        for _ in range(steps):
            out = fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), out


def run_gpu(args, world, rank, local):
    import torch

    import powspec_gb300 as ps
    from powspec_gb300 import learned
    wl = WORKLOADS[args.workload]
    torch.cuda.set_device(local)
    cat = make_catalogue(SEED + rank)
    nreal = len(cat)
    d_cat = torch.from_numpy(cat).to(f"cuda:{local}")
    pinned = torch.from_numpy(cat).pin_memory()
    host_arr = pinned.numpy()
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        with open(tf) as f:
            traffic = json.load(f)

    # plain fine-mesh context (the reference method; timed for comparison)
    pref = PLAIN_REF if wl["learned"] else dict(ng=wl["ng"], assign=wl["assign"],
                                                 interlace=wl["interlace"])
    plain = ps.Estimator(ng=pref["ng"], box=BOX, assign=pref["assign"],
                         interlace=pref["interlace"], poles=(0, 2, 4), dk=DK, device=local)
    s_plain = torch.cuda.ExternalStream(plain.stream(), device=local)
    phases_plain = np.zeros(6)
    tuning = {"plain": plain.autotune(d_cat.data_ptr(), nreal)}  # set-up, not timed

    rp_last = [None]

    def step_plain():
        plain.assign(0, d_cat.data_ptr(), on_device=True, n=nreal)
        r = plain.execute()
        phases_plain[:] += plain.timings()
        rp_last[0] = r
        return r

    if wl["learned"]:
        le = learned.LearnedEstimator(ng=wl["ng"], assign=wl["assign"], interlace=wl["interlace"],
                                      box=BOX, dk=DK, device=local)
        tuning["learned"] = le.autotune(d_cat.data_ptr(), nreal)
        stream = torch.cuda.ExternalStream(le.est.stream(), device=local)
        phases = np.zeros(6)
        launches = [0]

        def step():
            out = le.run(device_ptr=d_cat.data_ptr(), n=nreal)
            phases[:] += le.est.timings()
            launches[0] += le.est.launches()  # passes, features, network, combine
            return out

        def step_many(k):
            # k evaluations back to back on two contexts (LearnedEstimator.
            # run_many, lanes=2): each next assignment enqueued before the
            # previous results are waited for, two evaluations in flight.
            # Phase times come from evaluations run alone (below): with two
            # in flight each context's events also span the other's kernels.
            res = le.run_many([d_cat.data_ptr()] * k, nreal, lanes=LEARNED_LANES)
            launches[0] += le.est.launches() * k
            return res[-1]

        def e2e_stream(k):
            return le.run_stream(itertools.repeat(host_arr, k), lanes=LEARNED_LANES)
    else:
        le = None
        step_many = None
        stream, phases, launches = s_plain, phases_plain, [0]

        def step():
            r = step_plain()
            launches[0] += plain.launches()
            return r

        def e2e_stream(k):
            return plain.run_stream(itertools.repeat(host_arr, k))

    for _ in range(args.warmup):
        step()
        if le is not None:
            step_plain()
    if step_many is not None:
        step_many(2 * LEARNED_LANES)  # sets up and warms the second context too
    phases[:] = 0
    phases_plain[:] = 0
    launches[0] = 0

    with ClockSampler(local) as clk:
        barrier(world)
        dev_ms, out = timed(stream, args.steps, step, many=step_many)
        barrier(world)
    clocks = clk.summary()
    nlaunch = launches[0]
    if step_many is not None:  # phase times of evaluations run alone
        phases[:] = 0
        nalone = 3
        for _ in range(nalone):
            step()
        ph = phases / nalone
    else:
        ph = phases / args.steps
    t_max = reduce(world, dev_ms / 1e3, "max")
    value = reduce(world, float(args.steps), "sum") / t_max

    extra = {}
    if le is not None:
        # plain Ng = 1024 on the same catalogue: throughput and the error of the learned form
        phases_plain[:] = 0
        pl_ms, rp = timed(s_plain, args.steps, step_plain)
        k, pc, trusted = out
        ref = rp.pl[0][:, :len(k)]
        use = trusted & (rp.cnt[:len(k)] > 1) & (ref[0] > 0)
        err = np.abs(pc - ref)[:, use] / ref[0][use]
        err_plain = np.abs(le.last_cells.plain - ref)[:, use] / ref[0][use]
        plain_value = reduce(world, float(args.steps), "sum") / reduce(world, pl_ms / 1e3, "max")
        # the same coarse mesh without the correction (plain method, no |mu|
        # sub-bins, no network), timed on the same catalogue
        cg = wl["ng"]
        coarse = ps.Estimator(ng=cg, box=BOX, assign=wl["assign"], interlace=wl["interlace"],
                              poles=(0, 2, 4), dk=DK, device=local)
        coarse.autotune(d_cat.data_ptr(), nreal)
        s_coarse = torch.cuda.ExternalStream(coarse.stream(), device=local)

        def step_coarse():
            coarse.assign(0, d_cat.data_ptr(), on_device=True, n=nreal)
            return coarse.execute()

        for _ in range(args.warmup):
            step_coarse()
        co_ms, rco = timed(s_coarse, args.steps, step_coarse)
        coarse.close()
        err_co = np.abs(rco.pl[0][:, :len(k)] - ref)[:, use] / ref[0][use]
        coarse_value = reduce(world, float(args.steps), "sum") / reduce(world, co_ms / 1e3, "max")
        kmax = 0.8 * np.pi * cg / BOX
        extra["learned"] = {
            "plain_ng1024_evals_per_s": plain_value,
            "speedup_vs_plain_ng1024": value / plain_value,
            "max_err_vs_plain_ng1024": float(err.max()),
            "max_err_by_l": [float(v) for v in err.max(1)],
            f"max_err_uncorrected_ng{cg}": float(err_plain.max()),
            f"plain_ng{cg}_evals_per_s": coarse_value,
            f"plain_ng{cg}_max_err_vs_plain_ng1024": float(err_co.max()),
            "bins_compared": int(use.sum()),
            "bins_not_trusted_below_kmax": int((~trusted[:int(np.sum(k <= kmax))]).sum()),
            "bins_from_fine_fallback": int(le.last_fallback.sum()),
            "tolerance": 0.01,
        }
        extra["roofline_plain_ng1024"] = roofline(phases_plain / args.steps, 1024, True, nreal, traffic)

    # End to end through the public API with host (pinned) buffers: every
    # step copies its catalogue in (staged, overlapping the step before) and
    # reads its result back.  Staging slots allocated untimed first.
    for _ in e2e_stream(4):  # both slots of up to two contexts
        pass
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in e2e_stream(args.steps):
        pass
    torch.cuda.synchronize()
    e2e_s = reduce(world, time.perf_counter() - t0, "max")
    e2e = reduce(world, float(args.steps), "sum") / e2e_s
    if le is not None:
        d2h = 8 * 3 * le.est.nbin * 16 + 8 * 4 + 16 + 4 * le.est.nbin * 16
    else:
        d2h = 8 * 3 * plain.nbin + 8 * 4 + 16

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(args.workload, nreal),
            "phases_ms": {"assign": ph[0], "pass_z": ph[1], "pass_y": ph[2], "pass_x_bin": ph[3],
                          "reduce": ph[4], "device_total": ph[5]},
            "roofline": roofline(ph, wl["ng"], wl["interlace"], nreal, traffic),
            "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": nreal * 32,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": nlaunch, "clocks": clocks, "autotune": tuning,
        }
        line.update(extra)
        if world == 1 and not args.no_cpu:
            cpu_s, cpu_res = cpu_eval(cat, threads=os.cpu_count(), ref=pref)
            # the plain evaluation's error against the FP64 oracle, same catalogue
            line["parity"] = dict(parity(rp_last[0], cpu_res),
                                  evaluation=f"plain Ng={pref['ng']} PCS interlaced")
            line["cpu_baseline"] = {
                "value": 1.0 / cpu_s, "unit": "evals/s", "cores": os.cpu_count(), "kind": "port",
                "sample": "one plain Ng=1024 PCS interlaced evaluation of the same catalogue "
                          "(FP64 OpenMP restatement of the reference; FFT by the project's "
                          "FFTW-API shim)"}
        print(json.dumps(line))
    if le is not None:
        le.close()
    plain.close()
    return 0


def run_ensemble(args, world, rank, local):
    plan, cats = make_ensemble(SEED + rank)  # before any GPU call (spawn pool)
    import torch

    from powspec_gb300.ensemble import Ensemble
    torch.cuda.set_device(local)
    dev = [torch.from_numpy(c).to(f"cuda:{local}") for c in cats]
    pinned = [torch.from_numpy(c).pin_memory() for c in cats]
    configs = [(ng, a, True) for _, ng, a in plan]
    ntot = int(sum(len(c) for c in cats))
    t0 = time.perf_counter()
    ens = Ensemble(dev, configs, box=BOX, dk=DK, device=local)
    setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        ens.run()
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ens.launch()
            ens.wait()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        barrier(world)
    out = ens.results()
    t_max = reduce(world, el, "max")
    value = reduce(world, float(args.steps * len(cats)), "sum") / t_max
    # the per-context graphs launched one by one (each on its context's stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ens.launch_groups()
        ens.wait_groups()
    torch.cuda.synchronize()
    groups_value = reduce(world, float(args.steps * len(cats)), "sum") / reduce(
        world, time.perf_counter() - t0, "max")
    # the same evaluations one catalogue at a time (host round trip each)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = ens.run_plain()
    torch.cuda.synchronize()
    plain_s = reduce(world, time.perf_counter() - t0, "max")
    plain_value = reduce(world, float(len(cats)), "sum") / plain_s
    err = 0.0
    for g, r in zip(out, ref):
        use = r.cnt > 0
        scale = np.abs(r.pl[0][0][use]) + r.shot[0]
        err = max(err, float((np.abs(g.pl[0][:, use] - r.pl[0][:, use]) / scale).max()))
    # end to end: host catalogues copied in (pinned), graphs, results out
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for d, h in zip(dev, pinned):
            d.copy_(h, non_blocking=True)
        torch.cuda.synchronize()
        ens.launch()
        ens.wait()
        ens.results()
    e2e_s = reduce(world, time.perf_counter() - t0, "max")
    e2e = reduce(world, float(args.steps * len(cats)), "sum") / e2e_s
    nlaunch = ens.launches() * args.steps
    # algorithmic bytes of all evaluations (assignment, 3 FFT passes, binning)
    tot = 0
    for (n, ng, a), c in zip(plan, cats):
        tot += algorithmic_bytes(ng, True, len(c))["total"]
    peak, peak_kind = peaks()
    achieved = tot * args.steps / el / 1e9
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(args.workload, ntot),
            "step": "one step = all 256 catalogues: ONE launch of the ensemble graph, whose "
                    "child graphs (one per context; each configuration group split over up to "
                    "4 contexts) run concurrently",
            "groups": {f"ng{k[0]}_{['NGP', 'CIC', 'TSC', 'PCS'][k[1]]}": len(v)
                       for k, v in ens.groups.items()},
            "contexts": len(ens.lanes),
            "per_context_graph_launches_evals_per_s": groups_value,
            "autotune": {f"ng{k[0]}_{['NGP', 'CIC', 'TSC', 'PCS'][k[1]]}": v
                         for k, v in ens.tuning.items()},
            "setup_s": setup_s,
            "plain_per_catalogue_evals_per_s": plain_value,
            "speedup_vs_per_catalogue": value / plain_value,
            "max_err_vs_per_catalogue": err,
            "roofline": {"bound": "hbm", "kernel": "whole ensemble (all kernels)",
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": None},
            "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": ntot * 32,
                    "d2h_bytes_per_step": int(sum(len(part) * (3 * e.nbin + 6) * 8
                                                  for _, part, e, _ in ens.lanes))},
            "gpu_launches": nlaunch, "clocks": clk.summary(),
        }
        print(json.dumps(line))
    ens.close()
    return 0


def run_large(args, world, rank, local):
    import torch

    import powspec_gb300 as ps
    from powspec_gb300 import catalog
    wl = WORKLOADS[args.workload]
    x, y, z, w = catalog.lognormal(LARGE_N, box=LARGE_BOX, seed=SEED + rank, ngen=256,
                                   weights=(0.5, 1.5), soa=True)
    n = len(x)
    torch.cuda.set_device(local)
    dev = [torch.from_numpy(v).to(f"cuda:{local}") for v in (x, y, z, w)]
    host = [torch.from_numpy(v).pin_memory().numpy() for v in (x, y, z, w)]
    est = ps.Estimator(ng=wl["ng"], box=LARGE_BOX, assign=wl["assign"], interlace=wl["interlace"],
                       poles=(0, 2, 4), dk=LARGE_DK, device=local)
    stream = torch.cuda.ExternalStream(est.stream(), device=local)
    phases = np.zeros(6)
    launches = [0]

    def step():
        est.assign(0, x=dev[0].data_ptr(), y=dev[1].data_ptr(), z=dev[2].data_ptr(),
                   w=dev[3].data_ptr(), on_device=True, n=n)
        r = est.execute()
        phases[:] += est.timings()
        launches[0] += est.launches()
        return r

    for _ in range(args.warmup):
        step()
    phases[:] = 0
    launches[0] = 0
    with ClockSampler(local) as clk:
        barrier(world)
        dev_ms, _ = timed(stream, args.steps, step)
        barrier(world)
    ph = phases / args.steps
    t_max = reduce(world, dev_ms / 1e3, "max")
    value = reduce(world, float(args.steps), "sum") / t_max
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        est.assign(0, x=host[0], y=host[1], z=host[2], w=host[3])
        est.execute()
    e2e_s = reduce(world, time.perf_counter() - t0, "max")
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(args.workload, n),
            "phases_ms": {"assign": ph[0], "pass_z": ph[1], "pass_y": ph[2], "pass_x_bin": ph[3],
                          "reduce": ph[4], "device_total": ph[5]},
            "roofline": roofline(ph, wl["ng"], wl["interlace"], n, None, wl["assign"], bp=16),
            "e2e": {"value": args.steps / e2e_s, "unit": "evals/s", "h2d_bytes_per_step": n * 16,
                    "d2h_bytes_per_step": 8 * 3 * est.nbin + 8 * 4 + 16},
            "gpu_launches": launches[0], "clocks": clk.summary(),
            "cpu_baseline": None,
            "cpu_baseline_note": ("the FP64 reference at Ng=2048 needs about 0.3 TB of host memory"
                                  if wl["ng"] > 1024 else
                                  "one FP64 evaluation of 1.5e8 particles exceeds the few-minute "
                                  "sample budget of this run: bench.py --impl reference times it"),
        }
        print(json.dumps(line))
    est.close()
    return 0


def survey_bytes(ng, poles, interlace, n):
    """Algorithmic HBM bytes of one survey evaluation's phases.

    assignment: as for a periodic box; F_0: one r2c per mesh (4 B Ng^3 read,
    8 B Ncmplx written), with interlacing the combination and its c2r (8 B
    Ncmplx per field read, 4 B Ng^3 written); each harmonic term (2l + 1 per
    l > 0): the weighted mesh read (4 B Ng^3), its transform written and read
    (16 B Ncmplx), the field accumulated (16 B Ncmplx); each (F_0, F_l) pair
    binned: 16 B Ncmplx.
    """
    nmesh = 2 if interlace else 1
    ntot, ncx = ng ** 3, ng * ng * (ng // 2 + 1)
    terms = sum(2 * l + 1 for l in poles if l > 0)
    f0 = nmesh * (4 * ntot + 8 * ncx) + ((16 * ncx + 4 * ntot) if interlace else 0)
    harm = terms * (4 * ntot + 32 * ncx) + len(poles) * 16 * ncx
    return {"assign": nmesh * (n * 32 + 4 * ntot), "f0": f0, "harmonics": harm, "terms": terms}


def make_survey(seed):
    from powspec_gb300 import catalog
    d, r = catalog.survey(SURVEY_ND, centre=SURVEY_CENTRE, radius=SURVEY_RADIUS, seed=seed,
                          ngen=256)
    return catalog.prepare_survey([(d, r)])[0], len(d), len(r)


def survey_config(name, s, nd, nr):
    wl = WORKLOADS[name]
    return {"workload": name, "ng": wl["ng"], "assign": "PCS", "interlace": wl["interlace"],
            "poles": list(wl["poles"]), "box": list(s.box), "n_data": nd, "n_rand": nr, "dk": DK,
            "l2": "no flush: each evaluation's working set (128 MB of records, two 64 MB "
                  "meshes, seven 68 MB fields) is about 1 GB, far above the 129 MB L2"}


def survey_oracle_spec(name, s):
    import oracle
    wl = WORKLOADS[name]
    return oracle.Spec(ng=wl["ng"], box=s.box, assign=wl["assign"], interlace=wl["interlace"],
                       poles=wl["poles"], dk=DK, isauto=(True, False), iscross=False)


def run_reference_survey(args):
    """The oracle port's survey path on the survey workload's catalogue."""
    import oracle
    s, nd, nr = make_survey(SEED)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    spec = survey_oracle_spec(args.workload, s)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.survey(spec, [s.xyzw], s.origin, [s.shot], [s.norm])
        times.append(time.perf_counter() - t0)
        if sum(times) > 150.0:
            break
    total = sum(times)
    value = len(times) / total
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": len(times), "steps_requested": args.steps, "warmup": 0,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": survey_config(args.workload, s, nd, nr),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} evaluation(s) of the workload's catalogue, "
                                   "150 s cap; FFT by the project's FFTW-API shim"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def run_survey(args, world, rank, local):
    import torch

    import powspec_gb300 as ps
    wl = WORKLOADS[args.workload]
    s, nd, nr = make_survey(SEED + rank)
    n = len(s.xyzw)
    torch.cuda.set_device(local)
    dev = torch.from_numpy(s.xyzw).to(f"cuda:{local}")
    host = torch.from_numpy(s.xyzw).pin_memory().numpy()
    est = ps.Estimator(ng=wl["ng"], box=s.box, assign=wl["assign"], interlace=wl["interlace"],
                       poles=wl["poles"], dk=DK, device=local)
    est.set_survey(0, s.shot, s.norm, s.origin)
    stream = torch.cuda.ExternalStream(est.stream(), device=local)
    phases = np.zeros(6)
    launches = [0]

    def step():
        est.assign(0, dev.data_ptr(), on_device=True, n=n)
        out = est.execute()
        phases[:] += est.timings()
        launches[0] += est.launches()
        return out

    for _ in range(args.warmup):
        step()
    phases[:] = 0
    launches[0] = 0
    with ClockSampler(local) as clk:
        barrier(world)
        dev_ms, _ = timed(stream, args.steps, step)
        barrier(world)
    ph = phases / args.steps
    t_max = reduce(world, dev_ms / 1e3, "max")
    value = reduce(world, float(args.steps), "sum") / t_max
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        est.assign(0, host)
        est.execute()
    e2e_s = reduce(world, time.perf_counter() - t0, "max")
    if rank == 0:
        ab = survey_bytes(wl["ng"], wl["poles"], wl["interlace"], n)
        peak, peak_kind = peaks()
        frac = lambda b, ms: (b / (ms * 1e-3) / 1e9) / peak if ms > 0 else None
        cpu = None
        if not args.no_cpu:
            import oracle
            spec = survey_oracle_spec(args.workload, s)
            t0 = time.perf_counter()
            reps = 2
            for _ in range(reps):
                oracle.survey(spec, [s.xyzw], s.origin, [s.shot], [s.norm])
            cpu = {"value": reps / (time.perf_counter() - t0), "unit": "evals/s",
                   "cores": oracle.get_threads(), "kind": "port",
                   "sample": f"{reps} FP64 evaluations of the same survey catalogue and mesh"}
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": survey_config(args.workload, s, nd, nr),
            "phases_ms": {"assign": ph[0], "f0_and_c2r": ph[1], "harmonics_and_binning": ph[3],
                          "device_total": ph[5]},
            "roofline": {"bound": "hbm", "kernel": "harmonic terms (weight, r2c, accumulate) "
                         "and pair binning", "achieved": ab["harmonics"] / (ph[3] * 1e-3) / 1e9,
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": frac(ab["harmonics"], ph[3]), "traffic": None,
                         "per_phase_frac": {"assign": frac(ab["assign"], ph[0]),
                                            "f0_and_c2r": frac(ab["f0"], ph[1]),
                                            "harmonics_and_binning": frac(ab["harmonics"], ph[3])},
                         "harmonic_terms": ab["terms"]},
            "e2e": {"value": args.steps / e2e_s, "unit": "evals/s", "h2d_bytes_per_step": n * 32,
                    "d2h_bytes_per_step": 8 * 3 * est.nbin + 8 * 4 + 16},
            "gpu_launches": launches[0], "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    est.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_init()
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    elif WORKLOADS[args.workload].get("ensemble"):
        rc = run_ensemble(args, world, rank, local)
    elif WORKLOADS[args.workload].get("large"):
        rc = run_large(args, world, rank, local)
    elif WORKLOADS[args.workload].get("survey"):
        rc = run_survey(args, world, rank, local)
    else:
        rc = run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
