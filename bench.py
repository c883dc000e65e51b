"""Benchmark of the periodic-box P_l(k) path on GB300.

One step = one evaluation: a catalogue -> {P_0, P_2, P_4}(k) table (particle
assignment into two interlaced meshes, the r2c FFTs, interlace combine,
window compensation and Legendre binning, normalisation).

Workload (default): the plain form of the learned-vs-plain comparison: a
seeded lognormal catalogue of ~4e6 particles (spectrum A k^-1.5
exp(-(k/0.5)^2), sigma_G^2 = 1, Zel'dovich displacement along z), L = 1000
Mpc/h, PCS with interlacing at Ng = 1024, l = 0, 2, 4, dk = 0.005 h/Mpc.
Synthetic data stands in for simulation catalogues (none ship with the
reference).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank evaluates its own catalogues on its GPU
(replicas: the path has no exchange step); value = all evaluations / max
time over ranks.

--impl reference times the reference's CPU path: the oracle's FP64 OpenMP C
restatement of genr_mesh + powspec (the reference sources are not available
on the GPU machine), on rank 0 only, with all host threads.
"""
from __future__ import annotations

import argparse
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

WORKLOADS = {
    # name: (ng, assign, interlace, n_particles, box, dk, ngen)
    "plain_pcs_il_ng1024_n4e6": (1024, 3, True, 4_000_000, 1000.0, 0.005, 256),
    "plain_pcs_il_ng512_n4e6": (512, 3, True, 4_000_000, 1000.0, 0.005, 256),
    "plain_cic_ng256_n1e6_uniform": (256, 1, False, 1_000_000, 1000.0, 0.005, 0),
}
DEFAULT = "plain_pcs_il_ng1024_n4e6"
METRIC = "P_l(k) evals/s on 1 GB300"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_catalogue(wl, seed):
    from powspec_gb300 import catalog
    ng, assign, il, n, box, dk, ngen = WORKLOADS[wl]
    if ngen == 0:
        return catalog.uniform(n, box=box, seed=seed)
    return catalog.lognormal(n, box=box, seed=seed, ngen=ngen)


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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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


def allmax(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def algorithmic_bytes(wl, n):
    """Per-launch algorithmic HBM bytes of each phase (FP32 path).

    assignment: N * 32 B (AoS float64 records) + 4 B * Ng^3 per mesh;
    z pass: 4 B * Ng^3 read + 8 B * Ncmplx written; y pass: 8 B * Ncmplx
    read + written; x pass + binning: 8 B * Ncmplx per field read.
    """
    ng, assign, il, _, box, dk, _ = WORKLOADS[wl]
    nmesh = 2 if il else 1
    ntot = ng ** 3
    ncx = ng * ng * (ng // 2 + 1)
    return {
        "assign": n * 32 + 4 * ntot,          # per launch (one mesh)
        "pass_z": 4 * ntot + 8 * ncx,         # per launch (one field)
        "pass_y": 16 * ncx,                   # per launch (one field)
        "pass_x_bin": 8 * ncx * nmesh,        # one launch over all fields
        "nmesh": nmesh,
        "total": nmesh * (n * 32 + 4 * ntot) + nmesh * (4 * ntot + 8 * ncx) + nmesh * 8 * ncx * 2,
    }


def cpu_eval(wl, cat, threads=None):
    """One evaluation with the oracle's C restatement (FP64, OpenMP)."""
    import oracle
    ng, assign, il, n, box, dk, _ = WORKLOADS[wl]
    if threads:
        oracle.set_threads(threads)
    spec = oracle.Spec(ng=ng, box=box, assign=assign, interlace=il, poles=(0, 2, 4), dk=dk,
                       isauto=(True, False), iscross=False)
    t0 = time.perf_counter()
    oracle.run("port", spec, [cat])
    return time.perf_counter() - t0


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    import oracle
    wl = args.workload
    cat = make_catalogue(wl, seed=1)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    ng, assign, il, n, box, dk, _ = WORKLOADS[wl]
    # warm-up: W small evaluations of the same catalogue (Ng = 128)
    small = oracle.Spec(ng=128, box=box, assign=assign, interlace=il, poles=(0, 2, 4), dk=dk,
                        isauto=(True, False), iscross=False)
    for _ in range(args.warmup):
        oracle.run("port", small, [cat])
    times = []
    budget = 180.0
    for _ in range(args.steps):
        times.append(cpu_eval(wl, cat))
        if sum(times) > budget:
            break
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": len(times), "steps_requested": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(wl, n_actual=len(cat)),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} full evaluation(s) of the workload, "
                                   f"180 s cap; FFT by the project's FFTW-API shim"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def config_of(wl, n_actual):
    ng, assign, il, n, box, dk, ngen = WORKLOADS[wl]
    return {"workload": wl, "ng": ng, "assign": ["NGP", "CIC", "TSC", "PCS"][assign],
            "interlace": il, "n_particles": n_actual, "box": box, "dk": dk, "poles": [0, 2, 4],
            "catalogue": "lognormal" if ngen else "uniform",
            "l2": "working set per eval >> 129 MB L2 (int64 meshes 8 B/cell); no explicit flush"}


def run_gpu(args, world, rank, local):
    import torch

    import powspec_gb300 as ps
    wl = args.workload
    ng, assign, il, n, box, dk, _ = WORKLOADS[wl]
    torch.cuda.set_device(local)
    cat = make_catalogue(wl, seed=1 + rank)
    nreal = len(cat)
    est = ps.Estimator(ng=ng, box=box, assign=assign, interlace=il, poles=(0, 2, 4), dk=dk,
                       device=local)
    stream = torch.cuda.ExternalStream(est.stream(), device=local)
    d_cat = torch.from_numpy(cat).to(f"cuda:{local}")
    torch.cuda.synchronize()

    def step_device():
        est.assign(0, d_cat.data_ptr(), on_device=True, n=nreal)
        return est.execute()

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()

    # ---- device-resident timed region
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    phases = np.zeros(6)
    launches = 0
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step_device()
            phases += est.timings()
            launches += est.launches()
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    dev_ms = ev0.elapsed_time(ev1)
    clocks = clk.summary()
    t_max = allmax(world, dev_ms / 1e3)
    evals = allsum(world, float(args.steps))
    value = evals / t_max

    # ---- end to end through the public API with host buffers (pinned)
    pinned = torch.from_numpy(cat).pin_memory()
    host_arr = pinned.numpy()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        est.assign(0, host_arr)
        res = est.execute()
    torch.cuda.synchronize()
    e2e_s = allmax(world, time.perf_counter() - t0)
    e2e = allsum(world, float(args.steps)) / e2e_s
    d2h = 8 * 3 * est.nbin + 8 * 4 + 4 * 2  # sums, weight sums, error flags
    est.close()

    if rank != 0:
        return 0
    peak, peak_kind = peaks()
    ab = algorithmic_bytes(wl, nreal)
    per = phases / args.steps  # ms per eval: assign, z, y, x+bin, reduce, total
    kern = {
        "assign": (per[0] / ab["nmesh"], ab["assign"]),
        "pass_z": (per[1] / ab["nmesh"], ab["pass_z"]),
        "pass_y": (per[2] / ab["nmesh"], ab["pass_y"]),
        "pass_x_bin": (per[3], ab["pass_x_bin"]),
    }
    dom = max(kern, key=lambda k: kern[k][0])
    ms, nbytes = kern[dom]
    achieved = nbytes / (ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config_of(wl, nreal),
        "phases_ms": {"assign": per[0], "pass_z": per[1], "pass_y": per[2],
                      "pass_x_bin": per[3], "reduce": per[4], "total": per[5]},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": args.traffic.get(dom) if args.traffic else None,
                     "eval_algorithmic_GB": ab["total"] / 1e9,
                     "eval_frac": ab["total"] / (t_max / args.steps * world) / 1e9 / peak},
        "e2e": {"value": e2e, "unit": "evals/s", "h2d_bytes_per_step": nreal * 32,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu:
        cpu_s = cpu_eval(wl, cat, threads=os.cpu_count())
        line["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "evals/s", "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": "one full evaluation of the workload (FP64 OpenMP "
                                          "restatement; FFT by the project's FFTW-API shim)"}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--traffic", type=json.loads, default=None,
                    help='per-kernel ncu DRAM bytes per launch, e.g. {"pass_z": 1.2e10}')
    args = ap.parse_args()
    if args.traffic is None:
        # ncu DRAM read+write bytes per launch, summarised under profiles/
        tf = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.json")
        if os.path.exists(tf):
            with open(tf) as f:
                args.traffic = json.load(f).get("bytes_per_launch")
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_init()
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    else:
        rc = run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
