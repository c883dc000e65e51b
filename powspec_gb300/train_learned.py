"""Train the learned alias correction on the GPU and write its weights.

    python -m powspec_gb300.train_learned [--ntrain 48] [--nheld 16] [--steps 20000]

1. seeded lognormal catalogues (N = 4e6, L = 1000 Mpc/h, spectrum
   A k^-1.5 exp(-(k/0.5)^2), sigma_G^2 = 1, Zel'dovich displacement along z),
   generated by a spawn process pool while the GPU measures the previous ones;
2. labels: the plain estimator at Ng = 1024, PCS, interlaced; features: the
   plain estimator at Ng = 128 and 256 with CIC / TSC / PCS, interlacing
   on and off, with 16 |mu| sub-bins;
3. Adam (lr 1e-3) on the project's BF16 tensor-core training kernels;
4. held-out errors per k bin (max over held-out catalogues of
   |dP_l| / P_0 of the fine mesh), with the bins above 1% flagged.

Writes powspec_gb300/data/learned_alias.bin (checkpoint: parameters, Adam
state, step) and learned_alias_report.json.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ntrain", type=int, default=512)
    ap.add_argument("--nheld", type=int, default=64)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--n", type=int, default=4_000_000)
    ap.add_argument("--ngen", type=int, default=256)
    ap.add_argument("--out", default=None)
    ap.add_argument("--resume", action="store_true")
    args = ap.parse_args(argv)

    from . import learned
    out = args.out or learned.DEFAULT_WEIGHTS
    os.makedirs(os.path.dirname(out), exist_ok=True)
    t0 = time.time()
    seeds = list(range(1000, 1000 + args.ntrain + args.nheld))
    cats = learned.stream_catalogues(seeds, n=args.n, ngen=args.ngen)
    pairs = learned.measure_pairs(cats, log=lambda s: print(s, flush=True))
    print(f"catalogues + plain-method pairs: {len(pairs)} in {time.time() - t0:.1f} s", flush=True)

    m = learned.MLP(params=learned.init_params(0))
    if args.resume and os.path.exists(out):
        m.load(out)
    groups = learned.build_groups(pairs[:args.ntrain])
    t2 = time.time()
    losses = learned.train(m, groups, steps=args.steps, batch=args.batch, lr=args.lr,
                           log=lambda s: print(s, flush=True))
    print(f"training: {time.time() - t2:.1f} s, {len(groups[2])} groups", flush=True)
    m.save(out)
    err = learned.errors(pairs[args.ntrain:], m)
    rep = learned.save_report(out.replace(".bin", "_report.json"), err)
    rep["_meta"] = dict(ntrain=args.ntrain, nheld=args.nheld, steps=args.steps, batch=args.batch,
                        lr=args.lr, n=args.n, final_loss=float(losses[-500:].mean()),
                        seconds=time.time() - t0)
    with open(out.replace(".bin", "_report.json"), "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps(rep, indent=1))
    return 0


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.exit(main())
