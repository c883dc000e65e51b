"""Mock ensembles: many catalogues of uneven size, mesh and scheme.

Catalogues sharing (Ng, scheme, interlacing) share one Estimator context;
each group's evaluations are recorded once as a CUDA graph
(``ps_gpu_batch_create``) and replayed with one launch per group, the groups
on their own streams so that small meshes overlap.  The autotuner
(``ps_gpu_autotune``) picks each group's launch configuration on its
largest catalogue first.  ``run_plain`` is the per-catalogue path (assign +
execute, one host round trip each) for comparison.
"""
from __future__ import annotations

from collections import OrderedDict

from . import Estimator


class Ensemble:
    def __init__(self, cats, configs, box=1000.0, dk=0.005, poles=(0, 2, 4), autotune=True,
                 device=0):
        """cats: device tensors (N, 4) float64, or (pointer, n) pairs;
        configs: (ng, assign, interlace) per catalogue."""
        if len(cats) != len(configs):
            raise ValueError("one configuration per catalogue")
        self.ptrs, self.ns = [], []
        for c in cats:
            if isinstance(c, tuple):
                p, n = c
            else:
                p, n = c.data_ptr(), c.shape[0]
            self.ptrs.append(int(p))
            self.ns.append(int(n))
        self.configs = [tuple(cf) for cf in configs]
        self.groups = OrderedDict()
        for i, cf in enumerate(self.configs):
            self.groups.setdefault(cf, []).append(i)
        self.est, self.batch, self.tuning = {}, {}, {}
        for cf, idx in self.groups.items():
            ng, assign, interlace = cf
            e = Estimator(ng=ng, box=box, assign=assign, interlace=bool(interlace), poles=poles,
                          dk=dk, device=device)
            if autotune:
                big = max(idx, key=lambda i: self.ns[i])
                self.tuning[cf] = e.autotune(self.ptrs[big], self.ns[big])
            self.est[cf] = e
            self.batch[cf] = e.batch([self.ptrs[i] for i in idx], [self.ns[i] for i in idx])

    def launches(self):
        """Kernel launches recorded in all the groups' graphs."""
        return sum(b.launches() for b in self.batch.values())

    def launch(self):
        """One graph launch per group, all groups in flight together."""
        for b in self.batch.values():
            b.launch(wait=False)

    def wait(self):
        for b in self.batch.values():
            b.wait()

    def results(self):
        out = [None] * len(self.ns)
        for cf, idx in self.groups.items():
            b = self.batch[cf]
            for j, i in enumerate(idx):
                out[i] = b.result(j)
        return out

    def run(self):
        self.launch()
        self.wait()
        return self.results()

    def run_plain(self):
        """The same evaluations one catalogue at a time (assign + execute)."""
        out = [None] * len(self.ns)
        for cf, idx in self.groups.items():
            e = self.est[cf]
            for i in idx:
                e.assign(0, self.ptrs[i], on_device=True, n=self.ns[i])
                out[i] = e.execute()
        return out

    def close(self):
        for b in self.batch.values():
            b.close()
        for e in self.est.values():
            e.close()
