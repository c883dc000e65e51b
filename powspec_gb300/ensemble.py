"""Mock ensembles: many catalogues of uneven size, mesh and scheme.

Catalogues sharing (Ng, scheme, interlacing) form a group.  A group is
split over `lanes` contexts (Estimators), each holding its own meshes, so
that catalogues of one group can run at the same time; every context's
evaluations are recorded once as a CUDA graph (``ps_gpu_batch_create``), and
all of them become the child graphs of ONE ensemble graph
(``ps_gpu_ensemble_create``): a single graph launch evaluates the whole
ensemble, the contexts' branches running concurrently.  The autotuner
(``ps_gpu_autotune``) picks each group's launch configuration on its largest
catalogue, and the group's other contexts take the same configuration.

``launch_groups`` replays the per-context graphs one launch each on the
contexts' streams (the form before the ensemble graph), and ``run_plain``
is the per-catalogue path (assign + execute, one host round trip each), both
for comparison.
"""
from __future__ import annotations

import ctypes
from collections import OrderedDict

from . import Estimator, PowspecError, lib


class Ensemble:
    def __init__(self, cats, configs, box=1000.0, dk=0.005, poles=(0, 2, 4), autotune=True,
                 device=0, lanes=4, min_per_lane=4):
        """cats: device tensors (N, 4) float64, or (pointer, n) pairs;
        configs: (ng, assign, interlace) per catalogue; lanes: contexts per
        group at most (a lane gets at least min_per_lane catalogues)."""
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
        # lanes: (config, catalogue indices, Estimator, Batch)
        self.lanes, self.tuning = [], {}
        for cf, idx in self.groups.items():
            ng, assign, interlace = cf
            nl = max(1, min(lanes, len(idx) // max(1, min_per_lane)))
            parts = [idx[k::nl] for k in range(nl)]
            tuned = None
            for part in parts:
                e = Estimator(ng=ng, box=box, assign=assign, interlace=bool(interlace),
                              poles=poles, dk=dk, device=device)
                if autotune and tuned is None:
                    big = max(idx, key=lambda i: self.ns[i])
                    tuned = e.autotune(self.ptrs[big], self.ns[big])
                    self.tuning[cf] = tuned
                elif tuned is not None:
                    e.set_tuning(gather_threads=tuned["gather_threads"],
                                 z_radix32=tuned["z_radix32"], y_radix32=tuned["y_radix32"],
                                 pipelined_pass_c=tuned["pipelined_pass_c"],
                                 dense_lane_groups=tuned["dense_lane_groups"],
                                 region_gather=tuned["region_gather"])
                    e.warp_fft(tuned["warp_fft"])
                b = e.batch([self.ptrs[i] for i in part], [self.ns[i] for i in part])
                self.lanes.append((cf, part, e, b))
        L = lib()
        arr = (ctypes.c_void_p * len(self.lanes))(*[b._b for _, _, _, b in self.lanes])
        self._ens = ctypes.c_void_p()
        rc = L.ps_gpu_ensemble_create(arr, len(self.lanes), ctypes.byref(self._ens))
        if rc:
            msg = self.lanes[0][2].last_error()
            self.close()
            raise PowspecError(rc, msg)

    def launches(self):
        """Kernel launches recorded in the ensemble graph."""
        return sum(b.launches() for _, _, _, b in self.lanes)

    def launch(self):
        """One graph launch for the whole ensemble."""
        rc = lib().ps_gpu_ensemble_launch(self._ens, 0)
        if rc:
            raise PowspecError(rc, self.lanes[0][2].last_error())

    def wait(self):
        rc = lib().ps_gpu_ensemble_wait(self._ens)
        if rc:
            raise PowspecError(rc, self.lanes[0][2].last_error())

    def launch_groups(self):
        """The per-context graphs, one launch each on the contexts' streams."""
        for _, _, _, b in self.lanes:
            b.launch(wait=False)

    def wait_groups(self):
        for _, _, _, b in self.lanes:
            b.wait()

    def results(self):
        out = [None] * len(self.ns)
        for _, part, _, b in self.lanes:
            for j, i in enumerate(part):
                out[i] = b.result(j)
        return out

    def run(self):
        self.launch()
        self.wait()
        return self.results()

    def run_plain(self):
        """The same evaluations one catalogue at a time (assign + execute)."""
        out = [None] * len(self.ns)
        for _, part, e, _ in self.lanes:
            for i in part:
                e.assign(0, self.ptrs[i], on_device=True, n=self.ns[i])
                out[i] = e.execute()
        return out

    def close(self):
        if getattr(self, "_ens", None):
            lib().ps_gpu_ensemble_destroy(self._ens)
            self._ens = None
        for _, _, e, b in getattr(self, "lanes", []):
            b.close()
            e.close()
        self.lanes = []
