"""Ensembles of independent runs on one GPU (the batching pattern).

Every member is its own context (its own device arena, stream and two-step
CUDA graph), of any grid size and precision.  :meth:`Ensemble.step` calls
``fw_ensemble_step``, which enqueues the members' graphs round robin from
native code and then waits for all of them, so runs that are each too small
to fill the GPU execute concurrently.  With ``single_launch=True`` it calls
``fw_ensemble_run`` instead: one parent CUDA graph holds every member's
two-step graph as an independent child, so each two steps of the whole
ensemble are one graph launch.  Each member's results are those of
stepping it alone, bit for bit: the kernels are the same and deterministic.

The number of hardware queues the CUDA runtime spreads the streams over is
CUDA_DEVICE_MAX_CONNECTIONS (default 8, at most 32); set it before the first
CUDA call of the process for more concurrency.
"""
import ctypes

import numpy as np

from .params import with_defaults
from .solver import FwError, Solver


def max_runup(height_max, depth):
    """Highest land elevation the water reached: max(-h) over the interior
    cells that were dry land at rest (h < 0) and whose running maximum of
    eta (HeightMax, OUT_Hmax) rose above the land (eta > -h); 0 when the
    water reached no such cell."""
    g = 3
    hm = height_max[g:-g, g:-g]
    land = depth < 0.0
    wet = land & (hm > -depth)
    return float((-depth[wet]).max()) if wet.any() else 0.0


class Ensemble:
    """members: list of (params, depth, phases) as the case generators return.
    All members are created on ``device`` with ``precision``; OUT_Hmax is
    switched on so that each run's maximum run-up can be read.  autotune:
    choose each member's launch shapes with fw_autotune after its init
    (cached per size class, so the 512-member ensemble tunes a few dozen
    times, not 512); the results do not depend on it."""

    def __init__(self, members, precision="MIXED", device=0, autotune=False, single_launch=False):
        self.solvers = []
        self.depths = []
        for params, depth, phases in members:
            p = with_defaults(params)
            p["OUT_Hmax"] = True
            s = Solver(p, precision=precision, device=device)
            s.init(depth, phases=phases)
            if autotune:
                s.autotune()
            self.solvers.append(s)
            self.depths.append(np.asarray(depth))
        self.L = self.solvers[0].L if self.solvers else None
        self.handle = None
        if single_launch and self.solvers:
            n = len(self.solvers)
            arr = (ctypes.c_void_p * n)(*[s.ctx for s in self.solvers])
            h = ctypes.c_void_p()
            rc = self.L.fw_ensemble_create(arr, n, ctypes.byref(h))
            if rc != 0:
                raise FwError(rc, "fw_ensemble_create")
            self.handle = h

    def __len__(self):
        return len(self.solvers)

    def step(self, nsteps, check=True):
        """nsteps whole steps of every member, concurrently; the status of
        each (0, or FW_ERR_BLOWUP / FW_ERR_NAN)."""
        n = len(self.solvers)
        st = (ctypes.c_int * n)()
        if self.handle is not None:
            rc = self.L.fw_ensemble_run(self.handle, int(nsteps), st)
            if rc != 0:
                raise FwError(rc, "fw_ensemble_run")
        else:
            arr = (ctypes.c_void_p * n)(*[s.ctx for s in self.solvers])
            rc = self.L.fw_ensemble_step(arr, n, int(nsteps), st)
            if rc != 0:
                raise FwError(rc, "fw_ensemble_step")
        out = list(st)
        if check and any(out):
            raise FwError(next(v for v in out if v), "member %d" % next(k for k, v in enumerate(out) if v))
        return out

    def cells(self):
        return [s.Mloc - 6 for s in self.solvers], [s.Nloc - 6 for s in self.solvers]

    def max_runup(self):
        return [max_runup(s.get("HeightMax"), d) for s, d in zip(self.solvers, self.depths)]

    def close(self):
        if self.handle is not None:
            self.L.fw_ensemble_destroy(self.handle)
            self.handle = None
        for s in self.solvers:
            s.close()
        self.solvers = []
