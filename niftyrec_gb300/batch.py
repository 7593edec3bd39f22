"""Batched OSEM over many volumes of uneven size.

A ``Batch`` joins up to 64 fused ``Plan`` objects (each its own grid, camera
set, PSF, mu map and subset count).  One batched subset step runs

* one persistent projector launch for all volumes (per PSF width and
  attenuation kind): clusters of the GPU take (volume, row window, camera,
  x-tile) work items from a queue until none are left, so small volumes fill
  the SMs that one of them alone would leave idle;
* one ratio launch over all volumes' projections;
* the volumes' reference backprojections, concurrently on four side streams
  (largest volumes first, each to the least loaded stream; each volume's
  spread and gather on its own scratch), forked from and joined back into the
  caller's stream with events;
* one update launch over all volumes.

Nothing in a step allocates or copies from the host, so a step -- or a whole
reconstruction -- is captured once as a CUDA graph and replayed.  The update
is the reference's OSEM step (emission-lib/_et_array_interface.cpp:1017-1044),
identical to ``Plan.osem_step`` volume by volume.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import NiftyRecError, load
from .plan import COLUMN

_vp = ctypes.c_void_p


class Batch:
    def __init__(self, plans):
        import torch

        self.torch = torch
        self.L = load()
        self.plans = list(plans)
        if not 1 <= len(self.plans) <= 64:
            raise ValueError("a batch holds 1..64 plans")
        for p in self.plans:
            if not p.fused:
                raise ValueError("batched plans must use the fused y-gantry kernels")
            if p._osem_layout != COLUMN:
                p.osem_prepare("column")
        self.device = self.plans[0].device
        arr = (_vp * len(self.plans))(*[p.handle for p in self.plans])
        handle = _vp()
        st = self.L.nrgb_batch_create(ctypes.byref(handle), arr, len(self.plans), self._stream())
        if st:
            raise NiftyRecError("nrgb_batch_create", st)
        self.handle = handle
        self._graph = None

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.L.nrgb_batch_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    def _stream(self):
        return _vp(self.torch.cuda.current_stream(self.device).cuda_stream)

    def _call(self, name, *args):
        st = getattr(self.L, name)(self.handle, *args, self._stream())
        if st:
            raise NiftyRecError(name, st)

    def set_counts(self, v, counts):
        """Counts of volume v: CUDA (n_cameras, ny, nx) float32, original camera order."""
        c = counts.contiguous()
        self._call("nrgb_batch_set_counts", v, _vp(c.data_ptr()))

    def set_activity(self, v, activity):
        a = activity.contiguous()
        self._call("nrgb_batch_set_activity", v, _vp(a.data_ptr()))

    def get_activity(self, v):
        nz, ny, nx = self.plans[v].shape
        out = self.torch.empty((nz, ny, nx), dtype=self.torch.float32, device=self.device)
        self._call("nrgb_batch_get_activity", v, _vp(out.data_ptr()))
        return out

    def step(self, k, iterations=0, epsilon=1e-6):
        """Subset step k of every volume (subset k mod n_subsets_v)."""
        self._call("nrgb_batch_osem_step", int(k), int(iterations), float(epsilon))

    def n_steps(self, iterations):
        return iterations * max(p.n_subsets for p in self.plans)

    def osem(self, counts, iterations, activities=None, epsilon=1e-6, graph=False):
        """OSEM of every volume: `iterations` passes over its own subsets.
        counts: list of CUDA (n_cameras_v, ny_v, nx_v) tensors.  With graph=True
        the whole reconstruction is captured once as a CUDA graph and replayed.
        Returns the activities (nifti order)."""
        torch = self.torch
        for v, c in enumerate(counts):
            self.set_counts(v, c)

        def reset():
            for v, p in enumerate(self.plans):
                x = activities[v] if activities is not None else torch.ones(p.shape, dtype=torch.float32,
                                                                           device=self.device)
                self.set_activity(v, x)

        def run():
            for k in range(self.n_steps(iterations)):
                self.step(k, iterations, epsilon)

        reset()
        if graph:
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(side):
                self.step(0, iterations, epsilon)  # warm-up outside the capture (streams, attributes)
            torch.cuda.current_stream(self.device).wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                run()
            reset()
            g.replay()
            self._graph = g
        else:
            run()
        return [self.get_activity(v) for v in range(len(self.plans))]


def config_volumes(n_volumes=24, seed=0):
    """The batched workload's volume list: shapes cycling 64^3, 96x96x80,
    128^3, 160x160x128 (nifti (nx, ny, nz) -> arrays (nz, ny, nx)), camera
    counts cycling 60 / 90 / 120 / 180 over 360 degrees, subset counts cycling
    4, 8, 12, 16 (each dividing its camera count or not: subsets are
    interleaved), PSF 11x11 with a per-volume sigma slope."""
    shapes = [(64, 64, 64), (80, 96, 96), (128, 128, 128), (128, 160, 160)]
    cams = [60, 90, 120, 180]
    subsets = [4, 8, 12, 16]
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_volumes):
        out.append({"shape": shapes[i % 4], "ncam": cams[(i // 4 + i) % 4], "subsets": subsets[(i // 2) % 4],
                    "slope": float(rng.uniform(0.01, 0.03)), "seed": seed + i})
    return out
