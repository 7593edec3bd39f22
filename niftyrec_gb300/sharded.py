"""Angle-sharded OSEM across the processes of a torch.distributed group.

The projector is independent per camera, so every subset's cameras are dealt
round-robin over the ranks and each rank projects only its share: no data
moves between ranks for the projection.  A rank's backprojection of its share
is a partial volume; the subset's numerator B^T(y / A x) is the sum of the
partials, so each subset step makes exactly one collective, an all_reduce(SUM)
of the numerator volume (N^3 float32).  The normaliser B^T 1 depends only on
the geometry: it is reduced once, when the reconstructor is built.  Every rank
then applies the same update to the same sums, so the activity estimate stays
replicated on all ranks without a broadcast.

The update is et_array_osem_step's (emission-lib/_et_array_interface.cpp:972-1054):
p = A x with negatives truncated, r = y / p (y / eps where p < eps),
x <- x * (B^T r) / max(B^T 1, eps), both backprojections truncated.  With one
rank it is that step exactly; with several, the partial sums change only the
float32 summation order of the backprojection.

Ranks hold only their own cameras' counts.  The compute is an operator
object (``PlanOperator`` on the GPU, wrapping a device-resident Plan of the
rank's cameras); any object with the same four methods works, which is how
the multi-process logic is exercised with CPU ranks.
"""
from __future__ import annotations

import numpy as np


def camera_shares(subset_of_camera, rank: int, world: int):
    """This rank's cameras: each subset's cameras (ascending) dealt round-robin
    over the ranks.  Returns (camera indexes, subset id of each)."""
    sub = np.asarray(subset_of_camera, dtype=np.int64)
    cams, ids = [], []
    for s in range(int(sub.max()) + 1 if sub.size else 0):
        mine = np.flatnonzero(sub == s)[rank::world]
        cams.append(mine)
        ids.append(np.full(mine.size, s, dtype=np.int64))
    if not cams:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    return np.concatenate(cams), np.concatenate(ids)


class PlanOperator:
    """GPU operator over one rank's cameras (a Plan with the rank's share of
    every subset; subsets this rank has no camera of stay empty)."""

    def __init__(self, shape, cameras, camera_ids, subset_ids, n_subsets, psf=None, attenuation=None):
        import torch

        from ._lib import load
        from .plan import Plan

        self.torch = torch
        self.L = load()
        self.shape = tuple(shape)
        self.n_subsets = int(n_subsets)
        cams = np.asarray(cameras, dtype=np.float32)
        cams = cams[None, :] if cams.ndim == 1 else cams
        self.sizes = [int(np.sum(np.asarray(subset_ids) == s)) for s in range(self.n_subsets)]
        self.device = attenuation.device if attenuation is not None else torch.device("cuda", torch.cuda.current_device())
        self.plan = None
        if len(camera_ids):
            # camera_shares order is subset-major and stable, as the plan orders them
            self.plan = Plan(self.shape, np.ascontiguousarray(cams[:, camera_ids]), psf, attenuation,
                             subsets=np.asarray(subset_ids, dtype=np.int32), n_subsets=self.n_subsets)

    def _stream(self):
        import ctypes

        return ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def zeros(self):
        return self.torch.zeros(self.shape, dtype=self.torch.float32, device=self.device)

    def sensitivity(self, subset):
        if self.sizes[subset] == 0:
            return self.zeros()
        nz, ny, nx = self.shape
        ones = self.torch.ones((self.sizes[subset], ny, nx), dtype=self.torch.float32, device=self.device)
        return self.plan.backproject(ones, subset, truncate=True)

    def numerator(self, x, y, subset, epsilon):
        import ctypes

        if self.sizes[subset] == 0:
            return self.zeros()
        p = self.plan.project(x, subset, truncate=True)
        st = self.L.nrgb_osem_ratio_device(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(p.data_ptr()), p.numel(),
                                           float(epsilon), self._stream())
        if st:
            from ._lib import NiftyRecError

            raise NiftyRecError("nrgb_osem_ratio_device", st)
        return self.plan.backproject(p, subset, truncate=True)

    def update(self, x, num, den, epsilon):
        import ctypes

        st = self.L.nrgb_osem_update_device(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(num.data_ptr()),
                                            ctypes.c_void_p(den.data_ptr()), x.numel(), float(epsilon), self._stream())
        if st:
            from ._lib import NiftyRecError

            raise NiftyRecError("nrgb_osem_update_device", st)


class ShardedOSEM:
    """OSEM whose subsets are split over the ranks of a process group.

    operator: this rank's operator (PlanOperator, or an object with the
    methods zeros / sensitivity / numerator / update).
    counts: per subset, this rank's count sinogram (its share's cameras in
    camera_shares order), or None where the share is empty.
    group: torch.distributed group (None: the default group); world == 1
    makes no collective call at all."""

    def __init__(self, operator, counts, n_subsets, rank=0, world=1, group=None, epsilon=1e-6, sync=None):
        self.op = operator
        self.counts = counts
        self.n_subsets = int(n_subsets)
        self.rank, self.world, self.group = rank, world, group
        self.epsilon = float(epsilon)
        self.collectives = 0
        # collective timing (host clock, the device synchronised on both sides
        # by `sync`); off unless timing_collectives is set
        self.sync = sync or (lambda: None)
        self.timing_collectives = False
        self.collective_seconds = 0.0
        self.sens = []
        for s in range(self.n_subsets):
            den = self.op.sensitivity(s)
            self._sum(den)
            self.sens.append(den)

    def _sum(self, t):
        if self.world > 1:
            import time

            import torch.distributed as dist

            if self.timing_collectives:
                self.sync()
                t0 = time.perf_counter()
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
            if self.timing_collectives:
                self.sync()
                self.collective_seconds += time.perf_counter() - t0
            self.collectives += 1

    def step(self, x, subset):
        """One subset step, in place on the replicated activity x."""
        y = self.counts[subset]
        num = self.op.numerator(x, y, subset, self.epsilon) if y is not None else self.op.zeros()
        self._sum(num)
        self.op.update(x, num, self.sens[subset], self.epsilon)
        return x

    def run(self, x, iterations, start_iteration=0, start_subset=0, checkpoint=None, fingerprint="", every=1):
        """`iterations` passes over the subsets from (start_iteration,
        start_subset); with `checkpoint`, rank 0 saves the state (see
        niftyrec_gb300.checkpoint) after every `every` subset steps and at the
        end, and a run resumed from it continues exactly where it stopped."""
        from . import checkpoint as CK

        k = 0
        steps = list(CK.positions(self.n_subsets, iterations, start_iteration, start_subset))
        for i, (it, s) in enumerate(steps):
            self.step(x, s)
            k += 1
            if checkpoint and self.rank == 0 and (k % every == 0 or i == len(steps) - 1):
                nxt = (it, s + 1) if s + 1 < self.n_subsets else (it + 1, 0)
                self.sync()
                CK.save(checkpoint, x, nxt[0], nxt[1], fingerprint)
        return x


def split_counts(counts, camera_ids, subset_ids, n_subsets):
    """Per subset, the rows of a full count sinogram (n_cameras, ny, nx) that
    belong to this rank (camera_shares order), or None for an empty share."""
    out = []
    ids = np.asarray(subset_ids)
    cams = np.asarray(camera_ids)
    for s in range(n_subsets):
        sel = cams[ids == s]
        if sel.size == 0:
            out.append(None)
        elif hasattr(counts, "index_select"):
            import torch

            out.append(counts.index_select(0, torch.as_tensor(sel, device=counts.device)).contiguous())
        else:
            out.append(np.ascontiguousarray(counts[sel]))
    return out
