"""Device-resident projector plans and OSEM on torch tensors.

A ``Plan`` wraps the library's plan object (nrgb_plan_*): one grid, camera
set, PSF and attenuation map, with camera subsets for OSEM.  Tensors are CUDA
float32 in nifti memory order (volumes (nz, ny, nx), sinograms (n, ny, nx)) or,
with ``layout="column"``, in the fused kernels' native layout (volumes
(nz, nx, cy), sinograms (n, nx, cy), cy = ny rounded up to 4, zero pads).

``Plan.osem`` runs OSEM with the reference's update rule
(emission-lib/_et_array_interface.cpp:1017-1044); with ``graph=True`` one
iteration over all subsets is captured once as a CUDA graph and replayed.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import NiftyRecError, load

NIFTI, COLUMN = 0, 1
_vp = ctypes.c_void_p


def _layout(layout):
    return COLUMN if layout in ("column", COLUMN) else NIFTI


def interleaved_subsets(n_cameras, n_subsets):
    """Subset id per camera for interleaved subsets: camera k in subset k % n_subsets."""
    return np.arange(n_cameras, dtype=np.int32) % n_subsets


def opposed_subsets(n_cameras, n_subsets):
    """Subset id per camera for cameras evenly spaced over 360 degrees, with
    camera k and its opposite k + n/2 in the same subset (interleaved over the
    first half-turn: subset (k mod n/2) % n_subsets).  The library then serves
    each opposite pair from one set of samples (mirror units); an odd camera
    count falls back to interleaved subsets."""
    if n_cameras % 2:
        return interleaved_subsets(n_cameras, n_subsets)
    return (np.arange(n_cameras, dtype=np.int32) % (n_cameras // 2)) % n_subsets


class Plan:
    def __init__(self, shape, cameras, psf=None, attenuation=None, subsets=None, background=0.0,
                 background_attenuation=0.0, n_subsets=None):
        """subsets: None (one subset), a count (interleaved subsets) or the
        subset id of every camera; n_subsets overrides the count implied by
        the ids (subsets may then be empty)."""
        import torch

        self.torch = torch
        self.L = load()
        nz, ny, nx = shape
        self.shape = (nz, ny, nx)
        cams = np.ascontiguousarray(np.asarray(cameras, dtype=np.float32))
        self.cameras = cams
        ncam = cams.shape[0] if cams.ndim == 1 else cams.shape[1]
        ncols = 1 if cams.ndim == 1 else cams.shape[0]
        if subsets is None:
            sub = None
            self.n_subsets = 1
        elif np.isscalar(subsets):
            sub = interleaved_subsets(ncam, int(subsets))
            self.n_subsets = int(subsets)
        else:
            sub = np.ascontiguousarray(np.asarray(subsets, dtype=np.int32))
            self.n_subsets = int(sub.max()) + 1 if n_subsets is None else int(n_subsets)
        self._psf = None if psf is None else np.ascontiguousarray(np.asarray(psf, dtype=np.float32))
        self._mu_ref = attenuation  # for the checkpoint fingerprint
        self.device = attenuation.device if attenuation is not None else torch.device("cuda", torch.cuda.current_device())
        stream = torch.cuda.current_stream(self.device)
        handle = _vp()
        size = (ctypes.c_int * 3)(nx, ny, nz)
        psize = (ctypes.c_int * 3)(*(self._psf.shape[::-1] if self._psf is not None else (0, 0, 0)))
        st = self.L.nrgb_plan_create(ctypes.byref(handle), size, cams.ctypes.data_as(_vp),
                                     (ctypes.c_int * 2)(ncam, ncols),
                                     self._psf.ctypes.data_as(_vp) if self._psf is not None else None, psize,
                                     _vp(attenuation.data_ptr()) if attenuation is not None else None,
                                     float(background), float(background_attenuation),
                                     sub.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if sub is not None else None,
                                     self.n_subsets, _vp(stream.cuda_stream))
        if st:
            raise NiftyRecError("nrgb_plan_create", st)
        self.handle = handle
        info = (ctypes.c_int * 7)()
        self.L.nrgb_plan_shape(handle, info)
        self.cy = info[3]
        self.n_cameras = info[4]
        self.fused = bool(info[6])
        self._osem_layout = None
        self._graph = None

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.L.nrgb_plan_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    # ------------------------------------------------------------ helpers
    def _stream(self):
        return _vp(self.torch.cuda.current_stream(self.device).cuda_stream)

    def subset_cameras(self, subset):
        n = self.L.nrgb_plan_subset_cameras(self.handle, subset, None)
        idx = (ctypes.c_int * max(n, 1))()
        self.L.nrgb_plan_subset_cameras(self.handle, subset, idx)
        return np.array(idx[:n], dtype=np.int64)

    def subset_size(self, subset):
        return self.L.nrgb_plan_subset_cameras(self.handle, subset, None)

    def to_column(self, t):
        """nifti (planes, ny, nx) -> column (planes, nx, cy)."""
        planes, ny, nx = t.shape
        out = self.torch.empty((planes, nx, self.cy), dtype=self.torch.float32, device=t.device)
        st = self.L.nrgb_layout_convert(_vp(t.data_ptr()), _vp(out.data_ptr()), nx, ny, planes, 0, 0, self._stream())
        if st:
            raise NiftyRecError("nrgb_layout_convert", st)
        return out

    def from_column(self, t, ny=None, truncate=False):
        planes, nx, cy = t.shape
        ny = self.shape[1] if ny is None else ny
        out = self.torch.empty((planes, ny, nx), dtype=self.torch.float32, device=t.device)
        st = self.L.nrgb_layout_convert(_vp(t.data_ptr()), _vp(out.data_ptr()), nx, ny, planes, 1, int(truncate),
                                        self._stream())
        if st:
            raise NiftyRecError("nrgb_layout_convert", st)
        return out

    # ------------------------------------------------------------ operators
    def project(self, activity, subset=-1, layout="nifti", truncate=True, out=None):
        lay = _layout(layout)
        n = self.subset_size(subset)
        nz, ny, nx = self.shape
        if out is None:
            shp = (n, ny, nx) if lay == NIFTI else (n, nx, self.cy)
            out = self.torch.empty(shp, dtype=self.torch.float32, device=activity.device)
        st = self.L.nrgb_plan_project(self.handle, subset, _vp(activity.data_ptr()), _vp(out.data_ptr()), lay,
                                      int(truncate), self._stream())
        if st:
            raise NiftyRecError("nrgb_plan_project", st)
        return out

    def backproject(self, sinogram, subset=-1, layout="nifti", truncate=True, out=None):
        lay = _layout(layout)
        nz, ny, nx = self.shape
        if out is None:
            shp = (nz, ny, nx) if lay == NIFTI else (nz, nx, self.cy)
            out = self.torch.empty(shp, dtype=self.torch.float32, device=sinogram.device)
        st = self.L.nrgb_plan_backproject(self.handle, subset, _vp(sinogram.data_ptr()), _vp(out.data_ptr()), lay,
                                          int(truncate), self._stream())
        if st:
            raise NiftyRecError("nrgb_plan_backproject", st)
        return out

    # ------------------------------------------------------------ OSEM
    def osem_prepare(self, layout="column"):
        lay = _layout(layout)
        st = self.L.nrgb_plan_osem_prepare(self.handle, lay, self._stream())
        if st:
            raise NiftyRecError("nrgb_plan_osem_prepare", st)
        self._osem_layout = lay
        self._graph = None

    def split_counts(self, counts, layout="column"):
        """Per-subset count sinograms in subset camera order from a full (n, ny, nx) tensor."""
        out = []
        for s in range(self.n_subsets):
            idx = self.torch.as_tensor(self.subset_cameras(s), device=counts.device)
            y = counts.index_select(0, idx).contiguous()
            out.append(self.to_column(y) if _layout(layout) == COLUMN else y)
        return out

    def osem_step(self, activity, counts_subset, subset, epsilon=1e-6):
        st = self.L.nrgb_plan_osem_step(self.handle, subset, _vp(activity.data_ptr()), _vp(counts_subset.data_ptr()),
                                        float(epsilon), self._stream())
        if st:
            raise NiftyRecError("nrgb_plan_osem_step", st)

    def osmapem_step(self, activity, counts_subset, subset, beta, epsilon=1e-6):
        """One-step-late MAP-EM step with the quadratic MRF prior (et_osmapem_step
        of the reference's Python package; beta is its beta_osl)."""
        st = self.L.nrgb_plan_osmapem_step(self.handle, subset, _vp(activity.data_ptr()),
                                           _vp(counts_subset.data_ptr()), float(beta), float(epsilon),
                                           self._stream())
        if st:
            raise NiftyRecError("nrgb_plan_osmapem_step", st)

    def fingerprint(self):
        """Digest of the problem an OSEM state of this plan belongs to."""
        from .checkpoint import fingerprint

        return fingerprint(self.shape, self.cameras, self.n_subsets, self._psf, self._mu_ref)

    def osem(self, counts, iterations, activity=None, layout="column", epsilon=1e-6, graph=False, beta=None,
             checkpoint=None, resume=False, every=1):
        """OSEM from full-size counts (n, ny, nx); returns the activity in nifti order.
        beta: run one-step-late MAP-EM with the quadratic MRF prior instead
        (beta_osl of the reference's et_osmapem_step).
        checkpoint: file (.npz) that receives the state (activity, next
        iteration and subset) after every `every` subset steps and at the end;
        with resume=True an existing checkpoint of this problem is continued
        (iterations counts from the start of the run, not of the resume)."""
        torch = self.torch
        lay = _layout(layout)
        if self._osem_layout != lay:
            self.osem_prepare(layout)
        ys = self.split_counts(counts, layout)
        nz, ny, nx = self.shape
        start = (0, 0)
        if checkpoint is not None:
            import os

            from . import checkpoint as CK

            if graph:
                raise ValueError("checkpointing runs subset by subset; it does not combine with graph=True")
            fp = self.fingerprint()
            if resume and os.path.exists(checkpoint):
                state = CK.load(checkpoint)
                CK.check(state, fp)
                activity = torch.from_numpy(state["activity"]).to(counts.device)
                start = (state["iteration"], state["subset"])
        x = activity if activity is not None else torch.ones((nz, ny, nx), dtype=torch.float32, device=counts.device)
        x = self.to_column(x) if lay == COLUMN else x.clone()

        if checkpoint is not None:
            steps = list(CK.positions(self.n_subsets, iterations, *start))
            for i, (it, s) in enumerate(steps):
                if beta is None:
                    self.osem_step(x, ys[s], s, epsilon)
                else:
                    self.osmapem_step(x, ys[s], s, beta, epsilon)
                if (i + 1) % every == 0 or i == len(steps) - 1:
                    nxt = (it, s + 1) if s + 1 < self.n_subsets else (it + 1, 0)
                    CK.save(checkpoint, self.from_column(x) if lay == COLUMN else x, nxt[0], nxt[1], fp)
            return self.from_column(x) if lay == COLUMN else x

        def one_iteration():
            for s in range(self.n_subsets):
                if beta is None:
                    self.osem_step(x, ys[s], s, epsilon)
                else:
                    self.osmapem_step(x, ys[s], s, beta, epsilon)

        if graph:
            x0 = x.clone()
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(side):
                one_iteration()  # warm-up outside the capture (creates streams/events, sets attributes)
            torch.cuda.current_stream(self.device).wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                one_iteration()
            x.copy_(x0)
            for _ in range(iterations):
                g.replay()
            self._graph = (g, x, ys)
        else:
            for _ in range(iterations):
                one_iteration()
        return self.from_column(x) if lay == COLUMN else x
