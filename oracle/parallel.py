"""The C restatement of the oracle spread over host cores.  Test
infrastructure only (tests and the CPU legs of bench.py).

Projection, the reference backprojector and the reference attenuation gradient
are separable over cameras: each worker process computes a contiguous share of
the cameras and the shares are concatenated (projections) or summed
(backprojections, gradients).  The sum of shares changes only the float32
order of the accumulation over cameras (emission-lib/_et.cpp:497 accumulates
camera after camera).

Workers are started with the ``spawn`` method, so a pool may be created in a
process that already uses CUDA.
"""
from __future__ import annotations

import multiprocessing as mp
import os

import numpy as np

_W = {}


def _init(precision):
    from oracle.oracle import Restated

    _W["o"] = Restated(precision)


def _cams_slice(cams, lo, hi):
    cams = np.asarray(cams)
    return np.ascontiguousarray(cams[lo:hi] if cams.ndim == 1 else cams[:, lo:hi])


def _ncam(cams):
    cams = np.asarray(cams)
    return cams.shape[0] if cams.ndim == 1 else cams.shape[1]


def _project(args):
    act, cams, psf, mu, bg, bg_att, truncate = args
    return _W["o"].project(act, cams, psf, mu, bg, bg_att, truncate)


def _backproject(args):
    sino, cams, psf, mu, nz, bg, bg_att, truncate = args
    return _W["o"].backproject(sino, cams, psf, mu, bg, bg_att, truncate, nz=nz)


def _gradient(args):
    sino, act, mu, cams, psf, truncate = args
    return _W["o"].gradient_attenuation(sino, act, mu, cams, psf, truncate=truncate)


class Pool:
    """A pool of oracle processes (``precision`` "f32" or "f64")."""

    def __init__(self, workers=None, precision="f32"):
        self.workers = workers or os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(self.workers, initializer=_init, initargs=(precision,))

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _shares(self, n):
        k = min(self.workers, n)
        edges = np.linspace(0, n, k + 1).round().astype(int)
        return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]

    def project(self, act, cams, psf=None, mu=None, bg=0.0, bg_att=0.0, truncate=1):
        shares = self._shares(_ncam(cams))
        parts = self.pool.map(_project, [(act, _cams_slice(cams, a, b), psf, mu, bg, bg_att, truncate)
                                         for a, b in shares])
        return np.concatenate(parts, axis=0)

    def backproject(self, sino, cams, psf=None, mu=None, nz=None, bg=0.0, bg_att=0.0, truncate=1):
        shares = self._shares(_ncam(cams))
        parts = self.pool.map(_backproject, [(np.ascontiguousarray(sino[a:b]), _cams_slice(cams, a, b), psf, mu, nz,
                                              bg, bg_att, truncate) for a, b in shares])
        return np.sum(parts, axis=0, dtype=np.float64).astype(parts[0].dtype)

    def gradient_attenuation(self, sino, act, mu, cams, psf=None, truncate=0):
        shares = self._shares(_ncam(cams))
        parts = self.pool.map(_gradient, [(np.ascontiguousarray(sino[a:b]), act, mu, _cams_slice(cams, a, b), psf,
                                           truncate) for a, b in shares])
        return np.sum(parts, axis=0, dtype=np.float64).astype(parts[0].dtype)
