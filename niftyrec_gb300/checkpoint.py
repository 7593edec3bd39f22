"""Checkpoint and resume of an OSEM reconstruction.

The reference keeps its reconstruction state in memory only
(Python/NiftyRec/NiftyRec/NiftyRec.py:252-333).  Here the state of an OSEM
run is the activity estimate plus its position in the subset sequence (the
next iteration and subset to run) and a fingerprint of the problem (grid,
cameras, subset count, PSF, mu); ``save`` writes it atomically (a temporary
file renamed over the target), ``load`` reads it back and ``check`` refuses a
checkpoint of another problem.  The OSEM update is deterministic (the
reference-mode projector and backprojector use no atomics), so a resumed run
reproduces the uninterrupted one bit for bit.
"""
from __future__ import annotations

import hashlib
import os

import numpy as np


def fingerprint(shape, cameras, n_subsets, psf=None, attenuation=None) -> str:
    """Digest of what an OSEM state belongs to."""
    h = hashlib.sha256()
    h.update(np.asarray(shape, np.int64).tobytes())
    h.update(np.ascontiguousarray(np.asarray(cameras, np.float32)).tobytes())
    h.update(np.int64(n_subsets).tobytes())
    for a in (psf, attenuation):
        if a is None:
            h.update(b"-")
        else:
            if hasattr(a, "detach"):
                a = a.detach().float().cpu().numpy()
            h.update(np.ascontiguousarray(np.asarray(a, np.float32)).tobytes())
    return h.hexdigest()


def save(path, activity, iteration: int, subset: int, fp: str) -> None:
    """State before running `subset` of `iteration` (both counted from 0)."""
    if hasattr(activity, "detach"):
        activity = activity.detach().cpu().numpy()
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as f:
        np.savez(f, activity=np.asarray(activity, np.float32), iteration=np.int64(iteration),
                 subset=np.int64(subset), fingerprint=np.array(fp))
    os.replace(tmp, path)


def load(path) -> dict:
    with np.load(path) as z:
        return {"activity": z["activity"].copy(), "iteration": int(z["iteration"]), "subset": int(z["subset"]),
                "fingerprint": str(z["fingerprint"])}


def check(state: dict, fp: str) -> None:
    if state["fingerprint"] != fp:
        raise ValueError("checkpoint belongs to another problem (grid, cameras, subsets, PSF or mu differ)")


def positions(n_subsets: int, iterations: int, start_iteration: int = 0, start_subset: int = 0):
    """(iteration, subset) of every step from the start position to the end."""
    it, s = start_iteration, start_subset
    while it < iterations:
        yield it, s
        s += 1
        if s == n_subsets:
            it, s = it + 1, 0
