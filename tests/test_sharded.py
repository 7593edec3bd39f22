"""Angle-sharded OSEM (niftyrec_gb300.sharded) with CPU ranks over gloo.

Two processes each own a share of every subset's cameras; the per-rank
compute is an operator built on the oracle (test infrastructure only), so
these tests check the sharding, the one all_reduce per subset step and the
replicated update against the oracle's single-process et_array_osem_step
(emission-lib/_et_array_interface.cpp:972-1054) on the same subsets.
The GPU operator (PlanOperator) is checked in test_gpu_plan.py."""
import os
import socket

import numpy as np
import pytest

from niftyrec_gb300 import sharded as SH
from niftyrec_gb300 import synthetic as S

torch = pytest.importorskip("torch")

SHAPE = (16, 12, 16)


class OracleOperator:
    """The four operator methods on the oracle's float32 restatement."""

    def __init__(self, cameras, camera_ids, subset_ids, n_subsets, psf, mu):
        from oracle.oracle import Restated

        self.o = Restated("f32")
        self.psf, self.mu = psf, mu
        ids = np.asarray(subset_ids)
        self.cams = [np.ascontiguousarray(cameras[:, np.asarray(camera_ids)[ids == s]]) for s in range(n_subsets)]

    def zeros(self):
        return torch.zeros(SHAPE, dtype=torch.float32)

    def _back(self, sino, s):
        return torch.from_numpy(self.o.backproject(sino, self.cams[s], self.psf, self.mu, truncate=1, nz=SHAPE[0]))

    def sensitivity(self, s):
        if self.cams[s].shape[1] == 0:
            return self.zeros()
        return self._back(np.ones((self.cams[s].shape[1],) + SHAPE[1:], np.float32), s)

    def numerator(self, x, y, s, eps):
        p = self.o.project(x.numpy(), self.cams[s], self.psf, self.mu, truncate=1)
        y = np.asarray(y, np.float32)
        r = np.where(p < eps, y / np.float32(eps), y / np.where(p < eps, 1, p)).astype(np.float32)
        return self._back(r, s)

    def update(self, x, num, den, eps):
        x.mul_(num / torch.clamp(den, min=eps))


def problem(ncam, seed=3):
    act = S.ellipsoid_phantom(SHAPE, seed=seed)
    mu = S.mu_map(SHAPE, seed=seed)
    psf = S.gaussian_psf(5, SHAPE[2], 0.5, 0.05)
    cams = S.cameras_about_y(ncam, 2.0)
    from oracle.oracle import Restated

    y = S.poisson_counts(Restated("f32").project(act, cams, psf, mu), 40, seed=seed)
    return act, mu, psf, cams, y


def _rank_main(rank, world, port, ncam, n_subsets, iterations, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        act, mu, psf, cams, y = problem(ncam)
        sub = np.arange(ncam) % n_subsets
        ids, sids = SH.camera_shares(sub, rank, world)
        op = OracleOperator(cams, ids, sids, n_subsets, psf, mu)
        counts = SH.split_counts(y, ids, sids, n_subsets)
        rec = SH.ShardedOSEM(op, counts, n_subsets, rank=rank, world=world)
        x = torch.ones(SHAPE, dtype=torch.float32)
        rec.run(x, iterations)
        np.save(os.path.join(out_dir, f"x{rank}.npy"), x.numpy())
        np.save(os.path.join(out_dir, f"n{rank}.npy"), np.array([rec.collectives, len(ids)]))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _single_process(ncam, n_subsets, iterations):
    from oracle.oracle import Restated

    act, mu, psf, cams, y = problem(ncam)
    o = Restated("f32")
    x = np.ones(SHAPE, np.float32)
    for _ in range(iterations):
        for s in range(n_subsets):
            idx = np.flatnonzero(np.arange(ncam) % n_subsets == s)
            x = o.osem_step(x, y, cams, idx, mu, psf)
    return x


@pytest.mark.parametrize("ncam,n_subsets", [(12, 2), (3, 3)])
def test_two_ranks_match_single_process(tmp_path, ncam, n_subsets):
    """(12, 2): six cameras per subset, three per rank.  (3, 3): one camera per
    subset, so rank 1 owns nothing and contributes zeros to every sum."""
    import torch.multiprocessing as mp

    world, iterations = 2, 2
    mp.start_processes(_rank_main, args=(world, _free_port(), ncam, n_subsets, iterations, str(tmp_path)),
                       nprocs=world, start_method="spawn", join=True)
    x0, x1 = np.load(tmp_path / "x0.npy"), np.load(tmp_path / "x1.npy")
    np.testing.assert_array_equal(x0, x1)  # replicated without a broadcast
    n0, n1 = np.load(tmp_path / "n0.npy"), np.load(tmp_path / "n1.npy")
    # one reduce per subset for the normalisers, then one per subset step
    assert n0[0] == n1[0] == n_subsets + n_subsets * iterations
    assert n0[1] + n1[1] == ncam
    ref = _single_process(ncam, n_subsets, iterations)
    rel = np.linalg.norm(x0 - ref) / np.linalg.norm(ref)
    assert rel < 1e-5, rel


def _bench_rank_main(rank, world, port, ncam, n_subsets, iterations, out_dir):
    """One rank of bench.py's sharded mode, with the oracle operator on CPU."""
    import json
    import types

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    args = types.SimpleNamespace(steps=iterations, warmup=1, subsets=n_subsets)
    line = {}
    try:
        x = bench.run_sharded(args, make_operator=OracleOperator, make_workload=lambda: problem(ncam),
                              device=torch.device("cpu"), out=line)
        np.save(os.path.join(out_dir, f"x{rank}.npy"), x.numpy())
        if rank == 0:
            with open(os.path.join(out_dir, "line.json"), "w") as f:
                json.dump(line, f)
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def test_bench_sharded_mode_two_gloo_ranks(tmp_path):
    """bench.py --sharded, driven with two CPU ranks over gloo: the estimate
    after K timed iterations is replicated, equals the single-process OSEM, and
    the JSON line reports one collective per subset step."""
    import json

    import torch.multiprocessing as mp

    world, ncam, n_subsets, iterations = 2, 12, 3, 2
    mp.start_processes(_bench_rank_main, args=(world, _free_port(), ncam, n_subsets, iterations, str(tmp_path)),
                       nprocs=world, start_method="spawn", join=True)
    x0, x1 = np.load(tmp_path / "x0.npy"), np.load(tmp_path / "x1.npy")
    np.testing.assert_array_equal(x0, x1)
    ref = _single_process(ncam, n_subsets, iterations)
    assert np.linalg.norm(x0 - ref) / np.linalg.norm(ref) < 1e-5
    line = json.loads((tmp_path / "line.json").read_text())
    assert line["mode"] == "sharded" and line["backend"] == "gloo"
    assert line["collectives_per_iteration"] == n_subsets
    assert line["value"] > 0 and line["allreduce_ms_per_step"] >= 0
    assert line["allreduce_bytes_per_step"] == int(np.prod(SHAPE)) * 4


def test_camera_shares_partition():
    sub = np.arange(30) % 4
    seen = []
    for r in range(3):
        ids, sids = SH.camera_shares(sub, r, 3)
        assert np.all(sub[ids] == sids)
        assert np.all(np.diff(sids) >= 0)  # subset-major
        seen.extend(ids.tolist())
    assert sorted(seen) == list(range(30))
