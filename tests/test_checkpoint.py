"""OSEM checkpoint / resume (niftyrec_gb300.checkpoint) on the CPU: the
sharded reconstructor with one rank and the oracle operator, interrupted
mid-iteration and resumed from the saved state, reproduces the uninterrupted
run bit for bit; a checkpoint of another problem is refused."""
import numpy as np
import pytest

from niftyrec_gb300 import checkpoint as CK
from niftyrec_gb300 import sharded as SH

torch = pytest.importorskip("torch")


def _setup(ncam=9, n_subsets=3):
    from test_sharded import OracleOperator, problem

    act, mu, psf, cams, y = problem(ncam)
    ids, sids = SH.camera_shares(np.arange(ncam) % n_subsets, 0, 1)
    op = OracleOperator(cams, ids, sids, n_subsets, psf, mu)
    counts = SH.split_counts(y, ids, sids, n_subsets)
    fp = CK.fingerprint(act.shape, cams, n_subsets, psf, mu)
    return act.shape, op, counts, fp


def test_positions():
    assert list(CK.positions(3, 2, 1, 1)) == [(1, 1), (1, 2)]
    assert list(CK.positions(2, 2)) == [(0, 0), (0, 1), (1, 0), (1, 1)]
    assert list(CK.positions(2, 1, 1, 0)) == []


def test_resume_reproduces_uninterrupted_run(tmp_path):
    shape, op, counts, fp = _setup()
    full = SH.ShardedOSEM(op, counts, 3)
    x_full = full.run(torch.ones(shape, dtype=torch.float32), 2)

    ck = str(tmp_path / "osem.npz")
    a = SH.ShardedOSEM(op, counts, 3)
    x = torch.ones(shape, dtype=torch.float32)
    # stop after 4 of the 6 subset steps: run 1 iteration and one subset of the next
    a.run(x, 1, checkpoint=ck, fingerprint=fp)
    st = CK.load(ck)
    assert (st["iteration"], st["subset"]) == (1, 0)
    a.step(x, 0)
    CK.save(ck, x, 1, 1, fp)

    st = CK.load(ck)
    CK.check(st, fp)
    b = SH.ShardedOSEM(op, counts, 3)
    xr = torch.from_numpy(st["activity"])
    b.run(xr, 2, start_iteration=st["iteration"], start_subset=st["subset"], checkpoint=ck, fingerprint=fp)
    np.testing.assert_array_equal(xr.numpy(), x_full.numpy())
    st = CK.load(ck)
    assert (st["iteration"], st["subset"]) == (2, 0)


def test_checkpoint_of_another_problem_is_refused(tmp_path):
    shape, op, counts, fp = _setup()
    ck = str(tmp_path / "osem.npz")
    CK.save(ck, np.ones(shape, np.float32), 0, 1, fp)
    other = CK.fingerprint(shape, np.zeros((3, 9), np.float32), 3)
    with pytest.raises(ValueError):
        CK.check(CK.load(ck), other)
