"""intersecting_segments for a batch of states (pw_intersecting_segments_batch):
the same rows, in the same order, as one call per state, and as the oracle's
contact enumeration (unit_world.cc:959-1012, Moeller97d.cc:579), for colliding
and free states."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tori(oracle_mod, built_lib):
    import puzzletunneldiscovery_gb300 as pw
    m = W.cfg_interlocking_tori()
    uw = pw.UnitWorld()
    uw.load_env_mesh(m[0], m[1])
    uw.load_robot_mesh(m[2], m[3])
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, oracle_mod.OracleWorld(*m)


def ow_scale(uw):
    return uw.info()["scene_scale"]


def _states(uw, n, seed):
    q = W.uniform_states(8 * n, -0.6, 0.6, ow_scale(uw), seed=seed)
    hit = ~uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
    qs = q[hit][:n]
    far = W.uniform_states(n // 4, 30.0, 40.0, ow_scale(uw), seed=seed + 1)   # no contact
    h = qs.shape[0] // 2
    return np.concatenate([qs[:h], far, qs[h:]]), np.arange(h, h + far.shape[0])


def test_batch_equals_single_calls_and_oracle(tori):
    uw, ow = tori
    q, far = _states(uw, 200, 71)
    batch = uw.intersecting_segments_batch(q)
    assert len(batch) == q.shape[0]
    rows = 0
    for i, s in enumerate(q):
        one = uw.intersecting_segments(s)
        for x, y in zip(batch[i], one):
            assert x.shape == y.shape and (x == y).all()
        b2, e2, m2, p2, _ = ow.intersecting_segments(s)
        assert (batch[i][3] == p2).all() and (batch[i][0] == b2).all() and (batch[i][1] == e2).all()
        assert (batch[i][2] == m2).all()
        rows += batch[i][3].shape[0]
    assert rows > 200
    assert all(batch[i][3].shape[0] == 0 for i in far)


def test_batch_chunks_and_empty(tori, monkeypatch):
    uw, _ = tori
    assert len(uw.intersecting_segments_batch(np.zeros((0, 7)))) == 0
    q, _ = _states(uw, 40, 72)
    whole = uw.intersecting_segments_batch(q)
    # the same states in calls of 7: rows do not depend on the rest of the batch
    parts = [uw.intersecting_segments_batch(q[i:i + 7]) for i in range(0, q.shape[0], 7)]
    flat = [t for p in parts for t in p]
    for a, b in zip(whole, flat):
        for x, y in zip(a, b):
            assert (x == y).all()


def test_flat_rows_and_stats(tori):
    uw, _ = tori
    q, _ = _states(uw, 60, 73)
    per = uw.intersecting_segments_batch(q)
    b, e, m, p, off = uw.intersecting_segments_batch(q, flat=True)
    st = uw.last_stats()
    assert off.shape == (q.shape[0] + 1,) and off[0] == 0 and off[-1] == b.shape[0] == p.shape[0]
    assert (np.diff(off) >= 0).all()
    for i, t in enumerate(per):
        assert (t[3] == p[off[i]:off[i + 1]]).all() and (t[0] == b[off[i]:off[i + 1]]).all()
        # rows of one state sorted by (env face, robot face)
        k = t[3][:, 0].astype(np.int64) * (1 << 32) + t[3][:, 1]
        assert (np.diff(k) > 0).all()
    assert st["queries"] == q.shape[0] and st["retest_hits"] == off[-1]
    assert st["retests"] >= off[-1] and st["work_items"] >= 4
