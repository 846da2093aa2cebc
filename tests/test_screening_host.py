"""Host logic of the planner's screening stages against the reference's own
task partitioner and disjoint set (tests/golden/screening_golden.npz, made by
tests/golden/make_screening_golden.py from partt.py and disjoint_set.py)."""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden", "screening_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def test_partition_matches_the_reference_partitioner(golden):
    from puzzletunneldiscovery_gb300 import screening as S
    meta = golden["part_meta"]
    assert len(meta) >= 10
    for i, (nkey_total, quota, gran, total, task) in enumerate(meta):
        assert S.partition_screening(int(nkey_total), int(quota), int(gran)) == total
        f, t = S.partition_screening(int(nkey_total), int(quota), int(gran), index=int(task))
        assert np.array_equal(f, golden["part_from_%d" % i]), i
        assert np.array_equal(t, golden["part_to_%d" % i]), i


def test_chunks_tile_the_task_range():
    from puzzletunneldiscovery_gb300 import screening as S
    for ntask, num in [(1, 1), (10, 3), (1540, 15), (5050, 37), (7, 7), (1000003, 1000)]:
        b = S.chunk_bounds(ntask, num)
        assert b.shape == (num, 2)
        assert b[0, 0] == 0 and b[-1, 1] == ntask
        assert (b[1:, 0] == b[:-1, 1]).all() and (b[:, 1] >= b[:, 0]).all()


def test_tril_pairs_decode_flat_indices():
    from puzzletunneldiscovery_gb300 import screening as S
    for n in (1, 2, 3, 17, 300):
        r, c = np.tril_indices(n)
        i, j = S.tril_pairs(np.arange(r.shape[0]))
        assert np.array_equal(i, r) and np.array_equal(j, c)
    # far beyond float32 / at the float64 rounding edges: exact integer identities
    i0 = np.array([10**6, 3 * 10**6 + 7, 2**26 + 3], dtype=np.int64)
    base = i0 * (i0 + 1) // 2
    for off in (0, 1, -1):
        k = base + off
        i, j = S.tril_pairs(k)
        assert (i * (i + 1) // 2 + j == k).all() and (j >= 0).all() and (j <= i).all()


def test_root_selection_matches_the_reference_disjoint_set(golden):
    from puzzletunneldiscovery_gb300 import screening as S
    for c in range(int(golden["root_count"])):
        nkey = int(golden["root_%d_nkey" % c])
        keys = np.repeat(np.arange(nkey, dtype=np.float64)[:, None], 7, axis=1)
        out = S.assemble_roots(None, keys, golden["root_%d_bases" % c], golden["root_%d_from" % c],
                               golden["root_%d_to" % c], disentangled=golden["root_%d_dis" % c])
        assert set(out) == {"ge", "nt", "nn", "cmb"}
        for s, got in out.items():
            want = golden["root_%d_%s" % (c, s)]
            assert np.array_equal(got[:, 0].astype(np.int64), want), (c, s)


def test_edge_files_round_trip(tmp_path):
    from puzzletunneldiscovery_gb300 import screening as S
    rng = np.random.default_rng(0)
    parts = []
    for t in range(3):
        f = rng.integers(2, 50, size=10 + t)
        g = rng.integers(2, 50, size=10 + t)
        np.savez_compressed(tmp_path / ("edge_batch-%d.npz" % t), EDGE_FROM=f, EDGE_TO=g)
        parts.append((f, g))
    ef, et = S.load_edges(str(tmp_path))
    assert ef.shape == (33,) and et.shape == (33,)
    want = sorted(zip(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts])))
    assert sorted(zip(ef, et)) == want


class _FakeWorld:
    """A stand-in for UnitWorld on the CPU: key i is visible from key j unless
    i + j is a multiple of 3; counts the pairs it is asked about."""
    recommended_cres = 0.01
    _device = "cpu"

    def __init__(self):
        self.pairs = 0

    def translate_to_unit_state(self, q):
        return np.array(q, dtype=np.float64)

    def first_contact_steps(self, A, B, vm, kind):
        import torch
        from puzzletunneldiscovery_gb300 import _lib
        assert kind == _lib.PW_SEG_TRANSITION and vm == self.recommended_cres
        self.pairs += A.shape[0]
        s = (A[:, 0] + B[:, 0]).round().to(torch.int64)
        return torch.where(s % 3 != 0, torch.full_like(s, _lib.PW_STEP_FREE), torch.full_like(s, 4))


def test_screening_resume_checks_only_missing_tasks(tmp_path):
    from puzzletunneldiscovery_gb300 import screening as S
    n = 22
    keys = np.zeros((n, 7))
    keys[:, 0] = np.arange(n)
    keys[:, 3] = 1.0
    w = _FakeWorld()
    ef, et = S.screen_keyconf(w, keys, max_chunk_number=4, minimal_chunk_size=1, out_dir=str(tmp_path), batch=7)
    ntask = (n - S.RESERVED) * (n - S.RESERVED + 1) // 2
    assert w.pairs == ntask
    r, c = np.tril_indices(n - S.RESERVED)
    r, c = r + S.RESERVED, c + S.RESERVED
    m = (r + c) % 3 != 0
    assert np.array_equal(ef, r[m]) and np.array_equal(et, c[m])
    # a worker lost task 2: only its pairs are checked again
    b = S.chunk_bounds(ntask, 4)
    os.remove(tmp_path / "edge_batch-2.npz")
    w2 = _FakeWorld()
    ef2, et2 = S.screen_keyconf(w2, keys, max_chunk_number=4, minimal_chunk_size=1, out_dir=str(tmp_path),
                                batch=7, resume=True)
    assert w2.pairs == b[2, 1] - b[2, 0]
    assert np.array_equal(ef2, ef) and np.array_equal(et2, et)
    assert (tmp_path / "edge_batch-2.npz").exists()


class _FakeOmplLib:
    """pw_ompl_check_motions over host memory: motion i is valid unless
    from.x + to.x is a multiple of 3.  Records the arguments it was given."""

    def __init__(self):
        self.calls = []

    def pw_ompl_check_motions(self, h, pa, pb, m, lo, hi, cdres, pvalid, pchecked, stream):
        import ctypes
        A = np.ctypeslib.as_array((ctypes.c_double * (7 * m)).from_address(pa)).reshape(m, 7)
        B = np.ctypeslib.as_array((ctypes.c_double * (7 * m)).from_address(pb)).reshape(m, 7)
        self.calls.append((m, [lo[i] for i in range(3)], [hi[i] for i in range(3)], cdres, stream))
        v = (np.round(A[:, 0] + B[:, 0]).astype(np.int64) % 3 != 0).astype(np.uint8)
        ctypes.memmove(pvalid, v.ctypes.data, m)
        pchecked[0] = 5 * m
        return 0


class _FakeOmplWorld:
    recommended_cres = 0.01
    _device = "cpu"
    _h = None

    def __init__(self):
        self._L = _FakeOmplLib()


def test_screening_with_an_ompl_driver_checks_ompl_frame_key_pairs(tmp_path):
    """screen_keyconf(driver=OmplDriver) asks the driver about every lower-triangle
    pair (from = row, to = column, the OMPL-frame keys as stored), with the
    driver's bounds and resolution, in batches; the driver refuses to run
    before set_bb / set_cdres."""
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    from puzzletunneldiscovery_gb300 import screening as S
    n = 25
    keys = np.zeros((n, 7))
    keys[:, 0] = np.arange(n)
    keys[:, 6] = 1.0
    w = _FakeOmplWorld()
    d = OC.OmplDriver(w)
    with pytest.raises(RuntimeError):
        S.screen_keyconf(w, keys, driver=d)
    d.set_bb([-1, -2, -3], [4, 5, 6])
    d.set_cdres(0.02)
    ef, et = S.screen_keyconf(w, keys, max_chunk_number=3, out_dir=str(tmp_path), batch=11, driver=d)
    r, c = np.tril_indices(n - S.RESERVED)
    r, c = r + S.RESERVED, c + S.RESERVED
    m = (r + c) % 3 != 0
    assert np.array_equal(ef, r[m]) and np.array_equal(et, c[m])
    calls = w._L.calls
    assert sum(x[0] for x in calls) == r.shape[0] and max(x[0] for x in calls) <= 11
    assert all(x[1] == [-1, -2, -3] and x[2] == [4, 5, 6] and x[3] == 0.02 and x[4] is None for x in calls)
    assert d.last_states_checked == 5 * calls[-1][0]
    ef2, et2 = S.load_edges(str(tmp_path))
    assert sorted(zip(ef2, et2)) == sorted(zip(ef, et))
    # the host-array call goes through the same entry point
    out, checked = OC.check_motions_discrete(w, keys[2:8], keys[3:7], [-1, -2, -3], [4, 5, 6], 0.02)
    want = ((np.arange(2, 6) + np.arange(3, 7)) % 3 != 0).astype(np.int32)
    assert np.array_equal(out, np.concatenate([want, [0, 0]])) and checked == 20


class _FakeListingLib:
    """pw_ompl_motion_states over host memory: motion i lists i + 1 states, state r
    of motion i is filled with 10 i + r; refuses (PW_ERR_CAPACITY) below the total."""

    def __init__(self):
        self.capacities = []

    def pw_ompl_motion_states(self, h, pa, pb, m, lo, hi, cdres, capacity, pstates, poffs, ptotal, stream):
        import ctypes
        counts = np.arange(1, m + 1, dtype=np.int64)
        offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        ctypes.memmove(poffs, offs.ctypes.data, 8 * (m + 1))
        ptotal[0] = int(offs[-1])
        self.capacities.append(capacity)
        if capacity < offs[-1]:
            return 5
        rows = np.zeros((int(offs[-1]), 7))
        for i in range(m):
            rows[offs[i]:offs[i + 1], 0] = 10 * i + np.arange(counts[i])
        ctypes.memmove(pstates, rows.ctypes.data, rows.nbytes)
        return 0


def test_motion_state_listing_sizes_then_fills():
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    w = _FakeOmplWorld()
    w._L = _FakeListingLib()
    q = np.zeros((4, 7))
    q[:, 6] = 1.0
    states, offs = OC.motion_states(w, q, q, [-1, -1, -1], [1, 1, 1], 0.01)
    assert w._L.capacities == [0, 10]
    assert offs.tolist() == [0, 1, 3, 6, 10] and states.shape == (10, 7)
    assert states[:, 0].tolist() == [0, 10, 11, 20, 21, 22, 30, 31, 32, 33]
    empty, eoffs = OC.motion_states(w, np.zeros((0, 7)), np.zeros((0, 7)), [-1, -1, -1], [1, 1, 1], 0.01)
    assert empty.shape == (0, 7) and eoffs.tolist() == [0]
