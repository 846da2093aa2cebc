"""The planner's screening stages on the engine against the oracle: every
visible pair of the key-configuration screening, the edge files per reference
task, root assembly with the device's disentangled tests, and the PDS flags of
an assembled blooming forest."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = W.interlocking_tori(1.0, 0.25, 32, 16)
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    ow = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    # world-frame keys: half near the interlocked pose (mostly free), half uniform
    rng = np.random.default_rng(21)
    near = np.zeros((31, 7))
    near[:, 0] = 1.0 + rng.normal(0, 0.05, 31)
    near[:, 1:3] = rng.normal(0, 0.05, (31, 2))
    near[:, 3] = 1.0
    near[:, 4:] = rng.normal(0, 0.05, (31, 3))
    far = W.uniform_states(31, -2.0, 2.0, 1.0, seed=22)
    keys = np.concatenate([W.uniform_states(2, -2.0, 2.0, 1.0, seed=23), near, far])
    return uw, ow, keys


def _oracle_visible(uw, ow, keys, f, t, vm):
    u = uw.translate_to_unit_state(keys)
    e, _ = ow.segments_first_contact(u[f], u[t], vm, mode=1)
    return e == -1


def test_screening_finds_every_visible_pair(built_lib, setup, tmp_path):
    from puzzletunneldiscovery_gb300 import screening as S
    uw, ow, keys = setup
    vm = 0.01
    ef, et = S.screen_keyconf(uw, keys, max_chunk_number=8, minimal_chunk_size=100, out_dir=str(tmp_path),
                              verify_magnitude=vm, batch=257)
    nkey = keys.shape[0] - S.RESERVED
    r, c = np.tril_indices(nkey)
    r, c = r + S.RESERVED, c + S.RESERVED
    vis = _oracle_visible(uw, ow, keys, r, c, vm)
    assert 0 < vis.sum() < vis.size
    assert np.array_equal(ef, r[vis]) and np.array_equal(et, c[vis])
    total = S.partition_screening(keys.shape[0], 8, 100)
    assert len(list(tmp_path.glob("edge_batch-*.npz"))) == total
    lf, lt = S.load_edges(str(tmp_path))
    assert sorted(zip(lf, lt)) == sorted(zip(ef, et))
    # one task through the per-task entry point (the reference worker's call)
    f1, t1 = S.partition_screening(keys.shape[0], 8, 100, index=1)
    sf, st = S.screen_pairs(uw, keys, f1, t1, verify_magnitude=vm)
    d = np.load(tmp_path / "edge_batch-1.npz")
    assert np.array_equal(sf, d["EDGE_FROM"]) and np.array_equal(st, d["EDGE_TO"])
    # the same pairs through calculate_visibility_pair, as the reference's rerun path calls it
    v = uw.calculate_visibility_pair(keys[f1], False, keys[t1], False, vm)
    assert np.array_equal(f1[v.astype(bool)], sf)


def test_roots_and_pds_flags_follow_the_oracle(built_lib, setup, tmp_path):
    from puzzletunneldiscovery_gb300 import screening as S
    uw, ow, keys = setup
    vm = 0.01
    ef, et = S.screen_keyconf(uw, keys, verify_magnitude=vm)
    unit = uw.translate_ompl_to_unit(keys)
    dis = ow.is_disentangled(unit).astype(bool)
    assert np.array_equal(S.key_disentangled(uw, keys), dis)
    bases = np.array([2, 20, 40, keys.shape[0]])
    got = S.assemble_roots(uw, keys, bases, ef, et)
    want = S.assemble_roots(None, keys, bases, ef, et, disentangled=dis)
    for s in want:
        assert np.array_equal(got[s], want[s]), s
    assert got["cmb"].shape[0] >= 2
    # blooming forest: three trees, one of them without samples
    rng = np.random.default_rng(5)
    trees = [W.uniform_states(n, -6.0, 6.0, 1.0, seed=40 + n) for n in (5, 0, 9)]
    for i, q in enumerate(trees):
        m = q.shape[0]
        edge = np.stack([np.arange(1, m), rng.integers(0, np.maximum(np.arange(1, m), 1))]) if m else np.zeros((2, 0))
        np.savez(tmp_path / ("bloom-from_%d.npz" % i), BLOOM=q, BLOOM_EDGE=edge.astype(np.int64))
    pds = S.assemble_blooming(uw, str(tmp_path), str(tmp_path / "pds.npz"))
    Q = np.concatenate([trees[0], trees[2]])
    assert np.array_equal(pds["Q"], Q)
    assert pds["QB"] == [0, 5] and pds["QE"].shape == (12, 2) and pds["QEB"] == [0, 4]
    assert list(pds["BLOOM_NO_TO_INDEX"]) == [0, -1, 1] and pds["INDEX_TO_BLOOM_NO"] == [0, 2]
    qf = ow.is_disentangled(uw.translate_ompl_to_unit(Q)).astype(np.uint32).reshape(-1, 1)
    assert pds["QF"].dtype == np.uint32 and np.array_equal(pds["QF"], qf)
    assert qf.any()
    d = np.load(tmp_path / "pds.npz")
    assert set(d.files) == {"Q", "QF", "QB", "QE", "QEB", "BLOOM_NO_TO_INDEX", "INDEX_TO_BLOOM_NO"}
