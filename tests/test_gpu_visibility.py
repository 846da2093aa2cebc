"""The visibility batches (UnitWorld::calculateVisibilityMatrix / Matrix2 / Pair,
lib/osr/unit_world.cc:740-840, bound at lib/pyosr/module.cc:168-184) against
the oracle's isValidTransition on every pair: the N x N matrix over i < j
mirrored with a zero diagonal, the M x N grid, and aligned pairs, with unit and
non-unit inputs (the latter go through translateToUnitState)."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu

VERIFY = 0.01


@pytest.fixture(scope="module")
def world(oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)


def _free_keys(uw, n, seed, lo=-0.9, hi=0.9):
    """n free unit states close enough together that some transitions between them are free."""
    q = W.uniform_states(20 * n, lo, hi, uw.scene_scale, seed=seed)
    v = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
    return q[v][:n]


def _oracle_visible(ow, a, b):
    first, _ = ow.segments_first_contact(np.ascontiguousarray(a), np.ascontiguousarray(b), VERIFY, mode=1)
    return (first == -1).astype(np.int8)


def test_visibility_matrix_matches_oracle(built_lib, world):
    uw, ow = world
    q = _free_keys(uw, 41, 301)
    assert q.shape[0] == 41
    got = uw.calculate_visibility_matrix(q, True, VERIFY)
    assert got.dtype == np.int8 and got.shape == (41, 41)
    iu, ju = np.triu_indices(41, k=1)
    want = _oracle_visible(ow, q[iu], q[ju])            # from = qs[i], to = qs[j], i < j
    assert 0 < want.sum() < want.size                   # both verdicts occur
    assert (got[iu, ju] == want).all()
    assert (got == got.T).all()
    assert (np.diag(got) == 0).all()


def test_visibility_matrix_non_unit_inputs(built_lib, world):
    uw, ow = world
    qu = _free_keys(uw, 13, 302)
    qw = uw.translate_from_unit_state(qu)               # the same keys in the world frame
    got = uw.calculate_visibility_matrix(qw, False, VERIFY)
    qt = uw.translate_to_unit_state(qw)
    iu, ju = np.triu_indices(13, k=1)
    assert (got[iu, ju] == _oracle_visible(ow, qt[iu], qt[ju])).all()
    assert (got == got.T).all()


def test_visibility_matrix_small_sizes(built_lib, world):
    uw, _ = world
    q = _free_keys(uw, 2, 303)
    assert uw.calculate_visibility_matrix(q[:1], True, VERIFY).shape == (1, 1)
    assert (uw.calculate_visibility_matrix(q[:1], True, VERIFY) == 0).all()
    assert uw.calculate_visibility_matrix(np.zeros((0, 7)), True, VERIFY).shape == (0, 0)
    two = uw.calculate_visibility_matrix(q, True, VERIFY)
    assert two[0, 0] == 0 and two[1, 1] == 0 and two[0, 1] == two[1, 0]


def test_visibility_matrix2_matches_oracle(built_lib, world):
    uw, ow = world
    a = _free_keys(uw, 17, 304)
    b = _free_keys(uw, 23, 305)
    bw = uw.translate_from_unit_state(b)
    got = uw.calculate_visibility_matrix2(a, True, bw, False, VERIFY)
    assert got.dtype == np.int8 and got.shape == (17, 23)
    bt = uw.translate_to_unit_state(bw)
    want = _oracle_visible(ow, np.repeat(a, 23, axis=0), np.tile(bt, (17, 1))).reshape(17, 23)
    assert 0 < want.sum() < want.size
    assert (got == want).all()


def test_visibility_matrix2_chunked(built_lib, world, monkeypatch):
    """Pair chunks smaller than the grid: the flat indices of later chunks decode
    to the right (i, j)."""
    uw, ow = world
    a = _free_keys(uw, 9, 306)
    b = _free_keys(uw, 11, 307)
    whole = uw.calculate_visibility_matrix2(a, True, b, True, VERIFY)
    monkeypatch.setattr(type(uw), "_PAIR_CHUNK", 7)
    assert (uw.calculate_visibility_matrix2(a, True, b, True, VERIFY) == whole).all()
    m = uw.calculate_visibility_matrix(a, True, VERIFY)
    monkeypatch.setattr(type(uw), "_PAIR_CHUNK", 1 << 22)
    assert (uw.calculate_visibility_matrix(a, True, VERIFY) == m).all()


def test_visibility_pair_matches_oracle(built_lib, world):
    uw, ow = world
    a = _free_keys(uw, 64, 308)
    b = _free_keys(uw, 64, 309)
    got = uw.calculate_visibility_pair(a, True, b, True, VERIFY)
    assert got.dtype == np.int8 and got.shape == (64,)
    assert (got == _oracle_visible(ow, a, b)).all()
