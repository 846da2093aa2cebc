"""The rest of pyosr's UnitWorld surface that the planner's scripts call next to
the collision queries: discrete-action transits (transit_state /
transit_state_by) against the oracle's transit loop, the vanilla-frame
conversions, the kinetic-energy metric and the samplers' method names."""
import math

import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import state_ops as S
from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, oracle_mod.OracleWorld(Ve, Fe, Vr, Fr), (Ve, Fe, Vr, Fr)


def _free_starts(uw, n, seed):
    q = W.uniform_states(4000, -1.5, 1.5, uw.scene_scale, seed=seed)
    v = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
    return q[v][:n]


def _oracle_transit(ow, a, to, cvd):
    (lf, _, done, lt, _), _, _ = ow.transit_state_to_with_contact(a, to, float(cvd))
    return lf, done, lt


def test_transit_state_actions_match_the_oracle(built_lib, world):
    """Each of the 12 actions: the target the reference builds (float32 step,
    doubled for rotations), then the transit with the float32 step halved while
    there is no progress, checked against the oracle's transit loop."""
    uw, ow, _ = world
    vd = 0.02
    for st in _free_starts(uw, 4, 51):
        for action in range(12):
            free, done, prog = uw.transit_state(st, action, 0.0, vd)
            typ = 0 if action < 6 else 1
            cap = np.float32(vd) if typ == 0 else np.float32(vd * 2)
            sym = np.float32(1.0 if action % 2 == 0 else -1.0)
            ax = np.zeros(3)
            ax[(action - 6 * typ) // 2] = 1.0
            t, r = S.decompose(st)
            if typ == 0:
                t = t + float(cap) * ax * float(sym)
            else:
                r = S.quat_mul(S.quat_from_angleaxis(float(np.float32(cap * sym)), ax), r)
            to = S.compose(t, r)
            cvd = np.float32(vd)
            while True:
                lf, d, lt = _oracle_transit(ow, st, to, cvd)
                if lt > 0 or cvd == 0:
                    break
                cvd = np.float32(cvd / 2)
            assert np.array_equal(free, lf) and done == d and np.float32(prog) == lt, action
            assert uw.is_valid_state(free)
    # an invalid action, or a start in collision, returns the start unchanged
    st = _free_starts(uw, 1, 52)[0]
    q, d, p = uw.transit_state(st, 12, 0.0, vd)
    assert np.array_equal(q, st) and d is False and p == 0.0
    coll = np.array([0.0, 0, 0, 1, 0, 0, 0])       # coincident tori: in collision
    assert not uw.is_valid_state(coll)
    q, d, p = uw.transit_state(coll, 0, 0.0, vd)
    assert np.array_equal(q, coll) and d is False


def test_transit_state_by_matches_the_oracle(built_lib, world):
    uw, ow, _ = world
    rng = np.random.default_rng(53)
    for st in _free_starts(uw, 6, 54):
        tr = rng.normal(0, 0.05, 3)
        aav = rng.normal(0, 0.3, 3)
        free, done, prog = uw.transit_state_by(st, tr, aav, 0.005)
        n = np.linalg.norm(aav)
        to = np.concatenate([st[:3] + tr, S.quat_mul(S.quat_from_angleaxis(n, aav / n), st[3:])])
        lf, d, lt = _oracle_transit(ow, st, to, 0.005)
        assert np.array_equal(free, lf) and done == d and np.float32(prog) == lt


def test_vanilla_frames(built_lib, world):
    uw, _, (Ve, Fe, Vr, Fr) = world
    q = _free_starts(uw, 20, 55)
    wl = q[:, [0, 1, 2, 4, 5, 6, 3]]                 # w-last, as vanilla / OMPL states are
    back = uw.translate_ompl_to_vanilla(uw.translate_vanilla_to_ompl(wl))
    assert np.allclose(back, wl, atol=1e-12)
    assert np.array_equal(uw.translate_vanilla_to_unit(wl), uw.translate_ompl_to_unit(uw.translate_vanilla_to_ompl(wl)))
    # the OMPL centre maps to the unit-frame position of the robot's reference point
    oc = uw.get_ompl_center()
    R = S.quat_to_matrix(q[0, 3:7])
    assert np.allclose(uw.translate_vanilla_to_ompl(wl[:1])[0, :3], wl[0, :3] + R @ oc)
    # env mesh points in their own frame land on the env CD vertices
    Vcd, _ = uw._cd(0)
    assert np.allclose(uw.translate_vanilla_pts_to_unit(uw.GEO_ENV, Ve.astype(np.float64)), Vcd, atol=1e-6)
    assert uw.translate_vanilla_pts_to_unit(uw.GEO_ROB, np.zeros((0, 3))).shape == (0, 3)


def test_kinetic_energy_distance(built_lib, world):
    uw, _, _ = world
    q = _free_starts(uw, 10, 56)
    inertia, vol = uw._robot_mass_properties()
    s = uw.scene_scale
    # torus R = 1, r = 0.25 scaled by s: 2 pi^2 R r^2 s^3, the 64 x 32 tessellation a little less
    exact = 2 * math.pi ** 2 * 1.0 * 0.25 ** 2 * s ** 3
    assert 0.97 * exact < vol < exact
    assert np.allclose(inertia, inertia.T)
    assert abs(uw.kinetic_energy_distance(q[0], q[0])) < 1e-20    # q q^-1 leaves a rounding residue
    moved = q[0].copy()
    moved[:3] += [0.01, -0.02, 0.03]
    assert math.isclose(uw.kinetic_energy_distance(q[0], moved), 0.01 ** 2 + 0.02 ** 2 + 0.03 ** 2, rel_tol=1e-12)
    d = uw.multi_kinetic_energy_distance(q[0], q)
    assert d.shape == (10,) and abs(d[0]) < 1e-20
    assert all(math.isclose(d[i], uw.kinetic_energy_distance(q[0], q[i])) for i in range(10))


def test_sampler_method_names(built_lib, world):
    from puzzletunneldiscovery_gb300 import sampling
    uw, _, _ = world
    args = (np.array([0.0, 0.0, 0.1]), np.array([0.0, 0.0, 1.0]), np.array([0.3, 0.0, 0.0]),
            np.array([1.0, 0.0, 0.0]), 1e-4)
    a = uw.enum_free_configuration(*args, 64)
    b = sampling.enum_free_configuration(uw, *args, 64)
    assert np.array_equal(a, b)
    if a.shape[0] > 0:
        # max_trials -1 tries until a free spin is found; the enumeration shows one exists
        q = uw.sample_free_configuration(*args)
        assert uw.is_valid_state(q)
    q2 = uw.sample_free_configuration(*args, max_trials=0)
    assert q2.shape == (7,)
