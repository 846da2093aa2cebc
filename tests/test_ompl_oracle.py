"""The oracle's restatement of OMPL's discrete motion check (OMPL 1.x, un-vendored
by the reference; the check behind OmplDriver::validateMotionPairs,
lib/pyse3ompl/ompldriver.cc:597-621) against closed forms: the segment count of
pure translations and pure rotations, and the interpolated states of a rotation
about one axis.  No device needed."""
import math
import os

import numpy as np
import pytest

from conftest import ROOT


def _rot_z(phi, t=(0.0, 0.0, 0.0)):
    # OMPL state (x, y, z, qx, qy, qz, qw) of a rotation by phi about z
    return np.array([t[0], t[1], t[2], 0.0, 0.0, math.sin(phi / 2), math.cos(phi / 2)])


def test_segment_lengths(oracle_mod):
    O = oracle_mod
    lvs = O.ompl_lvs([-1, -2, -3], [1, 2, 3], 0.01)
    assert lvs[0] == pytest.approx(math.sqrt(4 + 16 + 36) * 0.01, rel=1e-15)
    assert lvs[1] == pytest.approx(math.pi / 2 * 0.01, rel=1e-15)


@pytest.mark.parametrize("length,cdres", [(0.5, 0.01), (1.0, 0.003), (3.7, 0.05), (0.0, 0.01)])
def test_translation_counts(oracle_mod, length, cdres):
    O = oracle_mod
    lo, hi = [-1, -1, -1], [1, 1, 1]
    a = _rot_z(0.0)
    b = _rot_z(0.0, (length, 0.0, 0.0))
    s = O.ompl_motion_states(a, b, lo, hi, cdres)
    nd = math.ceil(length / (math.sqrt(12.0) * cdres))
    assert s.shape[0] == max(nd, 1)
    assert np.array_equal(s[0], b)
    if nd >= 2:
        xs = s[1:, 0]
        want = np.arange(1, nd) / nd * length
        assert np.allclose(xs, want, rtol=0, atol=1e-15)
        # rotations untouched: the arc length is 0, OMPL copies `from`
        assert (s[1:, 3:] == a[3:]).all()


@pytest.mark.parametrize("phi,cdres", [(0.3, 0.01), (2.5, 0.02), (math.pi * 0.99, 0.1)])
def test_rotation_counts_and_slerp(oracle_mod, phi, cdres):
    O = oracle_mod
    a, b = _rot_z(0.0), _rot_z(phi)
    s = O.ompl_motion_states(a, b, [-1, -1, -1], [1, 1, 1], cdres)
    # SO(3) arc length of OMPL is acos|<q1, q2>| = phi / 2
    nd = math.ceil((phi / 2) / (math.pi / 2 * cdres))
    assert s.shape[0] == max(nd, 1)
    for k in range(1, nd):
        want = _rot_z(phi * k / nd)
        assert np.allclose(s[k], want, rtol=0, atol=1e-13), k


def test_long_way_round_takes_the_short_arc(oracle_mod):
    """q and -q are the same rotation: OMPL's slerp negates s1 for a negative dot,
    so a motion to -q(phi) rotates by phi, not by 2 pi - phi."""
    O = oracle_mod
    a, b = _rot_z(0.0), _rot_z(1.0)
    b[3:] = -b[3:]
    s = O.ompl_motion_states(a, b, [-1, -1, -1], [1, 1, 1], 0.05)
    nd = s.shape[0]
    assert nd == math.ceil(0.5 / (math.pi / 2 * 0.05))
    mid = s[nd // 2]
    angle = 2 * math.atan2(abs(mid[5]), abs(mid[6]))
    assert angle == pytest.approx(1.0 * (nd // 2) / nd, abs=1e-12)


def test_nearly_identical_rotations_are_not_interpolated(oracle_mod):
    """Above |<q1, q2>| > 1 - 1e-9 OMPL's arc length is 0 and interpolate copies
    the start rotation."""
    O = oracle_mod
    a = _rot_z(0.0)
    b = _rot_z(1e-5, (0.5, 0.0, 0.0))
    s = O.ompl_motion_states(a, b, [-1, -1, -1], [1, 1, 1], 0.01)
    assert s.shape[0] == math.ceil(0.5 / (math.sqrt(12.0) * 0.01))
    assert (s[1:, 3:] == a[3:]).all()


def test_count_is_symmetric(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(7)
    lo, hi = [-5, -5, -5], [5, 5, 5]
    for _ in range(200):
        a = np.concatenate([rng.uniform(-5, 5, 3), rng.normal(size=4)])
        b = np.concatenate([rng.uniform(-5, 5, 3), rng.normal(size=4)])
        a[3:] /= np.linalg.norm(a[3:])
        b[3:] /= np.linalg.norm(b[3:])
        assert O.ompl_motion_states(a, b, lo, hi, 0.01).shape[0] == O.ompl_motion_states(b, a, lo, hi, 0.01).shape[0]


@pytest.fixture(scope="module")
def alpha_ompl(oracle_mod):
    import bench
    (Ve, Fe, Vr, Fr), c, P = bench._alpha_ompl()
    return oracle_mod.OracleWorld(Ve, Fe, Vr, Fr, center=c), P


def test_ompl_frame_conversion_closed_form(alpha_ompl):
    """or_ompl_to_unit (translateOMPLStateToUnitState, unit_world.cc:689-711) is
    t' = s t - R(q) (m - c) s with the w-first rotation, m the robot's vertex
    mean and c its enforced centre; the path's OMPL-frame states come back free."""
    ow, P = alpha_ompl
    U = ow.ompl_to_unit(P)
    import bench
    s = ow.scene_scale
    g = np.load(os.path.join(ROOT, "tests", "golden", "alpha_puzzle.npz"))
    acc = np.zeros(3, dtype=np.float32)
    for v in g["Vr"].astype(np.float32):
        acc = acc + v
    # float mean summed in order, minus the float centre, as the world stores them
    d = (acc / np.float32(len(g["Vr"])) - g["center"].astype(np.float32)).astype(np.float64) * s
    for p, u in zip(P, U):
        q = np.array([p[6], p[3], p[4], p[5]])
        q /= np.linalg.norm(q)
        assert np.allclose(u[:3], p[:3] * s - bench._quat_matrix(q) @ d, rtol=0, atol=1e-14)
        assert np.allclose(u[3:], q, rtol=0, atol=1e-15)
    assert ow.is_valid(U).all()


def test_early_exit_check_agrees_with_every_state(alpha_ompl, oracle_mod):
    """or_ompl_check_motions (OMPL's order, stopping at the first colliding state)
    gives the verdict of checking every state checkMotion lists, with at most as
    many checks; the path's own edges are valid."""
    import bench
    ow, P = alpha_ompl
    A, B, lo, hi = bench._ompl_motions(P, 600, seed=5)
    A = np.concatenate([A, P[:-1]])
    B = np.concatenate([B, P[1:]])
    v, checks = ow.ompl_check_motions(A, B, lo, hi, 0.01)
    for i in range(len(A)):
        S = oracle_mod.ompl_motion_states(A[i], B[i], lo, hi, 0.01)
        ok = ow.is_valid(ow.ompl_to_unit(S)).astype(bool)
        assert v[i] == ok.all(), i
        assert 1 <= checks[i] <= len(S)
        if ok.all():
            assert checks[i] == len(S)
        elif not ok[0]:
            assert checks[i] == 1
    assert v[-(len(P) - 1):].all()
    assert 0 < v[:600].sum() < 600


def test_non_finite_motions_are_invalid(alpha_ompl):
    ow, P = alpha_ompl
    A, B = P[:4].copy(), P[1:5].copy()
    A[1, 0] = np.nan
    B[2, 5] = np.inf
    v, checks = ow.ompl_check_motions(A, B, P[:, :3].min(0) - 20, P[:, :3].max(0) + 20, 0.01)
    assert v[1] == 0 and v[2] == 0 and checks[1] == 0 and checks[2] == 0
    assert v[0] == 1 and v[3] == 1


def _ompl_states_libm(a, b, lo, hi, cdres):
    """OMPL's rule written again with numpy's libm arccos / sin (an independent
    restatement of the same published algorithm)."""
    ext = math.sqrt(sum((h - l) ** 2 for l, h in zip(lo, hi)))
    dq = float(np.dot(a[3:], b[3:]))
    arc = 0.0 if abs(dq) > 1.0 - 1e-9 else math.acos(abs(dq))
    nd = max(math.ceil(np.linalg.norm(a[:3] - b[:3]) / (ext * cdres)), math.ceil(arc / (math.pi / 2 * cdres)))
    out = [b.copy()]
    for k in range(1, nd):
        t = k / nd
        s = np.empty(7)
        s[:3] = a[:3] + (b[:3] - a[:3]) * t
        if arc > np.finfo(float).eps:
            s1 = math.sin(t * arc) * (-1.0 if dq < 0 else 1.0)
            s[3:] = (a[3:] * math.sin((1 - t) * arc) + b[3:] * s1) / math.sin(arc)
        else:
            s[3:] = a[3:]
        out.append(s)
    return np.array(out)


def test_restatement_agrees_with_a_libm_version(oracle_mod):
    """The oracle's OMPL states (with this project's own sin / acos) agree with a
    libm-based restatement to 1e-13, with the same segment counts on random motions."""
    rng = np.random.default_rng(11)
    lo, hi = [-3, -3, -3], [3, 3, 3]
    for _ in range(300):
        a = np.concatenate([rng.uniform(-3, 3, 3), rng.normal(size=4)])
        b = np.concatenate([rng.uniform(-3, 3, 3), rng.normal(size=4)])
        a[3:] /= np.linalg.norm(a[3:])
        b[3:] /= np.linalg.norm(b[3:])
        got = oracle_mod.ompl_motion_states(a, b, lo, hi, 0.02)
        want = _ompl_states_libm(a, b, lo, hi, 0.02)
        assert got.shape == want.shape
        assert np.allclose(got, want, rtol=0, atol=1e-13)
