"""The oracle against the reference's own golden data and analytic cases (CPU)."""
import math

import numpy as np
import pytest

from conftest import golden
from puzzletunneldiscovery_gb300 import workloads as W


def test_fclcontacts_kat(oracle_mod):
    """sancheck/fclcontacts/main.cc:17-64: the two unit triangles collide."""
    k = golden("fcl_kat.npz")
    h, v = k["tri_h"], k["tri_v"]
    assert oracle_mod.tri_tri(list(v), list(h)) is True
    assert oracle_mod.tri_tri(list(h), list(v)) is True
    hit, cop, p1, p2 = oracle_mod.tri_tri_isect(list(h), list(v), eps=1e-6)
    assert hit and not cop
    np.testing.assert_allclose(np.stack([p1, p2]), k["isect"], atol=1e-12)
    # moved apart along y by more than the overlap: no contact
    assert oracle_mod.tri_tri(list(v + [0, 0.6, 0]), list(h)) is False


def _alpha_world(O):
    g = golden("alpha_puzzle.npz")
    w = O.OracleWorld(g["Ve"], g["Fe"], g["Vr"], g["Fr"], center=g["center"].astype(np.float32))
    return w, g


def _to_unit(states, s, wlast):
    out = []
    for p in states:
        q = np.array([p[6], p[3], p[4], p[5]]) if wlast else np.array(p[3:7])
        out.append(np.concatenate([p[:3] * s, q / np.linalg.norm(q)]))
    return np.array(out)


def test_rl_alpha_states_expected_free(oracle_mod):
    """src/RL/test_collide.py:39-53 on res/alpha/env-1.2.obj + robot.obj: the two
    states it prints with "Expecting True" are free; the oracle's x sweep matches
    the committed regression vector and is free at both ends of the sweep."""
    g = golden("alpha_rl.npz")
    w = oracle_mod.OracleWorld(g["Ve"], g["Fe"], g["Vr"], g["Fr"])
    assert w.is_valid(g["expect_free"]).all()
    v = w.is_valid(g["sweep"])
    assert (v == g["sweep_valid"]).all()
    assert v[:5].all() and v[-5:].all() and not v.all()


def test_alpha_solution_path_is_free(oracle_mod):
    """Every state of the reference's alpha-puzzle OMPL solution is collision-free."""
    w, g = _alpha_world(oracle_mod)
    s = w.scene_scale
    for key, wlast in (("path_wlast", True), ("keys_wfirst", False), ("tunnel", False), ("tunnel_more", False)):
        U = _to_unit(g[key], s, wlast)
        assert w.is_valid(U).all(), key


def test_alpha_path_segments_are_free(oracle_mod):
    w, g = _alpha_world(oracle_mod)
    U = _to_unit(g["keys_wfirst"], w.scene_scale, False)
    first, checks = w.segments_first_contact(U[:-1], U[1:], 0.001)
    assert (first == -1).all()
    assert checks.sum() > 0


def test_alpha_perturbed_states_collide(oracle_mod):
    """Pushing the robot far into the obstacle along the solution path makes it collide."""
    w, g = _alpha_world(oracle_mod)
    U = _to_unit(g["keys_wfirst"], w.scene_scale, False)
    V = w.vertices(0)
    c = V.mean(axis=0)
    moved = U.copy()
    moved[:, :3] = c
    assert (~w.is_valid(moved)).sum() > len(moved) // 2


def test_torus_analytic_cases(oracle_mod):
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    w = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    info = w.info()
    s = info["scene_scale"]
    assert s == pytest.approx(0.4, rel=1e-7)
    c = info["center"]
    assert np.allclose(c, [1.0, 0.0, 0.0], atol=1e-5)
    interlocked = np.array([s * c[0], s * c[1], s * c[2], 1, 0, 0, 0])
    assert w.is_valid(interlocked)[0]                       # chain links at rest: free
    assert not w.is_valid(np.array([0, 0, 0, 1, 0, 0, 0.0]))[0]   # robot centred on the env: colliding
    far = np.array([5.0, 5.0, 5.0, 1, 0, 0, 0])
    assert w.is_valid(far)[0] and w.is_disentangled(far)[0]
    assert not w.is_disentangled(interlocked)[0]
    # sliding the interlocked ring along x by 0.25 unit brings the tubes into contact
    hit = interlocked.copy()
    hit[0] += 0.25
    assert not w.is_valid(hit)[0]


def test_bvh_matches_brute_force(oracle_mod):
    Ve, Fe = W.torus(1.0, 0.25, 12, 6)
    Vr, Fr = W.torus(0.6, 0.2, 10, 5)
    w = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    q = W.uniform_states(1500, -1.2, 1.2, w.scene_scale, seed=3)
    a = w.is_valid(q)
    b = w.is_valid(q, brute=True)
    assert (a == b).all()
    assert 0.1 < a.mean() < 0.95


def test_deterministic_math_accuracy(oracle_mod):
    xs = np.linspace(-0.78, math.pi / 2, 4001)
    for x in xs:
        assert abs(oracle_mod.det_sin(x) - math.sin(x)) <= 4 * np.spacing(abs(math.sin(x))) + 1e-300
    for a in np.linspace(0.0, 1.0, 4001)[:-1]:
        r = math.acos(a)
        assert abs(oracle_mod.det_acos(a) - r) <= 4 * np.spacing(r)
    rng = np.random.default_rng(0)
    for _ in range(4000):
        y, x = rng.random(2) * 10.0 ** rng.uniform(-6, 6, 2)
        r = math.atan2(y, x)
        assert abs(oracle_mod.det_atan2(y, x) - r) <= 4 * np.spacing(r)


def test_stepping_rules(oracle_mod):
    """unit_world.cc:445-486: delta >= dist checks nothing; steps end exactly at tau = dist*inv."""
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    w = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    a = np.array([3.0, 3.0, 3.0, 1, 0, 0, 0])
    b = np.array([3.05, 3.0, 3.0, 1, 0, 0, 0])
    tup, first, checks = w.transit_state_to_with_contact(a, b, 1.0)
    assert first == -2 and checks == 0 and tup[2] is False and tup[4] == np.float32(1.0)
    tup, first, checks = w.transit_state_to_with_contact(a, b, 0.01)
    assert first == -1 and tup[2] is True
    assert checks == oracle_mod.segment_steps(a, b, 0.01) == 5
    assert tup[4] == np.float32(0.0)            # the reference's shadowed outer tau
    assert tup[3] == np.float32(1.0)
    # is_valid_transition(q, q) is false: min(0 / 2, delta) = 0 >= 0 = dist
    f, _ = w.segments_first_contact(a[None], a[None], 0.01, mode=1)
    assert f[0] == -2
    # delta <= 0 would never terminate in the reference: reported as invalid
    tup, first, checks = w.transit_state_to_with_contact(a, b, 0.0)
    assert first == -3


def test_torus_regression_vectors(oracle_mod):
    g = golden("torus_regression.npz")
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    w = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    assert (w.is_valid(g["states"]) == g["valid"]).all()
    assert (w.is_disentangled(g["states"]) == g["disentangled"]).all()
    f, c = w.segments_first_contact(g["seg_from"], g["seg_to"], float(g["delta"]))
    assert (f == g["first"]).all() and (c == g["checks"]).all()


def test_intersecting_segments_oracle(oracle_mod):
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    w = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    b, e, m, p, c = w.intersecting_segments(np.array([0.0, 0.0, 0.0, 1, 0, 0, 0]))
    assert len(m) > 0
    assert (np.diff(p[:, 0]) >= 0).all()
    np.testing.assert_allclose(m, np.linalg.norm(e - b, axis=1), rtol=1e-12, atol=1e-15)
    b, e, m, p, c = w.intersecting_segments(np.array([5.0, 5.0, 5.0, 1, 0, 0, 0]))
    assert len(m) == 0


def _tri_cases(seed):
    """Random pairs, pairs sharing a vertex or an edge, coplanar pairs, pairs with a
    vertex on the other's plane, pairs nudged around touching, and tiny pairs."""
    rng = np.random.default_rng(seed)
    out = [(rng.uniform(-1, 1, (3, 3)), rng.uniform(-1, 1, (3, 3))) for _ in range(3000)]
    for _ in range(500):
        V = rng.uniform(-1, 1, (3, 3))
        U = rng.uniform(-1, 1, (3, 3))
        U[0] = V[rng.integers(0, 3)]
        out.append((V, U.copy()))
        U[1] = V[(rng.integers(0, 3))]
        out.append((V, U.copy()))
        Vc, Uc = V.copy(), U.copy()
        Vc[:, 2] = 0.0
        Uc[:, 2] = 0.0
        out.append((Vc, Uc))
        n = np.cross(V[1] - V[0], V[2] - V[0])
        n /= np.linalg.norm(n)
        W = U.copy()
        W[0] -= np.dot(W[0] - V[0], n) * n          # a vertex on V's plane (to rounding)
        out.append((V, W))
        for eps in (1e-9, 1e-7, 1e-5):
            out.append((V, W + eps * rng.normal(size=(3, 3))))
    for _ in range(500):
        s = 0.0025
        out.append((rng.uniform(-1, 1, (3, 3)) * s, rng.uniform(-1, 1, (3, 3)) * s))
    return out


def test_moller_restatement_matches_the_reference_source(oracle_mod):
    """The oracle's Moller test with the reference's 1e-6 snap against the
    reference's own lib/tritri/Moller97d.cc (built from its source by
    oracle/Makefile): verdict, coplanarity and intersection-line endpoints bit
    for bit, on random and near-degenerate pairs."""
    import ctypes
    ref = oracle_mod.ref_lib()
    if ref is None:
        pytest.skip("the reference checkout is not present (its Moller source cannot be built here)")
    p = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    cases = _tri_cases(8)
    hits = cops = 0
    random_diffs = tiny_diffs = 0
    for i, (V, U) in enumerate(cases):
        args = [p(v) for v in V] + [p(u) for u in U]
        want = bool(ref.ref_tri_tri(*args))
        assert oracle_mod.tri_tri(list(V), list(U), eps=1e-6) is want
        cop = ctypes.c_int(0)
        r1, r2 = np.zeros(3), np.zeros(3)
        wi = bool(ref.ref_tri_tri_isect(*args, ctypes.byref(cop), p(r1), p(r2)))
        hit, coplanar, q1, q2 = oracle_mod.tri_tri_isect(list(V), list(U), eps=1e-6)
        assert hit is wi and coplanar is bool(cop.value)
        if wi and not cop.value:
            assert np.array_equal(q1, r1) and np.array_equal(q2, r2)
        hits += wi
        cops += bool(cop.value)
        # the engine's verdict takes no snap: on generic pairs it agrees with the
        # snapped one; on 0.0025-unit triangles (plate cells) the absolute 1e-6
        # snap of unnormalised plane distances swallows real separations
        diff = oracle_mod.tri_tri(list(V), list(U), eps=0.0) is not want
        if i < 3000:
            random_diffs += diff
        elif i >= len(cases) - 500:
            tiny_diffs += diff
    assert hits > 500 and cops > 100
    assert random_diffs == 0
    assert tiny_diffs > 0
