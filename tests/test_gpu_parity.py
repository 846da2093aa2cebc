"""GPU path vs the CPU oracle: verdicts and first-contact steps must be identical.

All queries go through libpwcollide.so (UnitWorld -> C ABI).  Sizes are ones
the oracle finishes in seconds; the full-size workloads are covered by
size-independent properties in test_gpu_properties.py.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pair(O, Ve, Fe, Vr, Fr, center=None):
    import puzzletunneldiscovery_gb300 as pw
    uw = pw.UnitWorld()
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    if center is not None:
        uw.enforceRobotCenter(center)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    ow = O.OracleWorld(Ve, Fe, Vr, Fr, center=None if center is None else np.asarray(center, dtype=np.float32))
    return uw, ow


@pytest.fixture(scope="module")
def tori(oracle_mod, built_lib):
    return _pair(oracle_mod, *W.cfg_interlocking_tori())


@pytest.fixture(scope="module")
def alpha(oracle_mod, built_lib):
    g = golden("alpha_puzzle.npz")
    uw, ow = _pair(oracle_mod, g["Ve"], g["Fe"], g["Vr"], g["Fr"], center=g["center"].astype(np.float32))
    return uw, ow, g


def test_host_array_entry_points_match_device(tori):
    """is_valid_states_host / first_contact_steps_host (host batches streamed in
    chunks, copies overlapping checks) give the device path's answers, for numpy
    and pinned inputs and a batch that is no multiple of the chunk."""
    uw, ow = tori
    q = W.uniform_states(100_003, -2.0, 2.0, uw.scene_scale, seed=31)
    want = uw.is_valid_states(torch.from_numpy(q)).cpu()
    for src in (q, torch.from_numpy(q).pin_memory()):
        got = uw.is_valid_states_host(src, chunk=7_919)
        assert got.is_pinned() and got.dtype == torch.bool and torch.equal(got, want)
    q0, q1 = W.segment_batch(20_001, -2.0, 2.0, uw.scene_scale, seed=32)
    f = uw.first_contact_steps(torch.from_numpy(q0), torch.from_numpy(q1), 0.001).cpu()
    for chunk in (1 << 22, 4_999):
        got = uw.first_contact_steps_host(q0, q1, 0.001, chunk=chunk)
        assert got.dtype == torch.int32 and torch.equal(got, f)
    e, _ = ow.segments_first_contact(q0[:300], q1[:300], 0.001)
    assert (f[:300].numpy() == e).all()
    assert uw.is_valid_states_host(np.zeros((0, 7))).shape == (0,)
    with pytest.raises(ValueError):
        uw.first_contact_steps_host(q0, q1[:-1], 0.001)


def test_cd_vertices_and_scale_match(tori):
    uw, ow = tori
    assert uw.scene_scale == ow.scene_scale
    V, _ = uw._cd(0)
    assert (V == ow.vertices(0)).all()
    V, _ = uw._cd(1)
    assert (V == ow.vertices(1)).all()


def test_states_regression_vectors(tori):
    uw, ow = tori
    g = golden("torus_regression.npz")
    v = uw.is_valid_states(torch.from_numpy(g["states"])).cpu().numpy()
    assert (v == g["valid"]).all()
    d = uw.is_disentangled_states(torch.from_numpy(g["states"])).cpu().numpy()
    assert (d == g["disentangled"]).all()


def test_states_cfg0_parity(tori):
    """The interlocking-tori state workload (100k states) against the oracle."""
    uw, ow = tori
    q = W.uniform_states(100_000, -2.0, 2.0, ow.scene_scale, seed=0)
    gpu = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
    cpu = ow.is_valid(q)
    assert (gpu == cpu).all(), int((gpu != cpu).sum())
    st = uw.last_stats()
    assert st["queries"] == q.shape[0]
    d = uw.is_disentangled_states(torch.from_numpy(q)).cpu().numpy()
    assert (d == ow.is_disentangled(q)).all()


def test_segments_regression_vectors(tori):
    uw, ow = tori
    g = golden("torus_regression.npz")
    f = uw.first_contact_steps(torch.from_numpy(g["seg_from"]), torch.from_numpy(g["seg_to"]),
                               float(g["delta"])).cpu().numpy()
    assert (f == g["first"]).all()
    t = uw.first_contact_steps(torch.from_numpy(g["seg_from"]), torch.from_numpy(g["seg_to"]),
                               float(g["delta"]), mode=1).cpu().numpy()
    assert (t == g["transition_first"]).all()


def test_segments_cfg1_sample_parity(tori):
    uw, ow = tori
    q0, q1 = W.segment_batch(1500, -2.0, 2.0, ow.scene_scale, seed=7)
    gpu = uw.first_contact_steps(torch.from_numpy(q0), torch.from_numpy(q1), 0.001).cpu().numpy()
    cpu, _ = ow.segments_first_contact(q0, q1, 0.001)
    assert (gpu == cpu).all(), int((gpu != cpu).sum())


def test_near_contact_states(tori, oracle_mod):
    """States at and just before each segment's first contact: the FP32 band's hardest inputs."""
    uw, ow = tori
    q0, q1 = W.segment_batch(400, -2.0, 2.0, ow.scene_scale, seed=11)
    first, _ = ow.segments_first_contact(q0, q1, 0.001)
    rows = []
    for a, b, k in zip(q0, q1, first):
        if k > 0:
            for kk in (k - 1, k):
                s, _ = oracle_mod.segment_state(a, b, 0.001, kk)
                rows.append(s)
    rows = np.array(rows)
    # bisect each contact to ~1e-12 in tau to get states within rounding of touching
    fine = []
    for a, b, k in list(zip(q0, q1, first))[:120]:
        if k <= 0:
            continue
        lo, _ = oracle_mod.segment_state(a, b, 0.001, k - 1)
        hi, _ = oracle_mod.segment_state(a, b, 0.001, k)
        for _ in range(40):
            mid = oracle_mod.interpolate(lo, hi, 0.5)
            if ow.is_valid(mid)[0]:
                lo = mid
            else:
                hi = mid
        fine += [lo, hi]
    rows = np.concatenate([rows, np.array(fine)]) if fine else rows
    gpu = uw.is_valid_states(torch.from_numpy(rows)).cpu().numpy()
    cpu = ow.is_valid(rows)
    assert (gpu == cpu).all(), int((gpu != cpu).sum())
    assert uw.last_stats()["retests"] > 0   # the band was exercised


def test_rl_alpha_states_expected_free(built_lib):
    """src/RL/test_collide.py:39-53 (env-1.2.obj + robot.obj): the two states the
    reference expects free are free on the engine, and the script's x sweep
    gives the oracle's committed verdicts, through is_valid_state and the batch."""
    import puzzletunneldiscovery_gb300 as pw
    from conftest import golden
    g = golden("alpha_rl.npz")
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(g["Ve"], g["Fe"])
    uw.load_robot_mesh(g["Vr"], g["Fr"])
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    for q in g["expect_free"]:
        assert uw.is_valid_state(q) is True
    v = uw.is_valid_states(torch.from_numpy(g["sweep"])).cpu().numpy()
    assert (v == g["sweep_valid"]).all()


def test_alpha_puzzle_states_and_path(alpha):
    uw, ow, g = alpha
    s = uw.scene_scale
    U = []
    for p in g["keys_wfirst"]:
        U.append(np.concatenate([p[:3] * s, p[3:7] / np.linalg.norm(p[3:7])]))
    U = np.array(U)
    assert uw.is_valid_states(torch.from_numpy(U)).cpu().numpy().all()
    f = uw.first_contact_steps(torch.from_numpy(U[:-1]), torch.from_numpy(U[1:]), 0.0005).cpu().numpy()
    assert (f == -1).all()
    # random states around the puzzle
    q = W.uniform_states(20_000, -60.0, 60.0, s, seed=2)
    q[:, :3] += ow.vertices(0).mean(axis=0)
    assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()


def test_ompl_conversion_matches_unit_recipe(alpha):
    """translateOMPLStateToUnitState (unit_world.cc:689-711): w-last -> w-first, scale, then
    t' = t - R(q) (ompl_centre - centre) * scale, where the enforced centre differs from the
    vertex mean."""
    import puzzletunneldiscovery_gb300 as pw
    uw, ow, g = alpha
    U = uw.translate_ompl_to_unit(g["path_wlast"])
    info = uw.info()
    s = uw.scene_scale
    dc = (info["robot_ompl_center"].astype(np.float32) - info["robot_center"].astype(np.float32)).astype(np.float64) * s
    for p, u in zip(g["path_wlast"], U):
        q = np.array([p[6], p[3], p[4], p[5]])
        q = q / np.linalg.norm(q)
        R, _ = pw.state_transform(np.concatenate([[0, 0, 0], q]))
        np.testing.assert_allclose(u[:3], p[:3] * s - R @ dc, rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(u[3:], q, rtol=1e-12, atol=1e-15)
    # the reference's own scripts place the w-first keys with translate_to_unit_state
    K = uw.translate_to_unit_state(g["keys_wfirst"])
    assert uw.is_valid_states(torch.from_numpy(K)).cpu().numpy().all()
    back = uw.translate_from_unit_state(K)
    np.testing.assert_allclose(back[:, :3], g["keys_wfirst"][:, :3], rtol=1e-6)


def test_edge_cases(tori, oracle_mod):
    uw, ow = tori
    empty = torch.zeros((0, 7), dtype=torch.float64)
    assert uw.is_valid_states(empty).numel() == 0
    assert uw.first_contact_steps(empty, empty, 0.01).numel() == 0
    # non-unit quaternions are used raw, as translate_state_to_transform does
    q = W.uniform_states(3000, -2.0, 2.0, ow.scene_scale, seed=4)
    q[:, 3:] *= np.random.default_rng(0).uniform(0.5, 1.5, size=(3000, 1))
    assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()
    assert (uw.is_disentangled_states(torch.from_numpy(q)).cpu().numpy() == ow.is_disentangled(q)).all()
    # far away, identical endpoints, delta >= dist
    a = np.array([[4.0, 4.0, 4.0, 1, 0, 0, 0]])
    b = a.copy()
    b[0, 0] += 0.0001
    f = uw.first_contact_steps(torch.from_numpy(a), torch.from_numpy(b), 0.001).cpu().numpy()
    assert f[0] == -2
    f = uw.first_contact_steps(torch.from_numpy(a), torch.from_numpy(a), 0.001, mode=1).cpu().numpy()
    assert f[0] == -2
    with pytest.raises(RuntimeError):
        uw.first_contact_steps(torch.from_numpy(a), torch.from_numpy(b), 0.0)


def test_transit_tuple_matches_oracle(tori, oracle_mod):
    uw, ow = tori
    q0, q1 = W.segment_batch(40, -2.0, 2.0, ow.scene_scale, seed=9)
    for a, b in zip(q0, q1):
        got = uw.transit_state_to_with_contact(a, b, 0.002)
        exp, _, _ = ow.transit_state_to_with_contact(a, b, 0.002)
        assert (got[0] == exp[0]).all() and (got[1] == exp[1]).all()
        assert got[2] == exp[2] and got[3] == exp[3] and got[4] == exp[4]
        assert uw.is_valid_transition(a, b, 0.002) == (ow.segments_first_contact(a, b, 0.002, mode=1)[0][0] == -1)


def test_perturbation(tori, oracle_mod):
    uw, ow = tori
    p = np.array([0.05, -0.02, 0.01, 0.9, 0.1, 0.3, -0.2])
    p[3:] /= np.linalg.norm(p[3:])
    uw.set_perturbation(p)
    ow.set_perturbation(p)
    try:
        q = W.uniform_states(5000, -2.0, 2.0, ow.scene_scale, seed=6)
        assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()
        assert (uw.is_disentangled_states(torch.from_numpy(q)).cpu().numpy() == ow.is_disentangled(q)).all()
        # the rotated-perturbation form of the FP32 box test over many tiles per block
        q2 = W.uniform_states(1_500_007, -2.0, 2.0, ow.scene_scale, seed=7)
        assert (uw.is_disentangled_states(torch.from_numpy(q2)).cpu().numpy() == ow.is_disentangled(q2)).all()
    finally:
        ident = np.array([0, 0, 0, 1, 0, 0, 0.0])
        uw.set_perturbation(ident)
        ow.set_perturbation(ident)


def test_intersecting_segments_match(tori):
    uw, ow = tori
    for q in (np.array([0.0, 0.0, 0.0, 1, 0, 0, 0]), np.array([0.1, 0.05, 0.0, 0.96, 0.2, 0.1, 0.17]),
              np.array([5.0, 5.0, 5.0, 1, 0, 0, 0])):
        b, e, m, p = uw.intersecting_segments(q)
        b2, e2, m2, p2, c2 = ow.intersecting_segments(q)
        assert (p == p2).all()
        assert (b == b2).all() and (e == e2).all() and (m == m2).all()


def test_single_triangle_meshes(oracle_mod, built_lib):
    """The fclcontacts pair as one-triangle meshes: BVHs with a single leaf."""
    k = golden("fcl_kat.npz")
    Ve = k["tri_h"].astype(np.float32)
    Vr = k["tri_v"].astype(np.float32)
    F = np.array([[0, 1, 2]], dtype=np.uint32)
    uw, ow = _pair(oracle_mod, Ve, F, Vr, F)
    q = W.uniform_states(2000, -1.0, 1.0, ow.scene_scale, seed=1)
    assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()


@pytest.fixture(scope="module")
def plate(oracle_mod, built_lib):
    """Perforated plate (269k triangles) and a (2,3) torus knot (8192 triangles)."""
    return _pair(oracle_mod, *W.cfg_plate_knot())


def test_plate_knot_states_parity(plate):
    uw, ow = plate
    Ve = ow.Ve
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    q = W.uniform_states(60_000, lo, hi, ow.scene_scale, seed=5)
    gpu = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
    cpu = ow.is_valid(q)
    assert (gpu == cpu).all(), int((gpu != cpu).sum())
    assert 0.01 < cpu.mean() < 0.99
    info = uw.info()
    assert info["env_faces"] == ow.info()["nf_env"] and info["env_bvh_depth"] > 15


def test_plate_knot_segments_parity(plate):
    uw, ow = plate
    Ve = ow.Ve
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    q0, q1 = W.segment_batch(600, lo, hi, ow.scene_scale, sigma_t=0.3, seed=8)
    gpu = uw.first_contact_steps(torch.from_numpy(q0), torch.from_numpy(q1), 0.001).cpu().numpy()
    cpu, _ = ow.segments_first_contact(q0, q1, 0.001)
    assert (gpu == cpu).all(), int((gpu != cpu).sum())


def test_force_directions_from_contacts(tori):
    """force_direction_from_intersecting_segments (unit_world.cc:1038-1057) on the
    contacts of a colliding state: midpoints, and directions built from the
    oracle's vertices."""
    uw, ow = tori
    q = np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0])       # robot ring through the env ring
    b, e, mag, faces = uw.intersecting_segments(q)
    assert len(b) > 0
    pos, d = uw.force_direction_from_intersecting_segments(b, e, faces)
    assert np.allclose(pos, 0.5 * (b + e))
    Ve, Vr = ow.vertices(0), ow.vertices(1)
    _, Fe = uw._cd(0)
    _, Fr = uw._cd(1)

    def normals(V, F, idx):
        n = np.cross(V[F[idx, 1]] - V[F[idx, 0]], V[F[idx, 2]] - V[F[idx, 0]])
        return n / np.linalg.norm(n, axis=1, keepdims=True)

    nr = normals(Vr, Fr, faces[:, 1])
    ne = normals(Ve, Fe, faces[:, 0])
    want = np.cross(e - b, nr)
    want *= np.sign(np.sum(want * ne, axis=1))[:, None]
    assert np.allclose(d, want, atol=1e-12)
    assert np.allclose(uw.robot_face_normals_from_index_pairs(faces), nr)
    assert np.allclose(uw.scene_face_normals_from_indices(faces[:, 0]), ne)


def test_ompl_screening_of_the_alpha_path(alpha):
    """validate_states / validate_motion_pairs (ompldriver.cc:566-621) on OMPL-frame
    states made from the alpha puzzle's free keys (translate_unit_to_ompl, the
    inverse of the translateOMPLStateToUnitState rule they are checked with):
    every key and every edge between consecutive keys is valid; perturbed
    states collide exactly where the oracle says."""
    from puzzletunneldiscovery_gb300 import ompl_compat as OC
    uw, ow, g = alpha
    K = uw.translate_to_unit_state(g["keys_wfirst"])
    P = uw.translate_unit_to_ompl(K)
    np.testing.assert_allclose(uw.translate_ompl_to_unit(P), K, rtol=1e-9, atol=1e-12)
    v = OC.validate_states(uw, P)
    assert v.dtype == np.int32 and v.shape == (len(P),) and v.all()
    m = OC.validate_motion_pairs(uw, P[:-1], P[1:], 0.0005)
    assert m.shape == (len(P) - 1,) and m.all()
    # shorter second batch: trailing rows stay 0, as in the reference
    m2 = OC.validate_motion_pairs(uw, P[:10], P[1:6], 0.0005)
    assert m2.shape == (10,) and m2[:5].all() and not m2[5:].any()
    # perturbed states: verdicts equal the oracle's on the converted states
    rng = np.random.default_rng(4)
    Q = P[rng.integers(0, len(P), 2000)].copy()
    Q[:, :3] += rng.normal(0, 3.0, (2000, 3))
    U = uw.translate_ompl_to_unit(Q)
    got = OC.validate_states(uw, Q)
    assert 0 < got.sum() < len(Q)
    assert (got == ow.is_valid(U).astype(np.int32)).all()


def test_disentangled_fp32_and_fp64_paths(tori):
    """is_disentangled_states (FP32 box test, FP64 for undecided states queued to a
    second kernel) equals the oracle (unit_world.cc:249-264) on states built to lie
    within rounding of the boxes' contact, on a misaligned batch (scalar staging)
    and on a ragged tail."""
    uw, ow = tori
    s = ow.scene_scale
    q = W.uniform_states(300_001, -2.0, 2.0, s, seed=41)
    got = uw.is_disentangled_states(torch.from_numpy(q)).cpu().numpy()
    assert (got == ow.is_disentangled(q)).all()
    # near contact: bisect the translation scale between a touching and a separated state
    rng = np.random.default_rng(42)
    near = []
    for _ in range(2000):
        a = W.uniform_states(1, -0.3, 0.3, s, seed=int(rng.integers(1 << 30)))[0]
        v = rng.normal(size=3)
        lo, hi = 0.0, 8.0
        b = a.copy()
        b[:3] = a[:3] + hi * v
        if not ow.is_disentangled(a[None])[0] and ow.is_disentangled(b[None])[0]:
            for _ in range(60):
                mid = 0.5 * (lo + hi)
                c = a.copy()
                c[:3] = a[:3] + mid * v
                if ow.is_disentangled(c[None])[0]:
                    hi = mid
                else:
                    lo = mid
            for t in (lo, hi):
                c = a.copy()
                c[:3] = a[:3] + t * v
                near.append(c)
    near = np.array(near)
    got = uw.is_disentangled_states(torch.from_numpy(near)).cpu().numpy()
    assert (got == ow.is_disentangled(near)).all() and got.sum() > 100 and (got == 0).sum() > 100
    assert uw.last_stats()["retests"] > 0.5 * near.shape[0]        # near contact: the FP64 test decided
    # an offset view: 8-byte aligned rows, the scalar staging path
    dq = torch.from_numpy(q).cuda().reshape(-1)[7:].reshape(-1, 7)
    got = uw.is_disentangled_states(dq).cpu().numpy()
    assert (got == ow.is_disentangled(q[1:])).all()
    # a batch of many tiles per block: the bulk-copy ring wraps around its stages several times
    big = W.uniform_states(4_000_037, -2.0, 2.0, s, seed=43)
    got = uw.is_disentangled_states(torch.from_numpy(big)).cpu().numpy()
    assert (got == ow.is_disentangled(big)).all()
    assert uw.last_stats()["device_errors"] == 0
