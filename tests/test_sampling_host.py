"""Host logic of the batched samplers (puzzletunneldiscovery_gb300/sampling.py)
and the oracle's key-configuration states, on the CPU."""
import math

import numpy as np
import torch

from conftest import ROOT  # noqa: F401


def _S():
    from puzzletunneldiscovery_gb300 import sampling
    return sampling


def _rotate(q, v):
    w, u = q[0], q[1:]
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def _half(angles):
    h = 0.5 * np.asarray(angles, np.float64)
    return np.cos(h), np.sin(h)


def test_keyconf_states_place_points_with_opposed_normals(oracle_mod):
    """The oracle's key-configuration states (unit_world.cc:1301-1330): the robot
    point + margin x normal lands on the env point + margin x normal, the robot
    normal turns into the opposed env normal; opposite and equal normals
    included (the half-turn branch of the shortest arc)."""
    rng = np.random.default_rng(1)
    P, A = 6, 7
    rp, ep = rng.normal(size=(P, 3)), rng.normal(size=(P, 3))
    rn = rng.normal(size=(P, 3))
    en = rng.normal(size=(P, 3))
    rn /= np.linalg.norm(rn, axis=1, keepdims=True)
    en /= np.linalg.norm(en, axis=1, keepdims=True)
    en[0] = -rn[0]                   # normals opposed already: the identity arc
    en[1] = rn[1]                    # equal normals: a half turn
    hc, hs = _half(rng.uniform(0, 2 * math.pi, (P, A)))
    qs = oracle_mod.keyconf_states(rp, rn, ep, en, 0.01, hc, hs)
    assert qs.shape == (P, A, 7)
    for p in range(P):
        for i in range(A):
            q = qs[p, i]
            assert abs(np.linalg.norm(q[3:]) - 1.0) < 1e-15
            placed = _rotate(q[3:], rp[p] + 0.01 * rn[p]) + q[:3]
            assert np.allclose(placed, ep[p] + 0.01 * en[p], atol=1e-12)
            assert np.allclose(_rotate(q[3:], rn[p]), -en[p], atol=1e-12)
    # the shared spin table gives the per-pair table's states when every row repeats it
    hc1, hs1 = _half(np.arange(A) * (2 * math.pi / A))
    a = oracle_mod.keyconf_states(rp, rn, ep, en, 0.01, hc1, hs1)
    b = oracle_mod.keyconf_states(rp, rn, ep, en, 0.01, np.tile(hc1, (P, 1)), np.tile(hs1, (P, 1)))
    assert np.array_equal(a, b)


def test_free_spins_on_device_style_tensors(oracle_mod):
    """_free_spins takes the states as a tensor [P, A, 7] and gathers the picks by
    index; the picks equal the oracle's restatement of the reference loop."""
    from puzzletunneldiscovery_gb300 import sampling as S
    rng = np.random.default_rng(2)
    for _ in range(50):
        P, A = int(rng.integers(1, 12)), int(rng.integers(1, 30))
        valid = rng.random((P, A)) < rng.random()
        qs = rng.random((P, A, 7))
        for med in (False, True):
            got = S._free_spins(torch.from_numpy(qs), valid, med)
            want = oracle_mod.free_spins(qs, valid, med)
            assert all(np.array_equal(x, y) for x, y in zip(got, want))


def test_apply_batch_matches_single_apply():
    S = _S()
    from puzzletunneldiscovery_gb300.unit_world import apply
    rng = np.random.default_rng(4)
    q0 = np.array([0.1, -0.2, 0.3, 0.5, 0.5, -0.5, 0.5])
    tr = rng.normal(size=(20, 3))
    aa = rng.normal(size=(20, 3))
    aa[0] = 0.0
    out = S.apply_batch(q0, tr, aa)
    for i in range(20):
        assert np.allclose(out[i], apply(q0, tr[i], aa[i]), atol=1e-15)


def test_random_directions():
    S = _S()
    rng = np.random.default_rng(5)
    s = S.random_on_sphere(1000, 1.0, rng)
    assert np.allclose(np.linalg.norm(s, axis=1), 1.0)
    b = S.random_within_sphere(1000, 2 * math.pi, rng)
    assert (np.linalg.norm(b, axis=1) <= 2 * math.pi + 1e-12).all()
    assert abs(s.mean(axis=0)).max() < 0.1


def test_narrow_midpoint_is_the_slerp_midpoint(oracle_mod):
    """narrow.midpoints equals interpolate(a, b, 1/2) (osr_state.cc:27-44) to rounding."""
    from puzzletunneldiscovery_gb300 import narrow as N
    from puzzletunneldiscovery_gb300 import workloads as W
    q0, q1 = W.segment_batch(300, -2, 2, 0.4, seed=3)
    m = N.midpoints(torch.from_numpy(q0), torch.from_numpy(q1)).numpy()
    for i in range(300):
        assert np.abs(m[i] - oracle_mod.interpolate(q0[i], q1[i], 0.5)).max() < 1e-14


def test_autotune_cache_keys_and_file(tmp_path):
    """The tuned-configuration cache: keys separate mesh pairs, GPU models and
    kernels; the JSON file round-trips and is replaced atomically."""
    from puzzletunneldiscovery_gb300.autotune import TuneCache, tune_key
    V = np.zeros((3, 3), np.float32)
    F = np.array([[0, 1, 2]], np.uint32)
    V2 = V.copy()
    V2[1, 0] = 1.0
    k = tune_key([(V, F), (V, F)], "GB300", 152, "states")
    assert k == tune_key([(V.copy(), F.copy()), (V, F)], "GB300", 152, "states")
    assert k != tune_key([(V2, F), (V, F)], "GB300", 152, "states")
    assert k != tune_key([(V, F), (V, F)], "GB300", 148, "states")
    assert k != tune_key([(V, F), (V, F)], "GB300", 152, "segments")
    c = TuneCache(str(tmp_path / "sub" / "tune.json"))
    assert c.get(k) is None
    c.put(k, {"config": {"width": 16, "soft_cap": 0, "blocks": 0}, "default_ms": 2.0, "best_ms": 1.5})
    c.put("other", {"config": {}, "default_ms": 1.0, "best_ms": 1.0})
    assert TuneCache(str(tmp_path / "sub" / "tune.json")).get(k)["config"]["width"] == 16
    assert sorted(p.name for p in (tmp_path / "sub").iterdir()) == ["tune.json"]


def test_free_spins_follow_the_run_median_rule():
    """_free_spins (vectorised) against the reference's loop (unit_world.cc:1367-1386):
    each run of consecutive free spins contributes its middle spin, a run still
    open at the last spin contributes nothing; without only_median every free
    spin is kept."""
    from puzzletunneldiscovery_gb300 import sampling as S
    rng = np.random.default_rng(3)

    def loop(qs, valid):
        out = []
        for p in range(valid.shape[0]):
            picks, run = [], []
            for i in range(valid.shape[1]):
                if valid[p, i]:
                    run.append(i)
                elif run:
                    picks.append(run[len(run) // 2])
                    run = []
            out.append(qs[p][picks] if picks else np.zeros((0, 7)))
        return out

    for _ in range(200):
        P, D = int(rng.integers(1, 20)), int(rng.integers(1, 40))
        valid = rng.random((P, D)) < rng.random()
        qs = rng.random((P, D, 7))
        t = torch.from_numpy(qs)
        assert all(np.array_equal(x, y) for x, y in zip(loop(qs, valid), S._free_spins(t, valid, True)))
        assert all(np.array_equal(qs[p][valid[p]], r) for p, r in enumerate(S._free_spins(t, valid, False)))


def test_apply_rows_matches_apply_batch():
    from puzzletunneldiscovery_gb300 import sampling as S
    rng = np.random.default_rng(4)
    q = np.array([0.1, 0.2, 0.3, 0.9, 0.1, 0.2, 0.3])
    tr, aa = rng.normal(size=(10, 3)), rng.normal(size=(10, 3))
    aa[0] = 0.0
    assert np.array_equal(S.apply_batch(q, tr, aa), S.apply_rows(np.repeat(q[None], 10, 0), tr, aa))
