"""Host logic of the batched samplers (puzzletunneldiscovery_gb300/sampling.py),
on the CPU with a stand-in world whose verdicts are scripted."""
import math

import numpy as np
import torch

from conftest import ROOT  # noqa: F401


class ScriptedWorld:
    """Answers is_valid_states from a fixed pattern, in call order."""

    def __init__(self, pattern):
        self.pattern = np.asarray(pattern, bool).ravel()
        self._device = torch.device("cpu")
        self.calls = []

    def is_valid_states(self, q):
        self.calls.append(q.shape[0])
        assert q.shape[0] == self.pattern.shape[0]
        return torch.from_numpy(self.pattern.copy())


def _S():
    from puzzletunneldiscovery_gb300 import sampling
    return sampling


def test_quat_between_and_rotate():
    S = _S()
    rng = np.random.default_rng(0)
    a = rng.normal(size=(100, 3))
    b = rng.normal(size=(100, 3))
    b[0] = -a[0]                     # opposite directions
    b[1] = 2.0 * a[1]                # same direction
    q = S.quat_between(a, b)
    assert np.allclose(np.linalg.norm(q, axis=1), 1.0)
    ra = S.quat_rotate(q, a / np.linalg.norm(a, axis=1, keepdims=True))
    assert np.allclose(ra, b / np.linalg.norm(b, axis=1, keepdims=True), atol=1e-12)


def test_touch_states_place_points_with_opposed_normals():
    S = _S()
    rng = np.random.default_rng(1)
    P, A = 5, 7
    rp, ep = rng.normal(size=(P, 3)), rng.normal(size=(P, 3))
    rn = rng.normal(size=(P, 3))
    en = rng.normal(size=(P, 3))
    rn /= np.linalg.norm(rn, axis=1, keepdims=True)
    en /= np.linalg.norm(en, axis=1, keepdims=True)
    ang = rng.uniform(0, 2 * math.pi, (P, A))
    qs = S._touch_states(rp, rn, ep, en, 0.01, ang)
    for p in range(P):
        for i in range(A):
            q = qs[p, i]
            rob_o = rp[p] + 0.01 * rn[p]
            placed = S.quat_rotate(q[3:], rob_o) + q[:3]
            assert np.allclose(placed, ep[p] + 0.01 * en[p], atol=1e-12)
            assert np.allclose(S.quat_rotate(q[3:], rn[p]), -en[p], atol=1e-12)


def test_enum_free_configuration_median_runs():
    S = _S()
    # runs of free spins: [1..3] -> 2, [5] -> 5, trailing [8, 9] is not reported (reference quirk)
    pattern = np.array([0, 1, 1, 1, 0, 1, 0, 0, 1, 1], bool)
    uw = ScriptedWorld(pattern)
    z = np.zeros(3)
    n = np.array([0.0, 0.0, 1.0])
    all_free = S.enum_free_configuration(uw, z, n, z, n, 0.0, 10, only_median=False)
    assert all_free.shape == (6, 7)
    med = S.enum_free_configuration(uw, z, n, z, n, 0.0, 10, only_median=True)
    qs = S._touch_states(z, n, z, n, 0.0, (np.arange(10) * (2 * math.pi / 10))[None, :])[0]
    assert np.array_equal(med, qs[[2, 5]])


def test_sample_free_configuration_first_free_or_last_tried():
    S = _S()
    pattern = np.array([[0, 0, 1, 1], [0, 0, 0, 0]], bool)
    uw = ScriptedWorld(pattern)
    pts = np.zeros((2, 3))
    nrm = np.tile([0.0, 1.0, 0.0], (2, 1))
    rng = np.random.default_rng(3)
    q, found = S.sample_free_configurations(uw, pts, nrm, pts, nrm, 0.0, max_trials=3, rng=rng)
    assert list(found) == [True, False]
    rng = np.random.default_rng(3)
    ang = rng.uniform(0.0, 2 * math.pi, (2, 4))
    qs = S._touch_states(pts, nrm, pts, nrm, 0.0, ang)
    assert np.array_equal(q[0], qs[0, 2]) and np.array_equal(q[1], qs[1, 3])


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
        assert all(np.array_equal(x, y) for x, y in zip(loop(qs, valid), S._free_spins(qs, valid, True)))
        assert all(np.array_equal(qs[p][valid[p]], r) for p, r in enumerate(S._free_spins(qs, valid, False)))


def test_apply_rows_matches_apply_batch():
    from puzzletunneldiscovery_gb300 import sampling as S
    rng = np.random.default_rng(4)
    q = np.array([0.1, 0.2, 0.3, 0.9, 0.1, 0.2, 0.3])
    tr, aa = rng.normal(size=(10, 3)), rng.normal(size=(10, 3))
    aa[0] = 0.0
    assert np.array_equal(S.apply_batch(q, tr, aa), S.apply_rows(np.repeat(q[None], 10, 0), tr, aa))
