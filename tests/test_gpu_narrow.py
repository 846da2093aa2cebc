"""Narrow-passage search on the plate / torus-knot meshes: the crossing filter
on constructed cases, and a small search whose escapes are all exactly free
(re-checked by the oracle)."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_crossing_filter_constructed_cases(built_lib):
    from puzzletunneldiscovery_gb300 import narrow as N
    dev = torch.device("cuda", 0)
    probes = torch.tensor([[0.0, 0.0, 0.0]], dtype=torch.float64, device=dev)
    root = torch.tensor([[0.1, 0.2, 0.1, 1, 0, 0, 0]], dtype=torch.float64, device=dev)
    ends = torch.tensor([[0.1, 0.2, -0.1, 1, 0, 0, 0],      # crosses inside
                         [0.9, 0.2, -0.1, 1, 0, 0, 0],      # crosses at x = 0.5: outside extent 0.4
                         [0.1, 0.2, 0.05, 1, 0, 0, 0],      # stays above
                         [0.1, 0.2, 0.1, 0, 1, 0, 0]],      # rotation only: the probe at the origin stays
                        dtype=torch.float64, device=dev)
    roots = root.expand(1, 7).contiguous()
    got = N.crossings(roots, ends, 4, probes, 0.0, 0.4).cpu().numpy().tolist()
    assert got == [True, False, False, False]
    # a probe off the origin: a half turn about x carries it through the plane
    probes = torch.tensor([[0.0, 0.0, 0.15]], dtype=torch.float64, device=dev)
    ends = torch.tensor([[0.1, 0.2, 0.1, 0, 1, 0, 0]], dtype=torch.float64, device=dev)
    assert N.crossings(roots, ends, 1, probes, 0.0, 0.4).cpu().numpy().tolist() == [True]


def test_small_search_escapes_are_free(built_lib, oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import narrow as N
    from puzzletunneldiscovery_gb300.surrogate import Surrogate
    Ve, Fe, Vr, Fr = W.cfg_plate_knot(n=120)
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    s = uw.scene_scale
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    roots = N.draw_free_roots(uw, 20000, lo, hi, gen)
    assert uw.is_valid_states(roots).all()
    probes = N.centre_line_probes(uw, 256, 16, every=8)
    extent = float(np.abs(Ve[:, :2]).max()) * s
    net = Surrogate(0, 9)
    search = N.NarrowPassageSearch(uw, net, probes, 0.0, extent, k=4096, retrain_labels=8192, seed=1)
    rep = search.run(roots, guided=True, roots_per_round=5000, keep_escapes=True)
    assert rep.crossing > 0 and rep.validated > 0
    assert rep.retrains >= 1
    plain = N.NarrowPassageSearch(uw, None, probes, 0.0, extent, k=4096, seed=1)
    prep = plain.run(roots, guided=False, roots_per_round=5000)
    assert prep.validated > 0
    ow = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    checked = 0
    for frm, to in rep.escape_states:
        f, t = frm.cpu().numpy(), to.cpu().numpy()
        for i in range(min(len(f), 40)):
            (lf, st, done, _, _), _, _ = ow.transit_state_to_with_contact(f[i], t[i], min(0.001, 0.5 * pw.distance(f[i], t[i])))
            assert done
            checked += 1
    assert rep.escapes == 0 or checked > 0


def _mix64(z):
    M = (1 << 64) - 1
    z = (z + 0x9E3779B97F4A7C15) & M
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def _expand_ref(root, i, per_root, st, sr, seed):
    """A restatement of pw_expand_states for one candidate (FP32 noise, FP64 product)."""
    f32 = np.float32
    base = _mix64(seed ^ _mix64(i))
    g = []
    for k in (1, 2, 3):
        bits = _mix64((base + k) & ((1 << 64) - 1))
        u1 = (f32(bits >> 40) + f32(0.5)) * f32(1.0 / 16777216.0)
        u2 = (f32((bits >> 16) & 0xFFFFFF) + f32(0.5)) * f32(1.0 / 16777216.0)
        r = np.sqrt(f32(-2.0) * np.log(u1))
        g += [r * np.cos(f32(2.0) * np.pi * u2), r * np.sin(f32(2.0) * np.pi * u2)]
    g = np.asarray(g, dtype=np.float64)
    t = [root[c] + st * g[c] for c in range(3)]
    rv = sr * g[3:6]
    ang = np.linalg.norm(rv)
    w1, v1 = (np.cos(ang / 2), rv * np.sin(ang / 2) / ang) if ang > 0 else (1.0, np.zeros(3))
    q = np.asarray(root[3:], dtype=np.float64)
    q = q / np.linalg.norm(q)
    w2, v2 = q[0], q[1:]
    w = w1 * w2 - np.dot(v1, v2)
    v = w1 * v2 + w2 * v1 + np.cross(v1, v2)
    r4 = np.concatenate([[w], v])
    return np.concatenate([t, r4 / np.linalg.norm(r4)])


def test_expansion_kernel(built_lib):
    """pw_expand_states: deterministic per seed, matches a restatement of its
    generator and rotation, and has the requested spreads."""
    from puzzletunneldiscovery_gb300 import narrow as N
    from puzzletunneldiscovery_gb300 import workloads as W
    roots = torch.from_numpy(W.uniform_states(2000, -1.0, 1.0, 0.3, seed=8)).cuda()
    a = N.expand(roots, 64, 0.02, 0.1, 77)
    b = N.expand(roots, 64, 0.02, 0.1, 77)
    c = N.expand(roots, 64, 0.02, 0.1, 78)
    assert torch.equal(a, b) and not torch.equal(a, c)
    A = a.cpu().numpy()
    R = roots.cpu().numpy()
    for i in (0, 1, 63, 64, 5000, 127999):
        # FP32 noise and rotation: agreement to FP32 rounding
        np.testing.assert_allclose(A[i], _expand_ref(R[i // 64], i, 64, 0.02, 0.1, 77), rtol=0, atol=2e-6)
    d = A[:, :3] - np.repeat(R[:, :3], 64, axis=0)
    assert abs(d.std() - 0.02) < 0.001 and abs(d.mean()) < 0.001
    assert np.allclose(np.linalg.norm(A[:, 3:], axis=1), 1.0, atol=1e-6)
    qr = np.repeat(R[:, 3:] / np.linalg.norm(R[:, 3:], axis=1, keepdims=True), 64, axis=0)
    ang = 2 * np.arccos(np.clip(np.abs(np.sum(A[:, 3:] * qr, axis=1)), 0, 1))
    # |rotation vector| of a 3-D N(0, 0.1^2 I) draw: mean 0.1 * sqrt(8 / pi)
    assert abs(ang.mean() - 0.1 * np.sqrt(8 / np.pi)) < 0.005


def test_search_checkpoint_resumes_the_same_rounds(built_lib):
    """A narrow-passage search checkpointed between rounds (seeded counters,
    generator state, pending labels, network) and restored into a new search
    with a differently seeded network draws the same next rounds: same
    candidates, crossings and escapes.  Retraining is off during the compared
    rounds, so the network's scores are the restored ones."""
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import narrow as N
    from puzzletunneldiscovery_gb300.surrogate import Surrogate
    Ve, Fe, Vr, Fr = W.cfg_plate_knot(n=120)
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    s = uw.scene_scale
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    roots = N.draw_free_roots(uw, 10000, lo, hi, gen)
    probes = N.centre_line_probes(uw, 256, 16, every=8)
    extent = float(np.abs(Ve[:, :2]).max()) * s
    kw = dict(k=2048, retrain_labels=10**9)
    first = N.NarrowPassageSearch(uw, Surrogate(0, 3), probes, 0.0, extent, seed=7, **kw)
    assert first.pretrain(roots, 20000, roots_per_round=5000, batch=1024) >= 1
    first.run(roots[:5000], guided=True, roots_per_round=5000)
    sd = first.state_dict()
    assert sd["calls"] == first.calls and sd["net"]["step"] >= 1
    second = N.NarrowPassageSearch(uw, Surrogate(0, 4), probes, 0.0, extent, seed=0, **kw)
    second.load_state_dict(sd)
    for guided in (True, False):
        r1 = first.run(roots, guided=guided, roots_per_round=5000)
        r2 = second.run(roots, guided=guided, roots_per_round=5000)
        assert (r1.candidates, r1.crossing, r1.validated, r1.escapes) == (r2.candidates, r2.crossing, r2.validated,
                                                                          r2.escapes)
    assert first.calls == second.calls and first._nlab == second._nlab
