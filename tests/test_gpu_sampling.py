"""Batched samplers on the GPU against the oracle: the transit tuple of every
segment of a batch, touch sampling (touchq_util.calc_touch) and key
configurations (enumFreeConfiguration / sampleFreeConfiguration)."""
import math

import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tori(oracle_mod, built_lib):
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    uw = pw.UnitWorld()
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)


def _same_tuple(got, want):
    lf, st, done, lt, tt = got
    assert (lf == want[0]).all() and (st == want[1]).all()
    assert done == want[2] and lt == want[3] and tt == want[4]


def test_batched_transit_tuples_match_oracle(tori):
    uw, ow = tori
    q0, q1 = W.segment_batch(300, -2.0, 2.0, uw.scene_scale, seed=31)
    q1[:5] = q0[:5]                       # zero-length: delta >= dist
    q1[5:10] = q0[5:10] + 1e-5            # shorter than one step
    lf, st, done, lt, tt = uw.transit_states_to_with_contact(torch.from_numpy(q0), torch.from_numpy(q1), 0.001)
    lf, st, done, lt, tt = (x.cpu().numpy() for x in (lf, st, done, lt, tt))
    for i in range(300):
        want, _, _ = ow.transit_state_to_with_contact(q0[i], q1[i], 0.001)
        _same_tuple((lf[i], st[i], bool(done[i]), lt[i], tt[i]), want)


def test_calc_touch_matches_oracle(tori):
    from puzzletunneldiscovery_gb300 import sampling as S
    uw, ow = tori
    q0 = np.array([0.0, 0.0, 0.5, 1.0, 0.0, 0.0, 0.0])   # free: the robot ring above the env ring
    assert uw.is_valid_state(q0)
    rng = np.random.default_rng(7)
    lf, st, done, lt, tt = S.calc_touch(uw, q0, 256, 0.01, rng)
    rng = np.random.default_rng(7)
    to = S.apply_batch(q0, S.random_on_sphere(256, 1.0, rng), S.random_within_sphere(256, 2 * math.pi, rng))
    assert done.sum() < 256 and done.sum() > 0
    for i in range(256):
        want, _, _ = ow.transit_state_to_with_contact(q0, to[i], 0.01)
        _same_tuple((lf[i], st[i], bool(done[i]), lt[i], tt[i]), want)


def test_enum_free_configuration_verdicts_match_oracle(tori):
    from puzzletunneldiscovery_gb300 import sampling as S
    uw, ow = tori
    rng = np.random.default_rng(11)
    P, D = 40, 64
    Venv = ow.vertices(0)
    Vrob = ow.vertices(1)
    ep = Venv[rng.integers(0, Venv.shape[0], P)]
    rp = Vrob[rng.integers(0, Vrob.shape[0], P)]
    en = rng.normal(size=(P, 3))
    rn = rng.normal(size=(P, 3))
    en /= np.linalg.norm(en, axis=1, keepdims=True)
    rn /= np.linalg.norm(rn, axis=1, keepdims=True)
    got = S.enum_free_configurations(uw, rp, rn, ep, en, 1e-3, D)
    qs = S._touch_states(rp, rn, ep, en, 1e-3, np.broadcast_to(np.arange(D) * (2 * math.pi / D), (P, D)))
    valid = ow.is_valid(qs.reshape(-1, 7)).reshape(P, D)
    assert 0 < valid.sum() < P * D
    for p in range(P):
        assert np.array_equal(got[p], qs[p][valid[p]])
    q, found = S.sample_free_configurations(uw, rp, rn, ep, en, 1e-3, max_trials=15, rng=np.random.default_rng(2))
    assert ow.is_valid(q[found]).all()


def test_checkpointed_transit_tuples_equal_full_loop(tori):
    """pw_world_segments_contact_states (from the set-up kernel's checkpoints) and
    pw_segments_contact_states (the delta loop from step 0) give identical tuples."""
    from puzzletunneldiscovery_gb300 import _lib
    uw, _ = tori
    q0, q1 = W.segment_batch(20000, -2.0, 2.0, uw.scene_scale, seed=33)
    q1[:10] = q0[:10]
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    fast = uw.transit_states_to_with_contact(a, b, 0.001)      # checkpoint path (same batch as its query)
    steps = uw.first_contact_steps(a, b, 0.001)
    L = _lib.load()
    n = a.shape[0]
    outs = [torch.empty((n, 7), dtype=torch.float64, device="cuda"), torch.empty((n, 7), dtype=torch.float64,
                                                                                device="cuda"),
            torch.empty(n, dtype=torch.uint8, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"),
            torch.empty(n, dtype=torch.float32, device="cuda")]
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(L.pw_segments_contact_states(a.data_ptr(), b.data_ptr(), steps.data_ptr(), n, 0.001,
                                            *[o.data_ptr() for o in outs], err.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream), "contact states")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    for x, y in zip(fast, outs):
        assert torch.equal(x.to(y.dtype), y)
