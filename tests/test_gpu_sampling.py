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
    (lf, st, done, lt, tt), to = S.calc_touch_batch(uw, q0[None], 256, 0.01, np.random.default_rng(7))
    to = to.cpu().numpy()
    assert done.sum() < 256 and done.sum() > 0
    for i in range(256):
        want, _, _ = ow.transit_state_to_with_contact(q0, to[i], 0.01)
        _same_tuple((lf[i], st[i], bool(done[i]), lt[i], tt[i]), want)
    # the same rng state gives the same segments; calc_touch is calc_touch_batch of one key
    again = S.calc_touch(uw, q0, 256, 0.01, np.random.default_rng(7))
    assert all(np.array_equal(x, y) for x, y in zip(again, (lf, st, done, lt, tt)))


def test_touch_targets_follow_apply(tori):
    """pw_touch_targets: unit translations, rotations of angle <= 2 pi applied on the
    left (osr::apply), unit quaternions; from rows repeat their key."""
    from puzzletunneldiscovery_gb300 import sampling as S
    uw, _ = tori
    keys = W.uniform_states(50, -1.0, 1.0, uw.scene_scale, seed=5)
    frm, to = S.touch_segments(uw, keys, 400, 99)
    frm, to = frm.cpu().numpy(), to.cpu().numpy()
    assert np.array_equal(frm, np.repeat(keys, 400, axis=0))
    d = to[:, :3] - frm[:, :3]
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    assert abs(d.mean(axis=0)).max() < 0.05
    assert np.allclose(np.linalg.norm(to[:, 3:], axis=1), 1.0, atol=1e-15)
    # the left rotation r = to_rot * from_rot^-1 has angle 2 acos|w| uniform-in-ball distributed
    fr, tr = frm[:, 3:], to[:, 3:]
    w = np.abs(np.sum(tr * fr * np.array([1, 1, 1, 1]), axis=1))       # |<to, from>| = |cos(angle / 2)|
    ang = 2 * np.arccos(np.clip(w, 0, 1))
    assert ang.max() <= math.pi + 1e-6 and np.median(ang) > 1.0
    f2, t2 = S.touch_segments(uw, keys, 400, 99)
    assert np.array_equal(t2.cpu().numpy(), to)


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
    en[0] = rn[0]                          # the half-turn branch of the shortest arc
    got = S.enum_free_configurations(uw, rp, rn, ep, en, 1e-3, D)
    half = [0.5 * (i * (2 * math.pi / D)) for i in range(D)]
    hc, hs = [math.cos(h) for h in half], [math.sin(h) for h in half]
    qs = oracle_mod_keyconf(ow)(rp, rn, ep, en, 1e-3, hc, hs)
    # the device's states are the oracle's, bit for bit
    assert np.array_equal(S.keyconf_states(uw, rp, rn, ep, en, 1e-3, hc, hs).cpu().numpy(), qs)
    valid = ow.is_valid(qs.reshape(-1, 7)).reshape(P, D)
    assert 0 < valid.sum() < P * D
    for p in range(P):
        assert np.array_equal(got[p], qs[p][valid[p]])
    med = S.enum_free_configurations(uw, rp, rn, ep, en, 1e-3, D, only_median=True)
    from oracle import oracle as O
    assert all(np.array_equal(x, y) for x, y in zip(med, O.free_spins(qs, valid, True)))
    q, found = S.sample_free_configurations(uw, rp, rn, ep, en, 1e-3, max_trials=15, rng=np.random.default_rng(2))
    assert ow.is_valid(q[found]).all()
    # the random spins of sampleFreeConfiguration: first free spin, or the last one tried
    rng = np.random.default_rng(2)
    h = 0.5 * rng.uniform(0.0, 2 * math.pi, (P, 16))
    qs2 = O.keyconf_states(rp, rn, ep, en, 1e-3, np.cos(h), np.sin(h))
    v2 = ow.is_valid(qs2.reshape(-1, 7)).reshape(P, 16)
    first = np.where(v2.any(axis=1), np.argmax(v2, axis=1), 15)
    assert np.array_equal(q, qs2[np.arange(P), first]) and np.array_equal(found, v2.any(axis=1))


def oracle_mod_keyconf(ow):
    from oracle import oracle as O
    return O.keyconf_states


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
