"""Full-size workloads checked through properties that do not need the oracle to
run the whole batch: invariance under permutation and re-batching, the
meaning of a first-contact step (the state there collides, the one before is
free), and oracle agreement on random samples drawn from the full batch."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _world(meshes):
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = meshes
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw


@pytest.fixture(scope="module")
def tori():
    return W.cfg_interlocking_tori()


def test_segments_full_size_properties(built_lib, oracle_mod, tori):
    """1M segments (the headline workload): permutation invariance, chunked
    calls, first-contact semantics, and the oracle on a 300-segment sample."""
    uw = _world(tori)
    q0, q1 = W.segment_batch(1_000_000, -2.0, 2.0, uw.scene_scale, seed=0)
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    f = uw.first_contact_steps(a, b, 0.001)
    assert not uw.last_stats()["device_errors"]
    perm = torch.randperm(a.shape[0], generator=torch.Generator().manual_seed(1)).cuda()
    fp = uw.first_contact_steps(a[perm], b[perm], 0.001)
    assert torch.equal(fp, f[perm])
    parts = [uw.first_contact_steps(a[i:i + 333_333], b[i:i + 333_333], 0.001) for i in range(0, a.shape[0], 333_333)]
    assert torch.equal(torch.cat(parts), f)
    fc = f.cpu().numpy()
    assert set(np.unique(fc)) <= set(range(-2, 4097))
    assert 0.2 < (fc == -1).mean() < 0.8
    # the transit tuple of every colliding segment: the contact state collides, the last free one is free
    idx = torch.nonzero(f >= 0).flatten()[:200_000]
    lf, st, done, lt, tt = uw.transit_states_to_with_contact(a[idx], b[idx], 0.001)
    assert not done.any()
    assert not uw.is_valid_states(st).any()
    # the step before the first contact is free; at step 0 the "last free" state is the
    # segment's start, which the reference loop never checks (unit_world.cc:445-470)
    later = f[idx] >= 1
    assert later.any() and uw.is_valid_states(lf[later]).all()
    assert torch.equal(lf[~later], a[idx][~later])
    assert (lt < tt).all()
    # free segments: every step free, including the last
    jdx = torch.nonzero(f == -1).flatten()[:200_000]
    lf2, st2, done2, _, _ = uw.transit_states_to_with_contact(a[jdx], b[jdx], 0.001)
    assert done2.all() and uw.is_valid_states(st2).all()
    # the oracle on a sample of the full batch
    ow = oracle_mod.OracleWorld(*tori)
    rng = np.random.default_rng(7)
    sample = rng.choice(len(q0), 300, replace=False)
    e, _ = ow.segments_first_contact(q0[sample], q1[sample], 0.001)
    assert (fc[sample] == e).all()


def test_states_full_size_properties(built_lib, oracle_mod):
    """20M states on the plate / knot meshes (the scale-up workload): permutation
    invariance, chunked calls, the allocation-free entry point on a slice, and
    the oracle on a 20k sample."""
    Ve, Fe, Vr, Fr = W.cfg_plate_knot()
    uw = _world((Ve, Fe, Vr, Fr))
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    q = torch.from_numpy(W.uniform_states(20_000_000, lo, hi, uw.scene_scale, seed=0)).cuda()
    v = uw.is_valid_states(q)
    perm = torch.randperm(q.shape[0], generator=torch.Generator().manual_seed(2)).cuda()
    assert torch.equal(uw.is_valid_states(q[perm]), v[perm])
    parts = [uw.is_valid_states(q[i:i + 7_000_001]) for i in range(0, q.shape[0], 7_000_001)]
    assert torch.equal(torch.cat(parts), v)
    frac = float(v.float().mean())
    assert 0.0 < frac < 0.5
    ow = oracle_mod.OracleWorld(Ve, Fe, Vr, Fr)
    rng = np.random.default_rng(3)
    sample = torch.from_numpy(rng.choice(q.shape[0], 20_000, replace=False)).cuda()
    qs = q[sample].cpu().numpy()
    assert (v[sample].cpu().numpy() == ow.is_valid(qs)).all()
