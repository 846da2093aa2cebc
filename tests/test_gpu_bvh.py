"""The two BVH hierarchies (pw_world_set_bvh): top-down principal-axis splits
(the default) and Karras's Morton LBVH give the oracle's verdicts, first-contact
steps and contact rows (unit_world.cc:215-247, 405-474, 959-1012) with either
node-box kind."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _world(meshes, bvh):
    import puzzletunneldiscovery_gb300 as pw
    uw = pw.UnitWorld()
    uw.load_env_mesh(meshes[0], meshes[1])
    uw.load_robot_mesh(meshes[2], meshes[3])
    uw.scaleToUnit()
    uw.set_bvh(bvh)
    uw.angleModel(0.0, 0.0)
    assert uw.get_bvh() == bvh
    return uw


@pytest.fixture(scope="module")
def tori(oracle_mod, built_lib):
    m = W.cfg_interlocking_tori()
    return m, oracle_mod.OracleWorld(*m)


@pytest.mark.parametrize("bvh", ["topdown", "sah", "morton"])
@pytest.mark.parametrize("boxes", ["oriented", "aligned"])
def test_hierarchies_match_oracle(tori, bvh, boxes):
    m, ow = tori
    uw = _world(m, bvh)
    uw.set_node_boxes(boxes)
    s = ow.scene_scale
    q = W.uniform_states(20000, -1.0, 1.0, s, seed=3)
    assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()
    q0, q1 = W.segment_batch(800, -2.0, 2.0, s, seed=4)
    got = uw.first_contact_steps(torch.from_numpy(q0), torch.from_numpy(q1), 0.001).cpu().numpy()
    want, _ = ow.segments_first_contact(q0, q1, 0.001)
    assert (got == want).all()
    hit = q[~ow.is_valid(q)][:20]
    for x in hit:
        b, e, mg, p = uw.intersecting_segments(x)
        b2, e2, mg2, p2, _ = ow.intersecting_segments(x)
        assert (p == p2).all() and (b == b2).all() and (e == e2).all()
    assert 0 < uw.info()["env_bvh_depth"] < 64


def test_topdown_depth_is_bounded_on_the_plate(oracle_mod, built_lib):
    m = W.cfg_plate_knot(n=200)
    uw = _world(m, "topdown")
    d = uw.info()["env_bvh_depth"]
    assert 10 < d <= 60, d
    ow = oracle_mod.OracleWorld(*m)
    Ve = ow.Ve
    q = W.uniform_states(20000, Ve.min(0) - 0.5, Ve.max(0) + 0.5, ow.scene_scale, seed=9)
    assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()


def test_pick_bvh_keeps_the_fastest_and_the_verdicts(tori):
    from puzzletunneldiscovery_gb300.autotune import pick_bvh
    m, ow = tori
    uw = _world(m, "topdown")
    q = torch.from_numpy(W.uniform_states(200_000, -1.0, 1.0, ow.scene_scale, seed=12)).cuda()
    want = uw.is_valid_states(q).cpu().numpy()
    r = pick_bvh(uw, states=q)
    assert r["bvh"] in ("topdown", "morton") and uw.get_bvh() == r["bvh"]
    assert set(r["ms"]) == {"topdown", "morton"} and all(set(v) == {"aligned", "oriented"} for v in r["ms"].values())
    best = min(t for v in r["ms"].values() for t in v.values())
    assert r["ms"][r["bvh"]][r["boxes"]["states"]] == best
    assert (uw.is_valid_states(q).cpu().numpy() == want).all()
