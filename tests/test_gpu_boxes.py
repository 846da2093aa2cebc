"""Both kinds of BVH node box (pw_world_set_node_boxes): axis-aligned boxes in
each mesh's frame and oriented boxes along the principal axes of each node's
vertices (FCL's OBBRSS nodes, lib/osr/cdmodel.cc:17-18, are oriented boxes too).
The verdicts and first-contact steps must equal the oracle's under either kind
(unit_world.cc:215-247, 405-474); only the number of box and triangle tests
may differ."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _world(meshes):
    import puzzletunneldiscovery_gb300 as pw
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(meshes[0], meshes[1])
    uw.load_robot_mesh(meshes[2], meshes[3])
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw


@pytest.fixture(scope="module")
def tori(oracle_mod, built_lib):
    m = W.cfg_interlocking_tori()
    return _world(m), oracle_mod.OracleWorld(*m)


@pytest.fixture(scope="module")
def plate(oracle_mod, built_lib):
    m = W.cfg_plate_knot()
    return _world(m), oracle_mod.OracleWorld(*m), m[0]


def test_default_is_oriented(tori):
    uw, _ = tori
    assert uw.get_node_boxes(0) == "oriented" and uw.get_node_boxes(1) == "oriented"


@pytest.mark.parametrize("kind", ["aligned", "oriented"])
def test_tori_states_and_segments_match_oracle(tori, kind):
    uw, ow = tori
    uw.set_node_boxes(kind)
    try:
        q = W.uniform_states(60_000, -2.0, 2.0, ow.scene_scale, seed=41)
        got = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
        want = ow.is_valid(q)
        assert (got == want).all(), int((got != want).sum())
        q0, q1 = W.segment_batch(1500, -2.0, 2.0, ow.scene_scale, seed=42)
        f = uw.first_contact_steps(torch.from_numpy(q0), torch.from_numpy(q1), 0.001).cpu().numpy()
        e, _ = ow.segments_first_contact(q0, q1, 0.001)
        assert (f == e).all(), int((f != e).sum())
    finally:
        uw.set_node_boxes("oriented")


@pytest.mark.parametrize("kind", ["aligned", "oriented"])
def test_plate_states_match_oracle(plate, kind):
    uw, ow, Ve = plate
    uw.set_node_boxes(kind)
    try:
        lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
        q = W.uniform_states(20_000, lo, hi, ow.scene_scale, seed=43)
        got = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
        assert (got == ow.is_valid(q)).all()
    finally:
        uw.set_node_boxes("oriented")


def test_oriented_boxes_cut_the_tests(tori):
    """The same batch under both kinds: identical verdicts, and the oriented
    boxes' tighter fit leaves fewer box and triangle tests.  (Colliding states
    take about the same leaf tests under both kinds: a warp tests up to 32
    frontier pairs per round before its first certified contact ends the
    query.)"""
    uw, ow = tori
    q = torch.from_numpy(W.uniform_states(200_000, -2.0, 2.0, ow.scene_scale, seed=44)).cuda()
    out, stats = {}, {}
    for kind in ("aligned", "oriented"):
        uw.set_node_boxes(kind)
        out[kind] = uw.is_valid_states(q)
        stats[kind] = uw.last_stats()
    uw.set_node_boxes("oriented")
    assert torch.equal(out["aligned"], out["oriented"])
    assert stats["oriented"]["leaf_tests"] < 0.8 * stats["aligned"]["leaf_tests"], stats
    assert stats["oriented"]["node_tests"] < stats["aligned"]["node_tests"], stats


def test_node_boxes_refused_in_graph_mode(tori):
    from puzzletunneldiscovery_gb300 import _lib
    uw, _ = tori
    uw.set_graph_mode(True)
    try:
        with pytest.raises(_lib.PwError):
            uw.set_node_boxes("aligned")
    finally:
        uw.set_graph_mode(False)
    assert uw.get_node_boxes(0) == "oriented"


def test_node_boxes_per_kernel(tori):
    """Each kernel keeps its own kind: states aligned while segments stay oriented."""
    uw, ow = tori
    uw.set_node_boxes("aligned", 0)
    try:
        assert uw.get_node_boxes(0) == "aligned" and uw.get_node_boxes(1) == "oriented"
        q = W.uniform_states(5000, -2.0, 2.0, ow.scene_scale, seed=45)
        assert (uw.is_valid_states(torch.from_numpy(q)).cpu().numpy() == ow.is_valid(q)).all()
        q0, q1 = W.segment_batch(300, -2.0, 2.0, ow.scene_scale, seed=46)
        e, _ = ow.segments_first_contact(q0, q1, 0.001)
        assert (uw.first_contact_steps(torch.from_numpy(q0), torch.from_numpy(q1), 0.001).cpu().numpy() == e).all()
    finally:
        uw.set_node_boxes("oriented")
