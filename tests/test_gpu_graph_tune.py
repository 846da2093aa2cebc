"""Graph mode, CUDA-graph replay and the launch autotuner: none of them may
change a verdict or a first-contact step."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _world():
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw


def test_segment_graph_replay_matches_direct_call(built_lib):
    from puzzletunneldiscovery_gb300.autotune import SegmentGraph
    uw = _world()
    q0, q1 = W.segment_batch(20000, -2.0, 2.0, uw.scene_scale, seed=41)
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    want = uw.first_contact_steps(a, b, 0.001).clone()
    g = SegmentGraph(uw, a, b, 0.001)
    for _ in range(3):
        got = g.replay()
        torch.cuda.synchronize()
        assert torch.equal(got, want)
    assert g.errors() == 0
    # graph mode is off again: ordinary calls still size their own scratch, and a
    # call that grows (moves) it makes the next replay capture again
    q0b, q1b = W.segment_batch(60000, -2.0, 2.0, uw.scene_scale, seed=42)
    e0 = uw.scratch_epoch()
    uw.first_contact_steps(torch.from_numpy(q0b).cuda(), torch.from_numpy(q1b).cuda(), 0.001)
    assert uw.scratch_epoch() != e0
    got = g.replay()
    torch.cuda.synchronize()
    assert g.captures == 2
    assert torch.equal(got, want)


def test_graph_mode_over_capacity_reports_invalid(built_lib):
    """Reserved scratch too small for the batch: the device checks mark the
    segments PW_STEP_INVALID and raise the world's error count (no write past
    the reservation)."""
    uw = _world()
    q0, q1 = W.segment_batch(512, -2.0, 2.0, uw.scene_scale, seed=43)
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    uw.segments_reserve(512, 8, 64)
    uw.set_graph_mode(True)
    try:
        out = uw.first_contact_steps(a, b, 0.001).cpu().numpy()
        stats = uw.last_stats()
    finally:
        uw.set_graph_mode(False)
    assert stats["device_errors"] != 0
    assert (out == -3).sum() > 0
    ok = uw.first_contact_steps(a, b, 0.001).cpu().numpy()
    assert (ok != -3).all()
    # the segments that fit gave the ordinary answer
    fit = out != -3
    assert (out[fit] == ok[fit]).all()


def test_graph_mode_needs_reserved_scratch(built_lib):
    from puzzletunneldiscovery_gb300 import _lib
    uw = _world()
    q0, q1 = W.segment_batch(64, -2.0, 2.0, uw.scene_scale, seed=44)
    uw.set_graph_mode(True)
    try:
        with pytest.raises(_lib.PwError) as e:
            uw.first_contact_steps(torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda(), 0.001)
        assert e.value.code == _lib.PW_ERR_CAPACITY
    finally:
        uw.set_graph_mode(False)


def test_autotune_keeps_verdicts(built_lib, oracle_mod):
    from puzzletunneldiscovery_gb300.autotune import autotune
    uw = _world()
    q = torch.from_numpy(W.uniform_states(200000, -2.0, 2.0, uw.scene_scale, seed=45)).cuda()
    q0, q1 = W.segment_batch(10000, -2.0, 2.0, uw.scene_scale, seed=46)
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    before_v = uw.is_valid_states(q).clone()
    before_s = uw.first_contact_steps(a, b, 0.001).clone()
    rep = autotune(uw, states=q, segments=(a, b), verify_delta=0.001, soft_caps=(128, 0), blocks=(0, 2), reps=1)
    # the launch grid plus the two node-box kinds, timed first
    assert len(rep["states"].table) == 3 * 2 * 2 + 2 and len(rep["segments"].table) == 2 * 2 + 2
    assert rep["segments"].best["boxes"] == uw.get_node_boxes(1)
    assert rep["states"].best["boxes"] == uw.get_node_boxes(0)
    assert torch.equal(uw.is_valid_states(q), before_v)
    assert torch.equal(uw.first_contact_steps(a, b, 0.001), before_s)
    cfg = uw.get_launch_config(0)
    assert cfg["width"] in (8, 16, 32) and cfg["blocks"] >= 1
    # the oracle agrees on a sample under the tuned configuration
    ow = oracle_mod.OracleWorld(*W.cfg_interlocking_tori())
    qs = q[:5000].cpu().numpy()
    assert (uw.is_valid_states(torch.from_numpy(qs).cuda()).cpu().numpy() == ow.is_valid(qs)).all()


def test_autotune_cache_reapplies_a_tuned_configuration(built_lib, tmp_path):
    """A configuration tuned for a mesh pair on this GPU is stored; a second world
    with the same meshes gets it from the cache without timing anything, and a
    different mesh pair misses the cache."""
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300.autotune import TuneCache, autotune
    path = str(tmp_path / "tune.json")
    uw = _world()
    q = torch.from_numpy(W.uniform_states(100000, -2.0, 2.0, uw.scene_scale, seed=47)).cuda()
    first = autotune(uw, states=q, cache=path, soft_caps=(128, 0), blocks=(0, 2), reps=1)["states"]
    assert len(first.table) == 3 * 2 * 2 + 2
    applied = uw.get_launch_config(0)
    second_world = _world()
    again = autotune(second_world, states=q, cache=path, soft_caps=(128, 0), blocks=(0, 2), reps=1)["states"]
    assert again.table == [] and again.best == first.best
    assert second_world.get_launch_config(0) == applied
    assert second_world.get_node_boxes(0) == first.best["boxes"]
    assert torch.equal(second_world.is_valid_states(q), uw.is_valid_states(q))
    Ve, Fe, Vr, Fr = W.interlocking_tori(1.0, 0.25, 48, 24)
    other = pw.UnitWorld(0)
    other.load_env_mesh(Ve, Fe)
    other.load_robot_mesh(Vr, Fr)
    other.scaleToUnit()
    other.angleModel(0.0, 0.0)
    miss = autotune(other, states=q, cache=TuneCache(path), soft_caps=(0,), blocks=(0,), reps=1)["states"]
    assert len(miss.table) == 3 + 2
    assert len(TuneCache(path).load()) == 2
