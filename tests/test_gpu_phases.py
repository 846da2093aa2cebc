"""Round phases of segment queries (pw_world_set_segment_phases): the
first-contact codes of a large batch are the same in one phase and in eight
(the anchor frames of chunks behind a known contact are skipped in phases), and
equal the oracle's (unit_world.cc:405-474, 480-488) on a sample."""
import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tori(oracle_mod, built_lib):
    import puzzletunneldiscovery_gb300 as pw
    m = W.cfg_interlocking_tori()
    uw = pw.UnitWorld()
    uw.load_env_mesh(m[0], m[1])
    uw.load_robot_mesh(m[2], m[3])
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, oracle_mod.OracleWorld(*m)


def _codes(uw, a, b, mode, phases):
    uw.set_segment_phases(phases)
    try:
        return uw.first_contact_steps(a, b, 0.001, mode).cpu().numpy()
    finally:
        uw.set_segment_phases("auto")


@pytest.mark.parametrize("mode", [0, 1])
def test_phases_give_the_same_codes(tori, mode):
    uw, ow = tori
    assert uw.get_segment_phases() == "auto"
    s = uw.info()["scene_scale"]
    # about 6.7M 32-step chunks: "auto" runs this batch in phases
    q0, q1 = W.segment_batch(120_000, -2.0, 2.0, s, seed=21 + mode)
    a, b = torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda()
    auto = uw.first_contact_steps(a, b, 0.001, mode).cpu().numpy()
    off = _codes(uw, a, b, mode, "off")
    on = _codes(uw, a, b, mode, "on")
    assert (auto == off).all() and (on == off).all()
    assert (off >= 0).sum() > 10_000 and (off == -1).sum() > 10_000
    want, _ = ow.segments_first_contact(q0[:1500], q1[:1500], 0.001, mode=mode)
    assert (off[:1500] == want).all()
    # a small batch forced into phases
    on_small = _codes(uw, a[:3000], b[:3000], mode, "on")
    assert (on_small == off[:3000]).all()


def test_phase_mode_is_checked(tori):
    uw, _ = tori
    with pytest.raises(KeyError):
        uw.set_segment_phases("sometimes")
    assert uw.get_segment_phases() == "auto"
