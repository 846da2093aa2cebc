"""Host-side fault injection on the device path: bad meshes, queries before the
models exist, oversize batches, bad step sizes and non-finite states each end
in an error status (or, for a non-finite state, a "not free" verdict plus a
device_errors bit), and the world answers the next good query correctly.
Nothing here faults or stalls the GPU: every failure is made on the host or
is an input the kernels check."""
import ctypes

import numpy as np
import pytest
import torch

from puzzletunneldiscovery_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NONFINITE = 8   # PW_DEVERR_NONFINITE


@pytest.fixture(scope="module")
def tori():
    return W.interlocking_tori(1.0, 0.25, 24, 12)


def _ready(meshes):
    import puzzletunneldiscovery_gb300 as pw
    Ve, Fe, Vr, Fr = meshes
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw


def _code(exc):
    return getattr(exc.value, "code", None)


def test_bad_meshes_are_refused_and_the_world_stays_usable(built_lib, tori, oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import _lib
    Ve, Fe, Vr, Fr = tori
    uw = pw.UnitWorld(0)
    with pytest.raises(Exception) as e:                       # query before any model
        uw.is_valid_states(torch.zeros((4, 7), dtype=torch.float64, device="cuda"))
    assert _code(e) == _lib.PW_ERR_NO_MODEL
    bad_face = Fe.copy()
    bad_face[3, 1] = Ve.shape[0]                              # index one past the last vertex
    with pytest.raises(Exception) as e:
        uw.load_env_mesh(Ve, bad_face)
    assert _code(e) == _lib.PW_ERR_INVALID_ARG and b"face index" in uw._L.pw_last_error()
    nan_vertex = Vr.copy()
    nan_vertex[5, 2] = np.nan
    with pytest.raises(Exception) as e:
        uw.load_robot_mesh(nan_vertex, Fr)
    assert _code(e) == _lib.PW_ERR_INVALID_ARG and b"non-finite" in uw._L.pw_last_error()
    inf_vertex = Ve.copy()
    inf_vertex[0, 0] = np.inf
    with pytest.raises(Exception):
        uw.load_env_mesh(inf_vertex, Fe)
    rc = uw._L.pw_world_load_env(uw._h, None, -1, None, 0)
    assert rc == _lib.PW_ERR_INVALID_ARG
    # the refused loads left nothing behind: the good meshes load and answer like the oracle
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    q = W.uniform_states(2000, -2.0, 2.0, uw.scene_scale, seed=11)
    v = uw.is_valid_states(torch.from_numpy(q).cuda()).cpu().numpy()
    assert (v == oracle_mod.OracleWorld(*tori).is_valid(q)).all()


def test_oversize_batches_and_bad_step_sizes_are_refused(built_lib, tori):
    from puzzletunneldiscovery_gb300 import _lib
    uw = _ready(tori)
    q = torch.zeros((8, 7), dtype=torch.float64, device="cuda")
    q[:, 3] = 1.0
    out = torch.empty(8, dtype=torch.uint8, device="cuda")
    first = torch.empty(8, dtype=torch.int32, device="cuda")
    L, h = uw._L, uw._h
    # sizes are checked before any pointer is followed
    assert L.pw_states_valid(h, q.data_ptr(), 1 << 32, out.data_ptr(), None) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_states_valid(h, q.data_ptr(), -1, out.data_ptr(), None) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_states_valid_noalloc(h, q.data_ptr(), 1 << 32, out.data_ptr(), None) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_segments_first_contact(h, q.data_ptr(), q.data_ptr(), 1 << 31, 0.01, 0, first.data_ptr(),
                                       None) == _lib.PW_ERR_INVALID_ARG
    for delta in (0.0, -1.0, float("nan"), float("inf")):
        assert L.pw_segments_first_contact(h, q.data_ptr(), q.data_ptr(), 8, delta, 0, first.data_ptr(),
                                           None) == _lib.PW_ERR_INVALID_ARG, delta
    assert L.pw_segments_first_contact(h, q.data_ptr(), q.data_ptr(), 8, 0.01, 7, first.data_ptr(),
                                       None) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_world_set_launch_config(h, 0, 33, 0, 0) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_world_set_launch_config(h, 2, 32, 0, 0) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_last_error()
    # and the world still answers
    assert uw.is_valid_states(q).shape == (8,)
    assert not uw.last_stats()["device_errors"]


def test_non_finite_states_are_not_free(built_lib, tori, oracle_mod):
    """A NaN or infinite component makes the state's verdict 0 and sets the
    NONFINITE bit; the finite states of the same batch keep their verdicts."""
    uw = _ready(tori)
    q = W.uniform_states(5000, -2.0, 2.0, uw.scene_scale, seed=12)
    want = oracle_mod.OracleWorld(*tori).is_valid(q)
    assert want.any()
    bad = np.zeros(len(q), bool)
    rng = np.random.default_rng(4)
    for j, val in zip(rng.choice(len(q), 64, replace=False), [np.nan, np.inf, -np.inf, np.nan] * 16):
        q[j, rng.integers(0, 7)] = val
        bad[j] = True
    v = uw.is_valid_states(torch.from_numpy(q).cuda()).cpu().numpy()
    assert uw.last_stats()["device_errors"] & NONFINITE
    assert not v[bad].any()
    assert (v[~bad] == want[~bad]).all()
    v2 = uw.is_valid_states(torch.from_numpy(q[~bad]).cuda())
    assert uw.last_stats()["device_errors"] == 0
    assert (v2.cpu().numpy() == want[~bad]).all()
    # isDisentangled on the same batch: the non-finite states take the general FP64 box test
    d = uw.is_disentangled_states(torch.from_numpy(q).cuda()).cpu().numpy()
    assert (d == oracle_mod.OracleWorld(*tori).is_disentangled(q)).all()


def test_non_finite_segments_take_no_step(built_lib, tori, oracle_mod):
    """A segment with a NaN endpoint has a NaN distance: the reference loop
    (delta <= dist) checks no step, so it reports PW_STEP_NONE, flagged as
    NONFINITE; the other segments of the batch are unaffected."""
    from puzzletunneldiscovery_gb300 import _lib
    uw = _ready(tori)
    q0, q1 = W.segment_batch(400, -2.0, 2.0, uw.scene_scale, seed=13)
    want, _ = oracle_mod.OracleWorld(*tori).segments_first_contact(q0, q1, 0.01)
    q1[::37, 4] = np.nan
    f = uw.first_contact_steps(torch.from_numpy(q0).cuda(), torch.from_numpy(q1).cuda(), 0.01).cpu().numpy()
    assert uw.last_stats()["device_errors"] & NONFINITE
    bad = np.zeros(len(q0), bool)
    bad[::37] = True
    assert (f[bad] == _lib.PW_STEP_NONE).all()
    assert (f[~bad] == want[~bad]).all()


def test_network_refuses_bad_training_calls(built_lib):
    from puzzletunneldiscovery_gb300 import _lib
    from puzzletunneldiscovery_gb300.surrogate import Surrogate
    net = Surrogate(0, 1)
    L, h = net._L, net._h
    q = torch.zeros((4, 7), dtype=torch.float64, device="cuda")
    y = torch.zeros(4, dtype=torch.uint8, device="cuda")
    assert L.pw_mlp_train_step(h, q.data_ptr(), y.data_ptr(), 0, ctypes.c_float(1e-3), None, None) != _lib.PW_OK
    assert L.pw_mlp_set_adam(h, None, None, -1) == _lib.PW_ERR_INVALID_ARG
    assert L.pw_mlp_predict(h, None, 4, None, None) == _lib.PW_ERR_INVALID_ARG
    # a refused call changes nothing: the step count is still 0 and training works
    assert net.adam_state()["step"] == 0
    net.train_step(q, y, 1e-3)
    assert net.adam_state()["step"] == 1
