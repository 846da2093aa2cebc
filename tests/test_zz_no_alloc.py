"""pw_states_valid_noalloc: the state query for callers that may not allocate.

Some users cannot let a library call cudaMalloc once they are running -- a
planner embedded in a framework whose pool allocator owns the whole device
heap, or a tight loop that cannot take cudaMalloc's implicit device
synchronisation.  pw_states_valid_noalloc answers the same question as
pw_states_valid but keeps its scratch in a fixed array inside the library.
This test calls it through the C ABI twice in a row (the second call reuses
the array the first one left behind) and requires verdicts identical to the
allocating entry point.  It builds its own world, so it passes alone in a
fresh process as well as after the other tests; the file name makes pytest
collect it last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _world():
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import workloads as W
    Ve, Fe, Vr, Fr = W.cfg_interlocking_tori()
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw


def test_noalloc_matches_allocating_entry_point(built_lib):
    from puzzletunneldiscovery_gb300 import _lib
    from puzzletunneldiscovery_gb300 import workloads as W
    uw = _world()
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    # enough near-contact states that the FP64 re-test queue in the fixed array is used
    q = torch.from_numpy(W.uniform_states(200_000, -2.0, 2.0, uw.scene_scale, seed=21)).to(dev)
    expected = uw.is_valid_states(q).cpu().numpy()
    assert uw.last_stats()["retests"] > 0
    for call in range(2):
        out = torch.full((q.shape[0],), 7, dtype=torch.uint8, device=dev)
        rc = L.pw_states_valid_noalloc(uw._h, q.data_ptr(), q.shape[0], out.data_ptr(), stream)
        _lib.check(rc, "pw_states_valid_noalloc (call %d)" % call)
        got = out.cpu().numpy()
        assert set(np.unique(got)) <= {0, 1}
        assert (got.astype(bool) == expected).all(), "call %d: %d mismatches" % (call, int((got != expected).sum()))


def test_noalloc_rejects_oversized_batches(built_lib):
    from puzzletunneldiscovery_gb300 import _lib
    uw = _world()
    L = _lib.load()
    dev = torch.device("cuda", 0)
    q = torch.zeros((1, 7), dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.uint8, device=dev)
    # the size is checked before anything is launched, so the small buffers are never read
    rc = L.pw_states_valid_noalloc(uw._h, q.data_ptr(), (1 << 20) + 1, out.data_ptr(),
                                   torch.cuda.current_stream(dev).cuda_stream)
    assert rc == _lib.PW_ERR_INVALID_ARG
    assert b"1048576" in L.pw_last_error()
