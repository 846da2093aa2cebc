"""pw_states_valid_noalloc: the state query for callers that may not allocate.

Some users cannot let a library call cudaMalloc once they are running -- a
planner embedded in a framework whose pool allocator owns the whole device
heap, or a tight loop that cannot take cudaMalloc's implicit device
synchronisation.  pw_states_valid_noalloc answers the same question as
pw_states_valid but keeps its scratch in a fixed array inside the library.
These tests call it through the C ABI twice in a row (the second call reuses
the array the first one left behind) and require verdicts identical to the
allocating entry point, also when more pairs need the FP64 re-test than the
fixed queue holds, and that a warm call takes no device memory.  They build
their own worlds, so they pass alone in a fresh process as well as after the
other tests; the file name makes pytest collect them last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _world(meshes=None):
    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import workloads as W
    Ve, Fe, Vr, Fr = meshes if meshes is not None else W.cfg_interlocking_tori()
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


def _flat_grid(n):
    """A flat square plate in z = 0 over [-1, 1]^2, n x n cells, two triangles each."""
    x = np.linspace(-1.0, 1.0, n + 1, dtype=np.float32)
    X, Y = np.meshgrid(x, x, indexing="ij")
    V = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size, np.float32)], axis=1)
    F = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            F += [[a, b, c], [a, c, d]]
    return V, np.asarray(F, dtype=np.uint32)


def _call(L, uw, q, stream):
    from puzzletunneldiscovery_gb300 import _lib
    out = torch.full((q.shape[0],), 7, dtype=torch.uint8, device=q.device)
    _lib.check(L.pw_states_valid_noalloc(uw._h, q.data_ptr(), q.shape[0], out.data_ptr(), stream),
               "pw_states_valid_noalloc")
    return out


def test_noalloc_overflowing_retest_queue_and_no_allocation(built_lib):
    """Two coplanar plates: every overlapping triangle pair lies in the FP32
    band, so a few hundred states queue more FP64 re-tests than the fixed
    array's 1048576 entries and the rest are re-tested inline."""
    from puzzletunneldiscovery_gb300 import _lib
    V, F = _flat_grid(16)
    uw = _world((V, F, V, F))
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(5)
    n = 600
    a = rng.uniform(-np.pi, np.pi, n)
    q = np.zeros((n, 7))
    q[:, :2] = rng.uniform(-0.1, 0.1, (n, 2))       # unit frame: the plates overlap in z = 0
    q[:, 3] = np.cos(a / 2)
    q[:, 6] = np.sin(a / 2)                         # rotations about z keep the robot in the plane
    q[::10, 2] = 0.5                                # every tenth state lifted clear of the plate
    q = torch.from_numpy(q).to(dev)
    expected = uw.is_valid_states(q).cpu().numpy()
    st = uw.last_stats()
    assert st["retests"] + st["inline_retests"] > (1 << 20), st
    assert not expected[1::10].any() and expected[::10].all()
    for call in range(2):
        got = _call(L, uw, q, stream).cpu().numpy()
        assert (got.astype(bool) == expected).all(), "call %d: %d mismatches" % (call, int((got != expected).sum()))
    # a warm call takes no device memory (cudaMalloc hands out at least 2 MiB)
    out = torch.empty(q.shape[0], dtype=torch.uint8, device=dev)
    torch.cuda.synchronize(dev)
    free0, _ = torch.cuda.mem_get_info(dev)
    _lib.check(L.pw_states_valid_noalloc(uw._h, q.data_ptr(), q.shape[0], out.data_ptr(), stream),
               "pw_states_valid_noalloc")
    torch.cuda.synchronize(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free0 - free1 < (2 << 20), (free0, free1)
    assert (out.cpu().numpy().astype(bool) == expected).all()
