"""More uncertain triangle pairs than the FP64 re-test queue holds.

Two coplanar plates: every overlapping triangle pair lies inside the FP32
band, so each state (or segment step) queues thousands of FP64 re-tests.
When the queue (4,194,304 entries per call) is full, the slots that lost a pair
are answered again by a second traversal with inline FP64 re-tests.  Verdicts
and first-contact steps must equal the oracle's (unit_world.cc:215-247,
405-474) either way."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


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


@pytest.fixture(scope="module")
def plates(oracle_mod):
    import puzzletunneldiscovery_gb300 as pw
    V, F = _flat_grid(16)
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(V, F)
    uw.load_robot_mesh(V, F)
    uw.scaleToUnit()
    uw.angleModel(0.0, 0.0)
    return uw, oracle_mod.OracleWorld(V, F, V, F)


def _in_plane(rng, n, spread=0.1):
    """Unit states in the plate's plane: translation in x, y and a rotation about z
    (quaternion (cos a/2, 0, 0, sin a/2)), which keep every robot vertex at z = 0."""
    a = rng.uniform(-np.pi, np.pi, n)
    q = np.zeros((n, 7))
    q[:, :2] = rng.uniform(-spread, spread, (n, 2))
    q[:, 3] = np.cos(a / 2)
    q[:, 6] = np.sin(a / 2)
    return q


def test_states_past_the_queue_match_oracle(built_lib, plates):
    uw, ow = plates
    q = _in_plane(np.random.default_rng(11), 2000)
    q[::7, 2] = 0.5                                   # lifted clear of the plate
    got = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
    st = uw.last_stats()
    assert st["retests"] >= (1 << 22) and st["inline_retests"] > 0, st
    want = ow.is_valid(q)
    assert (got == want).all(), int((got != want).sum())
    assert want[::7].all() and not np.delete(want, np.s_[::7]).any()


def test_segments_past_the_queue_match_oracle(built_lib, plates):
    uw, ow = plates
    rng = np.random.default_rng(12)
    a = _in_plane(rng, 96)
    b = _in_plane(rng, 96)
    b[:, :2] = a[:, :2] + rng.uniform(-0.05, 0.05, (96, 2))
    b[:, 3:] = a[:, 3:]                               # translation only: up to about 70 steps each
    a[::8, 2] = b[::8, 2] = 0.5                       # a few segments clear of the plate
    delta = 0.001
    got = uw.first_contact_steps(torch.from_numpy(a), torch.from_numpy(b), delta).cpu().numpy()
    st = uw.last_stats()
    assert st["retests"] >= (1 << 22) and st["inline_retests"] > 0, st
    want, _ = ow.segments_first_contact(a, b, delta)
    assert (got == want).all(), (got[got != want][:8], want[got != want][:8])
    rest = np.delete(want, np.s_[::8])
    assert (want[::8] == -1).all() and np.isin(rest, [0, -2]).all() and (rest == 0).sum() > 80
