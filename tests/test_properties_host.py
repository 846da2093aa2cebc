"""Property-based checks on the CPU (hypothesis): the oracle's triangle
predicate is symmetric and invariant under cyclic vertex order on generic
pairs, state decompositions round-trip, and the screening partition tiles the
task range for any sizes."""
import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
from hypothesis import given, settings  # noqa: E402

coord = st.floats(min_value=-1.0, max_value=1.0, allow_nan=False, allow_infinity=False, width=64)
tri = st.lists(st.lists(coord, min_size=3, max_size=3), min_size=3, max_size=3)


def _generic(V):
    V = np.asarray(V)
    return np.linalg.norm(np.cross(V[1] - V[0], V[2] - V[0])) > 1e-3


def _clear(V, U):
    """No vertex of one triangle within 1e-6 of the other's plane: exact contacts
    (shared vertices, edges on the other's plane) are where Moller's test, the
    reference's included, depends on vertex order."""
    for A, B in ((V, U), (U, V)):
        A, B = np.asarray(A), np.asarray(B)
        n = np.cross(A[1] - A[0], A[2] - A[0])
        n /= np.linalg.norm(n)
        if (np.abs((B - A[0]) @ n) < 1e-6).any():
            return False
    return True


def _jitter(V, U):
    """A deterministic 1e-4 jitter of both triangles: hypothesis favours round
    coordinates, whose exact touches (an edge meeting an edge, not only a vertex
    on a plane) have measure zero once the pair is moved off them."""
    flat = tuple(float(x) for t in (V, U) for p in t for x in p)
    rng = np.random.default_rng(abs(hash(flat)) % (2 ** 32))
    return (np.asarray(V) + rng.uniform(-1e-4, 1e-4, (3, 3)), np.asarray(U) + rng.uniform(-1e-4, 1e-4, (3, 3)))


@settings(max_examples=300, deadline=None)
@given(tri, tri)
def test_tri_tri_symmetric_and_cyclic(oracle_mod, V, U):
    V, U = _jitter(V, U)
    if not (_generic(V) and _generic(U) and _clear(V, U)):
        return
    V, U = [np.array(v) for v in V], [np.array(u) for u in U]
    a = oracle_mod.tri_tri(V, U)
    assert oracle_mod.tri_tri(U, V) is a
    assert oracle_mod.tri_tri(V[1:] + V[:1], U) is a
    assert oracle_mod.tri_tri(V, U[2:] + U[:2]) is a


quat = st.lists(st.floats(min_value=-1.0, max_value=1.0, allow_nan=False, width=64), min_size=4, max_size=4)


@settings(max_examples=200, deadline=None)
@given(st.lists(coord, min_size=3, max_size=3), quat)
def test_state_round_trips(built_lib, t, r):
    from puzzletunneldiscovery_gb300 import state_ops as S
    r = np.array(r)
    if np.linalg.norm(r) < 1e-3:
        return
    q = np.concatenate([t, r / np.linalg.norm(r)])
    tt, angle, axis = S.decompose_3(q)
    back = S.compose_from_angleaxis(tt, angle, axis)
    assert np.allclose(back[:3], q[:3])
    assert min(np.abs(back[3:] - q[3:]).max(), np.abs(back[3:] + q[3:]).max()) < 1e-9
    tr, aav, se3 = S.differential(q, q)
    assert np.allclose(tr, 0) and np.linalg.norm(aav) < 1e-6


@settings(max_examples=200, deadline=None)
@given(st.integers(min_value=3, max_value=400), st.integers(min_value=1, max_value=512),
       st.integers(min_value=1, max_value=5000))
def test_partition_tiles_the_task_range(nkey_total, quota, gran):
    from puzzletunneldiscovery_gb300 import screening as S
    nkey = nkey_total - S.RESERVED
    ntask = nkey * (nkey + 1) // 2
    total = S.partition_screening(nkey_total, quota, gran)
    assert 1 <= total <= max(1, quota)
    try:
        b = S.chunk_bounds(ntask, total)
    except ValueError:
        # the reference's own partitioner asserts on the same sizes
        return
    assert b[0, 0] == 0 and b[-1, 1] == ntask and (b[1:, 0] == b[:-1, 1]).all()
    seen = 0
    for i in range(total):
        f, t = S.partition_screening(nkey_total, quota, gran, index=i)
        assert (f >= t).all() and (t >= S.RESERVED).all() and (f < nkey_total).all()
        seen += f.shape[0]
    assert seen == ntask
