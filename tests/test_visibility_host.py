"""Host logic of the visibility matrix: the flat-index decoding of the strict
lower triangle that the device uses to generate the (i, j) pairs of
calculate_visibility_matrix (unit_world.cc:740-759) without host arrays."""
import numpy as np
import torch

from puzzletunneldiscovery_gb300.unit_world import _strict_tril_pairs


def test_strict_triangle_decoding_is_numpy_order():
    for n in (1, 2, 3, 7, 64, 1000):
        k = torch.arange(n * (n - 1) // 2, dtype=torch.int64)
        r, c = _strict_tril_pairs(k)
        R, C = np.tril_indices(n, -1)
        assert (r.numpy() == R).all() and (c.numpy() == C).all()


def test_strict_triangle_decoding_at_large_indices():
    """Near perfect squares and at the end of the triangle of 2^20 and 3e6 keys,
    where the float square root is closest to an integer boundary."""
    for n in (1 << 20, 3_000_000):
        tot = n * (n - 1) // 2
        rows = np.array([2, 3, 1000, n // 2, n - 2, n - 1], dtype=np.int64)
        ks = np.concatenate([rows * (rows - 1) // 2 + d for d in (-1, 0, 1)] + [np.array([0, tot - 1])])
        ks = torch.from_numpy(ks[(ks >= 0) & (ks < tot)])
        r, c = _strict_tril_pairs(ks)
        assert ((c >= 0) & (c < r) & (r < n)).all()
        assert (r * (r - 1) // 2 + c == ks).all()
