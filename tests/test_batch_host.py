"""Host logic of the batch autotuner (no GPU): the clustering level that
keys its cache, the cache key, and the option bits of each tuned schedule."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_clustering_level_buckets():
    from jerald_gb300.batch import clustering_level
    n, L = 16, 32.0
    g = (np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * (L / n)
    lattice = torch.from_numpy(g.astype(np.float32))
    assert clustering_level(lattice, n, L) == 0
    # 5 % of the particles piled into one cell
    k = len(g) // 20
    some = lattice.clone()
    some[:k] = torch.tensor([3.1, 3.1, 3.1])
    assert clustering_level(some, n, L) == 1
    # every particle in one of ten cells
    dense = lattice.clone()
    dense[:] = torch.from_numpy(((np.arange(len(g)) % 10)[:, None] * 2.0 + 0.5).astype(np.float32))
    assert clustering_level(dense, n, L) == 2
    # the periodic wrap: x = L lands in cell 0, as in the paint
    edge = lattice.clone()
    edge[:, 0] = L
    assert clustering_level(edge, n, L) == 2  # n^2 cells of n particles each


def test_cache_key_separates_clustering_levels():
    from jerald_gb300.batch import _key
    assert _key(64, 1000, "sm", 2, 0) != _key(64, 1000, "sm", 2, 2)
    assert _key((64, 64, 64), 1000, "sm", 2) == _key(np.array([64, 64, 64]), 1000, "sm", 2, 0)


def test_schedule_option_bits():
    """FusedLDL.options of each tuned schedule, as include/jld.h documents
    them (bits 4, 5-6, 7-8), computed without a device."""
    from jerald_gb300.ldl import FusedLDL
    f = FusedLDL.__new__(FusedLDL)
    f.paint_method, f.pipelined, f.recompute = "atomic", True, False
    f.x_radix, f.min_cols, f.bin_tile = 8, 0, 16
    assert f.options == 0
    f.x_radix = 16
    assert f.options == 16
    f.x_radix, f.min_cols = 8, 8
    assert f.options == 2 << 5
    f.min_cols, f.paint_method, f.bin_tile = 0, "tiled", 20
    assert f.options == 4 | (2 << 7)
