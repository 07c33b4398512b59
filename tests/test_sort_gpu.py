"""Sort by cell key and the sorted paint, through the C ABI.

jld_cell_sort_f32 must give numpy.argsort(keys, kind="stable") bit for bit
(keys from the oracle's prelude and key restatement, lib/parops_fast.h:91-93)
on: uniform and lattice-ordered clustered particles, every particle in one
cell, the x mod L -> L edge, sizes that are not a multiple of the sort's
4096-pair tiles, one particle.  The sorted paint must match the oracle's
serial paint (the reference's lpaint, pinned in test_ref_pin.py) within 1e-5
of the mesh scale, and its dense cells (runs carried over a warp's rounds,
summed in FP64) the FP64 paint of the same float32 mesh positions within
1e-6 relative.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import cic  # noqa: E402


@pytest.fixture(scope="module")
def jl():
    from jerald_gb300 import _lib, build
    build.build()
    return _lib


def _st():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ct.c_void_p(t.data_ptr())


def _sort(jl, pos, nm, box):
    n = len(pos)
    b = np.asarray(box, dtype=np.float32)
    dpos = torch.from_numpy(pos).cuda()
    keys = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    order = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    ws = torch.empty(max(int(jl.load().jld_cell_sort_workspace(n)), 1), dtype=torch.uint8, device="cuda")
    jl.call("jld_cell_sort_f32", _st(), _p(dpos), n, *nm, b.ctypes.data_as(ct.c_void_p), _p(keys), _p(order),
            _p(ws), ws.numel())
    torch.cuda.synchronize()
    return keys[:n].cpu().numpy(), order[:n].cpu().numpy(), dpos, keys, order


def _expected(pos, nm, box):
    keys = cic.cell_keys(cic.box_to_mesh(pos, np.asarray(box, dtype=np.float32), nm), nm)
    order = np.argsort(keys, kind="stable")
    return keys[order].astype(np.int32), order.astype(np.int32)


def _uniform(n, box, seed):
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * np.asarray(box)).astype(np.float32)
    pos[:3] = [[-1e-10, 5e-9, -3e-12], [box[0], box[1], box[2]], [0.0, 0.0, 0.0]]
    return pos


def _clustered(n_side, box, seed):
    from jerald_gb300 import synth
    return np.ascontiguousarray(synth.clustered(n_side, box, seed=seed))


CASES = [
    ("uniform_64", lambda: _uniform(262144 + 77, (100.0, 100.0, 100.0), 1), (64, 64, 64), (100.0, 100.0, 100.0)),
    ("uniform_noncubic", lambda: _uniform(50001, (200.0, 30.0, 7.5), 2), (20, 12, 8), (200.0, 30.0, 7.5)),
    ("clustered_64", lambda: _clustered(64, 100.0, 3), (64, 64, 64), (100.0, 100.0, 100.0)),
    ("clustered_256", lambda: _clustered(256, 400.0, 4), (256, 256, 256), (400.0, 400.0, 400.0)),
    ("one_cell", lambda: (np.random.default_rng(5).random((100000, 3)) * 0.9 + 10.05).astype(np.float32),
     (32, 32, 32), (32.0, 32.0, 32.0)),
    ("one_particle", lambda: np.asarray([[1.5, 2.5, 3.5]], dtype=np.float32), (8, 8, 8), (8.0, 8.0, 8.0)),
]


@pytest.mark.parametrize("name,make,nm,box", CASES, ids=[c[0] for c in CASES])
def test_cell_sort_is_numpy_stable_argsort(jl, name, make, nm, box):
    pos = make()
    keys, order, *_ = _sort(jl, pos, nm, box)
    ek, eo = _expected(pos, nm, box)
    np.testing.assert_array_equal(keys, ek)
    np.testing.assert_array_equal(order, eo)


@pytest.mark.parametrize("name,make,nm,box", CASES, ids=[c[0] for c in CASES])
def test_sorted_paint_matches_oracle(jl, name, make, nm, box):
    pos = make()
    n = len(pos)
    rng = np.random.default_rng(9)
    mass = (rng.random(n) + 0.5).astype(np.float32)
    b = np.asarray(box, dtype=np.float32)
    q = cic.box_to_mesh(pos, b, nm)
    cic.set_threads(1)
    ref = cic.paint(q, mass, nm)
    dmass = torch.from_numpy(mass).cuda()
    out = torch.empty(nm, dtype=torch.float32, device="cuda")
    ws = torch.empty(int(jl.load().jld_ppaint_box_sorted_workspace(n)), dtype=torch.uint8, device="cuda")
    dpos = torch.from_numpy(pos).cuda()
    jl.call("jld_ppaint_box_sorted_f32", _st(), _p(dpos), n, _p(dmass), ct.c_float(0.0), *nm,
            b.ctypes.data_as(ct.c_void_p), _p(out), _p(ws), ws.numel())
    got = out.cpu().numpy()
    scale = max(1.0, float(np.abs(ref).max()))
    assert np.abs(got - ref).max() <= 1e-5 * scale
    # the paint-only entry point on a kept sort: the same mesh up to the
    # order in which runs of one cell meet in the mesh's atomics
    _, _, dpos2, keys, order = _sort(jl, pos, nm, box)
    out2 = torch.empty_like(out)
    jl.call("jld_ppaint_sorted_f32", _st(), _p(dpos2), n, _p(dmass), ct.c_float(0.0), *nm,
            b.ctypes.data_as(ct.c_void_p), _p(keys), _p(order), _p(out2))
    torch.cuda.synchronize()
    assert np.abs(out2.cpu().numpy() - got).max() <= 1e-6 * scale


def test_sorted_paint_dense_cells_are_fp64_sums(jl):
    """Forty cells of 4000 particles each on a clustered lattice: the cells
    they paint against the FP64 paint of the same float32 mesh positions,
    within 1e-6 relative."""
    nm, box = (64, 64, 64), (100.0, 100.0, 100.0)
    base = _clustered(64, 100.0, 6)
    rng = np.random.default_rng(7)
    cells = rng.integers(0, 64, (40, 3)) * (100.0 / 64)
    dense = (cells[:, None, :] + rng.random((40, 4000, 3)) * (100.0 / 64) * 0.98 + 0.01).reshape(-1, 3)
    pos = np.ascontiguousarray(np.concatenate([base, dense.astype(np.float32)]))
    n = len(pos)
    b = np.asarray(box, dtype=np.float32)
    q = cic.box_to_mesh(pos, b, nm)
    f64 = cic.paint(q.astype(np.float64), 1.0, nm)
    out = torch.empty(nm, dtype=torch.float32, device="cuda")
    ws = torch.empty(int(jl.load().jld_ppaint_box_sorted_workspace(n)), dtype=torch.uint8, device="cuda")
    jl.call("jld_ppaint_box_sorted_f32", _st(), _p(torch.from_numpy(pos).cuda()), n, None, ct.c_float(1.0), *nm,
            b.ctypes.data_as(ct.c_void_p), _p(out), _p(ws), ws.numel())
    got = out.cpu().numpy().astype(np.float64)
    dense_cells = f64 > 200.0   # the corner cells of the 4000-particle cells
    assert dense_cells.sum() >= 40
    rel = np.abs(got - f64)[dense_cells] / f64[dense_cells]
    assert rel.max() < 1e-6, rel.max()
    assert np.abs(got - f64).max() <= 1e-5 * f64.max()
