"""GPU parity of the drop-in primitives against the oracle (C ABI calls).

Bars: cell keys and readouts bit-exact (same operation order, no FMA);
paints within 1e-5 of the mesh scale in float32 (atomic summation order
differs), 1e-12 in float64; FFTs within float rounding of numpy's DFT.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import cic  # noqa: E402
from oracle.fft import pfft as o_pfft, pifft as o_pifft  # noqa: E402


@pytest.fixture(scope="module")
def jl():
    from jerald_gb300 import _lib, build
    build.build()
    return _lib


def _st():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ct.c_void_p(t.data_ptr())


_LIVE = []


@pytest.fixture(autouse=True)
def _release_inputs():
    yield
    torch.cuda.synchronize()
    _LIVE.clear()


def _cuda(a):
    # Device copies stay referenced until the test ends: a raw pointer handed
    # to the C ABI does not keep the tensor (and its allocator block) alive.
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    _LIVE.append(t)
    return t


def _box(box, dt):
    return np.ascontiguousarray(np.asarray(box, dtype=dt))


def _positions(n, nm, box, seed, dt, extra_edge=True):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-0.5, 1.5, (n, 3)) * np.asarray(box)
    if extra_edge:
        # exact grid points, exact box edges, tiny negatives that round to L
        pos[:4] = [[0.0, 0.0, 0.0], [box[0], box[1], box[2]], [-1e-10, 5e-9, -3e-12],
                   [box[0] / nm[0] * 3, box[1] / 2, -box[2]]]
    return pos.astype(dt)


CASES = [((16, 16, 16), (100.0, 100.0, 100.0)), ((20, 12, 8), (200.0, 30.0, 7.5)),
         ((64, 64, 64), (100.0, 100.0, 100.0))]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nm,box", CASES)
def test_cell_keys_bit_exact(jl, dt, nm, box):
    sfx = "f32" if dt == np.float32 else "f64"
    pos = _positions(5000, nm, box, 1, dt)
    ref = cic.cell_keys(cic.box_to_mesh(pos, box, nm), nm)
    keys = torch.empty(len(pos), dtype=torch.int32, device="cuda")
    b = _box(box, dt)
    jl.call(f"jld_cell_keys_{sfx}", _st(), _p(_cuda(pos)), len(pos), *nm, b.ctypes.data_as(ct.c_void_p),
            _p(keys))
    np.testing.assert_array_equal(keys.cpu().numpy(), ref)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nm,box", CASES)
@pytest.mark.parametrize("vjpdim", [-1, 0, 1, 2])
def test_readout_bit_exact(jl, dt, nm, box, vjpdim):
    sfx = "f32" if dt == np.float32 else "f64"
    pos = _positions(4000, nm, box, 2, dt)
    field = np.random.default_rng(3).standard_normal(nm).astype(dt)
    ref = cic.readout(cic.box_to_mesh(pos, box, nm), field, nm, box, vjpdim)
    out = torch.empty(len(pos), dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    b = _box(box, dt)
    jl.call(f"jld_preadout_box_{sfx}", _st(), _p(_cuda(pos)), len(pos), _p(_cuda(field)), *nm,
            b.ctypes.data_as(ct.c_void_p), vjpdim, _p(out))
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    # mesh-unit entry point on the oracle's mesh coordinates gives the same bits
    pm = cic.box_to_mesh(pos, box, nm)
    out2 = torch.empty_like(out)
    jl.call(f"jld_preadout_{sfx}", _st(), _p(_cuda(pm)), len(pos), _p(_cuda(field)), *nm,
            b.ctypes.data_as(ct.c_void_p), vjpdim, _p(out2))
    np.testing.assert_array_equal(out2.cpu().numpy(), ref)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("vjp", [0, 1])
def test_readout3d_bit_exact(jl, dt, vjp):
    nm, box = (16, 24, 32), (50.0, 60.0, 70.0)
    sfx = "f32" if dt == np.float32 else "f64"
    pos = _positions(3000, nm, box, 4, dt)
    shape = nm if vjp else (3,) + nm
    field = np.random.default_rng(5).standard_normal(shape).astype(dt)
    ref = cic.readout3d(cic.box_to_mesh(pos, box, nm), field, nm, box, bool(vjp))
    out = torch.empty((len(pos), 3), dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    b = _box(box, dt)
    jl.call(f"jld_preadout3d_box_{sfx}", _st(), _p(_cuda(pos)), len(pos), _p(_cuda(field)), *nm,
            b.ctypes.data_as(ct.c_void_p), vjp, _p(out))
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def _paint_tol(dt, ref):
    return (1e-5 if dt == np.float32 else 1e-12) * max(1.0, float(np.abs(ref).max()))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nm,box", CASES)
def test_paint_matches_oracle(jl, dt, nm, box):
    sfx = "f32" if dt == np.float32 else "f64"
    pos = _positions(20000, nm, box, 6, dt)
    mass = np.random.default_rng(7).uniform(0.5, 1.5, len(pos)).astype(dt)
    ref = cic.paint(cic.box_to_mesh(pos, box, nm), mass, nm)
    out = torch.empty(nm, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    b = _box(box, dt)
    cscal = ct.c_float(0) if sfx == "f32" else ct.c_double(0)
    jl.call(f"jld_ppaint_box_{sfx}", _st(), _p(_cuda(pos)), len(pos), _p(_cuda(mass)), cscal, *nm,
            b.ctypes.data_as(ct.c_void_p), _p(out))
    got = out.cpu().numpy()
    assert np.abs(got - ref).max() <= _paint_tol(dt, ref)
    # scalar-mass form
    out.fill_(7.0)
    cscal = ct.c_float(1.25) if sfx == "f32" else ct.c_double(1.25)
    jl.call(f"jld_ppaint_box_{sfx}", _st(), _p(_cuda(pos)), len(pos), None, cscal, *nm,
            b.ctypes.data_as(ct.c_void_p), _p(out))
    ref2 = cic.paint(cic.box_to_mesh(pos, box, nm), dt(1.25), nm)
    assert np.abs(out.cpu().numpy() - ref2).max() <= _paint_tol(dt, ref2)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nm,box,shift", [((16, 16, 16), (16.0, 16.0, 16.0), 0.0),
                                          ((12, 10, 18), (24.0, 5.0, 9.0), 0.37)])
def test_paint_lattice_order(jl, dt, nm, box, shift):
    # particles in lattice order (z fastest) pair up along z inside a warp;
    # the last z column wraps, one y row is displaced by a whole cell, the
    # count is not a multiple of the warp or block size
    g = np.stack(np.meshgrid(*[np.arange(n) for n in nm], indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    g[:, 1] += np.where(np.arange(len(g)) % (nm[1] * nm[2]) < nm[2], 1.0, 0.0)
    cell = np.asarray(box) / np.asarray(nm)
    pos = ((g + shift + 0.01 * np.sin(np.arange(len(g)))[:, None]) * cell)[:-5].astype(dt)
    sfx = "f32" if dt == np.float32 else "f64"
    mass = np.random.default_rng(3).uniform(0.5, 1.5, len(pos)).astype(dt)
    ref = cic.paint(cic.box_to_mesh(pos, box, nm), mass, nm)
    out = torch.empty(nm, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    b = _box(box, dt)
    cscal = ct.c_float(0) if sfx == "f32" else ct.c_double(0)
    jl.call(f"jld_ppaint_box_{sfx}", _st(), _p(_cuda(pos)), len(pos), _p(_cuda(mass)), cscal, *nm,
            b.ctypes.data_as(ct.c_void_p), _p(out))
    assert np.abs(out.cpu().numpy() - ref).max() <= _paint_tol(dt, ref)


@pytest.mark.parametrize("method", [0, 1])
def test_paint_methods_clustered(jl, method):
    # clustered: many particles per cell, signed weights
    nm, box = (32, 32, 32), (32.0, 32.0, 32.0)
    rng = np.random.default_rng(8)
    centers = rng.uniform(0, 32, (20, 3))
    pos = (centers[rng.integers(0, 20, 60000)] + rng.normal(0, 0.3, (60000, 3))).astype(np.float32)
    mass = rng.standard_normal(len(pos)).astype(np.float32)
    ref = cic.paint(cic.box_to_mesh(pos, box, nm), mass, nm)
    out = torch.empty(nm, dtype=torch.float32, device="cuda")
    b = _box(box, np.float32)
    jl.call("jld_ppaint_box_method_f32", _st(), _p(_cuda(pos)), len(pos), _p(_cuda(mass)), ct.c_float(0),
            *nm, b.ctypes.data_as(ct.c_void_p), method, _p(out))
    ref64 = cic.paint(cic.box_to_mesh(pos.astype(np.float64), box, nm), mass.astype(np.float64), nm)
    scale = np.abs(ref64).max()
    assert np.abs(out.cpu().numpy() - ref).max() <= 2e-5 * scale


def _paint_case(case):
    """(positions, masses or None, mesh, box) of the paint-method cases: lattice
    order (long z runs that the face pairing merges), clumps, both mixed,
    meshes whose cells do not line up with the lattice, and edge stencils."""
    from jerald_gb300 import synth
    rng = np.random.default_rng(21)
    if case == "exact_lattice":          # particles on cell corners: runs of 32
        g = np.arange(32, dtype=np.float64) + 0.25
        pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
        return pos, None, (32, 32, 32), (32.0, 32.0, 32.0)
    if case.startswith("lattice"):
        nm = {"lattice": (32, 32, 32), "lattice_nz34": (32, 32, 34), "lattice_nz33": (32, 32, 33)}[case]
        pos = synth.zeldovich(32, 32.0, 0.7, seed=5)
        return pos, rng.uniform(0.5, 1.5, len(pos)).astype(np.float32), nm, (32.0, 32.0, 32.0)
    if case == "mixed":
        pos = synth.clustered(16, 24.0, seed=3, extra_frac=0.6, nhalo=12, rms_cells=1.5)
        return pos, rng.standard_normal(len(pos)).astype(np.float32), (16, 16, 16), (24.0, 24.0, 24.0)
    if case == "ragged_edges":           # 1000 particles, prelude wraps, edge stencils
        pos = _positions(1000, (20, 20, 20), (20.0, 20.0, 20.0), 4, np.float32)
        return pos, rng.uniform(0.5, 1.5, len(pos)).astype(np.float32), (20, 20, 20), (20.0, 20.0, 20.0)
    raise ValueError(case)


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("case", ["exact_lattice", "lattice", "lattice_nz34", "lattice_nz33", "mixed",
                                  "ragged_edges"])
def test_paint_methods_lattice_and_clumps(jl, method, case):
    pos, mass, nm, box = _paint_case(case)
    m = np.ones(len(pos), np.float32) if mass is None else mass
    ref = cic.paint(cic.box_to_mesh(pos, box, nm), m, nm)
    ref64 = cic.paint(cic.box_to_mesh(pos.astype(np.float64), box, nm), m.astype(np.float64), nm)
    out = torch.empty(nm, dtype=torch.float32, device="cuda")
    b = _box(box, np.float32)
    mp = ct.c_void_p(None) if mass is None else _p(_cuda(mass))
    jl.call("jld_ppaint_box_method_f32", _st(), _p(_cuda(pos)), len(pos), mp, ct.c_float(1.0),
            *nm, b.ctypes.data_as(ct.c_void_p), method, _p(out))
    err = np.abs(out.cpu().numpy() - ref).max()
    assert err <= 2e-5 * np.abs(ref64).max(), (case, method, err)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_paint3d_matches_oracle(jl, dt):
    nm, box = (16, 16, 16), (10.0, 10.0, 10.0)
    sfx = "f32" if dt == np.float32 else "f64"
    pos = _positions(10000, nm, box, 9, dt)
    m3 = np.random.default_rng(10).standard_normal((len(pos), 3)).astype(dt)
    ref = cic.paint3d(cic.box_to_mesh(pos, box, nm), m3, nm)
    out = torch.empty((3,) + nm, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    b = _box(box, dt)
    jl.call(f"jld_ppaint3d_box_{sfx}", _st(), _p(_cuda(pos)), len(pos), _p(_cuda(m3)), *nm,
            b.ctypes.data_as(ct.c_void_p), _p(out))
    assert np.abs(out.cpu().numpy() - ref).max() <= _paint_tol(dt, ref)


def test_empty_inputs(jl):
    nm = (8, 8, 8)
    out = torch.full(nm, 3.0, device="cuda")
    b = _box((1.0, 1.0, 1.0), np.float32)
    jl.call("jld_ppaint_box_f32", _st(), None, 0, None, ct.c_float(1.0), *nm, b.ctypes.data_as(ct.c_void_p),
            _p(out))
    assert float(out.abs().sum()) == 0.0
    r = torch.empty(0, device="cuda")
    jl.call("jld_preadout_box_f32", _st(), None, 0, _p(out), *nm, b.ctypes.data_as(ct.c_void_p), -1, _p(out))
    del r


def test_error_statuses(jl):
    nm = (8, 8, 8)
    b = _box((1.0, 1.0, 1.0), np.float32)
    pos = torch.zeros((4, 3), device="cuda")
    f = torch.zeros(nm, device="cuda")
    out = torch.zeros(4, device="cuda")
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_preadout_box_f32", _st(), _p(pos), 4, _p(f), *nm, b.ctypes.data_as(ct.c_void_p), 3, _p(out))
    assert e.value.status == 1
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_ppaint_box_f32", _st(), _p(pos), -1, None, ct.c_float(1), *nm, b.ctypes.data_as(ct.c_void_p),
                _p(f))
    assert e.value.status == 1
    spec = torch.zeros((8, 8, 5), dtype=torch.complex64, device="cuda")
    ws = torch.zeros(10, dtype=torch.uint8, device="cuda")
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_pfft_c_f32", _st(), _p(f), 8, 8, 8, _p(spec), _p(ws), 10)
    assert e.value.status == 3
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_pfft_c_f32", _st(), _p(f), 8, 8, 7, _p(spec), _p(ws), 10 ** 6)
    assert e.value.status == 2
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_buildplan_f32", 7, 8, 8, None)
    assert e.value.status == 2


# -- FFT -------------------------------------------------------------------------

FFT_SHAPES = [(8, 8, 8), (16, 16, 16), (20, 20, 20), (12, 10, 8), (32, 48, 40), (64, 64, 64),
              (96, 96, 96), (2, 3, 2), (1, 1, 2), (128, 128, 128), (256, 64, 512), (30, 30, 30),
              (16, 256, 256), (16, 512, 512), (192, 192, 192), (160, 96, 144), (96, 192, 96),
              (192, 48, 384)]


def _ws(jl, nm, dt):
    sfx = "f32" if dt == np.float32 else "f64"
    n = getattr(jl.load(), f"jld_fft_workspace_{sfx}")(*nm)
    return torch.empty(int(n), dtype=torch.uint8, device="cuda")


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nm", FFT_SHAPES)
def test_pfft_matches_dft(jl, dt, nm):
    sfx = "f32" if dt == np.float32 else "f64"
    x = np.random.default_rng(11).standard_normal(nm).astype(dt)
    ref = o_pfft(x.astype(np.float64))
    cdt = torch.complex64 if dt == np.float32 else torch.complex128
    out = torch.empty((nm[0], nm[1], nm[2] // 2 + 1), dtype=cdt, device="cuda")
    ws = _ws(jl, nm, dt)
    jl.call(f"jld_pfft_c_{sfx}", _st(), _p(_cuda(x)), *nm, _p(out), _p(ws), ws.numel())
    got = out.cpu().numpy()
    scale = np.sqrt(np.mean(np.abs(ref) ** 2)) + 1e-30
    tol = 2e-6 * np.log2(max(x.size, 2)) if dt == np.float32 else 1e-13 * np.log2(max(x.size, 2))
    assert np.abs(got - ref).max() / scale < tol
    # split re/im variant gives identical values
    re = torch.empty(out.shape, dtype=out.real.dtype, device="cuda")
    im = torch.empty_like(re)
    jl.call(f"jld_pfft_{sfx}", _st(), _p(_cuda(x)), *nm, _p(re), _p(im), _p(ws), ws.numel())
    assert torch.equal(re, out.real) and torch.equal(im, out.imag)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nm", FFT_SHAPES)
def test_pifft_matches_definition(jl, dt, nm):
    sfx = "f32" if dt == np.float32 else "f64"
    rng = np.random.default_rng(12)
    h = nm[2] // 2 + 1
    y = (rng.standard_normal(nm[:2] + (h,)) + 1j * rng.standard_normal(nm[:2] + (h,)))
    ref = o_pifft(y, nm)
    cdt = np.complex64 if dt == np.float32 else np.complex128
    out = torch.empty(nm, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
    ws = _ws(jl, nm, dt)
    yin = _cuda(y.astype(cdt))
    jl.call(f"jld_pifft_c_{sfx}", _st(), _p(yin), *nm, _p(out), _p(ws), ws.numel())
    got = out.cpu().numpy()
    scale = np.sqrt(np.mean(ref ** 2)) + 1e-30
    tol = 2e-6 * np.log2(max(np.prod(nm), 2)) if dt == np.float32 else 1e-13 * np.log2(max(np.prod(nm), 2))
    assert np.abs(got - ref).max() / scale < tol
    re = _cuda(y.real.astype(dt))
    im = _cuda(y.imag.astype(dt))
    out2 = torch.empty_like(out)
    jl.call(f"jld_pifft_{sfx}", _st(), _p(re), _p(im), *nm, _p(out2), _p(ws), ws.numel())
    assert torch.equal(out, out2)


@pytest.mark.parametrize("nm", [(64, 64, 64), (256, 64, 512)])
def test_fft_alignment_fallback_and_rejection(jl, nm):
    # 8-byte aligned (not 16) input / output: no bulk or tensor copies, the
    # generic passes run and give the same transform.  4-byte aligned: the
    # complex-pair accesses cannot run at all, so the call is rejected on
    # the host before any launch.
    from jerald_gb300 import _lib
    x = torch.randn(nm, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    xo = torch.empty(x.numel() + 2, device="cuda")
    xo[2:] = x.reshape(-1)
    h = nm[2] // 2 + 1
    ws = _ws(jl, nm, np.float32)
    a = torch.empty(nm[:2] + (h,), dtype=torch.complex64, device="cuda")
    b = torch.empty_like(a)
    jl.call("jld_pfft_c_f32", _st(), _p(x), *nm, _p(a), _p(ws), ws.numel())
    jl.call("jld_pfft_c_f32", _st(), ct.c_void_p(xo.data_ptr() + 8), *nm, _p(b), _p(ws), ws.numel())
    scale = a.abs().pow(2).mean().sqrt().item()
    assert (a - b).abs().max().item() / scale < 2e-6 * np.log2(x.numel())
    yo = torch.empty(x.numel() + 2, device="cuda")
    ya = torch.empty(nm, device="cuda")
    jl.call("jld_pifft_c_f32", _st(), _p(a), *nm, _p(ya), _p(ws), ws.numel())
    jl.call("jld_pifft_c_f32", _st(), _p(a), *nm, ct.c_void_p(yo.data_ptr() + 8), _p(ws), ws.numel())
    yb = yo[2:].reshape(nm)
    assert (ya - yb).abs().max().item() / ya.abs().max().item() < 1e-5
    with pytest.raises(_lib.JLDError) as e:
        jl.call("jld_pfft_c_f32", _st(), ct.c_void_p(xo.data_ptr() + 4), *nm, _p(b), _p(ws), ws.numel())
    assert e.value.status == 1
    with pytest.raises(_lib.JLDError):
        jl.call("jld_pifft_c_f32", _st(), _p(a), *nm, ct.c_void_p(yo.data_ptr() + 4), _p(ws), ws.numel())
    v = ct.c_int32(-1)
    jl.call("jld_fft_pipe_status", ct.byref(v), 1)
    assert v.value == 0


def test_fft_roundtrip_large(jl):
    # size-independent property at 512^3: pifft(pfft(x)) = N x
    nm = (512, 512, 512)
    x = torch.randn(nm, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    spec = torch.empty((512, 512, 257), dtype=torch.complex64, device="cuda")
    ws = _ws(jl, nm, np.float32)
    jl.call("jld_pfft_c_f32", _st(), _p(x), *nm, _p(spec), _p(ws), ws.numel())
    # DC term equals the sum; Parseval holds
    s = x.double().sum()
    assert abs(spec[0, 0, 0].real.double() - s) < 1e-4 * x.numel() ** 0.5 * 10
    y = torch.empty_like(x)
    jl.call("jld_pifft_c_f32", _st(), _p(spec), *nm, _p(y), _p(ws), ws.numel())
    err = (y / x.numel() - x).abs().max().item()
    assert err < 2e-5


@pytest.mark.parametrize("nbytes", [16, 1000003, 64 << 20])
def test_copy_from_host_kernel(jl, nbytes):
    # the host-feed copy kernel reproduces the page-locked source exactly,
    # including a tail that is not a whole 16-byte word
    src = torch.randint(0, 256, (nbytes,), dtype=torch.uint8).pin_memory()
    dst = torch.zeros(nbytes + 16, dtype=torch.uint8, device="cuda")
    jl.call("jld_copy_from_host", _st(), _p(dst), _p(src), nbytes, 16)
    torch.cuda.synchronize()
    assert torch.equal(dst[:nbytes].cpu(), src)
    assert int(dst[nbytes:].sum()) == 0
    with pytest.raises(jl.JLDError):  # pageable source is rejected
        jl.call("jld_copy_from_host", _st(), _p(dst), _p(torch.empty(64, dtype=torch.uint8)), 64, 16)


def test_c1_scale_ops_match_oracle(jl):
    # the 256^3 validation configuration: clustered positions (1.85e7
    # particles), cell keys and readout bit-exact, paint within 1e-5 of the
    # mesh scale, all through the C ABI against the oracle's C loops
    from jerald_gb300 import synth
    n, box = 256, 400.0
    nm, b3 = (n, n, n), (box, box, box)
    pos = synth.clustered(n, box, seed=5).astype(np.float32)
    q = cic.box_to_mesh(pos, b3, nm)
    b = _box(b3, np.float32)
    dpos = _cuda(pos)
    keys = torch.empty(len(pos), dtype=torch.int32, device="cuda")
    jl.call("jld_cell_keys_f32", _st(), _p(dpos), len(pos), *nm, b.ctypes.data_as(ct.c_void_p), _p(keys))
    np.testing.assert_array_equal(keys.cpu().numpy(), cic.cell_keys(q, nm))
    field = np.random.default_rng(6).standard_normal(nm).astype(np.float32)
    out = torch.empty(len(pos), dtype=torch.float32, device="cuda")
    jl.call("jld_preadout_box_f32", _st(), _p(dpos), len(pos), _p(_cuda(field)), *nm,
            b.ctypes.data_as(ct.c_void_p), -1, _p(out))
    np.testing.assert_array_equal(out.cpu().numpy(), cic.readout(q, field, nm, b3, -1))
    mesh = torch.empty(nm, dtype=torch.float32, device="cuda")
    jl.call("jld_ppaint_box_f32", _st(), _p(dpos), len(pos), None, ct.c_float(1.0), *nm,
            b.ctypes.data_as(ct.c_void_p), _p(mesh))
    ref = cic.paint(q, np.float32(1.0), nm)
    assert np.abs(mesh.cpu().numpy() - ref).max() <= _paint_tol(np.float32, ref)
