"""The allocation-free r2c entry point (jld_pfft_c_static_f32).

Some callers of this library cannot allocate device memory themselves: a host
framework that owns every allocation, or code in a phase where allocating is
not allowed.  For them the library offers an r2c that takes no workspace and
keeps its scratch in a fixed device array inside the library.  This test
calls it through the C ABI on three meshes in a row (different shapes and
data, one of mixed radix, so each call runs over whatever the previous one
left in the shared scratch and twiddle table) and checks each result against
the workspace-taking jld_pfft_c_f32 and against the oracle's float64 DFT,
within the tolerance the FFT tests use.  It also checks that a mesh too large
for the fixed scratch is refused.  The file sorts last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _lib():
    from jerald_gb300 import _lib, build
    build.build()
    return _lib


def _st():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ct.c_void_p(t.data_ptr())


def _with_workspace(jl, x, nm):
    out = torch.empty((nm[0], nm[1], nm[2] // 2 + 1), dtype=torch.complex64, device="cuda")
    ws = torch.empty(int(jl.load().jld_fft_workspace_f32(*nm)), dtype=torch.uint8, device="cuda")
    jl.call("jld_pfft_c_f32", _st(), _p(x), *nm, _p(out), _p(ws), ws.numel())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _tol(nm):
    return 2e-6 * np.log2(max(int(np.prod(nm)), 2))


def test_no_alloc_r2c_matches_workspace_version_and_dft():
    from oracle.fft import pfft
    jl = _lib()
    rng = np.random.default_rng(5)
    for nm in [(64, 48, 32), (48, 40, 30), (32, 32, 32)]:
        xh = rng.standard_normal(nm).astype(np.float32)
        x = torch.from_numpy(xh).cuda()
        ref = _with_workspace(jl, x, nm)
        dft = pfft(xh.astype(np.float64))
        out = torch.full((nm[0], nm[1], nm[2] // 2 + 1), complex(7.0, 7.0), dtype=torch.complex64, device="cuda")
        jl.call("jld_pfft_c_static_f32", _st(), _p(x), *nm, _p(out))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        scale = np.sqrt(np.mean(np.abs(dft) ** 2))
        assert np.abs(got - ref).max() / scale < _tol(nm), nm
        assert np.abs(got - dft).max() / scale < _tol(nm), nm


def test_no_alloc_r2c_rejects_meshes_beyond_its_scratch():
    jl = _lib()
    x = torch.zeros(1, device="cuda")
    out = torch.zeros(1, device="cuda")
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_pfft_c_static_f32", _st(), _p(x), 512, 512, 512, _p(out))
    assert e.value.status == 3
    with pytest.raises(jl.JLDError) as e:
        jl.call("jld_pfft_c_static_f32", _st(), _p(x), 8192, 2, 2, _p(out))
    assert e.value.status == 2
