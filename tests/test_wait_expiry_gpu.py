"""A bounded device wait that runs out reports through the status words and
leaves the context usable (nothing hangs, nothing faults).

jld_wait_selftest arms an mbarrier for a copy that is never issued and polls
it with the pipelined passes' bounded wait; after the poll limit the CTA
writes its code (99) to the error word and returns.  The word is read back
through jld_fft_pipe_status (standalone FFT passes) and through
FusedLDL.error_word() (the fused step's word), and the next real call runs
and clears it.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SELFTEST_CODE = 99


@pytest.fixture(scope="module")
def jl():
    from jerald_gb300 import _lib, build
    build.build()
    return _lib


def _st():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _status(jl, reset):
    v = ct.c_int32(-1)
    jl.call("jld_fft_pipe_status", ct.byref(v), reset)
    return v.value


def test_fft_word_reports_expired_wait(jl):
    _status(jl, 1)
    assert _status(jl, 0) == 0
    jl.call("jld_wait_selftest", _st(), 4096, None)
    assert _status(jl, 1) == SELFTEST_CODE
    assert _status(jl, 0) == 0
    # a pipelined r2c afterwards runs normally and leaves the word clear
    from oracle.fft import pfft
    n = 32
    x = np.random.default_rng(1).standard_normal((n, n, n)).astype(np.float32)
    ws = torch.empty(jl.load().jld_fft_workspace_f32(n, n, n), dtype=torch.uint8, device="cuda")
    out = torch.empty((n, n, n // 2 + 1, 2), dtype=torch.float32, device="cuda")
    xd = torch.from_numpy(x).cuda()
    jl.call("jld_pfft_c_f32", _st(), ct.c_void_p(xd.data_ptr()), n, n, n, ct.c_void_p(out.data_ptr()),
            ct.c_void_p(ws.data_ptr()), ws.numel())
    got = out.cpu().numpy()
    ref = pfft(x.astype(np.float64))
    err = np.abs(got[..., 0] + 1j * got[..., 1] - ref).max() / np.abs(ref).max()
    assert err < 1e-5
    assert _status(jl, 0) == 0


def test_fused_word_reports_expired_wait(jl):
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    n, box = 16, 100.0
    X = torch.from_numpy(synth.zeldovich(n, box, 0.5, seed=3, dtype=np.float32)).cuda()
    tgt = torch.ones((n, n, n), dtype=torch.float32, device="cuda")
    step = FusedLDL(n, box, X.shape[0], nstep=2)
    p = synth.default_params(2)
    loss, _ = step(X, p, tgt)
    torch.cuda.synchronize()
    assert step.error_word() == 0
    ptr = ct.c_void_p()
    jl.call("jld_ldl_error_word_f32", ct.c_void_p(step.ws.data_ptr()), n, n, n, X.shape[0], 2, ct.byref(ptr))
    jl.call("jld_wait_selftest", _st(), 4096, ptr)
    torch.cuda.synchronize()
    assert step.error_word() == SELFTEST_CODE
    # the next step clears the word at its start and completes
    loss2, g2 = step(X, p, tgt)
    torch.cuda.synchronize()
    assert step.error_word() == 0
    assert np.isfinite(float(loss2)) and float(loss2) == pytest.approx(float(loss), rel=1e-6)
    assert torch.isfinite(g2).all()
