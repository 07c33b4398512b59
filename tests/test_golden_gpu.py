"""The CUDA path reproduces the committed fixtures (GPU, through the C ABI
for the CIC ops and the FFT, through the public Python API for the LDL)."""
import ctypes as ct
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

G = Path(__file__).resolve().parent / "golden"


def _st():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("name", ["cic_f32.npz", "cic_f64.npz"])
def test_cic_fixture_gpu(name):
    from jerald_gb300 import _lib
    f = np.load(G / name)
    dt = f["pos"].dtype
    sfx = "f32" if dt == np.float32 else "f64"
    tdt = torch.float32 if dt == np.float32 else torch.float64
    nm = tuple(int(v) for v in f["nmesh"])
    box = np.ascontiguousarray(f["box"].astype(dt))
    bp = box.ctypes.data_as(ct.c_void_p)
    pos = torch.from_numpy(f["pos"]).cuda()
    field = torch.from_numpy(f["field"]).cuda()
    field3 = torch.from_numpy(f["field3"]).cuda()
    mass = torch.from_numpy(f["mass"]).cuda()
    mass3 = torch.from_numpy(f["mass3"]).cuda()
    N = pos.shape[0]
    P = lambda t: ct.c_void_p(t.data_ptr())  # noqa: E731
    keys = torch.empty(N, dtype=torch.int32, device="cuda")
    _lib.call(f"jld_cell_keys_{sfx}", _st(), P(pos), N, *nm, bp, P(keys))
    np.testing.assert_array_equal(keys.cpu().numpy(), f["keys"])
    out = torch.empty(N, dtype=tdt, device="cuda")
    for d in (-1, 0, 1, 2):
        _lib.call(f"jld_preadout_box_{sfx}", _st(), P(pos), N, P(field), *nm, bp, d, P(out))
        np.testing.assert_array_equal(out.cpu().numpy(), f[f"readout_{d + 1}"])
    out3 = torch.empty((N, 3), dtype=tdt, device="cuda")
    _lib.call(f"jld_preadout3d_box_{sfx}", _st(), P(pos), N, P(field3), *nm, bp, 0, P(out3))
    np.testing.assert_array_equal(out3.cpu().numpy(), f["readout3d"])
    _lib.call(f"jld_preadout3d_box_{sfx}", _st(), P(pos), N, P(field), *nm, bp, 1, P(out3))
    np.testing.assert_array_equal(out3.cpu().numpy(), f["readout3d_vjp"])
    mesh = torch.empty(nm, dtype=tdt, device="cuda")
    cz = ct.c_float(0) if sfx == "f32" else ct.c_double(0)
    _lib.call(f"jld_ppaint_box_{sfx}", _st(), P(pos), N, P(mass), cz, *nm, bp, P(mesh))
    tol = (1e-5 if sfx == "f32" else 1e-12) * np.abs(f["paint"]).max()
    assert np.abs(mesh.cpu().numpy() - f["paint"]).max() <= tol
    mesh3 = torch.empty((3,) + nm, dtype=tdt, device="cuda")
    _lib.call(f"jld_ppaint3d_box_{sfx}", _st(), P(pos), N, P(mass3), *nm, bp, P(mesh3))
    tol = (1e-5 if sfx == "f32" else 1e-12) * np.abs(f["paint3d"]).max()
    assert np.abs(mesh3.cpu().numpy() - f["paint3d"]).max() <= tol


def test_fft_fixture_gpu():
    from jerald_gb300 import jaxpops_bind as jpo
    f = np.load(G / "fft.npz")
    x = torch.from_numpy(f["x"]).cuda()
    X = jpo.pfft(x, x.shape).cpu().numpy()
    np.testing.assert_allclose(X, f["X"], rtol=0, atol=1e-12)
    y = torch.from_numpy(f["y"]).cuda()
    np.testing.assert_allclose(jpo.pifft(y, x.shape).cpu().numpy(), f["yinv"], rtol=0, atol=1e-11)


def test_ldl_fixture_gpu():
    from jerald_gb300.ldl import FusedLDL
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    f = np.load(G / "ldl_sm16.npz")
    n, box = int(f["n"]), float(f["box"])
    X = torch.from_numpy(f["X"]).cuda()
    t = torch.from_numpy(f["target"]).cuda()
    model = JERALDModel(X, t, PMesh(n, box, dtype=torch.float64), Nstep=2, kind="sm")
    loss, g = model.loss_and_grad(torch.from_numpy(f["params"]))
    assert abs(float(loss) - float(f["loss"])) <= 1e-10 * abs(float(f["loss"]))
    ref = f["grad_reference"]
    assert np.max(np.abs(g.cpu().numpy() - ref) / np.maximum(np.abs(ref), 1e-6 * np.abs(ref).max())) < 1e-7
    fu = FusedLDL(n, box, X.shape[0], nstep=2, kind="sm", grad_mode="true")
    lf, gf = fu(X.float().contiguous(), f["params"], t.float().contiguous())
    torch.cuda.synchronize()
    assert abs(float(lf) - float(f["loss"])) <= 1e-5 * abs(float(f["loss"]))
    gt = f["grad_true"]
    assert np.max(np.abs(gf.cpu().numpy() - gt) / np.maximum(np.abs(gt), 1e-6 * np.abs(gt).max())) < 1e-3


def test_losstest_fixture_gpu():
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    f = np.load(G / "losstest20.npz")
    pos = torch.from_numpy(f["pos"]).cuda()
    tgt = torch.from_numpy(f["target"]).cuda()
    model = JERALDModel(pos, tgt, PMesh(20, 200, dtype=torch.float64), Nstep=2, kind="sm",
                        masktrain=torch.ones_like(tgt), maskvalid=torch.from_numpy(f["maskvalid"]).cuda())
    loss, lossv, g = model.lossv_and_grad(torch.from_numpy(f["params"]))
    assert abs(float(loss) - float(f["loss"])) <= 1e-11 * abs(float(f["loss"]))
    assert abs(float(lossv) - float(f["lossv"])) <= 1e-11 * abs(float(f["lossv"]))
    ref = f["grad"]
    assert np.max(np.abs(g.cpu().numpy() - ref) / np.maximum(np.abs(ref), 1e-6 * np.abs(ref).max())) < 1e-7
