"""The oracle reproduces the committed fixtures (CPU)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import cic
from oracle.fft import pfft, pifft
from oracle.ldl import LDLOracle

G = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["cic_f32.npz", "cic_f64.npz"])
def test_cic_fixture(name):
    f = np.load(G / name)
    nm, box = tuple(f["nmesh"]), tuple(f["box"])
    pm = cic.box_to_mesh(f["pos"], box, nm)
    np.testing.assert_array_equal(pm, f["mesh_pos"])
    np.testing.assert_array_equal(cic.cell_keys(pm, nm), f["keys"])
    np.testing.assert_array_equal(cic.paint(pm, f["mass"], nm), f["paint"])
    np.testing.assert_array_equal(cic.paint3d(pm, f["mass3"], nm), f["paint3d"])
    for d in (-1, 0, 1, 2):
        np.testing.assert_array_equal(cic.readout(pm, f["field"], nm, box, d), f[f"readout_{d + 1}"])
    np.testing.assert_array_equal(cic.readout3d(pm, f["field3"], nm, box, False), f["readout3d"])
    np.testing.assert_array_equal(cic.readout3d(pm, f["field"], nm, box, True), f["readout3d_vjp"])


def test_fft_fixture():
    f = np.load(G / "fft.npz")
    np.testing.assert_allclose(pfft(f["x"]), f["X"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(pifft(f["y"], f["x"].shape), f["yinv"], rtol=0, atol=1e-11)


def test_ldl_fixture():
    f = np.load(G / "ldl_sm16.npz")
    n = int(f["n"])
    o = LDLOracle((n,) * 3, float(f["box"]), kind="sm", L1=True)
    loss, g = o.loss_and_grad(f["params"], f["X"], f["target"], 2, mode="reference")
    assert abs(loss - float(f["loss"])) <= 1e-12 * abs(loss)
    np.testing.assert_allclose(g, f["grad_reference"], rtol=1e-9, atol=1e-20)
    np.testing.assert_allclose(o.backward("true"), f["grad_true"], rtol=1e-9, atol=1e-20)
    od = LDLOracle((n,) * 3, float(f["box"]), kind="dm", L1=False)
    loss_dm, g_dm = od.loss_and_grad(f["params"][:10], f["X"], np.ones((n,) * 3), 2, mode="true")
    assert abs(loss_dm - float(f["loss_dm"])) <= 1e-12 * abs(loss_dm)
    np.testing.assert_allclose(g_dm, f["grad_dm_true"], rtol=1e-9, atol=1e-20)


def test_ldl_hi_fixture():
    """The HI kind's FP64 forward (model.py:213-247, 313-336) and the central
    differences of its L2 loss; the differences agree with those at half the
    step to 4e-7 per component, so they pin the layer gradients (1e-7 of the
    final map's at these parameters) as well as the map's."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", G / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    from oracle.ldl import model_loss
    f = np.load(G / "ldl_hi16.npz")
    n, box = int(f["n"]), float(f["box"])
    args = (f["params"], f["X"], f["target"], 2)
    assert f["params"].shape == (32,)
    for L1, key in ((True, "loss_l1"), (False, "loss_l2")):
        loss = model_loss((n,) * 3, box, "HI", *args, starmap=f["starmap"], L1=L1)[0]
        assert abs(loss - float(f[key])) <= 1e-12 * abs(loss)
    g = mg.hi_fd_grad(n, box, f["params"], f["X"], f["target"], f["starmap"])
    # atol: a rounding change of the forward moves a difference by ~1e-12
    np.testing.assert_allclose(g, f["grad_l2_fd"], rtol=1e-7, atol=1e-10)


def test_losstest_fixture():
    f = np.load(G / "losstest20.npz")
    o = LDLOracle((20,) * 3, 200.0, kind="sm", L1=True)
    loss = o.forward(f["params"], f["pos"], f["target"], 2, mask=np.ones_like(f["target"]))
    np.testing.assert_allclose(loss, f["loss"], rtol=1e-12)
    np.testing.assert_allclose(o.backward("reference"), f["grad"], rtol=1e-9, atol=1e-20)
