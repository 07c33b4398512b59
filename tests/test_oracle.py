"""Known-answer tests that pin the oracle (CPU only).

The reference cannot run here (its ops need MPI and FFTW), so these tests
pin the restatement against definitions: a direct DFT, exact CIC weights,
mass conservation, adjointness, finite differences, and the committed
fixtures in tests/golden/.
"""
import numpy as np
import pytest

from oracle import cic
from oracle.fft import direct_irfft3, direct_rfft3, pfft, pifft
from oracle.ldl import LDLOracle

RNG = np.random.default_rng(1234)


# -- FFT conventions -------------------------------------------------------------

@pytest.mark.parametrize("shape", [(4, 6, 8), (5, 3, 6), (2, 2, 2)])
def test_pfft_is_unnormalised_sign_minus_dft(shape):
    x = RNG.standard_normal(shape)
    np.testing.assert_allclose(pfft(x), direct_rfft3(x), rtol=0, atol=1e-10)


@pytest.mark.parametrize("shape", [(4, 6, 8), (3, 5, 6)])
def test_pifft_matches_definition_on_non_hermitian_input(shape):
    h = shape[2] // 2 + 1
    y = RNG.standard_normal(shape[:2] + (h,)) + 1j * RNG.standard_normal(shape[:2] + (h,))
    np.testing.assert_allclose(pifft(y, shape), direct_irfft3(y, shape), rtol=0, atol=1e-9)


def test_pifft_pfft_roundtrip_is_n_times_identity():
    x = RNG.standard_normal((8, 6, 10))
    np.testing.assert_allclose(pifft(pfft(x), x.shape), x.size * x, rtol=1e-12, atol=1e-9)


# -- CIC ------------------------------------------------------------------------

NM = (6, 5, 4)
BOX = (6.0, 10.0, 2.0)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_particle_at_cell_centre_spreads_one_eighth(dt):
    pos = np.array([[2.5, 1.5, 0.5]], dtype=dt)
    m = cic.paint(pos, 1.0, NM)
    nz = np.argwhere(m != 0)
    assert len(nz) == 8
    assert np.all(m[m != 0] == dt(0.125))
    assert {tuple(v) for v in nz} == {(i, j, k) for i in (2, 3) for j in (1, 2) for k in (0, 1)}


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_particle_on_grid_point_lands_in_one_cell(dt):
    pos = np.array([[5.0, 4.0, 3.0]], dtype=dt)  # upper neighbours wrap to 0
    m = cic.paint(pos, 2.0, NM)
    assert m[5, 4, 3] == 2.0 and m.sum() == 2.0


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_mass_conservation(dt):
    pos = RNG.uniform(0, 1, (1000, 3)) * np.array(NM)
    mass = RNG.uniform(0.5, 1.5, 1000)
    m = cic.paint(pos.astype(dt), mass.astype(dt), NM)
    tol = 1e-4 if dt == np.float32 else 1e-10
    assert abs(m.sum() - mass.astype(dt).sum()) / mass.sum() < tol


def test_box_prelude_edge_case_drops_particle():
    # x mod L rounds up to exactly L in float32: the mesh coordinate is N, the
    # lower corner index N is out of range and its weight is dropped
    # (lib/parops_fast.h:388-402), so the particle paints nothing.
    box = (100.0, 100.0, 100.0)
    pos = np.array([[-1e-10, 50.0, 50.0]], dtype=np.float32)
    pm = cic.box_to_mesh(pos, box, (64, 64, 64))
    assert pm[0, 0] == np.float32(64.0)
    assert cic.cell_keys(pm, (64, 64, 64))[0] == (0 * 64 + 32) * 64 + 32
    assert cic.paint(pm, 1.0, (64, 64, 64)).sum() == 0.0
    # float64 keeps the tiny offset: the particle is conserved
    pm64 = cic.box_to_mesh(pos.astype(np.float64), box, (64, 64, 64))
    assert pm64[0, 0] < 64.0
    assert abs(cic.paint(pm64, 1.0, (64, 64, 64)).sum() - 1.0) < 1e-12


def test_box_prelude_is_jnp_remainder():
    box = (10.0, 10.0, 10.0)
    x = np.array([[-3.0, 13.0, 10.0], [-0.0, 0.0, 25.5]])
    pm = cic.box_to_mesh(x, box, (10, 10, 10))
    np.testing.assert_array_equal(pm, [[7.0, 3.0, 0.0], [-0.0, 0.0, 5.5]])


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_paint_readout_adjoint(dt):
    pos = RNG.uniform(0, 1, (500, 3)) * np.array(NM)
    mass = RNG.standard_normal(500)
    f = RNG.standard_normal(NM)
    lhs = np.sum(cic.paint(pos.astype(dt), mass.astype(dt), NM).astype(np.float64) * f)
    rhs = np.sum(mass * cic.readout(pos.astype(dt), f.astype(dt), NM, BOX).astype(np.float64))
    assert abs(lhs - rhs) <= (1e-4 if dt == np.float32 else 1e-10) * np.abs(lhs)


def test_readout_vjp_is_derivative_in_box_units():
    # d/dx_box readout(x_box) = readout with vjpdim (weights +-N/L), away from cell edges
    f = RNG.standard_normal(NM)
    pos_box = np.array([[2.3, 4.1, 0.7]])
    h = 1e-6
    for d in range(3):
        p1, p0 = pos_box.copy(), pos_box.copy()
        p1[0, d] += h; p0[0, d] -= h
        r1 = cic.readout(cic.box_to_mesh(p1, BOX, NM), f, NM, BOX)[0]
        r0 = cic.readout(cic.box_to_mesh(p0, BOX, NM), f, NM, BOX)[0]
        g = cic.readout(cic.box_to_mesh(pos_box, BOX, NM), f, NM, BOX, vjpdim=d)[0]
        assert abs((r1 - r0) / (2 * h) - g) < 1e-6 * max(1, abs(g))


def test_readout3d_and_paint3d_consistency():
    pos = (RNG.uniform(0, 1, (300, 3)) * np.array(NM)).astype(np.float64)
    f3 = RNG.standard_normal((3,) + NM)
    r3 = cic.readout3d(pos, f3, NM, BOX, vjp=False)
    for d in range(3):
        np.testing.assert_array_equal(r3[:, d], cic.readout(pos, f3[d], NM, BOX))
    rv = cic.readout3d(pos, f3[0], NM, BOX, vjp=True)
    for d in range(3):
        np.testing.assert_array_equal(rv[:, d], cic.readout(pos, f3[0], NM, BOX, vjpdim=d))
    m3 = RNG.standard_normal((300, 3))
    p3 = cic.paint3d(pos, m3, NM)
    for d in range(3):
        np.testing.assert_array_equal(p3[d], cic.paint(pos, m3[:, d], NM))


def test_out_of_range_mesh_coordinates_follow_reference_masking():
    # mesh-unit coordinates outside [0, N): the corner flags of lpaint decide
    pos = np.array([[-1.5, 0.5, 0.5], [6.25, 0.5, 0.5]])
    m = cic.paint(pos, 1.0, NM)
    # p = -1.5: i = int(-1.5) = -1 (invalid lower corner), i+1 = 0 valid with d = -0.5
    assert np.isclose(m[0].sum(), -0.5)
    # p = 6.25: i = 6 == N (invalid), i+1 = 7 % 6 = 1 valid with d = 0.25
    assert np.isclose(m[1].sum(), 0.25)


# -- LDL pipeline -----------------------------------------------------------------

def _small_case(kind="sm", L1=False, n=8):
    from jerald_gb300 import synth
    X = synth.zeldovich(n, 50.0, 0.5, seed=7, dtype=np.float64)
    p = synth.default_params(2)
    o = LDLOracle((n, n, n), 50.0, kind=kind, L1=L1)
    o.forward(p, X, np.ones((n, n, n)), 2)
    tgt = o.cache["F"] * synth.lognormal_noise(o.cache["F"].shape, 0.1, 3)
    return o, p, X, tgt


@pytest.mark.parametrize("kind", ["sm", "dm"])
def test_true_gradient_matches_central_differences(kind):
    o, p, X, tgt = _small_case(kind)
    _, g = o.loss_and_grad(p, X, tgt, 2, mode="true")
    fd = o.fd_grad(p, X, tgt, 2, step=1e-4, idx=range(10 if kind == "dm" else 13))
    idx = ~np.isnan(fd)
    rel = np.abs(g[idx] - fd[idx]) / np.maximum(np.abs(fd[idx]), 1e-3 * np.abs(fd[idx]).max())
    assert rel.max() < 1e-3, rel


def test_reference_rule_differs_only_in_alpha():
    o, p, X, tgt = _small_case("sm")
    _, gr = o.loss_and_grad(p, X, tgt, 2, mode="reference")
    gt = o.backward("true")
    alpha = [0, 5]
    others = [i for i in range(13) if i not in alpha]
    np.testing.assert_allclose(gr[others], gt[others], rtol=1e-12, atol=1e-18)
    assert np.all(np.abs(gr[alpha] - gt[alpha]) > 1e-3 * np.abs(gt[alpha]))


def test_model_loss_matches_pipeline_forward():
    # the general forward (all kinds and options) agrees with the pipeline
    # the gradient oracle differentiates, where both apply
    from jerald_gb300 import synth
    from oracle.ldl import LDLOracle, model_loss
    n, box = 16, 50.0
    X = synth.zeldovich(n, box, 0.5, seed=7).astype(np.float64)
    for kind in ("sm", "dm"):
        p = synth.default_params(2)
        if kind == "dm":
            p = p[:10]
        tgt = np.random.default_rng(1).uniform(0.5, 1.5, (n,) * 3)
        o = LDLOracle((n,) * 3, box, kind=kind, L1=(kind == "sm"))
        a = o.forward(p, X, tgt, 2)
        b, _ = model_loss((n,) * 3, box, kind, p, X, tgt, 2)
        assert abs(a - b) <= 1e-12 * abs(a)


def test_model_loss_smoothing_known_answer():
    """A residual that is the same constant c in every cell has only a k = 0
    mode; the smoothing kernel weights it (1e-8)^-n + 1 (|k| = 0 is read as
    1e-8, model.py:100-102), so the smoothed residual is c times that weight
    everywhere: L1 loss |c| ((1e-8)^-n + 1), L2 its square; the validation
    mask takes the same values over its own cells."""
    import numpy as np
    from oracle.ldl import model_loss
    n, box = 8, 10.0
    g = (np.arange(n) + 0.0) * box / n
    X = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)  # one particle per cell corner
    p = np.array([0.0, 1.0, 0.5, 2.0, 1.0] * 2)                           # alpha = 0: no displacement
    c = 0.25
    tgt = np.full((n,) * 3, 1.0 - c)                                      # dm map is 1 in every cell
    for nn in (0.25, 0.5):
        K0 = (1e-8) ** (-nn) + 1.0
        l1, _ = model_loss((n,) * 3, box, "dm", p, X, tgt, 2, n=nn, L1=True)
        assert abs(l1 - c * K0) <= 1e-9 * c * K0
        mv = np.zeros((n,) * 3)
        mv[:2] = 1.0
        l2, lv = model_loss((n,) * 3, box, "dm", p, X, tgt, 2, n=nn, L1=False, maskvalid=mv)
        assert abs(l2 - (c * K0) ** 2) <= 1e-9 * (c * K0) ** 2
        assert abs(lv - (c * K0) ** 2) <= 1e-9 * (c * K0) ** 2
    l0, _ = model_loss((n,) * 3, box, "dm", p, X, tgt, 2, n=0, L1=True)
    assert abs(l0 - c) <= 1e-12


def test_oracle_float32_position_storage():
    """pos_dtype=np.float32 keeps every layer's positions float32-representable
    and otherwise computes the same pipeline: at 16^3 its loss and gradient
    stay within 1e-6 of the FP64 oracle's."""
    from jerald_gb300 import synth
    from oracle import ldl as oldl
    n, L = 16, 25.0
    X = synth.zeldovich(n, L, 0.5, seed=1, dtype=np.float32).astype(np.float64)
    p = synth.default_params(2)
    t = synth.lognormal_noise((n,) * 3, 0.1, 2)
    a = oldl.LDLOracle((n,) * 3, L)
    b = oldl.LDLOracle((n,) * 3, L, pos_dtype=np.float32)
    la, lb = a.forward(p, X, t, 2), b.forward(p, X, t, 2)
    xf = b.cache["X_final"]
    assert np.array_equal(xf, xf.astype(np.float32).astype(np.float64))
    assert not np.array_equal(a.cache["X_final"], a.cache["X_final"].astype(np.float32).astype(np.float64))
    assert abs(la - lb) <= 1e-6 * abs(la)
    ga, gb = a.backward(), b.backward()
    assert np.abs(ga - gb).max() <= 1e-6 * np.abs(ga).max()
