"""Regenerates the committed fixtures in tests/golden/ from the oracle.

The reference cannot run in this environment (its custom calls need MPI and
FFTW, its bindings JAX), so these fixtures hold the oracle's outputs for
fixed seeded inputs; tests/test_golden.py pins the oracle to them on the CPU
and tests/test_golden_gpu.py holds the CUDA path to them.

    python tests/golden/make_golden.py [fixture ...]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import cic  # noqa: E402
from oracle.fft import pfft, pifft  # noqa: E402
from oracle.ldl import LDLOracle  # noqa: E402

NM = (16, 12, 8)
BOX = (40.0, 30.0, 10.0)


def cic_inputs(dt):
    rng = np.random.default_rng(2024)
    pos = rng.uniform(-0.5, 1.5, (2000, 3)) * np.asarray(BOX)
    pos[:6] = [[0.0, 0.0, 0.0], list(BOX), [-1e-10, 5e-9, -3e-12], [BOX[0] / NM[0] * 3, BOX[1] / 2, -BOX[2]],
               [BOX[0] - 1e-7, BOX[1] - 1e-6, BOX[2] - 1e-7], [2.5 * BOX[0], -3.25 * BOX[1], 1e3 * BOX[2]]]
    mass = rng.uniform(0.5, 1.5, len(pos))
    mass3 = rng.standard_normal((len(pos), 3))
    field = rng.standard_normal(NM)
    field3 = rng.standard_normal((3,) + NM)
    return pos.astype(dt), mass.astype(dt), mass3.astype(dt), field.astype(dt), field3.astype(dt)


def make_cic(dt, name):
    pos, mass, mass3, field, field3 = cic_inputs(dt)
    pm = cic.box_to_mesh(pos, BOX, NM)
    out = dict(pos=pos, mass=mass, mass3=mass3, field=field, field3=field3, box=np.asarray(BOX),
               nmesh=np.asarray(NM), mesh_pos=pm, keys=cic.cell_keys(pm, NM), paint=cic.paint(pm, mass, NM),
               paint3d=cic.paint3d(pm, mass3, NM), readout3d=cic.readout3d(pm, field3, NM, BOX, False),
               readout3d_vjp=cic.readout3d(pm, field, NM, BOX, True))
    for d in (-1, 0, 1, 2):
        out[f"readout_{d + 1}"] = cic.readout(pm, field, NM, BOX, d)
    np.savez_compressed(HERE / name, **out)


def make_fft():
    rng = np.random.default_rng(7)
    shape = (8, 6, 10)
    x = rng.standard_normal(shape)
    y = rng.standard_normal((8, 6, 6)) + 1j * rng.standard_normal((8, 6, 6))
    np.savez_compressed(HERE / "fft.npz", x=x, X=pfft(x), y=y, yinv=pifft(y, shape))


def make_ldl():
    from jerald_gb300 import synth
    n, box = 16, 100.0
    X = synth.zeldovich(n, box, 0.5, seed=3, dtype=np.float32).astype(np.float64)
    p = synth.default_params(2)
    o = LDLOracle((n, n, n), box, kind="sm", L1=True)
    o.forward(p, X, np.ones((n, n, n)), 2)
    tgt = (o.cache["F"] * synth.lognormal_noise((n, n, n), 0.1, 4)).astype(np.float32).astype(np.float64)
    loss, g_ref = o.loss_and_grad(p, X, tgt, 2, mode="reference")
    g_true = o.backward("true")
    od = LDLOracle((n, n, n), box, kind="dm", L1=False)
    loss_dm, g_dm = od.loss_and_grad(p[:10], X, np.ones((n, n, n)), 2, mode="true")
    np.savez_compressed(HERE / "ldl_sm16.npz", X=X, params=p, target=tgt, box=box, n=n, loss=loss,
                        grad_reference=g_ref, grad_true=g_true, loss_dm=loss_dm, grad_dm_true=g_dm)


def make_losstest():
    # inputs of the reference's losstest.py: 20^3 mesh, box 200, seed 83
    ng = 20
    rs = np.random.RandomState(83)
    pos = rs.rand(ng ** 3, 3) * 200
    pos = pos + (10 * np.cos(np.linalg.norm(pos, axis=1) / 19)).reshape(-1, 1)
    param = np.array([.1, .5, 1., 8., 0.] * 2 + [1., 1., 0.])
    target = rs.rand(ng, ng, ng)
    maskv = rs.randint(0, 2, target.shape).astype(np.float64)
    o = LDLOracle((ng,) * 3, 200.0, kind="sm", L1=True)
    loss = o.forward(param, pos, target, 2, mask=np.ones_like(target))
    grad = o.backward("reference")
    lossv = o.forward(param, pos, target, 2, mask=maskv)
    np.savez_compressed(HERE / "losstest20.npz", pos=pos, params=param, target=target, maskvalid=maskv,
                        loss=loss, lossv=lossv, grad=grad)


def hi_fd_grad(n, box, p, X, tgt, sm):
    """Central differences of the oracle's HI loss (L2), step 1e-4 max(|p|, 1)."""
    from oracle.ldl import model_loss
    g = np.empty(len(p))
    for i in range(len(p)):
        h = 1e-4 * max(abs(p[i]), 1.0)
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = model_loss((n,) * 3, box, "HI", pp, X, tgt, 2, starmap=sm, L1=False)[0]
        lm = model_loss((n,) * 3, box, "HI", pm, X, tgt, 2, starmap=sm, L1=False)[0]
        g[i] = (lp - lm) / (2 * h)
    return g


def make_ldl_hi():
    # the HI kind (model.py:213-247, 313-336): a sparse star map, a uniform target
    from jerald_gb300 import synth
    from oracle.ldl import model_loss
    n, box = 16, 100.0
    X = synth.zeldovich(n, box, 0.5, seed=5, dtype=np.float32).astype(np.float64)
    sm = synth.star_map(n, box, 6).astype(np.float64)
    tgt = np.random.default_rng(7).uniform(0.5, 1.5, (n, n, n))
    p = np.asarray(synth.default_params_hi(2), dtype=np.float64)
    loss_l1 = model_loss((n,) * 3, box, "HI", p, X, tgt, 2, starmap=sm, L1=True)[0]
    loss_l2 = model_loss((n,) * 3, box, "HI", p, X, tgt, 2, starmap=sm, L1=False)[0]
    np.savez_compressed(HERE / "ldl_hi16.npz", X=X, params=p, starmap=sm, target=tgt, box=box, n=n,
                        loss_l1=loss_l1, loss_l2=loss_l2, grad_l2_fd=hi_fd_grad(n, box, p, X, tgt, sm))


MAKERS = {
    "cic_f32": lambda: make_cic(np.float32, "cic_f32.npz"),
    "cic_f64": lambda: make_cic(np.float64, "cic_f64.npz"),
    "fft": make_fft,
    "ldl_sm16": make_ldl,
    "losstest20": make_losstest,
    "ldl_hi16": make_ldl_hi,
}

if __name__ == "__main__":
    # python tests/golden/make_golden.py [fixture ...]   (default: all)
    for name in sys.argv[1:] or MAKERS:
        MAKERS[name]()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)
