"""ORACLE — test infrastructure only.  Seeded CIC inputs that come out the
same bits on every host, for the reference-pinned hash fixtures
(tests/golden/ref_hashes.json, made by tests/golden/make_ref_hashes.py).

Only numpy's PCG64 generator and exactly rounded arithmetic (+, -, *, /,
mod, casts) are used: no exp, log, sin or FFT, whose last bits may differ
between x86-64 and Arm builds of numpy.  The cases cover what the GPU
kernels treat differently: particles in lattice order (the paint's
neighbour pairing), dense clumps (its shared-memory window), uniform random
order, positions that round to exactly N after the float32 cast (the
reference drops the lower corner there), and a non-cubic mesh.
"""
from __future__ import annotations

import hashlib

import numpy as np

# name -> (mesh, box, dtype, kind)
CASES = {
    "uniform_20x12x8_f32": ((20, 12, 8), (200.0, 30.0, 7.5), np.float32, "uniform"),
    "uniform_20x12x8_f64": ((20, 12, 8), (200.0, 30.0, 7.5), np.float64, "uniform"),
    "uniform_64_f32": ((64, 64, 64), (100.0, 100.0, 100.0), np.float32, "uniform"),
    "uniform_64_f64": ((64, 64, 64), (100.0, 100.0, 100.0), np.float64, "uniform"),
    "clustered_64_f32": ((64, 64, 64), (100.0, 100.0, 100.0), np.float32, "clustered"),
    "clustered_64_f64": ((64, 64, 64), (100.0, 100.0, 100.0), np.float64, "clustered"),
    "clustered_256_f32": ((256, 256, 256), (400.0, 400.0, 400.0), np.float32, "clustered"),
}

SEED = 20260


def _irwin_hall(rng, shape):
    # sum of three uniforms, centred: a bell-shaped offset with unit-ish
    # width from exactly rounded operations only
    return rng.random(shape) + rng.random(shape) + rng.random(shape) - 1.5


def positions(name: str) -> np.ndarray:
    """Mesh-unit positions (N, 3) of a case, in its dtype."""
    nm, _, dt, kind = CASES[name]
    rng = np.random.default_rng([SEED, sum(map(ord, name))])
    nmf = np.asarray(nm, dtype=np.float64)
    if kind == "uniform":
        n = int(np.prod(nm))
        pos = rng.random((n, 3)) * nmf
    else:
        # lattice order (x slowest) with a jitter of up to 1.5 cells, then
        # 10 % extra particles in 200 clumps of about 0.5-cell width
        ax = [np.arange(v, dtype=np.float64) + 0.5 for v in nm]
        lat = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3)
        lat += (rng.random(lat.shape) - 0.5) * 3.0
        nh = len(lat) // 10
        centres = rng.random((200, 3)) * nmf
        which = rng.integers(0, 200, nh)
        halo = centres[np.sort(which)] + _irwin_hall(rng, (nh, 3)) * 0.5
        pos = np.concatenate([lat, halo])
        pos = np.mod(pos, nmf)
    pos = pos.astype(dt)
    # exact corners and values that round to N in float32
    tiny = np.asarray(1e-9 * nmf)
    pos[:5] = np.asarray([[0.0, 0.0, 0.0], nmf - tiny, [nmf[0] - tiny[0], 0.5, 0.25],
                          [3.0, nmf[1] / 2, 0.0], nmf / 2], dtype=np.float64).astype(dt)
    return pos


def operands(name: str):
    """(pos, mass, mass3, field, field3, mesh, box, dtype) of a case."""
    nm, box, dt, _ = CASES[name]
    pos = positions(name)
    rng = np.random.default_rng([SEED + 1, sum(map(ord, name))])
    n = len(pos)
    mass = (rng.random(n) + 0.5).astype(dt)
    mass3 = (rng.random((n, 3)) - 0.5).astype(dt)
    field = (rng.random(nm) - 0.5).astype(dt)
    field3 = (rng.random((3,) + tuple(nm)) - 0.5).astype(dt)
    return pos, mass, mass3, field, field3, nm, box, dt


def digest(a: np.ndarray) -> str:
    """sha256 of the array's bytes (C order, little-endian on every host here)."""
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def outputs(mod, name: str) -> dict:
    """Every CIC op of `mod` (oracle.cic or oracle.ref) on the case: name -> array."""
    pos, mass, mass3, field, field3, nm, box, _ = operands(name)
    out = {"paint": mod.paint(pos, mass, nm), "paint3d": mod.paint3d(pos, mass3, nm)}
    for v in (-1, 0, 1, 2):
        out[f"readout{v}"] = mod.readout(pos, field, nm, box, v)
    out["readout3d"] = mod.readout3d(pos, field3, nm, box, False)
    out["readout3d_vjp"] = mod.readout3d(pos, field, nm, box, True)
    return out
