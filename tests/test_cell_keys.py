"""Cell keys of the fused step's division-free prelude against the
reference's, for every float32 position.

The reference's mesh coordinate is q = (x mod L) / (L/N) in float32
(jaxpops_bind.py:163-164), its cell key int(q) mod N (lib/parops_fast.h:91-93).
The fused step's kernels (box_to_mesh_fast in jerald_gb300/csrc/common.cuh)
take the same remainder and multiply by N/L instead; both L/N and N/L are
rounded to float32 on the host (make_src in csrc/cic.cu, BoxGeom in
csrc/ldl.cu). The remainder branches are the same code in both preludes, so
the two keys can differ only through the final division against the
multiplication; these tests enumerate every float32 remainder r that can
give a key other than 0 (r in [cell/2, L]: below half a cell both q round
to at most 0.5) and compare, in numpy float32 arithmetic (IEEE round to
nearest, as on the device).

* Geometries with cell = 25/16 (100 per 64 cells: the 64^3, 256^3, 512^3
  and 1024^3 workloads): no remainder gets another key, so the fused step's
  keys are the reference's for every position, displaced ones included.
* A geometry whose L/N is inexact: keys differ only for remainders on a cell
  boundary (one of the two q is an integer), by one cell, and every CIC
  weight of the axis moves by at most one ulp of q, so painted and gathered
  values stay continuous.
"""
import numpy as np
import pytest

f32 = np.float32


def _bits(x):
    return int(np.array([x], f32).view(np.uint32)[0])


def _remainders(L, n, chunk=1 << 24):
    """Every float32 in [cell/2, L], in chunks, with the host's cell and N/L."""
    cell = f32(f32(L) / f32(n))
    inv = f32(f32(n) / f32(L))
    lo, hi = _bits(cell / f32(2)), _bits(f32(L))
    for s in range(lo, hi + 1, chunk):
        yield np.arange(s, min(s + chunk, hi + 1), dtype=np.uint32).view(f32), cell, inv


def _axis_weights(k, d, m):
    """CIC weights of one axis on the cells m, m+1, m+2 (1-d on k, d on k+1)."""
    return [np.where(k == m + c, 1 - d, 0) + np.where(k + 1 == m + c, d, 0) for c in range(3)]


def test_keys_equal_for_every_position():
    # The four workloads share the cell and N/L, and the remainders of the
    # smaller boxes are a subset of 1600's: one exhaustive pass covers them.
    for L, n in [(100.0, 64), (400.0, 256), (800.0, 512), (1600.0, 1024)]:
        assert (f32(f32(L) / f32(n)), f32(f32(n) / f32(L))) == (f32(1.5625), f32(0.64))
    count = 0
    for r, cell, inv in _remainders(1600.0, 1024):
        count += len(r)
        assert np.array_equal(np.floor(r / cell), np.floor(r * inv))
    assert count > 9e7


def test_inexact_cell_keys_move_only_on_boundaries():
    L, n = 1000.0, 384  # L/N = 2.6041667 and N/L = 0.384 are both rounded
    flips = 0
    for r, cell, inv in _remainders(L, n):
        qr, qf = r / cell, r * inv
        kr, kf = np.floor(qr), np.floor(qf)
        dr, df = qr - kr, qf - kf
        fl = kr != kf
        flips += int(fl.sum())
        assert (np.abs(kf - kr) <= 1).all()
        assert ((dr[fl] == 0) | (df[fl] == 0)).all()
        m = np.minimum(kr, kf)
        ulp = np.spacing(np.maximum(qr, f32(1)))
        for a, b in zip(_axis_weights(kr, dr, m), _axis_weights(kf, df, m)):
            assert (np.abs(a - b) <= ulp).all()
    # keys differ for a few hundred of the 8e7 remainders (216 for this geometry)
    assert 0 < flips < 1000
