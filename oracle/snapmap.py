"""Oracle (test infrastructure only): CPU restatement of makemap's per-particle
steps and paint (JERALD/snaputils.py:253-406) with NumPy's own promotion
rules, for checking the GPU snapshot ingestion.  Not part of the product.

Parity: the reference's makemap cannot run here (h5py, bigfile and mpi4py
are absent and there is no snapshot); this follows its source line by line:
  weights    snaputils.py:360-376 (float32 fields, float64 coefficients;
             "Mstar", for which the reference defines no weight, uses the
             stellar Masses)
  positions  snaputils.py:378-380: pos /= 1000. in float32, then
             pos %= BoxSize against the float64 BoxSize
  dm mass    snaputils.py:383-385: prod(Nmesh) / total particle count
  paint      pm.paint -> the CIC oracle with the box prelude
"""
from __future__ import annotations

import numpy as np

from . import cic


def coefficients(redshift, BoxSize, Nmesh, h=0.678, XH=0.76):
    """snaputils.py:340-355 (a, coeff1, coeff2)."""
    a = 1 / (1 + np.float64(redshift))
    BoxSize = np.asarray(BoxSize, dtype=np.float64)
    Nmesh = np.asarray(Nmesh, dtype=np.int64)
    coeff1 = 4.0475e-07 * h ** 2 / a ** 3 * XH / BoxSize.prod() * Nmesh.prod()
    return a, coeff1, 323.06014


def weights(kind, f, a, coeff1, coeff2, XH=0.76):
    """snaputils.py:360-376 on float32 field arrays (float64 where NumPy
    promotes)."""
    M = f.get("Masses")
    Xe = f.get("ElectronAbundance")
    if kind == "ne":
        return coeff1 * M * Xe
    if kind == "nT":
        return coeff1 * M * Xe * coeff2 * f["InternalEnergy"] / (1 + 3 * XH + 4 * XH * Xe)
    if kind == "nHI":
        return coeff1 * M * f["NeutralHydrogenAbundance"]
    if kind == "neVz":
        return coeff1 * M * Xe * f["Velocities"] * a ** 0.5
    if kind == "MstarVz":
        return M * f["Velocities"] * a ** 0.5
    if kind == "XHI":
        return f["NeutralHydrogenAbundance"]
    if kind == "Mstar":
        return M
    raise ValueError(kind)


def positions(coords_kpc, BoxSize):
    """snaputils.py:378-380."""
    pos = np.array(coords_kpc, dtype=np.float32)
    pos /= 1000.
    pos %= np.asarray(BoxSize, dtype=np.float64)
    return pos


def makemap(fields, kind, Nmesh, BoxSize, redshift, h=0.678, XH=0.76):
    """Whole-snapshot map (float64 accumulation of the float32 CIC weights)."""
    a, c1, c2 = coefficients(redshift, BoxSize, Nmesh, h, XH)
    pos = positions(fields["Coordinates"], BoxSize)
    nm = tuple(int(v) for v in np.broadcast_to(np.asarray(Nmesh), (3,)))
    box = tuple(float(v) for v in np.broadcast_to(np.asarray(BoxSize, dtype=np.float64), (3,)))
    if kind == "dm":
        m = np.full(len(pos), np.float32(1.0 * np.prod(np.asarray(nm, dtype=np.int64)) / len(pos)))
    else:
        m = np.asarray(weights(kind, fields, a, c1, c2, XH)).astype(np.float32)
    q = cic.box_to_mesh(pos, np.asarray(box, dtype=np.float32), nm)
    return cic.paint(q.astype(np.float64), m.astype(np.float64), nm)
