"""ORACLE — test infrastructure only.  numpy wrappers over libjldref.so, the
reference's own CIC loops (lib/parops_fast.h:354-481, 484-567, 616-857 of
maurorigo/JERALD) compiled by build.build_ref() with a world-size-one MPI
stand-in.  Same calling convention as cic.py: positions in mesh units,
row-major arrays, float32 with int32 mesh sizes and float64 with int64
(lib/cpu.cc:276-285).

available() is False where the reference checkout is absent and no library
was built (the GPU hosts): tests that need it skip there, and the committed
hash fixtures (tests/golden/ref_hashes.json) carry the reference's outputs
instead.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .build import build_ref

_lib = None


def available() -> bool:
    try:
        return build_ref() is not None
    except RuntimeError:
        return False


def _load():
    global _lib
    if _lib is None:
        path = build_ref()
        if path is None:
            raise RuntimeError("the reference's CIC library is not built (no reference checkout)")
        _lib = ct.CDLL(str(path))
        for name in ("ppaint", "preadout", "ppaint3d", "preadout3d"):
            for sfx in ("f32", "f64"):
                getattr(_lib, f"jref_{name}_{sfx}").restype = None
    return _lib


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def _sfx(a):
    if a.dtype == np.float32:
        return "f32", np.int32
    if a.dtype == np.float64:
        return "f64", np.int64
    raise TypeError(f"unsupported dtype {a.dtype}")


def _nm(nmesh, it):
    return np.ascontiguousarray(np.asarray(nmesh, dtype=it).reshape(3))


def paint(pos_mesh, mass, nmesh):
    """ppaint -> lpaint at world size one: (Nx, Ny, Nz) mesh."""
    pos = np.ascontiguousarray(pos_mesh)
    sfx, it = _sfx(pos)
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, dtype=pos.dtype), (len(pos),)))
    nm = _nm(nmesh, it)
    out = np.empty(tuple(int(v) for v in nm), dtype=pos.dtype)
    getattr(_load(), f"jref_ppaint_{sfx}")(_p(pos), ct.c_int64(len(pos)), _p(m), _p(nm), _p(out))
    return out


def readout(pos_mesh, field, nmesh, box, vjpdim=-1):
    """preadout -> lreadout (after a ppaint on the same positions)."""
    pos = np.ascontiguousarray(pos_mesh)
    sfx, it = _sfx(pos)
    f = np.ascontiguousarray(field, dtype=pos.dtype)
    nm = _nm(nmesh, it)
    b = np.ascontiguousarray(np.asarray(box, dtype=pos.dtype).reshape(3))
    out = np.empty(len(pos), dtype=pos.dtype)
    getattr(_load(), f"jref_preadout_{sfx}")(_p(pos), ct.c_int64(len(pos)), _p(f), _p(nm), _p(b),
                                             ct.c_int32(int(vjpdim)), _p(out))
    return out


def paint3d(pos_mesh, mass3, nmesh):
    """ppaint3D -> lpaint3D: mass (N, 3) row-major -> (3, Nx, Ny, Nz)."""
    pos = np.ascontiguousarray(pos_mesh)
    sfx, it = _sfx(pos)
    m = np.ascontiguousarray(np.asarray(mass3, dtype=pos.dtype).reshape(len(pos), 3))
    nm = _nm(nmesh, it)
    out = np.empty((3,) + tuple(int(v) for v in nm), dtype=pos.dtype)
    getattr(_load(), f"jref_ppaint3d_{sfx}")(_p(pos), ct.c_int64(len(pos)), _p(m), _p(nm), _p(out))
    return out


def readout3d(pos_mesh, field, nmesh, box, vjp):
    """preadout3D -> lreadout3D: (N, 3) gathers of three fields, or the
    weight gradient of one field (vjp)."""
    pos = np.ascontiguousarray(pos_mesh)
    sfx, it = _sfx(pos)
    f = np.ascontiguousarray(field, dtype=pos.dtype)
    nm = _nm(nmesh, it)
    b = np.ascontiguousarray(np.asarray(box, dtype=pos.dtype).reshape(3))
    out = np.empty((len(pos), 3), dtype=pos.dtype)
    getattr(_load(), f"jref_preadout3d_{sfx}")(_p(pos), ct.c_int64(len(pos)), _p(f), _p(nm), _p(b),
                                               ct.c_int32(1 if vjp else 0), _p(out))
    return out
