"""ORACLE — test infrastructure only.  numpy wrappers over liborc.so, the C
restatement of the reference's single-rank CIC loops (cic_oracle.c).

Each function takes row-major numpy arrays and returns new arrays.  dtype
float32 follows the reference's f32 build, float64 its f64 build
(lib/cpu.cc:276-291).  Parity unpinned against the reference binary (it
needs MPI and FFTW to build); pinned by the known-answer tests in tests/.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .build import build

_lib = None
_THREADS = 1


def set_threads(n: int) -> None:
    """Host threads for the particle loops (1 = the reference's serial loops,
    the default the tests use).  With n > 1 the particles are split into n
    contiguous ranges run concurrently (the C calls release the GIL): gathers
    are unchanged bit for bit; each range paints into its own mesh and the
    meshes are summed in range order, as n ranks' slabs would be, which
    changes only the summation order of the deposits."""
    global _THREADS
    _THREADS = max(1, int(n))


def _ranges(n: int):
    k = _THREADS if n >= 4096 * _THREADS else 1
    edges = np.linspace(0, n, k + 1).astype(np.int64)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:])]


def _ranges_n(n: int, k: int):
    edges = np.linspace(0, n, max(1, min(k, n)) + 1).astype(np.int64)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:])]


def _pool_map(fn, ranges):
    if len(ranges) == 1:
        return [fn(*ranges[0])]
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(len(ranges)) as ex:
        return list(ex.map(lambda r: fn(*r), ranges))


def _load():
    global _lib
    if _lib is None:
        _lib = ct.CDLL(str(build()))
        for sfx in ("f32", "f64"):
            for name in ("box_to_mesh", "cell_keys", "paint", "paint3d", "readout", "readout3d"):
                getattr(_lib, f"orc_{name}_{sfx}").restype = None
    return _lib


def _sfx(a: np.ndarray) -> str:
    if a.dtype == np.float32:
        return "f32"
    if a.dtype == np.float64:
        return "f64"
    raise TypeError(f"unsupported dtype {a.dtype}")


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def _nm(nmesh):
    return np.ascontiguousarray(np.asarray(nmesh, dtype=np.int64).reshape(3))


def box_to_mesh(pos: np.ndarray, box, nmesh) -> np.ndarray:
    """(pos % box) / (box / nmesh) in pos.dtype (jaxpops_bind.py:163-164)."""
    pos = np.ascontiguousarray(pos)
    out = np.empty_like(pos)
    b = np.ascontiguousarray(np.asarray(box, dtype=pos.dtype).reshape(3))
    nm = _nm(nmesh)
    fn = getattr(_load(), f"orc_box_to_mesh_{_sfx(pos)}")
    _pool_map(lambda a, e: fn(_p(pos[a:]), ct.c_int64(e - a), _p(b), _p(nm), _p(out[a:])), _ranges(len(pos)))
    return out


def cell_keys(pos_mesh: np.ndarray, nmesh) -> np.ndarray:
    """Flattened cell index of int(pos) % N per axis (lib/parops_fast.h:91-93)."""
    pos_mesh = np.ascontiguousarray(pos_mesh)
    keys = np.empty(len(pos_mesh), dtype=np.int64)
    nm = _nm(nmesh)
    getattr(_load(), f"orc_cell_keys_{_sfx(pos_mesh)}")(_p(pos_mesh), ct.c_int64(len(pos_mesh)), _p(nm), _p(keys))
    return keys


def paint(pos_mesh: np.ndarray, mass, nmesh) -> np.ndarray:
    """lpaint at world size one: zeroed mesh plus CIC deposits in particle order."""
    pos_mesh = np.ascontiguousarray(pos_mesh)
    dt = pos_mesh.dtype
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, dtype=dt), (len(pos_mesh),)))
    nm = _nm(nmesh)
    fn = getattr(_load(), f"orc_paint_{_sfx(pos_mesh)}")

    def part(a, b):
        out = np.empty(tuple(int(v) for v in nm), dtype=dt)
        fn(_p(pos_mesh[a:]), ct.c_int64(b - a), _p(m[a:]), _p(nm), _p(out))
        return out
    meshes = _pool_map(part, _ranges(len(pos_mesh)))
    out = meshes[0]
    if len(meshes) > 1:
        # the range meshes are summed in range order, slab by slab in parallel
        def add(a, e):
            for extra in meshes[1:]:
                out[a:e] += extra[a:e]
        _pool_map(add, [(a, e) for a, e in _ranges_n(out.shape[0], len(meshes))])
    return out


def paint3d(pos_mesh: np.ndarray, mass3: np.ndarray, nmesh) -> np.ndarray:
    """lpaint3D: mass (N,3) row-major -> (3, Nx, Ny, Nz)."""
    pos_mesh = np.ascontiguousarray(pos_mesh)
    dt = pos_mesh.dtype
    m = np.ascontiguousarray(np.asarray(mass3, dtype=dt).reshape(len(pos_mesh), 3))
    nm = _nm(nmesh)
    out = np.empty((3,) + tuple(int(v) for v in nm), dtype=dt)
    getattr(_load(), f"orc_paint3d_{_sfx(pos_mesh)}")(_p(pos_mesh), ct.c_int64(len(pos_mesh)), _p(m), _p(nm), _p(out))
    return out


def readout(pos_mesh: np.ndarray, field: np.ndarray, nmesh, box, vjpdim: int = -1) -> np.ndarray:
    """lreadout: CIC gather, or its weight derivative along vjpdim."""
    pos_mesh = np.ascontiguousarray(pos_mesh)
    dt = pos_mesh.dtype
    f = np.ascontiguousarray(field, dtype=dt)
    nm = _nm(nmesh)
    b = np.ascontiguousarray(np.asarray(box, dtype=dt).reshape(3))
    out = np.empty(len(pos_mesh), dtype=dt)
    fn = getattr(_load(), f"orc_readout_{_sfx(pos_mesh)}")
    _pool_map(lambda a, e: fn(_p(pos_mesh[a:]), ct.c_int64(e - a), _p(f), _p(nm), _p(b), ct.c_int(int(vjpdim)),
                              _p(out[a:])), _ranges(len(pos_mesh)))
    return out


def readout3d(pos_mesh: np.ndarray, field: np.ndarray, nmesh, box, vjp: bool) -> np.ndarray:
    """lreadout3D: (N,3) gathers of three fields, or the weight gradient of one."""
    pos_mesh = np.ascontiguousarray(pos_mesh)
    dt = pos_mesh.dtype
    f = np.ascontiguousarray(field, dtype=dt)
    nm = _nm(nmesh)
    b = np.ascontiguousarray(np.asarray(box, dtype=dt).reshape(3))
    out = np.empty((len(pos_mesh), 3), dtype=dt)
    fn = getattr(_load(), f"orc_readout3d_{_sfx(pos_mesh)}")
    _pool_map(lambda a, e: fn(_p(pos_mesh[a:]), ct.c_int64(e - a), _p(f), _p(nm), _p(b), ct.c_int(1 if vjp else 0),
                              _p(out[a:])), _ranges(len(pos_mesh)))
    return out
