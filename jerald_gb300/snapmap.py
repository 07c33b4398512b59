"""Snapshot-map ingestion on the GPU: makemap (JERALD/snaputils.py:253-406).

The reference reads the particle fields a map kind needs from Gadget HDF5
snapshot files (readfields, snaputils.py:124-249), turns them into paint
weights (snaputils.py:338-376), converts positions from kpc/h to Mpc/h and
wraps them (snaputils.py:378-380), paints the map (snaputils.py:385-387) and
saves it as a bigfile "Field" (maputils.savefield).

Here the snapshot streams through the GPU in chunks: each chunk is copied
to the device (two staging slots, the copy of chunk i+1 overlapping the
work on chunk i), one CUDA kernel computes its wrapped positions and
weights (jld_snap_prep_f32) and the accumulating paint adds it to the map
(jld_ppaint_box_acc_f32).  The map never leaves the device until the end.

Sources of chunks:
  * HDF5Snapshot reads the reference's snapshot files (snapshot path
    resolution of snaputils.fname, the header, PartType<k>/<field>
    datasets).  It needs h5py, which this environment does not have: the
    tests run its logic against an in-memory stand-in, not real files.
  * ArraySnapshot wraps in-memory arrays (any other reader, synthetic data).
Positions and fields are float32 (the reference's default f32=True).
"""
from __future__ import annotations

import ctypes as ct
import os
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib

__all__ = ["KINDS", "fname", "mapPartNum", "map_fields", "map_coefficients", "Header", "HDF5Snapshot",
           "ArraySnapshot", "makemap"]

KINDS = {"dm": 0, "Mstar": 1, "ne": 2, "nT": 3, "nHI": 4, "neVz": 5, "MstarVz": 6, "XHI": 7}


def fname(path: str) -> str:
    """First file of a snapshot given a Pylians-style prefix (snaputils.py:30-48)."""
    if os.path.exists(path):
        if path[-4:] == "hdf5":
            return path
        raise ValueError("Unsupported file format")
    if os.path.exists(path + ".0"):
        raise ValueError("Binary type not supported")
    if os.path.exists(path + ".hdf5"):
        if path[-2:] != ".0":
            parts = path.split(".")[:-1]
            parts.append(".0")
            path = "".join(parts)
        return path + ".hdf5"
    if os.path.exists(path + ".0.hdf5"):
        return path + ".0.hdf5"
    raise FileNotFoundError("File not found")


def mapPartNum(kind: str) -> int:
    """Particle type of a map kind (snaputils.py:51-63): 0 gas, 1 dm, 4 stars."""
    if kind == "dm":
        return 1
    if kind in ("Mstar", "MstarVz"):
        return 4
    if kind in ("ne", "nT", "nHI", "neVz", "XHI"):
        return 0
    raise ValueError(f"Unkown required map type {kind}")


def map_fields(kind: str) -> tuple[list[str], list]:
    """(fields, mdi) that makemap reads for a kind (snaputils.py:281-318);
    mdi[i] = 2 selects vz of the 3-vector Velocities."""
    extra = {"dm": [], "Mstar": ["Masses"], "ne": ["Masses", "ElectronAbundance"],
             "nT": ["ElectronAbundance", "InternalEnergy", "Masses"],
             "nHI": ["Masses", "NeutralHydrogenAbundance"],
             "neVz": ["Masses", "ElectronAbundance", "Velocities"], "MstarVz": ["Masses", "Velocities"],
             "XHI": ["NeutralHydrogenAbundance"]}
    if kind not in extra:
        raise ValueError(f"Unknown kind to import {kind}")
    fields = ["Coordinates"] + extra[kind]
    return fields, [2 if f == "Velocities" else None for f in fields]


def map_coefficients(redshift: float, BoxSize, Nmesh, h: float = 0.678, XH: float = 0.76):
    """(a, coeff1, coeff2) of snaputils.py:340-355, in float64 as there."""
    a = 1 / (1 + redshift)
    BoxSize = np.asarray(BoxSize, dtype=np.float64)
    Nmesh = np.asarray(Nmesh, dtype=np.int64)
    coeff1 = 4.0475e-07 * h ** 2 / a ** 3 * XH / BoxSize.prod() * Nmesh.prod()
    coeff2 = 323.06014
    return a, float(coeff1), coeff2


class Header:
    """Header attributes of an HDF5 snapshot (snaputils.py:68-89); needs h5py."""

    def __init__(self, snapshot: str):
        import h5py
        with h5py.File(fname(snapshot), "r") as f:
            at = f["Header"].attrs
            self.time = at["Time"]
            self.redshift = at["Redshift"]
            self.boxsize = at["BoxSize"]
            self.filenum = at["NumFilesPerSnapshot"]
            self.omega_m = at["Omega0"]
            self.omega_l = at["OmegaLambda"]
            self.hubble = at["HubbleParam"]
            self.massarr = at["MassTable"]
            self.npart = at["NumPart_ThisFile"]
            self.nall = at["NumPart_Total"]
            self.cooling = at["Flag_Cooling"]
        self.Hubble = 100.0 * np.sqrt(self.omega_m * (1.0 + self.redshift) ** 3 + self.omega_l)


class HDF5Snapshot:
    """Chunks of a Gadget HDF5 snapshot (every file in turn, as readfields
    walks them at world size one).  Needs h5py."""

    def __init__(self, path: str):
        self.filename = fname(path)
        self.header = Header(self.filename)
        self.redshift = float(self.header.redshift)
        self.nall = np.asarray(self.header.nall, dtype=np.int64)

    def chunks(self, ptNum: int, fields, mdi, max_particles: int):
        import h5py
        name = f"PartType{ptNum}"
        for i in range(int(self.header.filenum)):
            with h5py.File(self.filename[:-6] + str(i) + ".hdf5", "r") as f:
                if name not in f:
                    continue
                n = int(f["Header"].attrs["NumPart_ThisFile"][ptNum])
                for lo in range(0, n, max_particles):
                    hi = min(n, lo + max_particles)
                    out = {}
                    for fld, m in zip(fields, mdi):
                        if fld not in f[name]:
                            raise KeyError(f"Particle type {ptNum} does not have field {fld}")
                        d = f[name][fld]
                        out[fld] = np.asarray(d[lo:hi] if m is None else d[lo:hi, m], dtype=np.float32)
                    yield out


@dataclass
class ArraySnapshot:
    """In-memory snapshot: redshift and, per particle type, a dict of field
    arrays (Coordinates (N, 3) in kpc/h, Velocities (N, 3) or vz (N,), ...)."""
    redshift: float
    parts: dict = field(default_factory=dict)

    @property
    def nall(self):
        out = np.zeros(6, dtype=np.int64)
        for t, d in self.parts.items():
            out[t] = len(d["Coordinates"])
        return out

    def chunks(self, ptNum: int, fields, mdi, max_particles: int):
        d = self.parts.get(ptNum, {})
        n = len(d["Coordinates"]) if d else 0
        for lo in range(0, n, max_particles):
            hi = min(n, lo + max_particles)
            out = {}
            for fld, m in zip(fields, mdi):
                if fld not in d:
                    raise KeyError(f"Particle type {ptNum} does not have field {fld}")
                a = np.asarray(d[fld][lo:hi])
                out[fld] = a[:, m] if (m is not None and a.ndim == 2) else a
            yield out


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class _Slot:
    """Pinned staging and device buffers for one chunk of up to cap particles."""

    def __init__(self, cap: int, names, device):
        self.host = {k: torch.empty((cap * (3 if k == "Coordinates" else 1),), dtype=torch.float32,
                                    pin_memory=True) for k in names}
        self.dev = {k: torch.empty_like(v, device=device) for k, v in self.host.items()}
        self.pos = torch.empty((cap * 3,), dtype=torch.float32, device=device)
        self.w = torch.empty((cap,), dtype=torch.float32, device=device)
        self.copied = torch.cuda.Event()
        self.used = torch.cuda.Event()


def makemap(path, kind, pm, f32=True, local=True, save=True, outpath=None, verbose=2, chunk=1 << 23,
            return_tensor=False, **kwargs):
    """snaputils.makemap on the GPU.  `path` is a snapshot prefix (read with
    HDF5Snapshot) or any object with redshift, nall and
    chunks(ptNum, fields, mdi, max_particles) (ArraySnapshot).  `pm` gives
    Nmesh, BoxSize and the device.  kwargs: h (0.678), XH (0.76).  Returns
    the map (numpy, or the device tensor with return_tensor=True).

    Differences from the reference: kind "Mstar" paints the stellar Masses
    (the reference reads them but defines no weight for it,
    snaputils.py:360-376, and stops with an unbound name); only float32
    snapshots (f32=True)."""
    if not f32:
        raise NotImplementedError("makemap on the GPU paints float32 snapshots (f32=True)")
    if kind not in KINDS:
        raise ValueError(f"Unknown kind to import {kind}")
    snap = HDF5Snapshot(path) if isinstance(path, (str, os.PathLike)) else path
    h = kwargs.get("h", 0.678)
    XH = kwargs.get("XH", 0.76)
    Nmesh = np.asarray(pm.Nmesh, dtype=np.int64).reshape(-1)
    BoxSize = np.asarray(pm.BoxSize, dtype=np.float64).reshape(-1)
    a, c1, c2 = map_coefficients(float(snap.redshift), BoxSize, Nmesh, h, XH)
    sqa = a ** 0.5
    ptNum = mapPartNum(kind)
    fields, mdi = map_fields(kind)
    ntot = int(np.asarray(snap.nall)[ptNum])
    if ntot == 0:
        raise ValueError(f"No particles of type {ptNum} in the snapshot")
    mscalar = 1.0 * Nmesh.prod() / ntot if kind == "dm" else 0.0
    dev = torch.device(getattr(pm, "device", "cuda"))
    if dev.type != "cuda":
        raise RuntimeError("makemap runs on a CUDA device")
    nm = tuple(int(v) for v in Nmesh)
    mesh = torch.zeros(nm, dtype=torch.float32, device=dev)
    box64 = np.ascontiguousarray(BoxSize, dtype=np.float64)
    box32 = np.ascontiguousarray(BoxSize, dtype=np.float32)
    names = ["Coordinates"] + [f for f in fields[1:]]
    slots = [_Slot(chunk, names, dev) for _ in range(2)]
    comp = torch.cuda.current_stream(dev)
    copy = torch.cuda.Stream(dev)
    P = lambda t: ct.c_void_p(t.data_ptr())  # noqa: E731
    for s in slots:
        s.used.record(comp)
    for i, ch in enumerate(snap.chunks(ptNum, fields, mdi, chunk)):
        s = slots[i % 2]
        n = int(ch["Coordinates"].shape[0])
        if n == 0:
            continue
        s.used.synchronize()                       # the GPU is done with this slot's buffers
        for k in names:
            v = ch[k]
            if isinstance(v, torch.Tensor):
                v = v.reshape(-1)
            else:
                v = torch.from_numpy(_f32(v).reshape(-1))
            s.host[k][:v.numel()].copy_(v)         # multi-threaded host copy into pinned staging
        with torch.cuda.stream(copy):
            for k in names:
                m = n * (3 if k == "Coordinates" else 1)
                s.dev[k][:m].copy_(s.host[k][:m], non_blocking=True)
            s.copied.record(copy)
        comp.wait_event(s.copied)
        sp = ct.c_void_p(comp.cuda_stream)
        fp = {k: (P(s.dev[k]) if k in s.dev else ct.c_void_p(None)) for k in
              ("Masses", "ElectronAbundance", "InternalEnergy", "NeutralHydrogenAbundance", "Velocities")}
        _lib.call("jld_snap_prep_f32", sp, P(s.dev["Coordinates"]), n, ct.c_float(1000.0),
                  box64.ctypes.data_as(ct.c_void_p), KINDS[kind], fp["Masses"], fp["ElectronAbundance"],
                  fp["InternalEnergy"], fp["NeutralHydrogenAbundance"], fp["Velocities"], 1, c1, c2, XH, sqa,
                  P(s.pos), P(s.w))
        wp = ct.c_void_p(None) if kind == "dm" else P(s.w)
        _lib.call("jld_ppaint_box_acc_f32", sp, P(s.pos), n, wp, ct.c_float(mscalar), *nm,
                  box32.ctypes.data_as(ct.c_void_p), P(mesh))
        s.used.record(comp)
    comp.synchronize()
    if save:
        from .fieldio import savefield
        if not outpath:
            outpath = "/".join(fname(path).split("/")[:-1]) if isinstance(path, (str, os.PathLike)) else "."
        savefield(mesh, f"{outpath}/{kind}map_Nmesh{nm[0]}", pm)
    if return_tensor:
        return mesh
    return mesh.cpu().numpy()
