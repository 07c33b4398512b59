"""Mesh files in the bigfile directory layout, without the bigfile module.

Restates maputils.savefield / loadfield (JERALD/maputils.py:26-77), which
store a painted map as the block "Field" of a bigfile with the attributes
ndarray.shape, BoxSize and Nmesh.  The bigfile module is not needed: this
module writes and reads its on-disk layout directly, as the bigfile project
documents it:

    <file>/                      the file: a directory
    <file>/<block>/header        "DTYPE: <f4", "NMEMB: 1", "NFILE: n", then
                                 one line per data file:
                                 "%06X: <items> : <cksum> : <sysvsum>"
    <file>/<block>/attr-v2       one attribute per line:
                                 "<name> <dtype> <nmemb> <hex bytes> #HUMANE [ ... ]"
    <file>/<block>/000000 ...    the items, row-major, split over n files

cksum is the byte sum modulo 2^32 of a data file and sysvsum its System V
fold ((s & 0xffff) + (s >> 16), folded once more), both written for
bigfile's readers; they are checked on load when asked.  Neither the bigfile
module nor a file written by it exists in this environment, so
compatibility with files the module itself wrote is not verified here; a
mismatch would show up as a header or attribute line this reader rejects.
"""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np

__all__ = ["savefield", "loadfield", "write_block", "read_block", "read_attrs", "sysv_checksums"]


def sysv_checksums(buf) -> tuple[int, int]:
    """(byte sum modulo 2^32, System V sum) of a byte buffer."""
    b = np.frombuffer(memoryview(buf).cast("B"), dtype=np.uint8)
    s = int(b.sum(dtype=np.uint64)) & 0xFFFFFFFF
    r = (s & 0xFFFF) + (s >> 16)
    return s, (r & 0xFFFF) + (r >> 16)


def _dtype_str(dt: np.dtype) -> str:
    dt = np.dtype(dt)
    if dt.kind == "S":
        return "|S1"
    return dt.newbyteorder("<").str if dt.byteorder in "=|" and dt.itemsize > 1 else dt.str


def _attr_line(name: str, value) -> str:
    if isinstance(value, str):
        raw = np.frombuffer(value.encode(), dtype="S1")
        human = value
    else:
        raw = np.atleast_1d(np.asarray(value))
        if raw.dtype.kind in "iu":
            raw = raw.astype("<i8")
        elif raw.dtype.kind == "f":
            raw = raw.astype("<f8")
        human = " ".join(repr(v.item()) for v in raw)
    return f"{name} {_dtype_str(raw.dtype)} {raw.size} {raw.tobytes().hex()} #HUMANE [ {human} ]\n"


def write_block(root, block: str, data: np.ndarray, attrs: dict | None = None, nfile: int = 1) -> Path:
    """Writes a flat array as block `block` of the file directory `root`."""
    data = np.ascontiguousarray(data).reshape(-1)
    dt = data.dtype.newbyteorder("<") if data.dtype.byteorder == ">" else data.dtype
    data = data.astype(dt, copy=False)
    d = Path(root) / block
    d.mkdir(parents=True, exist_ok=True)
    size = data.size
    nfile = max(1, int(nfile))
    lines = [f"DTYPE: {_dtype_str(data.dtype)}\n", "NMEMB: 1\n", f"NFILE: {nfile}\n"]
    for i in range(nfile):
        lo, hi = size * i // nfile, size * (i + 1) // nfile
        part = data[lo:hi]
        (d / f"{i:06X}").write_bytes(part.tobytes())
        ck, sv = sysv_checksums(part.tobytes())
        lines.append(f"{i:06X}: {hi - lo} : {ck} : {sv}\n")
    (d / "header").write_text("".join(lines))
    (d / "attr-v2").write_text("".join(_attr_line(k, v) for k, v in (attrs or {}).items()))
    return d


def _parse_header(d: Path):
    dtype, nmemb, nfile, files = None, 1, None, []
    for line in (d / "header").read_text().splitlines():
        line = line.strip()
        if not line:
            continue
        key, _, rest = line.partition(":")
        if key == "DTYPE":
            dtype = np.dtype(rest.strip())
        elif key == "NMEMB":
            nmemb = int(rest)
        elif key == "NFILE":
            nfile = int(rest)
        else:
            fields = [f.strip() for f in rest.split(":")]
            if len(fields) != 3:
                raise ValueError(f"{d / 'header'}: unexpected line {line!r}")
            files.append((int(key, 16), int(fields[0]), int(fields[1]), int(fields[2])))
    if dtype is None or nfile is None or len(files) != nfile:
        raise ValueError(f"{d / 'header'}: incomplete bigfile block header")
    return dtype, nmemb, sorted(files)


def read_attrs(root, block: str) -> dict:
    """Attributes of a block (attr-v2 lines), as numpy arrays or strings."""
    p = Path(root) / block / "attr-v2"
    out = {}
    if not p.exists():
        return out
    for line in p.read_text().splitlines():
        line = line.split("#HUMANE")[0].strip()
        if not line:
            continue
        name, dt, nmemb, hexdata = line.split()
        arr = np.frombuffer(bytes.fromhex(hexdata), dtype=np.dtype(dt))
        if arr.size != int(nmemb):
            raise ValueError(f"{p}: attribute {name} holds {arr.size} items, header says {nmemb}")
        out[name] = arr.tobytes().decode() if arr.dtype.kind == "S" else arr.copy()
    return out


def read_block(root, block: str, verify: bool = False) -> np.ndarray:
    """The flat array of a block (all data files concatenated)."""
    d = Path(root) / block
    dtype, nmemb, files = _parse_header(d)
    parts = []
    for idx, items, ck, sv in files:
        a = np.fromfile(d / f"{idx:06X}", dtype=dtype, count=items * nmemb)
        if a.size != items * nmemb:
            raise ValueError(f"{d / f'{idx:06X}'}: {a.size} items, header says {items * nmemb}")
        if verify and sysv_checksums(a.tobytes()) != (ck, sv):
            raise ValueError(f"{d / f'{idx:06X}'}: checksum mismatch")
        parts.append(a)
    out = np.concatenate(parts) if parts else np.zeros(0, dtype=dtype)
    return out.reshape(-1, nmemb) if nmemb > 1 else out


def savefield(data, filename, pm, nfile: int = 1) -> Path:
    """maputils.savefield (JERALD/maputils.py:26-41): the map, flattened in C
    order, as block "Field" with the attributes ndarray.shape (= Nmesh),
    BoxSize and Nmesh.  `data` may be a numpy array or a tensor."""
    if hasattr(data, "detach"):
        data = data.detach().cpu().numpy()
    data = np.asarray(data)
    Nmesh = np.asarray(pm.Nmesh, dtype=np.int64).reshape(-1)
    attrs = {"ndarray.shape": Nmesh, "BoxSize": np.asarray(pm.BoxSize, dtype=np.float64).reshape(-1),
             "Nmesh": Nmesh}
    os.makedirs(filename, exist_ok=True)
    return write_block(filename, "Field", data, attrs, nfile)


def loadfield(path, comm=None, local: bool = False, pm=None, verify: bool = False):
    """maputils.loadfield (JERALD/maputils.py:45-77): (map, Nmesh, BoxSize)
    from block "Field"; float64 items stay float64, others come back as
    float32.  With local=True and a mesh `pm`, the slab [fftss[0], fftss[1])
    of its decomposition; at world size one that is the whole map, which is
    also what local=True without `pm` returns."""
    attrs = {k: np.squeeze(v) if not isinstance(v, str) else v for k, v in read_attrs(path, "Field").items()}
    flat = read_block(path, "Field", verify)
    dtype = np.float64 if flat.dtype.itemsize == 8 else np.float32
    Nmesh = attrs["Nmesh"]
    out = flat.astype(dtype, copy=False).reshape(tuple(int(v) for v in np.atleast_1d(Nmesh)))
    if local and pm is not None:
        return out[pm.fftss[0]:pm.fftss[1], :, :], Nmesh, attrs["BoxSize"]
    return out, Nmesh, attrs["BoxSize"]
