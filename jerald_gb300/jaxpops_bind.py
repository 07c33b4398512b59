"""Drop-in mirror of the reference's primitive surface (jaxpops_bind.py) on
CUDA tensors, backed by libjld.so.

Same names, arguments, shapes and custom-VJP rules as the reference at world
size one:

    initLayout(commsize, lyidx=0)                     jaxpops_bind.py:57
    clean(lyidx=0)                                    jaxpops_bind.py:95
    ppaint(pos, mass, Nmesh, BoxSize, edges, dims, comm, lyidx=0, bwd=False)   :137
    preadout(pos, field, Nmesh, BoxSize, edges, dims, comm, lyidx=0, vjpdim=-1) :256
    ppaint3D(pos, mass, Nmesh, BoxSize, edges, dims, comm, lyidx=0)            :371
    preadout3D(pos, field, Nmesh, BoxSize, edges, dims, comm, lyidx=0, vjp=False) :472
    buildplan(Nmesh, comm)                            jaxpops_bind.py:597
    pfft(data, dims), pifft(data, dims)               jaxpops_bind.py:648, 710
    local_positions(pos, Nout, Nmesh, BoxSize, edges, commsize, commrank) :767

Differences, all deliberate:
  * Tensors are torch CUDA tensors and gradients flow through
    torch.autograd.Function objects whose backward passes apply the
    reference's rules (jaxpops_bind.py:233-249, 347-365, 569-590, 695-703,
    754-761).  torch stores the conjugate of JAX's complex cotangent, so the
    FFT rules appear conjugated: pfft's backward is pifft(g).real and
    pifft's backward is pfft(g).
  * The readouts use the positions they are given (the reference reads the
    positions stored by the last ppaint, lib/cpu.cc:93,137).
  * set_fft_adjoint("true") switches pifft/pfft to their exact adjoints
    (pifft's carries the half-spectrum multiplicity that the reference rule
    omits, which biases the reference's d/d alpha); the default "reference"
    reproduces the reference's gradient.
  * Only world size one: `comm` may be None or any object with size 1.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from . import _lib

__all__ = ["initLayout", "clean", "ppaint", "preadout", "ppaint3D", "preadout3D", "buildplan",
           "pfft", "pifft", "local_positions", "set_fft_adjoint", "fft_adjoint"]

_ADJOINT = {"mode": "reference"}


def set_fft_adjoint(mode: str) -> None:
    """'reference' (the reference's VJP rules) or 'true' (exact adjoints)."""
    if mode not in ("reference", "true"):
        raise ValueError("mode must be 'reference' or 'true'")
    _ADJOINT["mode"] = mode


def fft_adjoint() -> str:
    return _ADJOINT["mode"]


class _World1:
    rank = 0
    size = 1


WORLD = _World1()


def _check_comm(comm):
    size = getattr(comm, "size", 1) if comm is not None else 1
    if size != 1:
        raise NotImplementedError("only world size 1 is supported (one GPU, no MPI decomposition)")


def _stream(t: torch.Tensor):
    return ct.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _ptr(t: torch.Tensor):
    return ct.c_void_p(t.data_ptr())


def _sfx(t: torch.Tensor) -> str:
    if t.dtype == torch.float32:
        return "f32"
    if t.dtype == torch.float64:
        return "f64"
    raise NotImplementedError(f"Unsupported dtype {t.dtype}")


def _ints(v) -> tuple:
    a = np.asarray(v.detach().cpu() if isinstance(v, torch.Tensor) else v).reshape(-1)
    if a.size == 1:
        a = np.repeat(a, 3)
    return tuple(int(x) for x in a)


def _box(v, dtype) -> np.ndarray:
    a = np.asarray(v.detach().cpu() if isinstance(v, torch.Tensor) else v, dtype=np.float64).reshape(-1)
    if a.size == 1:
        a = np.repeat(a, 3)
    npdt = np.float32 if dtype == torch.float32 else np.float64
    return np.ascontiguousarray(a.astype(npdt))


def _check_pos(pos: torch.Tensor):
    if not isinstance(pos, torch.Tensor) or not pos.is_cuda:
        raise TypeError("pos must be a CUDA tensor")
    if pos.dim() != 2 or pos.shape[1] != 3:
        raise ValueError("pos must have shape (N, 3)")


def _check_edges(edges, nmesh):
    if edges is None:
        return
    e = np.asarray(edges.detach().cpu() if isinstance(edges, torch.Tensor) else edges)
    if e.shape[1] != 1:
        raise NotImplementedError("edges describe more than one rank; only world size 1 is supported")
    for a in range(3):
        if int(e[a, 0, 0]) != 0 or int(e[a, 0, 1]) != nmesh[a]:
            raise NotImplementedError("edges must cover the whole mesh at world size 1")


def _mesh_args(Nmesh, dims):
    nm = _ints(Nmesh)
    d = _ints(dims)
    if d != nm:
        raise ValueError(f"dims {d} must equal Nmesh {nm} at world size 1")
    return nm


# ---------------------------------------------------------------------------
# raw launches (no autograd)

def _paint(pos, mass, nm, box, out=None):
    pos = pos.detach().contiguous()
    sfx = _sfx(pos)
    n = pos.shape[0]
    if out is None:
        out = torch.empty(nm, dtype=pos.dtype, device=pos.device)
    b = _box(box, pos.dtype)
    if isinstance(mass, torch.Tensor) and mass.dim() > 0:
        m = mass.detach().to(pos.dtype).contiguous().reshape(-1)
        if m.numel() == 1:
            m = m.expand(n).contiguous()
        if m.numel() != n:
            raise ValueError("mass must be a scalar or have one entry per particle")
        mp, ms = _ptr(m), 0.0
    else:
        mp, ms = None, float(mass.item() if isinstance(mass, torch.Tensor) else mass)
    ctype = ct.c_float if sfx == "f32" else ct.c_double
    _lib.call(f"jld_ppaint_box_{sfx}", _stream(pos), _ptr(pos), n, mp, ctype(ms), *nm,
              b.ctypes.data_as(ct.c_void_p), _ptr(out))
    return out


def _readout(pos, field, nm, box, vjpdim=-1):
    pos = pos.detach().contiguous()
    field = field.detach().to(pos.dtype).contiguous()
    if field.numel() != nm[0] * nm[1] * nm[2]:
        raise ValueError("field size does not match Nmesh")
    sfx = _sfx(pos)
    out = torch.empty(pos.shape[0], dtype=pos.dtype, device=pos.device)
    b = _box(box, pos.dtype)
    _lib.call(f"jld_preadout_box_{sfx}", _stream(pos), _ptr(pos), pos.shape[0], _ptr(field), *nm,
              b.ctypes.data_as(ct.c_void_p), int(vjpdim), _ptr(out))
    return out


def _paint3d(pos, mass3, nm, box):
    pos = pos.detach().contiguous()
    m = mass3.detach().to(pos.dtype).contiguous()
    sfx = _sfx(pos)
    out = torch.empty((3,) + tuple(nm), dtype=pos.dtype, device=pos.device)
    b = _box(box, pos.dtype)
    _lib.call(f"jld_ppaint3d_box_{sfx}", _stream(pos), _ptr(pos), pos.shape[0], _ptr(m), *nm,
              b.ctypes.data_as(ct.c_void_p), _ptr(out))
    return out


def _readout3d(pos, field, nm, box, vjp):
    pos = pos.detach().contiguous()
    field = field.detach().to(pos.dtype).contiguous()
    sfx = _sfx(pos)
    out = torch.empty((pos.shape[0], 3), dtype=pos.dtype, device=pos.device)
    b = _box(box, pos.dtype)
    _lib.call(f"jld_preadout3d_box_{sfx}", _stream(pos), _ptr(pos), pos.shape[0], _ptr(field), *nm,
              b.ctypes.data_as(ct.c_void_p), 1 if vjp else 0, _ptr(out))
    return out


def _workspace(nm, dtype, device):
    sfx = "f32" if dtype == torch.float32 else "f64"
    nbytes = getattr(_lib.load(), f"jld_fft_workspace_{sfx}")(*nm)
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


def _pfft(data, nm):
    data = data.detach().contiguous()
    sfx = _sfx(data)
    cdt = torch.complex64 if sfx == "f32" else torch.complex128
    out = torch.empty((nm[0], nm[1], nm[2] // 2 + 1), dtype=cdt, device=data.device)
    ws = _workspace(nm, data.dtype, data.device)
    _lib.call(f"jld_pfft_c_{sfx}", _stream(data), _ptr(data), *nm, _ptr(out), _ptr(ws), ws.numel())
    return out


def _pifft(data, nm):
    data = data.detach()
    if not data.is_complex():
        data = data.to(torch.complex64 if data.dtype == torch.float32 else torch.complex128)
    data = data.contiguous()
    rdt = torch.float32 if data.dtype == torch.complex64 else torch.float64
    sfx = "f32" if rdt == torch.float32 else "f64"
    out = torch.empty(tuple(nm), dtype=rdt, device=data.device)
    ws = _workspace(nm, rdt, data.device)
    _lib.call(f"jld_pifft_c_{sfx}", _stream(out), _ptr(data), *nm, _ptr(out), _ptr(ws), ws.numel())
    return out


def _half_multiplicity(nm, device, dtype):
    h = nm[2] // 2 + 1
    m = torch.full((h,), 2.0, device=device, dtype=dtype)
    m[0] = 1.0
    if nm[2] % 2 == 0:
        m[-1] = 1.0
    return m


# ---------------------------------------------------------------------------
# layout bookkeeping

def initLayout(commsize, lyidx=0):
    """Validates commsize/lyidx; returns a (1,) int32 zero like the reference."""
    _lib.call("jld_init_layout", int(commsize), int(lyidx))
    return torch.zeros(1, dtype=torch.int32)


def clean(lyidx=0):
    _lib.call("jld_clean", int(lyidx))
    return torch.zeros(1, dtype=torch.int32)


# ---------------------------------------------------------------------------
# paint / readout with the reference's VJP rules

class _PaintFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, mass, nm, box):
        ctx.nm, ctx.box = nm, box
        ctx.save_for_backward(pos, mass if isinstance(mass, torch.Tensor) else None)
        ctx.mass_scalar = None if isinstance(mass, torch.Tensor) else float(mass)
        return _paint(pos, mass, nm, box)

    @staticmethod
    def backward(ctx, vimg):
        # ppaint_bwd, jaxpops_bind.py:236-247
        pos, mass = ctx.saved_tensors
        g_pos = g_mass = None
        if ctx.needs_input_grad[0]:
            out1 = _Readout3DFn.apply(pos, vimg, ctx.nm, ctx.box, True)
            m = mass if mass is not None else ctx.mass_scalar
            g_pos = out1 * (m.reshape(-1, 1) if isinstance(m, torch.Tensor) and m.dim() > 0 else m)
        if ctx.needs_input_grad[1]:
            g_mass = _ReadoutFn.apply(pos, vimg, ctx.nm, ctx.box, -1)
            if mass is not None and mass.dim() == 0:
                g_mass = g_mass.sum()
        return g_pos, g_mass, None, None


class _ReadoutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, field, nm, box, vjpdim):
        ctx.nm, ctx.box = nm, box
        ctx.save_for_backward(pos, field)
        return _readout(pos, field, nm, box, vjpdim)

    @staticmethod
    def backward(ctx, vmass):
        # preadout_bwd, jaxpops_bind.py:351-363
        pos, field = ctx.saved_tensors
        g_pos = g_field = None
        if ctx.needs_input_grad[0]:
            g_pos = _Readout3DFn.apply(pos, field, ctx.nm, ctx.box, True) * vmass.reshape(-1, 1)
        if ctx.needs_input_grad[1]:
            g_field = _PaintFn.apply(pos, vmass, ctx.nm, ctx.box).reshape(field.shape)
        return g_pos, g_field, None, None, None


class _Paint3DFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, mass3, nm, box):
        return _paint3d(pos, mass3, nm, box)

    @staticmethod
    def backward(ctx, g):  # the reference defines no VJP for ppaint3D
        raise NotImplementedError("ppaint3D has no VJP (as in the reference)")


class _Readout3DFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, field, nm, box, vjp):
        ctx.nm, ctx.box, ctx.vjp = nm, box, vjp
        ctx.save_for_backward(pos, field)
        return _readout3d(pos, field, nm, box, vjp)

    @staticmethod
    def backward(ctx, vmass):
        # preadout3D_bwd, jaxpops_bind.py:573-588
        if ctx.vjp:
            raise NotImplementedError("custom_vjp not implemented for 3D readout with vjp = True")
        pos, field = ctx.saved_tensors
        g_pos = g_field = None
        if ctx.needs_input_grad[0]:
            f = field.reshape((3,) + tuple(ctx.nm))
            g_pos = sum(_readout3d(pos, f[d], ctx.nm, ctx.box, True) * vmass[:, d:d + 1] for d in range(3))
        if ctx.needs_input_grad[1]:
            g_field = _paint3d(pos, vmass, ctx.nm, ctx.box).reshape(field.shape)
        return g_pos, g_field, None, None, None


def ppaint(pos, mass, Nmesh, BoxSize, edges, dims, comm, lyidx=0, bwd=False):
    """CIC paint of `pos` (N,3, box units) with masses `mass` (scalar or (N,))."""
    if lyidx > 4:
        raise Exception("lyidx needs to be smaller than 5")
    _check_comm(comm)
    _check_pos(pos)
    nm = _mesh_args(Nmesh, dims)
    _check_edges(edges, nm)
    box = tuple(float(v) for v in _box(BoxSize, torch.float64))
    return _PaintFn.apply(pos, mass, nm, box)


def preadout(pos, field, Nmesh, BoxSize, edges, dims, comm, lyidx=0, vjpdim=-1):
    """CIC readout of `field` at `pos`; vjpdim selects a weight derivative."""
    if lyidx > 4:
        raise Exception("lyidx needs to be smaller than 5")
    if vjpdim > 2:
        raise Exception("vjpdim must be between 0 and 2")
    _check_comm(comm)
    _check_pos(pos)
    nm = _mesh_args(Nmesh, dims)
    _check_edges(edges, nm)
    box = tuple(float(v) for v in _box(BoxSize, torch.float64))
    return _ReadoutFn.apply(pos, field, nm, box, int(vjpdim))


def ppaint3D(pos, mass, Nmesh, BoxSize, edges, dims, comm, lyidx=0):
    """Three-channel CIC paint: mass (N,3) -> (3, *dims)."""
    if lyidx > 4:
        raise Exception("lyidx needs to be smaller than 5")
    if mass.shape[1] != 3:
        raise Exception("Invalid input mass shape")
    _check_comm(comm)
    _check_pos(pos)
    nm = _mesh_args(Nmesh, dims)
    _check_edges(edges, nm)
    box = tuple(float(v) for v in _box(BoxSize, torch.float64))
    return _Paint3DFn.apply(pos, mass, nm, box)


def preadout3D(pos, field, Nmesh, BoxSize, edges, dims, comm, lyidx=0, vjp=False):
    """Reads three fields (vjp=False) or the three weight gradients of one."""
    if lyidx > 4:
        raise Exception("lyidx needs to be smaller than 5")
    if not vjp and len(field) != 3:
        raise Exception("Invalid input field shape")
    _check_comm(comm)
    _check_pos(pos)
    nm = _mesh_args(Nmesh, dims)
    _check_edges(edges, nm)
    box = tuple(float(v) for v in _box(BoxSize, torch.float64))
    return _Readout3DFn.apply(pos, field, nm, box, bool(vjp))


# ---------------------------------------------------------------------------
# FFT pair

def buildplan(Nmesh, comm):
    """Builds the FFT plans (both dtypes); returns int32 (localL, localstart)."""
    _check_comm(comm)
    nm = _ints(Nmesh)
    out = (ct.c_int32 * 2)()
    _lib.call("jld_buildplan_f32", *nm, ct.cast(out, ct.c_void_p))
    _lib.call("jld_buildplan_f64", *nm, ct.cast(out, ct.c_void_p))
    return torch.tensor([out[0], out[1]], dtype=torch.int32)


class _PfftFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, nm):
        ctx.nm = nm
        return _pfft(data, nm)

    @staticmethod
    def backward(ctx, g):
        # pfft_bwd (jaxpops_bind.py:699-701) in torch's conjugate convention
        if _ADJOINT["mode"] == "true":
            g = g / _half_multiplicity(ctx.nm, g.device, g.real.dtype)
        return _PifftFn.apply(g, ctx.nm), None


class _PifftFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, nm):
        ctx.nm = nm
        return _pifft(data, nm)

    @staticmethod
    def backward(ctx, g):
        # pifft_bwd (jaxpops_bind.py:758-759) in torch's conjugate convention
        out = _PfftFn.apply(g, ctx.nm)
        if _ADJOINT["mode"] == "true":
            out = out * _half_multiplicity(ctx.nm, g.device, g.dtype)
        return out, None


def pfft(data, dims):
    """Unnormalised r2c FFT of (L, M, N) real data -> complex (L, M, N//2+1)."""
    nm = _ints(dims)
    if tuple(data.shape) != nm and data.numel() != nm[0] * nm[1] * nm[2]:
        raise ValueError("data does not match dims")
    return _PfftFn.apply(data.reshape(nm), nm)


def pifft(data, dims):
    """Unnormalised c2r FFT of complex (L, M, N//2+1) -> real (L, M, N)."""
    nm = _ints(dims)
    return _PifftFn.apply(data.reshape(nm[0], nm[1], nm[2] // 2 + 1), nm)


# ---------------------------------------------------------------------------

def local_positions(pos, Nout, Nmesh, BoxSize, edges, commsize, commrank):
    """World-size-one form of the particle rebalancing of
    lib/parops_fast.h:860-925: every particle stays on rank 0 in input order,
    returned as (pos mod L) / cell * cell."""
    Nout = np.asarray(Nout)
    if Nout.sum() != len(pos):
        raise Exception(f"The sum of local sizes should match the total number of particles, "
                        f"got {Nout.sum()} and {len(pos)} instead.")
    if int(commsize) != 1 or int(commrank) != 0:
        raise NotImplementedError("only world size 1 is supported")
    nm = np.asarray(_ints(Nmesh), dtype=np.float64)
    b = _box(BoxSize, pos.dtype)
    box = torch.as_tensor(b, device=pos.device, dtype=pos.dtype)
    cell = box / torch.as_tensor(nm, device=pos.device, dtype=pos.dtype)
    return torch.remainder(pos, box) / cell * cell
