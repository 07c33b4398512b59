"""Fused LDL forward + adjoint step (libjld's jld_ldl_step_f32) with CUDA-graph
capture.

One call evaluates the loss of model.py (kinds "sm", "dm" and "HI") and its
gradient with respect to every parameter, the way
JERALDModel.loss_and_grad does through the primitives, but with the
elementwise source, filter and gradient kernels fused into the FFT passes,
a float4 force mesh for the readout, float4 vector atomics for the adjoint
paint and FP64 reductions for the loss and the parameter gradients.

    step = FusedLDL(nmesh=512, box=1000.0, nparts=N, nstep=2, kind="sm")
    loss, grad = step(pos, params, target)          # eager
    step.capture(pos, target)                        # CUDA graph on static inputs
    loss, grad = step.replay(params)                 # one graph launch per step
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from . import _lib

_KINDS = {"sm": 0, "dm": 1, "HI": 2}
_MODES = {"reference": 0, "true": 1}
_PAINT = {"atomic": 0, "warp": 1, "tiled": 4}


class _LossExt(ct.Structure):
    """jld_ldl_loss_ext of include/jld.h."""
    _fields_ = [("n", ct.c_float), ("index", ct.c_float), ("field2", ct.c_void_p), ("maskvalid", ct.c_void_p)]


def _new_graph():
    """A CUDA graph whose cudaGraph_t stays queryable after instantiation
    (for counting its kernel nodes) where torch supports that."""
    try:
        g = torch.cuda.CUDAGraph(keep_graph=True)
        g._jld_kept = True
    except TypeError:
        g = torch.cuda.CUDAGraph()
        g._jld_kept = False
    return g


def _finish_capture(g) -> None:
    """Instantiates a kept graph right after capture (a graph that is not
    kept was instantiated by the capture itself)."""
    if getattr(g, "_jld_kept", False):
        g.instantiate()


class FusedLDL:
    def __init__(self, nmesh, box, nparts: int, nstep: int = 2, kind: str = "sm", L1=None,
                 grad_mode: str = "reference", paint_method: str = "atomic", device="cuda",
                 pipelined: bool = True, recompute: bool = False, n: float = 0.0, index: float = 1.0,
                 starmap=None, x_radix: int = 8, min_cols: int = 0, bin_tile: int = 16):
        nm = np.broadcast_to(np.asarray(nmesh, dtype=np.int64).reshape(-1), (3,))
        self.nmesh = tuple(int(v) for v in nm)
        self.box = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float32).reshape(-1), (3,)))
        if kind not in _KINDS:
            raise ValueError("kind must be 'sm', 'dm' or 'HI'")
        self.kind = kind
        # HI kind (model.py:213-247, 313-336): the star map is a fixed input
        # of the model, a float32 mesh kept on the device
        self.starmap = None
        if kind == "HI":
            if starmap is None:
                raise ValueError("Star map required for HI target")
            if n != 0 or index != 1:
                raise ValueError("the fused HI step has no residual smoothing or map exponent")
            sm = torch.as_tensor(starmap, dtype=torch.float32, device=device).contiguous()
            if sm.numel() != int(np.prod(self.nmesh)):
                raise ValueError("starmap must be a mesh of the step's shape")
            self.starmap = sm
        self.L1 = (kind != "dm") if L1 is None else bool(L1)
        self.grad_mode = grad_mode
        self.paint_method = paint_method
        self.pipelined = bool(pipelined)
        self.recompute = bool(recompute)
        # schedule choices (the same step, different speed): radix of the x
        # passes' schedules where radix-8 ones fit (8 or 16), narrowest
        # pipelined tile (0 = automatic, 4, 8 or 16 columns), binning tile
        # edge of the "tiled" paint (16, 8 or 20 cells)
        if x_radix not in (8, 16) or min_cols not in (0, 4, 8, 16) or bin_tile not in (16, 8, 20):
            raise ValueError("x_radix must be 8 or 16, min_cols 0, 4, 8 or 16, bin_tile 16, 8 or 20")
        self.x_radix, self.min_cols, self.bin_tile = int(x_radix), int(min_cols), int(bin_tile)
        self.nparts = int(nparts)
        self.nstep = int(nstep)
        self.nparams = {"sm": 5 * self.nstep + 3, "dm": 5 * self.nstep, "HI": 10 * self.nstep + 12}[kind]
        self.device = torch.device(device)
        lib = _lib.load()
        ws_fn = lib.jld_ldl_workspace_hi_f32 if kind == "HI" else lib.jld_ldl_workspace_opt_f32
        nbytes = ws_fn(*self.nmesh, self.nparts, self.nstep, self.options)
        if nbytes == 0:
            raise ValueError("invalid fused-step geometry")
        self.ws = torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)
        if not (n >= 0):
            raise ValueError("n must be >= 0")
        self.n = float(n)          # loss smoothing exponent (model.py:376-381)
        self.index = float(index)  # map exponent (model.py:357)
        # [loss, grads..., validation loss]; `out` is the [loss, grads...] view
        self._buf = torch.zeros(2 + self.nparams, dtype=torch.float64, device=self.device)
        self.out = self._buf[:1 + self.nparams]
        self.params = torch.zeros(self.nparams, dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("jld_ldl_prepare_f32", *self.nmesh, self.box.ctypes.data_as(ct.c_void_p))
        self.graph = None
        self._static = None

    @property
    def options(self) -> int:
        """Option bits of jld_ldl_step_f32."""
        cols = {0: 0, 4: 1, 8: 2, 16: 3}[self.min_cols] << 5
        tile = {16: 0, 8: 1, 20: 2}[self.bin_tile] << 7
        return (_PAINT[self.paint_method] | (0 if self.pipelined else 2) | (8 if self.recompute else 0)
                | (16 if self.x_radix == 16 else 0) | cols | tile)

    @property
    def workspace_bytes(self) -> int:
        return self.ws.numel()

    def _launch(self, pos: torch.Tensor, target: torch.Tensor, mask, field2=None, maskvalid=None):
        if pos.dtype != torch.float32 or not pos.is_contiguous() or pos.shape != (self.nparts, 3):
            raise ValueError("pos must be a contiguous float32 (nparts, 3) CUDA tensor")
        C = int(np.prod(self.nmesh))
        if target.dtype != torch.float32 or not target.is_contiguous() or target.numel() != C:
            raise ValueError("target must be a contiguous float32 mesh")
        for name, m in (("mask", mask), ("field2", field2), ("maskvalid", maskvalid)):
            if m is not None and (m.dtype != torch.float32 or not m.is_contiguous() or m.numel() != C):
                raise ValueError(f"{name} must be a contiguous float32 mesh")
        ptr = lambda t: ct.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        st = ct.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        if self.kind == "HI":
            if field2 is not None or maskvalid is not None:
                raise ValueError("the fused HI step takes no field2 or validation mask")
            _lib.call("jld_ldl_step_hi_f32", st, ct.c_void_p(pos.data_ptr()), self.nparts, *self.nmesh,
                      self.box.ctypes.data_as(ct.c_void_p), self.nstep, int(self.L1), _MODES[self.grad_mode],
                      self.options, ct.c_void_p(self.params.data_ptr()), ct.c_void_p(target.data_ptr()),
                      ptr(mask), ct.c_void_p(self.starmap.data_ptr()), ct.c_void_p(self.ws.data_ptr()),
                      self.ws.numel(), ct.c_void_p(self._buf.data_ptr()))
            return
        ext = _LossExt(self.n, self.index, ptr(field2), ptr(maskvalid))
        _lib.call("jld_ldl_step_ext_f32", st, ct.c_void_p(pos.data_ptr()), self.nparts, *self.nmesh,
                  self.box.ctypes.data_as(ct.c_void_p), self.nstep, _KINDS[self.kind], int(self.L1),
                  _MODES[self.grad_mode], self.options,
                  ct.c_void_p(self.params.data_ptr()), ct.c_void_p(target.data_ptr()), ptr(mask),
                  ct.c_void_p(ct.addressof(ext)), ct.c_void_p(self.ws.data_ptr()), self.ws.numel(),
                  ct.c_void_p(self._buf.data_ptr()))

    @property
    def lossv(self) -> torch.Tensor:
        """Validation loss of the last step (model.py lossv; 0 without maskvalid)."""
        return self._buf[1 + self.nparams]

    def _set_params(self, params):
        p = torch.as_tensor(params, dtype=torch.float32).reshape(-1)
        if p.numel() != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.numel()}")
        self.params.copy_(p.to(self.device), non_blocking=True)

    def __call__(self, pos, params, target, mask=None, field2=None, maskvalid=None):
        """Eager step; returns (loss, grad) as float64 device tensors (the
        validation loss is `lossv`)."""
        self._set_params(params)
        self._launch(pos, target, mask, field2, maskvalid)
        return self.out[0], self.out[1:]

    def capture_graph(self, pos, target, mask=None, field2=None, maskvalid=None):
        """A new CUDA graph of the step on these (static) inputs; the step's
        own graph is left as it is."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self._launch(pos, target, mask, field2, maskvalid)  # builds plans, tables and kernel attributes
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = _new_graph()
        with torch.cuda.graph(g):
            self._launch(pos, target, mask, field2, maskvalid)
        _finish_capture(g)
        return g

    def capture(self, pos, target, mask=None, field2=None, maskvalid=None):
        """Captures the step on static inputs (they must stay alive and in place)."""
        self._static = (pos, target, mask, field2, maskvalid)
        self.graph = self.capture_graph(pos, target, mask, field2, maskvalid)
        return self.graph

    def replay(self, params=None):
        if self.graph is None:
            raise RuntimeError("capture() first")
        if params is not None:
            self._set_params(params)
        self.graph.replay()
        return self.out[0], self.out[1:]

    def graph_kernels(self):
        """Kernel launches one replay of the captured graph issues (None
        before capture or when torch does not expose the raw graph)."""
        if self.graph is None or not hasattr(self.graph, "raw_cuda_graph"):
            return None
        try:
            raw = self.graph.raw_cuda_graph()
        except RuntimeError:  # graph not kept after instantiation
            return None
        k = ct.c_int64(0)
        _lib.call("jld_graph_kernel_nodes", ct.c_void_p(raw), ct.byref(k))
        return int(k.value)

    def error_word(self) -> int:
        """Nonzero if a pipelined pass of the last step gave up waiting for a copy."""
        ptr = ct.c_void_p()
        _lib.call("jld_ldl_error_word_f32", ct.c_void_p(self.ws.data_ptr()), *self.nmesh, self.nparts, self.nstep,
                  ct.byref(ptr))
        off = ptr.value - self.ws.data_ptr()
        return int(self.ws[off: off + 4].view(torch.int32).item())

    def positions(self, layer: int) -> torch.Tensor:
        """(nparts, 3) view of the positions after `layer` layers of the last step."""
        ptr = ct.c_void_p()
        _lib.call("jld_ldl_positions_f32", ct.c_void_p(self.ws.data_ptr()), *self.nmesh, self.nparts,
                  self.nstep, int(layer), ct.byref(ptr))
        off = ptr.value - self.ws.data_ptr()
        x = self.ws[off: off + 12 * self.nparts].view(torch.float32).view(self.nparts, 3)
        if self.paint_method != "tiled":
            return x
        _lib.call("jld_ldl_order_f32", ct.c_void_p(self.ws.data_ptr()), *self.nmesh, self.nparts, self.nstep,
                  ct.byref(ptr))
        off = ptr.value - self.ws.data_ptr()
        perm = self.ws[off: off + 4 * self.nparts].view(torch.int32).long()
        out = torch.empty_like(x)
        out[perm] = x
        return out


class HostFeed:
    """Runs a FusedLDL from host-resident inputs, one step per input pair,
    with the host-to-device copies of step k+1 overlapped with the compute
    of step k: two device input buffers with one captured graph each, a copy
    stream and events.  Page-locked inputs are streamed in by a small kernel
    that reads host memory directly (jld_copy_from_host, copy="kernel") or
    by the copy engines (copy="engine"); others go through copy_.  Every step's positions and target are copied and its loss and
    gradient are read back; only the order of the copies changes, not their
    amount.
    """

    def __init__(self, step: FusedLDL, mask=None, copy: str = "kernel", ctas: int = 4):
        if copy not in ("kernel", "engine"):
            raise ValueError("copy must be 'kernel' or 'engine'")
        self.step = step
        self.copy_mode = copy
        dev = step.device
        self.pos = [torch.empty((step.nparts, 3), dtype=torch.float32, device=dev) for _ in range(2)]
        self.tgt = [torch.empty(step.nmesh, dtype=torch.float32, device=dev) for _ in range(2)]
        # capture_graph runs one eager step on these buffers first: spread
        # positions, since particles piled into one cell would make that
        # step's paint atomics contend (about 1 s at 1.5e8 particles)
        gen = torch.Generator(device=dev)
        gen.manual_seed(0)
        box = torch.as_tensor(step.box, dtype=torch.float32, device=dev)
        for t in self.pos:
            torch.rand(t.shape, generator=gen, device=dev, out=t)
            t.mul_(box)
        for t in self.tgt:
            t.fill_(1.0)
        self.mask = mask
        self.graphs = [step.capture_graph(self.pos[b], self.tgt[b], mask) for b in range(2)]
        self.copy = torch.cuda.Stream(dev)
        self.ctas = int(ctas)  # enough to saturate the host link; leaves the SMs to the step
        self.copied = [torch.cuda.Event() for _ in range(2)]
        self.free = [torch.cuda.Event() for _ in range(2)]

    def run(self, inputs, params, out_host: torch.Tensor) -> None:
        """inputs: sequence of (pos, target) host tensors (pinned for
        asynchronous copies); out_host: (len(inputs), 1 + nparams) float64
        host tensor (pinned) that receives each step's loss and gradient.
        Returns once everything is enqueued; synchronise before reading."""
        step = self.step
        comp = torch.cuda.current_stream(step.device)
        step._set_params(params)
        for b in range(2):
            self.free[b].record(comp)

        cs = ct.c_void_p(self.copy.cuda_stream)

        def put(dst: torch.Tensor, src: torch.Tensor) -> None:
            nbytes = dst.numel() * dst.element_size()
            if (self.copy_mode == "kernel" and src.is_pinned() and src.is_contiguous()
                    and src.numel() == dst.numel() and src.dtype == dst.dtype and src.data_ptr() % 16 == 0):
                # a few CTAs read the page-locked buffer directly (NVLink-C2C)
                _lib.call("jld_copy_from_host", cs, ct.c_void_p(dst.data_ptr()), ct.c_void_p(src.data_ptr()),
                          nbytes, self.ctas)
            else:
                dst.copy_(src, non_blocking=True)

        def feed(k):
            b = k % 2
            self.copy.wait_event(self.free[b])  # the graph that last read buffer b is done
            with torch.cuda.stream(self.copy):
                put(self.pos[b], inputs[k][0])
                put(self.tgt[b], inputs[k][1])
                self.copied[b].record(self.copy)

        n = len(inputs)
        if n:
            feed(0)
        for k in range(n):
            if k + 1 < n:
                feed(k + 1)
            b = k % 2
            comp.wait_event(self.copied[b])
            self.graphs[b].replay()
            self.free[b].record(comp)
            out_host[k].copy_(step.out, non_blocking=True)
