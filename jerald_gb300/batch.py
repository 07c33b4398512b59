"""Many independent boxes in one graph launch, with per-shape autotuning.

A batch holds one fused LDL step (FusedLDL) per box -- boxes may differ in
mesh, box size, particle count, kind and parameters -- and captures all of
their forward + adjoint evaluations into ONE CUDA graph.  Inside the graph
the boxes run on `streams` parallel branches, so small boxes fill the SMs
that a single small box leaves idle; one `replay()` launches every box's
step.  Parameters for all boxes live in one device buffer (one host->device
copy per replay).

Autotuning: for every distinct (mesh, particle count, kind, clustering
level) the first batch that meets it times candidate configurations of the
step for a few eager steps each and keeps the fastest.  The search runs in
stages, each from the best configuration so far: the FFT passes (pipelined
or generic) with the scatter method (plain, warp-aggregated or tiled
atomics); then, for pipelined passes, the x passes' radix schedule (8 or 16)
and the narrowest pipelined tile (4, 8 or 16 columns, or automatic); then,
for tiled scatters, the binning tile edge (8, 16 or 20 cells).  The
clustering level is the share of particles in cells that hold at least 8
(below 1 %, below 10 %, above), so a clustered box of the same shape is
tuned on its own.  Choices are cached for the process and optionally in a
JSON file, so later batches and captures reuse them.

There is no counterpart in the reference, which runs one box per process
(model.py's JERALDModel); the batch is how the GPU build serves many small
boxes at once.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field

import numpy as np
import torch

from .ldl import FusedLDL, _finish_capture, _new_graph

CANDIDATES = [
    {"pipelined": True, "paint_method": "atomic"},
    {"pipelined": False, "paint_method": "atomic"},
    {"pipelined": True, "paint_method": "tiled"},
    {"pipelined": True, "paint_method": "warp"},
]

# keys of a tuned configuration (FusedLDL keyword arguments)
TUNED = ("pipelined", "paint_method", "x_radix", "min_cols", "bin_tile")

_CACHE: dict[str, dict] = {}


def _key(nmesh, nparts, kind, nstep, level=0) -> str:
    nm = np.broadcast_to(np.asarray(nmesh, dtype=np.int64).reshape(-1), (3,))
    return f"{tuple(int(v) for v in nm)}:{int(nparts)}:{kind}:{int(nstep)}:c{int(level)}"


def clustering_level(pos: torch.Tensor, nmesh, box) -> int:
    """0, 1 or 2: share of the particles in cells holding at least 8 of them
    below 1 %, below 10 %, or above (cells of the paint's lower corner)."""
    nm = torch.as_tensor(np.broadcast_to(np.asarray(nmesh, dtype=np.int64).reshape(-1), (3,)).copy(),
                         device=pos.device)
    bx = torch.as_tensor(np.broadcast_to(np.asarray(box, dtype=np.float64).reshape(-1), (3,)).copy(),
                         device=pos.device)
    cell = torch.floor(pos.double() / bx * nm).long() % nm
    key = (cell[:, 0] * nm[1] + cell[:, 1]) * nm[2] + cell[:, 2]
    occ = torch.bincount(key, minlength=int(nm.prod()))
    share = float(occ[key].ge(8).double().mean())
    return 0 if share < 0.01 else (1 if share < 0.1 else 2)


def load_tuning(path: str) -> None:
    """Merges a JSON tuning file written by save_tuning into the cache."""
    if os.path.exists(path):
        with open(path) as f:
            _CACHE.update(json.load(f))


def save_tuning(path: str) -> None:
    with open(path, "w") as f:
        json.dump(_CACHE, f, indent=1, sort_keys=True)


def autotune(nmesh, box, pos, target, params, nstep=2, kind="sm", L1=None, grad_mode="reference",
             candidates=None, reps: int = 5, device="cuda") -> dict:
    """Fastest configuration of the fused step for this box shape and
    clustering level (cached).  Each candidate is captured into a CUDA graph
    and timed over `reps` replays after one untimed replay; the candidates
    must agree on the loss (they compute the same step).  `candidates`
    replaces the staged search by one list."""
    nm = np.broadcast_to(np.asarray(nmesh, dtype=np.int64).reshape(-1), (3,))
    level = clustering_level(pos, nm, box)
    key = _key(nm, pos.shape[0], kind, nstep, level)
    if key in _CACHE:
        return _CACHE[key]
    times, losses = {}, []

    def run(cand) -> float:
        name = json.dumps(cand, sort_keys=True)
        if name in times:
            return times[name]
        step = FusedLDL(nm, box, pos.shape[0], nstep=nstep, kind=kind, L1=L1, grad_mode=grad_mode,
                        device=device, **cand)
        # timed as the batch runs it: replays of a captured graph (eager
        # calls of a small box measure the host's launch work instead)
        step._set_params(params)
        g = step.capture_graph(pos, target)
        g.replay()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            g.replay()
        e1.record()
        torch.cuda.synchronize(device)
        times[name] = e0.elapsed_time(e1) / reps
        losses.append(float(step.out[0]))
        del g, step
        return times[name]

    def best_of(cands):
        return min(cands, key=run)

    if candidates:
        best = best_of(candidates)
    else:
        best = best_of(CANDIDATES)
        if best["pipelined"]:
            best = best_of([best, {**best, "x_radix": 16}])
            best = best_of([best] + [{**best, "min_cols": c} for c in (4, 8, 16)])
        if best["paint_method"] == "tiled":
            best = best_of([best] + [{**best, "bin_tile": t} for t in (8, 20)])
    ref = losses[0]
    if any(abs(v - ref) > 1e-4 * abs(ref) for v in losses):
        raise RuntimeError(f"autotune candidates disagree on the loss: {losses}")
    _CACHE[key] = {**best, "ms": times[json.dumps(best, sort_keys=True)], "timings": times,
                   "clustering_level": level}
    return _CACHE[key]


@dataclass
class Box:
    """One box of a batch: mesh, box size, positions (N, 3) and target mesh
    on the device, and its model configuration."""
    nmesh: object
    box: object
    pos: torch.Tensor
    target: torch.Tensor
    nstep: int = 2
    kind: str = "sm"
    L1: object = None
    mask: torch.Tensor | None = None
    grad_mode: str = "reference"
    config: dict = field(default_factory=dict)


class FusedLDLBatch:
    def __init__(self, boxes: list[Box], streams: int = 4, tune: bool = True, device="cuda"):
        self.boxes = boxes
        self.device = torch.device(device)
        self.steps: list[FusedLDL] = []
        nparams = []
        for b in boxes:
            cfg = dict(b.config)
            if tune and not cfg:
                t = autotune(b.nmesh, b.box, b.pos, b.target, _default_params(b), nstep=b.nstep, kind=b.kind,
                             L1=b.L1, grad_mode=b.grad_mode, device=self.device)
                cfg = {k: t[k] for k in TUNED if k in t}
            b.config = cfg
            st = FusedLDL(b.nmesh, b.box, b.pos.shape[0], nstep=b.nstep, kind=b.kind, L1=b.L1,
                          grad_mode=b.grad_mode, device=self.device, **cfg)
            self.steps.append(st)
            nparams.append(st.nparams)
        # one parameter buffer: each step reads its own slice
        self.offsets = np.concatenate([[0], np.cumsum(nparams)]).astype(np.int64)
        self.params = torch.zeros(int(self.offsets[-1]), dtype=torch.float32, device=self.device)
        for i, st in enumerate(self.steps):
            st.params = self.params[self.offsets[i]:self.offsets[i + 1]]
        self.nstreams = max(1, int(streams))
        self.graph = None

    def _set_params(self, params_list) -> None:
        flat = np.concatenate([np.asarray(p, dtype=np.float32).reshape(-1) for p in params_list])
        if flat.size != self.params.numel():
            raise ValueError(f"expected {self.params.numel()} parameters in total, got {flat.size}")
        self.params.copy_(torch.from_numpy(flat).to(self.device), non_blocking=True)

    def _launch_all(self) -> None:
        main = torch.cuda.current_stream(self.device)
        for i, (b, st) in enumerate(zip(self.boxes, self.steps)):
            s = self._streams[i % self.nstreams]
            s.wait_stream(main)
            with torch.cuda.stream(s):
                st._launch(b.pos, b.target, b.mask)
        for s in self._streams:
            main.wait_stream(s)

    def __call__(self, params_list):
        """Eager evaluation of every box: list of (loss, grad) device tensors."""
        self._set_params(params_list)
        self._streams = [torch.cuda.Stream(self.device) for _ in range(self.nstreams)]
        self._launch_all()
        return [(st.out[0], st.out[1:]) for st in self.steps]

    def capture(self):
        """Captures all boxes' steps into one CUDA graph (inputs must stay in place)."""
        self._streams = [torch.cuda.Stream(self.device) for _ in range(self.nstreams)]
        self._launch_all()  # plans, tables and kernel attributes exist before capture
        torch.cuda.synchronize(self.device)
        self.graph = _new_graph()
        with torch.cuda.graph(self.graph):
            self._launch_all()
        _finish_capture(self.graph)
        return self.graph

    def replay(self, params_list=None):
        if self.graph is None:
            raise RuntimeError("capture() first")
        if params_list is not None:
            self._set_params(params_list)
        self.graph.replay()
        return [(st.out[0], st.out[1:]) for st in self.steps]

    def graph_kernels(self):
        if self.graph is None or not hasattr(self.graph, "raw_cuda_graph"):
            return None
        try:
            raw = self.graph.raw_cuda_graph()
        except RuntimeError:  # graph not kept after instantiation
            return None
        import ctypes as ct
        from . import _lib
        k = ct.c_int64(0)
        _lib.call("jld_graph_kernel_nodes", ct.c_void_p(raw), ct.byref(k))
        return int(k.value)


def _default_params(b: Box) -> np.ndarray:
    from .synth import default_params
    p = default_params(b.nstep)
    return p if b.kind == "sm" else p[:5 * b.nstep]


def make_c3_boxes(seed: int = 0, nbox: int = 16, device="cuda", sizes=(64, 96, 128, 192, 256)):
    """The 16-box workload: meshes drawn from `sizes`^3, one particle per cell
    (a Zel'dovich lattice, 0.5-cell rms displacement, 100 * n / 64 box),
    parameters uniform within +-50% of the 64^3 configuration's, target the
    lognormal noise field (sigma 0.1)."""
    from . import synth
    rng = np.random.default_rng(seed)
    boxes, params = [], []
    base = synth.default_params(2)
    for i in range(nbox):
        n = int(rng.choice(sizes))
        L = 100.0 * n / 64
        pos = synth.zeldovich(n, L, 0.5, seed=seed * 1000 + i, device=device).contiguous()
        tgt = torch.from_numpy(synth.lognormal_noise((n, n, n), 0.1, seed=seed * 1000 + i + 500)
                               .astype(np.float32)).to(device)
        boxes.append(Box(n, L, pos, tgt))
        params.append(base * rng.uniform(0.5, 1.5, base.shape))
    return boxes, params
