"""LDL forward+adjoint benchmark on one GB300 (or N replicas under torchrun).

Workload (default, the 512^3 configuration of the metric): clustered 512^3
particles on a 512^3 mesh -- a Zel'dovich lattice with 3-cell rms
displacement plus 10% extra particles in 2000 Gaussian halos of 0.5-cell
width with Poisson counts -- two "sm" displacement layers (alpha, gamma, kh,
kl, nu) = (0.05, 1, 0.5, 2, 1), the ReLU bias map (mu, w, b) = (1.5, 1, -0.1),
L1 loss against the model's own output times lognormal noise (sigma 0.1).
Seeded synthetic data; box = 100 * n / 64 (the 64^3 configuration's cell
size).

A step is one fused, CUDA-graph-captured forward + adjoint evaluation
(loss and all 13 parameter gradients) with inputs resident in HBM.  The
inputs (1.8 GB of positions, 0.5 GB target) exceed the 129 MB L2, so no
flush is needed between steps.  `e2e` repeats the step through the public
API with host buffers: pinned-host -> device copies of positions and target
and a device -> host read of loss and gradients inside the timed region.

Both arms draw the same inputs: the positions are generated on the host
(numpy, seeded) and copied to the device.  --impl reference times the
oracle's FP64 CPU restatement of the same step (the reference's own ops need
MPI, FFTW and JAX, which neither host has): C CIC loops over particle ranges
and pocketFFT on every host thread, on the full workload, W untimed and K
timed steps, with the same config as this arm.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "LDL fwd+grad steps/s at 512³ (fused vs plain GPU ops, grad err≤1e-4); HBM %peak"
UNIT = "steps/s"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------

def host_workload(n: int, seed: int = 0):
    """Clustered positions (numpy float32, (N, 3)) and the box size."""
    from jerald_gb300 import synth
    box = 100.0 * n / 64
    return np.ascontiguousarray(synth.clustered(n, box, seed=seed)), box


def make_workload(n: int, device, seed: int = 0):
    import torch
    pos, box = host_workload(n, seed)
    return torch.from_numpy(pos).to(device).contiguous(), box


def noise_field(n: int):
    from jerald_gb300 import synth
    return synth.lognormal_noise((n, n, n), 0.1, seed=2)


def make_target(pos, n, box, params, device, nstep: int = 2):
    """The model's own output (plain primitives, float32, no autograd) times
    lognormal noise (sigma 0.1)."""
    import torch
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    pm = PMesh(n, box, device=device, dtype=torch.float32)
    model = JERALDModel(pos, None, pm, Nstep=nstep, kind="sm")
    with torch.no_grad():
        F = model.evaluate(torch.as_tensor(params, dtype=torch.float32, device=device), pos, nstep)
    del model, pm
    F *= torch.from_numpy(noise_field(n).astype(np.float32)).to(device)
    torch.cuda.empty_cache()
    return F.contiguous()


def workload_config(n: int, nparts: int, box: float, nstep: int, recompute: bool = False, world: int = 1):
    """The `config` object of both arms' lines."""
    inputs = 12 * int(nparts) + 4 * n ** 3  # positions and target
    return {"workload": f"clustered {n}^3 particles +10% halos on a {n}^3 mesh, {nstep} sm layers + "
                        f"ReLU map, L1 loss, fwd+adjoint ({5 * nstep + 3} grads)",
            "nmesh": n, "nparts": int(nparts), "box": box, "nstep": nstep, "kind": "sm",
            "memory_plan": "recompute force meshes" if recompute else "checkpoint",
            "l2": ("inputs larger than L2 (no flush)" if inputs > 129e6
                   else "inputs fit in L2 (no flush: a small configuration)"),
            "parallelism": f"{world} replicas" if world > 1 else "single GPU"}


def yardstick_bytes(N: int, nstep: int) -> int:
    """Plain-primitive byte yardstick of one fwd+adjoint step (N = C): per
    layer 108N forward and 224N adjoint, 16N final paint, 48N its adjoint."""
    return (332 * nstep + 64) * N


def time_primitives(pos, n, box, steps, warmup):
    """Per-kernel CUDA-event timings of the drop-in primitives on the workload,
    with algorithmic bytes (12N + 4C paint, 16N + 4C readout, 4C + 8H r2c)."""
    import ctypes as ct
    import torch
    from jerald_gb300 import _lib
    N = pos.shape[0]
    C = n ** 3
    H = n * n * (n // 2 + 1)
    b = np.asarray([box] * 3, dtype=np.float32)
    mesh = torch.empty((n, n, n), device=pos.device)
    out = torch.empty(N, device=pos.device)
    spec = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=pos.device)
    ws = torch.empty(int(_lib.load().jld_fft_workspace_f32(n, n, n)), dtype=torch.uint8, device=pos.device)
    field = torch.randn((n, n, n), device=pos.device)
    st = torch.cuda.current_stream()
    sp = ct.c_void_p(st.cuda_stream)
    P = lambda t: ct.c_void_p(t.data_ptr())  # noqa: E731
    bp = b.ctypes.data_as(ct.c_void_p)
    sws = torch.empty(int(_lib.load().jld_ppaint_box_sorted_workspace(N)), dtype=torch.uint8, device=pos.device)
    keys = sws[:4 * N].view(torch.int32)
    order = sws[(4 * N + 255) // 256 * 256:][:4 * N].view(torch.int32)
    cws = torch.empty(int(_lib.load().jld_cell_sort_workspace(N)), dtype=torch.uint8, device=pos.device)
    _lib.call("jld_cell_sort_f32", sp, P(pos), N, n, n, n, bp, P(keys), P(order), P(cws), cws.numel())
    ops = {
        "paint": (lambda: _lib.call("jld_ppaint_box_f32", sp, P(pos), N, None, ct.c_float(1.0), n, n, n, bp, P(mesh)),
                  12 * N + 4 * C),
        # warp-aggregated atomics (lanes on one cell merged first)
        "paint_warp": (lambda: _lib.call("jld_ppaint_box_method_f32", sp, P(pos), N, None, ct.c_float(1.0), n, n, n,
                                         bp, 1, P(mesh)), 12 * N + 4 * C),
        # stable sort by cell key (keys and order written: 12N in, 8N out)
        "cell_sort": (lambda: _lib.call("jld_cell_sort_f32", sp, P(pos), N, n, n, n, bp, P(keys), P(order), P(cws),
                                        cws.numel()), 20 * N),
        # paint from a kept cell-key order (the order read as well: 20N + 4C)
        "paint_sorted_reuse": (lambda: _lib.call("jld_ppaint_sorted_f32", sp, P(pos), N, None, ct.c_float(1.0),
                                                 n, n, n, bp, P(keys), P(order), P(mesh)), 20 * N + 4 * C),
        # sort and sorted paint in one call (the paint's algorithmic bytes)
        "paint_sorted": (lambda: _lib.call("jld_ppaint_box_sorted_f32", sp, P(pos), N, None, ct.c_float(1.0),
                                           n, n, n, bp, P(mesh), P(sws), sws.numel()), 12 * N + 4 * C),
        "readout": (lambda: _lib.call("jld_preadout_box_f32", sp, P(pos), N, P(field), n, n, n, bp, -1, P(out)),
                    16 * N + 4 * C),
        "r2c": (lambda: _lib.call("jld_pfft_c_f32", sp, P(field), n, n, n, P(spec), P(ws), ws.numel()),
                4 * C + 8 * H),
    }
    res = {}
    for name, (fn, nbytes) in ops.items():
        for _ in range(warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(steps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        res[name] = {"ms": ms, "algorithmic_bytes": int(nbytes), "gbs": nbytes / ms / 1e6}
    return res


def count_launches(nstep: int, kind: str, mask: bool, recompute: bool = False) -> int:
    """Kernel launches of one fused step on a power-of-two mesh with the
    pipelined passes and plain atomics (used only when the captured graph
    cannot be asked)."""
    force_mesh = 8                              # z r2c, y pass (2), x filter (2), inverse y (2), inverse z
    fwd = 1 + nstep * (force_mesh + 2)          # first paint; per layer force mesh, update, paint
    final = 1 + (2 if kind == "sm" else 1) + (1 if mask else 0)   # loss, its reductions (+ mask count)
    adj = nstep * 12                            # fused particle adjoint + 11 spectral / reduction kernels
    rec = force_mesh * max(0, nstep - 2) if recompute else 0
    return 1 + fwd + final + adj + rec


def _oracle_case(n_sample: int, threads: int):
    """The oracle's 2-layer fwd+grad set up at n_sample^3 (clustered recipe)."""
    from jerald_gb300 import synth
    from oracle import fft as offt
    from oracle import cic as ocic
    from oracle import ldl as oldl
    from oracle.ldl import LDLOracle
    offt.set_workers(threads)
    ocic.set_threads(threads)
    oldl.set_threads(threads)
    box = 100.0 * n_sample / 64
    X = synth.clustered(n_sample, box, seed=0).astype(np.float64)
    p = synth.default_params(2)
    o = LDLOracle((n_sample,) * 3, box, kind="sm", L1=True)
    o.forward(p, X, np.ones((n_sample,) * 3), 2)
    tgt = o.cache["F"] * synth.lognormal_noise(o.cache["F"].shape, 0.1, 2)
    return (lambda: o.loss_and_grad(p, X, tgt, 2)), len(X)


def _oracle_line(n_sample: int, n_full: int, threads: int, dt: float, n_part_sample: int):
    n_part_full = int(round(1.1 * n_full ** 3))
    value = (1.0 / dt) * n_part_sample / n_part_full
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle 2-layer fwd+grad at {n_sample}^3 ({n_part_sample} particles, "
                      f"{dt:.2f} s/step; CIC loops in C over {threads} particle ranges on {threads} threads, "
                      f"FFT pocketfft with {threads} workers, elementwise numpy on {threads} slabs), "
                      f"scaled by particle count to {n_full}^3"}


def cpu_baseline_sample(n_sample: int, n_full: int, steps: int = 1, threads: int | None = None):
    """Times the oracle's 2-layer fwd+grad at n_sample^3 (clustered recipe)."""
    threads = threads or os.cpu_count() or 1
    step, npart = _oracle_case(n_sample, threads)
    step()  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    return _oracle_line(n_sample, n_full, threads, (time.perf_counter() - t0) / steps, npart)


def run_reference(args):
    """The reference arm: the oracle's FP64 restatement of the reference's
    CPU ops (the reference itself needs MPI, FFTW and JAX, none of which
    exist on either host) on every host thread, on the full workload of this
    benchmark: W untimed and K timed forward+gradient steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))  # for the shared `config` only
    from jerald_gb300 import synth
    from oracle import cic as ocic
    from oracle import fft as offt
    from oracle import ldl as oldl
    threads = os.cpu_count() or 1
    offt.set_workers(threads)
    ocic.set_threads(threads)
    oldl.set_threads(threads)
    n, nstep = args.n, args.nstep
    pos, box = host_workload(n, seed=0)
    X = pos.astype(np.float64)
    del pos
    p = synth.default_params(nstep)
    o = oldl.LDLOracle((n,) * 3, box, kind="sm", L1=True)
    o.forward(p, X, np.zeros((n,) * 3), nstep)
    tgt = o.cache["F"] * noise_field(n)
    for _ in range(args.warmup):
        o.loss_and_grad(p, X, tgt, nstep)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss, _ = o.loss_and_grad(p, X, tgt, nstep)
    dt = (time.perf_counter() - t0) / args.steps
    v = 1.0 / dt
    cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": f"the full workload ({len(X)} particles, {n}^3 mesh): oracle FP64 fwd+grad, CIC loops in C "
                    f"over {threads} particle ranges, FFT pocketfft with {threads} workers, elementwise numpy "
                    f"on {threads} slabs"}
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dt, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Zel'dovich lattice + Gaussian halos)",
            "impl": "reference", "config": workload_config(n, len(X), box, nstep, args.recompute, world),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "loss": loss}
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """Eager fused steps only: the kernels ncu sees are the step's own."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    dev = torch.device("cuda", 0)
    n = args.n
    params = synth.default_params(2)
    pos, box = make_workload(n, dev, seed=0)
    target = torch.ones((n, n, n), device=dev)
    step = FusedLDL(n, box, pos.shape[0], nstep=2, kind="sm", L1=True, paint_method=args.paint, device=dev,
                    x_radix=args.x_radix, min_cols=args.min_cols)
    for _ in range(args.warmup + args.steps):
        step(pos, params, target)
    torch.cuda.synchronize()
    print(json.dumps({"profile": True, "n": n, "nparts": int(pos.shape[0]), "loss": float(step.out[0]),
                      "launches_per_step": count_launches(2, "sm", False)}))
    return 0


def run_batch(args):
    """Many independent boxes (meshes 64..256^3, one particle per cell,
    parameters within +-50% of the 64^3 configuration's) autotuned and
    captured into one CUDA graph; boxes/s and particle-steps/s."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from jerald_gb300.batch import FusedLDLBatch, make_c3_boxes
    dev = torch.device("cuda", 0)
    boxes, params = make_c3_boxes(seed=0, nbox=args.batch, device=dev)
    b = FusedLDLBatch(boxes, streams=args.streams, tune=True, device=dev)
    b.capture()
    for _ in range(args.warmup):
        b.replay(params)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        b.replay(params)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # the same boxes one after another, each as its own graph (no branches)
    serial = 0.0
    for bx, p in zip(boxes, params):
        one = FusedLDLBatch([bx], streams=1, tune=False, device=dev)
        one.capture()
        for _ in range(args.warmup):
            one.replay([p])
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(args.steps):
            one.replay([p])
        e1.record(st)
        torch.cuda.synchronize()
        serial += e0.elapsed_time(e1) / args.steps
        del one
    npart = sum(int(bx.pos.shape[0]) for bx in boxes)
    print(json.dumps({"workload": f"{len(boxes)} boxes, meshes {sorted(int(bx.nmesh) for bx in boxes)}, "
                                  f"one particle per cell, 2 sm layers, one graph",
                      "ms_per_batch": ms, "boxes_per_s": len(boxes) * 1000.0 / ms,
                      "particle_steps_per_s": npart * 1000.0 / ms, "serial_graphs_ms": serial,
                      "graph_kernels": b.graph_kernels(), "streams": args.streams,
                      "configs": [bx.config for bx in boxes]}), flush=True)
    return 0


def run_snapmap(args):
    """Snapshot-map ingestion (makemap, JERALD/snaputils.py:253-406): N gas
    particles in host memory (Coordinates, Masses, ElectronAbundance,
    InternalEnergy: map kind nT, 24 bytes per particle) streamed in chunks of
    2^23 onto an n^3 mesh; wall-clock particles/s and host bytes/s of the
    whole call (host staging copy, host-to-device copies, weights and paint),
    with the oracle's numpy restatement timed on a 1 % sample beside it."""
    import time
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import types
    from jerald_gb300 import snapmap
    from oracle import snapmap as osm
    N, n, box = int(args.snapmap), args.n, 25.0
    rng = np.random.default_rng(0)
    fields = {"Coordinates": (rng.random((N, 3), dtype=np.float32) * np.float32(box * 1000.0)),
              "Masses": rng.random(N, dtype=np.float32) * np.float32(1e-3),
              "ElectronAbundance": rng.random(N, dtype=np.float32) * np.float32(1.2),
              "InternalEnergy": rng.random(N, dtype=np.float32) * np.float32(1e4)}
    snap = snapmap.ArraySnapshot(redshift=2.0, parts={0: fields})
    pm = types.SimpleNamespace(Nmesh=np.asarray([n] * 3), BoxSize=np.asarray([box] * 3), device="cuda",
                               fftss=(0, n))
    for _ in range(max(1, args.warmup - 2)):
        snapmap.makemap(snap, "nT", pm, save=False, return_tensor=True)
    torch.cuda.synchronize()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        m = snapmap.makemap(snap, "nT", pm, save=False, return_tensor=True)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    sec = float(np.median(ts))
    k = max(1, N // 100)
    sample = {f: v[:k] for f, v in fields.items()}
    t0 = time.perf_counter()
    osm.makemap(sample, "nT", (n,) * 3, [box] * 3, 2.0)
    cpu = (time.perf_counter() - t0) * (N / k)
    print(json.dumps({"metric": "snapshot-map ingestion (makemap, kind nT)", "value": N / sec, "unit": "particles/s",
                      "seconds": sec, "host_gbs": N * 28 / sec / 1e9, "nparts": N, "nmesh": n,
                      "data": "synthetic uniform gas particles (seeded)", "map_sum": float(m.double().sum()),
                      "cpu_baseline": {"value": N / cpu, "unit": "particles/s", "cores": 1, "kind": "port",
                                       "sample": f"oracle numpy makemap on {k} particles, scaled"}}), flush=True)
    return 0


def run_loss_ext(args):
    """The fused step with the rest of model.py's loss (smoothing n = 0.5 of
    the residual, a validation mask) next to the plain-loss step on the same
    workload: ms per step of each."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    dev = torch.device("cuda", 0)
    n = args.n
    params = synth.default_params(2)
    pos, box = make_workload(n, dev)
    target = make_target(pos, n, box, params, dev)
    mv = torch.from_numpy(np.random.default_rng(3).integers(0, 2, (n,) * 3).astype(np.float32)).to(dev)
    out = {"workload": f"clustered {n}^3, 2 sm layers, L1 loss", "nmesh": n}
    for name, kw, extra in (("plain_loss", {}, {}), ("smooth_0.5_valid", {"n": 0.5}, {"maskvalid": mv})):
        step = FusedLDL(n, box, pos.shape[0], nstep=2, kind="sm", L1=True, device=dev, **kw)
        step(pos, params, target, **extra)
        step.capture(pos, target, **extra)
        for _ in range(args.warmup):
            step.replay(params)
        torch.cuda.synchronize()
        st = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            step.replay(params)
        e1.record(st)
        torch.cuda.synchronize()
        out[name] = {"ms_per_step": e0.elapsed_time(e1) / args.steps, "loss": float(step.out[0]),
                     "lossv": float(step.lossv), "graph_kernels": step.graph_kernels()}
        del step
    print(json.dumps(out), flush=True)
    return 0


def run_hi(args):
    """The fused step of the "HI" kind (star-map source in every layer,
    depletion map) next to the "sm" step on the same workload: ms per step
    of each, through captured graphs."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    dev = torch.device("cuda", 0)
    n = args.n
    pos, box = make_workload(n, dev)
    target = make_target(pos, n, box, synth.default_params(2), dev)
    sm = torch.from_numpy(synth.star_map(n, box, seed=5)).to(dev)
    out = {"workload": f"clustered {n}^3, 2 layers, L1 loss; star map nonzero in 5 % of the cells", "nmesh": n}
    for kind, params in (("sm", synth.default_params(2)), ("HI", synth.default_params_hi(2))):
        step = FusedLDL(n, box, pos.shape[0], nstep=2, kind=kind, L1=True, device=dev,
                        starmap=sm if kind == "HI" else None)
        step(pos, params, target)
        step.capture(pos, target)
        for _ in range(args.warmup):
            step.replay(params)
        torch.cuda.synchronize()
        st = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            step.replay(params)
        e1.record(st)
        torch.cuda.synchronize()
        out[kind] = {"ms_per_step": e0.elapsed_time(e1) / args.steps, "loss": float(step.out[0]),
                     "grad_norm": float(step.out[1:].norm()), "graph_kernels": step.graph_kernels(),
                     "workspace_gb": step.workspace_bytes / 1e9}
        if kind == "HI" and not args.no_plain:
            # the plain FP32 primitives one by one (JERALDModel, torch autograd)
            from jerald_gb300.model import JERALDModel
            from jerald_gb300.pmesh import PMesh
            grad = step.out[1:].cpu().numpy()
            del step
            pm = PMesh(n, box, device=dev, dtype=torch.float32)
            model = JERALDModel(pos, target, pm, Nstep=2, kind="HI", L1=True, starmap=sm)
            pt = torch.as_tensor(params, dtype=torch.float32)
            model.loss_and_grad(pt)
            torch.cuda.synchronize()
            e0.record(st)
            for _ in range(3):
                lp, gp = model.loss_and_grad(pt)
            e1.record(st)
            torch.cuda.synchronize()
            gp = gp.cpu().numpy()
            out[kind]["plain_ms_per_step"] = e0.elapsed_time(e1) / 3
            out[kind]["speedup_vs_plain"] = out[kind]["plain_ms_per_step"] / out[kind]["ms_per_step"]
            out[kind]["grad_rel_diff_vs_plain_f32"] = float(np.linalg.norm(grad - gp) / np.linalg.norm(gp))
            del model, pm
        else:
            del step
    print(json.dumps(out), flush=True)
    return 0


def run_precision(args):
    """Precision study on the benchmark workload: the fused FP32 step and the
    plain FP32 primitives against the FP64 oracle (the CPU restatement of the
    reference's pipeline) on the same positions and target; L1 loss in both
    gradient conventions and L2 loss.  The fused step is also compared with
    the FP64 oracle that keeps positions in float32 between layers
    (`*_vs_f32pos`), which separates the error of storing positions in
    float32 from the kernels' own.  Prints one JSON object."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from jerald_gb300 import synth
    from jerald_gb300 import jaxpops_bind as jpo
    from jerald_gb300.ldl import FusedLDL
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    from oracle import cic as ocic
    from oracle import fft as offt
    from oracle import ldl as oldl
    threads = os.cpu_count() or 1
    offt.set_workers(threads)
    ocic.set_threads(threads)
    oldl.set_threads(threads)
    dev = torch.device("cuda", 0)
    n, nstep = args.n, args.nstep
    params = synth.default_params(nstep)
    pos_h, box = host_workload(n, seed=0)
    pos = torch.from_numpy(pos_h).to(dev)
    target = make_target(pos, n, box, params, dev, nstep)
    tgt_h = target.cpu().numpy().astype(np.float64)
    X = pos_h.astype(np.float64)
    ib = 5 * nstep + 2

    def compare(g, g64):
        g, g64 = np.asarray(g, np.float64), np.asarray(g64, np.float64)
        rel = np.abs(g - g64) / np.abs(g64)
        return {"grad_norm_rel_err": float(np.linalg.norm(g - g64) / np.linalg.norm(g64)),
                "grad_rel_err": rel.tolist(),
                "grad_rel_err_max_excl_b": float(np.delete(rel, ib).max()),
                "grad_abs_err_b": float(abs(g[ib] - g64[ib]))}

    res = {"precision": True, "n": n, "nparts": int(len(X)), "oracle_threads": threads}
    for L1 in (True, False):
        o = oldl.LDLOracle((n,) * 3, box, kind="sm", L1=L1)
        t0 = time.perf_counter()
        l64 = o.forward(params, X, tgt_h, nstep)
        g64 = {m: o.backward(m) for m in ("reference", "true")}
        t_oracle = time.perf_counter() - t0
        F, diff = o.cache["F"], o.cache["diff"]
        ties = int(np.count_nonzero(np.abs(diff) < 1e-5 * np.abs(F)))
        key = "L1" if L1 else "L2"
        res[key] = {"loss_f64": l64, "oracle_s": t_oracle, "grad_f64": {m: g.tolist() for m, g in g64.items()}}
        if L1:
            res[key]["near_tie_pixels"] = ties
            res[key]["b_grad_tie_bound"] = 2.0 * ties / diff.size
        del o
        o = oldl.LDLOracle((n,) * 3, box, kind="sm", L1=L1, pos_dtype=np.float32)
        l64f = o.forward(params, X, tgt_h, nstep)
        g64f = {m: o.backward(m) for m in ("reference", "true")}
        res[key]["loss_f64_f32pos"] = l64f
        del o
        for mode in ("reference", "true"):
            step = FusedLDL(n, box, pos.shape[0], nstep=nstep, kind="sm", L1=L1, grad_mode=mode, device=dev)
            l32, g32 = step(pos, params, target)
            l32, g32 = float(l32), g32.cpu().numpy()
            del step
            torch.cuda.empty_cache()
            res[key][f"fused_{mode}"] = {"loss_rel_err": abs(l32 - l64) / abs(l64), **compare(g32, g64[mode])}
            res[key][f"fused_{mode}_vs_f32pos"] = {"loss_rel_err": abs(l32 - l64f) / abs(l64f),
                                                   **compare(g32, g64f[mode])}
        if L1:
            pm = PMesh(n, box, device=dev, dtype=torch.float32)
            model = JERALDModel(pos, target, pm, Nstep=nstep, kind="sm")
            lp, gp = model.loss_and_grad(torch.as_tensor(params, dtype=torch.float32))
            res[key]["plain_f32_reference"] = {"loss_rel_err": abs(float(lp) - l64) / abs(l64),
                                               **compare(gp.cpu().numpy(), g64["reference"])}
            del model, pm
            torch.cuda.empty_cache()
    jpo.set_fft_adjoint("reference")
    print(json.dumps(res), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512, help="mesh size per axis (workload scale)")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain primitive path")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile", action="store_true",
                    help="run only eager fused steps (warmup + steps) on the workload, for ncu")
    ap.add_argument("--precision", action="store_true",
                    help="compare the fused FP32 step with the FP64 primitive pipeline on the workload")
    ap.add_argument("--paint", default="atomic", choices=["atomic", "warp", "tiled"])
    ap.add_argument("--x-radix", type=int, default=8, choices=[8, 16],
                    help="x passes' schedule radix where radix-8 ones fit")
    ap.add_argument("--min-cols", type=int, default=0, choices=[0, 4, 8, 16],
                    help="narrowest pipelined tile (0: automatic)")
    ap.add_argument("--nstep", type=int, default=2, help="displacement layers")
    ap.add_argument("--batch", type=int, default=0,
                    help="instead of the main workload: N boxes of mixed meshes in one graph (prints its own line)")
    ap.add_argument("--streams", type=int, default=4, help="parallel graph branches of the --batch workload")
    ap.add_argument("--recompute", action="store_true",
                    help="memory plan: one force-mesh slot, recomputed in the adjoint")
    ap.add_argument("--snapmap", type=int, default=0,
                    help="instead of the main workload: makemap of N synthetic gas particles (prints its own line)")
    ap.add_argument("--loss-ext", action="store_true",
                    help="instead of the main workload: the fused step with residual smoothing and a validation mask")
    ap.add_argument("--hi", action="store_true",
                    help="instead of the main workload: the fused HI-kind step next to the sm step")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)
    if args.precision:
        return run_precision(args)
    if args.batch:
        return run_batch(args)
    if args.snapmap:
        return run_snapmap(args)
    if args.loss_ext:
        return run_loss_ext(args)
    if args.hi:
        return run_hi(args)

    import torch
    from jerald_gb300 import replicas
    world, rank, local = replicas.world()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import __graft_entry__
    __graft_entry__.build()
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL

    n, nstep = args.n, args.nstep
    params = synth.default_params(nstep)
    pos, box = make_workload(n, dev, seed=replicas.replica_seed(rank))
    target = make_target(pos, n, box, params, dev, nstep)
    N = pos.shape[0]
    step = FusedLDL(n, box, N, nstep=nstep, kind="sm", L1=True, grad_mode="reference", paint_method=args.paint,
                    device=dev, recompute=args.recompute, x_radix=args.x_radix, min_cols=args.min_cols)
    step(pos, params, target)
    step.capture(pos, target)
    launches_per_step = step.graph_kernels()
    for _ in range(args.warmup):
        step.replay(params)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    st = torch.cuda.current_stream(dev)
    with ClockSampler(local) as clk:
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            step.replay(params)
        e1.record(st)
        barrier()
    value, ms = replicas.aggregate_rate(e0.elapsed_time(e1) / args.steps, dev)
    loss, grad = step.out[0].item(), step.out[1:].cpu().numpy()
    assert step.error_word() == 0, "a pipelined pass gave up waiting for a copy"

    # e2e: host buffers -> device, step, loss+grads -> host, through the
    # public host feed (copies of step k+1 overlap the compute of step k)
    from jerald_gb300.ldl import HostFeed
    pos_h = pos.cpu().pin_memory()
    tgt_h = target.cpu().pin_memory()
    h2d = pos_h.numel() * 4 + tgt_h.numel() * 4
    feed = HostFeed(step)
    out_h = torch.empty((max(args.steps, args.warmup), step.out.numel()), dtype=torch.float64).pin_memory()
    d2h = step.out.numel() * 8
    feed.run([(pos_h, tgt_h)] * args.warmup, params, out_h)
    barrier()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(st)
    feed.run([(pos_h, tgt_h)] * args.steps, params, out_h)
    e3.record(st)
    barrier()
    e2e_loss_err = abs(float(out_h[args.steps - 1, 0]) - loss) / abs(loss)
    e2e_value, ms_e2e = replicas.aggregate_rate(e2.elapsed_time(e3) / args.steps, dev)
    del pos_h, tgt_h, feed

    extra = {}
    peak, peak_kind = _peaks()
    kern = time_primitives(pos, n, box, steps=5, warmup=3) if rank == 0 else {}
    prof = ROOT / "profiles" / "traffic.json"
    traffic = json.loads(prof.read_text()) if prof.exists() else {}
    dominant = "paint"
    dk = kern.get(dominant, {"gbs": 0.0, "algorithmic_bytes": 0})
    roofline = {"bound": "hbm", "achieved": dk["gbs"], "peak": peak, "unit": "GB/s",
                "frac": dk["gbs"] / peak, "traffic": traffic.get(dominant, {}).get("bytes_per_launch_full"),
                "kernel": dominant, "peak_kind": peak_kind,
                "kernels": {k: {"gbs": v["gbs"], "frac": v["gbs"] / peak, "ms": v["ms"]} for k, v in kern.items()}}

    if not args.no_plain and rank == 0 and n <= 512:
        from jerald_gb300.model import JERALDModel
        from jerald_gb300.pmesh import PMesh
        pm = PMesh(n, box, device=dev, dtype=torch.float32)
        model = JERALDModel(pos, target, pm, Nstep=nstep, kind="sm")
        pt = torch.as_tensor(params, dtype=torch.float32)
        lp, gp = model.loss_and_grad(pt)
        torch.cuda.synchronize()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record(st)
        kp = 3
        for _ in range(kp):
            lp, gp = model.loss_and_grad(pt)
        e5.record(st)
        torch.cuda.synchronize()
        plain_ms = e4.elapsed_time(e5) / kp
        gp = gp.cpu().numpy()
        extra["plain_ms_per_step"] = plain_ms
        extra["speedup_vs_plain"] = plain_ms / ms
        rel = np.abs(grad - gp) / np.maximum(np.abs(gp), 1e-6 * np.abs(gp).max())
        extra["grad_rel_diff_vs_plain"] = float(rel.max())
        extra["loss_rel_diff_vs_plain"] = abs(loss - float(lp)) / abs(float(lp))
        del model, pm

    cpu = None
    if not args.no_cpu and rank == 0:
        try:
            cpu = cpu_baseline_sample(min(256, n), n, steps=3)
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}

    ysb = yardstick_bytes(N, nstep)
    extra["yardstick"] = {"bytes_per_step": ysb, "gbs": ysb / ms / 1e6, "frac": ysb / ms / 1e6 / peak,
                          "note": "plain-primitive byte yardstick (332*nstep+64)*N over the fused step time"}
    extra["workspace_gb"] = step.workspace_bytes / 1e9
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Zel'dovich lattice + Gaussian halos)",
                "config": workload_config(n, N, box, nstep, args.recompute, world),
                "roofline": roofline, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e,
                        "path": "FusedLDL + HostFeed (double-buffered pinned-host copies)",
                        "loss_rel_diff_vs_device_run": e2e_loss_err},
                "gpu_launches": (launches_per_step if launches_per_step is not None
                                 else count_launches(nstep, "sm", False, args.recompute)) * args.steps,
                "clocks": clk.summary(), "loss": loss, **extra}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
