"""GPU tests of the multi-box batch: one graph replay evaluates every box as
its own fused step would, boxes of different meshes (power-of-two and mixed
radix), kinds and parameters side by side on parallel graph branches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _boxes():
    from jerald_gb300 import synth
    from jerald_gb300.batch import Box
    out, params = [], []
    for i, (n, kind) in enumerate([(32, "sm"), (48, "sm"), (64, "dm"), (32, "sm")]):
        L = 100.0 * n / 64
        pos = synth.zeldovich(n, L, 0.5, seed=40 + i, device="cuda").contiguous()
        tgt = torch.from_numpy(synth.lognormal_noise((n, n, n), 0.1, seed=60 + i).astype(np.float32)).cuda()
        out.append(Box(n, L, pos, tgt, kind=kind, config={"pipelined": True, "paint_method": "atomic"}))
        p = synth.default_params(2) * (1.0 + 0.1 * i)
        params.append(p if kind == "sm" else p[:10])
    return out, params


def test_batch_graph_matches_single_box_steps():
    from jerald_gb300.batch import FusedLDLBatch
    from jerald_gb300.ldl import FusedLDL
    boxes, params = _boxes()
    batch = FusedLDLBatch(boxes, streams=3, tune=False)
    batch.capture()
    res = [(float(l), g.cpu().numpy().copy()) for l, g in batch.replay(params)]
    torch.cuda.synchronize()
    for b, p, (lb, gb) in zip(boxes, params, res):
        single = FusedLDL(b.nmesh, b.box, b.pos.shape[0], nstep=2, kind=b.kind)
        ls, gs = single(b.pos, p, b.target)
        torch.cuda.synchronize()
        assert abs(lb - float(ls)) <= 1e-6 * abs(float(ls))
        gs = gs.cpu().numpy()
        assert np.abs(gb - gs).max() <= 1e-4 * np.abs(gs).max()
    k = batch.graph_kernels()
    assert k is None or k >= 4 * 30
    # new parameters through the same graph
    p2 = [p * 0.9 for p in params]
    res2 = [float(l) for l, _ in batch.replay(p2)]
    torch.cuda.synchronize()
    assert all(abs(a - b[0]) > 1e-7 * abs(b[0]) for a, b in zip(res2, res))


def test_autotune_picks_a_candidate_and_caches():
    from jerald_gb300 import batch as bt
    from jerald_gb300 import synth
    n, L = 32, 50.0
    pos = synth.zeldovich(n, L, 0.5, seed=3, device="cuda").contiguous()
    tgt = torch.ones((n, n, n), device="cuda")
    bt._CACHE.clear()
    t = bt.autotune(n, L, pos, tgt, synth.default_params(2), reps=2)
    assert {"pipelined", "paint_method", "ms", "timings", "clustering_level"} <= set(t)
    assert len(t["timings"]) >= len(bt.CANDIDATES)
    assert t["clustering_level"] == 0
    assert bt.autotune(n, L, pos, tgt, synth.default_params(2)) is t


@pytest.mark.parametrize("cfg", [{"x_radix": 16}, {"min_cols": 4}, {"min_cols": 8}, {"min_cols": 16},
                                 {"paint_method": "tiled", "bin_tile": 8},
                                 {"paint_method": "tiled", "bin_tile": 20}],
                         ids=["xr16", "cols4", "cols8", "cols16", "bin8", "bin20"])
def test_schedule_options_give_the_same_step(cfg):
    """Every schedule the autotuner can pick computes the same step: loss
    within 1e-6 and gradient within 1e-4 of the largest component of the
    default configuration's, at 64^3 and 128^3."""
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    for n in (64, 128):
        L = 100.0 * n / 64
        pos = synth.zeldovich(n, L, 0.5, seed=7, device="cuda").contiguous()
        tgt = torch.from_numpy(synth.lognormal_noise((n, n, n), 0.1, seed=8).astype(np.float32)).cuda()
        p = synth.default_params(2)
        l0, g0 = FusedLDL(n, L, pos.shape[0])(pos, p, tgt)
        f = FusedLDL(n, L, pos.shape[0], **cfg)
        l1, g1 = f(pos, p, tgt)
        torch.cuda.synchronize()
        assert f.error_word() == 0
        assert abs(float(l1) - float(l0)) <= 1e-6 * abs(float(l0))
        g0, g1 = g0.cpu().numpy(), g1.cpu().numpy()
        assert np.abs(g1 - g0).max() <= 1e-4 * np.abs(g0).max()


def test_batch_mixed_radix_boxes_match_fp64_oracle():
    """Boxes of 96^3 and 192^3 (mixed radix: generic FFT passes) in one
    batch graph, each against the FP64 oracle that keeps the positions in
    float32 between layers as the FP32 step does: loss within 1e-6,
    gradient within 1e-4 norm-wise; and against the plain FP64 oracle within
    5e-5 and 1e-3 (at 192^3, a 300-unit box, the layers' displacements of
    ~4e-5 units are about one float32 ulp of the coordinates, and their
    rounding alone moves the FP64 loss by 1.4e-5)."""
    import os
    from jerald_gb300 import synth
    from jerald_gb300.batch import Box, FusedLDLBatch
    from oracle import cic as ocic
    from oracle import fft as offt
    from oracle import ldl as oldl
    t = os.cpu_count() or 1
    offt.set_workers(t)
    ocic.set_threads(t)
    oldl.set_threads(t)
    try:
        boxes, params, X64 = [], [], []
        for i, n in enumerate((96, 192)):
            L = 100.0 * n / 64
            X = synth.zeldovich(n, L, 0.5, seed=80 + i, dtype=np.float32)
            p = synth.default_params(2) * (1.0 + 0.2 * (i - 0.5))
            tgt = synth.lognormal_noise((n, n, n), 0.1, seed=90 + i).astype(np.float32)
            boxes.append(Box(n, L, torch.from_numpy(X).cuda(), torch.from_numpy(tgt).cuda()))
            params.append(p)
            X64.append(X.astype(np.float64))
        batch = FusedLDLBatch(boxes, streams=2, tune=False)
        batch.capture()
        res = [(float(l), g.cpu().numpy().copy()) for l, g in batch.replay(params)]
        torch.cuda.synchronize()
        for b, p, X, (lb, gb) in zip(boxes, params, X64, res):
            n = int(b.nmesh)
            tgt = b.target.cpu().numpy().astype(np.float64)
            o = oldl.LDLOracle((n,) * 3, b.box, kind="sm", L1=True, pos_dtype=np.float32)
            lo, go = o.loss_and_grad(p, X, tgt, 2, mode="reference")
            assert abs(lb - lo) <= 1e-6 * abs(lo)
            assert np.linalg.norm(gb - go) / np.linalg.norm(go) < 1e-4
            o = oldl.LDLOracle((n,) * 3, b.box, kind="sm", L1=True)
            lo, go = o.loss_and_grad(p, X, tgt, 2, mode="reference")
            assert abs(lb - lo) <= 5e-5 * abs(lo)
            assert np.linalg.norm(gb - go) / np.linalg.norm(go) < 1e-3
    finally:
        offt.set_workers(1)
        ocic.set_threads(1)
        oldl.set_threads(1)
