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
    assert {"pipelined", "paint_method", "ms", "timings"} <= set(t)
    assert len(t["timings"]) == len(bt.CANDIDATES)
    assert bt.autotune(n, L, pos, tgt, synth.default_params(2)) is t
