"""GPU parity of the fused LDL step (C ABI jld_ldl_step_f32 via FusedLDL)
against the FP64 oracle, the plain primitive path, and its own CUDA graph.

Tolerances (FP32 bulk, FP64 reductions): loss within 1e-5 relative, each
gradient component within 1e-3 relative at these small meshes (FD-level
quantities; components below 1e-6 of the largest are compared absolutely).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle.ldl import LDLOracle  # noqa: E402


def _case(n, box, kind, L1, seed, rms=0.5, mask=False, nstep=2):
    from jerald_gb300 import synth
    X = synth.zeldovich(n, box, rms, seed=seed, dtype=np.float32).astype(np.float64)
    p = synth.default_params(nstep)
    if kind == "dm":
        p = p[:5 * nstep]
    o = LDLOracle((n, n, n), box, kind=kind, L1=L1)
    o.forward(p, X, np.ones((n, n, n)), nstep)
    tgt = (o.cache["F"] * synth.lognormal_noise((n, n, n), 0.1, seed + 1)).astype(np.float32)
    m = np.random.default_rng(seed + 2).integers(0, 2, (n, n, n)).astype(np.float32) if mask else None
    return X, p, tgt, o, m


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-6 * np.abs(b).max())


def _fused(n, box, N, kind, L1, mode, nstep=2, paint="atomic"):
    from jerald_gb300.ldl import FusedLDL
    return FusedLDL(n, box, N, nstep=nstep, kind=kind, L1=L1, grad_mode=mode, paint_method=paint)


@pytest.mark.parametrize("kind,L1,mask", [("sm", True, False), ("sm", False, True), ("dm", False, False)])
@pytest.mark.parametrize("mode", ["reference", "true"])
def test_fused_matches_fp64_oracle(kind, L1, mask, mode):
    n, box = 32, 100.0
    X, p, tgt, o, m = _case(n, box, kind, L1, 21, mask=mask)
    loss_o, g_o = o.loss_and_grad(p, X, tgt.astype(np.float64), 2,
                                  mask=None if m is None else m.astype(np.float64), mode=mode)
    f = _fused(n, box, len(X), kind, L1, mode)
    pos = torch.from_numpy(X.astype(np.float32)).cuda()
    t = torch.from_numpy(tgt).cuda()
    mk = torch.from_numpy(m).cuda() if m is not None else None
    loss, g = f(pos, p, t, mk)
    torch.cuda.synchronize()
    assert abs(float(loss) - loss_o) <= 1e-5 * abs(loss_o)
    g = g.cpu().numpy()
    # norm-wise within 1e-3; per component within 1e-2 (the nu and kh gradients
    # are small differences of large spectral sums, so FP32 FFT rounding shows
    # there first)
    assert np.linalg.norm(g - g_o) / np.linalg.norm(g_o) < 1e-3
    assert _rel(g, g_o).max() < 1e-2


@pytest.mark.parametrize("recompute", [False, True])
def test_fused_three_layers_memory_plans(recompute):
    # nstep = 3: the adjoint needs the force meshes of layers 1 and 2; with
    # recompute they share one slot and layer 1's is rebuilt from its density
    n, box = 32, 100.0
    X, p, tgt, o, _ = _case(n, box, "sm", True, 31, nstep=3)
    p = np.concatenate([synth_params3(), p[-3:]])
    loss_o, g_o = o.loss_and_grad(p, X, tgt.astype(np.float64), 3, mode="true")
    from jerald_gb300.ldl import FusedLDL
    f = FusedLDL(n, box, len(X), nstep=3, kind="sm", L1=True, grad_mode="true", recompute=recompute)
    pos = torch.from_numpy(X.astype(np.float32)).cuda()
    loss, g = f(pos, p, torch.from_numpy(tgt).cuda())
    torch.cuda.synchronize()
    assert f.error_word() == 0
    assert abs(float(loss) - loss_o) <= 1e-5 * abs(loss_o)
    g = g.cpu().numpy()
    assert np.linalg.norm(g - g_o) / np.linalg.norm(g_o) < 1e-3
    assert _rel(g, g_o).max() < 1e-2
    if recompute:
        full = FusedLDL(n, box, len(X), nstep=3, kind="sm", L1=True, grad_mode="true")
        assert f.workspace_bytes < full.workspace_bytes


def synth_params3():
    # three layers with different strengths (alpha, gamma, kh, kl, nu)
    return np.array([0.05, 1.0, 0.5, 2.0, 1.0, 0.04, 0.9, 0.6, 1.8, 1.1, 0.03, 1.1, 0.5, 2.2, 0.9])


def test_fused_positions_match_oracle_layers():
    n, box = 32, 100.0
    X, p, tgt, o, _ = _case(n, box, "sm", True, 5)
    f = _fused(n, box, len(X), "sm", True, "reference")
    pos = torch.from_numpy(X.astype(np.float32)).cuda()
    f(pos, p, torch.from_numpy(tgt).cuda())
    torch.cuda.synchronize()
    # X_1 of the oracle: rerun its first layer
    X1, _ = o.layer_forward(X, p[:5], float(n ** 3) / len(X))
    got = f.positions(1).cpu().numpy().astype(np.float64)
    disp = np.abs(X1 - X).max()
    assert np.abs(got - X1).max() < 1e-4 * max(disp, 1.0) + 2e-5 * box


@pytest.mark.parametrize("L1", [True, False])
def test_fused_matches_plain_primitives(L1):
    # Both paths in FP32.  With the L1 loss the gradient depends on
    # sign(F - t) per cell: rounding-level differences between the two paths
    # flip a few cells (each moves d/db by 2/Npix), so the L1 case compares
    # the loss and the gradient norm-wise; the smooth L2 case compares every
    # gradient component.
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    n, box = 64, 200.0
    X, p, tgt, o, _ = _case(n, box, "sm", L1, 9, rms=1.0)
    pos = torch.from_numpy(X.astype(np.float32)).cuda()
    t = torch.from_numpy(tgt).cuda()
    pm = PMesh(n, box, dtype=torch.float32)
    model = JERALDModel(pos, t, pm, Nstep=2, kind="sm", L1=L1)
    lp, gp = model.loss_and_grad(torch.from_numpy(p.astype(np.float32)))
    f = _fused(n, box, len(X), "sm", L1, "reference")
    lf, gf = f(pos, p, t)
    torch.cuda.synchronize()
    assert abs(float(lf) - float(lp)) <= 2e-5 * abs(float(lp))
    gf, gp = gf.cpu().numpy(), gp.cpu().numpy().astype(np.float64)
    if L1:
        assert np.linalg.norm(gf - gp) / np.linalg.norm(gp) < 5e-2
    else:
        assert _rel(gf, gp).max() < 5e-3


def test_tiled_scatters_match_atomic_scatters_clustered():
    # clustered particles (halos of many particles per cell), positions in
    # input order and well outside the box
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    n, box = 64, 100.0
    X = synth.clustered(n, box, seed=4, extra_frac=0.3, nhalo=20).astype(np.float32)
    X[:100] += 3 * box
    X[100:200] -= 2.5 * box
    pos = torch.from_numpy(X).cuda()
    t = torch.ones((n, n, n), device="cuda")
    p = synth.default_params(2)
    out = {}
    for m in ("atomic", "tiled"):
        f = FusedLDL(n, box, len(X), nstep=2, kind="sm", grad_mode="true", paint_method=m)
        lo, g = f(pos, p, t)
        torch.cuda.synchronize()
        out[m] = (float(lo), g.cpu().numpy(), f.positions(2).clone())
    assert abs(out["tiled"][0] - out["atomic"][0]) <= 1e-5 * abs(out["atomic"][0])
    assert _rel(out["tiled"][1], out["atomic"][1]).max() < 1e-3
    assert float((out["tiled"][2] - out["atomic"][2]).abs().max()) < 1e-3


@pytest.mark.parametrize("paint", ["atomic", "warp", "tiled"])
def test_fused_graph_replay_matches_eager(paint):
    n, box = 32, 100.0
    X, p, tgt, o, _ = _case(n, box, "sm", True, 13)
    f = _fused(n, box, len(X), "sm", True, "reference", paint=paint)
    pos = torch.from_numpy(X.astype(np.float32)).cuda()
    t = torch.from_numpy(tgt).cuda()
    l0, g0 = [v.clone() for v in f(pos, p, t)]
    f.capture(pos, t)
    l1, g1 = [v.clone() for v in f.replay(p)]
    torch.cuda.synchronize()
    assert abs(float(l1) - float(l0)) <= 1e-6 * abs(float(l0))
    # run-to-run atomic summation order only
    assert _rel(g1.cpu().numpy(), g0.cpu().numpy()).max() < 1e-3
    # new parameters through the same graph
    p2 = p * 1.1
    l2, g2 = [v.clone() for v in f.replay(p2)]
    l3, g3 = [v.clone() for v in f(pos, p2, t)]
    torch.cuda.synchronize()
    assert abs(float(l2) - float(l3)) <= 1e-6 * abs(float(l3))
    assert abs(float(l2) - float(l0)) > 1e-6 * abs(float(l0))


@pytest.mark.parametrize("n", [32, 64, 96, 128, 192])
def test_pipelined_passes_match_generic_passes(n):
    # L2 loss: with L1, rounding-level differences between two valid FP32
    # forward paths flip sign(F - t) in a few cells and move d/db visibly
    box = 100.0
    X, p, tgt, o, _ = _case(n, box, "sm", False, 17)
    pos = torch.from_numpy(X.astype(np.float32)).cuda()
    t = torch.from_numpy(tgt).cuda()
    fa = _fused(n, box, len(X), "sm", False, "true")
    from jerald_gb300.ldl import FusedLDL
    fb = FusedLDL(n, box, len(X), nstep=2, kind="sm", L1=False, grad_mode="true", pipelined=False)
    la, ga = [v.clone() for v in fa(pos, p, t)]
    lb, gb = [v.clone() for v in fb(pos, p, t)]
    torch.cuda.synchronize()
    assert fa.error_word() == 0 and fb.error_word() == 0
    assert abs(float(la) - float(lb)) <= 1e-6 * abs(float(lb))
    assert _rel(ga.cpu().numpy(), gb.cpu().numpy()).max() < 1e-3
    xa, xb = fa.positions(2), fb.positions(2)
    assert float((xa - xb).abs().max()) < 1e-4


@pytest.mark.parametrize("nm", [(512, 16, 32), (16, 512, 64), (64, 32, 1024), (1024, 16, 32), (96, 192, 48),
                                (192, 96, 96), (48, 64, 384)])
def test_pipelined_passes_match_generic_non_cubic(nm):
    # long x / y / z lines: narrower pipelined tiles (two CTAs per SM) and
    # few rows per z tile
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    rng = np.random.default_rng(23)
    box = np.asarray(nm, dtype=np.float64) * 1.5
    N = int(np.prod(nm))
    X = (rng.uniform(0, 1, (N, 3)) * box).astype(np.float32)
    pos = torch.from_numpy(X).cuda()
    t = torch.from_numpy(synth.lognormal_noise(nm, 0.1, seed=3).astype(np.float32)).cuda()
    p = synth.default_params(2)
    fa = FusedLDL(nm, box, N, nstep=2, kind="sm", L1=False, grad_mode="true")
    fb = FusedLDL(nm, box, N, nstep=2, kind="sm", L1=False, grad_mode="true", pipelined=False)
    la, ga = [v.clone() for v in fa(pos, p, t)]
    lb, gb = [v.clone() for v in fb(pos, p, t)]
    torch.cuda.synchronize()
    assert fa.error_word() == 0
    assert abs(float(la) - float(lb)) <= 1e-6 * abs(float(lb))
    assert _rel(ga.cpu().numpy(), gb.cpu().numpy()).max() < 1e-3


def test_fused_rejects_bad_arguments():
    from jerald_gb300 import _lib
    from jerald_gb300.ldl import FusedLDL
    with pytest.raises(ValueError):
        FusedLDL(16, 10.0, 100, kind="HI")
    f = FusedLDL(16, 10.0, 4096, kind="sm")
    pos = torch.zeros((4096, 3), device="cuda")
    with pytest.raises(ValueError):
        f(pos, np.zeros(3), torch.zeros((16, 16, 16), device="cuda"))
    f.grad_mode = "bogus"
    with pytest.raises(KeyError):
        f(pos, np.zeros(13), torch.zeros((16, 16, 16), device="cuda"))
    with pytest.raises(_lib.JLDError):
        FusedLDL((16, 16, 15), 10.0, 100)


def test_host_feed_matches_eager_steps():
    # three steps fed from pinned host memory (copies overlapped with the
    # previous step) give each step's own loss and gradient
    from jerald_gb300.ldl import FusedLDL, HostFeed
    n, box = 32, 100.0
    cases = [_case(n, box, "sm", True, s) for s in (41, 42, 43)]
    p = cases[0][1]
    f = FusedLDL(n, box, len(cases[0][0]), nstep=2, kind="sm", L1=True)
    feed = HostFeed(f)
    inputs = [(torch.from_numpy(X.astype(np.float32)).pin_memory(), torch.from_numpy(t).pin_memory())
              for X, _, t, _, _ in cases]
    out = torch.zeros((3, 1 + f.nparams), dtype=torch.float64).pin_memory()
    feed.run(inputs, p, out)
    torch.cuda.synchronize()
    for k, (ph, th) in enumerate(inputs):
        lo, go = f(ph.cuda(), p, th.cuda())
        torch.cuda.synchronize()
        assert abs(float(out[k, 0]) - float(lo)) <= 1e-6 * abs(float(lo))
        # float atomics sum in a different order on every run; d/d alpha is a
        # small difference of large sums, so allow 1e-3 per component
        assert _rel(out[k, 1:].numpy(), go.cpu().numpy()).max() < 1e-3
    assert float(out[0, 0]) != float(out[1, 0])


@pytest.mark.parametrize("case", ["sm_smooth_L1", "sm_smooth_L2_masks", "sm_index_field2_valid", "dm_smooth_L2"])
@pytest.mark.parametrize("mode", ["reference", "true"])
def test_fused_loss_options_match_plain_f64(case, mode):
    """The rest of model.py's loss in the fused step -- residual smoothing by
    |k|^-n + 1, the map exponent and second field, the validation loss --
    against the FP64 plain path on the same inputs (loss and validation loss
    within 1e-5, gradient 1e-3 norm-wise and 1e-2 per component) and the loss
    against the FP64 oracle's forward (1e-5)."""
    from jerald_gb300 import jaxpops_bind as jpo
    from jerald_gb300 import synth
    from jerald_gb300.ldl import FusedLDL
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    from oracle.ldl import model_loss
    n, box = 32, 100.0
    rng = np.random.default_rng(5)
    X = synth.zeldovich(n, box, 0.5, seed=6, dtype=np.float32).astype(np.float64)
    kind = "dm" if case.startswith("dm") else "sm"
    p = synth.default_params(2)[:10 if kind == "dm" else 13]
    tgt = rng.uniform(0.5, 1.5, (n,) * 3)
    if kind == "dm":
        # the dm map has mean 1 whatever the parameters (the paint conserves
        # mass), so a residual with a nonzero mean would put the loss in the
        # k = 0 mode, weighted (1e-8)^-n + 1, whose gradient is exactly zero
        # and drowns the rest in float32: give the target mean 1 as well
        tgt /= tgt.mean()
    tgt = tgt.astype(np.float32)
    L1 = "L1" in case
    o = dict(n=0.0, index=1.0, field2=None, mask=None, maskvalid=None)
    if "smooth" in case:
        # the k = 0 weight (1e-8)^-n + 1 multiplies the float32 rounding of
        # the residual's mean: 1e2 at n = 0.25, 1e4 at 0.5, 1e8 at 1
        o["n"] = 0.25 if kind == "dm" else 0.5
    if "masks" in case or "valid" in case:
        o["mask"] = rng.integers(0, 2, (n,) * 3).astype(np.float32)
        o["maskvalid"] = (1.0 - o["mask"]).astype(np.float32)
    if "index" in case:
        o["index"] = 2.0
        o["field2"] = rng.uniform(0.8, 1.2, (n,) * 3).astype(np.float32)
    ref, refv = model_loss((n,) * 3, box, kind, p, X, tgt.astype(np.float64), 2, L1=L1, n=o["n"], index=o["index"],
                           field2=o["field2"], mask=o["mask"], maskvalid=o["maskvalid"])
    d32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda() if a is not None else None  # noqa
    d64 = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64)).cuda() if a is not None else None  # noqa
    f = FusedLDL(n, box, len(X), nstep=2, kind=kind, L1=L1, grad_mode=mode, n=o["n"], index=o["index"])
    loss, g = f(d32(X), p, d32(tgt), d32(o["mask"]), d32(o["field2"]), d32(o["maskvalid"]))
    torch.cuda.synchronize()
    loss, lossv, g = float(loss), float(f.lossv), g.cpu().numpy()
    pm = PMesh(n, box, dtype=torch.float64)
    model = JERALDModel(d64(X), d64(tgt), pm, Nstep=2, kind=kind, L1=L1, n=o["n"], index=o["index"],
                        field2=d64(o["field2"]), masktrain=d64(o["mask"]), maskvalid=d64(o["maskvalid"]))
    jpo.set_fft_adjoint(mode)
    try:
        lp, lvp, gp = model.lossv_and_grad(torch.from_numpy(p))
    finally:
        jpo.set_fft_adjoint("reference")
    gp = gp.cpu().numpy()
    assert abs(loss - ref) <= 1e-5 * abs(ref), (loss, ref)
    assert abs(loss - float(lp)) <= 1e-5 * abs(float(lp))
    if o["maskvalid"] is not None:
        assert abs(lossv - refv) <= 1e-5 * abs(refv)
        assert abs(lossv - float(lvp)) <= 1e-5 * abs(float(lvp))
    else:
        assert lossv == 0.0
    assert np.linalg.norm(g - gp) / np.linalg.norm(gp) < 1e-3
    assert _rel(g, gp).max() < 1e-2
    # the same through a captured graph
    f.capture(d32(X), d32(tgt), d32(o["mask"]), d32(o["field2"]), d32(o["maskvalid"]))
    l2, g2 = f.replay(p)
    torch.cuda.synchronize()
    assert abs(float(l2) - loss) <= 1e-6 * abs(loss)
