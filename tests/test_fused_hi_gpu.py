"""GPU parity of the fused step's "HI" kind (jld_ldl_step_hi_f32 via
FusedLDL(kind="HI")): the star-map source in every layer's potential
(model.py:213-247) and the depletion map (model.py:313-336).

References, on the same float32 inputs:
* the FP64 plain model (JERALDModel(kind="HI"), primitives one by one,
  torch autograd) in both gradient conventions (jaxpops_bind's VJP rules and
  the exact adjoint): loss within 1e-5 relative, gradient within 1e-3
  norm-wise and 1e-2 per component (components below 1e-6 of the largest
  compared absolutely), as the other fused loss options;
* the FP64 oracle's forward (oracle.ldl.model_loss): loss within 1e-5.
Star maps: positive everywhere (lognormal), and zero outside 5 % of the cells
(where sm^e and its derivatives are 0).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-6 * np.abs(b).max())


def _inputs(n, box, sparse, seed, nstep=2):
    from jerald_gb300 import synth
    rng = np.random.default_rng(seed)
    X = synth.zeldovich(n, box, 0.5, seed=seed + 1, dtype=np.float32).astype(np.float64)
    sm = (synth.star_map(n, box, seed + 2) if sparse
          else np.exp(0.3 * rng.standard_normal((n,) * 3))).astype(np.float32)
    tgt = rng.uniform(0.5, 1.5, (n,) * 3).astype(np.float32)
    return X, synth.default_params_hi(nstep), sm, tgt


def _plain(n, box, X, p, sm, tgt, L1, mode, nstep=2, mask=None):
    from jerald_gb300 import jaxpops_bind as jpo
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    d64 = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64)).cuda() if a is not None else None  # noqa
    pm = PMesh(n, box, dtype=torch.float64)
    model = JERALDModel(d64(X), d64(tgt), pm, Nstep=nstep, kind="HI", L1=L1, starmap=d64(sm),
                        masktrain=d64(mask))
    jpo.set_fft_adjoint(mode)
    try:
        loss, g = model.loss_and_grad(torch.from_numpy(p))
    finally:
        jpo.set_fft_adjoint("reference")
    return float(loss), g.cpu().numpy()


def _fused(n, box, X, p, sm, tgt, L1, mode, nstep=2, mask=None, **kw):
    from jerald_gb300.ldl import FusedLDL
    d32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda() if a is not None else None  # noqa
    f = FusedLDL(n, box, len(X), nstep=nstep, kind="HI", L1=L1, grad_mode=mode, starmap=d32(sm), **kw)
    loss, g = f(d32(X), p, d32(tgt), d32(mask))
    torch.cuda.synchronize()
    assert f.error_word() == 0
    return f, float(loss), g.cpu().numpy()


@pytest.mark.parametrize("sparse", [False, True], ids=["lognormal", "sparse"])
@pytest.mark.parametrize("L1", [True, False], ids=["L1", "L2"])
@pytest.mark.parametrize("mode", ["reference", "true"])
def test_fused_hi_matches_plain_f64(sparse, L1, mode):
    from oracle.ldl import model_loss
    n, box = 32, 100.0
    X, p, sm, tgt = _inputs(n, box, sparse, 70 + 2 * sparse + L1)
    _, loss, g = _fused(n, box, X, p, sm, tgt, L1, mode)
    lp, gp = _plain(n, box, X, p, sm, tgt, L1, mode)
    ref, _ = model_loss((n,) * 3, box, "HI", p, X, tgt.astype(np.float64), 2, starmap=sm.astype(np.float64),
                        L1=L1)
    assert abs(loss - ref) <= 1e-5 * abs(ref), (loss, ref)
    assert abs(loss - lp) <= 1e-5 * abs(lp)
    assert g.shape == (10 * 2 + 12,)
    msg = np.array2string(_rel(g, gp), precision=2)
    assert np.linalg.norm(g - gp) / np.linalg.norm(gp) < 1e-3, msg
    assert _rel(g, gp).max() < 1e-2, msg


@pytest.mark.parametrize("variant", ["generic", "recompute_3", "mask_graph", "mesh_48"])
def test_fused_hi_variants(variant):
    """The generic (non-pipelined) passes, three layers with the recompute
    memory plan, a training mask through a captured CUDA graph, and a 48^3
    mesh (x and y passes on the 3 x 2^k pipelined schedules, the star map's
    own x pass included)."""
    n, box = (48, 150.0) if variant == "mesh_48" else (32, 100.0)
    nstep = 3 if variant == "recompute_3" else 2
    X, p, sm, tgt = _inputs(n, box, True, 90, nstep=nstep)
    mask = (np.random.default_rng(91).integers(0, 2, (n,) * 3).astype(np.float32)
            if variant == "mask_graph" else None)
    kw = {"generic": dict(pipelined=False), "recompute_3": dict(recompute=True)}.get(variant, {})
    f, loss, g = _fused(n, box, X, p, sm, tgt, True, "reference", nstep=nstep, mask=mask, **kw)
    lp, gp = _plain(n, box, X, p, sm, tgt, True, "reference", nstep=nstep, mask=mask)
    assert abs(loss - lp) <= 1e-5 * abs(lp)
    assert np.linalg.norm(g - gp) / np.linalg.norm(gp) < 1e-3
    assert _rel(g, gp).max() < 1e-2
    if variant == "mask_graph":
        d32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa
        statics = (d32(X), d32(tgt), d32(mask))
        f.capture(*statics)
        l2, g2 = f.replay(p)
        torch.cuda.synchronize()
        assert abs(float(l2) - loss) <= 1e-6 * abs(loss)
        assert _rel(g2.cpu().numpy(), g).max() < 1e-3


def test_fused_hi_rejects_bad_arguments():
    from jerald_gb300.ldl import FusedLDL
    sm = torch.ones((16, 16, 16), device="cuda")
    with pytest.raises(ValueError):
        FusedLDL(16, 10.0, 4096, kind="HI")
    with pytest.raises(ValueError):
        FusedLDL(16, 10.0, 4096, kind="HI", starmap=sm, n=1.0)
    with pytest.raises(ValueError):
        FusedLDL(16, 10.0, 4096, kind="HI", starmap=torch.ones(8, device="cuda"))
    f = FusedLDL(16, 10.0, 4096, kind="HI", starmap=sm)
    assert f.nparams == 32
    with pytest.raises(ValueError):
        f(torch.zeros((4096, 3), device="cuda"), np.zeros(13), torch.zeros((16, 16, 16), device="cuda"))
