"""GPU parity of the plain LDL model (primitives one by one, torch autograd)
against the FP64 oracle of the same pipeline."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle.ldl import LDLOracle  # noqa: E402


def _setup(n, box, kind, L1, dtype, seed=3, mask=False):
    from jerald_gb300 import synth
    X = synth.zeldovich(n, box, 0.5, seed=seed, dtype=np.float64)
    p = synth.default_params(2)
    o = LDLOracle((n, n, n), box, kind=kind, L1=L1)
    o.forward(p, X, np.ones((n, n, n)), 2)
    tgt = o.cache["F"] * synth.lognormal_noise((n, n, n), 0.1, seed + 1)
    m = (np.random.default_rng(seed + 2).integers(0, 2, (n, n, n)).astype(np.float64) if mask else None)
    return X, p, tgt, o, m


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    floor = 1e-6 * np.abs(b).max()
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.mark.parametrize("kind,L1", [("sm", True), ("dm", False), ("sm", False)])
@pytest.mark.parametrize("mode", ["reference", "true"])
def test_plain_model_f64_matches_oracle(kind, L1, mode):
    from jerald_gb300 import jaxpops_bind as jpo
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    n, box = 16, 100.0
    X, p, tgt, o, m = _setup(n, box, kind, L1, np.float64, mask=(kind == "sm" and not L1))
    loss_o, g_o = o.loss_and_grad(p, X, tgt, 2, mask=m, mode=mode)
    jpo.set_fft_adjoint(mode)
    try:
        pm = PMesh(n, box, dtype=torch.float64)
        mt = torch.from_numpy(m).cuda() if m is not None else None
        model = JERALDModel(torch.from_numpy(X).cuda(), torch.from_numpy(tgt).cuda(), pm, Nstep=2, kind=kind,
                            L1=L1, masktrain=mt)
        pp = p if kind != "dm" else p[:10]
        loss, g = model.loss_and_grad(torch.from_numpy(pp))
    finally:
        jpo.set_fft_adjoint("reference")
    assert abs(float(loss) - loss_o) <= 1e-10 * abs(loss_o)
    ng = len(pp)
    assert _rel(g.cpu().numpy(), g_o[:ng]).max() < 1e-7


def test_plain_model_f32_close_to_fp64_oracle():
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    n, box = 32, 100.0
    X, p, tgt, o, _ = _setup(n, box, "sm", True, np.float32)
    loss_o, g_o = o.loss_and_grad(p, X, tgt, 2, mode="reference")
    pm = PMesh(n, box, dtype=torch.float32)
    model = JERALDModel(torch.from_numpy(X.astype(np.float32)).cuda(),
                        torch.from_numpy(tgt.astype(np.float32)).cuda(), pm, Nstep=2, kind="sm")
    loss, g = model.loss_and_grad(torch.from_numpy(p.astype(np.float32)))
    assert abs(float(loss) - loss_o) <= 1e-5 * abs(loss_o)
    assert _rel(g.cpu().numpy(), g_o).max() < 2e-3


def _losstest_inputs():
    """Inputs of the reference's losstest.py (20^3 mesh, box 200, seed 83)."""
    ng = 20
    rs = np.random.RandomState(83)
    pos = rs.rand(ng ** 3, 3) * 200
    pos = pos + (10 * np.cos(np.linalg.norm(pos, axis=1) / 19)).reshape(-1, 1)
    param = np.array([.1, .5, 1., 8., 0.] * 2 + [1., 1., 0.])
    target = rs.rand(ng, ng, ng)
    maskl = np.ones_like(target)
    maskl2 = rs.randint(0, 2, target.shape).astype(np.float64)
    return ng, pos, param, target, maskl, maskl2


def test_losstest_replica_f64():
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    ng, pos, param, target, maskl, maskl2 = _losstest_inputs()
    o = LDLOracle((ng,) * 3, 200.0, kind="sm", L1=True)
    loss_o = o.forward(param, pos, target, 2, mask=maskl)
    g_o = o.backward("reference")
    lossv_o = o.forward(param, pos, target, 2, mask=maskl2)
    pm = PMesh(ng, 200, dtype=torch.float64)
    model = JERALDModel(torch.from_numpy(pos).cuda(), torch.from_numpy(target).cuda(), pm, Nstep=2, kind="sm",
                        masktrain=torch.from_numpy(maskl).cuda(), maskvalid=torch.from_numpy(maskl2).cuda())
    loss, lossv = model.lossv(torch.from_numpy(param).cuda())
    assert abs(float(loss) - loss_o) <= 1e-11 * abs(loss_o)
    assert abs(float(lossv) - lossv_o) <= 1e-11 * abs(lossv_o)
    l2, lv2, g = model.lossv_and_grad(torch.from_numpy(param))
    assert _rel(g.cpu().numpy(), g_o).max() < 1e-7



@pytest.mark.parametrize("case", ["HI", "sm_smooth", "sm_index_field2_valid"])
def test_plain_model_options_match_oracle_and_differences(case):
    """The model.py options outside the fused step -- the HI kind with its
    star map, residual smoothing |k|^-n + 1, the field exponent and second
    field, the validation mask -- on the FP64 plain path: loss (and lossv)
    against the oracle's forward, gradient against central differences of
    that forward (exact adjoint convention, smooth L2 loss)."""
    from jerald_gb300 import jaxpops_bind as jpo
    from jerald_gb300 import synth
    from jerald_gb300.model import JERALDModel
    from jerald_gb300.pmesh import PMesh
    from oracle.ldl import model_loss
    n, box = 16, 100.0
    rng = np.random.default_rng(11)
    X = synth.zeldovich(n, box, 0.5, seed=12, dtype=np.float64)
    tgt = rng.uniform(0.5, 1.5, (n,) * 3)
    kw = dict(L1=False)
    opts = {}
    if case == "HI":
        kind, p = "HI", synth.default_params_hi(2)
        opts["starmap"] = np.exp(0.3 * rng.standard_normal((n,) * 3))
    elif case == "sm_smooth":
        kind, p = "sm", synth.default_params(2)
        opts["n"] = 2
    else:
        kind, p = "sm", synth.default_params(2)
        opts["index"] = 2.0
        opts["field2"] = rng.uniform(0.8, 1.2, (n,) * 3)
        opts["mask"] = rng.integers(0, 2, (n,) * 3).astype(np.float64)
        opts["maskvalid"] = 1.0 - opts["mask"]
    ref, refv = model_loss((n,) * 3, box, kind, p, X, tgt, 2, **kw, **opts)
    dev = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64)).cuda() if a is not None else None  # noqa
    pm = PMesh(n, box, dtype=torch.float64)
    model = JERALDModel(dev(X), dev(tgt), pm, Nstep=2, kind=kind, L1=False, n=opts.get("n", 0),
                        index=opts.get("index", 1.0), field2=dev(opts.get("field2")),
                        masktrain=dev(opts.get("mask")), maskvalid=dev(opts.get("maskvalid")),
                        starmap=dev(opts.get("starmap")))
    jpo.set_fft_adjoint("true")
    try:
        loss, lossv, g = model.lossv_and_grad(torch.from_numpy(p))
    finally:
        jpo.set_fft_adjoint("reference")
    assert abs(float(loss) - ref) <= 1e-10 * abs(ref)
    if "maskvalid" in opts:
        assert abs(float(lossv) - refv) <= 1e-10 * abs(refv)
    g = g.cpu().numpy()
    fd = np.zeros_like(p)
    for i in range(len(p)):
        h = 1e-5 * max(abs(p[i]), 1e-2)
        pp, pm_ = p.copy(), p.copy()
        pp[i] += h
        pm_[i] -= h
        fd[i] = (model_loss((n,) * 3, box, kind, pp, X, tgt, 2, **kw, **opts)[0]
                 - model_loss((n,) * 3, box, kind, pm_, X, tgt, 2, **kw, **opts)[0]) / (2 * h)
    assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-4
