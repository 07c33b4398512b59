"""ORACLE — test infrastructure only.  FP64 restatement of the LDL pipeline
and of its gradient, used by tests/, the smoke check and bench.py's CPU
baseline to check results against.

Forward (model.py): per layer (model.py:186-212 "sm", 137-179 "dm")
    rho   = paint(X, 1) * fact                    fact = prod(Nmesh) / Npart
    s     = (rho + 1e-8) ** gamma
    shat  = pfft(s) / prod(Nmesh)                 (pmesh.py:112)
    G     = -exp(-k^2/kl^2 - kh^2/k^2) k^nu       ("sm";  "dm": -exp(-k/kl - kh/k) k^nu)
    P     = 1e-2 * alpha * shat * G
    g_d   = pifft(-1j * c_d(k) * P),  c_d = (45 sin(k h) - 9 sin(2kh) + sin(3kh)) / (30 h)
    X    += stack(readout(X, g_d))
final paint and bias (model.py:311, 344): F = ReLU(w (rho + 1e-8)^mu + b),
loss (model.py:373-403): sum(mask |F - target|^{1|2}) / Npixel.
Wavevectors (pmesh.py:175-186): k_d = 2 pi fftfreq(N_d, L_d/N_d), kz cut to
[0, Nz/2] (so the Nyquist plane carries the negative frequency), |k| = 0
replaced by 1e-8 (model.py:101-102).

Gradient, two modes:
  "reference": the composition of the reference's custom VJP rules as JAX
      applies them (jaxpops_bind.py:236-247, 351-363, 699-701, 758-759;
      model.py:23-29), with JAX's cotangent convention dL/dRe - i dL/dIm.
      pifft's rule omits the half-spectrum multiplicity m_k (2 for
      0 < kz < Nz/2), so d loss / d alpha is biased.
  "true": the exact adjoint: pifft's adjoint carries m_k, pfft's adjoint
      sums the half spectrum once, c2f's rule is the identity.
Both modes agree except in d/d alpha (on cubic meshes).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import cic
from .fft import pfft, pifft

PARAMS_PER_LAYER = 5  # alpha, gamma, kh, kl, nu (model.py:268-272)

_EW = {"threads": 1}


def set_threads(n: int) -> None:
    """Host threads for the large elementwise expressions and sums (1 = plain
    numpy, the default the tests use).  With n > 1 each expression runs on n
    slabs along the first axis at once (numpy releases the GIL inside its
    loops), which gives the same values; sums add n slab partials."""
    _EW["threads"] = max(1, int(n))


_POOL = {}


def _pool(n):
    if n not in _POOL:
        from concurrent.futures import ThreadPoolExecutor
        _POOL[n] = ThreadPoolExecutor(n)
    return _POOL[n]


def _slabs(length, n):
    e = np.linspace(0, length, n + 1).astype(np.int64)
    return [slice(int(a), int(b)) for a, b in zip(e[:-1], e[1:]) if b > a]


def _ew(fn, *arrs):
    """fn(*arrs) for an elementwise fn, evaluated slab by slab along axis 0
    of the largest argument (arguments of another first extent are passed
    whole and broadcast)."""
    n = _EW["threads"]
    big = max((a for a in arrs if isinstance(a, np.ndarray)), key=lambda a: a.size)
    if n <= 1 or big.size < (1 << 20) or big.ndim == 0:
        return fn(*arrs)
    L = big.shape[0]
    sl = _slabs(L, n)

    def part(s):
        return fn(*[a[s] if isinstance(a, np.ndarray) and a.ndim > 0 and a.shape[0] == L else a for a in arrs])
    first = part(sl[0])
    out = np.empty((L,) + first.shape[1:], dtype=first.dtype)
    out[sl[0]] = first

    def fill(s):
        out[s] = part(s)
    list(_pool(n).map(fill, sl[1:]))
    return out


def _sum(fn, *arrs):
    """np.sum(fn(*arrs)), slab partials summed in slab order when threaded."""
    n = _EW["threads"]
    big = max((a for a in arrs if isinstance(a, np.ndarray)), key=lambda a: a.size)
    if n <= 1 or big.size < (1 << 20) or big.ndim == 0:
        return np.sum(fn(*arrs))
    L = big.shape[0]

    def part(s):
        return np.sum(fn(*[a[s] if isinstance(a, np.ndarray) and a.ndim > 0 and a.shape[0] == L else a
                           for a in arrs]))
    return sum(_pool(n).map(part, _slabs(L, n)))


def fftfreq_signed(n: int) -> np.ndarray:
    """Integer frequency index of numpy's fftfreq ordering."""
    return np.fft.fftfreq(n, 1.0 / n)


@dataclass
class LDLOracle:
    """FP64 forward and adjoint of the LDL model (kinds "sm" and "dm").

    pos_dtype=np.float32 rounds the positions after every layer to float32
    (then computes on in FP64): the storage of an FP32 pipeline, which keeps
    each layer's particle positions in float32 as the reference's FP32 path
    does.  A displacement smaller than half a float32 ulp of the coordinate
    is then partly lost, an error no FP32 kernel arithmetic can avoid; this
    oracle separates it from the kernels' own."""
    nmesh: tuple
    box: tuple
    kind: str = "sm"
    L1: bool = True
    cache: dict = field(default_factory=dict)
    pos_dtype: object = np.float64

    def __post_init__(self):
        self.nmesh = tuple(int(v) for v in np.broadcast_to(np.asarray(self.nmesh), (3,)))
        self.box = tuple(float(v) for v in np.broadcast_to(np.asarray(self.box, dtype=float), (3,)))
        N, L = self.nmesh, self.box
        ks = []
        for a in range(3):
            k = np.fft.fftfreq(N[a], L[a] / N[a]) * 2 * np.pi
            if a == 2:
                k = k[: N[2] // 2 + 1]
            ks.append(k)
        KX, KY, KZ = np.meshgrid(*ks, indexing="ij")
        self.kvec = (KX, KY, KZ)
        kn = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
        self.knorm = np.where(kn == 0, 1e-8, kn)
        step = np.array(L) / np.array(N)
        self.coeff = [1.0 / (30 * step[a]) * (45 * np.sin(self.kvec[a] * step[a])
                                               - 9 * np.sin(2 * self.kvec[a] * step[a])
                                               + np.sin(3 * self.kvec[a] * step[a])) for a in range(3)]
        # half-spectrum multiplicity along z
        h = N[2] // 2 + 1
        m = np.full(h, 2.0)
        m[0] = 1.0
        if N[2] % 2 == 0:
            m[-1] = 1.0
        self.mult = m[None, None, :]
        self.ncell = float(np.prod(N))

    # -- pieces ---------------------------------------------------------------
    def mesh_pos(self, X):
        return cic.box_to_mesh(np.asarray(X, dtype=np.float64), self.box, self.nmesh)

    def green(self, kh, kl, nu):
        if self.kind == "dm":
            return _ew(lambda k: -np.exp(-k / kl - kh / k) * k ** nu, self.knorm)
        return _ew(lambda k: -np.exp(-k ** 2 / kl ** 2 - kh ** 2 / k ** 2) * k ** nu, self.knorm)

    def green_grads(self, G, kh, kl, nu):
        """dG/dkh, dG/dkl, dG/dnu."""
        k = self.knorm
        if self.kind == "dm":
            return (_ew(lambda G, k: G * (-1.0 / k), G, k), _ew(lambda G, k: G * (k / kl ** 2), G, k),
                    _ew(lambda G, k: G * np.log(k), G, k))
        return (_ew(lambda G, k: G * (-2.0 * kh / k ** 2), G, k), _ew(lambda G, k: G * (2.0 * k ** 2 / kl ** 3), G, k),
                _ew(lambda G, k: G * np.log(k), G, k))

    # -- forward --------------------------------------------------------------
    def layer_forward(self, X, prm, fact):
        alpha, gamma, kh, kl, nu = prm
        Xm = self.mesh_pos(X)
        rho = _ew(lambda r: r * fact, cic.paint(Xm, 1.0, self.nmesh))
        s = _ew(lambda r: (r + 1e-8) ** gamma, rho)
        shat = _ew(lambda v: v / self.ncell, pfft(s))
        G = self.green(kh, kl, nu)
        P = _ew(lambda v, G: 1e-2 * alpha * v * G, shat, G)
        g = [pifft(_ew(lambda c, P: -1j * c * P, self.coeff[d], P), self.nmesh) for d in range(3)]
        disp = np.empty_like(X)
        for d in range(3):
            disp[:, d] = cic.readout(Xm, g[d], self.nmesh, self.box)
        c = dict(Xm=Xm, rho=rho, s=s, shat=shat, G=G, g=g, prm=prm)
        return _ew(lambda a, b: a + b, X, disp), c

    def final_map(self, X, mu, w, b, fact):
        Xm = self.mesh_pos(X)
        rho = _ew(lambda r: r * fact, cic.paint(Xm, 1.0, self.nmesh))
        if self.kind == "dm":
            return rho, dict(Xm=Xm, rho=rho)
        base = _ew(lambda r: (r + 1e-8) ** mu, rho)
        u = _ew(lambda v: w * v + b, base)
        F = _ew(lambda u: np.where(u > 1e-12, u, 1e-12), u)
        return F, dict(Xm=Xm, rho=rho, base=base, u=u)

    def forward(self, params, X, target, nstep, mask=None):
        params = np.asarray(params, dtype=np.float64)
        X = np.asarray(X, dtype=np.float64)
        fact = self.ncell / len(X)
        layers = []
        for l in range(nstep):
            X, c = self.layer_forward(X, params[5 * l: 5 * l + 5], fact)
            if self.pos_dtype != np.float64:
                X = X.astype(self.pos_dtype).astype(np.float64)
            layers.append(c)
        if self.kind == "dm":
            mu = w = b = 0.0
        else:
            mu, w, b = params[5 * nstep: 5 * nstep + 3]
        F, fc = self.final_map(X, mu, w, b, fact)
        diff = _ew(lambda a, b: a - b, F, np.asarray(target, dtype=np.float64))
        if mask is not None:
            npix = float(np.sum(mask))
            ad = _ew(lambda d, m: np.abs(d) * m, diff, mask)
        else:
            npix = float(diff.size)
            ad = _ew(np.abs, diff)
        loss = (_sum(lambda a: a, ad) if self.L1 else _sum(lambda a: a ** 2, ad)) / npix
        self.cache = dict(layers=layers, final=fc, F=F, diff=diff, mask=mask, npix=npix,
                          fact=fact, params=params, nstep=nstep, X_final=X)
        return float(loss)

    # -- backward -------------------------------------------------------------
    def backward(self, mode="reference"):
        """Gradient of the last forward() loss w.r.t. the parameter vector."""
        if mode not in ("reference", "true"):
            raise ValueError("mode must be 'reference' or 'true'")
        c = self.cache
        params, nstep, fact = c["params"], c["nstep"], c["fact"]
        grad = np.zeros_like(params)
        diff, mask, npix = c["diff"], c["mask"], c["npix"]
        m = mask if mask is not None else np.float64(1.0)
        # d|diff|/d diff with JAX's abs rule (+1 at zero)
        if self.L1:
            ctF = _ew(lambda d, m: np.where(d >= 0, 1.0, -1.0) * m / npix, diff, m)
        else:
            ctF = _ew(lambda d, m: 2.0 * np.abs(d) * m * m * np.where(d >= 0, 1.0, -1.0) / npix, diff, m)
        fc = c["final"]
        if self.kind == "dm":
            ct_rho = ctF
        else:
            mu, w, b = params[5 * nstep: 5 * nstep + 3]
            ctu = _ew(lambda f, u: f * (u > 1e-12), ctF, fc["u"])
            grad[5 * nstep + 0] = _sum(lambda c, bs, r: c * w * bs * np.log(r + 1e-8), ctu, fc["base"], fc["rho"])
            grad[5 * nstep + 1] = _sum(lambda c, bs: c * bs, ctu, fc["base"])
            grad[5 * nstep + 2] = _sum(lambda c: c, ctu)
            ct_rho = _ew(lambda c, r: c * w * mu * (r + 1e-8) ** (mu - 1), ctu, fc["rho"])
        Xbar = cic.readout3d(fc["Xm"], _ew(lambda v: v * fact, ct_rho), self.nmesh, self.box, vjp=True)
        for l in reversed(range(nstep)):
            Xbar, g5 = self.layer_backward(c["layers"][l], Xbar, fact, mode)
            grad[5 * l: 5 * l + 5] = g5
        return grad

    def layer_backward(self, lc, Xbar_next, fact, mode):
        alpha, gamma, kh, kl, nu = lc["prm"]
        Xm, g = lc["Xm"], lc["g"]
        Xbar = Xbar_next.copy()
        ct_g = []
        for d in range(3):
            v = np.ascontiguousarray(Xbar_next[:, d])
            Xbar = _ew(lambda a, r, v: a + r * v[:, None], Xbar,
                       cic.readout3d(Xm, g[d], self.nmesh, self.box, vjp=True), v)
            ct_g.append(cic.paint(Xm, v, self.nmesh))
        ctP = np.zeros_like(lc["shat"])
        for d in range(3):
            if mode == "true":
                ctP = _ew(lambda acc, c, V: acc + (-1j * c) * (np.conj(V) * self.mult), ctP, self.coeff[d],
                          pfft(ct_g[d]))
            else:
                ctP = _ew(lambda acc, c, V: acc + (-1j * c) * np.conj(V), ctP, self.coeff[d], pfft(ct_g[d]))
        shat, G = lc["shat"], lc["G"]
        ctw = _ew(lambda G, P: G * P, G, ctP)              # w = 1e-2 alpha shat
        ctG = _ew(lambda P, s: np.real(P * (1e-2 * alpha * s)), ctP, shat)
        if mode == "reference":                          # c2f rule, model.py:23-29
            sz = ctG.shape[1]
            ctG[:, :, 1:sz // 2] *= 2.0
        g_alpha = 1e-2 * _sum(lambda w, s: np.real(w * s), ctw, shat)
        dkh, dkl, dnu = self.green_grads(G, kh, kl, nu)
        g_kh, g_kl, g_nu = (_sum(lambda a, b: a * b, ctG, dkh), _sum(lambda a, b: a * b, ctG, dkl),
                            _sum(lambda a, b: a * b, ctG, dnu))
        if mode == "reference":
            cts = pifft(_ew(lambda w: np.conj((1e-2 * alpha) * w / self.ncell), ctw), self.nmesh)
        else:
            cts = pifft(_ew(lambda w: np.conj((1e-2 * alpha) * w / self.ncell) / self.mult, ctw), self.nmesh)
        rho, s = lc["rho"], lc["s"]
        g_gamma = _sum(lambda c, s, r: c * s * np.log(r + 1e-8), cts, s, rho)
        ct_rho = _ew(lambda c, r: c * gamma * (r + 1e-8) ** (gamma - 1) * fact, cts, rho)
        Xbar = _ew(lambda a, b: a + b, Xbar, cic.readout3d(Xm, ct_rho, self.nmesh, self.box, vjp=True))
        return Xbar, np.array([g_alpha, g_gamma, g_kh, g_kl, g_nu])

    def loss_and_grad(self, params, X, target, nstep, mask=None, mode="reference"):
        loss = self.forward(params, X, target, nstep, mask)
        return loss, self.backward(mode)

    def fd_grad(self, params, X, target, nstep, mask=None, step=1e-3, idx=None):
        """Central finite differences of the loss, step `step` per parameter."""
        params = np.asarray(params, dtype=np.float64)
        idx = range(len(params)) if idx is None else idx
        out = np.full(len(params), np.nan)
        for i in idx:
            p1 = params.copy(); p1[i] += step
            p0 = params.copy(); p0[i] -= step
            out[i] = (self.forward(p1, X, target, nstep, mask) -
                      self.forward(p0, X, target, nstep, mask)) / (2 * step)
        return out


def model_loss(nmesh, box, kind, params, X, target, nstep, starmap=None, n=0, index=1.0, L1=None,
               field2=None, mask=None, maskvalid=None):
    """FP64 forward of model.py's full loss for every kind and option, by the
    oracle primitives: kinds "dm", "sm" and "HI" (potential_gradient_HI,
    model.py:213-247, with the star-map source; HI final map model.py:313-336),
    the field exponent `index` and second field (model.py:368-372), the
    residual smoothing |k|^-n + 1 without c2f (model.py:376-381), training
    and validation masks (model.py:384-390, 454-465).  Returns (loss, lossv)
    (lossv = 0 without a validation mask).  Forward only: gradients of the
    options are checked against its central differences."""
    o = LDLOracle(nmesh, box, kind="dm" if kind == "dm" else "sm")
    N = o.nmesh
    k = o.knorm
    params = np.asarray(params, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64).copy()
    relu = lambda v: np.where(v > 1e-12, v, 1e-12)  # noqa: E731  (model.py:55-57)
    r2c = lambda f: pfft(f) / o.ncell                 # noqa: E731  (pmesh.py:112)
    c2r = lambda fk: pifft(fk, N)                     # noqa: E731
    fact = o.ncell / len(X)
    npot = 10 if kind == "HI" else 5
    for layer in range(nstep):
        p = params[npot * layer: npot * (layer + 1)]
        Xm = o.mesh_pos(X)
        rho = cic.paint(Xm, 1.0, N) * fact
        if kind == "HI":
            a1, g1, kh1, kl1, nu1, a2, g2, kh2, kl2, nu2 = p
            G1 = -np.exp(-k ** 2 / kl1 ** 2 - kh1 ** 2 / k ** 2) * k ** nu1
            G2 = np.exp(-k ** 2 / kl2 ** 2 - kh2 ** 2 / k ** 2) * k ** nu2
            potk = 1e-3 * (a1 * G1 * r2c((rho + 1e-8) ** g1) + a2 * G2 * r2c(np.asarray(starmap) ** g2))
        else:
            a, g, kh, kl, nu = p
            potk = 1e-2 * a * r2c((rho + 1e-8) ** g) * o.green(kh, kl, nu)
        disp = [cic.readout(Xm, c2r(-1j * o.coeff[d] * potk), N, o.box) for d in range(3)]
        X = X + np.stack(disp, axis=-1)
    rho = cic.paint(o.mesh_pos(X), 1.0, N) * fact
    q = params[npot * nstep:]
    if kind == "HI":
        mu, w, b, beta1, khi, kli, nui, beta2, gamma3, xi, eta, zs = q[:12]
        sm = np.asarray(starmap, dtype=np.float64)
        filt = np.exp(-k / kli - khi / k) * k ** nui + xi
        depletion = relu(beta1 * c2r(r2c(sm) * filt) + eta) + beta2 * sm ** gamma3
        F = relu(w * relu(rho + zs) ** mu - depletion + b)
    elif kind == "sm":
        mu, w, b = q[:3]
        F = relu(w * (rho + 1e-8) ** mu + b)
    else:
        F = rho
    F = F ** index
    if field2 is not None:
        F = F * field2
    diff = F - target
    if n > 0:
        sk = np.where(k == 0, 1.0, k ** (-n) + 1.0)
        diff = np.abs(c2r(r2c(diff) * sk))
    else:
        diff = np.abs(diff)
    L1 = (kind != "dm") if L1 is None else L1

    def red(m):
        d = diff * m if m is not None else diff
        npix = float(np.sum(m)) if m is not None else float(diff.size)
        return float((np.sum(d) if L1 else np.sum(d * d)) / npix)
    return red(mask), (red(maskvalid) if maskvalid is not None else 0.0)
