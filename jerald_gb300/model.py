"""JERALD / LDL model on the drop-in primitives (torch autograd).

Mirrors the reference's model.py (JERALDModel, c2f, allbcast, ReLU) at
world size one: the same parameter layout (5 per layer alpha, gamma, kh, kl,
nu — 10 for "HI" — then the bias parameters), the same kinds ("dm", "sm",
"HI"), the same loss/lossv/loss_and_grad/lossv_and_grad entry points.  Every
paint, readout and FFT goes through jaxpops_bind (libjld.so); the elementwise
math between them is plain torch on the GPU, one primitive call at a time.
This is the "plain" LDL step; jerald_gb300.ldl holds the fused one.

Gradients follow the reference's custom VJP rules unless
jaxpops_bind.set_fft_adjoint("true") selects exact adjoints (then c2f's
backward is the identity too, because pifft's adjoint already carries the
half-spectrum multiplicity).
"""
from __future__ import annotations

import numpy as np
import torch

from . import jaxpops_bind as jpo


class _C2F(torch.autograd.Function):
    """Identity forward; backward doubles the cotangent of 1 <= kz < Ny/2
    (model.py:11-31) under the reference rules."""

    @staticmethod
    def forward(ctx, obj):
        return obj.clone()

    @staticmethod
    def backward(ctx, v):
        if jpo.fft_adjoint() == "true":
            return v
        sz = v.shape[1]
        v = v.clone()
        v[:, :, 1:sz // 2] = v[:, :, 1:sz // 2] + torch.conj(v[:, :, 1:sz // 2]) if v.is_complex() \
            else 2.0 * v[:, :, 1:sz // 2]
        return v


def c2f(obj):
    return _C2F.apply(obj)


def allbcast(val, comm=None):
    """World size one: the reference's allreduce in the backward is the identity."""
    return val


def ReLU(x, low=1e-12):
    return torch.where(x > low, x, torch.full_like(x, low))


def lReLU(x, alpha=.1):
    return torch.where(x > 0, x, alpha * x)


class JERALDModel:
    def __init__(self, X, target, pm, Nstep=2, kind="dm", n=0, index=1., L1=None, field2=None,
                 masktrain=None, maskvalid=None, starmap=None):
        self.pm = pm
        self.X = X
        self.target = target
        kv = pm.compute_wavevectors()
        self.kvals = kv
        kn = torch.linalg.norm(kv, dim=-1)
        self.knorms = torch.where(kn == 0, torch.full_like(kn, 1e-8), kn)
        self.Nstep = Nstep
        self.kind = kind if kind in ("dm", "sm", "HI") else "sm"
        self.n = n
        self.index = index
        self.field2 = field2
        self.masktrain = masktrain
        self.maskvalid = maskvalid
        if L1 is None:
            self.L1 = self.kind != "dm"
        else:
            self.L1 = L1
        self.starmap = starmap
        if starmap is not None:
            self.starmapk = self.pm.r2c(self.starmap)
        elif kind == "HI":
            raise Exception("Star map required for HI target")
        self.Npot = 10 if self.kind == "HI" else 5
        step = torch.as_tensor(pm.BoxSize / pm.Nmesh, device=kv.device, dtype=kv.dtype)
        self.coeff = 1 / (30 * step) * (45 * torch.sin(kv * step) - 9 * torch.sin(2 * kv * step) +
                                        torch.sin(3 * kv * step))

    # -- potential gradients (model.py:136-247) ------------------------------
    def _gradient_from_potk(self, potk, X):
        out = []
        for d in range(3):
            potgradk = -1j * self.coeff[..., d] * potk
            out.append(self.pm.readout(X, self.pm.c2r(potgradk)))
        return torch.stack(out, dim=-1)

    def potential_gradient_dm(self, params, X):
        fact, alpha, gamma, kh, kl, nu = params
        rho = self.pm.paint(X, 1.) * fact
        rhok = self.pm.r2c((rho + 1e-8) ** gamma)
        greenk = -torch.exp(-self.knorms / kl - kh / self.knorms) * self.knorms ** nu
        greenk = c2f(greenk)
        potk = 1e-2 * alpha * rhok * greenk
        return self._gradient_from_potk(potk, X)

    def potential_gradient_sm(self, params, X):
        fact, alpha, gamma, kh, kl, nu = params
        rho = self.pm.paint(X, 1.) * fact
        rhok = self.pm.r2c((rho + 1e-8) ** gamma)
        greenk = -torch.exp(-self.knorms ** 2 / kl ** 2 - kh ** 2 / self.knorms ** 2) * self.knorms ** nu
        greenk = c2f(greenk)
        potk = 1e-2 * alpha * rhok * greenk
        return self._gradient_from_potk(potk, X)

    def potential_gradient_HI(self, params, X):
        fact, alpha1, gamma1, kh1, kl1, nu1, alpha2, gamma2, kh2, kl2, nu2 = params
        rho = self.pm.paint(X, 1.) * fact
        rhok = self.pm.r2c((rho + 1e-8) ** gamma1)
        greenk1 = -torch.exp(-self.knorms ** 2 / kl1 ** 2 - kh1 ** 2 / self.knorms ** 2) * self.knorms ** nu1
        greenk1 = c2f(greenk1)
        starmapk = self.pm.r2c(self.starmap ** gamma2)
        greenk2 = torch.exp(-self.knorms ** 2 / kl2 ** 2 - kh2 ** 2 / self.knorms ** 2) * self.knorms ** nu2
        greenk2 = c2f(greenk2)
        potk = 1e-3 * (alpha1 * greenk1 * rhok + alpha2 * greenk2 * starmapk)
        return self._gradient_from_potk(potk, X)

    # -- model (model.py:249-347) --------------------------------------------
    def displace(self, params, X, Nstep):
        fact = float(np.prod(self.pm.Nmesh)) / len(X)
        for i in range(Nstep):
            p = params[self.Npot * i: self.Npot * (i + 1)]
            if self.kind == "dm":
                X = X + self.potential_gradient_dm((fact, *p[:5]), X)
            elif self.kind == "sm":
                X = X + self.potential_gradient_sm((fact, *p[:5]), X)
            else:
                X = X + self.potential_gradient_HI((fact, *p[:10]), X)
        return X

    def evaluate(self, params, X, Nstep):
        fact = float(np.prod(self.pm.Nmesh)) / len(X)
        X = self.displace(params, X, Nstep=Nstep)
        rho = self.pm.paint(X, 1.) * fact
        o = self.Npot * Nstep
        if self.kind == "HI":
            mu, w, b, beta1, khi, kli, nui, beta2, gamma3, xi, eta, zs = [params[o + j] for j in range(12)]
            starmapk = self.pm.r2c(self.starmap)
            filterk = torch.exp(-self.knorms / kli - khi / self.knorms) * self.knorms ** nui + xi
            filterk = c2f(filterk)
            depletion = ReLU(beta1 * self.pm.c2r(starmapk * filterk) + eta) + beta2 * self.starmap ** gamma3
            return ReLU(w * ReLU(rho + zs) ** mu - depletion + b)
        if self.kind == "sm":
            mu, w, b = params[o], params[o + 1], params[o + 2]
            return ReLU(w * (rho + 1e-8) ** mu + b)
        return rho

    def _residual(self, params):
        params = allbcast(params, self.pm.comm)
        F = self.evaluate(params, self.X, Nstep=self.Nstep) ** self.index
        if self.field2 is not None:
            F = F * self.field2
        diff = F - self.target
        if self.n > 0:
            sk = torch.where(self.knorms == 0, torch.ones_like(self.knorms), self.knorms ** (-self.n) + 1.)
            diffk = self.pm.r2c(diff) * sk
            diff = torch.abs(self.pm.c2r(diffk))
        else:
            diff = torch.abs(diff)
        return diff

    def _reduce(self, diff, mask):
        if mask is not None:
            d = diff * mask
            npix = torch.sum(mask)
        else:
            d = diff
            npix = diff.numel()
        s = torch.sum(d.double()) if self.L1 else torch.sum((d * d).double())
        return (s / npix).to(diff.dtype)

    def loss(self, params):
        return self._reduce(self._residual(params), self.masktrain)

    def lossv(self, params):
        diff = self._residual(params)
        loss = self._reduce(diff, self.masktrain)
        lossv = 0.
        if self.maskvalid is not None:
            lossv = self._reduce(diff, self.maskvalid)
        return loss, lossv

    def _param_leaf(self, params):
        p = params.detach().clone() if isinstance(params, torch.Tensor) else \
            torch.as_tensor(np.asarray(params), dtype=self.X.dtype, device=self.X.device)
        return p.to(device=self.X.device, dtype=self.X.dtype).requires_grad_(True)

    def loss_grad(self, params):
        return self.loss_and_grad(params)[1]

    def loss_and_grad(self, params):
        p = self._param_leaf(params)
        L = self.loss(p)
        (g,) = torch.autograd.grad(L, p)
        return L.detach(), g

    def lossv_and_grad(self, params):
        p = self._param_leaf(params)
        L, Lv = self.lossv(p)
        (g,) = torch.autograd.grad(L, p)
        Lv = Lv.detach() if isinstance(Lv, torch.Tensor) else Lv
        return L.detach(), Lv, g
