"""Seeded synthetic particle sets and parameters for the LDL workloads.

No public dataset is involved: every benchmark input is generated here from a
seed, with the shapes and distributions of the workload definitions:

* zeldovich(n, box, rms_cells, seed): n^3 particles on a lattice, displaced by
  the Zel'dovich field psi(k) = i k delta(k) / k^2 of a Gaussian random field
  with P(k) = k^-2.5 exp(-(k/kc)^2), kc = half the Nyquist wavenumber, scaled
  so the rms displacement is rms_cells mesh cells; positions wrapped into
  [0, box).
* halos(...): extra particles in Gaussian halos (width in cells) whose
  particle counts are Poisson distributed.
* default_params(nstep): per layer (alpha, gamma, kh, kl, nu) =
  (0.05, 1.0, 0.5, 2.0, 1.0), then (mu, w, b) = (1.5, 1.0, -0.1).  In the
  model's filter exp(-k^2/kl^2 - kh^2/k^2) these kh, kl give
  exp(-(k/2)^2) exp(-(0.5/k)^2).
* default_params_hi(nstep): the "HI" kind's per layer (a1, g1, kh1, kl1,
  nu1, a2, g2, kh2, kl2, nu2) = (0.5, 1.0, 0.5, 2.0, 1.0, 0.3, 0.8, 0.6,
  1.5, 0.5), then (mu, w, b, beta1, khi, kli, nui, beta2, gamma3, xi, eta,
  zs) = (1.2, 1.0, 0.2, 0.3, 0.5, 2.0, 0.5, 0.1, 0.9, 0.05, 0.1, 0.5).
* star_map(n, box, seed, frac): a stellar-mass mesh, zero outside the
  densest `frac` of the cells of a smoothed lognormal field.

Generation runs in numpy (CPU, float64) or in torch on a CUDA device (for the
large workloads); the two draw different random streams.
"""
from __future__ import annotations

import numpy as np

LAYER_DEFAULT = (0.05, 1.0, 0.5, 2.0, 1.0)
FINAL_DEFAULT = (1.5, 1.0, -0.1)


def default_params(nstep: int = 2) -> np.ndarray:
    return np.array(list(LAYER_DEFAULT) * nstep + list(FINAL_DEFAULT), dtype=np.float64)


HI_LAYER_DEFAULT = (0.5, 1.0, 0.5, 2.0, 1.0, 0.3, 0.8, 0.6, 1.5, 0.5)
HI_FINAL_DEFAULT = (1.2, 1.0, 0.2, 0.3, 0.5, 2.0, 0.5, 0.1, 0.9, 0.05, 0.1, 0.5)


def default_params_hi(nstep: int = 2) -> np.ndarray:
    return np.array(list(HI_LAYER_DEFAULT) * nstep + list(HI_FINAL_DEFAULT), dtype=np.float64)


def star_map(n: int, box: float, seed: int = 0, frac: float = 0.05) -> np.ndarray:
    """(n, n, n) float32 stellar-mass mesh: exp(2 g) of a Gaussian field g
    smoothed on two cells, kept in the densest `frac` of the cells and zero
    elsewhere, scaled to mean 1 over the cells it keeps."""
    import scipy.fft as sfft
    rng = np.random.default_rng(seed)
    W = sfft.rfftn(rng.standard_normal((n, n, n)), workers=-1)
    kx, ky, kz = _kgrid_np(n, box)
    r = 2.0 * box / n
    W *= np.exp(-0.5 * (kx ** 2 + ky ** 2 + kz ** 2) * r * r)
    g = sfft.irfftn(W, s=(n, n, n), workers=-1)
    g /= g.std()
    f = np.exp(2.0 * g)
    cut = np.quantile(f, 1.0 - frac)
    out = np.where(f > cut, f, 0.0)
    out /= out[out > 0].mean()
    return out.astype(np.float32)


def _kgrid_np(n: int, box: float):
    k = 2 * np.pi * np.fft.fftfreq(n, box / n)
    kz = k[: n // 2 + 1]
    return k[:, None, None], k[None, :, None], kz[None, None, :]


def zeldovich(n: int, box: float, rms_cells: float = 0.5, seed: int = 0,
              device=None, dtype=np.float32):
    """n^3 lattice particles plus a Zel'dovich displacement; returns (n^3, 3)."""
    if device is not None and str(device).startswith("cuda"):
        return _zeldovich_torch(n, box, rms_cells, seed, device, dtype)
    import scipy.fft as sfft
    rng = np.random.default_rng(seed)
    W = sfft.rfftn(rng.standard_normal((n, n, n)), workers=-1)
    kx, ky, kz = _kgrid_np(n, box)
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    kc = 0.5 * np.pi * n / box
    with np.errstate(divide="ignore", invalid="ignore"):
        # sqrt(P(k)) / k^2, zero at k = 0
        W *= np.where(k2 > 0, np.sqrt(k2 ** (-1.25) * np.exp(-k2 / kc ** 2)) / k2, 0.0)
    del k2
    out = np.empty((n ** 3, 3), dtype=np.float64)
    for d, kd in enumerate((kx, ky, kz)):
        out[:, d] = sfft.irfftn(1j * kd * W, s=(n, n, n), axes=(0, 1, 2), workers=-1).reshape(-1)
    del W
    rms = np.sqrt(np.einsum("ij,ij->", out, out) / out.shape[0])
    cell = box / n
    out *= rms_cells * cell / rms
    g = np.arange(n) * cell
    lat = out.reshape(n, n, n, 3)
    lat[..., 0] += g[:, None, None]
    lat[..., 1] += g[None, :, None]
    lat[..., 2] += g[None, None, :]
    np.mod(out, box, out=out)
    return out.astype(dtype)


def _zeldovich_torch(n, box, rms_cells, seed, device, dtype):
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    w = torch.randn((n, n, n), generator=gen, device=device, dtype=torch.float32)
    W = torch.fft.rfftn(w)
    del w
    k = 2 * np.pi * torch.fft.fftfreq(n, box / n, device=device)
    kx, ky, kz = k[:, None, None], k[None, :, None], k[: n // 2 + 1][None, None, :]
    kz = torch.abs(kz) * torch.sign(k[: n // 2 + 1])[None, None, :]
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    kc = 0.5 * np.pi * n / box
    pk = torch.where(k2 > 0, k2.clamp_min(1e-30) ** (-1.25) * torch.exp(-k2 / kc ** 2),
                     torch.zeros_like(k2))
    delta = W * torch.sqrt(pk)
    del W, pk
    inv = torch.where(k2 > 0, 1.0 / k2.clamp_min(1e-30), torch.zeros_like(k2))
    out = torch.empty((n * n * n, 3), device=device, dtype=torch.float32)
    cell = box / n
    g = torch.arange(n, device=device, dtype=torch.float32) * cell
    for d, kd in enumerate((kx, ky, kz)):
        psi = torch.fft.irfftn(1j * kd * delta * inv, s=(n, n, n))
        out[:, d] = psi.reshape(-1)
    rms = torch.sqrt(torch.mean(torch.sum(out.double() ** 2, dim=-1))).float()
    out *= rms_cells * cell / rms
    out[:, 0] += g[:, None, None].expand(n, n, n).reshape(-1)
    out[:, 1] += g[None, :, None].expand(n, n, n).reshape(-1)
    out[:, 2] += g[None, None, :].expand(n, n, n).reshape(-1)
    out = torch.remainder(out, box)
    return out if dtype in (np.float32, torch.float32) else out.double()


def halos(nhalo: int, total: int, box: float, n: int, width_cells: float = 0.5,
          seed: int = 1, dtype=np.float32) -> np.ndarray:
    """`total` particles in `nhalo` Gaussian halos with Poisson counts."""
    rng = np.random.default_rng(seed)
    lam = total / nhalo
    counts = rng.poisson(lam, nhalo).astype(np.int64)
    # trim/extend so the counts sum to `total`
    diff = total - int(counts.sum())
    idx = rng.integers(0, nhalo, abs(diff)) if diff else np.zeros(0, dtype=np.int64)
    np.add.at(counts, idx, 1 if diff > 0 else -1)
    counts = np.maximum(counts, 0)
    centers = rng.uniform(0, box, (nhalo, 3))
    sig = width_cells * box / n
    reps = np.repeat(np.arange(nhalo), counts)
    pts = centers[reps] + rng.normal(0, sig, (len(reps), 3))
    return np.mod(pts, box).astype(dtype)


def clustered(n: int, box: float, seed: int = 0, device=None, extra_frac: float = 0.1,
              nhalo: int = 2000, rms_cells: float = 3.0):
    """Clustered set: n^3 Zel'dovich particles (rms 3 cells) plus extra_frac * n^3
    halo particles in nhalo halos of 0.5-cell width."""
    base = zeldovich(n, box, rms_cells, seed, device=device)
    extra = halos(nhalo, int(round(extra_frac * n ** 3)), box, n, 0.5, seed + 1)
    if device is not None and str(device).startswith("cuda"):
        import torch
        return torch.cat([base, torch.from_numpy(extra).to(device)], dim=0)
    return np.concatenate([base, extra], axis=0)


def lognormal_noise(shape, sigma: float = 0.1, seed: int = 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(sigma * rng.standard_normal(shape))
