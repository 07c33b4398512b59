"""ORACLE — test infrastructure only.  FFT conventions of the reference.

pfft  (lib/parfft.h:78-94, lib/cpu.cc:169-200): unnormalised r2c, sign -1,
      half spectrum along z -> numpy.fft.rfftn.
pifft (lib/parfft.h:96-109, lib/cpu.cc:202-245): unnormalised c2r, sign +1:
      complex inverses along x, y then a c2r along z that ignores the
      imaginary parts of kz = 0 and kz = Nz/2 -> numpy.fft.irfftn * N.
r2c / c2r (pmesh.py:100-127): r2c = pfft / prod(Nmesh), c2r = pifft.
FFTW (unpinned version, pkg-config fftw3 in CMakeLists.txt:9) is not in the
image; numpy's pocketfft computes the same DFT.  tests/ pin numpy against a
direct O(n^2) DFT on small meshes.
"""
from __future__ import annotations

import numpy as np


_WORKERS = {"n": 1}


def set_workers(n: int) -> None:
    """Use scipy.fft (pocketfft) with n threads instead of numpy (1 thread)."""
    _WORKERS["n"] = max(1, int(n))


def pfft(x: np.ndarray) -> np.ndarray:
    if _WORKERS["n"] > 1:
        import scipy.fft
        return scipy.fft.rfftn(x, workers=_WORKERS["n"])
    return np.fft.rfftn(x)


def pifft(y: np.ndarray, shape) -> np.ndarray:
    shape = tuple(int(s) for s in shape)
    if _WORKERS["n"] > 1:
        import scipy.fft
        return scipy.fft.irfftn(y, s=shape, axes=(0, 1, 2), workers=_WORKERS["n"]) * float(np.prod(shape))
    return np.fft.irfftn(y, s=shape, axes=(0, 1, 2)) * float(np.prod(shape))


def r2c(x: np.ndarray) -> np.ndarray:
    return pfft(x) / float(np.prod(x.shape))


def c2r(y: np.ndarray, shape) -> np.ndarray:
    return pifft(y, shape)


def direct_rfft3(x: np.ndarray) -> np.ndarray:
    """O(N^2) DFT with sign -1, kz in [0, Nz/2]: a definition-level check."""
    nx, ny, nz = x.shape
    out = np.zeros((nx, ny, nz // 2 + 1), dtype=np.complex128)
    ix = np.arange(nx)[:, None, None]
    iy = np.arange(ny)[None, :, None]
    iz = np.arange(nz)[None, None, :]
    for kx in range(nx):
        for ky in range(ny):
            for kz in range(nz // 2 + 1):
                ph = np.exp(-2j * np.pi * (kx * ix / nx + ky * iy / ny + kz * iz / nz))
                out[kx, ky, kz] = np.sum(x * ph)
    return out


def direct_irfft3(y: np.ndarray, shape) -> np.ndarray:
    """O(N^2) c2r by definition: x = sum over kx, ky of Re-part-along-z terms.

    Along z the half spectrum is expanded as X[0].re + sum_{0<k<Nz/2}
    2 Re(X[k] e^{+i..}) + X[Nz/2].re (-1)^z after complex inverses along x
    and y, which is what FFTW's multi-dimensional c2r evaluates.
    """
    nx, ny, nz = shape
    h = nz // 2
    # complex inverse (unnormalised) along x and y
    t = np.fft.ifft2(y, axes=(0, 1)) * (nx * ny)
    out = np.zeros(shape)
    z = np.arange(nz)
    for kz in range(h + 1):
        ph = np.exp(2j * np.pi * kz * z / nz)
        if kz == 0 or (nz % 2 == 0 and kz == h):
            out += np.real(t[:, :, kz].real[:, :, None] * ph[None, None, :])
        else:
            out += 2.0 * np.real(t[:, :, kz][:, :, None] * ph[None, None, :])
    return out
