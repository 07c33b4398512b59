"""Particle-mesh facade mirroring the reference's pmesh.PMesh at world size one.

Same constructor and methods (pmesh.py:17-219): paint, readout, readout3D,
r2c (= pfft / prod(Nmesh), "forward normalisation to match LDL"), c2r
(= unnormalised pifft), compute_wavevectors, mesh_coordinates,
local_mesh_coordinates, local_mesh_indices, flattened_coordinates, preview,
printr, get_local_positions(_vanilla), clean, initLayouts.  Arrays are torch
tensors on a CUDA device; `dtype` picks the f32 or f64 primitives the way
jax_enable_x64 does in the reference.

One deviation: the reference's compute_edges sets the upper y edge to
Nmesh[2] (pmesh.py:62), which only matters for non-cubic meshes; here it is
Nmesh[1].
"""
from __future__ import annotations

import sys

import numpy as np
import torch

from . import jaxpops_bind as jpo


class PMesh:
    def __init__(self, Nmesh, BoxSize, comm=None, device="cuda", dtype=torch.float32):
        self.Nmesh = np.array(np.broadcast_to(np.asarray(Nmesh, dtype=np.int64).reshape(-1), (3,)))
        self.BoxSize = np.array(np.broadcast_to(np.asarray(BoxSize, dtype=np.float64).reshape(-1), (3,)))
        self.comm = comm if comm is not None else jpo.WORLD
        self.commrank = getattr(self.comm, "rank", 0)
        self.commsize = getattr(self.comm, "size", 1)
        self.device = torch.device(device)
        self.dtype = dtype
        jpo.initLayout(self.commsize)
        self.localL, self.localS = (int(v) for v in jpo.buildplan(self.Nmesh, self.comm))
        self._Nmesh = tuple(int(v) for v in self.Nmesh)
        self.fftss = (self.localS, self.localS + self.localL)
        self.fftdims = (self.localL, self._Nmesh[1], self._Nmesh[2])
        self.edges = self.compute_edges()
        r = self.commrank
        self.paintdims = tuple(int(self.edges[a, r, 1] - self.edges[a, r, 0]) for a in range(3))

    def initLayouts(self, N):
        for i in range(1, N):
            jpo.initLayout(self.commsize, lyidx=i)

    def compute_edges(self):
        edges = np.zeros((3, self.commsize, 2), dtype=np.int64)
        edges[2, :, 1] = self.Nmesh[2]
        edges[1, :, 1] = self.Nmesh[1]
        edges[0, 0, 0] = self.localS
        edges[0, 0, 1] = self.localS + self.localL
        return edges

    # -- particle <-> mesh ---------------------------------------------------
    def get_local_positions_vanilla(self, pos):
        box = torch.as_tensor(self.BoxSize, device=pos.device, dtype=pos.dtype)
        return torch.remainder(pos, box)

    def get_local_positions(self, pos, Nout):
        return jpo.local_positions(pos, Nout, self.Nmesh, self.BoxSize, self.edges, self.commsize,
                                   self.commrank)

    def paint(self, pos, mass, lyidx=0):
        return jpo.ppaint(pos, mass, self.Nmesh, self.BoxSize, self.edges, self.paintdims, self.comm, lyidx)

    def readout(self, pos, mesh, lyidx=0):
        return jpo.preadout(pos, mesh, self.Nmesh, self.BoxSize, self.edges, self.paintdims, self.comm, lyidx)

    def readout3D(self, pos, meshes, lyidx=0):
        return jpo.preadout3D(pos, meshes, self.Nmesh, self.BoxSize, self.edges, self.paintdims, self.comm,
                              lyidx)

    @staticmethod
    def clean(lyidx=0):
        return jpo.clean(lyidx)

    # -- FFT ------------------------------------------------------------------
    def r2c(self, localreal):
        """Forward r2c normalised by prod(Nmesh) (pmesh.py:100-112)."""
        return jpo.pfft(localreal, self.fftdims) / float(np.prod(self.Nmesh))

    def c2r(self, localcplx):
        """Unnormalised c2r (pmesh.py:115-127)."""
        return jpo.pifft(localcplx, self.fftdims)

    # -- coordinates ----------------------------------------------------------
    def _t(self, a):
        return torch.as_tensor(a, device=self.device, dtype=self.dtype)

    def mesh_coordinates(self):
        ax = [torch.arange(self._Nmesh[a], device=self.device, dtype=self.dtype) / self._Nmesh[a] *
              float(self.BoxSize[a]) for a in range(3)]
        return torch.stack(torch.meshgrid(*ax, indexing="ij"), dim=-1)

    def local_mesh_coordinates(self):
        x = torch.arange(self.fftss[0], self.fftss[1], device=self.device, dtype=self.dtype) / \
            self._Nmesh[0] * float(self.BoxSize[0])
        y = torch.arange(self._Nmesh[1], device=self.device, dtype=self.dtype) / self._Nmesh[1] * \
            float(self.BoxSize[1])
        z = torch.arange(self._Nmesh[2], device=self.device, dtype=self.dtype) / self._Nmesh[2] * \
            float(self.BoxSize[2])
        return torch.stack(torch.meshgrid(x, y, z, indexing="ij"), dim=-1)

    def local_mesh_indices(self):
        x = torch.arange(self.fftss[0], self.fftss[1], device=self.device)
        y = torch.arange(self._Nmesh[1], device=self.device)
        z = torch.arange(self._Nmesh[2], device=self.device)
        return torch.stack(torch.meshgrid(x, y, z, indexing="ij"), dim=-1)

    def flattened_coordinates(self):
        cell = self.BoxSize / self.Nmesh
        n = int(np.prod(self.Nmesh))
        r = torch.arange(n, device=self.device)
        out = torch.empty((n, 3), device=self.device, dtype=self.dtype)
        out[:, 2] = torch.remainder(r, self._Nmesh[2]).to(self.dtype) * float(cell[2])
        out[:, 1] = torch.remainder(r // self._Nmesh[2], self._Nmesh[1]).to(self.dtype) * float(cell[1])
        out[:, 0] = torch.remainder(r // (self._Nmesh[2] * self._Nmesh[1]), self._Nmesh[0]).to(self.dtype) * \
            float(cell[0])
        return out

    def compute_wavevectors(self):
        """(Nx, Ny, Nz//2+1, 3) wavevectors 2 pi fftfreq(N, L/N), kz cut to the
        half spectrum (its last entry is the negative Nyquist frequency)."""
        ks = []
        for a in range(3):
            k = np.fft.fftfreq(self._Nmesh[a], self.BoxSize[a] / self.Nmesh[a]) * 2 * np.pi
            ks.append(k)
        kx = ks[0][self.fftss[0]:self.fftss[1]]
        kz = ks[2][: self._Nmesh[2] // 2 + 1]
        grids = np.meshgrid(kx, ks[1], kz, indexing="ij")
        return torch.as_tensor(np.stack(grids, axis=-1), device=self.device, dtype=self.dtype)

    def preview(self, localfield, fullsize=None, comm=None):
        if fullsize is None:
            fullsize = self.Nmesh
        return localfield.detach().cpu().numpy().reshape(tuple(int(v) for v in fullsize))

    def printr(self, strings, rank=0, flush=True):
        if self.commrank == rank:
            if isinstance(strings, list):
                for s in strings:
                    print(s)
            else:
                print(strings)
            if flush:
                sys.stdout.flush()
