"""On-demand band queries for full-band Monte Carlo particles.

A particle of the reference's FBMC (src/FBMC/particle.cpp:52-63) asks, at its k-vector (SI, 1/m) and
band index, for its energy (update_energy) and group velocity v = grad_k E / h_bar_eV
(update_group_velocity), which the reference interpolates inside the mesh tetrahedron holding k
(mesh_tetra.hpp:226-227). ``BandQuery`` answers the same two questions exactly at arbitrary k: the
particles' k-vectors go through one batched device solve with Hellmann-Feynman gradients
(compute_gradient_at_level's kinetic-term gradient, eV m: exact for the local EPM, where V does not
depend on k), and each particle takes its own band. ``energy_and_velocity_device`` keeps everything
on the GPU for large ensembles. For FD velocities that include the nonlocal terms, see the request
server (``serve.Server`` with UEPM_SERVE_VELOCITY).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .api import Material, _Context, generate_basis_vectors

H_PLANCK = 6.62607015e-34   # src/Common/physical_constants.hpp:18-28
Q_E = 1.602176634e-19
H_BAR_EV = H_PLANCK / (2.0 * math.pi) / Q_E  # eV s


class BandQuery:
    def __init__(self, material: Material, nearest_neighbors: int = 10, nl: bool = False, soc: bool = False,
                 precision: int = N.UEPM_PREC_FP64, basis=None):
        self.material = material
        self.G = np.ascontiguousarray(basis if basis is not None else generate_basis_vectors(nearest_neighbors),
                                      dtype=np.int32)
        self.ctx = _Context(material, self.G, nl, soc, precision)
        self.n = self.ctx.n
        self.scale = material.get_lattice_constant_meter() / (2.0 * math.pi)  # SI -> reduced

    def close(self):
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def energy_and_velocity(self, k_si, band_index):
        """E [m] (eV) and v [m][3] (m/s) of each particle's band at its k (SI)."""
        k = np.ascontiguousarray(np.asarray(k_si, dtype=np.float64).reshape(-1, 3) * self.scale)
        bands = np.asarray(band_index, dtype=np.int64).reshape(-1)
        if len(bands) != len(k):
            raise ValueError("one band index per k-vector")
        if len(k) == 0:
            return np.zeros(0), np.zeros((0, 3))
        if bands.min() < 0 or bands.max() >= self.n:
            raise IndexError("band index out of range")
        nb = int(bands.max()) + 1
        E, _, g, st = self.ctx.solve(k, nb, gradient=True)
        if st.any():
            raise RuntimeError("Eigenvalue decomposition failed")
        rows = np.arange(len(k))
        return E[rows, bands], g[rows, bands] / H_BAR_EV

    def energy_and_velocity_device(self, d_k_si, d_band_index, stream=None):
        """The same on device tensors (torch, CUDA): d_k_si [m][3] float64, d_band_index [m] int64.
        Returns device tensors E [m] and v [m][3]."""
        import torch

        L = N.load()
        m = d_k_si.shape[0]
        dev = d_k_si.device
        if m == 0:
            return torch.zeros(0, dtype=torch.float64, device=dev), torch.zeros((0, 3), dtype=torch.float64, device=dev)
        nb = int(d_band_index.max().item()) + 1
        if nb > self.n or int(d_band_index.min().item()) < 0:
            raise IndexError("band index out of range")
        k = (d_k_si * self.scale).contiguous()
        E = torch.empty((m, nb), dtype=torch.float64, device=dev)
        g = torch.empty((m, nb, 3), dtype=torch.float64, device=dev)
        st = torch.empty(m, dtype=torch.int32, device=dev)
        s = stream if stream is not None else torch.cuda.current_stream()
        p = lambda t: C.c_void_p(t.data_ptr())
        N.check(L.uepm_solve_device(self.ctx.h, p(k), m, nb, N.UEPM_WANT_VALUES | N.UEPM_WANT_GRADIENT, p(E), None, p(g),
                                    p(st), C.c_void_p(s.cuda_stream)))
        rows = torch.arange(m, device=dev)
        b = d_band_index.to(dev).long()
        return E[rows, b], g[rows, b] / H_BAR_EV
