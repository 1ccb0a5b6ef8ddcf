"""Band states over a Brillouin-zone mesh and their dielectric function, on the GPU.

Mirrors ``uepm::mesh_bz::BZ_States`` (src/BZ_MESH/bz_states.hpp, bz_states.cpp), a ``MeshBZ`` that
keeps the eigenstates of every mesh vertex at k and at k + q:
  compute_eigenstates / compute_shifted_eigenstates   one device solve with vectors over all vertices
                                                      (local EPM, as the reference's m_nonlocal_epm =
                                                      false, bz_states.cpp:24-85); the states stay on
                                                      the device
  compute_dielectric_function                         the tetrahedron sums (bz_states.cpp:93-150): each
                                                      vertex enters with the volume / 4 of every
                                                      tetrahedron that holds it, so the sums are one
                                                      weighted pass of uepm_dielectric_sums_device;
                                                      then eps = 1 + q_e^2 / (eps_0 |q|^2) / q_e
                                                      * 2 / (2 pi)^3 * sum (:142-150)
  export_dielectric_function, get_eigen_states, export_full_eigenstates, compute_fermi_level (0, as
  in the reference).
Vertex positions and q are in SI (1/m) inside the mesh, reduced (2 pi / a) for the solves, as in
the reference.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _native as N
from .api import _Context
from .mesh import MeshBZ

Q_E = 1.602176634e-19   # src/Common/physical_constants.hpp:20
EPS_0 = 8.8541878128e-12  # physical_constants.hpp:31
FIRST_CONDUCTION_BAND = 4  # bz_states.cpp:95


class BZ_States(MeshBZ):  # noqa: N801 (reference name)
    def __init__(self, material):
        super().__init__(material)
        self.m_basisVectors = np.zeros((0, 3), dtype=np.int32)
        self.m_nb_bands_total = 0
        self.m_list_energies = np.zeros(0)
        self.m_dielectric_function_real = np.zeros(0)
        self.m_q_shift = np.zeros(3)
        self.total_volume = 0.0
        self._k = None   # device eigenstates: energies [nv][nb], vectors [nv][nb][n][2]
        self._kq = None

    def set_nb_bands(self, nb_bands: int) -> None:
        self.m_nb_bands_total = int(nb_bands)

    def set_basis_vectors(self, basis_vectors) -> None:
        self.m_basisVectors = np.ascontiguousarray(basis_vectors, dtype=np.int32)

    def get_basis_vectors(self) -> np.ndarray:
        return self.m_basisVectors

    def get_energies(self) -> np.ndarray:
        return self.m_list_energies

    def set_energies(self, energies) -> None:
        self.m_list_energies = np.ascontiguousarray(energies, dtype=np.float64)

    # ---- eigenstates -------------------------------------------------------------------------------
    def _solve(self, k_reduced: np.ndarray):
        import torch

        L = N.load()
        nb = self.m_nb_bands_total
        ctx = _Context(self.material, self.m_basisVectors, False, False, N.UEPM_PREC_FP64)
        try:
            n, m = ctx.n, len(k_reduced)
            dev = torch.device("cuda")
            dk = torch.from_numpy(np.ascontiguousarray(k_reduced, dtype=np.float64)).to(dev)
            E = torch.zeros((m, nb), dtype=torch.float64, device=dev)
            X = torch.zeros((m, nb, n, 2), dtype=torch.float64, device=dev)
            st = torch.zeros(m, dtype=torch.int32, device=dev)
            p = lambda t: C.c_void_p(t.data_ptr())
            sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
            N.check(L.uepm_solve_device(ctx.h, p(dk), m, nb, N.UEPM_WANT_VALUES | N.UEPM_WANT_VECTORS, p(E), p(X), None,
                                        p(st), sp))
            if st.any().item():
                raise RuntimeError("Eigenvalue decomposition failed")
            return E, X
        finally:
            ctx.close()

    def compute_eigenstates(self, nb_threads: int = 1) -> None:
        self._k = self._solve(self.reduced())

    def compute_shifted_eigenstates(self, q_shift, nb_threads: int = 1) -> None:
        """q_shift in reduced units (2 pi / a), kept in SI as the reference's m_q_shift."""
        q = np.asarray(q_shift, dtype=np.float64).reshape(3)
        self.m_q_shift = q * (2.0 * math.pi / self.material.get_lattice_constant_meter())
        self._kq = self._solve(self.reduced() + q[None, :])

    def get_eigen_states(self) -> np.ndarray:
        """The eigenvectors at k, [vertex][band][basis] complex (the reference holds n x nb matrices)."""
        if self._k is None:
            return np.zeros((0, self.m_nb_bands_total, 0), dtype=np.complex128)
        X = self._k[1].cpu().numpy()
        return X[..., 0] + 1j * X[..., 1]

    # ---- dielectric function -----------------------------------------------------------------------
    def vertex_weights(self) -> np.ndarray:
        """Sum over the tetrahedra holding each vertex of |signed volume| / 4."""
        w = np.zeros(len(self.positions))
        np.add.at(w, self.tetra.ravel(), np.repeat(np.abs(self.tetra_volumes) * 0.25, 4))
        return w

    def compute_dielectric_function(self, energies, eta_smearing: float, nb_threads: int = 1) -> None:
        import torch

        if self._k is None or self._kq is None:
            raise RuntimeError("compute_eigenstates and compute_shifted_eigenstates first")
        nb = self.m_nb_bands_total
        if nb <= FIRST_CONDUCTION_BAND:
            raise ValueError("the dielectric function needs bands above the first conduction band (index 4)")
        self.m_list_energies = np.ascontiguousarray(energies, dtype=np.float64)
        ne = len(self.m_list_energies)
        L = N.load()
        dev = torch.device("cuda")
        Ek, Xk = self._k
        Ekq, Xkq = self._kq
        w = self.vertex_weights()
        self.total_volume = float(np.abs(self.tetra_volumes).sum())
        dw = torch.from_numpy(w).to(dev)
        den = torch.from_numpy(self.m_list_energies).to(dev)
        sums = torch.zeros(max(ne, 1), dtype=torch.float64, device=dev)
        p = lambda t: C.c_void_p(t.data_ptr())
        sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        if ne and len(w):
            N.check(L.uepm_dielectric_sums_device(p(Xk), p(Xkq), p(Ek), p(Ekq), len(w), nb, Xk.shape[2],
                                                  FIRST_CONDUCTION_BAND, p(den), ne, float(eta_smearing), p(dw), p(sums),
                                                  sp))
        total = sums.cpu().numpy()[:ne]
        q2 = float(np.dot(self.m_q_shift, self.m_q_shift))
        coulomb = (Q_E * Q_E) / (EPS_0 * q2) / Q_E
        prefactor = coulomb * (2.0 / (2.0 * math.pi) ** 3)
        self.m_dielectric_function_real = 1.0 + prefactor * total

    def export_dielectric_function(self, prefix: str) -> None:
        with open(prefix + "_dielectric_function.csv", "w") as f:
            f.write("Energy (eV),Dielectric function\n")
            for e, v in zip(self.m_list_energies, self.m_dielectric_function_real):
                f.write(f"{float(e):g},{float(v):g}\n")

    def compute_fermi_level(self, doping_concentration: float, temperature: float) -> float:
        return 0.0  # bz_states.cpp:152-155 (not implemented there)

    def export_full_eigenstates(self) -> None:
        """eigenstates/eigenvalues/{eigenvalues,shiftedeigenvalues}_<k>.txt and the vectors, one file
        per vertex (bz_states.cpp:169-200)."""
        import shutil

        shutil.rmtree("eigenstates", ignore_errors=True)
        os.makedirs("eigenstates/eigenvectors")
        os.makedirs("eigenstates/eigenvalues")
        Ek = self._k[0].cpu().numpy()
        Ekq = self._kq[0].cpu().numpy()
        Xk = self.get_eigen_states()
        X2 = self._kq[1].cpu().numpy()
        Xkq = X2[..., 0] + 1j * X2[..., 1]
        for i in range(len(Ek)):
            np.savetxt(f"eigenstates/eigenvalues/eigenvalues_{i}.txt", Ek[i][None, :])
            np.savetxt(f"eigenstates/eigenvalues/shiftedeigenvalues_{i}.txt", Ekq[i][None, :])
            np.savetxt(f"eigenstates/eigenvectors/eigenvectors_{i}.txt", Xk[i].T)
            np.savetxt(f"eigenstates/eigenvectors/shiftedeigenvectors_{i}.txt", Xkq[i].T)
