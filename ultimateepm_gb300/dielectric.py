"""Dielectric function from the band states, computed on the GPU.

Mirrors ``uepm::pseudopotential::DielectricFunction`` (src/EPP/DielectricFunction.hpp:24-210,
DielectricFunction.cpp): the same class, method names, arguments and defaults. The eigenstates at k
and k + q come from the context's solve with vectors (``uepm_solve_device``), and the squared
overlaps with their smeared-pair sums over the energy grid from ``uepm_dielectric_sums_device``;
nothing leaves the device but the [q][energy] sums.

As in the reference:
- ``compute_dielectric_function`` covers the k range [offset, offset + nb_kpoints) set with
  ``set_offset_k_index`` / ``set_nb_kpoints`` (the per-process block of apps/epsilon.cpp), and its
  result per q is the un-normalised sum over that range (DielectricFunction.cpp:144-150);
- ``merge_results`` adds the instances' sums, divides by the total k count and forms
  1 + (2 pi / |q|^2) x (DielectricFunction.cpp:152-212);
- ``apply_kramers_kronig`` takes the imaginary part from the real one with the reference's matrix
  (DielectricFunction.cpp:214-251).
``generate_k_points_random`` takes an optional seed (the reference draws from std::random_device).
The band states are solved in FP64 (the drop-in precision) unless ``precision`` asks for the mixed
path; the k range is processed in chunks of ``chunk`` k-points, each solved once at k and once per q
at k + q.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _native as N
from .api import Material, _Context

FIRST_CONDUCTION_BAND = 4  # index_first_conduction_band (DielectricFunction.cpp:84)


def is_in_first_BZ(k, one_eighth: bool = False) -> bool:  # noqa: N802 (reference name)
    """is_in_first_BZ (DielectricFunction.cpp:35-40), reduced units."""
    x, y, z = (float(v) for v in k)
    c1 = abs(x) <= 1.0 and abs(y) <= 1.0 and abs(z) <= 1.0
    c2 = abs(x) + abs(y) + abs(z) <= 3.0 / 2.0
    return c1 and c2 and ((x >= 0.0 and y >= 0.0 and z >= 0.0) if one_eighth else True)


def is_in_irreducible_wedge(k) -> bool:
    """is_in_irreducible_wedge (DielectricFunction.cpp:31-33)."""
    x, y, z = (float(v) for v in k)
    return z >= 0.0 and y >= z and x >= y and x <= 1.0 and x + y + z <= 3.0 / 2.0


class DielectricFunction:
    def __init__(self, material: Material, basisVectors, nb_bands: int, precision: int = N.UEPM_PREC_FP64):
        self.m_material = material
        self.m_basisVectors = np.ascontiguousarray(basisVectors, dtype=np.int32)
        self.m_nb_bands = int(nb_bands)
        self.m_nonlocal_epm = False
        self.m_kpoints = np.zeros((0, 3))
        self.m_qpoints: list = []
        self.m_energies = np.zeros(0)
        self.m_offset_k_index = 0
        self.m_nb_kpoints = 0
        self.m_dielectric_function_real: list = []
        self.m_dielectric_function_imag: list = []
        self.m_export_prefix = "dielectric_function"
        self.precision = precision
        self.chunk = 4096

    # ---- k-points ---------------------------------------------------------------------------------
    def set_non_local_epm(self, new_value: bool) -> None:
        self.m_nonlocal_epm = bool(new_value)

    def generate_k_points_random(self, nb_points: int, seed: int | None = None) -> None:
        """Uniform in [-1, 1]^3, kept in the first zone until nb_points are held (appends, as the
        reference's loop does)."""
        rng = np.random.default_rng(seed)
        pts = [tuple(v) for v in self.m_kpoints]
        while len(pts) < nb_points:
            k = rng.uniform(-1.0, 1.0, size=3)
            if is_in_first_BZ(k):
                pts.append(tuple(k))
        self.m_kpoints = np.array(pts, dtype=np.float64).reshape(-1, 3)

    def generate_k_points_grid(self, Nx: int, Ny: int, Nz: int, shift: float, irreducible_wedge: bool) -> None:
        """DielectricFunction.cpp:59-76: N - 1 points per axis over [-1 - shift, 1 + shift]."""
        lo, hi = -1.0 - shift, 1.0 + shift
        i, j, k = np.meshgrid(np.arange(Nx - 1), np.arange(Ny - 1), np.arange(Nz - 1), indexing="ij")
        pts = np.stack([lo + (hi - lo) * i.ravel() / float(Nx - 1), lo + (hi - lo) * j.ravel() / float(Ny - 1),
                        lo + (hi - lo) * k.ravel() / float(Nz - 1)], axis=1)
        keep = [is_in_first_BZ(p) and (not irreducible_wedge or is_in_irreducible_wedge(p)) for p in pts]
        self.m_kpoints = np.ascontiguousarray(pts[np.array(keep, dtype=bool)]) if len(pts) else np.zeros((0, 3))

    def get_kpoints(self) -> np.ndarray:
        return self.m_kpoints

    def get_offset_k_index(self) -> int:
        return self.m_offset_k_index

    def get_nb_kpoints(self) -> int:
        return self.m_nb_kpoints

    def set_offset_k_index(self, offset_k_index: int) -> None:
        self.m_offset_k_index = int(offset_k_index)

    def set_nb_kpoints(self, nb_kpoints: int) -> None:
        self.m_nb_kpoints = int(nb_kpoints)

    def set_qpoints(self, qpoints) -> None:
        self.m_qpoints = [np.asarray(q, dtype=np.float64).reshape(3) for q in qpoints]

    def set_energies(self, energies) -> None:
        self.m_energies = np.ascontiguousarray(energies, dtype=np.float64)

    def set_export_prefix(self, prefix: str) -> None:
        self.m_export_prefix = prefix

    # ---- the sums ---------------------------------------------------------------------------------
    def compute_dielectric_function(self, eta_smearing: float = 1e-2, mpi_rank: int = 0) -> None:
        """One [energy] sum per q over the k range (DielectricFunction.cpp:83-150), appended to the
        results as the reference appends them."""
        import torch

        if self.m_nb_bands <= FIRST_CONDUCTION_BAND:
            raise ValueError("the dielectric function needs bands above the first conduction band (index 4)")
        L = N.load()
        ne = len(self.m_energies)
        nq = len(self.m_qpoints)
        a, b = self.m_offset_k_index, self.m_offset_k_index + self.m_nb_kpoints
        if b > len(self.m_kpoints):
            raise IndexError("k range beyond the k-points")
        ctx = _Context(self.m_material, self.m_basisVectors, self.m_nonlocal_epm, False, self.precision)
        try:
            n, nb = ctx.n, self.m_nb_bands
            stream = torch.cuda.current_stream()
            sp = C.c_void_p(stream.cuda_stream)
            dev = torch.device("cuda")
            den = torch.from_numpy(self.m_energies).to(dev)
            sums = torch.zeros((max(nq, 1), max(ne, 1)), dtype=torch.float64, device=dev)
            qs = []
            for q in self.m_qpoints:  # DielectricFunction.cpp:96-99
                qs.append(np.array([1e-15, 1e-15, 1e-15]) if math.sqrt(float(np.dot(q, q))) <= 1e-15 else q)
            want = N.UEPM_WANT_VALUES | N.UEPM_WANT_VECTORS
            for c0 in range(a, b, self.chunk):
                c1 = min(b, c0 + self.chunk)
                m = c1 - c0
                k = torch.from_numpy(np.ascontiguousarray(self.m_kpoints[c0:c1])).to(dev)
                Ek = torch.zeros((m, nb), dtype=torch.float64, device=dev)
                Xk = torch.zeros((m, nb, n, 2), dtype=torch.float64, device=dev)
                Ekq = torch.zeros_like(Ek)
                Xkq = torch.zeros_like(Xk)
                st = torch.zeros(m, dtype=torch.int32, device=dev)
                ptr = lambda t: C.c_void_p(t.data_ptr())
                N.check(L.uepm_solve_device(ctx.h, ptr(k), m, nb, want, ptr(Ek), ptr(Xk), None, ptr(st), sp))
                for iq, q in enumerate(qs):
                    kq = k + torch.from_numpy(q).to(dev)[None, :]
                    N.check(L.uepm_solve_device(ctx.h, ptr(kq), m, nb, want, ptr(Ekq), ptr(Xkq), None, ptr(st), sp))
                    if ne:
                        N.check(L.uepm_dielectric_sums_device(ptr(Xk), ptr(Xkq), ptr(Ek), ptr(Ekq), m, nb, n,
                                                              FIRST_CONDUCTION_BAND, ptr(den), ne, float(eta_smearing),
                                                              None, ptr(sums[iq]), sp))
                if st.any().item():
                    raise RuntimeError("Eigenvalue decomposition failed")
            host = sums.cpu().numpy()
        finally:
            ctx.close()
        for iq in range(nq):
            self.m_dielectric_function_real.append(host[iq, :ne].copy())

    def clear_eigen_states(self) -> None:
        """The reference frees its cached eigenstates; the device ones here live only per call."""

    def get_dielectric_function(self) -> list:
        return self.m_dielectric_function_real

    def get_flat_dielectric_function(self) -> np.ndarray:
        if not self.m_dielectric_function_real:
            return np.zeros(0)
        return np.concatenate([np.asarray(r, dtype=np.float64) for r in self.m_dielectric_function_real])

    @staticmethod
    def merge_results(RootDielectricFunction: "DielectricFunction", dielectric_function_results,
                      nb_kpoints_per_instance) -> "DielectricFunction":
        """DielectricFunction.cpp:152-212 (a copy of the root with the merged, normalised function)."""
        import copy

        if len(dielectric_function_results) == 0:
            raise RuntimeError("No results to merge")
        if len(dielectric_function_results) != len(nb_kpoints_per_instance):
            raise RuntimeError("Number of results and number of k-points per instance do not match")
        total = [np.array(r, dtype=np.float64).copy() for r in dielectric_function_results[0]]
        for inst in dielectric_function_results[1:]:
            for iq, r in enumerate(inst):
                total[iq] += np.asarray(r, dtype=np.float64)
        ren = 1.0 / float(sum(int(c) for c in nb_kpoints_per_instance))
        for iq in range(len(total)):
            q = RootDielectricFunction.m_qpoints[iq]
            q2 = math.sqrt(float(np.dot(q, q))) ** 2
            if q2 == 0.0:
                q2 = 1e-14
            total[iq] = 1.0 + (2.0 * math.pi / q2) * (total[iq] * ren)
        out = copy.copy(RootDielectricFunction)
        out.m_dielectric_function_real = total
        return out

    def apply_kramers_kronig(self) -> None:
        n = len(self.m_energies)
        K = create_kramers_matrix(n)
        self.m_dielectric_function_imag = [K @ (np.asarray(r, dtype=np.float64) - 1.0)
                                           for r in self.m_dielectric_function_real]

    # ---- export -----------------------------------------------------------------------------------
    def export_kpoints(self, filename: str) -> None:
        with open(filename, "w") as f:
            f.write("X,Y,Z\n")
            for k in self.m_kpoints:
                f.write(f"{_g(k[0])},{_g(k[1])},{_g(k[2])}\n")

    def export_dielectric_function_at_q(self, filename: str, idx_q: int, name_auto: bool) -> None:
        if name_auto:
            q = self.m_qpoints[idx_q]
            outname = f"{self.m_export_prefix}_{idx_q:05d}_{q[0]:.6f}_{q[1]:.6f}_{q[2]:.6f}.csv"
        else:
            outname = filename
        imag = self.m_dielectric_function_imag[idx_q] if idx_q < len(self.m_dielectric_function_imag) else None
        with open(outname, "w") as f:
            f.write("Energy (eV),EpsilonReal,EpsilonImaginary\n")
            for e in range(len(self.m_energies)):
                im = _g(imag[e]) if imag is not None else "0"
                f.write(f"{_g(self.m_energies[e])},{_g(self.m_dielectric_function_real[idx_q][e])},{im}\n")

    def export_dielectric_function(self, filename: str, name_auto: bool) -> None:
        for iq in range(len(self.m_qpoints)):
            self.export_dielectric_function_at_q(filename, iq, name_auto)


def create_kramers_matrix(N_: int) -> np.ndarray:
    """create_kramers_matrix (DielectricFunction.cpp:214-228)."""
    i = np.arange(N_, dtype=np.float64)[:, None]
    j = np.arange(N_, dtype=np.float64)[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        K = np.where(i == j, 0.0, i / (j * j - i * i))
    return K * (-2.0 / math.pi)


def _g(x: float) -> str:
    """std::ostream's default formatting of a double (6 significant digits, %g)."""
    return f"{float(x):g}"
