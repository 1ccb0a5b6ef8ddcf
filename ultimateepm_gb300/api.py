"""Python mirror of the reference's src/EPP interface over the GB300 C ABI.

Same class and method names as ``uepm::pseudopotential`` (Material / Materials / BandStructure /
Hamiltonian / SymmetryPoints), same argument meaning and the same error behaviour, mapped to Python
exceptions: std::invalid_argument -> ValueError, std::runtime_error -> RuntimeError,
std::out_of_range -> IndexError. Every computation runs through libuepm_gb300.so on the GPU.

Reference files: src/EPP/Material.{h,cpp}, BandStructure.{h,cpp}, Hamiltonian.{h,cpp},
SymmetryPoints.{h,cpp}.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _native as N


def _raise(code: int):
    msg = N.last_error()
    if code == N.UEPM_ERR_INVALID:
        raise ValueError(msg)
    if code == N.UEPM_ERR_OUT_OF_RANGE:
        raise IndexError(msg)
    raise RuntimeError(msg)


def _ok(code: int) -> int:
    if code < 0:
        _raise(code)
    return code


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Material:
    """uepm::pseudopotential::Material (src/EPP/Material.h:14-175). The constructor takes the form
    factors in eV, as the reference's does; YAML loading converts from Ry."""

    def __init__(self, name: str = "", a: float = 0.0, V3S=0.0, V4S=0.0, V8S=0.0, V11S=0.0,
                 V3A=0.0, V4A=0.0, V8A=0.0, V11A=0.0, raw: N.UepmMaterial | None = None):
        self.name = name
        self.raw = raw if raw is not None else N.UepmMaterial()
        if raw is None:
            self.raw.lattice_constant = a
            for k, v in dict(V3S=V3S, V4S=V4S, V8S=V8S, V11S=V11S, V3A=V3A, V4A=V4A, V8A=V8A, V11A=V11A).items():
                setattr(self.raw, k, v)

    def get_name(self) -> str:
        return self.name

    def get_lattice_constant_meter(self) -> float:
        return 1.0e-10 * self.raw.lattice_constant

    def is_non_local_parameters_populated(self) -> bool:
        return bool(self.raw.has_nonlocal)

    def is_spin_orbit_parameters_populated(self) -> bool:
        return bool(self.raw.has_soc)


class Materials:
    """uepm::pseudopotential::Materials: ``materials`` maps symbol -> Material."""

    def __init__(self):
        self.materials: dict[str, Material] = {}

    def load_material_parameters(self, filename: str) -> None:
        L = N.load()
        cnt = _ok(L.uepm_materials_load(filename.encode(), None, None, 0, 0))
        arr = (N.UepmMaterial * max(cnt, 1))()
        stride = 32
        syms = C.create_string_buffer(stride * max(cnt, 1))
        _ok(L.uepm_materials_load(filename.encode(), arr, syms, stride, cnt))
        for i in range(cnt):
            sym = syms.raw[i * stride:(i + 1) * stride].split(b"\0", 1)[0].decode()
            raw = N.UepmMaterial()
            C.memmove(C.byref(raw), C.byref(arr[i]), C.sizeof(raw))
            self.materials[sym] = Material(sym, raw=raw)


class SymmetryPoints:
    """uepm::pseudopotential::SymmetryPoints (L, G, X, W, K, U)."""

    def GeneratePoints(self, path, nrPoints: int):
        labels = "".join(path)
        k = np.zeros((max(nrPoints, 1), 3))
        pos = (C.c_uint32 * max(len(labels), 1))()
        cnt = _ok(N.load().uepm_generate_path(labels.encode(), nrPoints, _dp(k), nrPoints, pos))
        return k[:cnt].copy(), [int(pos[i]) for i in range(len(labels))]


def generate_basis_vectors(shells: int) -> np.ndarray:
    L = N.load()
    n = L.uepm_generate_basis(shells, None, 0)
    if n < 0:
        raise RuntimeError("BandStructure::Initialize: GenerateBasisVectors failed")
    G = np.zeros((n, 3), dtype=np.int32)
    L.uepm_generate_basis(shells, _ip(G), n)
    return G


class _Context:
    """One uepm_ctx: the material, basis and flags resident on the GPU."""

    def __init__(self, material: Material, G: np.ndarray, nl: bool, soc: bool, precision: int = N.UEPM_PREC_FP64,
                 force_complex: bool = False):
        L = N.load()
        self.G = np.ascontiguousarray(G, dtype=np.int32)
        flags = (N.UEPM_NONLOCAL if nl else 0) | (N.UEPM_SOC if soc else 0)
        h = C.c_void_p()
        _ok(L.uepm_ctx_create(C.byref(material.raw), _ip(self.G), self.G.shape[0], flags, C.byref(h)))
        self.h = h
        self.n = L.uepm_ctx_order(h)
        self.real = bool(_ok(L.uepm_ctx_force_complex(h, int(force_complex))))
        self.set_precision(precision)

    def set_precision(self, precision: int):
        _ok(N.load().uepm_ctx_set_precision(self.h, precision))
        self.precision = precision

    def solve(self, k: np.ndarray, nb: int, vectors=False, gradient=False):
        L = N.load()
        k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
        nk = k.shape[0]
        E = np.zeros((nk, nb))
        X = np.zeros((nk, nb, self.n), dtype=np.complex128) if vectors else None
        g = np.zeros((nk, nb, 3)) if gradient else None
        st = np.zeros(nk, dtype=np.int32)
        want = N.UEPM_WANT_VALUES | (N.UEPM_WANT_VECTORS if vectors else 0) | (N.UEPM_WANT_GRADIENT if gradient else 0)
        rc = L.uepm_solve(self.h, _dp(k), nk, nb, want, _dp(E), _dp(X) if vectors else None,
                          _dp(g) if gradient else None, _ip(st))
        if rc == N.UEPM_ERR_NOT_CONVERGED:
            raise RuntimeError("Eigenvalue decomposition failed: " + N.last_error())
        _ok(rc)
        return E, X, g, st

    def close(self):
        if getattr(self, "h", None):
            N.load().uepm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BandStructure:
    """uepm::pseudopotential::BandStructure (src/EPP/BandStructure.h:28-79) on the GPU."""

    def __init__(self):
        self.m_nb_points = 0
        self.m_nb_bands = 10
        self.m_nearestNeighborsNumber = 10
        self.m_computation_time_s = -1.0
        self.m_path: list[str] = []
        self.m_kpoints = np.zeros((0, 3))
        self.m_energies = np.zeros((0, 0))
        self.m_energies_gradient = None
        self.m_enable_spin_orbit_coupling = False
        self.m_enable_non_local_correction = False
        self.symmetryPointsPositions: list[int] = []
        self.basisVectors = np.zeros((0, 3), dtype=np.int32)
        self.precision = N.UEPM_PREC_FP64
        self._ctx: _Context | None = None

    def set_precision(self, precision: str | int):
        self.precision = {"fp64": N.UEPM_PREC_FP64, "mixed": N.UEPM_PREC_MIXED}.get(precision, precision)
        if self._ctx:
            self._ctx.set_precision(self.precision)

    def Initialize(self, material: Material, nb_bands: int, path_or_kpoints, nearestNeighborsNumber: int,
                   enable_non_local_correction: bool, enable_soc: bool, nrPoints: int | None = None):
        """Both reference overloads: a list of labels plus nrPoints (path), or an [nk, 3] k list."""
        self.m_material = material
        self.m_nb_bands = int(nb_bands)
        self.m_nearestNeighborsNumber = nearestNeighborsNumber
        self.m_enable_non_local_correction = bool(enable_non_local_correction)
        self.m_enable_spin_orbit_coupling = bool(enable_soc)
        if self.m_enable_spin_orbit_coupling:
            self.m_nb_bands *= 2  # BandStructure.cpp:78-82 / :109-113
        self.basisVectors = generate_basis_vectors(nearestNeighborsNumber)
        if isinstance(path_or_kpoints, (list, tuple)) and path_or_kpoints and isinstance(path_or_kpoints[0], str):
            self.m_path = list(path_or_kpoints)
            k, pos = SymmetryPoints().GeneratePoints(self.m_path, int(nrPoints))
            if len(k) == 0:
                raise RuntimeError("BandStructure::Initialize: GeneratePoints failed. No points generated.")
            self.m_kpoints, self.symmetryPointsPositions = k, pos
        else:
            self.m_path = []
            self.m_kpoints = np.ascontiguousarray(path_or_kpoints, dtype=np.float64).reshape(-1, 3)
        self.m_nb_points = len(self.m_kpoints)
        self._ctx = None

    def set_kpoints(self, kpoints):
        self.m_kpoints = np.ascontiguousarray(kpoints, dtype=np.float64).reshape(-1, 3)

    def _context(self) -> _Context:
        if self._ctx is None:
            self._ctx = _Context(self.m_material, self.basisVectors, self.m_enable_non_local_correction,
                                 self.m_enable_spin_orbit_coupling, self.precision)
        return self._ctx

    def Compute(self, compute_gradient: bool = False):
        # The reference's serial Compute keeps no gradients (BandStructure.cpp:124-149).
        self._run(False)

    def Compute_parallel(self, compute_gradient: bool = False, nb_threads: int = 1):
        self._run(bool(compute_gradient))

    def _run(self, grad: bool):
        t0 = time.perf_counter()
        ctx = self._context()
        self.m_nb_points = len(self.m_kpoints)
        nb = min(self.m_nb_bands, ctx.n)
        E, _, g, _ = ctx.solve(self.m_kpoints, nb, gradient=grad)
        self.m_energies = E
        self.m_energies_gradient = g
        # whole seconds, like the reference's duration_cast<seconds>
        self.m_computation_time_s = float(int(time.perf_counter() - t0))

    def AdjustValues(self, minConductionBandToZero: bool = False) -> float:
        E = np.ascontiguousarray(self.m_energies)
        gap = C.c_double(0.0)
        found = C.c_int32(0)
        _ok(N.load().uepm_adjust_values(_dp(E), E.shape[0], E.shape[1], int(self.m_enable_spin_orbit_coupling),
                                         int(minConductionBandToZero), C.byref(gap), C.byref(found)))
        self.m_energies = E
        return gap.value

    def get_band_energies(self):
        return self.m_energies

    def get_band_energy_gradients(self):
        return self.m_energies_gradient

    def get_basis_vectors(self):
        return self.basisVectors

    def get_kpoints(self):
        return self.m_kpoints

    def get_number_of_bands(self) -> int:
        return self.m_nb_bands

    def get_computation_time_s(self) -> float:
        return self.m_computation_time_s

    def is_soc_enabled(self) -> bool:
        return self.m_enable_spin_orbit_coupling

    def get_path_as_string(self) -> str:
        return "".join(self.m_path)

    def path_band_filename(self) -> str:
        return (f"EPM_{self.m_material.get_name()}_nb_bands_{self.m_energies.shape[1]}_path_"
                f"{self.get_path_as_string()}_size_basis_{len(self.basisVectors)}")

    def export_result_in_file(self, filename: str):
        """Band file read by python/plots/plot_band_structure.py (BandStructure.cpp:290-314)."""
        nbnd = self.m_energies.shape[1]
        with open(filename, "w") as f:
            f.write(f"# Material {self.m_material.get_name()}\n")
            f.write(f"# NBands {self.m_nb_bands}\n")
            f.write(f"# Nonlocal {'Yes' if self.m_enable_non_local_correction else 'No'}\n")
            f.write(f"# Path {self.get_path_as_string()}\n")
            f.write("# Symmetry points:" + "".join(f" {p}" for p in self.symmetryPointsPositions) + "\n")
            f.write(",".join(f"band_{i}" for i in range(nbnd)) + "\n")
            for row in self.m_energies:
                f.write(",".join(_fmt(v) for v in row) + "\n")


def _fmt(v: float) -> str:
    # std::ostream default formatting: 6 significant digits, %g style
    return f"{v:.6g}"


class Hamiltonian:
    """uepm::pseudopotential::Hamiltonian (src/EPP/Hamiltonian.h:10-32) for single k-points."""

    def __init__(self, material: Material, basisVectors: np.ndarray):
        self.m_material = material
        self.m_basisVectors = np.ascontiguousarray(basisVectors, dtype=np.int32)
        self._k = None
        self._flags = (False, False)
        self._ctx: dict = {}
        self._vals = None
        self._vecs = None

    def SetMatrix(self, k, add_non_local_correction: bool = False, enable_soc: bool = False):
        self._k = np.asarray(k, dtype=np.float64).reshape(1, 3)
        self._flags = (bool(add_non_local_correction), bool(enable_soc))

    def _context(self) -> _Context:
        if self._flags not in self._ctx:
            self._ctx[self._flags] = _Context(self.m_material, self.m_basisVectors, *self._flags)
        return self._ctx[self._flags]

    def Diagonalize(self, keep_eigenvectors: bool = False):
        ctx = self._context()
        E, X, _, _ = ctx.solve(self._k, ctx.n, vectors=keep_eigenvectors)
        self._vals = E[0]
        # Eigen layout: column c = eigenvector of eigenvalue c
        self._vecs = X[0].T.copy() if keep_eigenvectors else np.zeros((0, 0), dtype=np.complex128)

    def eigenvalues(self):
        return self._vals

    def get_eigenvalues(self):
        return self._vals

    def get_eigenvectors(self):
        return self._vecs

    def compute_gradient_at_level(self, k_point, level_index: int):
        if self._vecs is None or self._vecs.size == 0:
            raise RuntimeError("compute_gradient_at_level: eigenvectors not available. Call Diagonalize(true) first.")
        if level_index >= self._vecs.shape[1]:
            raise IndexError("compute_gradient_at_level: level_index out of range")
        ctx = self._context()
        _, _, g, _ = ctx.solve(np.asarray(k_point, dtype=np.float64).reshape(1, 3), level_index + 1, gradient=True)
        return g[0, level_index]
