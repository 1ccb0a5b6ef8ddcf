"""CPU ORACLE wrapper (test infrastructure only).

ctypes bindings over ``oracle/lib/liboracle.so`` (the restatement in ``epm_oracle.cpp``) and, where it
was built, ``oracle/_ref/libref.so`` (the reference's own Pseudopotential / SymmetryPoints / Bessel
code). Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module,
and only as the checker: nothing in the product imports it.

It also holds an independent reader for the reference's material YAML format
(src/EPP/Material.cpp:33-71 semantics: V* and alpha_0/A2 from Ry to eV, radii from Angstrom to m,
beta_0 and the spin-orbit numbers raw), so the product's own loader can be cross-checked.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liboracle.so")
FAST_LIB_PATH = os.path.join(HERE, "lib", "liboracle_fast.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")
# Root of the reference source tree (read only by the checker build and the fixture script; absent
# on machines that only run the committed fixtures).
REFERENCE_ROOT = os.environ.get("UEPM_REFERENCE_ROOT", "/root/reference")

# src/Common/physical_constants.hpp:18-44
H_PLANCK = 6.62607015e-34
Q_E = 1.602176634e-19
M_E = 9.1093837015e-31
PI = 3.141592653589793
H_BAR = H_PLANCK / (2.0 * PI)
RYD_TO_EV = (4.3597447222071e-18 / Q_E) / 2.0
ANGSTROM_TO_M = 1e-10


class OrMaterial(C.Structure):
    """Same layout as ``or_material`` (epm_oracle.cpp) and the product's ``uepm_material``."""

    _fields_ = [
        ("lattice_constant", C.c_double),
        ("V3S", C.c_double), ("V4S", C.c_double), ("V8S", C.c_double), ("V11S", C.c_double),
        ("V3A", C.c_double), ("V4A", C.c_double), ("V8A", C.c_double), ("V11A", C.c_double),
        ("nl_well", C.c_int32), ("has_nonlocal", C.c_int32),
        ("alpha0_cation", C.c_double), ("beta0_cation", C.c_double), ("A2_cation", C.c_double),
        ("alpha0_anion", C.c_double), ("beta0_anion", C.c_double), ("A2_anion", C.c_double),
        ("R0_cation", C.c_double), ("R2_cation", C.c_double), ("R0_anion", C.c_double), ("R2_anion", C.c_double),
        ("period_anion", C.c_uint32), ("period_cation", C.c_uint32),
        ("has_soc", C.c_int32), ("_pad", C.c_int32),
        ("radial_extent_anion", C.c_double), ("radial_extent_cation", C.c_double),
        ("alpha_soc", C.c_double), ("mu_soc", C.c_double),
    ]


# ---------------------------------------------------------------------------------------------
# Minimal reader for the reference's material YAML files (a block-style subset: maps, a sequence
# of maps, scalars, comments, document marker).

def _scalar(s: str):
    s = s.strip()
    if len(s) >= 2 and s[0] == s[-1] and s[0] in "\"'":
        return s[1:-1]
    try:
        if any(ch in s for ch in ".eE") and not s.isalpha():
            return float(s)
        return int(s)
    except ValueError:
        try:
            return float(s)
        except ValueError:
            return s


def parse_yaml_subset(text: str):
    lines = []
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip() or line.strip() == "---":
            continue
        lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    pos = 0

    def block(indent):
        nonlocal pos
        if pos >= len(lines):
            return None
        if lines[pos][1].startswith("- "):
            seq = []
            while pos < len(lines) and lines[pos][0] == indent and lines[pos][1].startswith("- "):
                ind, txt = lines[pos]
                lines[pos] = (ind + 2, txt[2:].lstrip())
                seq.append(block(ind + 2))
            return seq
        out = {}
        while pos < len(lines) and lines[pos][0] == indent and not lines[pos][1].startswith("- "):
            _, txt = lines[pos]
            key, _, val = txt.partition(":")
            pos += 1
            if val.strip():
                out[key.strip()] = _scalar(val)
            elif pos < len(lines) and lines[pos][0] > indent:
                out[key.strip()] = block(lines[pos][0])
            elif pos < len(lines) and lines[pos][0] == indent and lines[pos][1].startswith("- "):
                out[key.strip()] = block(indent)
            else:
                out[key.strip()] = None
        return out

    return block(lines[0][0]) if lines else {}


def load_materials(path: str) -> dict:
    """Materials::load_material_parameters (src/EPP/Material.cpp:33-71) -> {symbol: OrMaterial}."""
    with open(path) as f:
        doc = parse_yaml_subset(f.read())
    out = {}
    for m in doc["materials"]:
        pp = m["pseudo-potential-parameters"]
        mat = OrMaterial()
        mat.lattice_constant = float(m["lattice-constant"])
        for key in ("V3S", "V8S", "V11S", "V3A", "V4A", "V11A"):
            setattr(mat, key, RYD_TO_EV * float(pp[key]))
        mat.V4S = RYD_TO_EV * float(pp["V4S"]) if "V4S" in pp else 0.0
        mat.V8A = RYD_TO_EV * float(pp["V8A"]) if "V8A" in pp else 0.0
        nl = m.get("non-local-parameters")
        if nl:
            mat.has_nonlocal = 1
            for key in ("alpha_0_cation", "alpha_0_anion", "A2_cation", "A2_anion"):
                setattr(mat, key.replace("alpha_0", "alpha0"), RYD_TO_EV * float(nl[key]))
            mat.beta0_cation = float(nl["beta_0_cation"])
            mat.beta0_anion = float(nl["beta_0_anion"])
            for key in ("R0_cation", "R2_cation", "R0_anion", "R2_anion"):
                setattr(mat, key, float(nl[key]) * ANGSTROM_TO_M)
            well = nl["well_type"]
            if well not in ("square", "gaussian"):
                raise RuntimeError("Unknown non-local well type")
            mat.nl_well = 1 if well == "square" else 2
        so = m.get("spin-orbit-parameters")
        if so:
            mat.has_soc = 1
            mat.period_anion = int(so["period_anion"])
            mat.period_cation = int(so["period_cation"])
            mat.radial_extent_anion = float(so["radial_extent_anion"])
            mat.radial_extent_cation = float(so["radial_extent_cation"])
            mat.alpha_soc = float(so["alpha_soc"])
            mat.mu_soc = float(so["mu_soc"])
        out[m["symbol"]] = mat
    return out


# ---------------------------------------------------------------------------------------------

_lib = None
_ref = None


def reference_present() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "EPP"))


def build():
    """Compile liboracle.so, liboracle_fast.so (the timed baseline build) and, when the reference
    tree is present, libref.so."""
    env = dict(os.environ, UEPM_REFERENCE_ROOT=REFERENCE_ROOT)
    subprocess.run(["make", "-s", "-C", HERE, "oracle", "fast"], check=True, env=env)
    if reference_present():
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True, env=env)


_fast = None


def fast_lib():
    """The same restatement built with the reference's Release numerics flags (-O3 -ffast-math,
    OpenMP): the timed CPU baseline only, never a parity checker."""
    global _fast
    if _fast is None:
        if not os.path.exists(FAST_LIB_PATH):
            build()
        _fast = _bind(C.CDLL(FAST_LIB_PATH))
    return _fast


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = _bind(C.CDLL(LIB_PATH))
    return _lib


def _bind(L):
    if True:
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        mp = C.POINTER(OrMaterial)
        L.or_material_size.restype = C.c_int
        L.or_generate_basis.argtypes = [C.c_uint, ip, C.c_int]
        L.or_generate_basis.restype = C.c_int
        L.or_pp_value.argtypes = [mp, C.c_int, C.c_int, C.c_int, dp, C.c_double, dp]
        for name in ("or_cyl_bessel", "or_sph_bessel"):
            getattr(L, name).argtypes = [C.c_double, C.c_double]
            getattr(L, name).restype = C.c_double
        L.or_bessel_i2.argtypes = [C.c_double]
        L.or_bessel_i2.restype = C.c_double
        L.or_F_l.argtypes = [dp, dp, C.c_double, C.c_int]
        L.or_F_l.restype = C.c_double
        L.or_F2_gauss.argtypes = [dp, dp, C.c_double]
        L.or_F2_gauss.restype = C.c_double
        L.or_nl_correction.argtypes = [mp, dp, dp, dp, dp]
        L.or_soc_block.argtypes = [mp, dp, dp, dp, dp, dp, dp]
        L.or_soc_block.restype = C.c_int
        L.or_assemble.argtypes = [mp, ip, C.c_int, dp, C.c_int, C.c_int, dp]
        L.or_assemble.restype = C.c_int
        L.or_eigh.argtypes = [C.c_int, dp, dp, dp]
        L.or_eigh.restype = C.c_int
        L.or_gradient.argtypes = [mp, ip, C.c_int, dp, dp, C.c_int, dp]
        L.or_band_structure.argtypes = [mp, ip, C.c_int, dp, C.c_int64, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int, dp, dp, dp, ip]
        L.or_band_structure.restype = C.c_int
        L.or_is_irreducible_wedge.argtypes = [dp]
        L.or_is_irreducible_wedge.restype = C.c_int
        L.or_symmetry_operation.argtypes = [dp, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_symmetry_operation.restype = C.c_int
        L.or_adjust_values.argtypes = [dp, C.c_int64, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.or_adjust_values.restype = C.c_double
        L.or_generate_path.argtypes = [C.c_char_p, C.c_uint, dp, C.c_int, C.POINTER(C.c_uint32)]
        L.or_generate_path.restype = C.c_int
        assert L.or_material_size() == C.sizeof(OrMaterial)
    return L


def ref_lib():
    """The reference's own code for the buildable pieces, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        L = C.CDLL(REF_PATH)
        dp = C.POINTER(C.c_double)
        for name in ("ref_cyl_bessel", "ref_sph_bessel"):
            getattr(L, name).argtypes = [C.c_double, C.c_double]
            getattr(L, name).restype = C.c_double
        L.ref_bessel_i2.argtypes = [C.c_double]
        L.ref_bessel_i2.restype = C.c_double
        L.ref_pp_value.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp, C.c_double, dp]
        L.ref_generate_path.argtypes = [C.c_char_p, C.c_uint, dp, C.c_int, C.POINTER(C.c_uint32), C.c_int]
        L.ref_generate_path.restype = C.c_int
        cp = C.c_char_p
        ip = C.POINTER(C.c_int32)
        L.ref_material.argtypes = [cp, cp, C.POINTER(OrMaterial)]
        L.ref_hamiltonian.argtypes = [cp, cp, ip, C.c_int, dp, C.c_int, C.c_int, C.c_int, dp]
        L.ref_nl_correction.argtypes = [cp, cp, dp, dp, dp, dp]
        L.ref_soc_block.argtypes = [cp, cp, dp, dp, dp, dp, dp, dp]
        L.ref_band_file.argtypes = [cp, cp, C.c_int, cp, C.c_uint, C.c_uint, C.c_int, C.c_int, C.c_int, cp, dp,
                                    C.c_int]
        L.ref_gradient_shape.argtypes = [cp, cp, C.c_int, dp, C.c_int, C.c_uint, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), dp, C.c_int]
        assert L.ref_material_size() == C.sizeof(OrMaterial)
        _ref = L
    return _ref


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def generate_basis(shells: int) -> np.ndarray:
    """BandStructure::GenerateBasisVectors -> int32 [N, 3] in loop order."""
    L = lib()
    n = L.or_generate_basis(shells, None, 0)
    if n < 0:
        raise RuntimeError("BandStructure::Initialize: GenerateBasisVectors failed")
    G = np.zeros((n, 3), dtype=np.int32)
    L.or_generate_basis(shells, _ip(G), n)
    return G


def generate_path(labels: str, n_points: int):
    """SymmetryPoints::GeneratePoints -> (k [n,3], symmetry-point positions)."""
    L = lib()
    out = np.zeros((max(n_points, 1), 3))
    pos = (C.c_uint32 * max(len(labels), 1))()
    cnt = L.or_generate_path(labels.encode(), n_points, _dp(out), n_points, pos)
    if cnt < 0:
        raise ValueError("invalid path")
    return out[:cnt].copy(), [pos[i] for i in range(len(labels))]


def assemble(mat: OrMaterial, G: np.ndarray, k, nl=False, soc=False) -> np.ndarray:
    """H(k) after SetMatrix + the hermitisation of Diagonalize, complex [n, n]."""
    L = lib()
    G = np.ascontiguousarray(G, dtype=np.int32)
    N = G.shape[0]
    n = 2 * N if soc else N
    H = np.zeros((n, n), dtype=np.complex128, order="F")
    kk = np.ascontiguousarray(k, dtype=np.float64)
    st = L.or_assemble(C.byref(mat), _ip(G), N, _dp(kk), int(nl), int(soc), _dp(H))
    if st != 0:
        raise RuntimeError("SpinOrbitCorrection: Unsupported period")
    return H


def eigh(H: np.ndarray, vectors=False):
    """Restated Eigen SelfAdjointEigenSolver: ascending eigenvalues (and eigenvectors)."""
    L = lib()
    n = H.shape[0]
    A = np.array(H, dtype=np.complex128, order="F", copy=True)
    w = np.zeros(n)
    Z = np.zeros((n, n), dtype=np.complex128, order="F") if vectors else None
    info = L.or_eigh(n, _dp(A), _dp(w), _dp(Z) if vectors else None)
    if info != 0:
        raise RuntimeError("Eigenvalue decomposition failed")
    return (w, Z) if vectors else w


def band_structure(mat: OrMaterial, G: np.ndarray, kpts: np.ndarray, nb: int, nl=False, soc=False,
                   grad=False, vectors=False, nthreads=None, fast=False):
    """BandStructure::Compute_parallel over kpts -> dict(E [nk,nb], grad, vecs, status). fast: the
    Release-flags build (timing only)."""
    L = fast_lib() if fast else lib()
    G = np.ascontiguousarray(G, dtype=np.int32)
    k = np.ascontiguousarray(kpts, dtype=np.float64).reshape(-1, 3)
    nk = k.shape[0]
    N = G.shape[0]
    n = 2 * N if soc else N
    E = np.zeros((nk, nb))
    g = np.zeros((nk, nb, 3)) if grad else None
    X = np.zeros((nk, nb, n), dtype=np.complex128) if vectors else None
    st = np.zeros(nk, dtype=np.int32)
    nthreads = nthreads or os.cpu_count() or 1
    L.or_band_structure(C.byref(mat), _ip(G), N, _dp(k), nk, nb, int(nl), int(soc), int(grad), nthreads,
                        _dp(E), _dp(g) if grad else None, _dp(X) if vectors else None, _ip(st))
    return {"E": E, "grad": g, "vecs": X, "status": st}


def adjust_values(E: np.ndarray, soc=False, min_cond_zero=False):
    """BandStructure::AdjustValues in place; returns (gap, found)."""
    L = lib()
    assert E.flags.c_contiguous and E.dtype == np.float64
    found = C.c_int(0)
    gap = L.or_adjust_values(_dp(E), E.shape[0], E.shape[1], int(soc), int(min_cond_zero), C.byref(found))
    return gap, bool(found.value)


def is_irreducible_wedge(k_reduced) -> bool:
    """MeshBZ::is_irreducible_wedge on a reduced k-point."""
    k = np.ascontiguousarray(k_reduced, dtype=np.float64)
    return bool(lib().or_is_irreducible_wedge(_dp(k)))


def symmetry_operation(k_iw, k_bz):
    """apply_same_symmetry_operation's signed permutation: (found, perm[3], sign[3]) with
    v_bz[j] = sign[j] * v[perm[j]]."""
    a = np.ascontiguousarray(k_iw, dtype=np.float64)
    b = np.ascontiguousarray(k_bz, dtype=np.float64)
    perm = (C.c_int * 3)()
    sign = (C.c_int * 3)()
    found = lib().or_symmetry_operation(_dp(a), _dp(b), perm, sign)
    return bool(found), list(perm), list(sign)


def gradient(mat: OrMaterial, G: np.ndarray, k, ev: np.ndarray) -> np.ndarray:
    L = lib()
    G = np.ascontiguousarray(G, dtype=np.int32)
    ev = np.ascontiguousarray(ev, dtype=np.complex128)
    out = np.zeros(3)
    kk = np.ascontiguousarray(k, dtype=np.float64)
    L.or_gradient(C.byref(mat), _ip(G), G.shape[0], _dp(kk), _dp(ev), ev.shape[0], _dp(out))
    return out


def sample_first_bz(n: int, seed: int) -> np.ndarray:
    """Uniform k in the first BZ (truncated octahedron) by rejection from [-1,1]^3, the test used by
    is_in_first_BZ (src/EPP/DielectricFunction.cpp:35-40); seeded numpy generator."""
    rng = np.random.default_rng(seed)
    out = []
    have = 0
    while have < n:
        k = rng.uniform(-1.0, 1.0, size=(max(2 * (n - have), 64), 3))
        ok = (np.abs(k) <= 1.0).all(axis=1) & (np.abs(k).sum(axis=1) <= 1.5)
        out.append(k[ok])
        have += int(ok.sum())
    return np.concatenate(out)[:n].copy()


# ---- dielectric function (eigenvector consumer) ---------------------------------------------------
def is_in_first_bz(k, one_eighth=False) -> bool:
    """is_in_first_BZ (src/EPP/DielectricFunction.cpp:35-40)."""
    x, y, z = (float(v) for v in k)
    c1 = abs(x) <= 1.0 and abs(y) <= 1.0 and abs(z) <= 1.0
    c2 = abs(x) + abs(y) + abs(z) <= 3.0 / 2.0
    c8 = x >= 0.0 and y >= 0.0 and z >= 0.0
    return c1 and c2 and (c8 if one_eighth else True)


def is_in_irreducible_wedge_df(k) -> bool:
    """is_in_irreducible_wedge (src/EPP/DielectricFunction.cpp:31-33)."""
    x, y, z = (float(v) for v in k)
    return z >= 0.0 and y >= z and x >= y and x <= 1.0 and x + y + z <= 3.0 / 2.0


def dielectric_k_grid(nx: int, ny: int, nz: int, shift: float, irreducible_wedge: bool) -> np.ndarray:
    """DielectricFunction::generate_k_points_grid (src/EPP/DielectricFunction.cpp:59-76): i, j, k
    loops over N-1 points each of [-1 - shift, 1 + shift], kept in the first zone (and the wedge)."""
    lo, hi = -1.0 - shift, 1.0 + shift
    out = []
    for i in range(nx - 1):
        for j in range(ny - 1):
            for k in range(nz - 1):
                v = (lo + (hi - lo) * i / float(nx - 1), lo + (hi - lo) * j / float(ny - 1),
                     lo + (hi - lo) * k / float(nz - 1))
                if is_in_first_bz(v) and (not irreducible_wedge or is_in_irreducible_wedge_df(v)):
                    out.append(v)
    return np.array(out, dtype=np.float64).reshape(-1, 3)


def dielectric_pair_sums(Ek, Xk, Ekq, Xkq, energies, eta, first_cond=4, weights=None) -> np.ndarray:
    """The per-k sums of DielectricFunction::compute_dielectric_function
    (src/EPP/DielectricFunction.cpp:122-143), from eigenstates at k and k + q ([nk][nb][n] vectors,
    [nk][nb] energies): sum over k of weight_k * sum_{c >= first_cond > v} |sum_i u_c(k+q)_i u_v(k)_i|^2
    [(dE - w) / ((dE - w)^2 + eta^2) + (dE + w) / ((dE + w)^2 + eta^2)], dE = E_c(k+q) - E_v(k)."""
    en = np.asarray(energies, dtype=np.float64)
    total = np.zeros(len(en))
    nk, nb = Ek.shape
    for b in range(nk):
        ksum = np.zeros(len(en))
        for c in range(first_cond, nb):
            for v in range(first_cond):
                # col(c).adjoint().dot(col(v)) in Eigen: dot() conjugates its first operand, already
                # the adjoint, so the sum is unconjugated
                ov = abs(np.dot(Xkq[b, c], Xk[b, v])) ** 2
                d = Ekq[b, c] - Ek[b, v]
                f1 = (d - en) / ((d - en) * (d - en) + eta * eta)
                f2 = (d + en) / ((d + en) * (d + en) + eta * eta)
                ksum += ov * (f1 + f2)
        total += (1.0 if weights is None else float(weights[b])) * ksum
    return total


def dielectric_sums(mat: OrMaterial, G: np.ndarray, kpts: np.ndarray, q, nb: int, energies, eta: float, nl=False,
                    first_cond=4, weights=None) -> np.ndarray:
    """One q of DielectricFunction::compute_dielectric_function (src/EPP/DielectricFunction.cpp:
    83-150): eigenstates at k and at k + q (q of length <= 1e-15 replaced by (1e-15, 1e-15, 1e-15),
    :97-99), then the pair sums."""
    q = np.asarray(q, dtype=np.float64)
    if np.sqrt(np.dot(q, q)) <= 1e-15:
        q = np.array([1e-15, 1e-15, 1e-15])
    k = np.ascontiguousarray(kpts, dtype=np.float64).reshape(-1, 3)
    a = band_structure(mat, G, k, nb, nl=nl, vectors=True)
    b = band_structure(mat, G, k + q[None, :], nb, nl=nl, vectors=True)
    return dielectric_pair_sums(a["E"], a["vecs"], b["E"], b["vecs"], energies, eta, first_cond, weights)


def dielectric_merge(qpoints, results, nb_kpoints_per_instance) -> np.ndarray:
    """DielectricFunction::merge_results (src/EPP/DielectricFunction.cpp:152-212): the instances'
    [q][energy] sums added, divided by the total k count, then eps = 1 + (2 pi / |q|^2) * that
    (|q|^2 = 0 taken as 1e-14)."""
    if len(results) == 0:
        raise RuntimeError("No results to merge")
    if len(results) != len(nb_kpoints_per_instance):
        raise RuntimeError("Number of results and number of k-points per instance do not match")
    tot = np.array(results[0], dtype=np.float64).copy()
    for r in results[1:]:
        tot += np.array(r, dtype=np.float64)
    ren = 1.0 / float(sum(nb_kpoints_per_instance))
    out = np.empty_like(tot)
    for iq, q in enumerate(qpoints):
        q2 = float(np.sqrt(np.dot(q, q))) ** 2
        if q2 == 0.0:
            q2 = 1e-14
        out[iq] = 1.0 + (2.0 * PI / q2) * (tot[iq] * ren)
    return out


def kramers_matrix(n: int) -> np.ndarray:
    """create_kramers_matrix (src/EPP/DielectricFunction.cpp:214-228)."""
    K = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if i != j:
                K[i, j] = float(i) / float(j * j - i * i)
    return K * (-2.0 / PI)


def kramers_kronig(eps_real) -> np.ndarray:
    """apply_kramers_kronig (src/EPP/DielectricFunction.cpp:230-251): Im = K (Re - 1) per q."""
    e = np.atleast_2d(np.asarray(eps_real, dtype=np.float64))
    K = kramers_matrix(e.shape[1])
    return np.stack([K @ (row - 1.0) for row in e])


def bz_states_dielectric(Ek, Xk, Ekq, Xkq, tetra, signed_volumes, energies, eta, q_si, first_cond=4) -> np.ndarray:
    """BZ_States::compute_dielectric_function (src/BZ_MESH/bz_states.cpp:93-150) from the vertex
    eigenstates at k and k + q: per tetrahedron, the four vertices' pair sums times |volume| / 4,
    then eps = 1 + q_e^2 / (eps_0 |q|^2) / q_e * 2 / (2 pi)^3 * sum (q in SI)."""
    eps_0 = 8.8541878128e-12  # src/Common/physical_constants.hpp:31
    en = np.asarray(energies, dtype=np.float64)
    total = np.zeros(len(en))
    nb = Ek.shape[1]
    for t, vol in zip(tetra, signed_volumes):
        tsum = np.zeros(len(en))
        for idx in t:
            for c in range(first_cond, nb):
                for v in range(first_cond):
                    ov = abs(np.dot(Xkq[idx, c], Xk[idx, v])) ** 2
                    d = Ekq[idx, c] - Ek[idx, v]
                    f1 = (d - en) / ((d - en) * (d - en) + eta * eta)
                    f2 = (d + en) / ((d + en) * (d + en) + eta * eta)
                    tsum += ov * (f1 + f2)
        total += tsum * abs(vol) * 0.25
    q = np.asarray(q_si, dtype=np.float64)
    q2 = float(np.sqrt(np.dot(q, q))) ** 2
    pref = (Q_E * Q_E) / (eps_0 * q2) / Q_E * (2.0 / (2.0 * PI) ** 3)
    return 1.0 + pref * total
