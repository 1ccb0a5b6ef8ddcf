"""Generates the committed golden fixtures from the reference (run where the reference tree exists).

    python tests/golden/make_golden.py [REF_ROOT]

Outputs (all small, committed):
  bessel_table.json  the two 6 x 12 golden tables of the reference's own unit test
                     (tests/epp/test_bessel_functions.cpp:22-65), parsed from that file as text.
  ref_bessel.npz     generalized_bessel / generalized_bessel_cylindrical / bessel_2nd_order_first_kind
                     evaluated by the reference's bessel_func.hpp (compiled into oracle/_ref) on a grid
                     that covers the arguments the nonlocal terms use, including small x.
  ref_pp.npz         Pseudopotential::GetValue (the reference's Pseudopotential.cpp) for every
                     G_i - G_j of the 10-shell basis, for two form-factor sets.
  ref_paths.json     SymmetryPoints::GeneratePoints (the reference's SymmetryPoints.cpp) for several
                     paths and sizes, including the 2000-point L-G-X-W-K-U-L-W-X-K-G path.

From the reference's Material.cpp, SpinOrbitFunctional.cpp, Hamiltonian.cpp and BandStructure.cpp,
compiled against the project-written Eigen / yaml-cpp subsets in oracle/shim:
  ref_materials.json the fields Materials::load_material_parameters leaves in each Material of every
                     parameter file under params/ (units as the reference holds them).
  ref_hamiltonian.npz H(k) after Hamiltonian::SetMatrix and Diagonalize's hermitisation, for seven
                     material / nonlocal / spin-orbit cases at the eight fixed k (Gamma, L, X, W, K,
                     U and two seeded generic points): the lower triangles at basis 15 (3 shells),
                     and SHA-256 digests of the full column-major complex128 matrices at the
                     production bases (89 to 229 plane waves, orders up to 458), zeros unsigned.
  ref_elements.npz   Material::compute_pseudopotential_non_local_correction and
                     SpinOrbitCorrection::compute_soc_contribution on seeded (K1, K2) pairs, with
                     equal-norm and equal pairs for the reference's |K1| = |K2| branches.
  ref_band_*.txt     BandStructure::export_result_in_file after Initialize (path), Compute and
                     AdjustValues, for Si local and Ge nonlocal with spin-orbit; their energies in
                     ref_bands.npz.
  ref_gradients.npz  the shape of get_band_energy_gradients() after Compute_parallel(true, 1)
                     ([nk * nb] rows of nb) and its first nk rows.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

PATHS = [("LGXWKULWXKG", 2000), ("LGXWKULWXKG", 11), ("GXWKGLUWLK", 300), ("LGXUG", 57), ("KWXGLW", 61),
         ("GX", 2), ("GG", 10), ("LGXKG", 100)]


def parse_bessel_table(ref_root: str) -> dict:
    src = open(os.path.join(ref_root, "tests", "epp", "test_bessel_functions.cpp")).read()
    out = {}
    for name in ("nu_x_bessel_cyl_values", "nu_x_bessel_values"):
        body = re.search(name + r"\s*=\s*\{(.*?)\};", src, re.S).group(1)
        out[name] = [float(v) for v in re.findall(r"-?\d+\.\d+(?:[eE][-+]?\d+)?", body)]
    lists = re.findall(r"list_nu\s*=\s*\{([^}]*)\}", src)
    xs = re.findall(r"list_x\s*=\s*\{([^}]*)\}", src)
    out["list_nu"] = [float(v) for v in lists[0].split(",")]
    out["list_x"] = [float(v) for v in xs[0].split(",")]
    assert len(out["nu_x_bessel_cyl_values"]) == 72 and len(out["nu_x_bessel_values"]) == 72
    return out


PARAMS = os.path.join(ROOT, "params")
# (key, parameter file, symbol, nonlocal, spin-orbit, production shells)
HAM_CASES = [("si_local", "si-cohen-bergstresser.yaml", "Si", 0, 0, 10),
             ("si_nl", "materials.yaml", "Si", 1, 0, 10),
             ("si_d", "si-nonlocal-d.yaml", "Si", 1, 0, 10),
             ("inp_nl", "materials.yaml", "InP", 1, 0, 9),
             ("ge_nl_soc", "materials.yaml", "Ge", 1, 1, 12),
             ("gaas_nl_soc", "materials.yaml", "GaAs", 1, 1, 8),
             ("gap_soc", "materials.yaml", "GaP", 0, 1, 13)]
# Gamma, L, X, W, K, U, then two seeded generic points
FIXED_K = np.array([[0, 0, 0], [0.5, 0.5, 0.5], [1, 0, 0], [1, 0.5, 0], [0.75, 0.75, 0], [1, 0.25, 0.25],
                    [0.1237, -0.3318, 0.2871], [-0.4419, 0.0963, 0.6027]], dtype=np.float64)
BAND_FILES = [("si_local", "si-cohen-bergstresser.yaml", "Si", 16, "LGXWKULWXKG", 40, 10, 0, 0),
              ("ge_nl_soc", "materials.yaml", "Ge", 8, "LGX", 20, 8, 1, 1)]


def ref_hamiltonians(R, path, sym, G, k, nl, soc):
    N = len(G)
    n = 2 * N if soc else N
    H = np.zeros((len(k), n, n), dtype=np.complex128)  # [q][column][row]: column-major per k
    rc = R.ref_hamiltonian(path.encode(), sym.encode(), O._ip(np.ascontiguousarray(G, dtype=np.int32)), N,
                           O._dp(np.ascontiguousarray(k)), len(k), nl, soc, O._dp(H))
    assert rc == n, (path, sym, rc)
    return H


def make_reference_hamiltonians(R):
    small = O.generate_basis(3)
    out = {"k": FIXED_K, "G_small": small}
    for key, fname, sym, nl, soc, shells in HAM_CASES:
        path = os.path.join(PARAMS, fname)
        H = ref_hamiltonians(R, path, sym, small, FIXED_K, nl, soc)
        n = H.shape[1]
        r, c = np.tril_indices(n)
        out[key + "_lower"] = np.stack([H[q][c, r] for q in range(len(FIXED_K))])  # H(r, c), r >= c
        Gp = O.generate_basis(shells)
        Hp = ref_hamiltonians(R, path, sym, Gp, FIXED_K, nl, soc)
        # zeros are hashed unsigned (x + 0.0): the sign of a zero element depends on how the matrix
        # library scales a complex by a real (Diagonalize's 0.5 * (H + H^H)), not on the reference
        out[key + "_sha256"] = np.array([hashlib.sha256((Hp[q] + 0.0).tobytes()).hexdigest()
                                         for q in range(len(FIXED_K))])
        out[key + "_shells"] = np.array(shells)
    np.savez_compressed(os.path.join(HERE, "ref_hamiltonian.npz"), **out)


def make_reference_elements(R):
    rng = np.random.default_rng(20261204)
    K1 = rng.uniform(-3.0, 3.0, (96, 3))
    K2 = rng.uniform(-3.0, 3.0, (96, 3))
    # the reference's |K1| = |K2| branches: equal vectors, and signed permutations (equal norms)
    K2[:16] = K1[:16]
    K2[16:32] = -K1[16:32, ::-1]
    K1[32:36] = 0.0
    G1 = rng.integers(-3, 4, (96, 3)).astype(np.float64)
    G2 = rng.integers(-3, 4, (96, 3)).astype(np.float64)
    out = {"K1": K1, "K2": K2, "G1": G1, "G2": G2}
    for key, fname, sym, nl, soc, _ in HAM_CASES:
        path = os.path.join(PARAMS, fname).encode()
        mat = O.load_materials(os.path.join(PARAMS, fname))[sym]
        tau = np.full(3, (1.0 / 8.0) * 1e-10 * mat.lattice_constant)
        if nl:
            v = np.zeros((96, 2))
            for q in range(96):
                assert R.ref_nl_correction(path, sym.encode(), O._dp(K1[q]), O._dp(K2[q]), O._dp(tau), O._dp(v[q])) == 0
            out[key + "_nl"] = v
        if soc:
            b = np.zeros((96, 8))
            for q in range(96):
                assert R.ref_soc_block(path, sym.encode(), O._dp(K1[q]), O._dp(K2[q]), O._dp(G1[q]), O._dp(G2[q]),
                                       O._dp(tau), O._dp(b[q])) == 0
            out[key + "_soc"] = b
    np.savez_compressed(os.path.join(HERE, "ref_elements.npz"), **out)


def make_reference_materials(R):
    out = {}
    for fname in sorted(os.listdir(PARAMS)):
        if not fname.endswith(".yaml"):
            continue
        path = os.path.join(PARAMS, fname)
        for sym in O.load_materials(path):
            m = O.OrMaterial()
            assert R.ref_material(path.encode(), sym.encode(), C.byref(m)) == 0
            out.setdefault(fname, {})[sym] = {f: getattr(m, f) for f, _ in O.OrMaterial._fields_}
    with open(os.path.join(HERE, "ref_materials.json"), "w") as f:
        json.dump(out, f, indent=1)


def make_reference_band_files(R):
    out = {}
    for key, fname, sym, nb, labels, npts, shells, nl, soc in BAND_FILES:
        dst = os.path.join(HERE, f"ref_band_{key}.txt")
        cap = 4 * npts * nb
        E = np.zeros(cap)
        cnt = R.ref_band_file(os.path.join(PARAMS, fname).encode(), sym.encode(), nb, labels.encode(), npts, shells, nl,
                              soc, 0, dst.encode(), O._dp(E), cap)
        assert cnt > 0, (key, cnt)
        out[key] = E[:cnt].reshape(-1, nb * (2 if soc else 1))
    np.savez_compressed(os.path.join(HERE, "ref_bands.npz"), **out)


def make_reference_gradients(R):
    k = FIXED_K[[1, 6, 7]].copy()
    nb = 4
    G = O.generate_basis(4)
    rows, row_len = C.c_int(), C.c_int()
    g = np.zeros((len(k), nb, 3))
    assert R.ref_gradient_shape(os.path.join(PARAMS, "si-cohen-bergstresser.yaml").encode(), b"Si", nb,
                                O._dp(k), len(k), 4, C.byref(rows), C.byref(row_len), O._dp(g), len(k)) == 0
    np.savez(os.path.join(HERE, "ref_gradients.npz"), k=k, nb=nb, shells=4, rows=rows.value, row_len=row_len.value,
             grad=g, G=G)


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else O.REFERENCE_ROOT
    os.environ["UEPM_REFERENCE_ROOT"] = ref_root
    O.REFERENCE_ROOT = ref_root
    O.build()
    R = O.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libref.so was not built: the reference tree is required")

    with open(os.path.join(HERE, "bessel_table.json"), "w") as f:
        json.dump(parse_bessel_table(ref_root), f, indent=1)

    # Bessel grid: orders used by F_l (-1..3), x from 1e-16 to 40 (|K| R spans ~0..10 in practice)
    xs = np.concatenate([[0.0, 1e-16, 5e-15, 1e-14, 2e-14, 1e-12, 1e-9, 1e-6, 1e-4, 1e-3, 1e-2],
                         np.linspace(0.02, 3.0, 150), np.linspace(3.0, 40.0, 150)])
    nus = np.array([-1.0, 0.0, 1.0, 2.0, 3.0])
    sph = np.array([[R.ref_sph_bessel(nu, x) for x in xs] for nu in nus])
    cyl_nus = np.array([-0.5, 0.5, 1.5, 2.5, 3.5, -1.0, 0.0, 1.0, 2.0])
    xs_c = xs[xs > 0]
    cyl = np.array([[R.ref_cyl_bessel(nu, x) for x in xs_c] for nu in cyl_nus])
    xi = np.concatenate([[0.0, 1e-8, 1e-4, 1e-2], np.linspace(0.05, 8.0, 200)])
    i2 = np.array([R.ref_bessel_i2(x) for x in xi])
    np.savez(os.path.join(HERE, "ref_bessel.npz"), x=xs, nu=nus, sph=sph, cyl_nu=cyl_nus, cyl_x=xs_c, cyl=cyl,
             i2_x=xi, i2=i2)

    # Pseudopotential::GetValue over every difference vector of the 10-shell basis
    G = O.generate_basis(10)
    dG = np.unique((G[:, None, :] - G[None, :, :]).reshape(-1, 3), axis=0).astype(np.int32)
    sets = {
        "si_cb": ([-0.21, 0.0, 0.04, 0.08, 0.0, 0.0, 0.0, 0.0], 5.43),
        "gaas_pv": ([-0.214, -0.157, 0.014, 0.067, 0.055, 0.038, 0.008, 0.001], 5.65),
    }
    out = {"dG": dG}
    for key, (vry, a_ang) in sets.items():
        V = (C.c_double * 8)(*[O.RYD_TO_EV * v for v in vry])
        a = 1.0e-10 * a_ang
        tau = (C.c_double * 3)(*([(1.0 / 8.0) * a] * 3))
        vals = np.zeros((len(dG), 2))
        res = (C.c_double * 2)()
        for q, (x, y, z) in enumerate(dG):
            R.ref_pp_value(V, int(x), int(y), int(z), tau, a, res)
            vals[q] = (res[0], res[1])
        out[key + "_V"] = np.array([V[i] for i in range(8)])
        out[key + "_a"] = np.array(a)
        out[key] = vals
    np.savez(os.path.join(HERE, "ref_pp.npz"), **out)

    # SymmetryPoints::GeneratePoints
    paths = []
    for labels, npts in PATHS + [("LQ", 10), ("L", 5), ("LGX", 2)]:
        k = (C.c_double * (3 * max(npts, 1)))()
        pos = (C.c_uint32 * max(len(labels), 1))()
        cnt = R.ref_generate_path(labels.encode(), npts, k, npts, pos, len(labels))
        entry = {"labels": labels, "n": npts, "count": cnt}
        if cnt >= 0:
            entry["k"] = [k[i] for i in range(3 * cnt)]
            entry["sym"] = [pos[i] for i in range(len(labels))]
        paths.append(entry)
    with open(os.path.join(HERE, "ref_paths.json"), "w") as f:
        json.dump(paths, f)

    make_reference_materials(R)
    make_reference_hamiltonians(R)
    make_reference_elements(R)
    make_reference_band_files(R)
    make_reference_gradients(R)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
