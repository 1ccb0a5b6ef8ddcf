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
"""
from __future__ import annotations

import ctypes as C
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


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
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
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
