"""Generates tests/golden/oracle_bands.npz: the oracle's FP64 eigenvalues and Hellmann-Feynman
gradients at eight fixed k-points (Gamma, L, X, W, K, U and two seeded first-zone points) for the
parity configurations. The fixtures pin the oracle (a CPU test re-derives them) and give the GPU
tests an anchor that does not need the oracle at run time.

    python tests/golden/make_oracle_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# name: (parameter file, material, shells, nonlocal, spin-orbit, bands)
CONFIGS = {
    "si_cb_local": ("si-cohen-bergstresser.yaml", "Si", 10, False, False, 16),
    "si_d_nonlocal": ("si-nonlocal-d.yaml", "Si", 10, True, False, 12),
    "inp_nonlocal": ("materials.yaml", "InP", 9, True, False, 12),
    "gaas_nonlocal_soc": ("materials.yaml", "GaAs", 8, True, True, 16),
    "ge_nonlocal_soc": ("materials.yaml", "Ge", 12, True, True, 16),
}
SYMMETRY_POINTS = np.array([[0, 0, 0], [0.5, 0.5, 0.5], [1, 0, 0], [1, 0.5, 0], [0.75, 0.75, 0], [1, 0.25, 0.25]], float)


def k_points() -> np.ndarray:
    return np.concatenate([SYMMETRY_POINTS, O.sample_first_bz(2, 20261203)])


def compute(name: str):
    yaml, sym, shells, nl, soc, nb = CONFIGS[name]
    mat = O.load_materials(os.path.join(ROOT, "params", yaml))[sym]
    G = O.generate_basis(shells)
    r = O.band_structure(mat, G, k_points(), nb, nl=nl, soc=soc, grad=True)
    if r["status"].any():
        raise RuntimeError(f"{name}: oracle status {r['status']}")
    return r["E"], r["grad"]


def main():
    O.build()
    out = {"k": k_points()}
    for name in CONFIGS:
        E, g = compute(name)
        out[name + "_E"] = E
        out[name + "_grad"] = g
    np.savez(os.path.join(HERE, "oracle_bands.npz"), **out)


if __name__ == "__main__":
    main()
