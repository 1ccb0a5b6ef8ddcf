"""One batched solve of seeded first-zone k-points for a material, cutoff and flags: the quickest way
to time (or profile) the path on a given case.

    python -m ultimateepm_gb300.solve_sample materials.yaml Ge --shells 12 --nl --soc --bands 16 \\
        --k 2000 [--precision fp64|mixed] [--reduction R] [--repeat N]

Prints the first k-point's lowest energies and the mean wall time per solve after a small warm-up
solve (the solve runs through uepm_solve with host buffers, so the time includes the copies). Parameter files are looked up in
the package's params/ folder unless a path is given.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import time

import numpy as np

from . import _native as N
from .api import Materials, _Context, generate_basis_vectors
from .serve import PARAMS, sample_bz


def main(argv=None) -> int:
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("params")
    p.add_argument("material")
    p.add_argument("--shells", type=int, default=10)
    p.add_argument("--nl", action="store_true")
    p.add_argument("--soc", action="store_true")
    p.add_argument("--bands", type=int, default=16)
    p.add_argument("--k", type=int, default=2000)
    p.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    p.add_argument("--reduction", type=int, default=0, help="uepm_tuning.reduction (0: automatic)")
    p.add_argument("--repeat", type=int, default=1)
    p.add_argument("--seed", type=int, default=3)
    a = p.parse_args(argv)
    path = a.params if os.path.exists(a.params) else os.path.join(PARAMS, a.params)
    mats = Materials()
    mats.load_material_parameters(path)
    prec = N.UEPM_PREC_MIXED if a.precision == "mixed" else N.UEPM_PREC_FP64
    ctx = _Context(mats.materials[a.material], generate_basis_vectors(a.shells), a.nl, a.soc, prec)
    N.check(N.load().uepm_ctx_set_tuning(ctx.h, C.byref(N.UepmTuning(reduction=a.reduction))))
    k = sample_bz(a.k, np.random.default_rng(a.seed))
    ctx.solve(k[: min(len(k), 64)], a.bands)  # warm-up: workspace and module loading
    t0 = time.perf_counter()
    for _ in range(a.repeat):
        E, _, _, st = ctx.solve(k, a.bands)
    dt = (time.perf_counter() - t0) / a.repeat
    ctx.close()
    if st.any():
        print(f"{int((st != 0).sum())} k-points reported a non-zero status")
        return 1
    print(f"order {ctx.n}, {a.k} k-points, {a.bands} bands, {a.precision}: {dt * 1e3:.2f} ms per solve "
          f"({a.k / dt:.0f} k-points/s); E(k0) = {np.array2string(E[0, :4], precision=6)} eV")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
