"""Band structure along a path of high-symmetry points, on the GPU.

Mirrors apps/EmpiricalPseudoPotentialMain.cpp (same flags and output files):

    python -m ultimateepm_gb300.epm_main -m Si -b 16 -N 2000 -n 10 -p LGXWKULWXKG \
        -d params/si-cohen-bergstresser.yaml -r results [--precision mixed]

The band file (``<resultdir>/EPM_<mat>_nb_bands_<nb>_path_<path>_size_basis_<N>[_non_local].txt``) has
the reference's header and CSV layout, read by its python/plots/plot_band_structure.py.
Differences from the reference binary: ``-j`` is accepted and ignored (the whole batch runs on the GPU),
and ``-P`` (calling the plotting script) is not supported.
"""
from __future__ import annotations

import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PARAMS = os.path.join(os.path.dirname(HERE), "params")


def compute_path_mat(material, path, nb_points, nb_bands, nn, nl, soc, result_dir, precision, quiet=False):
    from .api import BandStructure

    bs = BandStructure()
    bs.set_precision(precision)
    bs.Initialize(material, nb_bands, list(path), nn, nl, soc, nrPoints=nb_points)
    bs.Compute_parallel(False, 1)
    bs.AdjustValues()
    if not quiet:
        print(f"Time to compute: {bs.get_computation_time_s()} s")
    out = os.path.join(result_dir, bs.path_band_filename() + ("_non_local" if nl else "") + ".txt")
    bs.export_result_in_file(out)
    return out


def main(argv=None) -> int:
    p = argparse.ArgumentParser(description="EPP PROGRAM. COMPUTE BAND STRUCTURE ON A PATH (GB300).")
    p.add_argument("-p", "--path", default=None, help="path of high symmetry points, e.g. LGXWKULWXK")
    p.add_argument("-m", "--material", default=None, help="symbol of the material (Si, Ge, GaAs, ...)")
    p.add_argument("-N", "--npoints", type=int, default=80)
    p.add_argument("-b", "--nbands", type=int, default=12)
    p.add_argument("-n", "--nearestNeighbors", type=int, default=10)
    p.add_argument("-j", "--nthreads", type=int, default=1)
    p.add_argument("-r", "--resultdir", default="./")
    p.add_argument("-d", "--file-data", default="materials.yaml")
    p.add_argument("-C", "--nonlocal-correction", action="store_true")
    p.add_argument("-S", "--soc", action="store_true")
    p.add_argument("-A", "--all", action="store_true")
    p.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    p.add_argument("-q", "--quiet", action="store_true")
    a = p.parse_args(argv)

    from .api import Materials

    os.makedirs(a.resultdir, exist_ok=True)
    fdata = a.file_data
    if not os.path.exists(fdata):
        alt = os.path.join(PARAMS, fdata)
        if not os.path.exists(alt):
            print(f"Error: material data file {fdata} does not exist!", file=sys.stderr)
            return -1
        fdata = alt
    mats = Materials()
    mats.load_material_parameters(fdata)
    if a.all:
        from .options import DEFAULT_PATHS

        for _, mat in mats.materials.items():
            for path in DEFAULT_PATHS:
                compute_path_mat(mat, path, a.npoints, a.nbands, a.nearestNeighbors, a.nonlocal_correction, a.soc,
                                 a.resultdir, a.precision, a.quiet)
        return 0
    if a.material and a.path:
        compute_path_mat(mats.materials[a.material], a.path, a.npoints, a.nbands, a.nearestNeighbors,
                         a.nonlocal_correction, a.soc, a.resultdir, a.precision, a.quiet)
        return 0
    if a.path:
        for _, mat in mats.materials.items():
            compute_path_mat(mat, a.path, a.npoints, a.nbands, a.nearestNeighbors, a.nonlocal_correction, a.soc,
                             a.resultdir, a.precision, a.quiet)
        return 0
    print("No material or path specified")
    return 1


if __name__ == "__main__":
    sys.exit(main())
