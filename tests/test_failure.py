"""Failure detection of the solve (no GPU fault involved: every failure is injected on the host).

The reference throws std::runtime_error("Eigenvalue decomposition failed") when Eigen's solver
reports a failure (Hamiltonian.cpp:129-133). Here the kernels write a per-k status: UEPM_K_NONFINITE
where NaN / Inf reaches H(k) or the reduction, UEPM_K_NOCONVERGE where an iteration cap ends the
bisection, the inverse iteration or the projected Jacobi before they converged; uepm_solve then
returns UEPM_ERR_NOT_CONVERGED, and the adapter throws the reference's exception. Injected here:
a NaN k-point, a NaN form factor, and an iteration cap of 1 (uepm_tuning.max_iter)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import PARAMS, ROOT
from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api

LIB = os.path.join(ROOT, "ultimateepm_gb300", "lib")


def _ctx(orm, G, nl=False, soc=False, precision=N.UEPM_PREC_FP64):
    return api._Context(api.Material("m", raw=N.UepmMaterial.from_buffer_copy(bytes(orm))), G, nl, soc, precision)


def _solve_raw(ctx, k, nb, want=0):
    L = N.load()
    k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
    E = np.zeros((len(k), nb))
    st = np.zeros(len(k), dtype=np.int32)
    n = ctx.n
    X = np.zeros((len(k), nb, n), dtype=np.complex128) if want & N.UEPM_WANT_VECTORS else None
    rc = L.uepm_solve(ctx.h, k.ctypes.data_as(C.POINTER(C.c_double)), len(k), nb, want,
                      E.ctypes.data_as(C.POINTER(C.c_double)),
                      X.ctypes.data_as(C.POINTER(C.c_double)) if X is not None else None, None,
                      st.ctypes.data_as(C.POINTER(C.c_int32)))
    return rc, E, st


def test_tuning_struct_has_the_iteration_cap():
    assert [f for f, _ in N.UepmTuning._fields_][-3:] == ["max_iter", "tensor_cores", "streams"]
    assert C.sizeof(N.UepmTuning) == 8 * 4


CASES = [("Si-CB", 8, False, False), ("Ge", 8, True, True), ("InP", 8, True, False)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [N.UEPM_PREC_FP64, N.UEPM_PREC_MIXED])
@pytest.mark.parametrize("key,shells,nl,soc", CASES)
def test_nan_k_point_reports_nonfinite(gpu, oracle, mats, key, shells, nl, soc, precision):
    ctx = _ctx(mats[key], oracle.generate_basis(shells), nl, soc, precision)
    k = oracle.sample_first_bz(6, 11)
    k[2, 0] = np.nan
    k[4, 2] = np.inf
    for want in (0, N.UEPM_WANT_VECTORS):
        rc, E, st = _solve_raw(ctx, k, 8, want)
        assert rc == N.UEPM_ERR_NOT_CONVERGED
        assert st.tolist() == [0, 0, N.UEPM_K_NONFINITE, 0, N.UEPM_K_NONFINITE, 0], st
        # the finite k-points are unaffected
        ref = oracle.band_structure(mats[key], oracle.generate_basis(shells), k[[0, 1, 3, 5]], 8, nl=nl, soc=soc)["E"]
        tol = 1e-10 if precision == N.UEPM_PREC_FP64 else 1e-6
        assert np.abs(E[[0, 1, 3, 5]] - ref).max() <= tol
    with pytest.raises(RuntimeError, match="Eigenvalue decomposition failed"):
        ctx.solve(k, 8)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [N.UEPM_PREC_FP64, N.UEPM_PREC_MIXED])
def test_nan_form_factor_reports_nonfinite(gpu, oracle, mats, precision):
    bad = N.UepmMaterial.from_buffer_copy(bytes(mats["Si-CB"]))
    bad.V3S = float("nan")
    ctx = api._Context(api.Material("m", raw=bad), oracle.generate_basis(8), False, False, precision)
    rc, _, st = _solve_raw(ctx, oracle.sample_first_bz(5, 3), 8)
    assert rc == N.UEPM_ERR_NOT_CONVERGED
    assert (st == N.UEPM_K_NONFINITE).all(), st
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [N.UEPM_PREC_FP64, N.UEPM_PREC_MIXED])
@pytest.mark.parametrize("key,shells,nl,soc", CASES)
def test_iteration_cap_of_one_reports_noconverge(gpu, oracle, mats, key, shells, nl, soc, precision):
    ctx = _ctx(mats[key], oracle.generate_basis(shells), nl, soc, precision)
    k = oracle.sample_first_bz(7, 5)
    t = N.UepmTuning()
    N.check(gpu.uepm_ctx_get_tuning(ctx.h, C.byref(t)))
    t.max_iter = 1
    N.check(gpu.uepm_ctx_set_tuning(ctx.h, C.byref(t)))
    for want in (0, N.UEPM_WANT_VECTORS):
        rc, _, st = _solve_raw(ctx, k, 8, want)
        assert rc == N.UEPM_ERR_NOT_CONVERGED
        assert (st == N.UEPM_K_NOCONVERGE).all(), st
    # back to the automatic caps: converged and correct
    t.max_iter = 0
    N.check(gpu.uepm_ctx_set_tuning(ctx.h, C.byref(t)))
    rc, E, st = _solve_raw(ctx, k, 8, N.UEPM_WANT_VECTORS)
    assert rc == N.UEPM_OK and not st.any()
    ref = oracle.band_structure(mats[key], oracle.generate_basis(shells), k, 8, nl=nl, soc=soc)["E"]
    assert np.abs(E - ref).max() <= (1e-10 if precision == N.UEPM_PREC_FP64 else 1e-6)
    for bad in (-1, 1001):
        t.max_iter = bad
        assert gpu.uepm_ctx_set_tuning(ctx.h, C.byref(t)) == N.UEPM_ERR_OUT_OF_RANGE
    ctx.close()


def _failure_driver(tmp_path):
    exe = str(tmp_path / "failure_driver")
    inc = [f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ROOT, 'include', 'uepm')}"]
    subprocess.run(["g++", "-O2", "-std=c++20", *inc, os.path.join(ROOT, "tests", "cpp", "failure_driver.cpp"), "-o", exe,
                    f"-L{LIB}", "-luepm_epp", "-luepm_gb300", f"-Wl,-rpath,{LIB}"], check=True, capture_output=True)
    return exe


def test_failure_driver_compiles(native, tmp_path):
    assert os.path.exists(_failure_driver(tmp_path))


@pytest.mark.gpu
def test_adapter_throws_the_reference_exception(gpu, tmp_path):
    r = subprocess.run([_failure_driver(tmp_path), os.path.join(PARAMS, "si-cohen-bergstresser.yaml"), "Si", "8"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    got = dict(l.split() for l in r.stdout.splitlines() if len(l.split()) == 2 and l.split()[1] in
               ("none", "runtime_error", "other"))
    assert got == {"finite_compute": "none", "hamiltonian_nan_k": "runtime_error",
                   "compute_parallel_nan_k": "runtime_error"}, r.stdout
