"""The FP64 bisection's pivot reciprocal (sturm_rcp in tridiag_eig.cu: rcp.approx.ftz.f64 refined by two
Newton-Raphson steps) against the correctly rounded 1.0 / q, over the pivot range the Sturm count
produces, through uepm_pivot_reciprocal_device.

Bounds: within 1 ulp of 1.0 / q wherever 1 / q is a normal number; exactly zero where 1 / q would be
subnormal (|q| > 2^1022: the approximation flushes it, a perturbation of e^2 / q below 2^-1022 in the
pivot recurrence); pivots within pivmin (subnormal ones included) replaced by -pivmin first, so their
reciprocal is 1 / -pivmin."""
import ctypes as C

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _run(gpu, q, pivmin):
    import torch

    dq = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float64)).cuda()
    dr = torch.full_like(dq, float("nan"))
    assert gpu.uepm_pivot_reciprocal_device(C.c_void_p(dq.data_ptr()), pivmin, len(q), C.c_void_p(dr.data_ptr()),
                                            None) == 0
    torch.cuda.synchronize()
    return dr.cpu().numpy()


def _ulps(a, b):
    return np.abs(a - b) / np.spacing(np.abs(b))


def test_reciprocal_within_one_ulp_over_the_pivot_range(gpu):
    rng = np.random.default_rng(5)
    tiny = np.finfo(np.float64).tiny
    # log-uniform magnitudes from just above DBL_MIN to 2^1021, both signs, plus mantissa sweeps
    mag = np.exp(rng.uniform(np.log(tiny) + 1e-3, np.log(2.0 ** 1021), 400000))
    sweep = np.concatenate([np.linspace(1.0, 2.0, 20001), np.linspace(0.5, 1.0, 20001)])
    q = np.concatenate([mag, -mag, sweep, -sweep * 3.0, [1.0, -1.0, 3.0, 7.0, tiny * 4, -tiny * 4]])
    r = _run(gpu, q, tiny)
    want = 1.0 / q
    ok = np.abs(want) >= tiny
    assert np.isfinite(r[ok]).all()
    assert _ulps(r[ok], want[ok]).max() <= 1.0
    assert (np.sign(r) == np.sign(q)).all()


def test_reciprocal_of_huge_pivots_flushes_to_zero(gpu):
    q = np.array([2.0 ** 1022 * 1.5, -(2.0 ** 1023), 1.7e308, -1.7e308])
    r = _run(gpu, q, np.finfo(np.float64).tiny)
    # 1 / q is subnormal here: the hardware approximation flushes it to a zero of the same sign
    assert (r == 0.0).all()


def test_pivots_within_pivmin_are_replaced_before_the_reciprocal(gpu):
    tiny = np.finfo(np.float64).tiny
    pivmin = tiny * 37.0
    q = np.array([0.0, -0.0, 5e-324, -5e-324, tiny / 3, tiny, -tiny * 36.0, pivmin, -pivmin])
    r = _run(gpu, q, pivmin)
    want = 1.0 / -pivmin
    assert (_ulps(r, np.full_like(r, want)) <= 1.0).all(), r
    # just above the guard's high-word window the pivot is kept
    q2 = np.array([pivmin * 4.0, -pivmin * 4.0])
    r2 = _run(gpu, q2, pivmin)
    assert (_ulps(r2, 1.0 / q2) <= 1.0).all()
