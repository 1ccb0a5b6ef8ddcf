"""The mixed path's double-single special functions (assemble.cu: ds_exp_pos, i2_ds), through
uepm_ds_special_device, against 40-digit decimal values of the same functions at the same arguments
(the FP32-pair rounding of each argument is applied on both sides).

e^x, 2 < x <= 80: Cody and Waite's reduction and a degree-13 Taylor series, relative error below
1e-14. i2(x) = ((x^2 + 3) sinh x - 3 x cosh x) / x^3 (the reference's closed form,
bessel_func.hpp:47-52), 2 < x <= 80, with that e^x: relative error below 2e-13 (the closed form's
cancellation just above x = 2 costs about a factor of 10; below x = 2 the mixed path takes the FP64
value, as the FP64 path does)."""
import ctypes as C
from decimal import Decimal, getcontext

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _run(gpu, fn, x):
    import torch

    dx = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    dy = torch.full_like(dx, float("nan"))
    assert gpu.uepm_ds_special_device(fn, C.c_void_p(dx.data_ptr()), len(x), C.c_void_p(dy.data_ptr()), None) == 0
    torch.cuda.synchronize()
    return dy.cpu().numpy()


def _pair(v):
    """The FP32 pair (h, l) of v, as the device forms it, summed exactly in decimal."""
    h = np.float32(v)
    l = np.float32(v - np.float64(h))
    return Decimal(float(h)) + Decimal(float(l))


def _i2(x: Decimal) -> Decimal:
    if x < Decimal(1) / 8:  # the series: no cancellation
        y, t, s, k = x * x, Decimal(1) / 15, Decimal(0), 0
        while True:
            s += t
            k += 1
            t = t * y / (2 * k * (2 * k + 5))
            if t < Decimal("1e-45") * s:
                return x * x * (s + t)
    e, ei = x.exp(), (-x).exp()
    return ((x * x + 3) * (e - ei) / 2 - 3 * x * (e + ei) / 2) / (x ** 3)


def test_ds_exp(gpu):
    getcontext().prec = 40
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.uniform(2.0, 80.0, 4000), [2.0000001, 10.0, 44.3614, 79.999]])
    y = _run(gpu, 0, x)
    rel = max(abs((Decimal(float(v)) - _pair(a).exp()) / _pair(a).exp()) for a, v in zip(x, y))
    assert rel <= Decimal("1e-14"), f"max relative error {rel:.3e}"


def test_ds_i2_closed_form(gpu):
    getcontext().prec = 40
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.uniform(2.0, 80.0, 4000), [2.000001, 2.5, 79.9]])
    y = _run(gpu, 1, x)
    rel = max(abs((Decimal(float(v)) - _i2(_pair(a))) / _i2(_pair(a))) for a, v in zip(x, y))
    assert rel <= Decimal("2e-13"), f"max relative error {rel:.3e}"


def test_ds_special_rejects_bad_arguments(gpu):
    assert gpu.uepm_ds_special_device(2, None, 0, None, None) == N.UEPM_ERR_INVALID
    assert gpu.uepm_ds_special_device(0, None, 4, None, None) == N.UEPM_ERR_INVALID
