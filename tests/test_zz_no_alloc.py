"""The allocation-free H(k) assembly (uepm_assemble_device_noalloc) against the regular one.

Callers that must not allocate device memory at call time (a serving loop whose memory was reserved
at start-up, a host program whose device memory belongs to its own allocator) use the no-alloc entry
point; its row table lives in a fixed 16 MiB device array of the library. This file sorts last so
that a run stopping at its first failure has already run every other test; it passes alone in a
fresh process as well as after the others.
"""
import ctypes as C

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("key,shells,nl,soc", [("Si-CB", 10, False, False), ("Ge", 9, True, True),
                                               ("GaAs", 8, True, False)])
def test_noalloc_assembly_matches_regular_entry_point(gpu, oracle, mats, key, shells, nl, soc):
    import torch

    G = oracle.generate_basis(shells)
    ctx = api._Context(api.Material(key, raw=N.UepmMaterial.from_buffer_copy(bytes(mats[key]))), G, nl, soc)
    n = ctx.n
    # both entry points run the same kernels on the same inputs: the results are bit-identical
    # two calls in a row, with different k-points, each compared with the regular entry point
    for seed in (3, 4):
        ks = np.concatenate([np.zeros((1, 3)), oracle.sample_first_bz(7, seed)])
        dk = torch.from_numpy(ks).cuda()
        ref = torch.zeros((len(ks), n, n), dtype=torch.complex128, device="cuda")
        out = torch.full((len(ks), n, n), float("nan"), dtype=torch.complex128, device="cuda")
        N.check(gpu.uepm_assemble_device(ctx.h, C.c_void_p(dk.data_ptr()), len(ks), C.c_void_p(ref.data_ptr()), None))
        N.check(gpu.uepm_assemble_device_noalloc(ctx.h, C.c_void_p(dk.data_ptr()), len(ks), C.c_void_p(out.data_ptr()),
                                                 None))
        torch.cuda.synchronize()
        r = ref.cpu().numpy()
        o = out.cpu().numpy()
        assert np.isfinite(o).all()
        np.testing.assert_array_equal(o, r)
    ctx.close()


def test_noalloc_allocates_nothing_on_a_fresh_context(gpu, oracle, mats):
    """Two no-alloc calls on a context that has never solved or assembled (its workspace is still
    unallocated) leave the device's free memory unchanged, then match the regular entry point bit
    for bit. A call on another context first does the once-per-device set-up (module load, address
    lookup)."""
    import torch

    G = oracle.generate_basis(9)
    raw = N.UepmMaterial.from_buffer_copy(bytes(mats["Ge"]))
    warm = api._Context(api.Material("Ge", raw=raw), G, True, True)
    ks = oracle.sample_first_bz(5, 9)
    dk = torch.from_numpy(ks).cuda()
    n = warm.n
    out = torch.zeros((len(ks), n, n), dtype=torch.complex128, device="cuda")
    N.check(gpu.uepm_assemble_device_noalloc(warm.h, C.c_void_p(dk.data_ptr()), len(ks), C.c_void_p(out.data_ptr()), None))
    ctx = api._Context(api.Material("Ge", raw=raw), G, True, True)
    out2 = torch.zeros_like(out)
    ref = torch.zeros_like(out)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for o in (out, out2):
        N.check(gpu.uepm_assemble_device_noalloc(ctx.h, C.c_void_p(dk.data_ptr()), len(ks), C.c_void_p(o.data_ptr()),
                                                 None))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    N.check(gpu.uepm_assemble_device(ctx.h, C.c_void_p(dk.data_ptr()), len(ks), C.c_void_p(ref.data_ptr()), None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), ref.cpu().numpy())
    np.testing.assert_array_equal(out2.cpu().numpy(), ref.cpu().numpy())
    ctx.close()
    warm.close()


def test_noalloc_rejects_requests_beyond_its_scratch(gpu, oracle, mats):
    import torch

    G = oracle.generate_basis(10)
    ctx = api._Context(api.Material("Si", raw=N.UepmMaterial.from_buffer_copy(bytes(mats["Si-CB"]))), G, False, False)
    per_k = len(G) * 24 * 8
    too_many = N.NOALLOC_SCRATCH_BYTES // per_k + 1
    dk = torch.zeros((too_many, 3), dtype=torch.float64, device="cuda")
    dH = torch.zeros((1,), dtype=torch.complex128, device="cuda")  # never written: the call is refused first
    rc = gpu.uepm_assemble_device_noalloc(ctx.h, C.c_void_p(dk.data_ptr()), too_many, C.c_void_p(dH.data_ptr()), None)
    assert rc == N.UEPM_ERR_INVALID
    assert "limit" in N.last_error()
    # more k-points than one assembly launch takes, with a one-plane-wave basis small enough for the
    # scratch to admit them
    G2 = np.zeros((1, 3), dtype=np.int32)
    small = api._Context(api.Material("Si", raw=N.UepmMaterial.from_buffer_copy(bytes(mats["Si-CB"]))), G2, False, False)
    nk = 32769
    assert nk * len(G2) * 24 * 8 <= N.NOALLOC_SCRATCH_BYTES
    dk2 = torch.zeros((nk, 3), dtype=torch.float64, device="cuda")
    rc = gpu.uepm_assemble_device_noalloc(small.h, C.c_void_p(dk2.data_ptr()), nk, C.c_void_p(dH.data_ptr()), None)
    assert rc == N.UEPM_ERR_INVALID
    assert "32768" in N.last_error()
    small.close()
    ctx.close()
