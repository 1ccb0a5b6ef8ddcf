"""Uneven batches over several contexts (uepm_batch_*) and kernel-shape tuning (uepm_ctx_*_tuning,
uepm_ctx_autotune). The batch runs each group exactly as a solve of that group alone would (same
kernels, same per-k-point arithmetic), so results must be bit-identical whether a group runs alone
or in the mix, eagerly, captured into a CUDA graph or replayed; every tuning choice must stay within
the parity tolerances against the oracle."""
import ctypes as C

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api

pytestmark = pytest.mark.gpu

# name: (material key, shells, nl, soc, precision, nb, nk, want)
GROUPS = {
    "si_fp64": ("Si-CB", 10, False, False, N.UEPM_PREC_FP64, 16, 50, N.UEPM_WANT_VALUES),
    "si_mixed": ("Si-CB", 10, False, False, N.UEPM_PREC_MIXED, 16, 300, N.UEPM_WANT_VALUES),
    "ge_soc_mixed": ("Ge", 12, True, True, N.UEPM_PREC_MIXED, 16, 12, N.UEPM_WANT_VALUES),
    "gaas_soc_fp64_vec": ("GaAs", 8, True, True, N.UEPM_PREC_FP64, 8, 10,
                          N.UEPM_WANT_VALUES | N.UEPM_WANT_VECTORS | N.UEPM_WANT_GRADIENT),
    "sid_mixed_vec": ("Si-d", 10, True, False, N.UEPM_PREC_MIXED, 12, 40,
                      N.UEPM_WANT_VALUES | N.UEPM_WANT_VECTORS | N.UEPM_WANT_GRADIENT),
}


def _mat(orm):
    return api.Material("m", raw=N.UepmMaterial.from_buffer_copy(bytes(orm)))


class _Group:
    def __init__(self, oracle, mats, name, seed):
        import torch

        key, shells, nl, soc, prec, nb, nk, want = GROUPS[name]
        self.name, self.key, self.nl, self.soc, self.prec, self.want = name, key, nl, soc, prec, want
        self.G = oracle.generate_basis(shells)
        self.ctx = api._Context(_mat(mats[key]), self.G, nl, soc, prec)
        self.nb = nb
        self.k = oracle.sample_first_bz(nk, seed)
        n = self.ctx.n
        dev = "cuda"
        self.dk = torch.from_numpy(self.k).to(dev)
        self.dE = torch.zeros((nk, nb), dtype=torch.float64, device=dev)
        self.dX = torch.zeros((nk, nb, n, 2), dtype=torch.float64, device=dev) if want & N.UEPM_WANT_VECTORS else None
        self.dg = torch.zeros((nk, nb, 3), dtype=torch.float64, device=dev) if want & N.UEPM_WANT_GRADIENT else None
        self.ds = torch.zeros(nk, dtype=torch.int32, device=dev)

    def ptrs(self):
        p = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
        return p(self.dk), len(self.k), self.nb, self.want, p(self.dE), p(self.dX), p(self.dg), p(self.ds)

    def zero(self):
        for t in (self.dE, self.dX, self.dg, self.ds):
            if t is not None:
                t.zero_()

    def solve_alone(self, L, stream):
        dk, nk, nb, want, dE, dX, dg, ds = self.ptrs()
        N.check(L.uepm_solve_device(self.ctx.h, dk, nk, nb, want, dE, dX, dg, ds, stream))

    def results(self):
        out = [self.dE.cpu().numpy().copy()]
        for t in (self.dX, self.dg):
            out.append(None if t is None else t.cpu().numpy().copy())
        out.append(self.ds.cpu().numpy().copy())
        return out


def _same(a, b):
    return all((x is None and y is None) or np.array_equal(x, y) for x, y in zip(a, b))


def test_batch_results_identical_alone_and_in_the_mix(gpu, oracle, mats):
    import torch

    L = gpu
    s = torch.cuda.current_stream()
    sp = C.c_void_p(s.cuda_stream)
    groups = [_Group(oracle, mats, name, 100 + q) for q, name in enumerate(GROUPS)]
    alone = []
    for g in groups:
        g.zero()
        g.solve_alone(L, sp)
        torch.cuda.synchronize()
        alone.append(g.results())
    b = C.c_void_p()
    N.check(L.uepm_batch_create(C.byref(b)))
    try:
        for g in groups:
            N.check(L.uepm_batch_add(b, g.ctx.h, *g.ptrs()))
        for run in ("eager", "captured", "replayed", "replayed again"):
            for g in groups:
                g.zero()
            l0 = L.uepm_kernel_launches()
            N.check(L.uepm_batch_run(b, sp))
            torch.cuda.synchronize()
            kpr = L.uepm_batch_kernels_per_run(b)
            assert kpr > 0 and L.uepm_kernel_launches() - l0 == kpr, run
            for g, ref in zip(groups, alone):
                assert _same(g.results(), ref), (run, g.name)
                assert not g.ds.any().item(), (run, g.name)
    finally:
        L.uepm_batch_destroy(b)
    # and the values are right: each group against the oracle
    tol = {N.UEPM_PREC_FP64: 1e-10, N.UEPM_PREC_MIXED: 1e-6}
    for g, ref in zip(groups, alone):
        Eo = oracle.band_structure(mats[g.key], g.G, g.k, g.nb, nl=g.nl, soc=g.soc)["E"]
        assert np.abs(ref[0] - Eo).max() <= tol[g.prec], g.name
    for g in groups:
        g.ctx.close()


def test_batch_replay_reads_the_registered_buffers(gpu, oracle, mats):
    import torch

    L = gpu
    s = torch.cuda.current_stream()
    sp = C.c_void_p(s.cuda_stream)
    g = _Group(oracle, mats, "si_mixed", 7)
    h = _Group(oracle, mats, "si_fp64", 8)
    b = C.c_void_p()
    N.check(L.uepm_batch_create(C.byref(b)))
    try:
        N.check(L.uepm_batch_add(b, g.ctx.h, *g.ptrs()))
        N.check(L.uepm_batch_add(b, h.ctx.h, *h.ptrs()))
        for _ in range(2):  # eager, then captured
            N.check(L.uepm_batch_run(b, sp))
        # new k-points in the same device buffers, then a replay
        k2 = oracle.sample_first_bz(len(g.k), 99)
        g.dk.copy_(torch.from_numpy(k2))
        N.check(L.uepm_batch_run(b, sp))
        torch.cuda.synchronize()
        got = g.results()[0]
        g.k = k2
        g.zero()
        g.solve_alone(L, sp)
        torch.cuda.synchronize()
        assert np.array_equal(got, g.results()[0])
        # adding a group drops the graph; the next runs still agree
        N.check(L.uepm_batch_clear(b))
        N.check(L.uepm_batch_add(b, h.ctx.h, *h.ptrs()))
        N.check(L.uepm_batch_run(b, sp))
    finally:
        L.uepm_batch_destroy(b)
    g.ctx.close()
    h.ctx.close()


@pytest.mark.parametrize("prec,tuning", [
    (N.UEPM_PREC_MIXED, dict(reduction=2)),
    (N.UEPM_PREC_MIXED, dict(reduction=1, vector_lanes=16, chunk=256)),
    (N.UEPM_PREC_MIXED, dict(reduction=3, cluster=2)),
    (N.UEPM_PREC_MIXED, dict(reduction=4)),
    (N.UEPM_PREC_MIXED, dict(reduction=5)),
    (N.UEPM_PREC_MIXED, dict(vector_lanes=32, chunk=64)),
    (N.UEPM_PREC_FP64, dict(ctas_per_sm=1, chunk=512)),
    (N.UEPM_PREC_FP64, dict(ctas_per_sm=8, vector_lanes=16)),
    (N.UEPM_PREC_FP64, dict(reduction=3, cluster=4)),
    (N.UEPM_PREC_MIXED, dict(streams=2, chunk=64)),
    (N.UEPM_PREC_MIXED, dict(streams=1)),
    (N.UEPM_PREC_FP64, dict(streams=2)),
])
def test_every_tuning_choice_keeps_parity(gpu, oracle, mats, prec, tuning):
    G = oracle.generate_basis(10)
    ks = oracle.sample_first_bz(700, 5)
    ctx = api._Context(_mat(mats["Si-CB"]), G, False, False, prec)
    t = N.UepmTuning(**tuning)
    N.check(gpu.uepm_ctx_set_tuning(ctx.h, C.byref(t)))
    back = N.UepmTuning()
    N.check(gpu.uepm_ctx_get_tuning(ctx.h, C.byref(back)))
    assert back.as_dict() == t.as_dict()
    E, X, g, st = ctx.solve(ks, 16, vectors=True, gradient=True)
    ref = oracle.band_structure(mats["Si-CB"], G, ks, 16)["E"]
    assert not st.any()
    assert np.abs(E - ref).max() <= (1e-10 if prec == N.UEPM_PREC_FP64 else 1e-6)
    ctx.close()


def test_set_tuning_rejects_out_of_range_fields(gpu, oracle, mats):
    ctx = api._Context(_mat(mats["Si-CB"]), oracle.generate_basis(8), False, False)
    for bad in (dict(reduction=7), dict(tensor_cores=2), dict(streams=3), dict(ctas_per_sm=9), dict(vector_lanes=12), dict(chunk=10), dict(cluster=3)):
        assert gpu.uepm_ctx_set_tuning(ctx.h, C.byref(N.UepmTuning(**bad))) == N.UEPM_ERR_OUT_OF_RANGE
    ctx.close()


def test_autotune_picks_a_valid_shape_and_caches_it(gpu, oracle, mats):
    import time

    import torch

    G = oracle.generate_basis(9)
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = api._Context(_mat(mats["Si-CB"]), G, False, False, N.UEPM_PREC_MIXED)
    N.check(gpu.uepm_ctx_autotune(a.h, 16, N.UEPM_WANT_VALUES, 1024, sp))
    ta = N.UepmTuning()
    N.check(gpu.uepm_ctx_get_tuning(a.h, C.byref(ta)))
    assert ta.reduction in (0, 1, 2, 3) and ta.vector_lanes in (0, 8, 16, 32) and ta.cluster in (0, 2, 4, 8, 16)
    assert ta.chunk == 0 or 64 <= ta.chunk <= 32768
    b = api._Context(_mat(mats["Si-CB"]), G, False, False, N.UEPM_PREC_MIXED)
    t0 = time.perf_counter()
    N.check(gpu.uepm_ctx_autotune(b.h, 16, N.UEPM_WANT_VALUES, 1024, sp))
    assert time.perf_counter() - t0 < 0.5  # served from the cache
    tb = N.UepmTuning()
    N.check(gpu.uepm_ctx_get_tuning(b.h, C.byref(tb)))
    assert tb.as_dict() == ta.as_dict()
    ks = oracle.sample_first_bz(200, 3)
    E, _, _, st = b.solve(ks, 16)
    assert not st.any()
    assert np.abs(E - oracle.band_structure(mats["Si-CB"], G, ks, 16)["E"]).max() <= 1e-6
    a.close()
    b.close()
