"""Dielectric function from the band states (DielectricFunction, src/EPP/DielectricFunction.cpp):
the k-point grids, the merge and Kramers-Kronig steps of the host mirror against the oracle's
restatement; the distributed form of apps/epsilon.cpp (per-rank k blocks, a gather and the merge)
over gloo ranks; and on the GPU, the overlap and smeared-pair sums (uepm_dielectric_sums_device)
and the whole compute_dielectric_function against the oracle."""
import ctypes as C
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from ultimateepm_gb300 import _native as N
from ultimateepm_gb300 import api
from ultimateepm_gb300 import dielectric as D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PARAMS = os.path.join(ROOT, "params")


def _mat(orm):
    return api.Material("m", raw=N.UepmMaterial.from_buffer_copy(bytes(orm)))


@pytest.mark.parametrize("nxyz,shift,iw", [((5, 5, 5), 0.0, False), ((9, 7, 8), 0.05, False), ((11, 11, 11), 0.0, True),
                                           ((2, 2, 2), 0.0, False)])
def test_k_grid_matches_the_reference_loops(oracle, nxyz, shift, iw):
    df = D.DielectricFunction(api.Material("m"), np.zeros((1, 3), dtype=np.int32), 8)
    df.generate_k_points_grid(*nxyz, shift, iw)
    np.testing.assert_array_equal(df.get_kpoints(), oracle.dielectric_k_grid(*nxyz, shift, iw))


def test_random_k_points_are_in_the_first_zone_and_seeded():
    a = D.DielectricFunction(api.Material("m"), np.zeros((1, 3), dtype=np.int32), 8)
    b = D.DielectricFunction(api.Material("m"), np.zeros((1, 3), dtype=np.int32), 8)
    a.generate_k_points_random(500, seed=3)
    b.generate_k_points_random(500, seed=3)
    k = a.get_kpoints()
    assert k.shape == (500, 3) and np.array_equal(k, b.get_kpoints())
    assert np.all(np.abs(k) <= 1.0) and np.all(np.abs(k).sum(axis=1) <= 1.5)


def test_kramers_matrix_and_merge_match_the_oracle(oracle):
    np.testing.assert_array_equal(D.create_kramers_matrix(7), oracle.kramers_matrix(7))
    rng = np.random.default_rng(4)
    qs = [np.array([0.0, 0.0, 0.0]), np.array([0.1, 0.0, 0.0]), np.array([0.02, 0.03, -0.01])]
    results = [[rng.normal(size=12) for _ in qs] for _ in range(3)]
    counts = [5, 7, 4]
    root = D.DielectricFunction(api.Material("m"), np.zeros((1, 3), dtype=np.int32), 8)
    root.set_qpoints(qs)
    root.set_energies(np.linspace(0, 5, 12))
    merged = D.DielectricFunction.merge_results(root, results, counts)
    ref = oracle.dielectric_merge(qs, results, counts)
    np.testing.assert_allclose(np.array(merged.get_dielectric_function()), ref, rtol=1e-15, atol=0)
    merged.apply_kramers_kronig()
    np.testing.assert_allclose(np.array(merged.m_dielectric_function_imag), oracle.kramers_kronig(ref), rtol=1e-14,
                               atol=1e-12)
    with pytest.raises(RuntimeError):
        D.DielectricFunction.merge_results(root, [], [])
    with pytest.raises(RuntimeError):
        D.DielectricFunction.merge_results(root, results, counts[:2])


def test_pair_sums_on_a_hand_case(oracle):
    """One k-point, one conduction band: O = |sum_i a_i b_i|^2 (no factor conjugated, as the
    reference's Eigen expression evaluates), and the smeared pair at each energy."""
    n, nb = 3, 5
    Xk = np.zeros((1, nb, n), dtype=np.complex128)
    Xkq = np.zeros((1, nb, n), dtype=np.complex128)
    Xk[0, 2] = [1j, 0.0, 0.0]           # valence band 2
    Xkq[0, 4] = [1j, 0.0, 0.0]          # conduction band 4: sum a_i b_i = -1, |.|^2 = 1
    Ek = np.array([[-1.0, -0.5, -0.25, 0.0, 9.0]])
    Ekq = np.array([[0.0, 0.0, 0.0, 0.0, 1.75]])
    en = np.array([0.0, 1.0, 2.0])
    eta = 0.1
    d = 1.75 - (-0.25)
    want = (d - en) / ((d - en) ** 2 + eta ** 2) + (d + en) / ((d + en) ** 2 + eta ** 2)
    got = oracle.dielectric_pair_sums(Ek, Xk, Ekq, Xkq, en, eta)
    np.testing.assert_allclose(got, want, rtol=1e-15)
    np.testing.assert_allclose(oracle.dielectric_pair_sums(Ek, Xk, Ekq, Xkq, en, eta, weights=[2.5]), 2.5 * want,
                               rtol=1e-15)


# ---- apps/epsilon.cpp's distributed form over gloo ranks -------------------------------------------
def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_path):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from oracle import oracle as O
    from ultimateepm_gb300 import partition as P
    from ultimateepm_gb300 import dielectric as DD
    from ultimateepm_gb300 import api as A

    dist.init_process_group("gloo", rank=rank, world_size=world)
    mat = O.load_materials(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))["Si"]
    G = O.generate_basis(4)
    k = O.sample_first_bz(11, 77)
    qs = [np.zeros(3), np.array([0.05, 0.02, 0.0])]
    en = np.linspace(0.0, 6.0, 9)
    counts = P.block_counts(len(k), world)
    a, b = P.shard_range(len(k), rank, world)
    # this rank's block (the oracle stands in for the device sums of compute_dielectric_function)
    local = np.stack([O.dielectric_sums(mat, G, k[a:b], q, 8, en, 0.05) if b > a else np.zeros(len(en)) for q in qs])
    flat = P.gather_blocks(local.reshape(1, -1), [1] * world, dst=0)  # one row of [q * ne] per rank
    if rank == 0:
        results = [list(row.reshape(len(qs), len(en))) for row in flat]
        root = DD.DielectricFunction(A.Material("m"), G, 8)
        root.set_qpoints(qs)
        root.set_energies(en)
        merged = DD.DielectricFunction.merge_results(root, results, list(counts))
        np.save(out_path, np.array(merged.get_dielectric_function()))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_distributed_dielectric_merge_equals_one_process(oracle, tmp_path, world):
    out = str(tmp_path / "eps.npy")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = np.load(out)
    mat = oracle.load_materials(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))["Si"]
    G = oracle.generate_basis(4)
    k = oracle.sample_first_bz(11, 77)
    qs = [np.zeros(3), np.array([0.05, 0.02, 0.0])]
    en = np.linspace(0.0, 6.0, 9)
    whole = [[oracle.dielectric_sums(mat, G, k, q, 8, en, 0.05) for q in qs]]
    ref = oracle.dielectric_merge(qs, whole, [len(k)])
    np.testing.assert_allclose(got, ref, rtol=1e-12)


# ---- GPU ------------------------------------------------------------------------------------------
@pytest.mark.gpu
def test_device_sums_match_the_oracle_on_the_same_states(gpu, oracle, mats):
    """The kernel alone: oracle eigenstates in, the oracle's pair sums out (with and without
    per-k weights, and accumulating into the output)."""
    import torch

    G = oracle.generate_basis(10)
    k = oracle.sample_first_bz(37, 5)
    q = np.array([0.03, -0.01, 0.02])
    nb = 12
    a = oracle.band_structure(mats["Si-CB"], G, k, nb, vectors=True)
    b = oracle.band_structure(mats["Si-CB"], G, k + q, nb, vectors=True)
    en = np.linspace(0.0, 12.0, 300)
    w = np.random.default_rng(1).uniform(0.5, 2.0, len(k))
    dev = "cuda"
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    Xk = t(a["vecs"].view(np.float64))
    Xkq = t(b["vecs"].view(np.float64))
    Ek, Ekq, den, dw = t(a["E"]), t(b["E"]), t(en), t(w)
    sums = torch.zeros(len(en), dtype=torch.float64, device=dev)
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda x: C.c_void_p(x.data_ptr())
    n = G.shape[0]
    N.check(gpu.uepm_dielectric_sums_device(p(Xk), p(Xkq), p(Ek), p(Ekq), len(k), nb, n, 4, p(den), len(en), 0.05, None,
                                            p(sums), sp))
    torch.cuda.synchronize()
    ref = oracle.dielectric_pair_sums(a["E"], a["vecs"], b["E"], b["vecs"], en, 0.05)
    np.testing.assert_allclose(sums.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    # weighted, added to what is there
    N.check(gpu.uepm_dielectric_sums_device(p(Xk), p(Xkq), p(Ek), p(Ekq), len(k), nb, n, 4, p(den), len(en), 0.05, p(dw),
                                            p(sums), sp))
    torch.cuda.synchronize()
    refw = ref + oracle.dielectric_pair_sums(a["E"], a["vecs"], b["E"], b["vecs"], en, 0.05, weights=w)
    np.testing.assert_allclose(sums.cpu().numpy(), refw, rtol=1e-12, atol=1e-12 * np.abs(refw).max())
    # argument errors
    bad = gpu.uepm_dielectric_sums_device(p(Xk), p(Xkq), p(Ek), p(Ekq), len(k), nb, n, nb, p(den), len(en), 0.05, None,
                                          p(sums), sp)
    assert bad == N.UEPM_ERR_INVALID
    bad = gpu.uepm_dielectric_sums_device(p(Xk), p(Xkq), p(Ek), p(Ekq), len(k), nb, n, 4, p(den), 5000, 0.05, None,
                                          p(sums), sp)
    assert bad == N.UEPM_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("case,nl", [("Si-CB", False), ("Si-d", True)])
def test_dielectric_function_matches_the_oracle(gpu, oracle, mats, case, nl):
    """compute_dielectric_function (device solves at k and k + q, then the device sums) against the
    oracle's restatement, two q (one of them 0, replaced by 1e-15 as the reference does), then the
    merge and Kramers-Kronig."""
    G = oracle.generate_basis(10)
    df = D.DielectricFunction(_mat(mats[case]), G, 12)
    df.set_non_local_epm(nl)
    df.generate_k_points_random(40, seed=9)
    k = df.get_kpoints()
    qs = [np.zeros(3), np.array([0.04, 0.01, -0.02])]
    en = np.linspace(0.0, 10.0, 200)
    df.set_qpoints(qs)
    df.set_energies(en)
    df.chunk = 16  # several chunks, the last one partial
    df.set_offset_k_index(3)
    df.set_nb_kpoints(len(k) - 5)
    df.compute_dielectric_function(0.1)
    got = np.array(df.get_dielectric_function())
    ks = k[3:len(k) - 2]
    ref = np.stack([oracle.dielectric_sums(mats[case], G, ks, q, 12, en, 0.1, nl=nl) for q in qs])
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * scale)
    merged = D.DielectricFunction.merge_results(df, [list(got)], [len(ks)])
    eps = np.array(merged.get_dielectric_function())
    np.testing.assert_allclose(eps, oracle.dielectric_merge(qs, [list(ref)], [len(ks)]), rtol=1e-9)
