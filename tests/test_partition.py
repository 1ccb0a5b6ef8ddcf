"""k-point partition over ranks and the gather to the owner (ultimateepm_gb300.partition): pure
functions, and world-size 2 and 3 runs over gloo on CPU in which each rank solves its block with the
oracle (the stand-in for its GPU) and rank 0 checks the gathered bands against one solve of the
whole list."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from conftest import PARAMS, ROOT
from ultimateepm_gb300 import partition as P


@pytest.mark.parametrize("nk,world", [(0, 1), (1, 1), (10, 3), (2000, 8), (7, 7), (5, 8), (1000003, 6)])
def test_block_counts_follow_the_reference_scheme(nk, world):
    c = P.block_counts(nk, world)
    base, rem = divmod(nk, world)
    assert c.sum() == nk and len(c) == world
    assert (c[:rem] == base + 1).all() and (c[rem:] == base).all()
    o = P.block_offsets(c)
    assert o[0] == 0 and (o[1:] == np.cumsum(c)[:-1]).all()
    covered = np.concatenate([np.arange(*P.shard_range(nk, r, world)) for r in range(world)])
    assert (covered == np.arange(nk)).all()


def test_partition_rejects_bad_arguments():
    with pytest.raises(ValueError):
        P.block_counts(10, 0)
    with pytest.raises(ValueError):
        P.shard_range(10, 3, 3)
    with pytest.raises(ValueError):
        P.cost_bins([1.0], 0)


def test_cost_bins_balance_uneven_groups():
    # config-4-like groups: orders 89..458, random k-point shares
    rng = np.random.default_rng(7)
    orders = [89, 113, 137, 169, 181, 229, 178, 226, 274, 338, 362, 458]
    nks = rng.multinomial(200000, rng.dirichlet(np.ones(len(orders))))
    costs = [P.solve_cost(n, k) for n, k in zip(orders, nks)]
    for world in (1, 2, 4, 8):
        bins = P.cost_bins(costs, world)
        assert sorted(i for b in bins for i in b) == list(range(len(costs)))
        loads = [sum(costs[i] for i in b) for b in bins]
        # the longest-processing-time rule: makespan <= 4/3 of the lower bound max(mean, largest item)
        assert max(loads) <= 4.0 / 3.0 * max(sum(costs) / world, max(costs)) + 1e-9


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, nk, out_path):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from oracle import oracle as O
    from ultimateepm_gb300 import partition as P

    dist.init_process_group("gloo", rank=rank, world_size=world)
    mat = O.load_materials(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))["Si"]
    G = O.generate_basis(8)
    k = O.sample_first_bz(nk, 123)
    nb = 8

    def solve(kb):
        if len(kb) == 0:
            return np.zeros((0, nb))
        return O.band_structure(mat, G, kb, nb, nthreads=1)["E"]

    E = P.distributed_solve(solve, k, dst=0)
    if rank == 0:
        np.save(out_path, E)
    else:
        assert E is None
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,nk", [(2, 37), (3, 2)])
def test_distributed_solve_gathers_the_same_bands(oracle, tmp_path, world, nk):
    """World 2 with an odd k count (uneven blocks); world 3 with an empty block."""
    out = str(tmp_path / "E.npy")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, nk, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    E = np.load(out)
    mat = oracle.load_materials(os.path.join(PARAMS, "si-cohen-bergstresser.yaml"))["Si"]
    ref = oracle.band_structure(mat, oracle.generate_basis(8), oracle.sample_first_bz(nk, 123), 8, nthreads=1)["E"]
    assert E.shape == ref.shape
    assert np.array_equal(E, ref)
