"""Multi-rank path on CPU: two gloo ranks split the ECP centres, compute their
shards (with the oracle standing in for the GPU engine) and all-reduce; the
sum equals the single-process matrix."""
import os
import socket

import numpy as np
import pytest

from libecp_gb300 import dist as D
from libecp_gb300 import workloads as W


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = W.random_system(31, n_atoms=5, n_centres=4, lmax_basis=2, lmax_ecp=3, kmax=2)
    I = D.distributed_get_integrals(s, lambda sub: O.oracle_matrix(sub)[1], rank, world)
    if rank == 0:
        np.save(out_path, I)
    dist.barrier()
    dist.destroy_process_group()


def test_centre_sharding_is_a_partition():
    s = W.batched_cluster(0)
    got = sorted(c for r in range(3) for c in D.centres_of_rank(s, r, 3))
    assert got == [a for a in range(s.n_atoms) if s.shellsECP[a] > 0]


def test_two_gloo_ranks_sum_to_single_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle import oracle as O
    out = str(tmp_path / "I.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    I = np.load(out)
    s = W.random_system(31, n_atoms=5, n_centres=4, lmax_basis=2, lmax_ecp=3, kmax=2)
    rc, ref = O.oracle_matrix(s)
    assert rc == 0
    assert np.max(np.abs(I - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
