"""Multi-process (gloo, CPU) tests of the N > 1 host logic: column sharding,
max/sum over ranks and result collection.  The per-rank compute is the CPU
oracle (test infrastructure) standing in for the GPU kernels, which see only
their own column block: sharded results must equal the single-process
result column for column."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
dist_mod = pytest.importorskip("fast_pauli.distributed")


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, S, one_d):
    import torch.distributed as dist

    from fast_pauli import distributed as fd

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(90 + n)
        strings = oracle.calculate_pauli_strings_max_weight(n, 2)[1:]
        P, K = len(strings), 3
        h = rng.standard_normal((P, K)) + 1j * rng.standard_normal((P, K))
        psi = oracle.unit_norm_states(rng, 1 << n, S)
        if one_d:
            psi = psi[:, 0]
        mine = fd.shard_columns(psi, world, rank)
        mine2 = mine.reshape(1 << n, -1)
        local = oracle.summed_expectation(strings, h, mine2) if mine2.shape[1] else np.zeros((K, 0), complex)
        n_cols = 1 if one_d else S
        full = fd.gather_columns(torch.from_numpy(np.ascontiguousarray(local)), n_cols, dist)
        # timings: the slowest rank sets the step time; units add up
        t = fd.max_over_ranks(0.5 + rank, dist)
        units = fd.sum_over_ranks(P * (1 << n) * mine2.shape[1], dist)
        dist.barrier()
        if rank == 0:
            want = oracle.summed_expectation(strings, h, psi.reshape(1 << n, -1))
            got = full.numpy()
            assert got.shape == want.shape, (got.shape, want.shape)
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-13)
            assert t == 0.5 + (world - 1)
            assert units == P * (1 << n) * n_cols
        else:
            assert full is None
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("S,one_d", [(7, False), (1, False), (4, True)])
def test_sharded_expectation_world2(S, one_d):
    oracle.lib()  # build the oracle once, before the ranks start
    port = _free_port()
    torch.multiprocessing.spawn(_worker, args=(2, port, 5, S, one_d), nprocs=2, join=True)


def test_column_shard_partitions():
    fd = dist_mod
    for S in (0, 1, 2, 7, 1024, 1025):
        for world in (1, 2, 3, 8):
            ranges = [fd.column_shard(S, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == S
            for (b0, e0), (b1, e1) in zip(ranges, ranges[1:]):
                assert e0 == b1 and e0 >= b0
            sizes = [e - b for b, e in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        fd.column_shard(4, 2, 2)
    assert fd.max_over_ranks(3.25) == 3.25  # no process group: the value itself
