"""Replica sharding of the stochastic trace on two gloo ranks (CPU).

Each rank runs the oracle recursion on its share of the Philox phase vectors
and the shares are reduced with reduce_moments; the result must equal the
single-process mean over all vectors (FP64 sums in a different order: 1e-12).
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from leo2d_gb300.replicas import reduce_moments, vector_share

P, R, SEED = 16, 7, 123


def test_vector_share_partitions():
    for total in (0, 1, 7, 13, 64):
        for world in (1, 2, 3, 8):
            got = [vector_share(total, r, world) for r in range(world)]
            assert sum(c for _, c in got) == total
            assert [f for f, _ in got] == [sum(c for _, c in got[:r]) for r in range(world)]
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        vector_share(4, 2, 2)


def _system():
    from oracle import oracle
    from leo2d_gb300 import make_geom, MODEL_SIMPLE
    g = oracle.geom_prepare(make_geom(model=MODEL_SIMPLE, size=8, angles_deg=(0.0, 5.0), energy_rescale=12.0))
    b = oracle.Built(g)
    return b.compact()


def _moments(rp, col, val, first, count):
    from oracle import oracle
    if count == 0:
        return np.zeros(P)
    re, im = oracle.phase_vectors(SEED, first, count, len(rp) - 1)
    mu = oracle.kpm_trace(rp, col, val, re, P) + oracle.kpm_trace(rp, col, val, im, P)
    return mu.sum(axis=0)


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rp, col, val = _system()
        first, count = vector_share(R, rank, world)
        mean = reduce_moments(_moments(rp, col, val, first, count), count, dist)
        out[rank] = mean
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_reduction_matches_one_process():
    rp, col, val = _system()
    ref = _moments(rp, col, val, 0, R) / R
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
        res = dict(out)
    for rank in (0, 1):
        np.testing.assert_allclose(res[rank], ref, rtol=1e-12, atol=1e-12)
