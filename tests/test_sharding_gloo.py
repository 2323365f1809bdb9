"""Multi-rank ket sharding on CPU: two gloo ranks each evolve their share of the kets (oracle
arithmetic standing in for the per-rank GPU step) and all-reduce the readouts."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "latticemodels.jl_gb300"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from lmgpu.sharding import allreduce_sum, shard_range
    from oracle import lm_oracle as o
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lat = o.SquareLattice(6, 5, periodic=(True, False))
        V = o.anderson_disorder(lat.N, 2.0, 3)
        H = o.tightbinding_hamiltonian(lat, field=o.LandauGauge(0.05), onsite=V)
        X = o.random_kets(lat.N, 7, 4)
        lo, hi = shard_range(7, rank, world)
        Y = X[:, lo:hi]
        for _ in range(3):
            Y = o.expm_multiply(H, 0.1, Y)
        bonds = o.nn_bonds(lat)
        src = np.array([b.src for b in bonds]); dst = np.array([b.dst for b in bonds])
        rho = allreduce_sum(o.localdensity(Y, weights=np.ones(hi - lo)))
        J = allreduce_sum(o.bond_currents(H, Y, src, dst, weights=np.ones(hi - lo), is_density=False))
        if rank == 0:
            out_q.put((rho, J))
    finally:
        dist.destroy_process_group()


def test_shard_range_partitions():
    from lmgpu.sharding import shard_range
    for M in (1, 7, 2048):
        for world in (1, 2, 3, 8):
            rs = [shard_range(M, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == M
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 1


def test_two_rank_sharded_readouts_match_unsharded():
    import multiprocessing as mp
    from oracle import lm_oracle as o
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    rho, J = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    lat = o.SquareLattice(6, 5, periodic=(True, False))
    V = o.anderson_disorder(lat.N, 2.0, 3)
    H = o.tightbinding_hamiltonian(lat, field=o.LandauGauge(0.05), onsite=V)
    X = o.random_kets(lat.N, 7, 4)
    for _ in range(3):
        X = o.expm_multiply(H, 0.1, X)
    bonds = o.nn_bonds(lat)
    src = np.array([b.src for b in bonds]); dst = np.array([b.dst for b in bonds])
    assert np.allclose(rho, o.localdensity(X, weights=np.ones(7)), atol=1e-13)
    assert np.allclose(J, o.bond_currents(H, X, src, dst, weights=np.ones(7), is_density=False), atol=1e-13)
