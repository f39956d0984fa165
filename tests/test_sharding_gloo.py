"""Visibility sharding of the operator across ranks (CPU, gloo, world size 2).

The reference's "distribute image" operator (cpp/purify/operators.h:416-461)
gives each rank a shard of the visibilities: the forward is local, and the
adjoint is the local Phi^H followed by an all-sum of the image
(operators.h:117-120, 433-435).  This checks that math with the oracle on two
gloo ranks: concatenated forward shards equal the unsharded forward, and the
all-reduced adjoint images equal the unsharded adjoint.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    rng = np.random.default_rng(4)
    M, n = 2000, 32
    u = rng.normal(0, 12, M)
    v = rng.normal(0, 12, M)
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    return u, v, wt, x, y, n


def _rank(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    u, v, wt, x, y, n = _problem()
    M = u.size
    lo, hi = rank * M // world, (rank + 1) * M // world
    op = oracle.Operator(u[lo:hi], v[lo:hi], None, wt[lo:hi], n, n, 2.0, kernel="kb", Ju=4, Jv=4)
    y_local = torch.from_numpy(op.forward(x))
    shards = [torch.empty(((r + 1) * M // world - r * M // world,), dtype=torch.complex128)
              for r in range(world)]
    dist.all_gather(shards, y_local)
    img = torch.from_numpy(op.adjoint(y[lo:hi]))
    dist.all_reduce(img, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(os.path.join(out_dir, "fwd.npy"), torch.cat(shards).numpy())
        np.save(os.path.join(out_dir, "adj.npy"), img.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_visibility_sharded_operator(tmp_path, oracle_mod):
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    u, v, wt, x, y, n = _problem()
    full = oracle_mod.Operator(u, v, None, wt, n, n, 2.0, kernel="kb", Ju=4, Jv=4)
    fwd = np.load(os.path.join(str(tmp_path), "fwd.npy"))
    adj = np.load(os.path.join(str(tmp_path), "adj.npy"))
    assert np.allclose(fwd, full.forward(x), rtol=0, atol=1e-12 * np.abs(fwd).max())
    ref = full.adjoint(y)
    assert np.linalg.norm(adj - ref) <= 1e-12 * np.linalg.norm(ref)
