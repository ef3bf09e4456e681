"""The reference's particle decomposition (maind.f:140) over two ranks.

Each rank deposits only its own particles, and the moments are then
summed across ranks, as the reference does with MPI_ALLREDUCE
(gutsp.f:1503,1812-1822). The C-ABI keeps that contract: a deposit entry
returns the folded, complete moments of the local particles, and the caller
all-reduces. This test runs that protocol with gloo on CPU. The oracle
stands in for the device, since the protocol is the same. The test checks
that the reduced moments match a single-rank deposit of all particles.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _make(n_local, offset, total, seed=5):
    """Particles offset..offset+n_local of a fixed random population."""
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root / "oracle"))
    import pyoracle

    nx, ny, nz = 10, 6, 8
    rng = np.random.default_rng(seed)
    xp_all = np.empty((total, 3))
    xp_all[:, 0] = 1.0 + rng.random(total) * (nx - 2)
    xp_all[:, 1] = 1.0 + rng.random(total) * (ny - 2)
    xp_all[:, 2] = 1.0 + rng.random(total) * (nz - 2)
    vp_all = 0.3 * rng.standard_normal((total, 3)) + np.array([2.0, 0, 0])
    o = pyoracle.Oracle(nx, ny, nz, max(n_local, 1), 0.05, 10, 1.0, 4.0)
    xp = np.asfortranarray(xp_all[offset:offset + n_local])
    vp = np.asfortranarray(vp_all[offset:offset + n_local])
    z3 = np.zeros((max(n_local, 1), 3), order="F")
    xp_b = np.array(z3, order="F")
    vp_b = np.array(z3, order="F")
    xp_b[:n_local] = xp
    vp_b[:n_local] = vp
    mrat = np.ones(max(n_local, 1))
    beta_p = np.ones(max(n_local, 1))
    ijkp = np.zeros((max(n_local, 1), 3), dtype=np.int32, order="F")
    ni = np.array([n_local], dtype=np.int32)
    o.bind_particles(xp_b, vp_b, np.array(vp_b, order="F"), mrat, beta_p, ijkp, ni)
    g = lambda n: np.zeros((nx, ny, nz, n), order="F") if n > 1 else np.zeros((nx, ny, nz), order="F")
    return o, xp_b, vp_b, g


def _rank(rank, world, port, total, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n_local = total // world
    o, xp, vp, g = _make(n_local, rank * n_local, total)
    np_ = g(1)
    up = g(3)
    o.get_interp_weights(xp)
    o.update_np(np_)  # complete local moments
    t = torch.from_numpy(np_.ravel(order="F").copy())
    dist.all_reduce(t)  # the caller's MPI_ALLREDUCE (gutsp.f:1503)
    np_global = np.asfortranarray(t.numpy().reshape(np_.shape, order="F"))
    o.update_up(vp, np_global, up)  # local particles, global np (gutsp.f:1704)
    t = torch.from_numpy(up.ravel(order="F").copy())
    dist.all_reduce(t)  # gutsp.f:1812-1822
    if rank == 0:
        q.put((np_global, t.numpy().reshape(up.shape, order="F")))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_deposit_matches_single_rank():
    total = 4000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, total, q)) for r in range(2)]
    for p in procs:
        p.start()
    np2, up2 = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    o, xp, vp, g = _make(total, 0, total)
    np1, up1 = g(1), g(3)
    o.get_interp_weights(xp)
    o.update_np(np1)
    o.update_up(vp, np1, up1)
    assert np.max(np.abs(np2 - np1)) <= 1e-12 * np.max(np.abs(np1))
    assert np.max(np.abs(up2 - up1)) <= 1e-12 * np.max(np.abs(up1))
