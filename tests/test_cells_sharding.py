"""Sharding the batched cells over ranks (CPU, gloo, world size 2).

The cells of a batch are independent, so a multi-GPU run gives each rank a share and needs no
collective on the data path.  Every rank computes the same largest-first assignment locally; the
test checks, across two gloo ranks, that the shares cover every cell exactly once and balance the
device bytes, and that the results gathered on the host come back in cell order."""
import os
import socket

import numpy as np
import pytest

from anisotropicfracture_gb300 import cells

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_partition_is_balanced_and_complete():
    rng = np.random.default_rng(4)
    edges = rng.choice([16, 24, 32, 48, 64], size=512)
    sizes = [int(e) ** 3 * 600 for e in edges]
    for nranks in (1, 2, 3, 8):
        parts = cells.partition_cells(sizes, nranks)
        flat = sorted(c for p in parts for c in p)
        assert flat == list(range(512))
        loads = [sum(sizes[c] for c in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)


def _rank(rank, world, port, sizes, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = cells.partition_cells(sizes, world)[rank]
    # each rank "solves" its cells (a stand-in value per cell) and the host gathers them
    vals = torch.tensor([[c, 1000.0 + c] for c in mine], dtype=torch.float64)
    n = torch.tensor([len(mine)])
    ns = [torch.zeros(1, dtype=torch.long) for _ in range(world)]
    dist.all_gather(ns, n)
    width = int(max(x.item() for x in ns))
    pad = torch.full((width, 2), -1.0, dtype=torch.float64)
    pad[:len(mine)] = vals
    got = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(got, pad)
    if rank == 0:
        rows = torch.cat(got)
        rows = rows[rows[:, 0] >= 0]
        order = torch.argsort(rows[:, 0])
        out_q.put(rows[order].numpy().tolist())
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_every_cell_once():
    import torch.multiprocessing as mp
    rng = np.random.default_rng(5)
    sizes = [int(e) ** 3 for e in rng.choice([16, 24, 32, 48, 64], size=37)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    rows = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [int(r[0]) for r in rows] == list(range(37))
    assert all(r[1] == 1000.0 + r[0] for r in rows)
