"""Sharding the batched cells over ranks (CPU, gloo, world size 2).

The cells of a batch are independent, so a multi-GPU run gives each rank a share and needs no
collective on the data path.  Every rank computes the same largest-first assignment locally.
Checked across two gloo ranks: the shares cover every cell exactly once and balance the device
bytes; each rank solves its own cells (the oracle's periodic-cell solve, one host thread) and the
results gathered on rank 0, put back in cell order, equal a single-process solve of all cells
bit for bit (iterations, fluctuation field, mean stress)."""
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


CELL_OPTS = dict(max_fmg_iter=0, nu1=2, nu2=2, sweeps=2, bottom=1, bottom_max_iter=200, bottom_reltol=1e-4, nuf=8,
                 max_iter=100)


def _work(ncells=10, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for c in range(ncells):
        n = int(rng.choice([8, 12, 16]))
        seeds, table = cells.rve_grains(n, int(rng.integers(3, 7)), int(rng.integers(1 << 30)))
        out.append((n, seeds, table))
    return out


def _solve(work, idx):
    """The oracle's cell solve of the cells idx (exx = 1e-3): {cell: (iters, w, mean stress)}."""
    from anisotropicfracture_gb300 import models
    from oracle import pyoracle as po
    po.set_threads(1)
    E = np.zeros((3, 3))
    E[0, 0] = 1e-3
    res = {}
    for c in idx:
        n, seeds, table = work[c]
        L = po.rve_level(n)
        Cf = cells.rve_stiffness(n, seeds, table)
        w, st, rc, _ = po.rve_solve(L, models.MAJORMINOR, Cf, E, **CELL_OPTS)
        assert rc == 0
        res[c] = (int(st.iters), w, po.rve_mean_stress(L, models.MAJORMINOR, Cf, E, w))
    return res


def _rank(rank, world, port, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    work = _work()
    sizes = [n ** 3 for n, _, _ in work]
    mine = cells.partition_cells(sizes, world)[rank]
    res = _solve(work, mine)  # this rank's share, no exchange on the data path
    got = [None] * world
    dist.all_gather_object(got, res)  # host-side gather of the results
    if rank == 0:
        merged = {}
        for part in got:
            assert not set(part) & set(merged)
            merged.update(part)
        out_q.put([(c,) + merged[c] for c in sorted(merged)])
    dist.destroy_process_group()


def test_two_gloo_ranks_solve_their_shares_like_one_process():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    rows = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    work = _work()
    ref = _solve(work, range(len(work)))
    assert [r[0] for r in rows] == list(range(len(work)))
    for c, iters, w, sig in rows:
        assert iters == ref[c][0]
        assert np.array_equal(w, ref[c][1])
        assert np.array_equal(sig, ref[c][2])
