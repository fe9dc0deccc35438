"""The serving loop (ae_server_*) on the GPU: continuous batching of cell homogenisation requests.

Each request's result is the same alone and in a mix whose membership changes while it runs,
bit for bit (tolerance 0): its arithmetic never depends on the other requests.  Results also equal
the batch entry point's for the same cell.  Admission respects the device-memory budget."""
import time

import numpy as np
import pytest

from anisotropicfracture_gb300 import _lib, cells, models

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SOLVER = dict(max_fmg_iter=0, nu1=2, nu2=2, sweeps=2, bottom=1, bottom_max_iter=200, bottom_reltol=1e-4, nuf=8,
              max_iter=100)


def _req(n, ngr, seed, nload=6):
    seeds, table = cells.rve_grains(n, ngr, seed)
    return n, cells.unit_strains()[:nload], seeds, table


@pytest.mark.parametrize("precision", [1, 0])
def test_each_result_is_the_same_alone_and_in_the_mix(precision):
    probe = _req(16, 8, 101)
    S = cells.CellServer(keep_solution=True, precision=precision, inner_cycles=2, **SOLVER)
    t = S.submit(probe[0], probe[1], probe[2], probe[3])
    alone = S.wait(t, 120.0)
    S.close()
    assert alone["status"] == 0
    S = cells.CellServer(keep_solution=True, precision=precision, inner_cycles=2, **SOLVER)
    others = [_req(24, 10, 102), _req(32, 12, 103, 3), _req(8, 4, 104, 2)]
    early = [S.submit(*r) for r in others[:2]]
    # wait until the first requests are on the device, then add the probe and one more
    for _ in range(2000):
        if S.poll(early[0])["status"] in (cells.CellServer.RUNNING, 0):
            break
        time.sleep(0.001)
    tp = S.submit(probe[0], probe[1], probe[2], probe[3])
    late = S.submit(*others[2])
    res = {t_: S.wait(t_, 300.0) for t_ in early + [tp, late]}
    for r in res.values():
        assert r["status"] == 0
        assert all(s["converged"] for s in r["stats"])
    mix = res[tp]
    assert np.array_equal(mix["w"], alone["w"])
    for a, b in zip(alone["stats"], mix["stats"]):
        assert a["iters"] == b["iters"]
        assert np.array_equal(a["mean_stress"], b["mean_stress"])
    st = S.stats()
    assert st["completed"] == 4 and st["failed"] == 0 and st["queued"] == 0 and st["hbm_used"] == 0
    S.close()


def test_server_matches_the_batch_entry_point():
    n, loads, seeds, table = _req(16, 6, 201, 2)
    S = cells.CellServer(keep_solution=True, precision=1, inner_cycles=2, **SOLVER)
    r = S.wait(S.submit(n, loads, seeds, table), 120.0)
    S.close()
    B = cells.CellBatch([(n, 2)])
    B.set_grains(0, seeds, table)
    for k, E in enumerate(loads):
        B.set_load(k, E)
    B.prepare()
    st, rc = B.solve(precision=1, inner_cycles=2, **SOLVER)
    for k in range(2):
        assert np.array_equal(B.solution(k), r["w"][k])
        assert np.array_equal(st[k]["mean_stress"], r["stats"][k]["mean_stress"])


def test_admission_waits_for_device_memory():
    reqs = [_req(16, 6, 300 + i, 2) for i in range(3)]
    need = cells.plan_bytes(16, 2)
    S = cells.CellServer(hbm_budget_bytes=int(1.5 * need), precision=1, inner_cycles=2, **SOLVER)
    ts = [S.submit(*r) for r in reqs]
    res = [S.wait(t, 300.0) for t in ts]
    assert all(r["status"] == 0 for r in res)
    # one request fits at a time: each is admitted only after the previous one finished
    for a, b in zip(res, res[1:]):
        assert b["t_admit"] >= a["t_done"]
    with pytest.raises(_lib.AeError) as e:
        S.submit(*_req(32, 6, 399, 2))
    assert e.value.code == _lib.AE_ERR_OOM
    S.close()


def test_requests_with_a_full_field_and_release():
    n = 12
    seeds, table = cells.rve_grains(n, 5, 401)
    Cf = cells.rve_stiffness(n, seeds, table)
    S = cells.CellServer(keep_solution=True, precision=0, **SOLVER)
    ta = S.submit(n, cells.unit_strains()[:1], field=Cf)
    tb = S.submit(n, cells.unit_strains()[:1], seeds=seeds, table=table)
    ra, rb = S.wait(ta, 120.0), S.wait(tb, 120.0)
    assert ra["status"] == 0 and np.array_equal(ra["w"], rb["w"])
    S.release(ta)
    with pytest.raises(_lib.AeError):
        S.poll(ta)
    S.close()
