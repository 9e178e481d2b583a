"""The serving loop: continuous batching of cavity-solve requests.

Requests arriving while others are resident join the running batch between
launches.  Each result must be the same alone and in the mix: the fields a
request gets from the server equal, bit for bit, the fields of the same case
solved alone through the batch API with the same settings.
"""
import math
import time

import numpy as np
import pytest

import cfdl

pytestmark = pytest.mark.gpu

REQS = [dict(n=8, tet=False, jitter=0.2, seed=1, re=100.0),
        dict(n=5, tet=True, jitter=0.1, seed=2, re=400.0),
        dict(n=10, tet=False, jitter=0.0, seed=3, re=30.0),
        dict(n=6, tet=True, jitter=0.2, seed=4, re=1000.0),
        dict(n=7, tet=False, jitter=0.1, seed=5, re=10.0),
        dict(n=4, tet=True, jitter=0.0, seed=6, re=200.0)]


def solve_alone(req, conv_tol, max_outer, precision, tile=4):
    z = cfdl.Zone(req["n"], req["tet"], req["jitter"], seed=req["seed"])
    cfg = cfdl.steady(mu=1.0 / req["re"], precision=precision)
    b = cfdl.Batch([cfdl.Setup(z)], [cfg])
    b.set_tile(tile)
    b.set_run(max_outer, 0, conv_tol)
    assert b.run(max_outer + 1) == 0
    st = b.case_stats(0)
    out = {f: b.case_get(0, f) for f in ("u", "v", "w", "p")}
    b.close()
    return out, st


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_results_same_alone_and_in_mix(need_gpu, precision):
    conv_tol, max_outer = 1e-4, 80
    srv = cfdl.Server(precision=precision, chunk=7, max_cases=4, prep_threads=3, hbm_budget=8e9, hbm_reserve=1e9)
    ids = []
    for r in REQS[:3]:
        ids.append(srv.submit(conv_tol=conv_tol, max_outer=max_outer, keep_fields=True, **r))
    first = srv.poll(wait_s=60.0, max_results=1)   # the others arrive while these run
    for r in REQS[3:]:
        ids.append(srv.submit(conv_tol=conv_tol, max_outer=max_outer, keep_fields=True, **r))
    srv.drain(timeout_s=300.0)
    results = {r.id: r for r in first + srv.poll(max_results=64)}
    assert sorted(results) == sorted(ids)
    for rid, req in zip(ids, REQS):
        res = results[rid]
        assert res.status == 0
        assert res.t_submit <= res.t_ready <= res.t_admit <= res.t_done
        ref, st = solve_alone(req, conv_tol, max_outer, precision)
        assert res.outer_done == st.outer_done and res.converged == st.converged
        for f in ("u", "v", "w", "p"):
            assert np.array_equal(srv.fields(rid, f), ref[f]), (rid, f)
    info = srv.info()
    assert info["done"] == len(REQS) and info["queued"] == 0 and info["cell_iters"] > 0
    srv.close()


def test_admission_respects_the_budget(need_gpu):
    # a budget below two cases: the second is admitted only after the first retires
    big = dict(n=12, tet=False, jitter=0.1, seed=9, re=100.0)
    est = cfdl.case_bytes_estimate(12 ** 3, 3 * 12 ** 3 + 3 * 12 ** 2, 6 * 12 ** 2)
    srv = cfdl.Server(chunk=5, hbm_budget=1.5 * est, hbm_reserve=0.0, prep_threads=2)
    a = srv.submit(conv_tol=0.0, max_outer=20, **big)
    b = srv.submit(conv_tol=0.0, max_outer=20, **big)
    srv.drain(timeout_s=300.0)
    res = {r.id: r for r in srv.poll(max_results=8)}
    assert res[a].status == 0 and res[b].status == 0
    assert res[a].outer_done == 20 and res[b].outer_done == 20
    # one resident at a time, whichever was prepared first
    assert res[b].t_admit >= res[a].t_done or res[a].t_admit >= res[b].t_done
    srv.close()


def test_invalid_requests_rejected(need_gpu):
    srv = cfdl.Server(prep_threads=1)
    with pytest.raises(cfdl.CfdlError):
        srv.submit(n=0)
    with pytest.raises(cfdl.CfdlError):
        srv.submit(n=4, re=-1.0)
    srv.close()
