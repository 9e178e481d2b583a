"""Batches and runs: many cases in one context, many outer iterations per launch.

A case's arithmetic must not depend on the other cases that share its
launches: every kernel works per case (tiles never span two cases), every
reduction sums a case's own tile partials in a fixed order, and a case whose
run is over is skipped by every kernel.  So a case solved in a batch, or
joining a batch later, gives bit-for-bit the fields it gives alone; these
tests check exactly that, and check a batched case against the oracle in the
tight mode (1e-9 relative L2, the end-to-end parity target).
"""
import math

import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "p", "mip")


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def case_setup(n, tet, jit, seed):
    return cfdl.Setup(cfdl.Zone(n, tet, jit, seed=seed))


def cavity_cfg(re, precision=0, **kw):
    # unit cube, lid speed 1, rho 1: Re = 1/mu
    return cfdl.steady(mu=1.0 / re, precision=precision, **kw)


SPECS = [(8, False, 0.2, 1, 100.0), (5, True, 0.1, 2, 400.0), (10, False, 0.0, 3, 30.0)]


def alone(spec, n_outer, precision=0, ncoef=0, graph=True):
    n, tet, jit, seed, re = spec
    g = cfdl.Solver(case_setup(n, tet, jit, seed), cavity_cfg(re, precision))
    g.set_graph_mode(graph)
    g.set_run(n_outer, ncoef)
    assert g.run(n_outer + 5) == 0
    out = {f: g.get(f) for f in FIELDS}
    g.close()
    return out


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_batch_equals_alone_bitwise(need_gpu, precision):
    setups = [case_setup(*s[:4]) for s in SPECS]
    cfgs = [cavity_cfg(s[4], precision) for s in SPECS]
    b = cfdl.Batch(setups, cfgs)
    b.set_run(12)
    assert b.run(100) == 0
    for cid, spec in enumerate(SPECS):
        ref = alone(spec, 12, precision)
        st = b.case_stats(cid)
        assert st.outer_done == 12 and st.run_left == 0
        for f in FIELDS:
            assert np.array_equal(b.case_get(cid, f), ref[f]), (cid, f)
    b.close()


def test_uneven_targets_and_budget(need_gpu):
    setups = [case_setup(*s[:4]) for s in SPECS]
    b = cfdl.Batch(setups, [cavity_cfg(s[4]) for s in SPECS])
    targets = [5, 12, 8]
    for cid, t in enumerate(targets):
        b.set_run(t, cid=cid)
    # a budget of 7 passes: case 0 finishes, the others are left running
    assert b.run(7) == 2
    assert [b.case_stats(c).outer_done for c in range(3)] == [5, 7, 7]
    assert b.run(100) == 0
    for cid, spec in enumerate(SPECS):
        ref = alone(spec, targets[cid])
        for f in FIELDS:
            assert np.array_equal(b.case_get(cid, f), ref[f]), (cid, f)
    b.close()


def test_run_equals_step_and_eager(need_gpu):
    spec = SPECS[0]
    n, tet, jit, seed, re = spec
    cfg = cfdl.default_config(rho=5.0)   # transient: update_time every 3 iterations
    g = cfdl.Solver(case_setup(n, tet, jit, seed), cfg)
    g.step(9, ncoef=3)
    ref = {f: g.get(f) for f in FIELDS + ("u0", "mip0")}
    g.close()
    for graph in (True, False):
        h = cfdl.Solver(case_setup(n, tet, jit, seed), cfg)
        h.set_graph_mode(graph)
        h.set_run(9, ncoef=3)
        assert h.run(9) == 0
        for f in FIELDS + ("u0", "mip0"):
            assert np.array_equal(h.get(f), ref[f]), (graph, f)
        h.close()


def test_cases_join_and_leave(need_gpu):
    b = cfdl.Batch([case_setup(*SPECS[0][:4])], [cavity_cfg(SPECS[0][4])])
    b.set_run(10, cid=0)
    assert b.run(4) == 1
    late = b.add(case_setup(*SPECS[1][:4]), cavity_cfg(SPECS[1][4]))
    b.set_run(6, cid=late)
    assert b.run(100) == 0
    assert b.case_stats(0).outer_done == 10 and b.case_stats(late).outer_done == 6
    ref0, ref1 = alone(SPECS[0], 10), alone(SPECS[1], 6)
    for f in FIELDS:
        assert np.array_equal(b.case_get(0, f), ref0[f]), f
        assert np.array_equal(b.case_get(late, f), ref1[f]), f
    b.remove(0)
    assert b.ids() == [late]
    b.set_run(2, cid=late)
    assert b.run(10) == 0
    ne, nbytes = b.case_info(late)
    assert ne == 6 * 5 ** 3 and nbytes > 0
    assert nbytes <= cfdl.case_bytes_estimate(ne, b._sizes[late][1], b._sizes[late][2])
    b.close()


def test_convergence_stop(need_gpu):
    spec = SPECS[2]
    b = cfdl.Batch([case_setup(*spec[:4])], [cavity_cfg(spec[4])])
    b.set_run(2000, conv_tol=1e-6)
    assert b.run(2000) == 0
    st = b.case_stats(0)
    assert st.converged == 1 and st.mass_ratio <= 1e-6 and st.outer_done < 2000
    b.close()


def test_batched_case_matches_oracle(need_gpu):
    """A case inside a tight-mode batch against the oracle run alone."""
    n, tet, jit, seed, re = 6, True, 0.1, 5, 100.0
    z = cfdl.Zone(n, tet, jit, seed=seed)
    s = cfdl.Setup(z)
    other = case_setup(7, False, 0.2, 9)
    gc = cavity_cfg(re, solve_mode=1, tight_rtol=1e-13)
    b = cfdl.Batch([other, s], [cavity_cfg(50.0, solve_mode=1, tight_rtol=1e-13), gc])
    b.set_run(8)
    assert b.run(8) == 0
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13, mu=1.0 / re))
    o.run(8, ncoef=0)
    for f in ("u", "v", "w", "p"):
        assert rel_l2(b.case_get(1, f), o.get(f)) < 1e-9, f
    b.close()
    o.close()


def test_form_mismatch_rejected(need_gpu):
    s = case_setup(4, False, 0.0, 1)
    with pytest.raises(cfdl.CfdlError):
        cfdl.Batch([s, s], [cavity_cfg(100.0, 0), cavity_cfg(100.0, 1)])
    b = cfdl.Batch([s], [cavity_cfg(100.0, 0)])
    with pytest.raises(cfdl.CfdlError):
        b.add(s, cavity_cfg(100.0, 1))
    with pytest.raises(cfdl.CfdlError):
        b.remove(0)          # the last case stays
    b.close()
    with pytest.raises(cfdl.CfdlError):   # FP32 momentum corrections need the 10x-drop stopping rule
        cfdl.Solver(s, cavity_cfg(100.0, 2, solve_mode=1))


def test_nonfinite_case_stops_alone(need_gpu):
    """A case whose state turns non-finite stops with CFDL_ERR_NONFINITE;
    the other cases of the batch run on, unaffected (failure injected on the
    host: a NaN written into one cell's velocity)."""
    setups = [case_setup(*s[:4]) for s in SPECS[:2]]
    b = cfdl.Batch(setups, [cavity_cfg(s[4]) for s in SPECS[:2]])
    u = b.case_get(1, "u")
    u[3] = float("nan")
    b.case_set(1, "u", u)
    b.set_run(6)
    assert b.run(6) == 0
    bad, good = b.case_stats(1), b.case_stats(0)
    assert bad.status == cfdl.CFDL_ERR_NONFINITE and bad.run_left == 0 and bad.outer_done == 1
    assert good.status == 0 and good.outer_done == 6
    ref = alone(SPECS[0], 6)
    for f in FIELDS:
        assert np.array_equal(b.case_get(0, f), ref[f]), f
    b.close()
    g = cfdl.Solver(case_setup(*SPECS[1][:4]), cavity_cfg(SPECS[1][4]))
    v = g.get("v")
    v[0] = float("inf")
    g.set("v", v)
    with pytest.raises(cfdl.CfdlError) as ei:
        g.solve_uvwp()
    assert ei.value.status == cfdl.CFDL_ERR_NONFINITE
    g.close()
