"""GPU parity of the energy equation (src/equations/mod_energy.f90) against
the CPU oracle, through the C-ABI.

Per routine, both sides start from the same seeded state (random flow,
temperature and per-cell cp, tc) and the outputs are compared with the
per-routine tolerance of the uvwp parity tests, 1e-12 of each array's scale.
End to end, both sides run in the tight mode (every inner solve, the energy
solve included, to ||r|| <= 1e-13 ||b||) with the energy equation solved after
solve_uvwp in every outer pass, and t, phi, u, v, w, p must agree within 1e-9
relative L2.  In the reference's own solve mode (Gauss-Seidel to a 10x drop on
the oracle, BiCGStab to a 10x drop on the GPU) the converged steady states
must agree within 1e-6.
"""
import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu

RTOL_KERNEL = 1e-12
RTOL_FIELD = 1e-9


def rel_max(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def tight_pair(n, tet, jit, steady):
    z = cfdl.Zone(n, tet, jit, seed=7)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    if steady:
        o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
        g = cfdl.Solver(s, cfdl.steady(solve_mode=1, tight_rtol=1e-13))
    else:
        o.physics_init(oracle_lib.config(rho=5.0, mode=1, tight_rtol=1e-13))
        g = cfdl.Solver(s, cfdl.default_config(rho=5.0, solve_mode=1, tight_rtol=1e-13))
    o.energy_init()
    g.energy_init()
    return s, o, g


def seed_state(o, g, rng):
    nc = o.ne + o.nbf
    vals = {f: rng.standard_normal(nc) for f in ("u", "v", "w", "p", "u0", "v0", "w0")}
    for f in ("gu", "gv", "gw", "gp"):
        vals[f] = rng.standard_normal(3 * nc)
    vals["mip"] = 1e-3 * rng.standard_normal(o.nf)
    vals["mip0"] = 1e-3 * rng.standard_normal(o.nf)
    cp = 1000.0 + 100.0 * rng.uniform(-1, 1, o.ne)
    tc = 5.0 + rng.uniform(-1, 1, o.ne)
    t = 300.0 + 20.0 * rng.standard_normal(nc)
    vals.update(cp=cp, tc=tc, t=t, e=np.concatenate([cp, np.full(o.nbf, 1000.0)]) * t,
                e0=1000.0 * (300.0 + 20.0 * rng.standard_normal(nc)))
    for f, v in vals.items():
        o.set(f, v)
        g.set(f, v)


@pytest.mark.parametrize("n,tet,jit", [(6, False, 0.2), (4, True, 0.0), (3, True, 0.1), (4, "mixed", 0.2),
                                       (4, "prism", 0.1)])
def test_energy_routines_match_oracle(need_gpu, n, tet, jit):
    s, o, g = tight_pair(n, tet, jit, steady=False)
    seed_state(o, g, np.random.default_rng(99))
    # update_boundaries: energy lid / dirichlet0 (exact)
    o.update_boundaries(); g.update_boundaries()
    for f in ("t", "e", "u", "p"):
        assert np.array_equal(g.get(f), o.get(f)), f
    # calc_grad of t and phi
    o.set("gt", o.calc_grad(o.get("t"), o.get("gt")))
    o.set("ge", o.calc_grad(o.get("e"), o.get("ge")))
    g.calc_grad("energy")
    for f in ("gt", "ge"):
        assert rel_max(g.get(f), o.get(f)) < RTOL_KERNEL, f
    # calc_coef_energy
    o.calc_coef_energy(); g.calc_coef_energy()
    for f in ("ap", "anb", "b"):
        assert rel_max(g.get(f), o.get(f)) < RTOL_KERNEL, f
    # solve_energy from the same state (gradients, assembly, tight solve, temperature)
    ost = o.solve_energy()
    gst = g.solve_energy()
    assert gst.status == 0 and gst.it_e > 0 and ost.it_e > 0
    for f in ("e", "t"):
        assert rel_l2(g.get(f), o.get(f)) < 1e-11, f
    assert abs(gst.res_e[0] - ost.res_e[0]) <= 1e-9 * ost.res_e[0]


@pytest.mark.parametrize("n,tet,jit,steady,nout", [
    (8, False, 0.2, True, 30),     # jittered hex, steady under-relaxed SIMPLE
    (6, False, 0.0, False, 12),    # reference physics: rho=5, dt=0.01, phi0 updated every 3 passes
    (4, True, 0.0, True, 20),      # tet split
    (4, "pyramid", 0.1, False, 9),  # six pyramids per cube
])
def test_energy_end_to_end_tight_parity(need_gpu, n, tet, jit, steady, nout):
    s, o, g = tight_pair(n, tet, jit, steady)
    o.run(nout, 3)
    st = g.step(nout, 3)
    assert st.status == 0 and st.it_e > 0
    for f in ("t", "e", "u", "v", "w", "p"):
        a, b = g.get(f)[:o.ne], o.get(f)[:o.ne]
        assert rel_l2(a, b) < RTOL_FIELD, (f, rel_l2(a, b))
    assert g.get("t")[:o.ne].max() > 273.0 + 1e-3     # the lid heats the cavity


def test_energy_converged_default_mode(need_gpu):
    z = cfdl.Zone(6, False, 0.1, seed=21)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=0, mu=0.01))
    o.energy_init()
    o.run(700, ncoef=0)
    for precision in (0, 1, 2, 3):
        g = cfdl.Solver(s, cfdl.steady(mu=0.01, precision=precision))
        g.energy_init()
        g.set_run(700)
        assert g.run(700) == 0
        for f in ("t", "u", "p"):
            err = rel_l2(g.get(f)[:s.ne], o.get(f)[:s.ne])
            assert err < 1e-6, (precision, f, err)
        g.close()


@pytest.mark.parametrize("graph", [True, False])
def test_energy_run_equals_step(need_gpu, graph):
    """cfdl_run (one graph launch with the energy solve as a device-side loop,
    or its eager form) gives the fields of cfdl_step bit for bit."""
    z = cfdl.Zone(6, True, 0.1, seed=3)
    s = cfdl.Setup(z)
    cfg = cfdl.default_config(rho=5.0)
    a, b = cfdl.Solver(s, cfg), cfdl.Solver(s, cfg)
    a.energy_init(); b.energy_init()
    b.set_graph_mode(graph)
    a.step(9, 3)
    b.set_run(9, 3)
    assert b.run(20) == 0
    for f in ("t", "e", "e0", "u", "p", "mip0"):
        assert np.array_equal(a.get(f), b.get(f)), f


def test_energy_batched_run_with_uneven_targets(need_gpu):
    """Two cases with the energy equation in one run graph, one stopping after
    4 outer passes, the other after 11: each equals the same case run alone."""
    zs = [cfdl.Zone(5, False, 0.2, seed=1), cfdl.Zone(4, True, 0.1, seed=2)]
    ss = [cfdl.Setup(z) for z in zs]
    cfg = cfdl.steady()
    bt = cfdl.Batch(ss, [cfg, cfg])
    bt.energy_init()
    ids = bt.ids()
    bt.set_run(4, 0, cid=ids[0])
    bt.set_run(11, 0, cid=ids[1])
    assert bt.run(50) == 0
    for cid, s, n in zip(ids, ss, (4, 11)):
        g = cfdl.Solver(s, cfg)
        g.energy_init()
        g.set_run(n, 0)
        assert g.run(50) == 0
        for f in ("t", "e", "u", "p"):
            assert np.array_equal(bt.case_get(cid, f), g.get(f)), (cid, f)
        g.close()


def test_energy_in_a_mixed_batch(need_gpu):
    """A batch where one case has the energy equation and one has not: each
    case's fields equal, bit for bit, the same case solved alone."""
    za, zb = cfdl.Zone(5, False, 0.2, seed=1), cfdl.Zone(4, True, 0.1, seed=2)
    sa, sb = cfdl.Setup(za), cfdl.Setup(zb)
    cfg = cfdl.default_config(rho=5.0)
    bt = cfdl.Batch([sa], [cfg])
    bt.energy_init(cp=900.0, tc=3.0, t_init=290.0)
    cb = bt.add(sb, cfg)
    bt.step(7, 3)
    ida = bt.ids()[0]
    alone_a = cfdl.Solver(sa, cfg)
    alone_a.energy_init(cp=900.0, tc=3.0, t_init=290.0)
    alone_a.step(7, 3)
    alone_b = cfdl.Solver(sb, cfg)
    alone_b.step(7, 3)
    for f in ("t", "e", "u", "p"):
        assert np.array_equal(bt.case_get(ida, f), alone_a.get(f)), f
    for f in ("u", "v", "p"):
        assert np.array_equal(bt.case_get(cb, f), alone_b.get(f)), f
    with pytest.raises(cfdl.CfdlError):
        bt.case_get(cb, "t")


def test_energy_needs_init(need_gpu):
    s = cfdl.Setup(cfdl.Zone(3))
    g = cfdl.Solver(s, cfdl.default_config())
    with pytest.raises(cfdl.CfdlError):
        g.solve_energy()
    with pytest.raises(cfdl.CfdlError):
        g.energy_init(cp=0.0)
    g.energy_init()
    st = g.solve_energy()
    assert st.status == 0


def test_energy_tile_shapes_and_autotune(need_gpu):
    """The energy solve's tile shape changes only the order of partial sums;
    the autotuner puts the state back exactly."""
    s = cfdl.Setup(cfdl.Zone(7, False, 0.2, seed=4))
    cfg = cfdl.steady()
    ref = None
    for vec in (1, 2, 4, 8):
        g = cfdl.Solver(s, cfg)
        g.energy_init()
        g.set_energy_tile(vec)
        assert g.get_energy_tile() == vec
        g.step(4, 0)
        t = g.get("t")
        if ref is None:
            ref = t
        assert rel_l2(t, ref) < 1e-12, vec
        before = {f: g.get(f) for f in ("t", "e", "u", "p")}
        g.autotune(outer=1)
        assert g.get_energy_tile() in (1, 2, 4, 8)
        for f, v in before.items():
            assert np.array_equal(g.get(f), v), f
        g.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_energy_graph_equals_eager(need_gpu, precision):
    """solve_energy as one graph launch (device-side BiCGStab loop) and as
    eager launches with host polls give the same fields bit for bit (FP64,
    and the FP32 correction form of precision >= 2)."""
    s = cfdl.Setup(cfdl.Zone(6, False, 0.2, seed=8))
    cfg = cfdl.default_config(rho=5.0, precision=precision)
    a, b = cfdl.Solver(s, cfg), cfdl.Solver(s, cfg)
    b.set_graph_mode(False)
    for g in (a, b):
        g.energy_init()
        g.step(5, 3)
    for f in ("t", "e", "e0", "ge", "u", "p"):
        assert np.array_equal(a.get(f), b.get(f)), f
    sa, sb = a.solve_energy(), b.solve_energy()
    assert sa.it_e == sb.it_e and sa.res_e[1] == sb.res_e[1]
    assert np.array_equal(a.get("t"), b.get("t"))
