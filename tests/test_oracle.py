"""Self-checks of the CPU oracle: hand-derivable invariants of the reference
discretisation and the committed golden runs (tests/golden/oracle_runs.json).
CPU only."""
import hashlib
import json
import math
import os

import numpy as np
import pytest

import cfdl
import oracle_lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("n,tet,jit", [(4, False, 0.0), (5, False, 0.2), (3, True, 0.0), (3, "prism", 0.2),
                                       (3, "pyramid", 0.2), (4, "mixed", 0.1)])
def test_grad_exact_for_linear_fields(n, tet, jit):
    """calc_grad is exact for linear fields, halos included: halo centres sit
    on the boundary face centroids (calc_vol_cv_centers.f90:37-42)."""
    z = cfdl.Zone(n, tet, jit, seed=1)
    o = oracle_lib.Oracle(z, n_subdomains=1)
    xc, yc, zc = o.get("xc"), o.get("yc"), o.get("zc")
    phi = 0.3 + 1.5 * xc - 2.0 * yc + 0.7 * zc
    g = o.calc_grad(phi).reshape(-1, 3)[:o.ne]
    assert np.abs(g - np.array([1.5, -2.0, 0.7])).max() < 1e-10


def _fresh(n=5, tet=False, jit=0.2, cfg=None, nsub=4):
    z = cfdl.Zone(n, tet, jit, seed=7)
    o = oracle_lib.Oracle(z, n_subdomains=nsub)
    o.physics_init(cfg or oracle_lib.steady(mode=1))
    return z, o


@pytest.mark.parametrize("kind", ["hex", "prism", "pyramid", "mixed"])
def test_pressure_matrix_symmetric_rows_sum_to_zero(kind):
    z, o = _fresh(tet=kind)
    o.run(3)
    o.update_boundaries()
    o.calc_coef_uvw()
    o.calc_coef_p()
    ap, anb, b = o.get("ap"), o.get("anb"), o.get("b")
    ef1, ef2, idx = o.get_int("ef2nb1"), o.get_int("ef2nb2"), o.get_int("ef2nb_idx")
    A = {}
    for e in range(o.ne):
        row = 0.0
        for h in range(idx[e] - 1, idx[e + 1] - 1):
            enb, lf = ef1[h] >> 5, ef1[h] & 31
            row += anb[h]
            if lf:
                A[(e, enb - 1)] = anb[h]
            else:
                assert anb[h] == 0.0            # boundary d = 0 (mod_uvwp.f90:354-363)
        assert abs(row - ap[e]) <= 1e-15 * ap[e]
    for (i, j), a in A.items():
        assert abs(a - A[(j, i)]) <= 1e-13 * abs(a)
    # b = net inflow: sums to minus the boundary net flux (zero at walls)
    assert abs(b.sum()) < 1e-14 * np.abs(o.get("mip")).sum()


def test_golden_runs():
    with open(os.path.join(ROOT, "tests", "golden", "oracle_runs.json")) as fh:
        gold = json.load(fh)["cases"]
    for key, rec in gold.items():
        kw = dict(rec["config"])
        if kw.get("dt") in ("inf", "Infinity"):
            kw["dt"] = math.inf
        z = cfdl.Zone(rec["n"], rec["tet"], rec["jitter"], seed=rec["seed"])
        o = oracle_lib.Oracle(z, n_subdomains=4)
        o.physics_init(oracle_lib.config(**kw))
        if rec.get("energy"):
            o.energy_init()
        st = o.run(rec["n_outer"], 3)
        assert [st.it_u, st.it_v, st.it_w, st.it_p] == rec["iters"], key
        if rec.get("energy"):
            assert st.it_e == rec["iters_e"], key
        for f, h in rec["hash"].items():
            assert sha(o.get(f)) == h, (key, f)


def test_cavity_fixture_checkpoints_reproduce():
    """The 32^3 cavity fixture (tests/golden/make_cavity_runs.py) is
    reproduced by the oracle here, bit for bit, at its first two checkpoints,
    with the thread count halved: the tight-mode oracle does not depend on
    how many threads run it."""
    with open(os.path.join(ROOT, "tests", "golden", "cavity_runs.json")) as fh:
        rec = json.load(fh)["cases"]["cavity32"]
    z = cfdl.Zone(rec["n"], rec["tet"], rec["jitter"], seed=rec["seed"])
    o = oracle_lib.Oracle(z, n_subdomains=1)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    threads = oracle_lib.num_threads()
    oracle_lib.set_num_threads(max(1, threads // 2))
    try:
        done = 0
        for k in sorted(int(c) for c in rec["checkpoints"])[:2]:
            st = o.run(k - done, 3)
            done = k
            cp = rec["checkpoints"][str(k)]
            assert [st.it_u, st.it_v, st.it_w, st.it_p] == cp["iters"], k
            for f, h in cp["hash"].items():
                assert sha(o.get(f)) == h, (k, f)
    finally:
        oracle_lib.set_num_threads(threads)


def test_reference_pressure_quirk_runs_full_nit():
    """multi_subdomain_solver never resets res_f_tot (mod_solver.f90:175-178),
    so for small residuals the 4-block pressure solve runs all nit sweeps."""
    z, o = _fresh(cfg=oracle_lib.config(rho=5.0, mode=0))
    o.update_boundaries()
    st = o.solve_uvwp()
    assert st.it_p == 100


def test_ref_and_tight_reach_the_same_steady_state():
    """The reference's sweep-based inner solves and the tight Krylov solves are
    two routes to the same discrete steady state."""
    runs = {}
    for mode in (0, 1):
        z, o = _fresh(n=5, cfg=oracle_lib.steady(mode=mode))
        o.run(220)
        runs[mode] = o
    for f in ("u", "v", "w"):
        a, b = runs[0].get(f)[:runs[0].ne], runs[1].get(f)[:runs[1].ne]
        assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b), f


def test_mass_conservation_improves():
    z, o = _fresh(n=6, cfg=oracle_lib.steady(mode=1))
    o.run(1)
    o.update_boundaries(); o.calc_coef_uvw(); o.calc_mip(True); o.calc_coef_p()
    b0 = np.linalg.norm(o.get("b"))
    o.run(40)
    o.update_boundaries(); o.calc_coef_uvw(); o.calc_mip(True); o.calc_coef_p()
    assert np.linalg.norm(o.get("b")) < 0.2 * b0


@pytest.mark.parametrize("kind,jit", [(False, 0.2), (True, 0.1), ("prism", 0.2), ("mixed", 0.2)])
def test_rhie_chow_term_vanishes_for_linear_pressure(kind, jit):
    """calc_mip's pressure-smoothing term -rho A d_ip/(dr.n) (p_nb - p_P -
    gp_ip.dr) (mod_uvwp.f90:438-490) is zero when p is linear and gp its exact
    gradient, on any mesh: the fluxes with and without the term agree to
    rounding, and differ at O(1) for a non-linear p."""
    z = cfdl.Zone(5, kind, jit, seed=7)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1))       # dt = inf: no transient term
    o.run(3)
    o.update_boundaries()
    o.calc_coef_uvw()                                # d = vol / ap, the term's weight
    assert np.abs(o.get("d")).max() > 0
    xc, yc, zc = o.get("xc"), o.get("yc"), o.get("zc")
    p = 0.4 + 2.0 * xc - 1.0 * yc + 3.0 * zc
    o.set("p", p)
    o.set("gp", np.tile([2.0, -1.0, 3.0], len(xc)))
    o.calc_mip(False)
    plain = o.get("mip").copy()
    o.calc_mip(True)
    assert np.abs(o.get("mip") - plain).max() < 1e-13 * np.abs(plain).max()
    o.set("p", p + 0.5 * xc ** 2)
    o.calc_mip(True)
    assert np.abs(o.get("mip") - plain).max() > 1e-2 * np.abs(plain).max()


def test_cavity_is_mirror_symmetric_across_the_lid_direction():
    """The lid moves in x on the top face, so on an unjittered hex mesh the
    discrete solution is symmetric under y -> 1 - y with v -> -v; the two
    other reflections are not symmetries of the flow."""
    z = cfdl.Zone(6, False, 0.0, seed=1)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    o.run(15)
    ne = o.ne
    xyz = np.stack([o.get(c)[:ne] for c in ("xc", "yc", "zc")], axis=1)
    where = {tuple(np.round(r, 9)): i for i, r in enumerate(xyz)}
    u, v, w, p = (o.get(f)[:ne] for f in "uvwp")
    scale = np.abs(u).max()
    for axis in range(3):
        r = xyz.copy()
        r[:, axis] = 1.0 - r[:, axis]
        m = np.array([where[tuple(np.round(q, 9))] for q in r])
        sign = [1.0, 1.0, 1.0]
        sign[axis] = -1.0
        err = max(np.abs(f - s * f[m]).max() for f, s in zip((u, v, w), sign)) / scale
        if axis == 1:
            assert err < 1e-12
            assert np.abs(p - p[m]).max() < 1e-12 * np.abs(p).max()
        else:
            assert err > 1e-2


@pytest.mark.parametrize("kind,jit", [(False, 0.2), (True, 0.1), ("pyramid", 0.1)])
def test_corrected_fluxes_satisfy_continuity(kind, jit):
    """calc_coef_p's face coefficient rho_ip dc_ip A/(dr.n) (mod_uvwp.f90:289-368)
    is the one update_uvwp corrects mip with (:370-436): after a tight
    pressure-correction solve, every cell's net face flux is the solve's
    residual, ~1e-13 of the imbalance before the correction."""
    z = cfdl.Zone(5, kind, jit, seed=7)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    o.run(4)
    o.update_boundaries(); o.calc_coef_uvw(); o.calc_mip(True); o.calc_coef_p()
    b0 = o.get("b").copy()
    o.solve_pc(); o.adjust_pc(); o.update_uvwp()
    mip = o.get("mip")
    ef2, idx = o.get_int("ef2nb2"), o.get_int("ef2nb_idx")
    owner = np.repeat(np.arange(o.ne), np.diff(idx))
    net = np.zeros(o.ne)
    np.add.at(net, owner, np.sign(ef2) * mip[np.abs(ef2) - 1])
    assert np.linalg.norm(b0) > 1e-3 * np.abs(mip).sum() / o.ne ** 0.5
    assert np.linalg.norm(net) < 1e-11 * np.linalg.norm(b0)


@pytest.mark.parametrize("kind", [False, True, "pyramid"])
def test_momentum_matrix_is_an_m_matrix(kind):
    """calc_coef_uvw (mod_uvwp.f90:161-286): upwind convection max(-mip, 0)
    plus diffusion mu A/ds gives non-negative neighbour coefficients, and the
    under-relaxed diagonal ap/alpha_u exceeds the row's neighbour sum."""
    z = cfdl.Zone(5, kind, 0.2, seed=3)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1))
    o.run(5)
    o.update_boundaries()
    o.calc_coef_uvw()
    ap, anb = o.get("ap"), o.get("anb")
    idx = o.get_int("ef2nb_idx")
    assert anb.min() >= 0.0
    rows = np.add.reduceat(anb, idx[:-1] - 1)
    assert (ap - rows > 0).all()


# ---- energy equation (src/equations/mod_energy.f90) ----------------------------

def test_energy_pure_diffusion_matrix():
    """With no flow and zero gradients, calc_coef_energy is pure diffusion:
    symmetric interior coefficients tc/cp*area/(dr.n), wall coefficients
    tc*area/ds/cp on the boundary half-faces, ap = sum of the row's anb
    (steady: ap0 = 0) and b = 0."""
    z, o = _fresh(n=4, jit=0.2, cfg=oracle_lib.steady(mode=1))
    o.energy_init(cp=800.0, tc=4.0)
    o.update_boundaries()
    assert np.all(o.get("mip") == 0.0)
    o.calc_coef_energy()
    ap, anb, b = o.get("ap"), o.get("anb"), o.get("b")
    ef1, idx = o.get_int("ef2nb1"), o.get_int("ef2nb_idx")
    A = {}
    nwall = 0
    for e in range(o.ne):
        row = 0.0
        for h in range(idx[e] - 1, idx[e + 1] - 1):
            enb, lf = ef1[h] >> 5, ef1[h] & 31
            row += anb[h]
            assert anb[h] > 0.0
            if lf:
                A[(e, enb - 1)] = anb[h]
            else:
                nwall += 1
        assert abs(row - ap[e]) <= 1e-14 * ap[e]
    assert nwall == o.nbf
    for (i, j), a in A.items():
        assert abs(a - A[(j, i)]) <= 1e-13 * a
    assert np.all(b == 0.0)
    # on the undistorted mesh every coefficient is tc/cp * h (area h^2, distance h; walls h/2)
    z, o = _fresh(n=4, jit=0.0, cfg=oracle_lib.steady(mode=1))
    o.energy_init(cp=800.0, tc=4.0)
    o.update_boundaries()
    o.calc_coef_energy()
    anb = o.get("anb")
    h = 1.0 / 4
    vals = np.unique(np.round(anb / (4.0 / 800.0 * h), 12))
    assert set(vals.tolist()) <= {1.0, 2.0}, vals


def test_energy_uniform_temperature_is_kept():
    """Walls and interior at one temperature stay there while the flow
    develops: the advection is conservative (b carries sumf*phi) and the
    fluxes are divergence-free to the tight pressure tolerance."""
    z, o = _fresh(n=5, jit=0.1, cfg=oracle_lib.config(mode=1))
    o.energy_init(t_init=300.0, t_lid=300.0, t_wall=300.0)
    for _ in range(6):
        o.update_boundaries()
        o.solve_uvwp()
        st = o.solve_energy()
    assert np.abs(o.get("t")[:o.ne] - 300.0).max() < 1e-8
    assert np.abs(o.get("u")).max() > 1e-3


def test_energy_ref_and_tight_reach_the_same_steady_state():
    """Gauss-Seidel (solve_gs 'e') and the tight BiCGStab energy solves reach
    the same steady temperature; the hot lid warms the cavity."""
    runs = {}
    for mode in (0, 1):
        z, o = _fresh(n=4, cfg=oracle_lib.steady(mode=mode))
        o.energy_init()
        o.run(260)
        runs[mode] = o
    a, b = runs[0].get("t")[:runs[0].ne], runs[1].get("t")[:runs[1].ne]
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
    assert b.min() > 273.0 - 1e-6 and b.max() < 373.0 and b.max() > 280.0


@pytest.mark.parametrize("kind,jit", [(False, 0.0), (False, 0.2), (True, 0.0)])
def test_energy_discrete_maximum_principle(kind, jit):
    """Upwind convection plus diffusion gives calc_coef_energy an M-matrix
    (mod_energy.f90:82-169), so the temperature stays between the wall
    temperatures (273 K walls, 373 K lid) at every outer pass."""
    z = cfdl.Zone(6, kind, jit, seed=3)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    o.energy_init(t_init=300.0)
    for _ in range(4):
        o.run(10)
        t = o.get("t")[:o.ne]
        assert t.min() >= 273.0 - 1e-9 and t.max() <= 373.0 + 1e-9
    assert t.max() > 300.0 and t.min() < 300.0      # heated by the lid, cooled by the walls
