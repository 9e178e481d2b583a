"""GPU parity: libcfdgpu (through its C-ABI) against the CPU oracle.

Per routine, both sides start from the same seeded state and the outputs are
compared with tolerance RTOL_KERNEL relative to each array's scale: the GPU
computes every face term once per face from precomputed geometry, so values
differ from the reference's per-half-face arithmetic by a few roundings.
End to end, both sides run in the tight mode (every inner solve to
||r|| <= 1e-13 ||b||) and the u, v, w, p fields must agree within 1e-9
relative L2 after the same number of outer iterations (the target the
reference comparison is stated in).
"""
import ctypes as C
import math

import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu

RTOL_KERNEL = 1e-12      # per routine, max-norm relative to the array scale
RTOL_FIELD = 1e-9        # end to end, relative L2 after the same iteration count


def rel_max(a, b):
    s = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / s


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make_pair(n=6, tet=False, jit=0.2, seed=7, gpu_cfg=None, or_cfg=None):
    z = cfdl.Zone(n, tet, jit, seed=seed)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(or_cfg)
    g = cfdl.Solver(s, gpu_cfg)
    return z, s, o, g


def tight_pair(n=6, tet=False, jit=0.2, steady=True, **kw):
    if steady:
        gc = cfdl.steady(solve_mode=1, tight_rtol=1e-13, **kw)
        oc = oracle_lib.steady(mode=1, tight_rtol=1e-13)
    else:
        gc = cfdl.default_config(rho=5.0, solve_mode=1, tight_rtol=1e-13, **kw)
        oc = oracle_lib.config(rho=5.0, mode=1, tight_rtol=1e-13)
    return make_pair(n, tet, jit, gpu_cfg=gc, or_cfg=oc)


def seed_state(o, g, rng):
    """Same random state on both sides (reference layouts)."""
    nc = o.ne + o.nbf
    vals = {}
    for f in ("u", "v", "w", "p", "u0", "v0", "w0"):
        vals[f] = rng.standard_normal(nc)
    for f in ("gu", "gv", "gw", "gp"):
        vals[f] = rng.standard_normal(3 * nc)
    vals["mip"] = 1e-3 * rng.standard_normal(o.nf)
    vals["mip0"] = 1e-3 * rng.standard_normal(o.nf)
    for f, v in vals.items():
        o.set(f, v)
        g.set(f, v)
    return vals


@pytest.mark.parametrize("n,tet,jit", [(6, False, 0.2), (4, True, 0.0), (3, True, 0.1), (4, "prism", 0.2),
                                       (3, "pyramid", 0.1), (4, "mixed", 0.2)])
def test_routines_match_oracle(need_gpu, n, tet, jit):
    z, s, o, g = tight_pair(n, tet, jit, steady=False)
    rng = np.random.default_rng(1234)
    seed_state(o, g, rng)
    # update_boundaries
    o.update_boundaries(); g.update_boundaries()
    for f in ("u", "v", "w", "p", "mip"):
        assert np.array_equal(g.get(f), o.get(f)), f
    # calc_grad (u, v, w fused and single)
    for f in ("u", "v", "w"):
        ref = o.calc_grad(o.get(f), o.get("g" + f))
        o.set("g" + f, ref)
    g.calc_grad("uvw")
    for f in ("gu", "gv", "gw"):
        assert rel_max(g.get(f), o.get(f)) < RTOL_KERNEL, f
    # calc_coef_uvw
    o.calc_coef_uvw(); g.calc_coef_uvw()
    for f in ("ap", "anb", "bu", "bv", "bw", "d", "dc"):
        assert rel_max(g.get(f), o.get(f)) < RTOL_KERNEL, f
    # calc_mip with Rhie-Chow
    o.calc_mip(True); g.calc_mip(True)
    assert rel_max(g.get("mip"), o.get("mip")) < RTOL_KERNEL
    # calc_coef_p
    o.calc_coef_p(); g.calc_coef_p()
    for f in ("ap", "anb", "b"):
        assert rel_max(g.get(f), o.get(f)) < RTOL_KERNEL, f
    # pressure-correction solve (tight), adjust_pc, grad(pc), update_uvwp
    o.solve_pc(); st = g.solve_pc()
    assert st.status == 0
    o.adjust_pc(); g.adjust_pc()
    assert rel_max(g.get("phic"), o.get("phic")) < 1e-9
    pc = o.get("phic")
    o.set("gpc", o.calc_grad(pc, o.get("gpc")))
    g.calc_grad("pc")
    assert rel_max(g.get("gpc"), o.get("gpc")) < 1e-9
    o.update_uvwp(); g.update_uvwp()
    for f in ("p", "gp", "mip"):
        assert rel_max(g.get(f), o.get(f)) < 1e-9, f


def test_momentum_solve_tight(need_gpu):
    z, s, o, g = tight_pair(6, False, 0.2, steady=True)
    rng = np.random.default_rng(5)
    seed_state(o, g, rng)
    o.update_boundaries(); g.update_boundaries()
    o.calc_coef_uvw(); g.calc_coef_uvw()
    for comp in range(3):
        o.solve_momentum(comp)
    st = g.solve_momentum()
    assert st.status == 0
    for f in ("u", "v", "w"):
        assert rel_l2(g.get(f), o.get(f)) < 1e-11, f


@pytest.mark.parametrize("n,tet,jit,steady,nout", [
    (8, False, 0.2, True, 40),     # jittered hex, steady under-relaxed SIMPLE
    (6, False, 0.0, False, 12),    # reference physics: pseudo-transient, rho=5, dt=0.01
    (4, True, 0.0, True, 25),      # tet split
    (5, "prism", 0.2, True, 20),   # two prisms per cube (W = 5, triangle and quad faces)
    (3, "pyramid", 0.1, False, 10),  # six pyramids per cube
    (5, "mixed", 0.2, True, 20),   # hex and pyramid cubes: ELL rows of 6 and 5 slots
])
def test_end_to_end_tight_parity(need_gpu, n, tet, jit, steady, nout):
    z, s, o, g = tight_pair(n, tet, jit, steady=steady)
    o.run(nout, 3)
    st = g.step(nout, 3)
    assert st.status == 0
    for f in ("u", "v", "w", "p"):
        a, b = g.get(f)[:o.ne], o.get(f)[:o.ne]
        assert rel_l2(a, b) < RTOL_FIELD, (f, rel_l2(a, b))


@pytest.mark.parametrize("precond,precision", [(1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("n,tet,jit", [(8, False, 0.2), (4, True, 0.0), (4, False, 0.0), (5, "mixed", 0.1)])
def test_pressure_solver_forms_tight_parity(need_gpu, n, tet, jit, precond, precision):
    """AMG-preconditioned CG and the mixed-precision form (FP32 inner PCG, FP64
    residual and refinement), tight, against the oracle after 20 iterations."""
    z, s, o, g = tight_pair(n, tet, jit, steady=True, precond=precond, precision=precision)
    o.run(20, 3)
    st = g.step(20, 3)
    assert st.status == 0
    for f in ("u", "v", "w", "p"):
        a, b = g.get(f)[:o.ne], o.get(f)[:o.ne]
        assert rel_l2(a, b) < RTOL_FIELD, (f, rel_l2(a, b))


@pytest.mark.parametrize("precond,precision", [(1, 0), (1, 1)])
def test_amg_default_mode_reaches_steady_state(need_gpu, precond, precision):
    """Production stopping rule with the AMG pressure solve, FP64 and mixed:
    the steady state is the oracle's within 1e-6 relative L2."""
    z = cfdl.Zone(10, False, 0.2, seed=7)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1))
    o.run(400)
    g = cfdl.Solver(s, cfdl.steady(solve_mode=0, precond=precond, precision=precision))
    g.step(400)
    for f in ("u", "v", "w"):
        assert rel_l2(g.get(f)[:o.ne], o.get(f)[:o.ne]) < 1e-6, f
    # this mesh's neighbours fit in 16-bit offsets, so the mixed form's FP32
    # mesh-level kernels ran on them; the FP64 form reads int32 indices
    assert cfdl.lib().cfdl_amg_index_bytes(g._h) == (2 if precision >= 1 else 4)


def test_default_mode_reaches_oracle_steady_state(need_gpu):
    """The production mode (each inner solve to a 10x residual drop, as the
    reference) converges to the same discrete steady state as the oracle."""
    z = cfdl.Zone(6, False, 0.2, seed=7)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1))
    o.run(300)
    g = cfdl.Solver(s, cfdl.steady(solve_mode=0))
    g.step(300)
    for f in ("u", "v", "w"):
        assert rel_l2(g.get(f)[:o.ne], o.get(f)[:o.ne]) < 1e-5, f


def test_deterministic_and_launches_counted(need_gpu):
    z = cfdl.Zone(10, False, 0.2, seed=9)
    s = cfdl.Setup(z)
    res = []
    for _ in range(2):
        g = cfdl.Solver(s, cfdl.steady())
        n0 = g.launch_count()
        g.step(5)
        assert g.launch_count() > n0
        res.append([g.get(f) for f in ("u", "v", "w", "p", "mip")])
        g.close()
    for a, b in zip(*res):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precond,precision,mode", [(0, 0, 0), (1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1)])
def test_graph_equals_eager(need_gpu, precond, precision, mode):
    """solve_uvwp as one CUDA graph with device-side loops runs the same
    kernels with the same device-side decisions as the host-polled launches,
    so the fields agree bit for bit."""
    z = cfdl.Zone(12, False, 0.2, seed=5)
    s = cfdl.Setup(z)
    out = []
    for graph in (True, False):
        g = cfdl.Solver(s, cfdl.steady(solve_mode=mode, precond=precond, precision=precision))
        g.set_graph_mode(graph)
        st = g.step(7, 3)
        assert st.status == 0
        out.append([g.get(f) for f in ("u", "v", "w", "p", "mip", "gp")])
        g.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_host_dropin_matches_resident(need_gpu):
    """cfdl_solve_uvwp_host (host arrays in and out) equals the resident path."""
    import ctypes as C
    z = cfdl.Zone(6, False, 0.1, seed=2)
    s = cfdl.Setup(z)
    g1 = cfdl.Solver(s, cfdl.steady())
    g2 = cfdl.Solver(s, cfdl.steady())
    nc, nf = s.ne + s.nbf, s.nf
    host = {f: np.zeros(nc) for f in ("u", "v", "w", "p", "u0", "v0", "w0")}
    host.update({f: np.zeros(3 * nc) for f in ("gu", "gv", "gw", "gp", "gpc")})
    host.update({"mip": g2.get("mip"), "mip0": g2.get("mip0")})
    fl = cfdl.Fields(**{k: v.ctypes.data_as(C.c_void_p) for k, v in host.items()})
    for _ in range(3):
        g1.update_boundaries(); g1.solve_uvwp()
        g2.update_boundaries()
        g2_dl = cfdl.lib().cfdl_download_fields(g2._h, C.byref(fl))
        assert g2_dl == 0
        st = cfdl.Stats()
        assert cfdl.lib().cfdl_solve_uvwp_host(g2._h, C.byref(fl), C.byref(st)) == 0
    for f in ("u", "v", "w", "p", "mip"):
        assert np.array_equal(g1.get(f), host[f]), f


@pytest.mark.parametrize("graph", [True, False])
def test_step_host_matches_resident(need_gpu, graph):
    """cfdl_step_host (upload, BC + solve_uvwp, overlapped download) equals
    the resident path, with only the steady state's arrays handed over."""
    import ctypes as C
    z = cfdl.Zone(7, True, 0.1, seed=4)
    s = cfdl.Setup(z)
    g1 = cfdl.Solver(s, cfdl.steady())
    g2 = cfdl.Solver(s, cfdl.steady())
    g1.set_graph_mode(graph)
    g2.set_graph_mode(graph)
    nc, nf = s.ne + s.nbf, s.nf
    host = {f: np.zeros(nc) for f in ("u", "v", "w", "p")}
    host.update({f: np.zeros(3 * nc) for f in ("gu", "gv", "gw", "gp", "gpc")})
    host["mip"] = g2.get("mip")
    fl = cfdl.Fields(**{k: v.ctypes.data_as(C.c_void_p) for k, v in host.items()})
    for _ in range(4):
        g1.step(1, ncoef=0)
        assert cfdl.lib().cfdl_step_host(g2._h, C.byref(fl), 1, 0, None) == 0
    for f in ("u", "v", "w", "p", "mip", "gu", "gp", "gpc"):
        assert np.array_equal(g1.get(f), host[f]), f


def test_step_host_keep_skips_only_safe_uploads(need_gpu):
    """cfdl_step_host_keep with the gradients and face fluxes declared
    unchanged equals the resident path bit for bit; when something else wrote
    the device in between (a kernel, set_array), the kept fields are uploaded
    again, so the result equals cfdl_step_host's."""
    import ctypes as C
    z = cfdl.Zone(7, False, 0.2, seed=6)
    s = cfdl.Setup(z)
    g1 = cfdl.Solver(s, cfdl.steady())
    g2 = cfdl.Solver(s, cfdl.steady())
    g3 = cfdl.Solver(s, cfdl.steady())
    nc = s.ne + s.nbf
    keep = sum(cfdl.FIELD_BITS[f] for f in ("gu", "gv", "gw", "gp", "gpc", "mip"))

    def host_for(g):
        h = {f: np.zeros(nc) for f in ("u", "v", "w", "p")}
        h.update({f: np.zeros(3 * nc) for f in ("gu", "gv", "gw", "gp", "gpc")})
        h["mip"] = g.get("mip")
        return h, cfdl.Fields(**{k: v.ctypes.data_as(C.c_void_p) for k, v in h.items()})

    h2, f2 = host_for(g2)
    h3, f3 = host_for(g3)
    L = cfdl.lib()
    for k in range(5):
        g1.step(1, ncoef=0)
        assert L.cfdl_step_host_keep(g2._h, C.byref(f2), keep, 1, 0, None) == 0
        if k == 2:
            # a device write between calls: the kept host arrays are stale for the
            # device now (here: its mip moved on), so they must be uploaded again
            g3.update_boundaries()
            g3.set("gp", h3["gp"] * 0.0)
        assert L.cfdl_step_host_keep(g3._h, C.byref(f3), keep, 1, 0, None) == 0
    for f in ("u", "v", "w", "p", "mip", "gu", "gp", "gpc"):
        assert np.array_equal(g1.get(f), h2[f]), f
        assert np.array_equal(h2[f], h3[f]), f


@pytest.mark.parametrize("tet", [False, "prism"])
def test_symmetry_bc_tight_parity(need_gpu, tet):
    """A wall rebound to the reference's symmetry procedure (mod_uvwp.f90:517-546,
    bc_type 'zero_flux'): reflected halo velocity, no wall shear term, the
    same diffusion coefficient in ap/anb.  Routines and the end-to-end tight
    run agree with the oracle."""
    n, jit = 5, 0.2
    z = cfdl.Zone(n, tet, jit, seed=11)
    s = cfdl.Setup(z)
    m = s.mesh(1.0)
    vel = np.ctypeslib.as_array(C.cast(m.bc_vel, C.POINTER(C.c_double)), (3 * m.nbc,))
    walls = [i for i in range(m.nbc) if vel[3 * i] == 0.0]
    sym = {walls[-1]: cfdl.BC_SYMMETRY, walls[0]: cfdl.BC_SYMMETRY}
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    for i in sym:
        o.set_bc_kind(i, "symmetry")
    g = cfdl.Solver(s, cfdl.steady(solve_mode=1, tight_rtol=1e-13), bc_kinds=sym)
    rng = np.random.default_rng(3)
    seed_state(o, g, rng)
    o.update_boundaries(); g.update_boundaries()
    for f in ("u", "v", "w", "p", "mip"):
        assert rel_max(g.get(f), o.get(f)) < 1e-14, f
    o.calc_coef_uvw(); g.calc_coef_uvw()
    for f in ("ap", "anb", "bu", "bv", "bw"):
        assert rel_max(g.get(f), o.get(f)) < RTOL_KERNEL, f
    # end to end from the construct state
    o2 = oracle_lib.Oracle(z, n_subdomains=4)
    o2.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    for i in sym:
        o2.set_bc_kind(i, "symmetry")
    g2 = cfdl.Solver(s, cfdl.steady(solve_mode=1, tight_rtol=1e-13), bc_kinds=sym)
    o2.run(15, 3)
    st = g2.step(15, 3)
    assert st.status == 0
    for f in ("u", "v", "w", "p"):
        a, b = g2.get(f)[:o2.ne], o2.get(f)[:o2.ne]
        assert rel_l2(a, b) < RTOL_FIELD, (f, rel_l2(a, b))


@pytest.mark.parametrize("precision", [0, 3])
def test_programmatic_launch_does_not_change_results(need_gpu, precision):
    """Programmatic dependent launch (the default) only overlaps launch
    latency, and the graph's parallel branches only reorder independent
    work: the fields equal those of ordinary launches, of the eager form and
    of the graph in one chain, bit for bit."""
    s = cfdl.Setup(cfdl.Zone(7, "mixed", 0.2, seed=9))
    out = []
    for pdl, graph in ((True, 1), (False, 1), (True, 0), (True, 2)):
        g = cfdl.Solver(s, cfdl.steady(precision=precision))
        g.set_pdl(pdl)
        g.set_graph_mode(graph)
        g.step(6, 3)
        out.append({f: g.get(f) for f in ("u", "v", "w", "p", "mip")})
        g.close()
    for f in out[0]:
        for o in out[1:]:
            assert np.array_equal(out[0][f], o[f]), f


def test_sixteen_bit_offsets_do_not_change_results(need_gpu):
    """The mixed form's FP32 mesh-level kernels read the neighbours as 16-bit
    offsets where they fit: the same neighbours and coefficients in the same
    order as the int32 indices, so the fields are the same bit for bit."""
    s = cfdl.Setup(cfdl.Zone(12, False, 0.2, seed=3))
    out = []
    for on in (True, False):
        g = cfdl.Solver(s, cfdl.steady(precision=3))
        g.set_index16(on)
        g.step(20, 3)
        assert g.index_bytes() == (2 if on else 4)
        out.append({f: g.get(f) for f in ("u", "v", "w", "p", "mip")})
        g.close()
    for f in out[0]:
        assert np.array_equal(out[0][f], out[1][f]), f
