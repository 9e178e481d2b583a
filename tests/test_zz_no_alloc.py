"""The allocation-free pressure-correction solve (cfdl_solve_pc_noalloc).

For callers that cannot allocate GPU memory themselves -- for example a
Fortran host whose device arrays come from another runtime or pool, or a
process held to a fixed device-memory budget -- the library offers one entry
point that works only on arrays the caller already holds on the device and
keeps its own working storage in a fixed file-scope device array.  These
tests play such a caller: they allocate the inputs and the output themselves
(through torch) and call the entry point through the C-ABI.  Two calls in a
row are checked against the regular context entry point (cfdl_solve_pc) on
the same pressure system, and against the oracle's tight pressure solve, with
the tolerance the other pressure-solve parity checks use.  The status cases
(iteration cap, an index outside the arrays, a zero diagonal entry, a
matrix that is not positive definite) and the argument checks, which run
before any device work and so need no GPU, follow.  The file is named so
that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import cfdl
import oracle_lib

RTOL_PC = 1e-9          # as the pressure-correction checks in test_gpu_parity.py
OK, INVALID, NONFINITE, ITER_CAP, TOO_LARGE, BREAKDOWN = 0, 1, 3, 4, 9, 10


def _assembled_case(n=20):
    z = cfdl.Zone(n, False, 0.2, seed=4)
    s = cfdl.Setup(z)
    g = cfdl.Solver(s, cfdl.steady(solve_mode=1, tight_rtol=1e-13, precond=0))
    g.step(3)
    # one pressure-correction system, assembled as solve_uvwp does
    g.update_boundaries()
    g.calc_coef_uvw()
    g.solve_momentum()
    g.calc_grad("uvw")
    g.calc_mip(True)
    g.calc_coef_p()
    return z, s, g


class _Device:
    """The caller's own device copies of one pressure system."""

    def __init__(self, torch, s, ap, anb, b, ef1=None, idx=None):
        dev = torch.device("cuda", 0)
        self.torch, self.dev, self.ne, self.nh = torch, dev, s.ne, s.H
        self.ef1 = torch.from_numpy(s.get_int("ef2nb1") if ef1 is None else ef1).to(dev)
        self.idx = torch.from_numpy(s.get_int("ef2nb_idx") if idx is None else idx).to(dev)
        self.ap = torch.from_numpy(np.ascontiguousarray(ap)).to(dev)
        self.anb = torch.from_numpy(np.ascontiguousarray(anb)).to(dev)
        self.b = torch.from_numpy(np.ascontiguousarray(b)).to(dev)
        torch.cuda.synchronize()

    def solve(self, rtol=1e-13, maxit=20000):
        x = self.torch.full((self.ne,), float("nan"), dtype=self.torch.float64, device=self.dev)
        self.torch.cuda.synchronize()
        iters, rnorm = C.c_int(-1), C.c_double(-1.0)
        status = cfdl.lib().cfdl_solve_pc_noalloc(self.ne, self.nh, self.ef1.data_ptr(), self.idx.data_ptr(),
                                                  self.ap.data_ptr(), self.anb.data_ptr(), self.b.data_ptr(),
                                                  x.data_ptr(), rtol, maxit, C.byref(iters), C.byref(rnorm))
        return status, x.cpu().numpy(), iters.value, rnorm.value


@pytest.mark.gpu
def test_noalloc_matches_context_and_oracle_solves_twice(need_gpu):
    torch = pytest.importorskip("torch")
    z, s, g = _assembled_case()
    ap, anb, b = g.get("ap"), g.get("anb"), g.get("b")
    st = g.solve_pc()                       # existing entry point, same algorithm
    assert st.status == 0
    ref = g.get("phic")[:s.ne]
    ref = ref - ref[0]
    # the oracle's tight pressure solve (Jacobi-PCG from zero) on the same system
    o = oracle_lib.Oracle(z, n_subdomains=1)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    o.set("ap", ap); o.set("anb", anb); o.set("b", b)
    o.solve_pc()
    ora = o.get("phic")[:s.ne]
    ora = ora - ora[0]
    assert np.linalg.norm(ref - ora) < RTOL_PC * np.linalg.norm(ora)

    d = _Device(torch, s, ap, anb, b)
    outs = []
    for call in range(2):
        status, x, iters, rnorm = d.solve()
        assert status == OK, cfdl.STATUS.get(status, status)
        assert iters > 0 and np.isfinite(rnorm)
        x = x - x[0]
        for what, want in (("context", ref), ("oracle", ora)):
            err = np.linalg.norm(x - want) / np.linalg.norm(want)
            assert err < RTOL_PC, (call, what, err)
        outs.append(x)
    assert np.linalg.norm(outs[0] - outs[1]) <= RTOL_PC * np.linalg.norm(outs[1])


@pytest.mark.gpu
def test_noalloc_status_cases(need_gpu):
    """Each way CG can stop short is reported, and a good call afterwards
    still succeeds (the shared array carries nothing over)."""
    torch = pytest.importorskip("torch")
    z, s, g = _assembled_case(8)
    ap, anb, b = g.get("ap"), g.get("anb"), g.get("b")
    # stopped at maxit above the tolerance
    status, x, iters, rnorm = _Device(torch, s, ap, anb, b).solve(rtol=1e-13, maxit=2)
    assert (status, iters) == (ITER_CAP, 2) and np.isfinite(rnorm)
    # a neighbour index beyond the cells: the access is skipped on the device
    ef1 = s.get_int("ef2nb1").copy()
    h = int(np.flatnonzero(ef1 & 31)[5])
    ef1[h] = ((s.ne + 7) << 5) | (ef1[h] & 31)
    assert _Device(torch, s, ap, anb, b, ef1=ef1).solve()[0] == INVALID
    # a CSR offset past the half-face arrays
    idx = s.get_int("ef2nb_idx").copy()
    idx[3] = s.H + 50
    assert _Device(torch, s, ap, anb, b, idx=idx).solve()[0] == INVALID
    # a zero diagonal entry: z = r/ap is not finite
    ap0 = ap.copy()
    ap0[4] = 0.0
    assert _Device(torch, s, ap0, anb, b).solve()[0] == NONFINITE
    # the negated operator is negative definite: p.Ap < 0 at the first step
    assert _Device(torch, s, -ap, -anb, b).solve()[0] == BREAKDOWN
    # and the shared scratch leaves no trace on the next good call
    status, x, iters, rnorm = _Device(torch, s, ap, anb, b).solve()
    assert status == OK and iters > 0


def test_noalloc_argument_checks_need_no_device():
    """Sizes and pointers are checked before the call touches a device."""
    L = cfdl.lib()
    buf = (C.c_double * 8)()
    ibuf = (C.c_int * 8)()
    p, ip = C.cast(buf, C.c_void_p), C.cast(ibuf, C.c_void_p)
    args = [4, 8, ip, ip, p, p, p, p, 1e-8, 10, None, None]

    def call(**over):
        a = list(args)
        names = ["ne", "nh", "ef1", "idx", "ap", "anb", "b", "x", "rtol", "maxit"]
        for k, v in over.items():
            a[names.index(k)] = v
        return L.cfdl_solve_pc_noalloc(*a)

    assert call(ne=0) == INVALID
    assert call(nh=0) == INVALID
    for k in ("ef1", "idx", "ap", "anb", "b", "x"):
        assert call(**{k: None}) == INVALID, k
    assert call(rtol=0.0) == INVALID
    assert call(rtol=float("nan")) == INVALID
    assert call(maxit=-1) == INVALID
    assert call(ne=131073) == TOO_LARGE
    assert L.cfdl_status_string(TOO_LARGE).decode().startswith("problem larger")
    assert L.cfdl_status_string(BREAKDOWN).decode().startswith("Krylov breakdown")
