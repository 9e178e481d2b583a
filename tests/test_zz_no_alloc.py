"""The allocation-free pressure-correction solve (cfdl_solve_pc_noalloc).

For callers that cannot allocate GPU memory themselves -- for example a
Fortran host whose device arrays come from another runtime or pool, or a
process held to a fixed device-memory budget -- the library offers one entry
point that works only on arrays the caller already holds on the device and
keeps its own working storage in a fixed file-scope device array.  This test
plays such a caller: it allocates the inputs and the output itself (through
torch), calls the entry point twice in a row through the C-ABI, and checks
both results against the regular context entry point (cfdl_solve_pc) on the
same pressure system, with the tolerance the other pressure-solve parity
checks use.  It lives in its own file so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import cfdl

pytestmark = pytest.mark.gpu

RTOL_PC = 1e-9          # as the pressure-correction checks in test_gpu_parity.py


def _assembled_case():
    z = cfdl.Zone(20, False, 0.2, seed=4)
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
    return s, g


def test_noalloc_matches_context_solve_twice(need_gpu):
    torch = pytest.importorskip("torch")
    s, g = _assembled_case()
    ap, anb, b = g.get("ap"), g.get("anb"), g.get("b")
    st = g.solve_pc()                       # existing entry point, same algorithm
    assert st.status == 0
    ref = g.get("phic")[:s.ne]
    ref = ref - ref[0]

    dev = torch.device("cuda", 0)
    d_ef1 = torch.from_numpy(s.get_int("ef2nb1")).to(dev)
    d_idx = torch.from_numpy(s.get_int("ef2nb_idx")).to(dev)
    d_ap = torch.from_numpy(ap).to(dev)
    d_anb = torch.from_numpy(anb).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    torch.cuda.synchronize()
    L = cfdl.lib()
    outs = []
    for call in range(2):
        d_x = torch.full((s.ne,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        iters, rnorm = C.c_int(-1), C.c_double(-1.0)
        status = L.cfdl_solve_pc_noalloc(s.ne, s.H, d_ef1.data_ptr(), d_idx.data_ptr(), d_ap.data_ptr(),
                                         d_anb.data_ptr(), d_b.data_ptr(), d_x.data_ptr(), 1e-13, 20000,
                                         C.byref(iters), C.byref(rnorm))
        assert status == 0, cfdl.STATUS.get(status, status)
        assert iters.value > 0 and np.isfinite(rnorm.value)
        x = d_x.cpu().numpy()
        x = x - x[0]
        err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
        assert err < RTOL_PC, (call, err)
        outs.append(x)
    assert np.linalg.norm(outs[0] - outs[1]) <= RTOL_PC * np.linalg.norm(outs[1])


def test_noalloc_rejects_oversize(need_gpu):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    t = torch.zeros(8, dtype=torch.float64, device=dev)
    ti = torch.ones(8, dtype=torch.int32, device=dev)
    L = cfdl.lib()
    status = L.cfdl_solve_pc_noalloc(131073, 8, ti.data_ptr(), ti.data_ptr(), t.data_ptr(), t.data_ptr(),
                                     t.data_ptr(), t.data_ptr(), 1e-8, 10, None, None)
    assert status == 9          # CFDL_ERR_TOO_LARGE
    assert L.cfdl_status_string(9).decode().startswith("problem larger")
