"""Precision 3: the explicit momentum face terms (sumss and the deferred
non-orthogonal correction of calc_coef_uvw) and the gradients of u, v, w they
use in FP32, on top of the mixed pressure solve and FP32 momentum
corrections.  The FP64<->FP32 conversions of these kernels are done in the
integer pipe; they must agree with the hardware conversions.  The host
drop-in, the tuner's snapshot and a switch of form mid-run must keep the
FP32 gradients in step with gu, gv, gw.  Converged states are checked
against the oracle with the other forms (test_gpu_converged.py)."""
import ctypes as C

import numpy as np
import pytest

import cfdl

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_integer_conversions_match_hardware(need_gpu):
    assert cfdl.check_conversions(1 << 22) == (0, 0)


def test_host_dropin_equals_resident(need_gpu):
    z = cfdl.Zone(7, False, 0.2, seed=4)
    s = cfdl.Setup(z)
    cfg = cfdl.steady(precision=3)
    a, b = cfdl.Solver(s, cfg), cfdl.Solver(s, cfg)
    a.step(6, 0)
    nc, nf = s.ne + s.nbf, s.nf
    sizes = {"u": nc, "v": nc, "w": nc, "p": nc, "gu": 3 * nc, "gv": 3 * nc, "gw": 3 * nc, "gp": 3 * nc,
             "gpc": 3 * nc, "mip": nf}
    host = {k: np.zeros(n) for k, n in sizes.items()}
    fl = cfdl.Fields(**{k: v.ctypes.data_as(C.c_void_p) for k, v in host.items()})
    L = cfdl.lib()
    cfdl._check(L.cfdl_download_fields(b._h, C.byref(fl)), "download")
    for _ in range(6):
        cfdl._check(L.cfdl_step_host(b._h, C.byref(fl), 1, 0, None), "step_host")
    for f in ("u", "v", "w", "p", "gu", "gp", "mip"):
        assert np.array_equal(host[f], a.get(f)), f


def test_autotune_and_form_switch_keep_state(need_gpu):
    s = cfdl.Setup(cfdl.Zone(8, True, 0.1, seed=5))
    g = cfdl.Solver(s, cfdl.steady(precision=0))
    g.step(4, 0)
    g.set_config(cfdl.steady(precision=3))      # gu, gv, gw of the FP64 run seed the FP32 gradients
    ref = cfdl.Solver(s, cfdl.steady(precision=0))
    ref.step(4, 0)
    ref.set_config(cfdl.steady(precision=3))
    before = {f: g.get(f) for f in ("u", "p", "gu")}
    g.autotune(outer=1)
    for f, v in before.items():
        assert np.array_equal(g.get(f), v), f
    g.set_tile(ref.get_tile())
    g.set_coarse_group(ref.get_coarse_group())
    g.step(5, 0)
    ref.step(5, 0)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(g.get(f), ref.get(f)), f


def test_close_to_fp64_after_the_same_iterations(need_gpu):
    s = cfdl.Setup(cfdl.Zone(10, False, 0.2, seed=6))
    out = {}
    for prec in (2, 3):
        g = cfdl.Solver(s, cfdl.steady(precision=prec))
        g.step(40, 0)
        out[prec] = {f: g.get(f)[: s.ne] for f in ("u", "v", "w", "p")}
        g.close()
    for f in ("u", "v", "w", "p"):
        assert rel_l2(out[3][f], out[2][f]) < 1e-5, f
