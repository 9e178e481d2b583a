"""FP64 thread-instructions per launch of the kernels that do FP64 arithmetic.

GB300 issues about two FP64 thread-instructions per SM per clock (the
cfdl_probe_fp64 DFMA probe measures 0.63 T instructions/s, 1.25 TFLOP/s), so
the assembly kernels of the outer iteration are bound by the FP64 pipe before
they are bound by HBM.  The per-unit figures are the FP64 instructions the
kernels execute (DADD, DMUL, DFMA and the rest of the double-precision
class, each one pipe slot), as ncu counted them
(sm__sass_thread_inst_executed_op_fp64_pred_on) on the 48^3 hex cavity
(profiles/fp64_instructions_cavity48.md); the source of each kernel accounts
for them:

  k_coef_uvw_face  40 per interior face: 1 - wt, nine gradient
                   interpolations (2 each), three components of
                   G^T A + G E (7 each)
  k_calc_mip       21 per interior face: velocity and pressure-gradient
                   interpolation, the flux and the Rhie-Chow correction
  k_coef_uvw_cell  70 per cell (6 per slot, the three right-hand sides, the
                   relaxation, the divisions of d and dc) and about 50 per
                   wall face (unit normal, tangential slip, wall terms)
  k_grad<N>        4 per slot and field (a difference and three FMAs)
  k_mom_*          BiCGStab with three active right-hand sides
  k_v_* , k_apc_q  the pressure solve's mesh-level rows

W = faces per cell; per-cell figures of the W-slot rows are scaled from the
hex counts by W / 6.
"""


def fp64_inst(name, ne, nf, nbf, W):
    nfi = nf - nbf
    w = W / 6.0
    table = {
        "k_coef_uvw_face": 40 * nfi,
        "k_calc_mip": 21 * nfi,
        "k_coef_uvw_cell": 70 * ne + 50 * nbf,
        "k_grad3": 12 * W * ne,
        "k_grad1": 4 * W * ne,
        "k_mom_init": 42.7 * w * ne,
        "k_mom_v": 26.5 * w * ne,
        "k_mom_t": 31.3 * w * ne,
        "k_mom_x": 17.3 * ne,
        "k_mom_s": 8.8 * ne,
        "k_v_jac_f": 9.0 * w * ne,
        "k_v_resid_f": 8.0 * w * ne,
        "k_apc_q": 9.3 * w * ne,
    }
    v = table.get(name)
    return int(round(v)) if v is not None else None
