"""FP64 thread-instructions per launch of the FP64-bound kernels.

GB300 issues about two FP64 thread-instructions per SM per clock, so the
assembly kernels of the outer iteration (one face or cell term after another,
each a handful of FP64 multiplies and adds) are bound by the FP64 pipe before
they are bound by HBM.  Each figure counts DADD, DMUL and DFMA (one pipe slot
each) and the FP64 instructions of the compiler's division sequence, per
unit of work, as the kernel source does them; W = faces per cell, ne cells,
nf faces, nbf boundary faces (steady form, W = 6 or 4).
"""

DIV = 9          # FP64 instructions of one IEEE division sequence (reciprocal seed and Newton steps)


def fp64_inst(name, ne, nf, nbf, W):
    nfi = nf - nbf
    table = {
        # per interior face: 1 - wt, nine gradient interpolations (2 each), three
        # components of (G^T A + G E) (3 + 3 + 1 each)
        "k_coef_uvw_face": nfi * (1 + 18 + 21),
        # per cell: 6 per interior slot (upwind sum, ap, sumf, three explicit sums),
        # bu/bv/bw (3 each), relaxation (6), d and dc (two divisions and a subtraction);
        # per wall face of a cell: unit normal (3 divisions), tangential slip and the
        # wall terms (about 20)
        "k_coef_uvw_cell": ne * (6 * W + 9 + 6 + 2 * DIV + 1) + nbf * (3 * DIV + 20),
        # per interior face: 1 - wt, velocity interpolation (6), flux (4), Rhie-Chow:
        # pressure-gradient interpolation (6), d_ip (2), the correction (8)
        "k_calc_mip": nfi * (1 + 6 + 4 + 6 + 2 + 8),
        # per cell and slot: a difference and three FMAs for each of the three fields
        "k_grad3": ne * W * 12,
        "k_grad1": ne * W * 4,
    }
    return table.get(name)
