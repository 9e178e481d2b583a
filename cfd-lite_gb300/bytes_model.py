"""Algorithmic (compulsory) HBM bytes per launch of each kernel.

Each array a kernel reads or writes is counted once per launch: FP64 = 8 B,
FP32 = 4 B, int32 = 4 B; a gathered neighbour value is counted once for the
cell that owns it, not once per gather.  W = faces per cell (6 for hex, 4 for
tet), ne cells, nf faces (interior + boundary), nbf boundary faces (halos).
These are the figures behind roofline.achieved in bench.py: bytes / average
launch duration.
"""


def kernel_bytes(name, ne, nf, nbf, W, ncomp_active=3):
    nfi = nf - nbf                    # interior faces
    ell_i = 4 * W * ne                # one int32 ELL plane
    ell_d = 8 * W * ne                # one FP64 ELL plane
    m = ncomp_active
    table = {
        # update_boundaries: halo tables + halo u,v,w,p writes, owner p, mip
        "k_bc": nbf * (4 + 4 + 4 + 24 + 32 + 8 + 8),
        # momentum face terms: own/nb, weight + 6 property planes, 3 outputs; 9 gradient comps per cell
        "k_coef_uvw_face": nfi * (8 + 56 + 24) + ne * 72,
        # momentum cell gather: ELL nb/fc, 5 face doubles, 13 cell doubles in, 6 out, anb ELL out
        "k_coef_uvw_cell": 2 * ell_i + nf * 40 + ne * (104 + 48) + ell_d + nbf * (24 + 4 + 32),
        "k_grad3": ell_i + 3 * ell_d + 24 * (ne + nbf) + 72 * ne,
        # precision 3: FP32 stencil, FP32 gradients out and the widened FP64 copies
        "k_grad3_f32": ell_i + 3 * 4 * W * ne + 24 * (ne + nbf) + 108 * ne,
        # precision 3: own/nb, 7 FP32 planes, 3 FP32 outputs; FP32 gradients of both cells
        "k_coef_uvw_face_f32": nfi * (8 + 28 + 12) + ne * 36,
        "k_narrow_grad": ne * (72 + 36),
        "k_grad1": ell_i + 3 * ell_d + 8 * (ne + nbf) + 24 * ne,
        # Rhie-Chow: own/nb, 8 geometry planes, mip0 in, mip out; 12 cell doubles
        "k_calc_mip": nfi * (8 + 72 + 16) + ne * 80,
        "k_coef_p_face": nfi * (8 + 16 + 8) + nbf * 8 + ne * 8,
        # matrix: ELL nb/fc, the face coefficient of every face; anb ELL and ap out
        "k_coef_p_mat": 2 * ell_i + nf * 8 + ell_d + ne * 8,
        # right-hand side: ELL nb/fc, the flux of every face, halo kinds; b out
        "k_coef_p_rhs": 2 * ell_i + nf * 8 + nbf * 4 + ne * 8,
        "k_adjust_pc": ell_i + ne * 16 + nbf * 8,
        "k_update_cells": ne * (8 + 8 + 8 + 24 + 24 + 24),
        "k_update_faces": nfi * (8 + 16 + 16) + ne * 32,
        "k_update_time": ne * 48,
        "k_update_time_halo": nbf * 48,
        "k_copy_mip0": nf * 16,
        # momentum BiCGStab, m active components
        # ap, rap out; per component: b, phi in, r and rh out
        "k_mom_init": ne * 16 + ell_d + ell_i + m * ne * (8 + 8 + 16) + m * nbf * 8,
        "k_mom_p": ne * 8 + m * ne * (24 + 16),
        "k_mom_v": ne * 8 + ell_d + ell_i + m * ne * (8 + 8 + 8),
        "k_mom_s": ne * 8 + m * ne * (16 + 16),
        "k_mom_t": ne * 8 + ell_d + ell_i + m * ne * (8 + 8 + 8),
        "k_mom_x": m * ne * (16 + 8 + 8 + 8 + 8 + 8 + 8),
        # pressure CG
        "k_pc_mean": ne * 8,
        "k_pc_init": ne * (8 + 8 + 8 * 4),
        "k_pc_q": ne * (8 + 8 + 8) + ell_d + ell_i,
        "k_pc_x": ne * (16 + 8 + 16 + 8 + 8 + 8),
        "k_pc_p": ne * 24,
        # energy equation: halo BC (kind, owner, wall t, owner cp in; t, phi out)
        "k_en_bc": nbf * (4 + 4 + 8 + 8 + 16),
        "k_en_time": ne * 16,
        "k_en_time_halo": nbf * 16,
        "k_grad2": ell_i + 3 * ell_d + 16 * (ne + nbf) + 48 * ne,
        # property planes (when cp/tc change): own/nb, weight, area/(dr.n), 3 outputs; cell tc, cp
        "k_en_props": nfi * (8 + 8 + 8 + 24) + nbf * (8 + 8 + 24) + ne * 16,
        # deferred face term: own/nb, weight, area vector, tc_ip and tc_ip/cp_ip, 1 output; the two gradients
        "k_en_face": nfi * (8 + 8 + 24 + 16 + 8) + ne * 48,
        # cell gather: ELL nb/fc, mip + coefficient plane (all faces), deferred term (interior);
        # phi, phi0, rho, vol in, ap, b out; anb ELL out; halo kinds
        "k_en_cell": 2 * ell_i + nf * 16 + nfi * 8 + ne * (32 + 16) + ell_d + nbf * 4,
        # solver init: ap, rap, b, phi, r, rh, anb ELL + halo phi
        "k_en_init": ne * 48 + ell_d + ell_i + nbf * 8,
        "k_en_p": ne * 8 + ne * (24 + 16),
        "k_en_v": ne * 8 + ell_d + ell_i + ne * (8 + 8 + 8),
        "k_en_s": ne * 8 + ne * (16 + 16),
        "k_en_t": ne * 8 + ell_d + ell_i + ne * (8 + 8 + 8),
        "k_en_x": ne * (16 + 8 + 8 + 8 + 8 + 8 + 8),
        "k_en_temp": ne * 24,
    }
    return table.get(name)


def _vcycle_level_bytes(kind, n, W, s, n_prev=0, n_next=0, ib=4):
    """One V-cycle kernel at one level of n cells and ELL width W; ib = bytes
    per neighbour index (2 for the mesh level's 16-bit offsets)."""
    ell_i = ib * W * n
    return {
        "jac0": 3 * s * n,                                  # r, w/D in; t out
        "jac": 4 * s * n + W * s * n + ell_i,               # t, r, w/D in; z out; ELL values and indices
        "jacr": 3 * s * n + W * s * n + ell_i,              # r, w/D in (t = w/D r formed); z out; ELL
        "resid": 4 * s * n + W * s * n + ell_i,             # z, r, D in; t out
        "prolong": (4 * s + 4) * n + W * s * n + ell_i + n_next * s,   # z, r, w/D, agg in; t out; coarse z
        "lift": (2 * s + 4) * n + n_next * s,               # z in and out, agg in; coarse z
        "restrict": n_prev * (s + 4) + n * (4 + s),     # into this level from the finer one
    }[kind]


def amg_kernel_bytes(name, levels, s, tail_rows=2048, ib=4):
    """Multigrid and CG-around-multigrid kernels.  levels = [(n_l, W_l)] for
    l = 0 (mesh) .. L (coarsest); s = value size (8 for the FP64 form, 4 for
    the FP32 inner solve of the mixed form); ib = bytes per mesh-level
    neighbour index (cfdl_amg_index_bytes: 2 for 16-bit offsets, else 4).
    Kernels suffixed _f run on the mesh level; _c kernels are averaged over
    the coarse levels they run on."""
    ne, W = levels[0]
    L = len(levels) - 1
    ell_i = ib * W * ne
    fixed = {
        "k_apc_rz": 16 * ne, "k_apc_p": 24 * ne, "k_apc_x": 48 * ne,
        "k_apc_q": ne * 24 + 8 * W * ne + ell_i,
        "k_mx_rz": 8 * ne, "k_mx_p": 12 * ne, "k_mx_x": 24 * ne,
        "k_mx_q": ne * 12 + 4 * W * ne + ell_i,
    }
    if name in fixed:
        return fixed[name]
    if name == "k_v_tail":
        # a case's levels of at most tail_rows rows, down and back up, and its
        # coarsest solve (dense inverse times the residual)
        lt = next((l for l in range(1, L + 1) if levels[l][0] <= tail_rows), L) if L >= 1 else 0
        b = 0
        for l in range(lt, L):
            n, w = levels[l]
            nn = levels[l + 1][0]
            b += _vcycle_level_bytes("jac0", n, w, s) + 3 * _vcycle_level_bytes("jac", n, w, s)
            b += _vcycle_level_bytes("resid", n, w, s) + _vcycle_level_bytes("restrict", nn, 0, s, n_prev=n)
            b += _vcycle_level_bytes("lift", n, w, s, n_next=nn)
        nL = levels[L][0]
        return b + nL * nL * s + 2 * nL * s
    if not name.startswith("k_v_") or L < 1:
        return None
    kind, where = name[4:].rsplit("_", 1)
    if where == "f":
        if kind == "restrict":
            return _vcycle_level_bytes(kind, levels[1][0], levels[1][1], s, n_prev=ne)
        return _vcycle_level_bytes(kind, ne, W, s, n_next=levels[1][0], ib=ib)
    # the coarse levels that run per-level kernels: those above the tail level
    # (the first of at most tail_rows rows, which k_v_tail runs with the rest);
    # each of them gets the same launches per V-cycle, so the mean over them
    # is the mean per launch
    lt = next((l for l in range(1, L + 1) if levels[l][0] <= tail_rows), L)
    if kind == "restrict":
        ls = list(range(2, lt + 1))
        vals = [_vcycle_level_bytes(kind, levels[l][0], levels[l][1], s, n_prev=levels[l - 1][0]) for l in ls]
    else:
        ls = list(range(1, lt))
        vals = [_vcycle_level_bytes(kind, levels[l][0], levels[l][1], s, n_next=levels[l + 1][0]) for l in ls]
    return sum(vals) / len(vals) if vals else None
