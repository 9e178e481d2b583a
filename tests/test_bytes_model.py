"""The algorithmic-bytes model behind bench.py's roofline.achieved, pinned to
hand counts for the kernels the benchmark reports as dominant.  CPU only."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cfd-lite_gb300"))

from bytes_model import amg_kernel_bytes, kernel_bytes  # noqa: E402


def hex_sizes(n):
    ne, nbf = n ** 3, 6 * n * n
    nf = 3 * n * n * (n - 1) + nbf
    return ne, nf, nbf


def test_mesh_level_jacobi_sweep_is_104_bytes_per_hex_cell():
    # t, r, w/D in and z out (4 doubles), 6 ELL coefficients (doubles) and
    # 6 ELL indices (int32): 32 + 48 + 24 = 104 B per cell
    ne, _, _ = hex_sizes(128)
    levels = [(ne, 6), (ne // 8, 26), (ne // 64, 26)]
    assert amg_kernel_bytes("k_v_jac_f", levels, 8) == 104 * ne
    assert amg_kernel_bytes("k_v_resid_f", levels, 8) == 104 * ne
    # the FP32 form of the mixed solve halves the values, not the indices
    assert amg_kernel_bytes("k_v_jac_f", levels, 4) == (16 + 24 + 24) * ne
    assert amg_kernel_bytes("k_v_jac0_f", levels, 8) == 24 * ne
    assert amg_kernel_bytes("k_v_jacr_f", levels, 4) == (12 + 24 + 24) * ne   # t = w/D r formed in the sweep
    assert 218103808 == amg_kernel_bytes("k_v_jac_f", levels, 8)   # the 128^3 bench figure
    # 16-bit neighbour offsets on the mesh level: 12 index bytes a row, not 24
    assert amg_kernel_bytes("k_v_jac_f", levels, 8, ib=2) == 92 * ne
    assert amg_kernel_bytes("k_apc_q", levels, 8, ib=2) == (24 + 48 + 12) * ne
    assert amg_kernel_bytes("k_v_jac_c", levels, 8, ib=2) == amg_kernel_bytes("k_v_jac_c", levels, 8)


def test_cg_and_bicgstab_spmv_counts():
    ne, nf, nbf = hex_sizes(64)
    levels = [(ne, 6), (ne // 8, 26)]
    # q = A p and (p, q): p in (own), q out, diagonal, ELL values and indices
    assert amg_kernel_bytes("k_apc_q", levels, 8) == (24 + 48 + 24) * ne
    # momentum t = A s for three components: diagonal, ELL, and per component s in, t out, t.s partial
    assert kernel_bytes("k_mom_t", ne, nf, nbf, 6) == (8 + 48 + 24 + 3 * 24) * ne
    # the energy solve's single right-hand side
    assert kernel_bytes("k_en_t", ne, nf, nbf, 6) == (8 + 48 + 24 + 24) * ne


def test_counts_grow_linearly_with_the_mesh():
    for name in ("k_coef_uvw_face", "k_coef_uvw_cell", "k_calc_mip", "k_grad3", "k_mom_init", "k_en_cell"):
        a = kernel_bytes(name, *hex_sizes(32), 6)
        b = kernel_bytes(name, *hex_sizes(64), 6)
        assert 7.5 < b / a < 8.2, name     # interior faces 3n^2(n-1) grow a little faster than n^3
    assert kernel_bytes("no_such_kernel", *hex_sizes(8), 6) is None


def test_coarse_kernels_average_over_the_levels_they_run_on():
    """_c kernels run on the coarse levels above the tail level (the first of
    at most 2048 rows); the levels the tail kernel runs are not in the mean."""
    levels = [(2097152, 6), (262144, 26), (32768, 26), (4096, 26), (512, 20), (64, 12)]
    jac = [4 * 8 * n + w * 8 * n + 4 * w * n for n, w in levels[1:4]]
    assert amg_kernel_bytes("k_v_jac_c", levels, 8) == sum(jac) / 3
    rst = [n_prev * (8 + 4) + n * (4 + 8) for (n_prev, _), (n, _) in zip(levels[1:4], levels[2:5])]
    assert amg_kernel_bytes("k_v_restrict_c", levels, 8) == sum(rst) / 3


def test_lift_and_tail_counts():
    """k_v_lift reads and writes z and reads the aggregate map (plus the coarse
    vector); the tail sums its levels' passes and the dense coarsest solve."""
    lv = [(4096, 6), (520, 20), (30, 12)]
    assert amg_kernel_bytes("k_v_lift_f", lv, 8) == (16 + 4) * 4096 + 520 * 8
    n, w, nn = 520, 20, 30
    per_level = (3 * 8 * n + 3 * (4 * 8 * n + w * 8 * n + 4 * w * n) + (4 * 8 * n + w * 8 * n + 4 * w * n)
                 + (n * (8 + 4) + nn * (4 + 8)) + ((16 + 4) * n + nn * 8))
    assert amg_kernel_bytes("k_v_tail", lv, 8) == per_level + nn * nn * 8 + 2 * nn * 8


def test_flops_model_matches_the_counted_instructions():
    """The FP64 model against ncu's counted FP64 instructions on the 48^3 hex
    cavity (profiles/fp64_instructions_cavity48.md): within 2% for each
    kernel the model covers."""
    from flops_model import fp64_inst
    ne, nf, nbf = hex_sizes(48)
    counted = {"k_coef_uvw_face": 12994560, "k_coef_uvw_cell": 8432640, "k_grad3": 7962624,
               "k_calc_mip": 6822144, "k_mom_init": 4718392, "k_mom_t": 3464964, "k_mom_v": 2930573,
               "k_grad1": 2654208, "k_mom_x": 1916710, "k_apc_q": 1026012, "k_v_jac_f": 995328,
               "k_mom_s": 976779, "k_v_resid_f": 884736}
    for k, c in counted.items():
        m = fp64_inst(k, ne, nf, nbf, 6)
        assert abs(m - c) <= 0.02 * c, (k, m, c)


def test_ncu_traffic_is_looked_up_per_precision():
    """bench.py's roofline traffic comes from profiles/ncu_traffic.txt, per
    kernel and precision (FP64 and FP32 sweeps move different bytes), scaled
    from the capture's cell count; a kernel or precision without a capture
    has none."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.ncu_traffic("k_v_jac_f", 112, 0) == 141687168
    assert bench.ncu_traffic("k_v_jac_f", 112, 3) == 67869696
    assert abs(bench.ncu_traffic("k_v_jac_f", 128, 3) - 67869696 * 128 ** 3 / 112 ** 3) < 1
    assert bench.ncu_traffic("k_v_jac_f", 128, 1) is None
    assert bench.ncu_traffic("k_v_jac_c", 128, 0) is None
