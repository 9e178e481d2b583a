"""Mesh set-up: the product's connectivity/geometry builder against the
oracle's line-by-line restatement of find_element_nb / calc_aip_xyzip_uns /
calc_vol_cv_centers_uns / calc_redblack (bit-exact), hand-derivable
invariants, the committed golden hashes, and the C-ABI symbol table.
No GPU is needed: these exercise host code only."""
import hashlib
import json
import os
import re

import numpy as np
import pytest

import cfdl
import oracle_lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "setup_hashes.json")

CASES = [(2, False, 0.0), (4, False, 0.2), (8, False, 0.2), (3, True, 0.0), (6, True, 0.1), (12, False, 0.1),
         (4, "prism", 0.2), (3, "pyramid", 0.1), (5, "mixed", 0.2), (1, "pyramid", 0.0)]


def expected_sizes(n, tet):
    """(cells, boundary faces, half-faces) of the synthetic zone of each kind."""
    c = n ** 3
    if tet is True or tet == "tet":
        return 6 * c, 12 * n * n, 24 * c
    if tet == "prism":
        return 2 * c, 8 * n * n, 10 * c
    if tet == "pyramid":
        return 6 * c, 6 * n * n, 30 * c
    if tet == "mixed":
        p = c // 2
        return (c - p) + 6 * p, 6 * n * n, 6 * (c - p) + 30 * p
    return c, 6 * n * n, 6 * c


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("n,tet,jit", CASES)
def test_setup_matches_oracle_bit_exact(n, tet, jit):
    z = cfdl.Zone(n, tet, jit, seed=7)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    assert (s.ne, s.nf, s.nbf) == (o.ne, o.nf, o.nbf)
    for name in ("ef2nb1", "ef2nb2", "ef2nb_idx", "s2g", "bs", "red"):
        np.testing.assert_array_equal(s.get_int(name), o.get_int(name), err_msg=name)
    for name in ("aip", "rip", "xc", "yc", "zc", "vol"):
        a, b = s.get_dbl(name), o.get(name)
        assert np.array_equal(a, b), name  # bit-exact doubles


@pytest.mark.parametrize("n,tet", [(2, False), (5, False), (3, True), (3, "prism"), (3, "pyramid"), (4, "mixed")])
def test_sizes_and_invariants(n, tet):
    z = cfdl.Zone(n, tet, 0.15, seed=3)
    s = cfdl.Setup(z)
    assert (s.ne, s.nbf, s.H) == expected_sizes(n, tet)
    vol = s.get_dbl("vol")
    assert (vol > 0).all()
    assert abs(vol.sum() - 1.0) < 1e-13                     # unit cube
    aip = s.get_dbl("aip").reshape(-1, 3)
    ef2 = s.get_int("ef2nb2")
    idx = s.get_int("ef2nb_idx")
    # closed surface: the outward area vectors of every cell sum to zero
    for e in range(s.ne):
        tot = np.zeros(3)
        for h in range(idx[e] - 1, idx[e + 1] - 1):
            fg = ef2[h]
            tot += np.sign(fg) * aip[abs(fg) - 1]
        assert np.abs(tot).max() < 1e-14
    # every face appears once with + (owner) and, if interior, once with -
    counts = np.bincount(np.abs(ef2), minlength=s.nf + 1)[1:]
    assert counts.max() == 2 and counts.min() == 1
    assert (counts == 1).sum() == s.nbf
    # the owner is the lower-numbered cell (mod_mg_lvl_uns.f90:397-410)
    ef1 = s.get_int("ef2nb1")
    for e in range(s.ne):
        for h in range(idx[e] - 1, idx[e + 1] - 1):
            enb, lf = ef1[h] >> 5, ef1[h] & 31
            if lf:
                assert (ef2[h] > 0) == (e + 1 < enb)
    # halo centres are boundary face centroids
    rip = s.get_dbl("rip").reshape(-1, 3)
    bs = np.abs(s.get_int("bs"))
    xc = s.get_dbl("xc")
    for k in range(s.nbf):
        e, lf = bs[k] >> 5, bs[k] & 31
        fg = ef2[idx[e - 1] - 1 + lf - 1]
        assert xc[s.ne + k] == rip[fg - 1, 0]


def test_face_numbering_closed_form():
    """find_element_nb numbers faces by (smallest vertex, lower element,
    local face); check that rule independently on a 3^3 hex zone."""
    z = cfdl.Zone(3, False, 0.0)
    s = cfdl.Setup(z)
    m = z.ne2vxmax
    faces_hexa8 = [(1, 4, 3, 2), (1, 2, 6, 5), (2, 3, 7, 6), (3, 4, 8, 7), (1, 5, 8, 4), (5, 6, 7, 8)]
    s2g = s.get_int("s2g")
    keys = []
    for fg in range(s.nf):
        e, lf = s2g[fg] >> 5, s2g[fg] & 31
        vx = z.e2vx[(e - 1) * m:(e - 1) * m + 8]
        keys.append((min(vx[v - 1] for v in faces_hexa8[lf - 1]), e, lf))
    assert keys == sorted(keys)


def test_golden_hashes():
    """Regression pin: hashes of the integer arrays (and the geometry) for the
    cases listed in tests/golden/setup_hashes.json, produced by the oracle
    with tests/golden/make_golden.py."""
    with open(GOLDEN) as fh:
        gold = json.load(fh)
    for key, ref in gold["cases"].items():
        n, tet, jit, seed = ref["n"], ref["tet"], ref["jitter"], ref["seed"]
        z = cfdl.Zone(n, tet, jit, seed=seed)
        s = cfdl.Setup(z)
        o = oracle_lib.Oracle(z, n_subdomains=4)
        for name, h in ref["int"].items():
            arr = o.get_int(name)
            assert sha(arr) == h, (key, name)
            if name in ("ef2nb1", "ef2nb2", "ef2nb_idx", "s2g", "bs", "red"):
                assert sha(s.get_int(name)) == h, (key, name)
        for name, h in ref["dbl"].items():
            assert sha(o.get(name)) == h, (key, name)
            assert sha(s.get_dbl(name)) == h, (key, name)


def test_partition_is_four_octree_blocks():
    z = cfdl.Zone(8, False, 0.2, seed=7)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    g = o.get_int("gf2g")
    assert sorted(np.unique(g)) == [1, 2, 3, 4]
    g2 = o.get_int("g2gf")
    assert sorted(g2) == list(range(1, o.ne + 1))
    idx = o.get_int("g2gf_idx")
    assert idx[0] == 1 and idx[-1] == o.ne + 1
    for c in range(4):
        assert (g[g2[idx[c] - 1:idx[c + 1] - 1] - 1] == c + 1).all()
    # subdomain CSR: local cells keep their face count; halos = cut + boundary faces
    tot_halo = 0
    for sd in range(1, 5):
        ne, nf, nbf, sidx, ef = o.subdomain(sd)
        assert ne == idx[sd] - idx[sd - 1]
        assert sidx[-1] - 1 == 2 * nf - nbf
        tot_halo += nbf
    assert tot_halo >= o.nbf


def test_library_exports_every_declared_symbol():
    with open(os.path.join(ROOT, "include", "cfdl.h")) as fh:
        text = fh.read()
    names = set(re.findall(r"\b(cfdl_[a-z0-9_]+)\s*\(", text))
    L = cfdl.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert len(names) > 25


def test_invalid_inputs_are_rejected():
    import ctypes as C
    L = cfdl.lib()
    a = C.c_int()
    assert L.cfdl_box_zone_sizes(0, 0, C.byref(a), C.byref(a), C.byref(a), C.byref(a)) == 1
    z = cfdl.Zone(2)
    bad = z.e2vx.copy()
    bad[0] = z.nvx + 5
    h = C.c_void_p()
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    st = L.cfdl_setup_create(z.nvx, p(z.x), p(z.y), p(z.z), z.nsec, z.names, p(z.etype), p(z.esec),
                             z.ne2vxmax, p(bad), C.byref(h))
    assert st == 1 and not h.value
    # a non-conforming mesh (one boundary quad dropped) is a mesh error
    esec = z.esec.copy()
    esec[-1] -= 1
    st = L.cfdl_setup_create(z.nvx, p(z.x), p(z.y), p(z.z), z.nsec, z.names, p(z.etype), p(esec),
                             z.ne2vxmax, p(z.e2vx), C.byref(h))
    assert st != 0


def test_ctx_create_without_device_fails_loudly():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("device present")
    s = cfdl.Setup(cfdl.Zone(2))
    with pytest.raises(cfdl.CfdlError) as ei:
        cfdl.Solver(s)
    assert ei.value.status == 7
    with pytest.raises(cfdl.CfdlError) as ei:
        cfdl.Batch([s, s], [cfdl.steady(), cfdl.steady()])
    assert ei.value.status == 7
    with pytest.raises(cfdl.CfdlError) as ei:
        cfdl.Server(prep_threads=1)
    assert ei.value.status == 7


def test_case_bytes_estimate_and_server_config():
    # the estimate grows linearly with the mesh and bounds ~2.1 kB per hex cell
    # (every form's arrays, the precision-3 FP32 copies included)
    e1 = cfdl.case_bytes_estimate(1000, 3300, 600)
    e8 = cfdl.case_bytes_estimate(8000, 26400, 2400)
    assert 0 < e1 < e8 <= 8.5 * e1
    assert e8 / 8000 < 2200
    c = cfdl.server_config()
    assert c.hbm_budget == 150e9 and c.max_cases > 0 and c.chunk > 0 and c.precision in (0, 1)
    with pytest.raises(KeyError):
        cfdl.server_config(no_such_field=1)


# ---- cfdl_mesh_check: the host-side validation of cfdl_ctx_create -----------

@pytest.mark.parametrize("kind", ["hex", "tet", "prism", "pyramid", "mixed"])
def test_mesh_check_accepts_every_kind(kind):
    s = cfdl.Setup(cfdl.Zone(4, kind if kind != "hex" else False, 0.2, seed=5))
    assert s.check() == 0


def _corrupted(s, **arrays):
    """s's mesh with some arrays replaced (the replacements kept alive on the struct)."""
    import ctypes as C
    m = s.mesh()
    keep = []
    for name, arr in arrays.items():
        arr = np.ascontiguousarray(arr)
        keep.append(arr)
        setattr(m, name, arr.ctypes.data_as(C.c_void_p))
    return m, keep


def test_mesh_check_refuses_corrupted_meshes():
    import ctypes as C
    s = cfdl.Setup(cfdl.Zone(4, True, 0.1, seed=5))
    L = cfdl.lib()
    ef1, ef2, idx = s.get_int("ef2nb1"), s.get_int("ef2nb2"), s.get_int("ef2nb_idx")
    s2g = s.get_int("s2g")
    ne, nbf = s.ne, s.nbf
    own0 = next(h for h in range(idx[0] - 1, idx[1] - 1) if ef2[h] > 0)
    other = next(h for h in range(idx[1] - 1, len(ef2)) if ef2[h] > 0)
    interior = next(h for h in range(len(ef1)) if 0 < (ef1[h] >> 5) <= ne and (ef1[h] & 31))

    def refused(**arrays):
        m, keep = _corrupted(s, **arrays)
        return L.cfdl_mesh_check(C.byref(m)) == 1

    a = ef2.copy(); a[own0] = ef2[other]                     # two owners of one face
    assert refused(ef2nb2=a)
    a = ef1.copy(); a[5] = ((ne + nbf + 3) << 5) | 1         # neighbour past the halos
    assert refused(ef2nb1=a)
    a = ef1.copy(); a[interior] = (ef1[interior] >> 5) << 5  # interior neighbour marked as boundary
    assert refused(ef2nb1=a)
    a = idx.copy(); a[0] = 2                                 # CSR offsets not 1-based
    assert refused(ef2nb_idx=a)
    a = s2g.copy(); a[0] = ((((s2g[0] >> 5) % ne) + 1) << 5) | (s2g[0] & 31)   # s2g names another owner
    assert refused(s2g=a)
    m = s.mesh()
    kinds = np.array([7] * m.nbc, np.int32)                  # no such boundary kind
    assert refused(bc_kind=kinds)
    esec = np.array(C.cast(m.bc_esec, C.POINTER(C.c_int))[:2 * m.nbc], np.int32)
    esec[0] = 1                                              # a boundary range over interior cells
    assert refused(bc_esec=esec)
    assert s.check() == 0                                    # the originals are untouched
    assert L.cfdl_mesh_check(None) == 1


@pytest.mark.parametrize("n,jit,seed", [(1, 0.0, 0), (5, 0.2, 7), (8, 0.0, 0), (12, 0.2, 3)])
def test_oracle_zone_equals_product_zone(n, jit, seed):
    """The oracle's own hex cavity zone (used where an oracle run must not
    load the GPU library, as the benchmark's reference arm) is the product's
    synthetic zone, bit for bit."""
    a, b = cfdl.Zone(n, False, jit, seed=seed), oracle_lib.BoxZone(n, jit, seed)
    assert (a.nvx, a.nelem, a.nsec, a.ne2vxmax) == (b.nvx, b.nelem, b.nsec, b.ne2vxmax)
    for f in ("x", "y", "z", "e2vx", "etype", "esec"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.names.raw == b.names
