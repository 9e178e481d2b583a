"""The device mesh set-up (cfdl_setup_create_device) against the oracle and
the host builder.

Face matching by smallest-vertex buckets on the GPU must number, orient and
pair every face exactly as the oracle's restatement of the reference's
set-up does (find_element_nb, calc_redblack, calc_aip_xyzip_uns,
calc_vol_cv_centers_uns), and the device geometry kernels, compiled without
FMA contraction, must give the same doubles.  The product's host builder is
held to the same arrays.
"""
import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu

INTS = ("ef2nb1", "ef2nb2", "ef2nb_idx", "s2g", "bs", "esec", "etype", "red")
DBLS = ("aip", "rip", "xc", "yc", "zc", "vol")


@pytest.mark.parametrize("n,tet,jit", [(5, False, 0.0), (7, True, 0.2), (12, False, 0.2), (9, True, 0.0), (1, True, 0.0),
                                       (6, "prism", 0.2), (5, "pyramid", 0.1), (7, "mixed", 0.2)])
def test_device_setup_equals_host(need_gpu, n, tet, jit):
    z = cfdl.Zone(n, tet, jit, seed=n)
    h, d = cfdl.Setup(z), cfdl.Setup(z, device=True)
    assert (h.ne, h.nf, h.nbf, h.nred) == (d.ne, d.nf, d.nbf, d.nred)
    for name in INTS:
        assert np.array_equal(h.get_int(name), d.get_int(name)), name
    for name in DBLS:
        assert np.array_equal(h.get_dbl(name), d.get_dbl(name)), name


@pytest.mark.parametrize("n,tet,jit,seed", [(5, False, 0.0, 5), (7, True, 0.2, 7), (12, False, 0.2, 12),
                                            (9, True, 0.0, 9), (1, True, 0.0, 1), (6, "prism", 0.2, 6),
                                            (5, "pyramid", 0.1, 5), (7, "mixed", 0.2, 7), (4, False, 0.2, 7),
                                            (32, False, 0.0, 0), (24, True, 0.2, 3)])
def test_device_setup_equals_oracle(need_gpu, n, tet, jit, seed):
    """The device builder against the oracle's own set-up restatement, bit
    for bit (connectivity, ordering, red/black colouring, geometry)."""
    z = cfdl.Zone(n, tet, jit, seed=seed)
    d = cfdl.Setup(z, device=True)
    o = oracle_lib.Oracle(z, n_subdomains=1)
    assert (d.ne, d.nf, d.nbf) == (o.ne, o.nf, o.nbf)
    for name in INTS:
        assert np.array_equal(d.get_int(name), o.get_int(name)), name
    for name in DBLS:
        assert np.array_equal(d.get_dbl(name), o.get(name)), name


def test_device_setup_drives_the_solver(need_gpu):
    z = cfdl.Zone(8, True, 0.1, seed=2)
    a = cfdl.Solver(cfdl.Setup(z), cfdl.steady())
    b = cfdl.Solver(cfdl.Setup(z, device=True), cfdl.steady())
    a.step(3, ncoef=0)
    b.step(3, ncoef=0)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(a.get(f), b.get(f)), f
