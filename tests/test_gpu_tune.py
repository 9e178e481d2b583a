"""Solver tile shapes and the autotuner.

Every tile shape must give the oracle's fields (tight mode, 1e-9 relative L2
after the same iteration count); the shape only reorders partial sums.  The
autotuner must leave the state of the cases as it found it.
"""
import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("vec", [1, 2, 8])
@pytest.mark.parametrize("precision", [0, 1])
def test_tile_shapes_match_oracle(need_gpu, vec, precision):
    z = cfdl.Zone(7, True, 0.15, seed=11)
    g = cfdl.Solver(cfdl.Setup(z), cfdl.steady(solve_mode=1, tight_rtol=1e-13, precision=precision))
    g.set_tile(vec)
    assert g.get_tile() == vec
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    g.step(5, ncoef=0)
    o.run(5, ncoef=0)
    for f in ("u", "v", "w", "p"):
        assert rel_l2(g.get(f), o.get(f)) < 1e-9, (vec, f)
    g.close()
    o.close()


def test_autotune_restores_state_and_picks_a_shape(need_gpu):
    setups = [cfdl.Setup(cfdl.Zone(n, t, 0.1, seed=n)) for n, t in ((12, False), (6, True), (9, False))]
    b = cfdl.Batch(setups, [cfdl.steady(mu=1.0 / re) for re in (100.0, 400.0, 50.0)])
    b.set_run(4)
    b.run(4)
    before = {(c, f): b.case_get(c, f) for c in range(3) for f in ("u", "v", "w", "p", "mip")}
    best, ms = b.autotune(outer=2)
    assert best in (1, 2, 4, 8) and b.get_tile() == best
    assert b.get_coarse_group() in (1, 2, 4)
    assert all(v > 0 for v in ms.values())
    for (c, f), v in before.items():
        assert np.array_equal(b.case_get(c, f), v), (c, f)
    # the tuned context still runs
    b.set_run(2)
    assert b.run(2) == 0
    b.close()


def test_invalid_tile_rejected(need_gpu):
    g = cfdl.Solver(cfdl.Setup(cfdl.Zone(3)), cfdl.steady())
    with pytest.raises(cfdl.CfdlError):
        g.set_tile(3)
    g.close()


def test_coarse_group_shapes_agree(need_gpu):
    """Large coarse levels (>= 65536 rows) run 1, 2 or 4 lanes per row; all
    three give the same tight-mode fields to rounding."""
    z = cfdl.Zone(84, False, 0.1, seed=3)
    s = cfdl.Setup(z)
    out = {}
    for lanes in (1, 2, 4):
        g = cfdl.Solver(s, cfdl.steady(solve_mode=1, tight_rtol=1e-12))
        g.set_coarse_group(lanes)
        assert g.get_coarse_group() == lanes
        g.step(3, ncoef=0)
        out[lanes] = {f: g.get(f) for f in ("u", "v", "w", "p")}
        g.close()
    for lanes in (2, 4):
        for f in ("u", "v", "w", "p"):
            assert rel_l2(out[lanes][f], out[1][f]) < 1e-9, (lanes, f)
