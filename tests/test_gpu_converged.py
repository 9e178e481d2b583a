"""Converged steady states against the oracle's.

A converged SIMPLE solution is a fixed point of the outer iteration: the
momentum equations hold, the pressure correction is zero and the face fluxes
are divergence-free, whatever inner solvers got there.  So the GPU forms --
FP64 AMG-PCG and the mixed-precision pressure solve, each with the
reference's stop-at-10x-drop inner solves -- must reach the oracle's
converged fields (the reference algorithm: Gauss-Seidel momentum solves,
4-block SSOR pressure solve) to within 1e-6 relative L2, the tolerance the
mixed form is held to.  The forms: precision 0 FP64; 1 mixed pressure
solve; 2 also FP32 momentum corrections; 3 also FP32 explicit momentum face
terms.
"""
import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu

TOL = 1e-6


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("n,tet,re", [(10, False, 100.0), (5, True, 400.0)])
def test_converged_fields_match_oracle(need_gpu, n, tet, re):
    outer = 1500
    z = cfdl.Zone(n, tet, 0.1, seed=21)
    s = cfdl.Setup(z)
    o = oracle_lib.Oracle(z, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=0, mu=1.0 / re))
    o.run(outer, ncoef=0)
    ref = {f: o.get(f)[: s.ne] for f in ("u", "v", "w", "p")}
    o.close()
    for precision in (0, 1, 2, 3):
        g = cfdl.Solver(s, cfdl.steady(mu=1.0 / re, precision=precision))
        g.set_run(outer)
        assert g.run(outer) == 0
        g.update_boundaries()
        st = g.solve_uvwp()
        # precision 3 recomputes its FP32 explicit face terms every pass, so
        # the iteration settles at their rounding level instead of at FP64's
        assert st.mass_imbalance < (1e-9 if precision == 3 else 1e-12), (precision, st.mass_imbalance)
        for f in ("u", "v", "w", "p"):
            err = rel_l2(g.get(f)[: s.ne], ref[f])
            assert err < TOL, (precision, f, err)
        g.close()
