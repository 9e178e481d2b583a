"""GPU parity at the plain-FP64 configurations, at their full iteration counts.

cavity32  -- 32^3 uniform hex cells, Re 100 (rho 1, mu 0.01), steady SIMPLE
             with alpha_u 0.7 / alpha_p 0.3: 200 outer iterations.
cavity128 -- 128^3 hex cells (2,097,152) with interior nodes jittered by a
             seeded U(-0.2, 0.2) of the spacing, same physics: 500 outer
             iterations.

Both sides run the tight mode (every inner solve to ||r|| <= 1e-13 ||b||), and
the GPU's u, v, w, p must agree with the oracle's within 1e-9 relative L2
after the same number of outer iterations.

At 32^3 the oracle runs beside the GPU for all 200 iterations.  At 128^3 the
oracle runs beside the GPU on this host for CAVITY128_ORACLE_ITERS outer
iterations (each takes the oracle seconds: a ~1300-iteration Jacobi-PCG
pressure solve on 2.1M cells), and the GPU's whole 500-iteration run is
checked against the committed fixture of a 500-iteration oracle run
(tests/golden/cavity_runs.json and .npz, made by make_cavity_runs.py): at
every checkpoint the 2-norms and eight random +-1 projections of each field
over all cells, and the values of every 1021st cell at three checkpoints.
The oracle run here must also reproduce the fixture's SHA-256 hashes, which
pins this host's oracle to the machine that made the fixture.
"""
import json
import os

import numpy as np
import pytest

import cfdl
import oracle_lib

pytestmark = pytest.mark.gpu

RTOL_FIELD = 1e-9
FIELDS = ("u", "v", "w", "p")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# about 8 minutes of the oracle on a 16-core Grace host (2.4 s per outer iteration)
CAVITY128_ORACLE_ITERS = int(os.environ.get("CFDL_CAVITY128_ORACLE_ITERS", "200"))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def fixture(key):
    with open(os.path.join(GOLDEN, "cavity_runs.json")) as fh:
        meta = json.load(fh)
    samples = np.load(os.path.join(GOLDEN, "cavity_runs.npz"))
    return meta, meta["cases"][key], samples


def signs(meta, ne):
    rng = np.random.default_rng(meta["proj_seed"])
    return (rng.integers(0, 2, size=(meta["nproj"], ne), dtype=np.int8) * 2 - 1).astype(np.float64)


def check_against_fixture(key, k, gpu_fields, meta, rec, samples, S):
    """GPU fields after k outer iterations against the fixture's checkpoint k."""
    cp = rec["checkpoints"][str(k)]
    ne = rec["ne"]
    worst = 0.0
    for f in FIELDS:
        x = gpu_fields[f][:ne]
        l2 = cp["l2"][f]
        # norms and projections: a field within rel L2 e moves each by about e * l2
        assert abs(np.linalg.norm(x) - l2) <= RTOL_FIELD * l2, (key, k, f, "l2")
        dproj = np.abs(S @ x - np.asarray(cp["proj"][f])).max() / l2
        assert dproj <= RTOL_FIELD, (key, k, f, "projection", dproj)
        name = "%s_%d_%s" % (key, k, f)
        if name in samples.files:
            err = rel_l2(x[::meta["stride"]], samples[name])
            assert err < RTOL_FIELD, (key, k, f, "sample", err)
            worst = max(worst, err)
        worst = max(worst, dproj)
    return worst


def make(n, jitter, seed=0):
    z = cfdl.Zone(n, False, jitter, seed=seed)
    s = cfdl.Setup(z)
    g = cfdl.Solver(s, cfdl.steady(solve_mode=1, tight_rtol=1e-13))
    return z, s, g


def test_cavity32_200_outer_iterations_tight(need_gpu):
    """32^3 cavity through all 200 outer iterations: GPU against the oracle
    run beside it (1e-9 relative L2 per field), the oracle against the
    committed hashes, and the GPU against the fixture at each checkpoint."""
    meta, rec, samples = fixture("cavity32")
    z, s, g = make(32, 0.0)
    o = oracle_lib.Oracle(z, n_subdomains=1)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    S = signs(meta, rec["ne"])
    done = 0
    for k in sorted(int(c) for c in rec["checkpoints"]):
        st = g.step(k - done, 3)
        assert st.status == 0
        o.run(k - done, 3)
        done = k
        gf = {f: g.get(f) for f in FIELDS}
        for f in FIELDS:
            of = o.get(f)
            assert rel_l2(gf[f][:o.ne], of[:o.ne]) < RTOL_FIELD, (k, f, rel_l2(gf[f][:o.ne], of[:o.ne]))
            assert oracle_lib.sha256(of) == rec["checkpoints"][str(k)]["hash"][f], (k, f, "oracle hash")
        check_against_fixture("cavity32", k, gf, meta, rec, samples, S)
    assert done == 200


def test_cavity128_tight_against_oracle(need_gpu):
    """The 128^3 jittered cavity: GPU and oracle side by side for
    CAVITY128_ORACLE_ITERS outer iterations, u, v, w, p within 1e-9 relative
    L2; the oracle's fields equal the fixture's hashes where it has a
    checkpoint."""
    meta, rec, samples = fixture("cavity128")
    z, s, g = make(128, 0.2)
    o = oracle_lib.Oracle(z, n_subdomains=1)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    stops = sorted({int(c) for c in rec["checkpoints"] if int(c) <= CAVITY128_ORACLE_ITERS}
                   | {CAVITY128_ORACLE_ITERS})
    done, report, t_oracle = 0, [], 0.0
    for k in stops:
        st = g.step(k - done, 3)
        assert st.status == 0
        t0 = oracle_lib.wtime()
        o.run(k - done, 3)
        t_oracle += oracle_lib.wtime() - t0
        done = k
        for f in FIELDS:
            a, b = g.get(f), o.get(f)
            err = rel_l2(a[:o.ne], b[:o.ne])
            report.append((k, f, err))
            assert err < RTOL_FIELD, (k, f, err)
            if str(k) in rec["checkpoints"]:
                assert oracle_lib.sha256(b) == rec["checkpoints"][str(k)]["hash"][f], (k, f, "oracle hash")
    print("cavity128 GPU vs oracle, worst rel L2 per checkpoint:",
          {k: max(e for kk, _, e in report if kk == k) for k in stops},
          "oracle %.1f s for %d outer iterations on %d threads" % (t_oracle, done, oracle_lib.num_threads()))


def test_cavity128_500_outer_iterations_against_fixture(need_gpu):
    """The 128^3 jittered cavity through its full 500 outer iterations on the
    GPU, checked at every checkpoint of the committed 500-iteration oracle
    run."""
    meta, rec, samples = fixture("cavity128")
    cps = sorted(int(c) for c in rec["checkpoints"])
    assert cps[-1] == 500, "fixture incomplete: %s" % cps
    z, s, g = make(128, 0.2)
    S = signs(meta, rec["ne"])
    done, worst = 0, {}
    for k in cps:
        st = g.step(k - done, 3)
        assert st.status == 0
        done = k
        worst[k] = check_against_fixture("cavity128", k, {f: g.get(f) for f in FIELDS}, meta, rec, samples, S)
    print("cavity128 GPU vs fixture, worst relative difference per checkpoint:", worst)
