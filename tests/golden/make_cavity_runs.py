"""Long oracle runs of the two plain-FP64 cavity configurations, as fixtures.

    python tests/golden/make_cavity_runs.py [cavity32|cavity128 ...]

cavity32:  32^3 uniform hex cells, Re = 100 (rho 1, mu 0.01), steady SIMPLE
           with alpha_u 0.7 / alpha_p 0.3, 200 outer iterations.
cavity128: 128^3 hex cells with interior nodes jittered by a seeded
           U(-0.2, 0.2) of the spacing (seed 0), same physics, 500 outer
           iterations.

Both run the oracle in its tight mode (every inner solve to a relative
residual of 1e-13), the mode in which the GPU library must reproduce the
u, v, w, p fields within 1e-9 relative L2 after the same number of outer
iterations.  The mesh is built by the oracle's own set-up restatement.  At
each checkpoint the fixture keeps, per field (interior cells):

  hash   SHA-256 of the whole array (cells and halos);
  l2     its 2-norm over the interior cells;
  proj   eight projections onto seeded random +-1 vectors over the interior
         cells (numpy PCG64, seed 2024) -- a GPU field within rel L2 e of the
         oracle's differs in each projection by about e * l2;
  sample the values of every 1021st interior cell (at the checkpoints in
         SAMPLE_AT), stored in cavity_runs.npz.

The oracle's results do not depend on its thread count (fixed-block dot
products) and use only IEEE +, -, *, /, sqrt without contraction, so the
hashes hold on any host.  The JSON is rewritten after every checkpoint, so an
interrupted run leaves the checkpoints it reached.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "cfd-lite_gb300"), os.path.join(ROOT, "tests")]

import cfdl  # noqa: E402
import oracle_lib  # noqa: E402

CASES = {
    "cavity32": dict(n=32, tet=False, jitter=0.0, seed=0, checkpoints=(15, 50, 100, 200), sample_at=(200,)),
    "cavity128": dict(n=128, tet=False, jitter=0.2, seed=0, checkpoints=(5, 10, 20, 40, 100, 200, 300, 400, 500),
                      sample_at=(40, 200, 500)),
}
FIELDS = ("u", "v", "w", "p")
STRIDE = 1021
NPROJ = 8
PROJ_SEED = 2024
JSON_PATH = os.path.join(HERE, "cavity_runs.json")
NPZ_PATH = os.path.join(HERE, "cavity_runs.npz")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def projection_signs(ne):
    rng = np.random.default_rng(PROJ_SEED)
    return rng.integers(0, 2, size=(NPROJ, ne), dtype=np.int8) * 2 - 1


def checkpoint_record(fields, ne, signs):
    rec = {"hash": {}, "l2": {}, "proj": {}}
    for f, a in fields.items():
        x = a[:ne]
        rec["hash"][f] = sha(a)
        rec["l2"][f] = float(np.linalg.norm(x))
        rec["proj"][f] = [float(v) for v in signs.astype(np.float64) @ x]
    return rec


def load():
    if os.path.exists(JSON_PATH):
        with open(JSON_PATH) as fh:
            meta = json.load(fh)
    else:
        meta = {"generator": "tests/golden/make_cavity_runs.py", "stride": STRIDE, "nproj": NPROJ,
                "proj_seed": PROJ_SEED, "cases": {}}
    samples = dict(np.load(NPZ_PATH)) if os.path.exists(NPZ_PATH) else {}
    return meta, samples


def save(meta, samples):
    with open(JSON_PATH, "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    np.savez_compressed(NPZ_PATH, **samples)


def run_case(key, meta, samples):
    spec = CASES[key]
    z = cfdl.Zone(spec["n"], spec["tet"], spec["jitter"], seed=spec["seed"])
    o = oracle_lib.Oracle(z, n_subdomains=1)
    o.physics_init(oracle_lib.steady(mode=1, tight_rtol=1e-13))
    signs = projection_signs(o.ne)
    rec = {"n": spec["n"], "tet": spec["tet"], "jitter": spec["jitter"], "seed": spec["seed"],
           "config": "steady rho 1 mu 0.01 alpha_u 0.7 alpha_p 0.3, tight 1e-13, ncoef 3", "ne": o.ne,
           "threads": oracle_lib.num_threads(), "checkpoints": {}}
    meta["cases"][key] = rec
    done, t0 = 0, time.time()
    for k in spec["checkpoints"]:
        st = o.run(k - done, 3)
        done = k
        fields = {f: o.get(f) for f in FIELDS}
        cp = checkpoint_record(fields, o.ne, signs)
        cp["iters"] = [st.it_u, st.it_v, st.it_w, st.it_p]
        cp["seconds"] = round(time.time() - t0, 1)
        rec["checkpoints"][str(k)] = cp
        if k in spec["sample_at"]:
            for f, a in fields.items():
                samples["%s_%d_%s" % (key, k, f)] = a[:o.ne:STRIDE].copy()
        save(meta, samples)
        print("%s: %d outer iterations, %.0f s, iters %s" % (key, k, time.time() - t0, cp["iters"]), flush=True)
    o.close()


def main():
    keys = sys.argv[1:] or list(CASES)
    meta, samples = load()
    for key in keys:
        run_case(key, meta, samples)


if __name__ == "__main__":
    main()
