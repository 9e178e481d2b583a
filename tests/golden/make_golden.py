"""Regenerate tests/golden/*.json from the CPU oracle.

The reference ships no tests, fixtures or sample mesh, and cannot be built
here (no Fortran compiler, no libcgns), so these fixtures pin the oracle's
restatement against regressions and across machines (the oracle uses only
IEEE +,-,*,/,sqrt without contraction, so x86 and aarch64 agree bit for bit).

    python tests/golden/make_golden.py
"""
import hashlib
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "cfd-lite_gb300"), os.path.join(ROOT, "tests")]

import cfdl  # noqa: E402
import oracle_lib  # noqa: E402

SETUP_CASES = {"hex4_j20": (4, False, 0.2, 7), "hex8_j20": (8, False, 0.2, 7),
               "tet3_j0": (3, True, 0.0, 7), "tet5_j10": (5, True, 0.1, 11),
               "prism4_j20": (4, "prism", 0.2, 7), "pyramid3_j10": (3, "pyramid", 0.1, 5),
               "mixed4_j20": (4, "mixed", 0.2, 9)}
INT_NAMES = ("ef2nb1", "ef2nb2", "ef2nb_idx", "s2g", "bs", "red", "gf2g", "g2gf", "g2gf_idx")
DBL_NAMES = ("aip", "rip", "xc", "yc", "zc", "vol")

# (n, tet, jitter, seed, config kwargs, outer iterations)
PHYS_CASES = {
    "ref_hex6_transient": (6, False, 0.2, 7, dict(rho=5.0, mu=0.01, dt=0.01, mode=0), 9),
    "ref_hex5_steady": (5, False, 0.1, 3, dict(rho=1.0, mu=0.01, dt=math.inf, alpha_u=0.7, alpha_p=0.3, mode=0), 12),
    "ref_tet3_transient": (3, True, 0.0, 5, dict(rho=1.0, mu=0.01, dt=0.01, mode=0), 6),
}
# with the energy equation solved after solve_uvwp in every pass
ENERGY_CASES = {
    "energy_hex5_transient": (5, False, 0.2, 7, dict(rho=5.0, mu=0.01, dt=0.01, mode=0), 9),
    "energy_mixed4_steady": (4, "mixed", 0.1, 3, dict(rho=1.0, mu=0.01, dt=math.inf, alpha_u=0.7, alpha_p=0.3,
                                                    mode=0), 10),
}
FIELDS = ("u", "v", "w", "p", "mip", "gp", "gu")
ENERGY_FIELDS = ("t", "e", "ge")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    setup = {}
    for key, (n, tet, jit, seed) in SETUP_CASES.items():
        z = cfdl.Zone(n, tet, jit, seed=seed)
        o = oracle_lib.Oracle(z, n_subdomains=4)
        setup[key] = {"n": n, "tet": tet, "jitter": jit, "seed": seed,
                      "int": {nm: sha(o.get_int(nm)) for nm in INT_NAMES},
                      "dbl": {nm: sha(o.get(nm)) for nm in DBL_NAMES}}
    with open(os.path.join(HERE, "setup_hashes.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": setup}, fh, indent=1, sort_keys=True)

    phys = {}
    cases = [(k, v, False) for k, v in PHYS_CASES.items()] + [(k, v, True) for k, v in ENERGY_CASES.items()]
    for key, (n, tet, jit, seed, kw, nout), energy in cases:
        z = cfdl.Zone(n, tet, jit, seed=seed)
        o = oracle_lib.Oracle(z, n_subdomains=4)
        o.physics_init(oracle_lib.config(**kw))
        if energy:
            o.energy_init()
        st = o.run(nout, 3)
        names = FIELDS + (ENERGY_FIELDS if energy else ())
        rec = {"n": n, "tet": tet, "jitter": jit, "seed": seed, "config": kw, "n_outer": nout,
               "iters": [st.it_u, st.it_v, st.it_w, st.it_p],
               "hash": {f: sha(o.get(f)) for f in names},
               "l2": {f: float(np.linalg.norm(o.get(f))) for f in names}}
        if energy:
            rec["energy"] = True
            rec["iters_e"] = st.it_e
        phys[key] = rec
    with open(os.path.join(HERE, "oracle_runs.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": phys}, fh, indent=1, sort_keys=True,
                  default=lambda x: "inf" if x == math.inf else x)
    print("wrote", len(setup), "set-up and", len(phys), "physics fixtures")


if __name__ == "__main__":
    main()
