"""Seeded synthetic workloads of the batched and served cavity benchmarks.

Batched: `count` independent lid-driven cavity cases drawn from one seed --
edge N uniform in {n_lo..n_hi} (N^3 hex cells), half of the cases (a seeded
choice) split into 6 tets per hex, Reynolds number log-uniform in
[re_lo, re_hi] (rho = 1, lid speed 1, mu = 1/Re).

Served: a Poisson stream of cavity-solve requests -- exponential
inter-arrival times at `rate` requests/s, edge N uniform in {n_lo..n_hi}, hex
or tet-split with equal odds, Re log-uniform in [re_lo, re_hi].
"""
import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np


def batched_cases(seed=0, count=64, n_lo=16, n_hi=64, re_lo=10.0, re_hi=1000.0):
    rng = np.random.default_rng(seed)
    n = rng.integers(n_lo, n_hi + 1, size=count)
    tet = np.zeros(count, dtype=bool)
    tet[rng.permutation(count)[: count // 2]] = True
    re = np.exp(rng.uniform(math.log(re_lo), math.log(re_hi), size=count))
    return [dict(n=int(n[i]), tet=bool(tet[i]), re=float(re[i])) for i in range(count)]


def served_requests(seed=0, count=16, rate=5.0, n_lo=24, n_hi=96, re_lo=10.0, re_hi=1000.0):
    rng = np.random.default_rng(seed)
    n = rng.integers(n_lo, n_hi + 1, size=count)
    tet = rng.random(count) < 0.5
    re = np.exp(rng.uniform(math.log(re_lo), math.log(re_hi), size=count))
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps) - gaps[0]
    return [dict(n=int(n[i]), tet=bool(tet[i]), re=float(re[i]), t=float(t[i])) for i in range(count)]


def cells(case):
    return case["n"] ** 3 * (6 if case["tet"] else 1)


def build_setups(cases, jitter=0.0, seed=0, threads=16):
    """Zones and mesh set-ups of the cases, built on host threads (the set-up
    runs in the library, outside the interpreter lock)."""
    import cfdl

    def one(c):
        return cfdl.Setup(cfdl.Zone(c["n"], c["tet"], jitter, seed=seed))

    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, cases))
