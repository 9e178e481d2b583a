#!/usr/bin/env python
"""Benchmark of the CFD-Lite SIMPLE outer iteration on GB300.

Workload (the reference-cavity configuration the metric is quoted on): the
lid-driven cavity in the unit cube on n^3 = 128^3 hex cells (2.1M cells),
interior nodes jittered by a seeded U(-0.2, 0.2) cell spacing, rho = 1,
mu = 0.01 (Re = 100), SIMPLE with under-relaxation 0.7 (velocity) and 0.3
(pressure), FP64.  One step = one outer iteration: update_boundaries +
solve_uvwp (+ update_time every ncoef = 3), with every inner solve stopped,
as in the reference, at a 10x residual drop or nit = 100 iterations.
Synthetic mesh: the reference's own sample mesh is not available.

The working set (~3 GB) is far larger than the 129 MB L2, so no L2 flush is
needed between steps.  Device time is taken with CUDA events on the solver's
own stream; `e2e` repeats the measurement through the host-array drop-in
(pinned host buffers uploaded and downloaded every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cfd-lite_gb300")
sys.path.insert(0, PKG)

METRIC = "SIMPLE cell-iters/s"
DTYPES = {0: "f64", 1: "f64+f32 (mixed pressure solve)",
          2: "f64+f32 (mixed pressure solve, FP32 momentum corrections)",
          3: "f64+f32 (mixed pressure solve, FP32 momentum corrections, FP32 explicit momentum face terms)"}
UNIT = "cell-iters/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--edge", dest="n", type=int, default=128, help="mesh edge: n^3 hex cells")
    ap.add_argument("--jitter", type=float, default=0.2)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tet", action="store_true")
    ap.add_argument("--mode", type=int, default=0, help="0: reference stopping rule, 1: tight")
    ap.add_argument("--precision", type=int, default=0, help="0: FP64, 1: mixed pressure solve, "
                    "2: also FP32 momentum corrections")
    ap.add_argument("--precond", type=int, default=1, help="pressure preconditioner: 0 Jacobi, 1 AMG")
    ap.add_argument("--eager", action="store_true", help="launch kernels one by one instead of the graph")
    ap.add_argument("--tile", type=int, default=0, help="solver tile shape (1, 2, 4, 8) instead of the autotuner's "
                    "choice (fewer launches, e.g. for a profiler's launch list)")
    ap.add_argument("--breakdown", action="store_true", help="print the per-kernel table to stderr")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="cavity",
                    choices=["cavity", "batched", "converged", "served", "pressure", "setup", "energy"],
                    help="cavity: one case (default); batched: 64 uneven cases in one run; served: request stream")
    ap.add_argument("--cases", type=int, default=64, help="batched: number of cases")
    ap.add_argument("--outer", type=int, default=300, help="batched: outer iterations per case")
    ap.add_argument("--forms", default="0,1,2,3", help="batched/served: precisions to run (0 FP64, 1 mixed pressure, "
                    "2 mixed pressure + FP32 momentum corrections, 3 also FP32 explicit momentum face terms)")
    ap.add_argument("--rates", default="5,20,50,100,200", help="served: request rates (req/s)")
    ap.add_argument("--requests", type=int, default=200, help="served: requests per rate")
    ap.add_argument("--err-sample", type=int, default=16, help="served: requests checked against FP64 converged "
                    "references")
    ap.add_argument("--max-outer", type=int, default=1000, help="served: outer-iteration cap per request")
    ap.add_argument("--conv-tol", type=float, default=1e-6, help="served/converged: mass-ratio tolerance")
    ap.add_argument("--ref-tol", type=float, default=1e-11, help="converged: mass ratio of the FP64 reference")
    ap.add_argument("--field-tol", type=float, default=1e-6, help="converged: rel L2 target against the reference")
    ap.add_argument("--chunk", type=int, default=20, help="converged: outer iterations between field checks")
    ap.add_argument("--conv-cap", type=int, default=16000, help="converged: outer-iteration cap per case")
    ap.add_argument("--n-range", default="", help="batched/served: override the mesh-edge range lo,hi")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed
class Dist:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)])
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)])
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi samples during the timed region (read-only query)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler is producing lines
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                if os.path.getsize(self.path) > 0:
                    break
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1])); smax.append(float(f[2]))
                except ValueError:
                    continue
                for k, nm in enumerate(names):
                    if f[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic(kernel, n, precision=0):
    """DRAM bytes per launch from a committed ncu summary (profiles/ncu_traffic.txt:
    lines 'kernel n_cells bytes_per_launch [precision]', precision 0 when
    absent), scaled to n^3 cells when the capture was taken on a smaller mesh;
    None when there is no capture of that kernel at that precision."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    best = None
    with open(path) as fh:
        for line in fh:
            f = line.split()
            if line.startswith("#") or len(f) < 3 or f[0] != kernel:
                continue
            if (int(f[3]) if len(f) >= 4 else 0) == precision:
                best = (int(f[1]), float(f[2]))
    if not best:
        return None
    cells, b = best
    return b * (n ** 3) / cells


# ---------------------------------------------------------------- our arm
def run_ours(a, dist):
    import numpy as np
    import cfdl
    from bytes_model import kernel_bytes

    cfdl.select_device(dist.local)
    zone = cfdl.Zone(a.n, a.tet, a.jitter, seed=a.seed)
    setup = cfdl.Setup(zone)
    cfg = cfdl.steady(solve_mode=a.mode, precision=a.precision, precond=a.precond)
    g = cfdl.Solver(setup, cfg)
    g.set_graph_mode(not a.eager)
    W = 4 if a.tet else 6
    ne, nf, nbf = setup.ne, setup.nf, setup.nbf
    state = {"it": 0}

    def step():
        g.update_boundaries()
        g.solve_uvwp(stats=False)
        state["it"] += 1
        if state["it"] % 3 == 0:
            g.update_time()

    for _ in range(a.warmup):
        step()
    if a.tile:
        g.set_tile(a.tile)
        tile, tile_ms = a.tile, {}
    else:
        tile, tile_ms = g.autotune(outer=2)     # solver tile shape by measurement (state restored)
    for _ in range(2):
        step()
    clocks = Clocks(dist.local)
    dist.barrier()
    g.timer_begin()
    clocks.start()
    l0 = g.launch_count()
    for _ in range(a.steps):
        step()
    ms = g.timer_end()
    launches = g.launch_count() - l0
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    cells_total = dist.sum(ne * a.steps)
    value = cells_total / (ms_max / 1e3)
    st = g.solve_uvwp() if False else g.last_stats

    # roofline: find the dominant kernel, then time its launches alone
    g.profile_start(None)
    for _ in range(min(3, a.steps)):
        step()
    prof = g.profile_stop()
    dominant = max(prof.items(), key=lambda kv: kv[1][1])[0]
    g.profile_start(dominant)
    for _ in range(a.steps):
        step()
    dp = g.profile_stop()[dominant]
    avg_s = dp[1] / dp[0] / 1e3
    peaks, peak_kind = measured_peaks()
    nbytes = kernel_bytes(dominant, ne, nf, nbf, W)
    if nbytes is None:
        import ctypes as C
        from bytes_model import amg_kernel_bytes
        nl = C.c_int()
        ns, ws = (C.c_int * 16)(), (C.c_int * 16)()
        cfdl._check(cfdl.lib().cfdl_amg_info(g._h, 15, C.byref(nl), ns, ws), "amg_info")
        levels = [(ns[l], ws[l]) for l in range(nl.value + 1)]
        val = 4 if (a.precision >= 1 and (dominant.startswith("k_v_") or dominant.startswith("k_mx_"))) else 8
        # bytes per mesh-level neighbour index (16-bit offsets in the FP32 kernels when they fit)
        ib = cfdl.lib().cfdl_amg_index_bytes(g._h) if val == 4 else 4
        nbytes = amg_kernel_bytes(dominant, levels, val, ib=ib)
    achieved = nbytes / avg_s / 1e9 if nbytes else None
    traffic = ncu_traffic(dominant, a.n, a.precision)
    # the FP64 pipe's ceiling: the probe's DFMA rate on this device, and each
    # FP64-bound kernel's FP64 instructions per launch (flops_model) over its
    # average launch time from the profile pass above
    fp64 = fp64_roofline(cfdl, prof, ne, nf, nbf, W, peaks) if a.precision == 0 else None
    breakdown = {k: {"launches": c, "ms": round(t, 3), "share": round(t / sum(v[1] for v in prof.values()), 4)}
                 for k, (c, t) in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    if a.breakdown and dist.rank == 0:
        sys.stderr.write(json.dumps(breakdown, indent=1) + "\n")

    # inner iteration counts of the last step
    g.update_boundaries()
    stl = g.solve_uvwp()

    # end to end through the host-array drop-in: every step uploads the fields
    # a Fortran host owns and may change between calls (u, v, w, p) from pinned
    # host buffers and downloads everything the outer iteration writes (the
    # same plus their gradients, gpc and mip).  The gradients and face fluxes
    # are the solver's own state, which such a host only reads: it declares
    # them unchanged (cfdl_step_host_keep), so they are not uploaded again.
    e2e = None
    if not a.no_e2e:
        import torch
        import ctypes as C
        nc = ne + nbf
        sizes = {"u": nc, "v": nc, "w": nc, "p": nc, "gu": 3 * nc, "gv": 3 * nc, "gw": 3 * nc, "gp": 3 * nc,
                 "gpc": 3 * nc, "mip": nf}
        host = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for k, n in sizes.items()}
        fl = cfdl.Fields(**{k: v.ctypes.data_as(C.c_void_p) for k, v in host.items()})
        L = cfdl.lib()
        cfdl._check(L.cfdl_download_fields(g._h, C.byref(fl)), "download")
        kept = ("gu", "gv", "gw", "gp", "gpc", "mip")
        keep = sum(cfdl.FIELD_BITS[k] for k in kept)
        h2d = sum(v.nbytes for k, v in host.items() if k not in kept)
        d2h = sum(v.nbytes for v in host.values())

        def e2e_step():
            cfdl._check(L.cfdl_step_host_keep(g._h, C.byref(fl), keep, 1, 0, None), "step_host_keep")

        for _ in range(2):
            e2e_step()
        dist.barrier()
        t0 = time.perf_counter()
        g.timer_begin()
        for _ in range(a.steps):
            e2e_step()
        ms_e = g.timer_end()
        wall = time.perf_counter() - t0
        ms_e = max(ms_e, wall * 1e3)
        ms_e = dist.max(ms_e)
        # the host link alone: the upload, and the part of the download that
        # cannot overlap the pressure correction (p, gp, gpc, mip)
        def wall_ms(fn, reps=5):
            fn()
            t = time.perf_counter()
            for _ in range(reps):
                fn()
            return (time.perf_counter() - t) * 1e3 / reps
        up = cfdl.Fields(**{k: v.ctypes.data_as(C.c_void_p) for k, v in host.items() if k not in kept})
        late_keys = ("p", "gp", "gpc", "mip")
        late = cfdl.Fields(**{k: host[k].ctypes.data_as(C.c_void_p) for k in late_keys})
        ms_up = wall_ms(lambda: cfdl._check(L.cfdl_upload_fields(g._h, C.byref(up)), "upload"))
        ms_dn = wall_ms(lambda: cfdl._check(L.cfdl_download_fields(g._h, C.byref(fl)), "download"))
        ms_late = ms_dn * sum(host[k].nbytes for k in late_keys) / d2h
        e2e = {"value": dist.sum(ne * a.steps) / (ms_e / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "api": "cfdl_step_host_keep (upload of u, v, w, p; update_boundaries + solve_uvwp; overlapped "
                      "download of all fields; gradients and mip declared unchanged by the host)",
               "ms_per_step": ms_e / a.steps,
               "link": {"h2d_gbs": h2d / ms_up / 1e6, "d2h_gbs": d2h / ms_dn / 1e6,
                        "floor_ms_per_step": ms_max / a.steps + ms_up + ms_late,
                        "floor": "device step + upload + non-overlapped download (p, gp, gpc, mip)"}}

    cpu = None
    if not a.no_cpu and dist.rank == 0 and dist.world == 1:
        cpu = cpu_baseline(a, budget_s=20.0)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES[a.precision],
        "data": "synthetic (seeded jittered unit-cube hex mesh; the reference's sample mesh is unavailable)",
        "config": {"workload": "lid-driven cavity %d^3 %s, jitter %.2f, Re=100 (rho=1, mu=0.01), SIMPLE "
                               "alpha_u=0.7 alpha_p=0.3, FP64" % (a.n, "tet-split" if a.tet else "hex", a.jitter),
                   "cells": ne, "faces": nf, "inner_solve": "10x residual drop / nit=100" if a.mode == 0 else "tight 1e-13",
                   "pressure_precond": ["jacobi", "amg"][a.precond], "tile": tile,
                   "coarse_group": g.get_coarse_group(),
                   "autotune_ms_per_outer": {str(k): round(v, 3) for k, v in tile_ms.items()},
                   "parallelism": "replicas" if dist.world > 1 else "single",
                   "l2": "working set > L2 (no flush needed)"},
        "gpu_launches": launches // max(1, 1),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
                     "traffic": traffic, "algorithmic_bytes": nbytes, "avg_launch_us": avg_s * 1e6,
                     "launches": dp[0], "peak_source": peak_kind},
        "inner_iterations": {"u": stl.it_u, "v": stl.it_v, "w": stl.it_w, "pc": stl.it_p},
        "kernel_shares": {k: v["share"] for k, v in list(breakdown.items())[:8]},
    }
    if fp64:
        out["fp64_roofline"] = fp64
    if clk:
        out["clocks"] = clk
    if e2e:
        out["e2e"] = e2e
    if cpu:
        out["cpu_baseline"] = cpu
    g.close()
    return out


def fp64_roofline(cfdl, prof, ne, nf, nbf, W, peaks):
    """FP64-pipe roofline of the kernels the flops model covers: FP64
    thread-instructions per launch / average launch time (the profile pass's
    CUDA events) against the probe's measured DFMA rate, beside each kernel's
    HBM fraction (its algorithmic bytes over the same time)."""
    from bytes_model import kernel_bytes
    try:
        from flops_model import fp64_inst
        rate, probe_ms = cfdl.probe_fp64()
    except Exception as e:          # no model or no probe: no FP64 ceiling in the line
        return {"unavailable": str(e)[:200]}
    rows = {}
    for k, (launches, ms) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
        inst = fp64_inst(k, ne, nf, nbf, W)
        if not inst or not launches:
            continue
        t = ms / launches / 1e3
        nb = kernel_bytes(k, ne, nf, nbf, W)
        rows[k] = {"fp64_inst_per_launch": inst, "avg_launch_us": round(t * 1e6, 2),
                   "fp64_frac": round(inst / t / rate, 3),
                   "hbm_frac": round(nb / t / 1e9 / peaks["hbm_gbs"], 3) if nb else None}
    return {"peak_fp64_inst_per_s": rate, "peak_fp64_tflops": 2 * rate / 1e12, "probe_ms": probe_ms,
            "peak_source": "measured (cfdl_probe_fp64: DFMA chains on every SM)", "kernels": rows}


# ---------------------------------------------------------- CPU reference
def oracle_case(a):
    """The reference algorithm's case, built entirely by the oracle: its own
    hex cavity zone (the same zone as the product's generator, tests/
    test_setup.py) and its own restatement of the reference's set-up, four
    subdomains, mode 0.  A tet-split mesh takes the product's zone as input
    (the oracle has no tet generator) and still the oracle's own set-up."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    if a.tet:
        import cfdl
        zone = cfdl.Zone(a.n, a.tet, a.jitter, seed=a.seed)
    else:
        zone = oracle_lib.BoxZone(a.n, a.jitter, a.seed)
    o = oracle_lib.Oracle(zone, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=0))
    return o, oracle_lib


def host_cpu():
    """The host's CPU model and logical core count, for the CPU baselines."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        try:
            with open("/proc/cpuinfo") as fh:
                for line in fh:
                    if line.lower().startswith("model name"):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"cpu": model or "unknown", "nproc": os.cpu_count()}


def cpu_baseline(a, budget_s=20.0):
    """The reference algorithm (CPU oracle, ref mode: Gauss-Seidel / 4-block
    SSOR inner solves, nsubd = 4) on the host's cores: its Gauss-Seidel
    sweeps are sequential, as in the reference; the loops whose iterations are
    independent (assembly, gradients, fluxes, corrections, the four pressure
    blocks) run on all host threads.  Timed over a bounded number of outer
    iterations of the same mesh."""
    o, oracle_lib = oracle_case(a)
    t0 = time.perf_counter()
    o.run(1, 3)                       # untimed warm iteration
    t1 = time.perf_counter() - t0
    k = max(1, min(4, int(budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.run(k, 3)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": o.ne * k / dt, "unit": UNIT, "cores": oracle_lib.num_threads(), "kind": "port", "host": host_cpu(),
            "sample": "%d outer iteration(s) of the full %d-cell mesh after 1 warm-up iteration, %.1f s; Gauss-Seidel "
                      "sweeps sequential, independent loops on %d threads" % (k, o.ne, dt, oracle_lib.num_threads())}


def run_reference(a, dist):
    if dist.rank != 0:
        return None
    o, oracle_lib = oracle_case(a)
    threads = oracle_lib.num_threads()
    t0 = time.perf_counter()
    o.run(1, 3)
    t_it = time.perf_counter() - t0
    warm = max(0, min(a.warmup, 1) - 1)
    if warm:
        o.run(warm, 3)
    steps = max(1, min(a.steps, int(150.0 / max(t_it, 1e-3))))
    t0 = time.perf_counter()
    o.run(steps, 3)
    dt = time.perf_counter() - t0
    value = o.ne * steps / dt
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
           "steps": steps, "steps_requested": a.steps, "warmup": 1 + warm, "ms_per_step": dt / steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded jittered unit-cube hex mesh)",
           "config": {"workload": "lid-driven cavity %d^3 %s, jitter %.2f, Re=100, SIMPLE alpha 0.7/0.3, FP64"
                                  % (a.n, "tet-split" if a.tet else "hex", a.jitter), "cells": o.ne},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "host": host_cpu(),
                            "sample": "%d outer iterations of the full mesh (reference algorithm: Gauss-Seidel "
                                      "sweeps sequential, independent loops on %d threads), %.1f s"
                                      % (steps, threads, dt)},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    o.close()
    return out


# ------------------------------------------------------------ batched cases
def run_batched(a, dist):
    """Uneven cases in one context, every outer iteration of every case in
    one graph launch (cfdl_run), one JSON line per pressure-solve form."""
    import numpy as np
    import cfdl
    import workloads

    cfdl.select_device(dist.local)
    kw = {}
    if a.n_range:
        lo, hi = (int(x) for x in a.n_range.split(","))
        kw = dict(n_lo=lo, n_hi=hi)
    cases = workloads.batched_cases(seed=a.seed, count=a.cases, **kw)
    t0 = time.perf_counter()
    setups = workloads.build_setups(cases)
    t_setup = time.perf_counter() - t0
    total_cells = sum(s.ne for s in setups)
    forms = [int(x) for x in a.forms.split(",")]
    fields = {}
    lines = []
    for prec in forms:
        cfgs = [cfdl.steady(mu=1.0 / c["re"], precision=prec) for c in cases]
        t0 = time.perf_counter()
        b = cfdl.Batch(setups, cfgs)
        t_create = time.perf_counter() - t0
        best, tune_ms = b.autotune(outer=2)
        # warm-up passes (graph build, multigrid set-up), then the timed run
        b.set_run(a.warmup)
        b.run(a.warmup)
        b.set_run(a.outer)
        clocks = Clocks(dist.local)
        dist.barrier()
        clocks.start()
        l0 = b.launch_count()
        b.timer_begin()
        t0 = time.perf_counter()
        left = b.run(a.outer)
        ms = b.timer_end()
        wall = time.perf_counter() - t0
        launches = b.launch_count() - l0
        clk = clocks.stop()
        ms = dist.max(max(ms, 0.0))
        ids = b.ids()
        stats = [b.case_stats(c) for c in ids]
        assert left == 0 and all(st.outer_done == a.outer for st in stats)
        value = dist.sum(total_cells * a.outer) / (ms / 1e3)
        fields[prec] = [{f: b.case_get(c, f) for f in ("u", "v", "w", "p")} for c in ids]
        # end to end: host fields in, the run, host fields out
        nb_in = sum((4 * (s.ne + s.nbf) + s.nf) * 8 for s in setups)
        nb_out = sum(4 * (s.ne + s.nbf) * 8 for s in setups)
        host = [{f: fields[prec][k][f].copy() for f in ("u", "v", "w", "p")} for k in range(len(ids))]
        mips = [b.case_get(c, "mip") for c in ids]
        b.set_run(a.outer)
        t0 = time.perf_counter()
        for k, c in enumerate(ids):
            for f in ("u", "v", "w", "p"):
                b.case_set(c, f, host[k][f])
            b.case_set(c, "mip", mips[k])
        b.run(a.outer)
        for k, c in enumerate(ids):
            for f in ("u", "v", "w", "p"):
                host[k][f] = b.case_get(c, f)
        e2e_s = dist.max(time.perf_counter() - t0)
        b.close()
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.outer,
            "warmup": a.warmup, "ms_per_step": ms / a.outer, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPES[prec],
            "data": "synthetic (seeded cavity meshes)",
            "config": {"workload": "batched: %d lid-driven cavity cases in one run, N~U{%d..%d} (seed %d), half "
                                   "tet-split, Re log-U[10,1000], %d SIMPLE iterations each" %
                                   (len(cases), min(c["n"] for c in cases), max(c["n"] for c in cases), a.seed,
                                    a.outer),
                       "cases": len(cases), "cells": total_cells, "tile": best,
                       "autotune_ms_per_outer": {str(k): round(v, 3) for k, v in tune_ms.items()},
                       "l2": "working set > L2 (no flush needed)", "parallelism": "single"},
            "gpu_launches": launches,
            "wall_s": wall, "host_setup_s": t_setup, "batch_create_s": t_create,
            "e2e": {"value": dist.sum(total_cells * a.outer) / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nb_in,
                    "d2h_bytes_per_step": nb_out, "step": "one run of %d outer iterations" % a.outer,
                    "api": "cfdl_case_set_array + cfdl_run + cfdl_case_get_array"},
        }
        if clk:
            out["clocks"] = clk
        lines.append(out)
    if 0 in fields:
        for out, prec in zip(lines, forms):
            if prec == 0:
                continue
            worst = {}
            for f in ("u", "v", "w", "p"):
                worst[f] = max(float(np.linalg.norm(m[f] - d[f]) / max(np.linalg.norm(d[f]), 1e-300))
                               for m, d in zip(fields[prec], fields[0]))
            out["vs_fp64_rel_l2_max_over_cases_after_run"] = worst
    return lines


# ------------------------------------------- batched, to the converged state
def converged_reference(setups, cases, tol, cap, tile=0):
    """The FP64 converged state of each case: the plain FP64 form run in one
    batch for cap outer iterations, a case stopping early once its mass ratio
    (mass imbalance / sum |mip|) is at or below tol (tol 0: never).  These
    fields stand in for the oracle's converged fields: the
    FP64 GPU path reproduces the oracle within 1e-9 per outer iteration in
    tight mode (tests/test_gpu_configs.py, test_gpu_parity.py) and the
    converged states agree within 1e-6 (tests/test_gpu_converged.py), while
    the oracle itself needs hours per case at these sizes."""
    import cfdl
    b = cfdl.Batch(setups, [cfdl.steady(mu=1.0 / c["re"], precision=0) for c in cases])
    if tile:
        b.set_tile(tile)
    b.set_run(cap, 0, tol)
    left = b.run(cap)
    ids = b.ids()
    stats = [b.case_stats(c) for c in ids]
    ref = [{f: b.case_get(c, f) for f in ("u", "v", "w", "p")} for c in ids]
    b.close()
    return ref, stats, left


def run_converged(a, dist):
    """The mixed forms against plain FP64 on one converged target: the
    batched cases (64 uneven cavities, N~U{16..64}, half tet-split, Re
    log-U[10,1000]) until each case's u, v, w and p are within --field-tol
    (relative L2, default 1e-6) of its FP64 converged state
    (converged_reference).  Each form runs from the initial state in timed
    graph launches of a few outer iterations; after each the cases within
    the tolerance are stopped.  The summed device time of the launches is the
    form's time to solution.  One JSON line per form, printed as it ends."""
    import numpy as np
    import cfdl
    import workloads

    cfdl.select_device(dist.local)
    kw = {}
    if a.n_range:
        lo, hi = (int(x) for x in a.n_range.split(","))
        kw = dict(n_lo=lo, n_hi=hi)
    cases = workloads.batched_cases(seed=a.seed, count=a.cases, **kw)
    setups = workloads.build_setups(cases)
    total_cells = sum(s_.ne for s_ in setups)
    cap = a.conv_cap
    # the FP64 form's tile shape first: the reference runs with it, so that the
    # FP64 form's timed run repeats the reference's arithmetic exactly
    b = cfdl.Batch(setups, [cfdl.steady(mu=1.0 / c["re"], precision=0) for c in cases])
    tile0, _ = b.autotune(outer=2)
    b.close()
    # the reference runs every case the whole cap, with no early stop: a mass
    # ratio of 1e-11 can still leave the fields 1e-4 from their limit on the
    # slowest cases (measured), while after the cap the mass ratio is at
    # rounding level (1e-15 and below)
    t0 = time.perf_counter()
    ref, ref_stats, ref_left = converged_reference(setups, cases, 0.0, cap, tile=tile0)
    t_ref = time.perf_counter() - t0
    ref_ratio = max(st.mass_ratio for st in ref_stats)

    def errors(b, ids, which):
        out = {}
        for k in which:
            e = 0.0
            for f in ("u", "v", "w", "p"):
                x, r = b.case_get(ids[k], f)[:setups[k].ne], ref[k][f][:setups[k].ne]
                e = max(e, float(np.linalg.norm(x - r) / max(np.linalg.norm(r), 1e-300)))
            out[k] = e
        return out

    t_fp64 = None
    for prec in [int(x) for x in a.forms.split(",")]:
        cfgs = [cfdl.steady(mu=1.0 / c["re"], precision=prec) for c in cases]
        if prec == 0:
            best = tile0
        else:
            b = cfdl.Batch(setups, cfgs)
            best, _ = b.autotune(outer=2)
            b.close()
        # one pass from the initial state: runs of --chunk outer iterations,
        # then of 5% of those done, each one graph launch timed on the device;
        # after each run the cases within the tolerance are stopped (their
        # count is at most one run above the least they need).  The host's
        # checks between runs are outside the timed launches.
        b = cfdl.Batch(setups, cfgs)
        b.set_tile(best)
        ids = b.ids()
        b.set_run(0, 0, 0.0)
        b.run(0)                         # builds the run graph outside the timing
        need, done_it, ms, launches = {}, 0, 0.0, 0
        todo = list(range(len(ids)))
        clocks = Clocks(dist.local)
        clocks.start()
        while todo and done_it < cap:
            step = min(max(a.chunk, done_it // 20), cap - done_it)
            for k in range(len(ids)):
                b.set_run(step if k in todo else 0, 0, 0.0, cid=ids[k])
            l0 = b.launch_count()
            b.timer_begin()
            b.run(step)
            ms += b.timer_end()
            launches += b.launch_count() - l0
            done_it += step
            for k, e in errors(b, ids, todo).items():
                if e <= a.field_tol:
                    need[k] = done_it
            todo = [k for k in todo if k not in need]
        clk = clocks.stop()
        for k in todo:
            need[k] = cap
        final = errors(b, ids, range(len(ids)))
        ratios = [b.case_stats(c).mass_ratio for c in ids]
        b.close()
        ms = dist.max(ms)
        iters = [need[k] for k in range(len(ids))]
        cell_iters = sum(s_.ne * n for s_, n in zip(setups, iters))
        errs = list(final.values())
        if prec == 0:
            t_fp64 = ms
        out = {
            "metric": "batched time to the FP64 converged fields within %.0e" % a.field_tol, "value": ms / 1e3,
            "unit": "s", "higher_is_better": False, "n_gpus": dist.world, "dtype": DTYPES[prec],
            "data": "synthetic (seeded cavity meshes)",
            "config": {"workload": "batched to convergence: %d lid-driven cavity cases, N~U{%d..%d} (seed %d), half "
                                   "tet-split, Re log-U[10,1000], each run until u, v, w, p are within %.0e (rel L2) "
                                   "of its FP64 converged state" %
                                   (len(cases), min(c["n"] for c in cases), max(c["n"] for c in cases), a.seed,
                                    a.field_tol),
                       "cases": len(cases), "cells": total_cells, "tile": best, "chunk": a.chunk, "cap": cap,
                       "reference": "the FP64 form, %d outer iterations of every case (largest mass ratio after "
                                    "them %.1e, %.0f s)" % (cap, ref_ratio, t_ref)},
            "cell_iters_per_s": cell_iters / (ms / 1e3),
            "cases_within_tol": int(sum(e <= a.field_tol for e in errs)),
            "outer_iterations": {"min": int(min(iters)), "median": float(np.median(iters)), "max": int(max(iters)),
                                 "total_cell_iters": cell_iters, "runs": "%d outer iterations in total" % done_it},
            "rel_l2_vs_fp64_converged": {"max": max(errs), "median": float(np.median(errs))},
            "not_within_tol": [{"case": k, "n": cases[k]["n"], "tet": cases[k]["tet"], "re": round(cases[k]["re"], 1),
                                "rel_l2": final[k], "mass_ratio_last_pass": ratios[k]}
                               for k in range(len(ids)) if final[k] > a.field_tol],
            "gpu_launches": launches,
        }
        if t_fp64 is not None and prec != 0:
            out["speedup_vs_fp64_time_to_solution"] = t_fp64 / ms
        if clk:
            out["clocks"] = clk
        yield out


# ------------------------------------------------------- pressure solve
def run_pressure(a, dist):
    """Seconds for one pressure-correction solve to a 1e-8 relative residual,
    FP64 AMG-PCG against the mixed form (FP32 AMG-PCG inside FP64 iterative
    refinement), on the same assembled system; then the per-field error of
    the mixed form against FP64 after the same outer iterations."""
    import numpy as np
    import cfdl

    cfdl.select_device(dist.local)
    n = a.n if a.n != 128 else 256
    mu = 0.0025
    t0 = time.perf_counter()
    zone = cfdl.Zone(n, a.tet, 0.1 if a.jitter == 0.2 else a.jitter, seed=a.seed)
    setup = cfdl.Setup(zone)
    t_setup = time.perf_counter() - t0
    base = dict(mu=mu, solve_mode=1, tight_rtol=1e-8, precond=1)
    g = cfdl.Solver(setup, cfdl.steady(precision=0, **base))
    g.step(a.warmup, ncoef=0)                      # a developed flow state
    names = ("u", "v", "w", "p", "u0", "v0", "w0", "gu", "gv", "gw", "gp", "gpc", "mip", "mip0")
    state = {f: g.get(f) for f in names}

    def assemble():
        for f, v in state.items():
            g.set(f, v)
        g.update_boundaries()
        g.calc_coef_uvw()
        g.solve_momentum()
        g.calc_grad("uvw")
        g.calc_mip(True)
        g.calc_coef_p()

    out_forms = {}
    for prec in (0, 1):
        g.set_config(cfdl.steady(precision=prec, **base))
        assemble()
        g.solve_pc()                               # warm: hierarchy, graph-free path
        times, st = [], None
        for _ in range(max(3, min(a.steps, 10))):
            assemble()
            g.timer_begin()
            st = g.solve_pc()
            times.append(g.timer_end())
        out_forms[prec] = {"ms": statistics.median(times), "iters": st.it_p, "res_rel": st.res_f[3] / st.res_i[3],
                           "phic": g.get("phic")}
    ref = out_forms[0]["phic"]
    err_pc = float(np.linalg.norm(out_forms[1]["phic"] - ref) / np.linalg.norm(ref))
    # fields after the same outer iterations with each form, from the same state
    fields = {}
    for prec in (0, 1):
        g.set_config(cfdl.steady(precision=prec, **base))
        for f, v in state.items():
            g.set(f, v)
        g.step(a.outer if a.outer != 300 else 5, ncoef=0)
        fields[prec] = {f: g.get(f) for f in ("u", "v", "w", "p")}
    field_err = {f: float(np.linalg.norm(fields[1][f] - fields[0][f]) / np.linalg.norm(fields[0][f]))
                 for f in ("u", "v", "w", "p")}
    ne = setup.ne
    g.close()
    out = {
        "metric": "pressure-correction solve time to 1e-8 relative residual", "value": out_forms[1]["ms"] / 1e3,
        "unit": "s", "higher_is_better": False, "n_gpus": dist.world, "dtype": "f64+f32 (mixed pressure solve)",
        "data": "synthetic (seeded jittered unit-cube hex mesh)",
        "config": {"workload": "pressure solve: cavity %d^3 hex (%d cells), jitter %.2f, Re=400 (mu=0.0025), "
                               "system of outer iteration %d" % (n, ne, 0.1 if a.jitter == 0.2 else a.jitter,
                                                                 a.warmup + 1),
                   "cells": ne, "host_setup_s": t_setup},
        "fp64": {"s": out_forms[0]["ms"] / 1e3, "pcg_iterations": out_forms[0]["iters"],
                 "final_rel_residual": out_forms[0]["res_rel"]},
        "mixed": {"s": out_forms[1]["ms"] / 1e3, "inner_iterations": out_forms[1]["iters"],
                  "final_rel_residual_fp64": out_forms[1]["res_rel"],
                  "phic_rel_l2_vs_fp64": err_pc},
        "speedup_mixed_vs_fp64": out_forms[0]["ms"] / out_forms[1]["ms"],
        "fields_rel_l2_mixed_vs_fp64_after_%d_outer" % (a.outer if a.outer != 300 else 5): field_err,
    }
    return out


# ------------------------------------------------------------ energy equation
def run_energy(a, dist):
    """The energy equation (src/equations/mod_energy.f90) on the cavity
    workload: one step = one solve_energy (calc_grad of t and phi,
    calc_coef_energy, the phi solve to the reference's 10x residual drop,
    calc_temperature) after an outer pass of solve_uvwp, so every solve sees a
    new flow field; value = cells x energy solves / s over the solve_energy
    calls alone.  Also: the outer pass with and without the energy solve, the
    dominant energy kernel against the HBM roofline, and the CPU oracle's
    solve_energy (the reference's Gauss-Seidel) on a bounded sample."""
    import cfdl
    from bytes_model import kernel_bytes

    cfdl.select_device(dist.local)
    zone = cfdl.Zone(a.n, a.tet, a.jitter, seed=a.seed)
    setup = cfdl.Setup(zone)
    cfg = cfdl.steady(solve_mode=a.mode, precision=a.precision, precond=a.precond)
    W = 4 if a.tet else 6
    ne, nf, nbf = setup.ne, setup.nf, setup.nbf
    g = cfdl.Solver(setup, cfg)
    g.set_graph_mode(not a.eager)
    g.energy_init()
    for _ in range(a.warmup):                  # developed flow and temperature
        g.step(1, ncoef=0)
    if a.tile:
        g.set_tile(a.tile)
        g.set_energy_tile(a.tile)
        tile = a.tile
    else:
        tile, _ = g.autotune(outer=2)          # solver and energy tile shapes by measurement (state restored)
    clocks = Clocks(dist.local)
    e_ms, o_ms, iters = [], [], []
    l0, launches_e = g.launch_count(), 0
    dist.barrier()
    clocks.start()
    for _ in range(a.steps):
        g.update_boundaries()
        g.timer_begin()
        g.solve_uvwp(stats=False)
        o_ms.append(g.timer_end())
        l1 = g.launch_count()
        g.timer_begin()
        st = g.solve_energy()
        e_ms.append(g.timer_end())
        launches_e += g.launch_count() - l1
        iters.append(st.it_e)
    clk = clocks.stop()
    dist.barrier()
    ms = dist.max(sum(e_ms))
    value = dist.sum(ne * a.steps) / (ms / 1e3)
    # per-kernel shares of the energy solve and the dominant kernel's launches
    g.profile_start(None)
    for _ in range(3):
        g.step(1, ncoef=0)
    prof = {k: v for k, v in g.profile_stop().items() if k.startswith("k_en_") or k == "k_grad2"}
    dominant = max(prof.items(), key=lambda kv: kv[1][1])[0]
    g.profile_start(dominant)
    for _ in range(a.steps):
        g.update_boundaries(); g.solve_uvwp(stats=False); g.solve_energy()
    dp = g.profile_stop()[dominant]
    avg_s = dp[1] / dp[0] / 1e3
    peaks, peak_kind = measured_peaks()
    nbytes = kernel_bytes(dominant, ne, nf, nbf, W)
    achieved = nbytes / avg_s / 1e9
    total = sum(v[1] for v in prof.values())
    shares = {k: round(t / total, 4) for k, (c, t) in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    per_launch = {k: {"launches": c, "avg_us": round(t / c * 1e3, 1),
                      "gbs": round(kernel_bytes(k, ne, nf, nbf, W) / (t / c / 1e3) / 1e9, 1)
                      if kernel_bytes(k, ne, nf, nbf, W) else None}
                  for k, (c, t) in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    energy_tile = g.get_energy_tile()
    # the outer pass without the energy equation, same mesh and state
    g2 = cfdl.Solver(setup, cfg)
    for _ in range(a.warmup):
        g2.step(1, ncoef=0)
    g2.timer_begin()
    for _ in range(a.steps):
        g2.update_boundaries(); g2.solve_uvwp(stats=False)
    ms_plain = g2.timer_end()
    g2.close()
    t_range = g.get("t")[:ne]
    g.close()
    cpu = None
    if not a.no_cpu and dist.rank == 0 and dist.world == 1:
        cpu = cpu_energy_baseline(a)
    ms_outer = statistics.median(o_ms)
    out = {
        "metric": "energy solve cell-updates/s", "value": value, "unit": "cells x solves/s",
        "n_gpus": dist.world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPES[a.precision],
        "data": "synthetic (seeded jittered unit-cube hex mesh)",
        "config": {"workload": "energy equation on the lid-driven cavity %d^3 %s, jitter %.2f, Re=100, hot lid "
                               "373 / walls 273, cp=1000, tc=5; solve_energy after each outer pass"
                               % (a.n, "tet-split" if a.tet else "hex", a.jitter),
                   "cells": ne, "inner_solve": "10x residual drop / nit=100" if a.mode == 0 else "tight 1e-13",
                   "tile": tile, "energy_tile": energy_tile,
                   "l2": "working set > L2 (no flush needed)"},
        "gpu_launches": launches_e,
        "energy_iterations_median": statistics.median(iters),
        "outer_pass_ms": {"solve_uvwp": ms_outer, "solve_energy": statistics.median(e_ms),
                          "solve_uvwp_without_energy_setup": ms_plain / a.steps},
        "temperature_range": [float(t_range.min()), float(t_range.max())],
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": ncu_traffic(dominant, a.n, a.precision),
                     "algorithmic_bytes": nbytes, "avg_launch_us": avg_s * 1e6, "launches": dp[0],
                     "peak_source": peak_kind},
        "kernel_shares": shares,
        "kernels": per_launch,
    }
    if clk:
        out["clocks"] = clk
    if cpu:
        out["cpu_baseline"] = cpu
    return out


def cpu_energy_baseline(a, budget_s=15.0):
    """The reference's solve_energy (CPU oracle, Gauss-Seidel to a 10x drop,
    sequential like the reference), on a 32^3 sample of the same cavity
    after a few outer passes; cells x solves / s."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    n = min(a.n, 32)
    if a.tet:
        import cfdl
        zone = cfdl.Zone(n, a.tet, a.jitter, seed=a.seed)
    else:
        zone = oracle_lib.BoxZone(n, a.jitter, a.seed)
    o = oracle_lib.Oracle(zone, n_subdomains=4)
    o.physics_init(oracle_lib.steady(mode=0))
    o.energy_init()
    o.run(3, 0)
    k, dt = 0, 0.0
    while dt < budget_s and k < 200:
        o.update_boundaries()
        o.solve_uvwp()
        t0 = time.perf_counter()
        o.solve_energy()
        dt += time.perf_counter() - t0
        k += 1
    ne = o.ne
    o.close()
    return {"value": ne * k / dt, "unit": "cells x solves/s", "cores": 1, "kind": "port", "host": host_cpu(),
            "sample": "%d solve_energy calls on a %d^3 mesh (%d cells) after 3 outer passes, %.1f s of solves"
                      % (k, n, ne, dt)}


# ------------------------------------------------------------ mesh set-up
def run_setup(a, dist):
    """Mesh set-up (face matching, numbering, geometry) of the largest served
    mesh, on the host builder and on the GPU; the arrays are compared."""
    import numpy as np
    import cfdl

    cfdl.select_device(dist.local)
    n = a.n if a.n != 128 else 96
    tet = True if not a.tet else a.tet
    zone = cfdl.Zone(n, tet, 0.1, seed=a.seed)
    cfdl.Setup(cfdl.Zone(4, tet), device=True)          # warm: CUDA context and module load
    times = {}
    setups = {}
    for dev in (False, True):
        best = None
        for _ in range(3):
            t0 = time.perf_counter()
            s = cfdl.Setup(zone, device=dev)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        times[dev] = best
        setups[dev] = s
    same = all(np.array_equal(setups[False].get_int(k), setups[True].get_int(k))
               for k in ("ef2nb1", "ef2nb2", "s2g", "bs", "red")) and \
        all(np.array_equal(setups[False].get_dbl(k), setups[True].get_dbl(k)) for k in ("aip", "rip", "xc", "vol"))
    return {"metric": "mesh set-up time", "value": times[True], "unit": "s", "higher_is_better": False,
            "n_gpus": dist.world, "dtype": "f64", "data": "synthetic (seeded jittered unit-cube mesh)",
            "config": {"workload": "mesh set-up of a %d^3 %s cavity (%d cells, %d faces)" %
                                   (n, "tet-split" if tet else "hex", setups[True].ne, setups[True].nf),
                       "host_threads": os.cpu_count()},
            "host_s": times[False], "device_s": times[True], "speedup": times[False] / times[True],
            "bit_identical": bool(same)}


# ------------------------------------------------------------ served stream
def run_served(a, dist):
    """A Poisson stream of cavity requests through the serving loop; one JSON
    line per (form, rate) with p50/p99 latency and throughput.  The first
    --err-sample requests of every stream are the same cases (the stream draws
    each request's mesh and Reynolds number before its arrival time), so their
    FP64 converged states are computed once (converged_reference) and each
    line reports those requests' relative L2 error against them."""
    import threading
    import numpy as np
    import cfdl
    import workloads

    cfdl.select_device(dist.local)
    kw = {}
    if a.n_range:
        lo, hi = (int(x) for x in a.n_range.split(","))
        kw = dict(n_lo=lo, n_hi=hi)
    ref, t_ref = None, 0.0
    nerr = min(a.err_sample, a.requests)
    if nerr > 0:
        sample = workloads.served_requests(seed=a.seed, count=a.requests, rate=1.0, **kw)[:nerr]
        setups = [cfdl.Setup(cfdl.Zone(r["n"], r["tet"], 0.0, seed=a.seed)) for r in sample]
        t0 = time.perf_counter()
        ref, ref_stats, _ = converged_reference(setups, sample, a.ref_tol, a.conv_cap)
        t_ref = time.perf_counter() - t0
        ref_ne = [s_.ne for s_ in setups]
        ref_conv = int(sum(st.converged for st in ref_stats))
        del setups
    for prec in [int(x) for x in a.forms.split(",")]:
        for rate in [float(x) for x in a.rates.split(",")]:
            reqs = workloads.served_requests(seed=a.seed, count=a.requests, rate=rate, **kw)
            srv = cfdl.Server(precision=prec, hbm_budget=150e9)
            t_start = srv.now()
            rids = []

            def feeder():
                for k, r in enumerate(reqs):
                    delay = t_start + r["t"] - srv.now()
                    if delay > 0:
                        time.sleep(delay)
                    rids.append(srv.submit(n=r["n"], tet=r["tet"], jitter=0.0, seed=a.seed, re=r["re"],
                                           conv_tol=a.conv_tol, max_outer=a.max_outer, keep_fields=k < nerr))

            clocks = Clocks(dist.local)
            clocks.start()
            th = threading.Thread(target=feeder)
            th.start()
            th.join()
            srv.drain()
            clk = clocks.stop()
            res = srv.poll(max_results=4 * len(reqs))
            info = srv.info()
            errs = []
            for k in range(nerr):
                e = {}
                for f in ("u", "v", "w", "p"):
                    x, r_ = srv.fields(rids[k], f)[:ref_ne[k]], ref[k][f][:ref_ne[k]]
                    e[f] = float(np.linalg.norm(x - r_) / max(np.linalg.norm(r_), 1e-300))
                errs.append(max(e.values()))
            srv.close()
            lat = np.array([r.t_done - r.t_submit for r in res])
            dev = np.array([r.t_done - r.t_admit for r in res])
            prep = np.array([r.t_ready - r.t_submit for r in res])
            span = max(r.t_done for r in res) - min(r.t_submit for r in res)
            out = {
                "metric": "served cavity requests: p50/p99 latency (s)", "value": float(np.percentile(lat, 99)),
                "unit": "s (p99 latency)", "higher_is_better": False, "n_gpus": dist.world,
                "dtype": DTYPES[prec],
                "data": "synthetic (seeded Poisson request stream)",
                "config": {"workload": "served: Poisson stream at %.0f req/s, %d requests, N~U{%d..%d}, hex or "
                                       "tet-split, Re log-U[10,1000], stop at mass ratio %.0e or %d iterations; "
                                       "admitted by free HBM against a 150 GB budget" %
                                       (rate, len(reqs), min(r["n"] for r in reqs), max(r["n"] for r in reqs),
                                        a.conv_tol, a.max_outer),
                           "rate_req_s": rate, "requests": len(reqs)},
                "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "device_p50_s": float(np.percentile(dev, 50)), "device_p99_s": float(np.percentile(dev, 99)),
                "host_prep_p50_s": float(np.percentile(prep, 50)), "host_prep_p99_s": float(np.percentile(prep, 99)),
                "throughput_req_s": len(res) / span, "cell_iters_per_s": info["cell_iters"] / span,
                "converged": int(sum(r.converged for r in res)), "failed": int(sum(r.status != 0 for r in res)),
                "outer_iterations": {"min": int(min(r.outer_done for r in res)),
                                     "median": float(np.median([r.outer_done for r in res])),
                                     "max": int(max(r.outer_done for r in res))},
                "launches": info["launches"], "makespan_s": span,
            }
            if nerr:
                out["rel_l2_vs_fp64_converged"] = {
                    "requests": nerr, "max": max(errs), "median": float(np.median(errs)),
                    "reference": "each request's case, FP64, to mass ratio <= %.0e (%d of %d converged, %.0f s)"
                                 % (a.ref_tol, ref_conv, nerr, t_ref)}
            if clk:
                out["clocks"] = clk
            yield out


def main():
    a = parse()
    dist = Dist()
    try:
        if a.impl == "reference":
            out = run_reference(a, dist)
        elif a.workload == "batched":
            out = run_batched(a, dist)
        elif a.workload == "served":
            out = run_served(a, dist)
        elif a.workload == "converged":
            out = run_converged(a, dist)
        elif a.workload == "pressure":
            out = run_pressure(a, dist)
        elif a.workload == "energy":
            out = run_energy(a, dist)
        elif a.workload == "setup":
            out = run_setup(a, dist)
        else:
            out = run_ours(a, dist)
        if out is not None:
            # lists print at the end, generators (the long workloads) as each line is ready
            for line in ([out] if isinstance(out, dict) else out):
                if dist.rank == 0:
                    print(json.dumps(line))
                    sys.stdout.flush()
    finally:
        dist.close()


if __name__ == "__main__":
    main()
