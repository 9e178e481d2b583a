"""Build libcfdgpu.so in-tree for sm_103a (GB300).

Each translation unit is compiled in parallel with nvcc (host files through
nvcc as well, so one toolchain drives the whole build), then linked into
``cfd-lite_gb300/libcfdgpu.so`` with the CUDA runtime linked statically.
Host code is compiled without floating-point contraction so the mesh set-up
and geometry precomputation round exactly like the reference's arithmetic.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcfdgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
SOURCES = ["cfdl_zone.cpp", "cfdl_setup.cpp", "cfdl_case.cpp", "cfdl_api.cpp",
           "cfdl_prof.cpp", "cfdl_tune.cpp", "cfdl_serve.cpp", "cfdl_amg_setup.cpp", "cfdl_kernels.cu", "cfdl_amg.cu", "cfdl_solvers.cu", "cfdl_graph.cu", "cfdl_run.cu", "cfdl_noalloc.cu", "cfdl_gsetup.cu", "cfdl_vtu.cpp", "cfdl_energy.cu", "cfdl_probe.cu"]
# the device mesh set-up reproduces the host builder's doubles: no FMA contraction
EXTRA = {"cfdl_gsetup.cu": ["-fmad=false"]}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [_nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + COMMON + EXTRA.get(src, [])
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if verbose else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "cfdl.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    """Compile every CUDA/C++ source for sm_103a and link libcfdgpu.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
