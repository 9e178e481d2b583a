"""The C-ABI from a plain-C host (tests/c_host/step_host.c): the program a
Fortran host's ISO_C_BINDING calls amount to, built with the system C
compiler against include/cfdl.h and libcfdgpu.so.  On CPU: it compiles and
links.  On a GB300: the fields it holds after its host-driven passes equal,
bit for bit, those of the same case stepped resident through the Python
mirror."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import cfdl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_host", "step_host.c")
LIBDIR = os.path.join(ROOT, "cfd-lite_gb300")


def build_host(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    cfdl.lib()                          # the library is built
    exe = str(tmp_path / "step_host")
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                        "-L", LIBDIR, "-lcfdgpu", "-Wl,-rpath," + LIBDIR, "-lm", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_compiles_against_the_header(tmp_path):
    build_host(tmp_path)


@pytest.mark.gpu
def test_c_host_equals_resident_stepping(need_gpu, tmp_path):
    exe = build_host(tmp_path)
    out = str(tmp_path / "fields.bin")
    n, tet, jit, seed, n_outer, ncoef = 6, 0, 0.2, 3, 9, 3
    r = subprocess.run([exe, str(n), str(tet), str(jit), str(seed), str(n_outer), str(ncoef), out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    z = cfdl.Zone(n, bool(tet), jit, seed=seed)
    s = cfdl.Setup(z)
    g = cfdl.Solver(s, cfdl.steady())
    g.step(n_outer, ncoef)
    nc, nf = s.ne + s.nbf, s.nf
    host = np.fromfile(out, dtype="<f8")
    assert host.size == 4 * nc + nf
    for q, f in enumerate(("u", "v", "w", "p")):
        assert np.array_equal(host[q * nc:(q + 1) * nc], g.get(f)), f
    assert np.array_equal(host[4 * nc:], g.get("mip"))


# ---- the C++ mirror of mod_physics / mod_uvwp (cfd-lite_gb300/host/cfdl_phys.hpp) ----

CPP_SRC = os.path.join(ROOT, "tests", "c_host", "phys_host.cpp")
CFDL_ERR_NO_DEVICE = 7


def build_cpp_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cfdl.lib()
    exe = str(tmp_path / "phys_host")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(LIBDIR, "host"), CPP_SRC, "-L", LIBDIR, "-lcfdgpu",
                        "-Wl,-rpath," + LIBDIR, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_host_compiles_against_the_mirror(tmp_path):
    build_cpp_host(tmp_path)


def test_cpp_host_stops_without_a_device(tmp_path):
    """The reference stops on an error; the mirror's stop_error does the same
    at construct_physics when there is no GPU (the set-up before it runs on
    the host)."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("device present")
    exe = build_cpp_host(tmp_path)
    r = subprocess.run([exe, "3", "0", "0.1", "1", "1", "1", str(tmp_path / "f.bin")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 10 + CFDL_ERR_NO_DEVICE, r.stdout + r.stderr
    assert "stop: construct_physics" in r.stderr


@pytest.mark.gpu
def test_cpp_host_equals_resident_stepping(need_gpu, tmp_path):
    """main.f90's loop through the C++ mirror (update_boundaries and
    solve_uvwp on host arrays, update_time on the host) gives the fields of
    the same case stepped resident, bit for bit."""
    exe = build_cpp_host(tmp_path)
    out = str(tmp_path / "fields.bin")
    n, kind, jit, seed, ntstep, ncoef = 6, 0, 0.2, 3, 3, 3
    r = subprocess.run([exe, str(n), str(kind), str(jit), str(seed), str(ntstep), str(ncoef), out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    s = cfdl.Setup(cfdl.Zone(n, False, jit, seed=seed))
    g = cfdl.Solver(s, cfdl.steady())
    g.step(ntstep * ncoef, ncoef)
    nc, nf = s.ne + s.nbf, s.nf
    host = np.fromfile(out, dtype="<f8")
    assert host.size == 4 * nc + nf
    for q, f in enumerate(("u", "v", "w", "p")):
        assert np.array_equal(host[q * nc:(q + 1) * nc], g.get(f)), f
    assert np.array_equal(host[4 * nc:], g.get("mip"))
