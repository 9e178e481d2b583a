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
