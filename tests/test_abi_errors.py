"""Error behaviour of the C-ABI without a device: every entry point that takes
a context, server or set-up handle refuses a NULL handle with a status code
(or -1 from a getter) instead of touching memory, and the set-up queries
reject unknown names.  The signatures are read from include/cfdl.h, so a new
entry point is covered when it is declared.  CPU only."""
import ctypes as C
import os
import re

import pytest

import cfdl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CFDL_ERR_INVALID = 1
# NULL is a no-op for the destroy call (as free(NULL)); the server clock of no
# server reads 0
NULL_OK = {"cfdl_setup_destroy": 0, "cfdl_server_now": 0.0}
# getters that return a value, not a status: -1 for no context
GETTERS = {"cfdl_get_tile", "cfdl_get_coarse_group", "cfdl_get_energy_tile", "cfdl_case_count", "cfdl_launch_count",
           "cfdl_amg_index_bytes"}


def handle_entry_points():
    with open(os.path.join(ROOT, "include", "cfdl.h")) as fh:
        hdr = fh.read()
    out = []
    for ret, name, args in re.findall(r"^(int|double|int64_t)\s+(cfdl_[a-z0-9_]+)\(([^)]*)\)", hdr, re.M):
        parts = [a.strip() for a in args.split(",")] if args.strip() else []
        if parts and re.search(r"\b(cfdl_ctx|cfdl_server|cfdl_setup)\s*\*", parts[0]):
            out.append((ret, name, parts))
    return out


def null_call(ret, name, parts):
    types, vals = [], []
    for a in parts:
        if "*" in a:
            types.append(C.c_void_p); vals.append(None)
        elif "double" in a:
            types.append(C.c_double); vals.append(1.0)
        elif "int64_t" in a:
            types.append(C.c_int64); vals.append(1)
        else:
            types.append(C.c_int); vals.append(1)
    f = getattr(C.CDLL(cfdl.LIB_PATH), name)
    f.argtypes = types
    f.restype = {"int": C.c_int, "double": C.c_double, "int64_t": C.c_int64}[ret]
    return f(*vals)


ENTRY = handle_entry_points()


def test_the_header_declares_handle_entry_points():
    names = {n for _, n, _ in ENTRY}
    assert len(names) > 50
    assert {"cfdl_step", "cfdl_solve_uvwp", "cfdl_step_host", "cfdl_run", "cfdl_server_submit"} <= names


@pytest.mark.parametrize("ret,name,parts", ENTRY, ids=[n for _, n, _ in ENTRY])
def test_null_handle_is_refused(ret, name, parts):
    r = null_call(ret, name, parts)
    if name in NULL_OK:
        assert r == NULL_OK[name]
    elif name in GETTERS:
        assert r == -1
    else:
        assert r == CFDL_ERR_INVALID


def test_setup_queries_reject_unknown_names():
    s = cfdl.Setup(cfdl.Zone(2))
    L = cfdl.lib()
    buf = (C.c_double * 64)()
    ibuf = (C.c_int * 64)()
    assert L.cfdl_setup_get_dbl(s._h, b"no_such_array", buf) != 0
    assert L.cfdl_setup_get_int(s._h, b"no_such_array", ibuf) != 0
    assert L.cfdl_setup_get_int(s._h, None, ibuf) != 0
