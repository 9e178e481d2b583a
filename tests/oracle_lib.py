"""ctypes access to the CPU oracle (oracle/liboracle.so) for the tests.

Test infrastructure only: the oracle checks the results of the code under
test and is never part of it.  It restates the reference Fortran line by line (see oracle/*.c).
"""
import ctypes as C
import hashlib
import math
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")


class OrConfig(C.Structure):
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("u_lid", C.c_double), ("dt", C.c_double),
                ("alpha_u", C.c_double), ("alpha_p", C.c_double), ("nit", C.c_int), ("mode", C.c_int),
                ("tight_rtol", C.c_double), ("tight_maxit", C.c_int)]


class OrStats(C.Structure):
    _fields_ = [("it_u", C.c_int), ("it_v", C.c_int), ("it_w", C.c_int), ("it_p", C.c_int),
                ("res_i", C.c_double * 4), ("res_f", C.c_double * 4), ("res_max", C.c_double * 4),
                ("it_e", C.c_int), ("res_e", C.c_double * 3)]


_lib = None


def build_oracle():
    r = subprocess.run(["make", "-s", "-C", ORACLE_DIR], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return ORACLE_LIB


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(ORACLE_LIB)
        vp = C.c_void_p
        L.or_create.restype = vp
        L.or_create.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_char_p, vp, vp, C.c_int, vp, C.c_int]
        L.or_create_from_arrays.restype = vp
        L.or_create_from_arrays.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p] + [vp] * 13 + [C.c_int]
        for n in ("or_destroy", "or_update_boundaries", "or_update_time", "or_calc_coef_uvw", "or_calc_coef_p",
                  "or_adjust_pc", "or_update_uvwp"):
            getattr(L, n).argtypes = [vp]
            getattr(L, n).restype = None
        L.or_sizes.argtypes = [vp, vp]
        L.or_get_int.argtypes = [vp, C.c_char_p, vp]
        L.or_get_dbl.argtypes = [vp, C.c_char_p, vp]
        L.or_set_dbl.argtypes = [vp, C.c_char_p, vp]
        L.or_physics_init.argtypes = [vp, C.POINTER(OrConfig)]
        L.or_set_config.argtypes = [vp, C.POINTER(OrConfig)]
        L.or_set_config.restype = None
        L.or_solve_uvwp.argtypes = [vp, C.POINTER(OrStats)]
        L.or_solve_uvwp.restype = None
        L.or_run.argtypes = [vp, C.c_int, C.c_int, C.POINTER(OrStats)]
        L.or_run.restype = None
        L.or_calc_grad.argtypes = [vp, vp, vp]
        L.or_calc_grad.restype = None
        L.or_calc_mip.argtypes = [vp, C.c_int]
        L.or_calc_mip.restype = None
        L.or_solve_pc.argtypes = [vp, C.POINTER(OrStats)]
        L.or_solve_pc.restype = None
        L.or_solve_momentum.argtypes = [vp, C.c_int, C.POINTER(OrStats)]
        L.or_solve_momentum.restype = None
        L.or_subdomain_sizes.argtypes = [vp, C.c_int, vp]
        L.or_subdomain_get.argtypes = [vp, C.c_int, vp, vp]
        L.or_energy_init.argtypes = [vp] + [C.c_double] * 5
        L.or_set_bc_kind.argtypes = [vp, C.c_int, C.c_int]
        L.or_calc_coef_energy.argtypes = [vp]
        L.or_calc_coef_energy.restype = None
        L.or_solve_energy.argtypes = [vp, C.POINTER(OrStats)]
        L.or_solve_energy.restype = None
        L.or_wtime.restype = C.c_double
        L.or_num_threads.restype = C.c_int
        L.or_box_zone_sizes.argtypes = [C.c_int, vp]
        L.or_box_zone_fill.argtypes = [C.c_int, C.c_double, C.c_uint64] + [vp] * 6 + [C.c_char_p]
        L.or_set_num_threads.argtypes = [C.c_int]
        L.or_set_num_threads.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def config(rho=5.0, mu=0.01, u_lid=1.0, dt=0.01, alpha_u=1.0, alpha_p=1.0, nit=100, mode=0,
           tight_rtol=1e-13, tight_maxit=20000):
    return OrConfig(rho, mu, u_lid, dt, alpha_u, alpha_p, nit, mode, tight_rtol, tight_maxit)


def steady(mode=1, **kw):
    base = dict(rho=1.0, mu=0.01, dt=math.inf, alpha_u=0.7, alpha_p=0.3, mode=mode)
    base.update(kw)
    return config(**base)


class Oracle:
    """One case in the CPU oracle, built from a zone (cfd-lite_gb300 Zone or any
    object with the same CGNS-shaped attributes)."""

    def __init__(self, zone, n_subdomains=4, setup=None):
        """Build from the zone with the oracle's own set-up restatement, or,
        when ``setup`` (a cfdl.Setup of the same zone) is given, from its
        arrays -- bit-identical to the restatement (tests/test_setup.py) and
        much faster on large meshes."""
        L = lib()
        if setup is None:
            h = L.or_create(zone.nvx, _p(zone.x), _p(zone.y), _p(zone.z), zone.nsec, zone.names,
                            _p(zone.etype), _p(zone.esec), zone.ne2vxmax, _p(zone.e2vx), n_subdomains)
        else:
            s = setup
            arrs = [s.get_int("esec"), s.get_int("etype")]
            ints = [s.get_int(n) for n in ("ef2nb1", "ef2nb2", "ef2nb_idx", "s2g", "bs")]
            dbls = [s.get_dbl(n) for n in ("aip", "rip", "xc", "yc", "zc", "vol")]
            self._keep = arrs + ints + dbls
            h = L.or_create_from_arrays(s.ne, s.nf, s.nbf, zone.nsec, zone.names, _p(arrs[1]), _p(arrs[0]),
                                        *[_p(a) for a in ints], *[_p(a) for a in dbls], n_subdomains)
        if not h:
            raise RuntimeError("oracle mesh set-up failed")
        self._h = C.c_void_p(h)
        sz = np.zeros(9, np.int32)
        L.or_sizes(self._h, _p(sz))
        (self.ne, self.nf, self.nbf, self.nvx, self.nelem, self.nsec, self.nred, self.nsubd,
         self.nintf) = (int(v) for v in sz)
        self.H = 2 * self.nf - self.nbf

    def _n(self, name):
        nc = self.ne + self.nbf
        table = {"ef2nb1": self.H, "ef2nb2": self.H, "ef2nb_idx": self.ne + 1, "s2g": self.nf, "bs": self.nbf,
                 "bs_idx": self.nsec + 1, "etype": self.nsec, "red": self.ne, "sec2intf": self.nsec,
                 "esec": 2 * self.nsec, "gf2g": self.ne, "g2gf": self.ne, "g2gf_idx": self.nsubd + 1,
                 "aip": 3 * self.nf, "rip": 3 * self.nf, "mip": self.nf, "mip0": self.nf, "anb": self.H}
        if name in table:
            return table[name]
        if name in ("xc", "yc", "zc", "u", "v", "w", "p", "u0", "v0", "w0", "phic", "t", "e", "e0"):
            return nc
        if name in ("gu", "gv", "gw", "gp", "gpc", "gt", "ge"):
            return 3 * nc
        return self.ne

    def get_int(self, name):
        out = np.zeros(self._n(name), np.int32)
        if lib().or_get_int(self._h, name.encode(), _p(out)) != 0:
            raise KeyError(name)
        return out

    def get(self, name):
        out = np.zeros(self._n(name))
        if lib().or_get_dbl(self._h, name.encode(), _p(out)) != 0:
            raise KeyError(name)
        return out

    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        assert a.size == self._n(name)
        if lib().or_set_dbl(self._h, name.encode(), _p(a)) != 0:
            raise KeyError(name)

    def physics_init(self, cfg):
        lib().or_physics_init(self._h, C.byref(cfg))

    def set_bc_kind(self, i, kind):
        """Rebind BC i (0-based, eqn%bcs order): 'lid', 'dirichlet0' or 'symmetry'."""
        k = {"lid": 1, "dirichlet0": 2, "symmetry": 3}[kind]
        if lib().or_set_bc_kind(self._h, int(i) + 1, k) != 0:
            raise ValueError("cannot rebind BC %d" % i)

    def set_config(self, cfg):
        lib().or_set_config(self._h, C.byref(cfg))

    def update_boundaries(self):
        lib().or_update_boundaries(self._h)

    def solve_uvwp(self):
        st = OrStats()
        lib().or_solve_uvwp(self._h, C.byref(st))
        return st

    def update_time(self):
        lib().or_update_time(self._h)

    def run(self, n_outer, ncoef=3):
        st = OrStats()
        lib().or_run(self._h, int(n_outer), int(ncoef), C.byref(st))
        return st

    def energy_init(self, cp=1000.0, tc=5.0, t_init=273.0, t_lid=373.0, t_wall=273.0):
        if lib().or_energy_init(self._h, cp, tc, t_init, t_lid, t_wall) != 0:
            raise RuntimeError("or_energy_init needs physics_init first")

    def calc_coef_energy(self):
        lib().or_calc_coef_energy(self._h)

    def solve_energy(self):
        st = OrStats()
        lib().or_solve_energy(self._h, C.byref(st))
        return st

    def calc_grad(self, phi, grad_in=None):
        g = np.zeros(3 * (self.ne + self.nbf)) if grad_in is None else np.array(grad_in, dtype=np.float64)
        ph = np.ascontiguousarray(phi, dtype=np.float64)
        lib().or_calc_grad(self._h, _p(ph), _p(g))
        return g

    def calc_coef_uvw(self):
        lib().or_calc_coef_uvw(self._h)

    def calc_mip(self, rhie_chow=True):
        lib().or_calc_mip(self._h, int(bool(rhie_chow)))

    def calc_coef_p(self):
        lib().or_calc_coef_p(self._h)

    def solve_pc(self):
        st = OrStats()
        lib().or_solve_pc(self._h, C.byref(st))
        return st

    def solve_momentum(self, comp):
        st = OrStats()
        lib().or_solve_momentum(self._h, int(comp), C.byref(st))
        return st

    def adjust_pc(self):
        lib().or_adjust_pc(self._h)

    def update_uvwp(self):
        lib().or_update_uvwp(self._h)

    def subdomain(self, sd):
        sz = np.zeros(3, np.int32)
        lib().or_subdomain_sizes(self._h, sd, _p(sz))
        ne, nf, nbf = (int(v) for v in sz)
        idx = np.zeros(ne + 1, np.int32)
        ef = np.zeros(2 * nf - nbf, np.int32)
        lib().or_subdomain_get(self._h, sd, _p(idx), _p(ef))
        return ne, nf, nbf, idx, ef

    def close(self):
        if getattr(self, "_h", None):
            lib().or_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def wtime():
    return lib().or_wtime()


class BoxZone:
    """The hex cavity zone made by the oracle (cfd_oracle_zone.c): the same
    attributes as the product's Zone, so an Oracle can be built from it
    without the GPU library."""

    def __init__(self, n, jitter=0.0, seed=0):
        L = lib()
        sz = np.zeros(4, np.int32)
        if L.or_box_zone_sizes(int(n), _p(sz)) != 0:
            raise ValueError("zone size out of range")
        self.nvx, self.nelem, self.nsec, self.ne2vxmax = (int(v) for v in sz)
        self.x, self.y, self.z = (np.zeros(self.nvx) for _ in range(3))
        self.e2vx = np.zeros(self.ne2vxmax * self.nelem, np.int32)
        self.etype = np.zeros(self.nsec, np.int32)
        self.esec = np.zeros(2 * self.nsec, np.int32)
        buf = C.create_string_buffer(33 * self.nsec)
        if L.or_box_zone_fill(int(n), float(jitter), int(seed), _p(self.x), _p(self.y), _p(self.z), _p(self.e2vx),
                              _p(self.etype), _p(self.esec), buf) != 0:
            raise RuntimeError("or_box_zone_fill failed")
        self.names = buf.raw


def sha256(a):
    """SHA-256 of an array's bytes (the golden fixtures' hash)."""
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def num_threads():
    """Host threads the oracle's parallel loops use."""
    return int(lib().or_num_threads())


def set_num_threads(n):
    """Threads for the oracle's parallel loops from now on."""
    lib().or_set_num_threads(int(n))
