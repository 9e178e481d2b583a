"""Host-side mirror of the CFD-Lite hot-path interface over libcfdgpu's C-ABI.

The reference drives one SIMPLE outer iteration from Fortran
(src/main.f90:50-63): ``update_boundaries`` (src/modules/mod_physics.f90:38),
``solve_uvwp`` (src/equations/mod_uvwp.f90:95) and, every ``ncoef`` outer
iterations, ``update_time`` (mod_physics.f90:101).  ``Solver`` exposes the
same routines, plus the individual routines solve_uvwp calls, on a case that
stays resident in GPU memory.  Arrays cross the boundary in the reference's
layouts (1-based index values, xyz-interleaved gradients).

There is no CPU fallback: constructing a ``Solver`` without the CUDA library
or without a GPU raises ``CfdlError``.
"""
import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcfdgpu.so")

CFDL_OK = 0
(CFDL_ERR_INVALID, CFDL_ERR_OOM, CFDL_ERR_NONFINITE, CFDL_ERR_ITER_CAP, CFDL_ERR_CUDA, CFDL_ERR_MESH,
 CFDL_ERR_NO_DEVICE, CFDL_ERR_NAME, CFDL_ERR_TOO_LARGE, CFDL_ERR_BREAKDOWN) = range(1, 11)
STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "non-finite value in a solve",
          4: "inner solve reached its iteration cap", 5: "CUDA runtime error", 6: "mesh connectivity error",
          7: "no CUDA device", 8: "unknown array name",
          9: "problem larger than the fixed scratch of the allocation-free entry point",
          10: "Krylov breakdown: p.Ap <= 0 above the tolerance (matrix not positive definite)"}
BC_WALL, BC_SYMMETRY = 1, 2
# cfdl_fields members as CFDL_F_* bits (cfdl_step_host_keep)
FIELD_BITS = {f: 1 << k for k, f in enumerate(("u", "v", "w", "p", "u0", "v0", "w0", "gu", "gv", "gw", "gp", "gpc",
                                                "mip", "mip0"))}
HEXA_8, TETRA_4, QUAD_4, TRI_3 = 17, 10, 7, 5


class CfdlError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s: %s (status %d)" % (what, STATUS.get(status, "unknown"), status))


class Config(C.Structure):
    """cfdl_config: physics constants and inner-solve controls."""
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("dt", C.c_double),
                ("alpha_u", C.c_double), ("alpha_p", C.c_double), ("nit", C.c_int),
                ("solve_mode", C.c_int), ("rtol_u", C.c_double), ("rtol_p", C.c_double),
                ("tight_rtol", C.c_double), ("tight_maxit", C.c_int), ("precision", C.c_int),
                ("precond", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("it_u", C.c_int), ("it_v", C.c_int), ("it_w", C.c_int), ("it_p", C.c_int),
                ("res_i", C.c_double * 4), ("res_f", C.c_double * 4),
                ("mass_imbalance", C.c_double), ("status", C.c_int),
                ("outer_done", C.c_int), ("run_left", C.c_int), ("converged", C.c_int),
                ("mass_ratio", C.c_double), ("it_e", C.c_int), ("res_e", C.c_double * 2)]

    def as_dict(self):
        return {"it": [self.it_u, self.it_v, self.it_w, self.it_p], "res_i": list(self.res_i),
                "res_f": list(self.res_f), "mass_imbalance": self.mass_imbalance, "status": self.status,
                "outer_done": self.outer_done, "run_left": self.run_left, "converged": self.converged,
                "mass_ratio": self.mass_ratio, "it_e": self.it_e, "res_e": list(self.res_e)}


class Request(C.Structure):
    _fields_ = [("n", C.c_int), ("tet", C.c_int), ("jitter", C.c_double), ("seed", C.c_uint64),
                ("re", C.c_double), ("conv_tol", C.c_double), ("max_outer", C.c_int), ("keep_fields", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_double), ("hbm_reserve", C.c_double),
                ("max_cases", C.c_int), ("chunk", C.c_int), ("prep_threads", C.c_int),
                ("precision", C.c_int), ("precond", C.c_int), ("tile", C.c_int),
                ("alpha_u", C.c_double), ("alpha_p", C.c_double), ("device_setup", C.c_int)]


class Result(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("ne", C.c_int), ("outer_done", C.c_int),
                ("converged", C.c_int), ("mass_ratio", C.c_double), ("t_submit", C.c_double),
                ("t_ready", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerInfo(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("done", C.c_int64), ("queued", C.c_int64), ("launches", C.c_int64),
                ("resident", C.c_int), ("held_bytes", C.c_double), ("cell_iters", C.c_double),
                ("busy_s", C.c_double), ("now", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Mesh(C.Structure):
    _fields_ = [("ne", C.c_int), ("nf", C.c_int), ("nbf", C.c_int),
                ("ef2nb1", C.c_void_p), ("ef2nb2", C.c_void_p), ("ef2nb_idx", C.c_void_p),
                ("s2g", C.c_void_p), ("bs", C.c_void_p), ("aip", C.c_void_p), ("rip", C.c_void_p),
                ("xc", C.c_void_p), ("yc", C.c_void_p), ("zc", C.c_void_p), ("vol", C.c_void_p),
                ("nbc", C.c_int), ("bc_esec", C.c_void_p), ("bc_kind", C.c_void_p), ("bc_vel", C.c_void_p),
                ("bc_temp", C.c_void_p)]


class Fields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("u", "v", "w", "p", "u0", "v0", "w0", "gu", "gv", "gw",
                                          "gp", "gpc", "mip", "mip0")]


_lib = None


def lib():
    """Load libcfdgpu.so (building it if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise CfdlError(5, "libcfdgpu.so is not built (run __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.cfdl_box_zone_sizes.argtypes = [C.c_int, C.c_int, ip, ip, ip, ip]
    L.cfdl_box_zone_fill.argtypes = [C.c_int, C.c_int, C.c_double, C.c_uint64, vp, vp, vp, vp, vp, vp, C.c_char_p]
    L.cfdl_setup_create.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_char_p, vp, vp, C.c_int, vp, C.POINTER(vp)]
    L.cfdl_setup_create_device.argtypes = L.cfdl_setup_create.argtypes
    L.cfdl_setup_sizes.argtypes = [vp, vp]
    L.cfdl_setup_mesh.argtypes = [vp, C.c_double, C.POINTER(Mesh)]
    L.cfdl_setup_get_int.argtypes = [vp, C.c_char_p, vp]
    L.cfdl_setup_get_dbl.argtypes = [vp, C.c_char_p, vp]
    L.cfdl_setup_destroy.argtypes = [vp]
    L.cfdl_config_default.argtypes = [C.POINTER(Config)]
    L.cfdl_config_default.restype = None
    L.cfdl_ctx_create.argtypes = [C.POINTER(Mesh), C.POINTER(Config), C.POINTER(vp)]
    L.cfdl_set_config.argtypes = [vp, C.POINTER(Config)]
    L.cfdl_upload_fields.argtypes = [vp, C.POINTER(Fields)]
    L.cfdl_download_fields.argtypes = [vp, C.POINTER(Fields)]
    L.cfdl_ctx_destroy.argtypes = [vp]
    L.cfdl_mesh_check.argtypes = [C.POINTER(Mesh)]
    for n in ("cfdl_update_boundaries", "cfdl_update_time", "cfdl_calc_coef_uvw", "cfdl_calc_coef_p",
              "cfdl_adjust_pc", "cfdl_update_uvwp"):
        getattr(L, n).argtypes = [vp]
    for n in ("cfdl_solve_uvwp", "cfdl_solve_momentum", "cfdl_solve_pc", "cfdl_solve_energy"):
        getattr(L, n).argtypes = [vp, C.POINTER(Stats)]
    L.cfdl_energy_init.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    L.cfdl_check_conversions.argtypes = [C.c_int, vp]
    L.cfdl_probe_fp64.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cfdl_set_pdl.argtypes = [vp, C.c_int]
    L.cfdl_set_index16.argtypes = [vp, C.c_int]
    L.cfdl_set_energy_tile.argtypes = [vp, C.c_int]
    L.cfdl_get_energy_tile.argtypes = [vp]
    L.cfdl_calc_coef_energy.argtypes = [vp]
    L.cfdl_step.argtypes = [vp, C.c_int, C.c_int, C.POINTER(Stats)]
    L.cfdl_solve_uvwp_host.argtypes = [vp, C.POINTER(Fields), C.POINTER(Stats)]
    L.cfdl_step_host.argtypes = [vp, C.POINTER(Fields), C.c_int, C.c_int, C.POINTER(Stats)]
    L.cfdl_step_host_keep.argtypes = [vp, C.POINTER(Fields), C.c_uint, C.c_int, C.c_int, C.POINTER(Stats)]
    L.cfdl_calc_grad.argtypes = [vp, C.c_int]
    L.cfdl_calc_mip.argtypes = [vp, C.c_int]
    L.cfdl_get_array.argtypes = [vp, C.c_char_p, vp]
    L.cfdl_set_array.argtypes = [vp, C.c_char_p, vp]
    L.cfdl_select_device.argtypes = [C.c_int]
    L.cfdl_timer_begin.argtypes = [vp]
    L.cfdl_timer_end.argtypes = [vp, dp]
    L.cfdl_profile_start.argtypes = [vp, C.c_char_p]
    L.cfdl_profile_stop.argtypes = [vp, ip]
    L.cfdl_profile_get.argtypes = [vp, C.c_int, C.c_char_p, C.POINTER(C.c_int64), dp]
    L.cfdl_solve_pc_noalloc.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, C.c_double, C.c_int,
                                        ip, dp]
    L.cfdl_amg_info.argtypes = [vp, C.c_int, ip, vp, vp]
    L.cfdl_amg_index_bytes.argtypes = [vp]
    L.cfdl_set_graph_mode.argtypes = [vp, C.c_int]
    L.cfdl_batch_create.argtypes = [C.c_int, vp, vp, C.POINTER(vp)]
    L.cfdl_case_add.argtypes = [vp, C.POINTER(Mesh), C.POINTER(Config), ip]
    L.cfdl_case_remove.argtypes = [vp, C.c_int]
    L.cfdl_case_count.argtypes = [vp]
    L.cfdl_case_ids.argtypes = [vp, vp]
    L.cfdl_case_get_array.argtypes = [vp, C.c_int, C.c_char_p, vp]
    L.cfdl_case_set_array.argtypes = [vp, C.c_int, C.c_char_p, vp]
    L.cfdl_case_stats.argtypes = [vp, C.c_int, C.POINTER(Stats)]
    L.cfdl_case_info.argtypes = [vp, C.c_int, ip, C.POINTER(C.c_size_t)]
    L.cfdl_case_bytes_estimate.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    L.cfdl_case_bytes_estimate.restype = C.c_size_t
    L.cfdl_case_set_run.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double]
    L.cfdl_run.argtypes = [vp, C.c_int, ip]
    L.cfdl_set_tile.argtypes = [vp, C.c_int]
    L.cfdl_write_vtu.argtypes = [vp, C.c_int, vp, C.c_char_p]
    L.cfdl_write_vtu_energy.argtypes = [vp, C.c_int, vp, C.c_char_p]
    L.cfdl_server_config_default.argtypes = [C.POINTER(ServerConfig)]
    L.cfdl_server_config_default.restype = None
    L.cfdl_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(vp)]
    L.cfdl_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_int64)]
    L.cfdl_server_poll.argtypes = [vp, C.POINTER(Result), C.c_int, ip, C.c_double]
    L.cfdl_server_fields.argtypes = [vp, C.c_int64, C.c_char_p, vp, C.POINTER(C.c_int64)]
    L.cfdl_server_drain.argtypes = [vp, C.c_double]
    L.cfdl_server_query.argtypes = [vp, C.POINTER(ServerInfo)]
    L.cfdl_server_now.argtypes = [vp]
    L.cfdl_server_now.restype = C.c_double
    L.cfdl_server_destroy.argtypes = [vp]
    L.cfdl_get_tile.argtypes = [vp]
    L.cfdl_autotune.argtypes = [vp, C.c_int, ip, dp]
    L.cfdl_set_coarse_group.argtypes = [vp, C.c_int]
    L.cfdl_get_coarse_group.argtypes = [vp]
    L.cfdl_launch_count.argtypes = [vp]
    L.cfdl_launch_count.restype = C.c_int64
    L.cfdl_status_string.argtypes = [C.c_int]
    L.cfdl_status_string.restype = C.c_char_p
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(st, what):
    if st != CFDL_OK:
        raise CfdlError(st, what)


ZONE_KINDS = {"hex": 0, "tet": 1, "prism": 2, "pyramid": 3, "mixed": 4}


class Zone:
    """CGNS-shaped zone of the synthetic cavity (what cell_input reads).
    tet=True is the six-tet split; kind ("hex", "tet", "prism", "pyramid",
    "mixed" = hex and pyramid cubes), or a kind name given as tet, overrides
    it."""

    def __init__(self, n, tet=False, jitter=0.0, seed=0, kind=None):
        L = lib()
        if isinstance(tet, str):
            kind = tet
        k = ZONE_KINDS[kind] if kind is not None else int(bool(tet))
        tet = k
        nvx, nelem, nsec, m = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(L.cfdl_box_zone_sizes(n, int(tet), C.byref(nvx), C.byref(nelem), C.byref(nsec), C.byref(m)), "zone sizes")
        self.n, self.tet, self.jitter, self.seed = n, k == 1, jitter, seed
        self.kind = k
        self.nvx, self.nelem, self.nsec, self.ne2vxmax = nvx.value, nelem.value, nsec.value, m.value
        self.x = np.zeros(self.nvx); self.y = np.zeros(self.nvx); self.z = np.zeros(self.nvx)
        self.e2vx = np.zeros(self.ne2vxmax * self.nelem, np.int32)
        self.etype = np.zeros(self.nsec, np.int32)
        self.esec = np.zeros(2 * self.nsec, np.int32)
        self.names = C.create_string_buffer(33 * self.nsec)
        _check(L.cfdl_box_zone_fill(n, int(tet), float(jitter), int(seed), _p(self.x), _p(self.y), _p(self.z),
                                    _p(self.e2vx), _p(self.etype), _p(self.esec), self.names), "zone fill")

    def section_names(self):
        raw = self.names.raw
        return [raw[33 * s:33 * s + 32].split(b"\0")[0].decode() for s in range(self.nsec)]


class Setup:
    """Connectivity and geometry of a zone, in the reference's arrays."""

    def __init__(self, zone, device=False):
        """device=True matches faces and computes the geometry on the GPU
        (cfdl_setup_create_device); the arrays are the same bit for bit."""
        L = lib()
        self._h = C.c_void_p()
        fn = L.cfdl_setup_create_device if device else L.cfdl_setup_create
        _check(fn(zone.nvx, _p(zone.x), _p(zone.y), _p(zone.z), zone.nsec, zone.names,
                  _p(zone.etype), _p(zone.esec), zone.ne2vxmax, _p(zone.e2vx), C.byref(self._h)),
               "mesh set-up")
        sz = np.zeros(5, np.int32)
        L.cfdl_setup_sizes(self._h, _p(sz))
        self.ne, self.nf, self.nbf, self.nsec, self.nred = (int(v) for v in sz)
        self.H = 2 * self.nf - self.nbf

    def get_int(self, name):
        n = {"ef2nb1": self.H, "ef2nb2": self.H, "ef2nb_idx": self.ne + 1, "s2g": self.nf, "bs": self.nbf,
             "esec": 2 * self.nsec, "etype": self.nsec, "red": self.ne}[name]
        out = np.zeros(n, np.int32)
        _check(lib().cfdl_setup_get_int(self._h, name.encode(), _p(out)), name)
        return out

    def get_dbl(self, name):
        n = {"aip": 3 * self.nf, "rip": 3 * self.nf, "xc": self.ne + self.nbf, "yc": self.ne + self.nbf,
             "zc": self.ne + self.nbf, "vol": self.ne}[name]
        out = np.zeros(n)
        _check(lib().cfdl_setup_get_dbl(self._h, name.encode(), _p(out)), name)
        return out

    def mesh(self, u_lid=1.0):
        m = Mesh()
        _check(lib().cfdl_setup_mesh(self._h, float(u_lid), C.byref(m)), "mesh")
        return m

    def check(self):
        """cfdl_mesh_check of this set-up's mesh: 0 when valid (no GPU needed)."""
        return lib().cfdl_mesh_check(C.byref(self.mesh()))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cfdl_setup_destroy(self._h)
            self._h = None


def select_device(device):
    _check(lib().cfdl_select_device(int(device)), "select_device")


def probe_fp64():
    """The current device's measured FP64 FMA rate: (FMA instructions/s, probe ms)."""
    rate, ms = C.c_double(), C.c_double()
    _check(lib().cfdl_probe_fp64(C.byref(rate), C.byref(ms)), "probe_fp64")
    return rate.value, ms.value


def default_config(**kw):
    cfg = Config()
    lib().cfdl_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


def steady(**kw):
    """The steady under-relaxed SIMPLE form (dt = inf, alpha_u, alpha_p)."""
    base = dict(rho=1.0, mu=0.01, dt=math.inf, alpha_u=0.7, alpha_p=0.3)
    base.update(kw)
    return default_config(**base)


class Solver:
    """One case resident on the GPU, driven like the reference's phys_t."""

    def __init__(self, setup, config=None, u_lid=1.0, bc_kinds=None):
        """bc_kinds (optional): {bc index: BC_WALL or BC_SYMMETRY} overriding the
        binding of cfdl_setup_mesh (eqn%bcs order)."""
        self.setup = setup
        self.mesh = setup.mesh(u_lid)
        if bc_kinds:
            kinds = np.ctypeslib.as_array(C.cast(self.mesh.bc_kind, C.POINTER(C.c_int)), (self.mesh.nbc,)).copy()
            for i, k in bc_kinds.items():
                kinds[i] = k
            self._bc_kinds = kinds
            self.mesh.bc_kind = kinds.ctypes.data_as(C.c_void_p)
        self.config = config if config is not None else default_config()
        self.ne, self.nf, self.nbf, self.H = setup.ne, setup.nf, setup.nbf, setup.H
        self._h = C.c_void_p()
        _check(lib().cfdl_ctx_create(C.byref(self.mesh), C.byref(self.config), C.byref(self._h)), "ctx_create")
        self.last_stats = Stats()

    # -- reference routines ------------------------------------------------
    def update_boundaries(self):
        _check(lib().cfdl_update_boundaries(self._h), "update_boundaries")

    def solve_uvwp(self, stats=True):
        if not stats:
            _check(lib().cfdl_solve_uvwp(self._h, None), "solve_uvwp")
            return None
        st = Stats()
        _check(lib().cfdl_solve_uvwp(self._h, C.byref(st)), "solve_uvwp")
        self.last_stats = st
        return st

    def update_time(self):
        _check(lib().cfdl_update_time(self._h), "update_time")

    def step(self, n_outer, ncoef=3):
        st = Stats()
        _check(lib().cfdl_step(self._h, int(n_outer), int(ncoef), C.byref(st)), "step")
        self.last_stats = st
        return st

    def calc_coef_uvw(self):
        _check(lib().cfdl_calc_coef_uvw(self._h), "calc_coef_uvw")

    def solve_momentum(self):
        st = Stats()
        _check(lib().cfdl_solve_momentum(self._h, C.byref(st)), "solve_momentum")
        return st

    def calc_grad(self, field):
        idx = {"u": 0, "v": 1, "w": 2, "phic": 3, "pc": 3, "uvw": 4, "energy": 5}[field]
        _check(lib().cfdl_calc_grad(self._h, idx), "calc_grad")

    def calc_mip(self, rhie_chow=True):
        _check(lib().cfdl_calc_mip(self._h, int(bool(rhie_chow))), "calc_mip")

    # -- energy equation (src/equations/mod_energy.f90) --------------------------
    def energy_init(self, cp=1000.0, tc=5.0, t_init=273.0):
        """construct_energy for every case; from then on update_boundaries,
        update_time, step and run include the energy equation."""
        _check(lib().cfdl_energy_init(self._h, float(cp), float(tc), float(t_init)), "energy_init")

    def solve_energy(self):
        st = Stats()
        _check(lib().cfdl_solve_energy(self._h, C.byref(st)), "solve_energy")
        return st

    def calc_coef_energy(self):
        _check(lib().cfdl_calc_coef_energy(self._h), "calc_coef_energy")

    def set_energy_tile(self, vec):
        _check(lib().cfdl_set_energy_tile(self._h, int(vec)), "set_energy_tile")

    def get_energy_tile(self):
        return lib().cfdl_get_energy_tile(self._h)

    def calc_coef_p(self):
        _check(lib().cfdl_calc_coef_p(self._h), "calc_coef_p")

    def solve_pc(self):
        st = Stats()
        _check(lib().cfdl_solve_pc(self._h, C.byref(st)), "solve_pc")
        return st

    def adjust_pc(self):
        _check(lib().cfdl_adjust_pc(self._h), "adjust_pc")

    def update_uvwp(self):
        _check(lib().cfdl_update_uvwp(self._h), "update_uvwp")

    def write_vtu(self, path, setup=None, cid=0):
        """The case's fields in the reference's VTU layout (write_vtubin)."""
        setup = setup if setup is not None else self.setup
        _check(lib().cfdl_write_vtu(self._h, int(cid), setup._h, str(path).encode()), "write_vtu")

    def write_vtu_energy(self, path, setup=None, cid=0):
        """The energy equation's fields in the reference's VTU layout."""
        setup = setup if setup is not None else self.setup
        _check(lib().cfdl_write_vtu_energy(self._h, int(cid), setup._h, str(path).encode()), "write_vtu_energy")

    def set_run(self, n_outer, ncoef=0, conv_tol=0.0, cid=-1):
        """Give case cid (-1: every case) n_outer outer iterations to run, an
        update_time cadence and an early-stop tolerance on the mass ratio."""
        _check(lib().cfdl_case_set_run(self._h, int(cid), int(n_outer), int(ncoef), float(conv_tol)), "case_set_run")

    def run(self, max_outer):
        """Up to max_outer passes; returns the number of cases with iterations left."""
        running = C.c_int()
        _check(lib().cfdl_run(self._h, int(max_outer), C.byref(running)), "run")
        return running.value

    def set_tile(self, vec):
        """Cells per thread of the inner-solve kernels (1, 2, 4 or 8)."""
        _check(lib().cfdl_set_tile(self._h, int(vec)), "set_tile")

    def get_tile(self):
        return int(lib().cfdl_get_tile(self._h))

    def set_coarse_group(self, lanes):
        """Lanes per row on the large coarse multigrid levels (1, 2 or 4)."""
        _check(lib().cfdl_set_coarse_group(self._h, int(lanes)), "set_coarse_group")

    def get_coarse_group(self):
        return int(lib().cfdl_get_coarse_group(self._h))

    def autotune(self, outer=3):
        """Times each tile shape on this context's cases (state restored) and
        keeps the fastest; returns (best, {vec: ms per outer iteration})."""
        best = C.c_int()
        ms = (C.c_double * 4)()
        _check(lib().cfdl_autotune(self._h, int(outer), C.byref(best), ms), "autotune")
        return best.value, dict(zip((1, 2, 4, 8), list(ms)))

    def set_pdl(self, on):
        _check(lib().cfdl_set_pdl(self._h, int(bool(on))), "set_pdl")

    def set_index16(self, on):
        """16-bit neighbour offsets in the FP32 mesh-level kernels (default on)."""
        _check(lib().cfdl_set_index16(self._h, int(bool(on))), "set_index16")

    def index_bytes(self):
        """Bytes per neighbour index of the FP32 mesh-level kernels (2 or 4)."""
        return lib().cfdl_amg_index_bytes(self._h)

    def set_graph_mode(self, on):
        """solve_uvwp as one CUDA graph (True or 1, default), as individual
        launches (False or 0), or as the graph in one chain without its
        parallel branches (2)."""
        mode = on if (isinstance(on, int) and not isinstance(on, bool)) else int(bool(on))
        _check(lib().cfdl_set_graph_mode(self._h, mode), "set_graph_mode")

    def set_config(self, cfg):
        _check(lib().cfdl_set_config(self._h, C.byref(cfg)), "set_config")
        self.config = cfg

    # -- arrays ------------------------------------------------------------
    def _len(self, name):
        nc = self.ne + self.nbf
        if name in ("u", "v", "w", "p", "u0", "v0", "w0", "phic", "t", "e", "e0"):
            return nc
        if name in ("gu", "gv", "gw", "gp", "gpc", "gt", "ge"):
            return 3 * nc
        if name in ("mip", "mip0"):
            return self.nf
        if name == "anb":
            return self.H
        return self.ne

    def get(self, name):
        out = np.zeros(self._len(name))
        _check(lib().cfdl_get_array(self._h, name.encode(), _p(out)), "get " + name)
        return out

    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        if a.size != self._len(name):
            raise ValueError("%s needs %d values" % (name, self._len(name)))
        _check(lib().cfdl_set_array(self._h, name.encode(), _p(a)), "set " + name)

    # -- measurement ---------------------------------------------------------
    def timer_begin(self):
        _check(lib().cfdl_timer_begin(self._h), "timer_begin")

    def timer_end(self):
        ms = C.c_double()
        _check(lib().cfdl_timer_end(self._h, C.byref(ms)), "timer_end")
        return ms.value

    def profile_start(self, kernel=None):
        _check(lib().cfdl_profile_start(self._h, kernel.encode() if kernel else None), "profile_start")

    def profile_stop(self):
        """Returns {kernel: (launches, total_ms)} for the profiled span."""
        n = C.c_int()
        _check(lib().cfdl_profile_stop(self._h, C.byref(n)), "profile_stop")
        out = {}
        name = C.create_string_buffer(64)
        cnt, tot = C.c_int64(), C.c_double()
        for i in range(n.value):
            _check(lib().cfdl_profile_get(self._h, i, name, C.byref(cnt), C.byref(tot)), "profile_get")
            out[name.value.decode()] = (cnt.value, tot.value)
        return out

    def launch_count(self):
        return int(lib().cfdl_launch_count(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().cfdl_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _array_len(name, ne, nf, nbf, H):
    nc = ne + nbf
    if name in ("u", "v", "w", "p", "u0", "v0", "w0", "phic", "t", "e", "e0"):
        return nc
    if name in ("gu", "gv", "gw", "gp", "gpc", "gt", "ge"):
        return 3 * nc
    if name in ("mip", "mip0"):
        return nf
    if name == "anb":
        return H
    return ne


class Batch(Solver):
    """Many independent cases resident in one context and advanced by the same
    launches.  The context-level routines of Solver act on every case; the
    case_* methods address one case by id.  All cases share the pressure-solve
    form (precision, precond)."""

    def __init__(self, setups, configs, u_lids=None):
        setups = list(setups)
        cfg_list = list(configs)
        if not setups or len(setups) != len(cfg_list):
            raise ValueError("one config per setup")
        u_lids = list(u_lids) if u_lids is not None else [1.0] * len(setups)
        self.setup = setups[0]
        self.config = cfg_list[0]
        meshes = (Mesh * len(setups))(*[s.mesh(u) for s, u in zip(setups, u_lids)])
        cfgs = (Config * len(cfg_list))(*cfg_list)
        self._h = C.c_void_p()
        _check(lib().cfdl_batch_create(len(setups), C.cast(meshes, C.c_void_p), C.cast(cfgs, C.c_void_p),
                                       C.byref(self._h)), "batch_create")
        self._sizes = {i: (s.ne, s.nf, s.nbf, s.H) for i, s in enumerate(setups)}
        self.ne, self.nf, self.nbf, self.H = self._sizes[0]
        self.last_stats = Stats()

    def add(self, setup, config, u_lid=1.0):
        mesh = setup.mesh(u_lid)
        cid = C.c_int()
        _check(lib().cfdl_case_add(self._h, C.byref(mesh), C.byref(config), C.byref(cid)), "case_add")
        self._sizes[cid.value] = (setup.ne, setup.nf, setup.nbf, setup.H)
        return cid.value

    def remove(self, cid):
        _check(lib().cfdl_case_remove(self._h, int(cid)), "case_remove")
        self._sizes.pop(cid, None)

    def ids(self):
        n = lib().cfdl_case_count(self._h)
        out = np.zeros(n, dtype=np.int32)
        _check(lib().cfdl_case_ids(self._h, _p(out)), "case_ids")
        return [int(i) for i in out]

    def case_get(self, cid, name):
        out = np.zeros(_array_len(name, *self._sizes[cid]))
        _check(lib().cfdl_case_get_array(self._h, int(cid), name.encode(), _p(out)), "case_get " + name)
        return out

    def case_set(self, cid, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        if a.size != _array_len(name, *self._sizes[cid]):
            raise ValueError("%s has the wrong size" % name)
        _check(lib().cfdl_case_set_array(self._h, int(cid), name.encode(), _p(a)), "case_set " + name)

    def case_stats(self, cid):
        st = Stats()
        _check(lib().cfdl_case_stats(self._h, int(cid), C.byref(st)), "case_stats")
        return st

    def case_info(self, cid):
        ne, nb = C.c_int(), C.c_size_t()
        _check(lib().cfdl_case_info(self._h, int(cid), C.byref(ne), C.byref(nb)), "case_info")
        return ne.value, nb.value


def check_conversions(n=1 << 20):
    """Mismatches (narrowing, widening) of the precision-3 integer conversions
    against the hardware ones; both 0 when they agree."""
    out = np.zeros(2, np.uint32)
    _check(lib().cfdl_check_conversions(int(n), _p(out)), "check_conversions")
    return int(out[0]), int(out[1])


def case_bytes_estimate(ne, nf, nbf, W=6):
    return int(lib().cfdl_case_bytes_estimate(int(ne), int(nf), int(nbf), int(W)))


def server_config(**kw):
    c = ServerConfig()
    lib().cfdl_server_config_default(C.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


class Server:
    """Continuous-batching cavity solver on one device (see cfdl_server_*)."""

    def __init__(self, config=None, **kw):
        self.config = config if config is not None else server_config(**kw)
        self._h = C.c_void_p()
        _check(lib().cfdl_server_create(C.byref(self.config), C.byref(self._h)), "server_create")

    def submit(self, n, tet=False, jitter=0.0, seed=0, re=100.0, conv_tol=1e-6, max_outer=1000, keep_fields=False):
        r = Request(int(n), int(bool(tet)), float(jitter), int(seed), float(re), float(conv_tol), int(max_outer),
                    int(bool(keep_fields)))
        rid = C.c_int64()
        _check(lib().cfdl_server_submit(self._h, C.byref(r), C.byref(rid)), "server_submit")
        return rid.value

    def poll(self, wait_s=0.0, max_results=256):
        out = (Result * max_results)()
        n = C.c_int()
        _check(lib().cfdl_server_poll(self._h, out, max_results, C.byref(n), float(wait_s)), "server_poll")
        return [out[i] for i in range(n.value)]

    def fields(self, rid, name):
        n = C.c_int64()
        _check(lib().cfdl_server_fields(self._h, int(rid), name.encode(), None, C.byref(n)), "server_fields")
        a = np.zeros(n.value)
        _check(lib().cfdl_server_fields(self._h, int(rid), name.encode(), _p(a), C.byref(n)), "server_fields")
        return a

    def drain(self, timeout_s=0.0):
        _check(lib().cfdl_server_drain(self._h, float(timeout_s)), "server_drain")

    def info(self):
        i = ServerInfo()
        _check(lib().cfdl_server_query(self._h, C.byref(i)), "server_query")
        return i.as_dict()

    def now(self):
        return lib().cfdl_server_now(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().cfdl_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
