"""ORACLE - test infrastructure only.

ctypes front end of the f64 CPU oracle (sph_oracle.cpp).  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module, to check
results or to time the CPU restatement; the product package never does.

``OracleSim(cfg)`` builds the initial particle arrays with the same host-side scene
builder every implementation uses, derives the solver's constants the way the reference's
solver constructors do (eng/solver_sph_wc.py:12-21, eng/solver_sph_muI.py:11-25,
eng/solver_sph_dp.py:11-35) and exposes each stage of ``SPHBase.step``
(eng/solver_sph_base.py:41-51) as a method.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

from tisphi_gb300.scene import build_scene, resolve_materials

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

ORC_SORT, ORC_KERNEL_CORR, ORC_INIT_TMP, ORC_ONE_STEP, ORC_ADVECT_FULL, ORC_ADVECT_LF_HALF, \
    ORC_SUBSTEP, ORC_ADVECT_POS, ORC_ADVECT_SOMETHING, ORC_ENFORCE_BOUNDARY, ORC_STEP = range(1, 12)


class orc_params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("solver", ctypes.c_int), ("kernel", ctypes.c_int),
        ("kernel_corr", ctypes.c_int), ("time_integration", ctypes.c_int), ("xsph", ctypes.c_int),
        ("boundary", ctypes.c_int), ("exponent_is_int", ctypes.c_int), ("init_geostatic", ctypes.c_int),
        ("grid_num", ctypes.c_int * 3), ("grid_num_total", ctypes.c_long),
        ("vdomain_start", ctypes.c_double * 3), ("domain_start", ctypes.c_double * 3),
        ("domain_end", ctypes.c_double * 3), ("grid_size", ctypes.c_double),
        ("support_radius", ctypes.c_double), ("smoothing_len", ctypes.c_double),
        ("particle_diameter", ctypes.c_double), ("particle_radius", ctypes.c_double),
        ("gravity", ctypes.c_double * 3), ("dt", ctypes.c_double), ("density0", ctypes.c_double),
        ("viscosity", ctypes.c_double), ("stiffness", ctypes.c_double), ("exponent", ctypes.c_double),
        ("coh", ctypes.c_double), ("fric", ctypes.c_double), ("E", ctypes.c_double),
        ("poi", ctypes.c_double), ("dila", ctypes.c_double), ("damping_eps", ctypes.c_double),
    ]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(orc_params), ctypes.c_int] + [dp] * 7 + [ip] * 4
        L.orc_destroy.argtypes = [P]
        L.orc_n.argtypes = [P]
        L.orc_call.argtypes = [P, ctypes.c_int]
        L.orc_steps.argtypes = [P, ctypes.c_int]
        L.orc_get.argtypes = [P, ctypes.c_char_p, dp]
        L.orc_grid.argtypes = [P, ip]
        L.orc_neighbors.restype = ctypes.c_long
        L.orc_neighbors.argtypes = [P, ip, ip, ctypes.c_long]
        L.orc_error.argtypes = [P]
        L.orc_density_sum.argtypes = [P, ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def calc_dt_cfl(cfl, h, vsound, dt_min):
    """``calc_dt_CFL`` (eng/solver_sph_base.py:209-212)."""
    dt = cfl * h / vsound
    return max(dt_min, dt - dt % dt_min)


def solver_params(cfg, geom):
    """orc_params from a scene, restating the solver constructors' constant set-up."""
    mats = resolve_materials(cfg)
    _, fluids, soils, _ = mats
    p = orc_params()
    p.dim = geom.dim
    p.solver = cfg.get_cfg("simulationMethod")
    p.kernel = cfg.get_cfg("kernel")
    p.kernel_corr = cfg.get_cfg("kernelCorrection")
    p.time_integration = cfg.get_cfg("timeIntegration")
    p.xsph = int(bool(cfg.get_cfg("xsph")))
    p.boundary = cfg.get_cfg("boundary")
    for d in range(3):
        p.grid_num[d] = int(geom.grid_num[d])
        p.vdomain_start[d] = float(geom.vdomain_start[d])
        p.domain_start[d] = float(geom.domain_start[d])
        p.domain_end[d] = float(geom.domain_end[d])
        p.gravity[d] = float(cfg.get_cfg("gravitation")[d])
    p.grid_num_total = geom.grid_num_total
    p.grid_size = geom.grid_size
    p.support_radius = geom.support_radius
    p.smoothing_len = geom.smoothing_len
    p.particle_diameter = geom.particle_diameter
    p.particle_radius = geom.particle_radius
    p.damping_eps = 5e-5
    dt_min = cfg.get_cfg("timeStepSizeMin")
    h = geom.smoothing_len
    if p.solver == 1:
        m = fluids[0]
        p.density0 = m["density0"]
        p.viscosity = m["viscosity"]
        p.stiffness = m["stiffness"]
        p.exponent = m["exponent"]
        p.exponent_is_int = int(float(m["exponent"]).is_integer())
        p.dt = calc_dt_cfl(0.2, h, 60, dt_min)
    else:
        m = soils[0]
        p.density0 = m["density0"]
        p.coh = m["cohesion"]
        p.fric = m["friction"] / 180 * math.pi
        p.E = m["EYoungMod"]
        p.poi = m["poison"]
        p.dila = m["dilatancy"] / 180 * math.pi
        if p.solver == 2:
            p.dt = calc_dt_cfl(0.2, h, 24.0, dt_min)
        else:
            p.dt = calc_dt_cfl(0.2, h, math.sqrt(p.E / p.density0), dt_min)
            p.init_geostatic = 1
    return p


VEC = {"x", "x0", "v", "v_tmp", "d_vel"}
MAT = {"stress", "stress_tmp", "d_stress", "v_grad", "CSPM_L"}


class OracleSim:
    """Oracle instance holding one scene's particles (array of structs, f64)."""

    def __init__(self, cfg, scene=None, params=None):
        self.scene = scene if scene is not None else build_scene(cfg)
        self.params = params if params is not None else solver_params(cfg, self.scene.geom)
        s = self.scene
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in
                      (s.x, s.v, s.density, s.mass, s.m_V, s.pressure, s.stress.reshape(-1, 9))]
        self._keepi = [np.ascontiguousarray(a, dtype=np.int32) for a in (s.mat_type, s.mat_id, s.obj_id, s.is_dynamic)]
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        self.h = lib().orc_create(ctypes.byref(self.params), s.n,
                                  *[a.ctypes.data_as(dp) for a in self._keep],
                                  *[a.ctypes.data_as(ip) for a in self._keepi])
        self.n = s.n

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_destroy(h)
            self.h = None

    def call(self, what):
        return lib().orc_call(self.h, what)

    def sort(self):
        return self.call(ORC_SORT)

    def step(self, nsteps=1):
        return lib().orc_steps(self.h, nsteps)

    def get(self, name):
        shape = (self.n, 3) if name in VEC else (self.n, 3, 3) if name in MAT else (self.n,)
        out = np.zeros(shape, dtype=np.float64)
        rc = lib().orc_get(self.h, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if rc != 0:
            raise KeyError(name)
        return out

    def grid(self):
        out = np.zeros(self.params.grid_num_total + 1, dtype=np.int32)
        lib().orc_grid(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return out

    def neighbors(self):
        """(counts, flat list) of neighbour indices in traversal order."""
        counts = np.zeros(self.n, dtype=np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        total = lib().orc_neighbors(self.h, counts.ctypes.data_as(ip), None, 0)
        lst = np.zeros(max(total, 1), dtype=np.int32)
        lib().orc_neighbors(self.h, counts.ctypes.data_as(ip), lst.ctypes.data_as(ip), total)
        return counts, lst[:total]

    def density_sum(self):
        """calc_density_task summed over every particle's neighbours (current order)."""
        out = np.zeros(self.n, dtype=np.float64)
        lib().orc_density_sum(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def error(self):
        return lib().orc_error(self.h)
