"""Solver constants from a scene, restating the reference solver constructors.

* time step: ``calc_dt_CFL(0.2, vsound, timeStepSizeMin)`` =
  ``max(dt_min, dt - dt % dt_min)`` with ``dt = 0.2 h / vsound``
  (eng/solver_sph_base.py:209-212); vsound is 60 for WCSPH (eng/solver_sph_wc.py:17),
  24 for mu(I) (eng/solver_sph_muI.py:23) and sqrt(E / rho0) for Drucker-Prager
  (eng/solver_sph_dp.py:18-19);
* material: the first fluid material for WCSPH (eng/solver_sph_wc.py:12-15), the first
  soil material otherwise, with angles converted from degrees
  (eng/solver_sph_muI.py:11-17, eng/solver_sph_dp.py:11-17).
"""
import math

from . import _native as nat
from .particle_func import MAT_FLUID, MAT_SOIL
from .scene import resolve_materials

PRECISIONS = {"fp64": nat.TSG_FP64, "fp32_mixed": nat.TSG_FP32_MIXED}


def calc_dt_cfl(cfl, h, vsound, dt_min):
    dt = cfl * h / vsound
    return max(dt_min, dt - dt % dt_min)


def solver_material(cfg):
    _, fluids, soils, _ = resolve_materials(cfg)
    method = cfg.get_cfg("simulationMethod")
    if method == 1:
        if not fluids:
            raise ValueError("WCSPH needs a fluid material (matType 1)")
        return fluids[0]
    if method in (2, 3):
        if not soils:
            raise ValueError("mu(I) / DP SPH needs a soil material (matType 2)")
        return soils[0]
    raise NotImplementedError(f"Solver type {method} has not been implemented.")


def solver_vsound(method, mat):
    if method == 1:
        return 60
    if method == 2:
        return 24.0
    return math.sqrt(mat["EYoungMod"] / mat["density0"])


def solver_dt(cfg, geom):
    method = cfg.get_cfg("simulationMethod")
    mat = solver_material(cfg)
    return calc_dt_cfl(0.2, geom.smoothing_len, solver_vsound(method, mat), cfg.get_cfg("timeStepSizeMin"))


def native_config(cfg, geom, precision="fp64") -> nat.tsg_config:
    method = cfg.get_cfg("simulationMethod")
    mat = solver_material(cfg)
    c = nat.tsg_config()
    c.dim = geom.dim
    c.solver = method
    c.kernel = cfg.get_cfg("kernel")
    c.kernel_corr = cfg.get_cfg("kernelCorrection")
    c.time_integration = cfg.get_cfg("timeIntegration")
    c.xsph = int(bool(cfg.get_cfg("xsph")))
    c.boundary = cfg.get_cfg("boundary")
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    c.precision = PRECISIONS[precision]
    for d in range(3):
        c.grid_num[d] = int(geom.grid_num[d])
        c.vdomain_start[d] = float(geom.vdomain_start[d])
        c.domain_start[d] = float(geom.domain_start[d])
        c.domain_end[d] = float(geom.domain_end[d])
        c.gravity[d] = float(cfg.get_cfg("gravitation")[d])
    c.grid_num_total = geom.grid_num_total
    c.grid_size = geom.grid_size
    c.support_radius = geom.support_radius
    c.smoothing_len = geom.smoothing_len
    c.particle_diameter = geom.particle_diameter
    c.particle_radius = geom.particle_radius
    c.dt = solver_dt(cfg, geom)
    c.density0 = mat["density0"]
    c.damping_eps = 5e-5
    # FP32-mixed neighbour-list skin (fraction of the support radius); extension key
    c.list_skin = float(cfg.get_cfg_opt("neighbourSkin", 0.05))
    if mat["matType"] == MAT_FLUID:
        c.viscosity = mat["viscosity"]
        c.stiffness = mat["stiffness"]
        c.exponent = mat["exponent"]
        c.exponent_is_int = int(float(mat["exponent"]).is_integer())
    elif mat["matType"] == MAT_SOIL:
        c.cohesion = mat["cohesion"]
        c.friction = mat["friction"] / 180 * math.pi
        c.E = mat["EYoungMod"]
        c.poisson = mat["poison"]
        c.dilatancy = mat["dilatancy"] / 180 * math.pi
        c.init_geostatic = int(method == 3)
    return c
