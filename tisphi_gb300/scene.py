"""Scene geometry and initial particle arrays, built on the host with numpy.

``SceneGeometry`` restates the discretisation block of the reference's
``ParticleSystem.__init__`` (eng/particle_system.py:32-59):

* ``particle_diameter = 2 r``, ``smoothing_len h = kh * 2r``, ``support_radius = kappa * h``,
  ``m_V0 = (2r) ** dim``;
* ``grid_size = ceil(kappa * kh) * 2r``; the virtual domain is the domain padded by one
  cell on every side, except that in 2D the z extent collapses to one particle diameter;
* ``grid_num = ceil(vdomain_size / grid_size)`` and ``grid_num_total`` is the product of
  the first ``dim`` entries.

``build_scene`` restates the particle generation of ``ParticleSystem.__init__`` /
``initialize_particles`` (eng/particle_system.py:71-148, eng/particle_func.py:176-208):
blocks first (in file order), then dummy-boundary boxes, then repulsive boxes.  Dummy
particles get ``density = 0`` and ``mass = 0`` (``add_cube`` defaults,
eng/particle_func.py:206) and ``obj_id = mat_type = -1`` (eng/particle_func.py:308-313).

The optional seeded jitter (``Configuration.jitter`` = amplitude in metres,
``Configuration.seed``) perturbs fluid/soil positions by uniform noise in
``[-jitter, +jitter]`` per active axis, drawn from numpy ``PCG64(seed)`` in particle
order.  The reference generates exact lattices; the jitter is an input transform that
every implementation receives identically.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from .particle_func import (MAT_DUMMY, MAT_FLUID, MAT_REP, MAT_RIGID, MAT_SOIL,
                            calc_cube_particle_num, calc_dummy_boundary, calc_rep_boundary,
                            chk_block_in_domain, cube_lattice)

BDY_NONE, BDY_COLLISION, BDY_DUMMY, BDY_REP, BDY_DUMMY_REP = 0, 1, 2, 3, 4


@dataclass
class SceneGeometry:
    dim: int
    domain_start: np.ndarray
    domain_end: np.ndarray
    vdomain_start: np.ndarray
    vdomain_end: np.ndarray
    particle_radius: float
    particle_diameter: float
    smoothing_len: float
    support_radius: float
    m_V0: float
    grid_size: float
    grid_num: np.ndarray
    grid_num_total: int


def scene_geometry(cfg) -> SceneGeometry:
    """Discretisation constants (eng/particle_system.py:14-59)."""
    dim = 3 if not cfg.get_cfg("is2D") else 2
    ds = np.array(cfg.get_cfg("domainStart"))
    de = np.array(cfg.get_cfg("domainEnd"))
    dsize = de - ds
    r = cfg.get_cfg("particleRadius")
    kappa = cfg.get_cfg("kappa")
    kh = cfg.get_cfg("kh")
    d = 2 * r
    h = kh * d
    R = kappa * h
    m_V0 = d ** dim
    g = math.ceil(kappa * kh) * d
    vs = ds - g
    ve = de + g
    vsize = ve - vs
    if dim == 2:
        de[2] = ds[2] + d
        dsize[2] = d
        vs[2] = ds[2]
        ve[2] = vs[2] + d
        vsize[2] = d
    grid_num = np.ceil(vsize / g).astype(int)
    G = int(np.prod(grid_num[0:dim]).item())
    return SceneGeometry(dim=dim, domain_start=ds.astype(np.float64), domain_end=de.astype(np.float64),
                         vdomain_start=vs.astype(np.float64), vdomain_end=ve.astype(np.float64),
                         particle_radius=r, particle_diameter=d, smoothing_len=h, support_radius=R,
                         m_V0=m_V0, grid_size=g, grid_num=grid_num, grid_num_total=G)


def resolve_materials(cfg):
    """(mat_index, fluids, soils, rigids) as ``set_material`` (eng/particle_func.py:218-236)."""
    mat_index, fluids, soils, rigids = [], [], [], []
    for mat in cfg.get_materials():
        t = mat["matType"]
        if t == MAT_FLUID:
            mat_index.append((MAT_FLUID, len(fluids)))
            fluids.append(mat)
        elif t == MAT_SOIL:
            mat_index.append((MAT_SOIL, len(soils)))
            soils.append(mat)
        elif t == MAT_RIGID:
            mat_index.append((MAT_RIGID, len(rigids)))
            rigids.append(mat)
    return mat_index, fluids, soils, rigids


def get_material(mats, i):
    """Material record by position in the Materials list (eng/particle_func.py:238-244)."""
    mat_index, fluids, soils, rigids = mats
    t, k = mat_index[i]
    return {MAT_FLUID: fluids, MAT_SOIL: soils, MAT_RIGID: rigids}[t][k]


@dataclass
class SceneArrays:
    geom: SceneGeometry
    x: np.ndarray            # (N, 3) f64
    v: np.ndarray            # (N, 3) f64
    density: np.ndarray      # (N,) f64
    pressure: np.ndarray     # (N,) f64
    mass: np.ndarray         # (N,) f64
    m_V: np.ndarray          # (N,) f64
    stress: np.ndarray       # (N, 3, 3) f64
    mat_type: np.ndarray     # (N,) int32
    mat_id: np.ndarray       # (N,) int32
    obj_id: np.ndarray       # (N,) int32
    is_dynamic: np.ndarray   # (N,) int32
    color: np.ndarray        # (N, 3) f32
    object_counts: dict = field(default_factory=dict)

    @property
    def n(self):
        return self.x.shape[0]

    def count(self, mat_type):
        return int(np.count_nonzero(self.mat_type == mat_type))


def build_scene(cfg, geom: SceneGeometry = None) -> SceneArrays:
    """Initial particle arrays in the reference's order (eng/particle_system.py:71-148)."""
    g = geom if geom is not None else scene_geometry(cfg)
    mats = resolve_materials(cfg)
    flag_boundary = cfg.get_cfg("boundary")
    parts = []
    object_counts = {}

    def add(pts, vel, density, mat_id, mat_type, obj_id, is_dynamic, color):
        n = pts.shape[0]
        parts.append(dict(
            x=pts,
            v=np.tile(np.asarray(vel, dtype=np.float64), (n, 1)) if vel is not None else np.zeros((n, 3)),
            density=np.full(n, float(density), dtype=np.float64),
            mat_id=np.full(n, mat_id, dtype=np.int32),
            mat_type=np.full(n, mat_type, dtype=np.int32),
            obj_id=np.full(n, obj_id, dtype=np.int32),
            is_dynamic=np.full(n, int(is_dynamic), dtype=np.int32),
            color=np.tile(np.asarray(color, dtype=np.float32), (n, 1))))

    for block in cfg.get_blocks():
        chk_block_in_domain(g.domain_start, g.domain_end, block["translation"], block["size"], g.dim)
        mat = get_material(mats, block["materialId"])
        mat_type = mat["matType"]
        if mat_type > 10:
            is_dynamic = bool(block["isDynamic"])
        else:
            is_dynamic = True
        pts = cube_lattice(np.array(block["translation"]), np.array(block["size"]), g.dim, g.particle_diameter)
        color = np.array([c / 255 for c in mat["color"]], dtype=np.float32)
        add(pts, block["velocity"], mat["density0"], block["materialId"], mat_type, block["objectId"],
            is_dynamic, color)
        object_counts[block["objectId"]] = pts.shape[0]

    # mesh bodies (eng/particle_system.py:82-91, :175-200): voxelised at the particle diameter
    for body in cfg.get_bodies() or []:
        if g.dim != 3:
            raise NotImplementedError("mesh bodies need a 3D scene (the voxel grid is 3D)")
        from .mesh_body import load_body
        mat = get_material(mats, body["materialId"])
        mat_type = mat["matType"]
        is_dynamic = bool(body["isDynamic"]) if mat_type > 10 else True
        pts = load_body(body, g.particle_diameter, base_dir=getattr(cfg, "base_dir", None))
        color = np.array([c / 255 for c in mat["color"]], dtype=np.float32)
        add(pts, body.get("velocity", [0.0, 0.0, 0.0]), mat["density0"], body["materialId"], mat_type,
            body["objectId"], is_dynamic, color)
        object_counts[body["objectId"]] = pts.shape[0]

    if flag_boundary in (BDY_DUMMY, BDY_DUMMY_REP):
        for lo, hi in calc_dummy_boundary(g.dim, g.domain_start, g.domain_end, g.vdomain_start, g.vdomain_end):
            pts = cube_lattice(lo, hi - lo, g.dim, g.particle_diameter)
            add(pts, None, 0.0, 0, MAT_DUMMY, MAT_DUMMY, True, np.array([153, 153, 255]) / 255)
    if flag_boundary in (BDY_REP, BDY_DUMMY_REP):
        for lo, hi in calc_rep_boundary(g.dim, g.domain_start, g.domain_end, g.particle_radius):
            pts = cube_lattice(lo, hi - lo, g.dim, g.particle_radius)
            add(pts, None, 0.0, 0, MAT_REP, MAT_REP, True, np.array([170, 17, 255]) / 255)

    cat = {k: np.concatenate([p[k] for p in parts], axis=0) for k in parts[0]}
    n = cat["x"].shape[0]
    x = cat["x"]
    jitter = cfg.get_cfg_opt("jitter", 0.0) or 0.0
    if jitter > 0.0:
        flow = np.nonzero((cat["mat_type"] == MAT_FLUID) | (cat["mat_type"] == MAT_SOIL))[0]
        rng = np.random.Generator(np.random.PCG64(int(cfg.get_cfg_opt("seed", 0))))
        noise = rng.uniform(-jitter, jitter, size=(flow.size, g.dim))
        x = x.copy()
        x[flow, :g.dim] += noise
    density = cat["density"]
    m_V = np.full(n, g.m_V0, dtype=np.float64)
    return SceneArrays(geom=g, x=np.ascontiguousarray(x), v=cat["v"], density=density,
                       pressure=np.zeros(n), mass=g.m_V0 * density, m_V=m_V,
                       stress=np.zeros((n, 3, 3)), mat_type=cat["mat_type"], mat_id=cat["mat_id"],
                       obj_id=cat["obj_id"], is_dynamic=cat["is_dynamic"], color=cat["color"],
                       object_counts=object_counts)
