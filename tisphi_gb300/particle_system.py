"""ParticleSystem with the reference's attribute names, backed by the GB300 library.

Mirrors eng/particle_system.py:10-545:

* geometry attributes (``dim``, ``particle_radius``, ``smoothing_len``, ``support_radius``,
  ``grid_size``, ``grid_num``, ``grid_num_total``, ``domain_*``, ``vdomain_*``, ``m_V0``)
  and material-type constants;
* ``particle_num[None]`` and ``particle_max_num``;
* ``pt`` - attribute access to particle fields (``pt.x``, ``pt.density``, ``pt.stress``, ...)
  as torch CUDA tensors that alias the library's device buffers, in the current cell-sorted
  order; re-read them after every step (the sort swaps buffers);
* ``initialize_particle_system()`` - cell hash + prefix sum + stable counting sort;
* ``grid_particle_num`` - inclusive per-cell end offsets after the last sort;
* ``dump()`` - the two dicts of numpy arrays that the reference's export writes
  (eng/particle_system.py:459-545).

The device instance (one ``tsg_handle``) is created here from the scene, including the
solver constants, because the library fuses the particle system and the solver state.
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from .params import native_config, solver_dt
from .particle_func import MAT_DUMMY, MAT_FLUID, MAT_REP, MAT_RIGID, MAT_SOIL
from .scene import (BDY_COLLISION, BDY_DUMMY, BDY_DUMMY_REP, BDY_NONE, BDY_REP, build_scene,
                    resolve_materials, scene_geometry)


class _Scalar:
    """``field[None]`` access for the reference's 0-d Taichi fields."""

    def __init__(self, getter, setter=None):
        self._get = getter
        self._set = setter

    def __getitem__(self, key):
        return self._get()

    def __setitem__(self, key, value):
        if self._set is None:
            raise AttributeError("this scalar is read-only")
        self._set(value)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Fields:
    """Attribute access to particle fields (the reference's ``pt`` struct field)."""

    NAMES = ("x", "v", "x0", "density", "mass", "m_V", "pressure", "stress", "strain_equ", "strain_equ_p",
             "flag_retmap", "mat_type", "mat_id", "obj_id", "is_dynamic", "id0", "v_tmp", "density_tmp",
             "stress_tmp", "d_density", "d_vel", "d_stress", "v_grad", "CSPM_f", "CSPM_L", "d_strain_equ",
             "d_strain_equ_p")

    def __init__(self, ps):
        object.__setattr__(self, "_ps", ps)

    def __getattr__(self, name):
        if name not in self.NAMES:
            raise AttributeError(name)
        return self._ps.field(name)

    def __setattr__(self, name, value):
        raise AttributeError("assign through the tensor view, e.g. ps.pt.v[:] = ...")


class ParticleSystem:
    mat_dummy_type, mat_rep_type = MAT_DUMMY, MAT_REP
    mat_fluid_type, mat_soil_type, mat_rigid_type = MAT_FLUID, MAT_SOIL, MAT_RIGID
    bdy_none, bdy_collision, bdy_dummy, bdy_rep, bdy_dummy_rep = (BDY_NONE, BDY_COLLISION, BDY_DUMMY,
                                                                  BDY_REP, BDY_DUMMY_REP)

    def __init__(self, config, precision=None, device=None) -> None:
        self.cfg = config
        g = scene_geometry(config)
        self.geom = g
        self.dim = g.dim
        self.dim3 = 3
        self.domain_start = g.domain_start
        self.domain_end = g.domain_end
        self.domain_size = g.domain_end - g.domain_start
        self.vdomain_start = g.vdomain_start
        self.vdomain_end = g.vdomain_end
        self.vdomain_size = g.vdomain_end - g.vdomain_start
        self.particle_radius = g.particle_radius
        self.particle_diameter = g.particle_diameter
        self.kappa = config.get_cfg("kappa")
        self.kh = config.get_cfg("kh")
        self.smoothing_len = g.smoothing_len
        self.support_radius = g.support_radius
        self.m_V0 = g.m_V0
        self.grid_size = g.grid_size
        self.grid_num = g.grid_num
        self.grid_num_total = g.grid_num_total
        self.flag_boundary = config.get_cfg("boundary")
        self.mat_index, self.mat_fluid, self.mat_soil, self.mat_rigid = resolve_materials(config)
        self.precision = precision or config.get_cfg_opt("precision", "fp64")
        self.scene = build_scene(config, g)
        self.object_collection = {b["objectId"]: b for b in config.get_blocks()}
        self.particle_max_num = self.scene.n
        self.dt_value = solver_dt(config, g)
        if device is not None:
            torch.cuda.set_device(device)
        self._lib = nat.load()
        self._cfg = native_config(config, g, self.precision)
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_create(ctypes.byref(self._cfg), ctypes.byref(h)), "tsg_create")
        self._h = h
        parts, keep = nat.host_particles(self.scene)
        nat.check(self._lib.tsg_upload(self._h, ctypes.byref(parts), 0, _stream()), "tsg_upload")
        del keep
        self.particle_num = _Scalar(lambda: int(self._lib.tsg_particle_num(self._h)))
        self.pt = _Fields(self)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.tsg_destroy(h)
            self._h = None

    # ---- field views -------------------------------------------------------------
    def field(self, name):
        """torch CUDA tensor aliasing one particle field (valid until the next sort)."""
        v = nat.tsg_view()
        nat.check(self._lib.tsg_field(self._h, name.encode(), ctypes.byref(v), _stream()), f"field {name}")
        return torch.as_tensor(nat.DeviceArray(v, self), device="cuda")

    def write_field(self, name, src):
        """Copy a row-major (n, k) buffer (numpy array or torch tensor, host or CUDA) into a field."""
        if isinstance(src, torch.Tensor):
            assert src.is_contiguous()
            ptr, dev = src.data_ptr(), int(src.is_cuda)
        else:
            src = np.ascontiguousarray(src)
            ptr, dev = src.ctypes.data, 0
        nat.check(self._lib.tsg_write(self._h, name.encode(), ctypes.c_void_p(ptr), dev, _stream()), f"write {name}")

    def read_field(self, name, dst, non_blocking=False):
        """Copy a field into a row-major (n, k) buffer (numpy array or torch tensor, host or CUDA).
        non_blocking (host buffers): return without synchronising - the copy completes in
        stream order, so synchronise (torch.cuda.synchronize) before reading dst; use pinned
        memory."""
        if isinstance(dst, torch.Tensor):
            assert dst.is_contiguous()
            ptr, dev = dst.data_ptr(), int(dst.is_cuda)
        else:
            assert dst.flags.c_contiguous
            ptr, dev = dst.ctypes.data, 0
        mode = dev if dev or not non_blocking else 2
        nat.check(self._lib.tsg_read(self._h, name.encode(), ctypes.c_void_p(ptr), mode, _stream()), f"read {name}")
        return dst

    def read_fields(self, names, dsts, non_blocking=False):
        """read_field for several fields in one call (the FP32-mixed form converts them in one
        pass before the copies); the destinations are all host or all CUDA buffers."""
        ptrs, devs = [], set()
        for dst in dsts:
            if isinstance(dst, torch.Tensor):
                assert dst.is_contiguous()
                ptrs.append(dst.data_ptr())
                devs.add(int(dst.is_cuda))
            else:
                assert dst.flags.c_contiguous
                ptrs.append(dst.ctypes.data)
                devs.add(0)
        if len(devs) != 1:
            raise ValueError("read_fields: mixed host and device destinations")
        dev = devs.pop()
        mode = dev if dev or not non_blocking else 2
        cnames = (ctypes.c_char_p * len(names))(*[nm.encode() for nm in names])
        cptrs = (ctypes.c_void_p * len(ptrs))(*ptrs)
        nat.check(self._lib.tsg_read_fields(self._h, len(names), cnames, cptrs, mode, _stream()), "read_fields")
        return dsts

    @property
    def grid_particle_num(self):
        """Inclusive end offset of every cell after the last sort (host numpy, int32)."""
        out = np.zeros(self.grid_num_total + 1, dtype=np.int32)
        nat.check(self._lib.tsg_grid(self._h, nat.as_ptr(out, ctypes.c_int32), _stream()), "tsg_grid")
        return out[: self.grid_num_total]

    # ---- hot path ----------------------------------------------------------------
    def initialize_particle_system(self):
        nat.check(self._lib.tsg_sort(self._h, _stream()), "tsg_sort")

    def neighbors(self):
        """(counts, flat list) of neighbour indices in the reference's traversal order."""
        n = self.particle_max_num
        counts = np.zeros(n, dtype=np.int32)
        total = ctypes.c_int64()
        nat.check(self._lib.tsg_neighbors(self._h, nat.as_ptr(counts, ctypes.c_int32), None, 0,
                                          ctypes.byref(total), _stream()), "tsg_neighbors")
        lst = np.zeros(max(total.value, 1), dtype=np.int32)
        nat.check(self._lib.tsg_neighbors(self._h, nat.as_ptr(counts, ctypes.c_int32),
                                          nat.as_ptr(lst, ctypes.c_int32), lst.size, ctypes.byref(total),
                                          _stream()), "tsg_neighbors")
        return counts, lst[: total.value]

    def diagnostics(self):
        """FP64 totals over flow particles: mass, momentum (3), kinetic, potential, max|v|, front."""
        out = np.zeros(8, dtype=np.float64)
        nat.check(self._lib.tsg_reduce_diag(self._h, nat.as_ptr(out, ctypes.c_double), _stream()), "diag")
        return {"mass": out[0], "momentum": out[1:4].copy(), "kinetic": out[4], "potential": out[5],
                "vmax": out[6], "front": out[7]}

    def visual(self, w2s_ratio=None, color_title=None, color_group=None, show_bdy=None, given_max=-1.0,
               given_min=-1.0, fix_max=False, fix_min=False, pos=None, color=None):
        """Headless replacement of the GUI inputs (assign_value_color + v_maxmin + set_color +
        copy2vis, eng/solver_sph_base.py:721-785, eng/particle_system.py:380-407): returns
        (pos2vis, color, (vmax, vmin)) with pos2vis / color float32 CUDA tensors (n, 3) indexed
        by id0.  Defaults come from the scene (colorTitle, colorGroup, showBdyPts) and
        w2s_ratio = 1 / max(domain size) as the reference's GUI sets it (eng/ui_sim.py:33)."""
        cfg = self.cfg
        vc = nat.tsg_visual_cfg()
        vc.color_title = int(cfg.get_cfg("colorTitle") if color_title is None else color_title)
        vc.color_group = int(cfg.get_cfg("colorGroup") if color_group is None else color_group)
        vc.show_bdy = int(bool(cfg.get_cfg("showBdyPts") if show_bdy is None else show_bdy))
        vc.fix_max, vc.fix_min = int(bool(fix_max)), int(bool(fix_min))
        vc.w2s_ratio = float(1.0 / max(self.domain_size) if w2s_ratio is None else w2s_ratio)
        vc.given_max, vc.given_min = float(given_max), float(given_min)
        n = self.particle_max_num
        pos = torch.zeros((n, 3), dtype=torch.float32, device="cuda") if pos is None else pos
        color = torch.zeros((n, 3), dtype=torch.float32, device="cuda") if color is None else color
        rng = np.zeros(2, dtype=np.float64)
        nat.check(self._lib.tsg_visual(self._h, ctypes.byref(vc), ctypes.c_void_p(pos.data_ptr()),
                                       ctypes.c_void_p(color.data_ptr()), nat.as_ptr(rng, ctypes.c_double),
                                       _stream()), "tsg_visual")
        return pos, color, (float(rng[0]), float(rng[1]))

    def list_stats(self):
        """FP32-mixed neighbour-list occupancy: entries of real / dummy particles, overflowed
        particles, list builds since upload and dummies with a non-empty list (raises for the
        FP64 form, which keeps no lists)."""
        out = np.zeros(5, dtype=np.int64)
        nat.check(self._lib.tsg_list_stats(self._h, nat.as_ptr(out, ctypes.c_int64), _stream()), "list_stats")
        return {"entries_real": int(out[0]), "entries_dummy": int(out[1]), "overflowed": int(out[2]),
                "builds": int(out[3]), "listed_dummies": int(out[4])}

    def check_errors(self):
        """Raise when the device error word has bits set (synchronises)."""
        rc = self._lib.tsg_last_error(self._h, _stream())
        if rc != 0:
            raise nat.NativeError(rc, "device error word")

    # ---- export ------------------------------------------------------------------
    def dump(self):
        """Host copies of the exported fields (eng/particle_system.py:459-545)."""
        f = lambda name: self.field(name).detach().cpu().numpy()
        x = f("x")
        v = f("v")
        out_pos = {"pos.x": x[:, 0].copy(), "pos.y": x[:, 1].copy(), "pos.z": x[:, 2].copy()}
        data = {
            "id0": f("id0").astype(np.int64),
            "objId": f("obj_id").astype(np.int64),
            "material": f("mat_type").astype(np.int64),
            "density": f("density"),
            "vel.x": v[:, 0].copy(), "vel.y": v[:, 1].copy(), "vel.z": v[:, 2].copy(),
            "vel.norm": np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]),
        }
        n = x.shape[0]
        if self.cfg.get_cfg("simulationMethod") != 1:
            s = f("stress")
            data.update({"stress.xx": s[:, 0, 0].copy(), "stress.yy": s[:, 1, 1].copy(),
                         "stress.zz": s[:, 2, 2].copy(), "stress.xy": s[:, 0, 1].copy(),
                         "stress.yz": s[:, 1, 2].copy(), "stress.zx": s[:, 2, 0].copy(),
                         "stress.hydro": ((s[:, 0, 0] + s[:, 1, 1]) + s[:, 2, 2]) / 3.0,
                         "strain_equ": f("strain_equ"), "strain_equ_p": f("strain_equ_p")})
            data["plas_behav"] = f("flag_retmap").astype(np.float64)
        else:
            z = np.zeros(n)
            data.update({"stress.xx": z, "stress.yy": z, "stress.zz": z, "stress.xy": z, "stress.yz": z,
                         "stress.zx": z, "stress.hydro": z, "strain_equ": z, "strain_equ_p": z,
                         "plas_behav": z})
        data["pressure"] = f("pressure")
        return out_pos, data
