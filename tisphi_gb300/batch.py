"""Batched ensembles: many independent WCSPH scenes stepped by one set of launches.

The reference runs one scene per process (run_simulation.py); sweeping stiffness,
viscosity or block size means hundreds of small runs that each leave a GB300 mostly idle.
``SceneBatch`` uploads every scene into one FP32-mixed handle (``tsg_batch_create``): the
scenes sit side by side along x, far enough apart that no neighbour pair crosses scenes,
each particle carries its scene number (for the per-scene stiffness and viscosity), and
every kernel of a step covers all scenes at once.  A step is a replay of a captured CUDA
graph whose re-sort runs only when the device-side displacement check asks for it, and
``autotune()`` picks the launch shape (threads per block, cells per CTA of the list build,
steps per graph) by timing candidates from a saved state.

Scenes must share the geometry, kernel, integrator and dummy boundary; stiffness,
viscosity and particle counts may differ (``scenes.dambreak_ensemble``).
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from .configer_builder import SimConfiger
from .params import native_config
from .particle_func import MAT_FLUID
from .scene import build_scene, scene_geometry

DIAG_KEYS = ("mass", "momentum_x", "momentum_y", "momentum_z", "kinetic", "potential", "vmax", "front")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class SceneBatch:
    def __init__(self, configs):
        self.cfgs = [c if isinstance(c, SimConfiger) else SimConfiger(config=c) for c in configs]
        if not self.cfgs:
            raise ValueError("a batch needs at least one scene")
        self.geoms = [scene_geometry(c) for c in self.cfgs]
        self.scenes = [build_scene(c, g) for c, g in zip(self.cfgs, self.geoms)]
        self.nscenes = len(self.scenes)
        self._lib = nat.load()
        ncfg = (nat.tsg_config * self.nscenes)(*[native_config(c, g, "fp32_mixed")
                                                 for c, g in zip(self.cfgs, self.geoms)])
        parts = (nat.tsg_particles * self.nscenes)()
        keep = []
        for q, sc in enumerate(self.scenes):
            p, k = nat.host_particles(sc)
            parts[q] = p
            keep.append(k)
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_batch_create(ncfg, ctypes.cast(parts, ctypes.c_void_p), self.nscenes, _stream(),
                                             ctypes.byref(h)), "tsg_batch_create")
        self._h = h
        del keep
        self.counts = np.array([sc.n for sc in self.scenes], dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)])
        self.n_fluid = np.array([sc.count(MAT_FLUID) for sc in self.scenes], dtype=np.int64)
        self.pitch = float(self._lib.tsg_batch_pitch(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.tsg_destroy(h)
            self._h = None

    @property
    def n(self):
        return int(self.offsets[-1])

    # ---- stepping and launch shape ----------------------------------------------------
    def step(self, nsteps=1):
        nat.check(self._lib.tsg_step(self._h, int(nsteps), _stream()), "tsg_step")

    def get_launch(self):
        c = nat.tsg_launch_cfg()
        nat.check(self._lib.tsg_get_launch(self._h, ctypes.byref(c)), "tsg_get_launch")
        return {"threads_per_block": c.threads_per_block, "cells_per_cta": c.cells_per_cta,
                "steps_per_graph": c.steps_per_graph}

    def set_launch(self, threads_per_block=128, cells_per_cta=0, steps_per_graph=1):
        c = nat.tsg_launch_cfg(threads_per_block, cells_per_cta, steps_per_graph)
        nat.check(self._lib.tsg_set_launch(self._h, ctypes.byref(c)), "tsg_set_launch")

    def autotune(self, trial_steps=10):
        """Time launch-shape candidates from the current state (which is restored) and keep
        the fastest; returns it with the best milliseconds per step."""
        c = nat.tsg_launch_cfg()
        ms = ctypes.c_double()
        nat.check(self._lib.tsg_autotune(self._h, int(trial_steps), ctypes.byref(c), ctypes.byref(ms), _stream()),
                  "tsg_autotune")
        return {"threads_per_block": c.threads_per_block, "cells_per_cta": c.cells_per_cta,
                "steps_per_graph": c.steps_per_graph, "ms_per_step": ms.value}

    # ---- results --------------------------------------------------------------------
    def diagnostics(self):
        """Per-scene FP64 totals of the flow particles (positions in each scene's own frame)."""
        out = np.zeros((self.nscenes, 8), dtype=np.float64)
        nat.check(self._lib.tsg_batch_diag(self._h, nat.as_ptr(out, ctypes.c_double), self.nscenes, _stream()),
                  "tsg_batch_diag")
        return [dict(zip(DIAG_KEYS, row)) for row in out]

    def field(self, name):
        """torch CUDA tensor over every particle of the batch (current sorted order; x carries
        the scene shift q * pitch)."""
        v = nat.tsg_view()
        nat.check(self._lib.tsg_field(self._h, name.encode(), ctypes.byref(v), _stream()), f"field {name}")
        return torch.as_tensor(nat.DeviceArray(v, self), device="cuda")

    def scene_field(self, name, q):
        """Field of scene q as numpy, in that scene's upload order (positions unshifted)."""
        ids = self.field("id0").long()
        lo, hi = int(self.offsets[q]), int(self.offsets[q + 1])
        sel = (ids >= lo) & (ids < hi)
        order = torch.argsort(ids[sel])
        a = self.field(name)[sel][order].to(torch.float64).cpu().numpy().copy()
        if name in ("x", "x0"):
            a[:, 0] -= q * self.pitch
        return a

    def check_errors(self):
        rc = self._lib.tsg_last_error(self._h, _stream())
        if rc != 0:
            raise nat.NativeError(rc, "device error word")

    def list_stats(self):
        out = np.zeros(5, dtype=np.int64)
        nat.check(self._lib.tsg_list_stats(self._h, nat.as_ptr(out, ctypes.c_int64), _stream()), "list_stats")
        return {"entries_real": int(out[0]), "entries_dummy": int(out[1]), "overflowed": int(out[2]),
                "builds": int(out[3]), "listed_dummies": int(out[4])}
