"""Differentiable WCSPH and mu(I) rollouts behind ``torch.autograd.Function``.

``WCRollout`` runs a 2D WCSPH scene and ``MuIRollout`` a 2D mu(I) scene (symplectic Euler,
dummy boundary, no kernel correction, no XSPH) in the FP32-mixed form and expose the final
fluid / soil positions as a function of two material parameters: the Tait stiffness B (Pa)
and the kinematic viscosity for WCSPH, the friction angle (degrees) and the cohesion (Pa)
for mu(I).  The backward pass is the library's hand-written adjoint (``tsg_adjoint_step``),
with checkpointed recomputation: the forward keeps a bitwise state snapshot every
``checkpoint_every`` steps; the backward walks the segments in reverse, re-runs each
segment from its checkpoint keeping a snapshot per step, then reverses the steps one by
one, each from its own snapshot (the adjoint step repeats the forward bit for bit before
reversing it).  Memory: one snapshot per checkpoint plus one per step of one segment.

Neighbour lists are rebuilt every step (skin 0), so a step re-run from a snapshot re-sorts
exactly as the original step did.

    model = MuIRollout(scenes.column_2d(method=2, spacing=0.002, dt=2e-5), nsteps=2000)
    params = torch.tensor([21.9, 0.0], dtype=torch.float64, requires_grad=True)
    x = model(params)                        # (n_soil, 2) final positions, f64
    sel = torch.topk(x[:, 0], k).indices     # the most distal particles (a fixed set)
    loss = ((x[sel, 0] - 0.35) ** 2).mean()
    loss.backward()                          # params.grad = (dL/dphi, dL/dcohesion)

    model = WCRollout(scenes.dambreak_2d(...), nsteps=2000)
    params = torch.tensor([5e4, 5e-3], dtype=torch.float64, requires_grad=True)  # B, nu
"""
import copy
import ctypes
import math

import numpy as np
import torch

from . import _native as nat
from .configer_builder import SimConfiger
from .particle_func import MAT_FLUID, MAT_SOIL


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class _AdjointRollout:
    """Shared machinery: snapshots, stepping and the output particles' positions."""
    METHOD = None        # simulationMethod the rollout covers
    OUT_TYPE = None      # material type whose final positions are the output

    def __init__(self, cfg, nsteps, checkpoint_every=100, precision="fp32_mixed"):
        from .simulation import Simulation
        d = copy.deepcopy(cfg.config if isinstance(cfg, SimConfiger) else cfg)
        d["Configuration"]["neighbourSkin"] = 0.0
        c = d["Configuration"]
        if c.get("simulationMethod") != self.METHOD or c.get("timeIntegration") != 1:
            raise ValueError(f"{type(self).__name__} covers simulationMethod {self.METHOD} with symplectic Euler")
        self.cfg_dict = d
        self.nsteps = int(nsteps)
        self.checkpoint_every = max(1, int(checkpoint_every))
        self.precision = precision
        self.sim = Simulation(SimConfiger(config=d), precision=precision)
        self.ps = self.sim.ps
        self._lib = nat.load()
        self._h = self.ps._h
        self.n = self.ps.particle_max_num
        mt = np.asarray(self.ps.scene.mat_type)
        self.out_ids = torch.as_tensor(np.nonzero(mt == self.OUT_TYPE)[0], device="cuda")
        if precision == "fp32_mixed":
            self.nbytes = int(self._lib.tsg_snapshot_bytes(self._h))
            self.initial = self.save()

    # ---- state ----------------------------------------------------------------------
    def save(self):
        buf = torch.empty(self.nbytes, dtype=torch.uint8, device="cuda")
        nat.check(self._lib.tsg_snapshot_save(self._h, _ptr(buf), _stream()), "tsg_snapshot_save")
        return buf

    def load(self, buf):
        nat.check(self._lib.tsg_snapshot_load(self._h, _ptr(buf), _stream()), "tsg_snapshot_load")

    def step(self, n=1):
        nat.check(self._lib.tsg_step(self._h, int(n), _stream()), "tsg_step")

    def positions(self):
        """Final (x, y) of the output particles in upload order, f64."""
        x = self.ps.field("x").to(torch.float64)
        ids = self.ps.field("id0").long()
        out = torch.empty_like(x)
        out[ids] = x
        return out[self.out_ids, :2].clone()

    def run(self, *params):
        """Final positions for the given parameters, without gradient (FP32-mixed)."""
        self.set_params(*params)
        self.load(self.initial)
        self.step(self.nsteps)
        return self.positions()

    def __call__(self, params):
        return _Rollout.apply(params, self)


class MuIRollout(_AdjointRollout):
    """mu(I) column: parameters (friction angle in degrees, cohesion in Pa)."""
    METHOD, OUT_TYPE = 2, MAT_SOIL

    def __init__(self, cfg, nsteps, checkpoint_every=100, precision="fp32_mixed"):
        super().__init__(cfg, nsteps, checkpoint_every, precision)
        self.soil_ids = self.out_ids
        self.friction_deg = float(self.ps.mat_soil[0]["friction"])
        self.cohesion = float(self.ps.mat_soil[0]["cohesion"])

    def set_params(self, friction_deg, cohesion):
        self.friction_deg, self.cohesion = float(friction_deg), float(cohesion)
        nat.check(self._lib.tsg_set_soil(self._h, self.friction_deg / 180.0 * math.pi, self.cohesion),
                  "tsg_set_soil")

    def soil_positions(self):
        return self.positions()

    def param_grads(self, pbar):
        mu_bar, coh_bar = pbar
        mu = math.tan(self.friction_deg / 180.0 * math.pi)
        return [mu_bar * (1.0 + mu * mu) * math.pi / 180.0, coh_bar]   # d tan(phi) / d phi_deg


class WCRollout(_AdjointRollout):
    """WCSPH scene: parameters (Tait stiffness B in Pa, kinematic viscosity)."""
    METHOD, OUT_TYPE = 1, MAT_FLUID

    def __init__(self, cfg, nsteps, checkpoint_every=100, precision="fp32_mixed"):
        super().__init__(cfg, nsteps, checkpoint_every, precision)
        self.fluid_ids = self.out_ids
        self.stiffness = float(self.ps.mat_fluid[0]["stiffness"])
        self.viscosity = float(self.ps.mat_fluid[0]["viscosity"])

    def set_params(self, stiffness, viscosity):
        self.stiffness, self.viscosity = float(stiffness), float(viscosity)
        nat.check(self._lib.tsg_set_fluid(self._h, self.stiffness, self.viscosity), "tsg_set_fluid")

    def param_grads(self, pbar):
        b_bar, nu_fac_bar = pbar
        return [b_bar, nu_fac_bar * 2.0 * (self.ps.dim + 2)]  # nu' = 2 (dim + 2) nu


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, model):
        model.set_params(*(float(v) for v in params.detach().cpu().tolist()))
        model.load(model.initial)
        ckpts = []
        for t in range(model.nsteps):
            if t % model.checkpoint_every == 0:
                ckpts.append(model.save())
            model.step(1)
        ctx.model = model
        ctx.ckpts = ckpts
        ctx.param_device = params.device
        return model.positions()

    @staticmethod
    def backward(ctx, gx):
        model = ctx.model
        lib, h, n = model._lib, model._h, model.n
        dev = "cuda"
        ax = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        ax[model.out_ids, :2] = gx.to(device=dev, dtype=torch.float64)
        av = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        ar = torch.zeros(n, dtype=torch.float64, device=dev)
        avt = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        pbar = torch.zeros(2, dtype=torch.float64, device=dev)
        K = model.checkpoint_every
        for seg in reversed(range(len(ctx.ckpts))):
            t0, t1 = seg * K, min(seg * K + K, model.nsteps)
            model.load(ctx.ckpts[seg])
            states = []
            for _ in range(t0, t1):
                states.append(model.save())
                model.step(1)
            for t in reversed(range(t1 - t0)):
                model.load(states[t])
                nat.check(lib.tsg_adjoint_step(h, _ptr(ax), _ptr(av), _ptr(ar), _ptr(avt), _ptr(pbar), _stream()),
                          "tsg_adjoint_step")
        grads = model.param_grads(pbar.cpu().tolist())
        return torch.tensor(grads, dtype=torch.float64, device=ctx.param_device), None


def distal_loss(x, target=0.35, fraction=0.01, sel=None):
    """Mean squared distance of the most distal particles' x from a target runout; the
    selection (top `fraction` by x) is returned so that perturbed runs reuse it."""
    if sel is None:
        k = max(1, int(round(fraction * x.shape[0])))
        sel = torch.topk(x[:, 0].detach(), k).indices
    return ((x[sel, 0] - target) ** 2).mean(), sel


def rollout_positions(cfg, nsteps, p0, p1, precision="fp64"):
    """Final output-particle positions (upload order, f64) of a fresh run with the given
    parameters - (friction in degrees, cohesion) for mu(I), (stiffness, viscosity) for
    WCSPH; the FP64 form is the finite-difference reference of the adjoint."""
    from .simulation import Simulation
    d = copy.deepcopy(cfg.config if isinstance(cfg, SimConfiger) else cfg)
    d["Configuration"]["neighbourSkin"] = 0.0
    sim = Simulation(SimConfiger(config=d), precision=precision)
    lib = nat.load()
    method = d["Configuration"].get("simulationMethod")
    if method == 1:
        nat.check(lib.tsg_set_fluid(sim.ps._h, float(p0), float(p1)), "tsg_set_fluid")
        out_type = MAT_FLUID
    else:
        nat.check(lib.tsg_set_soil(sim.ps._h, float(p0) / 180.0 * math.pi, float(p1)), "tsg_set_soil")
        out_type = MAT_SOIL
    sim.solver.step(int(nsteps))
    x = sim.ps.field("x").to(torch.float64)
    ids = sim.ps.field("id0").long()
    out = torch.empty_like(x)
    out[ids] = x
    mt = np.asarray(sim.ps.scene.mat_type)
    sel = torch.as_tensor(np.nonzero(mt == out_type)[0], device=x.device)
    return out[sel, :2].clone()
