"""Dense f64 torch restatement of the 2D mu(I) symplectic-Euler step, for autograd checks.

Test infrastructure only: it stands in for the reference kernels' own automatic
differentiation (Taichi is not installable here) when checking the library's hand-written
adjoint.  It follows the same step as the library's differentiable form:
eng/solver_sph_base.py:41-91 (step, init_real2tmp, advect_SE), :386-398 (Shepard factor),
:648-669 (boundary tasks), :714-715 (damping), :224-238 (advect_pos); eng/solver_sph_muI.py
:62-149 (mu(I) loops, density clamp); Wendland C2 kernel (eng/solver_sph_base.py:335-358).
Every pair interaction is evaluated densely (N x N), so keep N to a few hundred.
"""
import math

import numpy as np
import torch


class Consts:
    def __init__(self, scene, cfg):
        g = scene.geom
        self.soil = torch.as_tensor(scene.mat_type == 2)
        self.mass = torch.as_tensor(scene.mass, dtype=torch.float64)
        self.mV = torch.as_tensor(scene.m_V, dtype=torch.float64)
        self.h = g.smoothing_len
        self.R = g.support_radius
        self.kk = 7.0 / (4.0 * math.pi) / self.h ** 2
        mat = [m for m in cfg.get_materials() if m["matType"] == 2][0]
        self.rho0 = mat["density0"]
        self.E = mat["EYoungMod"]
        self.c2 = 24.0 ** 2
        self.dt = cfg.get_cfg("timeStepSizeMin")
        self.grav = torch.tensor(cfg.get_cfg("gravitation")[:2], dtype=torch.float64)
        self.damp_eps = 5e-5


def initial_state(scene):
    x = torch.as_tensor(scene.x[:, :2], dtype=torch.float64)
    v = torch.as_tensor(scene.v[:, :2], dtype=torch.float64)
    rho = torch.as_tensor(scene.density, dtype=torch.float64)
    vt = torch.zeros_like(v)
    return x, v, rho, vt


def step(x, v, rho, vt_prev, mu, coh, C):
    n = x.shape[0]
    soil = C.soil
    eye = torch.eye(n, dtype=torch.bool)
    mV = torch.where(soil, C.mass / rho, C.mV)
    d = x[:, None, :] - x[None, :, :]                       # d_ij = x_i - x_j
    r2 = (d * d).sum(-1)
    nbr = (r2 < C.R ** 2) & ~eye
    r = torch.sqrt(torch.where(nbr, r2, torch.ones_like(r2)))
    q = r / C.h
    q1 = torch.clamp(1.0 - 0.5 * q, min=0.0)
    W = torch.where(nbr, C.kk * q1 ** 4 * (1.0 + 2.0 * q), torch.zeros_like(r))
    G = torch.where(nbr, -5.0 * C.kk / C.h ** 2 * q1 ** 3, torch.zeros_like(r))
    vt = torch.where(soil[:, None], v, vt_prev)
    # Shepard factor of the dummies (soil neighbours only)
    Wb = W * (soil[None, :] * mV[None, :])
    S = Wb.sum(1)
    cf = torch.where(S != 0, 1.0 / torch.where(S != 0, S, torch.ones_like(S)), torch.ones_like(S))
    # mu(I) loop 1 (soil)
    u = vt[None, :, :] - vt[:, None, :]                      # u_ij = v~_j - v~_i
    g = G[..., None] * d
    A = nbr * mV[None, :]
    vg = torch.einsum("ij,ija,ijb->iab", A, u, g)
    dd = -torch.einsum("ij,ija,ija->i", A, u, g)
    p = torch.clamp(C.c2 * (rho - C.rho0), min=0.0)
    er = 0.5 * (vg + vg.transpose(1, 2))
    J = 0.5 * (er * er).sum((1, 2))
    pos = J > 0
    sJ = torch.sqrt(torch.where(pos, J, torch.ones_like(J))) * pos
    dbdot = sJ + 1e-8
    sc = (coh + p * mu) / dbdot
    I2 = torch.eye(2, dtype=x.dtype)
    sig = sc[:, None, None] * er - p[:, None, None] * I2
    # boundary extrapolation (dummies)
    B1 = Wb @ vt
    vt_b = 2.0 * v - cf[:, None] * B1
    B2 = Wb @ rho
    rho_b = torch.clamp(cf * B2, min=C.rho0)
    D = torch.einsum("bj,bja->ba", Wb * rho[None, :], C.grav[None, None, :] * d)
    B3 = torch.einsum("bj,jxy->bxy", Wb, sig) + torch.diag_embed(D)
    sig_b = cf[:, None, None] * B3
    SIG = torch.where(soil[:, None, None], sig, sig_b)
    RT = torch.where(soil, rho, rho_b)
    M = SIG[None, :, :, :] / RT[None, :, None, None] ** 2 + SIG[:, None, :, :] / RT[:, None, None, None] ** 2
    damp = -C.damp_eps * torch.sqrt(C.E / (rho * C.h ** 2))
    dv = torch.einsum("ij,ijab,ijb->ia", A * RT[None, :], M, g) + C.grav[None, :] + damp[:, None] * v
    # symplectic Euler, advect_pos, density clamp (soil only)
    rho1 = rho + C.dt * rho * dd
    v1 = v + C.dt * dv
    x1 = x + C.dt * v1
    rho2 = torch.clamp(rho1, min=C.rho0)
    x_n = torch.where(soil[:, None], x1, x)
    v_n = torch.where(soil[:, None], v1, v)
    rho_n = torch.where(soil, rho2, rho)
    vt_n = torch.where(soil[:, None], torch.zeros_like(vt_b), vt_b)
    return x_n, v_n, rho_n, vt_n


def rollout(scene, cfg, nsteps, friction_deg, cohesion):
    """Final soil positions (upload order) after nsteps, differentiable in both parameters."""
    C = Consts(scene, cfg)
    x, v, rho, vt = initial_state(scene)
    mu = torch.tan(friction_deg / 180.0 * math.pi)
    for _ in range(nsteps):
        x, v, rho, vt = step(x, v, rho, vt, mu, cohesion, C)
    return x[C.soil]


def soil_index(scene):
    return np.nonzero(scene.mat_type == 2)[0]
