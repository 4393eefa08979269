"""The dense torch restatement of the mu(I) step (used to check the adjoint through
autograd) against the f64 oracle on a small column: positions, velocities and densities
agree to 1e-9 relative after 20 steps (they differ only in summation order)."""
import numpy as np
import torch

from helpers import cfg_of
from tisphi_gb300 import scenes
from tisphi_gb300.scene import build_scene

import torch_mui


def tiny_column():
    return scenes.column_2d(method=2, spacing=0.002, dt=2e-5, width=0.02, height=0.02, domain=(0.06, 0.04))


def test_torch_restatement_matches_oracle(oracle_lib):
    d = tiny_column()
    cfg = cfg_of(d)
    scene = build_scene(cfg)
    C = torch_mui.Consts(scene, cfg)
    x, v, rho, vt = torch_mui.initial_state(scene)
    mu = torch.tan(torch.tensor(21.9 / 180.0 * np.pi, dtype=torch.float64))
    for _ in range(20):
        x, v, rho, vt = torch_mui.step(x, v, rho, vt, mu, 0.0, C)
    orc = oracle_lib.OracleSim(cfg)
    orc.step(20)
    ids = orc.get("id0").astype(np.int64)
    xo = np.empty((scene.n, 3))
    xo[ids] = orc.get("x")
    vo = np.empty((scene.n, 3))
    vo[ids] = orc.get("v")
    ro = np.empty(scene.n)
    ro[ids] = orc.get("density")
    soil = scene.mat_type == 2
    np.testing.assert_allclose(x.numpy()[soil], xo[soil, :2], rtol=0, atol=1e-12)
    vs = np.abs(vo[soil, :2]).max()
    np.testing.assert_allclose(v.numpy()[soil], vo[soil, :2], rtol=0, atol=1e-9 * vs)
    np.testing.assert_allclose(rho.numpy()[soil], ro[soil], rtol=1e-9)
