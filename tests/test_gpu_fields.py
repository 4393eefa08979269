"""Field transfers through the C ABI (tsg_read / tsg_write, ParticleSystem.read_field /
write_field): row-major host copies equal the device views, in both forms, blocking and
non-blocking; writing the values read back leaves every field unchanged (bit for bit), and
a written position moves the particle by exactly the written amount in the FP64 form."""
import numpy as np
import pytest
import torch

from helpers import cfg_of, small_column, small_dambreak_2d

pytestmark = pytest.mark.gpu

NAMES = {"wc": ["x", "v", "density", "pressure", "d_vel", "id0"],
         "dp": ["x", "v", "density", "pressure", "stress", "strain_equ", "id0"]}


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
@pytest.mark.parametrize("scene", ["wc", "dp"])
@pytest.mark.parametrize("non_blocking", [False, True])
def test_read_matches_views(native, precision, scene, non_blocking):
    from tisphi_gb300.simulation import Simulation
    d = small_dambreak_2d() if scene == "wc" else small_column(3)
    sim = Simulation(cfg_of(d), precision=precision)
    sim.solver.step(3)
    ps = sim.ps
    for nm in NAMES[scene]:
        view = ps.field(nm).cpu().numpy()
        dtype = np.int32 if nm == "id0" else np.float64
        host = torch.empty(view.shape, dtype=torch.int32 if nm == "id0" else torch.float64).pin_memory()
        ps.read_field(nm, host, non_blocking=non_blocking)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host.numpy(), view.astype(dtype), err_msg=nm)


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_write_read_round_trip(native, precision):
    from tisphi_gb300.simulation import Simulation
    sim = Simulation(cfg_of(small_dambreak_2d()), precision=precision)
    sim.solver.step(3)
    ps = sim.ps
    before = {nm: ps.read_field(nm, np.empty(ps.field(nm).shape, dtype=np.float64))
              for nm in ("x", "v", "density", "pressure")}
    for nm, a in before.items():
        ps.write_field(nm, a)
    for nm, a in before.items():
        np.testing.assert_array_equal(ps.read_field(nm, np.empty_like(a)), a, err_msg=nm)
    if precision == "fp64":
        x = before["x"].copy()
        x[:, 1] += 1e-3
        ps.write_field("x", x)
        np.testing.assert_array_equal(ps.read_field("x", np.empty_like(x)), x)


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_read_fields_equals_read_field(native, precision):
    from tisphi_gb300.simulation import Simulation
    sim = Simulation(cfg_of(small_dambreak_2d()), precision=precision)
    sim.solver.step(3)
    ps = sim.ps
    names = ["x", "v", "density", "pressure", "d_vel"]
    one = {nm: ps.read_field(nm, np.empty(ps.field(nm).shape, dtype=np.float64)) for nm in names}
    dsts = [torch.empty(ps.field(nm).shape, dtype=torch.float64).pin_memory() for nm in names]
    ps.read_fields(names, dsts, non_blocking=True)
    torch.cuda.synchronize()
    for nm, d in zip(names, dsts):
        np.testing.assert_array_equal(d.numpy(), one[nm], err_msg=nm)
    dev = [torch.empty(ps.field(nm).shape, dtype=torch.float64, device="cuda") for nm in names]
    ps.read_fields(names, dev)
    for nm, d in zip(names, dev):
        np.testing.assert_array_equal(d.cpu().numpy(), one[nm], err_msg=nm)
