"""Dynamic rigid bodies (shape matching, eng/solver_sph_base.py:467-518) in both forms.

The reference scatters the flow's reaction onto dynamic rigid particles without
synchronisation (eng/solver_sph_wc.py:70-71, eng/solver_sph_muI.py:45-46); both the oracle
and the GPU gather it per rigid particle in ascending neighbour order, the serial order of
that scatter, and replace ti.polar_decompose by the same scaled Newton iteration, so the FP64
form is bit-identical to the oracle (the golden fixture wc2d_rigid pins the oracle to the
reference's own rigid-body code run under the Taichi emulator).  Cases: a 2D water column
with a floating box (leap-frog over 300 steps, symplectic Euler + XSPH), a sinking box, the
3D counterpart with CSPM (also with the box given as a mesh body), two bodies of 1,200 and
300 particles on one water column, and a mu(I) column with a box resting on the sand.  The FP32-mixed
WCSPH form takes them too (reaction gathered over each rigid particle's list, shape matching
in f64 on its hi + lo positions), within its tolerances against the oracle; granular scenes
with dynamic rigid bodies take the FP64 form.
"""
import os
import tempfile

import numpy as np
import pytest

from helpers import cfg_of, describe_diff, mesh_box_scene_3d, small_column, write_box_obj

_OBJ_DIR = tempfile.mkdtemp(prefix="tsg_mesh_")

pytestmark = pytest.mark.gpu

FIELDS = ["x", "v", "density", "pressure", "m_V", "d_vel", "id0"]


def _compare(sim, orc, names, where):
    bad = []
    for nm in names:
        a = sim.ps.field(nm).detach().cpu().numpy().astype(np.float64)
        b = orc.get(nm)
        same = (a == b) | (np.isnan(a) & np.isnan(b))
        if not np.all(same):
            bad.append(describe_diff(nm, a, b))
    assert not bad, f"{where}: " + "; ".join(bad)


def _box_on_sand():
    d = small_column(2)
    d["Materials"].append({"matId": 1, "matType": 11, "color": [155, 55, 55], "density0": 3000.0})
    d["Blocks"].append({"objectId": 1, "size": [0.04, 0.02, 0.05], "translation": [0.04, 0.1, 0.0],
                        "velocity": [0.0, 0.0, 0.0], "materialId": 1, "isDynamic": True})
    return d


def _two_boxes():
    """Two dynamic bodies thrown onto a 2D water column: a 1,200-particle box (more than one
    chunk of the FP32-mixed form's object sums, three of the FP64 form's staged sums) and a
    300-particle denser one, so that the object lists, slices and per-object sums serve two
    objects."""
    from tisphi_gb300 import scenes
    d = scenes.floating_box_2d(spacing=0.004, dt=2e-5, jitter=4e-5, box=(0.16, 0.12), box_at=(0.1, 0.4))
    d["Blocks"][-1]["velocity"] = [0.5, -3.0, 0.0]
    d["Materials"].append({"matId": 2, "matType": 11, "color": [55, 155, 55], "density0": 2000.0})
    d["Blocks"].append({"objectId": 2, "size": [0.08, 0.06, 0.05], "translation": [0.4, 0.4, 0.0],
                        "velocity": [-0.5, -3.0, 0.0], "materialId": 2, "isDynamic": True})
    return d


def _cases():
    from tisphi_gb300 import scenes
    return {
        "2d_lf_float": (scenes.floating_box_2d(), 300),
        "2d_se_xsph": (scenes.floating_box_2d(integration=1, xsph=True), 100),
        "2d_sink": (scenes.floating_box_2d(box_density=3000.0, box_at=(0.3, 0.45)), 200),
        "3d_cspm": (scenes.floating_box_3d(), 20),
        "mui_box_on_sand": (_box_on_sand(), 100),
        # the box as a mesh body (a unit-box OBJ voxelised at the particle diameter)
        "3d_mesh_body": (mesh_box_scene_3d(write_box_obj(os.path.join(_OBJ_DIR, "unit_box.obj"))), 20),
        "2d_two_boxes": (_two_boxes(), 100),
    }


@pytest.mark.parametrize("name", list(_cases()))
def test_rigid_fp64_bit_exact(oracle_lib, native, name):
    from tisphi_gb300.simulation import Simulation
    d, steps = _cases()[name]
    cfg = cfg_of(d)
    sim = Simulation(cfg, precision="fp64")
    orc = oracle_lib.OracleSim(cfg)
    assert np.count_nonzero(orc.get("mat_type") == 11) > 0
    sim.solver.step(steps)
    orc.step(steps)
    _compare(sim, orc, FIELDS, f"{name} after {steps} steps")
    # every body moved and kept its shape: pairwise distances of its particles unchanged
    mt = orc.get("mat_type")
    xr = orc.get("x")[mt == 11]
    x0 = orc.scene.x[orc.get("id0")[mt == 11].astype(np.int64)]
    obj = orc.get("obj_id")[mt == 11]
    for o in np.unique(obj):
        sel = obj == o
        assert np.max(np.abs(xr[sel] - x0[sel])) > 1e-6
        d0 = np.linalg.norm(x0[sel][:, None, :] - x0[sel][None, :, :], axis=-1)
        d1 = np.linalg.norm(xr[sel][:, None, :] - xr[sel][None, :, :], axis=-1)
        assert np.max(np.abs(d1 - d0)) < 1e-9, f"body {o}"


def test_rigid_stage_calls_match_step(native):
    """solve_rigid_body is callable on its own: the reference's stage sequence through the
    object API equals step()."""
    from tisphi_gb300 import scenes
    from tisphi_gb300.simulation import Simulation
    cfg = cfg_of(scenes.floating_box_2d())
    a = Simulation(cfg, precision="fp64")
    b = Simulation(cfg, precision="fp64")
    a.solver.step(5)
    for _ in range(5):
        s = b.solver
        b.ps.initialize_particle_system()
        s.calc_kernel_corr()
        s.init_real2tmp()
        s.substep()
        s.advect_pos()
        s.advect_something()
        s.solve_rigid_body()
        s.enforce_boundary()
    for nm in FIELDS:
        assert np.array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy()), nm


def _by_id(ps_ids, v):
    out = np.empty_like(v)
    out[ps_ids.astype(np.int64)] = v
    return out


@pytest.mark.parametrize("name", ["2d_lf_float", "2d_sink", "3d_cspm", "3d_mesh_body", "2d_two_boxes"])
def test_rigid_fp32_mixed_close(oracle_lib, native, name):
    """The FP32-mixed WCSPH form with dynamic rigid bodies against the oracle: fluid density
    within 1e-5 relative, every position within 2e-6 m, the rigid particles' accelerations
    within 1e-4 of their largest (normwise)."""
    from tisphi_gb300.simulation import Simulation
    d, steps = _cases()[name]
    steps = min(steps, 100)
    cfg = cfg_of(d)
    sim = Simulation(cfg, precision="fp32_mixed")
    orc = oracle_lib.OracleSim(cfg)
    sim.solver.step(steps)
    orc.step(steps)
    mine_id = sim.ps.field("id0").cpu().numpy()
    oid = orc.get("id0")

    def get(nm):
        return _by_id(mine_id, sim.ps.field(nm).cpu().numpy().astype(np.float64))

    def ref(nm):
        return _by_id(oid, orc.get(nm))

    mt = ref("mat_type")
    fl, rg = mt == 1, mt == 11
    rho, rho_o = get("density")[fl], ref("density")[fl]
    assert np.max(np.abs(rho - rho_o) / rho_o) < 1e-5
    assert np.max(np.abs(get("x") - ref("x"))) < 2e-6
    dv, dv_o = get("d_vel")[rg], ref("d_vel")[rg]
    scale = np.max(np.linalg.norm(dv_o, axis=1))
    assert np.max(np.linalg.norm(dv - dv_o, axis=1)) < 1e-4 * scale


def test_rigid_fp32_mixed_granular_rejected(native):
    """Dynamic rigid bodies in a granular scene take the FP64 form; the FP32-mixed upload
    says so."""
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.simulation import Simulation
    with pytest.raises(nat.NativeError):
        Simulation(cfg_of(_box_on_sand()), precision="fp32_mixed")
