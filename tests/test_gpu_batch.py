"""Batched ensembles, captured step graphs and the autotuner (FP32-mixed form).

* A batch of dambreaks with different block sizes, stiffness and viscosity against the
  same scenes run one by one: neighbour sets identical (integer, exact); after 10
  leap-frog steps density within 1e-5 relative and positions within 1e-6 m (the FP32
  tolerances; the batch walks a different cell grid, so f32 sums run in another order);
  per-scene mass identical.
* One batch scene against the f64 oracle with the same tolerances.
* Graph replay against the eager step path (per-phase profiling forces eager steps):
  bit-identical, since both launch the same kernels in the same order; also one step per
  call through several list rebuilds (the graph's conditional node against the host's
  decision).
* The step sequence (fluid EOS inside init_real2tmp and the leap-frog half step; advect,
  advect_pos and the density clamp in one pass; Shepard factors from the first rates and
  boundary passes instead of the correction kernel) against the reference's stages called
  one by one (sort, calc_kernel_corr, init_real2tmp, substep, advect_pos,
  advect_something), lists rebuilt every step: bit-identical without CSPM and with CSPM
  under symplectic Euler (whose single rates pass keeps reading the correction kernel's
  CSPM matrix).
* Leap-frog with CSPM, where step() takes the fluid's CSPM factors from the first rates
  pass (the correction kernel then visits the boundary particles only), against the same
  stage calls: the factors bit-identical; the first pass's continuity, contracted with the
  inverse CSPM matrix after the neighbour loop instead of per neighbour, to rounding
  (density_tmp within 1e-9 relative, pressure within 1e-7 relative + 1e-4 Pa).  With
  the dynamic block holding fluid only, the dummies' Shepard factors come from the first
  boundary pass; with a static rigid obstacle in the dynamic block the correction kernel
  still runs for the non-fluid particles.  The obstacle scene also against the f64 oracle.
  A doubly dense block, whose fluid lists overflow, takes the same checks through the
  kernels' overflow passes (2 steps, and against the oracle).
* Threads per block changes no arithmetic: bit-identical.  Cells per CTA of the list
  build (and the per-particle builder) give the same neighbour sets; the entries of a list
  may be ordered differently, so steps agree within 1e-6 relative.
* The autotuner restores the particle state: every field equal after tuning.
"""
import ctypes

import numpy as np
import pytest

from helpers import cfg_of, small_dambreak_2d, small_dambreak_3d

pytestmark = pytest.mark.gpu


def _scenes():
    from tisphi_gb300 import scenes
    out = []
    for q, (w, h, b, nu) in enumerate([(0.3, 0.2, 2e4, 1e-3), (0.6, 0.4, 5e4, 5e-3), (0.44, 0.3, 1e5, 1e-2)]):
        out.append(scenes.dambreak_2d(spacing=0.02, width=w, height=h, stiffness=b, viscosity=nu, seed=11 + q,
                                      domain=(1.2, 0.8)))
    return out


def _single(d):
    from tisphi_gb300.simulation import Simulation
    return Simulation(cfg_of(d), precision="fp32_mixed")


def _by_id0(ps, name):
    ids = ps.field("id0").cpu().numpy()
    a = ps.field(name).cpu().numpy().astype(np.float64)
    out = np.empty_like(a)
    out[ids] = a
    return out


def test_batch_matches_single_scenes(native):
    from tisphi_gb300.batch import SceneBatch
    ds = _scenes()
    batch = SceneBatch(ds)
    singles = [_single(d) for d in ds]
    batch.step(10)
    for s in singles:
        s.solver.step(10)
    batch.check_errors()
    diag = batch.diagnostics()
    for q, s in enumerate(singles):
        mt = _by_id0(s.ps, "mat_type")
        f = mt == 1
        rho_b = batch.scene_field("density", q)[f]
        rho_s = _by_id0(s.ps, "density")[f]
        assert np.max(np.abs(rho_b - rho_s) / rho_s) < 1e-5, f"scene {q} density"
        x_b = batch.scene_field("x", q)[f]
        x_s = _by_id0(s.ps, "x")[f]
        assert np.max(np.abs(x_b - x_s)) < 1e-6, f"scene {q} positions"
        d_s = s.ps.diagnostics()
        assert diag[q]["mass"] == pytest.approx(d_s["mass"], rel=1e-12)
        assert diag[q]["front"] == pytest.approx(d_s["front"], abs=1e-6)


def test_batch_neighbor_sets_equal_single(native):
    """Neighbour sets of the batch (through tsg_neighbors after the first sort) per scene
    equal the scene's own, except pairs within 1e-6 R of the support radius, where the
    f32 rounding of the shifted positions may decide differently."""
    from tisphi_gb300 import _native as nat
    from tisphi_gb300.batch import SceneBatch
    ds = _scenes()
    batch = SceneBatch(ds)
    lib = nat.load()
    nat.check(lib.tsg_sort(batch._h, None), "sort")
    n = batch.n
    counts = np.zeros(n, dtype=np.int32)
    total = ctypes.c_int64()
    nat.check(lib.tsg_neighbors(batch._h, nat.as_ptr(counts, ctypes.c_int32), None, 0, ctypes.byref(total), None),
              "count")
    lst = np.zeros(total.value, dtype=np.int32)
    nat.check(lib.tsg_neighbors(batch._h, nat.as_ptr(counts, ctypes.c_int32), nat.as_ptr(lst, ctypes.c_int32),
                                total.value, ctypes.byref(total), None), "fill")
    gid = batch.field("id0").cpu().numpy()
    off = np.concatenate([[0], np.cumsum(counts)])
    pos_b = {int(g): k for k, g in enumerate(gid)}
    borderline = 0
    for q, d in enumerate(ds):
        s = _single(d)
        s.ps.initialize_particle_system()
        sc, sl = s.ps.neighbors()
        sid = s.ps.field("id0").cpu().numpy()
        soff = np.concatenate([[0], np.cumsum(sc)])
        lo = int(batch.offsets[q])
        x = batch.scenes[q].x
        R = s.ps.support_radius
        for k in range(sid.size):
            mine = set((sid[sl[soff[k]:soff[k + 1]]]).tolist())
            kb = pos_b[int(sid[k]) + lo]
            theirs = set((gid[lst[off[kb]:off[kb + 1]]] - lo).tolist())
            for j in mine ^ theirs:
                r = np.linalg.norm(x[sid[k]] - x[j])
                assert abs(r - R) < 1e-6 * R, f"scene {q} pair ({sid[k]}, {j}) at r = {r}"
                borderline += 1
    assert borderline <= 8


def test_batch_scene_vs_oracle(oracle_lib, native):
    from tisphi_gb300.batch import SceneBatch
    ds = _scenes()
    batch = SceneBatch(ds)
    batch.step(10)
    for q in (0, 2):
        orc = oracle_lib.OracleSim(cfg_of(ds[q]))
        orc.step(10)
        ids = orc.get("id0").astype(np.int64)
        f = orc.get("mat_type") == 1
        rho_o = np.empty_like(orc.get("density"))
        rho_o[ids] = orc.get("density")
        x_o = np.empty_like(orc.get("x"))
        x_o[ids] = orc.get("x")
        mt = np.empty_like(orc.get("mat_type"))
        mt[ids] = orc.get("mat_type")
        f = mt == 1
        rho_b = batch.scene_field("density", q)
        assert np.max(np.abs(rho_b[f] - rho_o[f]) / rho_o[f]) < 1e-5
        assert np.max(np.abs(batch.scene_field("x", q)[f] - x_o[f])) < 1e-6


def test_graph_replay_equals_eager(native):
    from tisphi_gb300 import _native as nat
    lib = nat.load()
    d = small_dambreak_2d()
    a, b = _single(d), _single(d)
    a.solver.step(12)           # graph replays
    lib.tsg_profile(1)          # per-phase events: eager steps
    try:
        b.solver.step(12)
    finally:
        ms = (ctypes.c_double * 16)()
        cnt = (ctypes.c_int64 * 16)()
        lib.tsg_profile_read(ms, cnt, len(nat.PHASES))
        lib.tsg_profile(0)
    for nm in ("x", "v", "density", "pressure", "id0"):
        np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy(), err_msg=nm)


def test_single_step_replays_through_rebuilds_equal_eager(native):
    """step() one step at a time (a graph replay per call, its list rebuilds taken by the
    graph's conditional node) through several list rebuilds: bit-identical to eager steps,
    which decide each rebuild on the host."""
    from tisphi_gb300 import _native as nat
    lib = nat.load()
    d = small_dambreak_2d()
    a, b = _single(d), _single(d)
    for _ in range(300):
        a.solver.step()
    lib.tsg_profile(1)
    try:
        for _ in range(300):
            b.solver.step()
    finally:
        ms = (ctypes.c_double * 16)()
        cnt = (ctypes.c_int64 * 16)()
        lib.tsg_profile_read(ms, cnt, len(nat.PHASES))
        lib.tsg_profile(0)
    ba, bb = a.ps.list_stats()["builds"], b.ps.list_stats()["builds"]
    assert ba == bb and ba >= 3, (ba, bb)
    for nm in ("x", "v", "density", "pressure", "id0"):
        np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy(), err_msg=nm)


@pytest.mark.parametrize("case", ["2d_se", "2d_lf", "3d_se_cspm"])
def test_step_sequence_equals_stage_calls(native, case):
    d = {"2d_se": lambda: small_dambreak_2d(integration=1), "2d_lf": lambda: small_dambreak_2d(integration=2),
         "3d_se_cspm": lambda: small_dambreak_3d(integration=1)}[case]()
    d["Configuration"]["neighbourSkin"] = 0.0
    a, b = _single(d), _single(d)
    a.solver.step(6)
    for _ in range(6):
        b.ps.initialize_particle_system()
        b.solver.calc_kernel_corr()
        b.solver.init_real2tmp()
        b.solver.substep()
        b.solver.advect_pos()
        b.solver.advect_something()
    for nm in ("x", "v", "density", "pressure", "id0", "CSPM_f"):
        np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy(), err_msg=nm)


def _stage_step(sim):
    sim.ps.initialize_particle_system()
    sim.solver.calc_kernel_corr()
    sim.solver.init_real2tmp()
    sim.solver.substep()
    sim.solver.advect_pos()
    sim.solver.advect_something()


def _with_obstacle(d):
    """A static rigid block (kinematic, in the dynamic block) beside the water column."""
    from tisphi_gb300 import scenes
    d["Materials"].append({"matId": 1, "matType": 11, "color": [120, 120, 120], "density0": 1000.0})
    b = scenes.block((0.1, 0.1, 0.1), translation=(0.8, 0.0, 0.0), material=1, obj=1)
    b["isDynamic"] = False
    d["Blocks"].append(b)
    return d


@pytest.mark.parametrize("case", ["2d", "3d", "2d_obstacle"])
def test_fused_cspm_step_matches_stage_calls(native, case):
    d = {"2d": lambda: small_dambreak_2d(corr=1), "3d": small_dambreak_3d,
         "2d_obstacle": lambda: _with_obstacle(small_dambreak_2d(corr=1))}[case]()
    d["Configuration"]["neighbourSkin"] = 0.0
    a, b = _single(d), _single(d)
    for step in range(4):
        a.solver.step(1)
        _stage_step(b)
        np.testing.assert_array_equal(a.ps.field("id0").cpu().numpy(), b.ps.field("id0").cpu().numpy())
        if step == 0:  # same positions: the factors are the same sums in the same order
            for nm in ("CSPM_f", "CSPM_L"):
                np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy(),
                                              err_msg=nm)
        f = a.ps.field("mat_type").cpu().numpy() == 1
        ra, rb = a.ps.field("density_tmp").cpu().numpy()[f], b.ps.field("density_tmp").cpu().numpy()[f]
        assert np.max(np.abs(ra - rb) / rb) < 1e-9, (step, np.max(np.abs(ra - rb) / rb))
        pa, pb = a.ps.field("pressure").cpu().numpy()[f], b.ps.field("pressure").cpu().numpy()[f]
        np.testing.assert_allclose(pa, pb, rtol=1e-7, atol=1e-4)
        np.testing.assert_allclose(a.ps.field("x").cpu().numpy(), b.ps.field("x").cpu().numpy(), rtol=0, atol=1e-9)


def _dense(d):
    """A second fluid block over the first, offset by half a spacing in x and y: every fluid
    particle has about twice the lattice's neighbours, more than a list holds, so the list
    kernels serve them from their overflow passes (direct cell traversal).  Densities start
    at the rest density (they evolve by continuity), so the block starts at rest."""
    import copy
    h = d["Configuration"]["particleRadius"]
    b = copy.deepcopy(d["Blocks"][0])
    b["translation"] = [b["translation"][0] + h, b["translation"][1] + h, b["translation"][2]]
    d["Blocks"].append(b)
    return d


def test_fused_cspm_overflow_passes(oracle_lib, native):
    d = _dense(small_dambreak_2d(corr=1))
    d["Configuration"]["neighbourSkin"] = 0.0
    a, b = _single(d), _single(d)
    a.ps.initialize_particle_system()
    assert a.ps.list_stats()["overflowed"] > 100
    for step in range(2):
        a.solver.step(1)
        _stage_step(b)
        np.testing.assert_array_equal(a.ps.field("id0").cpu().numpy(), b.ps.field("id0").cpu().numpy())
        if step == 0:
            for nm in ("CSPM_f", "CSPM_L"):
                np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy(),
                                              err_msg=nm)
        f = a.ps.field("mat_type").cpu().numpy() == 1
        ra, rb = a.ps.field("density_tmp").cpu().numpy()[f], b.ps.field("density_tmp").cpu().numpy()[f]
        assert np.max(np.abs(ra - rb) / rb) < 1e-9, (step, np.max(np.abs(ra - rb) / rb))
        pa, pb = a.ps.field("pressure").cpu().numpy()[f], b.ps.field("pressure").cpu().numpy()[f]
        np.testing.assert_allclose(pa, pb, rtol=1e-6, atol=1e-3)
    a.ps.check_errors()
    orc = oracle_lib.OracleSim(cfg_of(d))
    orc.step(2)
    ids = orc.get("id0").astype(np.int64)
    def by_id(v):
        out = np.empty_like(v)
        out[ids] = v
        return out
    f = by_id(orc.get("mat_type")) == 1
    rho_o, x_o = by_id(orc.get("density")), by_id(orc.get("x"))
    assert np.max(np.abs(_by_id0(a.ps, "density")[f] - rho_o[f]) / rho_o[f]) < 1e-5
    assert np.max(np.abs(_by_id0(a.ps, "x")[f] - x_o[f])) < 1e-6


def test_fused_cspm_obstacle_vs_oracle(oracle_lib, native):
    d = _with_obstacle(small_dambreak_2d(corr=1))
    a = _single(d)
    assert int(np.count_nonzero(a.ps.scene.mat_type == 11)) > 0
    a.solver.step(10)
    orc = oracle_lib.OracleSim(cfg_of(d))
    orc.step(10)
    ids = orc.get("id0").astype(np.int64)
    def by_id(v):
        out = np.empty_like(v)
        out[ids] = v
        return out
    f = by_id(orc.get("mat_type")) == 1
    rho_o, x_o = by_id(orc.get("density")), by_id(orc.get("x"))
    rho_a, x_a = _by_id0(a.ps, "density"), _by_id0(a.ps, "x")
    assert np.max(np.abs(rho_a[f] - rho_o[f]) / rho_o[f]) < 1e-5
    assert np.max(np.abs(x_a[f] - x_o[f])) < 1e-6


@pytest.mark.parametrize("tpb", [64, 256])
def test_threads_per_block_bit_identical(native, tpb):
    from tisphi_gb300 import _native as nat
    lib = nat.load()
    d = small_dambreak_2d()
    a, b = _single(d), _single(d)
    cfg = nat.tsg_launch_cfg(tpb, 0, 4)
    nat.check(lib.tsg_set_launch(b.ps._h, ctypes.byref(cfg)), "set_launch")
    a.solver.step(9)
    b.solver.step(9)
    for nm in ("x", "v", "density"):
        np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy(), err_msg=nm)


@pytest.mark.parametrize("cpc", [2, 4, 8])
def test_cells_per_cta_close(native, cpc):
    from tisphi_gb300 import _native as nat
    lib = nat.load()
    d = small_dambreak_2d()
    a, b = _single(d), _single(d)
    cfg = nat.tsg_launch_cfg(128, cpc, 1)
    nat.check(lib.tsg_set_launch(b.ps._h, ctypes.byref(cfg)), "set_launch")
    a.solver.step(10)
    b.solver.step(10)
    f = _by_id0(a.ps, "mat_type") == 1
    ra, rb = _by_id0(a.ps, "density")[f], _by_id0(b.ps, "density")[f]
    assert np.max(np.abs(ra - rb) / ra) < 1e-6
    assert np.max(np.abs(_by_id0(a.ps, "x") - _by_id0(b.ps, "x"))) < 1e-7


def test_autotune_restores_state(native):
    from tisphi_gb300.batch import SceneBatch
    batch = SceneBatch(_scenes())
    batch.step(5)
    before = {q: {nm: batch.scene_field(nm, q) for nm in ("x", "v", "density")} for q in range(batch.nscenes)}
    best = batch.autotune(trial_steps=4)
    assert best["threads_per_block"] in (64, 128, 256) and best["ms_per_step"] > 0
    assert best == {**batch.get_launch(), "ms_per_step": best["ms_per_step"]}
    for q in range(batch.nscenes):
        for nm, a in before[q].items():
            np.testing.assert_array_equal(batch.scene_field(nm, q), a, err_msg=f"scene {q} {nm}")
    batch.step(3)
    batch.check_errors()
