"""FP32-mixed GPU form vs the f64 CPU oracle, with stated tolerances.

The FP32-mixed form keeps real particles and static boundary particles in separate
cell-sorted blocks, so every comparison matches particles through id0.  Tolerances:

* neighbour sets: identical, except pairs whose f64 distance is within 1e-6 R of the
  support radius (f32 positions decide those; the kernel weight there is ~1e-20 of peak);
* single-step rates (CSPM factor, d_density, d_vel): normwise relative error <= 1e-4;
* density after a few steps: relative error <= 1e-5 (the headline accuracy bound);
* positions after a few steps: absolute error <= 1e-6 m;
* granular columns (mu(I), Drucker-Prager, with and without CSPM): single-step d_density,
  d_vel and stress_tmp normwise <= 1e-4, d_stress within 1e-4 of its largest entry for all
  but 2 % of the particles (the rest within 2e-2); after 20 steps density <= 1e-5 relative,
  positions <= 1e-7 m, stress normwise <= 1e-4 (Drucker-Prager: per particle, as d_stress)
  and the return-mapping case flag equal for >= 99 % of particles (the plastic-branch
  thresholds, f = +-1e-4 Pa and sqrt(J2) = 1e-8 Pa, sit at or below the f32 resolution of
  ~2 kPa stresses).
"""
import numpy as np
import pytest

from helpers import cfg_of, small_column, small_dambreak_2d, small_dambreak_3d

pytestmark = pytest.mark.gpu


def _pair(d, oracle_lib):
    from tisphi_gb300.simulation import Simulation
    cfg = cfg_of(d)
    sim = Simulation(cfg, precision="fp32_mixed")
    orc = oracle_lib.OracleSim(cfg)
    return sim, orc


def _by_id(sim, orc, name):
    """GPU field re-ordered to the oracle's current order (through id0)."""
    gid = sim.ps.field("id0").cpu().numpy()
    oid = orc.get("id0").astype(np.int64)
    a = sim.ps.field(name).cpu().numpy().astype(np.float64)
    inv = np.empty_like(gid)
    inv[gid] = np.arange(gid.size)
    return a[inv[oid]]


def _normwise(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _advance(sim, orc, oracle_lib, steps):
    sim.solver.step(steps)
    orc.step(steps)


@pytest.mark.parametrize("scene", ["2d", "3d"])
def test_neighbor_sets_match(oracle_lib, native, scene):
    d = small_dambreak_2d() if scene == "2d" else small_dambreak_3d()
    sim, orc = _pair(d, oracle_lib)
    sim.ps.initialize_particle_system()
    orc.sort()
    gc, gl = sim.ps.neighbors()
    oc, ol = orc.neighbors()
    gid = sim.ps.field("id0").cpu().numpy()
    oid = orc.get("id0").astype(np.int64)
    mt = orc.get("mat_type").astype(np.int64)
    x = orc.get("x")
    R = sim.ps.support_radius
    goff = np.concatenate([[0], np.cumsum(gc)])
    ooff = np.concatenate([[0], np.cumsum(oc)])
    g_of_id = {int(gid[k]): k for k in range(gid.size)}
    flow_ids = set(oid[(mt == 1) | (mt == 2)].tolist())
    mismatched = 0
    for oi in range(oid.size):
        gk = g_of_id[int(oid[oi])]
        glist = gid[gl[goff[gk]:goff[gk + 1]]].tolist()
        gset = set(glist)
        assert len(gset) == len(glist), f"duplicate list entries for particle {oid[oi]}"
        oset = set(oid[ol[ooff[oi]:ooff[oi + 1]]].tolist())
        if mt[oi] not in (1, 2):
            oset &= flow_ids  # boundary particles list flow neighbours only
        for idn in gset ^ oset:
            oj = int(np.nonzero(oid == idn)[0][0])
            r = np.linalg.norm(x[oi] - x[oj])
            assert abs(r - R) < 1e-6 * R, f"pair ({oid[oi]}, {idn}) at r={r} differs"
            mismatched += 1
    assert mismatched <= 4
    # the dummies visited per step: every dummy with a flow neighbour within R is listed
    gmt = sim.ps.field("mat_type").cpu().numpy()
    listed = sim.ps.list_stats()["listed_dummies"]
    assert np.count_nonzero((gmt < 0) & (gc > 0)) <= listed <= np.count_nonzero(gmt < 0)


def test_kernel_corr_close(oracle_lib, native):
    sim, orc = _pair(small_dambreak_3d(corr=1), oracle_lib)
    sim.ps.initialize_particle_system()
    orc.sort()
    sim.solver.calc_kernel_corr()
    orc.call(oracle_lib.ORC_KERNEL_CORR)
    # Compare the Shepard sum s = 1 / CSPM_f: f itself is ill-conditioned for boundary
    # particles whose only flow neighbours sit near the support radius (W -> 0 there).
    fg = _by_id(sim, orc, "CSPM_f")
    fo = orc.get("CSPM_f")
    sg, so = 1.0 / fg, 1.0 / fo
    both = (fg != 1.0) & (fo != 1.0)
    assert np.max(np.abs(sg[both] - so[both])) < 1e-5
    assert np.max(np.abs(sg[~both] - so[~both])) < 1e-5 or np.all(np.minimum(sg[~both], so[~both]) < 1e-5)
    mt = orc.get("mat_type")
    L = _by_id(sim, orc, "CSPM_L")
    Lo = orc.get("CSPM_L")
    f = mt == 1
    assert _normwise(L[f], Lo[f]) < 1e-4


@pytest.mark.parametrize("scene,corr", [("2d", 0), ("3d", 1)])
def test_one_step_rates_close(oracle_lib, native, scene, corr):
    d = small_dambreak_2d(corr=corr) if scene == "2d" else small_dambreak_3d(corr=corr)
    sim, orc = _pair(d, oracle_lib)
    _advance(sim, orc, oracle_lib, 3)
    sim.ps.initialize_particle_system()
    orc.sort()
    sim.solver.calc_kernel_corr()
    orc.call(oracle_lib.ORC_KERNEL_CORR)
    sim.solver.init_real2tmp()
    orc.call(oracle_lib.ORC_INIT_TMP)
    sim.solver.one_step()
    orc.call(oracle_lib.ORC_ONE_STEP)
    f = orc.get("mat_type") == 1
    for name in ("d_density", "d_vel", "pressure"):
        err = _normwise(_by_id(sim, orc, name)[f], orc.get(name)[f])
        assert err < 1e-4, f"{name}: normwise error {err:.3e}"
    # boundary extrapolation: dummies with flow neighbours, and those without (pressure 0,
    # written at the list build rather than every step).  The extrapolation is a Shepard
    # average; for a dummy whose flow neighbours all lie near the support radius (lattice
    # distance 3 spacings = R here) the weights W ~ (1 - q / 2)^4 carry the f32 rounding of
    # q amplified a thousandfold, so dummies with a Shepard sum below 1e-6 (CSPM_f > 1e6)
    # are left out of the 1e-4 bound.
    b = orc.get("mat_type") == -1
    pg, po = _by_id(sim, orc, "pressure")[b], orc.get("pressure")[b]
    e = np.abs(pg - po) / np.max(np.abs(po))
    bad = e > 1e-4
    assert np.all(orc.get("CSPM_f")[b][bad] > 1e6), f"boundary pressures off by {e.max():.3e}"
    idle = (po == 0) & ~bad
    assert np.count_nonzero(idle) > 0 and np.max(e[idle]) <= 1e-6


@pytest.mark.parametrize("scene,ti,skin", [("2d", 2, 0.1), ("2d", 1, 0.1), ("3d", 2, 0.1), ("2d", 2, 0.0),
                                           ("3d", 2, 0.0), ("2d", 2, 0.002), ("2d", 4, 0.1), ("3d", 4, 0.1),
                                           ("3d", 2, 0.05)])
def test_steps_density_position(oracle_lib, native, scene, ti, skin):
    """Neighbour-list skin 0.1 R: lists reused across steps; 0: rebuilt every step; 0.002 R:
    rebuilt whenever a particle moves 0.0009 R (several rebuilds within the run)."""
    d = small_dambreak_2d(integration=ti) if scene == "2d" else small_dambreak_3d(integration=ti)
    d["Configuration"]["neighbourSkin"] = skin
    sim, orc = _pair(d, oracle_lib)
    _advance(sim, orc, oracle_lib, 10)
    f = orc.get("mat_type") == 1
    rho = _by_id(sim, orc, "density")[f]
    rho_o = orc.get("density")[f]
    assert np.max(np.abs(rho - rho_o) / rho_o) < 1e-5
    x = _by_id(sim, orc, "x")[f]
    assert np.max(np.abs(x - orc.get("x")[f])) < 1e-6
    sim.ps.check_errors()


def test_fp32_determinism(oracle_lib, native):
    from tisphi_gb300.simulation import Simulation
    d = small_dambreak_2d()
    a = Simulation(cfg_of(d), precision="fp32_mixed")
    b = Simulation(cfg_of(d), precision="fp32_mixed")
    a.solver.step(10)
    b.solver.step(10)
    for nm in ("x", "v", "density"):
        np.testing.assert_array_equal(a.ps.field(nm).cpu().numpy(), b.ps.field(nm).cpu().numpy())


@pytest.mark.parametrize("method,corr", [(2, 0), (3, 0), (2, 1), (3, 1)])
def test_soil_one_step_rates_close(oracle_lib, native, method, corr):
    sim, orc = _pair(small_column(method, corr=corr), oracle_lib)
    _advance(sim, orc, oracle_lib, 3)
    sim.ps.initialize_particle_system()
    orc.sort()
    sim.solver.calc_kernel_corr()
    orc.call(oracle_lib.ORC_KERNEL_CORR)
    sim.solver.init_real2tmp()
    orc.call(oracle_lib.ORC_INIT_TMP)
    sim.solver.one_step()
    orc.call(oracle_lib.ORC_ONE_STEP)
    f = orc.get("mat_type") == 2
    names = ["d_density", "d_vel", "stress_tmp"]
    errs = {nm: _normwise(_by_id(sim, orc, nm)[f], orc.get(nm)[f]) for nm in names}
    assert all(e < 1e-4 for e in errs.values()), f"normwise errors {errs}"
    if method == 3:
        # Drucker-Prager stress rate per particle: the plastic branch needs sqrt(J2) > 1e-8 Pa
        # (eng/solver_sph_dp.py:194), a threshold far below the f32 resolution of kPa
        # stresses.  A particle whose stress is zero up to rounding (the free surface:
        # sqrt(J2) ~ 1e-16 Pa in f64, ~1e-7 Pa in f32) can take the plastic branch in one form
        # and not the other (with CSPM, two of this column's 1,250 particles at step 3); the
        # bound holds for all but 2 % of the particles, and those stay within 2e-2
        ds, ds_o = _by_id(sim, orc, "d_stress")[f], orc.get("d_stress")[f]
        e_p = np.abs(ds - ds_o).reshape(ds.shape[0], -1).max(axis=1) / np.abs(ds_o).max()
        off = float(np.mean(e_p >= 1e-4))
        assert off <= 2e-2 and e_p.max() < 2e-2, f"d_stress: {off:.4f} of particles off, max {e_p.max():.3e}"


@pytest.mark.parametrize("method,ti,skin,corr", [(2, 1, 0.05, 0), (3, 1, 0.05, 0), (3, 2, 0.05, 0), (3, 2, 0.1, 0),
                                                  (2, 4, 0.05, 0), (3, 4, 0.05, 0), (2, 1, 0.05, 1),
                                                  (3, 2, 0.05, 1)])
def test_soil_steps_close(oracle_lib, native, method, ti, skin, corr):
    """20 steps of mu(I) / Drucker-Prager against the f64 oracle (corr = 1: with the CSPM
    gradient correction).

    Density and positions within 1e-5 / 1e-7, stress within 1e-4 of its largest entry.  The
    Drucker-Prager stress rate switches its plastic term on where the previous yield value
    reaches -eps_f (eng/solver_sph_dp.py:194), a jump of about G |strain rate| dt in one
    step; a particle whose yield value lies within rounding of that threshold may take the
    other branch than the oracle (with skin 0.05, one particle of this column does at step
    11, and its neighbours' stress rates follow it; with skin 0.1, none within the 20 steps).
    For Drucker-Prager the stress bound therefore holds for all but 2 % of the particles, and
    those stay within 2e-2."""
    d = small_column(method, integration=ti, corr=corr)
    d["Configuration"]["neighbourSkin"] = skin
    sim, orc = _pair(d, oracle_lib)
    _advance(sim, orc, oracle_lib, 20)
    f = orc.get("mat_type") == 2
    rho = _by_id(sim, orc, "density")[f]
    rho_o = orc.get("density")[f]
    e_rho = float(np.max(np.abs(rho - rho_o) / rho_o))
    e_x = float(np.max(np.abs(_by_id(sim, orc, "x")[f] - orc.get("x")[f])))
    st, st_o = _by_id(sim, orc, "stress")[f], orc.get("stress")[f]
    e_p = np.abs(st - st_o).reshape(st.shape[0], -1).max(axis=1) / np.abs(st_o).max()
    e_s = float(e_p.max())
    report = f"density {e_rho:.3e}, x {e_x:.3e}, stress {e_s:.3e}"
    assert e_rho < 1e-5 and e_x < 1e-7, report
    if method == 3:
        fl = _by_id(sim, orc, "flag_retmap")[f]
        agree = float(np.mean(fl == orc.get("flag_retmap")[f]))
        off = float(np.mean(e_p >= 1e-4))
        report += f", flag agreement {agree:.4f}, particles off {off:.4f}"
        assert agree >= 0.99 and off <= 2e-2 and e_s < 2e-2, report
    else:
        assert e_s < 1e-4, report
    sim.ps.check_errors()
