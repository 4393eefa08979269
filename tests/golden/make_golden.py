"""Generate golden vectors by running the reference's own source (Rabmelon/tiSPHi, eng/*.py)
under the serial Taichi-API emulator in tests/golden/taichi_emul.

Run with a checkout of the reference (its eng/ package on the path):

    python tests/golden/make_golden.py --reference PATH   (or TISPHI_REFERENCE=PATH)

Each case builds a scene dict (tisphi_gb300.scenes), writes it to a temporary JSON file,
constructs the reference's ``Simulation`` from that file, runs ``solver.step()`` a few
times and stores the particle fields in tests/golden/<case>.npz together with the scene.

Where the reference's parallel loops race, the emulator is given the serialisation the
oracle defines:
* WCSPHSolver.one_step, first loop (eng/solver_sph_wc.py:86-106): all flow particles
  first, then boundary particles (a valid order of that parallel loop: each iteration
  writes only its own particle);
* advect_pos with XSPH (eng/solver_sph_base.py:228-238) and the mu(I) stress
  regularisation (eng/solver_sph_muI.py:134-156) are read-then-write across particles;
  for those cases the generator runs the reference's own ti.funcs (for_all_neighbors,
  xsph_task, chk_density, regu_stress_task) in two phases.
"""
import argparse
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def cases():
    from tisphi_gb300 import scenes
    small2d = dict(spacing=0.04, width=0.4, height=0.2, domain=(0.8, 0.6), jitter=4e-4, seed=11)
    return {
        "wc2d_lf": (scenes.dambreak_2d(**small2d), 3),
        "wc2d_se_cubic": (scenes.dambreak_2d(**small2d, kernel=0, integration=1), 3),
        "wc2d_rk4": (scenes.dambreak_2d(**small2d, integration=4), 2),
        "wc2d_cspm_xsph": (scenes.dambreak_2d(**small2d, corr=1, xsph=True), 2),
        "wc3d_cspm": (scenes.dambreak_3d(spacing=0.04, domain=(0.32, 0.24, 0.16), size=(0.16, 0.12, 0.08),
                                         jitter_frac=0.01, seed=12), 1),
        "mui2d": (scenes.column_2d(method=2, spacing=0.01, width=0.1, height=0.05, domain=(0.2, 0.1),
                                   seed=13), 2),
        "dp2d": (scenes.column_2d(method=3, spacing=0.01, width=0.1, height=0.05, domain=(0.2, 0.1),
                                  seed=14), 2),
        "dp2d_lf_xsph": (scenes.column_2d(method=3, spacing=0.01, width=0.1, height=0.05, domain=(0.2, 0.1),
                                          seed=15, integration=2, xsph=True), 2),
        # dynamic rigid box on the water surface: the reaction scatter and shape matching
        "wc2d_rigid": (scenes.floating_box_2d(spacing=0.04, water=(0.4, 0.2), box=(0.12, 0.08), box_at=(0.12, 0.2),
                                              domain=(0.8, 0.6), jitter=4e-4, seed=16), 3),
        # longer horizons: a finer 2D dambreak (200 fluid particles) over 40 leap-frog steps,
        # the 3D CSPM dambreak at half the spacing (192 fluid) over 3 steps, and the mu(I)
        # column over 40 steps
        "wc2d_lf_40": (scenes.dambreak_2d(spacing=0.02, width=0.4, height=0.2, domain=(0.8, 0.6), jitter=2e-4,
                                          seed=17), 40),
        "wc3d_cspm_fine": (scenes.dambreak_3d(spacing=0.02, domain=(0.32, 0.24, 0.16), size=(0.16, 0.12, 0.08),
                                              jitter_frac=0.01, seed=18), 3),
        "mui2d_40": (scenes.column_2d(method=2, spacing=0.01, width=0.1, height=0.05, domain=(0.2, 0.1),
                                      seed=19), 40),
        # Drucker-Prager with the reference sand scene's integrator (leap-frog + XSPH) and
        # RK4 over longer horizons
        "dp2d_lf_xsph_40": (scenes.column_2d(method=3, spacing=0.01, width=0.1, height=0.05, domain=(0.2, 0.1),
                                             seed=20, integration=2, xsph=True), 40),
        "wc2d_rk4_20": (scenes.dambreak_2d(spacing=0.02, width=0.4, height=0.2, domain=(0.8, 0.6), jitter=2e-4,
                                           seed=21, integration=4), 20),
    }


FIELDS = ["x", "v", "density", "pressure", "m_V", "id0", "mat_type", "stress", "strain_equ", "strain_equ_p",
          "flag_retmap", "CSPM_f", "d_density", "d_vel", "v_tmp", "density_tmp"]


def install_semantics(ti, sim):
    """Serialise the racy loops the way the oracle defines them (see module docstring)."""
    ps = sim.ps
    solver = sim.solver
    types = ps.pt.store["mat_type"]

    def flow_first(seq):
        t = types[: len(seq)]
        flow = [i for i in seq if t[i] in (1, 2)]
        rest = [i for i in seq if t[i] not in (1, 2)]
        return flow + rest

    ti.set_loop_order(("WCSPHSolver.one_step", 0), flow_first)

    if solver.flagXSPH:
        def advect_pos_two_phase():
            n = ps.particle_num[None]
            dt = solver.dt[None]
            sums = {}
            for i in range(n):
                if ps.pt[i].mat_type > 0 and ps.pt[i].is_dynamic:
                    box = ti.Vector.zero(float, 3)
                    _, _, box = ti.call_with_refs(ps.for_all_neighbors, i, solver.xsph_task, box)
                    sums[i] = box
            for i in range(n):
                if ps.pt[i].mat_type > 0:
                    if i in sums:
                        ps.pt[i].x = ps.pt[i].x + dt * (ps.pt[i].v + 0.5 * sums[i])
                    else:
                        ps.pt[i].x = ps.pt[i].x + dt * ps.pt[i].v
        solver.advect_pos = advect_pos_two_phase

    if type(solver).__name__ == "MUISPHSolver":
        def advect_something_two_phase():
            n = ps.particle_num[None]
            dt = solver.dt[None]
            soil = [i for i in range(n) if ps.pt[i].mat_type == 2]
            for i in soil:
                solver.chk_density(i, solver.density0)
                ps.pt[i].strain_equ = ps.pt[i].strain_equ + dt * ps.pt[i].d_strain_equ
                ps.pt[i].stress = ps.pt[i].stress_tmp
            reg = {}
            for i in soil:
                box = ti.Matrix(np.zeros((3, 3)))
                _, _, box = ti.call_with_refs(ps.for_all_neighbors, i, solver.regu_stress_task, box)
                reg[i] = box
            for i in soil:
                ps.pt[i].stress = reg[i] * ps.pt[i].CSPM_f
        solver.advect_something = advect_something_two_phase


def run_case(name, scene, steps, out_dir):
    import taichi as ti
    from eng.configer_builder import SimConfiger
    from eng.simulation import Simulation
    with tempfile.NamedTemporaryFile("w", suffix=".json", delete=False) as f:
        json.dump(scene, f)
        path = f.name
    try:
        sim = Simulation(SimConfiger(path))
    finally:
        os.unlink(path)
    ps = sim.ps
    n = ps.particle_num[None]
    # the seeded jitter every implementation applies to the generated lattice (fluid / soil
    # particles, active axes, numpy PCG64 in particle order)
    jit = scene["Configuration"].get("jitter", 0.0) or 0.0
    if jit > 0:
        mt = ps.pt.store["mat_type"][:n]
        flow = np.nonzero((mt == 1) | (mt == 2))[0]
        rng = np.random.Generator(np.random.PCG64(int(scene["Configuration"].get("seed", 0))))
        noise = rng.uniform(-jit, jit, size=(flow.size, ps.dim))
        ps.pt.store["x"][flow, :ps.dim, 0] += noise
        ps.pt.store["x0"][flow, :ps.dim, 0] = ps.pt.store["x"][flow, :ps.dim, 0]
    if type(sim.solver).__name__ == "DPSPHSolver":
        # the constructor's geostatic stress (eng/solver_sph_dp.py:35) must see the jittered
        # positions, as it does in every implementation that receives jittered input
        sim.solver.init_stress(sim.solver.density0, sim.solver.fric)
    x_init = ps.pt.store["x"][:n, :, 0].copy()
    install_semantics(ti, sim)
    ti.oob_reads[0] = 0
    for _ in range(steps):
        sim.solver.step()
    out = {}
    for fld in FIELDS:
        a = ps.pt.store[fld][:n]
        out[fld] = a[:, :, 0].copy() if (a.ndim == 3 and a.shape[2] == 1) else a.copy()
    out["grid_end"] = ps.grid_particle_num.data.copy()
    out["x_init"] = x_init
    out["scene_json"] = np.array(json.dumps(scene))
    out["steps"] = np.array(steps)
    out["dt"] = np.array(sim.solver.dt[None])
    np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **out)
    return n, ti.oob_reads[0]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("TISPHI_REFERENCE"),
                    help="checkout of the reference (or set TISPHI_REFERENCE)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if not args.reference:
        ap.error("--reference PATH (or TISPHI_REFERENCE) is required")
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(HERE, "taichi_emul"))
    sys.path.insert(1, args.reference)
    sys.path.insert(2, ROOT)
    for name, (scene, steps) in cases().items():
        if args.only and name != args.only:
            continue
        n, oob = run_case(name, scene, steps, HERE)
        print(f"{name}: {n} particles, {steps} steps, {oob} out-of-grid cell reads treated as empty")


if __name__ == "__main__":
    main()
