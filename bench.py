"""Benchmark: particle-updates/s of the 3D WCSPH dambreak step on one GB300.

Workload (default): 3D WCSPH dambreak, domain 3.22 x 1.6 x 0.5 m, fluid block
1.2 x 0.6 x 0.2 m at lattice spacing 0.0054 m (911,754 fluid + 1,413,114 dummy particles,
2,324,868 total) with seeded +-1 % jitter, Wendland C2, Tait rho0 1000 / B 5e4 / gamma 7,
viscosity 0.005, CSPM gradient correction on, XSPH off, leap-frog at dt = 2e-5.

A "step" is one full ``SPHBase.step()``: cell sort, CSPM, two one_step evaluations with
the half / full leap-frog updates, advect_pos and the density clamp.  particle-updates/s =
fluid particles x steps / second.  The per-step working set (~0.5 GB) exceeds the 129 MB
L2, so no flush is needed between steps.

Printed (rank 0, one JSON line): ``value`` = the FP32-mixed form when the library provides
it, else the FP64 form; the other form is reported beside it under ``forms``; ``e2e`` =
the same metric through the public API with the step's inputs copied from pinned host
memory and its results read back every step; ``roofline`` for the dominant kernel (the
rates kernel), timed live with CUDA events; ``cpu_baseline`` = the f64 CPU oracle on the
host cores for a bounded sample of the same workload.

``--impl reference`` times the reference algorithm's CPU restatement (the oracle) instead,
on all host cores, and prints the reference-arm line.

Other workloads (``--workload``): ``batch`` (the 256-scene ensemble, batched against scene
by scene), ``adjoint`` (the differentiable column's gradients against finite differences),
``rollout`` (2,000 steps of the 3D dambreak in both forms), ``column`` (the granular column
at its stated size), ``kernels`` (every kernel family of both forms once, the command of
the per-kernel profiler survey).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particle-updates/s, 1M 3D WCSPH: FP32-mixed vs plain FP64, 1 GB300, stated err"
UNIT = "particle-updates/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def workload(args):
    from tisphi_gb300 import scenes
    if args.workload == "3d":
        d, name = scenes.dambreak_3d(spacing=args.spacing), "3D WCSPH dambreak"
    elif args.workload == "2d":
        d, name = scenes.dambreak_2d(), "2D WCSPH dambreak"
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    if args.list_skin is not None:
        d["Configuration"]["neighbourSkin"] = args.list_skin
    return d, name


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


# ---------------------------------------------------------------- distributed plumbing
def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return rank, ws, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value):
    if dist is None:
        return value
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- CPU baseline (oracle)
def cpu_baseline(cfg_dict, budget_s=25.0):
    """f64 CPU oracle (the reference algorithm restated in C++/OpenMP) on the host cores."""
    from oracle.oracle import OracleSim
    from tisphi_gb300.configer_builder import SimConfiger
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cfg = SimConfiger(config=cfg_dict)
    orc = OracleSim(cfg)
    n_fluid = int(np.count_nonzero(orc.scene.mat_type == 1))
    t0 = time.perf_counter()
    orc.step(1)
    first = time.perf_counter() - t0
    steps = 1
    extra = max(0, min(4, int((budget_s - first) / max(first, 1e-3))))
    if extra:
        t1 = time.perf_counter()
        orc.step(extra)
        el = time.perf_counter() - t1
        rate = n_fluid * extra / el
        steps = extra
    else:
        rate = n_fluid / first
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} full step(s) of the same {orc.n:,}-particle scene after 1 untimed step, "
                      f"f64 C++/OpenMP oracle, {cores} threads"}


# ---------------------------------------------------------------- GPU measurement
def algorithmic_bytes(kernel, n_total, n_flow, precision, corr, lists=None, fused=None):
    """Unique bytes a kernel must move once per launch (neighbour re-reads excluded).

    Every per-particle array the kernel touches counts once (read or written), as does
    every neighbour-list entry it reads (4 B each: the list is data the kernel streams, not
    a re-read).  FP64 (cell traversal, no lists): rates read x (24) + m_V (8) + v_tmp (24) +
    density_tmp (8) + pressure (8) + mat_type (4) + f32 prefilter position (16) of every
    particle, and per flow particle its CSPM matrix (72 when corrected) plus the writes of
    d_density (8) and d_vel (24).  FP32-mixed (n_vis = flow particles + dummies with a
    non-empty list, the particles the list kernels visit; WCSPH scenes have no other real
    particles):
      rates:  lo (position offset, m_V) + (v_tmp, p / rho^2) of every visited particle (32);
              per flow particle its hi (16), density_tmp (4), list count (4), CSPM matrix
              (24, six planes, when corrected) and the writes of d_density (4) and d_vel
              (16); plus the flow particles' list entries;
      corr:   hi + lo + count of every visited particle (36), the listed dummies' index (4),
              writes CSPM_f (4) and CSPM_L (24 when corrected); plus every list entry;
      boundary: per listed dummy its index (4), hi + lo + velocity (48), count (4),
              CSPM_f (4) and the writes (v_tmp, p / rho^2) (16), (p, rho) (8),
              density_tmp (4), pressure (4); per flow particle lo + v_tmp + (p, rho)
              (16 + 16 + 8); plus the dummies' list entries.
    fused ("se" / "lf": the FP32-mixed WCSPH step, whose first rates pass computes the flow
    particles' Shepard factors, and with leap-frog + CSPM their CSPM matrices, and whose
    first boundary pass the dummies' Shepard factors): the rates figure is the mean over the
    step's rates passes — leap-frog: the first writes CSPM_f (4) and, with CSPM, CSPM_L (24)
    where the second reads CSPM_L (24), so 2 + 24 B per flow particle; symplectic Euler:
    the one pass writes CSPM_f (4) and reads CSPM_L (24 with CSPM).  The boundary pass
    writes the Shepard factor where it would read it (same bytes).  The correction kernel
    runs only with symplectic Euler + CSPM, over the flow particles.
    """
    if precision == "fp64":
        if kernel != "rates":
            return None
        return n_total * 92 + n_flow * (4 + (72 if corr else 0) + 32)
    lists = lists or {"entries_real": 0, "entries_dummy": 0}
    er, ed = lists["entries_real"], lists["entries_dummy"]
    na = lists.get("listed_dummies", n_total - n_flow)
    n_vis = n_flow + na
    if kernel == "rates":
        if fused == "lf":
            cspm = 2 + (24 if corr else 0)
        elif fused == "se":
            cspm = 4 + (24 if corr else 0)
        else:
            cspm = 24 if corr else 0
        return n_vis * 32 + n_flow * (16 + 4 + 4 + cspm + 20) + 4 * er
    if kernel == "kernel_corr":
        if fused:
            return n_flow * (36 + 4 + (24 if corr else 0)) + 4 * er
        return n_vis * (36 + 4 + (24 if corr else 0)) + na * 4 + 4 * (er + ed)
    if kernel == "boundary":
        return na * (4 + 48 + 4 + 4 + 32) + n_flow * 40 + 4 * ed
    return None


def measure(args, cfg_dict, precision, rank, dist):
    import ctypes

    import torch

    from tisphi_gb300 import _native as nat
    from tisphi_gb300.configer_builder import SimConfiger
    from tisphi_gb300.simulation import Simulation

    sim = Simulation(SimConfiger(config=cfg_dict), precision=precision)
    ps, solver = sim.ps, sim.solver
    lib = nat.load()
    n_total = ps.particle_max_num
    n_fluid = int(np.count_nonzero(ps.scene.mat_type == 1))
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        solver.step()
    torch.cuda.synchronize()
    ps.check_errors()
    try:
        builds0 = ps.list_stats()["builds"]
    except nat.NativeError:  # the FP64 form traverses cells and keeps no lists
        builds0 = None
    # ---- timed region: K steps, CUDA events on the launch stream
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        barrier(dist)
        torch.cuda.synchronize()
        l0 = lib.tsg_launch_count()
        start.record(stream)
        for _ in range(args.steps):
            solver.step()
        stop.record(stream)
        torch.cuda.synchronize()
        launches = lib.tsg_launch_count() - l0
        barrier(dist)
    ms = start.elapsed_time(stop) / args.steps
    ms = max_over_ranks(dist, ms)
    clocks = clk.summary()
    ps.check_errors()
    timed_builds = ps.list_stats()["builds"] - builds0 if builds0 is not None else None
    # ---- per-phase kernel timing (separate pass of the same steps, events on the stream)
    lib.tsg_profile(1)
    for _ in range(args.steps):
        solver.step()
    torch.cuda.synchronize()
    nph = len(nat.PHASES)
    pms = (ctypes.c_double * nph)()
    pcnt = (ctypes.c_int64 * nph)()
    lib.tsg_profile_read(pms, pcnt, nph)
    lib.tsg_profile(0)
    phases = {nat.PHASES[k]: {"ms_per_launch": (pms[k] / pcnt[k]) if pcnt[k] else 0.0,
                              "launches": int(pcnt[k]), "share": pms[k] / max(sum(pms), 1e-12)}
              for k in range(nph) if pcnt[k]}
    # ---- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        # The host owns the state between steps: every step writes x, v, density from pinned
        # host memory and reads x, v, density, pressure back (in the order the step leaves).
        host = {k: torch.empty((n_total, c), dtype=torch.float64).pin_memory()
                for k, c in (("x", 3), ("v", 3), ("density", 1), ("pressure", 1))}
        ins, outs = ("x", "v", "density"), ("x", "v", "density", "pressure")
        for k in outs:
            ps.read_field(k, host[k])
        torch.cuda.synchronize()
        e2e_steps = max(1, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            for k in ins:
                ps.write_field(k, host[k])
            solver.step()
            ps.read_fields(outs, [host[k] for k in outs], non_blocking=True)
            torch.cuda.synchronize()  # the step's results are on the host before the next step
        torch.cuda.synchronize()
        el = max_over_ranks(dist, time.perf_counter() - t0)
        h2d = sum(host[k].numel() * 8 for k in ins)
        d2h = sum(host[k].numel() * 8 for k in outs)
        e2e = {"value": n_fluid * e2e_steps / el, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": e2e_steps}
    diag = ps.diagnostics()
    try:
        list_stats = ps.list_stats()
    except nat.NativeError:  # the FP64 form traverses cells and keeps no lists
        list_stats = None
    del sim
    torch.cuda.synchronize()
    rebuilds = None
    if timed_builds is not None:
        rebuilds = {"in_timed_steps": timed_builds, "timed_steps": args.steps,
                    "since_upload": list_stats["builds"] if list_stats else None,
                    "steps_since_upload": 2 * args.steps + args.warmup + (e2e["steps"] if e2e else 0),
                    "note": "FP32-mixed neighbour lists hold pairs within support + skin and are rebuilt "
                            "(with the sort) only once a particle has moved 0.45 skin; the FP64 form "
                            "sorts and traverses cells every step"}
    return {"ms_per_step": ms, "value": n_fluid / (ms * 1e-3), "launches": launches,
            "list_rebuilds": rebuilds,
            "launches_per_step": launches / args.steps, "clocks": clocks, "phases": phases, "e2e": e2e,
            "n_total": n_total, "n_fluid": n_fluid, "diag_mass": diag["mass"], "lists": list_stats}


def error_report(cfg_dict, checkpoints=(1, 20)):
    """Per-field error of the FP32-mixed form against the FP64 form after each checkpoint.

    Both forms start from the same uploaded state.  The FP64 GPU form rounds every
    operation like the f64 CPU oracle (the parity tests require bit-identical results), so
    it stands in for the oracle at full size, where the oracle would need minutes.
    """
    import torch

    from tisphi_gb300 import compare
    from tisphi_gb300.configer_builder import SimConfiger
    from tisphi_gb300.simulation import Simulation

    sims = {p: Simulation(SimConfiger(config=cfg_dict), precision=p) for p in ("fp32_mixed", "fp64")}
    d0 = {p: s.ps.diagnostics() for p, s in sims.items()}
    out, done = {}, 0
    for n in checkpoints:
        for s in sims.values():
            s.solver.step(n - done)
        done = n
        torch.cuda.synchronize()
        rec = compare.field_errors(sims["fp32_mixed"].ps, sims["fp64"].ps)
        dr = {p: compare.drift(d0[p], s.ps.diagnostics()) for p, s in sims.items()}
        rec["conservation"] = {p: {"mass_rel": v["mass_rel"], "momentum_change": v["momentum"],
                                   "energy_rel": v["energy_rel"], "front": v["front"]} for p, v in dr.items()}
        out[f"after_{n}_steps"] = rec
    del sims
    torch.cuda.synchronize()
    return {"reference": "FP64 GPU form (bit-identical to the f64 oracle in the parity tests)",
            "matched_by": "id0", "particles": "fluid",
            "definitions": "density: |a-b|/|b| per particle; pressure, v, d_density, d_vel: |a-b| / max|b| "
                           "(Euclidean norm per particle for vectors); x: max |a-b| in metres",
            **out}


def full_run(cfg_dict, nsteps=1000):
    """The benchmark configuration's whole run (1,000 leap-frog steps from rest) in the
    FP32-mixed form, timed with CUDA events: the per-step cost including every neighbour-list
    rebuild the run needs (the K-step window of the headline starts from rest, where no
    rebuild is due yet)."""
    import torch

    from tisphi_gb300.configer_builder import SimConfiger
    from tisphi_gb300.simulation import Simulation
    sim = Simulation(SimConfiger(config=cfg_dict), precision="fp32_mixed")
    stream = torch.cuda.current_stream()
    sim.solver.step(1)
    torch.cuda.synchronize()
    b0 = sim.ps.list_stats()["builds"]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    sim.solver.step(nsteps - 1)
    stop.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(stop) / (nsteps - 1)
    sim.ps.check_errors()
    rebuilds = sim.ps.list_stats()["builds"] - b0
    n_fluid = int(np.count_nonzero(sim.ps.scene.mat_type == 1))
    return {"steps": nsteps, "ms_per_step": ms, "value": n_fluid / (ms * 1e-3), "list_rebuilds": rebuilds,
            "front": sim.ps.diagnostics()["front"]}


def read_profile_traffic(kernel_tag, entries_now):
    """DRAM traffic per launch of the rates kernel, from the committed ncu summary
    (profiles/<kernel_tag>.md) of a smaller capture of the same kernels, scaled to this run
    by its list entries (the list stream and the neighbour gathers, ~all of the traffic,
    grow with them).  The summary states its capture in three machine-read lines:
    ``capture_list_entries:``, ``capture_dram_bytes_per_launch:`` (read + write, mean of
    the step's rates passes) and ``capture:`` (what was captured).  Returns (bytes, source)
    or (None, reason)."""
    rel = os.path.join("profiles", f"{kernel_tag}.md")
    keys = {}
    try:
        for line in open(os.path.join(ROOT, rel)):
            k, sep, v = line.partition(":")
            if sep and k.strip() in ("capture_list_entries", "capture_dram_bytes_per_launch", "capture"):
                keys[k.strip()] = v.strip()
    except OSError:
        return None, f"{rel} missing"
    try:
        ent = float(keys["capture_list_entries"])
        byt = float(keys["capture_dram_bytes_per_launch"])
    except (KeyError, ValueError):
        return None, f"{rel} has no capture lines"
    scale = entries_now / ent if entries_now else None
    if not scale:
        return None, "no list entries in this run"
    return byt * scale, {"profile": rel, "capture": keys.get("capture", ""),
                         "capture_dram_bytes_per_launch": byt, "capture_list_entries": int(ent),
                         "scale": scale, "scaled_by": "list entries of this run / of the capture"}


def run_ours(args):
    import torch
    rank, ws, dist = dist_init(args)
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    cfg_dict, wname = workload(args)
    from tisphi_gb300 import build_native
    build_native.build()
    forms = {}
    order = ["fp32_mixed", "fp64"] if args.precision == "both" else [args.precision]
    for prec in order:
        try:
            forms[prec] = measure(args, cfg_dict, prec, rank, dist)
        except Exception as e:  # FP32-mixed may be absent from the library build
            forms[prec] = {"error": str(e)}
    head = "fp32_mixed" if "value" in forms.get("fp32_mixed", {}) else "fp64"
    h = forms[head]
    if "value" not in h:
        raise SystemExit(f"measurement failed: {forms}")
    peak, peak_kind = hbm_peak()
    corr = cfg_dict["Configuration"]["kernelCorrection"] == 1
    n_flow = h["n_fluid"]
    def roof(kernel):
        ph = h["phases"].get(kernel)
        conf = cfg_dict["Configuration"]
        ti = conf.get("timeIntegration")
        fused = None
        if head == "fp32_mixed" and conf.get("simulationMethod", 1) == 1 and ti in (1, 2):
            fused = "lf" if ti == 2 else "se"
        alg = algorithmic_bytes(kernel, h["n_total"], n_flow, head, corr, h.get("lists"), fused)
        if not ph or not alg or not ph["ms_per_launch"]:
            return None
        ach = alg / (ph["ms_per_launch"] * 1e-3) / 1e9
        return {"achieved": ach, "frac": ach / peak, "algorithmic_bytes_per_launch": alg,
                "ms_per_launch": ph["ms_per_launch"]}
    rates = roof("rates") or {"achieved": 0.0, "frac": 0.0, "algorithmic_bytes_per_launch": None,
                              "ms_per_launch": 0.0}
    entries_now = (h.get("lists") or {}).get("entries_real")
    traffic, traffic_source = read_profile_traffic(f"rates_{head}_3d_dambreak", entries_now)
    line = {
        "metric": METRIC, "value": h["value"] * ws, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": h["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if head == "fp32_mixed" else "f64", "data": "synthetic",
        "config": {"workload": f"{wname}, spacing {args.spacing} m, {h['n_fluid']:,} fluid + "
                               f"{h['n_total'] - h['n_fluid']:,} dummy particles, LF dt 2e-5, CSPM on, XSPH off",
                   "form": head, "n_fluid": h["n_fluid"], "n_total": h["n_total"],
                   "l2": "working set > 129 MB L2 (no flush needed)",
                   "list_skin": cfg_dict["Configuration"].get("neighbourSkin", 0.05),
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "forms": {k: ({"value": v["value"], "ms_per_step": v["ms_per_step"]} if "value" in v else v)
                  for k, v in forms.items()},
        "roofline": {"kernel": "rates: continuity + momentum (k_rates32 / k_wc_rates)", "bound": "hbm",
                     "achieved": rates["achieved"], "peak": peak, "unit": "GB/s", "frac": rates["frac"],
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": rates["algorithmic_bytes_per_launch"],
                     "ms_per_launch": rates["ms_per_launch"], "traffic": traffic,
                     "traffic_source": traffic_source,
                     "other_kernels": {k: roof(k) for k in ("kernel_corr", "boundary") if roof(k)}},
        "phases": h["phases"],
        "clocks": h["clocks"],
        "e2e": h["e2e"],
        "gpu_launches": int(h["launches"]),
        "list_rebuilds": h.get("list_rebuilds"),
        "lists": h.get("lists"),
    }
    if "fp32_mixed" in forms and "fp64" in forms and "value" in forms["fp32_mixed"] and "value" in forms["fp64"]:
        line["speedup_fp32_mixed_vs_fp64"] = forms["fp32_mixed"]["value"] / forms["fp64"]["value"]
    # the same rate counted over every particle of the step (fluid + dummies)
    line["particle_updates_per_s_all_particles"] = h["n_total"] * ws / (h["ms_per_step"] * 1e-3)
    if rank == 0 and head == "fp32_mixed" and args.workload == "3d" and not args.no_full_run:
        fr = full_run(cfg_dict)
        line["forms"]["fp32_mixed"]["full_1000_step_run"] = fr
        # the whole 1,000-step run, list rebuilds included (the K-step window above starts
        # from rest, where no rebuild is due yet)
        line["amortised"] = {"value": fr["value"] * ws, "unit": UNIT, "ms_per_step": fr["ms_per_step"],
                             "steps": fr["steps"], "list_rebuilds": fr["list_rebuilds"],
                             "how": "CUDA events around steps 2..1000 of one run from rest"}
    # The full-size accuracy check of the benchmark configuration runs once per job (N = 1):
    # both forms from the same state for error_steps leap-frog steps.
    if (rank == 0 and ws == 1 and not args.no_errors
            and all("value" in forms.get(p, {}) for p in ("fp32_mixed", "fp64"))):
        cps = tuple(sorted({1, 20, args.error_steps}))
        t0 = time.perf_counter()
        line["errors"] = error_report(cfg_dict, checkpoints=cps)
        line["errors"]["wall_s"] = time.perf_counter() - t0
        rel = line["errors"]["after_1_steps"].get("density", {}).get("max_rel")
        line["config"]["density_rel_err_1_step"] = rel
        last = line["errors"][f"after_{cps[-1]}_steps"]
        c32, c64 = last["conservation"]["fp32_mixed"], last["conservation"]["fp64"]
        line["accuracy"] = {
            "steps": cps[-1], "against": "FP64 GPU form (bit-identical to the f64 oracle in the parity tests)",
            "density_rel": {k: last["density"][k] for k in ("max_rel", "rms_rel")},
            "d_density_norm": {k: last["d_density"][k] for k in ("max_norm", "rms_norm")},
            "d_vel_norm": {k: last["d_vel"][k] for k in ("max_norm", "rms_norm")},
            "v_norm": {k: last["v"][k] for k in ("max_norm", "rms_norm")},
            "x_max_abs_m": last["x"]["max_abs"],
            "front_m": {"fp32_mixed": c32["front"], "fp64": c64["front"],
                        "difference": abs(c32["front"] - c64["front"])},
            "energy_change_rel": {"fp32_mixed": c32["energy_rel"], "fp64": c64["energy_rel"]},
            "momentum_change": {"fp32_mixed": c32["momentum_change"], "fp64": c64["momentum_change"]},
            "mass_rel": {"fp32_mixed": c32["mass_rel"], "fp64": c64["mass_rel"]}}
    # the other forms' headline checks, bounded: the 256-scene ensemble against sequential
    # launches, and short adjoint-vs-finite-difference checks (N = 1)
    if rank == 0 and ws == 1 and args.workload == "3d" and not args.no_forms:
        line["ensemble"] = ensemble_report(256, steps=20, warmup=3, seq_steps=5, tune=False)
        line["adjoint_check"] = adjoint_check()
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg_dict)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def ensemble_report(nscenes=256, steps=20, warmup=3, seq_steps=10, tune=True):
    """The 256-scene dambreak ensemble: one batched handle (graph replays, autotuned launch
    shape) against the same scenes stepped one after another through their own handles."""
    import torch

    from tisphi_gb300 import scenes
    from tisphi_gb300.batch import SceneBatch
    from tisphi_gb300.configer_builder import SimConfiger
    from tisphi_gb300.simulation import Simulation
    cfgs = scenes.dambreak_ensemble(nscenes)
    batch = SceneBatch(cfgs)
    nf = int(batch.n_fluid.sum())
    tuned = batch.autotune(trial_steps=10) if tune else None
    stream = torch.cuda.current_stream()
    batch.step(warmup)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        start.record(stream)
        batch.step(steps)
        stop.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop) / steps
    batch.check_errors()
    stats = batch.list_stats()
    del batch
    # sequential: every scene through its own handle, one after another
    sims = [Simulation(SimConfiger(config=c), precision="fp32_mixed") for c in cfgs]
    for s in sims:
        s.solver.step(1)
    torch.cuda.synchronize()
    k_seq = max(1, min(steps, seq_steps))
    start.record(stream)
    for s in sims:
        s.solver.step(k_seq)
    stop.record(stream)
    torch.cuda.synchronize()
    ms_seq = start.elapsed_time(stop) / k_seq
    del sims
    torch.cuda.synchronize()
    return {"scenes": nscenes, "n_fluid": nf, "ms_per_step": ms, "value": nscenes / (ms * 1e-3),
            "unit": "scenes*steps/s", "steps": steps, "warmup": warmup, "launch": tuned,
            "particle_updates_per_s": nf / (ms * 1e-3),
            "sequential": {"ms_per_step_all_scenes": ms_seq, "value": nscenes / (ms_seq * 1e-3),
                           "steps_timed": k_seq, "how": "each scene's own FP32-mixed handle, stepped in turn"},
            "speedup_vs_sequential": ms_seq / ms, "lists": stats, "clocks": clk.summary()}


def run_batch(args):
    """256-scene dambreak ensemble, batched vs sequential (ensemble_report)."""
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    from tisphi_gb300 import build_native
    build_native.build()
    rep = ensemble_report(args.scenes, args.steps, args.warmup)
    line = {"metric": "scenes*steps/s, 256-scene 2D WCSPH dambreak ensemble, batched vs sequential",
            "value": rep["value"], "unit": "scenes*steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rep["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"{args.scenes} 2D WCSPH dambreaks, spacing 0.01 m, block width U[0.3, 1.5] m, "
                                   f"height U[0.2, 0.8] m, B log-U[2e4, 1e5], nu log-U[1e-3, 1e-2], seed 7, "
                                   f"LF dt 1e-4", "n_fluid": rep["n_fluid"],
                       "l2": "working set ~0.15 GB > 129 MB L2 (no flush)"},
            **{k: rep[k] for k in ("launch", "particle_updates_per_s", "sequential", "speedup_vs_sequential",
                                   "lists", "clocks")}}
    print(json.dumps(line))


def adjoint_check():
    """Short adjoint checks against central finite differences of the FP64 form: the
    differentiable mu(I) column (0.2 x 0.1 m at spacing 0.002 m, symplectic Euler at dt 2e-5)
    over 200 steps (friction angle), and the 2D WCSPH dambreak (spacing 0.01 m, 0.6 x 0.4 m
    block, symplectic Euler at dt 1e-4) over 400 steps (stiffness and viscosity)."""
    import torch

    from tisphi_gb300 import scenes
    from tisphi_gb300.adjoint import MuIRollout, WCRollout, distal_loss, rollout_positions
    t0 = time.perf_counter()
    d = scenes.column_2d(method=2, spacing=0.002, dt=2e-5)
    model = MuIRollout(d, nsteps=200, checkpoint_every=100)
    params = torch.tensor([21.9, 0.0], dtype=torch.float64, requires_grad=True)
    loss, sel = distal_loss(model(params))
    loss.backward()
    g = params.grad.tolist()
    delta = 1e-4
    l_hi, _ = distal_loss(rollout_positions(d, 200, 21.9 + delta, 0.0), sel=sel)
    l_lo, _ = distal_loss(rollout_positions(d, 200, 21.9 - delta, 0.0), sel=sel)
    fd = (float(l_hi) - float(l_lo)) / (2 * delta)
    mui = {"steps": 200, "n_particles": model.n, "grad_friction_deg": g[0], "fd_friction_deg": fd,
           "rel_err": abs(g[0] - fd) / abs(fd)}
    dw = scenes.dambreak_2d(spacing=0.01, width=0.6, height=0.4, domain=(1.2, 0.8), integration=1)
    mw = WCRollout(dw, nsteps=400, checkpoint_every=100)
    B0, nu0 = mw.stiffness, mw.viscosity
    pw = torch.tensor([B0, nu0], dtype=torch.float64, requires_grad=True)
    lw, selw = distal_loss(mw(pw), target=0.7)
    lw.backward()
    gw = pw.grad.tolist()
    fdw = []
    for k in range(2):
        lo, hi = [B0, nu0], [B0, nu0]
        dk = 1e-4 * (B0, nu0)[k]
        lo[k] -= dk
        hi[k] += dk
        a, _ = distal_loss(rollout_positions(dw, 400, *hi), target=0.7, sel=selw)
        b, _ = distal_loss(rollout_positions(dw, 400, *lo), target=0.7, sel=selw)
        fdw.append((float(a) - float(b)) / (2 * dk))
    wc = {"steps": 400, "n_particles": mw.n, "grad": {"stiffness": gw[0], "viscosity": gw[1]},
          "fd": {"stiffness": fdw[0], "viscosity": fdw[1]},
          "rel_err": {"stiffness": abs(gw[0] - fdw[0]) / abs(fdw[0]), "viscosity": abs(gw[1] - fdw[1]) / abs(fdw[1])}}
    torch.cuda.synchronize()
    return {"against": "central finite differences of the FP64 form, relative step 1e-4",
            "mui_column": mui, "wcsph_dambreak": wc, "wall_s": time.perf_counter() - t0}


def run_adjoint(args):
    """Differentiable mu(I) column (0.2 x 0.1 m at spacing 0.002 m, symplectic Euler at
    dt 2e-5, checkpoints every 100 steps): loss = mean squared distance of the 1 % most
    distal particles' x from 0.35 m; gradient in friction angle (deg) and cohesion (Pa) from
    the hand-written adjoint, against central finite differences of the FP64 form at two
    step sizes, for a short horizon and for the full 2,000 steps."""
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    from tisphi_gb300 import build_native, scenes
    build_native.build()
    from tisphi_gb300.adjoint import MuIRollout, distal_loss, rollout_positions
    d = scenes.column_2d(method=2, spacing=0.002, dt=2e-5)
    # warm-up: first launches of every kernel, graph captures, allocator growth
    warm = MuIRollout(d, nsteps=20, checkpoint_every=10)
    wp = torch.tensor([21.9, 0.0], dtype=torch.float64, requires_grad=True)
    distal_loss(warm(wp))[0].backward()
    del warm
    runs = []
    for steps in sorted({200, args.adjoint_steps}):
        model = MuIRollout(d, nsteps=steps, checkpoint_every=100)
        params = torch.tensor([21.9, 0.0], dtype=torch.float64, requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x = model(params)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss, sel = distal_loss(x)
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        grad = params.grad.tolist()
        fd = {}
        for delta in (1e-4, 1e-2):
            vals = []
            for k in range(2):
                lo, hi = [21.9, 0.0], [21.9, 0.0]
                lo[k] -= delta
                hi[k] += delta
                l_hi, _ = distal_loss(rollout_positions(d, steps, *hi), sel=sel)
                l_lo, _ = distal_loss(rollout_positions(d, steps, *lo), sel=sel)
                vals.append((float(l_hi) - float(l_lo)) / (2 * delta))
            fd[str(delta)] = {"friction_deg": vals[0], "cohesion_pa": vals[1]}
        f4 = fd["0.0001"]
        rel = {"friction_deg": abs(grad[0] - f4["friction_deg"]) / abs(f4["friction_deg"]),
               "cohesion_pa": abs(grad[1] - f4["cohesion_pa"]) / abs(f4["cohesion_pa"])}
        runs.append({"steps": steps, "loss": float(loss.detach()),
                     "grad": {"friction_deg": grad[0], "cohesion_pa": grad[1]},
                     "central_fd_fp64": fd, "rel_err_vs_fd_1e-4": rel,
                     "seconds": {"forward": t1 - t0, "backward": t2 - t1}})
    # WCSPH: 2D dambreak (spacing 0.01 m, 0.6 x 0.4 m block, symplectic Euler at dt 1e-4),
    # gradient in the Tait stiffness B and the viscosity, same loss on the fluid front
    from tisphi_gb300.adjoint import WCRollout
    dw = scenes.dambreak_2d(spacing=0.01, width=0.6, height=0.4, domain=(1.2, 0.8), integration=1)
    wc_runs = []
    for steps in (400, 1000, 2000):
        model_w = WCRollout(dw, nsteps=steps, checkpoint_every=100)
        B0, nu0 = model_w.stiffness, model_w.viscosity
        params = torch.tensor([B0, nu0], dtype=torch.float64, requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x = model_w(params)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss, sel = distal_loss(x, target=0.7)
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        grad = params.grad.tolist()
        fd = {}
        for rel in (1e-4, 1e-2):
            vals = []
            for k in range(2):
                lo, hi = [B0, nu0], [B0, nu0]
                delta = rel * (B0, nu0)[k]
                lo[k] -= delta
                hi[k] += delta
                l_hi, _ = distal_loss(rollout_positions(dw, steps, *hi), target=0.7, sel=sel)
                l_lo, _ = distal_loss(rollout_positions(dw, steps, *lo), target=0.7, sel=sel)
                vals.append((float(l_hi) - float(l_lo)) / (2 * delta))
            fd[str(rel)] = {"stiffness": vals[0], "viscosity": vals[1]}
        f4 = fd["0.0001"]
        wc_runs.append({"steps": steps, "loss": float(loss.detach()),
                        "grad": {"stiffness": grad[0], "viscosity": grad[1]},
                        "central_fd_fp64_relative_step": fd,
                        "rel_err_vs_fd_1e-4": {"stiffness": abs(grad[0] - f4["stiffness"]) / abs(f4["stiffness"]),
                                               "viscosity": abs(grad[1] - f4["viscosity"]) / abs(f4["viscosity"])},
                        "seconds": {"forward": t1 - t0, "backward": t2 - t1}})
    line = {"metric": "adjoint gradient of the differentiable mu(I) column vs central FD (FP64)",
            "value": runs[0]["rel_err_vs_fd_1e-4"]["friction_deg"], "unit": "relative error, friction, 200 steps",
            "higher_is_better": False, "n_particles": model.n, "checkpoint_every": 100, "runs": runs,
            "wcsph": {"workload": "2D WCSPH dambreak, spacing 0.01 m, 0.6 x 0.4 m block, SE dt 1e-4; "
                                  "loss: mean squared distance of the 1 % most distal fluid particles from x = 0.7 m",
                      "n_particles": model_w.n, "checkpoint_every": 100, "runs": wc_runs},
            "data": "synthetic"}
    print(json.dumps(line))


def run_rollout(args):
    """The 3D dambreak of the benchmark (block, domain, CSPM, leap-frog at dt 2e-5) at twice
    the spacing (0.0108 m, one eighth of the particles) for 2,000 steps in both forms: the
    FP32-mixed form's per-field error and conservation figures against the FP64 form after
    1, 100 and 2,000 steps (mass, momentum and mechanical-energy change, dambreak front)."""
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    from tisphi_gb300 import build_native, scenes
    build_native.build()
    d = scenes.dambreak_3d(spacing=0.0108)
    t0 = time.perf_counter()
    rep = error_report(d, checkpoints=(1, 100, 2000))
    wall = time.perf_counter() - t0
    last = rep["after_2000_steps"]
    c32, c64 = last["conservation"]["fp32_mixed"], last["conservation"]["fp64"]
    line = {"metric": "FP32-mixed vs FP64 after 2,000 steps, 3D WCSPH dambreak at spacing 0.0108 m",
            "value": last["density"]["rms_rel"], "unit": "RMS relative density error after 2,000 steps",
            "higher_is_better": False,
            "front_difference_m": abs(c32["front"] - c64["front"]),
            "energy_change_rel": {"fp32_mixed": c32["energy_rel"], "fp64": c64["energy_rel"]},
            "momentum_change": {"fp32_mixed": c32["momentum_change"], "fp64": c64["momentum_change"]},
            "errors": rep, "wall_s": wall, "data": "synthetic"}
    print(json.dumps(line))


def run_column(args):
    """The granular column collapse of the benchmark configuration: 0.2 x 0.1 m of sand at
    spacing 0.001 m (20,000 particles + 2,418 dummies), seeded +-1 % jitter, Wendland C2,
    dummy boundary, symplectic Euler at dt 1e-5 for 6,100 steps (0.061 s).  mu(I): the
    FP32-mixed form against the FP64 form (runout = largest x of the soil, mean and
    per-particle equivalent strain, per-field errors) at checkpoints.  Drucker-Prager at the
    same settings: the FP64 form's mechanical energy against its initial value every
    50 steps, the record of why the Drucker-Prager comparisons use the reference's sand-scene
    integrator (leap-frog + XSPH) instead; then that comparison at this size."""
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    from tisphi_gb300 import build_native, compare, scenes
    build_native.build()
    from tisphi_gb300.configer_builder import SimConfiger
    from tisphi_gb300.simulation import Simulation

    def compare_forms(d, steps, checkpoints):
        cfg = SimConfiger(config=d)
        sims = {p: Simulation(cfg, precision=p) for p in ("fp32_mixed", "fp64")}
        d0 = {p: s.ps.diagnostics() for p, s in sims.items()}
        out, done, secs = {}, 0, {p: 0.0 for p in sims}
        for n in checkpoints:
            for p, s in sims.items():
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s.solver.step(n - done)
                torch.cuda.synchronize()
                secs[p] += time.perf_counter() - t0
            done = n
            dr = {p: compare.drift(d0[p], s.ps.diagnostics()) for p, s in sims.items()}
            ids = {p: s.ps.field("id0").cpu().numpy() for p, s in sims.items()}
            eqs = {}
            for p, s in sims.items():
                mt = s.ps.field("mat_type").cpu().numpy()
                e = s.ps.field("strain_equ").cpu().numpy().astype(np.float64)
                by_id = np.empty_like(e)
                by_id[ids[p]] = e
                soil = np.empty_like(mt)
                soil[ids[p]] = mt
                eqs[p] = by_id[soil == 2]
            rec = compare.field_errors(sims["fp32_mixed"].ps, sims["fp64"].ps,
                                       fields=("density", "x", "v", "stress"))
            e32, e64 = eqs["fp32_mixed"], eqs["fp64"]
            rec["runout_m"] = {p: dr[p]["front"] for p in sims}
            rec["runout_difference_in_spacings"] = abs(dr["fp32_mixed"]["front"] - dr["fp64"]["front"]) / d[
                "Configuration"]["particleRadius"] / 2
            rec["strain_equ_mean"] = {"fp32_mixed": float(e32.mean()), "fp64": float(e64.mean())}
            rec["strain_equ_mean_rel_diff"] = (abs(float(e32.mean()) - float(e64.mean()))
                                               / max(abs(float(e64.mean())), 1e-300))
            rec["strain_equ_max_abs_diff"] = float(np.max(np.abs(e32 - e64)))
            rec["energy_change_rel"] = {p: dr[p]["energy_rel"] for p in sims}
            out[f"after_{n}_steps"] = rec
        n_soil = int(np.count_nonzero(sims["fp64"].ps.scene.mat_type == 2))
        n_all = sims["fp64"].ps.particle_max_num
        del sims
        torch.cuda.synchronize()
        return {"n_soil": n_soil, "n_total": n_all, "seconds": secs,
                "particle_updates_per_s": {p: n_soil * steps / v for p, v in secs.items()}, **out}

    steps = args.column_steps
    cps = tuple(sorted({1, 100, 1000, steps}))
    t0 = time.perf_counter()
    mui = compare_forms(scenes.column_2d(method=2, spacing=0.001, dt=1e-5, integration=1), steps, cps)
    # Drucker-Prager at the stated settings, FP64 (bit-identical to the oracle): energy record
    dp_cfg = SimConfiger(config=scenes.column_2d(method=3, spacing=0.001, dt=1e-5, integration=1))
    dp = Simulation(dp_cfg, precision="fp64")
    dg0 = dp.ps.diagnostics()
    e0 = dg0["kinetic"] + dg0["potential"]
    energy = []
    for q in range(1, 21):
        dp.solver.step(50)
        dg = dp.ps.diagnostics()
        e = dg["kinetic"] + dg["potential"]
        energy.append({"steps": 50 * q, "kinetic_over_initial_mechanical": dg["kinetic"] / abs(e0),
                       "mechanical_change_rel": (e - e0) / abs(e0), "vmax": dg["vmax"]})
        if not np.isfinite(e):
            break
    del dp
    # Drucker-Prager with the reference sand scene's integrator (leap-frog + XSPH)
    dp_lf = compare_forms(scenes.column_2d(method=3, spacing=0.001, dt=1e-5, integration=2, xsph=True),
                          min(steps, 2000), tuple(sorted({1, 100, min(steps, 2000)})))
    last = mui[f"after_{steps}_steps"]
    line = {"metric": "mu(I) column collapse, FP32-mixed vs FP64 after the full run (0.061 s)",
            "value": last["runout_difference_in_spacings"], "unit": "runout difference, particle spacings",
            "higher_is_better": False,
            "config": {"workload": "2D sand column 0.2 x 0.1 m, spacing 0.001 m, +-1 % jitter, Wendland C2, "
                                   f"dummy boundary, symplectic Euler dt 1e-5, {steps} steps",
                       "n_soil": mui["n_soil"], "n_total": mui["n_total"]},
            "strain_equ_mean_rel_diff": last["strain_equ_mean_rel_diff"],
            "mui": mui,
            "dp_stated_settings_fp64_energy": energy,
            "dp_leapfrog_xsph": dp_lf,
            "wall_s": time.perf_counter() - t0, "data": "synthetic"}
    print(json.dumps(line))


def run_kernels(args):
    """Every kernel family of both forms at least once, at sizes above the 129 MB L2 where the
    scene allows: the command that the per-kernel DRAM / cache survey captures (one line of
    wall times per leg, no bench figure).  Each leg builds its scene in both forms, steps it
    three times and frees it; the particle-system extras (density summation, field export,
    the visual buffer, the allocation-free sort) run on the legs that name them, the
    ensemble and both adjoints on small scenes of their stated kind."""
    import ctypes

    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    from tisphi_gb300 import _native as nat
    from tisphi_gb300 import build_native, scenes
    build_native.build()
    from tisphi_gb300.adjoint import MuIRollout, WCRollout, distal_loss
    from tisphi_gb300.batch import SceneBatch
    from tisphi_gb300.configer_builder import SimConfiger
    from tisphi_gb300.simulation import Simulation
    lib = nat.load()
    # eager launches (the phase timer's mode) rather than graph replays, so that a
    # per-launch profiler sees every kernel of the step sequences
    lib.tsg_profile(1)

    def with_boundary(d, b):
        d["Configuration"]["boundary"] = b
        return d

    col = dict(spacing=0.0005, width=1.0, height=0.5, domain=(2.5, 0.6))
    legs = [
        ("3D WCSPH dambreak, spacing 0.0075 m, LF, CSPM", scenes.dambreak_3d(spacing=0.0075),
         {"density", "export", "visual"}),
        ("2D WCSPH dambreak, spacing 0.001 m, RK4, XSPH, CSPM",
         scenes.dambreak_2d(spacing=0.001, integration=4, xsph=True, corr=1), {"density"}),
        ("2D WCSPH dambreak, spacing 0.001 m, SE, cubic spline, dummy + repulsive boundary",
         with_boundary(scenes.dambreak_2d(spacing=0.001, integration=1, kernel=0), 4), set()),
        ("2D mu(I) column 1.0 x 0.5 m, spacing 0.0005 m, SE, CSPM",
         scenes.column_2d(method=2, integration=1, corr=1, **col), {"export"}),
        ("2D Drucker-Prager column 1.0 x 0.5 m, spacing 0.0005 m, LF, XSPH",
         scenes.column_2d(method=3, integration=2, xsph=True, **col), set()),
        # small enough for the allocation-free sort's fixed arrays (262,144 particles and cells)
        ("2D water with a dynamic rigid box, spacing 0.002 m, LF", scenes.floating_box_2d(spacing=0.002),
         {"noalloc"}),
    ]
    out = []
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for name, d, extras in legs:
        for precision in ("fp32_mixed", "fp64"):
            t0 = time.perf_counter()
            sim = Simulation(SimConfiger(config=d), precision=precision)
            sim.solver.step(3)
            ps = sim.ps
            if "density" in extras:
                sim.solver.calc_density()
            if "export" in extras:
                host = [torch.empty((ps.particle_max_num, 3), dtype=torch.float64).pin_memory() for _ in range(2)]
                ps.read_fields(("x", "v"), host)
            if "visual" in extras:
                ps.visual()
            if "noalloc" in extras and precision == "fp32_mixed":
                n, G = ps.particle_max_num, ps.grid_num_total
                cs = torch.empty(G + 2, dtype=torch.int32, device="cuda")
                perm = torch.empty(n, dtype=torch.int32, device="cuda")
                x = ps.field("x").contiguous()
                nat.check(lib.tsg_sort_noalloc(ctypes.byref(ps._cfg), ctypes.c_void_p(x.data_ptr()), n,
                                               ctypes.c_void_p(cs.data_ptr()), ctypes.c_void_p(perm.data_ptr()),
                                               stream), "tsg_sort_noalloc")
            torch.cuda.synchronize()
            out.append({"leg": name, "form": precision, "n_particles": ps.particle_max_num,
                        "seconds": time.perf_counter() - t0})
            del sim, ps
    t0 = time.perf_counter()
    batch = SceneBatch(scenes.dambreak_ensemble(64))
    batch.step(3)
    torch.cuda.synchronize()
    out.append({"leg": "64-scene 2D WCSPH ensemble, LF", "form": "fp32_mixed", "n_particles": batch.n,
                "seconds": time.perf_counter() - t0})
    del batch
    for name, model, params, target in (
            ("mu(I) column adjoint, spacing 0.002 m, 10 SE steps",
             MuIRollout(scenes.column_2d(method=2, spacing=0.002, dt=2e-5), nsteps=10, checkpoint_every=5),
             [21.9, 0.0], 0.35),
            ("WCSPH dambreak adjoint, spacing 0.01 m, 10 SE steps",
             WCRollout(scenes.dambreak_2d(spacing=0.01, width=0.6, height=0.4, domain=(1.2, 0.8), integration=1),
                       nsteps=10, checkpoint_every=5), None, 0.7)):
        t0 = time.perf_counter()
        p = torch.tensor(params if params else [model.stiffness, model.viscosity], dtype=torch.float64,
                         requires_grad=True)
        distal_loss(model(p), target=target)[0].backward()
        torch.cuda.synchronize()
        out.append({"leg": name, "form": "fp32_mixed", "n_particles": model.n, "seconds": time.perf_counter() - t0})
        del model
    nph = len(nat.PHASES)
    lib.tsg_profile_read((ctypes.c_double * nph)(), (ctypes.c_int64 * nph)(), nph)
    lib.tsg_profile(0)
    print(json.dumps({"workload": "kernel survey (every kernel family, both forms)", "legs": out,
                      "data": "synthetic"}))


def run_reference(args):
    rank, ws, dist = dist_init(args)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cfg_dict, wname = workload(args)
    from oracle import oracle as orc_mod
    orc_mod.build()
    from oracle.oracle import OracleSim
    from tisphi_gb300.configer_builder import SimConfiger
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    orc = OracleSim(SimConfiger(config=cfg_dict))
    n_fluid = int(np.count_nonzero(orc.scene.mat_type == 1))
    budget = 150.0
    t0 = time.perf_counter()
    orc.step(1)
    first = time.perf_counter() - t0
    warm = max(0, min(args.warmup - 1, int(budget * 0.2 / max(first, 1e-3))))
    if warm:
        orc.step(warm)
    k = max(1, min(args.steps, int(budget * 0.6 / max(first, 1e-3))))
    t1 = time.perf_counter()
    orc.step(k)
    el = time.perf_counter() - t1
    v = n_fluid * k / el
    sample = (f"{k} full step(s) of the {orc.n:,}-particle scene after {warm + 1} untimed, f64 C++/OpenMP "
              f"restatement of the reference's Taichi kernels (Taichi itself is not installable here), "
              f"{cores} threads")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": k, "warmup": warm + 1,
            "ms_per_step": el / k * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{wname}, spacing {args.spacing} m, {n_fluid:,} fluid + "
                                   f"{orc.n - n_fluid:,} dummy particles", "form": "cpu-f64"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["both", "fp32_mixed", "fp64"], default="both")
    ap.add_argument("--workload", choices=["3d", "2d", "batch", "adjoint", "rollout", "column", "kernels"], default="3d")
    ap.add_argument("--column-steps", type=int, default=6100, help="run length for --workload column")
    ap.add_argument("--adjoint-steps", type=int, default=2000, help="rollout length for --workload adjoint")
    ap.add_argument("--scenes", type=int, default=256, help="ensemble size for --workload batch")
    ap.add_argument("--spacing", type=float, default=0.0054)
    ap.add_argument("--list-skin", type=float, default=None,
                    help="FP32-mixed neighbour-list skin as a fraction of the support radius (scene default 0.05)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-full-run", action="store_true", help="skip the 1,000-step FP32-mixed run")
    ap.add_argument("--no-errors", action="store_true", help="skip the FP32-mixed vs FP64 error report")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the ensemble and adjoint checks of the default line")
    ap.add_argument("--error-steps", type=int, default=1000,
                    help="length of the FP32-mixed vs FP64 comparison of the default workload (N = 1)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "rollout":
        run_rollout(args)
    elif args.workload == "column":
        run_column(args)
    elif args.workload == "kernels":
        run_kernels(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
