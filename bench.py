#!/usr/bin/env python3
"""Benchmark: particle-updates/s of the coupled DEM-SPH step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config 0|1|2|3|4]

One bench step is one fluid period of the scene: `gap` solverBase::update()
calls (core/solverBase.cpp:47-67), the last of them the fluid step (the
reference integrates the fluid when step % gap == 0, core/integrate.cu:385-421);
for a scene with gap 1 that is one update() call.  Each update() runs the
neighbour search, the two solid half-step integrations, the fluid work of the
step and the contact phase.  particle-updates/s counts every mobile particle
once per update it is advanced: N_fluid per fluid step plus the solids with
non-zero inverse mass per update (dummy wall particles are not counted).

Workloads (synthetic, seeded, generated by dem-sphsource_gb300/scenes.py):
  0  48k-fluid WCSPH dam break (dx 0.01 m, 3-layer dummy walls), gap 1
  1  Hertz-Mindlin settle: 200k lognormal spheres + 5k four-pebble clumps, gap 1,
     timed from a contact-dense bed (--settle-steps of the settle run first, untimed)
  2  coupled dam break: 1.0M fluid (dx 0.004 m) against 64 bonded 8^3 cubes, gap 28 (default)
  3  256-scene batched mix through the scene server
  4  Poisson serving stream through the scene server

`value` is measured with the scene resident in HBM: K bench steps replayed as
CUDA graphs on the engine's stream, bracketed by CUDA events (the inputs are
far larger than L2 for configs 1 and 2; config 0's state fits in L2, and the
line says so).  `e2e` is the same metric through the C ABI with host buffers:
every bench step uploads the dynamic state from pinned host memory, runs the
step and downloads it again (demsph_update_io).  `roofline` times each stage
with CUDA events (an uncaptured pass) and relates the dominant stage's
algorithmic bytes to the measured HBM copy bandwidth.  `cpu_baseline` is the
FP64 oracle (a CPU restatement of the reference's step; the reference has no
CPU solver) on all host cores, on a bounded sample of whole bench steps, from
a scene the oracle assembles itself (oracle/scene.py).  `fp64_error` compares
a second engine, run through the same steps from the same state, with the
oracle's state at the end of that sample.

--impl reference times that CPU implementation on the same workload: W + K
bench steps (fewer if they would not fit --ref-budget seconds; the line then
says how many it timed), without loading the product library.  Under torchrun
(N > 1) every rank runs an independent replica of the scene on its own GPU
(the step has no inter-GPU exchange); `value` is the sum over ranks divided by
the slowest rank's time; the reference arm runs on rank 0 only.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def _package():
    name = "dem_sphsource_gb300"
    if name in sys.modules:
        return sys.modules[name]
    d = os.path.join(ROOT, "dem-sphsource_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _scenes():
    """dem-sphsource_gb300/scenes.py alone (numpy only): the workload recipes,
    without the package and its library."""
    name = "demsph_scenes"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "dem-sphsource_gb300", "scenes.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


WORKLOADS = {
    0: ("dam_break_48k", "WCSPH dam break: tank 1.6x0.4x0.6 m, column 0.4x0.4x0.3 m, dx 0.01 m, 3-layer walls"),
    1: ("granular_settle_200k_5k", "Hertz-Mindlin settle: 200k lognormal spheres (median 1 mm, sigma 0.2, radii "
                                   "clipped to [0.6, 1.2] mm: a 2.5 mm lattice cannot hold 2 mm radii without "
                                   "overlaps) + 5k 4-pebble clumps, floor wall, box sides of fixed 1 mm spheres "
                                   "(infinite side walls would hold only grains touching the floor: the reference "
                                   "stops its wall loop at the first wall not touched)"),
    2: ("coupled_dam_break_1M_64cubes", "1.0M fluid (dx 0.004 m) dam break onto 64 bonded 8^3 sphere cubes; bond "
                                        "strength per cube from 9 levels in [0.5, 2.0] MPa (the reference keys "
                                        "strength by material pair)"),
}
SETTLE_STEPS = {1: 200000}  # config 1: untimed steps of the settle (0.33 s) before the timed window


def make_recipe(config):
    sc = _scenes()
    if config == 1:
        return sc.granular_settle(side_walls="spheres")
    return {0: sc.dam_break, 2: sc.coupled_dam_break}[config]()


def mobile_counts(scene):
    import numpy as np
    nf = scene.n_fluid
    ns = scene.n_solid
    if ns:
        im = np.ctypeslib.as_array(scene.solid_inverse_mass, shape=(ns,))
        dummy = np.ctypeslib.as_array(scene.solid_is_dummy, shape=(ns,))
        n_mobile = int(((im > 0) & (dummy == 0)).sum())
        n_dummy = int((dummy == 1).sum())
    else:
        n_mobile = n_dummy = 0
    return nf, n_mobile, n_dummy


def updates_for(first, n, gap, nf, n_mobile):
    fluid_steps = sum(1 for s in range(first, first + n) if s % gap == 0)
    return nf * fluid_steps + n_mobile * n


def workload_config(config, scene, args, settle):
    """The config dict both arms print: the workload and its sizes, computed
    from the scene's arrays (the product's or the oracle's: the same bits)."""
    name, desc = WORKLOADS[config]
    nf, n_mobile, n_dummy = mobile_counts(scene)
    gap = scene.fluid_integrate_gap
    cfg = {"workload": name, "description": desc, "n_fluid": nf, "n_solid_mobile": n_mobile,
           "n_dummy_wall": n_dummy, "n_clump": scene.n_clump, "dt": scene.time_step, "fluid_integrate_gap": gap,
           "step": (f"one fluid period: {gap} solverBase::update() calls, the last of them the fluid step"
                    if gap > 1 else "one solverBase::update() call"),
           "updates_per_step": updates_for(1, gap, gap, nf, n_mobile),
           "l2": "inputs larger than L2 (129 MB)" if config in (1, 2) else
                 "the scene's state (about 20 MB) fits in L2 (129 MB): not flushed between steps",
           "parallelism": f"replicas x{args.gpus}"}
    return cfg


def workload_state(args, settle):
    """Where the timed steps start (a sibling of `config` in the line: the
    reference arm starts from the initial state, the GPU arm can settle first)."""
    if getattr(args, "load_state", None):
        start = f"the state saved in {os.path.basename(args.load_state)} (springs from zero)"
    else:
        start = (f"the bed after {settle} untimed steps of the settle (contact-dense), springs and all"
                 if settle else "the workload's initial state")
    return (start +
            f", then {args.warmup} warm-up, {args.latency_steps} latency and {args.profile_steps} profiled "
            "bench steps before the timed ones")


def scene_state(scene):
    """{name: writable numpy view} of the dynamic state arrays of a scene
    (either ctypes mirror of demsph_scene), for restarting from a state."""
    import ctypes as C
    import numpy as np

    def view(ptr, n, w):
        if not n or not ptr:
            return None
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double)), shape=(n, w))
    ns, nc = scene.n_solid, scene.n_clump
    return {"solid.pos": view(scene.solid_position, ns, 3), "solid.vel": view(scene.solid_velocity, ns, 3),
            "solid.acc": view(scene.solid_acceleration, ns, 3), "solid.torque": view(scene.solid_torque, ns, 3),
            "solid.angvel": view(scene.solid_angular_velocity, ns, 3),
            "clump.centroid": view(scene.clump_centroid, nc, 3), "clump.vel": view(scene.clump_velocity, nc, 3),
            "clump.acc": view(scene.clump_acceleration, nc, 3), "clump.angvel": view(scene.clump_angular_velocity, nc, 3),
            "clump.torque": view(scene.clump_torque, nc, 3)}


def engine_state(eng):
    """The solid and clump state of an engine, in the names of scene_state."""
    s = eng.download_solids()
    out = {"solid.pos": s["pos"], "solid.vel": s["vel"], "solid.acc": s["acc"], "solid.torque": s["torque"],
           "solid.angvel": s["angvel"]}
    if eng.nc:
        c = eng.download_clumps()
        out.update({"clump.centroid": c["centroid"], "clump.vel": c["vel"], "clump.acc": c["acc"],
                    "clump.angvel": c["angvel"], "clump.torque": c["torque"]})
    return out


def restart_scene(scene, state):
    """Writes a state (engine_state) into a scene's arrays: an engine or oracle
    created from the scene then starts from that state (contact springs and
    wall springs start at zero, as at any scene start)."""
    views = scene_state(scene)
    for k, v in state.items():
        if views.get(k) is not None and v is not None:
            views[k][...] = v


# ---- clocks during the timed region -------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons while the GPU
    works.  The window covers the timed region (up to mark_end) plus, when the
    caller keeps the same load going after it, that tail, so a timed region
    shorter than the sampling period still has samples; the summary says how
    many came from each."""
    FIELDS = ("clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 20

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t_end = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark_end(self):
        self.t_end = time.perf_counter()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        in_region = 0
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for t, ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            if self.t_end is None or t <= self.t_end:
                in_region += 1
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "samples_in_timed_region": in_region,
                "window": "the timed region plus about 1 s of the same bench steps replayed right after it"}


# ---- algorithmic bytes per stage (compulsory traffic) -------------------------
def stage_bytes(stage, c):
    """Bytes one launch of `stage` must move at least, from the scene counts `c`."""
    P, Ns, Nf, Nb = c["solid_pairs"], c["n_solid_active"], c["n_fluid"], c["bonds"]
    kff = c.get("fluid_partners", 0.0)
    kfs = c.get("fluid_solid_partners", 0.0)
    table = {
        # per pair, once: partner id 4 + springs in 48 + springs out 48 + F T TA TB out 64; per
        # active solid: cell ph pl vh vl wh wl rad flags 144 + count 4; per bond: 160 (below)
        "pair_forces": 164 * P + 148 * Ns + 160 * Nb,
        # per pair, from both sides: F and the torque on the side 32 each; per bond and side:
        # id 4 + pair 8 + F T 32; per active solid: counts 8 + bond range 8 + flags 16 + mass 16
        # + coupling force 16 + acc torque out 32
        "solid_forces": 64 * P + 88 * Nb + 96 * Ns,
        # the list and the forces of a step opened by a fused pass in one launch, each pair from
        # both sides: partner ids written 8 + springs in 48 + springs out 48 + F T 32; per active
        # solid: candidates' count 4 + cell ph pl at the step's end and middle, vh vl wh wl, rad
        # flags 176 + counts out 8 + acc torque out 32
        "contact_forces": 136 * P + 220 * Ns,
        # per active solid: cell ph pl rad flags 80 + list and candidate counts 12 + walk
        # centre 8; per pair: partner ids 8 + previous springs 48 in + springs 48 out + history id 8
        "solid_contact_list": 100 * Ns + 112 * P,
        # per solid and step: cell ph pl read and written 96 + key 4 + walk centre 16 (the sort
        # by cell runs only when lists need it)
        "solid_hash_sort": 116 * c["n_solid"],
        # per solid: ph pl vh vl wh wl acc torque flags rad (10 float4 read, 6 written)
        "integrate_before": 256 * c["n_solid"],
        "integrate_after": 256 * c["n_solid"],
        # per fluid particle: list entries 4/partner + own 112 + one neighbour copy 52 + out 4..64
        "continuity": (4 * (kff + kfs) + 200) * Nf,
        "momentum": (4 * (kff + kfs) + 260) * Nf,
        "density_reinit": (4 * (kff + kfs) + 120) * Nf,
        # per fluid particle: candidate ids read (about 4/3 of the partners) + list entries
        # written + own position 32
        "fluid_lists": (4 * 4 * (kff + kfs) // 3 + 4 * (kff + kfs) + 32) * Nf,
        # predicated: per launch that rebuilds, candidate ids written + own data 64
        "fluid_candidates": (4 * 4 * (kff + kfs) // 3 + 64) * Nf,
        "fluid_hash_reorder": 496 * Nf,
        "coupling_lists": 8 * kfs * Nf,
        "coupling_force": 64 * c.get("coupling_pairs", 0) + 96 * Ns,
        "clump_force": 64 * c.get("n_pebbles", 0),
    }
    if c.get("tiles"):
        # membership bits: no per-partner list reads; per fluid particle its own
        # state, its bit words (4 B each) and, per solid partner, the list entry
        # and the solid's state (96 B); the partners' fluid state is shared by
        # neighbouring particles' walks (L1 and L2 reads)
        w = c["bit_words"]
        table.update({
            # own ph pl vh vl drho fsc read 72 + drho ph pl written 36 ... (rounded up to whole float4s)
            "continuity": (128 + 4 * w + 68 * kfs) * Nf,
            # own ph pl vh vl drho fsc read 72 + acc vh vl ph pl written 80
            "momentum": (160 + 4 * w + 96 * kfs) * Nf,
            # own cell ph pl sumW0 drho read 64 + drho written
            "density_reinit": (72 + 4 * w + 96 * kfs) * Nf,
            # own cell ph pl read 48 + bits, counts, solid list entries written
            "fluid_lists": (56 + 4 * w + 4 * kfs) * Nf,
        })
    return table.get(stage)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# FP32 operations per partner of the fluid pair loops, counted from their pair
# formulas (core/integrate.cu:55-161 continuity, :163-280 momentum): each add,
# multiply, division and square root one operation, the compensated (Kahan)
# sum four per component.  The pair loops are bound by FP32 issue, not by
# DRAM, once their partners are on chip.
PAIR_FLOPS = {"continuity": 55, "momentum": 86}


def stage_flops(stage, c):
    """FP32 operations one launch of a fluid pair stage performs, from the counts."""
    per = PAIR_FLOPS.get(stage)
    if per is None:
        return None
    return per * (c.get("fluid_partners", 0.0) + c.get("fluid_solid_partners", 0.0)) * c["n_fluid"]


def fp32_peak_tflops(torch):
    """FP32 (non-tensor) throughput of this GPU: cuBLAS SGEMM 8192^3 with TF32
    off, best of 5, by CUDA events."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        torch.matmul(a, b)
        best = None
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        del a, b
        return 2.0 * n ** 3 / (best / 1000.0) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def load_traffic(stage, workload):
    """Measured DRAM bytes per unit for a stage on a workload, from the
    committed ncu summary; another workload's figure for the stage when this
    one was not captured (its source says which)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            by = json.load(f).get(stage) or {}
    except (OSError, ValueError):
        return None
    return by.get(workload) or next(iter(by.values()), None)


# ---- CPU baseline: the FP64 oracle ------------------------------------------------------------
def oracle_scene(recipe, state=None):
    """The workload assembled by the oracle itself (oracle/scene.py: the
    reference's setup calls restated, no product library), optionally
    restarted from a state."""
    from oracle.scene import build_scene
    asm, scene = build_scene(recipe)
    if state is not None:
        restart_scene(scene, state)
    return asm, scene


def cpu_baseline(recipe, state, budget_s, first_step=1):
    """Times the FP64 oracle on all host cores over whole bench steps (fluid
    periods) of the workload: one warm-up bench step, then as many as fit
    budget_s (at least one).  Returns (cpu_baseline dict, oracle, DEM steps
    run, assembly that keeps the scene alive)."""
    from oracle import oracle as orc_mod
    threads = os.cpu_count() or 1
    orc_mod.set_threads(threads)
    asm, scene = oracle_scene(recipe, state)
    gap, dt = scene.fluid_integrate_gap, scene.time_step
    nf, n_mobile, _ = mobile_counts(scene)
    orc = orc_mod.OracleSolver(scene)
    orc.initialize()
    t0 = time.perf_counter()
    orc.update(dt, first_step, gap, gap)
    t1 = time.perf_counter() - t0
    n = max(1, min(1000 // gap + 1, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    orc.update(dt, first_step + gap, n * gap, gap)
    el = time.perf_counter() - t0
    ups = updates_for(first_step + gap, n * gap, gap, nf, n_mobile) / el
    return ({"value": ups, "unit": "particle-updates/s", "cores": threads, "kind": "port",
             "sample": f"{n} bench steps ({n * gap} update() calls, steps {first_step + gap}.."
                       f"{first_step + gap + n * gap - 1}) of the full workload after one warm-up bench step; "
                       f"FP64 oracle (CPU restatement of the reference's step), OpenMP over particles, "
                       f"scene assembled by the oracle"},
            orc, (n + 1) * gap, asm)


def reference_arm(args, rank):
    """--impl reference: the reference's step restated for the CPU (the FP64
    oracle; the reference's own code exists only as CUDA kernels) on all host
    cores, W + K bench steps of the same workload.  Never loads the product
    library: the recipe comes from scenes.py alone and the scene from the
    oracle's own assembly."""
    if rank != 0:
        return
    from oracle import oracle as orc_mod
    threads = os.cpu_count() or 1
    orc_mod.set_threads(threads)
    recipe = make_recipe(args.config)
    asm, scene = oracle_scene(recipe)
    gap, dt = scene.fluid_integrate_gap, scene.time_step
    nf, n_mobile, _ = mobile_counts(scene)
    cfg = workload_config(args.config, scene, args, 0)
    orc = orc_mod.OracleSolver(scene)
    orc.initialize()
    step = 1
    t0 = time.perf_counter()
    orc.update(dt, step, gap, gap)
    t_step = time.perf_counter() - t0
    step += gap
    # untimed bench steps: the GPU arm's warm-up, latency and profiled ones, so
    # that both arms time the same steps of the run
    warm, timed = max(1, args.warmup + args.latency_steps + args.profile_steps), args.steps
    fit = int(args.ref_budget / max(t_step, 1e-9)) - 1
    if warm + timed > fit + 1:  # shrink both, keeping their ratio, to fit the budget
        timed = max(1, min(timed, int(fit * args.steps / max(1, args.steps + args.warmup))))
        warm = max(1, min(warm, fit - timed + 1))
    for _ in range(warm - 1):
        orc.update(dt, step, gap, gap)
        step += gap
    t0 = time.perf_counter()
    orc.update(dt, step, timed * gap, gap)
    el = time.perf_counter() - t0
    value = updates_for(step, timed * gap, gap, nf, n_mobile) / el
    sample = (f"{timed} bench steps ({timed * gap} update() calls, steps {step}..{step + timed * gap - 1}) after "
              f"{warm} warm-up bench steps; FP64 oracle, OpenMP over particles, scene assembled by the oracle")
    if args.config == 1:
        sample += "; from the workload's initial lattice (the contact-dense start needs the GPU settle)"
    print(json.dumps({
        "metric": "particle-updates/s", "value": value, "unit": "particle-updates/s", "n_gpus": 1,
        "steps": timed, "warmup": warm, "ms_per_step": 1000.0 * el / timed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic", "config": cfg,
        "state": f"the workload's initial state, then {warm} untimed bench steps before the timed ones (the GPU "
                 "arm's warm-up, latency and profiled steps)",
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "particle-updates/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "particle-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's step exists only as CUDA kernels (and its sources are not on the GPU box); its "
                "CPU restatement, pinned to the reference compiled for the CPU, is timed on the host cores"}))


def fp64_errors(ds, scene, orc, steps, dt, gap, device, first_step=1):
    """Error of the GPU step against the FP64 oracle after the CPU sample's
    steps (from the same state): a second engine runs the same steps through
    the timed path (graph replay), and each field's largest error is taken
    over all particles, scaled as named in `scale`."""
    import numpy as np
    g = 9.81
    eng = ds.Engine(scene, device=device)
    eng.initialize()
    eng.update(dt, first_step, steps, gap, use_graph=True)
    eng.synchronize()
    t = steps * dt
    err = {}

    def rel_rows(a, b, floor):
        return float(np.max(np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), floor)))

    if scene.n_fluid:
        pos, vel, acc, drho = eng.download_fluids()
        h = float(np.ctypeslib.as_array(scene.fluid_smoothing_length, shape=(scene.n_fluid,)).min())
        v64 = orc.get("fluid.vel")
        err["fluid.pos"] = float(np.max(np.abs(pos - orc.get("fluid.pos")))) / h
        err["fluid.vel"] = float(np.max(np.abs(vel - v64))) / max(float(np.abs(v64).max()), g * t)
        err["fluid.acc"] = rel_rows(acc, orc.get("fluid.acc"), g)
        err["fluid.dRho"] = float(np.max(np.abs(drho - orc.get("fluid.dRho")))) / 1000.0
    if scene.n_solid:
        s = eng.download_solids()
        r = float(np.ctypeslib.as_array(scene.solid_radius, shape=(scene.n_solid,)).min())
        v64 = orc.get("solid.vel")
        w64 = orc.get("solid.angvel")
        err["solid.pos"] = float(np.max(np.abs(s["pos"] - orc.get("solid.pos")))) / r
        err["solid.vel"] = float(np.max(np.abs(s["vel"] - v64))) / max(float(np.abs(v64).max()), g * t)
        # a grain at rest in a bed: contact forces of many weights cancel to a
        # net ~0, so the net acceleration is scaled by sum_j |F_ij| / m_i too
        im = np.ctypeslib.as_array(scene.solid_inverse_mass, shape=(scene.n_solid,))
        fsum = np.zeros(scene.n_solid)
        f64 = orc.get("ss.force")
        if len(f64):
            fm = np.linalg.norm(f64, axis=1)
            np.add.at(fsum, orc.get("ss.pointed"), fm)
            np.add.at(fsum, orc.get("ss.pointing"), fm)
        a64 = orc.get("solid.acc")
        err["solid.acc"] = float(np.max(np.linalg.norm(s["acc"] - a64, axis=1) /
                                        np.maximum(np.linalg.norm(a64, axis=1), np.maximum(g, fsum * im))))
        err["solid.angvel"] = float(np.max(np.abs(s["angvel"] - w64))) / max(float(np.abs(w64).max()), g * t / r)
    eng.close()
    return {"steps": steps, "fields": err,
            "scale": "largest |GPU - FP64| over the particles, divided by: the smallest smoothing length (fluid.pos) "
                     "or radius (solid.pos); the largest FP64 speed or g t (vel); the FP64 value per particle, at "
                     "least g (acc: force per mass) and, for solids, at least the sum of the magnitudes of its "
                     "contact forces per mass; rho0 = 1000 (dRho); the largest FP64 spin or g t / r (angvel)"}


# ---- ranks: replicas, no exchange on the data path -------------------------------------------
def rank_total(value, how, dist=None, device="cuda"):
    """Combines one number over the ranks of a replica run: "max" for times
    (the job ends with its slowest rank), "sum" for work.  Without a process
    group it returns the value itself."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if how == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def rank_share(items, rank, world):
    """This rank's share of independent work items (scenes): every world-th one."""
    return items[rank::world]


# ---- many scenes: batched (config 3) and served (config 4) -----------------------------------
def scene_updates(scene, steps):
    nf, n_mobile, _ = mobile_counts(scene)
    return updates_for(1, steps, scene.fluid_integrate_gap, nf, n_mobile)


RECIPES_AHEAD = 24  # serving: scene recipes made ahead of their arrival


def _serving_recipe(kind, n, steps, seed):
    """A serving request's recipe (in a spawned process)."""
    import dem_sphsource_gb300.scenes as sc
    return sc.make_request(kind, n, steps, seed)


def run_many(args, world, rank, local):
    """Config 3: the batched mix through the scene server, against the same
    scenes run one at a time.  Config 4: a Poisson stream of requests served
    for --duration seconds.  Under torchrun every rank runs its own server on
    its own GPU over its share of the scenes (no exchange between ranks)."""
    ds = _package()
    import dem_sphsource_gb300.scenes as sc
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    # warm-up: one small scene (module load, pool, graph instantiation)
    _, wsc = ds.build_scene(sc.tiny_coupled())
    warm = ds.Server(device=device, workers=1)
    warm.wait(warm.submit(wsc, 10), 600.0)
    warm.close()

    budget = 150 << 30
    if args.config == 3:
        steps = args.steps if args.steps != 2000 else 1000
        recipes = rank_share(sc.batch_mix(n_scenes=args.scenes, steps=steps), rank, world)
        built = [ds.build_scene(r) for r in recipes]
        total = sum(scene_updates(s, steps) for _, s in built)

        def mix(**kw):
            srv = ds.Server(device=device, workers=args.workers, hbm_budget_bytes=budget, autotune=True, **kw)
            if dist:
                dist.barrier()
            with ClockSampler(device) as clk:
                t0 = time.perf_counter()
                for _, s in built:
                    srv.submit(s, steps)
                srv.wait(-1, -1.0)
                w = time.perf_counter() - t0
            out = srv.stats()
            srv.close()
            return rank_total(w, "max", dist), out, clk

        # the mix in one graph launch per round (demsph_batch_update), then the
        # same mix on per-scene streams with direct launches
        wall, st, clocks = mix(batch=True, batch_round_steps=args.round_steps)
        s_wall, s_st, _ = mix()
        total = rank_total(total, "sum", dist)
        # plain: a spaced sample of the same scenes, one at a time, same engine path
        k = max(1, len(built) // max(1, args.plain_scenes))
        sample = built[::k][:args.plain_scenes]
        plain = ds.Server(device=device, workers=1, hbm_budget_bytes=budget, autotune=True)
        p_upd = sum(scene_updates(s, steps) for _, s in sample)
        t1 = time.perf_counter()
        for _, s in sample:
            plain.wait(plain.submit(s, steps), -1.0)
        p_wall = time.perf_counter() - t1
        pst = plain.stats()
        plain.close()
        if rank != 0:
            return
        g_value, s_value = total / wall, total / s_wall
        value = max(g_value, s_value)  # the faster of the two batched forms
        print(json.dumps({
            "metric": "particle-updates/s", "value": value, "unit": "particle-updates/s", "n_gpus": world,
            "steps": steps, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": f"batched_mix_{args.scenes}",
                       "description": f"{args.scenes} independent scenes, 60% SPH dam breaks and 40% coupled dam "
                                      "breaks, fluid counts log-uniform in [2k, 60k], column heights uniform in "
                                      f"[0.2, 0.5] m, {steps} steps each, through the scene server",
                       "workers": args.workers, "hbm_budget_bytes": budget,
                       "batched": "value: the faster of two forms of the server - one CUDA graph launch per "
                                  "round advancing every active scene (each scene's round of about "
                                  f"{args.round_steps} steps, whole Shepard periods, is a child graph; "
                                  "demsph_batch_update; workers create engines and download results), and "
                                  "per-scene streams with 8 worker threads launching directly",
                       "autotune": "threads per fluid particle timed per size class (demsph_autotune)",
                       "timing": "host wall clock from the first submission to the last completion (engine "
                                 "creation and initialisation included)"},
            "impl": "ours", "form": "one graph launch per round" if g_value >= s_value else "per-scene streams",
            "batched": {"value": g_value, "wall_s": wall, "p50_step_ms": st["p50_step_ms"],
                                        "p99_step_ms": st["p99_step_ms"], "peak_bytes": st["peak_bytes"],
                                        "scenes": st["completed"], "worker_create_s": st["create_s"],
                                        "step_s": st["step_s"], "worker_download_s": st["download_s"],
                                        "rounds": st["batch_rounds"], "graph_builds": st["batch_graph_builds"],
                                        "capture_s": st["batch_capture_s"],
                                        "instantiate_s": st["batch_instantiate_s"],
                                        "launch_s": st["batch_launch_s"]},
            "streams": {"value": s_value, "wall_s": s_wall, "p50_step_ms": s_st["p50_step_ms"],
                        "p99_step_ms": s_st["p99_step_ms"], "scenes": s_st["completed"],
                        "how": "the same mix on per-scene streams, 8 worker threads launching directly"},
            "plain": {"value": p_upd / p_wall, "wall_s": p_wall, "scenes": len(sample),
                      "p50_step_ms": pst["p50_step_ms"], "p99_step_ms": pst["p99_step_ms"],
                      "sample": f"every {k}-th scene of the mix, one at a time"},
            "batched_over_plain": value / (p_upd / p_wall), "clocks": clocks.summary(),
            "e2e": {"value": value, "unit": "particle-updates/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None, "path": "scene arrays copied in at submission, final state "
                                                        "copied out at completion"},
        }))
        return

    # config 4: serving.  The scene recipes (the particle lattices) are made by
    # a few spawned processes up to RECIPES_AHEAD arrivals ahead; the
    # submitting thread turns each into a scene before its arrival time and
    # submits it at that time.
    import multiprocessing as mp
    arrivals = rank_share(sc.serving_stream(duration=args.duration), rank, world)
    pool = mp.get_context("spawn").Pool(max(1, min(6, (os.cpu_count() or 2) // 2)), initializer=_package)
    made = {}
    nxt = [0]  # the first arrival whose recipe is not yet asked for

    def schedule(upto):
        while nxt[0] < min(upto, len(arrivals)):
            _, kind, n, steps, seed = arrivals[nxt[0]]
            made[nxt[0]] = pool.apply_async(_serving_recipe, (kind, n, steps, seed))
            nxt[0] += 1

    lag = []
    schedule(RECIPES_AHEAD)
    for k in range(min(RECIPES_AHEAD, len(arrivals))):
        made[k].wait()
    srv = ds.Server(device=device, workers=args.workers, hbm_budget_bytes=budget, autotune=True)
    if dist:
        dist.barrier()
    submitted = 0
    with ClockSampler(device) as clocks:
        t0 = time.perf_counter()
        for k, (ta, kind, n, steps, seed) in enumerate(arrivals):
            _, s = ds.build_scene(made.pop(k).get())
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            srv.submit(s, steps)
            submitted += 1
            lag.append(time.perf_counter() - t0 - ta)
            schedule(k + 1 + RECIPES_AHEAD)
        window = time.perf_counter() - t0
        st = srv.stats()
    pool.terminate()
    srv.close()  # requests still queued or running are dropped
    upd = rank_total(st["particle_updates"], "sum", dist)
    window = rank_total(window, "max", dist)
    if rank != 0:
        return
    lag.sort()
    print(json.dumps({
        "metric": "particle-updates/s", "value": upd / window, "unit": "particle-updates/s", "n_gpus": world,
        "steps": None, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "serving_stream",
                   "description": f"Poisson arrivals at 20/s for {args.duration:g} s (the workload names 300 s); "
                                  "SPH, DEM and coupled scenes in equal shares, sizes log-uniform in [5k, 500k], "
                                  "steps uniform in [200, 5000]; 150 GiB admission budget",
                   "workers": args.workers,
                   "graphs": "a scene replays CUDA graphs only while it is the only active one"},
        "impl": "ours",
        "serving": {"submitted": submitted, "admitted": st["admitted"], "completed": st["completed"],
                    "p50_step_ms": st["p50_step_ms"], "p99_step_ms": st["p99_step_ms"],
                    "peak_bytes": st["peak_bytes"], "window_s": window,
                    "submit_lag_p99_s": lag[int(0.99 * (len(lag) - 1))] if lag else None},
        "clocks": clocks.summary(),
        "e2e": {"value": upd / window, "unit": "particle-updates/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None},
    }))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed bench steps (fluid periods)")
    ap.add_argument("--warmup", type=int, default=5, help="untimed bench steps before the timed ones")
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", type=int, choices=(0, 1, 2, 3, 4), default=2)
    ap.add_argument("--settle-steps", type=int, default=None,
                    help="config 1: untimed settle steps before the warm-up (default 200000)")
    ap.add_argument("--scenes", type=int, default=256, help="batched workload: number of scenes")
    ap.add_argument("--plain-scenes", type=int, default=32,
                    help="batched workload: scenes (evenly spaced in the list) also run one at a time")
    ap.add_argument("--duration", type=float, default=60.0, help="serving workload: seconds of arrivals")
    ap.add_argument("--workers", type=int, default=8, help="batched/serving: server worker threads")
    ap.add_argument("--round-steps", type=int, default=20, help="batched workload: steps per scene and round")
    ap.add_argument("--e2e-steps", type=int, default=10, help="bench steps of the end-to-end leg")
    ap.add_argument("--latency-steps", type=int, default=20, help="bench steps timed one by one for p50/p99")
    ap.add_argument("--profile-steps", type=int, default=10,
                    help="bench steps of the per-stage timing pass, in one call (10: two Shepard "
                         "re-initialisation periods, so the stage shares weigh it as the timed region does, and "
                         "runs of plain DEM steps split into the timed region's 10-step runs)")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU-baseline stepping")
    ap.add_argument("--ref-budget", type=float, default=300.0, help="reference arm: seconds of stepping at most")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--save-state", default=None, help="config 1: writes the settled bed (.npz) for --load-state")
    ap.add_argument("--load-state", default=None,
                    help="starts from a state written by --save-state instead of settling (for profiling runs)")
    ap.add_argument("--clock-tail", type=float, default=1.0,
                    help="seconds of the same bench steps replayed after the timed region so that the clock sampler "
                         "sees the load (0 for a run under a profiler)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.config in (3, 4):
        return run_many(args, world, rank, local)
    if args.impl == "reference":
        return reference_arm(args, rank)

    ds = _package()
    import numpy as np
    import torch

    recipe = make_recipe(args.config)
    builder, scene = ds.build_scene(recipe)
    dt, gap = scene.time_step, scene.fluid_integrate_gap
    nf, n_mobile, n_dummy = mobile_counts(scene)
    settle = args.settle_steps if args.settle_steps is not None else SETTLE_STEPS.get(args.config, 0)
    cfg = workload_config(args.config, scene, args, settle)

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = local if world > 1 else 0
    torch.cuda.set_device(device)

    step = 1
    state0 = None
    if args.load_state:
        # a state saved by --save-state (the settled bed): the engine starts
        # from it (contact and wall springs from zero, as at any start)
        z = np.load(args.load_state)
        state0 = {k: z[k] for k in z.files if k != "step"}
        step = int(z["step"])
        restart_scene(scene, state0)
        settle = 0
    eng = ds.Engine(scene, device=device)
    eng.initialize()
    if settle:
        # the settle itself, untimed, up to a contact-dense bed; its state is
        # the start of the CPU baseline and of the FP64 comparison
        eng.update(dt, step, settle, gap, use_graph=True)
        step += settle
        eng.synchronize()
        state0 = engine_state(eng)
        if args.save_state:
            np.savez(args.save_state, step=step, **state0)
    first_sample_step = step
    eng.update(dt, step, args.warmup * gap, gap, use_graph=True)
    step += args.warmup * gap
    eng.synchronize()

    stream = torch.cuda.ExternalStream(eng.stream_ptr(), device=device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # ---- latency, then the stage timing, right before the timed region (the
    # same phase of the run: the clock tail after the timed region advances the
    # scene by up to a second of steps) ----
    # latency: bench steps one by one (graph replay), CUDA events on the engine stream
    lat = []
    for _ in range(max(1, args.latency_steps)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.update(dt, step, gap, gap, use_graph=True)
        e1.record(stream)
        e1.synchronize()
        lat.append(e0.elapsed_time(e1))
        step += gap
    lat.sort()

    # ---- stage timing pass for the roofline: the graphs' own launches (the
    # fused runs of the timed region) issued directly, CUDA events per stage ----
    eng.set_profiling(True)
    eng.profile_report()
    # (one call: the runs of plain DEM steps are split as in the timed region's call)
    eng.update(dt, step, max(1, args.profile_steps) * gap, gap, use_graph=True)
    step += max(1, args.profile_steps) * gap
    eng.synchronize()
    stages = eng.profile_report()
    eng.set_profiling(False)
    c = eng.counts()
    shapes = eng.launch_shapes()
    eng.synchronize()
    launches0 = eng.kernel_launches()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(device) as clocks:
        ev0.record(stream)
        eng.update(dt, step, args.steps * gap, gap, use_graph=True)
        ev1.record(stream)
        ev1.synchronize()
        clocks.mark_end()
        launches = eng.kernel_launches() - launches0
        # keep the GPU under the same load for a moment so the clock sampler
        # (nvidia-smi, 20 ms period at best) sees it when the timed region is short
        t_end = time.perf_counter() + args.clock_tail
        tail = step + args.steps * gap
        while time.perf_counter() < t_end:
            eng.update(dt, tail, gap, gap, use_graph=True)
            eng.synchronize()
            tail += gap
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    updates = updates_for(step, args.steps * gap, gap, nf, n_mobile)
    step = tail
    ms = rank_total(ms, "max", dist)
    updates = rank_total(updates, "sum", dist)
    value = updates / (ms / 1000.0)
    # the clock-tail steps launched kernels too; only the timed region's count is claimed
    launches_tail = eng.kernel_launches() - launches0 - launches

    counts = {"solid_pairs": c.solid_pairs, "n_solid": scene.n_solid, "n_solid_active": n_mobile,
              "n_fluid": nf, "bonds": c.bonds,
              "fluid_partners": 2.0 * c.fluid_pairs / max(nf, 1), "fluid_solid_partners": c.fluid_solid_pairs / max(nf, 1),
              "n_pebbles": 4 * scene.n_clump, "tiles": shapes.get("fluid_bit_lists", 0) > 0}
    if counts["tiles"]:
        # a particle's walk candidates: 27 cells of cell volume / particle volume
        # (a fluid particle's volume is (h / 1.3)^3, its mass rho0 (h / 1.3)^3)
        h = float(np.ctypeslib.as_array(scene.fluid_smoothing_length, shape=(nf,))[0])
        per_cell = c.cell_size[0] * c.cell_size[1] * c.cell_size[2] / (h / 1.3) ** 3
        counts["bit_words"] = math.ceil(27.0 * per_cell / 32.0)
    dom = max(stages.items(), key=lambda kv: kv[1][1]) if stages else None
    peak, peak_kind = load_peaks()
    roofline = None
    if dom:
        name, (n_launch, tot_ms) = dom
        avg_ms = tot_ms / max(n_launch, 1)
        alg = stage_bytes(name, counts)
        achieved = alg / (avg_ms / 1000.0) / 1e9 if alg else None
        tr = load_traffic(name, cfg["workload"])
        traffic = None
        if tr and tr.get("bytes_per_unit") is not None:
            traffic = tr["bytes_per_unit"] * counts.get(tr.get("unit_count", "solid_pairs"), 0)
        total_ms = sum(v[1] for v in stages.values())
        roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                    "traffic_source": tr.get("source") if tr else None,
                    "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                    "fallback 6.8 TB/s", "avg_launch_ms": avg_ms, "algorithmic_bytes_per_launch": alg,
                    "stage_share": {k: round(v[1] / total_ms, 4) for k, v in sorted(stages.items(),
                                                                                     key=lambda kv: -kv[1][1])}}
        # the fluid pair loops against the FP32 issue rate they are bound by
        sph = [(k, v) for k, v in stages.items() if k in PAIR_FLOPS and v[0] > 0]
        if sph and rank == 0:
            k, (n_launch, tot) = max(sph, key=lambda kv: kv[1][1])
            fl = stage_flops(k, counts)
            peak32 = fp32_peak_tflops(torch)
            ach = fl / (tot / n_launch / 1000.0) / 1e12 if fl else None
            roofline["fp32"] = {"kernel": k, "achieved": ach, "peak": peak32, "unit": "TFLOP/s",
                                "frac": (ach / peak32) if ach and peak32 else None,
                                "flops_per_pair": PAIR_FLOPS[k], "flops_per_launch": fl,
                                "peak_source": "measured here: cuBLAS SGEMM 8192^3, TF32 off"}

    # ---- end to end through the C ABI with host buffers ----
    ne = max(1, args.e2e_steps)
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    bi = bo = 0
    if scene.n_solid:
        sp, sv, sw = pin((scene.n_solid, 3)), pin((scene.n_solid, 3)), pin((scene.n_solid, 3))
        eng.download_solids(out={"pos": sp, "vel": sv, "angvel": sw})
        bi += 3 * sp.nbytes
        bo += 3 * sp.nbytes
    if nf:
        fp, fv, fd = pin((nf, 3)), pin((nf, 3)), pin((nf,))
        eng.download_fluids(out=(fp, fv, None, fd))
        bi += fp.nbytes + fv.nbytes + fd.nbytes
        bo += fp.nbytes + fv.nbytes + fd.nbytes
    torch.cuda.synchronize()
    s_io = (sp, sv, sw) if scene.n_solid else None
    f_io = (fp, fv, fd) if nf else None
    e2e_first = step
    t0 = time.perf_counter()
    for k in range(ne):
        # upload the state, one bench step, download the state: one C-ABI call, one synchronisation
        eng.update_io(dt, step, gap, gap, use_graph=True, fluid_in=f_io, solid_in=s_io, fluid_out=f_io,
                      solid_out=s_io)
        step += gap
    e2e_s = time.perf_counter() - t0
    e2e_updates = updates_for(e2e_first, ne * gap, gap, nf, n_mobile)
    e2e_val = e2e_updates / e2e_s
    if dist:
        e2e_val = e2e_updates * world / rank_total(e2e_s, "max", dist)
    live_contacts = eng.counts().solid_pairs

    cb = err64 = None
    if rank == 0 and not args.no_cpu:
        cb, orc, orc_steps, asm = cpu_baseline(recipe, state0, args.cpu_budget, first_sample_step)
        if state0 is not None:
            restart_scene(scene, state0)  # the second engine starts where the oracle started
        err64 = fp64_errors(ds, scene, orc, orc_steps, dt, gap, device, first_sample_step)
        del orc, asm

    if rank == 0:
        out = {
            "metric": "particle-updates/s", "value": value, "unit": "particle-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic", "config": cfg, "state": workload_state(args, settle), "impl": "ours",
            "p50_step_ms": lat[len(lat) // 2],
            "p99_step_ms": lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)],
            "roofline": roofline, "cpu_baseline": cb, "fp64_error": err64,
            "e2e": {"value": e2e_val, "unit": "particle-updates/s", "h2d_bytes_per_step": bi,
                    "d2h_bytes_per_step": bo, "steps": ne,
                    "path": "demsph_update_io per bench step: upload the state, the step's update() calls, download "
                            "the state, one synchronisation; pinned host buffers, FP64 reference layout"},
            "gpu_launches": launches, "clocks": clocks.summary(),
            "details": {"solid_pairs_live": live_contacts, "solid_pairs_per_mobile_solid":
                        live_contacts / max(n_mobile, 1), "fluid_pairs_half": c.fluid_pairs,
                        "fluid_solid_pairs": c.fluid_solid_pairs, "bonds": c.bonds,
                        "launch_shapes": eng.launch_shapes(), "clock_tail_launches": launches_tail,
                        "timing": "CUDA events on the engine stream around K bench steps replayed as CUDA graphs; "
                                  "p50/p99 from bench steps timed one by one",
                        "precision": "FP32 arithmetic with Kahan sums; double-float positions, velocities, overlaps, "
                                     "bond accumulators and clump states; FP64 clump orientation"},
        }
        print(json.dumps(out))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    eng.close()


if __name__ == "__main__":
    main()
