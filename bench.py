#!/usr/bin/env python3
"""Throughput of the GB300 simulation step (pkg/fluid Simulate) on the
2048x2048 lid-driven cavity.

Workload (one "step" = one Simulate call): 2048x2048 interior cells, density
1, h = 1, dt = 0.1, closed box, lid source row U = 1.0 under the top wall
(the app's cavity preset, without its smoke), BFECC advection on, the
New() default turbulence 0.02, 200 Jacobi pressure sweeps per step run in
temporal blocks of 8 sweeps per launch, FP64 residual reduction and one FP64
outer correction of 8 sweeps, fixed sweep count (no early exit), advection
departure points formed relative to their face (precise_coords).  Fields are
FP32; inputs are synthetic (zero initial state, seeded scene).

Arms:
  (default)          the CUDA path.  `value` is device-timed with CUDA events
                     on the library's stream, the lid held by device-resident
                     sources; `e2e` drives the same workload through the C ABI
                     from the host: per step the lid edits are uploaded, the
                     step runs and the smoke field is read back.
  --impl reference   the reference's CPU algorithm (serial lexicographic SOR
                     pressure, FP32) restated in C++, on the host cores.

Metric: Mcell-steps/s = 2048 * 2048 * steps / seconds / 1e6.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s fwd at 2048^2 (lid-driven cavity, BFECC, 200 Jacobi sweeps)"
W = H = 2048
DT = 0.1
ITERS = 200
TB = 8
REFINE = 8
# Algorithmic bytes per cell per Jacobi sweep (phi read + write, rhs, 1-byte mask).
JACOBI_BYTES_PER_CELL_SWEEP = 13
# Compulsory bytes per cell of one 8-sweep phase run in registers: phi read and
# written, w and w*b read once.
JACOBI_BYTES_PER_CELL_PHASE = 16
FALLBACK_HBM_GBS = 6800.0
# Compulsory bytes per cell of each stage of the headline step (each pass
# reads each of its inputs once and writes each output once; FP32 fields,
# 1-byte flags).  Keys are the step's profiled stages.
STAGE_BYTES_PER_CELL = {
    "sources+viscosity": 0,            # lid cells only; viscosity off
    "pressure setup": 21,              # U, V, flags -> b, w, w*b
    "jacobi sweeps": JACOBI_BYTES_PER_CELL_PHASE * ITERS // TB,  # 25 phases
    "outer correction": 17,            # phi, w, b, flags -> e (one launch of 8 sweeps)
    "gradient+div stats": 45,          # U, V, phi, e, b, flags, noise -> U, V, p
    "confinement/turbulence+borders": 0,  # confinement off, turbulence fused; perimeter only
    "advect velocity": 59,             # BFECC: fwd 17 + bwd/correct/clamp 25 + final 17
    "advect smoke+mass": 55,           # BFECC: 17 + 21 + 17
}


def workload_config(extra=None):
    cfg = {
        "workload": "lid-driven cavity 2048x2048, BFECC, turbulence 0.02, 200 Jacobi sweeps "
                    "(temporal blocks of 8), FP64 residual + 8-sweep FP64 outer correction, "
                    "face-relative departure points",
        "grid": [W, H],
        "dt": DT,
        "pressure_sweeps": ITERS,
        "tb_depth": TB,
        "refine_sweeps": REFINE,
        "l2": "per-step working set ~250 MB of fields > 129 MB L2; no flush between steps",
    }
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def committed_traffic():
    """DRAM bytes per Jacobi launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "jacobi_tb_traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None


def max_over_ranks(ms, device):
    """Max of a per-rank time over the process group (the slowest replica
    sets the job time)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, steps, t_max_ms, cells=W * H):
    """Whole-job Mcell-steps/s of `world` replicas of `steps` steps each."""
    return world * cells * steps / (t_max_ms / 1e3) / 1e6


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def build_cavity(fluid_gb300, auto_sync=False):
    f = fluid_gb300.Fluid(1.0, W, H, 1.0, auto_sync=auto_sync, scheme=fluid_gb300.SCHEME_JACOBI,
                          num_iters=ITERS, tb_depth=TB, refine_sweeps=REFINE, UseBFECC=True,
                          early_exit=False, precise_coords=True)
    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0
    f.mark_dirty(1 << fluid_gb300.FIELDS["S"])
    return f


def lid_cells(f):
    import numpy as np

    i = np.arange(2, f.NumX - 2, dtype=np.int32)
    j = np.full_like(i, f.NumY - 2)
    return i, j


def profile_leg(args, name):
    """With --profile-leg NAME, brackets that leg's timed region with
    cudaProfilerStart/Stop (for ncu --profile-from-start off); returns the
    closing call."""
    import torch

    if getattr(args, "profile_leg", None) != name:
        return lambda: None
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()

    def stop():
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStop()

    return stop


def jacobi_roofline(n_cells, phase_ms, peak, peak_kind, tr, clocks):
    """Roofline of the dominant kernel, k_jacobi_flow, per 8-sweep phase.

    `achieved` counts the phase's compulsory bytes: an 8-sweep phase run in
    registers must read phi, w and w*b and write phi once (16 B per cell),
    over the phase's CUDA-event time.  The solve's arrays stay in L2 across
    phases, so the DRAM traffic ncu measures (`traffic`) is below that, and
    the kernel's binding limit is instruction issue: `issue` compares the
    phase's warp instructions (ncu) with what 4 schedulers per SM issue at the
    sampled SM clock.  The per-sweep model (13 B per cell and sweep, every
    sweep of the phase counted) is kept beside it."""
    sec = phase_ms / 1e3
    comp = JACOBI_BYTES_PER_CELL_PHASE * n_cells
    model = JACOBI_BYTES_PER_CELL_SWEEP * TB * n_cells
    achieved = comp / sec / 1e9
    out = {
        "kernel": "k_jacobi_flow (one cooperative launch per solve: 25 phases of 8 sweeps; "
                  "figures per phase)",
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak,
        "peak_source": peak_kind + " MEASURED_PEAKS.json hbm_gbs" if peak_kind == "measured"
        else "fallback 6.8 TB/s",
        "bytes_per_launch": comp, "launch_ms": phase_ms,
        "traffic": tr.get("dram_bytes_per_launch_full") if tr else None,
        "traffic_source": tr.get("source") if tr else None,
        "model": "compulsory bytes of an 8-sweep phase run in registers: phi read and written, "
                 "w and w*b read (16 B per cell)",
        "per_sweep_model": {"bytes_per_launch": model, "achieved": model / sec / 1e9,
                            "ratio_to_peak": model / sec / 1e9 / peak,
                            "model": "13 B per cell-sweep (phi r/w 8, rhs 4, mask 1), all 8 "
                                     "sweeps of the phase counted; the sweeps run in registers, "
                                     "so this exceeds the HBM peak"},
    }
    inst = tr.get("warp_inst_per_phase") if tr else None
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if inst and mhz:
        sms = tr.get("sms", 152)
        peak_inst = sms * 4 * mhz * 1e6  # one warp instruction per scheduler per clock
        out["issue"] = {"warp_inst_per_phase": inst, "achieved_warp_inst_per_s": inst / sec,
                        "peak_warp_inst_per_s": peak_inst, "frac": inst / sec / peak_inst,
                        "source": tr.get("inst_source")}
    return out


def step_roofline(stage_ms, n_cells, ms_per_step, peak):
    """The whole step against HBM: the compulsory bytes of every stage
    (STAGE_BYTES_PER_CELL) over the device-timed step, and each stage's
    bytes over its own profiled time."""
    per_cell = sum(STAGE_BYTES_PER_CELL.values())
    total = per_cell * n_cells
    achieved = total / (ms_per_step / 1e3) / 1e9
    stages = {}
    for name, ms in stage_ms.items():
        b = STAGE_BYTES_PER_CELL.get(name)
        if b and ms > 0:
            gbs = b * n_cells / (ms / 1e3) / 1e9
            stages[name] = {"bytes_per_cell": b, "ms": ms, "gbs": gbs, "frac": gbs / peak}
    return {"bytes_per_cell": per_cell, "bytes_per_step": total, "ms_per_step": ms_per_step,
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "stages": stages}


def fp64_error(f):
    """One step of the FP64 oracle from the GPU's current state beside the
    GPU's own step: velocity max-abs error relative to max |U|, and the two
    post-projection divergence L2 norms."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes
    from oracle.pyoracle import OracleFluid

    o = OracleFluid(1.0, W, H, 1.0, prec=64, threads=os.cpu_count() or 1, scheme=1,
                    num_iters=ITERS, check_every=TB, UseBFECC=True, early_exit=False,
                    refine_sweeps=REFINE, precise_coords=True)
    f.synchronize()
    f.download()
    for k in ("U", "V", "M", "newU", "newV", "newM", "S"):
        getattr(o, k)[:] = getattr(f, k)
    f.Simulate(DT)
    scenes.cavity_lid(o)
    o.Simulate(DT)
    f.synchronize()
    f.download()
    scale = float(np.abs(o.U).max())
    err = max(float(np.abs(f.U.astype(np.float64) - o.U).max()),
              float(np.abs(f.V.astype(np.float64) - o.V).max())) / scale
    dg, do = f.stats()["div_l2_post"], o.stats()["div_l2_post"]
    return {"vel_maxabs_rel": err, "div_l2_post_gpu": dg, "div_l2_post_fp64": do,
            "div_l2_abs_diff": abs(dg - do), "bound": {"vel_maxabs_rel": 1e-4, "div_l2": 1e-5},
            "how": "after the timed steps the FP64 oracle is set to the GPU's state and both "
                   "take one step; tests/test_gpu_headline.py asserts the bounds every 100 "
                   "steps over 500"}


def config_rows(fluid_gb300, threads):
    """The two smaller configurations, each against its CPU port: the 128^2
    jet (walls left, top and bottom; 8-row jet U = 2 with smoke 1; BFECC and
    confinement off; 40 iterations) and the 512x256 Karman street (disc
    r = 24, inflow U = 1, BFECC, confinement 0.3, 100 Jacobi sweeps)."""
    import numpy as np
    import torch
    from oracle.pyoracle import LEXSOR, OracleFluid

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes

    rows = {}
    # Config 1: the reference scheme bit for bit, and the Jacobi scheme.
    for key, params in (("jet128_reference_sor", dict(num_iters=40)),
                        ("jet128_jacobi", dict(scheme=fluid_gb300.SCHEME_JACOBI, num_iters=40,
                                               tb_depth=8, early_exit=False))):
        f = fluid_gb300.Fluid(1.0, 128, 128, 1.0, auto_sync=False, **params)
        jet_setup(f)
        st = torch.cuda.ExternalStream(f.stream)
        for _ in range(3):
            f.Simulate(DT)
        ms = device_ms(st, lambda: f.Simulate(DT), 200)
        rows[key] = {"value": 128 * 128 / ms / 1e3, "unit": "Mcell-steps/s", "ms_per_step": ms,
                     "steps": 200}
        del f
    o = OracleFluid(1.0, 128, 128, 1.0, prec=32, threads=threads, scheme=LEXSOR, num_iters=40)
    scenes.jet_scene(o)
    for _ in range(3):
        scenes.jet_inject(o)
        o.Simulate(DT)
    t0 = time.perf_counter()
    for _ in range(200):
        scenes.jet_inject(o)
        o.Simulate(DT)
    sec = (time.perf_counter() - t0) / 200
    cpu1 = {"value": 128 * 128 / sec / 1e6, "unit": "Mcell-steps/s", "cores": threads,
            "kind": "port", "sample": "200 steps after 3 warm-up steps (reference SOR, 40 "
                                      "iterations with early exit; jet edits on the host)"}
    rows["jet128_reference_sor"]["cpu_baseline"] = cpu1
    rows["jet128_jacobi"]["cpu_baseline"] = cpu1
    rows["jet128_reference_sor"]["config"] = ("128x128 jet (config 1): reference lexicographic SOR "
                                              "bit for bit, 40 iterations with early exit, jet "
                                              "held by device sources; device-timed")
    rows["jet128_jacobi"]["config"] = ("128x128 jet (config 1) with the Jacobi scheme, 40 fixed "
                                       "sweeps; device-timed")
    # Config 2: Karman street.
    kw = dict(scheme=fluid_gb300.SCHEME_JACOBI, num_iters=100, tb_depth=4, early_exit=False,
              UseBFECC=True, Confinement=0.3)
    g = fluid_gb300.Fluid(1.0, 512, 256, 1.0, auto_sync=False, **kw)
    scenes.fast_walls(g, top=True, bottom=True, left=False, right=False)
    g.mark_dirty()
    g.SetCircularObstacle(128, 128, 24)
    g.download()
    rng = np.random.default_rng(2)
    U0 = ((1.0 + rng.uniform(-1e-3, 1e-3, g.numCells)) * (g.S != 0)).reshape(g.NumX, g.NumY)
    U0[0, :] = 0.0
    U0[:, 0] = U0[:, -1] = 0.0
    g.U[:] = U0.ravel()
    g.mark_dirty()
    S0 = g.S.copy()
    rr = np.arange(1, g.NumY - 1, dtype=np.int32)
    g.set_sources(np.ones_like(rr), rr, u=1.0, v=0.0, mode=g.SRC_SKIP_SOLID | g.SRC_SET_VELOCITY)
    st = torch.cuda.ExternalStream(g.stream)
    for _ in range(3):
        g.Simulate(DT)
    ms = device_ms(st, lambda: g.Simulate(DT), 200)
    rows["karman512x256_jacobi"] = {
        "value": 512 * 256 / ms / 1e3, "unit": "Mcell-steps/s", "ms_per_step": ms, "steps": 200,
        "config": "512x256 Karman street (config 2): disc r 24 at (128, 128), inflow U = 1, "
                  "BFECC, confinement 0.3, 100 Jacobi sweeps (blocks of 4); device-timed"}
    del g
    o = OracleFluid(1.0, 512, 256, 1.0, prec=32, threads=threads, scheme=LEXSOR, num_iters=100,
                    UseBFECC=True, Confinement=0.3)
    o.S[:] = S0
    o.U[:] = U0.ravel()
    for _ in range(2):
        scenes.karman_inflow(o)
        o.Simulate(DT)
    t0 = time.perf_counter()
    n = 5
    for _ in range(n):
        scenes.karman_inflow(o)
        o.Simulate(DT)
    sec = (time.perf_counter() - t0) / n
    rows["karman512x256_jacobi"]["cpu_baseline"] = {
        "value": 512 * 256 / sec / 1e6, "unit": "Mcell-steps/s", "cores": threads, "kind": "port",
        "sample": "%d steps after 2 warm-up steps (reference SOR, 100 iterations with the "
                  "reference's early exit, other stages on %d threads)" % (n, threads)}
    return rows


def multigrid_leg(fluid_gb300, f, args):
    """The headline cavity with the MULTIGRID pressure scheme (parallel
    V(2,2) cycles) in place of the 200 Jacobi sweeps and the outer
    correction: device-timed steps for 1 and 2 cycles from the main handle's
    state, and, from one snapshot of that state, one step of each scheme
    with its FP64-class pressure residual (resid_l2) and post-projection
    divergence."""
    import torch

    f.synchronize()
    f.download()
    snap = {k: getattr(f, k).copy() for k in ("U", "V", "M", "newU", "newV", "newM")}

    def load(h):
        for k, v in snap.items():
            getattr(h, k)[:] = v
        h.mark_dirty()

    out = {}
    for cycles in (1, 2):
        g = fluid_gb300.Fluid(1.0, W, H, 1.0, auto_sync=False, scheme=fluid_gb300.SCHEME_MULTIGRID,
                              num_iters=cycles, UseBFECC=True, early_exit=False,
                              precise_coords=True)
        S = g.S.reshape(g.NumX, g.NumY)
        S[:] = 1.0
        S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0
        load(g)
        li, lj = lid_cells(g)
        g.set_sources(li, lj, u=1.0, v=0.0, mode=g.SRC_SKIP_SOLID | g.SRC_SET_VELOCITY)
        g.Simulate(DT)  # the step from the snapshot
        st = g.stats()
        stream = torch.cuda.ExternalStream(g.stream)
        for _ in range(max(3, args.warmup)):
            g.Simulate(DT)
        l0 = g.launch_count()
        prof = profile_leg(args, "multigrid")
        ms = device_ms(stream, lambda: g.Simulate(DT), args.steps)
        prof()
        launches = (g.launch_count() - l0) / args.steps
        out["cycles_%d" % cycles] = {
            "value": W * H / ms / 1e3, "unit": "Mcell-steps/s", "ms_per_step": ms,
            "launches_per_step": launches, "resid_l2": st["resid_l2"],
            "div_l2_post": st["div_l2_post"]}
        del g
    load(f)
    f.Simulate(DT)
    st = f.stats()
    out["jacobi_200_refined"] = {"resid_l2": st["resid_l2"], "div_l2_post": st["div_l2_post"]}
    out["config"] = ("2048^2 cavity as the headline (BFECC, turbulence, face-relative departures), "
                     "pressure by MULTIGRID: V(2,2) cycles, damped Jacobi (0.8), levels down to a "
                     "side of 8; residuals compared on one step from the same snapshot against "
                     "the headline's 200 sweeps + 8-sweep correction; device-timed steps")
    return out


def fwd_adjoint(fluid_gb300, args):
    """Forward + adjoint rollout on the cavity with the headline step's
    settings (outer correction and face-relative departure points included):
    ROLL steps with a device-resident per-step force field, checkpoint every
    8 steps, loss ||M_T - target||_2, gradients w.r.t. the initial state and
    every step's forces.  Returns per-step times of the rollout (forward +
    recompute + adjoint) and of plain forward steps of the same
    configuration, both device-timed with CUDA events."""
    import numpy as np
    import torch

    roll, every = 16, 8
    f = build_cavity(fluid_gb300)
    li, lj = lid_cells(f)
    f.set_sources(li, lj, u=1.0, v=0.0, smoke=1.0,
                  mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY | f.SRC_ADD_SMOKE)
    stream = torch.cuda.ExternalStream(f.stream)
    n = f.numCells
    gen = torch.Generator(device="cuda").manual_seed(4)
    forces = (torch.rand((roll, 2, n), device="cuda", generator=gen) - 0.5) * 0.01
    ii = torch.arange(f.NumX, device="cuda", dtype=torch.float32)[:, None]
    jj = torch.arange(f.NumY, device="cuda", dtype=torch.float32)[None, :]
    target = torch.zeros((f.NumX, f.NumY), device="cuda")
    rng = np.random.default_rng(4)
    for _ in range(4):
        s, a = rng.uniform(10, 30), rng.uniform(0.5, 1.0)
        ci, cj = rng.uniform(1, f.NumX - 1), rng.uniform(1, f.NumY - 1)
        target += a * torch.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) / (2 * s * s))
    target = target.reshape(-1).contiguous()
    gfu = torch.empty((roll, n), device="cuda")
    gfv = torch.empty((roll, n), device="cuda")
    torch.cuda.synchronize()
    for _ in range(8):  # spin up the flow so the rollout starts from a moving state
        f.Simulate(DT)
    f.synchronize()

    def rollout():
        f.tape_begin(roll, every)
        for t in range(roll):
            f.step_forward(DT, forces[t, 0], forces[t, 1])
        loss = f.tape_seed_smoke_l2(target)
        for t in reversed(range(roll)):
            f.step_adjoint(gfu[t], gfv[t])
        f.tape_end()
        return loss

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    rollout()
    f.synchronize()
    reps = max(2, min(5, args.steps // 4))
    prof = profile_leg(args, "adjoint")
    e0.record(stream)
    for _ in range(reps):
        loss = rollout()
    e1.record(stream)
    f.synchronize()
    prof()
    ms_roll = e0.elapsed_time(e1) / (reps * roll)
    l0 = f.launch_count()
    e0.record(stream)
    for _ in range(roll):
        f.Simulate(DT)
    e1.record(stream)
    f.synchronize()
    ms_fwd = e0.elapsed_time(e1) / roll
    return {
        "metric": "Mcell-steps/s fwd+adjoint at 2048^2",
        "value": W * H / ms_roll / 1e3, "unit": "Mcell-steps/s", "ms_per_step": ms_roll,
        "fwd_ms_per_step": ms_fwd, "ratio_to_fwd": ms_roll / ms_fwd,
        "rollout_steps": roll, "checkpoint_every": every, "loss": loss,
        "config": "cavity 2048x2048 as above (outer correction included) with +1 smoke on "
                  "the lid row; per-step 2-channel force field on the device; one rollout = %d "
                  "recorded steps + seed + %d adjoint steps (the first %d steps recomputed "
                  "from their checkpoint); gradients w.r.t. the initial state and all forces; "
                  "%d rollouts timed" % (roll, roll, roll - every, reps),
        "checks": "tests/test_gpu_adjoint.py: FP64 central differences of the oracle "
                  "(with the outer correction: test_directional_derivative_with_outer_correction)",
        "fwd_launches_per_step": (f.launch_count() - l0) / roll,
    }


def rollout256(fluid_gb300, args):
    """The differentiable-rollout configuration: 256^2 jet (walls left, top,
    bottom; 8-row jet at U = 2 with smoke assigned to 1 before every step),
    FP32, 64 steps, BFECC, 60 Jacobi sweeps, checkpoint every 8, loss
    ||M_64 - target||_2 against 4 seeded Gaussian blobs (sigma 10-30 cells,
    amplitude 0.5-1.0), gradients w.r.t. U0, V0 and the 64 two-channel force
    fields.  Device-timed fwd+adjoint per step, and the adjoint's directional
    derivatives against central differences (eps 1e-3) of the FP32 forward
    pass on 32 seeded directions."""
    import numpy as np
    import torch

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes

    side, steps, iters, every = 256, 64, 60, 8
    f = fluid_gb300.Fluid(1.0, side, side, 1.0, auto_sync=False, scheme=1, num_iters=iters,
                          tb_depth=8, early_exit=False, UseBFECC=True)
    scenes.jet_rollout_scene(f)
    n = f.numCells
    target = torch.from_numpy(scenes.gaussian_target(f.NumX, f.NumY, seed=4)).cuda()
    gfu = torch.empty((steps, n), device="cuda")
    gfv = torch.empty((steps, n), device="cuda")
    dforce = torch.empty((steps, 2, n), device="cuda")
    stream = torch.cuda.ExternalStream(f.stream)
    torch.cuda.synchronize()

    def prep(dU=None, dV=None, s=0.0):
        f.Reset()
        f.download()
        if dU is not None:
            f.U[:] = s * dU
            f.V[:] = s * dV
            f.mark_dirty(3)
            fp = dforce * s
        else:
            fp = torch.zeros((steps, 2, n), device="cuda")
        torch.cuda.synchronize()
        return fp

    def run(fp, grads=True):
        f.tape_begin(steps, every)
        for t in range(steps):
            f.step_forward(DT, fp[t, 0], fp[t, 1])
        loss = f.tape_seed_smoke_l2(target)
        if grads:
            for t in reversed(range(steps)):
                f.step_adjoint(gfu[t], gfv[t])
        return loss

    run(prep())
    f.tape_end()
    fp = prep()
    f.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    loss = run(fp)
    e1.record(stream)
    f.synchronize()
    ms = e0.elapsed_time(e1) / steps
    g = f.tape_grad()
    f.tape_end()
    gu = (gfu.double().cpu().numpy(), gfv.double().cpu().numpy())
    prep()
    f.synchronize()
    e0.record(stream)
    for _ in range(steps):
        f.Simulate(DT)
    e1.record(stream)
    f.synchronize()
    ms_fwd = e0.elapsed_time(e1) / steps
    rel = []
    for k in range(32):
        rng = np.random.default_rng(4000 + k)
        dU = rng.standard_normal(n).astype(np.float32)
        dV = rng.standard_normal(n).astype(np.float32)
        df = rng.standard_normal((steps, 2, n)).astype(np.float32) * 0.1
        dforce.copy_(torch.from_numpy(df))
        torch.cuda.synchronize()
        ad = float(np.dot(g["U"].astype(np.float64), dU) + np.dot(g["V"].astype(np.float64), dV)
                   + np.sum(gu[0] * df[:, 0]) + np.sum(gu[1] * df[:, 1]))
        eps = 1e-3
        lp = run(prep(dU, dV, eps), grads=False)
        f.tape_end()
        lm = run(prep(dU, dV, -eps), grads=False)
        f.tape_end()
        fd = (lp - lm) / (2 * eps)
        rel.append(abs(ad - fd) / max(abs(fd), 1e-2))
    return {
        "config": "256x256 jet, FP32, 64 steps, BFECC, 60 Jacobi sweeps, checkpoint every 8; "
                  "loss ||M_64 - target||_2 (4 seeded Gaussians); grads w.r.t. U0, V0 and "
                  "64 x 2 force fields",
        "value": side * side / ms / 1e3, "unit": "Mcell-steps/s fwd+adjoint",
        "ms_per_step": ms, "fwd_ms_per_step": ms_fwd, "ratio_to_fwd": ms / ms_fwd, "loss": loss,
        "fd_check": {"directions": 32, "eps": 1e-3, "reference": "FP32 forward central differences",
                     "median_rel_err": float(np.median(rel)), "max_rel_err": float(np.max(rel)),
                     "note": "FP32 differences at eps 1e-3 switch BFECC clamps; the pin is "
                             "tests/test_gpu_adjoint.py::test_rollout256_vs_fp64_oracle_"
                             "differences (FP64 central differences, within 1e-4 relative)"},
    }


def ensemble(fluid_gb300, args, n=256, steps=20, roll=16, every=8):
    """The batched-ensemble configuration: n scenes (seed 5), square sides
    log-uniform in [64, 512], 0-5 discs of radius 4-32, 1-3 jets at U(0.5, 2)
    with smoke, 40-120 Jacobi sweeps per scene, BFECC, FP32.  One batch
    (autotuned block shape and sweeps per launch, each step one CUDA graph)
    against the same scenes stepped one handle at a time, forward and
    forward+adjoint (a `roll`-step rollout, checkpoint every `every`, loss
    ||M_s - target_s||_2 per scene, gradients w.r.t. each initial state)."""
    import numpy as np
    import torch

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import scenes

    sides = scenes.ensemble_sides(n, seed=5)
    iters = np.random.default_rng(5).integers(40, 121, n)

    def build():
        out = []
        for k, side in enumerate(sides):
            f = fluid_gb300.Fluid(1.0, side, side, 1.0, auto_sync=False, scheme=1,
                                  num_iters=int(iters[k]), tb_depth=8, early_exit=False,
                                  UseBFECC=True)
            scenes.ensemble_scene(f, np.random.default_rng(5000 + k))
            out.append(f)
        return out

    cells = sum(side * side for side in sides)
    one = build()
    mem = build()
    targets = [scenes.gaussian_target(f.NumX, f.NumY, seed=50 + k) for k, f in enumerate(one)]
    batch = fluid_gb300.Batch(mem)
    tb, bx, by, _ = batch.autotune(DT, reps=3)
    stream = torch.cuda.ExternalStream(batch.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        batch.step(DT)
    batch.synchronize()
    l0 = batch.launch_count()
    prof = profile_leg(args, "ensemble")
    e0.record(stream)
    for _ in range(steps):
        batch.step(DT)
    e1.record(stream)
    batch.synchronize()
    prof()
    ms_b = e0.elapsed_time(e1) / steps
    launches_b = (batch.launch_count() - l0) / steps

    for f in one:  # warm (graph capture)
        f.Simulate(DT)
        f.Simulate(DT)
    torch.cuda.synchronize()

    def device_span(work):
        # Device time from the first handle's start event to the last
        # handle's end event, each recorded on that handle's own stream (the
        # handles' streams run concurrently; the host issues their work in
        # turn).
        streams = [torch.cuda.ExternalStream(f.stream) for f in one]
        starts = [torch.cuda.Event(enable_timing=True) for _ in one]
        ends = [torch.cuda.Event(enable_timing=True) for _ in one]
        torch.cuda.synchronize()
        for k, st in enumerate(streams):
            starts[k].record(st)
        t0 = time.perf_counter()
        work()
        host = time.perf_counter() - t0
        for k, st in enumerate(streams):
            ends[k].record(st)
        torch.cuda.synchronize()
        span = max(starts[0].elapsed_time(e) for e in ends)
        return span, 1e3 * host

    def fwd_all():
        for _ in range(steps):
            for f in one:
                f.Simulate(DT)

    span_1, host_1 = device_span(fwd_all)
    ms_1 = span_1 / steps

    batch.rollout_grad(DT, roll, targets, every=every)
    batch.synchronize()
    e0.record(stream)
    losses, _ = batch.rollout_grad(DT, roll, targets, every=every)
    e1.record(stream)
    batch.synchronize()
    ms_ba = e0.elapsed_time(e1) / roll
    def adj_all():
        for k, f in enumerate(one):
            f.rollout_grad(DT, roll, targets[k], every=every)

    span_1a, host_1a = device_span(adj_all)
    ms_1a = span_1a / roll
    batch.close()
    return {
        "config": "%d scenes (seed 5): sides log-uniform 64-512, 0-5 discs r 4-32, 1-3 jets "
                  "U(0.5,2) with smoke, 40-120 Jacobi sweeps per scene, BFECC, FP32" % n,
        "interior_cells": cells,
        "autotune": {"tb_depth": tb, "block": [bx, by]},
        "batch_fwd": {"value": cells / ms_b / 1e3, "unit": "Mcell-steps/s", "ms_per_step": ms_b,
                      "launches_per_step": launches_b, "timing": "CUDA events, one graph per step"},
        "one_at_a_time_fwd": {"value": cells / ms_1 / 1e3, "unit": "Mcell-steps/s",
                              "ms_per_step": ms_1, "host_ms_per_step": host_1 / steps,
                              "timing": "device span (CUDA events on every handle's stream) of "
                                        "fg_simulate issued on each handle in turn"},
        "batch_speedup_fwd": ms_1 / ms_b,
        "batch_fwd_adjoint": {"value": cells / ms_ba / 1e3, "unit": "Mcell-steps/s",
                              "ms_per_step": ms_ba, "rollout_steps": roll,
                              "checkpoint_every": every},
        "one_at_a_time_fwd_adjoint": {"value": cells / ms_1a / 1e3, "unit": "Mcell-steps/s",
                                      "ms_per_step": ms_1a, "host_ms_per_step": host_1a / roll,
                                      "timing": "device span (CUDA events on every handle's "
                                                "stream) of each handle's rollout in turn"},
        "batch_speedup_fwd_adjoint": ms_1a / ms_ba,
        "loss_sum": float(np.sum(losses)),
    }


# ---------------------------------------------------------------- CPU legs
# ---------------------------------------------------------------- the app-side rows
APP_W, APP_H = 300, 251          # the app-size jet
N_PARTICLES = 10000              # the app's particle budget
MG_SIDE = 512                    # the multigrid (UseMultigrid) cavity


def jet_setup(f):
    """The app-size jet: walls left, top and bottom, jet of 8 rows at i = 1
    (U = 2, smoke 1) held by device sources."""
    import numpy as np

    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = 0.0
    f.mark_dirty()
    n = f.NumY
    rows = np.arange(n // 2 - 4, n // 2 + 4, dtype=np.int32)
    f.set_sources(np.ones_like(rows), rows, u=2.0, v=0.0, smoke=1.0,
                  mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY | f.SRC_SET_SMOKE)


def spawn_positions(nx, ny, n, seed=9):
    """n particle positions (world units, h = 1) at cell centres near the jet."""
    import numpy as np

    rng = np.random.default_rng(seed)
    i = rng.integers(1, min(nx - 1, 40), n)
    j = rng.integers(ny // 2 - 30, ny // 2 + 30, n)
    return (i + 0.5).astype(np.float32), (j + 0.5).astype(np.float32)


def device_ms(stream, fn, reps):
    """Mean milliseconds of fn() over reps calls, CUDA events on `stream`."""
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def app_rows(fluid_gb300):
    """The rows next to the step: the reference's multigrid V-cycle
    (UseMultigrid, bit for bit) as a whole step, the app's particle advection
    and field rendering, and a view (Vorticity), timed on the GPU."""
    import numpy as np
    import torch

    rows = {}
    # The CPU baseline's own workload on the GPU: the 2048^2 cavity with the
    # reference's serial SOR (200 sweeps, no early exit), bit for bit, as the
    # cluster wavefront -- the drop-in path for a caller who keeps the
    # reference's scheme.
    f = fluid_gb300.Fluid(1.0, W, H, 1.0, auto_sync=False, UseBFECC=True, num_iters=ITERS,
                          early_exit=False)
    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0
    f.mark_dirty()
    li, lj = lid_cells(f)
    f.set_sources(li, lj, u=1.0, v=0.0, mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY)
    st = torch.cuda.ExternalStream(f.stream)
    for _ in range(2):
        f.Simulate(DT)
    ms = device_ms(st, lambda: f.Simulate(DT), 3)
    rows["reference_sor_2048"] = {
        "value": W * H / ms / 1e3, "unit": "Mcell-steps/s", "ms_per_step": ms,
        "config": "the CPU baseline's workload (2048^2 cavity, BFECC, the reference's serial SOR "
                  "with 200 sweeps) bit for bit on the GPU (cluster wavefront on diagonal-major "
                  "copies); device-timed steps; its CPU baseline is the line's cpu_baseline"}
    del f
    # The reference scheme (serial SOR, bit for bit) as the wavefront kernel:
    # the 512^2 cavity, the reference's 8 iterations per step.
    f = fluid_gb300.Fluid(1.0, MG_SIDE, MG_SIDE, 1.0, auto_sync=False, UseBFECC=True, num_iters=8)
    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0
    f.mark_dirty()
    li, lj = lid_cells(f)
    f.set_sources(li, lj, u=1.0, v=0.0, mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY)
    st = torch.cuda.ExternalStream(f.stream)
    for _ in range(3):
        f.Simulate(DT)
    ms = device_ms(st, lambda: f.Simulate(DT), 10)
    rows["reference_sor"] = {"value": MG_SIDE * MG_SIDE / ms / 1e3, "unit": "Mcell-steps/s",
                             "ms_per_step": ms,
                             "config": "%dx%d cavity, the reference's lexicographic SOR bit for bit "
                                       "(8 sweeps with the reference's early exit, wavefront on an "
                                       "8-block cluster), BFECC; device-timed steps"
                                       % (MG_SIDE, MG_SIDE)}
    del f
    # Multigrid: a lid-driven cavity stepped with UseMultigrid (8 V-cycles).
    f = fluid_gb300.Fluid(1.0, MG_SIDE, MG_SIDE, 1.0, auto_sync=False, UseMultigrid=True,
                          UseBFECC=True, num_iters=8)
    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0
    f.mark_dirty()
    li, lj = lid_cells(f)
    f.set_sources(li, lj, u=1.0, v=0.0, mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY)
    st = torch.cuda.ExternalStream(f.stream)
    for _ in range(3):
        f.Simulate(DT)
    ms = device_ms(st, lambda: f.Simulate(DT), 10)
    rows["multigrid"] = {"value": MG_SIDE * MG_SIDE / ms / 1e3, "unit": "Mcell-steps/s",
                         "ms_per_step": ms,
                         "config": "%dx%d cavity, UseMultigrid (the reference's V-cycle bit for "
                                   "bit, 8 cycles), BFECC; device-timed steps" % (MG_SIDE, MG_SIDE)}
    del f
    # Particles and rendering on the app-size jet.
    f = fluid_gb300.Fluid(1.0, APP_W, APP_H, 1.0, auto_sync=False, scheme=fluid_gb300.SCHEME_JACOBI,
                          num_iters=40, early_exit=False, UseBFECC=True)
    jet_setup(f)
    for _ in range(20):
        f.Simulate(DT)
    x, y = spawn_positions(f.NumX, f.NumY, N_PARTICLES)
    rgb = np.full((N_PARTICLES, 3), 200, np.uint8)
    f.particles_add(x, y, 1e9, rgb)
    st = torch.cuda.ExternalStream(f.stream)
    f.particles_advect(DT)
    ms = device_ms(st, lambda: f.particles_advect(0.01), 200)
    live = len(f.particles()["X"])
    rows["particles"] = {"value": N_PARTICLES / ms / 1e3, "unit": "Mparticles/s",
                         "us_per_frame": 1e3 * ms, "live_after": live,
                         "config": "%d particles on the %dx%d jet (RK2 through SampleVelocity, "
                                   "culling, order-preserving compaction); device-timed calls"
                                   % (N_PARTICLES, APP_W, APP_H)}
    img = f.render(f.RENDER_SMOKE)
    t0 = time.perf_counter()
    for _ in range(50):
        img = f.render(f.RENDER_SMOKE)
    ms_app = 1e3 * (time.perf_counter() - t0) / 50
    del f
    g = build_cavity(fluid_gb300)
    gi, gj = lid_cells(g)
    g.set_sources(gi, gj, u=1.0, v=0.0, mode=g.SRC_SKIP_SOLID | g.SRC_SET_VELOCITY)
    for _ in range(3):
        g.Simulate(DT)
    g.render(g.RENDER_VORTICITY)
    t0 = time.perf_counter()
    for _ in range(10):
        img = g.render(g.RENDER_VORTICITY)
    ms_big = 1e3 * (time.perf_counter() - t0) / 10
    rows["render"] = {"value": g.NumX * g.NumY / ms_big / 1e3, "unit": "Mpixel/s",
                      "ms_per_frame_2048": ms_big, "ms_per_frame_app": ms_app,
                      "config": "fg_render (vorticity with getDivergingColor at 2048^2, smoke with "
                                "getSciValue at %dx%d) through the C ABI: min/max, colormap, "
                                "RGBA copied to the host; host wall clock" % (APP_W, APP_H)}
    g.Vorticity()
    t0 = time.perf_counter()
    for _ in range(10):
        g.Vorticity()
    ms_v = 1e3 * (time.perf_counter() - t0) / 10
    rows["views"] = {"value": g.NumX * g.NumY / ms_v / 1e3, "unit": "Mcell/s", "ms_per_view": ms_v,
                     "config": "Vorticity() of the 2048^2 cavity through the C ABI (curl kernel, "
                               "field copied to the host); host wall clock"}
    del g, img
    return rows


def cpu_app_rows(threads, warm=3, timed=3):
    """The CPU baseline of the app-side rows: the oracle's restatement of the
    reference on the same inputs, one bounded sample each (the step rows:
    `warm` warm-up steps, as the GPU rows take, then `timed` steps)."""
    import numpy as np
    from oracle.pyoracle import LEXSOR, OracleFluid

    out = {}
    for key, mg in (("reference_sor", False), ("multigrid", True)):
        o = OracleFluid(1.0, MG_SIDE, MG_SIDE, 1.0, prec=32, threads=threads, scheme=LEXSOR,
                        UseMultigrid=mg, UseBFECC=True, num_iters=8)
        S = o.S.reshape(o.NumX, o.NumY)
        S[:] = 1.0
        S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0
        def step():
            for i in range(2, o.NumX - 2):
                o.SetVelocity(i, o.NumY - 2, 1.0, 0.0)
            o.Simulate(DT)

        for _ in range(warm):
            step()
        t0 = time.perf_counter()
        for _ in range(timed):
            step()
        sec = (time.perf_counter() - t0) / timed
        out[key] = {"value": MG_SIDE * MG_SIDE / sec / 1e6, "unit": "Mcell-steps/s",
                    "cores": threads, "kind": "port",
                    "sample": "%d steps after %d warm-up steps" % (timed, warm)}
    o = OracleFluid(1.0, APP_W, APP_H, 1.0, prec=32, threads=threads, scheme=LEXSOR, num_iters=40,
                    UseBFECC=True)

    S = o.S.reshape(o.NumX, o.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = 0.0
    n = o.NumY
    for _ in range(5):
        for j in range(n // 2 - 4, n // 2 + 4):
            o.SetVelocity(1, j, 2.0, 0.0)
            o.M[n + j] = 1.0
        o.Simulate(DT)
    x, y = spawn_positions(o.NumX, o.NumY, N_PARTICLES)
    age = np.zeros(N_PARTICLES, np.float32)
    mx = np.full(N_PARTICLES, 1e9, np.float32)
    rgb = np.zeros(N_PARTICLES, np.uint32)
    t0 = time.perf_counter()
    reps, done = 20, 0
    for _ in range(reps):
        k = o.particles_advect(0.01, x, y, age, mx, rgb)
        done += x.size
        x, y, age, mx, rgb = x[:k], y[:k], age[:k], mx[:k], rgb[:k]
    sec = (time.perf_counter() - t0) / max(done, 1) * N_PARTICLES
    out["particles"] = {"value": N_PARTICLES / sec / 1e6, "unit": "Mparticles/s", "cores": 1,
                        "kind": "port", "sample": "%d calls over %d particles" % (reps, N_PARTICLES)}
    big = OracleFluid(1.0, W, H, 1.0, prec=32, threads=threads, scheme=LEXSOR)
    t0 = time.perf_counter()
    big.render(3)
    sec = time.perf_counter() - t0
    out["render"] = {"value": big.NumX * big.NumY / sec / 1e6, "unit": "Mpixel/s", "cores": 1,
                     "kind": "port", "sample": "1 vorticity frame at 2048^2"}
    t0 = time.perf_counter()
    big.Vorticity()
    sec = time.perf_counter() - t0
    out["views"] = {"value": big.NumX * big.NumY / sec / 1e6, "unit": "Mcell/s", "cores": 1,
                    "kind": "port", "sample": "1 Vorticity() at 2048^2"}
    return out


def cpu_reference_steps(steps, threads, warmup=0, budget_s=None):
    """Times the reference algorithm (FP32, serial SOR pressure, parallelRange
    stages on `threads` host threads) on the cavity workload: `warmup`
    untimed steps, then up to `steps` timed ones on the same state (fewer,
    but at least 2, when `budget_s` seconds, estimated from the last warm-up
    step, would not hold them all)."""
    from oracle.pyoracle import LEXSOR, OracleFluid

    o = OracleFluid(1.0, W, H, 1.0, prec=32, threads=threads, scheme=LEXSOR, num_iters=ITERS,
                    UseBFECC=True, early_exit=False)
    S = o.S.reshape(o.NumX, o.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = S[-1, :] = 0.0

    def step():
        for i in range(2, o.NumX - 2):
            o.SetVelocity(i, o.NumY - 2, 1.0, 0.0)
        t0 = time.perf_counter()
        o.Simulate(DT)
        return time.perf_counter() - t0

    last = None
    for _ in range(warmup):
        last = step()
    if budget_s is not None and last is not None:
        steps = max(2, min(steps, int(budget_s / max(last, 1e-3))))
    return [step() for _ in range(steps)]


# ---------------------------------------------------------------- arms
def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # Each step is one full 2048^2 step of the reference algorithm (~seconds
    # on the host, growing as the flow develops): W warm-up steps (1 to 10),
    # then timed steps on the same state, at least 2 and as many as
    # --cpu-budget seconds hold -- the protocol of the main arm's
    # cpu_baseline, so the two agree.
    warmup = max(1, min(args.warmup, 10))
    times = cpu_reference_steps(max(2, min(args.steps, args.cpu_steps)), threads, warmup=warmup,
                                budget_s=args.cpu_budget)
    sec = sum(times)
    value = W * H * len(times) / sec / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mcell-steps/s",
        "n_gpus": args.gpus, "steps": len(times), "warmup": warmup,
        "ms_per_step": 1e3 * sec / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config({"scheme": "reference serial lexicographic SOR (fluid.go:157-234)"}),
        "cpu_baseline": {"value": value, "unit": "Mcell-steps/s", "cores": threads, "kind": "port",
                         "sample": "%d full 2048x2048 steps after %d warm-up step(s); pressure "
                                   "loop serial as in the reference, other stages on %d threads"
                                   % (len(times), warmup, threads)},
        "e2e": {"value": value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import fluid_gb300

    fluid_gb300.build()
    f = build_cavity(fluid_gb300)
    li, lj = lid_cells(f)
    f.set_sources(li, lj, u=1.0, v=0.0, mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY)
    stream = torch.cuda.ExternalStream(f.stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        f.Simulate(DT)
    f.synchronize()

    # ------------------------------------------------------------ timed region
    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0] or 0) \
        if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else local
    sampler = ClockSampler(gpu_index)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with sampler:
        barrier()
        torch.cuda.synchronize()
        f.synchronize()
        launches0 = f.launch_count()
        t_host = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            f.Simulate(DT)
        e1.record(stream)
        f.synchronize()
        torch.cuda.synchronize()
        t_host = time.perf_counter() - t_host
        barrier()
    launches = f.launch_count() - launches0
    ms = e0.elapsed_time(e1)
    t_max = max_over_ranks(ms, "cuda") if world > 1 else ms
    value = replica_value(world, args.steps, t_max)
    st = f.stats()

    # ------------------------------------------------------------ dominant kernel
    f.profile(True)
    spans = []
    stages = {}
    for _ in range(min(args.steps, 5)):
        f.Simulate(DT)
        span, nl = f.jacobi_span()
        spans.append(span / nl)
        for name, ms_ in f.stage_times():
            stages.setdefault(name, []).append(ms_)
    f.profile(False)
    launch_ms = statistics.median(spans)
    stage_ms = {k: round(statistics.median(v), 4) for k, v in stages.items()}
    n_cells = f.NumX * f.NumY
    peak, peak_kind = measured_hbm()
    tr = committed_traffic()
    clocks = sampler.summary()
    roofline = jacobi_roofline(n_cells, launch_ms, peak, peak_kind, tr, clocks)
    step_roof = step_roofline(stage_ms, n_cells, t_max / args.steps, peak)

    # ------------------------------------------------------------ e2e through the C ABI
    e2e = None
    if rank == 0:
        g = build_cavity(fluid_gb300)
        mbit = 1 << fluid_gb300.FIELDS["M"]
        u = np.ones(li.size, np.float32)
        v = np.zeros(li.size, np.float32)
        # Frame loop of an app that reads the smoke every frame: the step's
        # smoke is copied to the host beside the next step and read one
        # step later (fg_download_async / fg_download_wait).
        chk = 0.0
        for _ in range(args.warmup):
            g.SetVelocityMany(li, lj, u, v)
            g.Simulate(DT)
            g.download_wait()
            g.download_async()
        g.download_wait()
        g.synchronize()
        b0 = g.edit_bytes()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g.SetVelocityMany(li, lj, u, v)
            g.Simulate(DT)
            g.download_wait()
            chk += float(g.M[g.NumY + 1])  # the host reads the previous step's smoke
            g.download_async()
        g.download_wait()
        chk += float(g.M[g.NumY + 1])
        t_e2e = time.perf_counter() - t0
        h2d = (g.edit_bytes() - b0) / args.steps
        e2e = {"value": W * H * args.steps / t_e2e / 1e6, "unit": "Mcell-steps/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 4 * g.NumX * g.NumY,
               "path": "per step: fg_set_velocity_many (lid edits) + fg_simulate + the smoke field "
                       "read back (fg_download_async of step k beside step k+1, "
                       "fg_download_wait before the host reads it)"}
        del g

    mgrow = multigrid_leg(fluid_gb300, f, args) if rank == 0 and not args.no_multigrid else None
    adj = fwd_adjoint(fluid_gb300, args) if rank == 0 and not args.no_adjoint else None
    roll = (rollout256(fluid_gb300, args)
            if rank == 0 and not (args.no_adjoint or args.no_rollout) else None)
    ens = ensemble(fluid_gb300, args) if rank == 0 and not args.no_ensemble else None
    app = None
    if rank == 0 and not args.no_app:
        stop_app = profile_leg(args, "app")
        app = app_rows(fluid_gb300)
        stop_app()

    # ------------------------------------------------------------ CPU baseline
    cpu = err64 = configs = ratios = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        # The reference arm's protocol: W warm-up steps of the reference
        # algorithm from the zero state (its step time grows as the flow
        # develops), then timed steps on the same state.
        warm = max(1, min(args.warmup, 10))
        times = cpu_reference_steps(max(2, args.cpu_steps), threads, warmup=warm,
                                    budget_s=args.cpu_budget)
        cpu = {"value": W * H * len(times) / sum(times) / 1e6, "unit": "Mcell-steps/s",
               "cores": threads, "kind": "port",
               "sample": "%d full 2048x2048 steps after %d warm-up step(s) of the reference "
                         "algorithm (serial SOR pressure, FP32), other stages on %d host threads "
                         "(the reference arm's protocol)" % (len(times), warm, threads)}
        if app is not None:
            for k, v in cpu_app_rows(threads).items():
                app[k]["cpu_baseline"] = v
            app["reference_sor_2048"]["cpu_baseline"] = dict(cpu)
        err64 = fp64_error(f)
        if not args.no_configs:
            configs = config_rows(fluid_gb300, threads)
        ratios = {"jacobi_gpu_over_sor_cpu": value / cpu["value"],
                  "note": "the line's value (Jacobi scheme) over cpu_baseline (the reference's "
                          "serial SOR on the host): same workload, different pressure algorithm"}
        if app is not None:
            ratios["sor_gpu_over_sor_cpu"] = app["reference_sor_2048"]["value"] / cpu["value"]
            ratios["note"] += ("; sor_gpu_over_sor_cpu: the reference's SOR bit for bit on the GPU "
                               "(app_rows.reference_sor_2048) over the same cpu_baseline")

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config({"parallelism": "replicas%d" % world if world > 1 else "single"}),
            "roofline": roofline, "step_roofline": step_roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "error_vs_fp64": err64, "ratios": ratios,
            "multigrid": mgrow, "fwd_adjoint": adj, "rollout_256": roll, "ensemble": ens,
            "app_rows": app,
            "configs": configs, "clocks": clocks,
            "host_ms_per_step": 1e3 * t_host / args.steps,
            "stage_ms": stage_ms,
            "step_stats": {"div_l2_post": st["div_l2_post"], "resid_l2": st["resid_l2"],
                           "smoke_mass": st["smoke_mass"], "sweeps": st["sweeps"],
                           "jacobi_kernel": {0: "none", 1: "sweep", 2: "tma",
                                             3: "dataflow"}[st["jacobi_kernel"]]},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=2,
                    help="timed CPU steps of the line's cpu_baseline (at least 2)")
    ap.add_argument("--cpu-budget", type=float, default=30.0,
                    help="seconds of timed CPU steps for the line's cpu_baseline")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 128^2 jet and 512x256 Karman rows")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-multigrid", action="store_true",
                    help="skip the MULTIGRID pressure-scheme rows")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-rollout", action="store_true")
    ap.add_argument("--no-app", action="store_true",
                    help="skip the multigrid, particle, rendering and view rows")
    ap.add_argument("--profile-leg", choices=["adjoint", "ensemble", "app", "multigrid"],
                    default=None,
                    help="bracket that leg's timed region for ncu --profile-from-start off")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
