#!/usr/bin/env python3
"""Benchmark of the PUNC++ per-timestep particle path on one GB300.

Headline workload (the mixed-precision configuration): the spherical probe,
cube [-10,10]^3 of 120^3 sub-cubes x 6 Kuhn tetrahedra (10.4M cells, 1.77M
dofs), cells with centroid inside r = 1 removed (the object), 10M electrons
(m = 1) and 10M ions (m = 1836), Maxwellian with T_e = T_i, lambda_D = omega_pe
= 1, the object held at -2 kT/e by a CircuitCM voltage source,
shifted-Maxwellian flux injection on the outer faces, absorption at the object
and the outer boundary, dt = 0.05; mixed form, with the FP64 form of the same
workload beside it and the errors of the mixed form against the FP64 run from
the same seed.  `--workload config3-40` is the same at 40^3; `probe-80` is the
FP64 probe configuration (80^3, 2M + 2M particles).  Inputs are seeded
synthetic data.

A step is one full timestep (interaction/interaction.cpp:342-480): deposit,
Poisson + circuit (one AMG-PCG solve; the object potential enters by
superposition of the set-up Laplace solutions), DG0 field, Boris push, move,
relocation, flux injection.  value = particle-steps/s = sum over timed steps of the particles
pushed / device time (CUDA events on the engine stream).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
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

METRIC = "particle-steps/s on 1 GB300: mixed-precision vs FP64 form at ≤1e-5 rel ρ error"
UNIT = "particle-steps/s"
HALF, RADIUS = 10.0, 1.0
N_SIDE, N_PER_SPECIES = 80, 2_000_000   # the probe configuration; --workload probe-N scales particles with N^3
CONFIG3_PER_SPECIES = 10_000_000         # config3-N: the probe at N^3 with 20M particles
LONG_STEPS = 500                          # the probe configuration's run length
INJECT_SEED = 0x5EED0002


def workload_name(n_side, n_per):
    label = f"config3-{n_side}" if n_per == CONFIG3_PER_SPECIES else f"probe-{n_side}"
    return (f"{label}: [-10,10]^3, {n_side}^3x6 Kuhn tets minus centroid r<1 (object), "
            f"{n_per / 1e6:g}M e- + {n_per / 1e6:g}M ions (m_i=1836), Maxwellian T_e=T_i, CM bias -2 kT/e, "
            f"flux injection, dt=0.05, Poisson rtol 1e-10 atol 1e-12")

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# dominant kernels on probe-80 in the mixed form, from one ncu capture each
# of this bench's command (the summaries under profiles/ give the commands)
# DRAM traffic of the dominant kernels from one ncu capture each: the
# particle pass per launch, the PCG per iteration at the AMG strength threshold
# of the capture (scaled by this run's iterations per solve)
PROFILED_TRAFFIC = {
    ("probe-80", "k_pcg_amg", 0.0): (1.204e9 / 17, "profiles/k_pcg_amg_probe80_mixed.md: 987 MB read + 217 MB "
                                                   "written per solve of 17 iterations"),
    ("probe-80", "k_mixed", None): (0.562e9, "profiles/k_mixed_probe80.md: 455 MB read + 106 MB written per launch"),
    ("config3-120", "k_pcg_amg", 0.0): (10.99e9 / 20, "profiles/k_pcg_amg_config3_120.md (threshold 0): 9.73 GB "
                                                      "read + 1.27 GB written per solve of 20 iterations"),
    ("config3-120", "k_pcg_amg", 0.01): (10.463e9 / 17, "profiles/k_pcg_amg_config3_120.md (threshold 0.01): 9.30 GB "
                                                        "read + 1.16 GB written per solve of 17 iterations"),
    ("config3-120", "k_mixed", None): (2.89e9, "profiles/k_mixed_config3_120.md: 2.30 GB read + 0.59 GB written per "
                                               "launch (untuned 256 x 4 launch configuration)"),
}

DT = 0.05
BIAS = -2.0
RTOL, ATOL = 1e-10, 1e-12
PRECONDS = {"amg": 0, "jacobi": 1}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling (every 100 ms) of SM clocks and throttle reasons,
    from the start of the warm-up to the end of the timed steps: the timed
    steps alone last well under one sampling interval."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0):
        self.rows = []
        self.times = []
        self.window = None       # (start, end) of the timed steps, perf_counter seconds
        self.proc = None
        self.dev = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])
            self.times.append(time.perf_counter())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        n_timed = (sum(1 for t in self.times if self.window[0] - 0.1 <= t <= self.window[1] + 0.1)
                   if self.window else None)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows), "samples_near_timed_steps": n_timed,
                "window": "every 100 ms from the start of the warm-up to the end of the timed steps"}


# ---------------------------------------------------------------------------
def make_workload(n_side=N_SIDE, n_per=N_PER_SPECIES):
    import numpy as np

    from puncpp_gb300 import meshgen
    ma = meshgen.probe_box(n_side, HALF, RADIUS)
    volume = (2 * HALF) ** 3 - 4.0 / 3.0 * math.pi * RADIUS ** 3
    w = volume / n_per                       # physical density 1 per simulation particle weight
    n_sim = n_per / volume
    mi = 1836.0
    species = [dict(q=-w, m=w, n=n_sim, vth=1.0), dict(q=w, m=mi * w, n=n_sim, vth=1.0 / math.sqrt(mi))]
    rng = np.random.default_rng(0x5EED0002)
    over = int(n_per * (2 * HALF) ** 3 / volume) + 1
    loads = []
    for s in species:
        x = -HALF + rng.random((over, 3)) * (2 * HALF)
        v = rng.normal(0.0, s["vth"], (over, 3))
        loads.append((x, v))
    return ma, species, loads


def run_ours(args):
    import numpy as np

    from puncpp_gb300 import _lib as L
    from puncpp_gb300 import punc

    ma, species, loads = make_workload(args.n_side, args.n_per)
    mesh = punc.Mesh(ma)
    prec = L.PG_MIXED if args.precision == "mixed" else L.PG_FP64
    pop = punc.Population(mesh, precision=prec, capacity=int(args.capacity_factor * args.n_per * 2), pcg_rtol=RTOL,
                          pcg_atol=ATOL, pcg_max_iter=4000, pcg_precond=PRECONDS[args.pcg_precond],
                          warm_start=2 if args.warm_start == "extrapolate" else 1)
    if args.amg_theta is not None and args.pcg_precond == "amg":
        punc.set_amg_strength(pop, args.amg_theta)
    for s, (x, v) in zip(species, loads):
        pop.add_particles(x, v, s["q"], s["m"])
    sp = [punc.Species(s["q"], s["m"], n=s["n"], vth=s["vth"]) for s in species]
    punc.create_flux(pop, sp)
    objs = [punc.Object(2)]
    circ = punc.CircuitCM(pop, objs, [(-1, 0, BIAS)], [], DT)
    lib = L.load()
    n0 = pop.num_of_particles()

    step_no = 0
    n_now = n0

    def one(first=False):
        nonlocal step_no, n_now
        r = punc.step(pop, objs, DT, first_step=first, inject=True, seed=INJECT_SEED, step_no=step_no,
                      efield_cg1=args.efield == "cg1")
        step_no += 1
        pushed = n_now
        n_now = r.n_particles
        return r, pushed

    clk = ClockSampler().__enter__()
    for k in range(max(3, args.warmup)):
        one(first=(k == 0))
    cg1 = args.efield == "cg1"
    graph = args.step_mode == "graph"
    tuning = None
    if args.autotune:
        # the autotuner's steps are part of the warm-up
        tuning = punc.autotune(pop, objs, DT, steps_per_trial=2, inject=True, seed=INJECT_SEED, step_no=step_no,
                               efield_cg1=cg1)
        step_no += (24 if prec == L.PG_MIXED else 12) * 2 + 41
        if args.pcg_precond == "amg" and args.amg_theta is None:
            # the AMG aggregation threshold of least PCG time, three candidates
            at = punc.autotune_amg(pop, objs, DT, steps_per_trial=6, inject=True, seed=INJECT_SEED, step_no=step_no,
                                   efield_cg1=cg1)
            tuning.update({"amg_theta": at["amg_theta"], "amg_pcg_ms": at["pcg_ms"]})
            step_no += 3 * 6
        n_now = pop.num_of_particles()
    if args.step_mode != "staged":
        # capture the step graph (and run one more warm-up step) outside the timed region
        rs = punc.run_steps(pop, objs, DT, 1, inject=True, seed=INJECT_SEED, step_no=step_no, efield_cg1=cg1,
                            use_graph=graph)
        step_no += 1
        n_now = rs[-1].n_particles
    L.check(lib.pg_synchronize(pop.handle))
    launches0 = launch_count()
    pushed_total = 0
    iters = 0
    first_timed = step_no
    L.check(lib.pg_event_record(pop.handle, 0))
    t_wall = time.perf_counter()
    t_start = t_wall
    if args.step_mode == "staged":
        punc.set_profiling(pop, True)
        punc.stage_times(pop)  # reset
        for _ in range(args.steps):
            r, pushed = one()
            pushed_total += pushed
            iters += r.pcg_iterations
    else:
        rs = punc.run_steps(pop, objs, DT, args.steps, inject=True, seed=INJECT_SEED, step_no=step_no,
                            efield_cg1=cg1, use_graph=graph)
        step_no += args.steps
        pushed_total = n_now + sum(r.n_particles for r in rs[:-1])
        n_now = rs[-1].n_particles
        iters = sum(r.pcg_iterations for r in rs)
    L.check(lib.pg_event_record(pop.handle, 1))
    last_timed = step_no - 1
    ms = ctypes_ms(lib, pop, 0, 1)
    t_wall = time.perf_counter() - t_wall
    clk.window = (t_start, t_start + t_wall)
    clk.__exit__(None, None, None)
    launches = launch_count() - launches0
    if args.step_mode == "staged":
        prof_steps = args.steps
        stages = punc.stage_times(pop)
        punc.set_profiling(pop, False)
    else:
        # stage shares from a separate profiled pass of staged steps (not timed)
        prof_steps = min(args.steps, 10)
        punc.set_profiling(pop, True)
        punc.stage_times(pop)
        prof_iters = 0
        for _ in range(prof_steps):
            r, _ = one()
            prof_iters += r.pcg_iterations
        stages = punc.stage_times(pop)
        punc.set_profiling(pop, False)
    value = pushed_total / (ms / 1e3)

    # e2e: step by step through the C ABI, each step's outputs read back to host
    # memory (potential, objects, the result row); the potential's read-back
    # (pg_get_phi_async, into two alternating page-locked buffers) overlaps
    # the next step and is complete at the final pg_synchronize
    phi_bufs = [pinned_host(mesh.n_dofs) for _ in range(2)]
    phi_host, pinned = phi_bufs[0]
    L.check(lib.pg_synchronize(pop.handle))
    e2e_pushed = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        if args.step_mode == "staged":
            r, pushed = one()
        else:
            r = punc.run_steps(pop, objs, DT, 1, inject=True, seed=INJECT_SEED, step_no=step_no, efield_cg1=cg1,
                               use_graph=graph)[0]
            step_no += 1
            pushed, n_now = n_now, r.n_particles
        e2e_pushed += pushed
        L.check(lib.pg_get_phi_async(pop.handle, L.dptr(phi_bufs[k % 2][0])))
    L.check(lib.pg_synchronize(pop.handle))
    e2e_s = time.perf_counter() - t0

    # long run: args.long_steps consecutive steps (the probe configuration's
    # length), device-timed like the headline
    long_run = None
    if args.long_steps > 0 and args.step_mode != "staged":
        n_first = n_now
        L.check(lib.pg_event_record(pop.handle, 2))
        rl = punc.run_steps(pop, objs, DT, args.long_steps, inject=True, seed=INJECT_SEED, step_no=step_no,
                            efield_cg1=cg1, use_graph=graph)
        L.check(lib.pg_event_record(pop.handle, 3))
        ms_long = ctypes_ms(lib, pop, 2, 3)
        pushed_long = n_now + sum(r.n_particles for r in rl[:-1])
        long_run = {"steps": args.long_steps, "first_step": step_no, "value": round(pushed_long / (ms_long / 1e3), 1),
                    "unit": UNIT, "ms_per_step": round(ms_long / args.long_steps, 4),
                    "particles_first": n_first, "particles_last": rl[-1].n_particles,
                    "pcg_iterations_per_step": round(sum(r.pcg_iterations for r in rl) / args.long_steps, 2),
                    "timing": "CUDA events on the engine stream around one pg_run_steps call (captured step graph)"}
        step_no += args.long_steps
        n_now = rl[-1].n_particles
    import ctypes as C
    h2d = C.sizeof(L.StepArgs) + C.sizeof(L.Object) * len(objs)
    d2h = phi_host.nbytes + C.sizeof(L.StepResult) + C.sizeof(L.Object) * len(objs)
    if args.step_mode != "staged":
        h2d += 4 * 8 + 32 * len(objs)                   # device counters and object state
        d2h += 4 * 8 + 32 * len(objs) + 8 * (6 + 3 * len(objs)) + 8

    # roofline of the dominant stage
    hbm, src = peaks()
    nc, nv = ma.n_cells, mesh.n_dofs
    lay = punc.poisson_layout(pop)
    nnz = lay["nnz"]
    n_avg = pushed_total / args.steps
    occ = nc * (1.0 - math.exp(-n_avg / nc))
    # stage times of the profiled steps, scaled to the timed steps
    sc = args.steps / max(1, prof_steps)
    part_ms = stages.get("push_move_update_deposit", 0.0) * sc
    pcg_ms = stages.get("pcg", 0.0) * sc
    mixed = args.precision == "mixed"
    # algorithmic bytes: particle pass per particle / occupied cell / dof,
    # PCG per iteration per nonzero / dof
    if mixed:
        pb, cb, pmodel = (n_avg * 57 + occ * 80 + nv * 16, None,
                          "Np*57 (FP32 x, v read+write, cell read+write, species) + occupied cells*80 (64-byte "
                          "cell record: FP32 barycentric rows + neighbours; dof ids 16) + Ndof*16 (phi read for "
                          "the in-pass DG0 field, int64 charge)")
    else:
        pb, cb, pmodel = n_avg * 104 + occ * 288 + nv * 8, None, "Np*104 + occupied cells*288 + Ndof*8"
    if lay["levels"]:
        kb, kmodel = amg_iteration_bytes(lay)
    elif mixed:
        kb, kmodel = nnz * 8 + nv * 52, "per iteration nnz*8 + Ndof*52"
    else:
        kb, kmodel = nnz * 12 + 7 * nv * 8, "per iteration nnz*12 + 7*Ndof*8"
    peak_src = (src + " (MEASURED_PEAKS.json hbm_gbs)") if src == "measured" else "fallback 6.8 TB/s"

    def roof_of(name, bytes_total, t_ms, model):
        ach = bytes_total / (t_ms / 1e3) / 1e9 if t_ms > 0 else 0.0
        out = {"bound": "hbm", "kernel": name, "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
               "frac": round(ach / hbm, 4), "peak_source": peak_src, "traffic": None,
               "algorithmic_bytes": model}
        kern = name.split(" ")[0]
        if kern == "k_pcg_amg":
            key = (args.workload, kern, punc.amg_strength(pop))
            per = iters / max(1, args.steps)          # iterations per solve (one solve a step)
        else:
            key, per = (args.workload, kern, None), 1.0
        if mixed and key in PROFILED_TRAFFIC and args.pcg_precond == "amg":
            t, srcs = PROFILED_TRAFFIC[key]
            out["traffic"], out["traffic_source"] = round(t * per), srcs
            out["traffic_unit"] = "bytes per launch" + (" (per iteration x %.2f iterations per solve)" % per
                                                        if kern == "k_pcg_amg" else "")
        return out

    r_part = roof_of("k_mixed (fused FP32 DG0 field+push+move+walk, fixed-point deposit)" if mixed
                     else "k_particles (fused FP64 push+move+walk+deposit)", args.steps * pb, part_ms, pmodel)
    pcg_kernel = ("k_pcg_amg (AMG-preconditioned mixed PCG, one cooperative launch per solve)" if lay["levels"]
                  else "k_pcg_rel (mixed Jacobi PCG, one cooperative launch per solve)" if mixed
                  else "k_pcg (FP64 Jacobi PCG, one cooperative launch per solve)")
    r_pcg = roof_of(pcg_kernel, iters * kb, pcg_ms, kmodel)
    roof = r_pcg if pcg_ms >= part_ms else r_part
    per_step = {k: v / max(1, prof_steps) for k, v in stages.items()}
    stages_share = {k: round(v / (ms / args.steps), 4) for k, v in per_step.items()}
    # the particle stages alone (push + move + relocate + deposit, injection, charge finalise)
    part_stage_ms = sum(per_step.get(k, 0.0) for k in ("push_move_update_deposit", "injector", "distributor")) * args.steps
    particle_stages = {"value": round(pushed_total / (part_stage_ms / 1e3), 1) if part_stage_ms > 0 else None,
                       "unit": UNIT, "ms_per_step": round(part_stage_ms / args.steps, 4),
                       "stages": ["push_move_update_deposit", "injector", "distributor"]}

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64" if args.precision == "mixed" else "f64",
        "precision_form": args.precision,
        "data": "synthetic: seeded uniform/Maxwellian particles on a generated Kuhn probe mesh (no dataset)",
        "config": {"workload": workload_name(args.n_side, args.n_per), "precision": args.precision,
                   "pcg_precond": args.pcg_precond, "warm_start": args.warm_start, "efield": args.efield,
                   "step_mode": args.step_mode, "tuning": tuning, "cells": nc, "dofs": nv, "nnz": nnz,
                   "amg_levels": [[v["rows"], v["nnz"]] for v in lay["levels"]],
                   "amg_theta": punc.amg_strength(pop) if lay["levels"] else None, "particles_initial": n0,
                   "particles_mean_pushed": round(n_avg), "pcg_iterations_per_step": round(iters / args.steps, 1),
                   "first_timed_step": first_timed, "last_timed_step": last_timed,
                   "l2": f"inputs larger than L2 (129 MB): particle records {(28 if mixed else 52) * n_avg / 1e6:.0f} MB, "
                         f"cell tables {(80 if mixed else 288) * nc / 1e6:.0f} MB per pass"},
        "particle_stages": particle_stages,
        "stage_ms_per_step": {k: round(v, 4) for k, v in per_step.items()},
        "stage_share": stages_share, "stage_source": ("the timed steps" if args.step_mode == "staged"
                                                      else f"{prof_steps} staged pg_step steps after the timed ones"),
        "roofline": roof, "roofline_particles": r_part, "roofline_pcg": r_pcg,
        "e2e": {"value": round(e2e_pushed / e2e_s, 1), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": ("per step through the C ABI: one step (pg_run_steps with K = 1, its result row and "
                         "objects read back, or pg_step), then pg_get_phi_async of the potential into one of two "
                         "host buffers; host wall clock up to the final pg_synchronize, which waits for every "
                         "read-back"),
                "host_buffer": "pinned" if pinned else "pageable"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s_timed": round(t_wall, 3),
        "long_run": long_run,
    }
    pop.close()
    return out


def interior_dofs(mesh):
    """Dofs of no cell that has a facet on the exterior boundary (tag 1)."""
    import numpy as np

    from puncpp_gb300 import _lib as L
    nbr = mesh.table(L.T_NEIGHBOURS).reshape(-1, 4)
    dofs = mesh.table(L.T_CELL_DOFS).reshape(-1, 4)
    keep = np.ones(mesh.n_dofs, bool)
    keep[np.unique(dofs[(nbr == -1).any(axis=1)])] = False
    return keep


def error_record(args, n_steps):
    """The mixed form against the FP64 form from the same seeded start and
    injection streams, in lockstep over n_steps fused steps (the steps the
    timed runs went through, and at least the probe configuration's 500):
    per step the charge density error in the L2 norm and the max-norm, over
    all dofs and over the interior dofs (of no cell with an exterior facet),
    the potential error, and whether the step is a boundary event (the forms'
    absorbed or injected counts, particle counts or object current differ: a
    particle within rounding distance of a boundary absorbed by one form and
    kept by the other, which changes the charge of one boundary cell's dofs).
    The interior error is the drift of the FP32 trajectories from the FP64
    ones.  The collected current per species (the object's share of each
    species' absorbed tally, over dt) is averaged over the run for both
    forms."""
    import numpy as np

    from puncpp_gb300 import _lib as L
    from puncpp_gb300 import punc
    ma, species, loads = make_workload(args.n_side, args.n_per)
    mesh = punc.Mesh(ma)
    inner = interior_dofs(mesh)
    runs = {}
    for prec in (L.PG_FP64, L.PG_MIXED):
        pop = punc.Population(mesh, precision=prec, capacity=int(2.6 * args.n_per * 2), pcg_rtol=RTOL, pcg_atol=ATOL,
                              pcg_max_iter=4000, pcg_precond=PRECONDS[args.pcg_precond],
                              warm_start=2 if args.warm_start == "extrapolate" else 1)
        if args.amg_theta is not None and args.pcg_precond == "amg":
            punc.set_amg_strength(pop, args.amg_theta)
        for s, (x, v) in zip(species, loads):
            pop.add_particles(x, v, s["q"], s["m"])
        punc.create_flux(pop, [punc.Species(s["q"], s["m"], n=s["n"], vth=s["vth"]) for s in species])
        objs = [punc.Object(2)]
        punc.CircuitCM(pop, objs, [(-1, 0, BIAS)], [], DT)
        runs[prec] = (pop, objs)
    l2, mx, l2i, mxi, phi_err, events = [], [], [], [], [], []
    cur = {L.PG_FP64: [], L.PG_MIXED: []}
    qs = None
    for n in range(n_steps):
        res = {}
        for prec, (pop, objs) in runs.items():
            res[prec] = punc.step(pop, objs, DT, first_step=(n == 0), inject=True, seed=INJECT_SEED, step_no=n,
                                  efield_cg1=args.efield == "cg1")
            counts, qs, _ = punc.absorbed_counts(pop)
            cur[prec].append(counts[2] * qs / DT)
        (p64, o64), (p32, o32) = runs[L.PG_FP64], runs[L.PG_MIXED]
        r64, r32 = punc.Function(p64, "rho").vector(), punc.Function(p32, "rho").vector()
        f64, f32 = punc.Function(p64, "phi").vector(), punc.Function(p32, "phi").vector()
        d = r32 - r64
        l2.append(float(np.linalg.norm(d) / np.linalg.norm(r64)))
        mx.append(float(np.abs(d).max() / np.abs(r64).max()))
        l2i.append(float(np.linalg.norm(d[inner]) / np.linalg.norm(r64[inner])))
        mxi.append(float(np.abs(d[inner]).max() / np.abs(r64[inner]).max()))
        phi_err.append(float(np.abs(f32 - f64).max() / np.abs(f64).max()))
        a, b = res[L.PG_FP64], res[L.PG_MIXED]
        events.append(bool(a.n_absorbed != b.n_absorbed or a.n_injected != b.n_injected
                           or a.n_particles != b.n_particles or not np.array_equal(cur[L.PG_FP64][-1], cur[L.PG_MIXED][-1])))
    for pop, _ in runs.values():
        pop.close()
    l2, mx, l2i, mxi, ev = np.array(l2), np.array(mx), np.array(l2i), np.array(mxi), np.array(events)

    def first_over(a, bar=1e-5):
        k = np.nonzero(a > bar)[0]
        return int(k[0]) if len(k) else None

    names = ["electrons" if q < 0 else "ions" for q in qs]
    cur_mean = {form: {nm: float(np.mean([c[k] for c in cur[prec]])) for k, nm in enumerate(names)}
                for form, prec in (("fp64", L.PG_FP64), ("mixed", L.PG_MIXED))}
    equal_steps = sum(np.array_equal(x, y) for x, y in zip(cur[L.PG_FP64], cur[L.PG_MIXED]))
    q3 = lambda a: [float("%.3g" % v) for v in a]
    return {
        "steps": n_steps, "bar": 1e-5,
        "step0": {"l2": float(l2[0]), "max": float(mx[0]),
                  "what": "the first deposit: the same loaded particles (FP32-rounded positions), fixed-point sums "
                          "against FP64"},
        "interior": {"first_step_above_bar_l2": first_over(l2i), "first_step_above_bar_max": first_over(mxi),
                     "l2_at_steps": {str(k): float(l2i[k]) for k in (0, 9, 49, 99, 199, 499) if k < n_steps},
                     "what": "dofs of no cell with an exterior facet: the drift of the FP32 trajectories"},
        "all_dofs": {"l2_median": float(np.median(l2)), "l2_max": float(l2.max()), "max_max": float(mx.max())},
        "event_steps": int(ev.sum()),
        "phi_max_err": float(max(phi_err)),
        "per_step_l2": q3(l2), "per_step_interior_l2": q3(l2i), "per_step_max": q3(mx),
        "collected_current_per_species": cur_mean,
        "collected_current_equal_steps": int(equal_steps),
        "collected_current_rel_diff": {nm: abs(cur_mean["mixed"][nm] - cur_mean["fp64"][nm]) /
                                           max(abs(cur_mean["fp64"][nm]), 1e-300) for nm in names},
        "how": "fresh FP64 and mixed engines, the workload's seeded particles and injection streams, pg_step per step "
               "(the trajectories of the timed runs: the mixed form is deterministic, the FP64 form's atomics "
               "reorder sums at 1e-16)",
    }


def pinned_host(n):
    """An FP64 host buffer in page-locked memory (a numpy view of a pinned
    torch tensor) for the per-step read-back of the e2e leg; pageable memory
    if torch cannot pin."""
    import numpy as np
    try:
        import torch
        t = torch.empty(n, dtype=torch.float64, pin_memory=True)
        return t.numpy(), True
    except Exception:
        return np.zeros(n), False


def amg_iteration_bytes(lay):
    """Algorithmic bytes of one AMG-preconditioned PCG iteration: the operator
    bytes the engine reports (stored entries, padding excluded, times their
    stored size: f32 or binary16 value + 32- or 16-bit column; A_0 twice, for
    the PCG product and the level-0 smoother; every other cycle operator once)
    plus the vectors, f32 except the f64 solution: 88 B per level-0 row (p, Ap,
    z, r, t, x, D^-1 streams of the iteration's phases), 16 B per row of levels
    1..L-1, 8 B per level-1 row (the up-sweep result)."""
    lv = lay["levels"]
    if not lv:
        return 0, "no AMG levels"
    L = len(lv) - 1
    b = lay["cycle_bytes"] + 88 * lv[0]["rows"]
    for l in range(1, L):
        b += 16 * lv[l]["rows"]
    b += 8 * lv[1]["rows"] if L >= 2 else 0
    return b, ("per iteration: operator bytes as stored (cycle_bytes: entries x stored size, A_0 twice) + "
               "88*rows(0) + 16*rows(1..L-1) + 8*rows(1); operators re-read from L2 count each time")


def ctypes_ms(lib, pop, a, b):
    import ctypes as C

    from puncpp_gb300 import _lib as L
    ms = C.c_double()
    L.check(lib.pg_event_elapsed(pop.handle, a, b, C.byref(ms)))
    return ms.value


def launch_count():
    import ctypes as C

    from puncpp_gb300 import _lib as L
    n = C.c_int64()
    L.check(L.load().pg_launch_count(C.byref(n)))
    return n.value


# ---------------------------------------------------------------------------
CPU_STAGES = ("distributor", "poisson", "efield", "accelerator", "move", "update", "injector")
PARTICLE_STAGES = ("distributor", "accelerator", "move", "update", "injector")


def oracle_workload(nthreads, n_side=N_SIDE, n_per=N_PER_SPECIES):
    """The workload on the oracle (the reference's algorithm restated in C++),
    with the Poisson solve by AMG-preconditioned CG (the reference's solver
    class: Krylov + hypre AMG, punc/src/poisson.cpp:297-304), warm-started
    from the previous potential, to the bench's tolerances."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O

    ma, species, loads = make_workload(n_side, n_per)
    o = O.Oracle(ma)
    for s, (x, v) in zip(species, loads):
        o.add_particles(x, v, s["q"], s["m"])
    o.create_flux(species)
    state = {"phi": None, "nthreads": nthreads, "iters": 0}

    def solve(rho, pots, laplace=False):
        r = np.zeros(o.ndof) if rho is None else rho
        x, it = o.poisson_amg(r, potentials=list(pots), x0=None if laplace else state["phi"], rtol=RTOL, atol=ATOL,
                              max_iter=4000, nthreads=state["nthreads"])
        if not laplace:
            state["phi"] = x
            state["iters"] += it
        return x

    circ = O.CircuitCM(o, [(-1, 0, BIAS)], [], DT, solve)
    objs = [dict(bnd_id=2, charge=0.0, current=0.0, potential=0.0)]
    return o, circ, objs, state


def oracle_step(o, circ, objs, n, nthreads, times=None):
    """One full step on the oracle, stage by stage (the reference Timer's task
    names, interaction/interaction.cpp:324-334); stage seconds add into times."""
    T = times if times is not None else {}
    clock = time.perf_counter

    def tick(name, t0):
        T[name] = T.get(name, 0.0) + clock() - t0

    t = clock(); rho = o.distribute_cg1(nthreads); tick("distributor", t)
    t = clock(); phi, _ = circ.solve_circuit(rho, objs); tick("poisson", t)
    t = clock(); E = o.efield(phi); tick("efield", t)
    pushed = o.num_particles()
    t = clock(); o.boris(E, (0.0, 0.0, 0.0), DT * (0.5 if n == 0 else 1.0), nthreads); tick("accelerator", t)
    t = clock(); o.move(DT, None, nthreads); tick("move", t)
    t = clock(); o.update(objs, DT, nthreads); tick("update", t)
    t = clock(); o.inject(DT, INJECT_SEED, n); tick("injector", t)
    return pushed


def _rates(pushed, elapsed, times, steps):
    part = sum(times.get(k, 0.0) for k in PARTICLE_STAGES)
    return {"value": round(pushed / elapsed, 1), "unit": UNIT,
            "particle_stages_value": round(pushed / part, 1) if part > 0 else None,
            "stage_s_per_step": {k: round(times.get(k, 0.0) / steps, 4) for k in CPU_STAGES}}


def cpu_baseline(args, budget=30.0):
    """The oracle on the machine's host cores: all threads on full steps of the
    workload, then one thread.  A single-threaded full step of a large workload
    would take minutes, so the single-thread leg times the Poisson solve and the
    field in full and the particle stages on a subsample of the particles
    (per-particle rates scaled to the full count)."""
    import numpy as np
    nthreads = os.cpu_count() or 1
    o, circ, objs, state = oracle_workload(nthreads, args.n_side, args.n_per)
    oracle_step(o, circ, objs, 0, nthreads)          # first step (half push, AMG set-up) untimed
    times, pushed, steps, n = {}, 0, 0, 1
    state["iters"] = 0
    t0 = time.perf_counter()
    while True:
        pushed += oracle_step(o, circ, objs, n, nthreads, times)
        n += 1
        steps += 1
        el = time.perf_counter() - t0
        if el > 0.5 * budget or steps >= 5:
            break
    allc = _rates(pushed, el, times, steps)
    allc.update({"cores": nthreads, "steps": steps, "amg_pcg_iterations_per_step": round(state["iters"] / steps, 1)})
    # one thread: Poisson and field in full, particle stages on a subsample
    n_full = o.num_particles()
    p = o.particles(sort=False)
    k = max(1, int(np.ceil(n_full * sum(times.get(s, 0.0) for s in PARTICLE_STAGES) / steps * nthreads * 0.8
                           / (0.25 * budget) / n_full))) if n_full else 1
    t1 = {}
    state["nthreads"] = 1
    clock = time.perf_counter
    rho = o.distribute_cg1(nthreads)
    t = clock(); phi, _ = circ.solve_circuit(rho, objs); t1["poisson"] = clock() - t
    t = clock(); E = o.efield(phi); t1["efield"] = clock() - t
    if k > 1:
        o.set_particles({key: val[::k] for key, val in p.items()})
    n_sub = o.num_particles()
    t = clock(); o.distribute_cg1(1); t1["distributor"] = clock() - t
    t = clock(); o.boris(E, (0.0, 0.0, 0.0), DT, 1); t1["accelerator"] = clock() - t
    t = clock(); o.move(DT, None, 1); t1["move"] = clock() - t
    t = clock(); o.update(objs, DT, 1); t1["update"] = clock() - t
    t = clock(); o.inject(DT, INJECT_SEED, n); t1["injector"] = clock() - t
    scale = n_full / max(1, n_sub)
    for key in ("distributor", "accelerator", "move", "update"):
        t1[key] *= scale
    one = _rates(n_full, sum(t1.values()), t1, 1)
    one.update({"cores": 1, "particle_subsample": f"1/{k}" if k > 1 else "none",
                "how": "Poisson and field timed on the full mesh; distributor, accelerator, move and update timed on "
                       "every k-th particle and scaled by k; injector in full"})
    return {"value": allc["value"], "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{steps} full steps of the same {args.workload} workload on the oracle (the reference's "
                      f"algorithm restated in C++, {nthreads} threads; Poisson by AMG-preconditioned CG like the "
                      f"reference's Krylov + hypre AMG) after one untimed step",
            "all_cores": allc, "single_thread": one}


def run_reference(args):
    nthreads = os.cpu_count() or 1
    o, circ, objs, state = oracle_workload(nthreads, args.n_side, args.n_per)
    n = 0
    for _ in range(max(1, args.warmup)):
        oracle_step(o, circ, objs, n, nthreads)
        n += 1
    pushed, t0, done = 0, time.perf_counter(), 0
    budget = 150.0
    times = {}
    state["iters"] = 0
    for _ in range(args.steps):
        pushed += oracle_step(o, circ, objs, n, nthreads, times)
        n += 1
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    rates = _rates(pushed, el, times, done)
    v = rates["value"]
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(el / done * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic: seeded uniform/Maxwellian particles on a generated Kuhn probe mesh (no dataset)",
            "config": {"workload": workload_name(args.n_side, args.n_per), "precision": "fp64"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{done} of {args.steps} timed steps (bounded to {budget:.0f} s) of the full "
                                       f"workload on the oracle, the reference's algorithm restated in C++ with its "
                                       f"solver class (AMG-preconditioned Krylov) for Poisson (the reference needs "
                                       f"DOLFIN/PETSc/Boost, absent here)",
                             "particle_stages_value": rates["particle_stages_value"],
                             "stage_s_per_step": rates["stage_s_per_step"],
                             "amg_pcg_iterations_per_step": round(state["iters"] / done, 1)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# Further workloads (not the headline): the Langmuir oscillation, a batch of
# independent probe runs, and the adjoint run.  Each prints one JSON line of
# the same shape.

def _event_ms(lib, pop, fn):
    from puncpp_gb300 import _lib as L
    L.check(lib.pg_synchronize(pop.handle))
    L.check(lib.pg_event_record(pop.handle, 0))
    out = fn()
    L.check(lib.pg_event_record(pop.handle, 1))
    return ctypes_ms(lib, pop, 0, 1), out


def langmuir_load(n_side, ppc, seed=0x5EED0001):
    """Periodic unit cube of n_side^3 x 6 cells, ppc electrons per cell
    uniform in the cube with x displaced by 0.01 sin(2 pi x), at rest; weight
    such that the density is 1 (omega_p = 1 with eps0 = 1)."""
    import numpy as np

    from puncpp_gb300 import meshgen
    ma = meshgen.langmuir_cube(n_side)
    n = ppc * ma.n_cells
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3))
    x[:, 0] = np.mod(x[:, 0] + 0.01 * np.sin(2 * np.pi * x[:, 0]), 1.0)
    w = 1.0 / n
    return ma, x, np.zeros((n, 3)), -w, w


def run_langmuir(args):
    """Config: periodic Langmuir cube, 16 electrons per cell, Boris dt = 0.251,
    P1 periodic Poisson with the mean fixed to zero, K steps; FP64 plain form
    (the headline of this workload) and the mixed form beside it; the oracle
    (single thread, like the reference) timed on a few steps."""
    from puncpp_gb300 import _lib as L
    from puncpp_gb300 import punc
    ma, x, v, q, m = langmuir_load(args.n_side, 16)
    lib = L.load()
    res = {}
    for form, prec in (("fp64", L.PG_FP64), ("mixed", L.PG_MIXED)):
        pop = punc.Population(punc.Mesh(ma), precision=prec, periodic=True, pcg_rtol=1e-10, pcg_atol=1e-12,
                              pcg_max_iter=4000)
        n0 = pop.add_particles(x, v, q, m)
        punc.run_steps(pop, [], 0.251, args.warmup, first_step=True, Ld=ma.Ld)
        punc.run_steps(pop, [], 0.251, 1, Ld=ma.Ld, step_no=args.warmup)        # graph capture
        ms, rs = _event_ms(lib, pop, lambda: punc.run_steps(pop, [], 0.251, args.steps, Ld=ma.Ld,
                                                             step_no=args.warmup + 1))
        res[form] = {"value": round(n0 * args.steps / (ms / 1e3), 1), "ms_per_step": round(ms / args.steps, 4),
                     "pcg_iterations_per_step": round(sum(r.pcg_iterations for r in rs) / args.steps, 1),
                     "particles": n0}
        pop.close()
    out = {"metric": "particle-steps/s on 1 GB300 (Langmuir oscillation, FP64 plain form)",
           "value": res["fp64"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": res["fp64"]["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic: seeded uniform electrons with a sin(2 pi x) "
           "displacement on a generated periodic Kuhn cube",
           "config": {"workload": f"langmuir-{args.n_side}: periodic unit cube {args.n_side}^3x6, 16 e- per cell, "
                                  f"v = 0, x += 0.01 sin(2 pi x), Boris dt = 0.251, Poisson rtol 1e-10",
                      "fp64": res["fp64"], "mixed": res["mixed"]}}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        o = O.Oracle(ma)
        o.add_particles(x, v, q, m)
        _, M = o.matrices()
        solve = O.PeriodicPoisson(o, 1)
        t0, k = time.perf_counter(), 0
        while k < 3 or (time.perf_counter() - t0 < 10.0 and k < 20):
            phi = solve(M @ o.distribute_cg1())
            o.boris(o.efield(phi), (0.0, 0.0, 0.0), 0.251 * (0.5 if k == 0 else 1.0))
            o.move(0.251, ma.Ld)
            o.update([], 0.251)
            k += 1
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(len(x) * k / el, 1), "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{k} full steps on the oracle, one thread (the reference is "
                                         f"single-threaded), Jacobi PCG"}
    return out


def batch_plan(R, seed=0x5EED0004):
    """The bias-sweep configuration's runs: per run r a probe box [-h, h]^3 of
    n^3 sub-cubes x 6 tetrahedra (n uniform in 30..70) around a sphere of
    radius 0.5, 1, 2 or 4 Debye lengths, a bias uniform in [-5, 5] kT/e and a
    particle count uniform in 0.2M..4M (electrons + ions).  All runs share the
    simulation density (250 particles per species per unit volume, the probe
    configuration's), so the species are common to all runs and a run's count
    fixes its box: (2h)^3 - 4/3 pi r^3 = count / 500, with h >= r + 2."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sides = rng.integers(30, 71, R)
    radii = rng.choice([0.5, 1.0, 2.0, 4.0], R)
    biases = rng.uniform(-5.0, 5.0, R)
    counts = rng.uniform(0.2e6, 4.0e6, R)
    n_sim = 250.0
    halves = 0.5 * np.cbrt(counts / (2 * n_sim) + 4.0 / 3.0 * math.pi * radii ** 3)
    halves = np.maximum(halves, radii + 2.0)
    return sides, halves, radii, biases, n_sim, rng


def run_batch(args):
    """Config: R independent probe runs in one engine (the bias sweep, R = 64
    by default), each step one launch per stage for all runs, captured as a
    CUDA graph, launch configuration from the autotuner."""
    import numpy as np

    from puncpp_gb300 import _lib as L
    from puncpp_gb300 import batch as B
    from puncpp_gb300 import meshgen, punc
    R = args.runs
    t_setup = time.perf_counter()
    sides, halves, radii, biases, n_sim, rng = batch_plan(R)
    mi = 1836.0
    w = 1.0 / n_sim
    meshes = [meshgen.probe_box(int(n), float(h), float(r)) for n, h, r in zip(sides, halves, radii)]
    nper = [int(n_sim * ((2 * h) ** 3 - 4.0 / 3.0 * math.pi * r ** 3)) for h, r in zip(halves, radii)]
    t_mesh = time.perf_counter()
    bt = B.Batch(meshes, precision=L.PG_MIXED, capacity=int(2.6 * 2 * sum(nper)), pcg_rtol=RTOL, pcg_atol=ATOL,
                 pcg_max_iter=4000)
    t_engine = time.perf_counter()
    species = ((-w, w, 1.0), (w, mi * w, 1.0 / math.sqrt(mi)))
    loaded = []
    for r in range(R):
        h = halves[r]
        box = (2 * h) ** 3
        k = 0
        for q, m_, vth in species:
            xs = -h + rng.random((int(nper[r] * box / (box - 4.0 / 3.0 * math.pi * radii[r] ** 3)) + 1, 3)) * (2 * h)
            k += bt.add_particles(r, xs, rng.normal(0.0, vth, xs.shape), q, m_)
        loaded.append(k)
    bt.create_flux([punc.Species(q, m_, n=n_sim, vth=vth) for q, m_, vth in species],
                   seeds=[0x5EED0004 + r for r in range(R)])
    objs = bt.objects()
    bt.circuit(objs, biases, DT)
    pop = bt.pop
    lib = L.load()
    t_loaded = time.perf_counter()
    punc.run_steps(pop, objs, DT, args.warmup, first_step=True, inject=True, seed=0x5EED0004)
    tuning = punc.autotune(pop, objs, DT, steps_per_trial=2, inject=True, seed=0x5EED0004, step_no=args.warmup)
    step_no = args.warmup + (24 * 2 + 41)
    at = punc.autotune_amg(pop, objs, DT, steps_per_trial=6, inject=True, seed=0x5EED0004, step_no=step_no)
    tuning.update({"amg_theta": at["amg_theta"], "amg_pcg_ms": at["pcg_ms"]})
    step_no += 3 * 6
    rs0 = punc.run_steps(pop, objs, DT, 1, inject=True, seed=0x5EED0004, step_no=step_no)
    n_now = rs0[-1].n_particles
    clk = ClockSampler().__enter__()
    t_w = time.perf_counter()
    ms, rs = _event_ms(lib, pop, lambda: punc.run_steps(pop, objs, DT, args.steps, inject=True, seed=0x5EED0004,
                                                         step_no=step_no + 1))
    clk.window = (t_w, time.perf_counter())
    clk.__exit__(None, None, None)
    pushed = n_now + sum(r.n_particles for r in rs[:-1])
    cells = sum(m.n_cells for m in meshes)
    per_run = bt.particles_per_run()
    lay = punc.poisson_layout(pop)
    pop.close()
    return {"metric": "particle-steps/s on 1 GB300 (batched independent probe runs, mixed form)",
            "value": round(pushed / (ms / 1e3), 1), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64",
            "data": "synthetic: seeded Maxwellian loads on generated Kuhn probe meshes",
            "config": {"workload": f"batch-{R}: {R} probe runs in one engine, boxes [-h,h]^3 of 30..70 sub-cubes per "
                                   f"side x 6, radii in {{0.5,1,2,4}}, biases in [-5,5], 0.2M..4M particles per run "
                                   f"(e- + ions, m_i = 1836), flux injection, dt = 0.05, captured step graph",
                       "runs": R, "cells": cells, "dofs": lay["n_rows"], "particles_loaded": int(sum(loaded)),
                       "particles_per_run_min_max": [int(per_run.min()), int(per_run.max())],
                       "sides_min_max": [int(sides.min()), int(sides.max())],
                       "particles_mean_pushed": round(pushed / args.steps),
                       "pcg_iterations_per_step": round(sum(r.pcg_iterations for r in rs) / args.steps, 1),
                       "tuning": tuning,
                       "setup_s": {"meshes": round(t_mesh - t_setup, 1), "engine": round(t_engine - t_mesh, 1),
                                   "particles_flux_circuit": round(t_loaded - t_engine, 1)}},
            "clocks": clk.summary()}


def run_adjoint(args):
    """Config: periodic Langmuir mesh 32^3 x 6, 2M electrons with v ~ N(0,
    0.1^2), uniform E0 = (0.01, 0, 0), K = 50 steps with checkpoints every 10,
    loss ||rho_K - target||^2; value = particle-steps of the forward K steps
    per second of forward + backward (checkpointed recompute and reverse
    sweep with a second PCG per step)."""
    import numpy as np

    from puncpp_gb300 import _lib as L
    from puncpp_gb300 import meshgen, punc
    ma = meshgen.langmuir_cube(args.n_side)
    n, K, Cc = args.adjoint_particles, 50, 10
    rng = np.random.default_rng(32)
    x = rng.random((n, 3))
    v0 = rng.normal(0.0, 0.1, size=(n, 3))
    w = 1.0 / n
    pop = punc.Population(punc.Mesh(ma), periodic=True, pcg_rtol=1e-12, pcg_atol=1e-30, pcg_max_iter=5000)
    target = rng.normal(0.0, 1.0, size=ma.n_dofs) * 0.05
    pop.add_particles(x, v0, -w, w)
    lib = L.load()
    L.check(lib.pg_synchronize(pop.handle))
    t0 = time.perf_counter()
    loss = punc.adjoint_forward(pop, [], 0.1, K, Cc, target, first_step=True, E0=(0.01, 0.0, 0.0), Ld=ma.Ld)
    t1 = time.perf_counter()
    gv, ge, gx = punc.adjoint_backward(pop, n)
    t2 = time.perf_counter()
    pop.close()
    return {"metric": "adjoint particle-steps/s on 1 GB300 (K forward steps per second of forward + backward)",
            "value": round(n * K / (t2 - t0), 1), "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": 0,
            "ms_per_step": round((t2 - t0) / K * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded uniform electrons, Gaussian velocities, seeded target charge vector",
            "config": {"workload": f"adjoint-{args.n_side}: periodic {args.n_side}^3x6, {n / 1e6:g}M e-, "
                                   f"v ~ N(0, 0.1^2), E0 = (0.01, 0, 0), K = {K}, checkpoints every {Cc}",
                       "forward_s": round(t1 - t0, 4), "backward_s": round(t2 - t1, 4), "loss": loss,
                       "grad_E0": [float(g) for g in ge], "host_wall_clock": True}}


def combine_replicas(res, world):
    """Whole-job line of N independent replicas (one per rank, process group
    initialised): the slowest rank's time per step, and the particle-steps
    all ranks processed divided by it."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([res["ms_per_step"]], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    v = torch.tensor([res["value"] * res["ms_per_step"]], dtype=torch.float64)
    dist.all_reduce(v)
    out = dict(res)
    out["config"] = dict(res["config"])
    out["ms_per_step"] = float(t.item())
    out["value"] = round(float(v.item()) / float(t.item()), 1)
    out["n_gpus"] = world
    out["config"]["parallelism"] = f"replicas x{world}"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1, help="GPUs of the job (N > 1: one replica per rank under torchrun)")
    ap.add_argument("--steps", type=int, default=20, help="timed steps")
    ap.add_argument("--warmup", type=int, default=3, help="untimed warm-up steps (at least 3)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"],
                    help="ours: the engine; reference: the reference's algorithm on the host cores")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the timed CPU baseline sample")
    ap.add_argument("--workload", default="config3-120",
                    help="config3-N (the headline: the probe at N^3 sub-cubes with 20M particles), probe-N (N^3 "
                         "sub-cubes, 2M + 2M particles scaled by (N/80)^3), langmuir-N, batch-R (R independent "
                         "probe runs), adjoint-N")
    ap.add_argument("--long-steps", type=int, default=LONG_STEPS,
                    help="probe workloads: a further device-timed run of this many consecutive steps (0: none)")
    ap.add_argument("--error-steps", type=int, default=LONG_STEPS,
                    help="mixed form: steps of the lockstep error record against the FP64 form (at least the "
                         "steps the timed runs went through; 0: none)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="mixed (the headline form: FP32 particles, fixed-point deposit, mixed PCG) or fp64")
    ap.add_argument("--no-fp64-form", dest="fp64_form", action="store_false",
                    help="skip the FP64-form run that the mixed form is compared with")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the engine's autotuners (launch configuration, sort interval, AMG strength threshold) in the warm-up")
    ap.add_argument("--step-mode", default="graph", choices=["graph", "stream", "staged"],
                    help="graph: pg_run_steps replaying a captured CUDA graph; stream: pg_run_steps without the "
                         "graph; staged: pg_step per step with stage timing")
    ap.add_argument("--warm-start", default="prev", choices=["prev", "extrapolate"],
                    help="PCG start: the previous potential, or 2 phi_n - phi_(n-1)")
    ap.add_argument("--efield", default="dg0", choices=["dg0", "cg1"],
                    help="field path: EFieldDG0 + accel/boris, or ESolver (CG1) + accel_cg1/boris_cg1")
    ap.add_argument("--pcg-precond", default="amg", choices=sorted(PRECONDS),
                    help="Poisson preconditioner: one AMG V-cycle or Jacobi per iteration")
    ap.add_argument("--amg-theta", type=float, default=None,
                    help="AMG aggregation strength threshold (default: chosen by pg_autotune_amg in the warm-up, "
                         "0 with --no-autotune)")
    ap.add_argument("--capacity-factor", type=float, default=2.6,
                    help="probe workloads: particle store slots per initial particle (the store grows if needed)")
    ap.add_argument("--runs", type=int, default=64, help="batch-R: runs in the batch (from the workload name)")
    ap.add_argument("--adjoint-particles", type=int, default=2_000_000, help="adjoint-N: particles of the run")
    args = ap.parse_args()
    kind = args.workload.split("-")[0]
    if kind not in ("config3", "probe", "langmuir", "batch", "adjoint"):
        ap.error("--workload must be config3-N, probe-N, langmuir-N, batch-R or adjoint-N")
    args.n_side = int(args.workload.split("-")[1])
    if kind not in ("probe", "config3"):
        if kind == "batch":
            args.runs = args.n_side
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm runs the probe workload"}))
            return
        fn = {"langmuir": run_langmuir, "batch": run_batch, "adjoint": run_adjoint}[kind]
        print(json.dumps(fn(args)))
        return
    if kind == "config3":
        args.n_per = CONFIG3_PER_SPECIES
    else:
        args.n_per = int(round(N_PER_SPECIES * (args.n_side / N_SIDE) ** 3))
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # replicas only: one independent run per GPU, no data-path collective
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    res = run_ours(args)
    if args.precision == "mixed" and args.fp64_form:
        # the same workload in the FP64 form: its throughput
        import copy
        a64 = copy.copy(args)
        a64.precision = "fp64"
        r64 = run_ours(a64)
        res["fp64_form"] = {"value": r64["value"], "unit": UNIT, "ms_per_step": r64["ms_per_step"],
                            "pcg_iterations_per_step": r64["config"]["pcg_iterations_per_step"],
                            "e2e": r64["e2e"]["value"], "roofline_particles_frac": r64["roofline_particles"]["frac"],
                            "particle_stages": r64["particle_stages"], "long_run": r64["long_run"],
                            "stage_ms_per_step": r64["stage_ms_per_step"], "tuning": r64["config"]["tuning"],
                            "amg_theta": r64["config"]["amg_theta"],
                            "poisson": "the same AMG-preconditioned PCG as the mixed form (FP32 recurrence and "
                                       "operators, FP64 solution, inner products and true-residual replacement, "
                                       "FP64 stopping test); the particle arithmetic is FP64"}
        # the full step shares the Poisson solve between the forms; the
        # particle stages (push, move, walk, deposit, injection) are where
        # they differ
        res["mixed_vs_fp64"] = round(res["value"] / r64["value"], 3)
        if res["particle_stages"]["value"] and r64["particle_stages"]["value"]:
            res["mixed_vs_fp64_particle_stages"] = round(res["particle_stages"]["value"] /
                                                         r64["particle_stages"]["value"], 3)
        if args.error_steps > 0:
            # the timed steps of both runs lie inside the first covered steps
            covered = max(args.error_steps, res["config"]["last_timed_step"] + 1,
                          r64["config"]["last_timed_step"] + 1)
            res["rho_rel_err"] = error_record(args, covered)
    if world > 1:
        res = combine_replicas(res, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(res))


if __name__ == "__main__":
    main()
