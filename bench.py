#!/usr/bin/env python
"""Contact-steps/s of SCISim's Ball2D contact path on one GB300, every step solved to residual <= 1e-6.

Workload (the headline configuration): the Ball2D dense pile, 262,144 discs with
radii log-uniform in [0.02, 0.06] (density 1), seeded non-overlapping fill of a
40 x 60 box with four walls, gravity -9.81, symplectic Euler dt 0.005, CoR 0,
mu 0.4, Coulomb residual tolerance 1e-6 (FP64-evaluated), at most 5,000
Gauss-Seidel sweeps per step.  The job starts from the fill: the pile falls and
forms during capped pre-roll phases (--schedule, untimed), then settles at the full
settings until --settle-converged consecutive steps reach the tolerance (untimed),
then --warmup steps, then --steps timed steps.  Every timed step's residual and
convergence are reported.

A step is one GeometricImpactFrictionMap::flow of the whole scene: predictor,
broad + narrow phase, contact assembly, coloured block Gauss-Seidel to tolerance,
impulse cache, final map.  value = sum of active contacts over the timed steps /
their device time (inputs resident in HBM, L2 flushed between steps).  e2e = the
same through the reference-facing C-ABI call sg_flow with pinned host buffers
(q0, v0 up; q1, v1 down) inside the timed region, from the same state and cache.

Solver forms, all from the state (positions, velocities, impulse cache) the timed
steps start from: "warm" (impulse cache NORMAL_AND_FRICTION, FP32 sweeps with FP64
residual and refinement, two-level sweeps) is the headline; "plain" is FP64 Gauss-Seidel,
with the impulse cache (plain_fp64_gpu) and cold (plain_fp64_cold_gpu, one step with a
larger sweep cap, which it does not reach the tolerance within).

--impl reference times the reference algorithm's CPU implementation (the oracle,
a restatement of SCISim + So-bogus; the reference itself needs Eigen/So-bogus,
absent here) on the same configuration: the same pile, formed and settled by the same
deterministic GPU pre-roll (untimed), stepped from the same state and impulse cache.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "contact-steps/s to Coulomb residual<=1e-6: warm-start+batched vs plain GPU"
UNIT = "contact-steps/s"
WORKLOAD = "ball2d_dense_pile_262144"
# Algorithmic bytes of the Gauss-Seidel kernel (FP64), per contact:
#   update: perm 4, ia 4, ib 4, n 16, c 16, W 24, mu 8, r 16+16, minv 2x8, v_a 16+16, v_b 16+16
#   residual: ia 4, ib 4, v_a 16, v_b 16, n 16, c 16, r 16, snapshot 16, mu 8
#   FP32 sweep: (ia, ib) 8, n 8, c 8, (w00, w01, w11, mu) 16, r 8+8, minv 2x4, v_a 8+8, v_b 8+8
#   FP32 -> FP64 lift: per contact perm 4, r32 8, r64 16 w, two adjacency visits x (adj 4, ia 4,
#   n 16, r 16); per body v0 16, minv 8, v 16 w
BYTES_PER_CONTACT_SWEEP = 188
BYTES_PER_CONTACT_SWEEP32 = 96
BYTES_PER_CONTACT_EVAL = 112
BYTES_PER_CONTACT_LIFT = 108
BYTES_PER_BODY_LIFT = 40
# 3D spheres (FP64), per contact:
#   update: perm 4, ia 4, ib 4, basis 72, angular rows 96, c 24, W 48, mu 8, r 24+24,
#           minv 2x8, Iinv 2x72, (v, omega) 2x(32+32) r + 2x(32+32) w
#   residual: ia 4, ib 4, basis 72, angular rows 96, c 24, (v, omega) 2x64, r 24, snapshot 24, mu 8
BYTES_PER_CONTACT_SWEEP_3D = 724
BYTES_PER_CONTACT_EVAL_3D = 384
#   FP32 sweep: (a, b) 8, basis 36, angular rows 48, c 12, W 24, mu 4, r 12+12, minv 2x4, Iinv 2x36,
#               (v, omega) 2x(16+16) r + 2x(16+16) w
#   FP32 -> FP64 lift: per contact perm 4, r32 12, r64 24 w, two adjacency visits x (adj 4, ia 4, basis 72,
#               angular rows 48, r 24); per body v0 48, minv 8, Iinv 72, (v, omega) 64 w + 32 w
BYTES_PER_CONTACT_SWEEP32_3D = 364
BYTES_PER_CONTACT_LIFT_3D = 344
BYTES_PER_BODY_LIFT_3D = 224


def step_roofline(kernel, bytes_total, ms_total, basis):
    """Algorithmic bytes of the sweeps over a measured time, against the measured HBM copy rate."""
    hbm, peak_kind = peaks()
    ach = bytes_total / (ms_total / 1e3) / 1e9 if ms_total > 0 else 0.0
    return {"kernel": kernel, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "peak_kind": peak_kind, "bytes": bytes_total, "ms": ms_total, "time_basis": basis, "traffic": None}


def gs3_bytes(prof):
    return (prof["contact_sweeps"] * BYTES_PER_CONTACT_SWEEP_3D + prof["contact_sweeps32"] * BYTES_PER_CONTACT_SWEEP32_3D +
            prof["contact_evals"] * BYTES_PER_CONTACT_EVAL_3D + prof["contact_lifts"] * BYTES_PER_CONTACT_LIFT_3D +
            prof["body_lifts"] * BYTES_PER_BODY_LIFT_3D)


def gs_bytes(prof):
    """Algorithmic bytes moved by the Gauss-Seidel kernel(s) counted in a profile."""
    return (prof["contact_sweeps"] * BYTES_PER_CONTACT_SWEEP + prof["contact_sweeps32"] * BYTES_PER_CONTACT_SWEEP32 +
            prof["contact_evals"] * BYTES_PER_CONTACT_EVAL + prof["contact_lifts"] * BYTES_PER_CONTACT_LIFT +
            prof["body_lifts"] * BYTES_PER_BODY_LIFT)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # The raw samples (the JSON line carries their summary); SG_CLOCKS_CSV keeps them.
        self.out = os.environ.get("SG_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(), "sg_clocks.csv")

    def start(self):
        try:
            self.fh = open(self.out, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.out):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_scene(n):
    """The dense-pile fill with n discs: the 40 x 60 box for 262,144 discs; other sizes
    keep the depth (60) and the area fraction by scaling the width."""
    from scisim_gb300 import scenes
    return scenes.dense_pile(n=n, seed=2, width=40.0 * n / 262144.0, height=60.0)


def solver_kw(s, **over):
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-6, max_iters=5000, eval_every=1)
    kw.update(over)
    return kw


# --------------------------------------------------------------------------- CPU leg
def cpu_from_state(s, q, v, cache, steps, first_iteration, budget_s=None):
    """The oracle (C++ restatement of SCISim + So-bogus, sequential block Gauss-Seidel in active-set
    order, one host thread) stepping the pile from the given state and impulse cache (the contacts and
    impulses of the step before, as the GPU left them) for `steps` steps at the full settings, each
    step timed on the host clock; with budget_s, no step starts once that many seconds have gone
    (at least one step runs).  Returns (contact-steps/s, description, per-step records)."""
    from oracle import oracle as O  # the oracle: CPU baseline only
    O.build()
    kw = solver_kw(s)
    sim = O.Ball2D(q, v, s["r"], s["m"], s["plane_x"], s["plane_n"], cache_mode=O.CACHE_NORMAL_AND_FRICTION, **kw)
    if cache is not None:
        sim.set_cache(cache["ia"], cache["ib"], cache["alpha"], cache["beta"])
    sim.iteration = first_iteration - 1
    recs, tot, wall = [], 0, 0.0
    for _ in range(steps):
        if budget_s is not None and recs and wall >= budget_s:
            break
        t0 = time.perf_counter()
        st = sim.step()
        dt = time.perf_counter() - t0
        wall += dt
        tot += st["n_contacts"]
        recs.append({"n_contacts": st["n_contacts"], "converged": bool(st["succeeded"]), "residual": st["error"],
                     "sweeps": st["iterations"], "s": dt})
    conv = sum(r["converged"] for r in recs)
    desc = ("oracle (C++ restatement of SCISim + So-bogus: grid broad phase, CCD, sequential block Gauss-Seidel "
            "in active-set order, 1 host thread) on the full %d-disc pile from the GPU's state and impulse cache, "
            "%d steps at the full settings: %d contact-steps in %.2f s, %d of %d steps converged, residuals %s, "
            "sweeps %s" % (s["r"].shape[0], len(recs), tot, wall, conv, len(recs),
                           [float("%.3g" % r["residual"]) for r in recs], [r["sweeps"] for r in recs]))
    return (tot / wall if wall > 0 else None), desc, recs


def cpu_strip_sample(args, steps):
    """Without a GPU (CPU-only runs of the reference arm): the oracle on a strip of the same fill
    (width 40/32 of the pile's at this depth), pre-rolled on the CPU with capped solves, then `steps`
    steps at the full settings.  Returns (contact-steps/s, description)."""
    from oracle import oracle as O  # the oracle: CPU baseline only
    O.build()
    n = max(2048, args.n // 32)
    s = make_scene(n)
    kw = solver_kw(s)
    sim = O.Ball2D(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"],
                   cache_mode=O.CACHE_NORMAL_AND_FRICTION, **kw)
    pre = sum(n_ for n_, _ in parse_schedule(args.schedule))
    sim.set_solver(kw["tol"], 50)
    sim.run(pre)
    sim.set_solver(kw["tol"], kw["max_iters"])
    sim.run(args.warmup)
    t0 = time.perf_counter()
    st, tot, bad = sim.run(steps)
    dt = time.perf_counter() - t0
    desc = ("no GPU: oracle (1 thread) on a %d-disc strip of the same fill pre-rolled %d capped steps on the "
            "CPU, then %d steps: %d contact-steps in %.2f s (%d not converged, last residual %.1e)" %
            (n, pre + args.warmup, steps, tot, dt, bad, st["error"]))
    return tot / dt, desc


def batch_cpu_sample(b, q0, v0, pick, steps):
    """The oracle on the scenes the plain GPU comparison samples, from the same state over the
    same number of steps, each scene on its own host thread (the oracle's C loop runs without the
    GIL and keeps no shared state), so all host cores up to one per scene work at once.  Scenes
    start from an empty impulse cache, then warm-start from their own.  Returns (contact-steps/s,
    threads, description)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O  # the oracle: CPU baseline only
    O.build()
    sims = []
    for sc in pick:
        b0, b1 = int(b["body_off"][sc]), int(b["body_off"][sc + 1])
        p0, p1 = int(b["plane_off"][sc]), int(b["plane_off"][sc + 1])
        sims.append(O.Ball2D(q0[2 * b0:2 * b1], v0[2 * b0:2 * b1], b["r"][b0:b1], b["m"][b0:b1], b["plane_x"][p0:p1],
                             b["plane_n"][p0:p1], dt=b["dt"], gravity=b["gravity"], mu=float(b["mu"][sc]),
                             CoR=float(b["CoR"][sc]), tol=1e-6, max_iters=5000, eval_every=1,
                             integrator=O.SYMPLECTIC_EULER, cache_mode=O.CACHE_NORMAL_AND_FRICTION))
    threads = max(1, min(len(sims), os.cpu_count() or 1))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(lambda sim: sim.run(steps), sims))
    wall = time.perf_counter() - t0
    tot = sum(r[1] for r in res)
    desc = ("oracle (C++ restatement of SCISim + So-bogus, sequential block GS per scene) on the %d sampled "
            "scenes (%d discs), one host thread per scene, %d threads, %d steps from the GPU's state: %d "
            "contact-steps in %.2f s" % (len(sims), sum(x.nb for x in sims), threads, steps, tot, wall))
    return (tot / wall if wall > 0 else None), threads, desc


def sphere_batch_cpu_sample(b, q0, v0, pick, steps, first_iteration):
    """As batch_cpu_sample for the sphere batch: the oracle on the sampled scenes from the GPU's
    state, steps numbered as the GPU's, one host thread per scene."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O  # the oracle: CPU baseline only
    from scisim_gb300 import scenes
    O.build()
    sims = []
    for sc in pick:
        x = scenes.batch_scene3(b, sc, q0, v0)
        sim = O.Sphere3D(x["q"], x["v"], x["r"], x["m"], x["I0"], x["plane_x"], x["plane_n"], dt=b["dt"],
                         gravity=b["gravity"], mu=x["mu"], CoR=x["CoR"], tol=1e-6, max_iters=5000, eval_every=1)
        sim.iteration = first_iteration - 1
        sims.append(sim)
    threads = max(1, min(len(sims), os.cpu_count() or 1))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(lambda sim: sim.run(steps), sims))
    wall = time.perf_counter() - t0
    tot = sum(r[1] for r in res)
    desc = ("oracle (C++ restatement of SCISim + So-bogus, sequential 3x3-block GS per scene) on the %d sampled "
            "scenes (%d spheres), one host thread per scene, %d threads, %d steps from the GPU's state: %d "
            "contact-steps in %.2f s" % (len(sims), sum(x.nb for x in sims), threads, steps, tot, wall))
    return (tot / wall if wall > 0 else None), threads, desc


def run_reference(args):
    """The reference arm: the oracle on the CPU, on the headline configuration (the same pile formed
    and settled by the same deterministic GPU pre-roll, untimed, then stepped on the CPU from the
    state and impulse cache the GPU arm's timed steps start from).  Rank 0 only."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    gpu = False
    try:
        import torch
        gpu = torch.cuda.is_available()
    except Exception:
        gpu = False
    if gpu:
        torch.cuda.set_device(local)
        ctx, s, it, info = form_pile(args, local)
        q, v = ctx.state()
        cache = ctx.last_contacts()
        ctx.close()
        value, desc, recs = cpu_from_state(s, q, v, cache, args.steps, it, args.cpu_budget)
        sample = "the full %d-disc pile from the GPU-formed state (%s)" % (s["r"].shape[0], pile_note(info))
        conv = {"steps_converged": sum(r["converged"] for r in recs), "steps": len(recs),
                "budget_s": args.cpu_budget,
                "max_residual": max(r["residual"] for r in recs) if recs else None,
                "sweeps_per_step": [r["sweeps"] for r in recs]}
        same = True
    else:
        value, desc = cpu_strip_sample(args, args.steps)
        sample, conv, same = "8,192-disc strip of the same fill (no GPU to form the pile)", None, False
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded dense-pile fill)",
            "config": {"workload": WORKLOAD if args.n == 262144 else "ball2d_dense_pile_%d" % args.n,
                       "sample": sample, "tol": 1e-6, "max_iters": 5000, "warm_start": "normal_and_friction",
                       "same_state_as_gpu_arm": same},
            "convergence": conv,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- GPU leg
def timed_steps(ctx, torch, stream, k, flush, first_iteration=1):
    """k steps, each bracketed by CUDA events on the library's stream; L2 flushed between.
    Returns (ms per step, contacts per step, per-step solve records)."""
    ms, contacts, recs = [], [], []
    for j in range(k):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = ctx.step(1, first_iteration=first_iteration + j)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        contacts.append(st["n_contacts"])
        recs.append({"converged": bool(st["succeeded"]), "residual": st["error"], "sweeps": st["iterations"]})
    return ms, contacts, recs


STAGES = ["predictor_and_grid", "pair_counting_and_plane_flags", "contact_writes_and_assembly", "colouring",
          "fp64_probe_partition_and_packing", "gauss_seidel", "final_velocity", "extract_cache_final_map"]


def headline_roofline(prof, total_ms, args, sweeps=()):
    """Roofline of the Gauss-Seidel kernel over the timed steps (algorithmic bytes per launch over its
    CUDA-event time per launch) and the step's stage times from the library's stage events.  sweeps:
    the timed steps' sweep counts (a solve of more than eight went on after the FP64 probe)."""
    hbm, peak_kind = peaks()
    gl = max(prof["gs_launches"], 1)
    bytes_per_launch = gs_bytes(prof) / gl
    gs_ms_per_launch = prof["gs_ms"] / gl
    achieved = bytes_per_launch / (gs_ms_per_launch / 1e3) / 1e9 if gs_ms_per_launch > 0 else 0.0
    n_two = prof.get("two_level_solves", 0)
    n_f64 = prof.get("fp64_start_solves", 0)
    two_level = n_two >= prof["gs_launches"] > 0 and n_f64 == 0
    if args.precision == 0:
        kname = "k_gs (cooperative coloured block Gauss-Seidel, FP64)"
    elif two_level:
        kname = "k_gs_patch (two-level FP32 sweeps: patches on shared memory, boundary contacts over the grid)"
    elif n_f64 >= prof["gs_launches"] > 0:
        n_cont = sum(1 for x in sweeps if x > 8)
        if n_cont == 0:
            kname = "k_gs (the FP64 probe, one-level: every solve converged in it)"
        else:
            kname = ("k_gs (the FP64 probe, one-level), then for the %d of %d solves it left unconverged "
                     "k_gs_ff1 (one-level FP64-precision sweeps in float-float pairs, up to 160) and, for %d "
                     "of them, k_gs_patch_ff (the same on the two-level partition), together"
                     % (n_cont, prof["gs_launches"], n_two))
    else:
        kname = "k_gs_mixed (cooperative FP32 sweeps, FP64 checks and refinement)"
    traffic = None
    tp = os.path.join(HERE, "profiles", "k_gs_patch_traffic.txt")
    if os.path.exists(tp) and two_level:
        for line in open(tp):
            if line.startswith("dram_bytes_per_algorithmic_byte"):
                traffic = float(line.split()[1]) * bytes_per_launch
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind, "kernel": kname,
                "bytes_per_launch": bytes_per_launch, "ms_per_launch": gs_ms_per_launch,
                "gs_share_of_step": prof["gs_ms"] / total_ms if total_ms else None}
    steps = max(prof["steps"], 1)
    stages = {name: round(ms / steps, 4) for name, ms in zip(STAGES, prof["stage_ms"])}
    return roofline, stages


def fp32_form_error(ck, s, it0, local, **tuning):
    """One step from the checkpointed state in the FP32 form and in plain FP64, to the same
    tolerance: the FP32 form's deviation from FP64 in impulses (alpha, beta), velocities and
    positions.  Both solves stop anywhere in the tolerance's neighbourhood of a frictional solution
    set, so the figures bound the form's effect at this tolerance rather than its rounding alone."""
    from scisim_gb300 import _lib
    out = {}
    for prec in (1, 0):
        c = _lib.Context(device=local, **solver_kw(s))
        c.restore(ck)
        c.reconfigure(precision=prec)
        if prec == 1 and tuning:
            c.set_tuning(**tuning)
        st = c.step(1, first_iteration=it0)
        q, v = c.state()
        out[prec] = (st, c.last_contacts(), q, v)
        c.close()
    (s32, c32, q32, v32), (s64, c64, q64, v64) = out[1], out[0]
    same = np.array_equal(c32["ia"], c64["ia"]) and np.array_equal(c32["ib"], c64["ib"])
    rec = {"same_contacts": bool(same), "residual_fp32_form": s32["error"], "residual_fp64": s64["error"],
           "sweeps_fp32_form": s32["iterations"], "sweeps_fp64": s64["iterations"],
           "velocity_abs": float(np.abs(v32 - v64).max()), "velocity_scale": float(np.abs(v64).max()),
           "position_abs": float(np.abs(q32 - q64).max())}
    if same and c64["alpha"].size:
        scale = float(np.abs(c64["alpha"]).max())
        da = float(np.abs(c32["alpha"] - c64["alpha"]).max())
        db = float(np.abs(c32["beta"] - c64["beta"]).max())
        rec.update({"alpha_abs": da, "beta_abs": db, "impulse_scale": scale,
                    "impulse_rel": max(da, db) / scale if scale > 0 else None})
    return rec


def convergence_record(recs):
    """Per-step convergence of timed steps: solve_succeeded (error < tol) as SCISim reports it
    (GeometricImpactFrictionMap.cpp:344-350), residuals and sweeps."""
    if not recs:
        return None
    return {"steps_converged": sum(r["converged"] for r in recs), "steps": len(recs),
            "all_converged": all(r["converged"] for r in recs),
            "max_residual": max(r["residual"] for r in recs), "tol": 1e-6,
            "residuals": [float("%.4g" % r["residual"]) for r in recs], "sweeps": [r["sweeps"] for r in recs]}


def batch_leg(args, torch, local, flush, ws=1, rank=0):
    """Batched Ball2D scenes (independent scenes of 16-4,096 discs stepped together from a
    CUDA graph, warm start from each scene's impulse cache) against the plain solver on a
    sample of the same scenes (one context per scene, FP64, cold start), over the same steps
    from the same state.  With several ranks the scenes are sharded by work (scisim_gb300.dist),
    each rank steps its shard, and the throughput is the sum of contact-steps over the slowest
    rank's time; the plain comparison runs on rank 0."""
    from scisim_gb300 import _lib, dist, scenes
    b = scenes.ball2d_batch(n_scenes=args.batch_scenes)
    S_all = len(b["mu"])
    if ws > 1:
        b = dist.batch_slice(b, dist.shard_scenes(dist.batch_work(b), ws)[rank])
    S, N = len(b["mu"]), int(b["body_off"][-1])
    kw = dict(dt=b["dt"], gravity=b["gravity"], tol=1e-6, max_iters=args.preroll_iters, device=local,
              integrator=_lib.SYMPLECTIC_EULER)
    ctx = _lib.Context(cache_mode=_lib.CACHE_NORMAL_AND_FRICTION, precision=args.precision, **kw)
    ctx.upload_batch2d(b["body_off"], b["q"], b["v"], b["r"], b["m"], b["plane_off"], b["plane_x"], b["plane_n"],
                       b["mu"], b["CoR"])
    t0 = time.perf_counter()
    ctx.step(args.batch_preroll)
    ctx.reconfigure(max_iters=5000)
    ctx.step(8)  # warm-up: one graph replay at the full settings (graph built here)
    log("batch preroll %d + 8 steps in %.1f s" % (args.batch_preroll, time.perf_counter() - t0))
    q0, v0 = ctx.state()
    stream = torch.cuda.ExternalStream(ctx.stream_ptr(), device=local)
    ctx.profile_read(reset=True)
    flush.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_batch")  # lets a profiler select the leg's timed launches
    e0.record(stream)
    st = ctx.step(args.batch_steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = e0.elapsed_time(e1)
    prof = ctx.profile_read(reset=True)
    stats = ctx.batch_scene_stats()
    job_contacts = dist.sum_over_ranks(st["total_contacts"], device="cuda")
    N_all = int(dist.sum_over_ranks(N, device="cuda"))
    ms = dist.max_over_ranks(ms, device="cuda")
    value = job_contacts / (ms / 1e3)
    log("batch: %d scenes, %d discs, %d contact-steps in %.1f ms" % (S, N, st["total_contacts"], ms))
    if rank != 0:
        ctx.close()
        return None
    # Plain: the first scenes of a fixed random sample, each alone, cold FP64, same steps.
    rng = np.random.default_rng(0)
    pick = rng.choice(S, min(args.batch_plain_scenes, S), replace=False)
    pc, pms = 0, 0.0
    for sc in pick:
        b0, b1 = int(b["body_off"][sc]), int(b["body_off"][sc + 1])
        p0, p1 = int(b["plane_off"][sc]), int(b["plane_off"][sc + 1])
        c = _lib.Context(cache_mode=_lib.CACHE_NONE, mu=float(b["mu"][sc]), CoR=float(b["CoR"][sc]),
                         precision=_lib.PRECISION_FP64, **dict(kw, max_iters=5000))
        c.upload_ball2d(q0[2 * b0:2 * b1], v0[2 * b0:2 * b1], b["r"][b0:b1], b["m"][b0:b1], b["plane_x"][p0:p1],
                        b["plane_n"][p0:p1])
        cs = torch.cuda.ExternalStream(c.stream_ptr(), device=local)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(cs)
        r = c.step(args.batch_steps)
        a1.record(cs)
        a1.synchronize()
        pc += r["total_contacts"]
        pms += a0.elapsed_time(a1)
        c.close()
    plain = pc / (pms / 1e3) if pms > 0 else None
    cpu_v, cpu_threads, cpu_desc = batch_cpu_sample(b, q0, v0, pick, args.batch_steps)
    log("batch cpu: %s" % cpu_desc)
    out = {"workload": "ball2d_batch_%d" % S_all, "scenes": S_all, "ranks": ws, "discs": N_all, "value": value,
           "unit": UNIT,
           "steps": args.batch_steps, "timed_steps": [args.batch_preroll + 9, args.batch_preroll + 8 + args.batch_steps],
           "ms_per_step": ms / args.batch_steps, "contacts_per_step": job_contacts / args.batch_steps,
           "form": "batched (one CUDA graph per 8 steps), warm start (cache), %s" % (
               "FP32 sweeps + FP64 residual and refinement per scene" if args.precision == 1 else "FP64 sweeps"),
           "fp32_sweep_share": prof["contact_sweeps32"] / max(prof["contact_sweeps"] + prof["contact_sweeps32"], 1),
           "scenes_converged_last_step": int(stats["succeeded"].sum()),
           "gs_iterations_mean_last_step": float(stats["iterations"].mean()),
           "plain_fp64_gpu": {"value": plain, "unit": UNIT, "sample_scenes": len(pick),
                              "form": "one context per scene, cold start, FP64, same steps from the same state"},
           "batched_over_plain": value / plain if plain else None, "gpu_launches": prof["kernel_launches"],
           "roofline": step_roofline("k_gs_scenes (one block per scene)" if int(np.diff(b["body_off"]).max()) <= 8192
                                     else "k_gs_mixed_batch", gs_bytes(prof), ms,
                                     "the whole timed graph replay (detection, assembly and sweeps), so a lower "
                                     "bound on the sweep kernel's rate"),
           "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_threads, "kind": "port", "sample": cpu_desc},
           "batched_over_cpu": value / cpu_v if cpu_v else None}
    ctx.close()
    return out


def sphere_batch_leg(args, torch, local, flush):
    """Batched sphere scenes (C5's 256 scenes of 64-1,024 spheres, FP64, no impulse cache) stepped
    together, against the plain solver on a sample of the same scenes (one context per scene,
    FP64), over the same steps from the same state."""
    from scisim_gb300 import _lib, scenes
    b = scenes.sphere_batch(n_scenes=args.sphere_batch_scenes)
    S, N = len(b["mu"]), int(b["body_off"][-1])
    kw = dict(dt=b["dt"], gravity=b["gravity"], tol=1e-6, max_iters=args.preroll_iters, device=local,
              integrator=_lib.SPLIT_HAM)
    ctx = _lib.Context(**kw)
    ctx.upload_sphere3d_batch(b["body_off"], b["q"], b["v"], b["r"], b["m"], b["I0"], b["plane_off"], b["plane_x"],
                              b["plane_n"], b["mu"], b["CoR"])
    t0 = time.perf_counter()
    ctx.step(args.sphere_batch_preroll)
    ctx.reconfigure(max_iters=5000)
    ctx.step(1)  # warm-up at the full settings
    log("sphere batch preroll %d + 1 steps in %.1f s" % (args.sphere_batch_preroll, time.perf_counter() - t0))
    q0, v0 = ctx.state()
    stream = torch.cuda.ExternalStream(ctx.stream_ptr(), device=local)
    ctx.profile_read(reset=True)
    flush.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    st = ctx.step(args.sphere_batch_steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    prof = ctx.profile_read(reset=True)
    stats = ctx.batch_scene_stats()
    q64, v64 = ctx.state()
    value = st["total_contacts"] / (ms / 1e3)
    log("sphere batch: %d scenes, %d spheres, %d contact-steps in %.1f ms" % (S, N, st["total_contacts"], ms))
    rng = np.random.default_rng(0)
    pick = rng.choice(S, min(args.batch_plain_scenes, S), replace=False)
    pc, pms = 0, 0.0
    for sc in pick:
        x = scenes.batch_scene3(b, sc, q0, v0)
        c = _lib.Context(mu=x["mu"], CoR=x["CoR"], **dict(kw, max_iters=5000))
        c.upload_sphere3d(x["q"], x["v"], x["r"], x["m"], x["I0"], x["plane_x"], x["plane_n"])
        cs = torch.cuda.ExternalStream(c.stream_ptr(), device=local)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(cs)
        r = c.step(args.sphere_batch_steps)
        a1.record(cs)
        a1.synchronize()
        pc += r["total_contacts"]
        pms += a0.elapsed_time(a1)
        c.close()
    plain = pc / (pms / 1e3) if pms > 0 else None
    cpu_v, cpu_threads, cpu_desc = sphere_batch_cpu_sample(b, q0, v0, pick, args.sphere_batch_steps,
                                                           args.sphere_batch_preroll + 2)
    log("sphere batch cpu: %s" % cpu_desc)
    # The same steps from the same state with FP32 sweeps and FP64 refinement, scene by scene.
    c32 = _lib.Context(precision=_lib.PRECISION_FP32_REFINE, **dict(kw, max_iters=5000))
    up = (b["body_off"], q0, v0, b["r"], b["m"], b["I0"], b["plane_off"], b["plane_x"], b["plane_n"], b["mu"], b["CoR"])
    c32.upload_sphere3d_batch(*up)
    c32.step(1)  # warm-up, then back to the timed state
    c32.upload_sphere3d_batch(*up)
    s32 = torch.cuda.ExternalStream(c32.stream_ptr(), device=local)
    c32.profile_read(reset=True)
    flush.zero_()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(s32)
    r32 = c32.step(args.sphere_batch_steps)
    f1.record(s32)
    f1.synchronize()
    ms32 = f0.elapsed_time(f1)
    st32 = c32.batch_scene_stats()
    q32, v32 = c32.state()
    # The FP32 form's deviation from FP64 after the same steps from the same state, over the bodies of
    # scenes that converged in both (linear parts: positions and velocities).
    both = stats["succeeded"].astype(bool) & st32["succeeded"].astype(bool)
    nbody = int(b["body_off"][-1])
    mask = np.zeros(nbody, bool)
    for sc in np.nonzero(both)[0]:
        mask[int(b["body_off"][sc]):int(b["body_off"][sc + 1])] = True
    m3 = np.repeat(mask, 3)
    form_err = {"scenes_compared": int(both.sum()),
                "position_abs": float(np.abs(q32[:3 * nbody] - q64[:3 * nbody])[m3].max()) if mask.any() else None,
                "velocity_abs": float(np.abs(v32[:3 * nbody] - v64[:3 * nbody])[m3].max()) if mask.any() else None,
                "velocity_scale": float(np.abs(v64[:3 * nbody])[m3].max()) if mask.any() else None,
                "angular_velocity_abs": float(np.abs(v32[3 * nbody:] - v64[3 * nbody:])[m3].max()) if mask.any() else None}
    p32 = c32.profile_read(reset=True)
    v32 = r32["total_contacts"] / (ms32 / 1e3)
    sw = p32["contact_sweeps32"] + p32["contact_sweeps"]
    log("sphere batch FP32+FP64 refinement: %d contact-steps in %.1f ms" % (r32["total_contacts"], ms32))
    c32.close()
    out = {"workload": "sphere_batch_%d" % S, "scenes": S, "spheres": N, "value": value, "unit": UNIT,
           "steps": args.sphere_batch_steps,
           "timed_steps": [args.sphere_batch_preroll + 2, args.sphere_batch_preroll + 1 + args.sphere_batch_steps],
           "ms_per_step": ms / args.sphere_batch_steps, "contacts_per_step": st["total_contacts"] / args.sphere_batch_steps,
           "form": "batched, one launch per step for all scenes, FP64, each scene to its own tolerance",
           "scenes_converged_last_step": int(stats["succeeded"].sum()),
           "gs_iterations_mean_last_step": float(stats["iterations"].mean()),
           "plain_fp64_gpu": {"value": plain, "unit": UNIT, "sample_scenes": len(pick),
                              "form": "one context per scene, FP64, same steps from the same state"},
           "batched_over_plain": value / plain if plain else None, "gpu_launches": prof["kernel_launches"],
           "roofline": step_roofline("k_gs3_batch", gs3_bytes(prof), prof["gs_ms"] or ms,
                                     "the sweep kernel's CUDA events" if prof["gs_ms"] else "the whole timed steps"),
           "fp32_refine": {"value": v32, "unit": UNIT, "ms_per_step": ms32 / args.sphere_batch_steps,
                           "scenes_converged_last_step": int(st32["succeeded"].sum()),
                           "fp32_sweep_share": p32["contact_sweeps32"] / sw if sw else None,
                           "over_fp64_batched": v32 / value, "over_plain": v32 / plain if plain else None,
                           "error_vs_fp64": form_err,
                           "form": "batched, FP32 sweeps with FP64 checks and refinement, each scene to its "
                                   "own tolerance"},
           "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_threads, "kind": "port", "sample": cpu_desc},
           "batched_over_cpu": value / cpu_v if cpu_v else None}
    ctx.close()
    return out


def sphere_leg(args, torch, local, flush):
    """RigidBody3D spheres (65,536 by default): FP64 3x3-block solve, no impulse cache (the
    reference's 3D geometric map keeps none), after a pre-roll with capped solves."""
    from scisim_gb300 import _lib, scenes
    s = scenes.sphere_pile(n=args.spheres)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-6, max_iters=args.preroll_iters,
              integrator=_lib.SPLIT_HAM, device=local)
    ctx = _lib.Context(precision=args.precision, **kw)
    ctx.upload_sphere3d(s["q"], s["v"], s["r"], s["m"], s["I0"], s["plane_x"], s["plane_n"])
    t0 = time.perf_counter()
    ctx.step(args.sphere_preroll)
    ctx.reconfigure(max_iters=5000)
    log("spheres preroll %d steps in %.1f s" % (args.sphere_preroll, time.perf_counter() - t0))
    stream = torch.cuda.ExternalStream(ctx.stream_ptr(), device=local)
    ctx.profile_enable(True)
    ctx.profile_read(reset=True)
    torch.cuda.nvtx.range_push("timed_spheres")
    ms, contacts, _ = timed_steps(ctx, torch, stream, args.sphere_steps, flush, args.sphere_preroll + 1)
    torch.cuda.nvtx.range_pop()
    prof = ctx.profile_read(reset=True)
    tot = float(sum(ms))
    value = sum(contacts) / (tot / 1e3)
    hbm, peak_kind = peaks()
    gl = max(prof["gs_launches"], 1)
    b_launch = (prof["contact_sweeps"] * BYTES_PER_CONTACT_SWEEP_3D + prof["contact_sweeps32"] * BYTES_PER_CONTACT_SWEEP32_3D +
                prof["contact_evals"] * BYTES_PER_CONTACT_EVAL_3D + prof["contact_lifts"] * BYTES_PER_CONTACT_LIFT_3D +
                prof["body_lifts"] * BYTES_PER_BODY_LIFT_3D) / gl
    ms_launch = prof["gs_ms"] / gl
    ach = b_launch / (ms_launch / 1e3) / 1e9 if ms_launch > 0 else 0.0
    out = {"workload": "sphere_pile_%d" % args.spheres, "value": value, "unit": UNIT, "steps": args.sphere_steps,
           "timed_steps": [args.sphere_preroll + 1, args.sphere_preroll + args.sphere_steps],
           "ms_per_step": tot / args.sphere_steps, "contacts_per_step": sum(contacts) / args.sphere_steps,
           "gs_iterations_per_step": (prof["contact_sweeps"] + prof["contact_sweeps32"]) / max(sum(contacts), 1),
           "fp32_sweep_share": prof["contact_sweeps32"] / max(prof["contact_sweeps"] + prof["contact_sweeps32"], 1),
           "form": ("FP32 sweeps + FP64 residual and refinement" if args.precision == 1 else "FP64 sweeps") +
                   ", cold start (no 3D impulse cache in the reference's geometric map)",
           "roofline": {"kernel": "k_gs3_mixed" if args.precision == 1 else "k_gs3", "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                        "frac": ach / hbm, "peak_kind": peak_kind, "bytes_per_launch": b_launch,
                        "ms_per_launch": ms_launch, "gs_share_of_step": prof["gs_ms"] / tot if tot else None},
           "gpu_launches": prof["kernel_launches"]}
    ctx.close()
    return out


def mlp_leg(args, torch, local):
    """Learned warm start on the hopper (C4: a V-wedge of two static planes): the hopper filled and
    settled on the GPU as the dense pile is (capped pre-roll phases, then steps at the full settings
    until consecutive steps converge), the plain FP64 solver's per-contact samples recorded over
    converged steps, the network trained on the GPU, then the same settled state stepped twice to
    the same tolerance in the bench's form: from the impulse cache, and from the cache-or-network
    start (per step the start with the smaller FP64 residual).  Sweeps, convergence and
    contact-steps/s of both."""
    from scisim_gb300 import _lib, scenes
    s = scenes.hopper(args.mlp_hopper)
    kw = dict(dt=s["dt"], gravity=s["gravity"], mu=s["mu"], CoR=s["CoR"], tol=1e-6, device=local)
    rec = _lib.Context(cache_mode=_lib.CACHE_NORMAL_AND_FRICTION, precision=args.precision, max_iters=50, **kw)
    rec.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    t0 = time.perf_counter()
    it = 1
    for n, cap in parse_schedule(args.mlp_schedule):
        rec.reconfigure(max_iters=cap)
        rec.step(n, first_iteration=it)
        it += n
    rec.reconfigure(max_iters=5000)
    run = settle = 0
    while settle < args.settle_max and run < 5:
        st = rec.step(1, first_iteration=it)
        it += 1
        settle += 1
        run = run + 1 if st["succeeded"] else 0
    t1 = time.perf_counter()
    ck = rec.checkpoint()
    # Samples of the plain FP64 solver over steps at the full settings.
    rec.reconfigure(precision=_lib.PRECISION_FP64)
    rec.mlp_load(_lib.mlp_init(0))
    rec.mlp_enable(warm_start=False, record=True)
    xs, ts = [], []
    rec_conv = 0
    for _ in range(args.mlp_record_steps):
        st = rec.step(1, first_iteration=it)
        it += 1
        rec_conv += int(st["succeeded"])
        x, t = rec.mlp_last_samples()
        xs.append(x)
        ts.append(t)
    X, T = np.concatenate(xs), np.concatenate(ts)
    t2 = time.perf_counter()
    p, losses = rec.mlp_train(X, T, _lib.mlp_init(1), epochs=args.mlp_epochs, batch=4096, lr=2e-3, seed=3)
    t_train = time.perf_counter() - t2
    rec.close()
    log("mlp: hopper formed and settled in %.1f s (%d settling steps), %d samples over %d steps (%d converged) in "
        "%.1f s, trained in %.2f s, epoch losses %s" % (t1 - t0, settle, X.shape[0], args.mlp_record_steps, rec_conv,
                                                         t2 - t1, t_train, [round(x, 4) for x in losses]))
    out = {"workload": "hopper_%d" % args.mlp_hopper, "samples": int(X.shape[0]), "epochs": args.mlp_epochs,
           "train_s": t_train, "epoch_loss": [float(x) for x in losses], "settling_steps": settle,
           "form": "from the settled hopper's checkpoint, %d steps each, tol 1e-6, 5,000 sweeps at most, %s" % (
               args.mlp_eval_steps, "FP32 sweeps + FP64 checks and refinement" if args.precision == 1 else "FP64")}
    for name, use in (("cache", False), ("cache_or_network", True)):
        ctx = _lib.Context(device=local, dt=s["dt"], gravity=s["gravity"])
        ctx.restore(ck)
        ctx.reconfigure(precision=args.precision, max_iters=5000)
        if use:
            ctx.mlp_load(p)
            ctx.mlp_enable(warm_start=True)
        stream = torch.cuda.ExternalStream(ctx.stream_ptr(), device=local)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its, cs, conv, lerr, sweeps = 0, 0, 0, 0.0, []
        for j in range(args.mlp_eval_steps):
            st = ctx.step(1, first_iteration=it + j)
            its += st["iterations"]
            sweeps.append(st["iterations"])
            cs += st["n_contacts"]
            conv += int(st["succeeded"])
            lerr += float(np.log10(max(st["error"], 1e-300)))
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"sweeps": its, "sweeps_per_step": sweeps, "contact_steps": cs, "converged_steps": conv,
                     "ms": ms, "value": cs / (ms / 1e3), "unit": UNIT,
                     "mean_log10_residual": lerr / args.mlp_eval_steps}
        if use:
            out[name]["network_start_steps"] = ctx.mlp_stats()["network_start"]
        ctx.close()
    out["sweeps_saved_frac"] = 1.0 - out["cache_or_network"]["sweeps"] / max(out["cache"]["sweeps"], 1)
    out["speedup"] = out["cache_or_network"]["value"] / out["cache"]["value"] if out["cache"]["value"] else None
    return out


def parse_schedule(txt):
    """'600:50,300:200' -> [(600, 50), (300, 200)]: pre-roll phases of (steps, sweep cap)."""
    out = []
    for part in txt.split(","):
        if part.strip():
            a, b = part.split(":")
            out.append((int(a), int(b)))
    return out


def pile_note(info):
    return ("pre-roll %s steps:sweep cap, then %d settling steps at the full settings (%d converged, %s), "
            "then %d warm-up steps" % (",".join("%d:%d" % (p["steps"], p["sweep_cap"]) for p in info["phases"]),
                                      info["settle_steps"], info["settle_converged_steps"],
                                      "settled" if info["settled"] else "not settled within the limit",
                                      info["warmup_steps"]))


def form_pile(args, local):
    """The dense pile formed and settled on the GPU, untimed: pre-roll phases with capped sweeps
    (--schedule: the fill falls, impacts and compacts), then steps at the full settings (tol 1e-6,
    5,000 sweeps) until --settle-converged consecutive steps reach the tolerance (at most
    --settle-max steps), then --warmup steps.  Deterministic: the same arguments give the same state.
    Returns (context, scene, next step index, record)."""
    from scisim_gb300 import _lib
    s = make_scene(args.n)
    ctx = _lib.Context(device=local, cache_mode=_lib.CACHE_NORMAL_AND_FRICTION, precision=args.precision,
                       **solver_kw(s))
    ctx.upload_ball2d(s["q"], s["v"], s["r"], s["m"], s["plane_x"], s["plane_n"])
    it = 1
    t0 = time.perf_counter()
    phases = []
    for n, cap in parse_schedule(args.schedule):
        ctx.reconfigure(max_iters=cap)
        st = ctx.step(n, first_iteration=it)
        it += n
        phases.append({"steps": n, "sweep_cap": cap, "last_residual": st["error"]})
    ctx.reconfigure(max_iters=5000)
    t1 = time.perf_counter()
    run = settle = conv = 0
    while settle < args.settle_max and run < args.settle_converged:
        st = ctx.step(1, first_iteration=it)
        it += 1
        settle += 1
        run = run + 1 if st["succeeded"] else 0
        conv += int(st["succeeded"])
    t2 = time.perf_counter()
    for _ in range(args.warmup):
        ctx.step(1, first_iteration=it)
        it += 1
    info = {"phases": phases, "settle_steps": settle, "settle_converged_steps": conv,
            "settled": run >= args.settle_converged, "warmup_steps": args.warmup,
            "preroll_s": round(t1 - t0, 2), "settle_s": round(t2 - t1, 2)}
    log("pile formed: %s" % info)
    return ctx, s, it, info


def run_ours(args):
    import torch

    from scisim_gb300 import _lib

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    fast, s, it0, pile = form_pile(args, local)
    nb = s["r"].shape[0]
    stream = torch.cuda.ExternalStream(fast.stream_ptr(), device=local)
    # Profiling cases only (the headline keeps tol 1e-6 and the library's tuning): another tolerance
    # and fp64_factor for the steps after the formed pile.
    if args.tol is not None:
        fast.reconfigure(tol=args.tol)
    if args.fp64_factor is not None:
        fast.set_tuning(fp64_factor=args.fp64_factor)
    # The state every arm starts from: positions, velocities and the impulse cache (the last step's
    # contacts and impulses; a restored context has no last step, so this is read before the
    # autotuner's trials, which end by restoring this state).
    ck = fast.checkpoint()
    q_snap, v_snap = fast.state()
    cache = fast.last_contacts()
    # Autotuner: each candidate tuning timed over a few steps from this state, which it restores.
    autotune = None
    if args.autotune_steps > 0:
        t0 = time.perf_counter()
        chosen, tms = fast.autotune(trial_steps=args.autotune_steps, first_iteration=it0)
        autotune = {"trial_steps": args.autotune_steps, "chosen": chosen,
                    "ms_per_step": [None if np.isnan(x) else round(float(x), 3) for x in tms],
                    "candidates": "two-level on: check interval 8, 16, 32; two-level off: 8, 16, 32"}
        log("autotune in %.1f s: %s" % (time.perf_counter() - t0, autotune))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    fast.profile_enable(True)
    fast.profile_read(reset=True)
    clocks = ClockSampler(local)
    clocks.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # NVTX range "timed": lets a profiler select the timed launches (--nvtx-include "timed/").
    torch.cuda.nvtx.range_push("timed")
    ms, contacts, recs = timed_steps(fast, torch, stream, args.steps, flush, it0)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    prof = fast.profile_read(reset=True)
    total_ms = float(sum(ms))
    if ws > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    csteps = int(sum(contacts))
    value = csteps * ws / (total_ms / 1e3)
    convergence = convergence_record(recs)
    log("fast: %d contact-steps in %.1f ms; per step ms %s; %s; profile %s" % (
        csteps, total_ms, [round(x, 2) for x in ms], convergence, prof))
    roofline, stages = headline_roofline(prof, total_ms, args, [r["sweeps"] for r in recs])

    def arm(**over):
        c = _lib.Context(device=local, **solver_kw(s))
        c.restore(ck)
        c.reconfigure(**over)
        c.profile_enable(True)
        c.profile_read(reset=True)
        return c

    # Plain FP64 Gauss-Seidel from the same state: with the impulse cache, then cold (one step,
    # a larger sweep cap).
    plain = plain_cold = None
    plain_steps = args.steps if args.plain_steps is None else args.plain_steps
    if plain_steps > 0:
        pctx = arm(precision=_lib.PRECISION_FP64)
        pms, pc, precs = timed_steps(pctx, torch, torch.cuda.ExternalStream(pctx.stream_ptr(), device=local),
                                     plain_steps, flush, it0)
        pst = pctx.profile_read()
        plain = {"value": sum(pc) / (sum(pms) / 1e3), "unit": UNIT, "steps": plain_steps,
                 "ms_per_step": sum(pms) / len(pms), "convergence": convergence_record(precs),
                 "form": "FP64 sweeps, warm start from the impulse cache, same state and steps"}
        log("plain FP64 (cache):", plain)
        pctx.close()
    if args.cold_steps > 0:
        cctx = arm(precision=_lib.PRECISION_FP64, cache_mode=_lib.CACHE_NONE, max_iters=args.cold_iters)
        cms, cc, crecs = timed_steps(cctx, torch, torch.cuda.ExternalStream(cctx.stream_ptr(), device=local),
                                     args.cold_steps, flush, it0)
        plain_cold = {"value": sum(cc) / (sum(cms) / 1e3), "unit": UNIT, "steps": args.cold_steps,
                      "ms_per_step": sum(cms) / len(cms), "max_iters": args.cold_iters,
                      "convergence": convergence_record(crecs),
                      "form": "FP64 sweeps, cold start (no impulse cache), sweep cap %d, same state" %
                              args.cold_iters}
        log("plain FP64 (cold):", plain_cold)
        cctx.close()

    # The FP32 form against FP64 from the timed state: as run (the start's residual picks FP64
    # sweeps near tol), and with FP32 sweeps from the first sweep.
    form_err = None
    if args.form_error:
        form_err = {"as_run": fp32_form_error(ck, s, it0, local),
                    "fp32_sweeps_from_start": fp32_form_error(ck, s, it0, local, fp64_factor=0)}
        log("fp32 form error:", form_err)

    # e2e through sg_flow with pinned host buffers, from the same state and impulse cache.
    e2e = None
    e2e_steps = args.steps if args.e2e_steps is None else args.e2e_steps
    if e2e_steps > 0:
        ectx = arm()
        bufs = [torch.empty(2 * nb, dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
        bufs[0][:] = q_snap
        bufs[1][:] = v_snap
        it = it0
        torch.cuda.synchronize()
        ec, econv, eerr = 0, 0, 0.0
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            _, _, st = ectx.flow(it, bufs[0], bufs[1], bufs[2], bufs[3])
            bufs = [bufs[2], bufs[3], bufs[0], bufs[1]]
            ec += st["n_contacts"]
            econv += int(st["succeeded"])
            eerr = max(eerr, st["error"])
            it += 1
        el = time.perf_counter() - t0
        e2e = {"value": ec / el, "unit": UNIT, "h2d_bytes_per_step": 2 * 16 * nb, "d2h_bytes_per_step": 2 * 16 * nb,
               "steps": e2e_steps, "steps_converged": econv, "max_residual": eerr,
               "api": "sg_flow (ImpactFrictionMap::flow), pinned host q/v, from the timed steps' state and cache"}
        log("e2e:", e2e)
        ectx.close()

    batched = None
    if args.batch_scenes > 0:
        batched = batch_leg(args, torch, local, flush, ws, rank)
        if rank == 0:
            log("batched:", batched)
    learned = None
    if rank == 0 and args.mlp_hopper > 0:
        learned = mlp_leg(args, torch, local)
        log("learned:", learned)
    spheres = None
    if rank == 0 and args.spheres > 0:
        spheres = sphere_leg(args, torch, local, flush)
        log("spheres:", spheres)
    sphere_batch = None
    if rank == 0 and args.sphere_batch_scenes > 0:
        sphere_batch = sphere_batch_leg(args, torch, local, flush)
        log("sphere batch:", sphere_batch)

    cpu = None
    if rank == 0 and args.cpu_steps > 0:
        v, desc, crecs = cpu_from_state(s, q_snap, v_snap, cache, args.cpu_steps, it0, args.cpu_budget)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": desc}
        log("cpu:", cpu)

    if rank == 0:
        timed0 = it0
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == 0 else "f32+f64",
                "data": "synthetic (seeded dense-pile fill, no dataset)",
                "config": {"workload": "ball2d_dense_pile_%d" % nb, "discs": nb, "box": [40, 60], "dt": s["dt"],
                           "mu": s["mu"], "CoR": s["CoR"], "tol": args.tol if args.tol is not None else 1e-6,
                           "max_iters": 5000,
                           "form": ("warm start (impulse cache), FP32 form: an FP64 probe of up to eight sweeps, then FP64 sweeps "
                                    "on the two-level partition near tol or FP32 sweeps with FP64 checks further "
                                    "away" if args.precision == 1 else "warm start (impulse cache), FP64 sweeps"),
                           "pile": pile_note(pile), "timed_steps": [timed0, timed0 + args.steps - 1],
                           "l2": "flushed between timed steps (256 MB write)",
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "convergence": convergence, "pile": pile,
                "contacts_per_step": csteps / args.steps,
                "gs_iterations_per_step": (prof["contact_sweeps"] + prof["contact_sweeps32"]) / max(csteps, 1),
                "fp32_sweep_share": prof["contact_sweeps32"] / max(prof["contact_sweeps"] + prof["contact_sweeps32"], 1),
                "fp64_start_solves": prof["fp64_start_solves"], "stage_ms_per_step": stages,
                "plain_fp64_gpu": plain,
                "warm_over_plain": (value / ws) / plain["value"] if plain and plain["steps"] == args.steps else None,
                "plain_fp64_cold_gpu": plain_cold, "fp32_form_error": form_err,
                "warm_over_plain_cold": (value / ws) / plain_cold["value"] if plain_cold else None,
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": prof["kernel_launches"], "autotune": autotune, "batched": batched,
                "spheres": spheres, "sphere_batch": sphere_batch, "learned": learned}
        print(json.dumps(line), flush=True)
    fast.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--autotune-steps", type=int, default=2, help="steps per autotuner candidate (0 = off)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=262144)
    ap.add_argument("--schedule", default="600:50,300:200,200:1000",
                    help="pre-roll phases steps:sweep cap of the pile (untimed)")
    ap.add_argument("--settle-converged", type=int, default=10,
                    help="settling ends after this many consecutive converged steps at the full settings")
    ap.add_argument("--settle-max", type=int, default=200, help="settling steps at most")
    ap.add_argument("--preroll-iters", type=int, default=50, help="sweep cap of the other legs' pre-rolls")
    ap.add_argument("--plain-steps", type=int, default=None,
                    help="steps of the plain FP64 arm (default: --steps, the timed steps themselves)")
    ap.add_argument("--cold-steps", type=int, default=1)
    ap.add_argument("--cold-iters", type=int, default=20000)
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="steps of the e2e leg (default: --steps, the timed steps themselves)")
    ap.add_argument("--form-error", type=int, default=1, help="FP32-form vs FP64 error from the timed state (0 = skip)")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--cpu-budget", type=float, default=60.0,
                    help="seconds of oracle stepping after which the CPU legs start no further step")
    ap.add_argument("--precision", type=int, default=1, help="0 = FP64 sweeps, 1 = FP32 sweeps + FP64 refinement")
    ap.add_argument("--tol", type=float, default=None,
                    help="profiling cases: tolerance of the steps after the formed pile (default: 1e-6 throughout)")
    ap.add_argument("--fp64-factor", type=int, default=None,
                    help="profiling cases: the FP32 form's fp64_factor for those steps (default: the library's)")
    ap.add_argument("--batch-scenes", type=int, default=4096, help="batched-scene leg (0 = skip)")
    ap.add_argument("--batch-preroll", type=int, default=40)
    ap.add_argument("--batch-steps", type=int, default=8)
    ap.add_argument("--batch-plain-scenes", type=int, default=16)
    ap.add_argument("--spheres", type=int, default=65536, help="sphere leg (0 = skip)")
    ap.add_argument("--sphere-preroll", type=int, default=800,
                    help="capped pre-roll steps of the sphere leg (the 65,536-sphere pile forms in ~600)")
    ap.add_argument("--sphere-steps", type=int, default=3)
    ap.add_argument("--sphere-batch-scenes", type=int, default=256, help="sphere-batch leg (0 = skip)")
    ap.add_argument("--sphere-batch-preroll", type=int, default=100)
    ap.add_argument("--sphere-batch-steps", type=int, default=3)
    ap.add_argument("--mlp-hopper", type=int, default=262144, help="learned-warm-start study on a hopper (0 = skip)")
    ap.add_argument("--mlp-schedule", default="800:50,300:200,200:1000",
                    help="pre-roll phases steps:sweep cap of the hopper (untimed)")
    ap.add_argument("--mlp-record-steps", type=int, default=30)
    ap.add_argument("--mlp-epochs", type=int, default=6)
    ap.add_argument("--mlp-eval-steps", type=int, default=20)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
