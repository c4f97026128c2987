"""Benchmark of the OSIRIS PIC time step on GB300: particle-steps/s of the 2D two-stream
workload (512 x 512 cells, two electron species x 32 particles per cell drifting at +-0.2 c,
uth = 0.01 c, 1e-3 density perturbation, quadratic splines, dx = 0.05, dt = 0.035), mixed
precision (FP32 particles and fields) on the tiled engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

One step = one full time step (guard replace, push + deposit + tile migration of both species,
current fold, Yee B/2-E-B/2), replayed from a CUDA graph.  Particle data (16.8 M particles,
537 MB per buffer) is far larger than L2, so no flush is needed between steps.

JSON line keys beyond the base contract:
  roofline      the push kernel (dominant): algorithmic bytes per launch / its CUDA-event time,
                the mean of 5 launches timed right before and 5 right after the timed steps
  cpu_baseline  the CPU oracle port on this host's cores, on a bounded sample of the workload
  e2e           the same metric through the reference-facing host-array C ABI
                (osg_vadvance_deposit_f32 per species, osg_periodic, osg_yee_advance) on pinned
                host buffers, every copy inside the timed region
  fp64_plain    the plain FP64 engine on the same workload (the "plain FP64 GPU form")
  fp64_error    normwise difference of E, B, J and the relative difference of the kinetic and
                field energies between the mixed-precision (tiled FP32) and the plain FP64
                engine after the same number of steps from the same load
  run_to_run    normwise difference of E, B, J between two identical runs of the tiled engine
  other_configs the other benchmark configurations (thermal 128^2 FP64, Weibel 128^3, 64
                batched boxes, laser wakefield with the moving window), each timed on this
                GPU with CUDA events (ms per step, particle-steps/s) with its push kernel's
                algorithmic bytes / CUDA-event time against the measured HBM peak, and the
                single-box autotuner's choice for this workload (--no-other-configs skips them)
--impl reference times the CPU oracle port (the reference's CPU path restated; the
reference's own AVX2 kernels do not build on this Arm host) with all host threads.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="2D two-stream 512x512, 2 species x 32 ppc, quadratic, FP32 mixed",
                nx=[512, 512], ppc=[8, 4], dx=[0.05, 0.05], dt=0.035, uth=0.01, ufl=0.2,
                amp=1e-3, order=2, seed=2)
METRIC = "particle-steps/s"
# algorithmic bytes (FP32 2D): particle read 32 B + write 28 B; per cell E,B gather 24 B + J 12 B
BYTES_PER_PARTICLE = 60
BYTES_PER_CELL_PUSH = 36


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one full-size push launch of this
# workload, from one ncu capture (one metric pass, --clock-control none) of the current kernel;
# the command and the figures are in profiles/push_tiled_c2.md.  None when no capture matches
# the kernel as built.
PUSH_TRAFFIC_BYTES = 1115267840


class Clocks:
    """nvidia-smi sampler for the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_species(osg, prec):
    w = WORKLOAD
    r = osg.Rng(w["seed"])
    return [osg.load_lattice(r, prec, w["nx"], w["ppc"], w["dx"], -1.0, [w["uth"]] * 3,
                             [s * w["ufl"], 0.0, 0.0], w["amp"], 1.0) for s in (1.0, -1.0)]


def cpu_oracle_rate(target_s, nthreads, steps=None):
    """CPU oracle (port) particle-steps/s on a square sub-box of the workload (same density,
    parameters and phases), sized so the timed part takes about target_s seconds."""
    from oracle import pyoracle as po
    po.build(with_ref=False)
    w = WORKLOAD

    def setup(n):
        r = po.mt_new(w["seed"])
        sp = []
        for s in (1.0, -1.0):
            ix, x, u, q = po.load(r, "f32", 2, [n, n], w["ppc"], w["dx"], -1.0, [w["uth"]] * 3,
                                  [s * w["ufl"], 0.0, 0.0], w["amp"], 1.0)
            sp.append(dict(ix=ix, x=x, u=u, q=q, rqm=-1.0))
        g = po.Grid([n, n], w["order"], w["dx"])
        return g, sp, g.zeros("f32"), g.zeros("f32"), g.zeros("f32")

    g, sp, e, b, j = setup(64)
    t = time.perf_counter()
    po.step(g, "f32", e, b, j, sp, w["dt"], nthreads=nthreads, fast=True)
    rate = 2 * 64 * 64 * 32 / (time.perf_counter() - t)
    nstep = steps or 3
    n = int(np.sqrt(rate * target_s / nstep / 64))
    n = max(32, min(512, n // 16 * 16))
    g, sp, e, b, j = setup(n)
    npart = sum(len(s["q"]) for s in sp)
    po.step(g, "f32", e, b, j, sp, w["dt"], nthreads=nthreads, fast=True)
    t = time.perf_counter()
    for _ in range(nstep):
        po.step(g, "f32", e, b, j, sp, w["dt"], nthreads=nthreads, fast=True)
    el = time.perf_counter() - t
    return npart * nstep / el, f"{n}x{n} cells ({npart} particles), {nstep} full steps", el


def cpu_config_rate(cfg, prec, nthreads, target_s, steps=2):
    """CPU oracle (port) particle-steps/s of another configuration (its density, parameters
    and phases) on a cubic sub-box no larger than the configuration's, sized so the timed part
    takes about target_s seconds.  Returns (rate, sample description)."""
    from oracle import pyoracle as po
    po.build(with_ref=False)
    dim = len(cfg["nx"])
    p = "f32" if prec == 32 else "f64"

    def setup(n):
        nx = [min(n, m) for m in cfg["nx"]]
        r = po.mt_new(cfg["seed"])
        sp = []
        for s in cfg["species"]:
            ix, x, u, q = po.load(r, p, dim, nx, cfg["ppc"], cfg["dx"], -1.0, [s["uth"]] * 3,
                                  s["ufl"], cfg["amp"], 1.0)
            sp.append(dict(ix=ix, x=x, u=u, q=q, rqm=-1.0))
        g = po.Grid(nx, cfg["order"], cfg["dx"])
        return nx, g, sp, g.zeros(p), g.zeros(p), g.zeros(p)

    n0 = 16 if dim == 3 else 64
    nx, g, sp, e, b, j = setup(n0)
    npart = sum(len(s["q"]) for s in sp)
    t = time.perf_counter()
    po.step(g, p, e, b, j, sp, cfg["dt"], nthreads=nthreads, fast=True)
    per = (time.perf_counter() - t) / npart
    n = int((target_s / steps / per / (npart / n0 ** dim)) ** (1.0 / dim))
    n = max(n0, n // 8 * 8)
    nx, g, sp, e, b, j = setup(n)
    npart = sum(len(s["q"]) for s in sp)
    po.step(g, p, e, b, j, sp, cfg["dt"], nthreads=nthreads, fast=True)
    t = time.perf_counter()
    for _ in range(steps):
        po.step(g, p, e, b, j, sp, cfg["dt"], nthreads=nthreads, fast=True)
    el = time.perf_counter() - t
    cells = "x".join(str(v) for v in nx)
    return npart * steps / el, f"{cells} cells ({npart} particles), {steps} full steps"


def e2e_host(osg, sp_host, steps):
    """Drop-in flow on host buffers (osiris_gb300.run.dropin_steps), all copies timed."""
    from osiris_gb300.run import dropin_steps
    w = WORKLOAD
    return dropin_steps(sp_host, w["nx"], w["dx"], w["dt"], w["order"], steps)


def run_native(args):
    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = (torch, tdist)
    import __graft_entry__ as ge
    ge.build_native()
    import osiris_gb300 as osg
    osg.set_device(local)
    w = WORKLOAD
    sp = load_species(osg, 32)
    npart = sum(len(s[3]) for s in sp)
    ncell = int(np.prod(w["nx"]))
    # slabs of 4x the mean tile load: the two-stream instability bunches particles up to
    # ~2.4x the mean per 8x8 tile around saturation, and the timed region has no re-binning
    sim = osg.Simulation(w["nx"], w["dx"], w["dt"], order=w["order"], precision=32,
                         engine=osg.ENGINE_TILED, capacity=4.0)
    for s in sp:
        sim.add_species(-1.0, *s)
    sim.step(args.warmup)
    # the push kernel's CUDA-event time right before the timed region (the beams are still cold:
    # few cell crossings) and right after it (heated: more); the roofline uses their mean, the
    # push time averaged over the timed region, which grows monotonically between the two
    prof0 = sim.profile(5)
    if dist:
        dist[1].barrier()
    with Clocks(local) as clk:
        ms = sim.time_steps(args.steps)
    if dist:
        t = dist[0].tensor([ms], device="cuda")
        dist[1].all_reduce(t, op=dist[1].ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * npart * args.steps / (ms / 1e3)
    prof = sim.profile(5)
    push_ms = 0.5 * (prof0["push"] + prof["push"])
    launches = sim.launches_per_step() * args.steps
    kin, fld = sim.energy()
    occupancy = sim.tile_occupancy()
    sim.close()
    if rank != 0:
        if dist:
            dist[1].destroy_process_group()
        return
    peak, peak_kind = peaks()
    push_bytes = npart * BYTES_PER_PARTICLE + ncell * BYTES_PER_CELL_PUSH
    achieved = push_bytes / (push_ms * 1e-3) / 1e9
    traffic = PUSH_TRAFFIC_BYTES
    # plain FP64 GPU form on the same workload
    sp64 = load_species(osg, 64)
    sim64 = osg.Simulation(w["nx"], w["dx"], w["dt"], order=w["order"], precision=64,
                           engine=osg.ENGINE_PLAIN, n_sort=25)
    for s in sp64:
        sim64.add_species(-1.0, *s)
    sim64.step(3)
    n64 = max(10, min(args.steps, 50))
    ms64 = sim64.time_steps(n64)
    v64 = npart * n64 / (ms64 / 1e3)
    # error of the mixed-precision result against the FP64 build: the tiled FP32 engine from
    # the same load, run for the same number of steps as the FP64 engine above
    n_err = 3 + n64
    sim32 = osg.Simulation(w["nx"], w["dx"], w["dt"], order=w["order"], precision=32,
                           engine=osg.ENGINE_TILED, capacity=4.0)
    for s in sp:
        sim32.add_species(-1.0, *s)
    sim32.step(n_err)
    # run-to-run spread of the mixed-precision engine: the same load and steps again (the tile
    # sums are deterministic; the in-tile particle order, which follows the arrival order of
    # migrating particles, is not, and the FP32 run sums follow it)
    sim32b = osg.Simulation(w["nx"], w["dx"], w["dt"], order=w["order"], precision=32,
                            engine=osg.ENGINE_TILED, capacity=4.0)
    for s in sp:
        sim32b.add_species(-1.0, *s)
    sim32b.step(n_err)
    spread = {"steps": n_err, "norm": "max|run1 - run2| / max|run2| over the grid"}
    for name, a, b in zip("EBJ", sim32.fields(), sim32b.fields()):
        spread[name] = float(np.abs(a.astype(np.float64) - b).max() / np.abs(b).max())
    sim32b.close()
    fp64_error = {"steps": n_err, "norm": "max|mixed - fp64| / max|fp64| over the grid"}
    f32, f64 = sim32.fields(), sim64.fields()
    for name, a, b in (("E", f32[0], f64[0]), ("B", f32[1], f64[1]), ("J", f32[2], f64[2])):
        fp64_error[name] = float(np.abs(a.astype(np.float64) - b).max() / np.abs(b).max())
    k32, fl32 = sim32.energy()
    k64, fl64 = sim64.energy()
    fp64_error["kinetic"] = float(abs(k32.sum() - k64.sum()) / abs(k64.sum()))
    fp64_error["field"] = float(abs(fl32.sum() - fl64.sum()) / abs(fl64.sum()))
    sim32.close()
    sim64.close()
    # end to end through the host-array C ABI
    e2e_v, h2d, d2h, e2e_steps = e2e_host(osg, sp, max(3, min(args.steps, 10)))
    # CPU baseline (oracle port) on rank 0
    from oracle import pyoracle as po
    nthr = po.max_threads()
    cpu_v, cpu_sample, _ = cpu_oracle_rate(15.0, nthr)
    others = None if args.no_other_configs or world > 1 else other_configs(osg, peak)
    if others is not None:
        # the CPU baselines the other configurations are reported with: configuration 1 (FP64)
        # on one thread and on all, configuration 3 (FP32) on all
        from osiris_gb300 import run as orun
        cb = {}
        for key, name, prec, thr in (("thermal_1_thread", "thermal", 64, 1),
                                     ("thermal_all_threads", "thermal", 64, nthr),
                                     ("weibel_all_threads", "weibel", 32, nthr)):
            v, smp = cpu_config_rate(orun.CONFIGS[name], prec, thr, 6.0)
            cb[key] = {"value": v, "unit": METRIC, "cores": thr, "kind": "port", "sample": smp}
        others["cpu_baseline"] = cb
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["workload"], "cells": w["nx"], "particles": npart,
                   "species": 2, "ppc_per_species": 32, "interpolation": "quadratic",
                   "dx": w["dx"], "dt": w["dt"], "engine": "tiled", "graph": True,
                   "l2": "inputs larger than L2 (537 MB particle buffer per step)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "kernel": "k_push_tiled<2,2>", "traffic": traffic,
                     "algorithmic_bytes_per_launch": push_bytes,
                     "launch_ms": push_ms,
                     "launch_ms_before_timed_steps": prof0["push"],
                     "launch_ms_after_timed_steps": prof["push"]},
        "phase_ms": prof,
        "cpu_baseline": {"value": cpu_v, "unit": METRIC, "cores": nthr, "kind": "port",
                         "sample": cpu_sample},
        "e2e": {"value": e2e_v, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                "path": "osg_vadvance_deposit_f32 + osg_particle_wrap per species, "
                        "osg_periodic x3, osg_yee_advance; pinned host buffers"},
        "fp64_plain": {"value": v64, "unit": METRIC, "steps": n64,
                       "ratio_mixed_over_fp64": value / world / v64},
        "fp64_error": fp64_error,
        "run_to_run": spread,
        "other_configs": others,
        "gpu_launches": launches,
        "tile_occupancy_max": occupancy,
        "clocks": clk.summary(),
        "energy": {"kinetic": [float(v) for v in kin], "field": [float(v) for v in fld]},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist[1].destroy_process_group()


# algorithmic push bytes: per particle (read + write) and per cell (E, B gathered, J)
PUSH_BYTES = {("tiled", 2): (60, 36), ("tiled", 3): (76, 36), ("plain64", 2): (104, 72)}


def other_configs(osg, peak):
    """The other benchmark configurations, timed on this GPU: ms per step and particle-steps/s
    over a few graph steps after a warm-up, the push phase's device time (osg_sim_profile) and
    its algorithmic bytes per launch against the measured HBM peak."""
    from osiris_gb300 import run as orun
    out = {}

    def push_roof(kind, dim, npart, ncell, push_ms):
        bp, bc = PUSH_BYTES[(kind, dim)]
        ach = (npart * bp + ncell * bc) / (push_ms * 1e-3) / 1e9
        return {"push_ms": push_ms, "achieved_gbs": ach, "frac": ach / peak}

    for name, steps, warm in (("thermal", 50, 5), ("weibel", 20, 3)):
        cfg = orun.CONFIGS[name]
        sim, npart = orun.build_sim(cfg)
        sim.step(warm)
        ms = sim.time_steps(steps)
        prof = sim.profile(3)
        ncell = int(np.prod(cfg["nx"]))
        kind = "plain64" if cfg["precision"] == 64 else "tiled"
        out[name] = {"cells": cfg["nx"], "particles": npart, "steps": steps,
                     "ms_per_step": ms / steps, "particle_steps_per_s": npart * steps / (ms / 1e3),
                     "engine": cfg["engine"], "precision": cfg["precision"],
                     **push_roof(kind, len(cfg["nx"]), npart, ncell, prof["push"])}
        sim.close()
    # the single-box autotuner on the benchmark workload itself (its choice; the timed run
    # above uses the default 8x8 tiles and 256 threads)
    sim, npart = orun.build_sim(orun.CONFIGS["two_stream"])
    out["autotune_two_stream"] = sim.autotune(steps=4)
    sim.close()
    bt, npart = orun.build_batch()
    tile, threads = bt.tuning()
    bt.step(3)
    ms = bt.time_steps(20)
    out["batch"] = {"boxes": 64, "particles": npart, "steps": 20, "ms_per_step": ms / 20,
                    "particle_steps_per_s": npart * 20 / (ms / 1e3), "tile": tile,
                    "threads": threads}
    bt.close()
    sim, n0 = orun.build_lwfa()
    sim.step(3)
    ms = sim.time_steps(25)
    n1 = sim.num_particles(0)
    out["lwfa"] = {"cells": orun.LWFA["nx"], "particles_start": n0, "particles_end": n1,
                   "steps": 25, "ms_per_step": ms / 25,
                   "particle_steps_per_s": n1 * 25 / (ms / 1e3),
                   "window_moves": sim.window_moves(), "note": "the first steps of the run"}
    sim.close()
    return out


def run_reference(args):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    from oracle import pyoracle as po
    po.build(with_ref=False)
    nthr = po.max_threads()
    # each step of this arm is a bounded sample: a sub-box of the workload sized so that the
    # whole --steps run takes about two minutes
    budget = 120.0
    v, sample, el = cpu_oracle_rate(budget, nthr, steps=args.steps)
    ms_step = el / args.steps * 1e3
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": _env_int("WORLD_SIZE", 1),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD["workload"], "sample": sample},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": nthr, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the timing of the other benchmark configurations")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_native(args)


if __name__ == "__main__":
    main()
