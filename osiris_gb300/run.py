"""Command-line runner of the device-resident simulation on the benchmark workloads.

    python -m osiris_gb300.run --config two_stream [--nx 128 128] [--steps 10] [--engine tiled]

Configurations (seeded OSIRIS lattice load, periodic box, electrons only over a fixed
neutralising background):
  thermal     2D 128x128, 16 ppc, uth 0.1, quadratic, dx 0.05, dt 0.035          (FP64 plain)
  two_stream  2D 512x512, 2 x 32 ppc, +-0.2 c drift, uth 0.01, 1e-3 perturbation  (FP32 tiled)
  weibel      3D 128^3, 2 x 8 ppc, +-0.5 c along z, uth 0.05, cubic, dx 0.1, dt 0.05
  lwfa        3D laser wakefield with a moving window: 1024 x 128 x 128 cells, dx 0.2,
              dy = dz = 0.6 c/w0, dt 0.18, 2 ppc electrons at n = 0.01 n_c (w_p = 0.1 w0)
              after a 50-cell linear ramp starting at x1 = 150, a0 = 2 Gaussian pulse (waist
              30, duration 10, centred at x1 = 130, focused at the ramp's end), cubic splines,
              window moving at c (--nx scales the box)
  batch       64 independent 2D thermal boxes in one batched engine: sizes drawn from
              {64^2, 128^2, 256^2, 512^2}, ppc from {4, 16, 64}, uth uniform in [0.01, 0.2]
              (MT19937 seed 4), quadratic, dx 0.05, dt 0.035, tile shape and CTA size
              autotuned (--boxes N takes the first N boxes)
Prints one JSON line per run with the device time per step and the energies; --fp64-check
adds the error of a mixed-precision run against the plain FP64 engine (same load, same
steps).  --dropin (2D
configurations) times the host-array drop-in flow instead, as an unchanged OSIRIS host drives
it: per species osg_vadvance_deposit_f32 and the particle wrap, guard updates and Yee on host
arrays, every copy included.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import osiris_gb300 as osg

CONFIGS = {
    "thermal": dict(nx=[128, 128], ppc=[4, 4], dx=[0.05, 0.05], dt=0.035, order=2,
                    species=[dict(uth=0.1, ufl=[0.0, 0.0, 0.0])], amp=0.0, precision=64,
                    engine="plain", seed=1),
    "two_stream": dict(nx=[512, 512], ppc=[8, 4], dx=[0.05, 0.05], dt=0.035, order=2,
                       species=[dict(uth=0.01, ufl=[0.2, 0.0, 0.0]),
                                dict(uth=0.01, ufl=[-0.2, 0.0, 0.0])],
                       amp=1e-3, precision=32, engine="tiled", seed=2),
    "weibel": dict(nx=[128, 128, 128], ppc=[2, 2, 2], dx=[0.1, 0.1, 0.1], dt=0.05, order=3,
                   species=[dict(uth=0.05, ufl=[0.0, 0.0, 0.5]),
                            dict(uth=0.05, ufl=[0.0, 0.0, -0.5])],
                   amp=0.0, precision=32, engine="tiled", seed=3),
}


def build_sim(cfg, engine=None, precision=None, tile=None, nx=None):
    nx = nx or cfg["nx"]
    dim = len(nx)
    precision = precision or cfg["precision"]
    engine = engine or cfg["engine"]
    eng = osg.ENGINE_TILED if engine == "tiled" else osg.ENGINE_PLAIN
    sim = osg.Simulation(nx, cfg["dx"][:dim], cfg["dt"], order=cfg["order"], precision=precision,
                         engine=eng, tile=tile, n_sort=25 if eng == osg.ENGINE_PLAIN else 0)
    r = osg.Rng(cfg["seed"])
    n = 0
    for s in cfg["species"]:
        ix, x, u, q = osg.load_lattice(r, precision, nx, cfg["ppc"][:dim], cfg["dx"][:dim], -1.0,
                                       [s["uth"]] * 3, s["ufl"], cfg["amp"], 1.0)
        sim.add_species(-1.0, ix, x, u, q)
        n += len(q)
    return sim, n


LWFA = dict(nx=[1024, 128, 128], dx=[0.2, 0.6, 0.6], dt=0.18, order=3, ppc=[2, 1, 1],
            n0=0.01, ramp_start=150.0, ramp_cells=50, a0=2.0, w0=30.0, duration=10.0,
            x0=130.0)


def build_lwfa(nx=None, tile=None, pml=False):
    """The laser-wakefield workload: seeded lattice load of the plasma already inside the box
    (density from the profile), the pulse launched into E/B, the window set.  pml=True: PML
    walls on the transverse axes (moving with the window) instead of periodic ones."""
    c = LWFA
    nx = nx or c["nx"]
    dx = c["dx"]
    ramp_end = c["ramp_start"] + c["ramp_cells"] * dx[0]
    px, pf = [c["ramp_start"], ramp_end, 1e9], [0.0, c["n0"], c["n0"]]
    sim = osg.Simulation(nx, dx, c["dt"], order=c["order"], precision=32,
                         engine=osg.ENGINE_TILED, tile=tile, pml=6 if pml else 0)
    gl, gu = osg.GUARD[c["order"]]
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape, np.float32), np.zeros(shape, np.float32)
    osg.zpulse_launch(c["order"], nx, dx, [0.0] * 3, e, b, omega0=1.0, a0=c["a0"], pol=0.0,
                      lon_x0=c["x0"], lon_duration=c["duration"], lon_range=4 * c["duration"],
                      per_w0=c["w0"], per_focus=ramp_end,
                      per_center=(nx[1] * dx[1] / 2, nx[2] * dx[2] / 2))
    sim.set_fields(e, b)
    ix, x, u, q = osg.load_lattice(osg.Rng(5), 32, nx, c["ppc"], dx, -1.0, [0.0] * 3,
                                   [0.0] * 3)
    xg = (ix[:, 0].astype(np.float64) - 0.5 + x[:, 0].astype(np.float64)) * dx[0]
    den = np.interp(xg, px, pf, left=0.0, right=c["n0"]).astype(np.float32)
    keep = den > 0
    sim.add_species(-1.0, np.ascontiguousarray(ix[keep]), np.ascontiguousarray(x[keep]),
                    np.ascontiguousarray(u[keep]), np.ascontiguousarray(q[keep] * den[keep]))
    sim.set_window(0, c["ppc"], px, pf)
    return sim, int(keep.sum())


def batch_boxes(nbox=64, seed=4):
    """The 64 box specifications of the batched workload: (nx, ppc per axis, uth)."""
    r = np.random.RandomState(seed)
    sizes = [64, 128, 256, 512]
    ppcs = {4: [2, 2], 16: [4, 4], 64: [8, 8]}
    out = []
    for _ in range(nbox):
        n = sizes[r.randint(len(sizes))]
        ppc = [4, 16, 64][r.randint(3)]
        uth = float(r.uniform(0.01, 0.2))
        out.append(([n, n], ppcs[ppc], uth))
    return out


def build_batch(nbox=64, tile=None, threads=0):
    """The batched thermal workload (one electron species per box over a fixed ion
    background), seeded OSIRIS lattice load per box."""
    bt = osg.Batch(2, 2, 0.035, tile=tile, threads=threads)
    n = 0
    for i, (nx, ppc, uth) in enumerate(batch_boxes()[:nbox]):
        k = bt.add_box(nx, [0.05, 0.05])
        r = osg.Rng(1000 + i)
        ix, x, u, q = osg.load_lattice(r, 32, nx, ppc, [0.05, 0.05], -1.0, [uth] * 3,
                                       [0.0, 0.0, 0.0])
        bt.add_species(k, -1.0, ix, x, u, q)
        n += len(q)
    return bt, n


def dropin_steps(sp_host, nx, dx, dt, order, steps, pinned=True):
    """Drop-in flow on host buffers, as an unchanged OSIRIS host would drive the library: field
    guard replace, per species osg_vadvance_deposit_f32 and the periodic particle boundary,
    current fold and Yee through the host-array C ABI (2D, FP32; every copy inside the timed
    part).  sp_host: per species (ix, x, u, q) host arrays, rqm -1.  Returns particle-steps/s,
    the host-to-device and device-to-host bytes per step (counted from the arrays each call
    copies) and the number of timed steps.  pinned=False keeps the particles in ordinary
    (pageable) host memory, as a Fortran host allocates them."""
    gl, gu = osg.GUARD[order]
    size = [n + gl + gu for n in nx]
    shape = tuple(reversed(size)) + (3,)
    e = osg.pinned_empty(shape, np.float32)
    b = osg.pinned_empty(shape, np.float32)
    j = osg.pinned_empty(shape, np.float32)
    e[...] = 0
    b[...] = 0
    pin = []
    for ix, x, u, q in sp_host:
        arrs = []
        for a in (ix, x, u, q):
            p = osg.pinned_empty(a.shape, a.dtype) if pinned else np.empty_like(a)
            p[...] = a
            arrs.append(p)
        pin.append(arrs)
    npart = sum(len(s[3]) for s in sp_host)
    gbytes = int(np.prod(shape)) * 4

    def one_step():
        osg.periodic(2, nx, [gl] * 2, [gu] * 2, e, 0)
        osg.periodic(2, nx, [gl] * 2, [gu] * 2, b, 0)
        j[...] = 0
        for ix, x, u, q in pin:
            osg.vadvance_deposit(2, order, ix, x, u, q, 1, len(q), -1.0, e, b, size, [gl] * 2, j,
                                 size, [gl] * 2, dx, dt)
            osg.particle_wrap(nx, ix)
        osg.periodic(2, nx, [gl] * 2, [gu] * 2, j, 1)
        osg.yee_advance(2, nx, [gl] * 2, [gu] * 2, e, b, j, dx, dt)

    one_step()
    t = time.perf_counter()
    for _ in range(steps):
        one_step()
    el = time.perf_counter() - t
    # bytes moved per step (counted from the arrays each call copies)
    h2d = 2 * gbytes + sum(len(p[3]) * 32 + 3 * gbytes for p in pin) + gbytes + 3 * gbytes
    d2h = 2 * gbytes + sum(len(p[3]) * 28 + gbytes + 12 for p in pin) + gbytes + 2 * gbytes
    for arrs in pin if pinned else ():
        for a in arrs:
            osg.pinned_free(a)
    for a in (e, b, j):
        osg.pinned_free(a)
    return npart * steps / el, h2d, d2h, steps


def run_batch(args):
    t0 = time.time()
    bt, npart = build_batch(args.boxes, args.tile, args.threads or 0)
    t_load = time.time() - t0
    t0 = time.time()
    tile, threads = bt.tuning()
    t_tune = time.time() - t0
    bt.step(args.warmup)
    ms = bt.time_steps(args.steps)
    print(json.dumps(dict(config="batch", boxes=args.boxes, particles=npart, steps=args.steps,
                          ms_per_step=ms / args.steps,
                          particle_steps_per_s=npart * args.steps / (ms / 1e3),
                          launches_per_step=bt.launches_per_step(), tile=tile,
                          threads=threads, load_s=t_load, tune_s=t_tune)))
    bt.close()


def fp64_error(cfg, sim, args):
    """Error of a mixed-precision run against the FP64 build of the same kernels: the plain FP64
    engine from the same load, run for the same number of steps; normwise E, B, J differences
    (max |a - b| / max |b| over the whole grid) and the relative kinetic / field energy
    differences."""
    steps = args.warmup + args.steps
    ref, _ = build_sim(cfg, "plain", 64, None, args.nx)
    ref.step(steps)
    out = {"steps": steps}
    for name, a, b in zip("EBJ", sim.fields(), ref.fields()):
        out[name] = float(np.abs(a.astype(np.float64) - b).max() / max(np.abs(b).max(), 1e-300))
    k32, f32 = sim.energy()
    k64, f64 = ref.energy()
    out["kinetic"] = float(abs(k32.sum() - k64.sum()) / abs(k64.sum()))
    out["field"] = float(abs(f32.sum() - f64.sum()) / max(abs(f64.sum()), 1e-300))
    ref.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="two_stream",
                    choices=sorted(CONFIGS) + ["batch", "lwfa"])
    ap.add_argument("--boxes", type=int, default=64)
    ap.add_argument("--threads", type=int)
    ap.add_argument("--nx", type=int, nargs="+")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--engine", choices=["tiled", "plain"])
    ap.add_argument("--precision", type=int, choices=[32, 64])
    ap.add_argument("--tile", type=int, nargs="+")
    ap.add_argument("--fp64-check", action="store_true",
                    help="mixed-precision runs: report the error against the plain FP64 "
                         "engine after the same steps from the same load")
    ap.add_argument("--pageable", action="store_true",
                    help="--dropin: particles in pageable host memory instead of pinned")
    ap.add_argument("--pml", action="store_true",
                    help="--config lwfa: PML walls on the transverse axes (moving with the window)")
    ap.add_argument("--dropin", action="store_true",
                    help="2D configurations: time the host-array drop-in flow instead "
                         "(osg_vadvance_deposit_f32 per species, guard updates and Yee on "
                         "host arrays, all copies included)")
    args = ap.parse_args()
    if args.config == "batch":
        run_batch(args)
        return
    if args.config == "lwfa":
        t0 = time.time()
        sim, n0 = build_lwfa(args.nx, args.tile, pml=args.pml)
        t_load = time.time() - t0
        sim.step(args.warmup)
        ms = sim.time_steps(args.steps)
        n1 = sim.num_particles(0)
        kin, fld = sim.energy()
        print(json.dumps(dict(config="lwfa", nx=args.nx or LWFA["nx"], particles_start=n0,
                              particles_end=n1, steps=args.steps, ms_per_step=ms / args.steps,
                              particle_steps_per_s=n1 * args.steps / (ms / 1e3),
                              window_moves=sim.window_moves(), load_s=t_load,
                              kinetic=[float(v) for v in kin], field=[float(v) for v in fld],
                              phase_ms=sim.profile(5))))
        sim.close()
        return
    cfg = CONFIGS[args.config]
    if args.dropin:
        nx = args.nx or cfg["nx"]
        r = osg.Rng(cfg["seed"])
        sp = [osg.load_lattice(r, 32, nx, cfg["ppc"], cfg["dx"], -1.0, [s["uth"]] * 3,
                               s["ufl"], cfg["amp"], 1.0) for s in cfg["species"]]
        rate, h2d, d2h, n = dropin_steps(sp, nx, cfg["dx"], cfg["dt"], cfg["order"], args.steps,
                                         pinned=not args.pageable)
        print(json.dumps(dict(config=args.config, path="host-array drop-in", nx=nx,
                              memory="pageable" if args.pageable else "pinned",
                              particles=sum(len(s[3]) for s in sp), steps=n,
                              particle_steps_per_s=rate, h2d_bytes_per_step=h2d,
                              d2h_bytes_per_step=d2h)))
        return
    t0 = time.time()
    sim, npart = build_sim(cfg, args.engine, args.precision, args.tile, args.nx)
    t_load = time.time() - t0
    sim.step(args.warmup)
    ms = sim.time_steps(args.steps)
    kin, fld = sim.energy()
    out = dict(config=args.config, particles=npart, steps=args.steps,
               ms_per_step=ms / args.steps,
               particle_steps_per_s=npart * args.steps / (ms / 1e3),
               launches_per_step=sim.launches_per_step(), load_s=t_load,
               kinetic=[float(v) for v in kin], field=[float(v) for v in fld])
    if args.fp64_check and sim.precision == 32:
        out["fp64_error"] = fp64_error(cfg, sim, args)
    # per-phase device ms of 5 more steps, each phase timed alone with CUDA events
    out["phase_ms"] = sim.profile(5)
    print(json.dumps(out))
    sim.close()


if __name__ == "__main__":
    main()
