"""Command-line runner of the device-resident simulation on the benchmark workloads.

    python -m osiris_gb300.run --config two_stream [--nx 128 128] [--steps 10] [--engine tiled]

Configurations (seeded OSIRIS lattice load, periodic box, electrons only over a fixed
neutralising background):
  thermal     2D 128x128, 16 ppc, uth 0.1, quadratic, dx 0.05, dt 0.035          (FP64 plain)
  two_stream  2D 512x512, 2 x 32 ppc, +-0.2 c drift, uth 0.01, 1e-3 perturbation  (FP32 tiled)
  weibel      3D 128^3, 2 x 8 ppc, +-0.5 c along z, uth 0.05, cubic, dx 0.1, dt 0.05
Prints one JSON line per run with the device time per step and the energies.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="two_stream", choices=sorted(CONFIGS))
    ap.add_argument("--nx", type=int, nargs="+")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--engine", choices=["tiled", "plain"])
    ap.add_argument("--precision", type=int, choices=[32, 64])
    ap.add_argument("--tile", type=int, nargs="+")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    t0 = time.time()
    sim, npart = build_sim(cfg, args.engine, args.precision, args.tile, args.nx)
    t_load = time.time() - t0
    sim.step(args.warmup)
    ms = sim.time_steps(args.steps)
    kin, fld = sim.energy()
    print(json.dumps(dict(config=args.config, particles=npart, steps=args.steps,
                          ms_per_step=ms / args.steps,
                          particle_steps_per_s=npart * args.steps / (ms / 1e3),
                          launches_per_step=sim.launches_per_step(), load_s=t_load,
                          kinetic=[float(v) for v in kin], field=[float(v) for v in fld])))
    sim.close()


if __name__ == "__main__":
    main()
