"""Run a simulation on the engine from the command line.

    python -m xmd_gb300.run --workload c4 --precision mixed --steps 960
    python -m xmd_gb300.run --workload c2 --yaml params.yml --steps 1000

The command-line counterpart of the reference's driver (xmd/main.cpp ->
freeform_main, src/freeform/main.cpp): YAML overrides over the defaults, a
system, a number of steps.  Systems are the seeded synthetic workloads of
xmd_gb300.synth (c1: one 100-bead chain; c2: 16 x 500 beads in a 300 A box;
c3: 512 x 60 beads at 1e-3 A^-3 with quasi-adiabatic contacts; c4: 256 uneven
single-chain replicas).  Prints one JSON line with wall time, bead-steps/s,
list statistics and (with --timing) per-kernel event timings.
"""
from __future__ import annotations

import argparse
import json
import os
import time

from . import synth
from .engine import Engine


def build_systems(workload: str, seed: int | None, workers: int):
    if workload == "c1":
        return [synth.config_c1(seed or 1)]
    if workload == "c2":
        return [synth.config_c2(seed or 2)]
    if workload == "c3":
        return [synth.config_c3(seed or 3)]
    if workload == "c4":
        return synth.config_c4(seed or 4, workers=workers)
    raise SystemExit(f"unknown workload {workload}")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--workload", default="c4", choices=["c1", "c2", "c3", "c4"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--yaml", default=None, help="extra YAML overrides (file)")
    ap.add_argument("--steps", type=int, default=960)
    ap.add_argument("--warmup", type=int, default=96)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--timing", action="store_true", help="CUDA events around every force/rebuild launch")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--shape", default=None,
                    help="launch shape fb,tile_per_sm,graph_steps,threads_per_bead (default: the engine's)")
    args = ap.parse_args(argv)

    y = synth.yaml_for(args.workload, args.precision) + f"  device: {args.device}\n"
    if args.yaml:
        with open(args.yaml) as f:
            y += "\n" + f.read()
    t0 = time.perf_counter()
    systems = build_systems(args.workload, args.seed, workers=min(16, os.cpu_count() or 1))
    t_gen = time.perf_counter() - t0
    nb = sum(s.n for s in systems)
    with Engine(y) as e:
        for s in systems:
            e.add_system(s)
        if args.shape:
            e.set_tuning(*(int(x) for x in args.shape.split(",")))
        e.step(args.warmup)
        e.synchronize()
        if args.timing:
            e.lib.xmd_gpu_set_kernel_timing(e.h, 1)
        s0 = e.stats()
        t1 = time.perf_counter()
        e.step(args.steps)
        e.synchronize()
        wall = time.perf_counter() - t1
        s1 = e.stats()
        out = {"workload": args.workload, "precision": args.precision, "beads": nb, "replicas": len(systems),
               "steps": args.steps, "wall_s": wall, "bead_steps_per_s": nb * args.steps / wall,
               "generate_s": t_gen, "rebuild_passes": None,
               "rebuilds": s1["rebuilds"] - s0["rebuilds"], "launches": s1["launches"] - s0["launches"],
               "nl_entries": s1["nl_entries"], "go_active": s1["go_active"], "qa_contacts": len(e.qa_contacts(0)[0])}
        if args.timing:
            import ctypes as C
            fms, nf, rms, nr = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
            e.lib.xmd_gpu_kernel_times(e.h, C.byref(fms), C.byref(nf), C.byref(rms), C.byref(nr))
            out.update(force_ms_total=fms.value, force_launches=nf.value, rebuild_ms_total=rms.value,
                       rebuild_launches=nr.value)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
