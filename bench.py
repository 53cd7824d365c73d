#!/usr/bin/env python3
"""Headline benchmark: batched mixed-precision MD steps on one GB300.

Workload (config 4 of the benchmark set): 256 independent single-chain
systems, lengths log-uniform in [50, 800] beads, Go native contacts +
Debye-Hueckel + Pauli + tether/angle/dihedral terms, per-replica temperature
uniform in [0.3, 0.6], all packed into one engine context.  A bench "step" is
--md-steps Langevin predictor-corrector steps of every replica.  The timed
window is fixed by the step counts: W warm-up bench steps, then K timed ones,
so MD steps [W*md, (W+K)*md) of every replica; the rebuild rate in that
window is reported.  L2 is flushed (256 MiB device write, not timed) before
each timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

One JSON line on rank 0.  --impl reference times the CPU implementation of
the same path (the C restatement of the reference's FP64 kernels, all host
threads, one thread per replica group) on the same workload and window; that
arm loads only the oracle's libraries.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bead-steps/s mixed+batched vs plain FP64 at ≤1e-5 force err; p99 req latency"
L2_FLUSH_BYTES = 256 << 20
# ncu DRAM read + write of one k_force<float,1> launch on this workload (the
# capture and its command are in profiles/k_force_mixed_c4.md); a committed
# figure, not measured by this run
FORCE_TRAFFIC_NCU = 25555712


# ---------------------------------------------------------------- helpers --
def cudart():
    """libcudart as already mapped into this process by the engine library."""
    from xmd_gb300 import abi
    abi.load()
    path = None
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart.so" in line:
                path = line.split()[-1]
                break
    return C.CDLL(path or "libcudart.so")


class Events:
    def __init__(self, rt, stream):
        self.rt, self.stream = rt, stream

    def new(self):
        e = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(e)) == 0
        return e

    def record(self, e):
        assert self.rt.cudaEventRecord(e, self.stream) == 0

    def ms(self, a, b):
        self.rt.cudaEventSynchronize(b)
        v = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(v), a, b) == 0
        return v.value


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def job_rate(nbeads: int, md_steps: int, steps: int, t_ms: float, world: int):
    """Whole-job bead-steps/s: the beads of every rank (each rank steps its own
    replicas) over the slowest rank's time.  Returns (value, t_max_ms,
    beads_all_ranks)."""
    t_max, beads = float(t_ms), float(nbeads)
    if world > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([t_ms], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        bb = torch.tensor([float(nbeads)], dtype=torch.float64)
        dist.all_reduce(bb, op=dist.ReduceOp.SUM)
        t_max, beads = float(tt.item()), float(bb.item())
    return beads * md_steps * steps / (t_max / 1e3), t_max, int(beads)


def make_workload(rank: int, workers: int):
    from xmd_gb300 import synth
    return synth.config_c4(seed=4 + 1000 * rank, workers=workers)


def workload_config(nbeads: int, nrep: int, md: int, warmup: int, steps: int) -> dict:
    """The `config` of both arms (identical for the same arguments)."""
    return {"workload": f"256 uneven single-chain replicas (log-uniform 50-800 beads, {nbeads} beads), "
                        "Go+Debye-Hueckel+Pauli+tether/angle/dihedral, per-replica T in [0.3,0.6], "
                        "seeded synthetic chains from extended starts",
            "beads_per_gpu": nbeads, "replicas_per_gpu": nrep, "md_steps_per_step": md,
            "window_md_steps": [warmup * md, (warmup + steps) * md]}


# ------------------------------------------------------------ engine arm --
def run_engine(args, rank, local, world):
    from xmd_gb300 import Engine, abi, synth
    dev = local
    workers = min(16, os.cpu_count() or 1)
    systems = make_workload(rank, workers)
    nbeads = sum(s.n for s in systems)
    nrep = len(systems)
    md, K, W = args.md_steps, args.steps, args.warmup
    y_mixed = synth.yaml_for("c4", "mixed") + f"  device: {dev}\n"
    y_fp64 = synth.yaml_for("c4", "fp64") + f"  device: {dev}\n"
    eng = Engine(y_mixed)
    for s in systems:
        eng.add_system(s)
    rt = cudart()
    rt.cudaSetDevice(dev)
    stream = C.c_void_p()
    abi.check(eng.lib.xmd_gpu_get_stream(eng.h, C.byref(stream)))
    ev = Events(rt, stream)
    flush = C.c_void_p()
    assert rt.cudaMalloc(C.byref(flush), C.c_size_t(L2_FLUSH_BYTES)) == 0
    pd = C.POINTER(C.c_double)

    def barrier():
        eng.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # launch shapes chosen by the autotuner on a clone (not timed; the
    # trajectory does not depend on them)
    tuned = eng.autotune(min(md, 96)) if args.autotune else None
    st_a = eng.stats()
    for _ in range(W):
        eng.step(md)
    barrier()
    st_w = eng.stats()
    # the state at the window start: snapshots (the end-to-end loop replays
    # the window from them) and histories (the CPU sample starts there)
    snaps = [eng.snapshot(r) for r in range(nrep)]
    hist0 = [eng.get_history(r) for r in range(nrep)]
    s0 = eng.stats()
    clocks = Clocks(dev)
    clocks.start()
    e0, e1 = ev.new(), ev.new()
    t_ms = 0.0
    for _ in range(K):
        rt.cudaMemsetAsync(flush, 1, C.c_size_t(L2_FLUSH_BYTES), stream)
        ev.record(e0)
        eng.step(md)
        ev.record(e1)
        t_ms += ev.ms(e0, e1)
    barrier()
    clk = clocks.stop()
    s1 = eng.stats()
    r_end = np.zeros(3 * nbeads)
    abi.check(eng.lib.xmd_gpu_download_positions_all(eng.h, r_end.ctypes.data_as(pd)))
    launches = int(s1["launches"] - s0["launches"])
    value, t_max, beads_all = job_rate(nbeads, md, K, t_ms, world)
    window = {"md_steps": [W * md, (W + K) * md],
              "replica_rebuilds_per_md_step": (s1["rebuilds"] - s0["rebuilds"]) / (K * md),
              "replica_rebuilds_per_md_step_warmup": (st_w["rebuilds"] - st_a["rebuilds"]) / max(1, W * md)}

    # end to end through the C ABI over the SAME window: restore the
    # window-start state, then every bench step uploads the whole state from
    # pinned host memory, runs md steps and reads the whole state back
    for r in range(nrep):
        eng.restore(r, snaps[r])
    ybytes = 18 * 8 * nbeads
    hbuf = C.c_void_p()
    assert rt.cudaHostAlloc(C.byref(hbuf), C.c_size_t(ybytes), 0) == 0
    hy = np.ctypeslib.as_array((C.c_double * (18 * nbeads)).from_address(hbuf.value))
    abi.check(eng.lib.xmd_gpu_download_history_all(eng.h, hy.ctypes.data_as(pd)))
    barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        abi.check(eng.lib.xmd_gpu_upload_history_all(eng.h, hy.ctypes.data_as(pd)))
        eng.step(md)
        abi.check(eng.lib.xmd_gpu_download_history_all(eng.h, hy.ctypes.data_as(pd)))
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = job_rate(nbeads, md, K, 1e3 * e2e_s, world)[0]
    e2e_same = bool(np.array_equal(hy[:3 * nbeads], r_end))

    # the dominant kernel, timed with events around each launch (per-step
    # path), continuing from the window's end
    abi.check(eng.lib.xmd_gpu_set_kernel_timing(eng.h, 1))
    eng.step(md)
    fms, nf, rms, nr = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
    abi.check(eng.lib.xmd_gpu_kernel_times(eng.h, C.byref(fms), C.byref(nf), C.byref(rms), C.byref(nr)))
    abi.check(eng.lib.xmd_gpu_set_kernel_timing(eng.h, 0))
    force_ms = fms.value / max(1, nf.value)
    rebuild_ms = rms.value / max(1, nr.value)
    st = eng.stats()
    P = st["nl_entries"] / 2.0          # unique pairs kept by the pair terms
    Cg = st["go_active"] / 2.0          # active Go contacts
    alg_bytes = 325.0 * nbeads + 4.0 * P + 12.0 * Cg     # mixed, per MD step (Q = 0)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (force_ms / 1e3) / 1e9
    eng.close()

    # plain FP64 on the same replicas, batched, the same protocol and window
    eng64 = Engine(y_fp64)
    for s in systems:
        eng64.add_system(s)
    tuned64 = eng64.autotune(min(md, 96)) if args.autotune else None
    for _ in range(W):
        eng64.step(md)
    eng64.synchronize()
    abi.check(eng64.lib.xmd_gpu_get_stream(eng64.h, C.byref(stream)))
    ev64 = Events(rt, stream)
    t64 = 0.0
    for _ in range(K):
        rt.cudaMemsetAsync(flush, 1, C.c_size_t(L2_FLUSH_BYTES), stream)
        ev64.record(e0)
        eng64.step(md)
        ev64.record(e1)
        t64 += ev64.ms(e0, e1)
    value64 = nbeads * md * K / (t64 / 1e3)
    eng64.close()
    # mixed force error against FP64 on identical states (every replica at t = 0)
    errs = []
    with Engine(y_mixed) as em, Engine(y_fp64) as ed:
        for s in systems:
            em.add_system(s)
            ed.add_system(s)
        for r in range(nrep):
            Fm, _ = em.eval_forces(r)
            Fd, _ = ed.eval_forces(r)
            errs.append(float(np.abs(Fm - Fd).max() / max(np.abs(Fd).max(), 1e-300)))
    rt.cudaFree(flush)
    rt.cudaFreeHost(hbuf)

    extras = {}
    if rank == 0 and args.extras:
        extras["c2_plain_fp64"] = bench_c2(args, dev, rt)
        if args.serve_requests > 0:
            extras["serving"] = serve_section(args, dev, workers)
        if args.accuracy_steps > 0:
            extras["mixed_vs_fp64_c3"] = accuracy_c3(args.accuracy_replicas, args.accuracy_steps,
                                                    args.accuracy_every, dev)
    cpu = cpu_baseline(systems, hist0, args.cpu_sample_steps) if rank == 0 else None
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": t_max / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": workload_config(nbeads, nrep, md, W, K),
        "precision": "mixed: FP32 pair/bond forces, float-float per-bead accumulation, FP64 positions, "
                     "history, integrator, energies and skin test",
        "l2": "256 MiB device write before each timed step (not timed)",
        "window": window,
        "comparisons": {
            "batched_fp64_value": value64, "mixed_over_batched_fp64": value / world / value64,
            "mixed_force_rel_err_max": max(errs), "mixed_force_rel_err_replicas": len(errs),
            "autotuned_shape": tuned, "autotuned_shape_fp64": tuned64,
            **extras},
        "p99_req_latency_ms": (extras.get("serving") or {}).get("latency", {}).get("p99_ms"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": FORCE_TRAFFIC_NCU,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, "
                                       "committed capture (profiles/k_force_mixed_c4.md), not this run",
                     "kernel": "k_force<float,1> (force+integrate)", "kernel_ms": force_ms,
                     "rebuild_pass_ms": rebuild_ms, "rebuild_passes_per_md_step": nr.value / md,
                     "alg_bytes_per_launch": alg_bytes, "peak_source": peak_kind,
                     "alg_bytes": "325 N + 4 P + 12 C (N beads, P kept pairs, C active Go contacts)"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "bead-steps/s", "h2d_bytes_per_step": ybytes,
                "d2h_bytes_per_step": ybytes, "same_window_as_value": e2e_same,
                "path": "xmd_gpu_upload_history_all + xmd_gpu_step + xmd_gpu_download_history_all, pinned host"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def bench_c2(args, dev, rt):
    """Config 2 (16 x 500 beads, 300 A periodic box, Debye-Hueckel): the
    plain FP64 GPU path on one system, beside the CPU restatement on the same
    system and window."""
    from oracle.pyoracle import Oracle, parse_params
    from xmd_gb300 import Engine, abi, synth
    s = synth.config_c2()
    y = synth.yaml_for("c2", "fp64") + f"  device: {dev}\n"
    warm, timed = args.c2_warmup, args.c2_steps
    out = {"system": f"16 x 500 beads ({s.n}), 300 A periodic, Go+Pauli+tether/angle/CND+Debye-Hueckel",
           "window_md_steps": [warm, warm + timed]}
    for prec in ("fp64", "mixed"):
        with Engine(y.replace("precision: fp64", f"precision: {prec}")) as e:
            e.add_system(s)
            e.step(warm)
            e.synchronize()
            stream = C.c_void_p()
            abi.check(e.lib.xmd_gpu_get_stream(e.h, C.byref(stream)))
            ev = Events(rt, stream)
            a, b = ev.new(), ev.new()
            s0 = e.stats()
            ev.record(a)
            e.step(timed)
            ev.record(b)
            ms = ev.ms(a, b)
            s1 = e.stats()
            out[f"gpu_{prec}_value"] = s.n * timed / (ms / 1e3)
            out[f"gpu_{prec}_rebuilds_per_md_step"] = (s1["rebuilds"] - s0["rebuilds"]) / timed
            if prec == "fp64":
                y0, t0, g0 = e.get_history(0)
    # the CPU restatement from the same window-start state, all host threads
    p = parse_params(synth.yaml_for("c2", "fp64"))
    o = Oracle(p, s, "port")
    o.set_history(y0, t0, g0)
    threads = os.cpu_count() or 1
    o.step_omp(1, threads)
    t = time.perf_counter()
    o.step_omp(args.c2_cpu_steps, threads)
    dt = time.perf_counter() - t
    out["cpu_port_value"] = s.n * args.c2_cpu_steps / dt
    out["cpu_port_sample"] = f"{args.c2_cpu_steps} MD steps from the window start, {threads} host threads"
    out["gpu_fp64_over_cpu"] = out["gpu_fp64_value"] / out["cpu_port_value"]
    return out


def serve_section(args, device, workers):
    """Config 5 serving: capacity of mixed and plain FP64 on the same request
    stream (every request offered at once, so throughput is the server's
    capacity, not the arrival rate), then latency percentiles of mixed under
    Poisson arrivals at a fraction of that capacity."""
    from xmd_gb300 import synth
    reqs = synth.config_c5(count=args.serve_requests, seed=5, workers=workers)
    cap_reqs = reqs[:args.serve_capacity_requests]
    cap = {prec: serve_run(cap_reqs, prec, args.serve_steps, None, device) for prec in ("mixed", "fp64")}
    mean_work = float(np.mean([rq.n for rq in reqs])) * args.serve_steps
    rate = args.serve_load * cap["mixed"]["bead_steps_per_s"] / mean_work
    lat = serve_run(reqs, "mixed", args.serve_steps, rate, device)
    lat["offered_load"] = args.serve_load
    # a small sweep of the offered load on the head of the same stream
    sweep = []
    for load in (float(x) for x in args.serve_sweep.split(",") if x):
        rq = reqs[:args.serve_sweep_requests]
        mw = float(np.mean([r.n for r in rq])) * args.serve_steps
        one = serve_run(rq, "mixed", args.serve_steps, load * cap["mixed"]["bead_steps_per_s"] / mw, device, seed=1)
        sweep.append({"offered_load": load, "requests": one["requests"], "p50_ms": one["p50_ms"],
                      "p99_ms": one["p99_ms"], "bead_steps_per_s": one["bead_steps_per_s"],
                      "completed": one["completed"]})
    return {"capacity": cap,
            "capacity_mixed_over_fp64": cap["mixed"]["bead_steps_per_s"] / cap["fp64"]["bead_steps_per_s"],
            "latency": lat, "load_sweep": sweep}


def serve_run(requests, precision, nsteps, rate_hz, device, seed=0):
    """Requests arrive as a Poisson process at `rate_hz` (None: all at once)
    and are served by the continuous-batching loop (HBM-budget admission,
    state resident on the device).  Returns latency percentiles and
    throughput."""
    from xmd_gb300 import Server, XmdError, synth
    yaml = synth.yaml_for("c5", precision) + f"  device: {device}\n"
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(requests)) if rate_hz else np.zeros(len(requests))
    with Server(yaml, hbm_budget=8 << 30, max_beads=200_000, chunk_steps=256) as srv:
        # warm-up request (graph capture, first list builds) outside the clock
        srv.result(srv.submit(requests[0], 256))
        t0 = time.perf_counter()
        ids = []
        due = t0
        for g, rq in zip(gaps, requests):
            due += g
            d = due - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids.append(srv.submit(rq, nsteps))
        # a request whose trajectory diverges (non-finite force, as the
        # reference's own kernels do for some states) fails alone
        lat, done_beads, failed = [], 0, []
        for k, i in enumerate(ids):
            try:
                lat.append(srv.result(i)[3])
                done_beads += requests[k].n
            except XmdError as ex:
                failed.append({"request": k, "beads": int(requests[k].n), "error": str(ex)[:120]})
        wall = time.perf_counter() - t0
        st = srv.stats()
    lat = np.sort(np.asarray(lat))
    work = float(done_beads) * nsteps
    pct = (lambda q: 1e3 * float(np.percentile(lat, q, method="inverted_cdf"))) if len(lat) else (lambda q: None)
    return {"p50_ms": pct(50), "p99_ms": pct(99), "max_ms": pct(100),
            "bead_steps_per_s": work / wall, "wall_s": wall, "peak_concurrent": int(st["peak_running"]),
            "worker_admit_s": st["admit_s"], "worker_step_s": st["step_s"], "chunks": int(st["chunks"]),
            "device_bytes": int(st["device_bytes"]), "bytes_per_bead_slot": st["bytes_per_bead"],
            "requests": len(requests), "completed": len(lat), "failed": failed,
            "steps_per_request": nsteps, "rate_hz": rate_hz,
            "beads_total": int(sum(rq.n for rq in requests))}


def accuracy_c3(nrep, steps, every, device):
    """Config 3 at full size (512 x 60 beads at 1e-3 A^-3, periodic, Go +
    Debye-Hueckel + quasi-adiabatic contacts): `nrep` replicas of the system,
    each with its own generator seed, run in mixed precision and in plain
    FP64 (one batched context per precision) from the same states with the
    same seeds.  Per replica: the energy change over the run and over its
    second half (least-squares slope x duration), and the means of E, Rg and
    Q over the second half.  Reported as paired mixed - FP64 differences,
    their mean and standard error over the replicas, and the drift
    criterion: |mean paired drift difference| <= 1 % of |FP64 drift|."""
    from xmd_gb300 import Engine, XmdError, observe, synth
    s = synth.config_c3()
    runs, forces, wall, frozen = {}, {}, {}, {}
    for prec in ("fp64", "mixed"):
        with Engine(synth.yaml_for("c3", prec) + f"  device: {device}\n") as e:
            for k in range(nrep):
                e.add_system(s, seed=s.seed + 7919 * k)
            forces[prec], _ = e.eval_forces(0)
            t0 = time.perf_counter()
            samples = [[(0.0, *[e.observables(k)[f] for f in observe.FIELDS])] for k in range(nrep)]
            frz = set()
            for t in range(every, steps + 1, every):
                try:
                    e.step(every)
                except XmdError as ex:
                    # a replica whose force went non-finite (the reference's
                    # terms are singular at some geometries) is frozen; the
                    # others go on, and it leaves the paired comparison
                    if "non-finite" not in str(ex):
                        raise
                    frz |= {int(k) for k in np.nonzero(e.steps_left()[:nrep] == -3)[0]}
                for k in range(nrep):
                    obs = (float("nan"),) * len(observe.FIELDS) if k in frz else \
                        tuple(e.observables(k)[f] for f in observe.FIELDS)
                    samples[k].append((float(t), *obs))
            frozen[prec] = sorted(frz)
            wall[prec] = time.perf_counter() - t0
            runs[prec] = [np.asarray(x) for x in samples]
    keep = [k for k in range(nrep) if k not in frozen["fp64"] and k not in frozen["mixed"]]
    runs = {prec: [runs[prec][k] for k in keep] for prec in runs}
    half = len(runs["fp64"][0]) // 2

    def per_rep(a):
        return {"drift_run": observe.drift(a[:, 0], a[:, 1]), "drift_half": observe.drift(a[half:, 0], a[half:, 1]),
                "E": a[half:, 1].mean(), "Rg": a[half:, 3].mean(), "Q": a[half:, 4].mean()}
    m = [per_rep(a) for a in runs["mixed"]]
    f = [per_rep(a) for a in runs["fp64"]]

    def paired(key):
        d = np.array([x[key] - y[key] for x, y in zip(m, f)])
        ref = np.array([y[key] for y in f])
        return {"fp64_mean": float(ref.mean()), "mixed_minus_fp64": float(d.mean()),
                "se": float(d.std(ddof=1) / np.sqrt(len(d))) if len(d) > 1 else None}
    res = {k: paired(k) for k in ("drift_run", "drift_half", "E", "Rg", "Q")}
    ferr = float(np.abs(forces["mixed"] - forces["fp64"]).max() / np.abs(forces["fp64"]).max())
    dr = res["drift_run"]
    rel = abs(dr["mixed_minus_fp64"]) / abs(dr["fp64_mean"])
    rel_hi = (abs(dr["mixed_minus_fp64"]) + 2.0 * (dr["se"] or 0.0)) / abs(dr["fp64_mean"])
    return {"system": f"{nrep} replicas x 512 x 60 beads ({s.n} each), periodic, Go + Debye-Hueckel + "
                      "quasi-adiabatic, own generator seed per replica",
            "steps": steps, "sample_every": every, "force_rel_err_t0": ferr, "paired": res,
            "replicas_paired": len(keep), "frozen_non_finite": frozen,
            "drift_rel_diff": rel, "drift_rel_diff_95": rel_hi, "drift_within_1pct": bool(rel <= 0.01),
            "drift_within_1pct_95": bool(rel_hi <= 0.01),
            "drift_definition": "energy change over the whole run (least-squares slope x duration), "
                                "per replica, paired mixed - FP64; 95 = mean + 2 SE",
            "wall_s": wall,
            "bead_steps_per_s": {prec: nrep * s.n * steps / wall[prec] for prec in wall},
            "bead_steps_note": "replicas x beads x steps / host wall time of the run, observables sampled "
                               "every sample_every steps; a frozen replica stops stepping when it freezes",
            "reference": "plain FP64 engine (pinned to the oracle by the parity tests)"}


# ------------------------------------------------------------- CPU arms --
class CpuReplicas:
    """All replicas on the CPU restatement of the reference's FP64 kernels,
    spread over `threads` host threads (ctypes releases the GIL during each
    call).  Loads only the oracle's library (parameters are parsed by the
    parser linked into it)."""

    def __init__(self, systems, threads):
        from oracle.pyoracle import Oracle, parse_params
        from xmd_gb300 import synth
        p = parse_params(synth.yaml_for("c4", "fp64"))
        self.orcs = [Oracle(p, s, "port") for s in systems]
        order = sorted(range(len(self.orcs)), key=lambda k: -systems[k].n)
        self.groups = [[] for _ in range(threads)]
        load = [0] * threads
        for k in order:   # longest-first greedy balance
            g = int(np.argmin(load))
            self.groups[g].append(k)
            load[g] += systems[k].n

    def run(self, n):
        def work(g):
            for k in self.groups[g]:
                self.orcs[k].step(n)
        ts = [threading.Thread(target=work, args=(g,)) for g in range(len(self.groups))]
        t0 = time.perf_counter()
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        return time.perf_counter() - t0


def cpu_baseline(systems, hist0, steps):
    """A bounded sample of the same workload on the CPU restatement: every
    replica, `steps` MD steps from the state at the start of the timed
    window (so the list-rebuild rate is the window's)."""
    threads = os.cpu_count() or 1
    nb = sum(s.n for s in systems)
    cpu = CpuReplicas(systems, threads)
    for o, (y, t, g) in zip(cpu.orcs, hist0):
        o.set_history(y, t, g)
    cpu.run(1)
    dt = cpu.run(steps)
    return {"value": nb * steps / dt, "unit": "bead-steps/s", "cores": threads, "kind": "port",
            "sample": f"all {len(systems)} replicas x {steps} MD steps ({nb} beads) from the timed window's "
                      f"start state, {dt:.1f} s wall on {threads} host threads"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    systems = make_workload(0, workers=min(16, os.cpu_count() or 1))
    nb = sum(s.n for s in systems)
    threads = os.cpu_count() or 1
    md, K, W = args.md_steps, args.steps, args.warmup
    cpu = CpuReplicas(systems, threads)
    for _ in range(W):
        cpu.run(md)
    t = 0.0
    for _ in range(K):
        t += cpu.run(md)
    value = nb * md * K / t
    maps = [ln.split()[-1] for ln in open("/proc/self/maps") if ".so" in ln and str(ROOT) in ln]
    out = {
        "metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": 1e3 * t / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": workload_config(nb, len(systems), md, W, K),
        "implementation": "C restatement of the reference's FP64 kernels (bit-exact to them on x86), "
                          "one host thread per replica group",
        "libraries_loaded": sorted(set(Path(m).name for m in maps)),
        "cpu_baseline": {"value": value, "unit": "bead-steps/s", "cores": threads, "kind": "port",
                         "sample": f"all {len(systems)} replicas x {md} MD steps per bench step, "
                                   f"MD steps [{W * md}, {(W + K) * md})"},
        "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--md-steps", type=int, default=240)
    ap.add_argument("--cpu-sample-steps", type=int, default=120)
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the config-2, serving and config-3 sections")
    ap.add_argument("--c2-warmup", type=int, default=480)
    ap.add_argument("--c2-steps", type=int, default=2400)
    ap.add_argument("--c2-cpu-steps", type=int, default=40)
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-capacity-requests", type=int, default=32)
    ap.add_argument("--serve-load", type=float, default=0.7)
    ap.add_argument("--serve-sweep", default="0.4,0.9", help="offered loads of the latency sweep")
    ap.add_argument("--serve-sweep-requests", type=int, default=64)
    ap.add_argument("--serve-steps", type=int, default=20000)
    ap.add_argument("--accuracy-replicas", type=int, default=8)
    ap.add_argument("--accuracy-steps", type=int, default=20000)
    ap.add_argument("--accuracy-every", type=int, default=1000)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, local, world = dist_env()
    if args.impl == "reference":
        # rank 0 alone times the CPU implementation; other ranks have no work
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from xmd_gb300 import build
    build.build_engine()
    build.build_oracle()
    run_engine(args, rank, local, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
