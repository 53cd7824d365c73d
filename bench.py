#!/usr/bin/env python3
"""Headline benchmark: batched mixed-precision MD steps on one GB300.

Workload (config 4 of the benchmark set): 256 independent single-chain
systems, lengths log-uniform in [50, 800] beads, Go native contacts +
Debye-Hueckel + Pauli + tether/angle/dihedral terms, per-replica temperature
uniform in [0.3, 0.6], all packed into one engine context.  A bench "step" is
--md-steps Langevin predictor-corrector steps over every replica (one chunk
of graph-captured device work); L2 is flushed (256 MiB device write) before
each timed step and is excluded from the timing.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

One JSON line on rank 0.  --impl reference times the CPU implementation of
the same path (the C restatement of the reference's kernels, all host
threads, one thread per replica group) on the same workload.
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
    lib = C.CDLL(path or "libcudart.so")
    return lib


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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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


def profile_value(key):
    """A figure of the dominant kernel's committed ncu summary (a line
    `<key>: <number>`), or None."""
    p = ROOT / "profiles" / "k_force_mixed_c4.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def profile_traffic():
    """Per-launch DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum)
    of the dominant kernel from the committed ncu summary, or None."""
    return profile_value("traffic_bytes_per_launch")


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


def pack_history(eng, nrep):
    hs = [eng.get_history(r)[0] for r in range(nrep)]     # each [6, n, 3]
    return np.ascontiguousarray(np.concatenate(hs, axis=1).reshape(6, -1))


# ------------------------------------------------------------ engine arm --
def run_engine(args, rank, local, world):
    from xmd_gb300 import Engine, abi, synth
    dev = local
    systems = make_workload(rank, workers=min(16, os.cpu_count() or 1))
    nbeads = sum(s.n for s in systems)
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

    def flush_l2():
        rt.cudaMemsetAsync(flush, 1, C.c_size_t(L2_FLUSH_BYTES), stream)

    def stats():
        out = np.zeros(abi_n_stats(), dtype=np.int64)
        abi.check(eng.lib.xmd_gpu_stats(eng.h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def abi_n_stats():
        return 8

    def barrier():
        eng.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    md = args.md_steps
    # launch shapes chosen by the autotuner on a clone (not timed; the
    # trajectory does not depend on them)
    tuned = eng.autotune(md) if args.autotune else None
    # warm-up (also builds the graphs and the first lists)
    for _ in range(args.warmup):
        eng.step(md)
    barrier()
    s0 = stats()
    clocks = Clocks(dev)
    clocks.start()
    e0, e1 = ev.new(), ev.new()
    t_ms = 0.0
    for _ in range(args.steps):
        flush_l2()
        ev.record(e0)
        eng.step(md)
        ev.record(e1)
        t_ms += ev.ms(e0, e1)
    barrier()
    clk = clocks.stop()
    s1 = stats()
    launches = int(s1[5] - s0[5])
    value, t_max, beads_all = job_rate(nbeads, md, args.steps, t_ms, world)

    # dominant kernel: force+integrate, timed with events around each launch
    abi.check(eng.lib.xmd_gpu_set_kernel_timing(eng.h, 1))
    eng.step(md)
    fms, nf, rms, nr = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
    abi.check(eng.lib.xmd_gpu_kernel_times(eng.h, C.byref(fms), C.byref(nf), C.byref(rms), C.byref(nr)))
    abi.check(eng.lib.xmd_gpu_set_kernel_timing(eng.h, 0))
    force_ms = fms.value / max(1, nf.value)
    st = stats()
    P = st[2] / 2.0          # unique pairs kept by the pair terms
    Cg = st[3] / 2.0         # active Go contacts
    alg_bytes = 325.0 * nbeads + 4.0 * P + 12.0 * Cg     # mixed, per MD step (Q = 0)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (force_ms / 1e3) / 1e9
    traffic = profile_traffic()

    # end-to-end through the C ABI with pinned host buffers: every bench step
    # uploads the packed history of all replicas, runs md steps, reads back
    # all positions
    nrep = len(systems)
    yh = pack_history(eng, nrep)
    hbuf = C.c_void_p()
    assert rt.cudaHostAlloc(C.byref(hbuf), C.c_size_t(yh.nbytes + 24 * nbeads), 0) == 0
    hy = np.ctypeslib.as_array((C.c_double * yh.size).from_address(hbuf.value))
    hy[:] = yh.reshape(-1)
    hr = np.ctypeslib.as_array((C.c_double * (3 * nbeads)).from_address(hbuf.value + yh.nbytes))
    e2e_steps = max(2, args.steps // 2)
    pd = C.POINTER(C.c_double)
    for _ in range(1):
        abi.check(eng.lib.xmd_gpu_upload_history_all(eng.h, hy.ctypes.data_as(pd)))
        eng.step(md)
        abi.check(eng.lib.xmd_gpu_download_positions_all(eng.h, hr.ctypes.data_as(pd)))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        abi.check(eng.lib.xmd_gpu_upload_history_all(eng.h, hy.ctypes.data_as(pd)))
        eng.step(md)
        abi.check(eng.lib.xmd_gpu_download_positions_all(eng.h, hr.ctypes.data_as(pd)))
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_value = job_rate(nbeads, md, e2e_steps, 1e3 * e2e_s, world)[0]

    # plain FP64 on the same replicas (same protocol), and the mixed force error
    eng64 = Engine(y_fp64)
    for s in systems:
        eng64.add_system(s)
    tuned64 = eng64.autotune(md) if args.autotune else None   # its own best shape
    for _ in range(args.warmup):
        eng64.step(md)
    eng64.synchronize()
    abi.check(eng64.lib.xmd_gpu_get_stream(eng64.h, C.byref(stream)))
    ev64 = Events(rt, stream)
    t64 = 0.0
    k64 = max(2, args.steps // 2)
    for _ in range(k64):
        rt.cudaMemsetAsync(flush, 1, C.c_size_t(L2_FLUSH_BYTES), stream)
        ev64.record(e0)
        eng64.step(md)
        ev64.record(e1)
        t64 += ev64.ms(e0, e1)
    value64 = nbeads * md * k64 / (t64 / 1e3)
    eng64.close()
    plain64 = plain_fp64(systems, y_fp64, md, args.warmup, rt, flush)
    # force error of the mixed path on identical states (fresh engines at t=0)
    errs = []
    with Engine(y_mixed) as em, Engine(y_fp64) as ed:
        for s in systems[:16]:
            em.add_system(s)
            ed.add_system(s)
        for r in range(16):
            Fm, _ = em.eval_forces(r)
            Fd, _ = ed.eval_forces(r)
            errs.append(float(np.abs(Fm - Fd).max() / max(np.abs(Fd).max(), 1e-300)))

    # serving (config 5): Poisson arrivals offered at ~70% of the batched
    # mixed throughput, mixed and plain FP64 on the same request stream
    serving = None
    if args.serve_requests > 0:
        from xmd_gb300 import synth as _s
        reqs = _s.config_c5(count=args.serve_requests, seed=5 + rank, workers=min(16, os.cpu_count() or 1))
        mean_work = float(np.mean([rq.n for rq in reqs])) * args.serve_steps
        rate = 0.7 * (value / world) / mean_work
        serving = {"mixed": serve_bench(reqs, "mixed", args.serve_steps, rate, dev),
                   "fp64": serve_bench(reqs, "fp64", args.serve_steps, rate, dev)}

    accuracy = accuracy_c3(args.accuracy_steps, args.accuracy_every, dev) \
        if (rank == 0 and args.accuracy_steps > 0) else None
    cpu = cpu_baseline(systems, sample_steps=args.cpu_sample_steps) if rank == 0 else None
    rt.cudaFree(flush)
    rt.cudaFreeHost(hbuf)
    eng.close()
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {
            "workload": f"256 uneven single-chain replicas (log-uniform 50-800 beads, {nbeads} beads), "
                        "Go+Debye-Hueckel+Pauli+tether/angle/dihedral, per-replica T in [0.3,0.6], "
                        "mixed precision (FP32 forces, FP64 accumulate/integrate), one context",
            "md_steps_per_step": md, "beads_per_gpu": nbeads, "replicas_per_gpu": nrep,
            "l2": "256 MiB device write before each timed step (not timed)",
            "plain_fp64_value": plain64["value"], "plain_fp64_sample": plain64["sample"],
            "mixed_over_plain_fp64": value / world / plain64["value"],
            "batched_fp64_value": value64, "mixed_over_batched_fp64": value / world / value64,
            "mixed_force_rel_err_max": max(errs),
            "graph_steps_per_launch": (tuned or {}).get("graph_steps", 16),
            "autotuned_shape": tuned, "autotuned_shape_fp64": tuned64,
            "p99_req_latency_ms": serving["mixed"]["p99_ms"] if serving else None,
            "serving": serving,
            "mixed_vs_fp64_c3": accuracy,
        },
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_force<float,1> (force+integrate)", "kernel_ms": force_ms,
                     "alg_bytes_per_launch": alg_bytes, "peak_source": peak_kind,
                     "fp64_pipe_active": profile_value("fp64_pipe_active_pct"),
                     "note": "working set (~30 MB) is L2-resident between steps; the step kernel is "
                             "latency-bound at 16 warps/SM with its FP64 integrator on GB300's 2-lane/clk FP64 "
                             "pipe (fp64_pipe_active: % of active cycles, ncu, profiles/k_force_mixed_c4.md)"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "bead-steps/s", "h2d_bytes_per_step": int(yh.nbytes),
                "d2h_bytes_per_step": int(24 * nbeads)},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)


def plain_fp64(systems, yaml_fp64, md, warmup, rt, flush, sample=16):
    """The plain FP64 path: each system alone in its own context (no packing,
    FP64 forces), over a size-stratified sample of the replicas.  Returns
    summed bead-steps over summed device time."""
    from xmd_gb300 import Engine, abi
    order = sorted(range(len(systems)), key=lambda k: systems[k].n)
    pick = [order[int(q)] for q in np.linspace(0, len(order) - 1, min(sample, len(order)))]
    work, t_ms = 0, 0.0
    stream = C.c_void_p()
    for k in pick:
        with Engine(yaml_fp64) as e:
            e.add_system(systems[k])
            for _ in range(max(1, warmup)):
                e.step(md)
            e.synchronize()
            abi.check(e.lib.xmd_gpu_get_stream(e.h, C.byref(stream)))
            ev = Events(rt, stream)
            a, b = ev.new(), ev.new()
            rt.cudaMemsetAsync(flush, 1, C.c_size_t(L2_FLUSH_BYTES), stream)
            ev.record(a)
            e.step(md)
            ev.record(b)
            t_ms += ev.ms(a, b)
            work += systems[k].n * md
    nb = sum(systems[k].n for k in pick)
    return {"value": work / (t_ms / 1e3),
            "sample": f"{len(pick)} size-stratified replicas ({nb} beads), each alone in an FP64 context, "
                      f"{md} steps each"}


def accuracy_c3(steps, every, device):
    """Config 3: mixed precision against plain FP64 on 512 chains x 60 beads at
    1e-3 A^-3 (periodic; Go + Debye-Hueckel + quasi-adiabatic contacts).
    Forces are compared on the starting state; then each precision runs
    `steps` steps from that state with the same generator seed, and the
    energy (mean and drift), Rg and Q are compared over the second half of
    the run (block-averaged standard errors)."""
    from xmd_gb300 import Engine, observe, synth
    s = synth.config_c3()
    runs, forces, wall = {}, {}, {}
    for prec in ("fp64", "mixed"):
        with Engine(synth.yaml_for("c3", prec) + f"  device: {device}\n") as e:
            e.add_system(s)
            forces[prec], _ = e.eval_forces(0)
            t0 = time.perf_counter()
            runs[prec] = observe.sample(e, steps, every)
            wall[prec] = time.perf_counter() - t0
    res = observe.compare(runs["mixed"], runs["fp64"], skip=0.5)
    ferr = float(np.abs(forces["mixed"] - forces["fp64"]).max() / np.abs(forces["fp64"]).max())
    return {"system": f"512 x 60 beads ({s.n}), periodic, Go + Debye-Hueckel + quasi-adiabatic",
            "steps": steps, "sample_every": every, "force_rel_err_t0": ferr,
            "E_mean_rel_diff": res["E"]["rel_diff"], "E_mean_diff": res["E"]["diff"], "E_se": res["E"]["se"],
            "E_drift_mixed": res["E_drift"]["drift"], "E_drift_fp64": res["E_drift"]["ref_drift"],
            "E_drift_diff_rel_to_energy_scale": res["E_drift"]["rel_to_ref_energy"],
            "Rg_mean_rel_diff": res["Rg"]["rel_diff"], "Rg_se": res["Rg"]["se"],
            "Q_mean_diff": res["Q"]["diff"], "Q_se": res["Q"]["se"],
            "wall_s": wall, "reference": "plain FP64 engine (pinned to the oracle by the parity tests)"}


def serve_bench(requests, precision, nsteps, rate_hz, device, seed=0):
    """Config 5: requests arrive as a Poisson process at `rate_hz` and are
    served by the continuous-batching loop (HBM-budget admission, state
    resident on the device).  Returns latency percentiles and throughput."""
    from xmd_gb300 import Server, XmdError, synth
    yaml = synth.yaml_for("c5", precision) + f"  device: {device}\n"
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(requests))
    with Server(yaml, hbm_budget=8 << 30, max_beads=200_000, chunk_steps=256) as srv:
        # warm-up request (graph capture, first list builds) outside the clock
        srv.result(srv.submit(requests[0], 256))
        t0 = time.perf_counter()
        ids = []
        for g, rq in zip(gaps, requests):
            time.sleep(g)
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
    return {"p50_ms": pct(50), "p99_ms": pct(99),
            "bead_steps_per_s": work / wall, "wall_s": wall, "peak_concurrent": int(st["peak_running"]),
            "requests": len(requests), "completed": len(lat), "failed": failed,
            "steps_per_request": nsteps, "rate_hz": rate_hz,
            "beads_total": int(sum(rq.n for rq in requests))}


# ------------------------------------------------------------- CPU arms --
def _cpu_run(systems, steps, threads, warm=0):
    """All replicas on the CPU restatement, replicas spread over `threads`
    host threads (ctypes releases the GIL during each call)."""
    from oracle.pyoracle import Oracle
    from xmd_gb300 import abi, synth
    p = abi.parse_params(synth.yaml_for("c4", "fp64"))
    orcs = [Oracle(p, s, "port") for s in systems]
    order = sorted(range(len(orcs)), key=lambda k: -systems[k].n)
    groups = [[] for _ in range(threads)]
    load = [0] * threads
    for k in order:   # longest-first greedy balance
        g = int(np.argmin(load))
        groups[g].append(k)
        load[g] += systems[k].n

    def work(g, n):
        for k in groups[g]:
            orcs[k].step(n)

    def run(n):
        ts = [threading.Thread(target=work, args=(g, n)) for g in range(threads)]
        t0 = time.perf_counter()
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        return time.perf_counter() - t0

    if warm:
        run(warm)
    return orcs, run


def cpu_baseline(systems, sample_steps=200):
    threads = os.cpu_count() or 1
    nb = sum(s.n for s in systems)
    _, run = _cpu_run(systems, sample_steps, threads, warm=1)
    dt = run(sample_steps)
    return {"value": nb * sample_steps / dt, "unit": "bead-steps/s", "cores": threads, "kind": "port",
            "sample": f"all {len(systems)} replicas x {sample_steps} steps ({nb} beads), "
                      f"{dt:.1f} s wall on {threads} host threads"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    systems = make_workload(0, workers=min(16, os.cpu_count() or 1))
    nb = sum(s.n for s in systems)
    threads = os.cpu_count() or 1
    md = args.md_steps_ref
    _, run = _cpu_run(systems, md, threads)
    for _ in range(args.warmup):
        run(md)
    t = 0.0
    for _ in range(args.steps):
        t += run(md)
    value = nb * md * args.steps / t
    out = {
        "metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": f"256 uneven single-chain replicas (log-uniform 50-800 beads, {nb} beads), "
                               "Go+Debye-Hueckel+Pauli+tether/angle/dihedral, per-replica T in [0.3,0.6]",
                   "md_steps_per_step": md,
                   "implementation": "C restatement of the reference's FP64 kernels (bit-exact to them), "
                                     "one host thread per replica group"},
        "cpu_baseline": {"value": value, "unit": "bead-steps/s", "cores": threads, "kind": "port",
                         "sample": f"all {len(systems)} replicas x {md} steps per bench step"},
        "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--md-steps", type=int, default=96)
    ap.add_argument("--md-steps-ref", type=int, default=5)
    ap.add_argument("--cpu-sample-steps", type=int, default=100)
    ap.add_argument("--serve-requests", type=int, default=12)
    ap.add_argument("--serve-steps", type=int, default=20000)
    ap.add_argument("--accuracy-steps", type=int, default=100000)
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
    if True:
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
