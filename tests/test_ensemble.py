"""Ensemble observables over longer runs (the reference's total energy,
gyration radius and native-contact fraction, src/stats/total_energy.cpp:4-11,
src/stats/gyration.cpp:4-19, src/io/report_structure.cpp:85).

* Plain FP64 on the GPU against the CPU restatement of the reference, both
  driven by the same seeded noise stream: mean E, Rg and Q over the second
  half of a 40,000-step run agree within four block-averaged standard errors.
* Mixed precision against plain FP64 from the same states and generator
  seeds: replica-averaged mean energy, energy drift (least-squares slope
  times window length), Rg and Q agree within statistical error.  The
  trajectories themselves decorrelate through the chaotic dynamics, as two
  FP64 runs with reordered force sums do, so agreement is statistical.

The reference's noise amplitude is sqrt(2 T gamma) per step with no
1/sqrt(dt) (lang_pc.cpp:11-16), so these runs are quenches from the extended
starts rather than equilibrium samples; both sides follow the same schedule.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from xmd_gb300 import Engine, abi, observe, synth

pytestmark = pytest.mark.gpu
ANGSTROM = 0.2


def oracle_sample(o, nsteps, every):
    out = []
    ob = o.observables()
    out.append((0, ob["E"], ob["K"], ob["Rg"], ob["Q"]))
    for s in range(every, nsteps + 1, every):
        o.step(every)
        ob = o.observables()
        out.append((s, ob["E"], ob["K"], ob["Rg"], ob["Q"]))
    return np.asarray(out)


def within(r, rel=0.0):
    return abs(r["diff"]) <= max(4.0 * r["se"], rel * abs(r["ref_mean"]), 1e-12 * abs(r["ref_mean"]))


@pytest.mark.parametrize("seed", [11, 12])
def test_fp64_ensemble_matches_oracle(seed):
    s = synth.config_c1(seed)
    y = synth.yaml_for("c1")
    o = Oracle(abi.parse_params(y), s, "port")
    with Engine(y) as e:
        e.add_system(s)
        a = observe.sample(e, 40000, 100)
    b = oracle_sample(o, 40000, 100)
    res = observe.compare(a, b, skip=0.5)
    for k in ("E", "Rg", "Q"):
        assert within(res[k]), (k, res[k])


def replica_means(runs, skip=0.5):
    """Per-replica means of E, Rg, Q over the second half, and per-replica
    energy drift over that window."""
    out = {}
    for prec, rs in runs.items():
        k = int(len(rs[0]) * skip)
        out[prec] = {
            "E": np.array([r[k:, 1].mean() for r in rs]),
            "Rg": np.array([r[k:, 3].mean() for r in rs]),
            "Q": np.array([r[k:, 4].mean() for r in rs]),
            "drift": np.array([observe.drift(r[k:, 0], r[k:, 1]) for r in rs]),
        }
    return out


def sample_all(engine, nrep, nsteps, every):
    """observe.sample over every replica of one batched engine."""
    out = [[] for _ in range(nrep)]
    for s in range(0, nsteps + 1, every):
        if s:
            engine.step(every)
        for r in range(nrep):
            o = engine.observables(r)
            out[r].append((s, o["E"], o["K"], o["Rg"], o["Q"]))
    return [np.asarray(x) for x in out]


def paired_check(systems, y, nsteps=20000, every=200):
    """Both precisions from the same states and generator seeds, one batched
    context each; per-replica means of E, energy drift, Rg and Q compared
    through their paired differences (mean within four standard errors)."""
    runs = {}
    for prec in ("fp64", "mixed"):
        with Engine(y.replace("precision: fp64", f"precision: {prec}")) as e:
            for s in systems:
                e.add_system(s)
            runs[prec] = sample_all(e, len(systems), nsteps, every)
    m = replica_means(runs)
    for k in ("E", "drift", "Rg", "Q"):
        d = m["mixed"][k] - m["fp64"][k]
        se = d.std(ddof=1) / np.sqrt(len(d))
        assert abs(d.mean()) <= 4.0 * se + 1e-12 * abs(m["fp64"][k].mean()), (k, d.mean(), se)


def test_mixed_ensemble_matches_fp64():
    """16 single-chain replicas (100 beads each, different chains), 20,000
    steps.  (Single trajectories decorrelate through the chaotic dynamics
    whatever the precision, so the agreement tested is statistical.)"""
    paired_check([synth.config_c1(200 + k) for k in range(16)], synth.yaml_for("c1"))


def small_c3(seed, chains=8, length=60):
    n = chains * length
    box = (n / 1e-3) ** (1.0 / 3.0) * ANGSTROM
    return synth.make_system([length] * chains, seed, box=box, types="uniform20", temperature=0.35)


def test_mixed_qa_ensemble_matches_fp64():
    """Config-3-like periodic systems with quasi-adiabatic contacts: 8
    replicas of 8 x 60 beads at 1e-3 A^-3, 20,000 steps."""
    paired_check([small_c3(300 + k) for k in range(8)], synth.yaml_for("c3"))
