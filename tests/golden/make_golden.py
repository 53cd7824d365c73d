"""Generate the golden fixtures of tests/golden/ from the reference's OWN kernels.

The reference ships no tests and no expected outputs, so the known answers
are produced by its compiled hot-path translation units (FP64 build,
oracle/_ref/libxmdref64.so, built by oracle/ref/build_ref.sh from the
reference tree).  Each fixture stores the full input (topology, native
structure, positions, YAML) and the reference's outputs, so the tests need
neither the reference tree nor the synthetic generator to replay it.

    python tests/golden/make_golden.py [case ...]    (all cases by default)

The full-size systems of the benchmark configurations (8,000 and 30,720
beads) keep only what their tests read: the inputs, the forces and energies
at step 0, the generator state and quasi-adiabatic contacts at each snapshot,
and the state at the last snapshot inside the parity horizon (the whole
predictor-corrector history for 8,000 beads, positions for 30,720).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.pyoracle import Oracle, rng_stream  # noqa: E402
from xmd_gb300 import abi, synth  # noqa: E402

OUT = Path(__file__).resolve().parent

QA_SHORT = "quasi-adiabatic potential:\n  phase duration: 0.25 tau\n"
# relative ES instead of const ES, simple native dihedrals instead of complex
REL_SND = """const ES:
  enabled: false
relative ES:
  enabled: true
  screening distance: 10.0 A
  factor: 4.0 eps_0/A
complex native dihedrals:
  enabled: false
simple native dihedrals:
  enabled: true
"""

CASES = {
    # 100-bead chain from the extended start, open boundary, Go + Pauli +
    # tether + angle + CND, 18 A + 2 A list
    "c1_chain100": dict(sys=lambda: synth.config_c1(seed=1), yaml=synth.yaml_for("c1"), steps=1000),
    # the same chain started in its native conformation at T = 0.1 (a start
    # near equilibrium: the 1000-step trajectory case)
    "c1_native100": dict(sys=lambda: synth.make_system([100], 1, box=None, temperature=0.1, start="native"),
                         yaml=synth.yaml_for("c1"), steps=1000),
    # 8 x 60 beads from extended starts, 80 A periodic box, + Debye-Hueckel
    "c2_periodic480": dict(sys=lambda: synth.make_system([60] * 8, 5, box=80 * 0.2, temperature=0.35),
                           yaml=synth.yaml_for("c2"), steps=1000),
    # 4 x 60 native chains in a 200 A periodic box, + Debye-Hueckel
    "c2_sparse240": dict(sys=lambda: synth.make_system([60] * 4, 5, box=200 * 0.2, temperature=0.35,
                                                       start="native"),
                         yaml=synth.yaml_for("c2"), steps=1000),
    # 20 x 30 beads, uniform 20-letter types, + quasi-adiabatic with a short phase
    "c3_qa600": dict(sys=lambda: synth.make_system([30] * 20, 11, box=(600 / 1e-3) ** (1 / 3) * 0.2 * 0.5,
                                                   types="uniform20", temperature=0.35),
                     yaml=synth.yaml_for("c3") + QA_SHORT, steps=500),
    # 8 x 60 beads from extended starts, 80 A periodic box, with the relative
    # ES term (es/relative.cpp) and simple native dihedrals
    # (dihedral/simple_native.cpp) in place of const ES and CND
    "c2_relsnd480": dict(sys=lambda: synth.make_system([60] * 8, 6, box=80 * 0.2, temperature=0.35),
                         yaml=synth.yaml_for("c2") + REL_SND, steps=1000),
    # the plain FP64 benchmark system at full size: 16 x 500 beads in a
    # 300 A periodic box, charges +-1 at p = 0.1 each, Debye-Hueckel
    "c2_full8000": dict(sys=lambda: synth.config_c2(), yaml=synth.yaml_for("c2"), steps=200, big="history"),
    # the mixed-precision benchmark system at full size: 512 x 60 beads at
    # 1e-3 A^-3, periodic, Go + Debye-Hueckel + quasi-adiabatic contacts
    # (its oracle agrees with itself to 1e-11 A for only ~20 steps, so its
    # state is kept at 10-step snapshots)
    "c3_full30720": dict(sys=lambda: synth.config_c3(), yaml=synth.yaml_for("c3"), steps=50, big="positions",
                         snapshots=(10, 20, 30, 40, 50)),
}


def pack_system(s):
    return dict(n=np.int64(s.n), chain=s.chain, seq=s.seq, atype=s.atype, cell=s.cell, r0=s.r,
                temperature=np.float64(s.temperature), seed=np.uint64(s.seed),
                teth_i1=s.tethers[0], teth_i2=s.tethers[1], teth_d=s.tethers[2],
                ang_i1=s.angles[0], ang_i2=s.angles[1], ang_i3=s.angles[2], ang_t=s.angles[3],
                dih_i1=s.dihedrals[0], dih_i2=s.dihedrals[1], dih_i3=s.dihedrals[2], dih_i4=s.dihedrals[3],
                dih_p=s.dihedrals[4], nat_i1=s.natives[0], nat_i2=s.natives[1], nat_d=s.natives[2])


SNAPSHOTS = (50, 100, 200)


def parity_horizon(s, p, total, snapshots=SNAPSHOTS):
    """Largest snapshot step count at which the oracle agrees with itself under
    a reordered force summation (its OpenMP driver, 4 threads) to <= 1e-11 A,
    a thousandth of the trajectory bar: a GPU build rounds differently in more
    places than a reordered sum (fused multiply-adds, its own libm), and the
    dynamics amplifies any rounding difference alike.  Beyond the horizon
    (and after Verlet-list decisions flip) trajectory parity between two
    correct FP64 implementations is not defined."""
    a, b = Oracle(p, s, "port"), Oracle(p, s, "port")
    done, best = 0, 0
    for n in sorted({k for k in snapshots if k <= total} | {total}):
        a.step(n - done)
        b.step_omp(n - done, 4)
        done = n
        ra, _, _ = a.get_state()
        rb, _, _ = b.get_state()
        if np.abs(ra - rb).max() / 0.2 <= 1e-11:
            best = n
        else:
            break
    return best


def make_case(name, c):
    s = c["sys"]()
    p = abi.parse_params(c["yaml"])
    big = c.get("big")
    shots = tuple(c.get("snapshots", SNAPSHOTS))
    horizon = parity_horizon(s, p, c["steps"], shots)
    ref = Oracle(p, s, "ref")
    F0, V0 = ref.eval_forces()
    counts0 = ref.counts()
    snaps = {}
    done = 0
    keep = max([k for k in shots + (c["steps"],) if k <= max(horizon, shots[0]) and k <= c["steps"]])
    for k in shots:
        if k > c["steps"]:
            break
        ref.step(k - done)
        done = k
        y, _, st = ref.get_history()
        if not big or k == keep:
            snaps[f"y_{k}"] = y if big != "positions" else y[0]
        snaps[f"rng_{k}"] = np.uint64(st)
        qk, _ = ref.qa_contacts()
        if qk.size:
            snaps[f"qa_{k}"] = qk
    ref.step(c["steps"] - done)
    y, t, rng = ref.get_history()
    snaps["parity_steps"] = np.int64(horizon)
    extra = {}
    if not big:
        F1, V1 = ref.eval_forces()
        qa, qa_t = ref.qa_contacts()
        extra = dict(F1=F1, V1=V1)
        if qa.size:
            extra.update(qa_contacts=qa, qa_ref_time=qa_t, sync=ref.sync())
        extra.update(y=y)
    np.savez_compressed(OUT / f"{name}.npz", yaml=np.array(c["yaml"]), steps=np.int64(c["steps"]),
                        F0=F0, V0=V0, n_go0=np.int64(counts0["go"]), n_pauli0=np.int64(counts0["pauli"]),
                        n_es0=np.int64(counts0["es"]), t=np.float64(t), rng=np.uint64(rng),
                        rebuilds=np.int64(ref.counts()["rebuilds"]),
                        **pack_system(s), **extra, **snaps)
    print(name, s.n, "atoms,", c["steps"], "steps, V0 =", V0.sum(), "rebuilds", ref.counts()["rebuilds"],
          "parity horizon", horizon, flush=True)


def main(names):
    for name in names or CASES:
        make_case(name, CASES[name])
    if not names:
        raw, st = rng_stream("ref", 42, 64)
        np.savez_compressed(OUT / "rng_seed42.npz", raw=raw, state_after=np.uint64(st))
        print("rng", raw[:3])


if __name__ == "__main__":
    main(sys.argv[1:])
