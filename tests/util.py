"""Shared helpers of the test suite."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from xmd_gb300.synth import System

GOLDEN = Path(__file__).resolve().parent / "golden"
GOLDEN_CASES = ["c1_chain100", "c1_native100", "c2_periodic480", "c2_sparse240", "c3_qa600", "c2_relsnd480"]
FP64_CASES = ["c1_chain100", "c1_native100", "c2_periodic480", "c2_sparse240", "c2_relsnd480"]
# the benchmark systems at full size (8,000 and 30,720 beads): inputs, step-0
# forces, and the state at the last snapshot inside the parity horizon
FULL_CASES = ["c2_full8000", "c3_full30720"]
ANGSTROM = 0.2
# YAML section of each force term, in xmd_gb300.abi.TERM_* order
SECTIONS = ["tether forces", "native angles", "complex native dihedrals", "simple native dihedrals",
            "native contacts", "Pauli exclusion", "const ES", "relative ES", "quasi-adiabatic potential",
            "chirality", "native ssbonds", "heurestic angles", "heurestic dihedrals", "velocity AFM",
            "force AFM", "solid walls", "LJ attractive walls",
            "pseudo-improper dihedral potential"]


def only_term(term: int, y: str) -> str:
    """y with every force term off but `term`."""
    return y + "".join(f"\n{SECTIONS[k]}:\n  enabled: {'true' if k == term else 'false'}\n"
                       for k in range(len(SECTIONS)))


def horizon_snapshot(z):
    """(steps, y[6,n,3], rng_state) of the fixture's last snapshot inside its
    parity horizon: the step count up to which the oracle agrees with itself
    under a reordered force summation to 1e-11 A (beyond it the dynamics
    amplifies rounding, so no two FP64 implementations stay within 1e-8 A)."""
    h = int(z["parity_steps"])
    if h >= int(z["steps"]) and "y" in z:
        return int(z["steps"]), z["y"], int(z["rng"])
    shots = sorted(int(k[2:]) for k in z.files if k.startswith("y_"))
    best = max(k for k in shots if k <= max(h, shots[0]))
    return best, z[f"y_{best}"], int(z[f"rng_{best}"])


def cudart():
    """ctypes handle on the CUDA runtime the engine library already mapped."""
    import ctypes

    from xmd_gb300 import abi
    abi.load()
    path = None
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart.so" in line:
                path = line.split()[-1]
                break
    return ctypes.CDLL(path or "libcudart.so")


def load_golden(name: str):
    z = np.load(GOLDEN / f"{name}.npz")
    s = System(
        n=int(z["n"]), chain=z["chain"], seq=z["seq"], atype=z["atype"], cell=z["cell"], r=z["r0"],
        tethers=(z["teth_i1"], z["teth_i2"], z["teth_d"]),
        angles=(z["ang_i1"], z["ang_i2"], z["ang_i3"], z["ang_t"]),
        dihedrals=(z["dih_i1"], z["dih_i2"], z["dih_i3"], z["dih_i4"], z["dih_p"]),
        natives=(z["nat_i1"], z["nat_i2"], z["nat_d"]),
        temperature=float(z["temperature"]), seed=int(z["seed"]),
    )
    return s, str(z["yaml"]), z


def rel_err(a, b, floor=1.0):
    """max |a - b| over max |b| (norm-wise relative error).  The denominator is
    floored (default 1 eps per internal length unit): at an energy minimum the
    net forces cancel to ~1e-13 while each contribution is O(1), so rounding
    would otherwise read as a large relative error.  Per-term comparisons use
    a tiny floor."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), floor)
    return float(np.abs(a - b).max() / den)


def energy_rel(Va, Vb, floor=1e-6):
    """Per-term relative energy errors.  The denominator is floored at 1e-6 eps:
    a term whose exact value is ~0 (e.g. bonds exactly at their rest length,
    V ~ 1e-25) carries only rounding noise, which a relative test would
    amplify without meaning."""
    out = []
    for x, y in zip(Va, Vb):
        out.append(abs(x - y) / max(abs(y), floor))
    return np.array(out)
