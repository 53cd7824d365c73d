"""Ensemble observables along a run, and their comparison between two runs.

The reference samples its observables on the master thread between steps,
gated by a period (total energy `src/stats/total_energy.cpp:4-11`, gyration
radius `src/stats/gyration.cpp:4-19`, native-contact fraction
`src/io/report_structure.cpp:85`).  `sample` does the same through the
engine's `observables` call.  `compare` reduces two sampled runs to the
figures the mixed-precision path reports against FP64: the mean-energy
difference, the energy drift of each run, the Rg difference and the Q
difference, each with a block-averaged standard error.
"""
from __future__ import annotations

import numpy as np

FIELDS = ("E", "K", "Rg", "Q")


def sample(engine, nsteps: int, every: int, rep: int = 0) -> np.ndarray:
    """Run `nsteps` steps on every replica of `engine`, sampling replica
    `rep` every `every` steps (and once before the first step).  Returns an
    array [samples, 5] of (t_step, E, K, Rg, Q)."""
    if every <= 0 or nsteps % every:
        raise ValueError("nsteps must be a positive multiple of every")
    def obs():
        o = engine.observables(rep)
        return tuple(o[k] for k in FIELDS) if isinstance(o, dict) else tuple(o)

    out = [(0, *obs())]
    for s in range(every, nsteps + 1, every):
        engine.step(every)
        out.append((s, *obs()))
    return np.asarray(out, dtype=np.float64)


def block_se(x: np.ndarray, blocks: int = 10) -> float:
    """Standard error of the mean of a correlated series from block averages."""
    x = np.asarray(x, dtype=np.float64)
    nb = min(blocks, len(x))
    if nb < 2:
        return float("inf")
    m = np.array([b.mean() for b in np.array_split(x, nb)])
    return float(m.std(ddof=1) / np.sqrt(nb))


def drift(t: np.ndarray, e: np.ndarray) -> float:
    """Least-squares slope of E(t) times the run length: the energy change a
    straight-line fit attributes to the run."""
    t = np.asarray(t, dtype=np.float64)
    if len(t) < 2 or t[-1] == t[0]:
        return 0.0
    return float(np.polyfit(t, e, 1)[0] * (t[-1] - t[0]))


def compare(a: np.ndarray, b: np.ndarray, skip: float = 0.5) -> dict:
    """Compare run `a` against reference run `b` (arrays from `sample`) over
    the samples after the first `skip` fraction of the run: means with their
    combined block standard error, and the energy drift over that window."""
    k = int(len(a) * skip)
    A, B = a[k:], b[k:]
    res = {"samples": int(len(A))}
    for col, name in ((1, "E"), (3, "Rg"), (4, "Q")):
        ma, mb = float(A[:, col].mean()), float(B[:, col].mean())
        se = float(np.hypot(block_se(A[:, col]), block_se(B[:, col])))
        res[name] = {"mean": ma, "ref_mean": mb, "diff": ma - mb, "se": se,
                     "rel_diff": (ma - mb) / abs(mb) if mb != 0 else None}
    # drift over the same window, against the reference run's energy scale
    # (its mean magnitude, or its spread where the mean is near zero)
    da, db = drift(A[:, 0], A[:, 1]), drift(B[:, 0], B[:, 1])
    scale = max(abs(float(B[:, 1].mean())), float(B[:, 1].std()))
    res["E_drift"] = {"drift": da, "ref_drift": db, "scale": scale,
                      "rel_to_ref_energy": abs(da - db) / scale if scale > 0 else None}
    return res
