"""Run reports of a replica: the statistics CSV of report_stats
(src/io/report_stats.cpp:8-41) and the structure YAML of report_structure
(src/io/report_structure.cpp:21-212), written from an Engine's state.

Both write numbers as std::to_string does (six decimals) in the reference's
units: time in tau, energies in eps, lengths in A (the asphericity, a squared
length, is divided by A once, as the reference divides it).  A reporter
fires when t - last_t >= period, like the reference's, and keeps last_t.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from .synth import ANGSTROM

QA_TYPES = {1: "BACK_BACK", 2: "BACK_SIDE", 3: "SIDE_BACK"}   # contact_type.h:10-14; others SIDE_SIDE
QA_STATUS = {0: "FORMING_OR_FORMED", 1: "BREAKING"}           # contact.h:6-9


def to_string(x) -> str:
    """std::to_string: integers as %d, floating point as %f."""
    if isinstance(x, (bool, np.bool_)):
        return "1" if x else "0"
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    return "%f" % float(x)


def asphericity(r: np.ndarray) -> float:
    """compute_asphericity (stats/asphericity.cpp:7-26) with unit masses:
    1.5 l_z^2 - 0.5 |l|^2 over the singular values of the centred positions."""
    if len(r) == 0:
        return 0.0
    R = (r - r.mean(axis=0)).T
    lam = np.linalg.svd(R, compute_uv=False)
    lam = np.pad(lam, (0, 3 - len(lam)))
    return 1.5 * lam[2] ** 2 - 0.5 * float((lam**2).sum())


class StatsReport:
    """report_stats: one CSV row t[tau], V[eps], K[eps], E[eps], Rg[A], W[A]
    per period; the header on the first row, appended afterwards."""
    HEADER = ["t[tau]", "V[eps]", "K[eps]", "E[eps]", "Rg[A]", "W[A]"]

    def __init__(self, path, period: float):
        self.path, self.period = Path(path), float(period)
        self.last_t, self.first = -math.inf, True

    def __call__(self, engine, rep: int = 0) -> bool:
        r, _, t = engine.get_state(rep)
        if t - self.last_t < self.period:
            return False
        ob = engine.observables(rep)
        row = [t, ob["E"] - ob["K"], ob["K"], ob["E"], ob["Rg"] / ANGSTROM, asphericity(r) / ANGSTROM]
        mode = "w" if self.first else "a"
        with open(self.path, mode) as f:
            if self.first:
                f.write(",".join(self.HEADER) + "\n")
            f.write(",".join(to_string(x) for x in row) + "\n")
        self.first, self.last_t = False, t
        return True


def _csv_block(header, rows) -> str:
    # emit_csv, report_structure.cpp:11-19: "|-" then the indented records
    out = "|-\n  " + ",".join(header)
    for r in rows:
        out += "\n  " + ",".join(r)
    return out


def structure_yaml(engine, system, rep: int = 0, active_threshold: float = 1.5) -> str:
    """The document report_structure writes: residues (with QA valences when
    the quasi-adiabatic term runs), native contacts with their current
    length and activity, QA contacts, angles and dihedrals with their native
    and current values.  system: the synth.System the replica was built from
    (its topology); active_threshold: `native contacts: active threshold`."""
    r, _, t = engine.get_state(rep)
    qa_on = bool(engine.params().on[8])
    head = ["idx", "x[A]", "y[A]", "z[A]"]
    sync = None
    if qa_on:
        head += ["back", "side-all", "side-polar", "side-hydrophobic"]
        sync = engine.qa_sync(rep)
    rows = []
    for i in range(len(r)):
        row = [to_string(i)] + [to_string(x / ANGSTROM) for x in r[i]]
        if sync is not None:
            row += [to_string(int(x)) for x in sync[i]]
        rows.append(row)
    doc = "residues: " + _csv_block(head, rows)

    n1, n2, nd = system.natives
    rows = []
    for k in range(len(n1)):
        a, b = int(n1[k]), int(n2[k])
        cur = float(np.linalg.norm(r[a] - r[b]))
        active = cur < active_threshold * 2.0 ** (-1.0 / 6.0) * nd[k]
        rows.append([to_string(k), to_string(a), to_string(b), "", to_string(nd[k] / ANGSTROM),
                     to_string(cur / ANGSTROM), to_string(bool(active))])
    ss = getattr(system, "ssbonds", None)
    if ss is not None:
        for k in range(len(ss[0])):
            a, b = int(ss[0][k]), int(ss[1][k])
            cur = float(np.linalg.norm(r[a] - r[b]))
            rows.append([to_string(len(n1) + k), to_string(a), to_string(b), "NAT_SS", "",
                         to_string(cur / ANGSTROM), to_string(False)])
    doc += "\n\nnative contacts: " + _csv_block(["idx", "i1", "i2", "type", "nat_dist[A]", "cur_dist[A]", "active"],
                                                rows)
    if qa_on:
        ct, rt = engine.qa_contacts(rep)
        rows = [[to_string(k), to_string(int(c[0])), to_string(int(c[1])),
                 QA_TYPES.get(int(c[2]), "SIDE_SIDE"), to_string(rt[k]), QA_STATUS.get(int(c[3]), "")]
                for k, c in enumerate(ct)]
        doc += "\n\nQA contacts: " + _csv_block(["idx", "i1", "i2", "type", "t0[tau]", "status"], rows)

    def theta(a, b, c):
        r12, r23 = r[b] - r[a], r[c] - r[b]
        return math.acos(-float(r12 @ r23) / (np.linalg.norm(r12) * np.linalg.norm(r23)))

    def phi(a, b, c, e):
        r12, r23, r34 = r[b] - r[a], r[c] - r[b], r[e] - r[c]
        x1, x2 = np.cross(r12, r23), np.cross(r23, r34)
        p = math.acos(max(-1.0, min(1.0, float(x1 @ x2) / (np.linalg.norm(x1) * np.linalg.norm(x2)))))
        return -p if float(x1 @ r34) < 0 else p

    angs = [(int(a), int(b), int(c), to_string(x)) for a, b, c, x in zip(*system.angles)]
    if getattr(system, "heur_angles", None) is not None:
        angs += [(int(a), int(b), int(c), "") for a, b, c in zip(*system.heur_angles)]
    rows = [[to_string(k), to_string(a), to_string(b), to_string(c), nat, to_string(theta(a, b, c))]
            for k, (a, b, c, nat) in enumerate(angs)]
    doc += "\n\nangles: " + _csv_block(["idx", "i1", "i2", "i3", "nat_theta[rad]", "cur_theta[rad]"], rows)
    dihs = [(int(a), int(b), int(c), int(e), to_string(x)) for a, b, c, e, x in zip(*system.dihedrals)]
    if getattr(system, "heur_dihedrals", None) is not None:
        dihs += [(int(a), int(b), int(c), int(e), "") for a, b, c, e in zip(*system.heur_dihedrals)]
    rows = [[to_string(k), to_string(a), to_string(b), to_string(c), to_string(e), nat, to_string(phi(a, b, c, e))]
            for k, (a, b, c, e, nat) in enumerate(dihs)]
    doc += "\n\ndihedrals: " + _csv_block(["idx", "i1", "i2", "i3", "i4", "nat_phi[rad]", "cur_phi[rad]"], rows)
    return doc


class StructureReport:
    """report_structure: one YAML file per period; path_fmt is formatted with
    the time in tau (printf style, e.g. "structure/%.0f.yml")."""

    def __init__(self, path_fmt: str, period: float, system, active_threshold: float = 1.5):
        self.path_fmt, self.period, self.system = path_fmt, float(period), system
        self.active_threshold = active_threshold
        self.last_t = -math.inf

    def __call__(self, engine, rep: int = 0):
        _, _, t = engine.get_state(rep)
        if t - self.last_t < self.period:
            return None
        path = Path(self.path_fmt % t)
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(structure_yaml(engine, self.system, rep, self.active_threshold))
        self.last_t = t
        return path
