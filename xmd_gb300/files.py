"""PDB structures in and out: real proteins as engine systems.

Reading restates the reference's PDB path (files/pdb.cpp:10-108 over the
fixed-column records of files/records.cpp and files/fields.cpp): ATOM,
SSBOND, LINK, CRYST1 and TER records, positions in A scaled to internal units
(x 0.2), parsing stopping at END.  `to_system` restates pdb::to_model
(pdb.cpp:201-323): one bead per residue at its CA atom, tethers at their
native lengths, native angles and dihedrals of consecutive residues,
contacts from LINK records (Go native contacts, CA-CA length) and SSBOND
records (native disulfides, kept apart as `ssbonds`), and the CRYST1 cell as
the box.  `derive_contacts` restates pdb::add_contacts (pdb.cpp:324-388) for
CA atoms: residues at least 3 apart in sequence whose CA atoms are closer than
the sum of their residue radii (defaults.yml `amino acid data`).

Two decisions differ from the shipped code, each for the intended meaning:
  * residue and chain order: the reference keeps chains, residues and atoms in
    unordered maps (include/xmd/files/pdb.h:52-64) and walks the residue map
    in to_model, so consecutive beads follow the hash order, not the chain.
    Here chains follow their first appearance, residues their order in the
    file (the order the reader already records, pdb.cpp:39-41);
  * native angles: to_model takes theta = acos(u12 . u23) (pdb.cpp:235-237),
    the supplement of the angle the force term measures
    (acos(-u12 . u23), angle/native.cpp:30).  Here theta uses the force
    term's convention, so a PDB structure sits at the angle minimum.
Writing emits CA-only models in the same columns (records.cpp write()), one
MODEL/ENDMDL block per frame, as export_pdb does (io/export_pdb.cpp:10-31).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .abi import AA
from .synth import ANGSTROM, System, bonded_natives, chirals_of

# CA radii of the residue types (defaults.yml amino-acid data, `radius`), in A
# (MET's entry, defaults.yml:183, lacks its unit; it is read as 4.5 A)
RADIUS_A = {
    "ALA": 3.35, "ARG": 3.95, "ASN": 3.65, "ASP": 3.5, "CYS": 3.7, "GLU": 3.65, "GLN": 3.9, "GLY": 3.15,
    "HIS": 4.0, "ILE": 4.5, "LEU": 4.6, "LYS": 3.65, "MET": 4.5, "PHE": 4.6, "PRO": 3.7, "SER": 3.3,
    "THR": 3.6, "TRP": 4.7, "TYR": 4.5, "VAL": 4.0,
}


@dataclass
class Residue:
    chain: str
    seq_num: int
    name: str
    atoms: list = field(default_factory=list)   # (atom name, serial) in order of appearance
    pos: dict = field(default_factory=dict)     # serial -> position (internal units)

    def find(self, name: str):
        """Position of the first atom of that name (residue::find_by_name)."""
        for nm, serial in self.atoms:
            if nm == name:
                return self.pos[serial]
        return None


@dataclass
class Pdb:
    chains: dict                  # chain id -> list of Residue in file order
    links: list                   # (chain1, seq1, atom1, chain2, seq2, atom2, length)
    ssbonds: list                 # (chain1, seq1, chain2, seq2, length)
    cell: np.ndarray              # CRYST1 a, b, c (internal units), zeros if absent


def _field(line: str, beg: int, end: int) -> str:
    # 1-based inclusive columns, as fields.cpp's (beg, end) pairs
    return line[beg - 1:end] if len(line) >= beg else ""


def _record(line: str) -> str:
    return line[:6].ljust(6)


def read_pdb(text: str) -> Pdb:
    """Parse PDB text (records.cpp columns)."""
    chains: dict = {}
    index: dict = {}
    ter: set = set()
    links, ssbonds = [], []
    cell = np.zeros(3)
    for line in text.splitlines():
        rec = _record(line)
        if rec == "ATOM  ":
            serial = int(_field(line, 7, 11))
            name = _field(line, 13, 16).strip()
            res = _field(line, 18, 20).strip()
            ch = _field(line, 22, 22) or " "
            seq = int(_field(line, 23, 26))
            pos = np.array([float(_field(line, 31, 38)), float(_field(line, 39, 46)),
                            float(_field(line, 47, 54))]) * ANGSTROM
            key = (ch, seq)
            r = index.get(key)
            if r is None:
                r = Residue(ch, seq, res)
                index[key] = r
                if ch not in ter:
                    chains.setdefault(ch, []).append(r)
            # atoms are keyed by serial (a later model overwrites the same
            # serial, pdb.cpp:58-62); a name's first atom is the one used
            if serial not in r.pos:
                r.atoms.append((name, serial))
            r.pos[serial] = pos
        elif rec == "SSBOND":
            if _field(line, 12, 14) != "CYS":
                continue
            ssbonds.append((_field(line, 16, 16), int(_field(line, 18, 21)), _field(line, 30, 30),
                            int(_field(line, 32, 35)), float(_field(line, 74, 78)) * ANGSTROM))
        elif rec == "LINK  ":
            links.append((_field(line, 22, 22), int(_field(line, 23, 26)), _field(line, 13, 16).strip(),
                          _field(line, 52, 52), int(_field(line, 53, 56)), _field(line, 43, 46).strip(),
                          float(_field(line, 74, 78)) * ANGSTROM))
        elif rec == "CRYST1":
            cell = np.array([float(_field(line, 7, 15)), float(_field(line, 16, 24)),
                             float(_field(line, 25, 33))]) * ANGSTROM
        elif rec == "TER   ":
            ter.add(_field(line, 22, 22) or " ")
        elif rec == "END   ":
            break
    return Pdb(chains=chains, links=links, ssbonds=ssbonds, cell=cell)


def derive_contacts(pdb: Pdb, radius_a: dict | None = None):
    """Native contacts from CA overlaps (pdb.cpp:324-388, CA atoms): residues
    at least 3 apart whose CA distance is below the sum of their radii.
    Returns (chain1, seq1, chain2, seq2, length) tuples, i < j by file order."""
    rad = RADIUS_A if radius_a is None else radius_a
    res = [r for ch in pdb.chains.values() for r in ch if r.find("CA") is not None]
    out = []
    for a in range(len(res)):
        ra = res[a]
        for b in range(a + 1, len(res)):
            rb = res[b]
            if abs(ra.seq_num - rb.seq_num) < 3:
                continue
            d = float(np.linalg.norm(ra.find("CA") - rb.find("CA")))
            if d < (rad[ra.name] + rad[rb.name]) * ANGSTROM:
                out.append((ra.chain, ra.seq_num, rb.chain, rb.seq_num, d))
    return out


def to_system(pdb: Pdb, temperature: float = 0.35, seed: int = 1, contacts: str = "links") -> System:
    """The engine system of a structure (pdb::to_model).  contacts: "links"
    (LINK records, as the reference), "derive" (CA overlaps, pdb::add_contacts)
    or "both"."""
    beads, chain, seq, atype = [], [], [], []
    bead_of = {}
    for ci, (ch, residues) in enumerate(pdb.chains.items()):
        k = 0
        for r in residues:
            ca = r.find("CA")
            if ca is None:
                continue
            bead_of[(ch, r.seq_num)] = len(beads)
            beads.append(ca)
            chain.append(ci)
            seq.append(k)
            atype.append(AA.index(r.name) if r.name in AA else 0)
            k += 1
    n = len(beads)
    if n == 0:
        raise ValueError("the structure has no CA atom")
    pos = np.asarray(beads, dtype=np.float64)
    chain = np.asarray(chain, dtype=np.int32)
    seq = np.asarray(seq, dtype=np.int32)
    t1, t2, td, ang, dih = [], [], [], ([], [], [], []), ([], [], [], [], [])
    for c in np.unique(chain):
        idx = np.nonzero(chain == c)[0]
        L = len(idx)
        if L >= 2:
            t1 += idx[:-1].tolist()
            t2 += idx[1:].tolist()
            td += np.linalg.norm(pos[idx[1:]] - pos[idx[:-1]], axis=1).tolist()
        if L >= 3:
            th, ph = bonded_natives(pos[idx])
            for k, t in enumerate(th):
                ang[0].append(idx[k]); ang[1].append(idx[k + 1]); ang[2].append(idx[k + 2]); ang[3].append(t)
            for k, p in enumerate(ph):
                dih[0].append(idx[k]); dih[1].append(idx[k + 1]); dih[2].append(idx[k + 2])
                dih[3].append(idx[k + 3]); dih[4].append(p)
    pairs = {}
    ss = []
    taken = set()
    for (c1, s1, c2, s2, _len) in pdb.ssbonds:
        a, b = bead_of.get((c1, s1)), bead_of.get((c2, s2))
        if a is None or b is None:
            continue
        a, b = min(a, b), max(a, b)
        if (a, b) in taken:
            continue
        taken.add((a, b))
        ss.append((a, b, float(np.linalg.norm(pos[a] - pos[b]))))
    srcs = []
    if contacts in ("links", "both"):
        srcs += [(l[0], l[1], l[3], l[4]) for l in pdb.links]
    if contacts in ("derive", "both"):
        srcs += [(d[0], d[1], d[2], d[3]) for d in derive_contacts(pdb)]
    for (c1, s1, c2, s2) in srcs:
        a, b = bead_of.get((c1, s1)), bead_of.get((c2, s2))
        if a is None or b is None or a == b:
            continue
        a, b = min(a, b), max(a, b)
        if (a, b) in taken or (a, b) in pairs:
            continue
        pairs[(a, b)] = float(np.linalg.norm(pos[a] - pos[b]))
    nat = sorted(pairs.items())
    as32 = lambda x: np.asarray(x, dtype=np.int32)
    asf = lambda x: np.asarray(x, dtype=np.float64)
    dihs = (as32(dih[0]), as32(dih[1]), as32(dih[2]), as32(dih[3]), asf(dih[4]))
    return System(
        n=n, chain=chain, seq=seq, atype=np.asarray(atype, dtype=np.uint8), cell=np.asarray(pdb.cell, dtype=np.float64),
        r=pos.copy(),
        tethers=(as32(t1), as32(t2), asf(td)),
        angles=(as32(ang[0]), as32(ang[1]), as32(ang[2]), asf(ang[3])),
        dihedrals=dihs,
        natives=(as32([p[0][0] for p in nat]), as32([p[0][1] for p in nat]), asf([p[1] for p in nat])),
        temperature=float(temperature), seed=int(seed),
        meta={"ssbonds": ss, "chains": [int((chain == c).sum()) for c in np.unique(chain)]},
        chirals=chirals_of(dihs, pos),
        ssbonds=(as32([x[0] for x in ss]), as32([x[1] for x in ss])),
    )


def _fmt_real(x: float, width: int, prec: int) -> str:
    s = f"{x:{width}.{prec}f}"
    if len(s) > width:
        raise ValueError(f"{x} does not fit a {width}-column PDB field")
    return s


def write_pdb(system: System, frames=None, chain_ids: str = "ABCDEFGHIJKLMNOPQRSTUVWXYZ") -> str:
    """CA-only PDB text of a system: its native contacts as LINK records and
    its disulfides as SSBOND records, then one MODEL block per frame
    (positions [n, 3] in internal units; default: the system's own)."""
    frames = [system.r] if frames is None else list(frames)
    cid = lambda c: chain_ids[int(c) % len(chain_ids)]
    lines = []
    if np.any(system.cell):
        c = np.asarray(system.cell) / ANGSTROM
        lines.append(f"CRYST1{_fmt_real(c[0], 9, 3)}{_fmt_real(c[1], 9, 3)}{_fmt_real(c[2], 9, 3)}".ljust(80))
    names = [AA[int(t)] for t in system.atype]
    for k, (a, b, d) in enumerate(system.meta.get("ssbonds", [])):
        line = list(" " * 80)
        line[0:6] = "SSBOND"
        line[7:10] = f"{k + 1:3d}"
        line[11:14] = "CYS"
        line[15] = cid(system.chain[a])
        line[17:21] = f"{int(system.seq[a]) + 1:4d}"
        line[25:28] = "CYS"
        line[29] = cid(system.chain[b])
        line[31:35] = f"{int(system.seq[b]) + 1:4d}"
        line[73:78] = _fmt_real(d / ANGSTROM, 5, 2)
        lines.append("".join(line))
    i1, i2, nd = system.natives
    for a, b, d in zip(i1.tolist(), i2.tolist(), nd.tolist()):
        line = list(" " * 80)
        line[0:6] = "LINK  "
        line[12:16] = " CA "
        line[17:20] = names[a]
        line[21] = cid(system.chain[a])
        line[22:26] = f"{int(system.seq[a]) + 1:4d}"
        line[42:46] = " CA "
        line[47:50] = names[b]
        line[51] = cid(system.chain[b])
        line[52:56] = f"{int(system.seq[b]) + 1:4d}"
        line[73:78] = _fmt_real(d / ANGSTROM, 5, 2)
        lines.append("".join(line))
    for m, r in enumerate(frames):
        r = np.asarray(r).reshape(-1, 3) / ANGSTROM
        if len(frames) > 1:
            lines.append(f"MODEL     {m + 1:4d}".ljust(80))
        for i in range(system.n):
            line = (f"ATOM  {i + 1:5d}  CA  {names[i]:>3s} {cid(system.chain[i])}{int(system.seq[i]) + 1:4d}    "
                    f"{_fmt_real(r[i, 0], 8, 3)}{_fmt_real(r[i, 1], 8, 3)}{_fmt_real(r[i, 2], 8, 3)}")
            lines.append(line.ljust(80))
            if i + 1 == system.n or system.chain[i + 1] != system.chain[i]:
                lines.append(f"TER   {i + 2:5d}      {names[i]:>3s} {cid(system.chain[i])}{int(system.seq[i]) + 1:4d}".ljust(80))
        if len(frames) > 1:
            lines.append("ENDMDL".ljust(80))
    lines.append("END".ljust(80))
    return "\n".join(lines) + "\n"
