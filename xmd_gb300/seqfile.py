"""Sequence files and contact maps: XMD's `model: seqfile:` input.

A sequence file (src/files/seq_file.cpp:9-134) lists chains, each a one-letter
residue string plus named maps.  A map (src/files/map_file.cpp:68-112) holds
three CSV tables: contacts (i1, i2, length), angles (i1, i2, i3, theta) and
dihedrals (i1, i2, i3, i4, phi), in chain-local indices, given inline or with
`from-file:`, and moved by `shift:`.  Lengths and angles are raw internal
units (radians, 5 A).

to_system() builds the replica as main.cpp does from such a model:

* tethers of every consecutive pair with the default bond length
  (main.cpp:408-413);
* native angles and dihedrals where a map gives them, heuristic ones on every
  other consecutive triple and quadruple (seq_file.cpp:97-129);
* Go contacts from the map contacts;
* starting positions from model::morph_into_saw (model.cpp:101-173) driven by
  the reference's generator seeded with `general: seed`, which the Langevin
  step then continues (main.cpp:112, 130, 214): the replica's noise seed is
  the generator's state after the morph.

Departures from the shipped reader, each for a defect: chain_idx is set and
seq_idx counts within each chain (the reader sets no chain and numbers
residues across chains, seq_file.cpp:12-32); `infer box` takes each axis'
extent (model.cpp:149-172 measures x for all three, from
numeric_limits::min()); a CSV `from-file:` inside a map is read relative to
the map, not the working directory.

The YAML reader below covers what these files use: block maps and sequences,
flow sequences, anchors and aliases, plain, single- and double-quoted scalars
(line folding, escaped line breaks) and literal block scalars.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .abi import AA
from .synth import ANGSTROM, System

LETTERS = "ARNDCEQGHILKMFPSTWYV"     # amino_acid(char), src/types/amino_acid.cpp:8-18
_LETTER_AA = {c: AA.index(n) for c, n in zip(LETTERS, ["ALA", "ARG", "ASN", "ASP", "CYS", "GLU", "GLN", "GLY",
                                                       "HIS", "ILE", "LEU", "LYS", "MET", "PHE", "PRO", "SER",
                                                       "THR", "TRP", "TYR", "VAL"])}


# ---- YAML subset ----------------------------------------------------------------

def _strip_comment(s: str) -> str:
    q = None
    for k, c in enumerate(s):
        if q:
            if c == q and not (q == '"' and k > 0 and s[k - 1] == "\\"):
                q = None
        elif c in "\"'":
            q = c
        elif c == "#" and (k == 0 or s[k - 1] in " \t"):
            return s[:k].rstrip()
    return s.rstrip()


def _split_key(body: str, lineno: int):
    q = None
    for k, c in enumerate(body):
        if q:
            if c == q:
                q = None
        elif c in "\"'":
            q = c
        elif c == ":" and (k + 1 == len(body) or body[k + 1] in " \t"):
            key = body[:k].strip()
            if key[:1] in "\"'":
                key = key[1:-1]
            return key, body[k + 1:].strip()
    raise ValueError(f"line {lineno}: expected 'key: value'")


_ESC = {"n": "\n", "t": "\t", "\\": "\\", '"': '"', "/": "/", "0": "\0", " ": " ", "r": "\r"}


def _fold_dquoted(raw: str) -> str:
    """Body of a double-quoted scalar (without the quotes): escapes, escaped
    line breaks (joined without a space, the next line's indentation
    dropped) and folded line breaks (one space; an empty line gives '\\n')."""
    lines = raw.split("\n")
    out = lines[0]
    k = 1
    while k < len(lines):
        nxt = lines[k].lstrip(" \t")
        if out.endswith("\\") and not out.endswith("\\\\"):
            out = out[:-1] + nxt
        else:
            out = out.rstrip(" \t")
            empties = 0
            while nxt == "" and k + 1 < len(lines):
                empties += 1
                k += 1
                nxt = lines[k].lstrip(" \t")
            out += ("\n" * empties if empties else " ") + nxt
        k += 1
    res, k = [], 0
    while k < len(out):
        c = out[k]
        if c == "\\" and k + 1 < len(out):
            e = out[k + 1]
            if e == "x":
                res.append(chr(int(out[k + 2:k + 4], 16)))
                k += 4
                continue
            if e == "u":
                res.append(chr(int(out[k + 2:k + 6], 16)))
                k += 6
                continue
            res.append(_ESC.get(e, e))
            k += 2
            continue
        res.append(c)
        k += 1
    return "".join(res)


class _Yaml:
    def __init__(self, text: str):
        self.lines = text.replace("\r\n", "\n").split("\n")
        self.i = 0
        self.anchors: dict = {}

    @staticmethod
    def _ind(line: str) -> int:
        return len(line) - len(line.lstrip(" "))

    def _skip(self):
        while self.i < len(self.lines):
            s = self.lines[self.i].strip()
            if s == "" or s.startswith("#") or s in ("---", "..."):
                self.i += 1
                continue
            break

    def parse(self):
        self._skip()
        if self.i >= len(self.lines):
            return None
        return self._block(self._ind(self.lines[self.i]))

    def _is_seq_line(self, k: int) -> bool:
        b = self.lines[k].strip()
        return b == "-" or b.startswith("- ")

    def _block(self, ind: int):
        self._skip()
        return self._seq(ind) if self._is_seq_line(self.i) else self._map(ind)

    def _map(self, ind: int) -> dict:
        out = {}
        while True:
            self._skip()
            if self.i >= len(self.lines):
                break
            line = self.lines[self.i]
            cur = self._ind(line)
            if cur < ind or (cur == ind and self._is_seq_line(self.i)):
                break
            if cur > ind:
                raise ValueError(f"line {self.i + 1}: unexpected indentation")
            key, rest = _split_key(_strip_comment(line.strip()), self.i + 1)
            self.i += 1
            out[key] = self._value(rest, ind, in_map=True)
        return out

    def _seq(self, ind: int) -> list:
        out = []
        while True:
            self._skip()
            if self.i >= len(self.lines):
                break
            line = self.lines[self.i]
            cur = self._ind(line)
            if cur < ind or not self._is_seq_line(self.i):
                break
            if cur > ind:
                raise ValueError(f"line {self.i + 1}: unexpected indentation")
            rest = line.strip()[1:].strip()
            body = _strip_comment(rest)
            if body and body[0] not in "\"'[{&*|>" and re.match(r"^[^:]+:(\s|$)", body):
                # "- key: value" opens a mapping whose keys sit at cur + 2
                self.lines[self.i] = " " * (cur + 2) + rest
                out.append(self._map(cur + 2))
            else:
                self.i += 1
                out.append(self._value(rest, ind, in_map=False))
        return out

    def _value(self, rest: str, ind: int, in_map: bool):
        anchor = None
        rest = rest.strip()
        if rest.startswith("&"):
            name, _, rest = rest[1:].partition(" ")
            anchor, rest = name, rest.strip()
        body = _strip_comment(rest)
        if body == "":
            self._skip()
            if self.i < len(self.lines):
                nind = self._ind(self.lines[self.i])
                if nind > ind:
                    val = self._block(nind)
                elif in_map and nind == ind and self._is_seq_line(self.i):
                    val = self._seq(ind)
                else:
                    val = None
            else:
                val = None
        elif body.startswith("*"):
            name = body[1:].strip()
            if name not in self.anchors:
                raise ValueError(f"line {self.i}: unknown alias *{name}")
            val = self.anchors[name]
        elif body[0] in "|>":
            val = self._block_scalar(body, ind)
        elif body[0] == '"':
            val = self._dquoted(rest)
        elif body[0] == "'":
            val = self._squoted(rest)
        elif body[0] in "[{":
            val = self._flow_text(body)
        else:
            val = body
        if anchor:
            self.anchors[anchor] = val
        return val

    def _dquoted(self, rest: str) -> str:
        buf = rest[1:]
        while True:
            k, esc = 0, False
            while k < len(buf):
                c = buf[k]
                if esc:
                    esc = False
                elif c == "\\":
                    esc = True
                elif c == '"':
                    return _fold_dquoted(buf[:k])
                k += 1
            if self.i >= len(self.lines):
                raise ValueError("unterminated double-quoted scalar")
            buf += "\n" + self.lines[self.i]
            self.i += 1

    def _squoted(self, rest: str) -> str:
        buf = rest[1:]
        while True:
            k = 0
            while k < len(buf):
                if buf[k] == "'":
                    if k + 1 < len(buf) and buf[k + 1] == "'":
                        k += 2
                        continue
                    return re.sub(r"[ \t]*\n[ \t]*", " ", buf[:k]).replace("''", "'")
                k += 1
            if self.i >= len(self.lines):
                raise ValueError("unterminated single-quoted scalar")
            buf += "\n" + self.lines[self.i]
            self.i += 1

    def _block_scalar(self, head: str, ind: int) -> str:
        m = re.match(r"^([|>])([+-]?)(\d?)([+-]?)$", head.strip())
        if not m:
            raise ValueError(f"line {self.i}: bad block scalar header {head!r}")
        style, chomp = m.group(1), m.group(2) or m.group(4)
        body, content_ind = [], int(m.group(3)) + ind if m.group(3) else None
        while self.i < len(self.lines):
            line = self.lines[self.i]
            if line.strip() == "":
                body.append("")
                self.i += 1
                continue
            cur = self._ind(line)
            if content_ind is None:
                if cur <= ind:
                    break
                content_ind = cur
            if cur < content_ind:
                break
            body.append(line[content_ind:])
            self.i += 1
        while body and body[-1] == "" and chomp != "+":
            body.pop()
        if style == "|":
            text = "\n".join(body)
        else:
            text = re.sub(r"(?<!\n)\n(?!\n)", " ", "\n".join(body))
        return text + ("\n" if chomp != "-" and body else "")

    def _flow_text(self, body: str):
        buf = body
        while True:
            depth, q = 0, None
            for c in buf:
                if q:
                    if c == q:
                        q = None
                elif c in "\"'":
                    q = c
                elif c in "[{":
                    depth += 1
                elif c in "]}":
                    depth -= 1
            if depth == 0:
                break
            if self.i >= len(self.lines):
                raise ValueError("unterminated flow collection")
            buf += " " + _strip_comment(self.lines[self.i].strip())
            self.i += 1
        val, _ = self._flow(buf.strip(), 0)
        return val

    def _flow(self, s: str, k: int):
        while s[k] == " ":
            k += 1
        if s[k] == "[":
            out, k = [], k + 1
            while True:
                while s[k] in " ,":
                    k += 1
                if s[k] == "]":
                    return out, k + 1
                v, k = self._flow(s, k)
                out.append(v)
        if s[k] == "{":
            out, k = {}, k + 1
            while True:
                while s[k] in " ,":
                    k += 1
                if s[k] == "}":
                    return out, k + 1
                j = k
                while s[j] not in ":}":
                    j += 1
                key = s[k:j].strip().strip("\"'")
                v, k = self._flow(s, j + 1)
                out[key] = v
        if s[k] == '"':
            j = k + 1
            while s[j] != '"' or s[j - 1] == "\\":
                j += 1
            return _fold_dquoted(s[k + 1:j]), j + 1
        if s[k] == "'":
            j = s.index("'", k + 1)
            return s[k + 1:j], j + 1
        j = k
        while j < len(s) and s[j] not in ",]}":
            j += 1
        tok = s[k:j].strip()
        if tok.startswith("*"):
            if tok[1:] not in self.anchors:
                raise ValueError(f"unknown alias {tok}")
            return self.anchors[tok[1:]], j
        return tok, j


def load_yaml(text: str):
    """Parse the YAML subset of sequence and map files (strings stay strings)."""
    return _Yaml(text).parse()


# ---- maps and sequence files ------------------------------------------------------

def _csv_records(text: str) -> list[dict]:
    """csv_file (src/files/csv.cpp): a header row, then records by column name."""
    rows = [ln.strip() for ln in str(text).split("\n") if ln.strip()]
    if not rows:
        return []
    head = [h.strip() for h in rows[0].split(",")]
    out = []
    for ln in rows[1:]:
        f = [x.strip() for x in ln.split(",")]
        out.append({h: f[k] for k, h in enumerate(head) if k < len(f)})
    return out


@dataclass
class ContactMap:
    """map_file: chain-local contacts, native angles and dihedrals."""
    contacts: list = field(default_factory=list)    # (i1, i2, length)
    angles: list = field(default_factory=list)      # (i1, i2, i3, theta)
    dihedrals: list = field(default_factory=list)   # (i1, i2, i3, i4, phi)

    def shift(self, k: int) -> "ContactMap":
        """map_file::shift (map_file.cpp:7-26)."""
        return ContactMap([(a + k, b + k, d) for a, b, d in self.contacts],
                          [(a + k, b + k, c + k, t) for a, b, c, t in self.angles],
                          [(a + k, b + k, c + k, e + k, p) for a, b, c, e, p in self.dihedrals])


def read_map(node, base: Path | None = None) -> ContactMap:
    """convert<map_file>::decode (map_file.cpp:68-112): node is a map file's
    text, or its parsed YAML mapping."""
    if isinstance(node, str):
        node = load_yaml(node)

    def table(key):
        v = node.get(key) if node else None
        if v is None:
            return []
        if isinstance(v, dict) and "from-file" in v:
            path = Path(v["from-file"])
            v = (path if path.is_absolute() or base is None else base / path).read_text()
        return _csv_records(v)

    m = ContactMap()
    for r in table("contacts"):
        m.contacts.append((int(r["i1"]), int(r["i2"]), float(r["length"])))
    for r in table("angles"):
        m.angles.append((int(r["i1"]), int(r["i2"]), int(r["i3"]), float(r["theta"])))
    for r in table("dihedrals"):
        m.dihedrals.append((int(r["i1"]), int(r["i2"]), int(r["i3"]), int(r["i4"]), float(r["phi"])))
    return m


@dataclass
class SeqChain:
    codes: str                                     # one-letter residue codes
    maps: list = field(default_factory=list)       # ContactMap, already shifted


@dataclass
class SeqModel:
    chains: list                                   # SeqChain


def read_seq(source, base: Path | None = None) -> SeqModel:
    """seq_file::seq_file (seq_file.cpp:9-134).  source: a path, or the
    file's text (then `from-file:` maps resolve against base)."""
    if isinstance(source, Path) or (isinstance(source, str) and "\n" not in source and Path(source).exists()):
        path = Path(source)
        text, base = path.read_text(), path.parent
    else:
        text = source
    root = load_yaml(text)
    chains = []
    for ch in root["model"]["chains"]:
        codes = re.sub(r"\s+", "", str(ch["seq"]))
        for c in codes:
            if c not in _LETTER_AA:
                raise ValueError(f"unknown residue code {c!r}")
        maps = []
        for _name, entry in (ch.get("maps") or {}).items():
            if "from-file" in entry:
                mpath = Path(entry["from-file"])
                mpath = mpath if mpath.is_absolute() or base is None else base / mpath
                mf = read_map(mpath.read_text(), mpath.parent)
            elif "map" in entry:
                mf = read_map(entry["map"], base)
            else:
                raise ValueError("map entry without 'from-file' or 'map'")
            if "shift" in entry:
                mf = mf.shift(int(entry["shift"]))
            maps.append(mf)
        chains.append(SeqChain(codes, maps))
    return SeqModel(chains)


# ---- the reference's generator and morph_into_saw -----------------------------------

_M64 = (1 << 64) - 1


class RandGen:
    """rand_gen (include/xmd/random/rand_gen.h): xorshift with a
    multiplicative output, uniform from the top 32 bits, Box-Muller normals."""

    def __init__(self, seed: int):
        self.state = int(seed) & _M64

    def next(self) -> int:
        res = (self.state * 0xd989bcacc137dcd5) & _M64
        s = self.state
        s ^= s >> 11
        s ^= (s << 31) & _M64
        s ^= s >> 18
        self.state = s
        return res

    def uniform(self, a: float = 0.0, b: float = 1.0) -> float:
        u = float(self.next() >> 32) * (1.0 / 4294967296.0)
        return (b - a) * u + a

    def normal_x2(self):
        r1, r2 = self.uniform(), self.uniform()
        r = math.sqrt(-2.0 * math.log(r1)) if r1 > 0 else math.inf
        if math.isnan(r):
            r = 0.0
        t = 2.0 * math.pi * r2
        return r * math.cos(t), r * math.sin(t)

    def normal(self) -> float:
        return self.normal_x2()[0]

    def sphere(self) -> np.ndarray:
        x, y = self.normal_x2()
        z = self.normal()
        v = np.array([x, y, z])
        return v / math.sqrt(float(v @ v))


def _rotate(axis: np.ndarray, angle: float, v: np.ndarray) -> np.ndarray:
    """Rotation of v by angle about the unit axis (Rodrigues)."""
    c, s = math.cos(angle), math.sin(angle)
    return v * c + np.cross(axis, v) * s + axis * float(axis @ v) * (1.0 - c)


def _perp(v: np.ndarray) -> np.ndarray:
    # perp_v, model.cpp:93-99
    p1, p2 = np.cross(v, [1.0, 0.0, 0.0]), np.cross(v, [0.0, 1.0, 0.0])
    p = p1 if np.linalg.norm(p1) > np.linalg.norm(p2) else p2
    return p / np.linalg.norm(p)


def morph_into_saw(lens, gen: RandGen, bond: float | None, density: float, infer_box: bool = False):
    """model::morph_into_saw (model.cpp:101-173): per chain a uniform start in
    the cube of side (n / density)^(1/3), a uniform direction, then steps of
    `bond` turned by a spread angle U(-pi/12, pi/12) about perp(dir) and an
    around angle U(-pi, pi) about dir.  Returns (r[n, 3], cell[3]); cell is
    zero unless infer_box (then each axis' extent)."""
    n = int(sum(lens))
    cell_a = (n / density) ** (1.0 / 3.0)
    r = np.zeros((n, 3))
    off = 0
    for L in lens:
        pos = np.array([gen.uniform(-cell_a / 2.0, cell_a / 2.0) for _ in range(3)])
        d = gen.sphere()
        for k in range(L):
            nxt = pos.copy()
            if k + 1 < L:
                b = bond if bond is not None else 0.0   # seq-file residues all sit at the origin
                nxt = nxt + d * b
                spread = gen.uniform(-math.pi / 12.0, math.pi / 12.0)
                d1 = _rotate(_perp(d), spread, d)
                around = gen.uniform(-math.pi, math.pi)
                d2 = _rotate(d, around, d1)
                d = d2 / np.linalg.norm(d2)
            r[off + k] = pos
            pos = nxt
        off += L
    cell = np.zeros(3)
    if infer_box and n:
        cell = r.max(axis=0) - r.min(axis=0)
    return r, cell


# ---- the replica -------------------------------------------------------------------

def to_system(model: SeqModel, seed: int = 42, bond: float | None = 3.8 * ANGSTROM,
              density: float = 1e-3 / ANGSTROM**3, infer_box: bool = False,
              temperature: float = 0.0, heuristic: bool = True) -> System:
    """The replica main.cpp builds from a sequence-file model (see the module
    docstring).  seed: `general: seed`; bond, density, infer_box: `model:
    morph into SAW`.  heuristic=False leaves out the heuristic angles and
    dihedrals (as the shipped driver, which builds no heuristic term)."""
    lens = [len(c.codes) for c in model.chains]
    n = sum(lens)
    chain = np.concatenate([np.full(L, c, np.int32) for c, L in enumerate(lens)]) if n else np.zeros(0, np.int32)
    seq = np.concatenate([np.arange(L, dtype=np.int32) for L in lens]) if n else np.zeros(0, np.int32)
    atype = np.array([_LETTER_AA[c] for ch in model.chains for c in ch.codes], dtype=np.uint8)
    t1, t2 = [], []
    ang, hang = ([], [], [], []), ([], [], [])
    dih, hdih = ([], [], [], [], []), ([], [], [], [])
    nat = {}
    off = 0
    for ch, L in zip(model.chains, lens):
        taken_a, taken_d = set(), set()
        for mf in ch.maps:
            for a, b, d in mf.contacts:
                if not (0 <= a < L and 0 <= b < L) or a == b:
                    raise ValueError(f"map contact ({a}, {b}) outside its chain")
                key = (off + min(a, b), off + max(a, b))
                nat[key] = d
            for a, b, c, t in mf.angles:
                if (a, b, c) in taken_a:
                    raise ValueError(f"map angle ({a}, {b}, {c}) given twice")
                taken_a.add((a, b, c))
                for q, x in zip(ang, (off + a, off + b, off + c, t)):
                    q.append(x)
            for a, b, c, e, p in mf.dihedrals:
                if (a, b, c, e) in taken_d:
                    raise ValueError(f"map dihedral ({a}, {b}, {c}, {e}) given twice")
                taken_d.add((a, b, c, e))
                for q, x in zip(dih, (off + a, off + b, off + c, off + e, p)):
                    q.append(x)
        for k in range(L - 1):
            t1.append(off + k)
            t2.append(off + k + 1)
            if heuristic and k + 2 < L and (k, k + 1, k + 2) not in taken_a:
                for q, x in zip(hang, (off + k, off + k + 1, off + k + 2)):
                    q.append(x)
            if heuristic and k + 3 < L and (k, k + 1, k + 2, k + 3) not in taken_d:
                for q, x in zip(hdih, (off + k, off + k + 1, off + k + 2, off + k + 3)):
                    q.append(x)
        off += L
    gen = RandGen(seed)
    r, cell = morph_into_saw(lens, gen, bond, density, infer_box)
    i32 = lambda x: np.asarray(x, dtype=np.int32)
    f64 = lambda x: np.asarray(x, dtype=np.float64)
    nk = sorted(nat)
    return System(
        n=n, chain=chain, seq=seq, atype=atype, cell=cell, r=r,
        tethers=(i32(t1), i32(t2), np.zeros(len(t1))),            # default bond length
        angles=(i32(ang[0]), i32(ang[1]), i32(ang[2]), f64(ang[3])),
        dihedrals=(i32(dih[0]), i32(dih[1]), i32(dih[2]), i32(dih[3]), f64(dih[4])),
        natives=(i32([a for a, _ in nk]), i32([b for _, b in nk]), f64([nat[k] for k in nk])),
        temperature=float(temperature), seed=gen.state,
        meta={"chains": lens, "source": "seqfile"},
        heur_angles=(i32(hang[0]), i32(hang[1]), i32(hang[2])) if heuristic else None,
        heur_dihedrals=(i32(hdih[0]), i32(hdih[1]), i32(hdih[2]), i32(hdih[3])) if heuristic else None,
    )


def write_map(m: ContactMap) -> str:
    """A map file holding m (the layout of convert<map_file>::encode,
    map_file.cpp:29-66, with each table's own records)."""
    def block(head, rows):
        body = "\n".join("  " + ",".join(repr(x) if isinstance(x, float) else str(x) for x in r) for r in rows)
        return f"{head}: |-\n  " + ",".join(
            {"contacts": ["i1", "i2", "length"], "angles": ["i1", "i2", "i3", "theta"],
             "dihedrals": ["i1", "i2", "i3", "i4", "phi"]}[head]) + ("\n" + body if rows else "") + "\n"
    return block("contacts", m.contacts) + block("angles", m.angles) + block("dihedrals", m.dihedrals)
