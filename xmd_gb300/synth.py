"""Seeded synthetic systems with the shapes of the benchmark configurations.

There is no dataset behind these configurations: chains are generated here.
Initial conformations restate the reference's chain generator
(model::morph_into_saw, src/model/model.cpp:101-147: random start in a cube of
side cbrt(n / density), direction on the sphere, each step turned by a
spread angle in [-pi/12, pi/12] about an axis perpendicular to the direction
and by an angle in [-pi, pi] about the direction), with a light overlap
rejection so that starting structures are self-avoiding.  Native structures
(contact maps with r < 7.5 A and |i-j| >= 3, native angles and dihedrals) come
from a second, compact random walk confined to a sphere.  numpy's PCG64 seeds
every draw, so a (config, seed) pair always yields the same system.

All lengths returned are in the engine's internal unit (1 = 5 A).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .abi import AA

ANGSTROM = 0.2  # include/xmd/utils/units.h:15
CHARGED_POS = [AA.index("ARG"), AA.index("LYS")]
CHARGED_NEG = [AA.index("ASP"), AA.index("GLU")]
NEUTRAL = [k for k in range(20) if k not in CHARGED_POS + CHARGED_NEG]


@dataclass
class System:
    """One replica: topology, native structure and initial state."""
    n: int
    chain: np.ndarray            # int32[n]
    seq: np.ndarray              # int32[n]
    atype: np.ndarray            # uint8[n]
    cell: np.ndarray             # float64[3], 0 = open
    r: np.ndarray                # float64[n, 3] initial positions
    tethers: tuple               # (i1, i2, nat_dist)
    angles: tuple                # (i1, i2, i3, theta0)
    dihedrals: tuple             # (i1, i2, i3, i4, phi0)
    natives: tuple               # (i1, i2, nat_dist)
    temperature: float = 0.0
    seed: int = 0
    meta: dict = field(default_factory=dict)
    chirals: tuple | None = None  # (i1, i2, i3, i4, nat_factor, nat_chir)
    ssbonds: tuple | None = None  # (i1, i2) native disulfide bonds
    heur_angles: tuple | None = None     # (i1, i2, i3): angles without a native value
    heur_dihedrals: tuple | None = None  # (i1, i2, i3, i4): dihedrals without a native value
    afm_vel: tuple | None = None         # (bead, orig[k, 3] (NaN: start position), vel[k, 3]) velocity AFM tips
    afm_force: tuple | None = None       # (bead, F[k, 3]) force AFM tips


def _unit(v):
    return v / np.linalg.norm(v)


def _perp(v):
    # perp_v: model.cpp:93-99
    p1 = np.cross(v, [1.0, 0.0, 0.0])
    p2 = np.cross(v, [0.0, 1.0, 0.0])
    p = p1 if np.linalg.norm(p1) > np.linalg.norm(p2) else p2
    return _unit(p)


def _rot(v, axis, ang):
    # Rodrigues rotation of v about the unit axis
    c, s = math.cos(ang), math.sin(ang)
    return v * c + np.cross(axis, v) * s + axis * np.dot(axis, v) * (1.0 - c)


def _sphere(rng):
    v = rng.normal(size=3)
    return _unit(v)


def saw_chain(rng, n, bond, start, min_sep=4.0 * ANGSTROM, tries=16, others=None, window=None):
    """A persistent random walk as in morph_into_saw with overlap rejection:
    each step turns the direction by a spread angle about perp_v(dir) and an
    around angle about dir; `tries` turns are drawn at once and the first
    whose bead keeps min_sep from earlier beads (the last `window` of them,
    or all) is taken (else the best)."""
    max_spread, max_around = math.pi / 12.0, math.pi
    pos = np.empty((n, 3))
    pos[0] = start
    d = _sphere(rng)
    for k in range(1, n):
        sp = rng.uniform(-max_spread, max_spread, size=tries)[:, None]
        ar = rng.uniform(-max_around, max_around, size=tries)[:, None]
        p = _perp(d)
        # Rodrigues rotations (p is perpendicular to d)
        v1 = d * np.cos(sp) + np.cross(p, d) * np.sin(sp)
        dv = (v1 * d).sum(axis=1, keepdims=True)
        v2 = v1 * np.cos(ar) + np.cross(d, v1) * np.sin(ar) + d * dv * (1.0 - np.cos(ar))
        v2 /= np.linalg.norm(v2, axis=1, keepdims=True)
        cand = pos[k - 1] + bond * v2
        dmin = np.full(tries, np.inf)
        if k >= 3:
            lo = 0 if window is None else max(0, k - 2 - window)
            dmin = np.sqrt(((cand[:, None, :] - pos[None, lo:k - 2, :]) ** 2).sum(axis=2).min(axis=1))
        if others is not None and len(others):
            do = np.sqrt(((cand[:, None, :] - others[None, :, :]) ** 2).sum(axis=2).min(axis=1))
            dmin = np.minimum(dmin, do)
        ok = np.nonzero(dmin >= min_sep)[0]
        pick = ok[0] if len(ok) else int(np.argmax(dmin))
        pos[k], d = cand[pick], v2[pick]
    return pos


def compact_walk(rng, n, bond, density=1.0 / 120.0, min_sep=4.2 * ANGSTROM, tries=48):
    """A random walk confined to a sphere holding n beads at `density` (per A^3),
    with overlap rejection: the native conformation of one chain.  Each step
    draws `tries` candidate directions at once and keeps the first admissible
    one (else the least bad)."""
    radius = (3.0 * n / (4.0 * math.pi * density)) ** (1.0 / 3.0) * ANGSTROM
    radius = max(radius, 2.0 * bond)
    pos = np.zeros((n, 3))
    batch = 8
    for k in range(1, n):
        best, best_score = None, -np.inf
        for _ in range(0, tries, batch):
            dirs = rng.normal(size=(batch, 3))
            dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
            cand = pos[k - 1] + bond * dirs
            if k >= 2:
                d2 = ((cand[:, None, :] - pos[None, :k - 1, :]) ** 2).sum(axis=2)
                dmin = np.sqrt(d2.min(axis=1))
            else:
                dmin = np.full(batch, np.inf)
            out = np.maximum(0.0, np.linalg.norm(cand, axis=1) - radius)
            score = np.minimum(dmin - min_sep, 0.0) - out
            ok = np.nonzero(score >= 0.0)[0]
            if len(ok):
                best = cand[ok[0]]
                break
            j = int(np.argmax(score))
            if score[j] > best_score:
                best_score, best = score[j], cand[j]
        pos[k] = best
    return pos


def bonded_natives(pos):
    """Native angles and dihedrals of one chain, with the force terms'
    conventions (angle/native.cpp:20-30, dihedral/complex_native.cpp:20-28)."""
    b = pos[1:] - pos[:-1]                      # bond vectors
    r12, r23 = b[:-1], b[1:]
    ct = -(r12 * r23).sum(axis=1) / (np.linalg.norm(r12, axis=1) * np.linalg.norm(r23, axis=1))
    th = np.arccos(np.clip(ct, -1.0, 1.0))
    r12, r23, r34 = b[:-2], b[1:-1], b[2:]
    x1, x2 = np.cross(r12, r23), np.cross(r23, r34)
    cp = (x1 * x2).sum(axis=1) / (np.linalg.norm(x1, axis=1) * np.linalg.norm(x2, axis=1))
    ph = np.arccos(np.clip(cp, -1.0, 1.0))
    ph = np.where((x1 * r34).sum(axis=1) < 0, -ph, ph)
    return th, ph


def chirals_of(dihedrals, pos):
    """Chiral quads over the dihedral quadruplets (i1..i4) with native
    positions pos[n, 3]: nat_factor = |r23|^-3 and nat_chir = r12 . (r23 x r34)
    * nat_factor, as main.cpp builds them from the model's dihedrals
    (src/freeform/main.cpp:376-393)."""
    i1, i2, i3, i4 = (np.asarray(x, dtype=np.int32) for x in dihedrals[:4])
    r12, r23, r34 = pos[i2] - pos[i1], pos[i3] - pos[i2], pos[i4] - pos[i3]
    fac = np.linalg.norm(r23, axis=1) ** -3 if len(i1) else np.zeros(0)
    chi = (r12 * np.cross(r23, r34)).sum(axis=1) * fac if len(i1) else np.zeros(0)
    return i1, i2, i3, i4, np.asarray(fac, dtype=np.float64), np.asarray(chi, dtype=np.float64)


def native_map(pos, cutoff=7.5 * ANGSTROM, min_sep=3):
    n = len(pos)
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=2)
    i1, i2 = np.nonzero(np.triu(d < cutoff, k=min_sep))
    return i1.astype(np.int32), i2.astype(np.int32), d[i1, i2].astype(np.float64)


def _types(rng, n, mode):
    if mode == "uniform20":
        return rng.integers(0, 20, size=n).astype(np.uint8)
    # +-1 charge with probability 0.1 each, realised through residue types
    u = rng.random(n)
    t = np.empty(n, dtype=np.uint8)
    pos_m, neg_m = u < 0.1, (u >= 0.1) & (u < 0.2)
    t[pos_m] = rng.choice(CHARGED_POS, size=pos_m.sum())
    t[neg_m] = rng.choice(CHARGED_NEG, size=neg_m.sum())
    rest = ~(pos_m | neg_m)
    t[rest] = rng.choice(NEUTRAL, size=rest.sum())
    return t


def make_system(chain_lengths, seed, box=None, density=1e-3, types="charged10",
                bond=3.8 * ANGSTROM, native=True, temperature=0.0, rng_seed=None, start="saw",
                saw_window=None, avoid_others=True):
    """Build one replica.  box: edge in internal units (periodic cube) or None
    for open boundaries; density (per A^3) sizes the starting cube.
    start="saw" begins from the extended walk (far from the native structure,
    as the benchmark configurations specify); start="native" places each chain
    in its native conformation, translated to its random start point (a start
    near equilibrium, where the dynamics does not amplify rounding)."""
    rng = np.random.default_rng(seed)
    lens = [int(x) for x in chain_lengths]
    n = sum(lens)
    chain = np.concatenate([np.full(L, c, dtype=np.int32) for c, L in enumerate(lens)])
    seq = np.concatenate([np.arange(L, dtype=np.int32) for L in lens])
    atype = _types(rng, n, types)
    if box is not None:
        a = box
    else:
        a = (n / density) ** (1.0 / 3.0) * ANGSTROM   # morph_into_saw cell_a
    r = np.empty((n, 3))
    tet_i1, tet_i2, tet_d = [], [], []
    ang = ([], [], [], [])
    dih = ([], [], [], [], [])
    nat = ([], [], [])
    natpos = np.zeros((n, 3))
    off = 0
    for c, L in enumerate(lens):
        start_pt = rng.uniform(-a / 2.0, a / 2.0, size=3)
        others = r[max(0, off - 2000):off] if (off and avoid_others) else None
        r[off:off + L] = saw_chain(rng, L, bond, start_pt, others=others, window=saw_window)
        if L >= 2:
            tet_i1 += list(range(off, off + L - 1))
            tet_i2 += list(range(off + 1, off + L))
            tet_d += [bond] * (L - 1)
        if native and L >= 3:
            npos = compact_walk(rng, L, bond)
            natpos[off:off + L] = npos
            if start == "native":
                r[off:off + L] = npos - npos.mean(axis=0) + start_pt
            th, ph = bonded_natives(npos)
            for k, t in enumerate(th):
                ang[0].append(off + k); ang[1].append(off + k + 1); ang[2].append(off + k + 2); ang[3].append(t)
            for k, p in enumerate(ph):
                dih[0].append(off + k); dih[1].append(off + k + 1); dih[2].append(off + k + 2)
                dih[3].append(off + k + 3); dih[4].append(p)
            i1, i2, dd = native_map(npos)
            nat[0].extend((i1 + off).tolist()); nat[1].extend((i2 + off).tolist()); nat[2].extend(dd.tolist())
        off += L
    cell = np.array([box, box, box], dtype=np.float64) if box is not None else np.zeros(3)
    as32 = lambda x: np.asarray(x, dtype=np.int32)
    asf = lambda x: np.asarray(x, dtype=np.float64)
    dihs = (as32(dih[0]), as32(dih[1]), as32(dih[2]), as32(dih[3]), asf(dih[4]))
    return System(
        n=n, chain=chain, seq=seq, atype=atype, cell=cell, r=r,
        tethers=(as32(tet_i1), as32(tet_i2), asf(tet_d)),
        angles=(as32(ang[0]), as32(ang[1]), as32(ang[2]), asf(ang[3])),
        dihedrals=dihs,
        natives=(as32(nat[0]), as32(nat[1]), asf(nat[2])),
        temperature=temperature, seed=int(rng_seed if rng_seed is not None else seed * 7919 + 17),
        meta={"chains": lens}, chirals=chirals_of(dihs, natpos),
    )


# ---- the benchmark configurations ------------------------------------------------

YAML_COMMON = """
langevin:
  enabled: true
  gamma factor: 2.0 1/tau
  temperature: 0.35 eps/kB
integrator:
  dt: 5e-3 tau
tether forces:
  enabled: true
native angles:
  enabled: true
complex native dihedrals:
  enabled: true
native contacts:
  enabled: true
  lj depth: 1 eps
Pauli exclusion:
  enabled: true
  r_excl: 4.0 A
"""


def yaml_for(config: str, precision: str = "fp64") -> str:
    """YAML overrides of a benchmark configuration (keys of defaults.yml)."""
    if config == "c1":   # 100 beads, no box, Go + Pauli + bonded, NL 18 A + 2 A skin
        extra = """
const ES:
  enabled: false
quasi-adiabatic potential:
  enabled: false
neighbor list:
  cutoff: 18 A
  skin: 2 A
"""
    elif config in ("c2", "c4", "c5"):   # + Debye-Hueckel, kappa^-1 = 10 A, eps_r = 80
        extra = """
const ES:
  enabled: true
  screening distance: 10.0 A
  permittivity: 80.0 eps_0
quasi-adiabatic potential:
  enabled: false
"""
    elif config == "c3":   # Go + DH + quasi-adiabatic
        extra = """
const ES:
  enabled: true
  screening distance: 10.0 A
  permittivity: 80.0 eps_0
quasi-adiabatic potential:
  enabled: true
"""
    else:
        raise ValueError(config)
    return YAML_COMMON + extra + f"engine:\n  precision: {precision}\n"


def config_c1(seed=1):
    return make_system([100], seed, box=None, types="charged10", temperature=0.35)


def config_c2(seed=2, chains=16, length=500):
    return make_system([length] * chains, seed, box=300.0 * ANGSTROM, types="charged10", temperature=0.35)


def config_c3(seed=3, chains=512, length=60):
    n = chains * length
    box = (n / 1e-3) ** (1.0 / 3.0) * ANGSTROM
    return make_system([length] * chains, seed, box=box, types="uniform20", temperature=0.35)


def c4_lengths(seed=4, count=256, lo=50, hi=800):
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), size=count))).astype(int)


def _c4_one(args):
    seed, k, L, T = args
    return make_system([int(L)], seed * 100003 + k, box=None, types="charged10",
                       temperature=float(T), rng_seed=seed * 7 + k * 131)


def config_c4(seed=4, count=256, workers=0):
    """256 single-chain replicas, lengths log-uniform in [50, 800], per-replica
    temperature uniform in [0.3, 0.6].  workers > 1 generates them in a spawned
    process pool (same systems, same order)."""
    lens = c4_lengths(seed, count)
    rng = np.random.default_rng(seed + 1000)
    temps = rng.uniform(0.3, 0.6, size=count)
    jobs = [(seed, k, int(L), float(temps[k])) for k, L in enumerate(lens)]
    if workers and workers > 1:
        import multiprocessing as mp
        from concurrent.futures import ProcessPoolExecutor
        with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            return list(ex.map(_c4_one, jobs, chunksize=4))
    return [_c4_one(j) for j in jobs]


def _perp_batch(d):
    # perp_v (model.cpp:93-99) of each row
    p1 = np.cross(d, [1.0, 0.0, 0.0])
    p2 = np.cross(d, [0.0, 1.0, 0.0])
    pick = (np.linalg.norm(p1, axis=1) > np.linalg.norm(p2, axis=1))[:, None]
    p = np.where(pick, p1, p2)
    return p / np.linalg.norm(p, axis=1, keepdims=True)


def _min_dist(cand, seg):
    """min over j of |cand[a, t] - seg[a, j]| for each chain a and try t
    (|c|^2 + |s|^2 - 2 c.s through batched matrix products)."""
    c2 = (cand * cand).sum(axis=2)[:, :, None]
    s2 = (seg * seg).sum(axis=2)[:, None, :]
    d2 = c2 + s2 - 2.0 * np.matmul(cand, seg.transpose(0, 2, 1))
    return np.sqrt(np.maximum(d2.min(axis=2), 0.0))


def saw_chains(rng, lens, bond, starts, window=256, min_sep=4.0 * ANGSTROM, tries=16):
    """saw_chain for many chains at once (each step advances every chain that
    is still growing); self-avoidance over the last `window` beads."""
    lens = np.asarray(lens)
    C, Lm = len(lens), int(lens.max())
    pos = np.zeros((C, Lm, 3))
    pos[:, 0] = starts
    d = rng.normal(size=(C, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ms, ma = math.pi / 12.0, math.pi
    for k in range(1, Lm):
        act = np.nonzero(lens > k)[0]
        A = len(act)
        dd = d[act][:, None, :]
        sp = rng.uniform(-ms, ms, size=(A, tries, 1))
        ar = rng.uniform(-ma, ma, size=(A, tries, 1))
        p = _perp_batch(d[act])[:, None, :]
        v1 = dd * np.cos(sp) + np.cross(p, dd) * np.sin(sp)
        dv = (v1 * dd).sum(axis=2, keepdims=True)
        v2 = v1 * np.cos(ar) + np.cross(dd, v1) * np.sin(ar) + dd * dv * (1.0 - np.cos(ar))
        v2 /= np.linalg.norm(v2, axis=2, keepdims=True)
        cand = pos[act, k - 1][:, None, :] + bond * v2
        if k >= 3:
            lo = max(0, k - 2 - window)
            dmin = _min_dist(cand, pos[act, lo:k - 2])
        else:
            dmin = np.full((A, tries), np.inf)
        ok = dmin >= min_sep
        pick = np.where(ok.any(axis=1), ok.argmax(axis=1), dmin.argmax(axis=1))
        ar_ = np.arange(A)
        pos[act, k] = cand[ar_, pick]
        d[act] = v2[ar_, pick]
    return [pos[c, :lens[c]] for c in range(C)]


def compact_walks(rng, lens, bond, density=1.0 / 120.0, min_sep=4.2 * ANGSTROM, tries=48, batch=8):
    """compact_walk for many chains at once."""
    lens = np.asarray(lens)
    C, Lm = len(lens), int(lens.max())
    radius = np.maximum((3.0 * lens / (4.0 * math.pi * density)) ** (1.0 / 3.0) * ANGSTROM, 2.0 * bond)
    pos = np.zeros((C, Lm, 3))
    for k in range(1, Lm):
        act = np.nonzero(lens > k)[0]
        A = len(act)
        best = np.zeros((A, 3))
        best_score = np.full(A, -np.inf)
        done = np.zeros(A, dtype=bool)
        for _ in range(0, tries, batch):
            todo = np.nonzero(~done)[0]
            if not len(todo):
                break
            ch = act[todo]
            dirs = rng.normal(size=(len(todo), batch, 3))
            dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
            cand = pos[ch, k - 1][:, None, :] + bond * dirs
            if k >= 2:
                dmin = _min_dist(cand, pos[ch, :k - 1])
            else:
                dmin = np.full((len(todo), batch), np.inf)
            out = np.maximum(0.0, np.linalg.norm(cand, axis=2) - radius[ch][:, None])
            score = np.minimum(dmin - min_sep, 0.0) - out
            ok = score >= 0.0
            has = ok.any(axis=1)
            j = np.where(has, ok.argmax(axis=1), score.argmax(axis=1))
            sj = score[np.arange(len(todo)), j]
            cj = cand[np.arange(len(todo)), j]
            better = has | (sj > best_score[todo])
            best[todo[better]] = cj[better]
            best_score[todo[better]] = sj[better]
            done[todo[has]] = True
        pos[act, k] = best
    return [pos[c, :lens[c]] for c in range(C)]


def make_request_system(chain_lengths, seed, temperature, rng_seed, density=1e-3, bond=3.8 * ANGSTROM):
    """A multi-chain open system built with the batched walks (config 5)."""
    rng = np.random.default_rng(seed)
    lens = [int(x) for x in chain_lengths]
    n = sum(lens)
    chain = np.concatenate([np.full(L, c, dtype=np.int32) for c, L in enumerate(lens)])
    seq = np.concatenate([np.arange(L, dtype=np.int32) for L in lens])
    atype = _types(rng, n, "charged10")
    a = (n / density) ** (1.0 / 3.0) * ANGSTROM
    starts = rng.uniform(-a / 2.0, a / 2.0, size=(len(lens), 3))
    walks = saw_chains(rng, lens, bond, starts)
    natives = compact_walks(rng, lens, bond)
    r = np.concatenate(walks)
    tet, ang, dih, nat = ([], [], []), ([], [], [], []), ([], [], [], [], []), ([], [], [])
    off = 0
    for L, npos in zip(lens, natives):
        if L >= 2:
            tet[0].append(np.arange(off, off + L - 1)); tet[1].append(np.arange(off + 1, off + L))
            tet[2].append(np.full(L - 1, bond))
        if L >= 3:
            th, ph = bonded_natives(npos)
            k = np.arange(len(th))
            ang[0].append(off + k); ang[1].append(off + k + 1); ang[2].append(off + k + 2); ang[3].append(th)
            k = np.arange(len(ph))
            dih[0].append(off + k); dih[1].append(off + k + 1); dih[2].append(off + k + 2)
            dih[3].append(off + k + 3); dih[4].append(ph)
            i1, i2, dd = native_map(npos)
            nat[0].append(i1 + off); nat[1].append(i2 + off); nat[2].append(dd)
        off += L
    cat32 = lambda xs: np.concatenate(xs).astype(np.int32) if xs else np.zeros(0, np.int32)
    catf = lambda xs: np.concatenate(xs).astype(np.float64) if xs else np.zeros(0)
    dihs = (cat32(dih[0]), cat32(dih[1]), cat32(dih[2]), cat32(dih[3]), catf(dih[4]))
    return System(
        n=n, chain=chain, seq=seq, atype=atype, cell=np.zeros(3), r=r,
        tethers=(cat32(tet[0]), cat32(tet[1]), catf(tet[2])),
        angles=(cat32(ang[0]), cat32(ang[1]), cat32(ang[2]), catf(ang[3])),
        dihedrals=dihs,
        natives=(cat32(nat[0]), cat32(nat[1]), catf(nat[2])),
        temperature=temperature, seed=int(rng_seed), meta={"chains": lens},
        chirals=chirals_of(dihs, np.concatenate(natives)),
    )


def c5_request(seed: int, max_chains=64, lo=30, hi=1500, max_beads=200_000):
    """One serving request: 1-64 chains with lengths log-uniform in [30, 1500]
    beads (total capped), open boundaries, Go + Debye-Hueckel topology, seeded
    temperature uniform in [0.3, 0.6]."""
    rng = np.random.default_rng(10_000 + seed)
    nch = int(rng.integers(1, max_chains + 1))
    lens = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), size=nch))).astype(int)
    lens = lens[np.cumsum(lens) <= max_beads]
    T = float(rng.uniform(0.3, 0.6))
    # self-avoidance over the last 256 beads of a chain; chains start at
    # random points of the density-sized cube and may meet (Pauli separates them)
    return make_request_system([int(L) for L in lens], 20_000 + seed, T, 30_000 + seed)


def _c5_one(args):
    return c5_request(*args)


def config_c5(count=24, seed=5, workers=0, max_chains=64):
    """`count` serving requests (config 5), optionally generated in a spawned
    process pool (same requests, same order)."""
    jobs = [(seed * 1000 + k, max_chains) for k in range(count)]
    if workers and workers > 1:
        import multiprocessing as mp
        from concurrent.futures import ProcessPoolExecutor
        with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            return list(ex.map(_c5_one, jobs, chunksize=1))
    return [_c5_one(j) for j in jobs]
