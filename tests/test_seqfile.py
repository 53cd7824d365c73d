"""Sequence files and contact maps (xmd_gb300.seqfile) and the heuristic
angle and dihedral terms they bring in: the reader against the format's rules,
morph_into_saw and the heuristic terms against the reference's own compiled
code, closed forms and numerical gradients; the GPU path against the
restatement."""
from pathlib import Path

import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Oracle, ref_morph_into_saw
from tests.util import ANGSTROM, energy_rel, only_term, rel_err
from xmd_gb300 import abi, seqfile, synth

have_ref = REF_LIB.exists()
# the reference checkout the reference oracle was built from (recorded by
# oracle/ref/build_ref.sh); its example inputs are read where they lie
_REF_ROOT = REF_LIB.parent / "ref_root.txt"
EXAMPLES = Path(_REF_ROOT.read_text().strip() if _REF_ROOT.exists() else "/nonexistent") / "xmd/data/examples"


def test_yaml_subset():
    text = """
# comment
parts:
  a: &A
    seq: "\\
      MKV\\
      GP"   # trailing comment
    maps:
      m1:
        map:
          contacts: |-
            i1,i2,length
            0,3,1.5
        shift: 2
  b: &B { seq: 'GG' }
model:
  chains: [ *A, *B,
            *A ]
  text: "one
    two"
  list:
    - x: 1
      y: 2
    - plain
"""
    y = seqfile.load_yaml(text)
    ch = y["model"]["chains"]
    assert [c["seq"] for c in ch] == ["MKVGP", "GG", "MKVGP"]
    assert ch[0]["maps"]["m1"]["shift"] == "2"
    assert ch[0]["maps"]["m1"]["map"]["contacts"] == "i1,i2,length\n0,3,1.5"
    assert y["model"]["text"] == "one two"
    assert y["model"]["list"] == [{"x": "1", "y": "2"}, "plain"]


def synthetic_seqfile(tmp: Path, seed=5):
    """Two chains (one used twice) with native maps from compact structures:
    contacts under 7.5 A with |i-j| >= 3, every other native angle and
    dihedral; one map from a file with a shift, one inline."""
    rng = np.random.default_rng(seed)
    lens = [48, 31]
    codes = []
    for L in lens:
        c = list(rng.choice(list(seqfile.LETTERS), size=L))
        c[3], c[4], c[9], c[10] = "G", "P", "P", "G"
        codes.append("".join(c))
    maps = []
    for L in lens:
        npos = synth.compact_walk(rng, L, 3.8 * ANGSTROM)
        i1, i2, d = synth.native_map(npos)
        th, ph = synth.bonded_natives(npos)
        m = seqfile.ContactMap(
            contacts=[(int(a), int(b), float(x)) for a, b, x in zip(i1, i2, d)],
            angles=[(k, k + 1, k + 2, float(th[k])) for k in range(0, L - 2, 2)],
            dihedrals=[(k, k + 1, k + 2, k + 3, float(ph[k])) for k in range(1, L - 3, 2)])
        maps.append(m)
    # chain 0's map is stored shifted down by 2 and shifted back by the file
    m0 = maps[0].shift(-2)
    (tmp / "a.map.yml").write_text(seqfile.write_map(m0))
    inline = "\n".join("          " + ln for ln in seqfile.write_map(maps[1]).splitlines())
    text = f"""parts:
  a: &a
    seq: "{codes[0][:20]}\\
      {codes[0][20:]}"
    maps:
      am:
        from-file: a.map.yml
        shift: 2
  b: &b
    seq: "{codes[1]}"
    maps:
      bm:
        map:
{inline}
model:
  chains: [ *a, *b, *a ]
"""
    (tmp / "model.yml").write_text(text)
    return tmp / "model.yml", codes, maps


def test_reader_builds_the_model(tmp_path):
    path, codes, maps = synthetic_seqfile(tmp_path)
    m = seqfile.read_seq(path)
    assert [c.codes for c in m.chains] == [codes[0], codes[1], codes[0]]
    got = m.chains[0].maps[0]
    assert got.contacts == maps[0].contacts and got.angles == maps[0].angles
    assert got.dihedrals == maps[0].dihedrals
    s = seqfile.to_system(m, seed=9)
    lens = [48, 31, 48]
    assert s.n == sum(lens) and list(s.meta["chains"]) == lens
    assert np.array_equal(s.chain, np.repeat([0, 1, 2], lens))
    assert np.array_equal(s.seq, np.concatenate([np.arange(L) for L in lens]))
    assert [seqfile.LETTERS[seqfile.LETTERS.index(c)] for c in codes[0]] == list(codes[0])
    # tethers on every bond, default length
    assert len(s.tethers[0]) == sum(L - 1 for L in lens) and np.all(s.tethers[2] == 0)
    # native angles where the map gives them, heuristic on the other triples
    nat_a = set(zip(*[x.tolist() for x in s.angles[:3]]))
    heur_a = set(zip(*[x.tolist() for x in s.heur_angles]))
    assert not nat_a & heur_a
    assert len(nat_a) + len(heur_a) == sum(L - 2 for L in lens)
    nat_d = set(zip(*[x.tolist() for x in s.dihedrals[:4]]))
    heur_d = set(zip(*[x.tolist() for x in s.heur_dihedrals]))
    assert not nat_d & heur_d and len(nat_d) + len(heur_d) == sum(L - 3 for L in lens)
    # contacts of chain 2 (the third) are chain 0's map moved by 79
    off = 48 + 31
    c2 = {(a - off, b - off) for a, b in zip(*[x.tolist() for x in s.natives[:2]]) if a >= off}
    assert c2 == {(a, b) for a, b, _ in maps[0].contacts}
    # bond lengths of the morphed start
    assert np.abs(np.linalg.norm(s.r[1:48] - s.r[:47], axis=1) - 3.8 * ANGSTROM).max() < 1e-12


def test_unknown_residue_and_bad_map_rejected(tmp_path):
    with pytest.raises(ValueError):
        seqfile.read_seq('model:\n  chains: [ { seq: "MKXB" } ]\n')
    bad = 'model:\n  chains:\n    - seq: "MKVL"\n      maps:\n        m:\n          map:\n' \
          '            contacts: |-\n              i1,i2,length\n              0,9,1.0\n'
    with pytest.raises(ValueError):
        seqfile.to_system(seqfile.read_seq(bad))


def test_generator_matches_the_oracle_stream():
    from oracle.pyoracle import rng_stream
    raw, st = rng_stream("port", 42, 64)
    g = seqfile.RandGen(42)
    assert [g.next() for _ in range(64)] == [int(x) for x in raw] and g.state == st


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
@pytest.mark.parametrize("seed", [42, 2024])
def test_morph_matches_the_reference(seed):
    lens = [140, 31, 7, 1]
    for bond in (3.8 * ANGSTROM, None):
        rr, st, _ = ref_morph_into_saw(lens, bond, 1e-3 / ANGSTROM**3, 0, seed)
        g = seqfile.RandGen(seed)
        r, _ = seqfile.morph_into_saw(lens, g, bond, 1e-3 / ANGSTROM**3)
        assert g.state == st
        assert np.abs(r - rr).max() <= 1e-12 * max(1.0, np.abs(rr).max())


@pytest.mark.skipif(not EXAMPLES.exists(), reason="reference examples not present")
def test_reference_examples_load():
    m = seqfile.read_seq(EXAMPLES / "glut" / "glut.yml")
    assert len(m.chains) == 14
    s = seqfile.to_system(m)
    off = 0
    for L in s.meta["chains"]:
        sel = (s.natives[0] >= off) & (s.natives[0] < off + L)
        assert np.all(s.natives[1][sel] < off + L)
        off += L
    assert len(s.natives[0]) > 0 and len(s.heur_angles[0]) > 0
    m = seqfile.read_seq(EXAMPLES / "9aac" / "9aac.yml")
    assert len(m.chains) == 1 and len(m.chains[0].codes) == 140


# ---- heuristic terms ----------------------------------------------------------------------

def seq_system(tmp, seed=5, noise=0.0, compact=False):
    """compact: chains folded as compact walks (bond angles away from the
    straight line, where the angle's derivatives grow without bound) instead
    of the morphed start."""
    path, _, _ = synthetic_seqfile(tmp, seed)
    s = seqfile.to_system(seqfile.read_seq(path), seed=seed + 1, temperature=0.35)
    rng = np.random.default_rng(seed)
    if compact:
        off = 0
        for c, L in enumerate(s.meta["chains"]):
            s.r[off:off + L] = synth.compact_walk(rng, L, 3.8 * ANGSTROM) + np.array([40.0 * c, 0, 0]) * ANGSTROM
            off += L
    if noise:
        s.r = s.r + rng.normal(0, noise * ANGSTROM, size=s.r.shape)
    return s


def yaml(prec="fp64"):
    return synth.yaml_for("c1", prec)


def heur_angle_energy(p, s, r):
    i1, i2, i3 = s.heur_angles
    r12, r23 = r[i2] - r[i1], r[i3] - r[i2]
    ct = -(r12 * r23).sum(1) / np.linalg.norm(r12, axis=1) / np.linalg.norm(r23, axis=1)
    th = np.arccos(np.clip(ct, -1, 1))
    cls = lambda a: np.where(a == abi.AA.index("GLY"), 0, np.where(a == abi.AA.index("PRO"), 1, 2))
    ty = 3 * cls(s.atype[i1]) + cls(s.atype[i2])
    A = np.array(p.heur_ang_coeffs)[ty]
    return sum((A[:, d] * th**d).sum() for d in range(7))


def heur_dih_energy(p, s, r, phi_of=np.arccos):
    i1, i2, i3, i4 = s.heur_dihedrals
    r12, r23, r34 = r[i2] - r[i1], r[i3] - r[i2], r[i4] - r[i3]
    x1, x2 = np.cross(r12, r23), np.cross(r23, r34)
    cp = (x1 * x2).sum(1) / np.linalg.norm(x1, axis=1) / np.linalg.norm(x2, axis=1)
    ph = phi_of(np.clip(cp, -1, 1))
    ph = np.where((x1 * r34).sum(1) < 0, -ph, ph)
    sp = np.sin(ph)
    cls = lambda a: np.where(a == abi.AA.index("GLY"), 0, np.where(a == abi.AA.index("PRO"), 1, 2))
    c = np.array(p.heur_dih_coeffs)[3 * cls(s.atype[i2]) + cls(s.atype[i3])]
    return (c[:, 0] + c[:, 1] * sp + c[:, 2] * cp + c[:, 3] * sp**2 + c[:, 4] * cp**2 + c[:, 5] * sp * cp).sum()


def num_grad(fn, r, h=1e-6):
    g = np.zeros_like(r)
    for i in range(len(r)):
        for x in range(3):
            rp, rm = r.copy(), r.copy()
            rp[i, x] += h
            rm[i, x] -= h
            g[i, x] = (fn(rp) - fn(rm)) / (2 * h)
    return g


@pytest.mark.parametrize("term", [abi.TERM_HEUR_ANG, abi.TERM_HEUR_DIH])
def test_port_heuristic_terms_match_closed_form(tmp_path, term):
    s = seq_system(tmp_path, compact=True)
    p = abi.parse_params(only_term(term, yaml()))
    F, V = Oracle(p, s, "port").eval_forces()
    fn = (lambda r: heur_angle_energy(p, s, r)) if term == abi.TERM_HEUR_ANG else (lambda r: heur_dih_energy(p, s, r))
    Vw = fn(s.r)
    assert abs(V[term] - Vw) <= 1e-9 * max(1.0, abs(Vw))
    # the angle polynomial's terms reach ~1e6 eps and cancel: each energy
    # evaluation carries ~1e-9 eps of rounding, so the central difference is
    # good to ~1e-6 relative only
    assert rel_err(F, -num_grad(fn, s.r, h=1e-5)) <= 1e-5


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
def test_shipped_heuristic_dihedral_takes_cos_of_cos(tmp_path):
    """The reference kernel's energy is the closed form at phi = cos(cos_phi)
    (dihedral/heurestic.cpp:43); the restatement uses acos."""
    s = seq_system(tmp_path)
    p = abi.parse_params(only_term(abi.TERM_HEUR_DIH, yaml()))
    _, V = Oracle(p, s, "ref").eval_forces()
    want = heur_dih_energy(p, s, s.r, phi_of=np.cos)
    assert abs(V[abi.TERM_HEUR_DIH] - want) <= 1e-9 * abs(want)
    assert abs(want - heur_dih_energy(p, s, s.r)) > 1e-3 * abs(want)


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
def test_port_bit_exact_vs_reference_on_a_seqfile_model(tmp_path):
    """Every term but the heuristic dihedral (which departs, above) against
    the reference's kernels: forces and 300 steps bit for bit."""
    s = seq_system(tmp_path)
    y = yaml() + "\nheurestic dihedrals:\n  enabled: false\n"
    p = abi.parse_params(y)
    a, b = Oracle(p, s, "port"), Oracle(p, s, "ref")
    Fa, Va = a.eval_forces()
    Fb, Vb = b.eval_forces()
    assert Va[abi.TERM_HEUR_ANG] != 0
    assert np.array_equal(Fa, Fb) and np.array_equal(Va, Vb)
    a.step(300)
    b.step(300)
    ya, ta, sa = a.get_history()
    yb, tb, sb = b.get_history()
    assert np.array_equal(ya, yb) and ta == tb and sa == sb


@pytest.mark.gpu
@pytest.mark.parametrize("term", [abi.TERM_HEUR_ANG, abi.TERM_HEUR_DIH])
def test_gpu_heuristic_term_forces(tmp_path, term):
    from xmd_gb300 import Engine
    s = seq_system(tmp_path, noise=0.2, compact=True)
    yy = only_term(term, yaml())
    Fo, Vo = Oracle(abi.parse_params(yy), s, "port").eval_forces()
    with Engine(yy) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-10
    assert energy_rel(V, Vo).max() <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("compact,steps", [(False, 60), (True, 200)])
def test_gpu_seqfile_trajectory(tmp_path, compact, steps):
    """Inside each start's parity horizon: from the morphed start (nearly
    straight triples, where the angle terms' derivatives diverge) the oracle
    reproduces itself under a reordered force sum to 1e-11 A for 50 steps
    and only to 2e-6 A at 200; from a compact start to 3e-11 A at 200."""
    from xmd_gb300 import Engine
    s = seq_system(tmp_path, compact=compact)
    y = yaml()
    o = Oracle(abi.parse_params(y), s, "port")
    Fo, _ = o.eval_forces()
    with Engine(y) as e:
        e.add_system(s)
        F, _ = e.eval_forces(0)
        assert rel_err(F, Fo) <= 1e-10
        e.step(steps)
        r, _, _ = e.get_state(0)
    o.step(steps)
    ro, _, _ = o.get_state()
    assert np.abs(r - ro).max() / ANGSTROM <= 1e-8


@pytest.mark.gpu
def test_gpu_mixed_heuristic_within_bound(tmp_path):
    from xmd_gb300 import Engine
    s = seq_system(tmp_path, noise=0.2, compact=True)
    Fo, Vo = Oracle(abi.parse_params(yaml()), s, "port").eval_forces()
    with Engine(yaml("mixed")) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-5
    for t in (abi.TERM_HEUR_ANG, abi.TERM_HEUR_DIH):
        assert abs(V[t] - Vo[t]) <= 1e-5 * max(1.0, abs(Vo[t]))
