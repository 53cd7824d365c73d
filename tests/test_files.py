"""PDB structures in and out (xmd_gb300.files), following the reference's PDB
path (files/pdb.cpp, records.cpp, fields.cpp) with its two documented
deviations (file order of residues; the force term's angle convention)."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tests.util import ANGSTROM, rel_err
from xmd_gb300 import abi, files, synth


def structure(seed=3):
    return synth.make_system([40, 25], seed, box=100 * ANGSTROM, types="uniform20", start="native")


def test_round_trip_keeps_structure_and_topology():
    s = structure()
    t = files.to_system(files.read_pdb(files.write_pdb(s)))
    assert t.n == s.n
    assert np.array_equal(t.chain, s.chain) and np.array_equal(t.seq, s.seq) and np.array_equal(t.atype, s.atype)
    assert np.abs(t.r - s.r).max() <= 0.5e-3 * ANGSTROM * (1 + 1e-9)        # 3 decimals in A
    assert np.allclose(t.cell, s.cell)
    assert [tuple(x) for x in zip(*t.natives[:2])] == [tuple(x) for x in zip(*s.natives[:2])]
    assert np.abs(t.natives[2] - s.natives[2]).max() <= 2e-3 * ANGSTROM
    assert np.abs(t.tethers[2] - np.linalg.norm(s.r[1:] - s.r[:-1], axis=1)[t.tethers[0]]).max() <= 2e-3 * ANGSTROM
    assert np.abs(t.angles[3] - s.angles[3]).max() < 1e-2
    d = (t.dihedrals[4] - s.dihedrals[4] + np.pi) % (2 * np.pi) - np.pi
    assert np.abs(d).max() < 1e-2


ATOM = "ATOM  {ser:5d}  {nm:<3s} {res:3s} {ch}{seq:4d}    {x:8.3f}{y:8.3f}{z:8.3f}"


def atom(ser, nm, res, ch, seq, x, y=0.0, z=0.0):
    return ATOM.format(ser=ser, nm=nm, res=res, ch=ch, seq=seq, x=x, y=y, z=z).ljust(80)


def test_reader_follows_the_record_rules():
    lines = [
        "CRYST1   50.000   60.000   70.000".ljust(80),
        atom(1, "CA", "GLY", "B", 5, 1.0),
        atom(2, "N", "GLY", "B", 5, 9.0),
        atom(3, "CA", "ALA", "A", 1, 2.0),
        atom(4, "CA", "ALA", "A", 1, 7.0),     # a second CA of the same residue: the first is used
        atom(5, "CA", "LYS", "B", 6, 3.0),
        "TER       6      LYS B   6".ljust(80),
        atom(7, "CA", "SER", "B", 9, 4.0),     # after chain B's TER: not part of the chain
        atom(8, "CA", "CYS", "A", 2, 5.0),
        "END".ljust(80),
        atom(9, "CA", "CYS", "A", 3, 6.0),     # after END: ignored
    ]
    p = files.read_pdb("\n".join(lines))
    assert list(p.chains) == ["B", "A"]                       # order of first appearance
    assert [r.seq_num for r in p.chains["B"]] == [5, 6]
    assert [r.seq_num for r in p.chains["A"]] == [1, 2]
    assert p.chains["A"][0].find("CA")[0] == pytest.approx(2.0 * ANGSTROM)
    assert np.allclose(p.cell, np.array([50, 60, 70]) * ANGSTROM)
    s = files.to_system(p)
    assert s.n == 4 and list(s.chain) == [0, 0, 1, 1] and list(s.seq) == [0, 1, 0, 1]
    assert [abi.AA[t] for t in s.atype] == ["GLY", "LYS", "ALA", "CYS"]


def test_later_model_overwrites_and_ssbond_is_kept_apart():
    s = structure(5)
    frames = [s.r, s.r + 1.0 * ANGSTROM]
    s.meta["ssbonds"] = [(2, 10, float(np.linalg.norm(s.r[2] - s.r[10])))]
    t = files.to_system(files.read_pdb(files.write_pdb(s, frames=frames)))
    # records keyed by atom serial: the second model's coordinates win
    assert np.abs(t.r - (s.r + 1.0 * ANGSTROM)).max() <= 0.5e-3 * ANGSTROM * (1 + 1e-9)
    assert [(a, b) for a, b, _ in t.meta["ssbonds"]] == [(2, 10)]
    assert (2, 10) not in set(zip(t.natives[0].tolist(), t.natives[1].tolist()))


def test_derived_contacts_are_ca_overlaps():
    s = structure(7)
    p = files.read_pdb(files.write_pdb(s))
    got = {(c1, s1, c2, s2) for c1, s1, c2, s2, _ in files.derive_contacts(p)}
    res = [r for ch in p.chains.values() for r in ch]
    want = set()
    for a in range(len(res)):
        for b in range(a + 1, len(res)):
            ra, rb = res[a], res[b]
            if abs(ra.seq_num - rb.seq_num) < 3:
                continue
            d = np.linalg.norm(ra.find("CA") - rb.find("CA"))
            if d < (files.RADIUS_A[ra.name] + files.RADIUS_A[rb.name]) * ANGSTROM:
                want.add((ra.chain, ra.seq_num, rb.chain, rb.seq_num))
    assert got == want and len(got) > 0


def test_structure_sits_at_its_bonded_minima():
    """With the force term's angle convention a structure is at the minimum
    of its own native angles and dihedrals (the shipped to_model's
    acos(u12 . u23) would put every angle off by pi - 2 theta)."""
    t = files.to_system(files.read_pdb(files.write_pdb(structure(9))))
    o = Oracle(abi.parse_params(synth.yaml_for("c1")), t, "port")
    _, V = o.eval_forces()
    assert abs(V[abi.TERM_NAT_ANG]) < 1e-20 and abs(V[abi.TERM_CND]) < 1e-20


@pytest.mark.gpu
def test_pdb_system_runs_at_parity():
    from xmd_gb300 import Engine
    t = files.to_system(files.read_pdb(files.write_pdb(structure(11))), temperature=0.35, seed=5,
                        contacts="both")
    y = synth.yaml_for("c2")
    o = Oracle(abi.parse_params(y), t, "port")
    Fo, Vo = o.eval_forces()
    with Engine(y) as e:
        e.add_system(t)
        F, V = e.eval_forces(0)
        assert rel_err(F, Fo) <= 1e-10
        e.step(200)
        r, _, _ = e.get_state(0)
    o.step(200)
    ro, _, _ = o.get_state()
    assert np.abs(r - ro).max() / ANGSTROM <= 1e-8
