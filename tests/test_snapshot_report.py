"""Snapshots (exact resume) and run reports (report_stats CSV,
report_structure YAML)."""
import math

import numpy as np
import pytest

from tests.util import ANGSTROM, load_golden
from xmd_gb300 import abi, report, seqfile, synth


def test_to_string_and_asphericity():
    assert report.to_string(3) == "3" and report.to_string(0.5) == "0.500000" and report.to_string(True) == "1"
    # a rod along x of half-length a: singular values (a sqrt(2n/3)-ish, 0, 0)
    x = np.linspace(-1, 1, 11)
    r = np.stack([x, 0 * x, 0 * x], axis=1)
    lam = np.linalg.norm(x)
    assert report.asphericity(r) == pytest.approx(-0.5 * lam**2)
    # a regular tetrahedron is isotropic: l1 = l2 = l3, W = 0
    t = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=float)
    assert abs(report.asphericity(t)) < 1e-12


class FakeEngine:
    """The Engine calls the reporters make, over a fixed state."""

    def __init__(self, s, t, qa=False):
        self.s, self.t, self.qa = s, t, qa

    def get_state(self, rep=0):
        return self.s.r, np.zeros_like(self.s.r), self.t

    def observables(self, rep=0):
        return {"E": -3.25, "K": 1.5, "Rg": 2.0, "Q": 0.5}

    def params(self):
        p = abi.parse_params("")
        p.on[abi.TERM_QA] = int(self.qa)
        return p

    def qa_sync(self, rep=0):
        return np.tile(np.array([2, 1, 0, 1], np.int8), (self.s.n, 1))

    def qa_contacts(self, rep=0):
        return np.array([[1, 7, 1, 0], [2, 9, 30, 1]], np.int32), np.array([0.5, 1.25])


def test_stats_report(tmp_path):
    s = synth.make_system([30], 3, box=None, types="uniform20", start="native")
    rep = report.StatsReport(tmp_path / "stats.csv", period=10.0)
    e = FakeEngine(s, 0.0)
    assert rep(e)
    e.t = 5.0
    assert not rep(e)            # within the period
    e.t = 10.0
    assert rep(e)
    lines = (tmp_path / "stats.csv").read_text().splitlines()
    assert lines[0] == "t[tau],V[eps],K[eps],E[eps],Rg[A],W[A]"
    f = lines[2].split(",")
    assert f[:5] == ["10.000000", "-4.750000", "1.500000", "-3.250000", "10.000000"]
    assert float(f[5]) == pytest.approx(report.asphericity(s.r) / ANGSTROM, abs=1e-6)


@pytest.mark.parametrize("qa", [False, True])
def test_structure_report(tmp_path, qa):
    s = synth.make_system([20, 12], 4, box=None, types="uniform20", start="native")
    s.ssbonds = (np.array([2], np.int32), np.array([15], np.int32))
    rep = report.StructureReport(str(tmp_path / "st" / "%.0f.yml"), period=1.0, system=s)
    path = rep(FakeEngine(s, 3.0, qa))
    doc = seqfile.load_yaml(path.read_text())
    res = doc["residues"].splitlines()
    assert res[0].startswith("idx,x[A],y[A],z[A]") and len(res) == s.n + 1
    assert ("back,side-all" in res[0]) == qa
    x0 = [float(v) for v in res[1].split(",")[1:4]]
    assert np.allclose(x0, s.r[0] / ANGSTROM, atol=1e-6)
    nat = doc["native contacts"].splitlines()
    assert len(nat) == len(s.natives[0]) + 2 and nat[-1].split(",")[3] == "NAT_SS"
    assert ("QA contacts" in doc) == qa
    if qa:
        q = doc["QA contacts"].splitlines()
        assert q[1] == "0,1,7,BACK_BACK,0.500000,FORMING_OR_FORMED" and q[2].endswith("SIDE_SIDE,1.250000,BREAKING")
    ang = doc["angles"].splitlines()[1:]
    assert len(ang) == len(s.angles[0])
    f = ang[0].split(",")
    assert float(f[4]) == pytest.approx(float(f[5]), abs=1e-6)     # the native structure sits at its angles
    dih = doc["dihedrals"].splitlines()[1:]
    assert len(dih) == len(s.dihedrals[0])
    assert not math.isnan(float(dih[0].split(",")[6]))


# ---- snapshots on the GPU -----------------------------------------------------------

def build(y, systems):
    from xmd_gb300 import Engine
    e = Engine(y)
    for s in systems:
        e.add_system(s)
    return e


@pytest.mark.gpu
@pytest.mark.parametrize("case,prec", [("c2_periodic480", "fp64"), ("c3_qa600", "fp64"), ("c3_qa600", "mixed")])
def test_snapshot_resumes_bit_for_bit(case, prec):
    s, y, _ = load_golden(case)
    if prec == "mixed":
        assert "precision: fp64" in y
        y = y.replace("precision: fp64", "precision: mixed")
    other = synth.make_system([40, 25], 8, box=None, types="charged10", temperature=0.4, rng_seed=3)
    systems = [other, s]
    with build(y, systems) as a:
        a.step(300)
        want = [a.get_history(r) for r in range(2)]
    with build(y, systems) as b, build(y, systems) as c:
        b.step(120)
        snaps = [b.snapshot(r) for r in range(2)]
        b.step(180)                                   # the snapshot leaves the run as it was
        for r in range(2):
            c.restore(r, snaps[r])
        c.step(180)
        for r in range(2):
            for got in (b.get_history(r), c.get_history(r)):
                assert np.array_equal(got[0], want[r][0]) and got[1] == want[r][1] and got[2] == want[r][2]
        if "qa" in case:
            assert np.array_equal(c.qa_contacts(1)[0], b.qa_contacts(1)[0])
            assert np.array_equal(c.qa_sync(1), b.qa_sync(1))


@pytest.mark.gpu
def test_snapshot_of_another_layout_rejected():
    s, y, _ = load_golden("c2_periodic480")
    other = synth.make_system([40, 25], 8, box=None, types="charged10", temperature=0.4, rng_seed=3)
    with build(y, [other, s]) as a, build(y, [s, other]) as b:
        a.step(10)
        snap = a.snapshot(1)
        with pytest.raises(abi.XmdError):
            b.restore(1, snap)
        with pytest.raises(abi.XmdError):
            a.restore(1, snap[:100])
        a.restore(1, snap)


@pytest.mark.gpu
@pytest.mark.parametrize("cut", [1, 4096])
def test_truncated_snapshot_leaves_replica_unchanged(cut):
    """A snapshot cut short anywhere past its header is rejected before any
    of the replica's state is written: the replica continues exactly as if no
    restore had been tried."""
    s, y, _ = load_golden("c3_qa600")
    other = synth.make_system([40, 25], 8, box=None, types="charged10", temperature=0.4, rng_seed=3)
    with build(y, [other, s]) as a, build(y, [other, s]) as b:
        a.step(60)
        b.step(60)
        snap = a.snapshot(1)
        a.step(30)
        b.step(30)
        before = b.get_history(1)
        with pytest.raises(abi.XmdError):
            b.restore(1, snap[:len(snap) - cut])
        after = b.get_history(1)
        assert np.array_equal(after[0], before[0]) and after[1:] == before[1:]
        a.step(40)
        b.step(40)
        ga, gb = a.get_history(1), b.get_history(1)
        assert np.array_equal(ga[0], gb[0]) and ga[1:] == gb[1:]
        assert np.array_equal(a.qa_contacts(1)[0], b.qa_contacts(1)[0])


@pytest.mark.gpu
def test_snapshot_with_other_wall_planes_rejected():
    """The saved LJ attractive wall states belong to the wall planes they
    were taken with: a context with other planes refuses the snapshot."""
    from xmd_gb300 import Engine
    s = synth.make_system([30], 4, box=None, types="charged10", temperature=0.4)
    y = synth.yaml_for("c1") + "LJ attractive walls:\n  enabled: true\n"
    planes = [(np.array([0.0, 0.0, -5.0]), np.array([0.0, 0.0, 1.0])),
              (np.array([0.0, 0.0, -6.0]), np.array([0.0, 0.0, 1.0]))]
    snaps = []
    for o, nrm in planes:
        with Engine(y) as e:
            e.set_walls(1, o[None, :], nrm[None, :])
            e.add_system(s)
            e.step(5)
            snaps.append(e.snapshot(0))
    with Engine(y) as e:
        e.set_walls(1, planes[0][0][None, :], planes[0][1][None, :])
        e.add_system(s)
        e.restore(0, snaps[0])
        with pytest.raises(abi.XmdError):
            e.restore(0, snaps[1])
