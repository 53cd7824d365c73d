"""Solid and LJ attractive walls (src/forces/walls/solid.cpp,
walls/lj_attr.cpp): the restatement against the closed form and the
reference's own kernels, the GPU path against the restatement."""
import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Oracle
from tests.util import ANGSTROM, energy_rel, only_term, rel_err
from xmd_gb300 import abi, synth

have_ref = REF_LIB.exists()
EPS, CUT = 1.0, 5.0 * ANGSTROM


def system(seed=6):
    return synth.make_system([60, 40], seed, box=None, types="charged10", start="native", temperature=0.4)


def walls_for(s, gap=2.0):
    """A floor gap A below the lowest bead (normal +z) and a side wall gap A
    beyond the largest x (normal -x)."""
    zmin, xmax = s.r[:, 2].min(), s.r[:, 0].max()
    o = np.array([[0.0, 0.0, zmin - gap * ANGSTROM], [xmax + gap * ANGSTROM, 0.0, 0.0]])
    n = np.array([[0.0, 0.0, 1.0], [-1.0, 0.0, 0.0]])
    return o, n


def yaml(prec="fp64", solid=True, lj=True):
    return (synth.yaml_for("c2", prec) + f"\nsolid walls:\n  enabled: {'true' if solid else 'false'}\n"
            f"\nLJ attractive walls:\n  enabled: {'true' if lj else 'false'}\n")


def solid_energy(r, o, n):
    V = 0.0
    for ow, nw in zip(o, n):
        x = (r - ow) @ nw
        m = x < CUT
        V += (EPS / (9.0 * x[m] ** 9)).sum()
    return V


def num_grad(fn, r, h=1e-6):
    g = np.zeros_like(r)
    for i in range(len(r)):
        for a in range(3):
            rp, rm = r.copy(), r.copy()
            rp[i, a] += h
            rm[i, a] -= h
            g[i, a] = (fn(rp) - fn(rm)) / (2 * h)
    return g


def test_port_solid_wall_is_the_energy_gradient():
    s = system()
    o, n = walls_for(s)
    p = abi.parse_params(only_term(abi.TERM_SOLID_WALL, yaml()))
    F, V = Oracle(p, s, "port", walls={0: (o, n)}).eval_forces()
    Vw = solid_energy(s.r, o, n)
    assert Vw > 0 and abs(V[abi.TERM_SOLID_WALL] - Vw) <= 1e-12 * Vw
    assert rel_err(F, -num_grad(lambda r: solid_energy(r, o, n), s.r)) <= 1e-6


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
def test_shipped_solid_wall_force():
    """The reference's force is dV_dx n with dV_dx = V (-9 x)
    (walls/solid.cpp:18-22), not -dV/dx n."""
    s = system()
    o, n = walls_for(s)
    p = abi.parse_params(only_term(abi.TERM_SOLID_WALL, yaml()))
    F, V = Oracle(p, s, "ref", walls={0: (o, n)}).eval_forces()
    want = np.zeros_like(s.r)
    for ow, nw in zip(o, n):
        x = (s.r - ow) @ nw
        m = x < CUT
        Vb = EPS / (9.0 * x[m] ** 9)
        want[m] += (Vb * (-9.0 * x[m]))[:, None] * nw
    assert np.abs(F - want).max() <= 1e-9 * np.abs(want).max()
    assert abs(V[abi.TERM_SOLID_WALL] - solid_energy(s.r, o, n)) <= 1e-12 * V[abi.TERM_SOLID_WALL]


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
def test_lj_walls_bit_exact_vs_reference_live():
    """The LJ attractive walls' pair states form, saturate and break as the
    reference's loop has them (forces and 400 steps bit for bit)."""
    s = system()
    o, n = walls_for(s, gap=1.0)
    y = yaml(solid=False)
    p = abi.parse_params(y)
    a = Oracle(p, s, "port", walls={1: (o, n)})
    b = Oracle(p, s, "ref", walls={1: (o, n)})
    for _ in range(4):
        a.step(100)
        b.step(100)
        ya, ta, sa = a.get_history()
        yb, tb, sb = b.get_history()
        assert np.array_equal(ya, yb) and ta == tb and sa == sb
    Fa, Va = a.eval_forces()
    Fb, Vb = b.eval_forces()
    assert Va[abi.TERM_LJ_WALL] != 0
    assert np.array_equal(Fa, Fb) and np.array_equal(Va, Vb)


@pytest.mark.gpu
def test_gpu_solid_wall_forces():
    from xmd_gb300 import Engine
    s = system()
    o, n = walls_for(s)
    yy = only_term(abi.TERM_SOLID_WALL, yaml())
    Fo, Vo = Oracle(abi.parse_params(yy), s, "port", walls={0: (o, n)}).eval_forces()
    with Engine(yy) as e:
        e.set_walls(0, o, n)
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-10
    assert energy_rel(V, Vo).max() <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_walls_trajectory(prec):
    """A solid floor and an LJ attractive side wall.  The pair states are
    discrete: a bead that crosses the formation distance one step apart on
    two FP64 paths (positions 1e-12 A apart) moves off, so the FP64 check
    stays within 120 steps (phase duration 2000 steps: no pair breaks); the
    mixed path is checked by its forces and a bounded run."""
    from xmd_gb300 import Engine
    s = system()
    o, n = walls_for(s, gap=2.0)
    wl = {0: (o[:1], n[:1]), 1: (o[1:] - np.array([1.0 * ANGSTROM, 0, 0]), n[1:])}
    y = yaml()
    orc = Oracle(abi.parse_params(y), s, "port", walls=wl)
    F0o, _ = orc.eval_forces()
    with Engine(yaml(prec)) as e:
        e.set_walls(0, *wl[0])
        e.set_walls(1, *wl[1])
        e.add_system(s)
        F0, V0 = e.eval_forces(0)
        assert rel_err(F0, F0o) <= (1e-10 if prec == "fp64" else 1e-5) and V0[abi.TERM_SOLID_WALL] > 0
        steps = 120 if prec == "fp64" else 600
        e.step(steps)
        r, _, _ = e.get_state(0)
        Fg, Vg = e.eval_forces(0)
    orc.step(steps)
    ro, _, _ = orc.get_state()
    Fo, Vo = orc.eval_forces()
    assert Vo[abi.TERM_LJ_WALL] != 0     # (the floor's repulsion acts at t = 0, checked above)
    if prec == "fp64":
        assert np.abs(r - ro).max() / ANGSTROM <= 1e-8
        assert rel_err(Fg, Fo) <= 1e-9
    else:
        assert np.isfinite(r).all() and np.abs(r - ro).max() / ANGSTROM < 5.0
        assert Vg[abi.TERM_LJ_WALL] != 0


@pytest.mark.gpu
def test_gpu_wall_state_in_snapshot():
    from xmd_gb300 import Engine
    s = system()
    o, n = walls_for(s, gap=1.0)

    def build():
        e = Engine(yaml(solid=False))
        e.set_walls(1, o, n)
        e.add_system(s)
        return e

    with build() as a, build() as b:
        a.step(150)
        snap = a.snapshot(0)
        a.step(150)
        b.restore(0, snap)
        b.step(150)
        assert np.array_equal(a.get_history(0)[0], b.get_history(0)[0])
