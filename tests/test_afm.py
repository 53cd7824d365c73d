"""AFM pulling (velocity and force tips, src/forces/velocity_afm.cpp and
force_afm.cpp): the restatement against the closed form and the reference's
own kernels, the GPU path against the restatement."""
import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Oracle
from tests.util import ANGSTROM, only_term, rel_err
from xmd_gb300 import abi, synth

have_ref = REF_LIB.exists()
H1 = 0.06 / ANGSTROM**2          # velocity AFM: H1 = 0.06 eps/A^2


def system(seed=3):
    s = synth.make_system([50, 30], seed, box=None, types="charged10", start="native", temperature=0.35)
    vel = np.array([[0.02, 0.0, 0.01], [-0.01, 0.03, 0.0]])
    orig = np.array([[np.nan] * 3, s.r[60] + np.array([3.0, -1.0, 0.5]) * ANGSTROM])
    s.afm_vel = (np.array([0, 60], np.int32), orig, vel)
    s.afm_force = (np.array([49, 49, 10], np.int32), np.array([[0.5, 0, 0], [0, -0.25, 0], [0.1, 0.2, 0.3]]))
    return s


def yaml(prec="fp64"):
    return synth.yaml_for("c2", prec) + "\nvelocity AFM:\n  enabled: true\n\nforce AFM:\n  enabled: true\n"


def afm_force(s, r, t):
    """Closed form: harmonic(H1, 0, 0) toward orig + t vel, clamped to 1000
    (harmonic.h:18-25), plus the summed pulling forces; no energy."""
    F = np.zeros_like(r)
    b, o, v = s.afm_vel
    o = np.where(np.isnan(o), s.r[b], o)
    for k, i in enumerate(b):
        ra = o[k] + t * v[k] - r[i]
        n = np.linalg.norm(ra)
        if n > 0:                # a spring at rest pulls nothing
            F[i] += np.clip(H1 * n, -1e3, 1e3) * ra / n
    if s.afm_force is not None:
        for i, f in zip(*s.afm_force):
            F[i] += f
    return F


def test_port_matches_closed_form():
    s = system()
    for term in (abi.TERM_VEL_AFM, abi.TERM_FORCE_AFM):
        p = abi.parse_params(only_term(term, yaml()))
        F, V = Oracle(p, s, "port").eval_forces()
        want = afm_force(s, s.r, 0.0)
        if term == abi.TERM_VEL_AFM:
            want -= afm_force(type(s)(**{**s.__dict__, "afm_vel": (np.zeros(0, np.int32), np.zeros((0, 3)),
                                                                     np.zeros((0, 3)))}), s.r, 0.0)
        else:
            want = np.zeros_like(want)
            for i, f in zip(*s.afm_force):
                want[i] += f
        assert np.abs(F - want).max() <= 1e-12 * max(1.0, np.abs(want).max())
        assert np.all(V == 0)


def test_tip_moves_with_time():
    """After k steps the velocity tip sits at orig + t vel."""
    s = system()
    s.afm_force = None
    p = abi.parse_params(only_term(abi.TERM_VEL_AFM, yaml()))
    o = Oracle(p, s, "port")
    o.step(40)
    r, _, t = o.get_state()
    F, _ = o.eval_forces()
    assert t > 0
    assert np.abs(F - afm_force(s, r, t)).max() <= 1e-9 * max(1.0, np.abs(F).max())


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
def test_port_bit_exact_vs_reference_live():
    """With explicit tip origins (a tip at its bead gives the reference
    0 * inf = NaN, which the restatement defines as no force)."""
    s = system()
    b, o, v = s.afm_vel
    s.afm_vel = (b, np.where(np.isnan(o), s.r[b] + 0.5 * ANGSTROM, o), v)
    p = abi.parse_params(yaml())
    a, b = Oracle(p, s, "port"), Oracle(p, s, "ref")
    Fa, Va = a.eval_forces()
    Fb, Vb = b.eval_forces()
    assert np.array_equal(Fa, Fb) and np.array_equal(Va, Vb)
    a.step(200)
    b.step(200)
    ya, ta, sa = a.get_history()
    yb, tb, sb = b.get_history()
    assert np.array_equal(ya, yb) and ta == tb and sa == sb


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_afm(prec):
    from xmd_gb300 import Engine
    s = system()
    o = Oracle(abi.parse_params(yaml()), s, "port")
    Fo, _ = o.eval_forces()
    with Engine(yaml(prec)) as e:
        e.add_system(s)
        F, _ = e.eval_forces(0)
        assert rel_err(F, Fo) <= (1e-10 if prec == "fp64" else 1e-5)
        if prec == "fp64":
            e.step(200)
            r, _, _ = e.get_state(0)
            o.step(200)
            ro, _, _ = o.get_state()
            assert np.abs(r - ro).max() / ANGSTROM <= 1e-8


@pytest.mark.gpu
def test_gpu_afm_rejects_bad_tips():
    from xmd_gb300 import Engine
    s = system()
    s.afm_vel = (np.array([0, 0], np.int32), np.zeros((2, 3)), np.zeros((2, 3)))
    with Engine(yaml()) as e:
        with pytest.raises(abi.XmdError):
            e.add_system(s)
