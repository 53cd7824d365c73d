"""Chirality (src/forces/chiral.cpp:15-37) and native disulfide bonds
(src/forces/native_ss.cpp:8-40): the restatement against closed forms and the
reference's own kernels, the GPU path against the restatement (FP64 to 1e-10,
mixed within its force bound)."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Oracle
from tests.util import ANGSTROM, energy_rel, only_term, rel_err
from xmd_gb300 import abi, synth

have_ref = REF_LIB.exists()
E_CHI = 1.0                             # chirality: e_chi = 1 eps
H1, NAT_R = 100.0 / ANGSTROM**2, 6.0 * ANGSTROM   # native ssbonds: H1 = 100 eps/A^2, 6 A

def system(seed=21, n_ss=5, noise=0.25, lens=(60, 45)):
    """Chains near their native structure (so chirality and the disulfides sit
    close to, not at, their minima); the n_ss native contacts nearest the 6 A
    disulfide length, between distinct beads, become disulfides (CYS pairs),
    taken out of the Go list."""
    s = synth.make_system(list(lens), seed, box=None, types="uniform20", start="native", temperature=0.35)
    rng = np.random.default_rng(seed + 1)
    s.r = s.r + rng.normal(0.0, noise * ANGSTROM, size=s.r.shape)
    n1, n2, nd = s.natives
    order = np.argsort(np.abs(nd - NAT_R), kind="stable")
    used, ss = set(), []
    for k in order:
        a, b = int(n1[k]), int(n2[k])
        if a in used or b in used:
            continue
        used |= {a, b}
        ss.append(k)
        if len(ss) == n_ss:
            break
    keep = np.setdiff1d(np.arange(len(n1)), ss)
    s.ssbonds = (n1[ss].astype(np.int32), n2[ss].astype(np.int32))
    s.natives = (n1[keep], n2[keep], nd[keep])
    s.atype = s.atype.copy()
    s.atype[np.concatenate(s.ssbonds)] = abi.AA.index("CYS")
    return s


def yaml(prec="fp64", chir=True, ss=True):
    return synth.yaml_for("c1", prec) + (f"\nchirality:\n  enabled: {'true' if chir else 'false'}\n"
                                         f"\nnative ssbonds:\n  enabled: {'true' if ss else 'false'}\n")


def only(term, y):
    return only_term(term, y)


def chiral_energy(s, r):
    i1, i2, i3, i4, fac, c0 = s.chirals
    r12, r23, r34 = r[i2] - r[i1], r[i3] - r[i2], r[i4] - r[i3]
    c = (r12 * np.cross(r23, r34)).sum(axis=1) * fac
    return 0.5 * E_CHI * ((c - c0) ** 2).sum()


def ss_energy(s, r):
    a, b = s.ssbonds
    d = np.linalg.norm(r[b] - r[a], axis=1)
    return np.clip(0.5 * H1 * (d - NAT_R) ** 2, -1e3, 1e3).sum()     # harmonic(H1, 0, nat_r), clamped


def num_grad(fn, s, h=1e-6):
    g = np.zeros_like(s.r)
    for i in range(s.n):
        for x in range(3):
            rp, rm = s.r.copy(), s.r.copy()
            rp[i, x] += h
            rm[i, x] -= h
            g[i, x] = (fn(s, rp) - fn(s, rm)) / (2 * h)
    return g


def test_chiral_quads_are_zero_at_the_native_structure():
    s = synth.make_system([40], 3, box=None, types="uniform20", start="native")
    i1, i2, i3, i4, fac, c0 = s.chirals
    assert len(i1) == 37 and np.array_equal(i2, i1 + 1) and np.array_equal(i4, i1 + 3)
    assert np.all(fac > 0) and np.abs(c0).max() > 0
    o = Oracle(abi.parse_params(only(abi.TERM_CHIR, yaml())), s, "port")
    F, V = o.eval_forces()
    assert abs(V[abi.TERM_CHIR]) < 1e-24 and np.abs(F).max() < 1e-10


def chiral_first_bead_offset(s, r):
    """The reference's force on i1 of each quad is f (r12 x r23)
    (chiral.cpp:33), where -dV/dr1 = f (r23 x r34); f = e_chi (chir -
    nat_chir) nat_factor.  Returns the per-bead difference to -grad V."""
    i1, i2, i3, i4, fac, c0 = s.chirals
    r12, r23, r34 = r[i2] - r[i1], r[i3] - r[i2], r[i4] - r[i3]
    f = E_CHI * ((r12 * np.cross(r23, r34)).sum(axis=1) * fac - c0) * fac
    out = np.zeros_like(r)
    np.add.at(out, i1, f[:, None] * (np.cross(r12, r23) - np.cross(r23, r34)))
    return out


@pytest.mark.parametrize("term,energy", [(abi.TERM_CHIR, chiral_energy), (abi.TERM_NAT_SS, ss_energy)])
def test_port_matches_closed_form(term, energy):
    """Energy equals the closed form; force = -grad V by central differences,
    up to the reference's first-bead chirality force."""
    s = system(n_ss=5)
    o = Oracle(abi.parse_params(only(term, yaml())), s, "port")
    F, V = o.eval_forces()
    Vw = energy(s, s.r)
    assert Vw > 0 and abs(V[term] - Vw) <= 1e-12 * Vw
    assert np.abs(np.delete(V, term)).max() == 0
    want = -num_grad(energy, s)
    if term == abi.TERM_CHIR:
        off = chiral_first_bead_offset(s, s.r)
        assert np.abs(off).max() > 1e-3 * np.abs(want).max()     # the offset is not negligible
        want = want + off
    assert rel_err(F, want) <= 1e-6


def test_ss_bonds_leave_the_active_list_beyond_cutoff_plus_pad():
    """update_nat_ssbonds keeps a disulfide only while |r12| < cutoff + pad at
    the list build (native_ss.cpp:8-19): a pair pulled apart contributes
    nothing, and the Go term does not take it over."""
    s = system(n_ss=2)
    a, b = int(s.ssbonds[0][0]), int(s.ssbonds[1][0])
    far = s.r.copy()
    far[b] = far[a] + np.array([40.0 * ANGSTROM, 0, 0])     # beyond 2 * 6 A + skin
    s.r = far
    p = abi.parse_params(only(abi.TERM_NAT_SS, yaml()))
    F, V = Oracle(p, s, "port").eval_forces()
    want = ss_energy(SimpleNamespace(ssbonds=(s.ssbonds[0][1:], s.ssbonds[1][1:])), s.r)
    assert want > 0 and abs(V[abi.TERM_NAT_SS] - want) <= 1e-12 * want
    assert np.all(F[a] == 0) and np.all(F[b] == 0)


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
@pytest.mark.parametrize("box", [None, 60.0])
def test_port_bit_exact_vs_reference_live(box):
    s = system(seed=31)
    if box is not None:
        s.cell = np.full(3, box * ANGSTROM)
    y = yaml()
    p = abi.parse_params(y)
    a, b = Oracle(p, s, "port"), Oracle(p, s, "ref")
    Fa, Va = a.eval_forces()
    Fb, Vb = b.eval_forces()
    assert Va[abi.TERM_CHIR] > 0 and Va[abi.TERM_NAT_SS] > 0
    assert np.array_equal(Fa, Fb) and np.array_equal(Va, Vb)
    a.step(300)
    b.step(300)
    ya, ta, sa = a.get_history()
    yb, tb, sb = b.get_history()
    assert np.array_equal(ya, yb) and ta == tb and sa == sb


@pytest.mark.gpu
@pytest.mark.parametrize("term", [abi.TERM_CHIR, abi.TERM_NAT_SS])
def test_gpu_term_forces(term):
    from xmd_gb300 import Engine
    s = system()
    full = abi.parse_params(yaml())
    mc = Oracle(full, s, "port").cutoffs()
    yy = only(term, yaml()) + (f"\nneighbor list:\n  cutoff: {float(mc[0] / ANGSTROM)!r} A\n"
                               f"  skin: {float(mc[1] / ANGSTROM)!r} A\n")
    Fo, Vo = Oracle(abi.parse_params(yy), s, "port").eval_forces()
    with Engine(yy) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-10
    assert energy_rel(V, Vo).max() <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("box", [None, 60.0])
def test_gpu_trajectory_with_all_terms(box):
    from xmd_gb300 import Engine
    s = system(seed=41)
    if box is not None:
        s.cell = np.full(3, box * ANGSTROM)
    y = yaml()
    o = Oracle(abi.parse_params(y), s, "port")
    Fo, Vo = o.eval_forces()
    with Engine(y) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
        assert rel_err(F, Fo) <= 1e-10
        assert energy_rel(V, Vo).max() <= 1e-10
        e.step(200)
        r, _, _ = e.get_state(0)
    o.step(200)
    ro, _, _ = o.get_state()
    assert np.abs(r - ro).max() / ANGSTROM <= 1e-8


@pytest.mark.gpu
def test_gpu_mixed_forces_within_bound():
    from xmd_gb300 import Engine
    s = system(seed=51)
    y = yaml("mixed")
    Fo, Vo = Oracle(abi.parse_params(yaml()), s, "port").eval_forces()
    with Engine(y) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-5
    for t in (abi.TERM_CHIR, abi.TERM_NAT_SS):
        assert abs(V[t] - Vo[t]) <= 1e-5 * abs(Vo[t])
