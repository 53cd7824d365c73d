"""The pseudo-improper dihedral potential (src/forces/pid/eval_forces.cpp,
bundle.cpp, lambda.h): the oracle's energies against the reference's own
kernel (its forces leave dpsi2_* unset, so the oracle's forces are checked
against the energy's numerical gradient); the engine's bundle lists against
the list rule, its per-term forces and energies and its trajectories against
the oracle."""
import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Oracle
from tests.util import only_term, rel_err
from xmd_gb300 import abi, synth

have_ref = REF_LIB.exists()


def system(seed=12):
    return synth.make_system([40, 35, 30], seed, box=None, types="uniform20", start="native", temperature=0.35)


def yaml(prec="fp64"):
    return synth.yaml_for("c1", prec) + "\npseudo-improper dihedral potential:\n  enabled: true\n"


def params(version):
    p = abi.parse_params(only_term(abi.TERM_PID, yaml()))
    p.pid_lambda = 1 if version == "algebraic" else 0
    return p


@pytest.mark.parametrize("version", ["cosine", "algebraic"])
def test_port_force_is_the_energy_gradient(version):
    """With depths small enough that lj and sink_lj never clamp dV/dr to
    1000 (their V is not clamped with it, so a clamped pair's force is not
    the gradient, as in the shipped Go and QA terms)."""
    s = system()
    p = params(version)
    p.pid_bbp[3] = p.pid_bbm[3] = 0.01
    for k in range(abi.NUM_SS):
        p.ss_depth[k] = 0.01
    o = Oracle(p, s, "port")
    F, V = o.eval_forces()
    assert V[abi.TERM_PID] != 0
    # the bundle set is fixed at the rebuild: differentiate with it frozen
    r0 = s.r.copy()
    g = np.zeros_like(r0)
    h = 1e-6
    for i in range(s.n):
        for a in range(3):
            for sg in (1, -1):
                rr = r0.copy()
                rr[i, a] += sg * h
                _, Vh = o.eval_at(rr)
                g[i, a] += sg * Vh[abi.TERM_PID] / (2 * h)
    assert rel_err(F, -g) <= 1e-6


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
@pytest.mark.parametrize("version", ["cosine", "algebraic"])
def test_energy_matches_the_reference_kernel(version):
    s = system()
    p = params(version)
    _, Va = Oracle(p, s, "port").eval_forces()
    _, Vb = Oracle(p, s, "ref").eval_forces()
    assert Va[abi.TERM_PID] != 0 and Va[abi.TERM_PID] == Vb[abi.TERM_PID]


ANGSTROM = 0.2


def pid_yaml(prec="fp64", version="cosine", base=None):
    y = synth.yaml_for("c1", prec) if base is None else base
    return y + f"\npseudo-improper dihedral potential:\n  enabled: true\n  lambda version: {version}\n"


def with_engine_key(y: str, line: str) -> str:
    if "\nengine:\n" in "\n" + y:
        return ("\n" + y).replace("\nengine:\n", "\nengine:\n  " + line + "\n", 1)[1:]
    return y + "\nengine:\n  " + line + "\n"


def periodic_system(seed=13):
    return synth.make_system([40, 35, 30], seed, box=60 * ANGSTROM, types="uniform20", start="native",
                             temperature=0.35)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("version", ["cosine", "algebraic"])
@pytest.mark.parametrize("box", ["open", "periodic"])
def test_engine_pid_term_matches_port(version, prec, box):
    """PID alone: the engine's forces and energy against the oracle's (the
    energy's gradient; the oracle's energy equals the reference kernel's).
    Both paths evaluate PID in FP64, so the bar is the FP64 one."""
    from xmd_gb300 import Engine
    s = system() if box == "open" else periodic_system()
    y = pid_yaml(prec, version, only_term(abi.TERM_PID, synth.yaml_for("c1", prec)))
    p = abi.parse_params(y)
    assert p.on[abi.TERM_PID] and p.pid_lambda == (1 if version == "algebraic" else 0)
    Fo, Vo = Oracle(p, s, "port").eval_forces()
    assert Vo[abi.TERM_PID] != 0
    with Engine(y) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo, floor=1e-12) <= 1e-10
    assert abs(V[abi.TERM_PID] - Vo[abi.TERM_PID]) <= 1e-10 * abs(Vo[abi.TERM_PID])


@pytest.mark.gpu
@pytest.mark.parametrize("build", ["cell", "tile"])
@pytest.mark.parametrize("box", ["open", "periodic"])
def test_engine_pid_bundles_match_rule(build, box):
    """Both Verlet builds flag exactly the bundles of update_pid_bundles
    (bundle.cpp:6-29): non-native list pairs within the PID cutoff + pad
    whose beads both have their chain neighbours."""
    import ctypes

    from xmd_gb300 import Engine
    s = system() if box == "open" else periodic_system()
    y = with_engine_key(pid_yaml(), f"nl build: {build}")
    p = abi.parse_params(y)
    o = Oracle(p, s, "port")
    o.eval_forces()
    nl = o.nl_pairs()
    mc, pad, _ = o.cutoffs()
    r = np.asarray(s.r)
    cell = np.asarray(s.cell)
    cinv = np.where(cell != 0, 1.0 / np.where(cell != 0, cell, 1.0), 0.0)
    dv = r[nl[:, 1]] - r[nl[:, 0]]
    dv = dv - cell * np.rint(dv * cinv)
    inv = 1.0 / np.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1] + dv[:, 2] * dv[:, 2])
    pid_cut = max(2.0 * p.lj_bb_r_min, 2.0 * p.lj_bs_r_min, 2.0 * max(p.ss_r_max[k] for k in range(abi.NUM_SS)))
    chain, seq = np.asarray(s.chain), np.asarray(s.seq)
    n = s.n
    has_prev = np.zeros(n, bool)
    has_next = np.zeros(n, bool)
    has_prev[1:] = (chain[1:] == chain[:-1]) & (seq[1:] == seq[:-1] + 1)
    has_next[:-1] = has_prev[1:]
    both = has_prev & has_next
    fl = ((inv > 1.0 / (p.pauli_r_excl + pad)) & bool(p.on[abi.TERM_PAULI])).astype(int)
    fl |= 4 * ((inv > 1.0 / (pid_cut + pad)) & both[nl[:, 0]] & both[nl[:, 1]]).astype(int)
    want = {(int(a), int(b)): int(f) for (a, b), f in zip(nl, fl) if f}
    assert any(f & 4 for f in want.values())
    with Engine(y) as e:
        e.add_system(s)
        e.eval_forces(0)
        cap = 4 * len(nl) + 16
        out = np.zeros(2 * cap, dtype=np.int32)
        flags = np.zeros(cap, dtype=np.uint8)
        cnt = ctypes.c_int32()
        abi.check(e.lib.xmd_gpu_verlet_pairs(e.h, 0, cap, abi.iptr(out),
                                              flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                              ctypes.byref(cnt)))
    got = {(int(out[2 * k]), int(out[2 * k + 1])): int(flags[k]) for k in range(cnt.value)}
    assert got == want


@pytest.mark.gpu
@pytest.mark.parametrize("box", ["open", "periodic"])
def test_engine_pid_trajectory_matches_port(box):
    """Go, Pauli, tether, angle, dihedral and PID together: all terms'
    forces at step 0, then 300 Langevin steps with the reference's noise
    stream, positions within 1e-8 A of the oracle's (native starts, inside
    the parity horizon)."""
    from xmd_gb300 import Engine
    s = system() if box == "open" else periodic_system()
    y = pid_yaml()
    p = abi.parse_params(y)
    o = Oracle(p, s, "port")
    Fo, Vo = o.eval_forces()
    with Engine(y) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
        assert rel_err(F, Fo) <= 1e-10
        assert abs(V[abi.TERM_PID] - Vo[abi.TERM_PID]) <= 1e-10 * abs(Vo[abi.TERM_PID])
        e.step(300)
        o.step(300)
        r, _, t = e.get_state(0)
    ro, _, to = o.get_state()
    assert np.abs(r - ro).max() / ANGSTROM <= 1e-8
    assert t == to
