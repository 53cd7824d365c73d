"""The pseudo-improper dihedral potential (src/forces/pid/eval_forces.cpp,
bundle.cpp, lambda.h): energies against the reference's own kernel (its
forces leave dpsi2_* unset, so forces are checked against the energy's
numerical gradient), bundles against the list rule.  The engine has no PID path and rejects
a context that enables it."""
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


@pytest.mark.gpu
def test_engine_rejects_pid():
    """The engine has no PID path: a context that enables it fails loudly."""
    from xmd_gb300 import Engine
    with pytest.raises(abi.XmdError):
        Engine(yaml())
