"""The CPU oracle against the reference's known answers (no GPU).

The golden fixtures were produced by the reference's own FP64 kernels
(tests/golden/make_golden.py); where the reference tree is present the
restatement is also compared with those kernels live.
"""
import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Oracle, rng_stream
from tests.util import GOLDEN, GOLDEN_CASES, energy_rel, horizon_snapshot, load_golden, rel_err
from xmd_gb300 import abi

have_ref = REF_LIB.exists()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_port_forces_match_golden(case):
    s, y, z = load_golden(case)
    o = Oracle(abi.parse_params(y), s, "port")
    F, V = o.eval_forces()
    assert rel_err(F, z["F0"]) <= 1e-13
    assert energy_rel(V, z["V0"]).max() <= 1e-13
    c = o.counts()
    assert (c["go"], c["pauli"], c["es"]) == (int(z["n_go0"]), int(z["n_pauli0"]), int(z["n_es0"]))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_port_trajectory_matches_golden(case):
    s, y, z = load_golden(case)
    o = Oracle(abi.parse_params(y), s, "port")
    n, y_ref, rng_ref = horizon_snapshot(z)
    o.step(n)
    yy, t, rng = o.get_history()
    assert rng == rng_ref
    # positions within 1e-8 A inside the parity horizon (the bar of the GPU path)
    assert np.abs(yy[0] - y_ref[0]).max() / 0.2 <= 1e-8
    assert np.abs(yy[1:] - y_ref[1:]).max() <= 1e-9
    if n == int(z["steps"]):
        assert t == float(z["t"])
        assert o.counts()["rebuilds"] == int(z["rebuilds"])
        F1, V1 = o.eval_forces()
        assert rel_err(F1, z["F1"]) <= 1e-8


def test_port_qa_state_matches_golden():
    s, y, z = load_golden("c3_qa600")
    o = Oracle(abi.parse_params(y), s, "port")
    o.step(100)
    qa100, _ = o.qa_contacts()
    assert np.array_equal(qa100, z["qa_100"])
    o.step(int(z["steps"]) - 100)
    qa, rt = o.qa_contacts()
    if have_ref:   # bit-exact on the reference's own platform; elsewhere chaos decides
        assert qa.shape == z["qa_contacts"].shape
        assert (qa == z["qa_contacts"]).all()
        assert np.array_equal(rt, z["qa_ref_time"])
        assert (o.sync() == z["sync"]).all()
    # the state machine went through every phase in this run
    assert (qa[:, 3] == 1).any() and (qa[:, 3] == 0).any()
    assert o.counts()["contact_slots"] > o.counts()["contacts"]


def test_rng_stream_matches_golden():
    z = np.load(GOLDEN / "rng_seed42.npz")
    raw, st = rng_stream("port", 42, 64)
    assert (raw == z["raw"]).all()
    assert st == int(z["state_after"])


@pytest.mark.skipif(not have_ref, reason="reference tree not built here")
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_port_bit_exact_vs_reference_live(case):
    s, y, _ = load_golden(case)
    p = abi.parse_params(y)
    a, b = Oracle(p, s, "port"), Oracle(p, s, "ref")
    Fa, Va = a.eval_forces()
    Fb, Vb = b.eval_forces()
    assert np.array_equal(Fa, Fb) and np.array_equal(Va, Vb)
    a.step(300)
    b.step(300)
    ya, ta, sa = a.get_history()
    yb, tb, sb = b.get_history()
    assert np.array_equal(ya, yb) and ta == tb and sa == sb


def test_omp_driver_matches_serial():
    """The OpenMP-structured driver (the timed CPU baseline) reproduces the
    serial step up to the reduction order of its atomic adds."""
    s, y, _ = load_golden("c2_periodic480")
    p = abi.parse_params(y)
    a, b = Oracle(p, s, "port"), Oracle(p, s, "port")
    a.step(50)
    b.step_omp(50, 4)
    ra, _, _ = a.get_state()
    rb, _, _ = b.get_state()
    assert np.abs(ra - rb).max() / 0.2 <= 1e-8


def test_oracle_edge_single_bead_and_open_box():
    from xmd_gb300.synth import System
    p = abi.parse_params("const ES:\n  enabled: false\nquasi-adiabatic potential:\n  enabled: false\n")
    s = System(n=1, chain=np.zeros(1, np.int32), seq=np.zeros(1, np.int32), atype=np.zeros(1, np.uint8),
               cell=np.zeros(3), r=np.zeros((1, 3)), tethers=(np.zeros(0, np.int32),) * 2 + (np.zeros(0),),
               angles=(np.zeros(0, np.int32),) * 3 + (np.zeros(0),),
               dihedrals=(np.zeros(0, np.int32),) * 4 + (np.zeros(0),),
               natives=(np.zeros(0, np.int32),) * 2 + (np.zeros(0),), temperature=0.35, seed=3)
    o = Oracle(p, s, "port")
    F, V = o.eval_forces()
    assert np.all(F == 0) and np.all(V == 0)
    o.step(10)
    r, _, t = o.get_state()
    assert np.isfinite(r).all() and abs(t - 0.05) < 1e-12


def test_serving_request_diverges_in_the_reference_kernels():
    """Serving request 15 of the seeded set (3,712 beads in 10 chains, open
    boundaries, seed 5015) goes non-finite in FP64 within 8,000 steps
    under the reference's own operations, as it does on the device: the
    server's failed requests are the reference's behaviour, not the engine's."""
    from oracle.pyoracle import parse_params
    from xmd_gb300 import synth
    s = synth._c5_one((5 * 1000 + 15, 64))
    o = Oracle(parse_params(synth.yaml_for("c5", "fp64")), s, "port")
    for _ in range(16):
        o.step_omp(500, 8)
        if not np.isfinite(o.get_state()[0]).all():
            break
    assert not np.isfinite(o.get_state()[0]).all()
