"""GPU parity at the benchmark systems' full size.

Two fixtures made by the reference's own FP64 kernels (tests/golden/
make_golden.py):

  * c2_full8000: 16 chains x 500 beads in a 300 A periodic box, Go + Pauli +
    tether + native angle + CND + Debye-Hueckel (const ES), charges +-1 at
    p = 0.1 each: the plain FP64 benchmark system;
  * c3_full30720: 512 chains x 60 beads at 1e-3 A^-3 (periodic), Go +
    Debye-Hueckel + quasi-adiabatic contacts over a uniform 20-letter
    alphabet: the mixed-precision benchmark system.

Both are above the tile build's 4,096-bead limit, so every list here comes
from the cell-grid build (k_cells ... k_nl_cells).  Bars: forces and per-term
energies within 1e-10 relative (all terms, and each term alone against the
CPU restatement); the Verlet pair set equal to the restatement's list
filters; positions within 1e-8 A and the generator state exact at the last
snapshot inside the fixture's parity horizon; for c3, the exact
quasi-adiabatic contact list (slots, types, statuses) after 50 steps; and
the mixed path's forces within 1e-5 of FP64.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tests.test_gpu_parity import verlet_pairs, with_engine_key
from tests.util import ANGSTROM, FULL_CASES, energy_rel, horizon_snapshot, load_golden, only_term, rel_err
from xmd_gb300 import Engine, abi

pytestmark = pytest.mark.gpu

QA_OFF = "\nquasi-adiabatic potential:\n  enabled: false\n"


@pytest.fixture(scope="module", params=FULL_CASES)
def full(request):
    return (request.param,) + load_golden(request.param)


def test_full_size_forces_match_golden(full):
    name, s, y, z = full
    # step-0 forces: no quasi-adiabatic contact exists yet (the reference's
    # QA term adds exactly zero there), so the engine runs without it
    yy = y + QA_OFF if "c3" in name else y
    with Engine(yy) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, z["F0"]) <= 1e-10, rel_err(F, z["F0"])
    assert energy_rel(V, z["V0"]).max() <= 1e-10, energy_rel(V, z["V0"])


@pytest.mark.parametrize("term", [0, 1, 2, 4, 5, 6])
def test_full_size_per_term_forces(full, term):
    """One term enabled at a time, the list cutoffs kept as with all terms,
    against the CPU restatement on the same input."""
    name, s, y, _ = full
    full_p = abi.parse_params(y)
    mc = Oracle(full_p, s, "port").cutoffs()
    yy = only_term(term, y)
    yy += f"\nneighbor list:\n  cutoff: {float(mc[0] / ANGSTROM)!r} A\n  skin: {float(mc[1] / ANGSTROM)!r} A\n"
    p = abi.parse_params(yy)
    Fo, Vo = Oracle(p, s, "port").eval_forces()
    with Engine(yy) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-10, rel_err(F, Fo)
    assert energy_rel(V, Vo).max() <= 1e-10


def test_full_size_verlet_pairs_cell_build(full):
    """The cell-grid build keeps exactly the pairs of the reference's list
    filters (legacy_update.cpp, pauli.cpp:9-24, es_pair.cpp:6-23)."""
    name, s, y, _ = full
    y = with_engine_key(y, "nl build: cell")
    p = abi.parse_params(y)
    o = Oracle(p, s, "port")
    o.eval_forces()
    nl = o.nl_pairs()
    _, pad, _ = o.cutoffs()
    r = np.asarray(s.r)
    cell = np.asarray(s.cell)
    cinv = np.where(cell != 0, 1.0 / np.where(cell != 0, cell, 1.0), 0.0)
    dv = r[nl[:, 1]] - r[nl[:, 0]]
    dv = dv - cell * np.rint(dv * cinv)
    inv = 1.0 / np.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1] + dv[:, 2] * dv[:, 2])
    q = np.array([p.charge[a] for a in s.atype])
    fl = np.zeros(len(nl), dtype=int)
    if p.on[abi.TERM_PAULI]:
        fl |= (inv > 1.0 / (p.pauli_r_excl + pad)).astype(int)
    if p.on[abi.TERM_CONST_ES]:
        fl |= 2 * ((inv > 1.0 / (2.0 * p.const_es_screen_dist + pad)) & (q[nl[:, 0]] * q[nl[:, 1]] != 0)).astype(int)
    want = {(int(a), int(b)): int(f) for (a, b), f in zip(nl, fl) if f}
    with Engine(y) as e:
        e.add_system(s)
        e.eval_forces(0)
        got = verlet_pairs(e, 0, 4 * len(nl) + 16)
    assert len(want) > 1000
    assert got == want


def test_full_size_trajectory_matches_golden(full):
    """Positions within 1e-8 A and the generator state exact at the last
    snapshot inside the parity horizon; for c3, then the exact
    quasi-adiabatic contact list at each stored snapshot up to 50 steps
    (the oracle's own contact lists agree under reordered sums that far)."""
    name, s, y, z = full
    n, y_ref, rng_ref = horizon_snapshot(z)
    qa_steps = sorted(int(k[3:]) for k in z.files if k.startswith("qa_"))
    with Engine(y) as e:
        e.add_system(s)
        e.step(n)
        yy, _, rng = e.get_history(0)
        qa = {}
        done = n
        for k in qa_steps:
            if k < n:
                continue
            e.step(k - done)
            done = k
            qa[k] = e.qa_contacts(0)[0]
    assert rng == rng_ref
    pos_ref = y_ref if y_ref.ndim == 2 else y_ref[0]
    dr = np.abs(yy[0] - pos_ref).max() / ANGSTROM
    assert dr <= 1e-8, (n, dr)
    if y_ref.ndim == 3:
        assert np.abs(yy[1:] - y_ref[1:]).max() <= 1e-9
    if "c3" in name:
        assert 50 in qa and len(z["qa_50"]) > 1000
        for k, got in qa.items():
            assert np.array_equal(got, z[f"qa_{k}"]), k


def test_full_size_mixed_force_error(full):
    name, s, y, z = full
    yy = (y + QA_OFF if "c3" in name else y).replace("precision: fp64", "precision: mixed")
    with Engine(yy) as e:
        e.add_system(s)
        F, _ = e.eval_forces(0)
    err = rel_err(F, z["F0"])
    assert err <= 1e-5, err
