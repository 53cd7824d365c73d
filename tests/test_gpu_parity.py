"""GPU parity: the sm_103a engine, called through its C ABI, against the
reference's known answers (golden fixtures from the reference's own FP64
kernels) and against the CPU restatement on fresh inputs.

Bars:
  * plain FP64: per-term forces and energies within 1e-10 relative;
  * positions within 1e-8 A after up to 1000 steps driven by the same
    generator stream (the engine reproduces the reference's xorshift stream
    bead by bead through a GF(2) jump-ahead), inside each system's parity
    horizon: the step count up to which the oracle agrees with ITSELF under a
    reordered force summation to 1e-9 A.  Near-equilibrium systems hold for
    the full 1000 steps; extended starts amplify rounding after 100-200 steps
    (measured in tests/golden/make_golden.py);
  * mixed precision: forces within 1e-5 relative of the FP64 oracle.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from tests.util import ANGSTROM, FP64_CASES, energy_rel, horizon_snapshot, load_golden, only_term, rel_err
from xmd_gb300 import Engine, abi, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", FP64_CASES + ["c3_qa600"])
def test_eval_forces_match_golden(case):
    s, y, z = load_golden(case)
    if case == "c3_qa600":
        y += "\nquasi-adiabatic potential:\n  enabled: false\n"
        p = abi.parse_params(y)
        Fo, Vo = Oracle(p, s, "port").eval_forces()
    else:
        Fo, Vo = z["F0"], z["V0"]
    with Engine(y) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-10, rel_err(F, Fo)
    assert energy_rel(V, Vo).max() <= 1e-10, energy_rel(V, Vo)


@pytest.mark.parametrize("case", FP64_CASES)
def test_trajectory_matches_golden(case):
    s, y, z = load_golden(case)
    n, y_ref, rng_ref = horizon_snapshot(z)
    with Engine(y) as e:
        e.add_system(s)
        e.step(n)
        yy, t, rng = e.get_history(0)
    assert rng == rng_ref
    dr = np.abs(yy[0] - y_ref[0]).max() / ANGSTROM
    assert dr <= 1e-8, (n, dr)
    assert np.abs(yy[1:] - y_ref[1:]).max() <= 1e-9
    if n == int(z["steps"]):
        assert abs(t - float(z["t"])) <= 1e-12


def test_qa_state_matches_golden():
    """Quasi-adiabatic contacts (sift, greedy acceptance in slot order,
    saturation ramps, breaking, re-freeing) against the reference's own QA
    kernels: identical contact list (slot order, types, statuses, ref times)
    after 50 steps, inside the parity horizon, with positions within 1e-8 A;
    the 0.25 tau phase has contacts breaking by then."""
    s, y, z = load_golden("c3_qa600")
    with Engine(y) as e:
        e.add_system(s)
        e.step(50)
        qa, rt = e.qa_contacts(0)
        yy, _, rng = e.get_history(0)
    assert np.array_equal(qa, z["qa_50"])
    assert rng == int(z["rng_50"])
    assert np.abs(yy[0] - z["y_50"][0]).max() / ANGSTROM <= 1e-8
    assert len(qa) > 100


def test_qa_long_run_state_machine():
    """Past the parity horizon the engine keeps the QA invariants: valence
    counters never go negative and equal the limits minus what live contacts
    hold; no pair is in two contacts."""
    s, y, _ = load_golden("c3_qa600")
    p = abi.parse_params(y)
    with Engine(y) as e:
        e.add_system(s)
        e.step(500)
        qa, _ = e.qa_contacts(0)
        sync = e.qa_sync(0).astype(int)
    assert (sync >= 0).all()
    pairs = {(a, b) for a, b, _, _ in qa}
    assert len(pairs) == len(qa)
    lim = np.array([p.limits[a][:] for a in s.atype], dtype=int)
    assert (sync <= lim).all()


@pytest.mark.parametrize("seed", [21, 22])
def test_fresh_system_matches_port(seed):
    """Systems not in the fixtures: periodic, charged, native starts."""
    s = synth.make_system([50] * 5, seed, box=150 * ANGSTROM, temperature=0.35, start="native")
    y = synth.yaml_for("c2")
    p = abi.parse_params(y)
    o = Oracle(p, s, "port")
    Fo, Vo = o.eval_forces()
    with Engine(y) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
        assert rel_err(F, Fo) <= 1e-10
        assert energy_rel(V, Vo).max() <= 1e-10
        e.step(500)
        o.step(500)
        r, v, t = e.get_state(0)
    ro, vo, to = o.get_state()
    assert np.abs(r - ro).max() / ANGSTROM <= 1e-8
    assert t == to


@pytest.mark.parametrize("case", ["c1_chain100", "c2_periodic480", "c2_relsnd480"])
def test_mixed_precision_force_error(case):
    s, y, z = load_golden(case)
    with Engine(y.replace("precision: fp64", "precision: mixed")) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    err = rel_err(F, z["F0"])
    assert err <= 1e-5, err


def test_batched_replicas_equal_alone():
    """Replicas packed into one context give bit-identical results to the
    same systems run alone (per-replica streams, grids and lists)."""
    systems = [synth.make_system([L], 300 + k, box=None, temperature=0.3 + 0.1 * k)
               for k, L in enumerate([57, 120, 33])]
    y = synth.yaml_for("c2")
    alone = []
    for s in systems:
        with Engine(y) as e:
            e.add_system(s)
            e.step(300)
            alone.append(e.get_history(0))
    with Engine(y) as e:
        for s in systems:
            e.add_system(s)
        e.step(300)
        for k in range(len(systems)):
            yy, t, st = e.get_history(k)
            assert np.array_equal(yy, alone[k][0])
            assert t == alone[k][1] and st == alone[k][2]


def test_graph_and_stream_paths_agree():
    """Graph-captured chunks (device-side rebuild decisions) and the plain
    per-step path give identical trajectories; a step count that is not a
    multiple of the graph length runs its rest in graphs of 4, 2 and 1 steps
    (the last one leaves the position buffers swapped)."""
    s, y, _ = load_golden("c2_periodic480")
    with Engine(y) as a, Engine(y) as b:
        a.add_system(s)
        b.add_system(s)
        a.set_tuning(64, 0, 16, 1)
        a.step(71)                       # graphs of 16, 16, 16, 16, 4, 2, 1 steps
        abi.check(b.lib.xmd_gpu_set_kernel_timing(b.h, 1))   # timing forces the per-step path
        b.step(71)
        ya, ta, sa = a.get_history(0)
        yb, tb, sb = b.get_history(0)
    assert np.array_equal(ya, yb) and ta == tb and sa == sb


@pytest.mark.parametrize("case,build", [("c2_periodic480", "cell"), ("c3_qa600", "tile"), ("c3_qa600", "cell")])
def test_gated_graphs_agree_with_stream_path(case, build):
    """Cell-path and quasi-adiabatic contexts run graphs without rebuild
    nodes that halt at a flagged skin check (the host rebuilds), and graphs
    with IF rebuild nodes while rebuilds come every few steps; both give the
    per-step path's trajectory bit for bit (200 steps from the fixture's
    start, where the lists are rebuilt often and then rarely)."""
    s, y, _ = load_golden(case)
    y = with_engine_key(y, f"nl build: {build}")
    with Engine(y) as a, Engine(y) as b:
        a.add_system(s)
        b.add_system(s)
        a.step(200)
        abi.check(b.lib.xmd_gpu_set_kernel_timing(b.h, 1))   # timing forces the per-step path
        b.step(200)
        ya, ta, sa = a.get_history(0)
        yb, tb, sb = b.get_history(0)
        assert a.stats()["rebuilds"] == b.stats()["rebuilds"]
        if "qa" in case:
            ca, cb = a.qa_contacts(0), b.qa_contacts(0)
            assert np.array_equal(ca[0], cb[0]) and np.array_equal(ca[1], cb[1])
    assert np.array_equal(ya, yb) and ta == tb and sa == sb


def test_packed_upload_download_roundtrip():
    systems = [synth.make_system([L], 500 + k, temperature=0.4) for k, L in enumerate([40, 75])]
    with Engine(synth.yaml_for("c2")) as e:
        for s in systems:
            e.add_system(s)
        e.step(20)
        hs = [e.get_history(k)[0] for k in range(2)]
        packed = np.ascontiguousarray(np.concatenate(hs, axis=1).reshape(6, -1))
        abi.check(e.lib.xmd_gpu_upload_history_all(e.h, abi.dptr(packed)))
        r = np.zeros(3 * (40 + 75))
        abi.check(e.lib.xmd_gpu_download_positions_all(e.h, abi.dptr(r)))
        assert np.array_equal(r.reshape(-1, 3), np.concatenate([h[0] for h in hs]))
        yall = np.zeros(18 * (40 + 75))
        abi.check(e.lib.xmd_gpu_download_history_all(e.h, abi.dptr(yall)))
        assert np.array_equal(yall, packed.reshape(-1))


def test_host_round_trip_keeps_the_trajectory():
    """Carrying the whole state through host memory between chunks
    (download_history_all, upload_history_all) leaves the trajectory
    bit-identical to a run that never leaves the device."""
    systems = [synth.make_system([L], 600 + k, temperature=0.4) for k, L in enumerate([60, 90])]
    y = synth.yaml_for("c2")
    with Engine(y) as a, Engine(y) as b:
        for s in systems:
            a.add_system(s)
            b.add_system(s)
        a.step(200)
        host = np.zeros(18 * 150)
        for _ in range(5):
            abi.check(b.lib.xmd_gpu_download_history_all(b.h, abi.dptr(host)))
            abi.check(b.lib.xmd_gpu_upload_history_all(b.h, abi.dptr(host)))
            b.step(40)
        for k in range(2):
            ya, ta, sa = a.get_history(k)
            yb, tb, sb = b.get_history(k)
            assert np.array_equal(ya, yb) and ta == tb and sa == sb


def with_engine_key(y: str, line: str) -> str:
    """YAML with `line` added to its engine section (one section per key)."""
    if "\nengine:\n" in "\n" + y:
        return ("\n" + y).replace("\nengine:\n", "\nengine:\n  " + line + "\n", 1)[1:]
    return y + "\nengine:\n  " + line + "\n"


def verlet_pairs(e, rep, cap):
    import ctypes
    out = np.zeros(2 * cap, dtype=np.int32)
    flags = np.zeros(cap, dtype=np.uint8)
    cnt = ctypes.c_int32()
    abi.check(e.lib.xmd_gpu_verlet_pairs(e.h, rep, cap, abi.iptr(out),
                                          flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                          ctypes.byref(cnt)))
    assert cnt.value <= cap
    return {(int(out[2 * k]), int(out[2 * k + 1])): int(flags[k]) for k in range(cnt.value)}


@pytest.mark.parametrize("build", ["cell", "tile"])
@pytest.mark.parametrize("case", ["c2_periodic480", "c1_chain100", "c3_qa600"])
def test_verlet_pairs_match_oracle(case, build):
    """Both Verlet builds (cell grid, whole-replica tiles) keep exactly the
    pairs of the reference's list filters: non-native pairs within the Verlet
    radius (legacy_update.cpp), Pauli within r_excl + pad (pauli.cpp:9-24), ES
    within 2D + pad with q1 q2 != 0 (es_pair.cpp:6-23); as sets, with
    identical membership."""
    s, y, _ = load_golden(case)
    y = with_engine_key(y, f"nl build: {build}")
    p = abi.parse_params(y)
    assert p.nl_build == {"cell": 1, "tile": 2}[build]
    o = Oracle(p, s, "port")
    o.eval_forces()
    nl = o.nl_pairs()
    mc, pad, _ = o.cutoffs()
    r = np.asarray(s.r)
    cell = np.asarray(s.cell)
    cinv = np.where(cell != 0, 1.0 / np.where(cell != 0, cell, 1.0), 0.0)
    dv = r[nl[:, 1]] - r[nl[:, 0]]
    dv = dv - cell * np.rint(dv * cinv)
    dd = np.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1] + dv[:, 2] * dv[:, 2])
    inv = 1.0 / dd
    q = np.array([p.charge[a] for a in s.atype])
    pauli = p.on[abi.TERM_PAULI] and True
    fl = np.zeros(len(nl), dtype=int)
    if pauli:
        fl |= (inv > 1.0 / (p.pauli_r_excl + pad)).astype(int)
    if p.on[abi.TERM_CONST_ES]:
        fl |= 2 * ((inv > 1.0 / (2.0 * p.const_es_screen_dist + pad)) & (q[nl[:, 0]] * q[nl[:, 1]] != 0)).astype(int)
    want = {(int(a), int(b)): int(f) for (a, b), f in zip(nl, fl) if f}
    with Engine(y) as e:
        e.add_system(s)
        e.eval_forces(0)
        got = verlet_pairs(e, 0, 4 * len(nl) + 16)
    assert got == want


@pytest.mark.parametrize("case", ["c2_periodic480", "c2_sparse240", "c3_qa600", "c1_native100"])
def test_cell_and_tile_builds_agree(case):
    """Along a trajectory (lists rebuilt many times), the cell-grid and the
    tile build keep the same pairs, the same Go list and the same QA state;
    forces differ only by the summation order of each bead's pair row."""
    s, y, _ = load_golden(case)
    res = {}
    for build in ("cell", "tile"):
        with Engine(with_engine_key(y, f"nl build: {build}")) as e:
            e.add_system(s)
            e.step(40)
            pairs = verlet_pairs(e, 0, 1 << 20)
            F, V = e.eval_forces(0)
            st = e.stats()
            res[build] = (pairs, F, V, st, e.qa_contacts(0) if "qa" in case else None, e.get_state(0)[0])
    a, b = res["cell"], res["tile"]
    assert a[0] == b[0]
    # the two builds order a row's entries differently: FP64 sums in another
    # order (a few ulps of the largest pair force, clamped at 1e3)
    assert rel_err(b[1], a[1]) <= 1e-11
    assert a[3]["go_active"] == b[3]["go_active"] and a[3]["rebuilds"] == b[3]["rebuilds"]
    assert np.abs(a[5] - b[5]).max() <= 1e-9
    if a[4] is not None:
        assert np.array_equal(a[4][0], b[4][0])


def test_verlet_capacity_overflow_is_reported():
    s, y, _ = load_golden("c2_periodic480")
    with Engine(y + "\nengine:\n  nl capacity: 1\n  nl grow: false\n") as e:
        e.add_system(s)
        with pytest.raises(abi.XmdError) as ei:
            e.eval_forces(0)
        assert ei.value.code == -5


def test_verlet_rows_grow_on_demand():
    """With growth on (the default) a too-small initial capacity is raised at
    the first rebuild and the forces are unaffected."""
    s, y, z = load_golden("c2_periodic480")
    with Engine(y + "\nengine:\n  nl capacity: 2\n") as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
        e.step(40)
    assert rel_err(F, z["F0"], floor=1.0) <= 1e-10


# one term at a time: tether 0, native angle 1, CND 2, SND 3, Go 4, Pauli 5,
# const ES 6, relative ES 7
PER_TERM = [(c, k) for c in ("c1_chain100", "c2_periodic480", "c3_qa600") for k in (0, 1, 2, 4, 5, 6)] + \
           [("c2_relsnd480", k) for k in (0, 1, 3, 4, 5, 7)]


@pytest.mark.parametrize("case,term", PER_TERM)
def test_per_term_forces(case, term):
    """One term enabled at a time (the list cutoffs kept as with all terms):
    forces and energy of that term alone within 1e-10 of the oracle,
    normalised by that term's own force scale."""
    s, y, _ = load_golden(case)
    full = abi.parse_params(y)
    mc = Oracle(full, s, "port").cutoffs()
    yy = only_term(term, y)
    yy += f"\nneighbor list:\n  cutoff: {float(mc[0] / ANGSTROM)!r} A\n  skin: {float(mc[1] / ANGSTROM)!r} A\n"
    p = abi.parse_params(yy)
    Fo, Vo = Oracle(p, s, "port").eval_forces()
    with Engine(yy) as e:
        e.add_system(s)
        F, V = e.eval_forces(0)
    assert rel_err(F, Fo) <= 1e-10, rel_err(F, Fo)
    assert energy_rel(V, Vo).max() <= 1e-10


def test_bad_topology_rejected():
    s = synth.make_system([20], 5)
    bad = (s.angles[0][:1], s.angles[1][:1] + 1, s.angles[2][:1], s.angles[3][:1])
    s.angles = bad
    with Engine(synth.yaml_for("c1")) as e:
        with pytest.raises(abi.XmdError) as ei:
            e.add_system(s)
        assert ei.value.code == -1
