"""Dynamic membership and the continuous-batching server: a replica's
trajectory is the same, bit for bit, whether it runs alone or shares the
context with replicas that arrive and leave while it runs."""
import time

import numpy as np
import pytest

from xmd_gb300 import Engine, Server, abi, synth

pytestmark = pytest.mark.gpu

YAML = synth.yaml_for("c5", "mixed")


def systems():
    out = []
    for k, lens in enumerate([[120], [60, 90], [300], [45, 45, 45], [200]]):
        s = synth.make_system(lens, 500 + k, box=None, types="charged10", temperature=0.3 + 0.05 * k,
                              rng_seed=900 + k)
        out.append(s)
    return out


def alone(s, nsteps, yaml=YAML):
    with Engine(yaml) as e:
        e.add_system(s)
        e.step(nsteps)
        r, v, t = e.get_state(0)
    return r, v, t


def test_replicas_come_and_go_without_changing_each_other():
    ss = systems()
    with Engine(YAML) as e:
        e.reserve(2000, 4, 8 * 2000)
        a = e.add_system(ss[0])
        e.set_steps(a, 80)
        b = e.add_system(ss[1])
        e.set_steps(b, 200)
        e.step(48)                      # a, b run
        c = e.add_system(ss[2])         # arrives while a and b run
        e.set_steps(c, 100)
        e.step(48)                      # a stops at 80 inside this call
        ra, va, ta = e.get_state(a)
        e.remove_replica(a)             # leaves; its slot is reused next
        d = e.add_system(ss[3])
        e.set_steps(d, 64)
        assert d == a
        e.step(160)
        got = {k: e.get_state(rid) for k, rid in (("b", b), ("c", c), ("d", d))}
    want = {"a": alone(ss[0], 80), "b": alone(ss[1], 200), "c": alone(ss[2], 100), "d": alone(ss[3], 64)}
    got["a"] = (ra, va, ta)
    for k in "abcd":
        assert np.array_equal(got[k][0], want[k][0]), k
        assert np.array_equal(got[k][1], want[k][1]), k
        assert got[k][2] == pytest.approx(want[k][2], abs=0, rel=1e-12), k


def test_capacity_is_enforced():
    ss = systems()
    with Engine(YAML) as e:
        e.reserve(400, 2, 4000)
        e.add_system(ss[0])
        e.add_system(ss[1])
        with pytest.raises(abi.XmdError) as ei:
            e.add_system(ss[2])       # no third slot
        assert ei.value.code == -5
        e.step(4)


def test_server_results_equal_alone():
    """Requests submitted while others run (continuous batching) finish with
    the state each reaches alone."""
    ss = systems()
    steps = [96, 160, 64, 128, 200]
    with Server(YAML, hbm_budget=64 << 20, max_beads=4000, chunk_steps=32) as srv:
        ids = []
        for k, s in enumerate(ss):
            ids.append(srv.submit(s, steps[k]))
            time.sleep(0.01)
        res = [srv.result(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(ss)
    assert st["p99_s"] >= st["p50_s"] > 0
    for k, s in enumerate(ss):
        r, v, t = alone(s, steps[k])
        assert np.array_equal(res[k][0], r), k
        assert np.array_equal(res[k][1], v), k
        assert res[k][3] > 0


def test_server_rejects_oversized_request():
    big = synth.make_system([700], 77, box=None, types="charged10", temperature=0.4, rng_seed=1)
    with Server(YAML, hbm_budget=64 << 20, max_beads=500, chunk_steps=32) as srv:
        with pytest.raises(abi.XmdError) as ei:
            srv.submit(big, 10)
        assert ei.value.code == -5


def diverging(seed=610):
    """A chain with two beads far apart in sequence placed on the same spot:
    its first pair force is non-finite."""
    s = synth.make_system([80], seed, box=None, types="charged10", temperature=0.4, rng_seed=seed)
    s.r[40] = s.r[10]
    return s


def test_diverged_request_fails_alone():
    """A request whose trajectory goes non-finite is frozen and failed; the
    requests sharing the context finish with the state each reaches alone."""
    ss = systems()[:3]
    bad = diverging()
    steps = [96, 160, 64]
    with Server(YAML, hbm_budget=64 << 20, max_beads=4000, chunk_steps=32) as srv:
        ids = [srv.submit(ss[0], steps[0]), srv.submit(bad, 128), srv.submit(ss[1], steps[1]),
               srv.submit(ss[2], steps[2])]
        with pytest.raises(abi.XmdError) as ei:
            srv.result(ids[1])
        assert "non-finite" in str(ei.value)
        res = [srv.result(i) for i in (ids[0], ids[2], ids[3])]
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 3
    for k, s in enumerate(ss):
        r, v, t = alone(s, steps[k])
        assert np.array_equal(res[k][0], r), k
        assert np.array_equal(res[k][1], v), k


def test_static_context_reports_non_finite_and_freezes():
    """Outside the server a non-finite force fails the step call; the
    replica is frozen with finite positions and thaws on a new state."""
    bad = diverging()
    with Engine(YAML) as e:
        e.add_system(bad)
        with pytest.raises(abi.XmdError):
            e.step(8)
        r, _, _ = e.get_state(0)
        assert np.isfinite(r).all()
        good = synth.make_system([80], 611, box=None, types="charged10", temperature=0.4, rng_seed=611)
        e.set_state(0, good.r)
        e.step(8)
        r2, _, _ = e.get_state(0)
        assert np.isfinite(r2).all() and not np.array_equal(r2, good.r)


def test_budget_is_the_real_allocation():
    """The server sizes its reservation from the engine's measured device
    cost per bead slot, so the context it holds stays within the budget and
    uses most of it; the per-bead figure is the allocation's, not a guess."""
    budget = 1 << 30
    with Server(YAML, hbm_budget=budget, max_beads=10_000_000, chunk_steps=64) as srv:
        st = srv.stats()
    assert st["budget_bytes"] == budget
    assert 0.9 * budget <= st["device_bytes"] <= budget
    # the per-slot figure is the slope of the measured cost (its fixed part
    # can be slightly negative), so the product only approximates the budget
    assert st["cap_beads"] * st["bytes_per_bead"] <= 1.01 * budget
    assert 500 <= st["bytes_per_bead"] <= 4096


def test_frozen_replica_does_not_fail_the_others_evaluation():
    """After a replica is frozen by a non-finite force, evaluating (and
    observing) another replica of the context still works; evaluating the
    frozen one reports the non-finite force."""
    bad = diverging()
    good = synth.make_system([80], 611, box=None, types="charged10", temperature=0.4, rng_seed=611)
    with Engine(YAML) as e:
        g = e.add_system(good)
        b = e.add_system(bad)
        with pytest.raises(abi.XmdError):
            e.step(8)
        assert e.steps_left()[b] == -3
        F, _ = e.eval_forces(g)
        assert np.isfinite(F).all()
        assert np.isfinite(e.observables(g)["E"])
        with pytest.raises(abi.XmdError):
            e.eval_forces(b)


def test_server_queues_until_capacity_frees():
    """Requests that do not fit beside the running ones wait in the queue and
    are admitted when capacity frees (admission overlaps the running chunk);
    each still finishes with the state it reaches alone."""
    ss = [synth.make_system([300], 700 + k, box=None, types="charged10", temperature=0.35, rng_seed=710 + k)
          for k in range(4)]
    steps = [64, 96, 32, 128]
    with Server(YAML, hbm_budget=64 << 20, max_beads=650, chunk_steps=32) as srv:
        ids = [srv.submit(s, steps[k]) for k, s in enumerate(ss)]
        res = [srv.result(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == 4 and st["failed"] == 0
    assert st["peak_running"] <= 2
    for k, s in enumerate(ss):
        r, v, t = alone(s, steps[k])
        assert np.array_equal(res[k][0], r), k
