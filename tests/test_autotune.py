"""Launch shapes and the autotuner: the trajectory never depends on the shape
(step-kernel block size and threads per bead, resident tile-build blocks,
steps per graph), and
autotuning leaves the context's state as it was."""
import numpy as np
import pytest

from xmd_gb300 import Engine, abi, synth

pytestmark = pytest.mark.gpu


def replicas():
    lens = [57, 130, 301, 75, 612]
    return [synth.make_system([L], 700 + k, box=None, types="charged10", temperature=0.3 + 0.05 * k,
                              rng_seed=800 + k) for k, L in enumerate(lens)]


def qa_replicas():
    """Two periodic systems with quasi-adiabatic contacts (20 x 30 beads)."""
    box = (600 / 1e-3) ** (1 / 3) * 0.2 * 0.5
    return [synth.make_system([30] * 20, 11 + k, box=box, types="uniform20", temperature=0.35) for k in range(2)]


def run(prec, shape, nsteps=200, workload="c4"):
    systems = replicas() if workload == "c4" else qa_replicas()
    with Engine(synth.yaml_for(workload, prec)) as e:
        for s in systems:
            e.add_system(s)
        if shape is not None:
            e.set_tuning(*shape)
        e.step(nsteps)
        return [e.get_state(r)[0] for r in range(len(systems))]


SHAPES = [(32, 0, 8, 1), (64, 2, 32, 2), (128, 1, 16, 4), (128, 0, 16, 1), (32, 0, 64, 2)]


@pytest.mark.parametrize("workload", ["c4", "c3"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_shapes_give_identical_trajectories(prec, workload):
    """Every shape, threads per bead included, gives the same bits: the
    pair sums run over four virtual lanes in a fixed tree whatever the
    number of threads holding them."""
    ref = run(prec, None, workload=workload)
    for shape in SHAPES:
        got = run(prec, shape, workload=workload)
        for r in range(len(ref)):
            assert np.array_equal(got[r], ref[r]), (shape, r)


def test_autotune_keeps_state_and_picks_a_valid_shape():
    with Engine(synth.yaml_for("c4", "mixed")) as e, Engine(synth.yaml_for("c4", "mixed")) as f:
        for s in replicas():
            e.add_system(s)
            f.add_system(s)
        e.step(32)
        f.step(32)
        best = e.autotune(64)
        assert best["fb"] in (32, 64, 128) and best["graph_steps"] in (8, 16, 32, 64) and best["lpb"] in (1, 2, 4)
        assert best["ms_per_step"] > 0
        assert e.tuning() == {k: best[k] for k in ("fb", "tile_per_sm", "graph_steps", "lpb")}
        e.step(96)
        f.step(96)
        for r in range(5):
            assert np.array_equal(e.get_state(r)[0], f.get_state(r)[0]), r


def test_bad_shape_rejected():
    with Engine(synth.yaml_for("c4", "mixed")) as e:
        e.add_system(replicas()[0])
        with pytest.raises(abi.XmdError):
            e.set_tuning(100, 0, 16)
        with pytest.raises(abi.XmdError):
            e.set_tuning(64, 0, 12)
        with pytest.raises(abi.XmdError):
            e.set_tuning(64, 0, 16, 3)
