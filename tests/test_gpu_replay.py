"""Bit-exact replay: the device's generations against the oracle replaying
the same Philox stream on the CPU (every selection decided in FP64).

The device decides selections in FP32 and re-decides in FP64 those whose
fitness gap lies within the rounding window, so its populations must equal
the FP64-decided replay exactly (bit for bit), generation after generation.
Operators: DE/rand/1/bin and DE/current/1/bin (proposed model/
SG-EMTF_DE.cu:474-600), SBX + polynomial mutation (SG-EMTF.cu:548-831)."""
import numpy as np
import pytest

from gpu_util import make_engine, oracle_params

pytestmark = pytest.mark.gpu


def replay(orc, p, tasks, X, gens, gen0=0):
    out = []
    for t, x in zip(tasks, X):
        x = x.copy()
        f32 = np.zeros(t.NP, np.float32)
        f64 = np.array([t.eval64(r)[0] for r in x])
        f32[:] = f64
        for g in range(gen0 + 1, gen0 + gens + 1):
            orc.generation(p, t, x, f32, f64, g, 0)
        out.append(x)
    return out


def test_initial_population_bit_exact(sgemtf, orc):
    specs = [(f, D, NP, 1) for f, D, NP in [(0, 50, 64), (3, 7, 5), (6, 128, 16), (2, 1, 4)]]
    eng, tasks = make_engine(sgemtf, orc, specs, seed=77)
    eng.reset()
    for i, t in enumerate(tasks):
        X, f = eng.population(i)
        want = orc.gen_population(77, i, t.NP, t.D, t.c.lo, t.c.hi)
        assert np.array_equal(X, want)
        # shift vectors are drawn from the same stream
        assert np.array_equal(t.o, orc.gen_shift(77, i, t.D, t.c.lo, t.c.hi))


@pytest.mark.parametrize("alg", [0, 1, 2])
def test_replay_all_functions(sgemtf, orc, alg):
    specs = [(f, 10, 16, 1) for f in range(7)]
    eng, tasks = make_engine(sgemtf, orc, specs, seed=5, algorithm=alg)
    eng.reset()
    X0 = [eng.population(i)[0] for i in range(len(tasks))]
    gens = 25
    eng.run(gens)
    want = replay(orc, oracle_params(orc, eng), tasks, X0, gens)
    for i in range(len(tasks)):
        got = eng.population(i)[0]
        assert np.array_equal(got, want[i]), (alg, i, np.argwhere(got != want[i])[:5])


@pytest.mark.parametrize("D,NP", [(1, 4), (3, 5), (50, 64), (50, 100), (100, 128), (33, 256)])
def test_replay_shapes(sgemtf, orc, D, NP):
    specs = [(f, D, NP, 1) for f in (0, 2, 6)]
    eng, tasks = make_engine(sgemtf, orc, specs, seed=11)
    eng.reset()
    X0 = [eng.population(i)[0] for i in range(len(tasks))]
    gens = 6
    eng.run(gens)
    want = replay(orc, oracle_params(orc, eng), tasks, X0, gens)
    for i in range(len(tasks)):
        assert np.array_equal(eng.population(i)[0], want[i])


def test_split_runs_equal_one_run(sgemtf, orc):
    """Philox counters come from the generation number: 3 x 10 == 1 x 30."""
    specs = [(f, 20, 32, 1) for f in range(7)]
    a, _ = make_engine(sgemtf, orc, specs, seed=21)
    b, _ = make_engine(sgemtf, orc, specs, seed=21)
    a.run(30)
    for _ in range(3):
        b.run(10)
    for i in range(7):
        assert np.array_equal(a.population(i)[0], b.population(i)[0])


def test_config1_shape_identity_rotation(sgemtf, orc):
    """8 tasks, NP 100, D 50, identity rotation, functions in the config
    order sphere..weierstrass, sphere (first generations replayed)."""
    fids = [0, 1, 2, 3, 4, 5, 6, 0]
    specs = [(f, 50, 100, 0) for f in fids]
    eng, tasks = make_engine(sgemtf, orc, specs, seed=2)
    eng.reset()
    X0 = [eng.population(i)[0] for i in range(8)]
    eng.run(5)
    want = replay(orc, oracle_params(orc, eng), tasks, X0, 5)
    for i in range(8):
        assert np.array_equal(eng.population(i)[0], want[i])


@pytest.mark.parametrize("precision,flags", [(0, 0), (1, 0), (3, 0), (0, 0x40)])
def test_replay_converged_islands(sgemtf, orc, precision, flags):
    """Long runs of small islands converge until trial and parent differ by a
    few ulps and most selections are near-ties: every re-check path (the
    differential decision with its cached anchors, the tiered FP64-class
    values) must still decide as the FP64 replay does."""
    specs = [(f, 10, 16, 1) for f in range(7)]
    try:
        eng, tasks = make_engine(sgemtf, orc, specs, seed=21, precision=precision, flags=flags)
    except sgemtf.EngineError as e:
        pytest.skip(str(e))
    eng.reset()
    X0 = [eng.population(i)[0] for i in range(len(tasks))]
    gens = 600
    eng.run(gens)
    st = eng.stats()
    assert st["rechecks"] > 1000
    if flags & 0x40:
        assert st["recheck_differential"] == 0
    else:
        assert st["recheck_differential"] > 0
    want = replay(orc, oracle_params(orc, eng), tasks, X0, gens)
    for i in range(len(tasks)):
        got = eng.population(i)[0]
        assert np.array_equal(got, want[i]), (i, np.argwhere(got != want[i])[:5])
