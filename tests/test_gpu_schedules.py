"""Launch schedules for islands of uneven shape (config 3): one launch over
all islands, occupancy buckets on side streams, one launch per island, each
with and without CUDA-graph replay of the epoch sequence.  The schedule only
changes where and when CTAs run, so populations must be bit-identical to the
single launch and to the oracle replay."""
import numpy as np
import pytest

from gpu_util import make_engine, oracle_params

pytestmark = pytest.mark.gpu

# D, NP pairs from config 3's classes plus odd sizes; (100, 128) needs most of
# an SM's shared memory, the small ones fit three per SM
SHAPES = [(10, 32), (30, 64), (50, 128), (100, 128), (100, 32), (10, 128), (3, 8), (64, 64)]


def specs(n=24):
    return [(t % 7, SHAPES[t % len(SHAPES)][0], SHAPES[t % len(SHAPES)][1], 1) for t in range(n)]


def islands(eng, n):
    return [eng.population(i)[0] for i in range(n)]


def run_with(sgemtf, orc, schedule, graph, gens_list, interval=5):
    eng, _ = make_engine(sgemtf, orc, specs(), seed=13, schedule=schedule, use_graph=graph,
                         transfer_interval=interval)
    eng.reset()
    for g in gens_list:
        eng.run(g)
    out = islands(eng, 24), eng.stats()
    eng.close()
    return out


@pytest.mark.parametrize("schedule,graph", [(2, 0), (3, 0), (4, 0), (1, 1), (2, 1), (3, 1), (4, 1)])
def test_schedules_bit_identical(sgemtf, orc, schedule, graph):
    gens = [3, 7, 5, 5, 1]  # epochs that start and end off the transfer boundaries
    ref, st_ref = run_with(sgemtf, orc, 1, 0, gens)
    got, st = run_with(sgemtf, orc, schedule, graph, gens)
    for i, (a, b) in enumerate(zip(ref, got)):
        assert np.array_equal(a, b), (schedule, graph, i)
    assert st["transfers_accepted"] == st_ref["transfers_accepted"]
    assert st["evaluations"] == st_ref["evaluations"]


def test_buckets_match_oracle(sgemtf, orc):
    from test_gpu_replay import replay
    eng, tasks = make_engine(sgemtf, orc, specs(14), seed=4, schedule=2, use_graph=1)
    eng.reset()
    X0 = islands(eng, 14)
    eng.run(9)
    want = replay(orc, oracle_params(orc, eng), tasks, X0, 9)
    for i, w in enumerate(want):
        assert np.array_equal(eng.population(i)[0], w), i
    eng.close()


def test_graph_replayed_across_calls(sgemtf, orc):
    # the same plan recurs (no transfer, equal calls): one capture, replays
    eng, _ = make_engine(sgemtf, orc, specs(), seed=3, schedule=2, use_graph=1)
    eng.reset()
    for _ in range(4):
        eng.run(6)
    a = islands(eng, 24)
    eng.close()
    eng, _ = make_engine(sgemtf, orc, specs(), seed=3, schedule=1)
    eng.reset()
    eng.run(24)
    b = islands(eng, 24)
    eng.close()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_tune_keeps_results(sgemtf, orc):
    eng, _ = make_engine(sgemtf, orc, specs(), seed=8, transfer_interval=4)
    eng.reset()
    chosen = eng.tune(4)
    assert chosen & 0xFF in (1, 2)
    eng.run(6)
    a = islands(eng, 24)
    total = eng.stats()["generations"] // 24  # the tuner's candidates ran real generations
    eng.close()
    assert total >= 4 * 2 + 6
    eng, _ = make_engine(sgemtf, orc, specs(), seed=8, transfer_interval=4, schedule=1)
    eng.reset()
    eng.run(total)
    b = islands(eng, 24)
    eng.close()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_rejects_bad_schedule(sgemtf):
    with pytest.raises(sgemtf.EngineError):
        sgemtf.Engine(sgemtf.Config(schedule=5))
    with pytest.raises(sgemtf.EngineError):
        sgemtf.Engine(sgemtf.Config(use_graph=2))
