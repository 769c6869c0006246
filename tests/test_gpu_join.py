"""Tasks joining a running handle (the reference admits batches of tasks into
a running service, proposed model/SG-EMTF.cu:1842-1912): emt_add_tasks on a
handle that has run keeps the running islands and the generation counter,
gives the new islands the initial populations a handle created with every
task draws, and from then on every island evolves as the oracle replays it
(SG-EMTF.cu:548-831 GA, SG-EMTF_DE.cu:474-706 DE, :1514-1591 transfer)."""
import numpy as np
import pytest

from gpu_util import make_engine, oracle_params

pytestmark = pytest.mark.gpu

FUSED_A = [(0, 20, 32, 1), (2, 12, 48, 1), (6, 30, 16, 1), (4, 8, 24, 1)]
FUSED_B = [(1, 16, 32, 1), (5, 10, 16, 1), (3, 50, 64, 1)]
LARGE_A = [(0, 150, 16, 1), (6, 129, 16, 1)]
LARGE_B = [(3, 200, 12, 1), (2, 40, 300, 1)]


def _oracle_epochs(orc, eng, tasks, gen, interval, epochs, rate, every=4):
    """Epochs of `interval` generations from generation `gen` on, each replayed
    by the oracle from the device's state (transfer import first when `gen` is
    a multiple of the transfer interval `every`)."""
    p = oracle_params(orc, eng)
    n = len(tasks)
    state = [eng.population(i) for i in range(n)]
    for _ in range(epochs):
        eng.run(interval)
        X = [s[0].copy() for s in state]
        f32 = [s[1].copy() for s in state]
        f64 = [np.full(t.NP, np.nan) for t in tasks]
        if rate > 0 and gen > 0 and gen % every == 0:
            elites = [state[i][0][np.argsort(orc.rank(state[i][1]))] for i in range(n)]
            for i, t in enumerate(tasks):
                q = orc.transfer_partner(p, i, n, gen)
                k = min(max(1, int(rate * t.NP + 0.5)), max(1, int(rate * tasks[q].NP + 0.5)))
                orc.transfer_in(p, t, tasks[q], elites[q][:k], X[i], f32[i], f64[i], gen, 0)
        for i, t in enumerate(tasks):
            for g in range(gen + 1, gen + interval + 1):
                orc.generation(p, t, X[i], f32[i], f64[i], g, 0)
        gen += interval
        state = [eng.population(i) for i in range(n)]
        for i in range(n):
            assert np.array_equal(state[i][0], X[i]), (gen, i)
    return gen


@pytest.mark.parametrize("layout", ["fused", "large"])
@pytest.mark.parametrize("alg", [0, 2])
def test_join_running_handle(sgemtf, orc, layout, alg):
    A, B = (FUSED_A, FUSED_B) if layout == "fused" else (LARGE_A, LARGE_B)
    kw = dict(algorithm=alg, transfer_interval=4, transfer_rate=0.25, transfer_mix=0.5)
    # every task from the start: the initial islands the joining tasks must get
    ref, tasks = make_engine(sgemtf, orc, A + B, seed=11, **kw)
    ref.reset()
    init = [ref.population(i) for i in range(len(A) + len(B))]
    run, _ = make_engine(sgemtf, orc, A, seed=11, **kw)
    run.reset()
    run.run(6)  # not a transfer boundary
    before = [run.population(i) for i in range(len(A))]
    ev = run.stats()["evaluations"]
    run.add_tasks([sgemtf.TaskDesc(f, D, NP, rotation=r) for f, D, NP, r in B])
    for i in range(len(A)):
        X, f = run.population(i)
        assert np.array_equal(X, before[i][0]) and np.array_equal(f, before[i][1]), i
    for i in range(len(A), len(A) + len(B)):
        Q, o = run.task_params(i)
        Qr, orr = ref.task_params(i)
        assert np.array_equal(Q, Qr) and np.array_equal(o, orr)
        X, f = run.population(i)
        assert np.array_equal(X, init[i][0]) and np.array_equal(f, init[i][1]), i
    st = run.stats()
    assert st["evaluations"] == ev + sum(b[2] for b in B)
    assert st["generations"] == 6 * len(A)
    # two generations to the next transfer boundary, then whole epochs
    gen = _oracle_epochs(orc, run, tasks, 6, 2, 1, 0.25)
    _oracle_epochs(orc, run, tasks, gen, 4, 3, 0.25)
    assert run.stats()["generations"] == 20 * len(A) + 14 * len(B)
    run.close()
    ref.close()


def test_join_at_transfer_boundary(sgemtf, orc):
    """At a boundary the running islands' elites were exported at the end of
    the last epoch; after the join every island's are exported again, the new
    ones from their initial members, and the next epoch imports them."""
    kw = dict(algorithm=0, transfer_interval=4, transfer_rate=0.25)
    _, tasks = make_engine(sgemtf, orc, FUSED_A + FUSED_B, seed=5, **kw)
    run, _ = make_engine(sgemtf, orc, FUSED_A, seed=5, **kw)
    run.run(8)
    run.add_tasks([sgemtf.TaskDesc(f, D, NP, rotation=r) for f, D, NP, r in FUSED_B])
    _oracle_epochs(orc, run, tasks, 8, 4, 3, 0.25)
    assert run.stats()["transfers_accepted"] > 0
    run.close()


def test_refused_join_keeps_running_islands(sgemtf, orc):
    """An explicit tensor-core form takes islands of <= 128 members; a joining
    island of 200 is refused and the handle runs on as if nothing happened."""
    try:
        a, _ = make_engine(sgemtf, orc, FUSED_A, seed=3, precision=sgemtf.ROT_TF32X3)
        a.run(5)
    except sgemtf.EngineError as e:
        pytest.skip(str(e))
    b, _ = make_engine(sgemtf, orc, FUSED_A, seed=3, precision=sgemtf.ROT_TF32X3)
    b.run(5)
    with pytest.raises(sgemtf.EngineError) as e:
        a.add_tasks([sgemtf.TaskDesc(0, 20, 200)])
    assert e.value.status == sgemtf.ERR_UNSUPPORTED
    assert a.stats()["n_tasks"] == len(FUSED_A)
    a.run(4)
    b.run(4)
    for i in range(len(FUSED_A)):
        assert np.array_equal(a.population(i)[0], b.population(i)[0]), i
    assert a.stats()["evaluations"] == b.stats()["evaluations"]
    a.close()
    b.close()
