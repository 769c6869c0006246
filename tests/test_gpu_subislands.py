"""Sub-islands and ring migration on the device (IslandMigration,
proposed model/SG-EMTF.cu:1138-1218) against the oracle.

Migration runs before the trials of generation g when (g - 1) is a multiple
of the interval, so with epochs of exactly `interval` generations it opens
each epoch: the oracle starts from the device's own state (its FP32 fitness
fixes the ranking), migrates, then runs the epoch's generations in FP64.
"""
import numpy as np
import pytest

from gpu_util import make_engine, oracle_params

pytestmark = pytest.mark.gpu

SPECS = [(0, 20, 32, 1), (1, 20, 32, 1), (2, 12, 48, 1), (6, 20, 16, 1), (4, 8, 24, 1),
         (3, 50, 64, 1), (5, 30, 32, 1)]


def _replay(sgemtf, orc, specs, S, interval, epochs, transfer=False, **cfg):
    kw = dict(subislands=S, migration_interval=interval, **cfg)
    if transfer:
        kw.update(transfer_interval=interval, transfer_rate=0.25, transfer_mix=0.5)
    eng, tasks = make_engine(sgemtf, orc, specs, seed=41, **kw)
    p = oracle_params(orc, eng)
    eng.reset()
    n = len(tasks)
    state = [eng.population(i) for i in range(n)]
    gen, migrated, transferred = 0, 0, 0
    for epoch in range(epochs):
        eng.run(interval)
        X = [s[0].copy() for s in state]
        f32 = [s[1].copy() for s in state]
        f64 = [np.full(t.NP, np.nan) for t in tasks]
        if transfer and gen > 0:
            elites = [state[i][0][np.argsort(orc.rank(state[i][1]))] for i in range(n)]
            for i, t in enumerate(tasks):
                q = orc.transfer_partner(p, i, n, gen)
                k = min(max(1, int(0.25 * t.NP + 0.5)), max(1, int(0.25 * tasks[q].NP + 0.5)))
                transferred += orc.transfer_in(p, t, tasks[q], elites[q][:k], X[i], f32[i],
                                               f64[i], gen, 0)
        for i, t in enumerate(tasks):
            for g in range(gen + 1, gen + interval + 1):
                if orc.migration_due(p, g):
                    migrated += orc.migrate(p, t, X[i], f32[i], f64[i], 0)
                orc.generation(p, t, X[i], f32[i], f64[i], g, 0)
        gen += interval
        state = [eng.population(i) for i in range(n)]
        for i in range(n):
            assert np.array_equal(state[i][0], X[i]), (epoch, i)
    st = eng.stats()
    assert st["migrations_accepted"] == migrated
    if transfer:
        assert st["transfers_accepted"] == transferred
    return migrated


@pytest.mark.parametrize("alg", [0, 2])
@pytest.mark.parametrize("S", [2, 4])
def test_migration_epochs_bit_exact(sgemtf, orc, alg, S):
    migrated = _replay(sgemtf, orc, SPECS, S, 4, 5, algorithm=alg)
    assert migrated > 0


@pytest.mark.parametrize("alg", [0, 2])
def test_migration_with_transfer_tc(sgemtf, orc, alg):
    """Transfer import, then migration, then the trials, on the tensor-core
    form (islands of <= 128 members)."""
    specs = [s for s in SPECS if s[2] <= 128]
    _replay(sgemtf, orc, specs, 2, 3, 5, transfer=True, algorithm=alg,
            precision=sgemtf.ROT_TF32X3, migration_count=3)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("alg", [0, 2])
def test_migration_large_islands(sgemtf, orc, precision, alg):
    """The HBM-resident pipeline (any D > 128 in the handle): sub-island
    draws in its trial kernel, migration through its selection pipeline."""
    specs = [(0, 150, 32, 1), (4, 200, 32, 1), (6, 129, 16, 1), (2, 10, 24, 1)]
    try:
        migrated = _replay(sgemtf, orc, specs, 2, 3, 4, algorithm=alg, precision=precision,
                           migration_count=3)
    except sgemtf.EngineError as e:
        pytest.skip(str(e))
    assert migrated > 0


def test_migration_np512_sixteen_subislands(sgemtf, orc):
    """The reference's layout: 512 members per task in sub-islands of 32
    (SG-EMTF.cu:29-31, 856-896), migration every few generations, on the
    HBM-resident pipeline that islands of more than 256 members take."""
    specs = [(6, 50, 512, 1), (0, 30, 512, 1), (3, 20, 64, 1)]
    migrated = _replay(sgemtf, orc, specs, 16, 3, 3, algorithm=2, eta_c=2.0, p_c=1.0,
                       eta_m=5.0, p_m=1.0, migration_count=2)
    assert migrated > 0


def test_migration_inside_long_epochs(sgemtf, orc):
    """One run of many generations migrates at every interval inside the
    kernel; the same run cut into interval-long epochs gives the same state."""
    specs = SPECS[:4]
    a, _ = make_engine(sgemtf, orc, specs, seed=7, subislands=2, migration_interval=3)
    b, _ = make_engine(sgemtf, orc, specs, seed=7, subislands=2, migration_interval=3)
    a.run(24)
    for _ in range(8):
        b.run(3)
    for i in range(len(specs)):
        assert np.array_equal(a.population(i)[0], b.population(i)[0])
    assert a.stats()["migrations_accepted"] == b.stats()["migrations_accepted"] > 0


def test_one_subisland_changes_nothing(sgemtf, orc):
    specs = SPECS[:4]
    a, _ = make_engine(sgemtf, orc, specs, seed=9)
    b, _ = make_engine(sgemtf, orc, specs, seed=9, subislands=1, migration_interval=2,
                       migration_count=3)
    a.run(10)
    b.run(10)
    for i in range(len(specs)):
        assert np.array_equal(a.population(i)[0], b.population(i)[0])
    assert b.stats()["migrations_accepted"] == 0


def test_subisland_arguments(sgemtf):
    eng = sgemtf.Engine(sgemtf.Config(seed=1, subislands=4))
    for bad in [dict(function=0, dim=4, pop=18), dict(function=0, dim=4, pop=12)]:
        with pytest.raises(sgemtf.EngineError) as e:
            eng.add_tasks([sgemtf.TaskDesc(**bad)])
        assert e.value.status == sgemtf.ERR_INVALID_ARG
    eng.add_tasks([sgemtf.TaskDesc(0, 200, 32)])  # large islands split too
    eng2 = sgemtf.Engine(sgemtf.Config(seed=1, subislands=2, migration_count=5))
    with pytest.raises(sgemtf.EngineError) as e:
        eng2.add_tasks([sgemtf.TaskDesc(0, 4, 16)])
    assert e.value.status == sgemtf.ERR_INVALID_ARG
    with pytest.raises(sgemtf.EngineError):
        sgemtf.Engine(sgemtf.Config(seed=1, subislands=-1))
