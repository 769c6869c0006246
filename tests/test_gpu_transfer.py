"""Elite transfer (knowledgeTransfer, proposed model/SG-EMTF.cu:1514-1591):
epoch by epoch, the device against the oracle started from the device's own
state, so that ranking by FP32 fitness uses the same values on both sides."""
import numpy as np
import pytest

from gpu_util import make_engine, oracle_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("alg", [0, 2])
def test_transfer_epochs_bit_exact(sgemtf, orc, alg):
    specs = [(0, 20, 20, 1), (1, 20, 20, 1), (2, 12, 30, 1), (6, 20, 16, 1), (4, 8, 10, 1)]
    interval = 4
    eng, tasks = make_engine(sgemtf, orc, specs, seed=31, algorithm=alg,
                             transfer_interval=interval, transfer_rate=0.25, transfer_mix=0.5)
    p = oracle_params(orc, eng)
    eng.reset()
    n = len(tasks)
    state = [eng.population(i) for i in range(n)]
    gen = 0
    replaced_total = 0
    for epoch in range(4):
        eng.run(interval)
        # oracle: import (if not the first epoch) from the partner's top-k of
        # the previous state, then `interval` generations, all in FP64.
        X = [s[0].copy() for s in state]
        f32 = [s[1].copy() for s in state]
        f64 = [np.full(t.NP, np.nan) for t in tasks]
        if gen > 0:
            elites = []
            for i, t in enumerate(tasks):
                r = orc.rank(state[i][1])
                order = np.argsort(r)
                elites.append(state[i][0][order])
            for i, t in enumerate(tasks):
                q = orc.transfer_partner(p, i, n, gen)
                k = min(max(1, int(0.25 * t.NP + 0.5)), max(1, int(0.25 * tasks[q].NP + 0.5)))
                replaced_total += orc.transfer_in(p, t, tasks[q], elites[q][:k], X[i], f32[i],
                                                  f64[i], gen, 0)
        for i, t in enumerate(tasks):
            for g in range(gen + 1, gen + interval + 1):
                orc.generation(p, t, X[i], f32[i], f64[i], g, 0)
        gen += interval
        state = [eng.population(i) for i in range(n)]
        for i in range(n):
            assert np.array_equal(state[i][0], X[i]), (epoch, i)
    assert eng.stats()["transfers_accepted"] == replaced_total


def test_config1_with_transfer(sgemtf, orc):
    """8 tasks, NP 100, D 50, identity rotation (sphere..weierstrass, sphere),
    DE/rand/1/bin F 0.5 CR 0.9, 10 % of the island every 10 generations."""
    fids = [0, 1, 2, 3, 4, 5, 6, 0]
    specs = [(f, 50, 100, 0) for f in fids]
    interval, rate = 10, 0.1
    eng, tasks = make_engine(sgemtf, orc, specs, seed=23, transfer_interval=interval,
                             transfer_rate=rate)
    p = oracle_params(orc, eng)
    eng.reset()
    n = len(tasks)
    state = [eng.population(i) for i in range(n)]
    gen, replaced = 0, 0
    for epoch in range(3):
        eng.run(interval)
        X = [s[0].copy() for s in state]
        f32 = [s[1].copy() for s in state]
        f64 = [np.full(t.NP, np.nan) for t in tasks]
        if gen > 0:
            elites = [state[i][0][np.argsort(orc.rank(state[i][1]))] for i in range(n)]
            for i, t in enumerate(tasks):
                q = orc.transfer_partner(p, i, n, gen)
                k = max(1, int(rate * t.NP + 0.5))
                replaced += orc.transfer_in(p, t, tasks[q], elites[q][:k], X[i], f32[i], f64[i],
                                            gen, 0)
        for i, t in enumerate(tasks):
            for g in range(gen + 1, gen + interval + 1):
                orc.generation(p, t, X[i], f32[i], f64[i], g, 0)
        gen += interval
        state = [eng.population(i) for i in range(n)]
        for i in range(n):
            assert np.array_equal(state[i][0], X[i]), (epoch, i)
    assert eng.stats()["transfers_accepted"] == replaced
