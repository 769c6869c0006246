"""Parity at the workloads' own sizes and full lengths: the device's
populations against the oracle replaying the same Philox stream with every
selection decided in FP64 (proposed model/SG-EMTF_DE.cu:474-706 for DE,
SG-EMTF.cu:548-831 for the GA, :1514-1591 for elite transfer).

- 1000 rotated tasks of D = 50, NP = 64, DE/rand/1/bin F 0.5 CR 0.9, all 2000
  generations, in the three rotation forms (FP32, TF32X3, BF16X3): 14 of the
  tasks (two per function) replayed from their initial populations, and the
  forms' final populations identical for all 1000 tasks.  Converged islands spend their
  late generations on near ties, which is where a wrong re-check would show.
- 8 tasks of D = 50, NP = 100, identity rotation, transfer of 10 % every 10
  generations, all 1000 generations, epoch by epoch from the device's state
  (transfer ranks members by the device's FP32 fitness).
- 2 tasks of D = 1000, NP = 256, GA (SBX eta 15 p_c 0.9, PM eta 15 p_m 1/D),
  transfer every 20, 40 generations (one transfer crossed), both forms."""
import hashlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from gpu_util import make_engine, oracle_params

pytestmark = pytest.mark.gpu

CONFIG2_TASKS, CONFIG2_GENS = 1000, 2000
# two tasks per function: the first seven and the last seven of the 1000
CONFIG2_CHECKED = list(range(7)) + list(range(CONFIG2_TASKS - 7, CONFIG2_TASKS))


def _hash_populations(eng, n):
    """SHA-256 over every task's population (the forms' FP32 fitness values
    differ by their rounding; the populations must not)."""
    h = hashlib.sha256()
    for i in range(n):
        h.update(eng.population(i)[0].tobytes())
    return h.hexdigest()


def test_config2_full_length_both_forms(sgemtf, orc):
    descs = [sgemtf.TaskDesc(t % 7, 50, 64, rotation=sgemtf.ROTATION_SEEDED_QR)
             for t in range(CONFIG2_TASKS)]
    digests, finals = {}, {}
    X0 = None
    forms = (sgemtf.ROT_FP32, sgemtf.ROT_TF32X3, sgemtf.ROT_BF16X3)
    for prec in forms:
        eng = sgemtf.Engine(sgemtf.Config(seed=1, precision=prec))
        eng.add_tasks(descs)
        eng.reset()
        if X0 is None:
            X0 = {t: eng.population(t)[0] for t in CONFIG2_CHECKED}
            tasks = []
            for t in CONFIG2_CHECKED:
                Q, o = eng.task_params(t)
                lo, hi = sgemtf.function_box(t % 7)
                tasks.append(orc.OTask(t % 7, 50, 64, lo, hi, Q, o, 0, t))
            p = oracle_params(orc, eng)
        eng.run(CONFIG2_GENS)
        st = eng.stats()
        assert st["precision_used"] == prec
        assert st["rechecks"] > 1_000_000  # the late generations are near-tie bound
        digests[prec] = _hash_populations(eng, CONFIG2_TASKS)
        finals[prec] = {t: eng.population(t)[0] for t in CONFIG2_CHECKED}
        eng.close()
    assert len(set(digests.values())) == 1, digests
    # the oracle: FP64 decisions for every selection, one native thread per task
    X = [X0[t].copy() for t in CONFIG2_CHECKED]
    f64 = [np.array([tk.eval64(r)[0] for r in x]) for tk, x in zip(tasks, X)]
    f32 = [v.astype(np.float32) for v in f64]
    orc.run_threads(p, tasks, X, f32, f64, 0, CONFIG2_GENS, 0, len(tasks))
    for k, t in enumerate(CONFIG2_CHECKED):
        for prec in forms:
            got = finals[prec][t]
            assert np.array_equal(got, X[k]), (prec, t, np.argwhere(got != X[k])[:5])


def _epochs_against_oracle(orc, eng, tasks, interval, rate, gens, threads):
    """Runs `gens` generations epoch by epoch; each epoch the oracle starts
    from the device's state (import of the partners' top-k when due, then
    the epoch's generations in FP64) and must end on the device's state."""
    p = oracle_params(orc, eng)
    n = len(tasks)
    state = [eng.population(i) for i in range(n)]
    gen, replaced = 0, 0
    pool = ThreadPoolExecutor(threads)
    while gen < gens:
        eng.run(interval)
        X = [s[0].copy() for s in state]
        f32 = [s[1].copy() for s in state]
        f64 = [np.full(t.NP, np.nan) for t in tasks]
        if gen > 0:
            elites = [state[i][0][np.argsort(orc.rank(state[i][1]))] for i in range(n)]
            for i, t in enumerate(tasks):
                q = orc.transfer_partner(p, i, n, gen)
                k = min(max(1, int(rate * t.NP + 0.5)), max(1, int(rate * tasks[q].NP + 0.5)))
                replaced += orc.transfer_in(p, t, tasks[q], elites[q][:k], X[i], f32[i], f64[i],
                                            gen, 0)

        def work(i, g0=gen):
            for g in range(g0 + 1, g0 + interval + 1):
                orc.generation(p, tasks[i], X[i], f32[i], f64[i], g, 0)

        list(pool.map(work, range(n)))
        gen += interval
        state = [eng.population(i) for i in range(n)]
        for i in range(n):
            assert np.array_equal(state[i][0], X[i]), (gen, i)
    pool.shutdown()
    return replaced


def test_config1_full_length_with_transfer(sgemtf, orc):
    fids = [0, 1, 2, 3, 4, 5, 6, 0]
    specs = [(f, 50, 100, sgemtf.ROTATION_IDENTITY) for f in fids]
    eng, tasks = make_engine(sgemtf, orc, specs, seed=1, transfer_interval=10, transfer_rate=0.1)
    eng.reset()
    replaced = _epochs_against_oracle(orc, eng, tasks, 10, 0.1, 1000, 8)
    assert eng.stats()["transfers_accepted"] == replaced
    assert replaced > 0
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_config4_two_tasks_across_a_transfer(sgemtf, orc, precision):
    specs = [(sgemtf.GRIEWANK, 1000, 256, 1), (sgemtf.WEIERSTRASS, 1000, 256, 1)]
    try:
        eng, tasks = make_engine(sgemtf, orc, specs, seed=1, precision=precision, algorithm=2,
                                 eta_c=15.0, p_c=0.9, eta_m=15.0, p_m=-1.0,
                                 transfer_interval=20, transfer_rate=0.1)
    except sgemtf.EngineError as e:
        pytest.skip(str(e))
    eng.reset()
    _epochs_against_oracle(orc, eng, tasks, 20, 0.1, 40, 2)
    assert eng.stats()["rechecks"] > 0
    eng.close()
