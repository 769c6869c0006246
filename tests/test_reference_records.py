"""Statistical pin of the oracle against the reference's own recorded runs.

The fixture (tests/golden/reference_records_T100.json, made by
tests/golden/make_reference_records.py) holds, for 18 recorded GA runs of 100
tasks, the best and the 481st-best fitness of each task's initial population
of 512 members (data process/ANO_Tnum/data_record_T_ANO_100.txt).

The oracle in reference mode re-creates those populations' distribution: the
reference's diagonal instances z = M (x + b), M ~ U(0, 1], b ~ U(0, range]
(proposed model/SG-EMTF.cu:181-195), its box table (:197-214), its GA-file
function variants (Griewank without the product, :1029; the host-computed
Weierstrass offset, :354-361; E = 2.718282), 512 uniform members per task.
Per function, the median over tasks of each recorded statistic must match the
oracle's (100 simulated instances) within 3 standard deviations of the
difference of the two medians, estimated by bootstrap from the instance
spread: the reference recorded only 8-18 instances per function, all sharing
its seed-0 M and b across runs.  This pins Ackley, Weierstrass and Schwefel
to 1-7 % and the heavy-tailed functions more loosely; a wrong box (e.g. the
standard table instead of the reference's) moves every median by far more."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
# (best, 481st best) relative tolerances by reference type
TOL = {0: (0.28, 0.18), 1: (0.57, 0.33), 2: (0.01, 0.01), 3: (0.26, 0.17), 4: (0.29, 0.19),
       5: (0.06, 0.05), 6: (0.07, 0.03)}


@pytest.fixture(scope="module")
def records():
    with open(os.path.join(HERE, "golden", "reference_records_T100.json")) as f:
        d = json.load(f)
    return d["types"], np.array(d["runs"])


def test_fixture_layout(records):
    types, runs = records
    assert runs.shape == (18, 100, 3)
    assert types[:10] == [6, 4, 2, 5, 1, 3, 3, 2, 1, 3]  # glibc srand(0), rand() % 7
    # best-so-far never increases from generation 0 to 1000
    assert (runs[:, :, 1] <= runs[:, :, 0] + 1e-6 * np.abs(runs[:, :, 0])).all()


@pytest.mark.parametrize("ref_type", range(7))
def test_initial_population_statistics(orc, records, ref_type):
    types, runs = records
    fid = orc.lib().orc_function_from_reference(ref_type)
    lo, hi = orc.box(fid, True)
    flags = orc.FLAG_REF_GRIEWANK_NO_PRODUCT | orc.FLAG_REF_WEIERSTRASS_CONST | orc.FLAG_REF_ACKLEY_E
    idx = [i for i in range(100) if types[i] == ref_type]
    ref_best = np.median(runs[:, idx, 0])
    ref_481 = np.median(runs[:, idx, 2])
    rng = np.random.default_rng(1000 + ref_type)
    D = 50
    best, r481 = [], []
    for _ in range(100):
        M = (1.0 - rng.uniform(0, 1, D)).astype(np.float32)   # (0, 1]
        b = ((1.0 - rng.uniform(0, 1, D)) * (hi - lo)).astype(np.float32)
        t = orc.OTask(fid, D, 8, lo, hi, np.diag(M), -b, flags)
        X = rng.uniform(lo, hi, (512, D)).astype(np.float32)
        f = np.sort([t.eval64(x)[0] for x in X])
        best.append(f[0])
        r481.append(f[480])
    for got, want, tol in ((np.median(best), ref_best, TOL[ref_type][0]),
                           (np.median(r481), ref_481, TOL[ref_type][1])):
        assert abs(got / want - 1.0) <= tol, (ref_type, got, want)


def test_standard_boxes_do_not_fit(orc, records):
    """The same statistic with the standard Rastrigin box (+-5.12) instead of
    the reference's (+-50) misses the record by far: the check has power."""
    types, runs = records
    lo, hi = orc.box(orc.RASTRIGIN, False)
    assert (lo, hi) != orc.box(orc.RASTRIGIN, True)
    idx = [i for i in range(100) if types[i] == 3]
    rng = np.random.default_rng(5)
    best = []
    for _ in range(20):
        M = (1.0 - rng.uniform(0, 1, 50)).astype(np.float32)
        b = ((1.0 - rng.uniform(0, 1, 50)) * (hi - lo)).astype(np.float32)
        t = orc.OTask(orc.RASTRIGIN, 50, 8, lo, hi, np.diag(M), -b, 0)
        X = rng.uniform(lo, hi, (512, 50)).astype(np.float32)
        best.append(min(t.eval64(x)[0] for x in X))
    assert np.median(best) / np.median(runs[:, idx, 0]) < 0.2
