"""Statistical quality against the reference's own recorded runs: 30 seeded
runs of the reference's GA setting (sgemtf/quality.py: 100 tasks, D = 50,
512 members in 4 islands of 128) beside its 18 recorded runs of 100 tasks
(data process/ANO_Tnum/data_record_T_ANO_100.txt) and the ANO curve its tool
computed from them.

Which setting the recorded runs came from.  The GA file mutates every gene
(P = 1.f, proposed model/SG-EMTF.cu:555); its DE variant mutates each gene
with probability 1/DIMENSION (SG-EMTF_DE.cu:481).  With 1/D (RECORDED_GA)
the median best of every function type lands near the recorded one and the
ANO curve follows the recorded curve within 0.01; with every gene mutated
(SHIPPED_GA) Schwefel ends ~5x and Weierstrass ~2.3x above the record.
So the recorded runs used the 1/D mutation probability.

Stated tolerances (measured; 30 seeds):
  - RECORDED_GA, median best at generation 1000 per reference type, ours
    over the reference's: at most 2 for every type (measured 0.88-1.17 for
    six types).  Schwefel ends better than the record: 0.48 on this instance
    draw, 0.44-1.04 over three draws (8 of the 100 tasks are Schwefel, so
    their instances move its median), hence a lower bound of 0.35.  The
    other types stay within [0.5, 2];
  - RECORDED_GA, ANO: within 0.03 absolute at every recording point
    (measured 0.009);
  - SHIPPED_GA: Schwefel above 3 and Weierstrass above 2 (measured about
    5.3 and 2.3): the shipped probability does not give the recorded runs."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
WEIERSTRASS, SCHWEFEL = 5, 6  # reference types
LOWER = {t: (0.35 if t == SCHWEFEL else 0.5) for t in range(7)}
UPPER = {t: 2.0 for t in range(7)}


def _reference():
    with open(os.path.join(HERE, "golden", "reference_records_T100.json")) as f:
        d = json.load(f)
    with open(os.path.join(HERE, "golden", "reference_ano_T100.json")) as f:
        ano = np.array([float(v) for v in json.load(f)["ano"]])
    return np.array(d["runs"]), np.array(d["types"]), ano


def _ratios(types, summary, runs, rtypes):
    assert list(types) == list(rtypes)
    return {rt: v["median"] / float(np.median(runs[:, rtypes == rt, 1]))
            for rt, v in summary["per_type"].items()}


@pytest.fixture(scope="module")
def recorded(sgemtf):
    from sgemtf import quality
    types, rec = quality.run(seeds=30, operators=quality.RECORDED_GA)
    return types, rec, quality.summarise(types, rec)


def test_ano_tracks_the_reference(recorded):
    _, _, ref = _reference()
    ano = np.array(recorded[2]["ano"])
    assert ano.shape == ref.shape == (21,)
    assert np.abs(ano - ref).max() <= 0.03
    assert (np.diff(ano) <= 1e-6).all()  # normalised progress never reverses


def test_final_medians_by_type(recorded):
    runs, rtypes, _ = _reference()
    types, _, s = recorded
    for rt, ratio in _ratios(types, s, runs, rtypes).items():
        assert LOWER[rt] <= ratio <= UPPER[rt], (rt, ratio)


def test_records_are_best_so_far(recorded):
    _, rec, _ = recorded
    best = rec[:, :, :-1]
    # no transfer: a task's recorded best never rises beyond the FP32 error
    # (migration moves members between a task's own islands only)
    assert (np.diff(best, axis=2) <= 1e-5 * np.abs(best[:, :, 1:]) + 2e-2).all()
    assert (rec[:, :, -1] >= rec[:, :, 0]).all()  # near-worst >= best at generation 0


def test_shipped_mutation_probability_misses_the_record(sgemtf):
    from sgemtf import quality
    runs, rtypes, _ = _reference()
    types, rec = quality.run(seeds=30, operators=quality.SHIPPED_GA)
    r = _ratios(types, quality.summarise(types, rec), runs, rtypes)
    assert r[SCHWEFEL] > 3.0 and r[WEIERSTRASS] > 2.0, r
