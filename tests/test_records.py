"""Run records and the average normalised objective (host code of the
library, no GPU).

emt_ano restates the reference's analysis tool (data process/源.cpp:172-203).
It is pinned by the reference's own output: the tool's ANO curve for 100
tasks (data process/ANO_Tnum/data_record_T_ANO_100_1677482963.txt), which it
computed from the 18 recorded runs of data_record_T_ANO_100.txt; both are
committed fixtures (tests/golden/make_reference_records.py)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def trajectories():
    return np.load(os.path.join(HERE, "golden", "reference_trajectories_T100.npy"))


def _ano_restatement(R):
    """numpy restatement of the tool: per task min over runs of the last
    recording point, max over runs of the near-worst column."""
    runs, tasks, cols = R.shape
    P = cols - 1
    mn = R[:, :, P - 1].min(0)
    mx = R[:, :, P].max(0)
    span = mx - mn
    ok = (span != 0)[None, :, None]
    norm = np.where(ok, (R[:, :, :P] - mn[None, :, None]) /
                    np.where(span != 0, span, 1)[None, :, None], 0.0)
    return norm.sum(axis=(0, 1)) / (runs * tasks)


def test_ano_reproduces_the_reference_tool(sgemtf, trajectories):
    with open(os.path.join(HERE, "golden", "reference_ano_T100.json")) as f:
        want = json.load(f)["ano"]
    got = sgemtf.ano(trajectories)
    assert trajectories.shape == (18, 100, 22)
    assert len(got) == len(want) == 21
    # printed the way the tool printed it (6 significant digits)
    assert ["%g" % v for v in got] == want


def test_ano_matches_restatement(sgemtf, trajectories):
    got = sgemtf.ano(trajectories)
    ref = _ano_restatement(trajectories.astype(np.float64))
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-7)
    # degenerate tasks (max == min) contribute zero
    flat = np.ones((2, 3, 5), np.float32)
    assert np.array_equal(sgemtf.ano(flat), np.zeros(4, np.float32))


def test_ano_arguments(sgemtf):
    with pytest.raises(sgemtf.EngineError):
        sgemtf.ano(np.zeros((1, 1, 1), np.float32))


def _read_runs(path):
    """The tool's reader (data process/源.cpp:127-149): rows of numbers, runs
    separated by blank lines."""
    runs, cur = [], []
    for line in open(path):
        if not line.strip():
            if cur:
                runs.append(cur)
                cur = []
            continue
        cur.append([float(v) for v in line.split()])
    if cur:
        runs.append(cur)
    return np.array(runs, np.float32)


def test_write_record_round_trip(sgemtf, tmp_path, trajectories):
    path = tmp_path / "data_record.txt"
    for r in trajectories[:3]:
        sgemtf.write_record(path, r)
    back = _read_runs(path)
    assert back.shape == (3, 100, 22)
    # 6 significant digits, the precision the reference wrote them with
    assert np.allclose(back, trajectories[:3], rtol=1e-5)
    text = open(path).read()
    assert text.endswith("\n\n") and text.count("\n\n") == 3
    assert np.allclose(sgemtf.ano(back), sgemtf.ano(trajectories[:3]), rtol=1e-4)
