"""Run records and the reference's output files through a live engine:
emt_record_run (SG-EMTF_DE.cu:1575-1632), output_0.txt (SG-EMTF.cu:1971-1983)
and para.txt (SG-EMTF.cu:244-264)."""
import numpy as np
import pytest

from gpu_util import make_engine

pytestmark = pytest.mark.gpu


def test_record_run_matches_stepwise_run(sgemtf, orc):
    specs = [(f, 12, 40, 1) for f in range(7)]
    a, _ = make_engine(sgemtf, orc, specs, seed=3)
    b, _ = make_engine(sgemtf, orc, specs, seed=3)
    a.reset()
    b.reset()
    pops = [b.population(i)[1] for i in range(7)]
    rec = a.record_run(100, 20)
    assert rec.shape == (7, 7)
    want = [b.best_all()]
    for _ in range(5):
        b.run(20)
        want.append(b.best_all())
    assert np.array_equal(rec[:, :6], np.array(want).T)
    # the near-worst: rank 32 * ((NP - 1) / 32) = 32 of the population on entry
    assert np.array_equal(rec[:, 6], [np.sort(p)[32] for p in pops])
    # a best-so-far never increases without transfer (FP64 decides the
    # selections, so the FP32 best may move within its stated error)
    assert (np.diff(rec[:, :6], axis=1) <= 1e-5 * np.abs(rec[:, 1:6]) + 5e-3).all()
    for i in range(7):
        assert np.array_equal(a.population(i)[0], b.population(i)[0])


def test_record_run_arguments(sgemtf, orc):
    eng, _ = make_engine(sgemtf, orc, [(0, 4, 8, 1)], seed=1)
    eng.reset()
    for g, k in [(10, 3), (10, 0), (-5, 5)]:
        with pytest.raises(sgemtf.EngineError) as e:
            eng.record_run(g, k)
        assert e.value.status == sgemtf.ERR_INVALID_ARG


def test_write_fitness_is_sorted_population(sgemtf, orc, tmp_path):
    specs = [(f, 10, 16 + 8 * f, 1) for f in range(4)]
    eng, _ = make_engine(sgemtf, orc, specs, seed=2)
    eng.run(15)
    path = tmp_path / "output_0.txt"
    eng.write_fitness(path)
    eng.write_fitness(path)  # appends, one blank line per call
    lines = open(path).read().split("\n")
    rows = [ln for ln in lines if ln.strip()]
    assert len(rows) == 8 and lines.count("") == 3
    for i in range(4):
        got = np.array([float(v) for v in rows[i].split()], np.float32)
        want = np.sort(eng.population(i)[1])
        assert got.shape == want.shape
        assert np.allclose(got, want, rtol=1e-5, atol=0)


def test_write_para_diagonal_instances(sgemtf, orc, tmp_path):
    rng = np.random.default_rng(4)
    D = 6
    descs, Ms, bs = [], [], []
    for ref_type in (6, 4, 2):
        fid = sgemtf.lib().emt_function_from_reference(ref_type)
        M = (1.0 - rng.uniform(0, 1, D)).astype(np.float32)
        b = rng.uniform(0.5, 10, D).astype(np.float32)
        descs.append(sgemtf.TaskDesc(fid, D, 8, rotation=sgemtf.ROTATION_DIAG, diag=M, shift=-b))
        Ms.append(M)
        bs.append(b)
    eng = sgemtf.Engine(sgemtf.Config(seed=1))
    eng.add_tasks(descs)
    path = tmp_path / "para.txt"
    eng.write_para(path)
    lines = open(path).read().split("\n")
    assert lines[3] == "" and lines[4].split() == ["6", "4", "2"]
    for t in range(3):
        v = np.array([float(x) for x in lines[t].split()], np.float32).reshape(D, 2)
        assert np.allclose(v[:, 0], Ms[t], rtol=1e-5) and np.allclose(v[:, 1], bs[t], rtol=1e-5)
    qr = sgemtf.Engine(sgemtf.Config(seed=1))
    qr.add_tasks([sgemtf.TaskDesc(0, D, 8, rotation=sgemtf.ROTATION_SEEDED_QR)])
    with pytest.raises(sgemtf.EngineError) as e:
        qr.write_para(tmp_path / "p2.txt")
    assert e.value.status == sgemtf.ERR_UNSUPPORTED
