"""Service mode (emt_service_*): batches of tasks arriving over time, served
concurrently, as the reference's host scheduler serves them
(proposed model/SG-EMTF.cu:1836-1958)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(sgemtf, first, n, D=20, NP=32):
    return [sgemtf.TaskDesc((first + t) % 7, D, NP) for t in range(n)]


def test_batches_equal_standalone_handles(sgemtf):
    gens, epoch = 60, 25
    cfg = sgemtf.Config(seed=11, transfer_interval=20, transfer_rate=0.2)
    svc = sgemtf.Service(cfg, generations=gens, epoch=epoch)
    batches = [_batch(sgemtf, 0, 5), _batch(sgemtf, 3, 9), _batch(sgemtf, 1, 3, D=50, NP=64)]
    ids = [svc.submit(b, arrival_ms=20.0 * i) for i, b in enumerate(batches)]
    info, best = svc.batch(ids[2])
    assert best is None and info["state"] in (0, 1)
    svc.drain()
    evals = 0
    for i, b in zip(ids, batches):
        info, best = svc.batch(i)
        assert info["state"] == 2 and info["generations"] == gens
        assert info["arrival_ms"] <= info["admit_ms"] <= info["done_ms"]
        solo = sgemtf.Engine(sgemtf.Config(seed=11 + i, transfer_interval=20, transfer_rate=0.2))
        solo.add_tasks(b)
        solo.run(gens)
        assert np.array_equal(best, solo.best_all()), i
        evals += solo.stats()["evaluations"]  # generations and transfer candidates
    st = svc.stats()
    assert st["batches_submitted"] == st["batches_done"] == 3
    assert st["tasks_done"] == 17
    assert 0.0 <= st["mean_response_ms"] <= st["mean_solve_ms"]
    assert st["evaluations"] == evals
    assert st["max_device_mem_mb"] >= st["mean_device_mem_mb"] > 0.0
    svc.close()


def test_batches_overlap_on_the_device(sgemtf):
    """Two batches admitted together are both running before either is done."""
    svc = sgemtf.Service(sgemtf.Config(seed=3), generations=200, epoch=10)
    a = svc.submit(_batch(sgemtf, 0, 40))
    b = svc.submit(_batch(sgemtf, 2, 40))
    svc.step()
    ia, _ = svc.batch(a)
    ib, _ = svc.batch(b)
    assert ia["state"] == 1 and ib["state"] == 1
    svc.drain()
    assert svc.batch(a)[0]["state"] == 2 and svc.batch(b)[0]["state"] == 2


def test_service_arguments(sgemtf):
    svc = sgemtf.Service(sgemtf.Config(seed=1), generations=10, epoch=5)
    with pytest.raises(sgemtf.EngineError) as e:
        svc.submit([sgemtf.TaskDesc(0, 200, 16)])
    assert e.value.status == sgemtf.ERR_INVALID_ARG
    with pytest.raises(sgemtf.EngineError) as e:
        svc.submit([])
    assert e.value.status == sgemtf.ERR_INVALID_ARG
    with pytest.raises(sgemtf.EngineError):
        sgemtf.Service(sgemtf.Config(seed=1), generations=10, epoch=0)
    with pytest.raises(sgemtf.EngineError):
        svc.batch(7)


def test_failed_batch_is_released_and_skipped(sgemtf):
    """A batch that cannot be admitted (here a bad function id, caught by
    emt_add_tasks) fails once: the round that met it returns the error, the
    batch is marked failed, and the remaining batches are served."""
    svc = sgemtf.Service(sgemtf.Config(seed=5), generations=20, epoch=10)
    bad = svc.submit([sgemtf.TaskDesc(99, 10, 16)])
    good = svc.submit(_batch(sgemtf, 0, 3))
    with pytest.raises(sgemtf.EngineError) as e:
        svc.drain()
    assert e.value.status == sgemtf.ERR_INVALID_ARG
    info, best = svc.batch(bad)
    assert info["state"] == 3 and best is None
    svc.drain()
    info, best = svc.batch(good)
    assert info["state"] == 2 and best.shape == (3,)
    st = svc.stats()
    assert st["batches_submitted"] == 2 and st["batches_done"] == 1 and st["tasks_done"] == 3
    svc.close()


def test_unsupported_batch_is_released_and_skipped(sgemtf):
    """Admission also rejects a batch the configured form cannot hold (a
    tensor-core handle with islands of NP > 128): EMT_ERR_UNSUPPORTED, the
    batch fails alone and the next one is served."""
    svc = sgemtf.Service(sgemtf.Config(seed=6, precision=sgemtf.ROT_BF16X3), generations=20,
                         epoch=10)
    bad = svc.submit([sgemtf.TaskDesc(0, 50, 200)])
    good = svc.submit(_batch(sgemtf, 0, 3))
    with pytest.raises(sgemtf.EngineError) as e:
        svc.drain()
    assert e.value.status == sgemtf.ERR_UNSUPPORTED
    assert svc.batch(bad)[0]["state"] == 3
    svc.drain()
    info, best = svc.batch(good)
    assert info["state"] == 2 and best.shape == (3,)
    svc.close()
