"""Failure detection on the device without a GPU fault: every mbarrier wait
of the tensor-core form is bounded by emt_config.wait_limit_ms.  The test
switch EMT_FLAG_TEST_LOST_COMPLETION makes the rotation issue no MMA and no
commit, so the wait for the MMA barrier runs out with nothing in flight (the
TMA copy of the rotation tiles has landed before).  The kernel records
CHECK_TIMEOUT, skips the rest of the epoch, frees its tensor memory and
returns; the host reads EMT_ERR_DEVICE_CHECK and the context stays usable."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _descs(sgemtf):
    return [sgemtf.TaskDesc(f, 20, 32) for f in range(3)]


@pytest.mark.parametrize("precision", [3, 1])  # BF16X3, TF32X3
def test_lost_completion_reports_and_context_survives(sgemtf, precision):
    cfg = dict(seed=4, precision=precision)
    bad = sgemtf.Engine(sgemtf.Config(wait_limit_ms=20, flags=sgemtf.FLAG_TEST_LOST_COMPLETION,
                                      **cfg))
    bad.add_tasks(_descs(sgemtf))
    t0 = time.perf_counter()
    bad.reset()  # the initial evaluation's rotation waits in vain
    with pytest.raises(sgemtf.EngineError) as e:
        bad.sync()
    waited = time.perf_counter() - t0
    assert e.value.status == sgemtf.ERR_DEVICE_CHECK
    assert "wait ran out" in str(e.value)
    assert waited < 10.0  # the 20 ms limit, not the 2 s default per wait
    bad.close()
    # a fresh handle on the same context runs normally and matches the FP32 form
    good = sgemtf.Engine(sgemtf.Config(**cfg))
    ref = sgemtf.Engine(sgemtf.Config(seed=4, precision=sgemtf.ROT_FP32))
    for eng in (good, ref):
        eng.add_tasks(_descs(sgemtf))
        eng.run(8)
    assert good.stats()["precision_used"] == precision
    for i in range(3):
        assert np.array_equal(good.population(i)[0], ref.population(i)[0])


def test_wait_limit_is_validated(sgemtf):
    with pytest.raises(sgemtf.EngineError) as e:
        sgemtf.Engine(sgemtf.Config(wait_limit_ms=-1))
    assert e.value.status == sgemtf.ERR_INVALID_ARG
