"""Calls on a non-blocking caller stream.  The library uploads tasks, restores
snapshots and replaces populations with copies and memsets on the legacy
default stream, which a stream created non-blocking does not wait for; the
library finishes those before it returns (or issues them on the handle's
stream), so a run launched on such a stream sees them.  Each case is checked
against the same calls on the default stream."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

LAYOUTS = {
    "fused": [(0, 50, 64, 1), (5, 50, 64, 1), (3, 30, 32, 1)],
    "large": [(0, 150, 16, 1), (3, 200, 12, 1)],  # HBM-resident islands
}


def _engine(sgemtf, layout, **kw):
    eng = sgemtf.Engine(sgemtf.Config(seed=4, transfer_interval=5, transfer_rate=0.2, **kw))
    eng.add_tasks([sgemtf.TaskDesc(f, D, NP, rotation=r) for f, D, NP, r in LAYOUTS[layout]])
    return eng


def _pops(eng):
    return [eng.population(t)[0].copy() for t in range(len(eng.tasks))]


@pytest.mark.parametrize("layout", ["fused", "large"])
@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_reset_and_run_on_a_nonblocking_stream(sgemtf, layout, precision):
    prec = sgemtf.ROT_FP32 if precision == "fp32" else sgemtf.ROT_TF32X3
    ref = _engine(sgemtf, layout, precision=prec)
    ref.reset()
    ref.run(12)
    want = _pops(ref)
    side = torch.cuda.Stream()  # created non-blocking
    eng = _engine(sgemtf, layout, precision=prec)
    eng.reset(side.cuda_stream)
    eng.run(12, side.cuda_stream)
    for a, b in zip(_pops(eng), want):
        assert np.array_equal(a, b)
    ref.close()
    eng.close()


@pytest.mark.parametrize("layout", ["fused", "large"])
def test_restore_and_set_population_on_a_nonblocking_stream(sgemtf, layout):
    side = torch.cuda.Stream()
    ref = _engine(sgemtf, layout)
    ref.reset()
    ref.run(7)
    blob = ref.snapshot()
    x = ref.population(1)[0].copy()
    x[3] = x[5]
    ref.set_population(1, x)
    ref.run(8)
    want = _pops(ref)

    eng = _engine(sgemtf, layout)
    eng.reset(side.cuda_stream)
    eng.run(3, side.cuda_stream)
    eng.restore(blob)
    eng.run(0, side.cuda_stream)  # the handle's stream becomes the side stream
    eng.set_population(1, x)
    eng.run(8, side.cuda_stream)
    for a, b in zip(_pops(eng), want):
        assert np.array_equal(a, b)
    ref.close()
    eng.close()
