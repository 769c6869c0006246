"""emt_run_noalloc: the generation loop for callers that cannot allocate
device memory at run time (a service whose GPU memory belongs to its own
pool allocator, or a loop that must not call cudaMalloc/cudaFree because
they synchronize the device).  Its elite-exchange scratch is a fixed
4 MiB device array in the library instead of a per-handle allocation.

Checked through the C ABI against emt_run on the same handle configuration:
populations must be bit-identical (the repository's tolerance for selection
replay), after each of two calls in a row.  This file is collected last so
that a run stopping at the first failure has already run everything else;
it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(sgemtf, seed, transfer_interval, tasks=7, D=20, NP=24):
    eng = sgemtf.Engine(sgemtf.Config(seed=seed, transfer_interval=transfer_interval,
                                      transfer_rate=0.25))
    eng.add_tasks([sgemtf.TaskDesc(f % 7, D, NP) for f in range(tasks)])
    return eng


@pytest.mark.parametrize("precision", [0, 1, 3])
def test_noalloc_matches_run_two_calls(sgemtf, precision):
    ref = sgemtf.Engine(sgemtf.Config(seed=23, transfer_interval=5, transfer_rate=0.25,
                                      precision=precision))
    new = sgemtf.Engine(sgemtf.Config(seed=23, transfer_interval=5, transfer_rate=0.25,
                                      precision=precision))
    descs = [sgemtf.TaskDesc(f % 7, 20, 24) for f in range(7)]
    ref.add_tasks(descs)
    new.add_tasks(descs)
    ref.reset()
    new.reset()
    L = sgemtf.lib()
    for gens in (12, 13):  # the first call ends mid-interval, the second on a boundary
        ref.run(gens)
        assert L.emt_run_noalloc(new._h, gens, None) == sgemtf.OK, L.emt_last_error(new._h)
        new.sync()
        for i in range(7):
            assert np.array_equal(ref.population(i)[0], new.population(i)[0]), (gens, i)
            assert np.array_equal(ref.population(i)[1], new.population(i)[1]), (gens, i)
    # the handle carries the exchange state on: a following emt_run agrees too
    ref.run(6)
    new.run(6)
    for i in range(7):
        assert np.array_equal(ref.population(i)[0], new.population(i)[0])


def test_noalloc_without_transfer(sgemtf):
    ref = _engine(sgemtf, 3, 0)
    new = _engine(sgemtf, 3, 0)
    ref.reset()
    new.reset()
    ref.run(9)
    new.run_noalloc(9)
    for i in range(7):
        assert np.array_equal(ref.population(i)[0], new.population(i)[0])


def test_noalloc_refusals(sgemtf):
    L = sgemtf.lib()
    eng = _engine(sgemtf, 1, 5)
    # not prepared by emt_reset: it would have to allocate
    assert L.emt_run_noalloc(eng._h, 3, None) == sgemtf.ERR_STATE
    assert b"emt_reset" in L.emt_last_error(eng._h)
    # exchange larger than the static buffer
    big = sgemtf.Engine(sgemtf.Config(seed=1, transfer_interval=5))
    n = sgemtf.NOALLOC_EXCHANGE_FLOATS // (128 * 64) + 1  # NP * round4(D) per task
    big.add_tasks([sgemtf.TaskDesc(0, 64, 128) for _ in range(n)])
    big.reset()
    assert L.emt_run_noalloc(big._h, 3, None) == sgemtf.ERR_UNSUPPORTED
    assert b"static buffer" in L.emt_last_error(big._h)
    assert L.emt_run_noalloc(None, 3, None) == sgemtf.ERR_INVALID_ARG
