"""The library's seeded rotations (EMT_ROTATION_SEEDED_QR), computed on the
host left-looking in blocks of columns and rows, against the oracle's
step-by-step Householder QR (orc_gen_rotation): the same FP64 matrix bit for
bit, sizes across the block edges (16) included.  Host code only: runs
without a GPU."""
import numpy as np
import pytest


@pytest.mark.parametrize("D", [1, 2, 3, 15, 16, 17, 31, 50, 129, 300])
def test_seeded_rotation_matches_the_oracle(sgemtf, orc, D):
    for seed, task in ((1, 0), (7, 5), (123456789, 41)):
        q = sgemtf.seeded_rotation(seed, task, D)
        ref = orc.gen_rotation(seed, task, D)
        assert np.array_equal(q.view(np.uint64), ref.view(np.uint64)), (D, seed, task)


def test_seeded_rotation_is_orthogonal(sgemtf):
    q = sgemtf.seeded_rotation(3, 2, 200)
    assert np.abs(q @ q.T - np.eye(200)).max() < 1e-12


def test_seeded_rotation_rejects_bad_arguments(sgemtf):
    for dim in (0, 1025):
        with pytest.raises(sgemtf.EngineError) as e:
            sgemtf.seeded_rotation(1, 0, dim)
        assert e.value.status == sgemtf.ERR_INVALID_ARG
    with pytest.raises(sgemtf.EngineError):
        sgemtf.seeded_rotation(1, -1, 10)
