"""Device fitness against the FP64 oracle (the reference's evaluate kernel,
proposed model/SG-EMTF.cu:1428-1479, and evaluation(), :898-1111).

Tolerance: |f - f64| <= 1e-5 * scale, where scale is the sum of the absolute
sub-terms of f (so cancellation against a constant, e.g. Schwefel's
418.9829 D, does not turn rounding into a large relative error).  For
Weierstrass the bound adds the rounding of the FP32 rotation propagated
through its terms (3^k amplification, capped at each term's range)."""
import numpy as np
import pytest

from gpu_util import make_engine, tolerance

pytestmark = pytest.mark.gpu

CASES = [(1, 0), (2, 1), (10, 1), (50, 1), (50, 0), (100, 1), (128, 1)]


@pytest.mark.parametrize("fid", range(7))
@pytest.mark.parametrize("D,rot", CASES)
def test_evaluate_matches_fp64(sgemtf, orc, fid, D, rot):
    eng, (t,) = make_engine(sgemtf, orc, [(fid, D, 8, rot)], seed=3)
    lo, hi = t.c.lo, t.c.hi
    rng = np.random.default_rng(fid * 1000 + D)
    X = rng.uniform(lo, hi, (200, D)).astype(np.float32)
    X[0] = t.o                      # z = 0
    X[1] = lo                       # box corners
    X[2] = hi
    X[3] = np.clip(t.o + 1e-3, lo, hi)
    f, z = eng.evaluate(0, X, want_z=True)
    worst = 0.0
    for i, x in enumerate(X):
        f64, s, z64 = t.eval64(x)
        assert abs(float(f[i]) - f64) <= tolerance(orc, t, x, s), (i, float(f[i]), f64, s)
        if s > 0:
            worst = max(worst, abs(float(f[i]) - f64) / s)
        # rotation: rigorous FP32 dot-product bound gamma_{D+1} * sum |Q||x - o|
        sa = np.abs(t.Q.astype(np.float64)) @ np.abs(x.astype(np.float64) - t.o)
        g = (D + 1) * 2.0 ** -24 / (1 - (D + 1) * 2.0 ** -24)
        assert np.all(np.abs(z[i] - z64[:D]) <= g * sa + 1e-30)
    # Weierstrass: within its default near-tie half-window, 5e-5 of the scale
    assert worst <= (5e-5 if fid == orc.WEIERSTRASS else 1e-5)


@pytest.mark.parametrize("D", [1, 17, 50])
def test_weierstrass_epilogue_exact_argument(sgemtf, orc, D):
    """With z exactly representable (identity, zero shift) the only error is
    the epilogue's: exact reduction of 2*3^k*z mod 2, then cosines."""
    eng = sgemtf.Engine(sgemtf.Config(seed=1))
    eng.add_tasks([sgemtf.TaskDesc(sgemtf.WEIERSTRASS, D, 8, rotation=sgemtf.ROTATION_IDENTITY,
                                   shift=np.zeros(D, np.float32))])
    t = orc.OTask(orc.WEIERSTRASS, D, 8, -0.5, 0.5, None, np.zeros(D, np.float32))
    rng = np.random.default_rng(D)
    X = rng.uniform(-0.5, 0.5, (300, D)).astype(np.float32)
    X[0] = 0.0
    X[1, :] = 2.0 ** -30
    X[2, :] = 0.5
    f = eng.evaluate(0, X)
    for i, x in enumerate(X):
        f64, s, _ = t.eval64(x)
        assert abs(float(f[i]) - f64) <= 1e-5 * s + 2e-6 * D, (i, float(f[i]), f64)


def test_reference_mode_diag_rotation(sgemtf, orc):
    """z = M (x + b) of the reference (SG-EMTF.cu:922) through DIAG with o = -b."""
    D = 50
    rng = np.random.default_rng(5)
    M = rng.uniform(0, 1, D).astype(np.float32)
    b = rng.uniform(0, 200, D).astype(np.float32)
    flags = sgemtf.FLAG_REF_BOXES | sgemtf.FLAG_REF_GRIEWANK_NO_PRODUCT | \
        sgemtf.FLAG_REF_WEIERSTRASS_CONST | sgemtf.FLAG_REF_ACKLEY_E
    for fid in range(7):
        eng = sgemtf.Engine(sgemtf.Config(seed=1, flags=flags))
        eng.add_tasks([sgemtf.TaskDesc(fid, D, 8, rotation=sgemtf.ROTATION_DIAG, diag=M, shift=-b)])
        lo, hi = sgemtf.function_box(fid, True)
        t = orc.OTask(fid, D, 8, lo, hi, np.diag(M), -b, flags)
        X = rng.uniform(lo, hi, (64, D)).astype(np.float32)
        f, z = eng.evaluate(0, X, want_z=True)
        # the reference's single FP32 product M * (x + b) is exactly what FMA
        # against a diagonal Q computes
        assert np.array_equal(z, (M * (X + b)).astype(np.float32))
        for i, x in enumerate(X):
            f64, s, _ = t.eval64(x)
            assert abs(float(f[i]) - f64) <= tolerance(orc, t, x, s)
