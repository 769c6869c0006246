"""CPU checks of the oracle itself: known-answer vectors and analytic optima.

The reference ships no golden vectors (its only checks are printf probes with
0.1-1 tolerances, proposed model/SG-EMTF.cu:833-855,1263-1286), so the oracle
is pinned by published known answers (Philox4x32-10), by the functions'
analytic optima and by the reference's recorded trajectories
(test_reference_records.py).
"""
import math

import numpy as np
import pytest


# Random123 known-answer vectors for Philox4x32-10.
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_kat(orc, ctr, key, want):
    assert tuple(orc.philox(ctr, key)) == want


def test_u01_range_and_exactness(orc):
    L = orc.lib()
    assert L.orc_u01(0) == 0.0
    assert L.orc_u01(0xFFFFFFFF) == 1.0 - 2.0 ** -24
    assert L.orc_u01(0x80000000) == 0.5


def _identity_task(orc, fid, D, flags=0, o=None):
    lo, hi = orc.box(fid)
    return orc.OTask(fid, D, 8, lo, hi, None, o, flags)


@pytest.mark.parametrize("D", [1, 2, 10, 50, 128])
def test_analytic_optima(orc, D):
    """f(z*) at the known optimum of each function (shift o, identity Q)."""
    o = np.linspace(-0.3, 0.3, D).astype(np.float32)
    cases = {orc.SPHERE: 0.0, orc.RASTRIGIN: 0.0, orc.ACKLEY: 0.0, orc.GRIEWANK: 0.0,
             orc.WEIERSTRASS: 0.0}
    for fid, want in cases.items():
        t = _identity_task(orc, fid, D, o=o)
        f, _, _ = t.eval64(o)
        assert abs(f - want) < 1e-9 * D, (fid, f)
    # Rosenbrock: minimum 0 at z = 1 (reference form, SG-EMTF.cu:939-962)
    t = _identity_task(orc, orc.ROSENBROCK, D, o=np.zeros(D, np.float32))
    f, _, _ = t.eval64(np.ones(D, np.float32))
    assert abs(f) < 1e-12
    # Schwefel: 418.9829 D - sum z sin sqrt|z|, minimum near z = 420.9687
    t = _identity_task(orc, orc.SCHWEFEL, D, o=np.zeros(D, np.float32))
    f, _, _ = t.eval64(np.full(D, 420.9687, np.float32))
    assert abs(f) < 1e-3 * D


def test_known_values(orc):
    """Hand-computed values at simple points (z = x, o = 0)."""
    D = 2
    x = np.array([1.0, 2.0], np.float32)
    t = _identity_task(orc, orc.SPHERE, D)
    assert t.eval64(x)[0] == 5.0
    t = _identity_task(orc, orc.ROSENBROCK, D)
    assert t.eval64(x)[0] == 100.0 * (1 - 2) ** 2 + 0.0
    t = _identity_task(orc, orc.RASTRIGIN, D)
    assert abs(t.eval64(x)[0] - 5.0) < 1e-12  # integers: cos(2 pi z) = 1
    t = _identity_task(orc, orc.GRIEWANK, D)
    want = 1 + 5.0 / 4000 - math.cos(1.0) * math.cos(2.0 / math.sqrt(2))
    assert abs(t.eval64(x)[0] - want) < 1e-12
    t = _identity_task(orc, orc.ACKLEY, D)
    want = -20 * math.exp(-0.2 * math.sqrt(2.5)) - math.exp(1.0) + 20 + math.e
    assert abs(t.eval64(x)[0] - want) < 1e-12
    t = _identity_task(orc, orc.SCHWEFEL, D)
    want = 418.9829 * 2 - (math.sin(1.0) + 2 * math.sin(math.sqrt(2.0)))
    assert abs(t.eval64(x)[0] - want) < 1e-9


def test_reference_flags(orc):
    D = 3
    x = np.array([0.5, -1.0, 2.0], np.float32)
    t = orc.OTask(orc.GRIEWANK, D, 8, -100, 100, None, None, orc.FLAG_REF_GRIEWANK_NO_PRODUCT)
    assert abs(t.eval64(x)[0] - (0.25 + 1 + 4) / 4000) < 1e-15
    # reference host offset: float accumulation with PI = 3.1415926 (SG-EMTF.cu:354-361)
    w0 = orc.lib().orc_weierstrass_reference_offset()
    assert -2.0 < w0 < -1.9999
    t = orc.OTask(orc.WEIERSTRASS, D, 8, -0.5, 0.5, None, None, orc.FLAG_REF_WEIERSTRASS_CONST)
    f, _, _ = t.eval64(np.zeros(D, np.float32))
    assert abs(f - D * (-(2 - 2 ** -20) - w0)) < 1e-6


def test_reference_type_map_and_boxes(orc):
    L = orc.lib()
    assert [L.orc_function_from_reference(t) for t in range(7)] == [
        orc.SPHERE, orc.ROSENBROCK, orc.ACKLEY, orc.RASTRIGIN, orc.GRIEWANK, orc.WEIERSTRASS,
        orc.SCHWEFEL]
    # SG-EMTF.cu:197-214 by reference type
    ref = {0: 100, 1: 50, 2: 50, 3: 50, 4: 100, 5: 0.5, 6: 500}
    for rt, half in ref.items():
        lo, hi = orc.box(L.orc_function_from_reference(rt), True)
        assert (lo, hi) == (-half, half)


@pytest.mark.parametrize("D", [1, 2, 7, 50, 100])
def test_rotation_orthogonal(orc, D):
    Q = orc.gen_rotation(3, 11, D)
    assert np.abs(Q @ Q.T - np.eye(D)).max() < 1e-12
    Q2 = orc.gen_rotation(3, 11, D)
    assert np.array_equal(Q, Q2)
    if D > 1:
        assert not np.array_equal(Q, orc.gen_rotation(3, 12, D))


def test_shift_and_population_in_box(orc):
    for fid in range(7):
        lo, hi = orc.box(fid)
        o = orc.gen_shift(5, fid, 50, lo, hi)
        assert (o >= 0.8 * lo).all() and (o < 0.8 * hi + 1e-6).all()
        X = orc.gen_population(5, fid, 64, 50, lo, hi)
        assert (X >= lo).all() and (X <= hi).all()
        assert len(np.unique(X)) > 0.99 * X.size


def test_powf_accuracy(orc):
    rng = np.random.default_rng(0)
    xs = rng.uniform(1e-6, 1e6, 2000).astype(np.float32)
    ys = rng.uniform(-3, 3, 2000).astype(np.float32)
    L = orc.lib()
    for x, y in zip(xs, ys):
        want = float(x) ** float(y)
        if want < 1e-30 or want > 1e30:
            continue
        got = L.orc_powf(float(x), float(y))
        # exp2(t) with t = y log2 x rounded to FP32: relative error grows with |t|
        t = abs(float(y) * math.log2(float(x)))
        assert abs(got / want - 1) < (t + 8) * 2.0 ** -23, (x, y, got, want)
    assert L.orc_powf(0.0, 0.5) == 0.0
    assert L.orc_powf(1.0, 7.0) == 1.0


def test_de_trial_indices_distinct(orc):
    """r1, r2, r3 distinct and != i; the mutant uses them (DE/rand/1/bin)."""
    p = orc.params(seed=9, CR=0.0)  # CR = 0: only gene jrand is mutated
    for NP in (4, 5, 64, 100):
        D = 6
        lo, hi = -5.0, 5.0
        t = orc.OTask(orc.SPHERE, D, NP, lo, hi, None, None)
        X = orc.gen_population(9, 0, NP, D, lo, hi)
        for i in range(NP):
            u = orc.trial(p, t, X, 3, i)
            diff = np.nonzero(u != X[i])[0]
            assert len(diff) <= 1
            w = orc.draw(9, 0, 3, i, orc.P_DE_INDEX, 0)
            r1 = w[0] % (NP - 1)
            r1 += r1 >= i
            assert r1 != i


def test_selection_ties_go_to_trial(orc):
    """A trial equal in fitness to its parent replaces it (SG-EMTF_DE.cu:679-706)."""
    D, NP = 4, 8
    t = orc.OTask(orc.SPHERE, D, NP, -1.0, 1.0, None, None)
    X = np.zeros((NP, D), np.float32)
    f32 = np.zeros(NP, np.float32)
    f64 = np.zeros(NP)
    p = orc.params(seed=1, F=0.0, CR=1.0)  # trial = x_r1 = 0 vector: same fitness
    acc, _ = orc.generation(p, t, X, f32, f64, 1, 0)
    assert acc.all()


@pytest.mark.parametrize("fid", range(7))
def test_fp32_cpu_path_within_tolerance(orc, fid):
    """The oracle's FP32 arithmetic (the CPU baseline) against its FP64."""
    D, NP = 50, 32
    lo, hi = orc.box(fid)
    Q = orc.gen_rotation(4, fid, D).astype(np.float32)
    o = orc.gen_shift(4, fid, D, lo, hi)
    t = orc.OTask(fid, D, NP, lo, hi, Q, o, 0, fid)
    X = orc.gen_population(4, fid, NP, D, lo, hi)
    for x in X:
        f64, s, _ = t.eval64(x)
        f32, _ = t.eval32(x)
        tol = 1e-5 * s + (t.weier_bound(x) if fid == orc.WEIERSTRASS else 0.0)
        assert abs(f32 - f64) <= tol
