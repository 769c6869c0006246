"""The oracle's reference mode against fitness values computed by the
reference's own evaluate kernel (proposed model/SG-EMTF.cu:1428-1479,
evaluation() :898-1111), compiled from its source and run on a GPU by
tests/golden/make_reference_evaluate.py: 7 function types x 512 individuals
of D = 50 on diagonal instances z = M (x + b).

The reference sums its terms with FP32 shared-memory atomics in an
order-dependent way and computes z and every term in FP32; the oracle
evaluates the same definitions in FP64.  For six function types agreement
within 1e-6 of the scale (the sum of absolute sub-terms) pins the oracle's
definitions, constants (E = 2.718282), box table, the Griewank variant
without its product, and the diagonal-instance convention o = -b against
the reference's arithmetic.

Weierstrass is the exception, and the reason is the reference's own FP32
arithmetic: it forms each argument as the FP32 product 2 (z + 1/2) * 3^k
(:1057-1064), which for 3^k |2z + 1| >= 2^25 (k >= 16 for most z) is an
even integer, so cospif returns exactly 1 for those terms, and for k around
12-15 the product has lost most of its fraction bits.  The test restates
that FP32 recipe term by term and requires the reference's values within
1e-6 of it; the oracle's exact definition (also the engine's) differs from
the reference by that artifact, a bias of about 1.5e-5 of the scale, and
within 3e-5 (the offset, from PI = 3.1415926, agrees to the bit)."""
import ctypes
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_evaluate.json")
sys.path.insert(0, os.path.join(HERE, "golden"))

REF_FLAGS = 0x1 | 0x2 | 0x4 | 0x8  # no Griewank product, Weierstrass const, Ackley E, boxes
# worst |f_ref - f64| / scale allowed per reference type (SG-EMTF.cu numbering)
TOL = {0: 1e-6, 1: 1e-6, 2: 1e-6, 3: 1e-6, 4: 1e-6, 5: 3e-5, 6: 1e-6}
WEIERSTRASS = 5


def weierstrass_fp32_recipe(X, M, b, para):
    """The reference's Weierstrass in its own FP32 steps (SG-EMTF.cu:1049-1078):
    x = M (x + b), t = 2 (x + 0.5), terms 0.5^k cospi(t * 3^k) with the
    product and the powers rounded to FP32, minus DIMENSION * para.  cospi is
    taken in FP64 on the exactly reduced FP32 argument; sums in FP64."""
    f32 = np.float32
    z = (M.astype(f32) * (X.astype(f32) + b.astype(f32)).astype(f32)).astype(f32)
    t = (f32(2) * (z + f32(0.5)).astype(f32)).astype(f32)
    a, p = f32(1), f32(1)
    total = np.zeros(X.shape[0])
    for _ in range(21):
        arg = (t * p).astype(f32).astype(np.float64)
        r = np.fmod(np.abs(arg), 2.0)
        total += float(a) * np.cos(np.pi * r).sum(axis=1)
        a = f32(a * f32(0.5))
        p = f32(p * f32(3))
    return total - X.shape[1] * float(para)


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(GOLDEN):
        pytest.fail("missing %s (tests/golden/make_reference_evaluate.py makes it)" % GOLDEN)
    with open(GOLDEN) as fh:
        return json.load(fh)


def test_reference_evaluate_pins_oracle(orc, golden):
    import make_reference_evaluate as mk
    lib = orc.lib()
    lib.orc_function_from_reference.restype = ctypes.c_int
    lib.orc_function_from_reference.argtypes = [ctypes.c_int]
    assert golden["seed"] == mk.SEED and golden["np"] == mk.NP and golden["dim"] == mk.D
    assert np.float32(golden["weierstrass_para"]) == np.float32(lib.orc_weierstrass_reference_offset())
    worst = {}
    for rtype in range(7):
        X, M, b = mk.reference_inputs(orc, rtype)
        f_ref = np.array(golden["fitness"][str(rtype)], np.uint32).view(np.float32)
        fid = lib.orc_function_from_reference(rtype)
        lo, hi = orc.box(fid, reference_boxes=True)
        t = orc.OTask(fid, mk.D, mk.NP, lo, hi, np.diag(M.astype(np.float32)), -b, REF_FLAGS)
        w = 0.0
        for i in range(mk.NP):
            f64, s, _ = t.eval64(X[i])
            assert np.isfinite(f_ref[i])
            w = max(w, abs(float(f_ref[i]) - f64) / s)
        worst[rtype] = w
        if rtype == WEIERSTRASS:
            emu = weierstrass_fp32_recipe(X, M, b, np.float32(golden["weierstrass_para"]))
            scale = np.array([t.eval64(X[i])[1] for i in range(mk.NP)])
            assert np.max(np.abs(f_ref - emu) / scale) <= 1e-6
    for rtype, w in worst.items():
        assert w <= TOL[rtype], (rtype, w, worst)
