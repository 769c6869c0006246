"""Golden fitness values from the reference's own evaluate kernel.

Runs the reference's `evaluate` kernel (proposed model/SG-EMTF.cu:1428-1479,
which calls evaluation(), :898-1111) from the cubin that `make -C oracle ref`
compiles out of the reference's source (oracle/_ref/sgemtf_ref.cubin), on one
GPU, through the CUDA driver API, and writes reference_evaluate.json beside
this script.  tests/test_reference_evaluate.py checks the oracle's reference
mode against those values on the CPU.

Inputs (regenerated from seeds by the test, so only the outputs are stored):
for each reference function type t = 0..6 (SG-EMTF.cu numbering), one
population of INDIVNUM = 512 individuals of DIMENSION = 50 drawn uniformly in
the type's reference box (Range, :197-214) by the oracle's Philox stream
(orc.gen_population(SEED, t, 512, 50, lo, hi)), and one instance
z = M (x + b) with M ~ U[0, 1) (orc.gen_population(SEED, 100 + t, 1, 50, 0, 1))
and b ~ U[0, hi - lo) (orc.gen_population(SEED, 200 + t, 1, 50, 0, hi - lo)),
as para_init draws them (:181-195).

Launch as iter() does (:1661-1663): BLOCK_NUM = 16 blocks of
THREAD_FOR_OPERA = 416 threads, one task of 512 individuals.  The reference
passes 576 bytes of dynamic shared memory while evaluation() addresses
3 x 64 floats (768 bytes) of it; this launch passes 1024 so that every access
stays inside the allocation.  Weierstrass_para is set as initialization()
sets it (:354-361): the host's float sum of 0.5^k cosf(2 PI 3^k 0.5) with
PI = 3.1415926, computed by the oracle's C restatement of that loop.

Usage (on a machine with the GPU and the cubin):
    make -C oracle ref        # where the reference tree is present
    python tests/golden/make_reference_evaluate.py [out.json]
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

SEED = 97
NP, D = 512, 50
GRID, BLOCK, DYN_SMEM = 16, 416, 1024
CUBIN = os.path.join(ROOT, "oracle", "_ref", "sgemtf_ref.cubin")
KERNEL = b"_Z8evaluatePfS_S_S_Pi"  # evaluate(float*, float*, float*, float*, int*)


def reference_inputs(orc, rtype):
    """Population, M and b of reference type rtype (see the module doc)."""
    fid = orc.lib().orc_function_from_reference(rtype)
    lo, hi = orc.box(fid, reference_boxes=True)
    X = orc.gen_population(SEED, rtype, NP, D, lo, hi)
    M = orc.gen_population(SEED, 100 + rtype, 1, D, 0.0, 1.0)[0]
    b = orc.gen_population(SEED, 200 + rtype, 1, D, 0.0, hi - lo)[0]
    return X, M, b


class Driver:
    """The few CUDA driver calls the launch needs."""

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.ctx = ctypes.c_void_p()
        self.check(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self.check(self.cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        self.check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "ctx retain")
        self.check(self.cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")

    @staticmethod
    def check(rc, what):
        if rc != 0:
            raise RuntimeError("%s failed (CUresult %d)" % (what, rc))

    def alloc(self, nbytes):
        p = ctypes.c_uint64()
        self.check(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(nbytes)), "cuMemAlloc")
        return p

    def h2d(self, dst, arr):
        arr = np.ascontiguousarray(arr)
        self.check(self.cu.cuMemcpyHtoD_v2(dst, arr.ctypes.data_as(ctypes.c_void_p),
                                           ctypes.c_size_t(arr.nbytes)), "cuMemcpyHtoD")

    def d2h(self, arr, src):
        self.check(self.cu.cuMemcpyDtoH_v2(arr.ctypes.data_as(ctypes.c_void_p), src,
                                           ctypes.c_size_t(arr.nbytes)), "cuMemcpyDtoH")


def main(out_path):
    import orc
    orc.build()
    orc.lib().orc_function_from_reference.restype = ctypes.c_int
    orc.lib().orc_function_from_reference.argtypes = [ctypes.c_int]
    orc.lib().orc_weierstrass_reference_offset.restype = ctypes.c_double
    if not os.path.exists(CUBIN):
        raise SystemExit("missing %s: run `make -C oracle ref` where the reference is" % CUBIN)
    drv = Driver()
    cu = drv.cu
    mod = ctypes.c_void_p()
    drv.check(cu.cuModuleLoad(ctypes.byref(mod), CUBIN.encode()), "cuModuleLoad")
    fn = ctypes.c_void_p()
    drv.check(cu.cuModuleGetFunction(ctypes.byref(fn), mod, KERNEL), "cuModuleGetFunction")
    wp, wsize = ctypes.c_uint64(), ctypes.c_size_t()
    drv.check(cu.cuModuleGetGlobal_v2(ctypes.byref(wp), ctypes.byref(wsize), mod,
                                      b"Weierstrass_para"), "cuModuleGetGlobal")
    assert wsize.value == 4
    # initialization() stores the float sum; the oracle restates its loop in C
    wpara = np.array([orc.lib().orc_weierstrass_reference_offset()], np.float32)
    drv.h2d(wp, wpara)

    d_x, d_f = drv.alloc(NP * D * 4), drv.alloc(NP * 4)
    d_m, d_b, d_t = drv.alloc(D * 4), drv.alloc(D * 4), drv.alloc(4)
    result = {"seed": SEED, "np": NP, "dim": D, "launch": [GRID, BLOCK, DYN_SMEM],
              "weierstrass_para": float(wpara[0]), "fitness": {}}
    for rtype in range(7):
        X, M, b = reference_inputs(orc, rtype)
        drv.h2d(d_x, X.astype(np.float32))
        drv.h2d(d_f, np.zeros(NP, np.float32))
        drv.h2d(d_m, M.astype(np.float32))
        drv.h2d(d_b, b.astype(np.float32))
        drv.h2d(d_t, np.array([rtype], np.int32))
        args = [ctypes.c_uint64(p.value) for p in (d_x, d_f, d_m, d_b, d_t)]
        params = (ctypes.c_void_p * 5)(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
        drv.check(cu.cuLaunchKernel(fn, GRID, 1, 1, BLOCK, 1, 1, DYN_SMEM, None, params, None),
                  "cuLaunchKernel")
        drv.check(cu.cuCtxSynchronize(), "cuCtxSynchronize")
        f = np.zeros(NP, np.float32)
        drv.d2h(f, d_f)
        # float32 values as their bit patterns, so the file is exact
        result["fitness"][str(rtype)] = [int(v) for v in f.view(np.uint32)]
        print("type %d: f[0..3] = %s" % (rtype, f[:4]), flush=True)
    for p in (d_x, d_f, d_m, d_b, d_t):
        cu.cuMemFree_v2(p)
    cu.cuModuleUnload(mod)
    with open(out_path, "w") as fh:
        json.dump(result, fh)
    print("wrote", out_path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "reference_evaluate.json"))
