"""The C ABI from a compiled C++ host program (tests/cpp/host_example.cpp,
built here with g++ against include/sgemtf.h and the library): the
reference's GA setting on diagonal instances, run by the C++ program and by
the Python binding with the same configuration, must give the same best
fitness for every task and the same population of task 0, bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_host_program_matches_binding(sgemtf, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(sgemtf.LIB_PATH)
    exe = str(tmp_path / "host_example")
    subprocess.run([gxx, "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cpp", "host_example.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lsgemtf",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    T, D, NP, gens, epoch = 14, 50, 64, 100, 20
    rng = np.random.default_rng(3)
    ref_type = (np.arange(T) % 7).astype(np.int32)
    M = rng.uniform(0.0, 1.0, (T, D)).astype(np.float32)
    b = np.zeros((T, D), np.float32)
    for t in range(T):
        lo, hi = sgemtf.function_box(sgemtf.lib().emt_function_from_reference(int(ref_type[t])), True)
        b[t] = rng.uniform(0.0, 0.8 * (hi - lo) / 2, D).astype(np.float32)
    inp = tmp_path / "tasks.bin"
    with open(inp, "wb") as f:
        f.write(np.array([T, D, NP, gens, epoch], np.int32).tobytes())
        f.write(ref_type.tobytes())
        f.write(M.tobytes())
        f.write(b.tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.float32)
    best_cpp, pop_cpp = raw[:T], raw[T:].reshape(NP, D)

    cfg = sgemtf.Config(algorithm=sgemtf.GA_SBX_PM, eta_c=2.0, p_c=1.0, eta_m=5.0, p_m=1.0,
                        transfer_interval=epoch, transfer_rate=50.0 / 512.0, transfer_mix=0.4,
                        flags=sgemtf.FLAG_REF_BOXES | sgemtf.FLAG_REF_GRIEWANK_NO_PRODUCT |
                        sgemtf.FLAG_REF_WEIERSTRASS_CONST | sgemtf.FLAG_REF_ACKLEY_E, seed=12345)
    eng = sgemtf.Engine(cfg)
    eng.add_tasks([sgemtf.TaskDesc(sgemtf.lib().emt_function_from_reference(int(ref_type[t])), D, NP,
                                   rotation=sgemtf.ROTATION_DIAG, diag=M[t], shift=-b[t])
                   for t in range(T)])
    for _ in range(gens // epoch):
        eng.run(epoch)
    assert np.array_equal(eng.best_all(), best_cpp)
    assert np.array_equal(eng.population(0)[0], pop_cpp)
    eng.close()
