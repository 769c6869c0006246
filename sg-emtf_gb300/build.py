"""In-tree build of the engine's shared library for sm_103a.

    python sg-emtf_gb300/build.py        # -> sg-emtf_gb300/_build/libsgemtf.so
    python sg-emtf_gb300/build.py --phases   # -> _build/libsgemtf_phases.so, the
                                             # measurement build with phase clocks

Each translation unit compiles in parallel with one -gencode (sm_103a); the
objects link into one shared library exporting the C ABI of include/sgemtf.h.
Host code is built with -ffp-contract=off so that the library's host-side
FP32 arithmetic (shift vectors) is identical on x86-64 and AArch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsgemtf.so")
PHASES_LIB = os.path.join(OUT, "libsgemtf_phases.so")
SOURCES = ["emt_kernels.cu", "emt_api.cu", "emt_cvrp.cu", "emt_records.cpp", "emt_service.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, phases=False):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + (".phases.o" if phases else ".o"))
    extra = ["-DEMT_PHASE_CLOCKS"] if phases else []
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(ROOT, "include", "sgemtf.h"), os.path.abspath(__file__)]
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, phases=False):
    lib = PHASES_LIB if phases else LIB
    if not force and up_to_date(lib):
        return lib
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda f: _compile(f, phases), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, phases="--phases" in sys.argv))
