"""Builds the fixtures of the reference's own recorded GA runs,
data process/ANO_Tnum/data_record_T_ANO_100.txt (18 runs x 100 tasks x 22
columns: best fitness at generations 0, 50, ..., 1000, then the 481st-best
member of the initial population; writer commented at proposed
model/SG-EMTF.cu:2015-2026):
  reference_records_T100.json       the initial and final columns, by type
  reference_trajectories_T100.npy   every column, float32 [18, 100, 22]
  reference_ano_T100.json           the ANO curve the reference's tool
                                    (data process/源.cpp:122-209) computed
                                    from those runs, as it printed it
                                    (data process/ANO_Tnum/
                                    data_record_T_ANO_100_1677482963.txt)

The task -> function map is the reference's: glibc srand(0); rand() % 7 per
task with task 0 forced to type 6 (SG-EMTF.cu:307-313).  Reference types are
stored as recorded (0 Sphere, 1 Rosenbrock, 2 Ackley, 3 Rastrigin,
4 Griewank, 5 Weierstrass, 6 Schwefel).

Usage (wherever the reference tree is available):
    python tests/golden/make_reference_records.py <reference root>
"""
import ctypes
import json
import os
import sys

import numpy as np

REC = os.path.join("data process", "ANO_Tnum", "data_record_T_ANO_100.txt")
REC_ANO = os.path.join("data process", "ANO_Tnum", "data_record_T_ANO_100_1677482963.txt")
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_records_T100.json")


def reference_types(n):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(0)
    t = [libc.rand() % 7 for _ in range(n)]
    t[0] = 6
    return t


def main(root):
    src, src_ano = os.path.join(root, REC), os.path.join(root, REC_ANO)
    runs, cur = [], []
    for line in open(src):
        line = line.strip()
        if not line:
            if cur:
                runs.append(cur)
                cur = []
            continue
        cur.append([float(v) for v in line.split()])
    if cur:
        runs.append(cur)
    assert all(len(r) == 100 and all(len(row) == 22 for row in r) for r in runs), "layout"
    out = {
        "source": "data process/ANO_Tnum/data_record_T_ANO_100.txt",
        "columns": "gen0_best, gen1000_best, gen0_rank481",
        "types": reference_types(100),
        "runs": [[[row[0], row[20], row[21]] for row in r] for r in runs],
    }
    with open(OUT, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    np.save(os.path.join(HERE, "reference_trajectories_T100.npy"), np.array(runs, np.float32))
    ano = [v.strip() for v in open(src_ano).read().split(",") if v.strip()]
    with open(os.path.join(HERE, "reference_ano_T100.json"), "w") as f:
        json.dump({"source": "data process/ANO_Tnum/data_record_T_ANO_100_1677482963.txt",
                   "ano": ano}, f, indent=0)
    print(OUT, len(runs), "runs;", len(ano), "ANO points")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_reference_records.py <reference root>")
    main(sys.argv[1])
