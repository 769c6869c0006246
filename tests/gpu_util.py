"""Helpers shared by the GPU parity tests: build an engine and the matching
oracle tasks from the engine's own rotation and shift."""
import numpy as np


def make_engine(sgemtf, orc, specs, seed=1, **cfg):
    """specs: list of (fid, D, NP, rotation).  Returns (engine, oracle tasks)."""
    eng = sgemtf.Engine(sgemtf.Config(seed=seed, **cfg))
    eng.add_tasks([sgemtf.TaskDesc(f, D, NP, rotation=r) for f, D, NP, r in specs])
    tasks = []
    for t, (f, D, NP, r) in enumerate(specs):
        Q, o = eng.task_params(t)
        lo, hi = sgemtf.function_box(f, bool(eng.config.flags & sgemtf.FLAG_REF_BOXES))
        tasks.append(orc.OTask(f, D, NP, lo, hi, Q, o, eng.config.flags, t))
    return eng, tasks


def oracle_params(orc, eng):
    c = eng.config
    return orc.params(algorithm=c.algorithm, F=c.F, CR=c.CR, eta_c=c.eta_c, p_c=c.p_c,
                      eta_m=c.eta_m, p_m=c.p_m, transfer_mix=c.transfer_mix, seed=c.seed,
                      recheck_rel=c.recheck_rel, flags=c.flags, subislands=max(1, c.subislands),
                      mig_interval=c.migration_interval, mig_count=c.migration_count)


def tolerance(orc, t, x, scale):
    tol = 1e-5 * scale
    if t.c.fid == orc.WEIERSTRASS:
        tol += t.weier_bound(x)
    return tol
