"""ctypes binding of the CPU oracle (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
as the checker; the product never imports it.  `build()` compiles
oracle/emt_oracle.c with the committed Makefile.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libemt_oracle.so")

SPHERE, RASTRIGIN, ACKLEY, GRIEWANK, ROSENBROCK, SCHWEFEL, WEIERSTRASS = range(7)
FUNCTION_NAMES = ["sphere", "rastrigin", "ackley", "griewank", "rosenbrock", "schwefel",
                  "weierstrass"]
DE_RAND1, DE_CURRENT1, GA = 0, 1, 2
FLAG_REF_GRIEWANK_NO_PRODUCT = 0x1
FLAG_REF_WEIERSTRASS_CONST = 0x2
FLAG_REF_ACKLEY_E = 0x4
FLAG_REF_BOXES = 0x8
FLAG_NO_RECHECK = 0x10
FLAG_RIGOROUS_WINDOW = 0x20

P_POP_INIT, P_SHIFT, P_QR_NORMAL, P_DE_INDEX, P_DE_CR = 1, 2, 3, 4, 5
P_GA_PARENT, P_GA_SBX, P_GA_PM, P_TRANSFER_PARTNER, P_TRANSFER_MIX = 6, 7, 8, 9, 10
P_CVRP_NODE, P_CVRP_POP_INIT, P_CVRP_SELECT, P_CVRP_OX, P_CVRP_MUTATE, P_CVRP_PARTNER = range(16, 22)

_F32P = ctypes.POINTER(ctypes.c_float)
_F64P = ctypes.POINTER(ctypes.c_double)
_U8P = ctypes.POINTER(ctypes.c_uint8)


class Task(ctypes.Structure):
    _fields_ = [("fid", ctypes.c_int), ("D", ctypes.c_int), ("NP", ctypes.c_int),
                ("lo", ctypes.c_float), ("hi", ctypes.c_float), ("Q", _F32P),
                ("o", _F32P), ("flags", ctypes.c_uint32), ("id", ctypes.c_uint32)]


class Params(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int), ("F", ctypes.c_float), ("CR", ctypes.c_float),
                ("eta_c", ctypes.c_float), ("p_c", ctypes.c_float), ("eta_m", ctypes.c_float),
                ("p_m", ctypes.c_float), ("transfer_mix", ctypes.c_float),
                ("seed", ctypes.c_uint64), ("recheck_rel", ctypes.c_double),
                ("flags", ctypes.c_uint32), ("subislands", ctypes.c_int),
                ("mig_interval", ctypes.c_int), ("mig_count", ctypes.c_int)]


class CvrpParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("p_cross", ctypes.c_float), ("p_swap", ctypes.c_float),
                ("p_2opt", ctypes.c_float), ("subislands", ctypes.c_int),
                ("mig_interval", ctypes.c_int), ("mig_count", ctypes.c_int)]


def build(quiet=True):
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_u01.restype = ctypes.c_float
        L.orc_u01.argtypes = [ctypes.c_uint32]
        L.orc_eval64.restype = ctypes.c_double
        L.orc_eval64.argtypes = [ctypes.POINTER(Task), _F32P, _F64P, _F64P]
        L.orc_eval32.restype = ctypes.c_float
        L.orc_eval32.argtypes = [ctypes.POINTER(Task), _F32P, _F32P]
        L.orc_weierstrass_rotation_bound.restype = ctypes.c_double
        L.orc_weierstrass_rotation_bound.argtypes = [ctypes.POINTER(Task), _F32P]
        L.orc_weierstrass_reference_offset.restype = ctypes.c_double
        L.orc_powf.restype = ctypes.c_float
        L.orc_powf.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc_gen_shift.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                    ctypes.c_float, ctypes.c_float, _F32P]
        L.orc_gen_population.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_float, ctypes.c_float, _F32P]
        L.orc_gen_rotation.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, _F64P]
        L.orc_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                               ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                               ctypes.POINTER(ctypes.c_uint32)]
        L.orc_generation.restype = ctypes.c_int
        L.orc_generation.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Task), _F32P, _F32P,
                                     _F64P, ctypes.c_uint32, ctypes.c_int, _U8P]
        L.orc_trial.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Task), _F32P,
                                ctypes.c_uint32, ctypes.c_int, _F32P]
        L.orc_rank.argtypes = [_F32P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_transfer_partner.restype = ctypes.c_int
        L.orc_transfer_partner.argtypes = [ctypes.POINTER(Params), ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.c_uint32]
        L.orc_transfer_in.restype = ctypes.c_int
        L.orc_transfer_in.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Task),
                                      ctypes.POINTER(Task), _F32P, ctypes.c_int, _F32P, _F32P,
                                      _F64P, ctypes.c_uint32, ctypes.c_int]
        L.orc_migration_due.restype = ctypes.c_int
        L.orc_migration_due.argtypes = [ctypes.POINTER(Params), ctypes.c_uint32]
        L.orc_migration_count.restype = ctypes.c_int
        L.orc_migration_count.argtypes = [ctypes.POINTER(Params), ctypes.c_int]
        L.orc_migrate.restype = ctypes.c_int
        L.orc_migrate.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Task), _F32P, _F32P,
                                  _F64P, ctypes.c_int]
        L.orc_run_threads.restype = ctypes.c_double
        L.orc_run_threads.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Task), ctypes.c_int,
                                      ctypes.POINTER(_F32P), ctypes.POINTER(_F32P),
                                      ctypes.POINTER(_F64P), ctypes.c_uint32, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int]
        L.orc_box.argtypes = [ctypes.c_int, ctypes.c_int, _F32P, _F32P]
        I32P = ctypes.POINTER(ctypes.c_int32)
        L.orc_cvrp_round_sqrt.restype = ctypes.c_uint32
        L.orc_cvrp_round_sqrt.argtypes = [ctypes.c_uint64]
        L.orc_cvrp_gen_instance.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, I32P,
                                            I32P, I32P]
        L.orc_cvrp_distances.argtypes = [ctypes.c_int, I32P, I32P, I32P]
        L.orc_cvrp_split.restype = ctypes.c_int32
        L.orc_cvrp_split.argtypes = [ctypes.c_int, I32P, I32P, ctypes.c_int32, _U8P, I32P]
        L.orc_cvrp_child.argtypes = [ctypes.POINTER(CvrpParams), ctypes.c_uint32, ctypes.c_int,
                                     ctypes.c_int, _U8P, I32P, ctypes.c_uint32, ctypes.c_int, _U8P]
        L.orc_cvrp_init_population.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int,
                                               ctypes.c_int, _U8P]
        L.orc_cvrp_generation.restype = ctypes.c_int
        L.orc_cvrp_generation.argtypes = [ctypes.POINTER(CvrpParams), ctypes.c_uint32, ctypes.c_int,
                                          ctypes.c_int, I32P, I32P, ctypes.c_int32, _U8P, I32P,
                                          ctypes.c_uint32]
        L.orc_cvrp_rank.argtypes = [I32P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_cvrp_migrate.restype = ctypes.c_int
        L.orc_cvrp_migrate.argtypes = [ctypes.POINTER(CvrpParams), ctypes.c_int, ctypes.c_int, _U8P,
                                       I32P, ctypes.c_uint32]
        L.orc_cvrp_transfer_in.restype = ctypes.c_int
        L.orc_cvrp_transfer_in.argtypes = [ctypes.c_int, ctypes.c_int, I32P, I32P, ctypes.c_int32,
                                           _U8P, ctypes.c_int, _U8P, I32P]
        _lib = L
    return _lib


def _p32(a):
    return a.ctypes.data_as(_F32P)


def _p64(a):
    return a.ctypes.data_as(_F64P)


def box(fid, reference_boxes=False):
    lo, hi = ctypes.c_float(), ctypes.c_float()
    lib().orc_box(fid, int(reference_boxes), ctypes.byref(lo), ctypes.byref(hi))
    return lo.value, hi.value


def draw(seed, task, gen, member, purpose, block):
    out = (ctypes.c_uint32 * 4)()
    lib().orc_draw(seed, task, gen, member, purpose, block, out)
    return list(out)


def philox(ctr, key):
    out = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32_10((ctypes.c_uint32 * 4)(*ctr), (ctypes.c_uint32 * 2)(*key), out)
    return list(out)


def gen_shift(seed, task, D, lo, hi):
    o = np.zeros(D, np.float32)
    lib().orc_gen_shift(seed, task, D, lo, hi, _p32(o))
    return o


def gen_population(seed, task, NP, D, lo, hi):
    X = np.zeros((NP, D), np.float32)
    lib().orc_gen_population(seed, task, NP, D, lo, hi, _p32(X))
    return X


def gen_rotation(seed, task, D):
    Q = np.zeros((D, D), np.float64)
    lib().orc_gen_rotation(seed, task, D, _p64(Q))
    return Q


class OTask:
    """An oracle task: keeps the numpy buffers alive behind the C struct."""

    def __init__(self, fid, D, NP, lo, hi, Q=None, o=None, flags=0, tid=0):
        self.Q = None if Q is None else np.ascontiguousarray(Q, np.float32)
        self.o = np.zeros(D, np.float32) if o is None else np.ascontiguousarray(o, np.float32)
        self.c = Task(fid, D, NP, lo, hi, _p32(self.Q) if self.Q is not None else None,
                      _p32(self.o), flags, tid)

    @property
    def D(self):
        return self.c.D

    @property
    def NP(self):
        return self.c.NP

    def eval64(self, x):
        x = np.ascontiguousarray(x, np.float32)
        s = ctypes.c_double()
        z = np.zeros(max(self.D, 1), np.float64)
        f = lib().orc_eval64(ctypes.byref(self.c), _p32(x), ctypes.byref(s), _p64(z))
        return f, s.value, z

    def eval32(self, x):
        x = np.ascontiguousarray(x, np.float32)
        s = ctypes.c_float()
        f = lib().orc_eval32(ctypes.byref(self.c), _p32(x), ctypes.byref(s))
        return f, s.value

    def weier_bound(self, x):
        x = np.ascontiguousarray(x, np.float32)
        return lib().orc_weierstrass_rotation_bound(ctypes.byref(self.c), _p32(x))


def params(algorithm=DE_RAND1, F=0.5, CR=0.9, eta_c=15.0, p_c=0.9, eta_m=15.0, p_m=-1.0,
           transfer_mix=0.4, seed=1, recheck_rel=0.0, flags=0, subislands=1, mig_interval=0,
           mig_count=0):
    return Params(algorithm, F, CR, eta_c, p_c, eta_m, p_m, transfer_mix, seed, recheck_rel,
                  flags, subislands, mig_interval, mig_count)


def generation(p, t, X, fit32, fit64, gen, mode):
    acc = np.zeros(t.NP, np.uint8)
    n = lib().orc_generation(ctypes.byref(p), ctypes.byref(t.c), _p32(X), _p32(fit32),
                             _p64(fit64), gen, mode, acc.ctypes.data_as(_U8P))
    return acc, n


def trial(p, t, X, gen, i):
    u = np.zeros(t.D, np.float32)
    lib().orc_trial(ctypes.byref(p), ctypes.byref(t.c), _p32(X), gen, i, _p32(u))
    return u


def rank(fit32):
    fit32 = np.ascontiguousarray(fit32, np.float32)
    r = np.zeros(len(fit32), np.int32)
    lib().orc_rank(_p32(fit32), len(fit32), r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return r


def transfer_partner(p, t, n_tasks, gen):
    return lib().orc_transfer_partner(ctypes.byref(p), t, n_tasks, gen)


def transfer_in(p, t, pt, elites, X, fit32, fit64, gen, mode):
    elites = np.ascontiguousarray(elites, np.float32)
    return lib().orc_transfer_in(ctypes.byref(p), ctypes.byref(t.c), ctypes.byref(pt.c),
                                 _p32(elites), elites.shape[0], _p32(X), _p32(fit32),
                                 _p64(fit64), gen, mode)


def migration_due(p, gen):
    return bool(lib().orc_migration_due(ctypes.byref(p), gen))


def migration_count(p, NP):
    return lib().orc_migration_count(ctypes.byref(p), NP)


def migrate(p, t, X, fit32, fit64, mode):
    """Ring migration between the sub-islands of task t; returns replacements."""
    return lib().orc_migrate(ctypes.byref(p), ctypes.byref(t.c), _p32(X), _p32(fit32),
                             _p64(fit64), mode)


def run_threads(p, tasks, X, fit32, fit64, gen0, gens, mode, threads):
    n = len(tasks)
    arr = (Task * n)(*[t.c for t in tasks])
    xp = (_F32P * n)(*[_p32(a) for a in X])
    fp = (_F32P * n)(*[_p32(a) for a in fit32])
    dp = (_F64P * n)(*[_p64(a) for a in fit64])
    return lib().orc_run_threads(ctypes.byref(p), arr, n, xp, fp, dp, gen0, gens, mode, threads)


# ---- CVRP ----
def _i32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _u8(a):
    return a.ctypes.data_as(_U8P)


class CvrpInstance:
    """One seeded CVRP instance: coordinates, demands, rounded-Euclidean
    distances, capacity."""

    def __init__(self, seed, inst, n=100, capacity=50, x=None, y=None, demand=None):
        self.n, self.capacity, self.inst = n, capacity, inst
        if x is None:
            self.x = np.zeros(n + 1, np.int32)
            self.y = np.zeros(n + 1, np.int32)
            self.demand = np.zeros(n + 1, np.int32)
            lib().orc_cvrp_gen_instance(seed, inst, n, _i32(self.x), _i32(self.y), _i32(self.demand))
        else:
            self.x = np.ascontiguousarray(x, np.int32)
            self.y = np.ascontiguousarray(y, np.int32)
            self.demand = np.ascontiguousarray(demand, np.int32)
        self.dist = np.zeros((n + 1) * (n + 1), np.int32)
        lib().orc_cvrp_distances(n, _i32(self.x), _i32(self.y), _i32(self.dist))

    def split(self, perm, with_pred=False):
        perm = np.ascontiguousarray(perm, np.uint8)
        pred = np.zeros(self.n + 1, np.int32)
        c = lib().orc_cvrp_split(self.n, _i32(self.dist), _i32(self.demand), self.capacity,
                                 _u8(perm), _i32(pred))
        return (c, pred) if with_pred else c


def cvrp_params(seed=1, p_cross=0.9, p_swap=0.2, p_2opt=0.2, subislands=1, mig_interval=0,
                mig_count=0):
    return CvrpParams(seed, p_cross, p_swap, p_2opt, subislands, mig_interval, mig_count)


def cvrp_init_population(seed, inst, n, NP):
    pop = np.zeros((NP, n), np.uint8)
    lib().orc_cvrp_init_population(seed, inst, n, NP, _u8(pop))
    return pop


def cvrp_generation(p, ins, pop, cost, g):
    NP = pop.shape[0]
    return lib().orc_cvrp_generation(ctypes.byref(p), ins.inst, ins.n, NP, _i32(ins.dist),
                                     _i32(ins.demand), ins.capacity, _u8(pop), _i32(cost), g)


def cvrp_rank(cost):
    cost = np.ascontiguousarray(cost, np.int32)
    r = np.zeros(len(cost), np.int32)
    lib().orc_cvrp_rank(_i32(cost), len(cost), r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return r


def cvrp_transfer_in(ins, elites, pop, cost):
    elites = np.ascontiguousarray(elites, np.uint8)
    return lib().orc_cvrp_transfer_in(ins.n, pop.shape[0], _i32(ins.dist), _i32(ins.demand),
                                      ins.capacity, _u8(elites), elites.shape[0], _u8(pop),
                                      _i32(cost))


def cvrp_transfer_k(rate, NP):
    k = int(np.float32(np.float32(rate) * np.float32(NP)) + np.float32(0.5))
    return max(1, min(NP, k))


def cvrp_partner(seed, t, n_inst, gen):
    """Partner instance of instance t for the transfer at generation gen."""
    p = int(draw(seed, t, gen, 0, P_CVRP_PARTNER, 0)[0]) % (n_inst - 1)
    return p + 1 if p >= t else p


class CvrpReplay:
    """Host replay of the CVRP engine's schedule: generations with elite
    transfer every `interval` generations (exported at the end of the epoch
    that closes an interval, imported at the start of the next epoch)."""

    def __init__(self, seed, instances, NP, p_cross=0.9, p_swap=0.2, p_2opt=0.2,
                 interval=0, rate=0.1, subislands=1, mig_interval=0, mig_count=0):
        self.p = cvrp_params(seed, p_cross, p_swap, p_2opt, subislands, mig_interval, mig_count)
        self.seed, self.ins, self.NP = seed, instances, NP
        self.interval = interval if len(instances) > 1 else 0
        self.rate = rate
        self.pop = [cvrp_init_population(seed, t, ins.n, NP) for t, ins in enumerate(instances)]
        self.cost = [np.array([ins.split(r) for r in pop], np.int32)
                     for ins, pop in zip(instances, self.pop)]
        self.gen = 0
        self.elites = None
        self.accepted = 0

    def _export(self):
        k = cvrp_transfer_k(self.rate, self.NP)
        return [pop[cvrp_rank(cost)[:k]].copy() for pop, cost in zip(self.pop, self.cost)]

    def run(self, gens):
        left = gens
        T = len(self.ins)
        while left > 0:
            g = left
            if self.interval:
                if self.gen > 0 and self.gen % self.interval == 0 and self.elites is not None:
                    for t in range(T):
                        pt = cvrp_partner(self.seed, t, T, self.gen)
                        if self.ins[pt].n == self.ins[t].n:
                            self.accepted += cvrp_transfer_in(self.ins[t], self.elites[pt],
                                                              self.pop[t], self.cost[t])
                g = min(left, self.interval - self.gen % self.interval)
            for t in range(T):
                for k in range(1, g + 1):
                    cvrp_generation(self.p, self.ins[t], self.pop[t], self.cost[t], self.gen + k)
            self.gen += g
            left -= g
            if self.interval and self.gen % self.interval == 0:
                self.elites = self._export()
