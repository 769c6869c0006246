"""Python binding of the engine's C ABI (include/sgemtf.h).

A thin ctypes layer over sg-emtf_gb300/_build/libsgemtf.so: every call goes
straight to the CUDA library.  There is no Python or CPU implementation of
the engine behind it; if the library is missing, importing `lib()` raises.

    eng = Engine(Config(seed=1))
    eng.add_tasks([TaskDesc(function=SPHERE, dim=50, pop=64, rotation=ROTATION_SEEDED_QR)])
    eng.run(2000)
    f, x = eng.best(0)
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libsgemtf.so")
# the measurement build (phase clocks), loaded instead when SGEMTF_PHASE_CLOCKS=1
PHASES_LIB_PATH = os.path.join(PKG_DIR, "_build", "libsgemtf_phases.so")

# ---- enums (include/sgemtf.h) ----
OK, ERR_INVALID_ARG, ERR_OUT_OF_MEMORY, ERR_CUDA, ERR_DEVICE_TIMEOUT, ERR_STATE, \
    ERR_UNSUPPORTED, ERR_DEVICE_CHECK = range(8)
DE_RAND1_BIN, DE_CURRENT1_BIN, GA_SBX_PM = range(3)
ROT_FP32, ROT_TF32X3, ROT_AUTO, ROT_BF16X3 = range(4)
SPHERE, RASTRIGIN, ACKLEY, GRIEWANK, ROSENBROCK, SCHWEFEL, WEIERSTRASS = range(7)
FUNCTION_NAMES = ["sphere", "rastrigin", "ackley", "griewank", "rosenbrock", "schwefel",
                  "weierstrass"]
ROTATION_IDENTITY, ROTATION_SEEDED_QR, ROTATION_DENSE, ROTATION_DIAG = range(4)
FLAG_REF_GRIEWANK_NO_PRODUCT = 0x1
FLAG_REF_WEIERSTRASS_CONST = 0x2
FLAG_REF_ACKLEY_E = 0x4
FLAG_REF_BOXES = 0x8
FLAG_NO_RECHECK = 0x10
FLAG_RIGOROUS_WINDOW = 0x20
FLAG_NO_DIFF_RECHECK = 0x40
FLAG_TEST_LOST_COMPLETION = 0x80
SCHEDULE_AUTO, SCHEDULE_SINGLE, SCHEDULE_BUCKETS, SCHEDULE_PER_TASK, SCHEDULE_QUEUE = 0, 1, 2, 3, 4
MAX_DIM, MAX_POP = 128, 256  # fused islands; larger ones run the HBM-resident pipeline
MAX_DIM_LARGE, MAX_POP_LARGE = 1024, 512
NOALLOC_EXCHANGE_FLOATS = 1 << 19

EXPORTED = [
    "emt_config_default", "emt_function_from_reference", "emt_function_box",
    "emt_seeded_rotation", "emt_create",
    "emt_add_tasks", "emt_reset", "emt_run", "emt_run_noalloc", "emt_tune", "emt_time_rotation",
    "emt_get_phase_cycles",
    "emt_sync", "emt_get_best", "emt_get_best_all",
    "emt_get_population", "emt_set_population", "emt_get_task_info", "emt_get_task_params",
    "emt_evaluate", "emt_get_stats", "emt_snapshot_size", "emt_snapshot", "emt_restore",
    "emt_record_run", "emt_write_record", "emt_ano", "emt_write_fitness", "emt_write_para",
    "emt_service_create", "emt_service_submit", "emt_service_step", "emt_service_drain",
    "emt_service_batch", "emt_service_get_stats", "emt_service_last_error",
    "emt_service_destroy",
    "emt_last_error", "emt_status_string", "emt_destroy",
    "emt_cvrp_config_default", "emt_cvrp_create", "emt_cvrp_add_instances", "emt_cvrp_reset",
    "emt_cvrp_run", "emt_cvrp_sync", "emt_cvrp_get_best_all", "emt_cvrp_get_population",
    "emt_cvrp_get_instance", "emt_cvrp_evaluate", "emt_cvrp_get_stats", "emt_cvrp_last_error", "emt_cvrp_destroy",
]


class Config(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("F", ctypes.c_float), ("CR", ctypes.c_float), ("eta_c", ctypes.c_float),
                ("p_c", ctypes.c_float), ("eta_m", ctypes.c_float), ("p_m", ctypes.c_float),
                ("transfer_interval", ctypes.c_int32), ("transfer_rate", ctypes.c_float),
                ("transfer_mix", ctypes.c_float), ("flags", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("recheck_rel", ctypes.c_double),
                ("device", ctypes.c_int32), ("schedule", ctypes.c_int32),
                ("use_graph", ctypes.c_int32), ("subislands", ctypes.c_int32),
                ("migration_interval", ctypes.c_int32), ("migration_count", ctypes.c_int32),
                ("wait_limit_ms", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        lib().emt_config_default(ctypes.byref(self))
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class TaskDescC(ctypes.Structure):
    _fields_ = [("function", ctypes.c_int32), ("dim", ctypes.c_int32), ("pop", ctypes.c_int32),
                ("lo", ctypes.c_float), ("hi", ctypes.c_float), ("rotation", ctypes.c_int32),
                ("rotation_matrix", ctypes.POINTER(ctypes.c_double)),
                ("diag", ctypes.POINTER(ctypes.c_float)),
                ("shift", ctypes.POINTER(ctypes.c_float))]


class Stats(ctypes.Structure):
    _fields_ = [("evaluations", ctypes.c_uint64), ("generations", ctypes.c_uint64),
                ("rechecks", ctypes.c_uint64), ("recheck_flips", ctypes.c_uint64),
                ("transfers_accepted", ctypes.c_uint64), ("device_ms", ctypes.c_double),
                ("n_tasks", ctypes.c_int32), ("precision_used", ctypes.c_int32),
                ("recheck_differential", ctypes.c_uint64), ("anchor_rotations", ctypes.c_uint64),
                ("recheck_identical", ctypes.c_uint64), ("epoch_launches", ctypes.c_int32),
                ("schedule_used", ctypes.c_int32), ("migrations_accepted", ctypes.c_uint64),
                ("max_rel_err", ctypes.c_double), ("recheck_fp64_terms", ctypes.c_uint64)]


class TaskDesc:
    """One task; arrays are kept alive here until add_tasks copies them.  The
    fields are fixed at construction (the C descriptor is built once)."""

    def __init__(self, function, dim, pop, lo=0.0, hi=0.0, rotation=ROTATION_SEEDED_QR,
                 rotation_matrix=None, diag=None, shift=None):
        self.function, self.dim, self.pop = int(function), int(dim), int(pop)
        self.lo, self.hi, self.rotation = float(lo), float(hi), int(rotation)
        self.rotation_matrix = None if rotation_matrix is None else np.ascontiguousarray(
            rotation_matrix, np.float64)
        self.diag = None if diag is None else np.ascontiguousarray(diag, np.float32)
        self.shift = None if shift is None else np.ascontiguousarray(shift, np.float32)

        def ptr(a, t):
            return None if a is None else a.ctypes.data_as(ctypes.POINTER(t))
        self._c = TaskDescC(self.function, self.dim, self.pop, self.lo, self.hi, self.rotation,
                            ptr(self.rotation_matrix, ctypes.c_double),
                            ptr(self.diag, ctypes.c_float), ptr(self.shift, ctypes.c_float))

    def c(self):
        return self._c


class ServiceBatchInfo(ctypes.Structure):
    _fields_ = [("n_tasks", ctypes.c_int32), ("state", ctypes.c_int32),
                ("generations", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("arrival_ms", ctypes.c_double), ("admit_ms", ctypes.c_double),
                ("done_ms", ctypes.c_double)]


class ServiceStats(ctypes.Structure):
    _fields_ = [("batches_submitted", ctypes.c_int32), ("batches_done", ctypes.c_int32),
                ("tasks_done", ctypes.c_int64), ("mean_response_ms", ctypes.c_double),
                ("mean_solve_ms", ctypes.c_double), ("max_device_mem_mb", ctypes.c_double),
                ("mean_device_mem_mb", ctypes.c_double), ("evaluations", ctypes.c_uint64),
                ("rounds", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class CvrpConfig(ctypes.Structure):
    _fields_ = [("pop", ctypes.c_int32), ("p_cross", ctypes.c_float), ("p_swap", ctypes.c_float),
                ("p_2opt", ctypes.c_float), ("transfer_interval", ctypes.c_int32),
                ("transfer_rate", ctypes.c_float), ("seed", ctypes.c_uint64),
                ("device", ctypes.c_int32), ("subislands", ctypes.c_int32),
                ("migration_interval", ctypes.c_int32), ("migration_count", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 4)]

    def __init__(self, **kw):
        super().__init__()
        lib().emt_cvrp_config_default(ctypes.byref(self))
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class CvrpInstanceC(ctypes.Structure):
    _fields_ = [("customers", ctypes.c_int32), ("capacity", ctypes.c_int32),
                ("x", ctypes.POINTER(ctypes.c_int32)), ("y", ctypes.POINTER(ctypes.c_int32)),
                ("demand", ctypes.POINTER(ctypes.c_int32))]


class EngineError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (status_string(status), status, message))
        self.status = status


_lib = None


def lib():
    """The loaded CUDA library.  Raises if it was not built: there is no
    fallback implementation."""
    global _lib
    if _lib is None:
        path = PHASES_LIB_PATH if os.environ.get("SGEMTF_PHASE_CLOCKS") == "1" else LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError("%s not built: run `python sg-emtf_gb300/build.py` "
                               "(--phases for the measurement build)" % os.path.basename(path))
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        i32 = ctypes.c_int32
        f32p = ctypes.POINTER(ctypes.c_float)
        L.emt_config_default.argtypes = [ctypes.POINTER(Config)]
        L.emt_config_default.restype = None
        L.emt_function_from_reference.argtypes = [i32]
        L.emt_function_from_reference.restype = i32
        L.emt_function_box.argtypes = [i32, i32, f32p, f32p]
        L.emt_seeded_rotation.argtypes = [ctypes.c_uint64, i32, i32, ctypes.POINTER(ctypes.c_double)]
        L.emt_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.emt_add_tasks.argtypes = [vp, i32, ctypes.POINTER(TaskDescC)]
        L.emt_reset.argtypes = [vp, vp]
        L.emt_run.argtypes = [vp, i32, vp]
        L.emt_run_noalloc.argtypes = [vp, i32, vp]
        L.emt_tune.argtypes = [vp, i32, vp, ctypes.POINTER(ctypes.c_int32)]
        L.emt_time_rotation.argtypes = [vp, i32, vp, ctypes.POINTER(ctypes.c_float)]
        L.emt_get_phase_cycles.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), i32]
        L.emt_sync.argtypes = [vp]
        L.emt_get_best.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_double), f32p]
        L.emt_get_best_all.argtypes = [vp, f32p]
        L.emt_get_population.argtypes = [vp, i32, f32p, f32p]
        L.emt_set_population.argtypes = [vp, i32, f32p]
        L.emt_get_task_params.argtypes = [vp, i32, f32p, f32p]
        L.emt_get_task_info.argtypes = [vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                        ctypes.POINTER(i32)]
        L.emt_record_run.argtypes = [vp, i32, i32, vp, f32p]
        L.emt_write_record.argtypes = [ctypes.c_char_p, i32, i32, f32p]
        L.emt_ano.argtypes = [i32, i32, i32, f32p, f32p]
        L.emt_write_fitness.argtypes = [vp, ctypes.c_char_p]
        L.emt_write_para.argtypes = [vp, ctypes.c_char_p]
        L.emt_service_create.argtypes = [ctypes.POINTER(Config), i32, i32, ctypes.POINTER(vp)]
        L.emt_service_submit.argtypes = [vp, i32, ctypes.POINTER(TaskDescC), ctypes.c_double,
                                         ctypes.POINTER(i32)]
        L.emt_service_step.argtypes = [vp, ctypes.POINTER(i32)]
        L.emt_service_drain.argtypes = [vp]
        L.emt_service_batch.argtypes = [vp, i32, ctypes.POINTER(ServiceBatchInfo), f32p]
        L.emt_service_get_stats.argtypes = [vp, ctypes.POINTER(ServiceStats)]
        L.emt_service_last_error.argtypes = [vp]
        L.emt_service_last_error.restype = ctypes.c_char_p
        L.emt_service_destroy.argtypes = [vp]
        L.emt_service_destroy.restype = None
        L.emt_evaluate.argtypes = [vp, i32, i32, f32p, f32p, f32p]
        L.emt_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.emt_snapshot_size.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
        L.emt_snapshot.argtypes = [vp, vp, ctypes.c_size_t]
        L.emt_restore.argtypes = [vp, vp, ctypes.c_size_t]
        L.emt_last_error.argtypes = [vp]
        L.emt_last_error.restype = ctypes.c_char_p
        L.emt_status_string.argtypes = [ctypes.c_int]
        L.emt_status_string.restype = ctypes.c_char_p
        L.emt_destroy.argtypes = [vp]
        L.emt_destroy.restype = None
        i32p = ctypes.POINTER(ctypes.c_int32)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        L.emt_cvrp_config_default.argtypes = [ctypes.POINTER(CvrpConfig)]
        L.emt_cvrp_config_default.restype = None
        L.emt_cvrp_create.argtypes = [ctypes.POINTER(CvrpConfig), ctypes.POINTER(vp)]
        L.emt_cvrp_add_instances.argtypes = [vp, i32, ctypes.POINTER(CvrpInstanceC)]
        L.emt_cvrp_reset.argtypes = [vp, vp]
        L.emt_cvrp_run.argtypes = [vp, i32, vp]
        L.emt_cvrp_sync.argtypes = [vp]
        L.emt_cvrp_get_best_all.argtypes = [vp, i32p]
        L.emt_cvrp_get_population.argtypes = [vp, i32, u8p, i32p]
        L.emt_cvrp_get_instance.argtypes = [vp, i32, i32p, i32p, i32p, i32p]
        L.emt_cvrp_evaluate.argtypes = [vp, i32, i32, u8p, i32p]
        L.emt_cvrp_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.emt_cvrp_last_error.argtypes = [vp]
        L.emt_cvrp_last_error.restype = ctypes.c_char_p
        L.emt_cvrp_destroy.argtypes = [vp]
        L.emt_cvrp_destroy.restype = None
        _lib = L
    return _lib


def status_string(s):
    return lib().emt_status_string(s).decode()


def seeded_rotation(seed, task, dim):
    """emt_seeded_rotation: the FP64 rotation EMT_ROTATION_SEEDED_QR gives task
    `task` of a handle with this seed (host only)."""
    q = np.zeros((dim, dim), np.float64)
    rc = lib().emt_seeded_rotation(int(seed), int(task), int(dim),
                                   q.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc:
        raise EngineError(rc, "seeded_rotation")
    return q


def function_box(fid, reference_boxes=False):
    lo, hi = ctypes.c_float(), ctypes.c_float()
    rc = lib().emt_function_box(fid, int(reference_boxes), ctypes.byref(lo), ctypes.byref(hi))
    if rc:
        raise EngineError(rc, "function_box")
    return lo.value, hi.value


def ano(records):
    """Average normalised objective of runs x tasks x cols records (cols - 1
    recording points, then the near-worst), data process/源.cpp:172-203."""
    r = np.ascontiguousarray(records, np.float32)
    runs, tasks, cols = r.shape
    out = np.zeros(cols - 1, np.float32)
    rc = lib().emt_ano(runs, tasks, cols, _f32(r), _f32(out))
    if rc:
        raise EngineError(rc, "emt_ano: %s" % status_string(rc))
    return out


def write_record(path, record):
    """Appends one run's tasks x cols record and a blank line (data_record_*)."""
    r = np.ascontiguousarray(record, np.float32)
    rc = lib().emt_write_record(os.fsencode(path), r.shape[0], r.shape[1], _f32(r))
    if rc:
        raise EngineError(rc, "emt_write_record: %s" % status_string(rc))


def _f32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Engine:
    """One emt_handle: a set of tasks resident on one GPU."""

    def __init__(self, config=None, **kw):
        self.config = config if config is not None else Config(**kw)
        self._h = ctypes.c_void_p()
        rc = lib().emt_create(ctypes.byref(self.config), ctypes.byref(self._h))
        if rc:
            raise EngineError(rc, "emt_create")
        self.tasks = []

    def _check(self, rc, what):
        if rc:
            raise EngineError(rc, "%s: %s" % (what, lib().emt_last_error(self._h).decode()))

    def add_tasks(self, descs):
        descs = list(descs)
        arr = (TaskDescC * len(descs)).from_buffer_copy(b"".join(bytes(d.c()) for d in descs)) \
            if descs else (TaskDescC * 0)()
        self._check(lib().emt_add_tasks(self._h, len(descs), arr), "emt_add_tasks")
        self.tasks.extend(descs)

    def reset(self, stream=None):
        self._check(lib().emt_reset(self._h, stream), "emt_reset")

    def run(self, generations, stream=None, sync=True):
        self._check(lib().emt_run(self._h, int(generations), stream), "emt_run")
        if sync:
            self.sync()

    def tune(self, generations, stream=None):
        """emt_tune: time the launch schedules on real generations, keep the
        fastest; returns schedule | 0x100 when graph replay won."""
        out = ctypes.c_int32(0)
        self._check(lib().emt_tune(self._h, int(generations), stream, ctypes.byref(out)), "emt_tune")
        return out.value

    def time_rotation(self, reps, stream=None):
        """Mean duration (ms) of one rotation-GEMM launch (large islands)."""
        out = ctypes.c_float(0.0)
        self._check(lib().emt_time_rotation(self._h, int(reps), stream, ctypes.byref(out)),
                    "emt_time_rotation")
        return out.value

    def run_noalloc(self, generations, stream=None, sync=True):
        """emt_run_noalloc: allocates nothing (needs a prior reset())."""
        self._check(lib().emt_run_noalloc(self._h, int(generations), stream), "emt_run_noalloc")
        if sync:
            self.sync()

    def sync(self):
        self._check(lib().emt_sync(self._h), "emt_sync")

    # "rotate" is the FP32 rotation, or the tensor-core forms' operand hand-off;
    # their MMAs, the wait for them and the accumulator drain follow
    PHASES = ["other", "build", "rotate", "eval", "select", "recheck", "mma_issue", "mma_wait",
              "drain"]
    ROTATION_PHASES = ("rotate", "mma_issue", "mma_wait", "drain")

    def phase_cycles(self):
        """emt_get_phase_cycles (measurement build only): SM cycles per phase."""
        out = (ctypes.c_uint64 * len(self.PHASES))()
        self._check(lib().emt_get_phase_cycles(self._h, out, len(self.PHASES)),
                    "emt_get_phase_cycles")
        return dict(zip(self.PHASES, [int(v) for v in out]))

    def _dim(self, task):
        if 0 <= task < len(self.tasks):
            return self.tasks[task].dim, self.tasks[task].pop
        return 1, 1  # the library reports the bad index

    def best(self, task):
        x = np.zeros(self._dim(task)[0], np.float32)
        f = ctypes.c_double()
        self._check(lib().emt_get_best(self._h, task, ctypes.byref(f), _f32(x)), "emt_get_best")
        return f.value, x

    def best_all(self):
        out = np.zeros(len(self.tasks), np.float32)
        self._check(lib().emt_get_best_all(self._h, _f32(out)), "emt_get_best_all")
        return out

    def population(self, task):
        D, NP = self._dim(task)
        x = np.zeros((NP, D), np.float32)
        f = np.zeros(NP, np.float32)
        self._check(lib().emt_get_population(self._h, task, _f32(x), _f32(f)),
                    "emt_get_population")
        return x, f

    def set_population(self, task, x):
        x = np.ascontiguousarray(x, np.float32)
        self._check(lib().emt_set_population(self._h, task, _f32(x)), "emt_set_population")

    def task_info(self, task):
        f, d, p = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(lib().emt_get_task_info(self._h, task, ctypes.byref(f), ctypes.byref(d),
                                            ctypes.byref(p)), "emt_get_task_info")
        return f.value, d.value, p.value

    def record_run(self, generations, interval, stream=None):
        """Runs in steps of `interval`; returns tasks x (generations/interval + 2):
        best FP32 fitness at each recording point, then the near-worst."""
        cols = generations // interval + 2 if interval > 0 else 2
        rec = np.zeros((len(self.tasks), cols), np.float32)
        self._check(lib().emt_record_run(self._h, generations, interval, stream, _f32(rec)),
                    "emt_record_run")
        return rec

    def write_fitness(self, path):
        self._check(lib().emt_write_fitness(self._h, os.fsencode(path)), "emt_write_fitness")

    def write_para(self, path):
        self._check(lib().emt_write_para(self._h, os.fsencode(path)), "emt_write_para")

    def task_params(self, task):
        D, _ = self._dim(task)
        Q = np.zeros((D, D), np.float32)
        o = np.zeros(D, np.float32)
        self._check(lib().emt_get_task_params(self._h, task, _f32(Q), _f32(o)),
                    "emt_get_task_params")
        return Q, o

    def evaluate(self, task, x, want_z=False):
        x = np.ascontiguousarray(np.atleast_2d(x), np.float32)
        n = x.shape[0]
        f = np.zeros(n, np.float32)
        z = np.zeros_like(x) if want_z else None
        self._check(lib().emt_evaluate(self._h, task, n, _f32(x), _f32(f),
                                       _f32(z) if want_z else None), "emt_evaluate")
        return (f, z) if want_z else f

    def stats(self):
        s = Stats()
        self._check(lib().emt_get_stats(self._h, ctypes.byref(s)), "emt_get_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def snapshot(self):
        n = ctypes.c_size_t()
        self._check(lib().emt_snapshot_size(self._h, ctypes.byref(n)), "emt_snapshot_size")
        buf = ctypes.create_string_buffer(n.value)
        self._check(lib().emt_snapshot(self._h, buf, n.value), "emt_snapshot")
        return buf.raw

    def restore(self, blob):
        buf = ctypes.create_string_buffer(blob, len(blob))
        self._check(lib().emt_restore(self._h, buf, len(blob)), "emt_restore")

    def close(self):
        if self._h:
            lib().emt_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Service:
    """Service mode (emt_service_*): batches of tasks that arrive over time,
    each served by its own handle and stream, concurrently on one GPU."""

    def __init__(self, config=None, generations=1000, epoch=50):
        self.config = config or Config()
        self._s = ctypes.c_void_p()
        self._tasks = {}
        rc = lib().emt_service_create(ctypes.byref(self.config), generations, epoch,
                                      ctypes.byref(self._s))
        if rc:
            raise EngineError(rc, "emt_service_create: %s" % status_string(rc))

    def _check(self, rc, what):
        if rc:
            raise EngineError(rc, "%s: %s" % (what, lib().emt_service_last_error(self._s).decode()))

    def submit(self, tasks, arrival_ms=0.0):
        arr = (TaskDescC * len(tasks))(*[t.c() for t in tasks])
        b = ctypes.c_int32()
        self._check(lib().emt_service_submit(self._s, len(tasks), arr, float(arrival_ms),
                                             ctypes.byref(b)), "emt_service_submit")
        self._tasks[b.value] = len(tasks)
        return b.value

    def step(self):
        left = ctypes.c_int32()
        self._check(lib().emt_service_step(self._s, ctypes.byref(left)), "emt_service_step")
        return left.value

    def drain(self):
        self._check(lib().emt_service_drain(self._s), "emt_service_drain")

    def batch(self, b):
        info = ServiceBatchInfo()
        self._check(lib().emt_service_batch(self._s, b, ctypes.byref(info), None),
                    "emt_service_batch")
        d = {k: getattr(info, k) for k, _ in ServiceBatchInfo._fields_ if k != "reserved"}
        best = None
        if info.state == 2:
            best = np.zeros(info.n_tasks, np.float32)
            self._check(lib().emt_service_batch(self._s, b, None, _f32(best)), "emt_service_batch")
        return d, best

    def stats(self):
        st = ServiceStats()
        self._check(lib().emt_service_get_stats(self._s, ctypes.byref(st)), "emt_service_get_stats")
        return {k: getattr(st, k) for k, _ in ServiceStats._fields_ if k != "reserved"}

    def close(self):
        if self._s:
            lib().emt_service_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CvrpEngine:
    """One emt_cvrp_handle: CVRP instances, one island of permutations each."""

    def __init__(self, config=None, **kw):
        self.config = config if config is not None else CvrpConfig(**kw)
        self._h = ctypes.c_void_p()
        rc = lib().emt_cvrp_create(ctypes.byref(self.config), ctypes.byref(self._h))
        if rc:
            raise EngineError(rc, "emt_cvrp_create")
        self.sizes = []

    def _check(self, rc, what):
        if rc:
            raise EngineError(rc, "%s: %s" % (what, lib().emt_cvrp_last_error(self._h).decode()))

    def add_instances(self, specs):
        """specs: (customers, capacity) for seeded instances, or
        (customers, capacity, x, y, demand) with n + 1 entries each."""
        keep, arr = [], []
        for sp in specs:
            n, cap = int(sp[0]), int(sp[1])
            if len(sp) > 2:
                x, y, d = (np.ascontiguousarray(a, np.int32) for a in sp[2:5])
                keep += [x, y, d]
                p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
                arr.append(CvrpInstanceC(n, cap, p(x), p(y), p(d)))
            else:
                arr.append(CvrpInstanceC(n, cap, None, None, None))
        carr = (CvrpInstanceC * len(arr))(*arr)
        self._check(lib().emt_cvrp_add_instances(self._h, len(arr), carr), "emt_cvrp_add_instances")
        self.sizes += [int(sp[0]) for sp in specs]

    def reset(self, stream=None):
        self._check(lib().emt_cvrp_reset(self._h, stream), "emt_cvrp_reset")

    def run(self, generations, stream=None, sync=True):
        self._check(lib().emt_cvrp_run(self._h, int(generations), stream), "emt_cvrp_run")
        if sync:
            self.sync()

    def sync(self):
        self._check(lib().emt_cvrp_sync(self._h), "emt_cvrp_sync")

    def population(self, inst):
        n = self.sizes[inst] if 0 <= inst < len(self.sizes) else 1
        perms = np.zeros((self.config.pop, n), np.uint8)
        costs = np.zeros(self.config.pop, np.int32)
        self._check(lib().emt_cvrp_get_population(
            self._h, inst, perms.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
            costs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))), "emt_cvrp_get_population")
        return perms, costs

    def best_all(self):
        out = np.zeros(len(self.sizes), np.int32)
        self._check(lib().emt_cvrp_get_best_all(self._h, out.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int32))), "emt_cvrp_get_best_all")
        return out

    def instance(self, inst):
        n = self.sizes[inst]
        x, y, d = (np.zeros(n + 1, np.int32) for _ in range(3))
        dist = np.zeros((n + 1) * (n + 1), np.int32)
        p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        self._check(lib().emt_cvrp_get_instance(self._h, inst, p(x), p(y), p(d), p(dist)),
                    "emt_cvrp_get_instance")
        return x, y, d, dist

    def evaluate(self, inst, perms):
        """Device costs of giant tours (rows of customer ids 1..n)."""
        perms = np.ascontiguousarray(perms, np.uint8)
        out = np.zeros(perms.shape[0], np.int32)
        self._check(lib().emt_cvrp_evaluate(
            self._h, inst, perms.shape[0], perms.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))), "emt_cvrp_evaluate")
        return out

    def stats(self):
        st = Stats()
        self._check(lib().emt_cvrp_get_stats(self._h, ctypes.byref(st)), "emt_cvrp_get_stats")
        return {k: getattr(st, k) for k, _ in Stats._fields_}

    def close(self):
        if self._h:
            lib().emt_cvrp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
