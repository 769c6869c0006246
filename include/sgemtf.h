/*
 * sgemtf.h -- C ABI of the GB300 evolutionary-multitasking engine.
 *
 * One handle owns a set of optimisation tasks.  Each task is one island of
 * NP individuals in D dimensions that evolves on one benchmark function of a
 * shifted, rotated argument z = Q (x - o).  All populations stay resident on
 * one GPU; one emt_run() call advances every task by a number of generations
 * (DE/rand/1/bin, DE/current/1/bin or SBX + polynomial-mutation GA), with
 * periodic elite transfer between tasks.
 *
 * The reference program has no library interface: its replaceable unit is the
 * per-task host function
 *     void iter(int task_idx, int cthread_idx, cudaStream_t* streams)
 *         (proposed model/SG-EMTF.cu:1646, SG-EMTF_DE.cu:1576)
 * with the kernels it launches.  Each entry point below names the reference
 * code it replaces.
 *
 * Conventions
 *   - Every call returns EMT_OK (0) or an emt_status error code; the message
 *     of the last failure on a handle is in emt_last_error().
 *   - The handle owns all device memory.  Caller buffers are HOST memory and
 *     are copied in or out; no device pointer crosses this interface except
 *     the optional CUDA stream (a cudaStream_t passed as void*; NULL = the
 *     legacy default stream).
 *   - A handle is used by one host thread at a time.  Calls on different
 *     handles are independent: apart from emt_run_noalloc's shared device
 *     array, the library keeps no global mutable state.
 *   - Random numbers come from a counter-based Philox4x32-10 stream keyed by
 *     emt_config.seed, so a run is reproducible bit for bit: the same seed and
 *     call sequence give the same populations on every run.
 *
 * Function ids follow the order sphere, rastrigin, ackley, griewank,
 * rosenbrock, schwefel, weierstrass.  The reference numbers the same functions
 * 0 Sphere, 1 Rosenbrock, 2 Ackley, 3 Rastrigin, 4 Griewank, 5 Weierstrass,
 * 6 Schwefel (proposed model/SG-EMTF.cu:917-1101); emt_function_from_reference
 * converts.
 */
#ifndef SGEMTF_H
#define SGEMTF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMT_ABI_VERSION 1

#if defined(__GNUC__)
#define EMT_API __attribute__((visibility("default")))
#else
#define EMT_API
#endif

/* Opaque engine handle; owns the device state of its tasks. */
typedef struct emt_handle emt_handle_t;

typedef enum emt_status {
  EMT_OK = 0,
  EMT_ERR_INVALID_ARG = 1,   /* bad pointer, size or enum value           */
  EMT_ERR_OUT_OF_MEMORY = 2, /* a device or host allocation failed         */
  EMT_ERR_CUDA = 3,          /* a CUDA runtime call or kernel failed       */
  EMT_ERR_DEVICE_TIMEOUT = 4,/* a bounded device-side wait gave up         */
  EMT_ERR_STATE = 5,         /* call out of order (e.g. no tasks yet)      */
  EMT_ERR_UNSUPPORTED = 6,   /* valid request this build cannot serve      */
  EMT_ERR_DEVICE_CHECK = 7   /* a kernel's own bounds/descriptor check fired */
} emt_status;

typedef enum emt_algorithm {
  EMT_DE_RAND1_BIN = 0,    /* v = x_r1 + F (x_r2 - x_r3), binomial crossover  */
  EMT_DE_CURRENT1_BIN = 1, /* v = x_i  + F (x_r2 - x_r3): the reference's DE,
                              proposed model/SG-EMTF_DE.cu:547-600,474-495    */
  EMT_GA_SBX_PM = 2        /* SBX crossover + polynomial mutation: the
                              reference's GA, SG-EMTF.cu:548-750,772-831      */
} emt_algorithm;

/* Arithmetic of the rotation z = Q (x - o) behind every evaluation. */
typedef enum emt_precision {
  EMT_ROT_FP32 = 0,   /* FP32 FMA on CUDA cores                          */
  EMT_ROT_TF32X3 = 1, /* tcgen05 tensor cores, kind::tf32: hi/lo TF32 split
                         of both operands (both parts rounded to nearest),
                         FP32 accumulation in tensor memory, hi.hi apart
                         from hi.lo + lo.hi + lo.lo, added in FP32         */
  EMT_ROT_AUTO = 2,   /* the tensor-core form when the device and the
                         islands allow it (BF16X3), else FP32              */
  EMT_ROT_BF16X3 = 3  /* tcgen05 tensor cores, kind::f16: each operand split
                         exactly into three BF16 parts (x = x0 + x1 + x2),
                         eight of the nine products of parts (x2.y2, at most
                         2^-32 of x0.y0, is dropped), every product exact;
                         x0.y0 accumulated apart from the other seven in
                         FP32 tensor memory.  Islands of D <= 128; a
                         large-island handle runs TF32X3 instead.  (A plain
                         one-part TF32 form is not offered: its 2^-11
                         operand rounding is ~100x the 1e-5 tolerance.)     */
} emt_precision;

typedef enum emt_function {
  EMT_SPHERE = 0,
  EMT_RASTRIGIN = 1,
  EMT_ACKLEY = 2,
  EMT_GRIEWANK = 3,
  EMT_ROSENBROCK = 4,
  EMT_SCHWEFEL = 5,
  EMT_WEIERSTRASS = 6,
  EMT_NUM_FUNCTIONS = 7
} emt_function;

typedef enum emt_rotation {
  EMT_ROTATION_IDENTITY = 0,  /* z = x - o                                  */
  EMT_ROTATION_SEEDED_QR = 1, /* Q = orthogonal factor of the FP64 QR of a
                                 seeded N(0,1) D x D matrix, stored FP32     */
  EMT_ROTATION_DENSE = 2,     /* Q given by the caller (FP64, row-major)    */
  EMT_ROTATION_DIAG = 3       /* z = m .* (x - o): the reference's
                                 z = M[d] * (x + b[d]) with o = -b
                                 (SG-EMTF.cu:181-195, use at :922)          */
} emt_rotation;

/* Reference-compatibility switches (emt_config.flags). */
#define EMT_FLAG_REF_GRIEWANK_NO_PRODUCT 0x1u /* GA file drops the product
                                                 term (SG-EMTF.cu:1029)      */
#define EMT_FLAG_REF_WEIERSTRASS_CONST 0x2u   /* offset computed as the host
                                                 code does, PI = 3.1415926,
                                                 float cosf (SG-EMTF.cu:354-361) */
#define EMT_FLAG_REF_ACKLEY_E 0x4u            /* E = 2.718282 (SG-EMTF.cu:54) */
#define EMT_FLAG_REF_BOXES 0x8u               /* box table of SG-EMTF.cu:197-214 */
#define EMT_FLAG_NO_RECHECK 0x10u             /* select on FP32 fitness only */
#define EMT_FLAG_RIGOROUS_WINDOW 0x20u        /* Weierstrass near-tie window from the
                                                 rigorous 3^k conditioning bound */
#define EMT_FLAG_NO_DIFF_RECHECK 0x40u        /* re-check near ties by FP64-class values
                                                 only, without the differential form */
#define EMT_FLAG_TEST_LOST_COMPLETION 0x80u   /* test switch, tensor-core form: the
                                                 rotation issues no MMA and no commit, so
                                                 its bounded wait runs out; the epoch stops
                                                 and emt_sync returns EMT_ERR_DEVICE_CHECK */

typedef struct emt_config {
  int32_t algorithm;         /* emt_algorithm                                */
  int32_t precision;         /* emt_precision                                */
  float F;                   /* DE scale factor (reference 0.5, SG-EMTF_DE.cu:43) */
  float CR;                  /* DE crossover rate (reference 0.6, :39)       */
  float eta_c;               /* SBX distribution index (reference 2, SG-EMTF.cu:46) */
  float p_c;                 /* per-gene SBX probability (reference 1, :718)  */
  float eta_m;               /* PM distribution index (reference 5, :49)      */
  float p_m;                 /* per-gene PM probability; < 0 means 1/D (reference 1, :555) */
  int32_t transfer_interval; /* generations between elite transfers; 0 = off */
  float transfer_rate;       /* fraction of the island sent (reference 50/512) */
  float transfer_mix;        /* probability that a candidate gene comes from
                                the partner (reference 1 - 0.6, SG-EMTF.cu:1551) */
  uint32_t flags;            /* EMT_FLAG_*                                    */
  uint64_t seed;             /* Philox key                                    */
  double recheck_rel;        /* FP64 re-check window, relative to the fitness
                                scale; 0 = library default                   */
  int32_t device;            /* CUDA device ordinal                           */
  int32_t schedule;          /* emt_schedule: how an epoch's islands are launched */
  int32_t use_graph;         /* 1: emt_run captures its epoch sequence in a CUDA
                                graph once and replays it when it recurs        */
  /* Sub-islands (the reference's slots of one block, IslandMigration,
   * SG-EMTF.cu:1138-1218): each island of NP members splits into subislands
   * groups of NP / subislands (NP must divide; 0 or 1 = one group).  DE and GA
   * draw partners within the member's own group.  Before the trials of
   * generation g, when g > 1 and (g - 1) % migration_interval == 0, the r-th
   * best of group s replaces the r-th worst of group s + 1 (mod subislands),
   * r < migration_count, when strictly better, all from the pre-migration
   * state; near ties are decided like any selection. */
  int32_t subislands;
  int32_t migration_interval; /* generations between migrations; 0 = none       */
  int32_t migration_count;    /* members each group sends; 0 = NP/subislands/8,
                                 at least 1; 2 * count <= NP / subislands       */
  int32_t wait_limit_ms;      /* limit of every bounded device-side wait (TMA and
                                 MMA completion on mbarriers); 0 = 2000 ms.  A
                                 wait that runs out sets the kernel's error word
                                 (emt_sync: EMT_ERR_DEVICE_CHECK)              */
  int32_t reserved;
} emt_config;

/* How emt_run launches an epoch's islands (results are identical).  The
 * reference launches one kernel per task from one host thread per task on 8
 * streams (SG-EMTF.cu:1660-1676, 1839-1915); EMT_SCHEDULE_PER_TASK keeps that
 * shape for comparison. */
typedef enum emt_schedule {
  EMT_SCHEDULE_AUTO = 0,     /* tuned by emt_tune, else BUCKETS for mixed shapes */
  EMT_SCHEDULE_SINGLE = 1,   /* one launch over every island, shared memory sized
                                for the largest, longest islands first         */
  EMT_SCHEDULE_BUCKETS = 2,  /* islands grouped by resident CTAs per SM, one
                                launch per group with its own shared-memory size,
                                groups concurrent on side streams               */
  EMT_SCHEDULE_PER_TASK = 3, /* one single-CTA launch per island, 8 streams     */
  EMT_SCHEDULE_QUEUE = 4     /* one persistent launch, SMs x resident CTAs, each
                                CTA taking the next island (longest first) from
                                a device work queue                            */
} emt_schedule;

typedef struct emt_task_desc {
  int32_t function;              /* emt_function                             */
  int32_t dim;                   /* D, 1..EMT_MAX_DIM                        */
  int32_t pop;                   /* NP, 4..EMT_MAX_POP                       */
  float lo, hi;                  /* box; lo >= hi selects the function's box */
  int32_t rotation;              /* emt_rotation                             */
  const double* rotation_matrix; /* DENSE: D*D row-major, else ignored      */
  const float* diag;             /* DIAG: D scale factors, else ignored     */
  const float* shift;            /* D floats; NULL draws o ~ U(0.8 * box)   */
} emt_task_desc;

/* Islands with D <= EMT_MAX_FUSED_DIM and NP <= EMT_MAX_FUSED_POP run in the
 * fused kernel (one CTA per island, state in shared memory).  A handle
 * holding any task with a larger D (up to EMT_MAX_DIM, e.g. 256 tasks of
 * D = 1000) or a larger NP (up to EMT_MAX_POP, the reference's 512-member
 * islands, SG-EMTF.cu:29) runs every island as an HBM-resident pipeline
 * instead: trial kernel, rotation GEMM (tcgen05 tensor cores or FP32 CUDA
 * cores), evaluation, selection; emt_evaluate and emt_run_noalloc return
 * EMT_ERR_UNSUPPORTED for such a handle. */
#define EMT_MAX_DIM 1024
#define EMT_MAX_FUSED_DIM 128
#define EMT_MAX_POP 512
#define EMT_MAX_FUSED_POP 256

typedef struct emt_stats {
  uint64_t evaluations;       /* fitness evaluations on the device         */
  uint64_t generations;       /* sum over tasks of generations completed    */
  uint64_t rechecks;          /* selections re-decided in FP64              */
  uint64_t recheck_flips;     /* of those, how many FP32 would have got wrong */
  uint64_t transfers_accepted;/* elite-transfer candidates that replaced a member */
  double device_ms;           /* device time of the last emt_run            */
  int32_t n_tasks;
  int32_t precision_used;     /* emt_precision actually run                 */
  uint64_t recheck_differential; /* re-checks decided by the differential form,
                                    without FP64-class values               */
  uint64_t anchor_rotations;  /* compensated member rotations computed for it */
  uint64_t recheck_identical; /* re-checks of a trial bit-identical to its parent */
  int32_t epoch_launches;     /* kernel launches per epoch under the schedule in use */
  int32_t schedule_used;      /* emt_schedule in use | 0x100 when graphs replay  */
  uint64_t migrations_accepted; /* sub-island migrants that replaced a member   */
  double max_rel_err;         /* largest |f32 - f64| / scale over the tasks' best
                                 members (scale: the sum of |sub-terms| the FP32
                                 evaluation states); 0 before emt_reset        */
  uint64_t recheck_fp64_terms; /* Weierstrass near ties whose FP32-term values
                                  were closer than their error bound, decided
                                  with every term in double precision         */
} emt_stats;

/* Fills *cfg with DE/rand/1/bin, F = 0.5, CR = 0.9, SBX eta 15 / p_c 0.9,
 * PM eta 15 / p_m = 1/D, no transfer, FP32 rotation, seed 1. */
EMT_API void emt_config_default(emt_config* cfg);

/* Reference function number (SG-EMTF.cu:917-1101) -> emt_function, or -1. */
EMT_API int32_t emt_function_from_reference(int32_t reference_type);

/* The function's box [lo, hi]; reference_boxes != 0 gives SG-EMTF.cu:197-214. */
EMT_API int emt_function_box(int32_t function, int32_t reference_boxes, float* lo, float* hi);

/* The rotation EMT_ROTATION_SEEDED_QR gives task number `task` (its index in
 * the handle) of a handle configured with `seed`: the orthogonal factor of
 * the FP64 Householder QR of a seeded N(0,1) dim x dim matrix, row-major in
 * q (dim * dim doubles), before the handle rounds it to FP32.  Host code
 * only; no device is needed.  No reference counterpart: the reference's
 * rotation is a diagonal scale (SG-EMTF.cu:181-195). */
EMT_API int emt_seeded_rotation(uint64_t seed, int32_t task, int32_t dim, double* q);

/* Replaces the reference's initialization() (SG-EMTF.cu:293-380): validates
 * the configuration and binds the device.  No task exists yet. */
EMT_API int emt_create(const emt_config* cfg, emt_handle_t** out);

/* Adds n tasks (para_init + pop_init, SG-EMTF.cu:146-195): copies the
 * rotation and shift, generates what the descriptors leave to the seed.
 * Before emt_reset the tasks simply join the handle.  On a handle that has
 * been reset or run, the tasks join the running handle (the reference's
 * batch arrivals, SG-EMTF.cu:1842-1912): the running islands keep their
 * state and generation counter, the new islands get the initial populations
 * a handle created with every task would draw and evolve from the handle's
 * next generation on (transfer partners are then drawn over all tasks).  The
 * call synchronises the handle's stream.  If the grown handle is refused
 * (e.g. an explicit tensor-core form the new islands do not fit), the call
 * returns that error and the handle keeps its running islands unchanged. */
EMT_API int emt_add_tasks(emt_handle_t* h, int32_t n, const emt_task_desc* tasks);

/* Draws every task's initial population from the seed and evaluates it
 * (pop_init + evaluate, SG-EMTF.cu:146-159,1428-1479).  emt_run calls it
 * on first use; calling it again restarts every task from generation 0. */
EMT_API int emt_reset(emt_handle_t* h, void* stream);

/* Advances every task by `generations` generations: the per-task loop of
 * iter() (SG-EMTF.cu:1669-1723) over GeneticOpera (:1289-1426), popSort
 * (:462-486) and knowledgeTransfer (:1514-1591), for all tasks at once.
 * Asynchronous on `stream`; emt_sync waits and reports device errors. */
EMT_API int emt_run(emt_handle_t* h, int32_t generations, void* stream);

/* Same as emt_run, but allocates nothing.  For callers that cannot allocate
 * device memory while they run: a service whose GPU memory is reserved up
 * front by its own pool allocator, or a host loop that must not call
 * cudaMalloc/cudaFree because those calls synchronize the device.  No
 * counterpart in the reference.
 *
 * The handle must have been prepared with emt_reset (which allocates the
 * islands); this call then only launches kernels and copies device to
 * device.  The elite exchange between epochs goes through one file-scope
 * device array of 2 x EMT_NOALLOC_EXCHANGE_FLOATS floats (4 MiB) that every
 * GPU loading the library holds until the process exits.  Limit: the sum
 * over tasks of NP * round4(D) must not exceed EMT_NOALLOC_EXCHANGE_FLOATS,
 * else EMT_ERR_UNSUPPORTED and nothing runs.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current and keeps it for the life of the process; make that first
 * call before any stream capture, and do not call it again on a device the
 * process has reset with cudaDeviceReset (the kept address would be stale).
 * All calls share the array and it keeps the last call's contents: calls
 * that overlap on the GPU (other handles, other streams) race on it.
 * Nothing in it needs to start at zero: each call first copies in the
 * exchange state its handle carries.  Every epoch is one launch over all
 * islands; the handle's schedule, use_graph and emt_tune choices do not
 * apply here.  Results are bit-identical to emt_run. */
#define EMT_NOALLOC_EXCHANGE_FLOATS (1 << 19)
EMT_API int emt_run_noalloc(emt_handle_t* h, int32_t generations, void* stream);

/* Autotuner for EMT_SCHEDULE_AUTO: runs `generations` generations with each
 * candidate schedule in turn (single launch; occupancy buckets; each with and
 * without graph replay), times them with events on `stream`, and keeps the
 * fastest for later emt_run calls on this handle.  The generations are real
 * work (the run continues; results do not depend on the schedule).  Blocking.
 * *chosen (may be NULL) receives schedule | (graph ? 0x100 : 0).  Replaces
 * the reference's fixed 8-stream, one-launch-per-task shape
 * (SG-EMTF.cu:1660-1676). */
EMT_API int emt_tune(emt_handle_t* h, int32_t generations, void* stream, int32_t* chosen);

/* Measurement hook for roofline reports: times `reps` launches of the
 * rotation GEMM (Z = S Q^T for every island) of a large-island handle on its
 * current operands, with CUDA events on `stream`; *ms receives the mean
 * duration of one launch.  Blocking.  EMT_ERR_UNSUPPORTED for fused-kernel
 * handles, whose rotation runs inside the epoch kernel.  No counterpart in
 * the reference. */
EMT_API int emt_time_rotation(emt_handle_t* h, int32_t reps, void* stream, float* ms);

/* Measurement hook: SM cycles the fused epoch kernel's CTAs spent per phase
 * since emt_reset, summed over CTAs: [0] loading and writing back islands
 * and transfer bookkeeping, [1] trial vectors, [2] rotation (tensor-core
 * forms: the operand hand-off), [3] function epilogue, [4] FP32 selection,
 * [5] near-tie re-checks, and for the tensor-core forms [6] the issuing
 * thread's MMAs and commit, [7] the wait for their completion, [8] the
 * accumulator drain.  Only the library's
 * measurement build counts them (compiled with EMT_PHASE_CLOCKS, which adds
 * a barrier at each phase boundary); the regular build returns
 * EMT_ERR_UNSUPPORTED.  No counterpart in the reference. */
EMT_API int emt_get_phase_cycles(emt_handle_t* h, uint64_t* cycles, int32_t n);

/* Waits for the handle's work and reports a kernel's error word. */
EMT_API int emt_sync(emt_handle_t* h);

/* Best member of one task (messageTransfer, SG-EMTF.cu:1601-1615).  The
 * fitness is re-evaluated in FP64 on the host from the stored vector. */
EMT_API int emt_get_best(emt_handle_t* h, int32_t task, double* fitness, float* x);

/* FP32 fitness of every task's best member, n_tasks floats. */
EMT_API int emt_get_best_all(emt_handle_t* h, float* fitness);

/* One task's population (NP * D floats, row-major) and FP32 fitness (NP). */
EMT_API int emt_get_population(emt_handle_t* h, int32_t task, float* x, float* fitness);

/* Replaces one task's population and evaluates it on the device. */
EMT_API int emt_set_population(emt_handle_t* h, int32_t task, const float* x);

/* A task's function id, dimension and island size, as added. */
EMT_API int emt_get_task_info(emt_handle_t* h, int32_t task, int32_t* function, int32_t* dim,
                              int32_t* pop);

/* The rotation (D*D FP32, row-major) and shift (D) the device uses. */
EMT_API int emt_get_task_params(emt_handle_t* h, int32_t task, float* rotation, float* shift);

/* Evaluates n arbitrary points of one task on the device (the reference's
 * evaluate kernel, SG-EMTF.cu:1428-1479).  x: n*D floats; fitness: n floats;
 * z: optional n*D floats receiving the rotated argument. */
EMT_API int emt_evaluate(emt_handle_t* h, int32_t task, int32_t n, const float* x,
                 float* fitness, float* z);

EMT_API int emt_get_stats(emt_handle_t* h, emt_stats* out);

/* Size in bytes of a checkpoint, then the checkpoint itself: populations,
 * fitness and per-task generation counters.  Philox counters are derived
 * from those, so a restored run continues bit for bit. */
EMT_API int emt_snapshot_size(emt_handle_t* h, size_t* bytes);
EMT_API int emt_snapshot(emt_handle_t* h, void* buf, size_t bytes);
EMT_API int emt_restore(emt_handle_t* h, const void* buf, size_t bytes);

/* ---- CVRP multitask engine ------------------------------------------------
 * One island of giant-tour permutations per instance, decoded into
 * capacity-feasible routes by the split procedure (Prins 2004; evaluated on
 * the device in O(n) with Vidal's 2016 deque form); costs are exact int32.  Replaces
 * the reference's CVRP variant (proposed model/SG-EMTF_cvrp.cu: iter() at
 * :1487-1607 with per-task params {dimension, cars, customers} at :1496-1500);
 * that variant is unfinished (its crossover sets every gene to 1, :731-736),
 * so this engine follows the published methods instead: order crossover,
 * swap and 2-opt mutation, binary tournaments, elite transfer of whole
 * permutations between instances with the same customer count. */
typedef struct emt_cvrp_handle emt_cvrp_handle_t;

#define EMT_CVRP_MAX_CUSTOMERS 255

typedef struct emt_cvrp_config {
  int32_t pop;               /* island size (2..256)                         */
  float p_cross;             /* order-crossover probability                  */
  float p_swap, p_2opt;      /* mutation probabilities                       */
  int32_t transfer_interval; /* generations between transfers; 0 = off       */
  float transfer_rate;       /* fraction of the island sent                  */
  uint64_t seed;
  int32_t device;
  /* Sub-islands (the reference's IslandMigration, SG-EMTF_cvrp.cu:965-1020):
   * the island of pop members splits into subislands groups of pop /
   * subislands (>= 4; pop must divide; 0 or 1 = one group).  Tournaments
   * draw parents within the member's own group.  Before the children of
   * generation g, when g > 1 and (g - 1) % migration_interval == 0, the r-th
   * cheapest of group s replaces the r-th dearest of group s + 1 (mod
   * subislands), r < migration_count, when strictly cheaper, all from the
   * pre-migration state.  emt_cvrp_get_stats counts the replacements in
   * migrations_accepted. */
  int32_t subislands;
  int32_t migration_interval; /* generations between migrations; 0 = none     */
  int32_t migration_count;    /* members each group sends; 0 = group size / 8,
                                 at least 1; 2 * count <= group size          */
  int32_t reserved[4];
} emt_cvrp_config;

typedef struct emt_cvrp_instance {
  int32_t customers;     /* n, 1..EMT_CVRP_MAX_CUSTOMERS                    */
  int32_t capacity;
  const int32_t* x;      /* n + 1 integer coordinates in [0, 40000], node 0 = depot; */
  const int32_t* y;      /* NULL for all three: uniform on [0, 1000)^2      */
  const int32_t* demand; /* n + 1 (demand[0] ignored); NULL: uniform 1..10  */
} emt_cvrp_instance;

EMT_API void emt_cvrp_config_default(emt_cvrp_config* cfg);
EMT_API int emt_cvrp_create(const emt_cvrp_config* cfg, emt_cvrp_handle_t** out);
/* Distances are rounded Euclidean, round(sqrt(dx^2 + dy^2)) in integers. */
EMT_API int emt_cvrp_add_instances(emt_cvrp_handle_t* h, int32_t n, const emt_cvrp_instance* inst);
EMT_API int emt_cvrp_reset(emt_cvrp_handle_t* h, void* stream);
EMT_API int emt_cvrp_run(emt_cvrp_handle_t* h, int32_t generations, void* stream);
EMT_API int emt_cvrp_sync(emt_cvrp_handle_t* h);
/* Best cost of every instance (n_instances int32). */
EMT_API int emt_cvrp_get_best_all(emt_cvrp_handle_t* h, int32_t* costs);
/* One island: pop * customers bytes (customer ids 1..n), pop int32 costs. */
EMT_API int emt_cvrp_get_population(emt_cvrp_handle_t* h, int32_t inst, uint8_t* perms,
                                    int32_t* costs);
/* The instance as the device holds it: n + 1 x, y, demand; (n + 1)^2 distances. */
EMT_API int emt_cvrp_get_instance(emt_cvrp_handle_t* h, int32_t inst, int32_t* x, int32_t* y,
                                  int32_t* demand, int32_t* dist);
/* Cost of `count` caller-given giant tours of instance `inst` (count *
 * customers bytes, each a permutation of 1..n; anything else is rejected),
 * decoded on the device by the same split as the engine.  Blocking. */
EMT_API int emt_cvrp_evaluate(emt_cvrp_handle_t* h, int32_t inst, int32_t count,
                              const uint8_t* perms, int32_t* costs);
EMT_API int emt_cvrp_get_stats(emt_cvrp_handle_t* h, emt_stats* out);
EMT_API const char* emt_cvrp_last_error(const emt_cvrp_handle_t* h);
EMT_API void emt_cvrp_destroy(emt_cvrp_handle_t* h);

/* ---- run records and the reference's output files (emt_records.cpp) ----
 *
 * emt_record_run runs `generations` (a multiple of `interval`) in steps of
 * `interval` and fills record[t * (P + 2) + c], P = generations / interval:
 * the best FP32 fitness of task t at generation g0 + c * interval for
 * c = 0..P (g0 = the handle's generation count on entry), then the fitness
 * of rank 32 * ((NP - 1) / 32) (ascending) of the population on entry, the
 * reference's "near-worst" (SG-EMTF_DE.cu:1575,1594-1595,1632: best and
 * first entry of the last 32-member bank of the sorted population). */
EMT_API int emt_record_run(emt_handle_t* h, int32_t generations, int32_t interval, void* stream,
                           float* record);

/* Appends one run's rows (tasks x cols floats, "%g " each, newline per task)
 * and a blank line, the data_record_* layout (SG-EMTF_DE.cu:1791-1809) that
 * the reference's ANO tool reads run by run (data process/源.cpp:127-149). */
EMT_API int emt_write_record(const char* path, int32_t tasks, int32_t cols, const float* record);

/* The average normalised objective (data process/源.cpp:172-203) of `runs`
 * records of `tasks` x `cols` (cols - 1 recording points, then the
 * near-worst): per task, min over runs of the last point and max over runs
 * of the near-worst; ano[j] = mean over tasks and runs of
 * (record - min) / (max - min), 0 where max == min; FP32 arithmetic in the
 * tool's order.  ano receives cols - 1 floats. */
EMT_API int emt_ano(int32_t runs, int32_t tasks, int32_t cols, const float* records, float* ano);

/* Appends every task's FP32 fitness in ascending order, one line per task,
 * then a blank line (output_0.txt, SG-EMTF.cu:1971-1983). */
EMT_API int emt_write_fitness(emt_handle_t* h, const char* path);

/* Writes para.txt (SG-EMTF.cu:244-264): per task, D pairs "M b" of its
 * diagonal instance z = M (x + b), i.e. the diagonal rotation's factors and
 * b = -shift; a blank line; then the tasks' reference type ids.  Tasks whose
 * rotation is not diagonal have no such form: EMT_ERR_UNSUPPORTED. */
EMT_API int emt_write_para(emt_handle_t* h, const char* path);

/* ---- service mode (emt_service.cpp) ----
 *
 * Tasks arrive in batches over time and are served concurrently, the
 * reference's host scheduler (SG-EMTF.cu:1836-1958: T tasks split into
 * BATCH_NUM batches that arrive after random gaps, one host thread per task,
 * average response and solve times, memory use).  Here an admitted batch is
 * one handle on its own CUDA stream, created with seed = config seed + batch
 * number; each round of emt_service_step launches the next epoch of every
 * running batch whose previous epoch has finished, so batches overlap on the
 * device, and retires batches that have run the service's generation
 * budget.  A batch's results equal those of a standalone handle with the
 * same configuration, seed and tasks.  Times are milliseconds on the
 * service's steady clock, which starts at emt_service_create.  Islands of
 * D <= 128 (the fused kernel). */
typedef struct emt_service emt_service_t;

typedef struct emt_service_batch_info {
  int32_t n_tasks;
  int32_t state;        /* 0 waiting for its arrival time, 1 running, 2 done,
                           3 failed (admission or a launch failed: the step
                           that met it returned the error; the batch's handle
                           is released and it is not tried again)          */
  int32_t generations;  /* generations completed                            */
  int32_t reserved;
  double arrival_ms;    /* as submitted                                      */
  double admit_ms;      /* its handle created and its first launch queued    */
  double done_ms;       /* its last epoch seen complete                      */
} emt_service_batch_info;

typedef struct emt_service_stats {
  int32_t batches_submitted, batches_done;
  int64_t tasks_done;
  double mean_response_ms;    /* admit - arrival, averaged over finished tasks */
  double mean_solve_ms;       /* done - arrival, averaged over finished tasks  */
  double max_device_mem_mb;   /* device memory in use (cudaMemGetInfo), the
                                 largest sample, one sample per round        */
  double mean_device_mem_mb;  /* and the mean over rounds                    */
  uint64_t evaluations;       /* over finished batches                        */
  int32_t rounds;
  int32_t reserved;
} emt_service_stats;

/* generations: budget per batch; epoch: generations per launch (> 0). */
EMT_API int emt_service_create(const emt_config* cfg, int32_t generations, int32_t epoch,
                               emt_service_t** out);
/* Queues a batch that arrives at arrival_ms (0 or a past time: at once);
 * the task descriptors are copied.  *batch receives its number. */
EMT_API int emt_service_submit(emt_service_t* s, int32_t n, const emt_task_desc* tasks,
                               double arrival_ms, int32_t* batch);
/* One round: admit arrived batches, launch ready epochs, retire finished
 * batches.  *active (optional) receives the batches still waiting or
 * running. */
EMT_API int emt_service_step(emt_service_t* s, int32_t* active);
/* Rounds until every submitted batch is done or failed; sleeps until the
 * next arrival when nothing runs.  Returns at the first failure; calling it
 * again serves the remaining batches. */
EMT_API int emt_service_drain(emt_service_t* s);
/* A batch's times and state; best (n_tasks floats, optional) receives each
 * task's best FP32 fitness once the batch is done. */
EMT_API int emt_service_batch(emt_service_t* s, int32_t batch, emt_service_batch_info* info,
                              float* best);
EMT_API int emt_service_get_stats(emt_service_t* s, emt_service_stats* out);
EMT_API const char* emt_service_last_error(const emt_service_t* s);
EMT_API void emt_service_destroy(emt_service_t* s);

EMT_API const char* emt_last_error(const emt_handle_t* h);
EMT_API const char* emt_status_string(int status);
EMT_API void emt_destroy(emt_handle_t* h);

#ifdef __cplusplus
}
#endif

#endif /* SGEMTF_H */
