// emt_internal.h -- device-side task table, launch arguments and the shared
// memory layout of the fused epoch kernel.  Shared by emt_kernels.cu (device
// code) and emt_api.cu (host orchestration); not part of the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>

#include "emt_common.cuh"

namespace emt {

constexpr int kThreads = 256;  // one CTA per task, 8 warps
constexpr int kWarps = kThreads / 32;
constexpr int kMaxDim = 128;
constexpr int kMaxPop = 256;       // members of a fused (shared-memory) island
constexpr int kMaxPopLarge = 512;  // members of an HBM-resident island (the reference's 512)

// Per-task descriptor resident in HBM.  Row strides are padded to DP (a
// multiple of 4 floats) so every population row starts 16-byte aligned and
// moves as float4.
struct TaskDev {
  int32_t fid, D, NP, DP;
  float lo, hi;
  float woff;   // Weierstrass offset added to the term sum
  float qnorm;  // max row 2-norm of Q (rounding bound of the rotation)
  double woff64;  // the same offset in double precision
  int64_t pop_off;    // floats, into pop[]: NP rows of DP
  int64_t q_off;      // floats, into qt[]: D rows of DP, qt[k][n] = Q[n][k]
  int64_t o_off;      // floats, into shift[]: DP
  int64_t elite_off;  // floats, into elites[]: kmax rows of DP
  int32_t fit_off;    // into fit32[], tol32[], fit64[]: NP
  uint32_t flags;
  int32_t qt_in_smem;  // 1: Q staged in shared memory; 0: read through L1
  int32_t pad_;
};

// Largest dynamic shared memory a CTA may use (GB300: 227 KB).
constexpr size_t kSmemLimit = 227 * 1024;

enum Mode : int { MODE_EPOCH = 0, MODE_INIT = 1, MODE_EVAL = 2 };

// device counters, indexed as in EpochArgs::stats; [8, 8 + kPhases) hold the
// per-phase SM cycles of the phase-clock build (EMT_PHASE_CLOCKS)
constexpr int kPhases = 9;
// [8 + kPhases]: Weierstrass near ties decided with double-precision terms
constexpr int kStatWeierFp64 = 8 + kPhases;
constexpr int kStats = kStatWeierFp64 + 1;
enum Phase : int {
  PH_OTHER = 0,    // loading and writing back islands, transfer bookkeeping, migration ranks
  PH_BUILD = 1,    // trial vectors and the rotation operand
  PH_ROTATE = 2,   // the rotation (FP32 tiles, or the MMAs and the TMEM drain)
  PH_EVAL = 3,     // the function epilogue: f and its near-tie window
  PH_SELECT = 4,   // FP32 decisions, anchors carried forward, copies of accepted trials
  PH_RECHECK = 5,  // near ties re-decided: differential form, FP64-class tiers
  // the tensor-core rotation after its operands are published (PH_ROTATE):
  PH_MMA_ISSUE = 6,  // the issuing thread's MMA instructions and commit
  PH_MMA_WAIT = 7,   // from the commit to the completion seen by every warp
  PH_DRAIN = 8       // accumulators out of tensor memory into the rotated rows
};
// MMA descriptors of one island: at most 8 products of parts x 8 K-steps
// (BF16, K <= 128) or 4 x 16 (TF32); each entry {A and B descriptor low
// words, accumulator column, accumulate flag}
constexpr int kMaxMmas = 64;

struct EpochArgs {
  const TaskDev* tasks;
  const int32_t* order;  // CTA -> task (longest-first)
  int32_t single_task;   // >= 0: the grid's one CTA works on this task
  int32_t n_tasks;
  int32_t mode;
  float* pop;
  float* fit32;
  float* tol32;
  double* fit64;
  const float* qt;
  const float* shift;
  uint32_t* gen;  // generations completed per task
  int32_t gens;   // generations in this launch
  int32_t algorithm;
  float F, CR, eta_c, p_c, eta_m, p_m;
  uint64_t seed;
  float recheck_rel;
  uint32_t flags;
  // elite transfer
  int32_t transfer_import, transfer_export;
  float transfer_rate, transfer_mix;
  const float* elites_in;
  float* elites_out;
  unsigned long long* stats;  // [0] rechecks [1] flips [2] transfers [3] evaluations
                              // [4] re-checks decided by the differential form
                              // [5] member anchors (compensated rotations) computed
                              // [6] re-checks of bit-identical trials
                              // [7] sub-island migrants accepted
  // per member: compensated rotation z_h, z_l (2 * DP floats, at 2 * pop_off)
  // and {error bound, refresh limit} (at 2 * fit_off); NaN bound = not cached
  float* zc;
  float* zcb;
  int32_t* err;               // first kernel-side check that fired (0 = none)
  size_t smem_bytes;          // dynamic shared memory the launch provides
  int32_t tc_np, tc_kp;       // tensor-core form: padded N and K (elements) of the B tiles
  int32_t tc_bf16;            // 1: exact 3 x BF16 split (kind::f16); 0: TF32 hi/lo
  // sub-islands: groups per island (1 = none), migration interval and count
  int32_t subislands, mig_interval, mig_count;
  int32_t* queue;  // non-null: persistent grid taking islands from this counter
  uint64_t wait_ns;  // limit of every bounded device wait (tensor-core form)
};

// Islands too large for one CTA's shared memory (D > kMaxDim, up to
// kMaxDimLarge): each generation runs as a pipeline of kernels over
// HBM-resident islands (emt_large.cuh).  Rotation operands: S holds one row
// per member (rows of a task padded to a multiple of 128, Kp columns, zero
// beyond D); Z receives Q (s) per row, Nq columns.
constexpr int kMaxDimLarge = 1024;
constexpr int kLargeBM = 128;  // GEMM tile rows (members)
constexpr int kLargeBN = 256;  // GEMM tile columns (rotated genes), tensor-core form

struct LargeArgs {
  const TaskDev* tasks;
  int32_t n_tasks;
  int32_t max_np;         // largest island of the handle (sizes the per-row grids)
  int32_t Kp, Nq;        // padded GEMM K (multiple of 32) and N (multiple of 256)
  int32_t tc;            // 1: S holds the TF32 hi part, S + split the lo part
  const int64_t* srow;   // per task: first row of its block in S and Z
  const int64_t* qrow;   // per task: first row of its Q tiles (tensor-core form)
  int64_t split;         // floats between the hi and lo planes of S
  float* pop;            // members, stride DP (TaskDev::pop_off)
  float* U;              // trials, same layout
  float* fit32;
  float* tol32;
  double* fit64;
  float* ftr;            // trial fitness and window, same offsets as fit32
  float* ttr;
  const float* qt;       // FP32 Q^T per task (TaskDev::q_off)
  const float* shift;
  float* S;
  float* Z;
  uint32_t* gen;
  int32_t* rank;         // per member: rank order of the task (byrank)
  int32_t* flag;         // per trial row: 0 keep, 1 replace (FP32), 2 near tie, 3 replace (re-checked)
  int32_t* ties;         // per task (fit offsets): its near-tie rows, in order found
  int32_t* ntie;         // per task: their number
  int32_t* tjob;         // per near tie (fit offsets): trial job | (member job + 1) << 16
  float* wprec;          // per member (fit offsets): 0 when fit64 holds a float-float
                         // Weierstrass value, anything else when not
  int32_t* jobs;         // per task (2 x fit offsets): rows to rotate, row | 1 << 16 for a member
  int32_t* njob;         // per task: their number
  double* zr;            // FP64-class rotations of the jobs, 2 x pop offsets, stride DP
  int32_t* work;         // decision work items: task << 16 | tie; Weierstrass ties
                         // from the front, the others from the back (work_cap slots)
  int32_t* rwork;        // rotation work items: task << 16 | column block << 12 | job chunk
  int32_t* nwork;        // [0] Weierstrass decision items, [1] rotation items, [2] [3]
                         // the next rotation / decision item to hand out, [4] the
                         // other decision items
  int32_t work_cap;
  int32_t rot_grid, decide_grid;  // persistent grids of the two re-check kernels
  int32_t algorithm;
  float F, CR, eta_c, p_c, eta_m, p_m;
  uint64_t seed;
  float recheck_rel;
  uint32_t flags;
  float transfer_rate, transfer_mix;
  const float* elites_in;
  float* elites_out;
  unsigned long long* stats;
  int32_t* err;
  size_t select_smem;    // dynamic shared memory of the selection kernel
  int32_t subislands, mig_interval, mig_count;  // sub-islands per island (1 = none)
  uint64_t wait_ns;      // limit of every bounded device wait
};

namespace large {
enum BuildMode : int { BUILD_X = 0, BUILD_TRIALS = 1, BUILD_CANDIDATES = 2 };
// SEL_MIGRATE: the select kernel prepares the migrants (trial rows, their
// fitness, targets in the rank buffer); the selection pipeline then decides
// them strictly, as a transfer import
enum SelectMode : int {
  SEL_GENERATION = 0, SEL_IMPORT = 1, SEL_EXPORT = 2, SEL_RANK = 3, SEL_MIGRATE = 4
};
// Near-tie rotation work items (rot_kernel): 2 kRotCols outputs of up to
// kRotJobs rows of one task on kRotCols threads, two outputs per thread
// (registers: 4 per job and thread).  A build may set other shapes through
// EMT_ROT_COLS / EMT_ROT_JOBS.
#ifndef EMT_ROT_COLS
#define EMT_ROT_COLS 128
#endif
#ifndef EMT_ROT_JOBS
#define EMT_ROT_JOBS 8
#endif
constexpr int kRotCols = EMT_ROT_COLS;
constexpr int kRotJobs = EMT_ROT_JOBS;
// Rotation items a task can list in one selection step: column blocks x job
// chunks, with up to two jobs (trial and member) per selected row
EMT_HD int64_t rot_items_max(int D, int NP) {
  return (int64_t)((D + 2 * kRotCols - 1) / (2 * kRotCols)) * ((2 * NP + kRotJobs - 1) / kRotJobs);
}
}  // namespace large

// Dynamic shared memory of the large-island ranking / export / migration
// kernel: the flag/list/target/misc arrays (no re-checks run there; the
// stride DP is kept for the launch's interface).
EMT_HD size_t large_select_smem(int DP) {
  (void)DP;
  return sizeof(int) * (4 * kMaxPopLarge + 16);
}

// Arguments of the standalone evaluation kernel (emt_evaluate).
struct EvalArgs {
  const TaskDev* tasks;
  int32_t task;
  int32_t n;
  const float* x;  // n * D, unpadded
  float* f;        // n
  float* z;        // n * D or null
  const float* qt;
  const float* shift;
  int32_t* err;
  size_t smem_bytes;
};

EMT_HD int round4(int v) { return (v + 3) & ~3; }
EMT_HD size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

constexpr size_t kQueueSlot = 16;

struct Layout {
  int DP, NPP;
  size_t fit64, z64, X, U, ST, Z, QT, o, fit, tol, ftr, ttr, idx, flag, list, misc, total;
};

// Shared-memory carve-up for one task; identical on host and device.  With
// qt_in_smem false the rotation is read from global memory (L1/L2) instead,
// for islands too large to hold Q next to the population.
EMT_HD Layout smem_layout(int D, int NP, bool qt_in_smem = true) {
  Layout L;
  L.DP = round4(D);
  L.NPP = round4(NP);
  size_t off = 0;
  L.fit64 = off; off = align16(off + sizeof(double) * NP);
  L.z64 = off;   off = align16(off + sizeof(double) * kWarps * 2 * L.DP);
  L.X = off;     off = align16(off + sizeof(float) * NP * L.DP);
  L.U = off;     off = align16(off + sizeof(float) * NP * L.DP);
  L.ST = off;    off = align16(off + sizeof(float) * L.DP * L.NPP);
  L.Z = off;     off = align16(off + sizeof(float) * NP * L.DP);
  L.QT = off;    off = align16(off + (qt_in_smem ? sizeof(float) * D * L.DP : 0));
  L.o = off;     off = align16(off + sizeof(float) * L.DP);
  L.fit = off;   off = align16(off + sizeof(float) * NP);
  L.tol = off;   off = align16(off + sizeof(float) * NP);
  L.ftr = off;   off = align16(off + sizeof(float) * NP);
  L.ttr = off;   off = align16(off + sizeof(float) * NP);
  L.idx = off;   off = align16(off + sizeof(int) * 4 * NP);
  L.flag = off;  off = align16(off + sizeof(int) * NP);
  L.list = off;  off = align16(off + sizeof(int) * NP);
  L.misc = off;  off = align16(off + sizeof(int) * 8);
  // the last kQueueSlot bytes of a launch's allocation: the persistent queue
  // kernel's island slot (at the same place whatever island a CTA works on)
  L.total = off + kQueueSlot;
  return L;
}

// Shared-memory carve-up of the tensor-core form.  The dynamic shared memory
// starts 1024-byte aligned (the kernel checks it) with the operand tiles,
// `planes` split parts of each operand (TF32: hi, lo; BF16: three parts),
// each part nkb tiles of 128-byte rows (32 TF32 or 64 BF16 values per row):
// A = planes x nkb tiles of MA rows.  With NP <= 64 the A tiles hold 64 rows
// and the MMAs are M = 64; above, 128 rows and M = 128, so no MMA reads past
// A.  B holds Q's parts in tiles of Np rows:
//  - paired form, Np = 64 (every island of the handle has D <= 64): per K
//    block the parts' tiles side by side, kb-major, plus (BF16) a zero tile,
//    so an MMA of N = 128 over two adjacent tiles takes two parts of Q;
//  - otherwise Np = round8(D) of the widest island, part-major: an MMA of
//    N = round16(D) columns reads up to 8 rows (1 KB) past a part, whose
//    output columns (>= D) are never used; past the last part that stays
//    inside the allocation, which ends with at least the 1 KB MMA table and
//    the header.  The FP32 rotated rows Z alias the A region once the MMAs have
// completed.  The last kTcHeader bytes of the launch's allocation hold the
// CTA's own tensor-core state, at the same place whatever island it works on
// (the persistent queue kernel runs many): two mbarriers (MMA completion, TMA
// arrival), the TMEM base and the "a bounded wait gave up" flag.
constexpr size_t kTcHeader = 64;
struct TcHeader {
  uint64_t mma_bar, tma_bar;
  uint32_t tmem;
  int32_t dead;
  int32_t item;  // the persistent queue kernel's current island
};
static_assert(sizeof(TcHeader) <= kTcHeader, "tensor-core header");

struct TcLayout {
  int DP, Np, Kp, nkb, MA, planes, epr;
  int bplanes;  // B tiles per K block: planes, and a zero tile in the paired BF16 form
  size_t A, B, fit64, z64, X, U, o, fit, tol, ftr, ttr, idx, flag, list, misc, mdesc, total;
};

EMT_HD TcLayout tc_layout(int D, int NP, int Np, int Kp, bool bf16) {
  TcLayout L;
  L.DP = round4(D);
  L.Np = Np;
  L.Kp = Kp;
  L.planes = bf16 ? 3 : 2;
  L.epr = bf16 ? 64 : 32;
  L.nkb = Kp / L.epr;
  L.MA = NP <= 64 ? 64 : 128;
  size_t off = 0;
  L.A = off;
  off += (size_t)L.planes * L.nkb * L.MA * 128;
  L.B = off;
  L.bplanes = (Np == 64 && bf16) ? 4 : L.planes;
  off += (size_t)L.bplanes * L.nkb * Np * 128;
  L.fit64 = off; off = align16(off + sizeof(double) * NP);
  // FP64 re-check scratch: idle A-region space past Z (the re-checks run
  // after the epilogue has consumed Z and before the next operands are staged)
  const size_t zend = align16(L.A + sizeof(float) * NP * L.DP);
  const size_t zbuf = sizeof(double) * kWarps * 2 * L.DP;
  if (zend + zbuf <= L.B) {
    L.z64 = zend;
  } else {
    L.z64 = off;
    off = align16(off + zbuf);
  }
  L.X = off;     off = align16(off + sizeof(float) * NP * L.DP);
  L.U = off;     off = align16(off + sizeof(float) * NP * L.DP);
  L.o = off;     off = align16(off + sizeof(float) * L.DP);
  L.fit = off;   off = align16(off + sizeof(float) * NP);
  L.tol = off;   off = align16(off + sizeof(float) * NP);
  L.ftr = off;   off = align16(off + sizeof(float) * NP);
  L.ttr = off;   off = align16(off + sizeof(float) * NP);
  L.idx = off;   off = align16(off + sizeof(int) * 4 * NP);
  L.flag = off;  off = align16(off + sizeof(int) * NP);
  L.list = off;  off = align16(off + sizeof(int) * NP);
  L.misc = off;  off = align16(off + sizeof(int) * 8);
  L.mdesc = off; off = align16(off + sizeof(uint32_t) * 4 * kMaxMmas);
  L.total = off + kTcHeader;  // the header closes the allocation
  return L;
}

EMT_HD int round8(int v) { return (v + 7) & ~7; }
EMT_HD int round16(int v) { return (v + 15) & ~15; }
EMT_HD int round32(int v) { return (v + 31) & ~31; }
EMT_HD int round64(int v) { return (v + 63) & ~63; }

// MMAs of one island's tensor-core rotation, in issue order: K-step outer,
// product of parts inner.  Products (a of s, b of Q), the leading one first;
// BF16 takes eight of the nine (s2 q2, at most 2^-32 of s0 q0, is below the
// FP32 accumulation's rounding).  Two accumulators of 128 TMEM columns, the
// leading product alone in the first.
//  - paired form (Q in 64-row tiles, N = 128): an MMA on B tile b reads tiles
//    b and b + 1 of the K block, so its columns 0-63 take part b of Q and
//    columns 64-127 part b + 1.  Per K-step, TF32: hi [q_hi q_lo] -> acc 0,
//    lo [q_hi q_lo] -> acc 1.  BF16: s0 [q0 q1] -> acc 0; s1 [q0 q1],
//    s2 [q0 q1], s0 [q2 0], s1 [q2 0] -> acc 1 (the zero tile keeps columns
//    64-127 of the last two clean);
//  - otherwise one MMA per product (N = round16(D), part-major B tiles).
struct MmaEntry {
  uint32_t a_off, b_off;  // bytes from the A and B regions to the MMA's tiles
  uint32_t k_off;         // bytes of the K-step inside the 128-byte rows
  uint32_t acc;           // accumulator 0 or 1
  uint32_t accumulate;    // 0 for the first MMA into its accumulator
};
EMT_HD int mma_per_kstep(int planes, bool paired) {
  return paired ? (planes == 3 ? 5 : 2) : (planes == 3 ? 8 : 4);
}
EMT_HD MmaEntry mma_entry(int i, int MA, int Np, int planes, int nkb, int bplanes, bool paired) {
  // per K-step: part of s, part (paired: first B tile) of Q, accumulator; 4 bits each
  uint32_t pa, pb, pk;
  if (paired && planes == 3) {
    pa = 0x10210u; pb = 0x22000u; pk = 0x11110u;
  } else if (paired) {
    pa = 0x10u; pb = 0x00u; pk = 0x10u;
  } else if (planes == 3) {
    pa = 0x21201100u; pb = 0x12021010u; pk = 0x11111110u;
  } else {
    pa = 0x1100u; pb = 0x1010u; pk = 0x1110u;
  }
  const int per = mma_per_kstep(planes, paired);
  const int st = i / per, p = i - st * per;
  const uint32_t kb = (uint32_t)st >> 2, ks = (uint32_t)st & 3u;
  const uint32_t ap = (pa >> (4 * p)) & 15u, bp = (pb >> (4 * p)) & 15u, k = (pk >> (4 * p)) & 15u;
  const uint32_t btile = paired ? kb * (uint32_t)bplanes + bp : bp * (uint32_t)nkb + kb;
  MmaEntry e;
  e.a_off = (kb * (uint32_t)planes + ap) * (uint32_t)MA * 128u;
  e.b_off = btile * (uint32_t)Np * 128u;
  e.k_off = 32u * ks;
  e.acc = k;
  // the first MMA into each accumulator (K-step 0, the first product with
  // that accumulator) overwrites it
  e.accumulate = (st > 0 || p > (int)k) ? 1u : 0u;
  return e;
}

// One island of a tensor-core handle (Q tiles of np rows, K padded to kp,
// launch allocation smem bytes): every MMA reads its tiles inside the
// allocation (A reads inside A, paired B reads inside B), every TMA copy of
// Q's parts lands inside B, and the MMA table fits.  The host checks it
// before configuring a tensor-core launch.
inline bool tc_island_reads_inside(int D, int NP, int np, int kp, bool bf16, size_t smem) {
  const TcLayout L = tc_layout(D, NP, np, kp, bf16);
  if (L.total > smem) return false;
  const bool paired = L.Np == 64;
  const size_t N = paired ? 128 : (size_t)round16(D);
  if (N > 128) return false;  // two accumulators of 128 TMEM columns
  const size_t bend = L.B + (size_t)L.bplanes * L.nkb * L.Np * 128;
  const int ksteps = bf16 ? (D + 15) >> 4 : (D + 7) >> 3;
  const int n = mma_per_kstep(L.planes, paired) * ksteps;
  if (n > kMaxMmas) return false;
  for (int i = 0; i < n; ++i) {
    const MmaEntry e = mma_entry(i, L.MA, L.Np, L.planes, L.nkb, L.bplanes, paired);
    if (L.A + e.a_off + (size_t)L.MA * 128 > L.B) return false;
    const size_t b_end = L.B + e.b_off + N * 128;
    if (b_end > smem || (paired && b_end > bend)) return false;
  }
  for (int h = 0; h < L.planes; ++h)
    for (int kb = 0; kb < L.nkb; ++kb) {
      const int tile = paired ? kb * L.bplanes + h : h * L.nkb + kb;
      if (L.B + (size_t)(tile + 1) * L.Np * 128 > bend) return false;
    }
  return true;
}

// Error codes written to EpochArgs::err by the kernels' own checks.
enum DeviceCheck : int32_t {
  CHECK_OK = 0,
  CHECK_BAD_DESCRIPTOR = 1,
  CHECK_SMEM_TOO_SMALL = 2,
  CHECK_BAD_PARTNER = 3,
  CHECK_TIMEOUT = 4,      // a bounded mbarrier wait gave up
  CHECK_TC_SHAPE = 5,     // island outside the tensor-core form's limits
  CHECK_SMEM_ALIGN = 6    // dynamic shared memory not 1024-byte aligned (tensor-core form)
};

// Arguments of the best-member kernel (popSort + messageTransfer,
// SG-EMTF.cu:462-486,1601-1615): per task, warp-shuffle argmin of the FP32
// fitness, then the winner's fitness in FP64.
struct BestArgs {
  const TaskDev* tasks;
  int32_t n_tasks;
  const float* pop;
  const float* fit32;
  const double* fit64;
  const float* qt;
  const float* shift;
  int32_t* best_idx;
  float* best_f32;
  double* best_f64;
  // relative error of the best member's FP32 fitness, |f32 - f64| / scale,
  // with the scale the FP32 evaluation stated (its near-tie half-window tol32
  // over rel; Weierstrass: 2D + |offset|)
  const float* tol32;
  float rel;
  float* best_err;
};

// The tensor-core forms' split copies of each task's Q, written on the
// device by emt_prepare_rotations: part p of Q[r][c] of task t at
// base + t * task_stride + p * plane_stride + r * row_stride + c (elements),
// TF32 hi and lo (float; each rounded to nearest, ties away, as
// cvt.rna.tf32.f32 does; lo = tf32(Q - hi)) or the three exact BF16 parts
// (round to nearest even, each part of the remainder of the previous ones).
enum QPlaneKind : int32_t { QPLANES_NONE = 0, QPLANES_TF32 = 1, QPLANES_BF16 = 2 };
struct QPlanes {
  void* base = nullptr;
  int64_t task_stride = 0;
  int64_t plane_stride = 0;
  int32_t row_stride = 0;
  int32_t kind = QPLANES_NONE;
};

}  // namespace emt

// Kernel launchers (emt_kernels.cu).  tmap: the CUtensorMap of the B
// operand tiles (tensor-core form), or null for the FP32 form.
int emt_launch_epoch(const emt::EpochArgs& a, int grid, void* stream, const void* tmap = nullptr);
int emt_launch_epoch_noattr(const emt::EpochArgs& a, int grid, void* stream, const void* tmap);
int emt_epoch_smem_attr(bool tc, size_t bytes);
// resident CTAs per SM of the epoch kernel (queue: its persistent-queue twin)
int emt_epoch_occupancy(bool tc, size_t bytes, bool queue = false);
int emt_launch_eval(const emt::EvalArgs& a, void* stream);
// large islands (emt_large.cuh)
int emt_large_init(const emt::LargeArgs& a, void* stream);
int emt_large_build(const emt::LargeArgs& a, int mode, void* stream);
int emt_large_gemm(const emt::LargeArgs& a, const void* smap, const void* qmap, void* stream);
int emt_large_eval(const emt::LargeArgs& a, int which, int rows, void* stream);
int emt_large_select(const emt::LargeArgs& a, int mode, void* stream);
int emt_large_best(const emt::BestArgs& a, int maxD, void* stream);
// persistent grids of the re-check rotation and decision kernels on sms SMs
void emt_large_recheck_grids(int sms, int32_t* rot, int32_t* decide);
// selection of a generation (SEL_GENERATION), a transfer import (SEL_IMPORT)
// or a migration (SEL_MIGRATE): classify, rotate the near ties' rows, decide
// them, apply
int emt_large_selection(const emt::LargeArgs& a, int mode, void* stream);
int emt_launch_best(const emt::BestArgs& a, void* stream);
// Rotation matrices arrive in qt row-major (Q[r][c] at q_off + r * DP + c,
// zero columns from D to DP); transposes them in place to the kernels'
// layout (qt[q_off + k * DP + n] = Q[n][k]) and writes the split planes
// (whose buffer the caller has zeroed).  max_dim: the largest D.
int emt_prepare_rotations(const emt::TaskDev* tasks, int n_tasks, int max_dim, float* qt,
                          const emt::QPlanes& planes, void* stream);
