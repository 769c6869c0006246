// emt_api.cu -- the C ABI (include/sgemtf.h): handle, task packing and the
// host orchestration of the device kernels.
//
// Replaces the reference's host layer: initialization() (proposed model/
// SG-EMTF.cu:293-380), one std::thread per task running iter() (:1646-1745)
// over 8 shared streams, and the pthread/cudaEvent hand-shake for transfers
// (:1678-1722).  Here every task advances in the same launch; transfers are
// epoch boundaries between launches, so no host thread waits on another.
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sgemtf.h"
#include "emt_internal.h"

// NVTX range over a host call (header-only NVTX 3: without a profiler
// attached a push/pop costs a branch), so timelines show the library's
// calls and each epoch's launches.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

namespace {

using emt::TaskDev;

struct HostTask {
  int fid = 0, D = 0, NP = 0;
  float lo = 0.f, hi = 0.f;
  std::vector<float> Q;  // D*D row-major, the operator the device applies
  std::vector<float> o;  // D
  float woff = 0.f, qnorm = 1.f;
  uint32_t qr_id = UINT32_MAX;    // task id whose seeded rotation is still to be generated
  const double* dense = nullptr;  // caller's FP64 matrix still to be checked and converted
  double woff64 = 0.0;
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }  // every buffer of a handle goes with it
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace

struct emt_handle {
  emt_config cfg{};
  int device = 0;
  std::vector<HostTask> tasks;
  std::vector<TaskDev> table;
  std::vector<int32_t> order;
  bool uploaded = false, initialized = false;
  uint32_t gdone = 0;  // generation counter of the handle (every task's next draw is gdone + 1)
  uint64_t gen_joined = 0;  // sum over joined tasks of gdone at their join (stats)
  int elite_parity = 0;
  size_t smem_bytes = 0;
  std::string err;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timing_pending = false;
  double device_ms = 0.0;
  unsigned long long stats_base[4] = {0, 0, 0, 0};

  // launch schedules: islands grouped by resident CTAs per SM (each group a
  // contiguous range of the bucketed order, d_order[n ..]), per-island shared
  // memory, side streams and fork/join events, the cached epoch-loop graph
  struct Bucket {
    int first = 0, count = 0;
    size_t smem = 0;
  };
  std::vector<Bucket> buckets;
  std::vector<size_t> task_smem;
  int tuned = 0;  // schedule | 0x100 (graph) chosen by emt_tune; 0 = not tuned
  static constexpr int kSide = 8;
  cudaStream_t side[kSide] = {};
  cudaStream_t cap = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev[kSide] = {};
  cudaGraphExec_t gexec = nullptr;
  std::vector<int64_t> gkey;

  DevBuf<TaskDev> d_tasks;
  DevBuf<int32_t> d_order;
  DevBuf<float> d_pop, d_fit32, d_tol32, d_qt, d_shift, d_elites[2], d_best_f32, d_best_err;
  DevBuf<float> d_zc, d_zcb;  // per-member compensated rotations and their bounds
  DevBuf<double> d_fit64, d_best_f64;
  DevBuf<uint32_t> d_gen;
  DevBuf<unsigned long long> d_stats;
  DevBuf<int32_t> d_err, d_best_idx, d_queue;
  int queue_grid = 1;  // persistent grid of EMT_SCHEDULE_QUEUE: SMs x resident CTAs
  // tensor-core form: Q hi/lo tiles [task][2][Np][Kp] and their TMA map
  bool use_tc = false;
  bool tc_bf16 = false;  // exact 3 x BF16 split (else TF32 hi/lo)
  int tc_np = 0, tc_kp = 0;
  DevBuf<float> d_qtc;
  CUtensorMap tmap;
  // large islands (any D > 128): HBM-resident pipeline (emt_large.cuh)
  bool large = false, large_tc = false;
  int lKp = 0, lNq = 0;
  int32_t lrot_grid = 1, ldecide_grid = 1;
  int64_t lrows = 0;
  size_t lsel_smem = 0;
  DevBuf<float> d_U, d_ftr, d_ttr, d_S, d_Z, d_qbig;
  DevBuf<int64_t> d_srow, d_qrow;
  DevBuf<int32_t> d_rank, d_flag, d_ties, d_ntie, d_work, d_nwork, d_tjob, d_jobs, d_njob, d_rwork;
  DevBuf<float> d_wprec;  // large islands: which cached FP64-class values are float-float
  DevBuf<double> d_zr;  // re-check rotations of the large-island pipeline
  CUtensorMap smap, qmap;

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? EMT_ERR_OUT_OF_MEMORY : EMT_ERR_CUDA;
  }
};

namespace {

const float kBoxStd[7][2] = {{-100.f, 100.f}, {-5.12f, 5.12f},   {-32.768f, 32.768f},
                             {-600.f, 600.f}, {-2.048f, 2.048f}, {-500.f, 500.f},
                             {-0.5f, 0.5f}};
// SG-EMTF.cu:197-214 by reference type; kRefToFid maps the type to our id.
const float kBoxRef[7][2] = {{-100.f, 100.f}, {-50.f, 50.f},   {-50.f, 50.f}, {-50.f, 50.f},
                             {-100.f, 100.f}, {-0.5f, 0.5f}, {-500.f, 500.f}};
const int kRefToFid[7] = {EMT_SPHERE,   EMT_ROSENBROCK,  EMT_ACKLEY,  EMT_RASTRIGIN,
                          EMT_GRIEWANK, EMT_WEIERSTRASS, EMT_SCHWEFEL};

// Relative cost per gene of one island's generation beyond the rotation
// (D + 40), for the longest-first order.  Fitted to measured island times of
// 2000-generation runs (D = 50, NP = 64, GB300), where the near-tie re-checks
// of converged islands dominate: a Rosenbrock island then costs 2.3x and a
// Weierstrass island 2.8x a Sphere island, Griewank 1.3x, the rest ~1x.
const float kFnCost[7] = {0.f, 3.f, 0.f, 26.f, 114.f, 7.f, 160.f};

// The Weierstrass offset as the reference's host code computes it
// (SG-EMTF.cu:354-361): PI = 3.1415926 (double), b_ *= 3 in float, cosf.
float weierstrass_reference_offset() {
  float a = 1.f, b = 1.f, res = 0.f;
  for (int i = 0; i <= 20; ++i) {
    double arg = 2 * 3.1415926 * (double)b * 0.5;
    res += a * cosf((float)arg);
    a *= 0.5f;
    b *= 3.f;
  }
  return res;
}

// Orthogonal factor of the FP64 Householder QR of a seeded N(0,1) D x D
// matrix (Box-Muller on Philox words, purpose P_QR_NORMAL), column signs
// fixed so that R has a positive diagonal.
// For each of the vectors w_j = M + j * stride, j in [j0, j1): s = sum over
// i in [k, D) of v_i w_j[i] (in order of i), s = 2 s / vn, w_j[i] -= s v_i.
// Four vectors at a time; each vector's operations are exactly the
// one-vector loop's.
void reflect4(double* M, size_t stride, int j0, int j1, int D, const double* v, double vn,
              int k) {
  int j = j0;
  for (; j + 4 <= j1; j += 4) {
    double* w0 = M + (size_t)j * stride;
    double* w1 = w0 + stride;
    double* w2 = w1 + stride;
    double* w3 = w2 + stride;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int i = k; i < D; ++i) {
      s0 += v[i] * w0[i];
      s1 += v[i] * w1[i];
      s2 += v[i] * w2[i];
      s3 += v[i] * w3[i];
    }
    s0 = 2.0 * s0 / vn;
    s1 = 2.0 * s1 / vn;
    s2 = 2.0 * s2 / vn;
    s3 = 2.0 * s3 / vn;
    for (int i = k; i < D; ++i) {
      w0[i] -= s0 * v[i];
      w1[i] -= s1 * v[i];
      w2[i] -= s2 * v[i];
      w3[i] -= s3 * v[i];
    }
  }
  for (; j < j1; ++j) {
    double* w = M + (size_t)j * stride;
    double s = 0.0;
    for (int i = k; i < D; ++i) s += v[i] * w[i];
    s = 2.0 * s / vn;
    for (int i = k; i < D; ++i) w[i] -= s * v[i];
  }
}

// Orthogonal factor Q (row-major, D x D) of the Householder QR of A, held
// column-major in At (At[c][i] = A[i][c]; overwritten); Q's columns are
// negated where A's diagonal ends negative.
void householder_q(std::vector<double>& At, int D, std::vector<double>& Q) {
  // Householder QR: step k reflects with v_k = a_k - alpha e_k (a_k: column
  // k of A from row k on, after steps 0..k-1; alpha = -sign(a_kk) |a_k|);
  // every column c >= k of A and every row of Q gets
  // w -= (2 (v_k . w) / |v_k|^2) v_k.  Each column and each row thus sees the
  // reflectors in the order k = 0, 1, ..., and nothing else: the steps are
  // applied left-looking, a block of kBlk columns (rows) at a time, so each
  // v_k is read once per block instead of streaming all of A and Q per step.
  // Four vectors of a block at a time (reflect4): their dot products are
  // independent chains.  Every operation and every sum's order over i are
  // the step-by-step loop's, so Q is the same bit for bit.
  constexpr int kBlk = 16;
  std::vector<double> V((size_t)D * D, 0.0), vn(D, 0.0);
  std::vector<char> valid(D, 0);
  double* A = At.data();
  for (int c0 = 0; c0 < D; c0 += kBlk) {
    const int c1 = std::min(D, c0 + kBlk);
    for (int k = 0; k < c0 && k < D - 1; ++k)
      if (valid[k]) reflect4(A, (size_t)D, c0, c1, D, V.data() + (size_t)k * D, vn[k], k);
    for (int k = c0; k < c1 && k < D - 1; ++k) {
      double nrm = 0.0;
      const double* ak = A + (size_t)k * D;
      for (int i = k; i < D; ++i) nrm += ak[i] * ak[i];
      nrm = std::sqrt(nrm);
      if (nrm == 0.0) continue;
      const double alpha = ak[k] > 0 ? -nrm : nrm;
      double* v = V.data() + (size_t)k * D;
      for (int i = k; i < D; ++i) v[i] = ak[i];
      v[k] -= alpha;
      double n2 = 0.0;
      for (int i = k; i < D; ++i) n2 += v[i] * v[i];
      if (n2 == 0.0) continue;
      vn[k] = n2;
      valid[k] = 1;
      reflect4(A, (size_t)D, k, c1, D, v, n2, k);  // this column and the block's later ones
    }
  }
  Q.assign((size_t)D * D, 0.0);
  for (int i = 0; i < D; ++i) Q[(size_t)i * D + i] = 1.0;
  for (int r0 = 0; r0 < D; r0 += kBlk) {
    const int r1 = std::min(D, r0 + kBlk);
    for (int k = 0; k < D - 1; ++k)
      if (valid[k]) reflect4(Q.data(), (size_t)D, r0, r1, D, V.data() + (size_t)k * D, vn[k], k);
  }
  for (int c = 0; c < D; ++c)
    if (At[(size_t)c * D + c] < 0)
      for (int r = 0; r < D; ++r) Q[(size_t)r * D + c] = -Q[(size_t)r * D + c];
}

void seeded_rotation(uint64_t seed, uint32_t task, int D, std::vector<double>& Q) {
  // A is held column-major (At[c][i] = A[i][c]) so the Householder column
  // updates run over contiguous memory; every sum keeps its order.
  std::vector<double> At((size_t)D * D);
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; c += 4) {
      emt::U4 w = emt::draw(seed, task, 0, (uint32_t)r, emt::P_QR_NORMAL, (uint32_t)(c >> 2));
      uint32_t ww[4] = {w.x, w.y, w.z, w.w};
      for (int h = 0; h < 2; ++h) {
        double u1 = ((double)ww[2 * h] + 1.0) * 0x1p-32;
        double u2 = (double)ww[2 * h + 1] * 0x1p-32;
        double rad = std::sqrt(-2.0 * std::log(u1));
        double th = 6.283185307179586 * u2;
        if (c + 2 * h < D) At[(size_t)(c + 2 * h) * D + r] = rad * std::cos(th);
        if (c + 2 * h + 1 < D) At[(size_t)(c + 2 * h + 1) * D + r] = rad * std::sin(th);
      }
    }
  householder_q(At, D, Q);
}

int max_smem_optin(int device) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess)
    return 0;
  return v;
}

bool device_has_tcgen05(int device) {
  int major = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device) != cudaSuccess)
    return false;
  return major == 10;
}

// Whether every island fits the tensor-core form (NP <= 128, one 128-row MMA
// tile; operands and state within the shared-memory limit).  np: rows of the
// B tiles, kp: their K extent in elements.
// emt::tc_island_reads_inside for every island at the launch's allocation
bool tc_reads_inside(const std::vector<HostTask>& tasks, int np, int kp, bool bf16) {
  size_t smem = 0;
  for (const auto& t : tasks) smem = std::max(smem, emt::tc_layout(t.D, t.NP, np, kp, bf16).total);
  for (const auto& t : tasks)
    if (!emt::tc_island_reads_inside(t.D, t.NP, np, kp, bf16, smem)) return false;
  return true;
}

bool tc_fits(const std::vector<HostTask>& tasks, bool bf16, int& np, int& kp) {
  int dmax = 1;
  for (const auto& t : tasks) dmax = std::max(dmax, t.D);
  // islands of D <= 64 take Q in 64-row tiles (the paired form, N = 128)
  np = std::max(64, emt::round8(dmax));
  kp = bf16 ? emt::round64(dmax) : emt::round32(dmax);
  for (const auto& t : tasks)
    if (t.NP > 128 || emt::tc_layout(t.D, t.NP, np, kp, bf16).total > emt::kSmemLimit) return false;
  return tc_reads_inside(tasks, np, kp, bf16);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor map over the Q tiles: dims (Kp, Np, planes * tasks), FP32 (TF32
// parts) or BF16, box (one 128-byte row, Np, 1), 128-byte swizzle, i.e. one
// K-major B tile of one part of one task per TMA load.
int encode_qtc_map(emt_handle* h) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
    return h->fail(EMT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const int planes = h->tc_bf16 ? 3 : 2, esz = h->tc_bf16 ? 2 : 4;
  const cuuint64_t dims[3] = {(cuuint64_t)h->tc_kp, (cuuint64_t)h->tc_np,
                              (cuuint64_t)(planes * h->tasks.size())};
  const cuuint64_t strides[2] = {(cuuint64_t)h->tc_kp * esz,
                                 (cuuint64_t)h->tc_kp * h->tc_np * esz};
  const cuuint32_t box[3] = {(cuuint32_t)(128 / esz), (cuuint32_t)h->tc_np, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = ((EncodeTiledFn)fn)(&h->tmap, h->tc_bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                        : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                                   3, h->d_qtc.p, dims,
                                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return h->fail(EMT_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return EMT_OK;
}

// 3-D FP32 tensor map (K, rows, 2 planes), box (32, brows, 1), 128B swizzle.
int encode_planes(emt_handle* h, CUtensorMap* map, float* base, int K, int64_t rows, int brows) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
    return h->fail(EMT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, 2};
  const cuuint64_t strides[2] = {(cuuint64_t)K * 4, (cuuint64_t)K * (cuuint64_t)rows * 4};
  const cuuint32_t box[3] = {32, (cuuint32_t)brows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = ((EncodeTiledFn)fn)(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box,
                                   estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return h->fail(EMT_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return EMT_OK;
}

// Buffers of the large-island pipeline: trials, trial fitness, ranks, the
// rotation operands S (rows of a task padded to 128, Kp columns; FP32, or
// TF32 hi and lo planes) and results Z (Nq columns), and for the tensor-core
// form Q's TF32 hi/lo planes, Nq rows per task, with their TMA maps.
int large_upload(emt_handle* h, int64_t pop, int32_t fit, emt::QPlanes* qp) {
  const int n = (int)h->tasks.size();
  int dmax = 1, dpmax = 4;
  for (const auto& t : h->tasks) dmax = std::max(dmax, t.D);
  dpmax = emt::round4(dmax);
  h->lKp = emt::round32(dmax);
  h->lNq = (dmax + emt::kLargeBN - 1) / emt::kLargeBN * emt::kLargeBN;
  std::vector<int64_t> srow(n), qrow(n);
  int64_t rows = 0;
  for (int t = 0; t < n; ++t) {
    srow[t] = rows;
    rows += (h->tasks[t].NP + emt::kLargeBM - 1) / emt::kLargeBM * emt::kLargeBM;
    qrow[t] = (int64_t)t * h->lNq;
  }
  h->lrows = rows;
  int64_t ritems = 0;  // rotation work items of one selection step, at most
  for (const auto& t : h->tasks) ritems += emt::large::rot_items_max(t.D, t.NP);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  emt_large_recheck_grids(sms, &h->lrot_grid, &h->ldecide_grid);  // persistent re-check grids
  h->lsel_smem = emt::large_select_smem(dpmax);
  const int planes = h->large_tc ? 2 : 1;
  cudaError_t e;
  if ((e = h->d_U.ensure((size_t)pop)) || (e = h->d_ftr.ensure((size_t)fit)) ||
      (e = h->d_ttr.ensure((size_t)fit)) || (e = h->d_rank.ensure((size_t)fit)) ||
      (e = h->d_flag.ensure((size_t)fit)) || (e = h->d_ties.ensure((size_t)fit)) ||
      (e = h->d_ntie.ensure(n)) || (e = h->d_work.ensure((size_t)fit)) || (e = h->d_nwork.ensure(5)) ||
      (e = h->d_tjob.ensure((size_t)fit)) || (e = h->d_jobs.ensure(2 * (size_t)fit)) ||
      (e = h->d_wprec.ensure((size_t)fit)) ||
      (e = h->d_njob.ensure(n)) || (e = h->d_rwork.ensure((size_t)ritems)) ||
      (e = h->d_zr.ensure(2 * (size_t)pop)) ||
      (e = h->d_srow.ensure(n)) || (e = h->d_qrow.ensure(n)) ||
      (e = h->d_S.ensure((size_t)planes * rows * h->lKp)) ||
      (e = h->d_Z.ensure((size_t)rows * h->lNq)))
    return h->cuda_fail(e, "cudaMalloc");
  if ((e = cudaMemcpy(h->d_srow.p, srow.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(h->d_qrow.p, qrow.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(h->d_S.p, 0, sizeof(float) * h->d_S.n)) ||
      (e = cudaMemset(h->d_Z.p, 0, sizeof(float) * h->d_Z.n)) ||
      (e = cudaMemset(h->d_U.p, 0, sizeof(float) * (size_t)pop)) ||
      (e = cudaMemset(h->d_wprec.p, 0xFF, sizeof(float) * (size_t)fit)))
    return h->cuda_fail(e, "upload");
  if (!h->large_tc) return EMT_OK;
  const size_t plane = (size_t)n * h->lNq * h->lKp, per = (size_t)h->lNq * h->lKp;
  if ((e = h->d_qbig.ensure(2 * plane))) return h->cuda_fail(e, "cudaMalloc");
  if ((e = cudaMemset(h->d_qbig.p, 0, sizeof(float) * 2 * plane))) return h->cuda_fail(e, "upload");
  // TF32 hi and lo of Q, the lo part rounded as the S planes' is
  qp->base = h->d_qbig.p;
  qp->task_stride = (int64_t)per;
  qp->plane_stride = (int64_t)plane;
  qp->row_stride = h->lKp;
  qp->kind = emt::QPLANES_TF32;
  int rc = encode_planes(h, &h->smap, h->d_S.p, h->lKp, rows, emt::kLargeBM);
  if (!rc) rc = encode_planes(h, &h->qmap, h->d_qbig.p, h->lKp, (int64_t)n * h->lNq, emt::kLargeBN);
  return rc;
}

int upload(emt_handle* h) {
  if (h->uploaded) return EMT_OK;
  const int n = (int)h->tasks.size();
  if (n == 0) return h->fail(EMT_ERR_STATE, "no tasks");
  h->table.resize(n);
  int64_t pop = 0, q = 0, o = 0, el = 0;
  int32_t fit = 0;
  size_t smem = 0;
  for (int t = 0; t < n; ++t) {
    const HostTask& ht = h->tasks[t];
    TaskDev& d = h->table[t];
    d.fid = ht.fid;
    d.D = ht.D;
    d.NP = ht.NP;
    d.DP = emt::round4(ht.D);
    d.lo = ht.lo;
    d.hi = ht.hi;
    d.woff = ht.woff;
    d.woff64 = ht.woff64;
    d.qnorm = ht.qnorm;
    d.pop_off = pop;
    pop += (int64_t)ht.NP * d.DP;
    d.q_off = q;
    q += (int64_t)ht.D * d.DP;
    d.o_off = o;
    o += d.DP;
    d.elite_off = el;
    el += (int64_t)ht.NP * d.DP;
    d.fit_off = fit;
    fit += ht.NP;
    d.flags = h->cfg.flags;
    d.qt_in_smem = emt::smem_layout(ht.D, ht.NP, true).total <= emt::kSmemLimit ? 1 : 0;
    d.pad_ = 0;
    smem = std::max(smem, emt::smem_layout(ht.D, ht.NP, d.qt_in_smem != 0).total);
  }
  h->use_tc = false;
  h->tc_bf16 = false;
  h->large = false;
  for (const auto& t : h->tasks) h->large |= t.D > emt::kMaxDim || t.NP > emt::kMaxPop;
  if (h->large) {
    // the pipeline's work items carry the task index in 15 bits
    if (h->tasks.size() > 32767)
      return h->fail(EMT_ERR_UNSUPPORTED, "a handle with islands of D > 128 or NP > 256 holds at most 32767 tasks");
    // (large islands run the TF32 hi/lo GEMM for either tensor-core form)
    h->large_tc = h->cfg.precision != EMT_ROT_FP32 && device_has_tcgen05(h->device);
    if (!h->large_tc && (h->cfg.precision == EMT_ROT_TF32X3 || h->cfg.precision == EMT_ROT_BF16X3))
      return h->fail(EMT_ERR_UNSUPPORTED, "tensor-core form needs an sm_10x device");
    smem = 0;
  } else if (h->cfg.precision != EMT_ROT_FP32) {
    int np = 0, kp = 0;
    const bool bf16 = h->cfg.precision != EMT_ROT_TF32X3;  // BF16X3, and AUTO's choice
    const bool ok = device_has_tcgen05(h->device) && tc_fits(h->tasks, bf16, np, kp);
    if (!ok && h->cfg.precision != EMT_ROT_AUTO)
      return h->fail(EMT_ERR_UNSUPPORTED, "tensor-core form needs an sm_10x device and islands "
                                          "with NP <= 128 whose tiles fit in shared memory");
    if (ok) {
      h->use_tc = true;
      h->tc_bf16 = bf16;
      h->tc_np = np;
      h->tc_kp = kp;
      smem = 0;
      for (const auto& t : h->tasks)
        smem = std::max(smem, emt::tc_layout(t.D, t.NP, np, kp, bf16).total);
    }
  }
  h->smem_bytes = smem;
  // longest-first order: the hardware hands CTAs to free SM slots in block
  // order, so costly islands start first and the tail is made of cheap ones.
  h->order.resize(n);
  std::iota(h->order.begin(), h->order.end(), 0);
  std::vector<double> cost(n);
  for (int t = 0; t < n; ++t) {
    const HostTask& ht = h->tasks[t];
    cost[t] = (double)ht.NP * ht.D * (ht.D + 40.0 + kFnCost[ht.fid]);
  }
  std::stable_sort(h->order.begin(), h->order.end(),
                   [&](int a, int b) { return cost[a] > cost[b]; });
  // occupancy buckets: islands with the same resident CTAs per SM share a
  // launch whose shared memory is the largest of the group; in LPT order
  cudaError_t e0 = cudaSetDevice(h->device);
  if (e0 != cudaSuccess) return h->cuda_fail(e0, "cudaSetDevice");
  h->task_smem.assign(n, 0);
  std::vector<int> occ(n, 1);
  std::map<size_t, int> occ_of;  // one occupancy query per distinct shared-memory size
  for (int t = 0; t < n && !h->large; ++t) {
    const HostTask& ht = h->tasks[t];
    h->task_smem[t] = h->use_tc ? emt::tc_layout(ht.D, ht.NP, h->tc_np, h->tc_kp, h->tc_bf16).total
                                : emt::smem_layout(ht.D, ht.NP, h->table[t].qt_in_smem != 0).total;
    auto it = occ_of.find(h->task_smem[t]);
    if (it == occ_of.end())
      it = occ_of.emplace(h->task_smem[t], emt_epoch_occupancy(h->use_tc, h->task_smem[t])).first;
    occ[t] = it->second;
    if (occ[t] <= 0) return h->fail(EMT_ERR_UNSUPPORTED, "an island does not fit on an SM");
  }
  std::vector<int32_t> border(h->order);
  std::stable_sort(border.begin(), border.end(), [&](int a, int b) { return occ[a] < occ[b]; });
  h->buckets.clear();
  for (int i = 0; i < n && !h->large; ++i) {
    const int t = border[i];
    if (h->buckets.empty() || occ[border[h->buckets.back().first]] != occ[t]) {
      emt_handle::Bucket b;
      b.first = i;
      h->buckets.push_back(b);
    }
    h->buckets.back().count++;
    h->buckets.back().smem = std::max(h->buckets.back().smem, h->task_smem[t]);
  }
  h->order.insert(h->order.end(), border.begin(), border.end());
  if (!h->large) {  // the persistent grid: every SM slot the largest island allows
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    h->queue_grid =
        std::max(1, sms * std::max(1, emt_epoch_occupancy(h->use_tc, h->smem_bytes, true)));
  }
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->gkey.clear();
  }
  h->tuned = 0;

  // rotations go up row-major (rows padded to DP with zeros) and are
  // transposed and split on the device (emt_prepare_rotations)
  std::unique_ptr<float[]> hq(new float[(size_t)q]);
  std::vector<float> ho((size_t)o, 0.f);
  for (int t = 0; t < n; ++t) {
    const HostTask& ht = h->tasks[t];
    const TaskDev& d = h->table[t];
    for (int r = 0; r < ht.D; ++r) {
      float* row = hq.get() + d.q_off + (size_t)r * d.DP;
      std::memcpy(row, ht.Q.data() + (size_t)r * ht.D, sizeof(float) * ht.D);
      std::fill(row + ht.D, row + d.DP, 0.f);
    }
    for (int j = 0; j < ht.D; ++j) ho[(size_t)d.o_off + j] = ht.o[j];
  }
  cudaError_t e;
  if ((e = cudaSetDevice(h->device)) != cudaSuccess) return h->cuda_fail(e, "cudaSetDevice");
  if ((e = h->d_tasks.ensure(n)) != cudaSuccess ||
      (e = h->d_order.ensure(2 * (size_t)n)) != cudaSuccess ||
      (e = h->d_pop.ensure((size_t)pop)) != cudaSuccess ||
      (e = h->d_fit32.ensure((size_t)fit)) != cudaSuccess ||
      (e = h->d_tol32.ensure((size_t)fit)) != cudaSuccess ||
      (e = h->d_fit64.ensure((size_t)fit)) != cudaSuccess ||
      (e = h->d_zc.ensure((size_t)2 * pop)) != cudaSuccess ||
      (e = h->d_zcb.ensure((size_t)2 * fit)) != cudaSuccess ||
      (e = h->d_qt.ensure((size_t)q)) != cudaSuccess ||
      (e = h->d_shift.ensure((size_t)o)) != cudaSuccess ||
      (e = h->d_gen.ensure(n)) != cudaSuccess ||
      (e = h->d_stats.ensure(emt::kStats)) != cudaSuccess || (e = h->d_err.ensure(1)) != cudaSuccess ||
      (e = h->d_queue.ensure(1)) != cudaSuccess ||
      (e = h->d_best_idx.ensure(n)) != cudaSuccess ||
      (e = h->d_best_f32.ensure(n)) != cudaSuccess ||
      (e = h->d_best_f64.ensure(n)) != cudaSuccess || (e = h->d_best_err.ensure(n)) != cudaSuccess)
    return h->cuda_fail(e, "cudaMalloc");
  if (h->cfg.transfer_interval > 0 && n > 1)
    for (int b = 0; b < 2; ++b)
      if ((e = h->d_elites[b].ensure((size_t)el)) != cudaSuccess) return h->cuda_fail(e, "cudaMalloc");
  if ((e = cudaMemcpy(h->d_tasks.p, h->table.data(), sizeof(TaskDev) * n, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(h->d_order.p, h->order.data(), sizeof(int32_t) * 2 * n, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(h->d_qt.p, hq.get(), sizeof(float) * (size_t)q, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(h->d_shift.p, ho.data(), sizeof(float) * ho.size(), cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(h->d_gen.p, 0, sizeof(uint32_t) * n)) ||
      (e = cudaMemset(h->d_pop.p, 0, sizeof(float) * (size_t)pop)) ||
      (e = cudaMemset(h->d_stats.p, 0, sizeof(unsigned long long) * emt::kStats)) ||
      (e = cudaMemset(h->d_zcb.p, 0xFF, sizeof(float) * 2 * (size_t)fit)) ||
      (e = cudaMemset(h->d_err.p, 0, sizeof(int32_t))))
    return h->cuda_fail(e, "upload");
  emt::QPlanes planes;
  if (h->use_tc) {
    // Q's split parts, part-major per task: TF32 hi and lo (both rounded to
    // nearest, as the A tiles are), or the exact three BF16 parts
    const size_t plane = (size_t)h->tc_np * h->tc_kp;
    const size_t per = (h->tc_bf16 ? 3 : 2) * plane;
    const size_t bytes = per * n * (h->tc_bf16 ? sizeof(uint16_t) : sizeof(float));
    if ((e = h->d_qtc.ensure((bytes + 3) / 4)) != cudaSuccess) return h->cuda_fail(e, "cudaMalloc");
    if ((e = cudaMemset(h->d_qtc.p, 0, bytes)) != cudaSuccess) return h->cuda_fail(e, "upload");
    planes.base = h->d_qtc.p;
    planes.task_stride = (int64_t)per;
    planes.plane_stride = (int64_t)plane;
    planes.row_stride = h->tc_kp;
    planes.kind = h->tc_bf16 ? emt::QPLANES_BF16 : emt::QPLANES_TF32;
    int rc = encode_qtc_map(h);
    if (rc) return rc;
  }
  if (h->large) {
    int rc = large_upload(h, pop, fit, &planes);
    if (rc) return rc;
  }
  int dmax = 1;
  for (const auto& t : h->tasks) dmax = std::max(dmax, t.D);
  int pe = emt_prepare_rotations(h->d_tasks.p, n, dmax, h->d_qt.p, planes, nullptr);
  // the uploads and memsets above run on the legacy default stream: finish
  // them before the caller's stream (possibly a non-blocking one) runs
  if (!pe) pe = (int)cudaStreamSynchronize(nullptr);
  if (pe) return h->cuda_fail((cudaError_t)pe, "rotation preparation");
  h->uploaded = true;
  h->initialized = false;
  return EMT_OK;
}

emt::EpochArgs base_args(emt_handle* h, int mode) {
  emt::EpochArgs a{};
  a.tasks = h->d_tasks.p;
  a.order = h->d_order.p;
  a.single_task = -1;
  a.n_tasks = (int32_t)h->tasks.size();
  a.mode = mode;
  a.pop = h->d_pop.p;
  a.fit32 = h->d_fit32.p;
  a.tol32 = h->d_tol32.p;
  a.fit64 = h->d_fit64.p;
  a.zc = h->d_zc.p;
  a.zcb = h->d_zcb.p;
  a.qt = h->d_qt.p;
  a.shift = h->d_shift.p;
  a.gen = h->d_gen.p;
  a.gens = 0;
  a.algorithm = h->cfg.algorithm;
  a.F = h->cfg.F;
  a.CR = h->cfg.CR;
  a.eta_c = h->cfg.eta_c;
  a.p_c = h->cfg.p_c;
  a.eta_m = h->cfg.eta_m;
  a.p_m = h->cfg.p_m;
  a.seed = h->cfg.seed;
  a.recheck_rel = (float)(h->cfg.recheck_rel > 0 ? h->cfg.recheck_rel : 1e-5);
  a.flags = h->cfg.flags;
  a.transfer_import = 0;
  a.transfer_export = 0;
  a.transfer_rate = h->cfg.transfer_rate;
  a.transfer_mix = h->cfg.transfer_mix;
  a.stats = h->d_stats.p;
  a.err = h->d_err.p;
  a.smem_bytes = h->smem_bytes;
  a.tc_np = h->tc_np;
  a.tc_kp = h->tc_kp;
  a.tc_bf16 = h->tc_bf16 ? 1 : 0;
  a.subislands = h->cfg.subislands > 1 ? h->cfg.subislands : 1;
  a.mig_interval = h->cfg.migration_interval;
  a.mig_count = h->cfg.migration_count;
  a.wait_ns = h->cfg.wait_limit_ms > 0 ? (uint64_t)h->cfg.wait_limit_ms * 1000000ull : 0ull;
  return a;
}

int launch_epoch(emt_handle* h, const emt::EpochArgs& a, int grid, void* stream) {
  return emt_launch_epoch(a, grid, stream, h->use_tc ? (const void*)&h->tmap : nullptr);
}

// ---- epoch plans, launch schedules, graph replay ----

struct EpochStep {
  int gens, imp, exp, parity;
};

int transfer_interval_of(const emt_handle* h) {
  return (h->cfg.transfer_interval > 0 && h->tasks.size() > 1) ? h->cfg.transfer_interval : 0;
}

// The epochs emt_run(generations) launches from the handle's current state:
// an epoch ends at every transfer boundary.
std::vector<EpochStep> plan_epochs(const emt_handle* h, int generations) {
  std::vector<EpochStep> plan;
  const int interval = transfer_interval_of(h);
  uint32_t gdone = h->gdone;
  int parity = h->elite_parity, left = generations;
  while (left > 0) {
    EpochStep s{left, 0, 0, parity};
    if (interval) {
      s.imp = (gdone > 0 && gdone % (uint32_t)interval == 0) ? 1 : 0;
      s.gens = std::min(left, interval - (int)(gdone % (uint32_t)interval));
      s.exp = ((gdone + (uint32_t)s.gens) % (uint32_t)interval == 0) ? 1 : 0;
    }
    plan.push_back(s);
    if (s.exp) parity ^= 1;
    gdone += (uint32_t)s.gens;
    left -= s.gens;
  }
  return plan;
}

void apply_plan(emt_handle* h, const std::vector<EpochStep>& plan) {
  for (const EpochStep& s : plan) {
    if (s.exp) h->elite_parity ^= 1;
    h->gdone += (uint32_t)s.gens;
  }
}

int effective_schedule(const emt_handle* h) {
  if (h->cfg.schedule != EMT_SCHEDULE_AUTO) return h->cfg.schedule;
  if (h->tuned) return h->tuned & 0xFF;
  return h->buckets.size() > 1 ? EMT_SCHEDULE_BUCKETS : EMT_SCHEDULE_SINGLE;
}

bool effective_graph(const emt_handle* h) {
  if (h->cfg.schedule == EMT_SCHEDULE_AUTO && h->tuned) return (h->tuned & 0x100) != 0;
  return h->cfg.use_graph != 0;
}

int ensure_side(emt_handle* h) {
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < emt_handle::kSide && e == cudaSuccess; ++i) {
    if (!h->side[i]) e = cudaStreamCreateWithFlags(&h->side[i], cudaStreamNonBlocking);
    if (e == cudaSuccess && !h->join_ev[i])
      e = cudaEventCreateWithFlags(&h->join_ev[i], cudaEventDisableTiming);
  }
  if (e == cudaSuccess && !h->fork_ev) e = cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess && !h->cap) e = cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking);
  return e == cudaSuccess ? EMT_OK : h->cuda_fail(e, "side streams");
}

// ---- large islands: argument block and launch sequences ----

emt::LargeArgs large_args(emt_handle* h) {
  emt::LargeArgs a{};
  a.tasks = h->d_tasks.p;
  a.n_tasks = (int32_t)h->tasks.size();
  a.max_np = 4;
  for (const auto& t : h->tasks) a.max_np = std::max(a.max_np, t.NP);
  a.Kp = h->lKp;
  a.Nq = h->lNq;
  a.tc = h->large_tc ? 1 : 0;
  a.srow = h->d_srow.p;
  a.qrow = h->d_qrow.p;
  a.split = (int64_t)h->lrows * h->lKp;
  a.pop = h->d_pop.p;
  a.U = h->d_U.p;
  a.fit32 = h->d_fit32.p;
  a.tol32 = h->d_tol32.p;
  a.fit64 = h->d_fit64.p;
  a.ftr = h->d_ftr.p;
  a.ttr = h->d_ttr.p;
  a.qt = h->d_qt.p;
  a.shift = h->d_shift.p;
  a.S = h->d_S.p;
  a.Z = h->d_Z.p;
  a.gen = h->d_gen.p;
  a.rank = h->d_rank.p;
  a.flag = h->d_flag.p;
  a.ties = h->d_ties.p;
  a.ntie = h->d_ntie.p;
  a.tjob = h->d_tjob.p;
  a.wprec = h->d_wprec.p;
  a.jobs = h->d_jobs.p;
  a.njob = h->d_njob.p;
  a.zr = h->d_zr.p;
  a.work = h->d_work.p;
  a.rwork = h->d_rwork.p;
  a.nwork = h->d_nwork.p;
  a.work_cap = (int32_t)h->d_work.n;
  a.rot_grid = h->lrot_grid;
  a.decide_grid = h->ldecide_grid;
  a.algorithm = h->cfg.algorithm;
  a.F = h->cfg.F;
  a.CR = h->cfg.CR;
  a.eta_c = h->cfg.eta_c;
  a.p_c = h->cfg.p_c;
  a.eta_m = h->cfg.eta_m;
  a.p_m = h->cfg.p_m;
  a.seed = h->cfg.seed;
  a.recheck_rel = (float)(h->cfg.recheck_rel > 0 ? h->cfg.recheck_rel : 1e-5);
  a.flags = h->cfg.flags;
  a.transfer_rate = h->cfg.transfer_rate;
  a.transfer_mix = h->cfg.transfer_mix;
  a.stats = h->d_stats.p;
  a.err = h->d_err.p;
  a.select_smem = h->lsel_smem;
  a.subislands = h->cfg.subislands > 1 ? h->cfg.subislands : 1;
  a.mig_interval = h->cfg.migration_interval;
  a.mig_count = h->cfg.migration_count;
  a.wait_ns = h->cfg.wait_limit_ms > 0 ? (uint64_t)h->cfg.wait_limit_ms * 1000000ull : 0ull;
  return a;
}

// fitness of every member: operands from the islands, rotation, evaluation
int large_eval_members(emt_handle* h, cudaStream_t stream) {
  const emt::LargeArgs a = large_args(h);
  int e = emt_large_build(a, emt::large::BUILD_X, stream);
  if (!e) e = emt_large_gemm(a, &h->smap, &h->qmap, stream);
  if (!e) e = emt_large_eval(a, 0, emt::kMaxPopLarge, stream);
  return e;
}

// One generation: trials, rotation, evaluation, selection (7 launches: the
// selection is classify, re-check rotations, decisions, apply).
int large_generation(emt_handle* h, const emt::LargeArgs& a, cudaStream_t stream) {
  int e = emt_large_build(a, emt::large::BUILD_TRIALS, stream);
  if (!e) e = emt_large_gemm(a, &h->smap, &h->qmap, stream);
  if (!e) e = emt_large_eval(a, 1, emt::kMaxPopLarge, stream);
  if (!e) e = emt_large_selection(a, emt::large::SEL_GENERATION, stream);
  return e;
}

int large_epoch(emt_handle* h, int gens, int imp, int exp, int parity, cudaStream_t stream) {
  emt::LargeArgs a = large_args(h);
  if (transfer_interval_of(h)) {
    a.elites_in = h->d_elites[parity ^ 1].p;
    a.elites_out = h->d_elites[parity].p;
  }
  int e = 0;
  if (imp) {  // elite transfer in: rank, candidates, their fitness, strict selection
    e = emt_large_select(a, emt::large::SEL_RANK, stream);
    if (!e) e = emt_large_build(a, emt::large::BUILD_CANDIDATES, stream);
    if (!e) e = emt_large_gemm(a, &h->smap, &h->qmap, stream);
    if (!e) e = emt_large_eval(a, 1, emt::kMaxPopLarge, stream);
    if (!e) e = emt_large_selection(a, emt::large::SEL_IMPORT, stream);
  }
  const bool migrate = a.subislands > 1 && a.mig_interval > 0;
  for (int g = 0; g < gens && !e; ++g) {
    // ring migration before the trials when the generation calls for it; the
    // kernels decide that from each task's counter, so a replayed graph of
    // this sequence stays right whatever generation it starts at
    if (migrate) {
      e = emt_large_select(a, emt::large::SEL_MIGRATE, stream);
      if (!e) e = emt_large_selection(a, emt::large::SEL_MIGRATE, stream);
    }
    if (!e) e = large_generation(h, a, stream);
  }
  if (!e && exp) e = emt_large_select(a, emt::large::SEL_EXPORT, stream);
  return e;
}

// One epoch's islands under a schedule; stream receives every launch or
// waits for them (fork/join through events), so the next epoch's transfer
// sees all of this epoch's exports.
int launch_sched(emt_handle* h, emt::EpochArgs a, int sched, cudaStream_t stream) {
  const void* tm = h->use_tc ? (const void*)&h->tmap : nullptr;
  const int n = (int)h->tasks.size();
  if (sched == EMT_SCHEDULE_SINGLE || (sched == EMT_SCHEDULE_BUCKETS && h->buckets.size() == 1))
    return emt_launch_epoch_noattr(a, n, stream, tm);
  if (sched == EMT_SCHEDULE_QUEUE) {  // one persistent launch over the work queue
    int e = (int)cudaMemsetAsync(h->d_queue.p, 0, sizeof(int32_t), stream);
    a.queue = h->d_queue.p;
    if (!e) e = emt_launch_epoch_noattr(a, std::min(n, h->queue_grid), stream, tm);
    return e;
  }
  int e = (int)cudaEventRecord(h->fork_ev, stream);
  const int nside = sched == EMT_SCHEDULE_BUCKETS ? (int)h->buckets.size() : emt_handle::kSide;
  for (int i = 0; i < nside && !e; ++i) e = (int)cudaStreamWaitEvent(h->side[i], h->fork_ev, 0);
  if (sched == EMT_SCHEDULE_BUCKETS) {
    for (int i = 0; i < nside && !e; ++i) {
      const emt_handle::Bucket& b = h->buckets[i];
      emt::EpochArgs ab = a;
      ab.order = h->d_order.p + n + b.first;
      ab.smem_bytes = b.smem;
      e = emt_launch_epoch_noattr(ab, b.count, h->side[i], tm);
    }
  } else {
    for (int k = 0; k < n && !e; ++k) {
      const int t = h->order[k];
      emt::EpochArgs at = a;
      at.single_task = t;
      at.smem_bytes = h->task_smem[t];
      e = emt_launch_epoch_noattr(at, 1, h->side[k % emt_handle::kSide], tm);
    }
  }
  for (int i = 0; i < nside && !e; ++i) {
    e = (int)cudaEventRecord(h->join_ev[i], h->side[i]);
    if (!e) e = (int)cudaStreamWaitEvent(stream, h->join_ev[i], 0);
  }
  return e;
}

int enqueue_plan(emt_handle* h, const std::vector<EpochStep>& plan, int sched, cudaStream_t stream) {
  const int interval = transfer_interval_of(h);
  if (h->large) {
    for (const EpochStep& s : plan) {
      const NvtxRange range("emt epoch (large islands)");
      const int e = large_epoch(h, s.gens, s.imp, s.exp, s.parity, stream);
      if (e) return e;
    }
    return 0;
  }
  for (const EpochStep& s : plan) {
    const NvtxRange range("emt epoch");
    emt::EpochArgs a = base_args(h, emt::MODE_EPOCH);
    a.gens = s.gens;
    if (interval) {
      a.transfer_import = s.imp;
      a.transfer_export = s.exp;
      a.elites_in = h->d_elites[s.parity ^ 1].p;
      a.elites_out = h->d_elites[s.parity].p;
    }
    const int e = launch_sched(h, a, sched, stream);
    if (e) return e;
  }
  return 0;
}

// Launches a plan on `stream` (directly, or as a CUDA graph captured once
// per distinct plan and replayed), between the handle's timing events.
int run_plan(emt_handle* h, const std::vector<EpochStep>& plan, int sched, bool graph,
             cudaStream_t stream) {
  if (sched != EMT_SCHEDULE_SINGLE || graph) {
    const int rc = ensure_side(h);
    if (rc) return rc;
  }
  int e = emt_epoch_smem_attr(h->use_tc, h->smem_bytes);
  if (e) return h->cuda_fail((cudaError_t)e, "shared-memory attribute");
  cudaEventRecord(h->ev0, stream);
  if (graph && !plan.empty()) {
    std::vector<int64_t> key{sched};
    for (const EpochStep& s : plan) {
      key.push_back(s.gens);
      key.push_back(s.imp | (s.exp << 1) | (s.parity << 2));
    }
    if (!h->gexec || key != h->gkey) {
      if (h->gexec) cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
      h->gkey.clear();
      cudaGraph_t g = nullptr;
      e = (int)cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal);
      if (!e) {
        const int le = enqueue_plan(h, plan, sched, h->cap);
        e = (int)cudaStreamEndCapture(h->cap, &g);
        if (le) e = le;
      }
      if (!e) e = (int)cudaGraphInstantiate(&h->gexec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e) {
        h->gexec = nullptr;
        return h->cuda_fail((cudaError_t)e, "epoch graph capture");
      }
      h->gkey = key;
    }
    e = (int)cudaGraphLaunch(h->gexec, stream);
  } else {
    e = enqueue_plan(h, plan, sched, stream);
  }
  if (e) return h->cuda_fail((cudaError_t)e, "epoch launch");
  cudaEventRecord(h->ev1, stream);
  h->timing_pending = true;
  return EMT_OK;
}

int check_task(const emt_handle* h, int32_t task) {
  return (task >= 0 && task < (int32_t)h->tasks.size()) ? EMT_OK : EMT_ERR_INVALID_ARG;
}

}  // namespace

extern "C" {

void emt_config_default(emt_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->algorithm = EMT_DE_RAND1_BIN;
  cfg->precision = EMT_ROT_FP32;
  cfg->F = 0.5f;
  cfg->CR = 0.9f;
  cfg->eta_c = 15.f;
  cfg->p_c = 0.9f;
  cfg->eta_m = 15.f;
  cfg->p_m = -1.f;
  cfg->transfer_interval = 0;
  cfg->transfer_rate = 0.1f;
  cfg->transfer_mix = 0.4f;
  cfg->flags = 0;
  cfg->seed = 1;
  cfg->recheck_rel = 0.0;
  cfg->device = 0;
}

int32_t emt_function_from_reference(int32_t t) { return (t >= 0 && t < 7) ? kRefToFid[t] : -1; }

int emt_seeded_rotation(uint64_t seed, int32_t task, int32_t dim, double* q) {
  if (!q || task < 0 || dim < 1 || dim > EMT_MAX_DIM) return EMT_ERR_INVALID_ARG;
  std::vector<double> Q;
  try {
    seeded_rotation(seed, (uint32_t)task, dim, Q);
  } catch (const std::bad_alloc&) {
    return EMT_ERR_OUT_OF_MEMORY;
  }
  std::memcpy(q, Q.data(), sizeof(double) * Q.size());
  return EMT_OK;
}

int emt_function_box(int32_t fid, int32_t reference_boxes, float* lo, float* hi) {
  if (fid < 0 || fid >= EMT_NUM_FUNCTIONS || !lo || !hi) return EMT_ERR_INVALID_ARG;
  if (reference_boxes) {
    for (int t = 0; t < 7; ++t)
      if (kRefToFid[t] == fid) {
        *lo = kBoxRef[t][0];
        *hi = kBoxRef[t][1];
        return EMT_OK;
      }
  }
  *lo = kBoxStd[fid][0];
  *hi = kBoxStd[fid][1];
  return EMT_OK;
}

const char* emt_status_string(int s) {
  switch (s) {
    case EMT_OK: return "ok";
    case EMT_ERR_INVALID_ARG: return "invalid argument";
    case EMT_ERR_OUT_OF_MEMORY: return "out of memory";
    case EMT_ERR_CUDA: return "CUDA error";
    case EMT_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case EMT_ERR_STATE: return "call out of order";
    case EMT_ERR_UNSUPPORTED: return "unsupported";
    case EMT_ERR_DEVICE_CHECK: return "device-side check failed";
    default: return "unknown status";
  }
}

int emt_create(const emt_config* cfg, emt_handle_t** out) {
  if (!cfg || !out) return EMT_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->algorithm < EMT_DE_RAND1_BIN || cfg->algorithm > EMT_GA_SBX_PM) return EMT_ERR_INVALID_ARG;
  if (cfg->precision < EMT_ROT_FP32 || cfg->precision > EMT_ROT_BF16X3) return EMT_ERR_INVALID_ARG;
  if (!(cfg->CR >= 0.f && cfg->CR <= 1.f) || !(cfg->p_c >= 0.f && cfg->p_c <= 1.f) ||
      !(cfg->eta_c >= 0.f) || !(cfg->eta_m >= 0.f) || !(cfg->p_m <= 1.f) ||
      !std::isfinite(cfg->F) || cfg->transfer_interval < 0 ||
      !(cfg->transfer_rate > 0.f && cfg->transfer_rate <= 1.f) ||
      !(cfg->transfer_mix >= 0.f && cfg->transfer_mix <= 1.f) || !(cfg->recheck_rel >= 0.0) ||
      cfg->subislands < 0 || cfg->subislands > EMT_MAX_POP / 4 || cfg->migration_interval < 0 ||
      cfg->migration_count < 0 || cfg->wait_limit_ms < 0)
    return EMT_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return EMT_ERR_CUDA;
  if (cfg->device < 0 || cfg->device >= ndev) return EMT_ERR_INVALID_ARG;
  if (cfg->schedule < EMT_SCHEDULE_AUTO || cfg->schedule > EMT_SCHEDULE_QUEUE ||
      (cfg->use_graph != 0 && cfg->use_graph != 1))
    return EMT_ERR_INVALID_ARG;
  emt_handle* h = new (std::nothrow) emt_handle();
  if (!h) return EMT_ERR_OUT_OF_MEMORY;
  h->cfg = *cfg;
  h->device = cfg->device;
  if (cudaSetDevice(h->device) != cudaSuccess || cudaEventCreate(&h->ev0) != cudaSuccess ||
      cudaEventCreate(&h->ev1) != cudaSuccess) {
    delete h;
    return EMT_ERR_CUDA;
  }
  *out = h;
  return EMT_OK;
}

// Tasks joining an initialized handle (the reference admits batches of
// tasks into a running service, SG-EMTF.cu:1842-1912).  The islands already
// running keep their members, fitness values and generation counter; the new
// ones start from the initial populations a handle created with every task
// would draw (the draws depend on the seed and the task index only) and take
// part from generation gdone + 1 on, transfer partners included.  The layout
// of the device arrays changes, so the running islands travel through a
// snapshot: state out, new layout and initial islands in, state back.
int join_tasks(emt_handle* h, std::vector<HostTask>& add) {
  const size_t n_old = h->tasks.size();
  size_t bytes = 0;
  emt_snapshot_size(h, &bytes);
  std::vector<unsigned char> before(bytes);
  int rc = emt_snapshot(h, before.data(), bytes);  // synchronises the handle
  if (rc) return rc;
  unsigned long long st[emt::kStats];
  cudaError_t e = cudaMemcpy(st, h->d_stats.p, sizeof(st), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return h->cuda_fail(e, "copy stats");
  const uint32_t gdone = h->gdone;
  const uint64_t joined = h->gen_joined;
  uint64_t np_new = 0;
  for (auto& t : add) {
    np_new += (uint64_t)t.NP;
    h->tasks.push_back(std::move(t));
  }
  h->uploaded = false;
  h->initialized = false;
  if ((rc = emt_reset(h, h->stream))) {  // new layout; every island initial
    // refused (e.g. a form the new islands do not fit): the handle goes back
    // to its running islands, and the error stays the refusal's
    const std::string why = h->err;
    h->tasks.resize(n_old);
    h->uploaded = false;
    h->initialized = false;
    if (!emt_reset(h, h->stream) && !emt_restore(h, before.data(), before.size()) &&
        cudaMemcpy(h->d_stats.p, st, sizeof(st), cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaStreamSynchronize(nullptr) == cudaSuccess)
      h->gen_joined = joined;
    h->err = why;
    return rc;
  }
  emt_snapshot_size(h, &bytes);
  std::vector<unsigned char> after(bytes);
  if ((rc = emt_snapshot(h, after.data(), bytes))) return rc;
  // the running islands' records, then the new islands' initial ones with
  // the handle's generation counter
  std::vector<unsigned char> merged(after.size());
  const size_t hdr = 3 * sizeof(uint64_t);
  const size_t old_body = before.size() - hdr;
  std::memcpy(merged.data(), after.data(), hdr);
  const uint64_t g64 = gdone;
  std::memcpy(merged.data() + 2 * sizeof(uint64_t), &g64, sizeof(g64));
  std::memcpy(merged.data() + hdr, before.data() + hdr, old_body);
  size_t at = hdr + old_body;
  std::memcpy(merged.data() + at, after.data() + at, after.size() - at);
  for (size_t t = n_old; t < h->tasks.size(); ++t) {
    const HostTask& ht = h->tasks[t];
    at += (size_t)ht.NP * ht.D * 4 + (size_t)ht.NP * (4 + 4 + 8);
    std::memcpy(merged.data() + at, &gdone, sizeof(gdone));
    at += 4;
  }
  if ((rc = emt_restore(h, merged.data(), merged.size()))) return rc;
  st[3] += np_new;  // the new islands' initial evaluation
  if ((e = cudaMemcpy(h->d_stats.p, st, sizeof(st), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaStreamSynchronize(nullptr)) != cudaSuccess)
    return h->cuda_fail(e, "restore stats");
  h->gen_joined = joined + (uint64_t)gdone * (h->tasks.size() - n_old);
  return EMT_OK;
}

static int add_tasks_impl(emt_handle_t* h, int32_t n, const emt_task_desc* td) {
  if (!h) return EMT_ERR_INVALID_ARG;
  const NvtxRange range("emt_add_tasks");
  if (n < 0 || (n > 0 && !td)) return h->fail(EMT_ERR_INVALID_ARG, "bad task array");
  const int smem_cap = max_smem_optin(h->device);
  std::vector<HostTask> add;
  add.reserve(n);
  for (int i = 0; i < n; ++i) {
    const emt_task_desc& d = td[i];
    const uint32_t id = (uint32_t)(h->tasks.size() + add.size());
    if (d.function < 0 || d.function >= EMT_NUM_FUNCTIONS)
      return h->fail(EMT_ERR_INVALID_ARG, "task " + std::to_string(i) + ": bad function id");
    if (d.dim < 1 || d.dim > EMT_MAX_DIM)
      return h->fail(EMT_ERR_INVALID_ARG, "task " + std::to_string(i) + ": dim out of range");
    if (d.pop < 4 || d.pop > EMT_MAX_POP)
      return h->fail(EMT_ERR_INVALID_ARG, "task " + std::to_string(i) + ": pop out of range");
    if (h->cfg.subislands > 1) {
      const int S = h->cfg.subislands, NPs = d.pop / S;
      const int m = h->cfg.migration_count > 0 ? h->cfg.migration_count : std::max(1, NPs / 8);
      if (d.pop % S != 0 || NPs < 4 || 2 * m > NPs)
        return h->fail(EMT_ERR_INVALID_ARG, "task " + std::to_string(i) +
                                                ": pop must split into sub-islands of >= 4 "
                                                "members, each sending at most half");
    }
    if (d.dim <= emt::kMaxDim && d.pop <= emt::kMaxPop &&
        (size_t)smem_cap < emt::smem_layout(d.dim, d.pop, false).total)
      return h->fail(EMT_ERR_UNSUPPORTED, "task " + std::to_string(i) +
                                              ": island does not fit in shared memory");
    HostTask ht;
    ht.fid = d.function;
    ht.D = d.dim;
    ht.NP = d.pop;
    if (d.lo < d.hi && std::isfinite(d.lo) && std::isfinite(d.hi)) {
      ht.lo = d.lo;
      ht.hi = d.hi;
    } else {
      emt_function_box(d.function, (h->cfg.flags & EMT_FLAG_REF_BOXES) ? 1 : 0, &ht.lo, &ht.hi);
    }
    const int D = d.dim;
    ht.Q.assign((size_t)D * D, 0.f);
    switch (d.rotation) {
      case EMT_ROTATION_IDENTITY:
        for (int k = 0; k < D; ++k) ht.Q[(size_t)k * D + k] = 1.f;
        break;
      case EMT_ROTATION_SEEDED_QR:
        ht.qr_id = id;
        break;
      case EMT_ROTATION_DENSE:
        if (!d.rotation_matrix) return h->fail(EMT_ERR_INVALID_ARG, "dense rotation without matrix");
        ht.dense = d.rotation_matrix;  // checked and converted below, in parallel
        break;
      case EMT_ROTATION_DIAG:
        if (!d.diag) return h->fail(EMT_ERR_INVALID_ARG, "diagonal rotation without factors");
        for (int k = 0; k < D; ++k) ht.Q[(size_t)k * D + k] = d.diag[k];
        break;
      default:
        return h->fail(EMT_ERR_INVALID_ARG, "bad rotation kind");
    }
    ht.o.assign(D, 0.f);
    if (d.shift) {
      for (int k = 0; k < D; ++k) ht.o[k] = d.shift[k];
    } else {
      const float a = emt::fmul(0.8f, ht.lo), r = emt::fmul(0.8f, emt::fsub(ht.hi, ht.lo));
      for (int k = 0; k < D; k += 4) {
        emt::U4 w = emt::draw(h->cfg.seed, id, 0, 0, emt::P_SHIFT, (uint32_t)(k >> 2));
        for (int qd = 0; qd < 4 && k + qd < D; ++qd) ht.o[k + qd] = emt::ffma(emt::u01(emt::word(w, qd)), r, a);
      }
    }
    if (h->cfg.flags & EMT_FLAG_REF_WEIERSTRASS_CONST)
      ht.woff64 = -(double)D * (double)weierstrass_reference_offset();
    else
      ht.woff64 = (double)D * (2.0 - 0x1p-20);
    ht.woff = (float)ht.woff64;
    add.push_back(std::move(ht));
  }
  // the O(D^2) and O(D^3) work per task on all host cores: seeded rotations
  // (an FP64 QR each), caller matrices (checked finite, rounded to FP32) and
  // every rotation's largest row norm
  std::vector<char> bad(add.size(), 0);
  auto finish = [&](size_t i, std::vector<double>& Q) {
    HostTask& ht = add[i];
    const int D = ht.D;
    if (ht.qr_id != UINT32_MAX) {
      seeded_rotation(h->cfg.seed, ht.qr_id, D, Q);
      for (size_t e = 0; e < Q.size(); ++e) ht.Q[e] = (float)Q[e];
    } else if (ht.dense) {
      for (size_t k = 0; k < (size_t)D * D; ++k) {
        if (!std::isfinite(ht.dense[k])) {
          bad[i] = 1;
          return;
        }
        ht.Q[k] = (float)ht.dense[k];
      }
    }
    ht.dense = nullptr;
    double qn = 0.0;
    for (int r = 0; r < D; ++r) {
      double s = 0.0;
      for (int c = 0; c < D; ++c) s += (double)ht.Q[(size_t)r * D + c] * ht.Q[(size_t)r * D + c];
      qn = std::max(qn, std::sqrt(s));
    }
    ht.qnorm = (float)qn;
  };
  size_t work = 0;
  for (const auto& ht : add) work += (size_t)ht.D * ht.D * (ht.qr_id != UINT32_MAX ? ht.D : 1);
  const int nth = work < 200000 ? 1
                              : (int)std::min<size_t>(add.size(),
                                                      std::max(1u, std::thread::hardware_concurrency()));
  if (nth <= 1) {
    std::vector<double> Q;
    for (size_t i = 0; i < add.size(); ++i) finish(i, Q);
  } else {
    std::vector<std::thread> pool;
    for (int w = 0; w < nth; ++w)
      pool.emplace_back([&, w] {
        std::vector<double> Q;
        for (size_t i = w; i < add.size(); i += nth) finish(i, Q);
      });
    for (auto& th : pool) th.join();
  }
  for (size_t i = 0; i < add.size(); ++i)
    if (bad[i]) return h->fail(EMT_ERR_INVALID_ARG, "task " + std::to_string(i) + ": non-finite rotation");
  if (h->initialized && !add.empty()) return join_tasks(h, add);
  for (auto& t : add) h->tasks.push_back(std::move(t));
  h->uploaded = false;
  h->initialized = false;
  return EMT_OK;
}

// Host allocations that grow with the handle (task matrices, staging
// buffers) fail as EMT_ERR_OUT_OF_MEMORY instead of unwinding through the C ABI.
int emt_add_tasks(emt_handle_t* h, int32_t n, const emt_task_desc* td) {
  try {
    return add_tasks_impl(h, n, td);
  } catch (const std::bad_alloc&) {
    return h ? h->fail(EMT_ERR_OUT_OF_MEMORY, "host memory") : EMT_ERR_OUT_OF_MEMORY;
  }
}

static int reset_impl(emt_handle_t* h, void* stream) {
  if (!h) return EMT_ERR_INVALID_ARG;
  const NvtxRange range("emt_reset");
  int rc = upload(h);
  if (rc) return rc;
  h->stream = (cudaStream_t)stream;
  int e;
  if (h->large) {
    e = emt_large_init(large_args(h), stream);
    if (!e) e = large_eval_members(h, h->stream);
  } else {
    emt::EpochArgs a = base_args(h, emt::MODE_INIT);
    e = launch_epoch(h, a, (int)h->tasks.size(), stream);
  }
  if (e) return h->cuda_fail((cudaError_t)e, "init launch");
  h->initialized = true;
  h->gdone = 0;
  h->gen_joined = 0;
  h->elite_parity = 0;
  return EMT_OK;
}

int emt_reset(emt_handle_t* h, void* stream) {
  try {
    return reset_impl(h, stream);
  } catch (const std::bad_alloc&) {
    return h ? h->fail(EMT_ERR_OUT_OF_MEMORY, "host memory") : EMT_ERR_OUT_OF_MEMORY;
  }
}

int emt_run(emt_handle_t* h, int32_t generations, void* stream) {
  if (!h) return EMT_ERR_INVALID_ARG;
  const NvtxRange range("emt_run");
  if (generations < 0) return h->fail(EMT_ERR_INVALID_ARG, "negative generation count");
  if (!h->initialized) {
    int rc = emt_reset(h, stream);
    if (rc) return rc;
  }
  h->stream = (cudaStream_t)stream;
  const std::vector<EpochStep> plan = plan_epochs(h, generations);
  const int rc = run_plan(h, plan, effective_schedule(h), effective_graph(h), h->stream);
  if (rc) return rc;
  apply_plan(h, plan);
  return EMT_OK;
}

int emt_time_rotation(emt_handle_t* h, int32_t reps, void* stream, float* ms) {
  if (!h || !ms || reps < 1) return EMT_ERR_INVALID_ARG;
  if (!h->initialized) {
    int rc = emt_reset(h, stream);
    if (rc) return rc;
  }
  if (!h->large) return h->fail(EMT_ERR_UNSUPPORTED, "the rotation of fused islands runs inside the epoch kernel");
  h->stream = (cudaStream_t)stream;
  const emt::LargeArgs a = large_args(h);
  cudaEventRecord(h->ev0, h->stream);
  int e = 0;
  for (int r = 0; r < reps && !e; ++r) e = emt_large_gemm(a, &h->smap, &h->qmap, h->stream);
  if (e) return h->cuda_fail((cudaError_t)e, "rotation launch");
  cudaEventRecord(h->ev1, h->stream);
  cudaError_t ce = cudaEventSynchronize(h->ev1);
  float t = 0.f;
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, h->ev0, h->ev1);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "rotation timing");
  h->timing_pending = false;
  *ms = t / (float)reps;
  return emt_sync(h);
}

int emt_tune(emt_handle_t* h, int32_t generations, void* stream, int32_t* chosen) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (generations <= 0) return h->fail(EMT_ERR_INVALID_ARG, "tuning needs generations > 0");
  if (!h->initialized) {
    int rc = emt_reset(h, stream);
    if (rc) return rc;
  }
  h->stream = (cudaStream_t)stream;
  std::vector<int> cands{EMT_SCHEDULE_SINGLE, EMT_SCHEDULE_SINGLE | 0x100, EMT_SCHEDULE_QUEUE,
                         EMT_SCHEDULE_QUEUE | 0x100};
  if (h->buckets.size() > 1) {
    cands.push_back(EMT_SCHEDULE_BUCKETS);
    cands.push_back(EMT_SCHEDULE_BUCKETS | 0x100);
  }
  int best = 0;
  float best_ms = 0.f;
  for (int c : cands) {
    const std::vector<EpochStep> plan = plan_epochs(h, generations);
    int rc = run_plan(h, plan, c & 0xFF, (c & 0x100) != 0, h->stream);
    if (rc) return rc;
    apply_plan(h, plan);
    cudaError_t e = cudaEventSynchronize(h->ev1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    if (e != cudaSuccess) return h->cuda_fail(e, "tuning");
    h->timing_pending = false;
    if (!best || ms < best_ms) {
      best = c;
      best_ms = ms;
    }
  }
  h->tuned = best;
  if (chosen) *chosen = best;
  return emt_sync(h);
}

// ---------------------------------------------------------------------------
// emt_run_noalloc: the epoch loop of emt_run with the elite-exchange scratch
// in a file-scope device array instead of the handle's allocation.
// ---------------------------------------------------------------------------
static __device__ __align__(256) float g_noalloc_exchange[2 * EMT_NOALLOC_EXCHANGE_FLOATS];

static std::mutex g_noalloc_mu;
static float* g_noalloc_ptr[256];  // device address of g_noalloc_exchange per ordinal

// Host code cannot use g_noalloc_exchange's name as a device address (it is a
// host-side stand-in): look the address up once per device, with that device
// current, and reuse it for the life of the process (a cudaDeviceReset by the
// caller would make it stale; the header says so).
static int noalloc_scratch(emt_handle* h, float** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (h->device < 0 || h->device >= 256) return h->fail(EMT_ERR_INVALID_ARG, "device ordinal");
  if (!g_noalloc_ptr[h->device]) {
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return h->cuda_fail(e, "cudaSetDevice");
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_exchange);
    if (e != cudaSuccess || !p) return h->cuda_fail(e, "cudaGetSymbolAddress");
    g_noalloc_ptr[h->device] = (float*)p;
  }
  *out = g_noalloc_ptr[h->device];
  return EMT_OK;
}

int emt_run_noalloc(emt_handle_t* h, int32_t generations, void* stream) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (generations < 0) return h->fail(EMT_ERR_INVALID_ARG, "negative generation count");
  if (!h->initialized || !h->uploaded)
    return h->fail(EMT_ERR_STATE, "emt_run_noalloc needs a handle prepared by emt_reset");
  if (h->large)
    return h->fail(EMT_ERR_UNSUPPORTED, "emt_run_noalloc serves islands of D <= 128 only");
  const int n = (int)h->tasks.size();
  const int interval = (h->cfg.transfer_interval > 0 && n > 1) ? h->cfg.transfer_interval : 0;
  float* buf[2] = {nullptr, nullptr};
  size_t need = 0;
  if (interval) {
    for (const auto& t : h->table) need += (size_t)t.NP * t.DP;
    if (need > (size_t)EMT_NOALLOC_EXCHANGE_FLOATS)
      return h->fail(EMT_ERR_UNSUPPORTED,
                     "emt_run_noalloc: the elite exchange needs " + std::to_string(need) +
                         " floats per buffer; the static buffer holds " +
                         std::to_string(EMT_NOALLOC_EXCHANGE_FLOATS));
    float* base = nullptr;
    int rc = noalloc_scratch(h, &base);
    if (rc) return rc;
    buf[0] = base;
    buf[1] = base + EMT_NOALLOC_EXCHANGE_FLOATS;
  }
  h->stream = (cudaStream_t)stream;
  cudaError_t ce = cudaSetDevice(h->device);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaSetDevice");
  // the exchange state the handle carries in: elites of the last boundary
  if (interval && h->gdone > 0 && h->gdone % (uint32_t)interval == 0) {
    const int in = h->elite_parity ^ 1;
    ce = cudaMemcpyAsync(buf[in], h->d_elites[in].p, sizeof(float) * need, cudaMemcpyDeviceToDevice,
                         h->stream);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "exchange copy in");
  }
  cudaEventRecord(h->ev0, h->stream);
  bool exported_last = false;
  int left = generations;
  while (left > 0) {
    int g = left;
    bool do_import = false, do_export = false;
    if (interval) {
      do_import = h->gdone > 0 && (h->gdone % (uint32_t)interval) == 0;
      int to_boundary = interval - (int)(h->gdone % (uint32_t)interval);
      g = std::min(left, to_boundary);
      do_export = ((h->gdone + (uint32_t)g) % (uint32_t)interval) == 0;
    }
    emt::EpochArgs a = base_args(h, emt::MODE_EPOCH);
    a.gens = g;
    if (interval) {
      a.transfer_import = do_import ? 1 : 0;
      a.transfer_export = do_export ? 1 : 0;
      a.elites_in = buf[h->elite_parity ^ 1];
      a.elites_out = buf[h->elite_parity];
    }
    int e = launch_epoch(h, a, n, stream);
    if (e) return h->cuda_fail((cudaError_t)e, "epoch launch");
    exported_last = interval && do_export;
    if (exported_last) h->elite_parity ^= 1;
    h->gdone += (uint32_t)g;
    left -= g;
  }
  // the exchange state the handle carries out, for its next emt_run
  if (exported_last) {
    const int in = h->elite_parity ^ 1;
    ce = cudaMemcpyAsync(h->d_elites[in].p, buf[in], sizeof(float) * need, cudaMemcpyDeviceToDevice,
                         h->stream);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "exchange copy out");
  }
  cudaEventRecord(h->ev1, h->stream);
  h->timing_pending = true;
  return EMT_OK;
}

int emt_sync(emt_handle_t* h) {
  if (!h) return EMT_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "stream synchronize");
  e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "kernel");
  if (h->timing_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev0, h->ev1) == cudaSuccess) h->device_ms = ms;
    h->timing_pending = false;
  }
  if (h->d_err.p) {
    int32_t code = 0;
    e = cudaMemcpy(&code, h->d_err.p, sizeof(code), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "error word");
    if (code) {
      cudaMemset(h->d_err.p, 0, sizeof(int32_t));
      cudaStreamSynchronize(nullptr);  // cleared before the next launch on any stream
      return h->fail(EMT_ERR_DEVICE_CHECK, "device check " + std::to_string(code) +
                                               (code == emt::CHECK_BAD_DESCRIPTOR ? " (bad task descriptor)"
                                                : code == emt::CHECK_SMEM_TOO_SMALL ? " (shared memory too small)"
                                                : code == emt::CHECK_BAD_PARTNER ? " (bad transfer partner)"
                                                : code == emt::CHECK_TIMEOUT ? " (a bounded device wait ran out)"
                                                : code == emt::CHECK_TC_SHAPE ? " (island outside the tensor-core form's limits)"
                                                : code == emt::CHECK_SMEM_ALIGN ? " (shared memory not 1024-byte aligned)"
                                                                                 : ""));
    }
  }
  return EMT_OK;
}

static int ensure_ready(emt_handle* h) {
  if (h->tasks.empty()) return h->fail(EMT_ERR_STATE, "no tasks");
  if (!h->initialized) {
    int rc = emt_reset(h, h->stream);
    if (rc) return rc;
  }
  return emt_sync(h);
}

emt::BestArgs best_args(emt_handle* h) {
  return emt::BestArgs{h->d_tasks.p,  (int32_t)h->tasks.size(), h->d_pop.p, h->d_fit32.p,
                       h->d_fit64.p,  h->d_qt.p, h->d_shift.p, h->d_best_idx.p,
                       h->d_best_f32.p, h->d_best_f64.p, h->d_tol32.p,
                       (float)(h->cfg.recheck_rel > 0 ? h->cfg.recheck_rel : 1e-5),
                       h->d_best_err.p};
}

int emt_get_best(emt_handle_t* h, int32_t task, double* fitness, float* x) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (check_task(h, task)) return h->fail(EMT_ERR_INVALID_ARG, "task index out of range");
  int rc = ensure_ready(h);
  if (rc) return rc;
  const emt::BestArgs b = best_args(h);
  int e = h->large ? emt_large_best(b, h->lKp, h->stream) : emt_launch_best(b, h->stream);
  if (e) return h->cuda_fail((cudaError_t)e, "best launch");
  if ((rc = emt_sync(h))) return rc;
  int32_t idx = 0;
  double f = 0.0;
  cudaMemcpy(&idx, h->d_best_idx.p + task, sizeof(idx), cudaMemcpyDeviceToHost);
  cudaMemcpy(&f, h->d_best_f64.p + task, sizeof(f), cudaMemcpyDeviceToHost);
  if (fitness) *fitness = f;
  if (x) {
    const TaskDev& d = h->table[task];
    cudaError_t ce = cudaMemcpy(x, h->d_pop.p + d.pop_off + (size_t)idx * d.DP, sizeof(float) * d.D,
                                cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "copy best");
  }
  return EMT_OK;
}

int emt_get_best_all(emt_handle_t* h, float* fitness) {
  if (!h || !fitness) return EMT_ERR_INVALID_ARG;
  int rc = ensure_ready(h);
  if (rc) return rc;
  const emt::BestArgs b = best_args(h);
  int e = h->large ? emt_large_best(b, h->lKp, h->stream) : emt_launch_best(b, h->stream);
  if (e) return h->cuda_fail((cudaError_t)e, "best launch");
  cudaError_t ce = cudaMemcpyAsync(fitness, h->d_best_f32.p, sizeof(float) * h->tasks.size(),
                                   cudaMemcpyDeviceToHost, h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "copy best");
  return emt_sync(h);
}

int emt_get_population(emt_handle_t* h, int32_t task, float* x, float* fitness) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (check_task(h, task)) return h->fail(EMT_ERR_INVALID_ARG, "task index out of range");
  int rc = ensure_ready(h);
  if (rc) return rc;
  const TaskDev& d = h->table[task];
  cudaError_t e = cudaSuccess;
  if (x)
    e = cudaMemcpy2D(x, sizeof(float) * d.D, h->d_pop.p + d.pop_off, sizeof(float) * d.DP,
                     sizeof(float) * d.D, d.NP, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && fitness)
    e = cudaMemcpy(fitness, h->d_fit32.p + d.fit_off, sizeof(float) * d.NP, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return h->cuda_fail(e, "copy population");
  return EMT_OK;
}

int emt_set_population(emt_handle_t* h, int32_t task, const float* x) {
  if (!h || !x) return EMT_ERR_INVALID_ARG;
  if (check_task(h, task)) return h->fail(EMT_ERR_INVALID_ARG, "task index out of range");
  int rc = ensure_ready(h);
  if (rc) return rc;
  const TaskDev& d = h->table[task];
  for (size_t k = 0; k < (size_t)d.NP * d.D; ++k)
    if (!(x[k] >= d.lo && x[k] <= d.hi)) return h->fail(EMT_ERR_INVALID_ARG, "member outside the box");
  // on the handle's stream, ahead of the evaluation launched there
  cudaError_t e = cudaMemcpy2DAsync(h->d_pop.p + d.pop_off, sizeof(float) * d.DP, x,
                                    sizeof(float) * d.D, sizeof(float) * d.D, d.NP,
                                    cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "copy population");
  int le;
  if (h->large) {  // re-evaluates every island (unchanged ones get the same values)
    e = cudaMemsetAsync(h->d_fit64.p + d.fit_off, 0xFF, sizeof(double) * d.NP, h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "reset cache");
    le = large_eval_members(h, h->stream);
  } else {
    emt::EpochArgs a = base_args(h, emt::MODE_EVAL);
    a.single_task = task;
    le = launch_epoch(h, a, 1, h->stream);
  }
  if (le) return h->cuda_fail((cudaError_t)le, "evaluate launch");
  return emt_sync(h);
}

int emt_get_task_info(emt_handle_t* h, int32_t task, int32_t* function, int32_t* dim,
                      int32_t* pop) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (check_task(h, task)) return h->fail(EMT_ERR_INVALID_ARG, "task index out of range");
  const HostTask& t = h->tasks[task];
  if (function) *function = t.fid;
  if (dim) *dim = t.D;
  if (pop) *pop = t.NP;
  return EMT_OK;
}

int emt_get_task_params(emt_handle_t* h, int32_t task, float* rotation, float* shift) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (check_task(h, task)) return h->fail(EMT_ERR_INVALID_ARG, "task index out of range");
  const HostTask& t = h->tasks[task];
  if (rotation) std::memcpy(rotation, t.Q.data(), sizeof(float) * t.Q.size());
  if (shift) std::memcpy(shift, t.o.data(), sizeof(float) * t.o.size());
  return EMT_OK;
}

int emt_evaluate(emt_handle_t* h, int32_t task, int32_t n, const float* x, float* fitness,
                 float* z) {
  if (!h || (n > 0 && (!x || !fitness)) || n < 0) return EMT_ERR_INVALID_ARG;
  if (check_task(h, task)) return h->fail(EMT_ERR_INVALID_ARG, "task index out of range");
  int rc = upload(h);
  if (rc) return rc;
  if (n == 0) return EMT_OK;
  if (h->large)
    return h->fail(EMT_ERR_UNSUPPORTED, "emt_evaluate serves islands of D <= 128; read a large "
                                        "island's fitness with emt_get_population");
  const HostTask& t = h->tasks[task];
  float *dx = nullptr, *df = nullptr, *dz = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&dx, sizeof(float) * (size_t)n * t.D)) != cudaSuccess) return h->cuda_fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&df, sizeof(float) * (size_t)n)) != cudaSuccess) {
    cudaFree(dx);
    return h->cuda_fail(e, "cudaMalloc");
  }
  if (z && (e = cudaMalloc(&dz, sizeof(float) * (size_t)n * t.D)) != cudaSuccess) {
    cudaFree(dx);
    cudaFree(df);
    return h->cuda_fail(e, "cudaMalloc");
  }
  e = cudaMemcpyAsync(dx, x, sizeof(float) * (size_t)n * t.D, cudaMemcpyHostToDevice, h->stream);
  int out = EMT_OK;
  if (e == cudaSuccess) {
    emt::EvalArgs a{h->d_tasks.p, task, n, dx, df, dz, h->d_qt.p, h->d_shift.p, h->d_err.p,
                    emt::smem_layout(t.D, 64).total};
    int le = emt_launch_eval(a, h->stream);
    if (le) out = h->cuda_fail((cudaError_t)le, "evaluate launch");
    else if ((out = emt_sync(h)) == EMT_OK) {
      e = cudaMemcpy(fitness, df, sizeof(float) * n, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && z) e = cudaMemcpy(z, dz, sizeof(float) * (size_t)n * t.D, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) out = h->cuda_fail(e, "copy results");
    }
  } else {
    out = h->cuda_fail(e, "copy points");
  }
  cudaFree(dx);
  cudaFree(df);
  if (dz) cudaFree(dz);
  return out;
}

int emt_get_stats(emt_handle_t* h, emt_stats* out) {
  if (!h || !out) return EMT_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  out->n_tasks = (int32_t)h->tasks.size();
  out->precision_used = h->use_tc ? (h->tc_bf16 ? EMT_ROT_BF16X3 : EMT_ROT_TF32X3)
                       : (h->large && h->large_tc) ? EMT_ROT_TF32X3 : EMT_ROT_FP32;
  if (h->d_stats.p) {
    int rc = emt_sync(h);
    if (rc) return rc;
    unsigned long long s[emt::kStats];
    cudaError_t e = cudaMemcpy(s, h->d_stats.p, sizeof(s), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "copy stats");
    out->recheck_differential = s[4];
    out->anchor_rotations = s[5];
    out->recheck_identical = s[6];
    out->rechecks = s[0];
    out->recheck_flips = s[1];
    out->transfers_accepted = s[2];
    out->evaluations = s[3];
    out->migrations_accepted = s[7];
    out->recheck_fp64_terms = s[emt::kStatWeierFp64];
    out->generations = h->initialized ? (uint64_t)h->gdone * h->tasks.size() - h->gen_joined : 0;
  }
  if (h->initialized && !h->tasks.empty()) {
    // the largest relative error of a task's best FP32 fitness against its
    // FP64-class value
    const emt::BestArgs b = best_args(h);
    int e = h->large ? emt_large_best(b, h->lKp, h->stream) : emt_launch_best(b, h->stream);
    if (e) return h->cuda_fail((cudaError_t)e, "best launch");
    std::vector<float> err(h->tasks.size());
    cudaError_t ce = cudaMemcpyAsync(err.data(), h->d_best_err.p, sizeof(float) * err.size(),
                                     cudaMemcpyDeviceToHost, h->stream);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "copy best error");
    int rc = emt_sync(h);
    if (rc) return rc;
    for (float v : err) out->max_rel_err = std::max(out->max_rel_err, (double)v);
  }
  out->device_ms = h->device_ms;
  if (h->uploaded) {
    const int sched = effective_schedule(h);
    out->schedule_used = sched | (effective_graph(h) ? 0x100 : 0);
    out->epoch_launches = sched == EMT_SCHEDULE_SINGLE || sched == EMT_SCHEDULE_QUEUE ? 1
                          : sched == EMT_SCHEDULE_BUCKETS ? (int32_t)h->buckets.size()
                                                          : (int32_t)h->tasks.size();
  }
  return EMT_OK;
}

int emt_get_phase_cycles(emt_handle_t* h, uint64_t* cycles, int32_t n) {
  if (!h || !cycles || n < 0) return EMT_ERR_INVALID_ARG;
#ifndef EMT_PHASE_CLOCKS
  return h->fail(EMT_ERR_UNSUPPORTED, "phase clocks need the measurement build (EMT_PHASE_CLOCKS)");
#else
  if (!h->d_stats.p) return h->fail(EMT_ERR_STATE, "no run yet");
  int rc = emt_sync(h);
  if (rc) return rc;
  unsigned long long s[emt::kStats];
  cudaError_t e = cudaMemcpy(s, h->d_stats.p, sizeof(s), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return h->cuda_fail(e, "copy phase clocks");
  for (int k = 0; k < n; ++k) cycles[k] = k < emt::kPhases ? (uint64_t)s[8 + k] : 0u;
  return EMT_OK;
#endif
}

// Checkpoint layout: magic, task count, generation counter, then per task
// pop (NP*D floats), fit32, tol32 (NP floats), fit64 (NP doubles), gen.
static const uint64_t kSnapMagic = 0x31504E5354464D45ull;  // "EMFTSNP1"

int emt_snapshot_size(emt_handle_t* h, size_t* bytes) {
  if (!h || !bytes) return EMT_ERR_INVALID_ARG;
  size_t s = 3 * sizeof(uint64_t);
  for (const auto& t : h->tasks) s += (size_t)t.NP * t.D * 4 + (size_t)t.NP * (4 + 4 + 8) + 4;
  *bytes = s;
  return EMT_OK;
}

int emt_snapshot(emt_handle_t* h, void* buf, size_t bytes) {
  if (!h || !buf) return EMT_ERR_INVALID_ARG;
  size_t need = 0;
  emt_snapshot_size(h, &need);
  if (bytes < need) return h->fail(EMT_ERR_INVALID_ARG, "snapshot buffer too small");
  int rc = ensure_ready(h);
  if (rc) return rc;
  unsigned char* p = (unsigned char*)buf;
  uint64_t hdr[3] = {kSnapMagic, (uint64_t)h->tasks.size(), (uint64_t)h->gdone};
  std::memcpy(p, hdr, sizeof(hdr));
  p += sizeof(hdr);
  for (size_t t = 0; t < h->tasks.size(); ++t) {
    const TaskDev& d = h->table[t];
    cudaError_t e = cudaMemcpy2D(p, sizeof(float) * d.D, h->d_pop.p + d.pop_off, sizeof(float) * d.DP,
                                 sizeof(float) * d.D, d.NP, cudaMemcpyDeviceToHost);
    p += (size_t)d.NP * d.D * 4;
    if (e == cudaSuccess) e = cudaMemcpy(p, h->d_fit32.p + d.fit_off, 4 * (size_t)d.NP, cudaMemcpyDeviceToHost);
    p += 4 * (size_t)d.NP;
    if (e == cudaSuccess) e = cudaMemcpy(p, h->d_tol32.p + d.fit_off, 4 * (size_t)d.NP, cudaMemcpyDeviceToHost);
    p += 4 * (size_t)d.NP;
    if (e == cudaSuccess) e = cudaMemcpy(p, h->d_fit64.p + d.fit_off, 8 * (size_t)d.NP, cudaMemcpyDeviceToHost);
    p += 8 * (size_t)d.NP;
    if (e == cudaSuccess) e = cudaMemcpy(p, h->d_gen.p + t, 4, cudaMemcpyDeviceToHost);
    p += 4;
    if (e != cudaSuccess) return h->cuda_fail(e, "snapshot");
  }
  return EMT_OK;
}

int emt_restore(emt_handle_t* h, const void* buf, size_t bytes) {
  if (!h || !buf) return EMT_ERR_INVALID_ARG;
  size_t need = 0;
  emt_snapshot_size(h, &need);
  if (bytes < need) return h->fail(EMT_ERR_INVALID_ARG, "snapshot too small");
  const unsigned char* p = (const unsigned char*)buf;
  uint64_t hdr[3];
  std::memcpy(hdr, p, sizeof(hdr));
  p += sizeof(hdr);
  if (hdr[0] != kSnapMagic || hdr[1] != h->tasks.size())
    return h->fail(EMT_ERR_INVALID_ARG, "snapshot does not match this handle");
  int rc = upload(h);
  if (rc) return rc;
  for (size_t t = 0; t < h->tasks.size(); ++t) {
    const TaskDev& d = h->table[t];
    cudaError_t e = cudaMemcpy2D(h->d_pop.p + d.pop_off, sizeof(float) * d.DP, p, sizeof(float) * d.D,
                                 sizeof(float) * d.D, d.NP, cudaMemcpyHostToDevice);
    p += (size_t)d.NP * d.D * 4;
    if (e == cudaSuccess) e = cudaMemcpy(h->d_fit32.p + d.fit_off, p, 4 * (size_t)d.NP, cudaMemcpyHostToDevice);
    p += 4 * (size_t)d.NP;
    if (e == cudaSuccess) e = cudaMemcpy(h->d_tol32.p + d.fit_off, p, 4 * (size_t)d.NP, cudaMemcpyHostToDevice);
    p += 4 * (size_t)d.NP;
    if (e == cudaSuccess) e = cudaMemcpy(h->d_fit64.p + d.fit_off, p, 8 * (size_t)d.NP, cudaMemcpyHostToDevice);
    p += 8 * (size_t)d.NP;
    if (e == cudaSuccess) e = cudaMemcpy(h->d_gen.p + t, p, 4, cudaMemcpyHostToDevice);
    p += 4;
    if (e != cudaSuccess) return h->cuda_fail(e, "restore");
  }
  // the cached compensated rotations belong to the replaced islands
  cudaError_t ez = cudaMemset(h->d_zcb.p, 0xFF, sizeof(float) * h->d_zcb.n);
  if (ez == cudaSuccess && h->d_wprec.p)  // restored values are not known to be float-float
    ez = cudaMemset(h->d_wprec.p, 0xFF, sizeof(float) * h->d_wprec.n);
  // the copies and memsets above run on the legacy default stream, which a
  // non-blocking caller stream does not wait for
  if (ez == cudaSuccess) ez = cudaStreamSynchronize(nullptr);
  if (ez != cudaSuccess) return h->cuda_fail(ez, "restore");
  h->gdone = (uint32_t)hdr[2];
  h->initialized = true;
  h->elite_parity = 0;
  // At a transfer boundary the next epoch imports the elites exported at the
  // end of the last one: export them again from the restored islands (they
  // rank by the same restored FP32 fitness, so the rows are identical).
  const int interval = (h->cfg.transfer_interval > 0 && h->tasks.size() > 1) ? h->cfg.transfer_interval : 0;
  if (interval && h->gdone > 0 && h->gdone % (uint32_t)interval == 0) {
    int e;
    if (h->large) {
      emt::LargeArgs la = large_args(h);
      la.elites_out = h->d_elites[0].p;
      e = emt_large_select(la, emt::large::SEL_EXPORT, h->stream);
    } else {
      emt::EpochArgs a = base_args(h, emt::MODE_EPOCH);
      a.gens = 0;
      a.transfer_export = 1;
      a.elites_out = h->d_elites[0].p;
      e = launch_epoch(h, a, (int)h->tasks.size(), h->stream);
    }
    if (e) return h->cuda_fail((cudaError_t)e, "elite export");
    h->elite_parity = 1;
    return emt_sync(h);
  }
  return EMT_OK;
}

const char* emt_last_error(const emt_handle_t* h) { return h ? h->err.c_str() : "null handle"; }

void emt_destroy(emt_handle_t* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->d_tasks.release();
  h->d_order.release();
  h->d_pop.release();
  h->d_fit32.release();
  h->d_tol32.release();
  h->d_qt.release();
  h->d_shift.release();
  h->d_elites[0].release();
  h->d_elites[1].release();
  h->d_best_f32.release();
  h->d_fit64.release();
  h->d_zc.release();
  h->d_zcb.release();
  h->d_best_f64.release();
  h->d_best_err.release();
  h->d_gen.release();
  h->d_stats.release();
  h->d_err.release();
  h->d_best_idx.release();
  h->d_qtc.release();
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  for (int i = 0; i < emt_handle::kSide; ++i) {
    if (h->side[i]) cudaStreamDestroy(h->side[i]);
    if (h->join_ev[i]) cudaEventDestroy(h->join_ev[i]);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->cap) cudaStreamDestroy(h->cap);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  delete h;
}

}  // extern "C"
