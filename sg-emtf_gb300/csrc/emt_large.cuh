// emt_large.cuh -- islands too large for one CTA's shared memory (D up to
// 1024 or NP up to 512; D = 1000, NP = 256 GA islands, or the reference's
// D = 50, NP = 512 GA islands).  Included at the end of
// emt_kernels.cu, whose selection and ranking code it reuses.
//
// A generation is a pipeline of kernels over HBM-resident islands:
//   build   trial genes (DE or GA, the same arithmetic and Philox stream as
//           the fused kernel) and the rotation operand s = u - o, split into
//           TF32 hi/lo planes for the tensor-core form;
//   gemm    Z = S Q^T for every task: tcgen05.mma kind::tf32 (4 products of
//           the rounded hi/lo pairs, FP32 accumulation in tensor memory), 128 x
//           256 tiles fed by TMA (128B swizzle) through a 2-stage mbarrier
//           pipeline; or FP32 CUDA-core tiles (128 x 128, 8 x 8 per thread);
//   eval    one warp per row: f and its rounding window from the Z row;
//   select  one CTA per task: the fused kernel's selection with its near-tie
//           re-check (global-memory operands, shared-memory scratch).
// Elite transfer reuses rank/select with the candidates in the trial rows.
#pragma once

namespace emt {
namespace large {

__device__ __forceinline__ bool large_ok(const TaskDev& t) {
  return t.D >= 1 && t.D <= kMaxDimLarge && t.NP >= 4 && t.NP <= kMaxPopLarge && t.DP == round4(t.D);
}

__device__ __forceinline__ FnConst fn_const(const TaskDev& td, float rel) {
  FnConst fc;
  fc.fid = td.fid;
  fc.D = td.D;
  fc.flags = td.flags;
  fc.woff = td.woff;
  fc.qnorm = td.qnorm;
  fc.rel = rel;
  fc.woff64 = td.woff64;
  return fc;
}

// Transfer partner and candidate count of task t at generation gen0 (the
// fused kernel's rule); -1 when there is none.
// migrants each sub-island sends, and whether generation gen[t] + 1 opens
// with a migration (as the fused kernel's epoch loop decides it)
__device__ __forceinline__ int migration_count(const LargeArgs& a, int NP) {
  const int NPs = NP / a.subislands;
  return a.mig_count > 0 ? a.mig_count : max(1, NPs / 8);
}
__device__ __forceinline__ bool migration_due(const LargeArgs& a, int t) {
  const uint32_t G = a.gen[t] + 1u;
  return a.subislands > 1 && a.mig_interval > 0 && G > 1u &&
         (G - 1u) % (uint32_t)a.mig_interval == 0u;
}

__device__ __forceinline__ int transfer_partner(const LargeArgs& a, int t, uint32_t gen0, int& k) {
  if (a.n_tasks < 2) return -1;
  const U4 w = draw(a.seed, (uint32_t)t, gen0, 0u, P_TRANSFER_PARTNER, 0);
  uint32_t p = w.x % (uint32_t)(a.n_tasks - 1);
  if (p >= (uint32_t)t) ++p;
  const TaskDev pd = a.tasks[p];
  if (!large_ok(pd)) return -1;
  const int kt = transfer_k(a.transfer_rate, a.tasks[t].NP), kp = transfer_k(a.transfer_rate, pd.NP);
  k = kt < kp ? kt : kp;
  return (int)p;
}

// Operand row of s = v - o: FP32 (FP32 form) or TF32 hi/lo planes, both
// rounded to nearest TF32 (v = hi + lo + r, |r| <= 2^-24 |v|, unbiased; the
// tensor core would otherwise truncate lo, and over K = 1000 products that
// bias reaches 1e-5 of the fitness scale).
__device__ __forceinline__ void put_s(const LargeArgs& a, int64_t row, int j, float v) {
  float* p = a.S + row * a.Kp + j;
  if (a.tc) {
    const float hi = tc::tf32_round(v);
    p[0] = hi;
    p[a.split] = tc::tf32_round(v - hi);
  } else {
    p[0] = v;
  }
}

// ---------------------------------------------------------------------------
// initial islands (the fused kernel's MODE_INIT draw)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) init_kernel(const LargeArgs a) {
  const int task = blockIdx.y;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) {
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicCAS(a.err, 0, CHECK_BAD_DESCRIPTOR);
    return;
  }
  const int D = td.D, NP = td.NP, DP = td.DP, nb = (D + 3) >> 2;
  const float r = fsub(td.hi, td.lo);
  float* X = a.pop + td.pop_off;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < NP * nb; it += gridDim.x * blockDim.x) {
    const int i = it / nb, b = it - i * nb;
    const U4 w = draw(a.seed, (uint32_t)task, 0u, (uint32_t)i, P_POP_INIT, (uint32_t)b);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = 4 * b + q;
      if (j < D) X[(size_t)i * DP + j] = fminf(ffma(u01(word(w, q)), r, td.lo), td.hi);
    }
    if (4 * b + 4 >= DP)
      for (int j = D; j < DP; ++j) X[(size_t)i * DP + j] = 0.f;
    if (b == 0) a.fit64[td.fit_off + i] = __longlong_as_double(0x7FF8000000000000ll);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.gen[task] = 0u;
    if (a.stats) atomicAdd(a.stats + 3, (unsigned long long)NP);  // the initial evaluation
  }
}

// ---------------------------------------------------------------------------
// trial rows and rotation operands; one CTA per (task, 8 members)
// ---------------------------------------------------------------------------
constexpr int kBuildRows = 8;

__global__ void __launch_bounds__(256) build_kernel(const LargeArgs a, int mode) {
  __shared__ int sidx[kBuildRows][4];
  __shared__ int spart[kBuildRows];
  const int task = blockIdx.y;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  const int D = td.D, NP = td.NP, DP = td.DP;
  const int i0 = blockIdx.x * kBuildRows;
  if (i0 >= NP) return;
  const int nrow = min(kBuildRows, NP - i0);
  const float* X = a.pop + td.pop_off;
  float* U = a.U + td.pop_off;
  const float* o = a.shift + td.o_off;
  const int64_t srow = a.srow[task];
  const float lo = td.lo, hi = td.hi;

  if (mode == BUILD_X) {  // operands of the members themselves
    for (int it = threadIdx.x; it < nrow * D; it += blockDim.x) {
      const int r = it / D, j = it - r * D, i = i0 + r;
      put_s(a, srow + i, j, fsub(X[(size_t)i * DP + j], o[j]));
    }
    return;
  }
  const uint32_t gen0 = a.gen[task];
  if (mode == BUILD_CANDIDATES) {
    int k = 0;
    const int p = transfer_partner(a, task, gen0, k);
    if (p < 0 || i0 >= k) return;
    const TaskDev pd = a.tasks[p];
    const float* el = a.elites_in + pd.elite_off;
    const int* byrank = a.rank + td.fit_off;
    const float rp = fsub(pd.hi, pd.lo), rt = fsub(td.hi, td.lo);
    const int nc = min(nrow, k - i0);
    for (int it = threadIdx.x; it < nc * D; it += blockDim.x) {
      const int r = it / D, j = it - r * D, c = i0 + r;
      const U4 wm = draw(a.seed, (uint32_t)task, gen0, (uint32_t)c, P_TRANSFER_MIX, (uint32_t)(j >> 2));
      float v = X[(size_t)byrank[c] * DP + j];
      if (j < pd.D && u01(word(wm, j & 3)) < a.transfer_mix) {
        const float q = fdiv(fsub(el[(size_t)c * pd.DP + j], pd.lo), rp);
        v = clamp_box(ffma(q, rt, td.lo), td.lo, td.hi);
      }
      U[(size_t)c * DP + j] = v;
      put_s(a, srow + c, j, fsub(v, o[j]));
    }
    return;
  }
  // ---- trials of generation G (partners from the member's sub-island) ----
  const uint32_t G = gen0 + 1u;
  const int NPs = NP / a.subislands;
  if (a.algorithm == 0 || a.algorithm == 1) {
    if (threadIdx.x < nrow) {
      const int i = i0 + threadIdx.x;
      const int base = a.subislands > 1 ? (i / NPs) * NPs : 0;
      const U4 w = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_DE_INDEX, 0);
      int r1, r2, r3, jr;
      de_indices(w, i - base, NPs, D, r1, r2, r3, jr);
      sidx[threadIdx.x][0] = a.algorithm == 0 ? base + r1 : i;
      sidx[threadIdx.x][1] = base + r2;
      sidx[threadIdx.x][2] = base + r3;
      sidx[threadIdx.x][3] = jr;
    }
    __syncthreads();
    const int nb = (D + 3) >> 2;
    for (int it = threadIdx.x; it < nrow * nb; it += blockDim.x) {
      const int r = it / nb, b = it - r * nb, i = i0 + r;
      const U4 w = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_DE_CR, (uint32_t)b);
      const float* xb = X + (size_t)sidx[r][0] * DP;
      const float* x2 = X + (size_t)sidx[r][1] * DP;
      const float* x3 = X + (size_t)sidx[r][2] * DP;
      const float* xi = X + (size_t)i * DP;
      const int jr = sidx[r][3];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = 4 * b + q;
        if (j < D) {
          const float m = clamp_box(ffma(a.F, fsub(x2[j], x3[j]), xb[j]), lo, hi);
          const float t = (u01(word(w, q)) < a.CR || j == jr) ? m : xi[j];
          U[(size_t)i * DP + j] = t;
          put_s(a, srow + i, j, fsub(t, o[j]));
        }
      }
    }
    return;
  }
  // GA: parent per member (CrossPrep), SBX on the pair (i, i^1), polynomial
  // mutation -- the fused kernel's build_trials, gene for gene
  if (threadIdx.x < nrow) {
    const int i = i0 + threadIdx.x;
    const int base = a.subislands > 1 ? (i / NPs) * NPs : 0;
    sidx[threadIdx.x][0] =
        base + (int)(draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_GA_PARENT, 0).x % (uint32_t)NPs);
    const int pi = i ^ 1;
    const bool paired = pi < NP && (a.subislands == 1 || pi / NPs == i / NPs);
    spart[threadIdx.x] =
        paired ? base + (int)(draw(a.seed, (uint32_t)task, G, (uint32_t)pi, P_GA_PARENT, 0).x %
                              (uint32_t)NPs)
               : sidx[threadIdx.x][0];
  }
  __syncthreads();
  const float ec = fdiv(1.f, fadd(a.eta_c, 1.f));
  const float em1 = fadd(a.eta_m, 1.f), em = fdiv(1.f, em1);
  const float pm = a.p_m < 0.f ? fdiv(1.f, (float)D) : a.p_m;
  const float range = fsub(hi, lo);
  const int nb = (D + 1) >> 1;
  for (int it = threadIdx.x; it < nrow * nb; it += blockDim.x) {
    const int r = it / nb, b = it - r * nb, i = i0 + r;
    const int r0 = sidx[r][0], partner = spart[r];
    const U4 ws = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_GA_SBX, (uint32_t)b);
    const U4 wm = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_GA_PM, (uint32_t)b);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = 2 * b + h;
      if (j >= D) break;
      const float x0 = X[(size_t)r0 * DP + j], x1 = X[(size_t)partner * DP + j];
      float c;
      if (u01(word(ws, 2 * h)) < a.p_c) {
        const float pu = u01(word(ws, 2 * h + 1));
        const float tv = pu <= 0.5f ? fmul(2.f, pu) : fdiv(0.5f, fsub(1.f, pu));
        float beta = det_powf(tv, ec);
        if (i & 1) beta = -beta;
        c = fmul(0.5f, ffma(fadd(1.f, beta), x0, fmul(fsub(1.f, beta), x1)));
        c = clamp_box(c, lo, hi);
      } else {
        c = x0;
      }
      if (u01(word(wm, 2 * h)) < pm) {
        const float um = u01(word(wm, 2 * h + 1));
        float dq;
        if (um <= 0.5f) {
          const float d1 = fdiv(fsub(c, lo), range);
          const float v = ffma(fsub(1.f, fmul(2.f, um)), det_powf(fsub(1.f, d1), em1), fmul(2.f, um));
          dq = fsub(det_powf(v, em), 1.f);
        } else {
          const float d2 = fdiv(fsub(hi, c), range);
          const float v = ffma(fmul(2.f, fsub(um, 0.5f)), det_powf(fsub(1.f, d2), em1),
                               fmul(2.f, fsub(1.f, um)));
          dq = fsub(1.f, det_powf(v, em));
        }
        c = clamp_box(ffma(dq, range, c), lo, hi);
      }
      U[(size_t)i * DP + j] = c;
      put_s(a, srow + i, j, fsub(c, o[j]));
    }
  }
}

// ---------------------------------------------------------------------------
// Z = S Q^T, FP32 form: 128 x 128 tiles, K step 16, 8 x 8 outputs per thread
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) gemm_f32_kernel(const LargeArgs a) {
  constexpr int BM = 128, BN = 128, BK = 16;
  __shared__ __align__(16) float As[BK][BM + 4];
  __shared__ __align__(16) float Bs[BK][BN + 4];
  const int task = blockIdx.z;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if (m0 >= td.NP || n0 >= td.D) return;
  const int D = td.D, DP = td.DP;
  const float* S = a.S + (a.srow[task] + m0) * (int64_t)a.Kp;
  const float* QT = a.qt + td.q_off;  // QT[k * DP + n] = Q[n][k]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[8][8];
#pragma unroll
  for (int r = 0; r < 8; ++r)
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[r][c] = 0.f;
  for (int k0 = 0; k0 < D; k0 += BK) {
    // A tile: 128 rows x 16 k, transposed into As[k][row]
    for (int it = threadIdx.x; it < BM * BK / 4; it += 256) {
      const int r = it >> 2, kq = (it & 3) * 4;
      const float4 v = *reinterpret_cast<const float4*>(S + (int64_t)r * a.Kp + k0 + kq);
      As[kq + 0][r] = v.x;
      As[kq + 1][r] = v.y;
      As[kq + 2][r] = v.z;
      As[kq + 3][r] = v.w;
    }
    // B tile: Q^T rows k0..k0+15, columns n0..n0+127 (zero beyond D)
    for (int it = threadIdx.x; it < BK * BN; it += 256) {
      const int kk = it / BN, n = it - kk * BN;
      const int k = k0 + kk, col = n0 + n;
      Bs[kk][n] = (k < D && col < D) ? QT[(int64_t)k * DP + col] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float av[8], bv[8];
      const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][64 + tx * 4]);
      av[0] = a0.x; av[1] = a0.y; av[2] = a0.z; av[3] = a0.w;
      av[4] = a1.x; av[5] = a1.y; av[6] = a1.z; av[7] = a1.w;
      bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
      bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
#pragma unroll
      for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
    }
    __syncthreads();
  }
  float* Z = a.Z + (a.srow[task] + m0) * (int64_t)a.Nq + n0;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int row = (r < 4 ? ty * 4 + r : 64 + ty * 4 + r - 4);
    if (m0 + row >= td.NP) continue;
    float* zr = Z + (int64_t)row * a.Nq;
    *reinterpret_cast<float4*>(zr + tx * 4) = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
    *reinterpret_cast<float4*>(zr + 64 + tx * 4) =
        make_float4(acc[r][4], acc[r][5], acc[r][6], acc[r][7]);
  }
}

// ---------------------------------------------------------------------------
// Z = S Q^T, tensor-core form: one CTA per (task, 128-row, 256-column) tile.
// warp 0: TMA producer; warp 1: TMEM owner and MMA issuer; warps 2-5: epilogue
// (tcgen05.ld lane quadrant = warp mod 4).  Every wait gives up after 2 s.
// ---------------------------------------------------------------------------
constexpr int kTcStages = 2;
constexpr uint32_t kTileA = kLargeBM * 128;  // bytes of one 128-row x 32-float plane
constexpr uint32_t kTileB = kLargeBN * 128;
constexpr uint32_t kStageBytes = 2 * kTileA + 2 * kTileB;  // hi + lo of A and B
constexpr size_t kGemmTcSmem = kTcStages * kStageBytes + 1024 + 128;

__global__ void __launch_bounds__(192, 1)
    gemm_tc_kernel(const LargeArgs a, const __grid_constant__ CUtensorMap smap,
                   const __grid_constant__ CUtensorMap qmap) {
  extern __shared__ __align__(16) unsigned char raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + kTcStages * kStageBytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 8);
  int* ctl = reinterpret_cast<int*>(tslot + 1);  // [0] failed, [1] issued, [2] consumed
  const int task = blockIdx.z;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  const int m0 = blockIdx.y * kLargeBM, n0 = blockIdx.x * kLargeBN;
  if (m0 >= td.NP || n0 >= td.D) return;  // uniform: before any barrier
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t sbase = tc::smem_addr(base);
  const uint32_t full0 = tc::smem_addr(bars), empty0 = tc::smem_addr(bars + 2),
                 done = tc::smem_addr(bars + 4);
  const int nkb = (td.D + 31) >> 5;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      tc::mbar_init(full0 + 8 * s, 1);
      tc::mbar_init(empty0 + 8 * s, 1);
    }
    tc::mbar_init(done, 1);
    ctl[0] = ctl[1] = ctl[2] = 0;
  }
  // two accumulators of kLargeBN columns: hi.hi, and the three small products
  if (warp == 1) tc::tmem_alloc(tslot, 2 * kLargeBN);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;
  const int64_t srow = a.srow[task] + m0, qrow = a.qrow[task] + n0;
  const uint64_t wait_ns = a.wait_ns ? a.wait_ns : tc::kWaitLimitNs;

  if (warp == 0 && lane == 0) {  // producer
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % kTcStages;
      if (kb >= kTcStages && !tc::mbar_wait(empty0 + 8 * s, ((kb / kTcStages) - 1) & 1, wait_ns)) {
        atomicExch(&ctl[0], 1);
        break;
      }
      if (ctl[0]) break;
      const uint32_t st = sbase + s * kStageBytes;
      tc::mbar_expect_tx(full0 + 8 * s, kStageBytes);
      tc::tma_load_3d(st, &smap, kb * 32, (int)srow, 0, full0 + 8 * s);
      tc::tma_load_3d(st + kTileA, &smap, kb * 32, (int)srow, 1, full0 + 8 * s);
      tc::tma_load_3d(st + 2 * kTileA, &qmap, kb * 32, (int)qrow, 0, full0 + 8 * s);
      tc::tma_load_3d(st + 2 * kTileA + kTileB, &qmap, kb * 32, (int)qrow, 1, full0 + 8 * s);
      ctl[1] = kb + 1;
    }
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    const uint32_t idesc = tc::idesc_tf32(kLargeBM, kLargeBN);
    int kb = 0;
    for (; kb < nkb; ++kb) {
      const int s = kb % kTcStages;
      if (!tc::mbar_wait(full0 + 8 * s, (kb / kTcStages) & 1, wait_ns)) {
        atomicExch(&ctl[0], 1);
        break;
      }
      tc::fence_after();
      const uint32_t st = sbase + s * kStageBytes;
      // all four products of the hi/lo pairs.  Each MMA step loses about
      // 2^-24 of its accumulator's magnitude (measured: with the four products
      // in one accumulator |f - f64| reached 1.3e-5 of the scale at K = 1000),
      // so hi.hi accumulates alone and hi.lo + lo.hi + lo.lo, 2^-11 smaller,
      // in the second accumulator; the epilogue adds the two in FP32.
      const uint32_t pa[4] = {0u, 0u, kTileA, kTileA}, pb[4] = {0u, kTileB, 0u, kTileB};
      for (int p = 0; p < 4; ++p)
        for (int ks = 0; ks < 4; ++ks) {
          const uint64_t ad = tc::sdesc_sw128(st + pa[p] + 32u * ks);
          const uint64_t bd = tc::sdesc_sw128(st + 2 * kTileA + pb[p] + 32u * ks);
          const uint32_t acc = p == 0 ? ((kb | ks) ? 1u : 0u) : ((kb | (p - 1) | ks) ? 1u : 0u);
          tc::mma_tf32(tmem + (p ? (uint32_t)kLargeBN : 0u), ad, bd, idesc, acc);
        }
      tc::mma_commit(empty0 + 8 * s);
      ctl[2] = kb + 1;
    }
    if (kb == nkb) tc::mma_commit(done);
  } else if (warp >= 2) {  // epilogue
    const bool ok = tc::mbar_wait(done, 0, wait_ns);
    if (!ok && lane == 0) atomicExch(&ctl[0], 1);
    tc::fence_after();
    const int q = warp & 3;
    const int row = m0 + 32 * q + lane;
    if (ok) {
      float* zr = a.Z + (a.srow[task] + row) * (int64_t)a.Nq + n0;
      for (int c0 = 0; c0 < kLargeBN; c0 += 16) {
        float v[16], w[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
        tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(kLargeBN + c0), w);
#pragma unroll
        for (int g = 0; g < 16; ++g) v[g] = __fadd_rn(v[g], w[g]);
        if (row < td.NP)
#pragma unroll
          for (int g = 0; g < 4; ++g)
            reinterpret_cast<float4*>(zr + c0)[g] = make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2], v[4 * g + 3]);
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (ctl[0]) {
    if (threadIdx.x == 0) {
      atomicCAS(a.err, 0, CHECK_TIMEOUT);
      // let copies still in flight land before the CTA's shared memory goes
      for (int kb = ctl[2]; kb < ctl[1]; ++kb)
        tc::mbar_wait(full0 + 8 * (kb % kTcStages), (kb / kTcStages) & 1);
    }
    __syncthreads();
  }
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, 2 * kLargeBN);
  }
}

// ---------------------------------------------------------------------------
// f and its window for one Z row, by the calling warp (lanes over genes; the
// fused kernel's FP32 forms and scale)
// ---------------------------------------------------------------------------
__device__ void eval_row_lanes(const FnConst& fc, const float* __restrict__ z,
                               const float* __restrict__ x, const float* __restrict__ o,
                               float* fout, float* tout) {
  const int lane = threadIdx.x & 31, D = fc.D;
  const bool griewank_prod = !(fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT);
  float a = 0.f, b = 0.f, c = 1.f, sa = 0.f, ss = 0.f;
  int neg = 0;
  switch (fc.fid) {
    case F_SPHERE:
      for (int j = lane; j < D; j += 32) a = fmaf(z[j], z[j], a);
      sa = a;
      break;
    case F_RASTRIGIN:
      for (int j = lane; j < D; j += 32) {
        const float v = z[j], sp = sinpif(v);
        a += fmaf(20.f * sp, sp, v * v);
      }
      sa = a;
      break;
    case F_ACKLEY:
      for (int j = lane; j < D; j += 32) {
        const float v = z[j], sp = sinpif(v);
        a = fmaf(v, v, a);
        b = fmaf(sp, sp, b);
      }
      break;
    case F_GRIEWANK:
      for (int j = lane; j < D; j += 32) {
        const float v = z[j];
        a = fmaf(v, v, a);
        if (griewank_prod) {
          const float th = __fdiv_rn(v, sqrtf((float)(j + 1)));
          const float ct = cosf(th);
          c *= ct;
          if (ct > 0.f) {
            const float sh = sinf(0.5f * th);
            b += log1pf(-2.f * sh * sh);
          } else {
            neg = 1;
          }
        }
      }
      break;
    case F_ROSENBROCK:
      for (int j = lane; j + 1 < D; j += 32) {
        const float v = z[j], n = z[j + 1];
        const float t1 = fmaf(v, v, -n), t2 = v - 1.f;
        const float t = fmaf(100.f * t1, t1, t2 * t2);
        a += t;
        sa += t + 200.f * fabsf(t1) * fmaf(v, v, fabsf(n)) + 2.f * fabsf(t2) * (fabsf(v) + 1.f);
      }
      break;
    case F_SCHWEFEL:
      for (int j = lane; j < D; j += 32) {
        const float v = z[j], t = v * sinf(sqrtf(fabsf(v)));
        a += t;
        sa += fabsf(t);
      }
      break;
    case F_WEIERSTRASS:
      for (int j = lane; j < D; j += 32) {
        a += weier_gene_f32(z[j]);
        const float d = x[j] - o[j];
        ss = fmaf(d, d, ss);
      }
      break;
    default:
      break;
  }
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_prod(c);
  sa = warp_sum(sa);
  ss = warp_sum(ss);
  neg = __any_sync(0xFFFFFFFFu, neg);
  float f, scale;
  switch (fc.fid) {
    case F_ACKLEY: {
      const float e = 2.71828183f;
      const float eref = (fc.flags & FLAG_REF_ACKLEY_E) ? 2.718282f - e : 0.f;
      const float t1 = -20.f * expm1f(-0.2f * sqrtf(a / (float)D));
      const float t2 = -e * expm1f(-2.f * b / (float)D);
      f = t1 + t2 + eref;
      scale = t1 + t2 + fabsf(eref);
      break;
    }
    case F_GRIEWANK: {
      const float om = !griewank_prod ? 0.f : (neg ? 1.f - c : -expm1f(b));
      f = om + a / 4000.f;
      scale = a / 4000.f + fabsf(om) + ((griewank_prod && neg) ? fabsf(c) + 1.f : 0.f);
      break;
    }
    case F_SCHWEFEL:
      f = 418.9829f * (float)D - a;
      scale = 418.9829f * (float)D + sa;
      break;
    case F_WEIERSTRASS:
      f = a + fc.woff;
      scale = 2.f * (float)D + fabsf(fc.woff);
      break;
    default:
      f = a;
      scale = sa;
      break;
  }
  float t = fc.rel * scale;
  if (fc.fid == F_WEIERSTRASS)
    t = (fc.flags & FLAG_RIGOROUS_WINDOW) ? t + weier_rotation_bound(D, fc.qnorm, sqrtf(ss))
                                          : 5.f * t;
  *fout = f;
  *tout = t;
}

// which = 0: members (fit32/tol32); 1: trials (ftr/ttr); rows < limit
__global__ void __launch_bounds__(256) eval_kernel(const LargeArgs a, int which, int limit) {
  const int task = blockIdx.y;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  const int row = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row >= td.NP || row >= limit) return;  // warp-uniform
  const FnConst fc = fn_const(td, a.recheck_rel);
  const float* z = a.Z + (a.srow[task] + row) * (int64_t)a.Nq;
  const float* x = (which ? a.U : a.pop) + td.pop_off + (size_t)row * td.DP;
  float f, t;
  eval_row_lanes(fc, z, x, a.shift + td.o_off, &f, &t);
  if ((threadIdx.x & 31) == 0) {
    (which ? a.ftr : a.fit32)[td.fit_off + row] = f;
    (which ? a.ttr : a.tol32)[td.fit_off + row] = t;
  }
}

// ---------------------------------------------------------------------------
// ranking, elite export and the migrants' preparation: one CTA (256 threads)
// per task over global-memory rows (the selections themselves run through
// the split pipeline below)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) select_kernel(const LargeArgs a, int mode) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int task = blockIdx.x;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  if (large_select_smem(td.DP) > a.select_smem) {
    if (threadIdx.x == 0) atomicCAS(a.err, 0, CHECK_SMEM_TOO_SMALL);
    return;
  }
  const int NP = td.NP, DP = td.DP;
  Smem s{};
  s.z64 = nullptr;
  int* ip = reinterpret_cast<int*>(smraw);
  s.flag = ip;
  s.list = ip + kMaxPopLarge;
  s.idx = ip + 2 * kMaxPopLarge;  // targets (transfer)
  s.misc = ip + 4 * kMaxPopLarge;
  s.X = a.pop + td.pop_off;
  s.U = a.U + td.pop_off;
  s.fit = a.fit32 + td.fit_off;
  s.tol = a.tol32 + td.fit_off;
  s.ftr = a.ftr + td.fit_off;
  s.ttr = a.ttr + td.fit_off;
  s.fit64 = a.fit64 + td.fit_off;
  s.o = const_cast<float*>(a.shift + td.o_off);
  s.QT = const_cast<float*>(a.qt + td.q_off);
  s.zc = s.zcb = nullptr;
  int* byrank = a.rank + td.fit_off;
  if (mode == SEL_RANK || mode == SEL_EXPORT) {
    rank_members(s, NP, s.idx);
    if (mode == SEL_RANK) {
      for (int i = threadIdx.x; i < NP; i += kThreads) byrank[i] = s.idx[i];
    } else {
      const int k = transfer_k(a.transfer_rate, NP);
      float* el = a.elites_out + td.elite_off;
      for (int it = threadIdx.x; it < k * DP; it += kThreads) {
        const int c = it / DP, j = it - c * DP;
        el[(size_t)c * DP + j] = s.X[(size_t)s.idx[c] * DP + j];
      }
    }
  } else if (mode == SEL_MIGRATE) {
    // ring migration between sub-islands (IslandMigration, SG-EMTF.cu:1138-1218),
    // as the fused kernel's migrate(): rank each sub-island by FP32 fitness,
    // copy the r-th best of sub-island s to trial row s*m + r with its
    // fitness, target the r-th worst of s + 1 (the pipeline decides)
    if (!migration_due(a, task)) return;  // uniform over the CTA
    const int S = a.subislands, NPs = NP / S, m = migration_count(a, NP), k = S * m;
    int* rk = s.idx;  // NP ints: member of each within-sub-island rank
    for (int i = threadIdx.x; i < NP; i += kThreads) {
      const int base = (i / NPs) * NPs;
      const float fi = s.fit[i];
      int r = 0;
      for (int j = base; j < base + NPs; ++j) {
        const float fj = s.fit[j];
        r += (fj < fi || (fj == fi && j < i)) ? 1 : 0;
      }
      rk[base + r] = i;
    }
    __syncthreads();
    for (int it = threadIdx.x; it < k * DP; it += kThreads) {
      const int c = it / DP, j = it - c * DP, sc = c / m;
      s.U[(size_t)c * DP + j] = s.X[(size_t)rk[sc * NPs + (c - sc * m)] * DP + j];
    }
    for (int c = threadIdx.x; c < k; c += kThreads) {
      const int sc = c / m, r = c - sc * m, src = rk[sc * NPs + r];
      const int dst = sc + 1 == S ? 0 : sc + 1;
      byrank[c] = rk[dst * NPs + NPs - 1 - r];
      s.ftr[c] = s.fit[src];
      s.ttr[c] = s.tol[src];
    }
  }
  // SEL_GENERATION and SEL_IMPORT run through the split selection below
  // (emt_large_selection), never here
}

// ---------------------------------------------------------------------------
// selection split for parallelism.  The per-task CTA above would re-check a
// task's near ties with its 8 warps while most SMs idle; at D = 1000 each
// re-check rotates 10^6 compensated products.  Instead:
//   classify (CTA per task): FP32 decisions; near ties listed, identical
//            trials decided, the rows to rotate listed as jobs;
//   rot      (persistent grid): a task's jobs in chunks of 8, 128 outputs
//            per item, every load of Q shared by the chunk's rows (the same
//            per-output arithmetic as precise_rotation, so the same bits);
//   decide   (persistent grid, a warp per near tie): tiers 2/3, exact
//            Weierstrass, from the stored rotations;
//   apply    (CTA per task): accepted rows into the island, counters.
// ---------------------------------------------------------------------------

// rows of the step and the member each one competes with
__device__ __forceinline__ int sel_rows(const LargeArgs& a, int task, int mode, int& k) {
  const TaskDev td = a.tasks[task];
  if (mode == SEL_MIGRATE) {
    k = migration_due(a, task) ? a.subislands * migration_count(a, td.NP) : 0;
    return k;
  }
  if (mode == SEL_IMPORT) {
    k = 0;
    if (transfer_partner(a, task, a.gen[task], k) < 0) return 0;
    return k;
  }
  return td.NP;
}
__device__ __forceinline__ int sel_target(const LargeArgs& a, const TaskDev& td, int mode, int k, int c) {
  return mode == SEL_IMPORT    ? a.rank[td.fit_off + td.NP - k + c]
         : mode == SEL_MIGRATE ? a.rank[td.fit_off + c]
                               : c;
}

// the k-tile of the rows' exact splits staged in shared memory (the item
// shape kRotCols x kRotJobs is in emt_internal.h)
constexpr int kRotTile = 128;
// work-item encodings: rotation items task << 16 | block << 12 | chunk, jobs
// row | member << 16, tie jobs trial | (member + 1) << 16, decisions
// task << 16 | tie (tasks < 2^15, checked on the host).  Rotation items per
// task: at most rot_items_max(D, NP), which the host allocates per task.
static_assert((kMaxDimLarge + 2 * kRotCols - 1) / (2 * kRotCols) <= 16, "column block in 4 bits");
static_assert((2 * kMaxPopLarge + kRotJobs - 1) / kRotJobs < 4096, "job chunk in 12 bits");
static_assert(2 * kMaxPopLarge + 1 < 0xFFFF, "job and tie indices in 16 bits");
static_assert(kRotCols >= kRotJobs && kRotCols % 32 == 0, "row pointers set by the first threads");

__global__ void __launch_bounds__(256) classify_kernel(const LargeArgs a, int mode) {
  const int task = blockIdx.x;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  int k = 0;
  const int nrows = sel_rows(a, task, mode, k);
  const bool strict = mode == SEL_IMPORT || mode == SEL_MIGRATE;  // candidates must be better
  const bool recheck = !(a.flags & FLAG_NO_RECHECK);
  const int D = td.D, DP = td.DP;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ int nt, nj;
  if (threadIdx.x == 0) nt = nj = 0;
  __syncthreads();
  for (int c = threadIdx.x; c < nrows; c += blockDim.x) {
    const int m = sel_target(a, td, mode, k, c);
    const float ft = a.ftr[td.fit_off + c], fp = a.fit32[td.fit_off + m];
    const bool d32 = strict ? (ft < fp) : (ft <= fp);
    int f = d32 ? 1 : 0;
    if (recheck && fabsf(ft - fp) <= a.ttr[td.fit_off + c] + a.tol32[td.fit_off + m]) {
      f = 2;
      a.ties[td.fit_off + atomicAdd(&nt, 1)] = c;
    }
    a.flag[td.fit_off + c] = f;
  }
  __syncthreads();
  // a warp per near tie: an identical trial is decided here (the same vector
  // has the same fitness: accepted unless the selection is strict); any other
  // gets a rotation job, and one for its member when that member's
  // FP64-class value is not cached, and a decision item
  const int ties = nt;
  for (int i = warp; i < ties; i += blockDim.x >> 5) {
    const int c = a.ties[td.fit_off + i], m = sel_target(a, td, mode, k, c);
    const float* u = a.U + td.pop_off + (size_t)c * DP;
    const float* x = a.pop + td.pop_off + (size_t)m * DP;
    bool diff = false;
    for (int j = lane; j < D; j += 32) diff |= __float_as_uint(u[j]) != __float_as_uint(x[j]);
    diff = __any_sync(0xFFFFFFFFu, diff);
    if (lane != 0) continue;
    if (!diff) {
      const float f32t = a.ftr[td.fit_off + c], f32p = a.fit32[td.fit_off + m];
      const bool d32 = strict ? (f32t < f32p) : (f32t <= f32p), d64 = !strict;
      a.flag[td.fit_off + c] = d64 ? 3 : 0;  // member m keeps its cached FP64 value
      a.tjob[td.fit_off + i] = -1;
      if (a.stats) {
        atomicAdd(a.stats + 0, 1ull);
        if (d64 != d32) atomicAdd(a.stats + 1, 1ull);
        atomicAdd(a.stats + 6, 1ull);
      }
      continue;
    }
    const bool member = isnan(a.fit64[td.fit_off + m]);
    const int j = atomicAdd(&nj, member ? 2 : 1);
    a.jobs[2 * td.fit_off + j] = c;
    if (member) a.jobs[2 * td.fit_off + j + 1] = (1 << 16) | m;
    a.tjob[td.fit_off + i] = j | ((member ? j + 2 : 0) << 16);
    // Weierstrass decisions are handed out first: their rare float-float
    // escalations are the longest items, and started early they end under
    // the other items instead of after them (config 4: 1.789 -> 1.760 s;
    // handed out last, 1.786 s)
    if (td.fid == F_WEIERSTRASS)
      a.work[atomicAdd(a.nwork + 0, 1)] = (task << 16) | i;
    else
      a.work[a.work_cap - 1 - atomicAdd(a.nwork + 4, 1)] = (task << 16) | i;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a.ntie[task] = ties;
    a.njob[task] = nj;
    const int blocks = (D + 2 * kRotCols - 1) / (2 * kRotCols), chunks = (nj + kRotJobs - 1) / kRotJobs;
    if (chunks) {
      const int w0 = atomicAdd(a.nwork + 1, blocks * chunks);
      for (int b = 0; b < blocks; ++b)
        for (int q = 0; q < chunks; ++q) a.rwork[w0 + b * chunks + q] = (task << 16) | (b << 12) | q;
    }
  }
}

// Rotation work item: outputs [2 kRotCols b, 2 kRotCols (b + 1)) of up to
// kRotJobs rows of one task (small items keep the grid busy when few islands
// have near ties).  A persistent grid takes items from the queue; each thread
// owns outputs n and n + kRotCols and streams their columns of Q once for all
// the item's rows, the exact splits x - o of the rows staged in shared memory
// a k-tile at a time (each staged pair serves both outputs: 1.5% faster at
// D = 1000 than one output per thread).  Each output keeps dot2_pair's order
// over k, so the values equal precise_rotation's.
// Compensated product q * (h + l) into the running sums S, C of one output.
__device__ __forceinline__ void comp_step(float q, float2 hl, float& S, float& C) {
  const float pp = __fmul_rn(q, hl.x);
  const float e = __fmaf_rn(q, hl.x, -pp);
  float t, te;
  two_sum(S, pp, t, te);
  S = t;
  C = __fmaf_rn(q, hl.y, __fadd_rn(C, __fadd_rn(te, e)));
}
// The compensated products of J rows (J = the item's job count, fixed at
// compile time so a partial chunk costs in proportion to its rows) for the
// k-tile in pr, into S[0..J), C[0..J) (output n, column qa of Q) and
// S[J..2J), C[J..2J) (output n + kRotCols, column qb).
template <int J>
__device__ __forceinline__ void rot_tile(const float2 (*pr)[kRotJobs], const float* qa,
                                         const float* qb, int k0, int kt, int DP, float* S,
                                         float* C) {
  constexpr int kAhead = 8;  // Q loads issued ahead of the dependent updates
  int kk = 0;
  for (; kk + kAhead <= kt; kk += kAhead) {
    float va[kAhead], vb[kAhead];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      va[u] = __ldg(qa + (size_t)(k0 + kk + u) * DP);
      vb[u] = __ldg(qb + (size_t)(k0 + kk + u) * DP);
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const float2 hl = pr[kk + u][j];
        comp_step(va[u], hl, S[j], C[j]);
        comp_step(vb[u], hl, S[J + j], C[J + j]);
      }
    }
  }
  for (; kk < kt; ++kk) {
    const float a = __ldg(qa + (size_t)(k0 + kk) * DP), b = __ldg(qb + (size_t)(k0 + kk) * DP);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const float2 hl = pr[kk][j];
      comp_step(a, hl, S[j], C[j]);
      comp_step(b, hl, S[J + j], C[J + j]);
    }
  }
}

// One rotation work item with J jobs: stage each k-tile of the rows' exact
// splits, accumulate, write the FP64-class outputs.
template <int J>
__device__ __forceinline__ void rot_item(const LargeArgs& a, const TaskDev& td, int blk, int j0,
                                         float2 (*pr)[kRotJobs], const float* const* jrow) {
  const int D = td.D, DP = td.DP;
  const float* o = a.shift + td.o_off;
  const int n = blk * 2 * kRotCols + threadIdx.x, m = n + kRotCols;
  const bool live = n < D, live2 = m < D;
  const float* qa = a.qt + td.q_off + (live ? n : 0);
  const float* qb = live2 ? a.qt + td.q_off + m : qa;
  float S[2 * J], C[2 * J];
#pragma unroll
  for (int j = 0; j < 2 * J; ++j) S[j] = C[j] = 0.f;
  for (int k0 = 0; k0 < D; k0 += kRotTile) {
    const int kt = min(kRotTile, D - k0);
    __syncthreads();
    for (int it = threadIdx.x; it < J * kt; it += blockDim.x) {
      const int j = it / kt, kk = it - j * kt;
      float sh, sl;
      two_sum(jrow[j][k0 + kk], -o[k0 + kk], sh, sl);
      pr[kk][j] = make_float2(sh, sl);
    }
    __syncthreads();
    if (live) rot_tile<J>(pr, qa, qb, k0, kt, DP, S, C);
  }
  double* z = a.zr + 2 * td.pop_off + (size_t)j0 * DP;
  if (live) {
#pragma unroll
    for (int j = 0; j < J; ++j) z[(size_t)j * DP + n] = (double)S[j] + (double)C[j];
  }
  if (live2) {
#pragma unroll
    for (int j = 0; j < J; ++j) z[(size_t)j * DP + m] = (double)S[J + j] + (double)C[J + j];
  }
}

// Next work item of a persistent grid: one atomic on a device-wide counter
// per item, broadcast to the CTA through shared memory, so CTAs that draw
// cheap items take more of them.
__device__ __forceinline__ int next_item(int* counter, int* slot) {
  __syncthreads();  // every thread has read the previous item's index
  if (threadIdx.x == 0) *slot = atomicAdd(counter, 1);
  __syncthreads();
  return *slot;
}

__global__ void __launch_bounds__(kRotCols) rot_kernel(const LargeArgs a) {
  static_assert(kRotJobs == 8, "the job-count dispatch below covers 1..8");
  __shared__ __align__(16) float2 pr[kRotTile][kRotJobs];
  __shared__ const float* jrow[kRotJobs];
  __shared__ int slot;
  const int items = a.nwork[1];
  for (int w = next_item(a.nwork + 2, &slot); w < items; w = next_item(a.nwork + 2, &slot)) {
    const int code = a.rwork[w];
    const int task = code >> 16, blk = (code >> 12) & 15, chunk = code & 0xFFF;
    const TaskDev td = a.tasks[task];
    const int DP = td.DP;
    const int j0 = chunk * kRotJobs, nj = min(kRotJobs, a.njob[task] - j0);
    if (threadIdx.x < kRotJobs) {
      const int t = threadIdx.x;
      const float* r = nullptr;
      if (t < nj) {
        const int jc = a.jobs[2 * td.fit_off + j0 + t];
        r = ((jc >> 16) ? a.pop : a.U) + td.pop_off + (size_t)(jc & 0xFFFF) * DP;
      }
      jrow[t] = r;
    }
    switch (nj) {  // uniform over the CTA
      case 1: rot_item<1>(a, td, blk, j0, pr, jrow); break;
      case 2: rot_item<2>(a, td, blk, j0, pr, jrow); break;
      case 3: rot_item<3>(a, td, blk, j0, pr, jrow); break;
      case 4: rot_item<4>(a, td, blk, j0, pr, jrow); break;
      case 5: rot_item<5>(a, td, blk, j0, pr, jrow); break;
      case 6: rot_item<6>(a, td, blk, j0, pr, jrow); break;
      case 7: rot_item<7>(a, td, blk, j0, pr, jrow); break;
      default: rot_item<8>(a, td, blk, j0, pr, jrow); break;
    }
    __syncthreads();  // jrow of the next item
  }
}

// Writes the decision of near tie i (trial row c against member m).
__device__ __forceinline__ void decide_write(const LargeArgs& a, const TaskDev& td, bool strict,
                                             int c, int m, bool d64, double ft, double fpv) {
  const float f32t = a.ftr[td.fit_off + c], f32p = a.fit32[td.fit_off + m];
  const bool d32 = strict ? (f32t < f32p) : (f32t <= f32p);
  a.flag[td.fit_off + c] = d64 ? 3 : 0;
  // FP64 value of whichever vector member m holds afterwards
  a.fit64[td.fit_off + m] = d64 ? ft : fpv;
  if (a.stats) {
    atomicAdd(a.stats + 0, 1ull);
    if (d64 != d32) atomicAdd(a.stats + 1, 1ull);
  }
}

// Decisions of the near ties: a persistent grid, a CTA per tie.  Tier 2,
// then tier 3 (exact Weierstrass terms for that function), as
// select_and_replace decides, from the stored rotations of the trial and
// (when not cached) the member, with the genes over all 256 threads: the
// FP64 terms of one tie on one warp take ~0.2 ms at D = 1000 on this GPU's
// FP64 pipe, and a few such ties would set the launch length.
__global__ void __launch_bounds__(256) decide_kernel(const LargeArgs a, int mode) {
  __shared__ double scratch[8];
  __shared__ double zmem[kMaxDimLarge];  // a member's rotation, when a tie needs it here
  const CtaTeam tm{scratch};
  const bool strict = mode == SEL_IMPORT || mode == SEL_MIGRATE;  // candidates must be better
  __shared__ int slot;
  const int front = a.nwork[0], items = front + a.nwork[4];
  for (int w = next_item(a.nwork + 3, &slot); w < items; w = next_item(a.nwork + 3, &slot)) {
    const int code = w < front ? a.work[w] : a.work[a.work_cap - 1 - (w - front)];
    const int task = code >> 16, i = code & 0xFFFF;
    const TaskDev td = a.tasks[task];
    int k = 0;
    sel_rows(a, task, mode, k);
    const int c = a.ties[td.fit_off + i], m = sel_target(a, td, mode, k, c);
    const int tj = a.tjob[td.fit_off + i];
    const double* zb = a.zr + 2 * td.pop_off;
    const double* zt = zb + (size_t)(tj & 0xFFFF) * td.DP;
    const double* zp = (tj >> 16) ? zb + (size_t)((tj >> 16) - 1) * td.DP : nullptr;
    const FnConst fc = fn_const(td, a.recheck_rel);
    const double fp = a.fit64[td.fit_off + m];
    double ft = __longlong_as_double(0x7FF8000000000000ll), fpv = fp;
    bool d64 = false, decided = false;
    if (fc.fid != F_WEIERSTRASS && fc.fid != F_SPHERE && fc.fid != F_ROSENBROCK) {
      double et, ep = 0.0;
      const double t2 = eval_tier2_t(fc, zt, &et, tm);
      double p2 = fp;
      if (zp) p2 = eval_tier2_t(fc, zp, &ep, tm);
      if (fabs(t2 - p2) > et + ep) {
        d64 = strict ? (t2 < p2) : (t2 <= p2);
        decided = true;
      }
    }
    // Weierstrass: whether fit64[m] is a float-float value afterwards (1) or
    // not (0); -1 for the other functions
    int wprec = -1;
    if (!decided) {
      const bool weier = fc.fid == F_WEIERSTRASS;
      ft = weier ? eval_weier_precise_pair_t(fc, zt, tm) : eval_tier3_t(fc, zt, tm);
      if (zp) fpv = weier ? eval_weier_precise_pair_t(fc, zp, tm) : eval_tier3_t(fc, zp, tm);
      if (weier) {
        // the member's cached value is already float-float (exact to ~1e-12)
        const bool pprec = !zp && !isnan(fp) && a.wprec[td.fit_off + m] == 0.f;
        const double bound = weier_precise_bound(fc.D);
        wprec = 0;
        if (fabs(ft - fpv) <= (pprec ? bound : 2.0 * bound)) {
          // closer than the FP32 terms' error: every term in float-float, the
          // member's too unless already so, its rotation computed here when
          // only its value was cached
          if (!pprec) {
            double* zm = zmem;
            if (zp) {
              zm = const_cast<double*>(zp);
            } else {
              precise_rotation_team(a.pop + td.pop_off + (size_t)m * td.DP, a.shift + td.o_off,
                                    a.qt + td.q_off, td.DP, td.D, zmem, tm);
            }
            fpv = eval_weier_ff_pair_t(fc, zm, tm);
          }
          ft = eval_weier_ff_pair_t(fc, zt, tm);
          wprec = 1;
          if (threadIdx.x == 0 && a.stats) atomicAdd(a.stats + kStatWeierFp64, 1ull);
        }
        d64 = strict ? (ft < fpv) : (ft <= fpv);
        if (!wprec && !d64 && pprec) wprec = 1;  // the member keeps its float-float value
      } else {
        d64 = strict ? (ft < fpv) : (ft <= fpv);
      }
    }
    if (threadIdx.x == 0) {
      decide_write(a, td, strict, c, m, d64, ft, fpv);
      if (wprec >= 0) a.wprec[td.fit_off + m] = wprec ? 0.f : __int_as_float(0x7FC00000);
    }
  }
}

// A task's accepted rows are copied by kApplySlices CTAs (its float4s
// interleaved over them); the first also moves the fitness values and counts.
constexpr int kApplySlices = 4;

__global__ void __launch_bounds__(256) apply_kernel(const LargeArgs a, int mode) {
  const int task = blockIdx.x;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  int k = 0;
  const int nrows = sel_rows(a, task, mode, k);
  const int DP = td.DP, nq = DP >> 2;
  for (int it = blockIdx.y * blockDim.x + threadIdx.x; it < nrows * nq;
       it += kApplySlices * blockDim.x) {
    const int c = it / nq, q = it - c * nq;
    if (a.flag[td.fit_off + c] & 1) {
      const int m = sel_target(a, td, mode, k, c);
      reinterpret_cast<float4*>(a.pop + td.pop_off + (size_t)m * DP)[q] =
          reinterpret_cast<const float4*>(a.U + td.pop_off + (size_t)c * DP)[q];
    }
  }
  if (blockIdx.y != 0) return;
  __shared__ int acc;
  if (threadIdx.x == 0) acc = 0;
  __syncthreads();
  for (int c = threadIdx.x; c < nrows; c += blockDim.x) {
    const int f = a.flag[td.fit_off + c];
    if (f & 1) {
      const int m = sel_target(a, td, mode, k, c);
      a.fit32[td.fit_off + m] = a.ftr[td.fit_off + c];
      a.tol32[td.fit_off + m] = a.ttr[td.fit_off + c];
      if (f == 1) a.fit64[td.fit_off + m] = __longlong_as_double(0x7FF8000000000000ll);
      atomicAdd(&acc, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (mode == SEL_GENERATION) {
      a.gen[task] += 1u;
      if (a.stats) atomicAdd(a.stats + 3, (unsigned long long)td.NP);
    } else if (mode == SEL_MIGRATE) {  // copies carry their fitness: no evaluations
      if (acc && a.stats) atomicAdd(a.stats + 7, (unsigned long long)acc);
    } else if (a.stats) {
      if (acc) atomicAdd(a.stats + 2, (unsigned long long)acc);
      atomicAdd(a.stats + 3, (unsigned long long)k);
    }
  }
}

// best member per task and its FP64-class fitness; zbuf in dynamic smem
__global__ void __launch_bounds__(32) best_kernel(const BestArgs a) {
  extern __shared__ double zb[];
  const int task = blockIdx.x;
  if (task >= a.n_tasks) return;
  const TaskDev td = a.tasks[task];
  if (!large_ok(td)) return;
  const int lane = threadIdx.x;
  float bf = __int_as_float(0x7F800000);
  int bi = 0x7FFFFFFF;
  for (int i = lane; i < td.NP; i += 32) {
    const float f = a.fit32[td.fit_off + i];
    if (f < bf || (f == bf && i < bi)) {
      bf = f;
      bi = i;
    }
  }
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    const float of = __shfl_xor_sync(0xFFFFFFFFu, bf, m);
    const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, m);
    if (of < bf || (of == bf && oi < bi)) {
      bf = of;
      bi = oi;
    }
  }
  if (bi < 0 || bi >= td.NP) bi = 0;
  double f64 = a.fit64[td.fit_off + bi];
  if (isnan(f64))
    f64 = eval_row_f64(fn_const(td, 0.f), a.pop + td.pop_off + (size_t)bi * td.DP,
                       a.shift + td.o_off, a.qt + td.q_off, td.DP, zb);
  if (lane == 0) {
    a.best_idx[task] = bi;
    a.best_f32[task] = bf;
    a.best_f64[task] = f64;
    if (a.best_err) a.best_err[task] = best_rel_err(td, bf, f64, a.tol32[td.fit_off + bi], a.rel);
  }
}

}  // namespace large
}  // namespace emt

// ---- host launchers ----
int emt_large_init(const emt::LargeArgs& a, void* stream) {
  emt::large::init_kernel<<<dim3(16, a.n_tasks), 256, 0, (cudaStream_t)stream>>>(a);
  return (int)cudaGetLastError();
}

int emt_large_build(const emt::LargeArgs& a, int mode, void* stream) {
  const int gx = (a.max_np + emt::large::kBuildRows - 1) / emt::large::kBuildRows;
  emt::large::build_kernel<<<dim3(gx, a.n_tasks), 256, 0, (cudaStream_t)stream>>>(a, mode);
  return (int)cudaGetLastError();
}

int emt_large_gemm(const emt::LargeArgs& a, const void* smap, const void* qmap, void* stream) {
  const int gy = (a.max_np + emt::kLargeBM - 1) / emt::kLargeBM;
  if (a.tc) {
    static_assert(emt::large::kGemmTcSmem <= 227 * 1024, "tile pipeline");
    cudaError_t e = cudaFuncSetAttribute(emt::large::gemm_tc_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)emt::large::kGemmTcSmem);
    if (e != cudaSuccess) return (int)e;
    emt::large::gemm_tc_kernel<<<dim3(a.Nq / emt::kLargeBN, gy, a.n_tasks), 192,
                                 emt::large::kGemmTcSmem, (cudaStream_t)stream>>>(
        a, *reinterpret_cast<const CUtensorMap*>(smap), *reinterpret_cast<const CUtensorMap*>(qmap));
  } else {
    emt::large::gemm_f32_kernel<<<dim3((a.Nq + 127) / 128, gy, a.n_tasks), 256, 0,
                                  (cudaStream_t)stream>>>(a);
  }
  return (int)cudaGetLastError();
}

int emt_large_eval(const emt::LargeArgs& a, int which, int rows, void* stream) {
  const int gx = (a.max_np + 7) / 8;
  emt::large::eval_kernel<<<dim3(gx, a.n_tasks), 256, 0, (cudaStream_t)stream>>>(a, which, rows);
  return (int)cudaGetLastError();
}

int emt_large_select(const emt::LargeArgs& a, int mode, void* stream) {
  cudaError_t e = cudaFuncSetAttribute(emt::large::select_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)a.select_smem);
  if (e != cudaSuccess) return (int)e;
  emt::large::select_kernel<<<a.n_tasks, emt::kThreads, a.select_smem, (cudaStream_t)stream>>>(a, mode);
  return (int)cudaGetLastError();
}

int emt_large_selection(const emt::LargeArgs& a, int mode, void* stream) {
  cudaError_t e = cudaMemsetAsync(a.nwork, 0, 5 * sizeof(int32_t), (cudaStream_t)stream);
  if (e != cudaSuccess) return (int)e;
  emt::large::classify_kernel<<<a.n_tasks, 256, 0, (cudaStream_t)stream>>>(a, mode);
  emt::large::rot_kernel<<<a.rot_grid, emt::large::kRotCols, 0, (cudaStream_t)stream>>>(a);
  emt::large::decide_kernel<<<a.decide_grid, 256, 0, (cudaStream_t)stream>>>(a, mode);
  emt::large::apply_kernel<<<dim3(a.n_tasks, emt::large::kApplySlices), 256, 0, (cudaStream_t)stream>>>(
      a, mode);
  return (int)cudaGetLastError();
}

void emt_large_recheck_grids(int sms, int32_t* rot, int32_t* decide) {
  int r = 0, d = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, emt::large::rot_kernel, emt::large::kRotCols, 0) != cudaSuccess)
    r = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, emt::large::decide_kernel, 256, 0) != cudaSuccess)
    d = 1;
  if (sms < 1) sms = 1;
  *rot = sms * (r > 1 ? r : 1);
  *decide = sms * (d > 1 ? d : 1);
}

int emt_large_best(const emt::BestArgs& a, int maxD, void* stream) {
  if (a.n_tasks <= 0) return 0;
  emt::large::best_kernel<<<a.n_tasks, 32, sizeof(double) * (size_t)(maxD + 4), (cudaStream_t)stream>>>(a);
  return (int)cudaGetLastError();
}
