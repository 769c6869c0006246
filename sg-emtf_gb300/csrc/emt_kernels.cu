// emt_kernels.cu -- the fused generation kernel (FP32 CUDA-core and tcgen05
// tensor-core rotation forms) and the standalone evaluation kernel.
//
// One CTA owns one task for a whole epoch (all generations between two elite
// transfers).  Its island lives in shared memory across generations, as the
// reference's GeneticOpera keeps its sub-population in shared memory
// (proposed model/SG-EMTF.cu:1289-1426), but without the reference's
// cross-block shuffle and its unbounded grid spin (:1384-1392): an island is
// owned by exactly one CTA, so no CTA ever waits on another.
//
// Per generation (all in shared memory):
//   1. trial vectors: DE/rand/1/bin, DE/current/1/bin or SBX + polynomial
//      mutation, from the counter-based Philox stream (bit-exact with the
//      host replay);
//   2. rotation Z = (U - o) Q^T, in one of three forms:
//      FP32:   4x4 register tiles on CUDA cores, float4 operand loads;
//      BF16X3: tcgen05 MMA, kind::f16, both operands split exactly into
//              three BF16 parts, eight products of parts;
//      TF32X3: tcgen05 MMA, kind::tf32, hi/lo TF32 parts, four products;
//      (FP32 accumulation in tensor memory, the leading product in its own
//      accumulator; the trial builder writes the split A operand into
//      128B-swizzled shared-memory tiles, Q's parts arrive by TMA once per
//      island);
//   3. function epilogue: f and its rounding-error scale per trial;
//   4. selection (ties go to the trial, SG-EMTF_DE.cu:679-706): a trial whose
//      FP32 fitness lies within the rounding window of its parent's is
//      re-decided in FP64 so that selections do not depend on FP32 rounding.
#include <cuda.h>
#include <cuda_runtime.h>

#include "emt_functions.cuh"
#include "emt_recheck.cuh"
#include "emt_tc.cuh"

namespace emt {

// Phase clocks (build with -DEMT_PHASE_CLOCKS, the measurement build): thread
// 0 of each CTA charges the SM cycles between CTA-wide barriers to the phase
// the CTA was in (the Phase enum), and adds its totals to the stats array at
// the end of the island.  mark() adds a barrier at boundaries that lack one.
// The product build compiles every mark away.
#ifdef EMT_PHASE_CLOCKS
struct PhaseClock {
  long long t0, acc[kPhases];
  int cur;
  __device__ __forceinline__ void begin() {
    if (threadIdx.x == 0) {
      t0 = clock64();
      cur = PH_OTHER;
      for (int k = 0; k < kPhases; ++k) acc[k] = 0;
    }
  }
  __device__ __forceinline__ void mark(int next) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const long long t = clock64();
      acc[cur] += t - t0;
      t0 = t;
      cur = next;
    }
  }
  // thread 0 alone (no barrier): the rest of the current phase is `next`
  __device__ __forceinline__ void lap(int next) {
    if (threadIdx.x == 0) {
      const long long t = clock64();
      acc[cur] += t - t0;
      t0 = t;
      cur = next;
    }
  }
  __device__ __forceinline__ void flush(unsigned long long* stats) {
    mark(PH_OTHER);
    if (threadIdx.x == 0 && stats)
      for (int k = 0; k < kPhases; ++k) atomicAdd(stats + 8 + k, (unsigned long long)acc[k]);
  }
};
#define EMT_PHASE(s, k) \
  do {                      \
    if ((s).ph) (s).ph->mark(k); \
  } while (0)
#define EMT_PHASE_LAP(s, k) \
  do {                          \
    if ((s).ph) (s).ph->lap(k); \
  } while (0)
#else
struct PhaseClock {};
#define EMT_PHASE(s, k) ((void)0)
#define EMT_PHASE_LAP(s, k) ((void)0)
#endif

struct Smem {
  double *fit64, *z64;
  float *zc, *zcb;  // this task's anchor cache (global memory)
  float *X, *U, *ST, *Z, *QT, *o, *fit, *tol, *ftr, *ttr;
  int *idx, *flag, *list, *misc;
  // tensor-core form
  unsigned char *A, *B;
  uint32_t a_saddr, b_saddr, mma_bar, tma_bar, tmem;
  // two accumulators of 128 TMEM columns: accumulator k at column 128 k
  int nmma;           // MMAs per rotation
  int bplanes;        // B tiles per K block
  bool paired;        // Q in 64-row tiles, N = 128 MMAs over two of them
  int MA, nkb, Np, N, ksteps;
  int planes;     // split parts per operand: 2 (TF32 hi/lo) or 3 (BF16)
  bool bf16;      // exact 3 x BF16 split, kind::f16 MMAs
  uint32_t idesc;
  // the island's MMAs in issue order (mma_descriptors): descriptor low
  // words, accumulator column and accumulate flag in shared memory; the
  // descriptors' high words are the same for every MMA
  const uint4* mdesc;
  uint32_t ad_hi, bd_hi;
  int* dead;         // CTA-wide: a bounded wait gave up (the MMAs are skipped)
  uint64_t wait_ns;  // limit of each bounded wait
  bool lose_completion;  // test switch: issue no MMA and no commit
  PhaseClock* ph;        // thread 0's phase clocks (measurement build only)
};

// The tensor-core state of one CTA, set up once per CTA: TMEM is allocated
// once (the allocation permit is relinquished right after, so a CTA that
// works on several islands, as the persistent queue kernel does, must not
// allocate again), the mbarriers are initialised once and their phases run
// on across islands.  Every thread keeps the same copy of the phases.
struct TcCta {
  TcHeader* hdr;
  uint32_t tmem, ncols, mma_bar, tma_bar;
  uint32_t mphase, tphase;  // parity each barrier completes next
};

__device__ __forceinline__ Smem carve_tc(unsigned char* base, const TcLayout& L) {
  Smem s;
  s.A = base + L.A;
  s.B = base + L.B;
  s.fit64 = (double*)(base + L.fit64);
  s.z64 = (double*)(base + L.z64);
  s.X = (float*)(base + L.X);
  s.U = (float*)(base + L.U);
  s.ST = nullptr;
  s.Z = (float*)(base + L.A);  // rotated rows alias the A operand after the MMAs
  s.QT = nullptr;
  s.zc = s.zcb = nullptr;
  s.ph = nullptr;
  s.o = (float*)(base + L.o);
  s.fit = (float*)(base + L.fit);
  s.tol = (float*)(base + L.tol);
  s.ftr = (float*)(base + L.ftr);
  s.ttr = (float*)(base + L.ttr);
  s.idx = (int*)(base + L.idx);
  s.flag = (int*)(base + L.flag);
  s.list = (int*)(base + L.list);
  s.misc = (int*)(base + L.misc);
  s.mdesc = (const uint4*)(base + L.mdesc);
  s.a_saddr = tc::smem_addr(s.A);
  s.b_saddr = tc::smem_addr(s.B);
  s.MA = L.MA;
  s.planes = L.planes;
  s.bf16 = L.planes == 3;
  s.nkb = L.nkb;
  s.Np = L.Np;
  s.bplanes = L.bplanes;
  s.paired = L.Np == 64;
  return s;
}

__device__ __forceinline__ Smem carve(unsigned char* base, const Layout& L) {
  Smem s;
  s.fit64 = (double*)(base + L.fit64);
  s.z64 = (double*)(base + L.z64);
  s.X = (float*)(base + L.X);
  s.U = (float*)(base + L.U);
  s.ST = (float*)(base + L.ST);
  s.Z = (float*)(base + L.Z);
  s.QT = (float*)(base + L.QT);
  s.zc = s.zcb = nullptr;
  s.ph = nullptr;
  s.o = (float*)(base + L.o);
  s.fit = (float*)(base + L.fit);
  s.tol = (float*)(base + L.tol);
  s.ftr = (float*)(base + L.ftr);
  s.ttr = (float*)(base + L.ttr);
  s.idx = (int*)(base + L.idx);
  s.flag = (int*)(base + L.flag);
  s.list = (int*)(base + L.list);
  s.misc = (int*)(base + L.misc);
  return s;
}

__device__ __forceinline__ void report(int32_t* err, int32_t code) {
  if (err) atomicCAS(err, 0, code);
}

__device__ __forceinline__ bool descriptor_ok(const TaskDev& t) {
  return t.D >= 1 && t.D <= kMaxDim && t.NP >= 4 && t.NP <= kMaxPop && t.DP == round4(t.D) &&
         t.fid >= 0 && t.fid <= F_WEIERSTRASS && t.lo < t.hi;
}

// Z[0..nrows) = ST^T Q^T over k < D; ST is [DP][NPP] (column i = row i of
// U - o), QT is [D][DP] with zero padding beyond D.
__device__ void rotate_f32(const Smem& s, int D, int DP, int NPP, int nrows) {
  const int ncg = DP >> 2;
  const int nrg = (nrows + 3) >> 2;
  const int ntile = nrg * ncg;
  for (int tt = threadIdx.x; tt < ntile; tt += kThreads) {
    const int rg = tt / ncg, cg = tt - rg * ncg;
    const float* a = s.ST + 4 * rg;
    const float* b = s.QT + 4 * cg;
    float c[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q) c[r][q] = 0.f;
#pragma unroll 2
    for (int k = 0; k < D; ++k) {
      const float4 av = *reinterpret_cast<const float4*>(a + k * NPP);
      const float4 bv = *reinterpret_cast<const float4*>(b + k * DP);
      const float ar[4] = {av.x, av.y, av.z, av.w};
      const float br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) c[r][q] = fmaf(ar[r], br[q], c[r][q]);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int row = 4 * rg + r;
      if (row < nrows)
        *reinterpret_cast<float4*>(s.Z + row * DP + 4 * cg) =
            make_float4(c[r][0], c[r][1], c[r][2], c[r][3]);
    }
  }
}

// Stores the rotation input s = x_j - o_j of row i: FP32 form into ST[j][i];
// tensor-core form as its split parts in the swizzled A tiles:
//   TF32: hi = round-to-nearest TF32 of s, lo = round-to-nearest TF32 of
//         s - hi, so s = hi + lo + r with |r| <= 2^-22 |s| and r unbiased (a
//         lo left for the tensor core to truncate would carry a one-signed
//         error that grows linearly over K);
//   BF16: three round-to-nearest BF16 parts with s = p0 + p1 + p2 exactly.
template <bool TC>
__device__ __forceinline__ void stage(const Smem& s, int i, int j, float v, int NPP) {
  if constexpr (TC) {
    if (s.bf16) {
      uint32_t p0, p1, p2;
      tc::split3_bf16x2(v, 0.f, p0, p1, p2);
      const uint32_t off = tc::sw128_offset_b16(i, j & 63);
      unsigned char* t = s.A + (size_t)((j >> 6) * 3) * s.MA * 128 + off;
      const size_t pl = (size_t)s.MA * 128;
      *reinterpret_cast<uint16_t*>(t) = (uint16_t)p0;
      *reinterpret_cast<uint16_t*>(t + pl) = (uint16_t)p1;
      *reinterpret_cast<uint16_t*>(t + 2 * pl) = (uint16_t)p2;
    } else {
      const float hi = tc::tf32_round(v);
      const float lo = tc::tf32_round(v - hi);
      const uint32_t off = tc::sw128_offset(i, j & 31);
      unsigned char* t = s.A + (size_t)((j >> 5) * 2) * s.MA * 128;
      *reinterpret_cast<float*>(t + off) = hi;
      *reinterpret_cast<float*>(t + (size_t)s.MA * 128 + off) = lo;
    }
  } else {
    s.ST[j * NPP + i] = v;
  }
}

// Four consecutive inputs s_{4b..4b+3} of row i (zeros beyond D).  TF32:
// they fill one 16-byte chunk of each part's swizzled tile, so a
// quarter-warp on 8 consecutive rows writes 8 distinct chunks (no bank
// conflicts).  BF16: half a chunk of each part; item_ib below hands a
// half-warp 8 rows x 2 neighbouring blocks, which covers the 32 banks once.
template <bool TC>
__device__ __forceinline__ void stage4(const Smem& s, int i, int b, float4 v, int NPP) {
  if constexpr (TC) {
    if (s.bf16) {
      uint2 p0, p1, p2;
      tc::split3_bf16x2(v.x, v.y, p0.x, p1.x, p2.x);
      tc::split3_bf16x2(v.z, v.w, p0.y, p1.y, p2.y);
      const uint32_t off = (uint32_t)((i >> 3) * 1024 + (i & 7) * 128 +
                                      ((((b >> 1) & 7) ^ (i & 7)) << 4) + ((b & 1) << 3));
      unsigned char* t = s.A + (size_t)((b >> 4) * 3) * s.MA * 128 + off;
      const size_t pl = (size_t)s.MA * 128;
      *reinterpret_cast<uint2*>(t) = p0;
      *reinterpret_cast<uint2*>(t + pl) = p1;
      *reinterpret_cast<uint2*>(t + 2 * pl) = p2;
    } else {
      float4 hi, lo;
      hi.x = tc::tf32_round(v.x); lo.x = tc::tf32_round(v.x - hi.x);
      hi.y = tc::tf32_round(v.y); lo.y = tc::tf32_round(v.y - hi.y);
      hi.z = tc::tf32_round(v.z); lo.z = tc::tf32_round(v.z - hi.z);
      hi.w = tc::tf32_round(v.w); lo.w = tc::tf32_round(v.w - hi.w);
      const uint32_t off = (uint32_t)((i >> 3) * 1024 + (i & 7) * 128 + (((b & 7) ^ (i & 7)) << 4));
      unsigned char* t = s.A + (size_t)((b >> 3) * 2) * s.MA * 128 + off;
      *reinterpret_cast<float4*>(t) = hi;
      *reinterpret_cast<float4*>(t + (size_t)s.MA * 128) = lo;
    }
  } else {
    s.ST[(4 * b + 0) * NPP + i] = v.x;
    s.ST[(4 * b + 1) * NPP + i] = v.y;
    s.ST[(4 * b + 2) * NPP + i] = v.z;
    s.ST[(4 * b + 3) * NPP + i] = v.w;
  }
}

// Work item `it` of a loop over (row i < nrows, 4-gene block b < nb): row
// fastest (consecutive threads on consecutive rows), or, for the BF16
// staging, 16 consecutive items on 8 rows x 2 neighbouring blocks.  Returns
// false for the padding items of the BF16 order.  The order of the items
// changes nothing but which thread does which.
__device__ __forceinline__ bool item_ib(int it, int nrows, int nb, bool pairs, int& i, int& b) {
  if (!pairs) {
    b = it / nrows;
    i = it - b * nrows;
    return true;
  }
  const int r8 = (nrows + 7) >> 3, g = it >> 4, l = it & 15;
  const int bp = g / r8, ro = g - bp * r8;
  i = 8 * ro + (l & 7);
  b = 2 * bp + (l >> 3);
  return i < nrows && b < nb;
}

__device__ __forceinline__ int items_ib(int nrows, int nb, bool pairs) {
  return pairs ? ((nrows + 7) >> 3) * ((nb + 1) >> 1) * 16 : nrows * nb;
}

// 4-gene blocks a staging loop covers: the row's DP / 4, and in the
// tensor-core form every block up to the operand tiles' K extent, so that
// the pad columns [D, Kp) are written (as zeros) with the rest of the row.
template <bool TC>
__device__ __forceinline__ int staged_blocks(const Smem& s, int DP) {
  if constexpr (TC) return (s.nkb * (s.bf16 ? 64 : 32)) >> 2;
  return DP >> 2;
}

template <bool TC>
__device__ void stage_differences(const Smem& s, const float* rows, int nrows, int D, int DP,
                                  int NPP) {
  const int nb = staged_blocks<TC>(s, DP), nbx = DP >> 2;
  const bool pairs = TC && s.bf16;
  const int nit = items_ib(nrows, nb, pairs);
  for (int it = threadIdx.x; it < nit; it += kThreads) {
    int i, b;
    if (!item_ib(it, nrows, nb, pairs, i, b)) continue;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (b < nbx) {
      const float4 x = reinterpret_cast<const float4*>(rows + i * DP)[b];
      const float4 o = reinterpret_cast<const float4*>(s.o)[b];
      v.x = 4 * b + 0 < D ? fsub(x.x, o.x) : 0.f;
      v.y = 4 * b + 1 < D ? fsub(x.y, o.y) : 0.f;
      v.z = 4 * b + 2 < D ? fsub(x.z, o.z) : 0.f;
      v.w = 4 * b + 3 < D ? fsub(x.w, o.w) : 0.f;
    }
    stage4<TC>(s, i, b, v, NPP);
  }
}

// Zeros in the pad columns [D, Kp) of the tensor-core operand rows [0,
// nrows), for the staging paths that write gene by gene (the GA trials).
// The columns must hold finite values: they meet Q's zero columns, and the
// rotated rows and the re-check scratch alias this region between
// rotations.
__device__ void zero_pads(const Smem& s, int D, int nrows) {
  const int epr = s.bf16 ? 64 : 32;
  const int kp = s.nkb * epr, npad = kp - D;
  const size_t pl = (size_t)s.MA * 128;
  for (int it = threadIdx.x; it < nrows * npad; it += kThreads) {
    const int i = it / npad, j = D + (it - i * npad);
    if (s.bf16) {
      unsigned char* t = s.A + (size_t)((j >> 6) * 3) * pl + tc::sw128_offset_b16(i, j & 63);
      *reinterpret_cast<uint16_t*>(t) = 0;
      *reinterpret_cast<uint16_t*>(t + pl) = 0;
      *reinterpret_cast<uint16_t*>(t + 2 * pl) = 0;
    } else {
      unsigned char* t = s.A + (size_t)((j >> 5) * 2) * pl + tc::sw128_offset(i, j & 31);
      *reinterpret_cast<float*>(t) = 0.f;
      *reinterpret_cast<float*>(t + pl) = 0.f;
    }
  }
}

// The island's MMAs (mma_entry, issue order), written once per island by all
// threads (read after the next barrier); returns their number.  Each entry:
// descriptor low words (the tile's base descriptor plus its offset >> 4 in
// the start-address field, bits 0-13: shared addresses stay below 256 KB, so
// there is no carry and the high words are the base descriptors'),
// accumulator column, accumulate flag.
__device__ __noinline__ int mma_descriptors(uint4* tab, uint32_t a_saddr, uint32_t b_saddr,
                                            int MA, int Np, int planes, int nkb, int bplanes,
                                            int ksteps, bool paired) {
  const uint64_t a0 = tc::sdesc_sw128(a_saddr), b0 = tc::sdesc_sw128(b_saddr);
  const int n = mma_per_kstep(planes, paired) * ksteps;
  for (int i = threadIdx.x; i < n && i < kMaxMmas; i += kThreads) {
    const MmaEntry e = mma_entry(i, MA, Np, planes, nkb, bplanes, paired);
    const uint64_t ad = a0 + ((e.a_off + e.k_off) >> 4);
    const uint64_t bd = b0 + ((e.b_off + e.k_off) >> 4);
    tab[i] = make_uint4((uint32_t)ad, (uint32_t)bd, e.acc * 128u, e.accumulate);
  }
  return n < kMaxMmas ? n : kMaxMmas;
}

// Tensor-core rotation of rows [0, nrows) staged with their pad columns:
// the island's MMAs (mma_descriptors) over the K steps that cover D (32
// bytes of each 128-byte row per step: 8 TF32 or 16 BF16 values) from one
// issuing thread, completion on an mbarrier.  The product of the two leading
// parts accumulates alone, so the large partial sums do not swallow the small
// products (each MMA step rounds its accumulator to FP32).  Each warp that
// drains rows waits on the mbarrier itself, reads its TMEM lanes (warp w
// reads the lanes of sub-partition w mod 4, its half of the columns), adds
// the small products, then the leading one, in FP32 and stores Z.
// phase: the mbarrier parity this CTA expects next.
__device__ void rotate_tc(const Smem& s, int D, int DP, int nrows, uint32_t& phase) {
  tc::fence_async_smem();  // generic-proxy operand writes -> async proxy
  __syncthreads();
  const bool dead = *s.dead != 0;  // an earlier wait gave up: skip the MMAs
  EMT_PHASE(s, PH_MMA_ISSUE);
  if (threadIdx.x == 0 && !dead && !s.lose_completion) {
    tc::fence_after();
    // the table of mma_descriptors, in issue order
    for (int i = 0; i < s.nmma; ++i) {
      const uint4 w = s.mdesc[i];
      const uint64_t ad = ((uint64_t)s.ad_hi << 32) | w.x, bd = ((uint64_t)s.bd_hi << 32) | w.y;
      if (s.bf16)
        tc::mma_bf16(s.tmem + w.z, ad, bd, s.idesc, w.w);
      else
        tc::mma_tf32(s.tmem + w.z, ad, bd, s.idesc, w.w);
    }
    tc::mma_commit(s.mma_bar);
  }
  EMT_PHASE_LAP(s, PH_MMA_WAIT);
  // Each warp that drains rows waits for the completion itself, so no CTA
  // barrier stands between the completion and the drain; the others go on
  // to the closing barrier.  A wait that gives up marks the CTA dead; its
  // warp writes finite zeros instead, and the epoch stops at the end of this
  // generation with CHECK_TIMEOUT reported.
  // TMEM holds row r of an M = 128 result in lane r; an M = 64 result puts
  // rows 16q .. 16q + 15 in lanes 32q .. 32q + 15 of sub-partition q
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rpq = s.MA >> 2;  // rows per sub-partition: 16 or 32
  if (rpq * (warp & 3) < nrows) {  // warp-uniform: the loads are .sync.aligned
    bool ok = !dead;
    if (ok) {
      ok = tc::mbar_wait(s.mma_bar, phase, s.wait_ns);
      ok = __all_sync(0xFFFFFFFFu, ok);
      if (!ok && lane == 0) atomicExch(s.dead, 1);
      if (ok) tc::fence_after();
    }
    EMT_PHASE_LAP(s, PH_DRAIN);
    const int q = warp & 3, row = lane < rpq ? rpq * q + lane : nrows;  // nrows: no row
    // output columns: the paired form's first 64 (its columns 64-127 hold the
    // second part of Q), else N
    const int nch = (s.paired ? 64 : s.N) >> 4, half = (nch + 1) >> 1;
    const int c_lo = (warp >> 2) ? half : 0, c_hi = (warp >> 2) ? nch : half;
    for (int c = c_lo; c < c_hi; ++c) {
      const int c0 = 16 * c;
      float v[16], w[16];
      if (ok) {
        // the small products first, then the leading one
        const uint32_t t0 = s.tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0;
        tc::tmem_ld16(t0 + 128u, w);
        if (s.paired) {
          tc::tmem_ld16(t0 + 64u, v);
#pragma unroll
          for (int g = 0; g < 16; ++g) w[g] = __fadd_rn(w[g], v[g]);
          tc::tmem_ld16(t0 + 192u, v);
#pragma unroll
          for (int g = 0; g < 16; ++g) w[g] = __fadd_rn(w[g], v[g]);
        }
        tc::tmem_ld16(t0, v);
#pragma unroll
        for (int g = 0; g < 16; ++g) v[g] = __fadd_rn(v[g], w[g]);
      } else {
#pragma unroll
        for (int g = 0; g < 16; ++g) v[g] = 0.f;
      }
      if (row < nrows)
#pragma unroll
        for (int g = 0; g < 4; ++g)
          if (c0 + 4 * g < DP)
            reinterpret_cast<float4*>(s.Z + row * DP)[(c0 >> 2) + g] =
                make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2], v[4 * g + 3]);
    }
  }
  if (!dead) phase ^= 1u;
  tc::fence_before();
  __syncthreads();
}

// Evaluates rows [0, nrows) of `rows` (shared memory, stride DP) whose
// differences rows - o are already staged: rotation, then one warp per row.
template <bool TC>
__device__ void evaluate_rows(const Smem& s, const FnConst& fc, const float* rows, int nrows,
                              int DP, int NPP, float* fout, float* tout, uint32_t& phase) {
  EMT_PHASE(s, PH_ROTATE);
  if constexpr (TC) {
    rotate_tc(s, fc.D, DP, nrows, phase);
  } else {
    rotate_f32(s, fc.D, DP, NPP, nrows);
    __syncthreads();
  }
  EMT_PHASE(s, PH_EVAL);
  eval_rows_f32<kThreads>(fc, s.Z, rows, s.o, nrows, DP, fout, tout);
  __syncthreads();
}

// Trial vectors of generation G into U (and U - o into the rotation input).
template <bool TC>
__device__ void build_trials(const Smem& s, const EpochArgs& a, const TaskDev& td, int task,
                             uint32_t G, int DP, int NPP) {
  const int D = td.D, NP = td.NP;
  const float lo = td.lo, hi = td.hi;
  // partners come from the member's own sub-island of NPs members
  const int NPs = NP / a.subislands;
  if (a.algorithm == 0 || a.algorithm == 1) {
    for (int i = threadIdx.x; i < NP; i += kThreads) {
      const U4 w = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_DE_INDEX, 0);
      const int base = a.subislands > 1 ? (i / NPs) * NPs : 0;
      int r1, r2, r3, jr;
      de_indices(w, i - base, NPs, D, r1, r2, r3, jr);
      s.idx[4 * i + 0] = a.algorithm == 0 ? base + r1 : i;
      s.idx[4 * i + 1] = base + r2;
      s.idx[4 * i + 2] = base + r3;
      s.idx[4 * i + 3] = jr;
    }
    __syncthreads();
    const int nbd = (D + 3) >> 2, nb = TC ? staged_blocks<TC>(s, DP) : nbd;
    const bool pairs = TC && s.bf16;
    const int nit = items_ib(NP, nb, pairs);
    for (int it = threadIdx.x; it < nit; it += kThreads) {
      int i, b;
      if (!item_ib(it, NP, nb, pairs, i, b)) continue;
      if (TC && b >= nbd) {  // pad columns of the operand only
        stage4<TC>(s, i, b, make_float4(0.f, 0.f, 0.f, 0.f), NPP);
        continue;
      }
      const U4 w = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_DE_CR, (uint32_t)b);
      const int base = s.idx[4 * i], r2 = s.idx[4 * i + 1], r3 = s.idx[4 * i + 2],
                jr = s.idx[4 * i + 3];
      const float* xb = s.X + base * DP;
      const float* x2 = s.X + r2 * DP;
      const float* x3 = s.X + r3 * DP;
      const float* xi = s.X + i * DP;
      float tr[4], sv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = 4 * b + q;
        tr[q] = 0.f;
        sv[q] = 0.f;
        if (j < D) {
          const float m = clamp_box(ffma(a.F, fsub(x2[j], x3[j]), xb[j]), lo, hi);
          tr[q] = (u01(word(w, q)) < a.CR || j == jr) ? m : xi[j];
          sv[q] = fsub(tr[q], s.o[j]);
        }
      }
      reinterpret_cast<float4*>(s.U + i * DP)[b] = make_float4(tr[0], tr[1], tr[2], tr[3]);
      stage4<TC>(s, i, b, make_float4(sv[0], sv[1], sv[2], sv[3]), NPP);
    }
    return;
  }
  // GA: parent index per member (CrossPrep, SG-EMTF.cu:803-812), SBX on the
  // pair (i, i^1) (:711-749) and polynomial mutation (:565-605).
  for (int i = threadIdx.x; i < NP; i += kThreads) {
    const int base = a.subislands > 1 ? (i / NPs) * NPs : 0;
    s.idx[i] = base + (int)(draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_GA_PARENT, 0).x %
                            (uint32_t)NPs);
  }
  __syncthreads();
  const float ec = fdiv(1.f, fadd(a.eta_c, 1.f));
  const float em1 = fadd(a.eta_m, 1.f), em = fdiv(1.f, em1);
  const float pm = a.p_m < 0.f ? fdiv(1.f, (float)D) : a.p_m;
  const float range = fsub(hi, lo);
  const int nb = (D + 1) >> 1;
  for (int it = threadIdx.x; it < NP * nb; it += kThreads) {
    const int b = it / NP, i = it - b * NP;
    const int r0 = s.idx[i];
    const int pi = i ^ 1;
    const bool paired = pi < NP && (a.subislands == 1 || pi / NPs == i / NPs);
    const int partner = paired ? s.idx[pi] : r0;
    const U4 ws = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_GA_SBX, (uint32_t)b);
    const U4 wm = draw(a.seed, (uint32_t)task, G, (uint32_t)i, P_GA_PM, (uint32_t)b);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = 2 * b + h;
      if (j >= D) break;
      const float x0 = s.X[r0 * DP + j], x1 = s.X[partner * DP + j];
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
      s.U[i * DP + j] = c;
      stage<TC>(s, i, j, fsub(c, s.o[j]), NPP);
    }
  }
  if constexpr (TC) zero_pads(s, D, NP);
}

// Selection of nrows candidates (rows of U, fitness ftr/ttr) against members
// target[c] (X rows).  strict: candidate must be strictly better (transfer);
// otherwise ties go to the candidate (generation step).  Returns the number
// of replacements (valid in thread 0).
__device__ int select_and_replace(const Smem& s, const EpochArgs& a, const FnConst& fc,
                                  int nrows, const int* target, bool strict, int DP,
                                  unsigned long long* rechecks, unsigned long long* flips) {
  const bool recheck = !(a.flags & FLAG_NO_RECHECK);
  const bool anchors = recheck && s.zcb && !(a.flags & FLAG_NO_DIFF_RECHECK) &&
                       diff_pays(fc.fid);
  EMT_PHASE(s, PH_SELECT);
  if (threadIdx.x == 0) s.misc[0] = s.misc[1] = 0;
  __syncthreads();
  // flag bits: 1 accept, 2 re-checked, 4 anchor carried forward
  for (int c = threadIdx.x; c < nrows; c += kThreads) {
    const int m = target ? target[c] : c;
    const float ft = s.ftr[c], fp = s.fit[m];
    const bool d32 = strict ? (ft < fp) : (ft <= fp);
    if (recheck && fabsf(ft - fp) <= s.ttr[c] + s.tol[m]) {
      s.flag[c] = 2;
      s.list[atomicAdd(&s.misc[0], 1)] = c;
    } else if (d32 && anchors && s.zcb[2 * m] <= s.zcb[2 * m + 1]) {
      // accepted on FP32 fitness with a cached anchor: carry it forward (the
      // island is converging, so the member is likely re-checked again)
      s.flag[c] = 5;
      s.list[nrows - 1 - atomicAdd(&s.misc[1], 1)] = c;
    } else {
      s.flag[c] = d32 ? 1 : 0;
    }
  }
  __syncthreads();
  const int nre = s.misc[0], nadv = s.misc[1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  EMT_PHASE(s, PH_RECHECK);
  for (int r = warp; r < nre; r += kWarps) {
    const int c = s.list[r];
    const int m = target ? target[c] : c;
    double* zt = s.z64 + warp * 2 * DP;  // trial z, then parent z
    double* zp = zt + DP;
    // a candidate bit-identical to the member it would replace is a tie in
    // any precision: no re-evaluation needed
    bool same = true;
    for (int j = lane; j < fc.D; j += 32)
      same &= __float_as_uint(s.U[c * DP + j]) == __float_as_uint(s.X[m * DP + j]);
    same = __all_sync(0xFFFFFFFFu, same);
    double fp = s.fit64[m], ft = 0.0;
    bool d64;
    // the differential decision: sign of f(u) - f(x) from the parent's cached
    // compensated rotation and dz = Q (u - x), FP32/INT pipes only; -1 when
    // its bound cannot separate the two
    int dd = -1;
    // Weierstrass: whether fit64[m] is a float-float value afterwards (1),
    // a tier-3 value (0), or unchanged (-1); kept in the member's first
    // anchor-bound slot, which this function's islands do not use otherwise
    int wprec = -1;
    if (!same && anchors) {
      float* zh = s.zc + (size_t)m * 2 * DP;
      float* zl = zh + DP;
      float* buf = reinterpret_cast<float*>(zt);
      float ez = s.zcb[2 * m], lim = s.zcb[2 * m + 1];
      if (!(ez <= lim)) {  // not cached, or its bound has grown: recompute
        float zmax;
        ez = anchor_rotation(s.X + m * DP, s.o, s.QT, DP, fc.D, fc.qnorm * (1.f + 0x1p-20f), zh,
                             zl, &zmax, reinterpret_cast<float2*>(buf + 2 * DP));
        // carried-forward anchors may drift to 64x the fresh bound, or to
        // 2^-26 max|z| (below the rounding of the difference forms themselves)
        lim = fmaxf(64.f * ez, 0x1p-26f * zmax) + 1e-30f;
        if (lane == 0 && rechecks) atomicAdd(rechecks + 5, 1ull);
      }
      dd = diff_decide(fc, zh, zl, ez, s.X + m * DP, s.U + c * DP, s.QT, DP, buf);
      if (dd == 1) ez = anchor_advance(zh, zl, buf, DP, fc.D, ez);  // the trial replaces x
      if (lane == 0) {
        s.zcb[2 * m] = ez;
        s.zcb[2 * m + 1] = lim;
      }
    }
    if (same) {
      ft = fp;
      d64 = !strict;
    } else if (dd >= 0) {
      d64 = dd == 1;
      ft = __longlong_as_double(0x7FF8000000000000ll);  // exact values unknown
    } else {
      precise_rotation(s.U + c * DP, s.o, s.QT, DP, fc.D, zt);
      const bool tier2 = fc.fid != F_WEIERSTRASS && fc.fid != F_SPHERE && fc.fid != F_ROSENBROCK;
      bool decided = false;
      if (tier2) {
        // tier 2: FP32 terms on the precise rotation, with error bounds
        double et, ep = 0.0;
        const double t2 = eval_tier2(fc, zt, &et);
        double p2 = fp;
        if (isnan(fp)) {
          precise_rotation(s.X + m * DP, s.o, s.QT, DP, fc.D, zp);
          p2 = eval_tier2(fc, zp, &ep);
        }
        if (fabs(t2 - p2) > et + ep) {
          d64 = strict ? (t2 < p2) : (t2 <= p2);
          ft = __longlong_as_double(0x7FF8000000000000ll);  // exact values unknown
          decided = true;
        }
      }
      if (!decided) {
        // tier 3 (or the exact Weierstrass terms): FP64-class values, cached
        const bool weier = fc.fid == F_WEIERSTRASS;
        ft = weier ? eval_weier_precise(fc, zt) : eval_tier3(fc, zt);
        // the member's cached value is already float-float
        const bool pprec = weier && s.zcb && s.zcb[2 * m] == 0.f && !isnan(fp);
        bool zp_ready = false;
        if (isnan(fp)) {
          if (!tier2) precise_rotation(s.X + m * DP, s.o, s.QT, DP, fc.D, zp);
          fp = weier ? eval_weier_precise(fc, zp) : eval_tier3(fc, zp);
          zp_ready = true;
        }
        if (weier) {
          const double bound = weier_precise_bound(fc.D);
          if (fabs(ft - fp) <= (pprec ? bound : 2.0 * bound)) {
            // closer than the FP32 terms' error: every term in float-float
            if (!pprec) {
              if (!zp_ready) precise_rotation(s.X + m * DP, s.o, s.QT, DP, fc.D, zp);
              fp = eval_weier_ff_warp(fc, zp);
            }
            ft = eval_weier_ff_warp(fc, zt);
            wprec = 1;
            if (lane == 0 && rechecks) atomicAdd(rechecks + kStatWeierFp64, 1ull);
          }
        }
        d64 = strict ? (ft < fp) : (ft <= fp);
        if (weier && wprec < 0) wprec = (!d64 && pprec) ? 1 : 0;
      }
    }
    const bool d32 = strict ? (s.ftr[c] < s.fit[m]) : (s.ftr[c] <= s.fit[m]);
    if (lane == 0) {
      if (rechecks) {
        if (dd >= 0) atomicAdd(rechecks + 4, 1ull);
        if (same) atomicAdd(rechecks + 6, 1ull);
      }
      // a trial accepted through the FP64-class tiers has no cached anchor
      if (!same && dd < 0 && d64 && s.zcb) s.zcb[2 * m] = __int_as_float(0x7FC00000);
      if (wprec >= 0 && s.zcb) s.zcb[2 * m] = wprec ? 0.f : __int_as_float(0x7FC00000);
      s.flag[c] = d64 ? 3 : 0;
      // FP64 value of whichever vector member m holds after this selection,
      // cached for its next re-check.  Targets are distinct, so no race.
      s.fit64[m] = d64 ? ft : fp;
      if (rechecks) atomicAdd(rechecks, 1ull);
      if (flips && d64 != d32) atomicAdd(flips, 1ull);
    }
    __syncwarp();
  }
  for (int r = warp; r < nadv; r += kWarps) {
    const int c = s.list[nrows - 1 - r];
    const int m = target ? target[c] : c;
    float* buf = reinterpret_cast<float*>(s.z64 + warp * 2 * DP);
    float* zh = s.zc + (size_t)m * 2 * DP;
    row_offset(s.X + m * DP, s.U + c * DP, s.QT, DP, fc.D, fc.qnorm * (1.f + 0x1p-20f), buf,
               reinterpret_cast<float2*>(buf + 2 * DP));
    const float ez = anchor_advance(zh, zh + DP, buf, DP, fc.D, s.zcb[2 * m]);
    if (lane == 0) s.zcb[2 * m] = ez;  // refreshed on its next use if above the limit
    __syncwarp();
  }
  EMT_PHASE(s, PH_SELECT);
  __syncthreads();
  // copy accepted candidates into the population
  const int nq = DP >> 2;
  for (int it = threadIdx.x; it < nrows * nq; it += kThreads) {
    const int c = it / nq, q = it - c * nq;
    if (s.flag[c] & 1) {
      const int m = target ? target[c] : c;
      reinterpret_cast<float4*>(s.X + m * DP)[q] = reinterpret_cast<const float4*>(s.U + c * DP)[q];
    }
  }
  int acc = 0;
  for (int c = threadIdx.x; c < nrows; c += kThreads) {
    if (s.flag[c] & 1) {
      const int m = target ? target[c] : c;
      s.fit[m] = s.ftr[c];
      s.tol[m] = s.ttr[c];
      if (!(s.flag[c] & 2)) s.fit64[m] = __longlong_as_double(0x7FF8000000000000ll);
      if (s.flag[c] == 1 && s.zcb) s.zcb[2 * m] = __int_as_float(0x7FC00000);
      ++acc;
    }
  }
  __syncthreads();
  (void)fc;
  return acc;
}

// rank[i] = #{j : fit[j] < fit[i] or (fit[j] == fit[i] and j < i)}; writes
// byrank[rank[i]] = i.
__device__ void rank_members(const Smem& s, int NP, int* byrank) {
  for (int i = threadIdx.x; i < NP; i += kThreads) {
    const float fi = s.fit[i];
    int r = 0;
    for (int j = 0; j < NP; ++j) {
      const float fj = s.fit[j];
      r += (fj < fi || (fj == fi && j < i)) ? 1 : 0;
    }
    byrank[r] = i;
  }
  __syncthreads();
}

// Ring migration between the sub-islands of one island (IslandMigration,
// SG-EMTF.cu:1138-1218, which exchanges between the two slots of a block):
// each sub-island is ranked by FP32 fitness (ties by index, as the
// reference's odd-even transposition sort keeps them); candidate c = s*m + r
// is a copy of the r-th best of sub-island s and targets the r-th worst of
// s + 1 (mod S).  Candidates are copied before any replacement, so every
// exchange starts from the pre-migration state; the decision is the strict
// transfer selection, re-checks included.  No evaluations: a copy carries its
// source's FP32 fitness and tolerance.
__device__ void migrate(const Smem& s, const EpochArgs& a, const FnConst& fc, int NP, int DP,
                        unsigned long long* st_re, unsigned long long* st_fl) {
  const int S = a.subislands, NPs = NP / S;
  const int m = a.mig_count > 0 ? a.mig_count : max(1, NPs / 8), k = S * m;
  int* byrank = s.idx;       // NP ints
  int* target = s.idx + NP;  // k <= NP / 2 ints
  for (int i = threadIdx.x; i < NP; i += kThreads) {
    const int base = (i / NPs) * NPs;
    const float fi = s.fit[i];
    int r = 0;
    for (int j = base; j < base + NPs; ++j) {
      const float fj = s.fit[j];
      r += (fj < fi || (fj == fi && j < i)) ? 1 : 0;
    }
    byrank[base + r] = i;
  }
  __syncthreads();
  const int nq = DP >> 2;
  for (int it = threadIdx.x; it < k * nq; it += kThreads) {
    const int c = it / nq, q = it - c * nq;
    const int sc = c / m, src = byrank[sc * NPs + (c - sc * m)];
    reinterpret_cast<float4*>(s.U + c * DP)[q] = reinterpret_cast<const float4*>(s.X + src * DP)[q];
  }
  for (int c = threadIdx.x; c < k; c += kThreads) {
    const int sc = c / m, r = c - sc * m, src = byrank[sc * NPs + r];
    const int dst = sc + 1 == S ? 0 : sc + 1;
    target[c] = byrank[dst * NPs + NPs - 1 - r];
    s.ftr[c] = s.fit[src];
    s.ttr[c] = s.tol[src];
  }
  __syncthreads();
  const int acc = select_and_replace(s, a, fc, k, target, true, DP, st_re, st_fl);
  if (acc && a.stats) atomicAdd(a.stats + 7, (unsigned long long)acc);
}

__device__ __forceinline__ int transfer_k(float rate, int NP) {
  int k = (int)(rate * (float)NP + 0.5f);
  return k < 1 ? 1 : (k > NP ? NP : k);
}

template <bool TC>
__device__ __forceinline__ void epoch_body(const EpochArgs& a, const void* tmap,
                                           unsigned char* smem_raw, int task, TcCta& cta) {
  if (task < 0 || task >= a.n_tasks) {
    if (threadIdx.x == 0) report(a.err, CHECK_BAD_DESCRIPTOR);
    return;
  }
  const TaskDev td = a.tasks[task];
  if (!descriptor_ok(td)) {
    if (threadIdx.x == 0) report(a.err, CHECK_BAD_DESCRIPTOR);
    return;
  }
  const int D = td.D, NP = td.NP;
  Smem s;
  int DP, NPP;
  if constexpr (TC) {
    if (NP > 128 || round8(D) > a.tc_np || (a.tc_bf16 ? round64(D) : round32(D)) > a.tc_kp) {
      if (threadIdx.x == 0) report(a.err, CHECK_TC_SHAPE);
      return;
    }
    const TcLayout L = tc_layout(D, NP, a.tc_np, a.tc_kp, a.tc_bf16 != 0);
    if (L.total > a.smem_bytes) {
      if (threadIdx.x == 0) report(a.err, CHECK_SMEM_TOO_SMALL);
      return;
    }
    s = carve_tc(smem_raw, L);
    s.mma_bar = cta.mma_bar;
    s.tma_bar = cta.tma_bar;
    s.tmem = cta.tmem;
    s.dead = &cta.hdr->dead;
    s.wait_ns = a.wait_ns ? a.wait_ns : tc::kWaitLimitNs;
    s.lose_completion = (a.flags & FLAG_TEST_LOST_COMPLETION) != 0;
    s.QT = const_cast<float*>(a.qt + td.q_off);  // FP32 Q^T for the re-checks
    DP = L.DP;
    NPP = round4(NP);
    s.N = s.paired ? 128 : round16(D);
    s.ksteps = s.bf16 ? (D + 15) >> 4 : (D + 7) >> 3;
    // M = 64 for islands of <= 64 members (the A tiles' own rows), else 128
    s.idesc = s.bf16 ? tc::idesc_bf16(s.MA, s.N) : tc::idesc_tf32(s.MA, s.N);
    s.nmma = mma_descriptors(const_cast<uint4*>(s.mdesc), s.a_saddr, s.b_saddr, s.MA, s.Np,
                             s.planes, s.nkb, s.bplanes, s.ksteps, s.paired);
    s.ad_hi = (uint32_t)(tc::sdesc_sw128(s.a_saddr) >> 32);
    s.bd_hi = (uint32_t)(tc::sdesc_sw128(s.b_saddr) >> 32);
    // zero the operand tiles once: padded K columns meet zero Q columns, so
    // they only need to hold finite values; and the paired BF16 form's zero
    // tiles of B (the fourth of each K block), which no TMA copy writes
    for (size_t it = threadIdx.x; it < (L.B - L.A) / 16; it += kThreads)
      reinterpret_cast<float4*>(s.A)[it] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (s.bplanes > s.planes)
      for (int it = threadIdx.x; it < s.nkb * s.Np * 8; it += kThreads) {
        const int kb = it / (s.Np * 8), r = it - kb * s.Np * 8;
        reinterpret_cast<float4*>(s.B + (size_t)(kb * s.bplanes + s.planes) * s.Np * 128)[r] =
            make_float4(0.f, 0.f, 0.f, 0.f);
      }
    // B operand: Q's part tiles of this task by TMA (box one 128-byte row x
    // Np x 1 per tile) into the B region, which no MMA reads any more (the
    // previous island's last MMAs completed before its selection)
    if (threadIdx.x == 0 && !*s.dead) {
      tc::mbar_expect_tx(s.tma_bar, (uint32_t)(s.planes * s.nkb * s.Np * 128));
      for (int h = 0; h < s.planes; ++h)
        for (int kb = 0; kb < s.nkb; ++kb) {
          const int tile = s.paired ? kb * s.bplanes + h : h * s.nkb + kb;
          tc::tma_load_3d(s.b_saddr + (uint32_t)(tile * s.Np * 128), tmap, L.epr * kb, 0,
                          s.planes * task + h, s.tma_bar);
        }
    }
  } else {
    const Layout L = smem_layout(D, NP, td.qt_in_smem != 0);
    if (L.total > a.smem_bytes) {
      if (threadIdx.x == 0) report(a.err, CHECK_SMEM_TOO_SMALL);
      return;
    }
    s = carve(smem_raw, L);
    if (!td.qt_in_smem) s.QT = const_cast<float*>(a.qt + td.q_off);
    DP = L.DP;
    NPP = L.NPP;
  }
  FnConst fc;
  fc.fid = td.fid;
  fc.D = D;
  fc.flags = td.flags;
  fc.woff = td.woff;
  fc.qnorm = td.qnorm;
  fc.rel = a.recheck_rel;
  fc.woff64 = td.woff64;
  if (a.zc && a.zcb) {
    s.zc = a.zc + 2 * td.pop_off;
    s.zcb = a.zcb + 2 * (size_t)td.fit_off;
  }
  uint32_t phase = TC ? cta.mphase : 0u;
#ifdef EMT_PHASE_CLOCKS
  PhaseClock ph;
  ph.begin();
  s.ph = &ph;
#endif

  // ---- load the task into shared memory ----
  const float* gq = a.qt + td.q_off;
  if (!TC && td.qt_in_smem)
    for (int it = threadIdx.x; it < D * (DP >> 2); it += kThreads)
      reinterpret_cast<float4*>(s.QT)[it] = reinterpret_cast<const float4*>(gq)[it];
  for (int j = threadIdx.x; j < DP; j += kThreads) s.o[j] = j < D ? a.shift[td.o_off + j] : 0.f;
  if (!TC)
    for (int it = threadIdx.x; it < DP * NPP; it += kThreads) s.ST[it] = 0.f;
  float* gpop = a.pop + td.pop_off;
  if (a.mode == MODE_INIT) {
    const float r = fsub(td.hi, td.lo);
    const int nb = (D + 3) >> 2;
    for (int it = threadIdx.x; it < NP * nb; it += kThreads) {
      const int i = it / nb, b = it - i * nb;
      const U4 w = draw(a.seed, (uint32_t)task, 0u, (uint32_t)i, P_POP_INIT, (uint32_t)b);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = 4 * b + q;
        if (j < D) s.X[i * DP + j] = fminf(ffma(u01(word(w, q)), r, td.lo), td.hi);
      }
      if (4 * b + 4 >= DP)
        for (int j = D; j < DP; ++j) s.X[i * DP + j] = 0.f;
    }
  } else {
    for (int it = threadIdx.x; it < NP * (DP >> 2); it += kThreads)
      reinterpret_cast<float4*>(s.X)[it] = reinterpret_cast<const float4*>(gpop)[it];
    for (int i = threadIdx.x; i < NP; i += kThreads) {
      s.fit[i] = a.fit32[td.fit_off + i];
      s.tol[i] = a.tol32[td.fit_off + i];
      s.fit64[i] = a.fit64[td.fit_off + i];
    }
  }
  for (int it = threadIdx.x; it < NP * DP; it += kThreads) s.U[it] = 0.f;
  if constexpr (TC) {
    if (!*s.dead) {
      if ((threadIdx.x >> 5) == 0 && !tc::mbar_wait(s.tma_bar, cta.tphase, s.wait_ns))
        atomicExch(s.dead, 1);
      cta.tphase ^= 1u;
    }
  }
  __syncthreads();

  unsigned long long* st_re = a.stats ? a.stats + 0 : nullptr;
  unsigned long long* st_fl = a.stats ? a.stats + 1 : nullptr;

  if (a.mode == MODE_INIT || a.mode == MODE_EVAL) {
    stage_differences<TC>(s, s.X, NP, D, DP, NPP);
    __syncthreads();
    evaluate_rows<TC>(s, fc, s.X, NP, DP, NPP, s.fit, s.tol, phase);
    for (int i = threadIdx.x; i < NP; i += kThreads) {
      s.fit64[i] = __longlong_as_double(0x7FF8000000000000ll);
      if (s.zcb) s.zcb[2 * i] = __int_as_float(0x7FC00000);  // anchors not cached
    }
    if (threadIdx.x == 0) {
      a.gen[task] = a.mode == MODE_INIT ? 0u : a.gen[task];
      if (a.stats) atomicAdd(a.stats + 3, (unsigned long long)NP);
    }
  } else {
    const uint32_t gen0 = a.gen[task];
    // ---- elite transfer in (knowledgeTransfer, SG-EMTF.cu:1514-1591) ----
    if (a.transfer_import && a.elites_in && a.n_tasks > 1) {
      const U4 w = draw(a.seed, (uint32_t)task, gen0, 0u, P_TRANSFER_PARTNER, 0);
      uint32_t p = w.x % (uint32_t)(a.n_tasks - 1);
      if (p >= (uint32_t)task) ++p;
      const TaskDev pd = a.tasks[p];
      if (!descriptor_ok(pd)) {
        if (threadIdx.x == 0) report(a.err, CHECK_BAD_PARTNER);
      } else {
        int* byrank = s.idx;  // NP ints (idx has 4*NP)
        rank_members(s, NP, byrank);
        const int kt = transfer_k(a.transfer_rate, NP), kp = transfer_k(a.transfer_rate, pd.NP);
        const int k = kt < kp ? kt : kp;
        const float* el = a.elites_in + pd.elite_off;
        const float rp = fsub(pd.hi, pd.lo), rt = fsub(td.hi, td.lo);
        for (int it = threadIdx.x; it < k * D; it += kThreads) {
          const int c = it / D, j = it - c * D;
          const U4 wm = draw(a.seed, (uint32_t)task, gen0, (uint32_t)c, P_TRANSFER_MIX, (uint32_t)(j >> 2));
          float v = s.X[byrank[c] * DP + j];
          if (j < pd.D && u01(word(wm, j & 3)) < a.transfer_mix) {
            const float r = fdiv(fsub(el[c * pd.DP + j], pd.lo), rp);
            v = clamp_box(ffma(r, rt, td.lo), td.lo, td.hi);
          }
          s.U[c * DP + j] = v;
        }
        __syncthreads();
        stage_differences<TC>(s, s.U, k, D, DP, NPP);
        __syncthreads();
        evaluate_rows<TC>(s, fc, s.U, k, DP, NPP, s.ftr, s.ttr, phase);
        int* target = s.idx + NP;  // member of rank NP - k + c
        for (int c = threadIdx.x; c < k; c += kThreads) target[c] = byrank[NP - k + c];
        __syncthreads();
        const int acc = select_and_replace(s, a, fc, k, target, true, DP, st_re, st_fl);
        if (acc && a.stats) atomicAdd(a.stats + 2, (unsigned long long)acc);
        if (threadIdx.x == 0 && a.stats) atomicAdd(a.stats + 3, (unsigned long long)k);
      }
      __syncthreads();
    }
    // ---- generations ----
    for (int g = 0; g < a.gens; ++g) {
      const uint32_t G = gen0 + (uint32_t)g + 1u;
      if (a.subislands > 1 && a.mig_interval > 0 && G > 1u &&
          (G - 1u) % (uint32_t)a.mig_interval == 0u)
        migrate(s, a, fc, NP, DP, st_re, st_fl);
      EMT_PHASE(s, PH_BUILD);
      build_trials<TC>(s, a, td, task, G, DP, NPP);
      __syncthreads();
      evaluate_rows<TC>(s, fc, s.U, NP, DP, NPP, s.ftr, s.ttr, phase);
      select_and_replace(s, a, fc, NP, nullptr, false, DP, st_re, st_fl);
      EMT_PHASE(s, PH_OTHER);
      if constexpr (TC) {
        if (*s.dead) break;  // read after the selection's barrier: CTA-uniform
      }
    }
    if (threadIdx.x == 0) {
      a.gen[task] = gen0 + (uint32_t)a.gens;
      if (a.stats) atomicAdd(a.stats + 3, (unsigned long long)NP * (unsigned long long)a.gens);
    }
    // ---- elite export: top-k rows for the next epoch's receivers ----
    if (a.transfer_export && a.elites_out) {
      __syncthreads();
      int* byrank = s.idx;
      rank_members(s, NP, byrank);
      const int k = transfer_k(a.transfer_rate, NP);
      float* el = a.elites_out + td.elite_off;
      for (int it = threadIdx.x; it < k * DP; it += kThreads) {
        const int c = it / DP, j = it - c * DP;
        el[c * DP + j] = s.X[byrank[c] * DP + j];
      }
    }
  }
  __syncthreads();
  // ---- write the island back ----
  for (int it = threadIdx.x; it < NP * (DP >> 2); it += kThreads)
    reinterpret_cast<float4*>(gpop)[it] = reinterpret_cast<const float4*>(s.X)[it];
  for (int i = threadIdx.x; i < NP; i += kThreads) {
    a.fit32[td.fit_off + i] = s.fit[i];
    a.tol32[td.fit_off + i] = s.tol[i];
    a.fit64[td.fit_off + i] = s.fit64[i];
  }
#ifdef EMT_PHASE_CLOCKS
  ph.flush(a.stats);
#endif
  if constexpr (TC) cta.mphase = phase;
}

// Sets up the CTA's tensor-core state in the header of its dynamic shared
// memory: both mbarriers, the flag, and 2 x pow2(tc_np) TMEM columns (two
// accumulators of the rotation).
__device__ __forceinline__ void tc_cta_begin(const EpochArgs& a, unsigned char* smem_raw,
                                             TcCta& cta) {
  cta.hdr = reinterpret_cast<TcHeader*>(smem_raw + a.smem_bytes - kTcHeader);
  cta.mma_bar = tc::smem_addr(&cta.hdr->mma_bar);
  cta.tma_bar = tc::smem_addr(&cta.hdr->tma_bar);
  // two accumulators of 128 columns (N <= 128): two CTAs per SM stay within
  // the SM's 512 columns
  cta.ncols = 256;
  cta.mphase = cta.tphase = 0;
  if (threadIdx.x == 0) {
    tc::mbar_init(cta.mma_bar, 1);
    tc::mbar_init(cta.tma_bar, 1);
    cta.hdr->dead = 0;
  }
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&cta.hdr->tmem, cta.ncols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  cta.tmem = *reinterpret_cast<volatile uint32_t*>(&cta.hdr->tmem);
}

// Reports a wait that gave up and frees the CTA's TMEM (no MMA is in
// flight: every commit issued was waited for, or none was issued).
__device__ __forceinline__ void tc_cta_end(const EpochArgs& a, TcCta& cta) {
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (threadIdx.x == 0 && cta.hdr->dead) report(a.err, CHECK_TIMEOUT);
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(cta.tmem, cta.ncols);
}

// One island per CTA (order[blockIdx.x], or single_task), or (QUEUE) a
// persistent grid: each CTA takes the next island of the longest-first
// order from the counter until none is left.  Separate instantiations keep
// the one-island kernels' registers as they are.
template <bool TC, bool QUEUE>
__device__ __forceinline__ void epoch_entry(const EpochArgs& a, const void* tmap,
                                            unsigned char* smem_raw) {
  TcCta cta{};
  if constexpr (TC) {
    // the swizzled operand tiles need 1024-byte alignment; the layout keeps
    // no slack for it, so a launch that does not provide it stops here
    if ((tc::smem_addr(smem_raw) & 1023u) != 0u || a.smem_bytes < kTcHeader) {
      if (threadIdx.x == 0) report(a.err, CHECK_SMEM_ALIGN);
      return;
    }
    tc_cta_begin(a, smem_raw, cta);
  }
  if constexpr (!QUEUE) {
    epoch_body<TC>(a, tmap, smem_raw,
                   a.single_task >= 0 ? a.single_task
                                      : (a.order ? a.order[blockIdx.x] : (int)blockIdx.x),
                   cta);
  } else {
    // the island slot, in dynamic shared memory at a place no island's
    // layout uses (the TC header; the FP32 layout's last bytes): static
    // shared memory would push the dynamic allocation, whose alignment in
    // this module is 1024 bytes (the TC kernels ask for it), back by 1 KB
    int* item;
    if constexpr (TC)
      item = &cta.hdr->item;
    else
      item = reinterpret_cast<int*>(smem_raw + a.smem_bytes - kQueueSlot);
    for (;;) {
      __syncthreads();  // the previous island is written back; item is free
      if (threadIdx.x == 0) *item = atomicAdd(a.queue, 1);
      __syncthreads();
      const int i = *item;
      if (i >= a.n_tasks) break;
      if constexpr (TC) {
        if (cta.hdr->dead) break;  // written before the barrier above: CTA-uniform
      }
      epoch_body<TC>(a, tmap, smem_raw, a.order ? a.order[i] : i, cta);
    }
  }
  if constexpr (TC) tc_cta_end(a, cta);
}

// FP32 form: three islands of D = 50, NP = 64 share an SM (~68 KB each).
__global__ void __launch_bounds__(kThreads, 3) epoch_kernel(const EpochArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  epoch_entry<false, false>(a, nullptr, smem_raw);
}
__global__ void __launch_bounds__(kThreads, 3) epoch_kernel_queue(const EpochArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  epoch_entry<false, true>(a, nullptr, smem_raw);
}

// Tensor-core forms: two islands per SM with up to 128 registers a thread
// (no spills).  Three per SM at 80 registers, which the BF16 form's ~76 KB
// of shared memory would allow, spilled and ran slower (D = 50, NP = 64:
// 165 against 155 ms per config-2 step).
__global__ void __launch_bounds__(kThreads, 2) epoch_kernel_tc(const EpochArgs a,
                                                                const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(1024) unsigned char smem_tc[];
  epoch_entry<true, false>(a, &tmap, smem_tc);
}
__global__ void __launch_bounds__(kThreads, 2) epoch_kernel_tc_queue(
    const EpochArgs a, const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(1024) unsigned char smem_tc[];
  epoch_entry<true, true>(a, &tmap, smem_tc);
}

// Evaluates n caller points of one task in chunks of up to 64 rows per CTA
// (the reference's evaluate kernel, SG-EMTF.cu:1428-1479).
__global__ void __launch_bounds__(kThreads) eval_kernel(const EvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const TaskDev td = a.tasks[a.task];
  if (!descriptor_ok(td)) {
    if (threadIdx.x == 0) report(a.err, CHECK_BAD_DESCRIPTOR);
    return;
  }
  const int D = td.D;
  const int rows = 64;
  const Layout L = smem_layout(D, rows);
  if (L.total > a.smem_bytes) {
    if (threadIdx.x == 0) report(a.err, CHECK_SMEM_TOO_SMALL);
    return;
  }
  const int DP = L.DP, NPP = L.NPP;
  const Smem s = carve(smem_raw, L);
  FnConst fc;
  fc.fid = td.fid;
  fc.D = D;
  fc.flags = td.flags;
  fc.woff = td.woff;
  fc.qnorm = td.qnorm;
  fc.rel = 0.f;
  fc.woff64 = td.woff64;
  const float* gq = a.qt + td.q_off;
  for (int it = threadIdx.x; it < D * DP; it += kThreads) s.QT[it] = gq[it];
  for (int j = threadIdx.x; j < DP; j += kThreads) s.o[j] = j < D ? a.shift[td.o_off + j] : 0.f;
  for (int it = threadIdx.x; it < DP * NPP; it += kThreads) s.ST[it] = 0.f;
  const int r0 = blockIdx.x * rows;
  const int nr = min(rows, a.n - r0);
  for (int it = threadIdx.x; it < rows * DP; it += kThreads) {
    const int i = it / DP, j = it - i * DP;
    s.U[it] = (i < nr && j < D) ? a.x[(size_t)(r0 + i) * D + j] : 0.f;
  }
  __syncthreads();
  stage_differences<false>(s, s.U, nr, D, DP, NPP);
  __syncthreads();
  uint32_t phase = 0;
  evaluate_rows<false>(s, fc, s.U, nr, DP, NPP, s.ftr, s.ttr, phase);
  for (int i = threadIdx.x; i < nr; i += kThreads) a.f[r0 + i] = s.ftr[i];
  if (a.z)
    for (int it = threadIdx.x; it < nr * D; it += kThreads) {
      const int i = it / D, j = it - i * D;
      a.z[(size_t)(r0 + i) * D + j] = s.Z[i * DP + j];
    }
}

__global__ void __launch_bounds__(32) best_kernel(const BestArgs a) {
  __shared__ double zbuf[kMaxDim];
  const int task = blockIdx.x;
  if (task >= a.n_tasks) return;
  const TaskDev td = a.tasks[task];
  if (!descriptor_ok(td)) return;
  const int lane = threadIdx.x;
  float bf = __int_as_float(0x7F800000);
  int bi = 0x7FFFFFFF;
  for (int i = lane; i < td.NP; i += 32) {
    const float f = a.fit32[td.fit_off + i];
    if (f < bf || (f == bf && i < bi)) { bf = f; bi = i; }
  }
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    const float of = __shfl_xor_sync(0xFFFFFFFFu, bf, m);
    const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, m);
    if (of < bf || (of == bf && oi < bi)) { bf = of; bi = oi; }
  }
  if (bi < 0 || bi >= td.NP) bi = 0;
  double f64 = a.fit64[td.fit_off + bi];
  if (isnan(f64)) {
    FnConst fc;
    fc.fid = td.fid;
    fc.D = td.D;
    fc.flags = td.flags;
    fc.woff = td.woff;
    fc.qnorm = td.qnorm;
    fc.rel = 0.f;
    fc.woff64 = td.woff64;
    f64 = eval_row_f64(fc, a.pop + td.pop_off + (size_t)bi * td.DP, a.shift + td.o_off,
                       a.qt + td.q_off, td.DP, zbuf);
  }
  if (lane == 0) {
    a.best_idx[task] = bi;
    a.best_f32[task] = bf;
    a.best_f64[task] = f64;
    if (a.best_err) a.best_err[task] = best_rel_err(td, bf, f64, a.tol32[td.fit_off + bi], a.rel);
  }
}

// TF32 part of x: round to nearest, ties away from zero, on the bit pattern
// (finite x); x - tf32_rna(x) is exact in FP32.
__device__ __forceinline__ float tf32_rna(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// BF16 part of x: round to nearest even on the bit pattern (finite x).
__device__ __forceinline__ uint32_t bf16_rne(float x) {
  const uint32_t b = __float_as_uint(x);
  return (b + 0x7FFFu + ((b >> 16) & 1u)) >> 16;
}
__device__ __forceinline__ float bf16_val(uint32_t h) { return __uint_as_float(h << 16); }

__device__ __forceinline__ void put_planes(const QPlanes& pl, int t, int r, int c, float v) {
  const size_t at = (size_t)t * pl.task_stride + (size_t)r * pl.row_stride + c;
  if (pl.kind == QPLANES_BF16) {
    uint16_t* q = static_cast<uint16_t*>(pl.base);
    const uint32_t p0 = bf16_rne(v);
    const float r1 = __fsub_rn(v, bf16_val(p0));  // exact
    const uint32_t p1 = bf16_rne(r1);
    q[at] = (uint16_t)p0;
    q[at + pl.plane_stride] = (uint16_t)p1;
    q[at + 2 * pl.plane_stride] = (uint16_t)bf16_rne(__fsub_rn(r1, bf16_val(p1)));
  } else if (pl.kind == QPLANES_TF32) {
    float* q = static_cast<float*>(pl.base);
    const float vh = tf32_rna(v);
    q[at] = vh;
    q[at + pl.plane_stride] = tf32_rna(__fsub_rn(v, vh));
  }
}

// One CTA per task and pair of 32 x 32 tiles (i, j), (j, i) with i <= j: both
// tiles are read into shared memory before either is written, so the in-place
// transpose has one writer per element; the split planes are written from the
// same tiles, along rows of Q.
__global__ void __launch_bounds__(256) prepare_rotations_kernel(const TaskDev* tasks, float* qt,
                                                                const QPlanes pl) {
  const int t = blockIdx.x, bi = blockIdx.y, bj = blockIdx.z;
  if (bi > bj) return;
  const TaskDev td = tasks[t];
  const int D = td.D, DP = td.DP;
  if (bj * 32 >= D) return;
  __shared__ float ta[32][33], tb[32][33];  // Q[32 bi + y][32 bj + x], Q[32 bj + y][32 bi + x]
  float* q = qt + td.q_off;
  const int x = threadIdx.x & 31, y0 = threadIdx.x >> 5;
  for (int y = y0; y < 32; y += 8) {
    const int ra = 32 * bi + y, ca = 32 * bj + x, rb = 32 * bj + y, cb = 32 * bi + x;
    ta[y][x] = (ra < D && ca < D) ? q[(size_t)ra * DP + ca] : 0.f;
    tb[y][x] = (rb < D && cb < D) ? q[(size_t)rb * DP + cb] : 0.f;
  }
  __syncthreads();
  for (int y = y0; y < 32; y += 8) {
    const int ra = 32 * bi + y, ca = 32 * bj + x;
    if (ra < D && ca < D) {
      if (pl.kind != QPLANES_NONE) put_planes(pl, t, ra, ca, ta[y][x]);
      q[(size_t)ra * DP + ca] = tb[x][y];  // Q^T[ra][ca] = Q[ca][ra]
    }
    const int rb = 32 * bj + y, cb = 32 * bi + x;
    if (bi != bj && rb < D && cb < D) {
      if (pl.kind != QPLANES_NONE) put_planes(pl, t, rb, cb, tb[y][x]);
      q[(size_t)rb * DP + cb] = ta[x][y];
    }
  }
}

}  // namespace emt

int emt_prepare_rotations(const emt::TaskDev* tasks, int n_tasks, int max_dim, float* qt,
                          const emt::QPlanes& planes, void* stream) {
  if (n_tasks <= 0 || max_dim <= 0) return 0;
  const unsigned tiles = (unsigned)(max_dim + 31) / 32;
  emt::prepare_rotations_kernel<<<dim3((unsigned)n_tasks, tiles, tiles), 256, 0,
                                  (cudaStream_t)stream>>>(tasks, qt, planes);
  return (int)cudaGetLastError();
}

int emt_launch_best(const emt::BestArgs& a, void* stream) {
  if (a.n_tasks <= 0) return 0;
  emt::best_kernel<<<a.n_tasks, 32, 0, (cudaStream_t)stream>>>(a);
  return (int)cudaGetLastError();
}

int emt_launch_epoch(const emt::EpochArgs& a, int grid, void* stream, const void* tmap) {
  if (grid <= 0) return 0;
  static_assert(sizeof(emt::EpochArgs) < 2048, "kernel parameter block");
  cudaError_t e;
  if (tmap) {
    e = cudaFuncSetAttribute(emt::epoch_kernel_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)a.smem_bytes);
    if (e != cudaSuccess) return (int)e;
    emt::epoch_kernel_tc<<<grid, emt::kThreads, a.smem_bytes, (cudaStream_t)stream>>>(
        a, *reinterpret_cast<const CUtensorMap*>(tmap));
  } else {
    e = cudaFuncSetAttribute(emt::epoch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)a.smem_bytes);
    if (e != cudaSuccess) return (int)e;
    emt::epoch_kernel<<<grid, emt::kThreads, a.smem_bytes, (cudaStream_t)stream>>>(a);
  }
  return (int)cudaGetLastError();
}

// Epoch launch without touching the function's shared-memory attribute (the
// caller has raised it to cover a.smem_bytes); usable inside stream capture.
int emt_launch_epoch_noattr(const emt::EpochArgs& a, int grid, void* stream, const void* tmap) {
  if (grid <= 0) return 0;
  const cudaStream_t st = (cudaStream_t)stream;
  if (tmap) {
    const CUtensorMap& m = *reinterpret_cast<const CUtensorMap*>(tmap);
    if (a.queue)
      emt::epoch_kernel_tc_queue<<<grid, emt::kThreads, a.smem_bytes, st>>>(a, m);
    else
      emt::epoch_kernel_tc<<<grid, emt::kThreads, a.smem_bytes, st>>>(a, m);
  } else if (a.queue) {
    emt::epoch_kernel_queue<<<grid, emt::kThreads, a.smem_bytes, st>>>(a);
  } else {
    emt::epoch_kernel<<<grid, emt::kThreads, a.smem_bytes, st>>>(a);
  }
  return (int)cudaGetLastError();
}

// Raises the epoch kernel's dynamic shared-memory limit to bytes.
int emt_epoch_smem_attr(bool tc, size_t bytes) {
  const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e = tc ? cudaFuncSetAttribute(emt::epoch_kernel_tc, at, (int)bytes)
                     : cudaFuncSetAttribute(emt::epoch_kernel, at, (int)bytes);
  if (e == cudaSuccess)  // the persistent-queue twin of the same form
    e = tc ? cudaFuncSetAttribute(emt::epoch_kernel_tc_queue, at, (int)bytes)
           : cudaFuncSetAttribute(emt::epoch_kernel_queue, at, (int)bytes);
  return (int)e;
}

// Resident CTAs per SM of the epoch kernel with `bytes` of dynamic shared
// memory (0 if it cannot launch).
int emt_epoch_occupancy(bool tc, size_t bytes, bool queue) {
  int n = 0;
  if (emt_epoch_smem_attr(tc, bytes) != 0) return 0;
  cudaError_t e;
  if (queue)
    e = tc ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, emt::epoch_kernel_tc_queue, emt::kThreads, bytes)
           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, emt::epoch_kernel_queue, emt::kThreads, bytes);
  else
    e = tc ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, emt::epoch_kernel_tc, emt::kThreads, bytes)
           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, emt::epoch_kernel, emt::kThreads, bytes);
  return e == cudaSuccess ? n : 0;
}

int emt_launch_eval(const emt::EvalArgs& a, void* stream) {
  const int grid = (a.n + 63) / 64;
  if (grid <= 0) return 0;
  cudaError_t e = cudaFuncSetAttribute(emt::eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)a.smem_bytes);
  if (e != cudaSuccess) return (int)e;
  emt::eval_kernel<<<grid, emt::kThreads, a.smem_bytes, (cudaStream_t)stream>>>(a);
  return (int)cudaGetLastError();
}

#include "emt_large.cuh"
