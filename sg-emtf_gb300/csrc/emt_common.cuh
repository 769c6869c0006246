// emt_common.cuh -- arithmetic shared by the engine's host and device code:
// the Philox4x32-10 counter RNG and its stream layout, the deterministic
// FP32 power used by the GA operators, and small helpers.
//
// Everything here is written so that host and device produce identical bits:
// every intended fused multiply-add is an explicit fmaf()/__fmaf_rn, host code
// is compiled with -ffp-contract=off, and device code on the trial path uses
// explicitly rounded intrinsics (__fadd_rn, __fmul_rn, ...), which the
// compiler never contracts.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define EMT_HD __host__ __device__ __forceinline__
#else
#define EMT_HD inline
#endif

namespace emt {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Replaces the reference's per-thread cuRAND XORWOW
// states (SG-EMTF.cu:163-179), which were reseeded from time(0) and shared by
// every task mapped to the same stream (:1660,1676).
//
// Stream layout (all engine randomness):
//   key = (seed low 32 bits, seed high 32 bits)
//   ctr = (task, generation, member, purpose << 24 | block)
// ---------------------------------------------------------------------------
enum Purpose : uint32_t {
  P_POP_INIT = 1,         // gen 0, member i, block b -> genes 4b..4b+3
  P_SHIFT = 2,            // gen 0, member 0, block b -> dims 4b..4b+3
  P_QR_NORMAL = 3,        // gen 0, member = row, block b -> columns 4b..4b+3
  P_DE_INDEX = 4,         // gen g, member i, block 0 -> r1, r2, r3, jrand
  P_DE_CR = 5,            // gen g, member i, block b -> genes 4b..4b+3
  P_GA_PARENT = 6,        // gen g, member i, block 0 -> parent index
  P_GA_SBX = 7,           // gen g, member i, block b -> (rate, p) for genes 2b, 2b+1
  P_GA_PM = 8,            // gen g, member i, block b -> (r, u) for genes 2b, 2b+1
  P_TRANSFER_PARTNER = 9, // gen g, member 0, block 0 -> partner task
  P_TRANSFER_MIX = 10,    // gen g, member c, block b -> genes 4b..4b+3 of candidate c
  // CVRP engine (emt_cvrp.cu): node data, Fisher-Yates words, tournaments,
  // order-crossover cuts, mutation draws, transfer partner (purposes 16..21)
};

struct U4 {
  uint32_t x, y, z, w;
};

EMT_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

EMT_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
  }
  return c;
}

EMT_HD U4 draw(uint64_t seed, uint32_t task, uint32_t gen, uint32_t member, uint32_t purpose,
               uint32_t block) {
  U4 c{task, gen, member, (purpose << 24) | (block & 0xFFFFFFu)};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// 24 random bits -> [0, 1), exact in FP32.
EMT_HD float u01(uint32_t w) { return (float)(w >> 8) * 0x1p-24f; }

EMT_HD uint32_t word(const U4& v, int q) {
  return q == 0 ? v.x : (q == 1 ? v.y : (q == 2 ? v.z : v.w));
}

// ---------------------------------------------------------------------------
// explicit-rounding FP32 arithmetic (never contracted into an FMA)
// ---------------------------------------------------------------------------
EMT_HD float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;
  return r;
#endif
}
EMT_HD float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
EMT_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
EMT_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  volatile float r = a / b;
  return r;
#endif
}
EMT_HD float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}
EMT_HD float frint(float a) {
#if defined(__CUDA_ARCH__)
  return rintf(a);
#else
  return __builtin_rintf(a);
#endif
}

EMT_HD float clamp_box(float v, float lo, float hi) {
  if (v > hi) return hi;
  if (v < lo) return lo;
  return v;
}

EMT_HD float bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  union {
    uint32_t u;
    float f;
  } b;
  b.u = u;
  return b.f;
#endif
}
EMT_HD uint32_t float_to_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  union {
    float f;
    uint32_t u;
  } b;
  b.f = f;
  return b.u;
#endif
}

// x^y for x >= 0 as exp2(y log2 x), built only from correctly rounded FP32
// +, -, *, / and fma so that host and device agree bit for bit.
//   log2 m = (2 / ln 2) atanh(s), s = (m - 1)/(m + 1), m in [sqrt(1/2), sqrt(2)):
//            odd Taylor series of atanh to s^9 (|s| < 0.172, truncation < 4e-10)
//   2^f    = e^(f ln 2), f in [-1/2, 1/2]: Taylor series to degree 7 (< 6e-9)
// Replaces CUDA powf in SBX and polynomial mutation (SG-EMTF.cu:590,728).
EMT_HD float det_powf(float x, float y) {
  if (!(x > 0x1p-100f)) return 0.f;
  uint32_t b = float_to_bits(x);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  float m = bits_to_float((b & 0x7FFFFFu) | 0x3F800000u);
  if (m > 1.41421354f) {
    m = fmul(m, 0.5f);
    e += 1;
  }
  float s = fdiv(fsub(m, 1.f), fadd(m, 1.f));
  float s2 = fmul(s, s);
  float p = ffma(s2, 0x1.c71c72p-4f, 0x1.24924ap-3f);
  p = ffma(s2, p, 0x1.99999ap-3f);
  p = ffma(s2, p, 0x1.555556p-2f);
  p = ffma(s2, p, 1.f);
  float lm = fmul(fmul(s, p), 0x1.715476p+1f);
  float L = fadd((float)e, lm);
  float t = fmul(y, L);
  if (t > 126.f) t = 126.f;
  if (t < -126.f) return 0.f;
  float n = frint(t);
  float f = fsub(t, n);
  float g = fmul(f, 0x1.62e430p-1f);
  float q = ffma(g, 0x1.a01a02p-13f, 0x1.6c16c2p-10f);
  q = ffma(g, q, 0x1.111112p-7f);
  q = ffma(g, q, 0x1.555556p-5f);
  q = ffma(g, q, 0x1.555556p-3f);
  q = ffma(g, q, 0.5f);
  q = ffma(g, q, 1.f);
  q = ffma(g, q, 1.f);
  return fmul(q, bits_to_float((uint32_t)((int)n + 127) << 23));
}

// Three distinct indices in [0, NP) \ {i} and a dimension in [0, D), drawn
// without rejection: r <- w mod (N - |S|), then r += 1 for every excluded
// value s (ascending) with r >= s.  Requires NP >= 4.
EMT_HD void de_indices(const U4& w, int i, int NP, int D, int& r1, int& r2, int& r3, int& jr) {
  r1 = (int)(w.x % (uint32_t)(NP - 1));
  if (r1 >= i) r1++;
  int a = i < r1 ? i : r1, b = i < r1 ? r1 : i;
  r2 = (int)(w.y % (uint32_t)(NP - 2));
  if (r2 >= a) r2++;
  if (r2 >= b) r2++;
  int s0 = i, s1 = r1, s2 = r2, t;
  if (s0 > s1) { t = s0; s0 = s1; s1 = t; }
  if (s1 > s2) { t = s1; s1 = s2; s2 = t; }
  if (s0 > s1) { t = s0; s0 = s1; s1 = t; }
  r3 = (int)(w.z % (uint32_t)(NP - 3));
  if (r3 >= s0) r3++;
  if (r3 >= s1) r3++;
  if (r3 >= s2) r3++;
  jr = (int)(w.w % (uint32_t)D);
}

}  // namespace emt
