// emt_functions.cuh -- the seven benchmark functions on the device.
//
// FP32 form (every evaluation): one warp per individual, lanes over genes,
// butterfly reductions (a fixed order, so results repeat run to run).  Besides
// f it returns the "scale", the sum of absolute sub-terms, which bounds the
// rounding error of f and sets the FP64 re-check window.
//
// FP64-class form (re-check of near-tie selections): the rotation by a
// compensated double-FP32 dot product (precise_rotation); then tier 2, FP32
// terms with a per-row error bound, and only if that cannot decide, tier 3,
// the terms in double precision.  Weierstrass reduces each argument exactly
// (eval_weier_precise).
//
// Definitions follow the reference's evaluation() (proposed model/
// SG-EMTF.cu:898-1111): Sphere :918, Rosenbrock :939, Ackley :963 (E =
// 2.718282 in reference mode), Rastrigin :991, Griewank :1014 (product as in
// SG-EMTF_DE.cu:989; EMT_FLAG_REF_GRIEWANK_NO_PRODUCT drops it as the GA file
// does), Weierstrass :1049 (a = 0.5, b = 3, k = 0..20), Schwefel :1079.
#pragma once

#include "emt_internal.h"

namespace emt {

enum Fid : int {
  F_SPHERE = 0,
  F_RASTRIGIN = 1,
  F_ACKLEY = 2,
  F_GRIEWANK = 3,
  F_ROSENBROCK = 4,
  F_SCHWEFEL = 5,
  F_WEIERSTRASS = 6
};

constexpr uint32_t FLAG_REF_GRIEWANK_NO_PRODUCT = 0x1u;
constexpr uint32_t FLAG_REF_WEIERSTRASS_CONST = 0x2u;
constexpr uint32_t FLAG_REF_ACKLEY_E = 0x4u;
constexpr uint32_t FLAG_REF_BOXES = 0x8u;
constexpr uint32_t FLAG_NO_RECHECK = 0x10u;
constexpr uint32_t FLAG_RIGOROUS_WINDOW = 0x20u;
// Test switch of the tensor-core form: the rotation issues no MMA and no
// commit, so the first bounded wait on the MMA barrier runs out with nothing
// in flight; the kernel reports CHECK_TIMEOUT and stops the epoch.
constexpr uint32_t FLAG_TEST_LOST_COMPLETION = 0x80u;

// Weierstrass terms k = 0..20 of one gene: sum of 0.5^k cos(2 pi 3^k (z + 1/2)).
// cos(2 pi 3^k (z + 1/2)) = -cos(pi y_k) with y_k = 2 * 3^k * |z| (3^k is odd).
// Anchors k = 0, 5, 10, 15 reduce y_k mod 2 exactly from the FP32 significand
// of z (r_k = M 3^k mod 2^(sh+1), unsigned wrap-around arithmetic) and take
// cospif; the other terms follow the angle-tripling identity
// cos(3t) = cos t (4 cos^2 t - 3), whose error grows 3x per step but at most
// 4 steps from an anchor and weighted 0.5^k: below 14 anchor errors per gene.
__device__ __forceinline__ float weier_gene_f32(float z) {
  const float az = fabsf(z);
  const uint32_t bits = __float_as_uint(az);
  const uint32_t E = bits >> 23;
  const uint32_t M = (bits & 0x7FFFFFu) | 0x800000u;
  const int sh = 149 - (int)E;  // y_0 = M / 2^sh for normal az
  float y[4];
  if (E == 0u || sh > 61) {  // |z| < 2^-37: y_k is tiny, plain FP32 is exact enough
    y[0] = 2.f * az;
    y[1] = 486.f * az;
    y[2] = 118098.f * az;
    y[3] = 28697814.f * az;
  } else if (sh <= 0) {  // |z| >= 2^22: y_k integer, parity of M 3^k = parity of M (sh = 0)
    const float p = (sh == 0 && (M & 1u)) ? 1.f : 0.f;
    y[0] = y[1] = y[2] = y[3] = p;
  } else if (sh <= 31) {
    const uint32_t mask = (2u << sh) - 1u;
    const float scale = __uint_as_float((uint32_t)(127 - sh) << 23);
    uint32_t r = M & mask;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      y[a] = (float)r * scale;
      r = (r * 243u) & mask;  // 3^5
    }
  } else {
    const unsigned long long mask = (2ull << sh) - 1ull;
    const float scale = __uint_as_float((uint32_t)(127 - sh) << 23);
    unsigned long long r = M;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      y[a] = (float)r * scale;
      r = (r * 243ull) & mask;
    }
  }
  // k = 0 anchor, then k = 1..20 with anchors at k = 5, 10, 15
  float c = cospif(y[0]);
  float s = -c, ak = 1.f;
#pragma unroll
  for (int k = 1; k <= 20; ++k) {
    ak *= 0.5f;
    if (k == 5 || k == 10 || k == 15)
      c = cospif(y[k / 5]);
    else
      c = c * fmaf(4.f * c, c, -3.f);
    s = fmaf(-ak, c, s);
  }
  return s;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, m);
  return v;
}
__device__ __forceinline__ float warp_prod(float v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v *= __shfl_xor_sync(0xFFFFFFFFu, v, m);
  return v;
}
__device__ __forceinline__ double warp_sum64(double v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, m);
  return v;
}
__device__ __forceinline__ double warp_prod64(double v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v *= __shfl_xor_sync(0xFFFFFFFFu, v, m);
  return v;
}

// Reduction teams for the FP64-class evaluations: a warp (lanes over genes,
// as the fused kernel runs them) or a whole CTA (the large-island decisions,
// where one warp alone would set the launch length on the FP64 pipe).  With
// WarpTeam the evaluations below run exactly the warp operations.
struct WarpTeam {
  __device__ __forceinline__ int rank() const { return threadIdx.x & 31; }
  __device__ __forceinline__ int size() const { return 32; }
  __device__ __forceinline__ double sum(double v) const { return warp_sum64(v); }
  __device__ __forceinline__ double prod(double v) const { return warp_prod64(v); }
  __device__ __forceinline__ int any(int p) const { return __any_sync(0xFFFFFFFFu, p); }
};
struct CtaTeam {
  double* scratch;  // shared memory, one double per warp of the CTA
  __device__ __forceinline__ int rank() const { return threadIdx.x; }
  __device__ __forceinline__ int size() const { return blockDim.x; }
  // warp partials combined in warp order, the same value in every thread
  __device__ __forceinline__ double sum(double v) const {
    v = warp_sum64(v);
    if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += scratch[w];
    __syncthreads();
    return r;
  }
  __device__ __forceinline__ double prod(double v) const {
    v = warp_prod64(v);
    if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 1.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r *= scratch[w];
    __syncthreads();
    return r;
  }
  __device__ __forceinline__ int any(int p) const { return __syncthreads_or(p); }
};

// Bound on the Weierstrass error caused by rounding of the rotation, per
// member: |dz_j| <= (gamma_{D+1} + 2^-20) * |q_j|_2 * |x - o|_2 (Cauchy-Schwarz
// on the worst-case FP32 dot-product bound, plus the TF32 split error), pushed
// through every term and capped by the term's range.
__device__ __forceinline__ float weier_rotation_bound(int D, float qnorm, float snorm) {
  const float u = 0x1p-24f;
  const float g = (float)(D + 1) * u / (1.f - (float)(D + 1) * u) + 0x1p-20f;
  const float dz = g * qnorm * snorm + u * snorm;
  float b = 0.f, ak = 1.f, e = 6.2831855f * dz;
#pragma unroll
  for (int k = 0; k <= 20; ++k) {
    b = fmaf(ak, fminf(e, 2.f), b);
    ak *= 0.5f;
    e *= 3.f;
  }
  return (float)D * (b + 4e-6f);
}

struct FnConst {
  int fid, D;
  uint32_t flags;
  float woff, qnorm, rel;
  double woff64;
};

// FP32 fitness of rows [0, nrows) of Z (rotated, shared memory, stride DP),
// evaluated by the whole CTA: tpr consecutive threads share a row (4 rows
// per warp-octet for nrows <= 64), each summing a contiguous chunk of genes,
// then a tpr-lane butterfly.  x rows (unrotated) and o give x - o for the
// Weierstrass rounding bound.  fout/tout receive f and the half-width of the
// near-tie window, rel * scale, where scale is the sum of absolute
// sub-terms of f and rel the stated accuracy of the FP32 form (1e-5; the
// parity tests check |f - f64| <= 1e-5 scale).  Weierstrass, whose terms
// amplify the rotation's rounding by 3^k, gets 5 x rel * scale (five times
// the largest error measured on the FP32 form; the parity tests check it),
// or with EMT_FLAG_RIGOROUS_WINDOW the rigorous conditioning bound
// (weier_rotation_bound), which sends most late-run selections to the
// re-check.  Weierstrass term magnitudes are bounded by 2 per gene.  Near an optimum the forms
// below avoid cancellation: Ackley uses expm1 of sum z^2 and of sum
// sin^2(pi z), Griewank 1 - prod cos = -expm1(sum log1p(-2 sin^2(theta/2))),
// Rastrigin z^2 + 20 sin^2(pi z).
template <int kBlock>
__device__ void eval_rows_f32(const FnConst& fc, const float* __restrict__ Z,
                              const float* __restrict__ rows, const float* __restrict__ o,
                              int nrows, int DP, float* __restrict__ fout,
                              float* __restrict__ tout) {
  const int D = fc.D;
  const int tpr = nrows <= kBlock / 4 ? 4 : (nrows <= kBlock / 2 ? 2 : 1);
  const int per_pass = kBlock / tpr;
  const int sub = threadIdx.x & (tpr - 1);
  const int chunk = (D + tpr - 1) / tpr;
  const int j0 = sub * chunk, j1 = min(D, j0 + chunk);
  const bool griewank_prod = !(fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT);
  for (int base = 0; base < nrows; base += per_pass) {
    const int row = base + (int)threadIdx.x / tpr;
    float a = 0.f, b = 0.f, c = 1.f, sa = 0.f, ss = 0.f;
    int neg = 0;
    if (row < nrows) {
      const float* z = Z + row * DP;
      switch (fc.fid) {
        case F_SPHERE:
          for (int j = j0; j < j1; ++j) a = fmaf(z[j], z[j], a);
          sa = a;
          break;
        case F_RASTRIGIN:
          for (int j = j0; j < j1; ++j) {
            const float v = z[j], sp = sinpif(v);
            a += fmaf(20.f * sp, sp, v * v);
          }
          sa = a;
          break;
        case F_ACKLEY:
          for (int j = j0; j < j1; ++j) {
            const float v = z[j], sp = sinpif(v);
            a = fmaf(v, v, a);
            b = fmaf(sp, sp, b);  // sum sin^2(pi z)
          }
          break;
        case F_GRIEWANK:
          for (int j = j0; j < j1; ++j) {
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
          for (int j = j0; j < j1 && j + 1 < D; ++j) {
            const float v = z[j], n = z[j + 1];
            const float t1 = fmaf(v, v, -n), t2 = v - 1.f;
            const float t = fmaf(100.f * t1, t1, t2 * t2);
            a += t;
            sa += t + 200.f * fabsf(t1) * fmaf(v, v, fabsf(n)) + 2.f * fabsf(t2) * (fabsf(v) + 1.f);
          }
          break;
        case F_SCHWEFEL:
          for (int j = j0; j < j1; ++j) {
            const float v = z[j], t = v * sinf(sqrtf(fabsf(v)));
            a += t;
            sa += fabsf(t);
          }
          break;
        case F_WEIERSTRASS: {
          const float* x = rows + row * DP;
          for (int j = j0; j < j1; ++j) {
            a += weier_gene_f32(z[j]);
            const float d = x[j] - o[j];
            ss = fmaf(d, d, ss);
          }
          break;
        }
        default:
          break;
      }
    }
    for (int m = 1; m < tpr; m <<= 1) {
      a += __shfl_xor_sync(0xFFFFFFFFu, a, m);
      b += __shfl_xor_sync(0xFFFFFFFFu, b, m);
      c *= __shfl_xor_sync(0xFFFFFFFFu, c, m);
      sa += __shfl_xor_sync(0xFFFFFFFFu, sa, m);
      ss += __shfl_xor_sync(0xFFFFFFFFu, ss, m);
      neg |= __shfl_xor_sync(0xFFFFFFFFu, neg, m);
    }
    if (row < nrows && sub == 0) {
      float f, scale;
      switch (fc.fid) {
        case F_ACKLEY: {
          const float e = 2.71828183f;
          const float eref = (fc.flags & FLAG_REF_ACKLEY_E) ? 2.718282f - e : 0.f;
          const float t1 = -20.f * expm1f(-0.2f * sqrtf(a / (float)D));  // 20 - 20 exp(-0.2 r)
          const float t2 = -e * expm1f(-2.f * b / (float)D);            // e - exp(B / D)
          f = t1 + t2 + eref;
          scale = t1 + t2 + fabsf(eref);
          break;
        }
        case F_GRIEWANK: {
          const float om = !griewank_prod ? 0.f : (neg ? 1.f - c : -expm1f(b));  // 1 - prod cos
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
        default:  // sphere, rastrigin, rosenbrock: non-negative sums
          f = a;
          scale = sa;
          break;
      }
      float t = fc.rel * scale;
      if (fc.fid == F_WEIERSTRASS)
        t = (fc.flags & FLAG_RIGOROUS_WINDOW) ? t + weier_rotation_bound(D, fc.qnorm, sqrtf(ss))
                                              : 5.f * t;
      fout[row] = f;
      tout[row] = t;
    }
  }
}

// s + e = a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// One Weierstrass gene from a high-precision argument z (double holding a
// double-FP32 value): y_k = 2 * 3^k * |z| mod 2 is reduced exactly on the
// 53-bit significand (r <- 3 r mod 2^(sh+1)), then cos(pi y_k) in FP32
// (the reduced argument carries 24 bits, so each term is good to ~2^-23);
// the 21 terms are summed with Kahan compensation.
__device__ __forceinline__ float weier_gene_precise(double z) {
  // |z| = M 2^-sh with M the 53-bit significand; y_k = 2 3^k |z| mod 2 is
  // reduced exactly in integers (64-bit for sh < 64, 128-bit up to sh = 127)
  // and rounded once to FP32 for cospif.  No FP64 arithmetic.
  const unsigned long long b =
      (unsigned long long)__double_as_longlong(z) & 0x7FFFFFFFFFFFFFFFull;
  const int E = (int)(b >> 52);
  const unsigned long long M = (b & ((1ull << 52) - 1ull)) | (1ull << 52);
  const int sh = 1074 - E;  // y_0 = M / 2^sh for normal |z|
  float s = 0.f, comp = 0.f, ak = 1.f;
  auto add = [&](float c) {
    const float v = __fsub_rn(__fmul_rn(-ak, c), comp);
    const float t = __fadd_rn(s, v);
    comp = __fsub_rn(__fsub_rn(t, s), v);
    s = t;
    ak *= 0.5f;
  };
  if (b == 0ull || E == 0 || sh > 127) {
    // |z| < 2^-75: every 2 3^k |z| < 2^-41 and cospif rounds to 1
    for (int k = 0; k <= 20; ++k) add(1.f);
  } else if (sh <= 0) {
    const float c = (sh == 0 && (M & 1ull)) ? -1.f : 1.f;
    for (int k = 0; k <= 20; ++k) add(c);
  } else if (sh < 64) {
    const unsigned long long mask = (2ull << sh) - 1ull;
    unsigned long long r = M & mask;
    const int drop = sh > 24 ? sh - 24 : 0;
    const float scale = __uint_as_float((uint32_t)(127 - (sh - drop)) << 23);
    for (int k = 0; k <= 20; ++k) {
      // r >> drop < 2^25: a 32-bit conversion rounds it exactly as a 64-bit
      // one would, and stays off the FP64 pipe
      add(cospif(__uint2float_rn((uint32_t)(r >> drop)) * scale));
      r = (r * 3ull) & mask;
    }
  } else {
    // 64 <= sh <= 127: r = (r1 : r0) < 2^(sh+1) <= 2^128, drop = sh - 24 >= 40
    unsigned long long r0 = M, r1 = 0ull;
    const unsigned long long mask1 = sh >= 127 ? ~0ull : ((2ull << (sh - 64)) - 1ull);
    const int drop = sh - 24;
    const float scale = __uint_as_float((uint32_t)(127 - 24) << 23);
    for (int k = 0; k <= 20; ++k) {
      const unsigned long long top =
          drop >= 64 ? (r1 >> (drop - 64)) : ((r0 >> drop) | (r1 << (64 - drop)));
      add(cospif(__uint2float_rn((uint32_t)top) * scale));
      // r <- 3 r mod 2^(sh+1)
      const unsigned long long lo = r0 * 3ull;
      const unsigned long long carry = __umul64hi(r0, 3ull);
      r1 = (r1 * 3ull + carry) & mask1;
      r0 = lo;
    }
  }
  return s;
}

// Two outputs z_n, z_m (m = n + 32, or none) of sum_k q_nk (x_k - o_k) to
// FP64-class accuracy on the FP32 pipe: the compensated dot product of Ogita,
// Rump and Oishi ("Dot2", SIAM J. Sci. Comput. 26, 2005) over the exact split
// x_k - o_k = sh_k + sl_k, so |z - z_exact| <~ u |z| + gamma_D^2 sum |q||x - o|.
// The two chains are interleaved for instruction-level parallelism.  This
// GPU's FP64 pipe runs at ~1/45 of its FP32 rate, so ~12 FP32 operations per
// product beat one FP64 FMA.
__device__ __forceinline__ void dot2_pair(const float* __restrict__ x, const float* __restrict__ o,
                                          const float* __restrict__ qt, int DP, int D, int n,
                                          bool two, double& zn, double& zm) {
  float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
  const int m = two ? n + 32 : n;
  for (int k = 0; k < D; ++k) {
    float sh, sl;
    two_sum(x[k], -o[k], sh, sl);
    const float q0 = qt[k * DP + n], q1 = qt[k * DP + m];
    const float p0 = __fmul_rn(q0, sh), p1 = __fmul_rn(q1, sh);
    const float e0 = __fmaf_rn(q0, sh, -p0), e1 = __fmaf_rn(q1, sh, -p1);
    float t0, te0, t1, te1;
    two_sum(S0, p0, t0, te0);
    two_sum(S1, p1, t1, te1);
    S0 = t0;
    S1 = t1;
    C0 = __fmaf_rn(q0, sl, __fadd_rn(C0, __fadd_rn(te0, e0)));
    C1 = __fmaf_rn(q1, sl, __fadd_rn(C1, __fadd_rn(te1, e1)));
  }
  zn = (double)S0 + (double)C0;
  zm = (double)S1 + (double)C1;
}

// The calling team fills zbuf[0..D) with the FP64-class rotation of row x,
// one output per member of the team at a time (the team synchronises before
// returning).
// Outputs n + i st (i < 4) of the same compensated rotation, their four Dot2
// chains interleaved for instruction-level parallelism; each keeps
// dot2_pair's operations and order over k, so the values are the same.
// Outputs at or beyond D repeat output n and are not stored.
__device__ __forceinline__ void dot2_quad(const float* __restrict__ x, const float* __restrict__ o,
                                          const float* __restrict__ qt, int DP, int D, int n,
                                          int st, double* zbuf) {
  int m[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) m[i] = n + i * st < D ? n + i * st : n;
  float S[4] = {0.f, 0.f, 0.f, 0.f}, C[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k = 0; k < D; ++k) {
    float sh, sl;
    two_sum(x[k], -o[k], sh, sl);
    const float* qk = qt + (size_t)k * DP;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float q = qk[m[i]];
      const float p = __fmul_rn(q, sh);
      const float e = __fmaf_rn(q, sh, -p);
      float t, te;
      two_sum(S[i], p, t, te);
      S[i] = t;
      C[i] = __fmaf_rn(q, sl, __fadd_rn(C[i], __fadd_rn(te, e)));
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (n + i * st < D) zbuf[n + i * st] = (double)S[i] + (double)C[i];
}

template <class Team>
__device__ void precise_rotation_team(const float* __restrict__ x, const float* __restrict__ o,
                                      const float* __restrict__ qt, int DP, int D, double* zbuf,
                                      const Team& tm) {
  const int st = tm.size();
  for (int n = tm.rank(); n < D; n += 4 * st) dot2_quad(x, o, qt, DP, D, n, st, zbuf);
  tm.sum(0.0);  // a barrier of the team
}

// The calling warp fills zbuf[0..D) with the FP64-class rotation of row x.
__device__ __forceinline__ void precise_rotation(const float* __restrict__ x,
                                                 const float* __restrict__ o,
                                                 const float* __restrict__ qt, int DP, int D,
                                                 double* zbuf) {
  const int lane = threadIdx.x & 31;
  for (int n = lane; n < D; n += 64) {
    double a, b;
    const bool two = n + 32 < D;
    dot2_pair(x, o, qt, DP, D, n, two, a, b);
    zbuf[n] = a;
    if (two) zbuf[n + 32] = b;
  }
  __syncwarp();
}

// sin(pi v) and cos(v) for |pi v|, |v| < 2^-10 by Taylor series (error below
// 1e-25); the double-precision library calls cost ~10 SM-clocks each here.
__device__ __forceinline__ double sinpi_small(double v) {
  const double x = 3.141592653589793 * v, x2 = x * x;
  return x * fma(x2, fma(x2, 1.0 / 120.0, -1.0 / 6.0), 1.0);
}
__device__ __forceinline__ double cos_small(double t) {
  const double t2 = t * t;
  return fma(t2, fma(t2, fma(t2, -1.0 / 720.0, 1.0 / 24.0), -0.5), 1.0);
}
// 1/sqrt(v) and sqrt(v) for v > 0 in double: FP32 estimate, two Newton steps.
__device__ __forceinline__ double rsqrt_d(double v) {
  double r = (double)rsqrtf((float)v);
  r = r * fma(-0.5 * v * r, r, 1.5);
  r = r * fma(-0.5 * v * r, r, 1.5);
  return r;
}

// Tier 3: f in double precision from the FP64-class rotation zbuf, by the
// calling team.
template <class Team>
__device__ double eval_tier3_t(const FnConst& fc, const double* zbuf, const Team& tm) {
  const int r0 = tm.rank(), st = tm.size();
  const int D = fc.D;
  double a = 0.0, b = 0.0, c = 1.0;
  switch (fc.fid) {
    case F_SPHERE:
      for (int j = r0; j < D; j += st) a = fma(zbuf[j], zbuf[j], a);
      break;
    case F_RASTRIGIN:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        const double sp = fabs(v) < 0x1p-12 ? sinpi_small(v) : sinpi(v);
        a += fma(20.0 * sp, sp, v * v);
      }
      break;
    case F_ACKLEY:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        const double sp = fabs(v) < 0x1p-12 ? sinpi_small(v) : sinpi(v);
        a = fma(v, v, a);
        b = fma(sp, sp, b);
      }
      break;
    case F_GRIEWANK:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        a = fma(v, v, a);
        if (!(fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT)) {
          const double th = v * rsqrt_d((double)(j + 1));
          c *= fabs(th) < 0x1p-10 ? cos_small(th) : cos(th);
        }
      }
      break;
    case F_ROSENBROCK:
      for (int j = r0; j + 1 < D; j += st) {
        const double v = zbuf[j], n = zbuf[j + 1];
        const double t1 = v * v - n, t2 = v - 1.0;
        a += 100.0 * t1 * t1 + t2 * t2;
      }
      break;
    case F_SCHWEFEL:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j], av = fabs(v);
        if (av > 0.0) a += v * sin(av * rsqrt_d(av));
      }
      break;
    default:
      break;
  }
  a = tm.sum(a);
  double f;
  switch (fc.fid) {
    case F_ACKLEY: {
      b = tm.sum(b);
      const double e = 2.718281828459045;
      const double eref = (fc.flags & FLAG_REF_ACKLEY_E) ? 2.718282 - e : 0.0;
      f = -20.0 * expm1(-0.2 * sqrt(a / D)) - e * expm1(-2.0 * b / D) + eref;
      break;
    }
    case F_GRIEWANK:
      c = tm.prod(c);
      f = (1.0 - c) + a / 4000.0;
      break;
    case F_SCHWEFEL:
      f = 418.9829 * D - a;
      break;
    default:
      f = a;
      break;
  }
  return f;
}
__device__ __noinline__ double eval_tier3(const FnConst& fc, const double* zbuf) {
  return eval_tier3_t(fc, zbuf, WarpTeam{});
}

// Tier 2: f from the FP64-class rotation zbuf with FP32 function terms on the
// rounded z, summed in double, and *err, a first-order bound on |f - f(z)|:
// per gene |g'(z)| |z - fl(z)| + 8u (|g| + |sub-terms|).  Sphere and
// Rosenbrock need no transcendental and go straight to tier 3.
template <class Team>
__device__ double eval_tier2_t(const FnConst& fc, const double* zbuf, double* err, const Team& tm) {
  const int r0 = tm.rank(), st = tm.size();
  const int D = fc.D;
  const double u = 0x1p-24;
  double a = 0.0, b = 0.0, e = 0.0, eb = 0.0, lg = 0.0, c = 1.0;
  int neg = 0;
  switch (fc.fid) {
    case F_RASTRIGIN:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        const float zf = (float)v;
        const double dz = fabs(v - (double)zf);
        const float sp = sinpif(zf), cp = cospif(zf);
        const double g = (double)zf * zf + 20.0 * (double)sp * sp;
        a += g;
        e += fabs(2.0 * zf + 125.66370614359172 * sp * cp) * dz + 8.0 * u * g;
      }
      break;
    case F_ACKLEY:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        const float zf = (float)v;
        const double dz = fabs(v - (double)zf);
        const float sp = sinpif(zf), cp = cospif(zf);
        a = fma(v, v, a);
        b += (double)sp * sp;
        eb += 6.283185307179586 * fabs(sp * cp) * dz + 4.0 * u * (double)sp * sp;
      }
      break;
    case F_GRIEWANK:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        a = fma(v, v, a);
        if (!(fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT)) {
          const double th = v * rsqrt_d((double)(j + 1));
          const float tf = (float)th;
          const double dt = fabs(th - (double)tf);
          const float ct = cosf(tf), st = sinf(tf);
          c *= (double)ct;
          if (ct > 0.f) {
            const float sh = sinf(0.5f * tf);
            lg += (double)log1pf(-2.f * sh * sh);
            eb += fabs((double)st / (double)ct) * dt + 8.0 * u;
          } else {
            neg = 1;
            eb += 1.0;  // no relative bound through a non-positive cosine
          }
        }
      }
      break;
    case F_SCHWEFEL:
      for (int j = r0; j < D; j += st) {
        const double v = zbuf[j];
        const float zf = (float)v;
        const double dz = fabs(v - (double)zf);
        const float r = sqrtf(fabsf(zf)), sr = sinf(r), cr = cosf(r);
        const double g = (double)zf * sr;
        a += g;
        e += fabs((double)sr + 0.5 * r * cr) * dz + 8.0 * u * fabs((double)zf) * (1.0 + r);
      }
      break;
    default:
      break;
  }
  a = tm.sum(a);
  e = tm.sum(e);
  double f;
  switch (fc.fid) {
    case F_ACKLEY: {
      b = tm.sum(b);
      eb = tm.sum(eb);
      const double ee = 2.718281828459045;
      const double eref = (fc.flags & FLAG_REF_ACKLEY_E) ? 2.718282 - ee : 0.0;
      const double x2 = exp(-2.0 * b / D);
      f = -20.0 * expm1(-0.2 * sqrt(a / D)) - ee * expm1(-2.0 * b / D) + eref;
      e = ee * x2 * (2.0 / D) * eb + 1e-15 * fabs(f);
      break;
    }
    case F_GRIEWANK: {
      double om;
      if (fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT) {
        om = 0.0;
        e = 0.0;
      } else {
        c = tm.prod(c);
        lg = tm.sum(lg);
        eb = tm.sum(eb);
        neg = tm.any(neg);
        om = neg ? 1.0 - c : -expm1(lg);
        e = neg ? 1e300 : fabs(c) * eb;  // a sign change: leave it to tier 3
      }
      f = om + a / 4000.0;
      break;
    }
    case F_SCHWEFEL:
      f = 418.9829 * D - a;
      break;
    default:
      f = a;
      break;
  }
  *err = 2.0 * e;  // safety factor on the first-order bound
  return f;
}
__device__ __noinline__ double eval_tier2(const FnConst& fc, const double* zbuf, double* err) {
  return eval_tier2_t(fc, zbuf, err, WarpTeam{});
}

// |f32 - f64| / scale of one member, as BestArgs::best_err defines it: the
// scale the FP32 evaluation stated, tol / rel (Weierstrass: 2D + |offset|).
__device__ __forceinline__ float best_rel_err(const TaskDev& td, float f32, double f64, float tol,
                                              float rel) {
  const double scale = td.fid == F_WEIERSTRASS ? 2.0 * td.D + fabs((double)td.woff)
                                               : (double)tol / (double)rel;
  return scale > 0.0 ? (float)(fabs((double)f32 - f64) / scale) : 0.f;
}

// Weierstrass from the FP64-class rotation: exactly reduced terms (FP32/INT).
template <class Team>
__device__ double eval_weier_precise_t(const FnConst& fc, const double* zbuf, const Team& tm) {
  double acc = 0.0;
  for (int n = tm.rank(); n < fc.D; n += tm.size()) acc += (double)weier_gene_precise(zbuf[n]);
  acc = tm.sum(acc);
  return acc + fc.woff64;
}
__device__ __noinline__ double eval_weier_precise(const FnConst& fc, const double* zbuf) {
  return eval_weier_precise_t(fc, zbuf, WarpTeam{});
}

// weier_gene_precise of two genes, the two reductions and compensated sums
// interleaved when both arguments take the 64-bit path (the usual case);
// every operation of each gene is weier_gene_precise's.
__device__ __forceinline__ void weier_gene_precise2(double z0, double z1, float& g0, float& g1) {
  const unsigned long long b0 = (unsigned long long)__double_as_longlong(z0) & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long b1 = (unsigned long long)__double_as_longlong(z1) & 0x7FFFFFFFFFFFFFFFull;
  const int E0 = (int)(b0 >> 52), E1 = (int)(b1 >> 52);
  const int sh0 = 1074 - E0, sh1 = 1074 - E1;
  if (b0 == 0ull || E0 == 0 || sh0 <= 0 || sh0 >= 64 || b1 == 0ull || E1 == 0 || sh1 <= 0 ||
      sh1 >= 64) {
    g0 = weier_gene_precise(z0);
    g1 = weier_gene_precise(z1);
    return;
  }
  const unsigned long long mask0 = (2ull << sh0) - 1ull, mask1 = (2ull << sh1) - 1ull;
  unsigned long long r0 = ((b0 & ((1ull << 52) - 1ull)) | (1ull << 52)) & mask0;
  unsigned long long r1 = ((b1 & ((1ull << 52) - 1ull)) | (1ull << 52)) & mask1;
  const int drop0 = sh0 > 24 ? sh0 - 24 : 0, drop1 = sh1 > 24 ? sh1 - 24 : 0;
  const float scale0 = __uint_as_float((uint32_t)(127 - (sh0 - drop0)) << 23);
  const float scale1 = __uint_as_float((uint32_t)(127 - (sh1 - drop1)) << 23);
  float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f, ak = 1.f;
  for (int k = 0; k <= 20; ++k) {
    const float u0 = cospif(__uint2float_rn((uint32_t)(r0 >> drop0)) * scale0);
    const float u1 = cospif(__uint2float_rn((uint32_t)(r1 >> drop1)) * scale1);
    const float v0 = __fsub_rn(__fmul_rn(-ak, u0), c0);
    const float v1 = __fsub_rn(__fmul_rn(-ak, u1), c1);
    const float t0 = __fadd_rn(s0, v0), t1 = __fadd_rn(s1, v1);
    c0 = __fsub_rn(__fsub_rn(t0, s0), v0);
    c1 = __fsub_rn(__fsub_rn(t1, s1), v1);
    s0 = t0;
    s1 = t1;
    ak *= 0.5f;
    r0 = (r0 * 3ull) & mask0;
    r1 = (r1 * 3ull) & mask1;
  }
  g0 = s0;
  g1 = s1;
}

// eval_weier_precise_t with two genes per step of each team member, summed
// in the same order (the same value).
template <class Team>
__device__ double eval_weier_precise_pair_t(const FnConst& fc, const double* zbuf, const Team& tm) {
  const int st = tm.size();
  double acc = 0.0;
  int n = tm.rank();
  for (; n + st < fc.D; n += 2 * st) {
    float g0, g1;
    weier_gene_precise2(zbuf[n], zbuf[n + st], g0, g1);
    acc += (double)g0;
    acc += (double)g1;
  }
  if (n < fc.D) acc += (double)weier_gene_precise(zbuf[n]);
  acc = tm.sum(acc);
  return acc + fc.woff64;
}

// Largest error of an eval_weier_precise value, per gene: each term's
// argument y_k = 2 3^k |z| mod 2 reaches cospif as a 24-bit float after the
// low bits are cut (< 2^-24) and the 25-bit rest rounded (<= 2^-24), so
// |dy| < 2^-23 and the term moves by < pi 2^-23; cospif adds <= 1 ulp
// (<= 2^-24 for |cos| <= 1); times 0.5^k summed over k (< 2) that is
// < 8.7e-7, and the compensated sum of 21 terms adds < 2 u sum |terms|
// (< 2.4e-7).  Over D genes: D x 1.2e-6.  Near ties closer than twice this
// are decided by eval_weier_ff_t instead.
__device__ __forceinline__ double weier_precise_bound(int D) { return 1.2e-6 * (double)D; }

// Float-float arithmetic (pairs h + l of FP32 values, ~2^-44 relative) on
// the FP32 pipe, for the Weierstrass ties the FP32 terms cannot separate:
// this GPU's FP64 pipe runs at ~1/64 of its FP32 rate, so a double-precision
// cosine costs far more than the float-float one below.
struct FF {
  float h, l;
};
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return ff_fast_two_sum(s, e);
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  return ff_fast_two_sum(p, e);
}
// a double constant as a float-float pair
#define EMT_FF(v) FF{(float)(v), (float)((v) - (double)(float)(v))}

// cos(pi y) for y = r 2^-sh in [0, 2) (r < 2^(sh+1), 1 <= sh <= 127) to
// ~1e-13: y is split exactly as m/2 + t with m = round(2 y) and
// |t| <= 1/4 in integers, t goes to float-float (48 significant bits), and
// cos or sin of x = pi t comes from its Taylor series (|x| <= pi/4; the
// first omitted terms are below 1e-15), the five leading coefficients in
// float-float and the small tail in FP32.
__device__ __forceinline__ FF cospi_ff(unsigned __int128 r, int sh) {
  const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
  const unsigned __int128 q = (r + (half >> 1)) >> (sh - 1);  // round(2 y)
  __int128 d = (__int128)r - (__int128)(q * half);            // t = d 2^-sh, |d| <= 2^(sh-2)
  int e = sh;
  if (sh > 64) {  // keep 62 bits of d: the cut is below 2^-64 of t's scale
    d >>= (sh - 64);
    e = 64;
  }
  const long long dl = (long long)d;
  const float th = __ll2float_rn(dl);
  const float tl = __ll2float_rn(dl - (long long)th);
  const FF t{ldexpf(th, -e), ldexpf(tl, -e)};
  const FF x = ff_mul(t, EMT_FF(3.14159265358979323846));
  const FF u = ff_mul(x, x);
  const int quadrant = (int)(q & 3u);
  FF v;
  if (quadrant & 1) {  // sin x = x (1 - u/3! + u^2/5! - ...)
    float tail = __fmaf_rn(u.h, -1.0f / 1307674368000.0f, 1.0f / 6227020800.0f);
    tail = __fmaf_rn(u.h, tail, -1.0f / 39916800.0f);
    FF w = FF{tail, 0.f};
    w = ff_add(EMT_FF(1.0 / 362880.0), ff_mul(u, w));
    w = ff_add(EMT_FF(-1.0 / 5040.0), ff_mul(u, w));
    w = ff_add(EMT_FF(1.0 / 120.0), ff_mul(u, w));
    w = ff_add(EMT_FF(-1.0 / 6.0), ff_mul(u, w));
    w = ff_add(FF{1.f, 0.f}, ff_mul(u, w));
    v = ff_mul(x, w);
    if (quadrant == 1) v = FF{-v.h, -v.l};  // cos(pi t + pi/2) = -sin(pi t)
  } else {  // cos x = 1 - u/2! + u^2/4! - ...
    float tail = __fmaf_rn(u.h, -1.0f / 87178291200.0f, 1.0f / 479001600.0f);
    tail = __fmaf_rn(u.h, tail, -1.0f / 3628800.0f);
    FF w = FF{tail, 0.f};
    w = ff_add(EMT_FF(1.0 / 40320.0), ff_mul(u, w));
    w = ff_add(EMT_FF(-1.0 / 720.0), ff_mul(u, w));
    w = ff_add(EMT_FF(1.0 / 24.0), ff_mul(u, w));
    w = ff_add(FF{-0.5f, 0.f}, ff_mul(u, w));
    v = ff_add(FF{1.f, 0.f}, ff_mul(u, w));
    if (quadrant == 2) v = FF{-v.h, -v.l};  // cos(pi t + pi) = -cos(pi t)
  }
  return v;
}

// One Weierstrass gene with every term in float-float: the same exact
// reduction of y_k = 2 3^k |z| mod 2 as weier_gene_precise (here in 128-bit
// integers), then cospi_ff; the terms are summed in float-float.
__device__ __forceinline__ double weier_gene_ff(double z) {
  const unsigned long long b =
      (unsigned long long)__double_as_longlong(z) & 0x7FFFFFFFFFFFFFFFull;
  const int E = (int)(b >> 52);
  const unsigned long long M = (b & ((1ull << 52) - 1ull)) | (1ull << 52);
  const int sh = 1074 - E;  // y_0 = M / 2^sh for normal |z|
  FF s{0.f, 0.f};
  float ak = 1.f;
  if (b == 0ull || E == 0 || sh > 127) {
    // |z| < 2^-75: every 2 3^k |z| < 2^-41, cos = 1 to far below the bound
    for (int k = 0; k <= 20; ++k, ak *= 0.5f) s = ff_add(s, FF{-ak, 0.f});
  } else if (sh <= 0) {
    const float c = (sh == 0 && (M & 1ull)) ? -1.f : 1.f;
    for (int k = 0; k <= 20; ++k, ak *= 0.5f) s = ff_add(s, FF{-ak * c, 0.f});
  } else {
    const unsigned __int128 mask = sh >= 127 ? ~(unsigned __int128)0
                                             : (((unsigned __int128)2 << sh) - 1);
    unsigned __int128 r = (unsigned __int128)M & mask;
    for (int k = 0; k <= 20; ++k, ak *= 0.5f) {
      const FF c = cospi_ff(r, sh);
      s = ff_add(s, FF{-ak * c.h, -ak * c.l});  // scaling by 0.5^k is exact
      r = (r * 3u) & mask;
    }
  }
  return (double)s.h + (double)s.l;
}

// weier_gene_ff of two genes, interleaved when both take the general path;
// every operation of each gene is weier_gene_ff's.
__device__ __forceinline__ void weier_gene_ff2(double z0, double z1, double& g0, double& g1) {
  const unsigned long long b0 = (unsigned long long)__double_as_longlong(z0) & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long b1 = (unsigned long long)__double_as_longlong(z1) & 0x7FFFFFFFFFFFFFFFull;
  const int E0 = (int)(b0 >> 52), E1 = (int)(b1 >> 52);
  const int sh0 = 1074 - E0, sh1 = 1074 - E1;
  if (b0 == 0ull || E0 == 0 || sh0 <= 0 || sh0 > 127 || b1 == 0ull || E1 == 0 || sh1 <= 0 ||
      sh1 > 127) {
    g0 = weier_gene_ff(z0);
    g1 = weier_gene_ff(z1);
    return;
  }
  const unsigned __int128 mask0 = sh0 >= 127 ? ~(unsigned __int128)0
                                             : (((unsigned __int128)2 << sh0) - 1);
  const unsigned __int128 mask1 = sh1 >= 127 ? ~(unsigned __int128)0
                                             : (((unsigned __int128)2 << sh1) - 1);
  unsigned __int128 r0 = (unsigned __int128)((b0 & ((1ull << 52) - 1ull)) | (1ull << 52)) & mask0;
  unsigned __int128 r1 = (unsigned __int128)((b1 & ((1ull << 52) - 1ull)) | (1ull << 52)) & mask1;
  FF s0{0.f, 0.f}, s1{0.f, 0.f};
  float ak = 1.f;
  for (int k = 0; k <= 20; ++k, ak *= 0.5f) {
    const FF c0 = cospi_ff(r0, sh0);
    const FF c1 = cospi_ff(r1, sh1);
    s0 = ff_add(s0, FF{-ak * c0.h, -ak * c0.l});
    s1 = ff_add(s1, FF{-ak * c1.h, -ak * c1.l});
    r0 = (r0 * 3u) & mask0;
    r1 = (r1 * 3u) & mask1;
  }
  g0 = (double)s0.h + (double)s0.l;
  g1 = (double)s1.h + (double)s1.l;
}

// eval_weier_ff_t with two genes per step of each team member, summed in the
// same order (the same value).
template <class Team>
__device__ double eval_weier_ff_pair_t(const FnConst& fc, const double* zbuf, const Team& tm) {
  const int st = tm.size();
  double acc = 0.0;
  int n = tm.rank();
  for (; n + st < fc.D; n += 2 * st) {
    double g0, g1;
    weier_gene_ff2(zbuf[n], zbuf[n + st], g0, g1);
    acc += g0;
    acc += g1;
  }
  if (n < fc.D) acc += weier_gene_ff(zbuf[n]);
  acc = tm.sum(acc);
  return acc + fc.woff64;
}

template <class Team>
__device__ double eval_weier_ff_t(const FnConst& fc, const double* zbuf, const Team& tm) {
  double acc = 0.0;
  for (int n = tm.rank(); n < fc.D; n += tm.size()) acc += weier_gene_ff(zbuf[n]);
  acc = tm.sum(acc);
  return acc + fc.woff64;
}
// The warp form, out of line: a rare path that should not raise the
// register needs of the fused kernel around it.
__device__ __noinline__ double eval_weier_ff_warp(const FnConst& fc, const double* zbuf) {
  return eval_weier_ff_t(fc, zbuf, WarpTeam{});
}

// FP64-class fitness of x (shared or global memory row) by the calling warp
// (qt[k*DP + n] = Q[n][k]); zbuf: DP doubles of per-warp scratch.
__device__ double eval_row_f64(const FnConst& fc, const float* __restrict__ x,
                               const float* __restrict__ o, const float* __restrict__ qt,
                               int DP, double* zbuf) {
  precise_rotation(x, o, qt, DP, fc.D, zbuf);
  const double f = fc.fid == F_WEIERSTRASS ? eval_weier_precise(fc, zbuf) : eval_tier3(fc, zbuf);
  __syncwarp();
  return f;
}

}  // namespace emt
