/*
 * emt_oracle.c -- CPU ORACLE (test infrastructure only; see emt_oracle.h).
 *
 * Plain C restatement of the reference's generation step with the engine's
 * Philox stream.  Every fused multiply-add that the engine performs is an
 * explicit fmaf() here and the file is compiled with -ffp-contract=off, so
 * trial vectors agree with the device bit for bit on x86 and on Arm.
 */
#define __STDC_WANT_IEC_60559_TYPES_EXT__ 1
#include "emt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)                   */
/* ------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += PHILOX_W0; k1 += PHILOX_W1; }
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_draw(uint64_t seed, uint32_t task, uint32_t gen, uint32_t member, uint32_t purpose,
              uint32_t block, uint32_t out[4]) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {task, gen, member, (purpose << 24) | (block & 0xFFFFFFu)};
  orc_philox4x32_10(ctr, key, out);
}

float orc_u01(uint32_t w) { return (float)(w >> 8) * 0x1p-24f; }

/* ------------------------------------------------------------------ */
/* boxes and ids                                                        */
/* ------------------------------------------------------------------ */
static const float kBoxStd[ORC_NFUNC][2] = {
    {-100.f, 100.f},     /* sphere      */
    {-5.12f, 5.12f},     /* rastrigin   */
    {-32.768f, 32.768f}, /* ackley      */
    {-600.f, 600.f},     /* griewank    */
    {-2.048f, 2.048f},   /* rosenbrock  */
    {-500.f, 500.f},     /* schwefel    */
    {-0.5f, 0.5f},       /* weierstrass */
};
/* SG-EMTF.cu:197-214, indexed by reference type 0..6 */
static const float kBoxRef[7][2] = {{-100.f, 100.f}, {-50.f, 50.f}, {-50.f, 50.f}, {-50.f, 50.f},
                                    {-100.f, 100.f}, {-0.5f, 0.5f}, {-500.f, 500.f}};
/* reference type -> function id (SG-EMTF.cu:917-1101) */
static const int kRefToFid[7] = {ORC_SPHERE,    ORC_ROSENBROCK,  ORC_ACKLEY,  ORC_RASTRIGIN,
                                 ORC_GRIEWANK,  ORC_WEIERSTRASS, ORC_SCHWEFEL};

int orc_function_from_reference(int t) { return (t >= 0 && t < 7) ? kRefToFid[t] : -1; }

int orc_box(int fid, int reference_boxes, float* lo, float* hi) {
  if (fid < 0 || fid >= ORC_NFUNC) return -1;
  if (reference_boxes) {
    for (int t = 0; t < 7; ++t)
      if (kRefToFid[t] == fid) { *lo = kBoxRef[t][0]; *hi = kBoxRef[t][1]; return 0; }
  }
  *lo = kBoxStd[fid][0];
  *hi = kBoxStd[fid][1];
  return 0;
}

/* SG-EMTF.cu:354-361: float a_=1, b_=1, res=0; for i<=20: res += a_*cosf(2*PI*b_*0.5);
 * with PI the double literal 3.1415926, b_ *= 3 in float. */
double orc_weierstrass_reference_offset(void) {
  float a = 1.f, b = 1.f, res = 0.f;
  for (int i = 0; i <= 20; ++i) {
    double arg = 2 * 3.1415926 * (double)b * 0.5;
    res += a * cosf((float)arg);
    a *= 0.5f;
    b *= 3.f;
  }
  return (double)res;
}

/* ------------------------------------------------------------------ */
/* instance generation                                                  */
/* ------------------------------------------------------------------ */
void orc_gen_shift(uint64_t seed, uint32_t task, int D, float lo, float hi, float* o) {
  float a = 0.8f * lo, r = 0.8f * (hi - lo);
  uint32_t w[4];
  for (int d = 0; d < D; ++d) {
    if ((d & 3) == 0) orc_draw(seed, task, 0, 0, ORC_P_SHIFT, (uint32_t)(d >> 2), w);
    o[d] = fmaf(orc_u01(w[d & 3]), r, a);
  }
}

void orc_gen_population(uint64_t seed, uint32_t task, int NP, int D, float lo, float hi,
                        float* X) {
  float r = hi - lo;
  uint32_t w[4];
  for (int i = 0; i < NP; ++i)
    for (int d = 0; d < D; ++d) {
      if ((d & 3) == 0) orc_draw(seed, task, 0, (uint32_t)i, ORC_P_POP_INIT, (uint32_t)(d >> 2), w);
      float x = fmaf(orc_u01(w[d & 3]), r, lo);
      X[(size_t)i * D + d] = x > hi ? hi : x;
    }
}

/* Orthogonal factor of the Householder QR of a seeded N(0,1) matrix, with
 * the sign of each column fixed so that R has a positive diagonal (the Haar
 * measure).  Gaussians: Box-Muller on Philox words, u1 in (0,1]. */
void orc_gen_rotation(uint64_t seed, uint32_t task, int D, double* Q) {
  double* A = (double*)malloc(sizeof(double) * D * D);
  double* v = (double*)malloc(sizeof(double) * D);
  uint32_t w[4];
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; c += 4) {
      orc_draw(seed, task, 0, (uint32_t)r, ORC_P_QR_NORMAL, (uint32_t)(c >> 2), w);
      for (int h = 0; h < 2; ++h) {
        double u1 = ((double)w[2 * h] + 1.0) * 0x1p-32;
        double u2 = (double)w[2 * h + 1] * 0x1p-32;
        double rad = sqrt(-2.0 * log(u1));
        double th = 6.283185307179586 * u2;
        if (c + 2 * h < D) A[r * D + c + 2 * h] = rad * cos(th);
        if (c + 2 * h + 1 < D) A[r * D + c + 2 * h + 1] = rad * sin(th);
      }
    }
  /* Q starts as identity; apply reflectors H_k from the left to A and
   * accumulate Q = H_0 H_1 ... on the right. */
  for (int i = 0; i < D * D; ++i) Q[i] = 0.0;
  for (int i = 0; i < D; ++i) Q[i * D + i] = 1.0;
  for (int k = 0; k < D - 1; ++k) {
    double nrm = 0.0;
    for (int i = k; i < D; ++i) nrm += A[i * D + k] * A[i * D + k];
    nrm = sqrt(nrm);
    if (nrm == 0.0) continue;
    double alpha = A[k * D + k] > 0 ? -nrm : nrm;
    for (int i = 0; i < D; ++i) v[i] = 0.0;
    for (int i = k; i < D; ++i) v[i] = A[i * D + k];
    v[k] -= alpha;
    double vn = 0.0;
    for (int i = k; i < D; ++i) vn += v[i] * v[i];
    if (vn == 0.0) continue;
    for (int c = k; c < D; ++c) { /* A <- H A */
      double s = 0.0;
      for (int i = k; i < D; ++i) s += v[i] * A[i * D + c];
      s = 2.0 * s / vn;
      for (int i = k; i < D; ++i) A[i * D + c] -= s * v[i];
    }
    for (int r = 0; r < D; ++r) { /* Q <- Q H */
      double s = 0.0;
      for (int i = k; i < D; ++i) s += Q[r * D + i] * v[i];
      s = 2.0 * s / vn;
      for (int i = k; i < D; ++i) Q[r * D + i] -= s * v[i];
    }
  }
  for (int c = 0; c < D; ++c)
    if (A[c * D + c] < 0)
      for (int r = 0; r < D; ++r) Q[r * D + c] = -Q[r * D + c];
  free(A);
  free(v);
}

/* ------------------------------------------------------------------ */
/* FP64 evaluation                                                      */
/* ------------------------------------------------------------------ */
static double cospi64(double x) {
  double r = fmod(fabs(x), 2.0); /* exact */
  if (r > 1.0) r = 2.0 - r;      /* cos(pi r) symmetric about 1 */
  return cos(3.141592653589793 * r);
}

static void rotate64(const orc_task* t, const float* x, double* z) {
  int D = t->D;
  for (int n = 0; n < D; ++n) {
    if (!t->Q) { z[n] = (double)x[n] - (double)t->o[n]; continue; }
    double acc = 0.0;
    for (int k = 0; k < D; ++k)
      acc += (double)t->Q[(size_t)n * D + k] * ((double)x[k] - (double)t->o[k]);
    z[n] = acc;
  }
}

static double weier_offset(uint32_t flags, int D) {
  /* standard: - D * sum_k 0.5^k cos(pi 3^k) = + D (2 - 2^-20) */
  if (flags & ORC_FLAG_REF_WEIERSTRASS_CONST) return -(double)D * orc_weierstrass_reference_offset();
  return (double)D * (2.0 - 0x1p-20);
}

static double fvalue64(int fid, uint32_t flags, int D, const double* z, double* scale) {
  double f = 0.0, s = 0.0;
  switch (fid) {
    case ORC_SPHERE:
      for (int j = 0; j < D; ++j) f += z[j] * z[j];
      s = f;
      break;
    case ORC_RASTRIGIN:
      for (int j = 0; j < D; ++j) {
        double c = cospi64(2.0 * z[j]);
        f += z[j] * z[j] - 10.0 * c + 10.0;
        s += z[j] * z[j] + 10.0 * fabs(c) + 10.0;
      }
      break;
    case ORC_ACKLEY: {
      double a = 0.0, b = 0.0;
      for (int j = 0; j < D; ++j) { a += z[j] * z[j]; b += cospi64(2.0 * z[j]); }
      double e = (flags & ORC_FLAG_REF_ACKLEY_E) ? 2.718282 : 2.718281828459045;
      double t1 = 20.0 * exp(-0.2 * sqrt(a / D)), t2 = exp(b / D);
      f = -t1 - t2 + 20.0 + e;
      s = t1 + t2 + 20.0 + e;
      break;
    }
    case ORC_GRIEWANK: {
      double a = 0.0, p = 1.0;
      for (int j = 0; j < D; ++j) {
        a += z[j] * z[j];
        if (!(flags & ORC_FLAG_REF_GRIEWANK_NO_PRODUCT)) p *= cos(z[j] / sqrt((double)(j + 1)));
      }
      f = 1.0 + a / 4000.0 - p;
      s = 1.0 + a / 4000.0 + fabs(p);
      break;
    }
    case ORC_ROSENBROCK:
      for (int j = 0; j + 1 < D; ++j) {
        double a = z[j] * z[j] - z[j + 1], b = z[j] - 1.0;
        f += 100.0 * a * a + b * b;
        double aa = z[j] * z[j] + fabs(z[j + 1]), bb = fabs(z[j]) + 1.0;
        s += 100.0 * aa * aa + bb * bb;
      }
      break;
    case ORC_SCHWEFEL: {
      double a = 0.0, sa = 0.0;
      for (int j = 0; j < D; ++j) {
        double g = z[j] * sin(sqrt(fabs(z[j])));
        a += g;
        sa += fabs(g);
      }
      f = 418.9829 * D - a;
      s = 418.9829 * D + sa;
      break;
    }
    case ORC_WEIERSTRASS: {
      double off = weier_offset(flags, D);
      for (int j = 0; j < D; ++j) {
        double ak = 1.0, bk = 1.0;
        for (int k = 0; k <= 20; ++k) {
          double c = cospi64(2.0 * bk * (z[j] + 0.5));
          f += ak * c;
          s += ak * fabs(c);
          ak *= 0.5;
          bk *= 3.0;
        }
      }
      f += off;
      s += fabs(off);
      break;
    }
    default:
      f = NAN;
      s = NAN;
  }
  if (scale) *scale = s;
  return f;
}

/* ------------------------------------------------------------------ */
/* _Float128 evaluation: the replay's arbiter of near ties              */
/* ------------------------------------------------------------------ */
/* Near its optimum a function value can be the small difference of large
 * terms (Ackley: 20 + e - 20 exp(-0.2 r) - exp(B / D); Schwefel:
 * 418.9829 D - sum z sin sqrt|z|), so two FP64 evaluations may tie although
 * the exact values differ (observed: Ackley, f = 3.1e-6, exact gap 2.7e-15,
 * FP64 gap 0).  The replay's decision is the exact one: FP64 values decide
 * when they differ by more than 1e-10 of the scale (every FP64 form here
 * is far more accurate than that), and IEEE binary128 evaluations (113-bit
 * significand; the rotation's FP32 x FP32 products are exact in it; glibc's
 * *f128 functions) decide the rest. */
typedef _Float128 q128;
static const q128 kPiQ = 3.14159265358979323846264338327950288q;

static void rotate128(const orc_task* t, const float* x, q128* z) {
  int D = t->D;
  for (int n = 0; n < D; ++n) {
    if (!t->Q) { z[n] = (q128)x[n] - (q128)t->o[n]; continue; }
    q128 acc = 0;
    for (int k = 0; k < D; ++k)
      acc += (q128)t->Q[(size_t)n * D + k] * ((q128)x[k] - (q128)t->o[k]);
    z[n] = acc;
  }
}

static q128 cospi128(q128 x) {
  q128 r = fmodf128(fabsf128(x), 2); /* exact */
  if (r > 1) r = 2 - r;
  return cosf128(kPiQ * r);
}

static q128 fvalue128(int fid, uint32_t flags, int D, const q128* z) {
  q128 f = 0;
  switch (fid) {
    case ORC_SPHERE:
      for (int j = 0; j < D; ++j) f += z[j] * z[j];
      break;
    case ORC_RASTRIGIN:
      for (int j = 0; j < D; ++j) f += z[j] * z[j] - 10 * cospi128(2 * z[j]) + 10;
      break;
    case ORC_ACKLEY: {
      q128 a = 0, b = 0;
      for (int j = 0; j < D; ++j) { a += z[j] * z[j]; b += cospi128(2 * z[j]); }
      q128 e = (flags & ORC_FLAG_REF_ACKLEY_E) ? (q128)2.718282 : expf128(1);
      f = -20 * expf128(-(q128)0.2q * sqrtf128(a / D)) - expf128(b / D) + 20 + e;
      break;
    }
    case ORC_GRIEWANK: {
      q128 a = 0, p = 1;
      for (int j = 0; j < D; ++j) {
        a += z[j] * z[j];
        if (!(flags & ORC_FLAG_REF_GRIEWANK_NO_PRODUCT)) p *= cosf128(z[j] / sqrtf128((q128)(j + 1)));
      }
      f = 1 + a / 4000 - p;
      break;
    }
    case ORC_ROSENBROCK:
      for (int j = 0; j + 1 < D; ++j) {
        q128 a = z[j] * z[j] - z[j + 1], b = z[j] - 1;
        f += 100 * a * a + b * b;
      }
      break;
    case ORC_SCHWEFEL: {
      q128 a = 0;
      for (int j = 0; j < D; ++j) a += z[j] * sinf128(sqrtf128(fabsf128(z[j])));
      f = (q128)418.9829 * D - a;
      break;
    }
    case ORC_WEIERSTRASS: {
      for (int j = 0; j < D; ++j) {
        q128 ak = 1, bk = 1;
        for (int k = 0; k <= 20; ++k) {
          f += ak * cospi128(2 * bk * (z[j] + (q128)0.5q));
          ak *= (q128)0.5q;
          bk *= 3;
        }
      }
      f += (q128)weier_offset(flags, D);
      break;
    }
    default:
      f = NAN;
  }
  return f;
}

static q128 eval128(const orc_task* t, const float* x) {
  q128 zb[1024];
  rotate128(t, x, zb);
  return fvalue128(t->fid, t->flags, t->D, zb);
}

/* Whether u replaces x in the replay (mode 0): f(u) <= f(x), or f(u) < f(x)
 * when strict.  fu, fx: FP64 values; su: u's FP64 scale.  Identical vectors
 * tie. */
static int decide_exact(const orc_task* t, const float* u, double fu, double su,
                        const float* x, double fx, int strict) {
  if (memcmp(u, x, sizeof(float) * (size_t)t->D) == 0) return !strict;
  if (!(fabs(fu - fx) <= 1e-10 * (su + fabs(fu) + fabs(fx))))
    return strict ? fu < fx : fu <= fx;
  const q128 qu = eval128(t, u), qx = eval128(t, x);
  return strict ? qu < qx : qu <= qx;
}

double orc_eval64(const orc_task* t, const float* x, double* scale, double* zout) {
  double zb[1024]; /* D <= 1024, the engine's largest island */
  double* z = zout ? zout : zb;
  rotate64(t, x, z);
  return fvalue64(t->fid, t->flags, t->D, z, scale);
}

/* Rounding of the FP32 rotation: |dz_j| <= (gamma_{D+1} + 2^-20) sum_k |Q_jk||s_k|
 * (FP32 sequential FMA dot product, or the TF32 hi/lo split), propagated
 * through each Weierstrass term and capped by the term's range. */
double orc_weierstrass_rotation_bound(const orc_task* t, const float* x) {
  int D = t->D;
  double u = 0x1p-24, g = (D + 1) * u / (1.0 - (D + 1) * u) + 0x1p-20;
  double b = 0.0;
  for (int j = 0; j < D; ++j) {
    double sa = 0.0;
    for (int k = 0; k < D; ++k) {
      double q = t->Q ? fabs((double)t->Q[(size_t)j * D + k]) : (k == j ? 1.0 : 0.0);
      sa += q * fabs((double)x[k] - (double)t->o[k]);
    }
    double dz = g * sa + u * fabs((double)x[j] - (double)t->o[j]);
    double ak = 1.0, bk = 1.0;
    for (int k = 0; k <= 20; ++k) {
      double e = 6.283185307179586 * bk * dz;
      b += ak * (e < 2.0 ? e : 2.0);
      ak *= 0.5;
      bk *= 3.0;
    }
    b += 4e-6; /* the epilogue's own rounding per dimension */
  }
  return b;
}

/* ------------------------------------------------------------------ */
/* FP32 evaluation (CPU baseline arithmetic)                            */
/* ------------------------------------------------------------------ */
static float cospi32(float x) { /* exact reduction mod 2, then cosf */
  float r = fmodf(fabsf(x), 2.f);
  if (r > 1.f) r = 2.f - r;
  return cosf(3.14159265f * r);
}
static float sinpi32(float x) {
  float r = fmodf(x, 2.f); /* (-2, 2) */
  if (r > 1.f) r -= 2.f;
  if (r < -1.f) r += 2.f;
  if (r > 0.5f) r = 1.f - r;
  if (r < -0.5f) r = -1.f - r;
  return sinf(3.14159265f * r);
}

/* cos(2 pi 3^k (z + 0.5)) = -cos(pi * (2 * 3^k * z mod 2)); the reduction is
 * exact integer arithmetic on the FP32 significand of z. */
static void weier_terms32(float z, float* sum, float* sabs) {
  float s = 0.f, sa = 0.f;
  float az = fabsf(z);
  if (az == 0.f) {
    for (int k = 0; k <= 20; ++k) { float a = ldexpf(1.f, -k); s -= a; sa += a; }
    *sum = s; *sabs = sa; return;
  }
  int e;
  float m = frexpf(az, &e);                 /* az = m 2^e, m in [0.5,1) */
  uint64_t M = (uint64_t)ldexpf(m, 24);     /* az = M 2^(e-24) */
  int sh = 23 - e;                          /* y_k = M 3^k / 2^sh */
  uint64_t P = M;
  for (int k = 0; k <= 20; ++k) {
    float y;
    if (sh < 0) y = 0.f;
    else if (sh >= 62) y = (float)P * ldexpf(1.f, -sh);
    else y = (float)(P & ((2ull << sh) - 1ull)) * ldexpf(1.f, -sh);
    float c = -cospi32(y);
    float a = ldexpf(1.f, -k);
    s += a * c;
    sa += a * fabsf(c);
    if (sh >= 0 && sh < 62) P = (P & ((2ull << sh) - 1ull)) * 3ull; else P *= 3ull;
  }
  *sum = s;
  *sabs = sa;
}

float orc_eval32(const orc_task* t, const float* x, float* scale) {
  int D = t->D;
  float z[1024]; /* D <= 1024 */
  for (int n = 0; n < D; ++n) {
    if (!t->Q) { z[n] = x[n] - t->o[n]; continue; }
    float acc = 0.f;
    const float* q = t->Q + (size_t)n * D;
    for (int k = 0; k < D; ++k) acc = fmaf(q[k], x[k] - t->o[k], acc);
    z[n] = acc;
  }
  float f = 0.f, s = 0.f;
  switch (t->fid) {
    case ORC_SPHERE:
      for (int j = 0; j < D; ++j) f = fmaf(z[j], z[j], f);
      s = f;
      break;
    case ORC_RASTRIGIN:
      for (int j = 0; j < D; ++j) {
        float sp = sinpi32(z[j]);
        f += z[j] * z[j] + 20.f * sp * sp;
        s += z[j] * z[j] + 10.f * fabsf(1.f - 2.f * sp * sp) + 10.f;
      }
      break;
    case ORC_ACKLEY: {
      float a = 0.f, b = 0.f;
      for (int j = 0; j < D; ++j) { a = fmaf(z[j], z[j], a); b += cospi32(2.f * z[j]); }
      float e = (t->flags & ORC_FLAG_REF_ACKLEY_E) ? 2.718282f : 2.71828183f;
      float t1 = 20.f * expf(-0.2f * sqrtf(a / D)), t2 = expf(b / D);
      f = (20.f - t1) + (e - t2);
      s = t1 + t2 + 20.f + e;
      break;
    }
    case ORC_GRIEWANK: {
      float a = 0.f, p = 1.f;
      for (int j = 0; j < D; ++j) {
        a = fmaf(z[j], z[j], a);
        if (!(t->flags & ORC_FLAG_REF_GRIEWANK_NO_PRODUCT)) p *= cosf(z[j] / sqrtf((float)(j + 1)));
      }
      f = (1.f - p) + a / 4000.f;
      s = 1.f + a / 4000.f + fabsf(p);
      break;
    }
    case ORC_ROSENBROCK:
      for (int j = 0; j + 1 < D; ++j) {
        float a = z[j] * z[j] - z[j + 1], b = z[j] - 1.f;
        f += 100.f * a * a + b * b;
        float aa = z[j] * z[j] + fabsf(z[j + 1]), bb = fabsf(z[j]) + 1.f;
        s += 100.f * aa * aa + bb * bb;
      }
      break;
    case ORC_SCHWEFEL: {
      float a = 0.f, sa = 0.f;
      for (int j = 0; j < D; ++j) {
        float g = z[j] * sinf(sqrtf(fabsf(z[j])));
        a += g;
        sa += fabsf(g);
      }
      f = 418.9829f * D - a;
      s = 418.9829f * D + sa;
      break;
    }
    case ORC_WEIERSTRASS: {
      float a = 0.f, sa = 0.f;
      for (int j = 0; j < D; ++j) {
        float tj, taj;
        weier_terms32(z[j], &tj, &taj);
        a += tj;
        sa += taj;
      }
      float off = (float)weier_offset(t->flags, D);
      f = a + off;
      s = sa + fabsf(off);
      break;
    }
    default:
      f = NAN;
      s = NAN;
  }
  if (scale) *scale = s;
  return f;
}

/* ------------------------------------------------------------------ */
/* deterministic power: exp2(y * log2(x)) from FP32 +,-,*,/ and fma     */
/* log2 m = (2/ln 2) atanh(s), s = (m-1)/(m+1), odd series to s^9;      */
/* exp2 f = e^(f ln 2), Taylor to degree 7 (Horner).                   */
/* ------------------------------------------------------------------ */
static float ldexp_exact(float v, int n) {
  union { uint32_t u; float f; } b;
  b.u = (uint32_t)(n + 127) << 23;
  return v * b.f;
}

float orc_powf(float x, float y) {
  if (!(x > 0x1p-100f)) return 0.f;
  union { float f; uint32_t u; } b;
  b.f = x;
  int e = (int)((b.u >> 23) & 0xFF) - 127;
  b.u = (b.u & 0x7FFFFFu) | 0x3F800000u; /* m in [1, 2) */
  float m = b.f;
  if (m > 1.41421354f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.f) / (m + 1.f);
  float s2 = s * s;
  float p = fmaf(s2, 0x1.c71c72p-4f /* 1/9 */, 0x1.24924ap-3f /* 1/7 */);
  p = fmaf(s2, p, 0x1.99999ap-3f /* 1/5 */);
  p = fmaf(s2, p, 0x1.555556p-2f /* 1/3 */);
  p = fmaf(s2, p, 1.f);
  float lm = (s * p) * 0x1.715476p+1f; /* 2 / ln 2 */
  float L = (float)e + lm;
  float t = y * L;
  if (t > 126.f) t = 126.f;
  if (t < -126.f) return 0.f;
  float n = rintf(t);
  float f = t - n;
  float g = f * 0x1.62e430p-1f; /* ln 2 */
  float q = fmaf(g, 0x1.a01a02p-13f /* 1/5040 */, 0x1.6c16c2p-10f /* 1/720 */);
  q = fmaf(g, q, 0x1.111112p-7f /* 1/120 */);
  q = fmaf(g, q, 0x1.555556p-5f /* 1/24 */);
  q = fmaf(g, q, 0x1.555556p-3f /* 1/6 */);
  q = fmaf(g, q, 0.5f);
  q = fmaf(g, q, 1.f);
  q = fmaf(g, q, 1.f);
  return ldexp_exact(q, (int)n);
}

/* ------------------------------------------------------------------ */
/* trial vectors                                                        */
/* ------------------------------------------------------------------ */
static inline float clampf_box(float v, float lo, float hi) {
  if (v > hi) return hi;
  if (v < lo) return lo;
  return v;
}

/* members per sub-island: operators draw partners within the member's own
 * sub-island (the reference's two slots of one block, SG-EMTF.cu:1138-1218,
 * evolve apart between migrations) */
static int sub_size(const orc_params* p, const orc_task* t) {
  return p->subislands > 1 ? t->NP / p->subislands : t->NP;
}

static void de_indices(const orc_params* p, const orc_task* t, uint32_t gen, int i, int* r1o,
                       int* r2o, int* r3o, int* jro) {
  uint32_t w[4];
  const int NP = sub_size(p, t), base = (i / NP) * NP;
  orc_draw(p->seed, t->id, gen, (uint32_t)i, ORC_P_DE_INDEX, 0, w);
  i -= base;
  int r1 = (int)(w[0] % (uint32_t)(NP - 1));
  if (r1 >= i) r1++;
  int a = i < r1 ? i : r1, b = i < r1 ? r1 : i;
  int r2 = (int)(w[1] % (uint32_t)(NP - 2));
  if (r2 >= a) r2++;
  if (r2 >= b) r2++;
  int s0 = i, s1 = r1, s2 = r2, tmp; /* sort three */
  if (s0 > s1) { tmp = s0; s0 = s1; s1 = tmp; }
  if (s1 > s2) { tmp = s1; s1 = s2; s2 = tmp; }
  if (s0 > s1) { tmp = s0; s0 = s1; s1 = tmp; }
  int r3 = (int)(w[2] % (uint32_t)(NP - 3));
  if (r3 >= s0) r3++;
  if (r3 >= s1) r3++;
  if (r3 >= s2) r3++;
  *r1o = r1 + base; *r2o = r2 + base; *r3o = r3 + base;
  *jro = (int)(w[3] % (uint32_t)t->D);
}

static int ga_parent(const orc_params* p, const orc_task* t, uint32_t gen, int i) {
  uint32_t w[4];
  const int NP = sub_size(p, t), base = (i / NP) * NP;
  orc_draw(p->seed, t->id, gen, (uint32_t)i, ORC_P_GA_PARENT, 0, w);
  return base + (int)(w[0] % (uint32_t)NP);
}

void orc_trial(const orc_params* p, const orc_task* t, const float* X, uint32_t gen, int i,
               float* u) {
  int D = t->D, NP = t->NP;
  float lo = t->lo, hi = t->hi;
  uint32_t w[4];
  if (p->algorithm == ORC_DE_RAND1 || p->algorithm == ORC_DE_CURRENT1) {
    int r1, r2, r3, jr;
    de_indices(p, t, gen, i, &r1, &r2, &r3, &jr);
    int base = p->algorithm == ORC_DE_RAND1 ? r1 : i;
    const float *xb = X + (size_t)base * D, *x2 = X + (size_t)r2 * D, *x3 = X + (size_t)r3 * D,
                *xi = X + (size_t)i * D;
    for (int j = 0; j < D; ++j) {
      if ((j & 3) == 0) orc_draw(p->seed, t->id, gen, (uint32_t)i, ORC_P_DE_CR, (uint32_t)(j >> 2), w);
      float m = clampf_box(fmaf(p->F, x2[j] - x3[j], xb[j]), lo, hi);
      u[j] = (orc_u01(w[j & 3]) < p->CR || j == jr) ? m : xi[j];
    }
    return;
  }
  /* GA: SBX on the pair (i, i^1) of drawn parents, then polynomial mutation */
  int r0 = ga_parent(p, t, gen, i);
  int pi = i ^ 1, NPs = sub_size(p, t);
  int partner = (pi < NP && pi / NPs == i / NPs) ? ga_parent(p, t, gen, pi) : r0;
  const float *x0 = X + (size_t)r0 * D, *x1 = X + (size_t)partner * D;
  float ec = 1.f / (p->eta_c + 1.f);
  float em1 = p->eta_m + 1.f, em = 1.f / em1;
  float pm = p->p_m < 0.f ? 1.f / (float)D : p->p_m;
  float range = hi - lo;
  uint32_t ws[4], wm[4];
  for (int j = 0; j < D; ++j) {
    if ((j & 1) == 0) {
      orc_draw(p->seed, t->id, gen, (uint32_t)i, ORC_P_GA_SBX, (uint32_t)(j >> 1), ws);
      orc_draw(p->seed, t->id, gen, (uint32_t)i, ORC_P_GA_PM, (uint32_t)(j >> 1), wm);
    }
    int h = (j & 1) * 2;
    float c;
    if (orc_u01(ws[h]) < p->p_c) {
      float pu = orc_u01(ws[h + 1]);
      float tv = pu <= 0.5f ? 2.f * pu : 0.5f / (1.f - pu);
      float beta = orc_powf(tv, ec);
      if (i & 1) beta = -beta;
      c = 0.5f * fmaf(1.f + beta, x0[j], (1.f - beta) * x1[j]);
      c = clampf_box(c, lo, hi);
    } else {
      c = x0[j];
    }
    if (orc_u01(wm[h]) < pm) {
      float um = orc_u01(wm[h + 1]);
      float dq;
      if (um <= 0.5f) {
        float d1 = (c - lo) / range;
        float v = fmaf(1.f - 2.f * um, orc_powf(1.f - d1, em1), 2.f * um);
        dq = orc_powf(v, em) - 1.f;
      } else {
        float d2 = (hi - c) / range;
        float v = fmaf(2.f * (um - 0.5f), orc_powf(1.f - d2, em1), 2.f * (1.f - um));
        dq = 1.f - orc_powf(v, em);
      }
      c = clampf_box(fmaf(dq, range, c), lo, hi);
    }
    u[j] = c;
  }
}

/* ------------------------------------------------------------------ */
/* selection                                                            */
/* ------------------------------------------------------------------ */
static double recheck_window(const orc_params* p, const orc_task* t, const float* x, float f32,
                             float s32) {
  double rel = p->recheck_rel > 0 ? p->recheck_rel : 1e-5;
  double w = rel * (double)s32;
  (void)f32;
  if (t->fid == ORC_WEIERSTRASS)
    w = (p->flags & ORC_FLAG_RIGOROUS_WINDOW) ? w + orc_weierstrass_rotation_bound(t, x) : 5.0 * w;
  return w;
}

int orc_generation(const orc_params* p, const orc_task* t, float* X, float* fit32,
                   double* fit64, uint32_t gen, int mode, uint8_t* accepted) {
  int D = t->D, NP = t->NP, rechecks = 0;
  float* U = (float*)malloc(sizeof(float) * (size_t)NP * D);
  for (int i = 0; i < NP; ++i) orc_trial(p, t, X, gen, i, U + (size_t)i * D);
  for (int i = 0; i < NP; ++i) {
    const float* u = U + (size_t)i * D;
    float* xi = X + (size_t)i * D;
    int acc;
    double ft64 = NAN;
    float ft32 = NAN;
    if (mode == 0) {
      double su;
      ft64 = orc_eval64(t, u, &su, NULL);
      if (isnan(fit64[i])) fit64[i] = orc_eval64(t, xi, NULL, NULL);
      acc = decide_exact(t, u, ft64, su, xi, fit64[i], 0);
    } else {
      float st, sp;
      ft32 = orc_eval32(t, u, &st);
      double wt = recheck_window(p, t, u, ft32, st);
      orc_eval32(t, xi, &sp);
      double wp = recheck_window(p, t, xi, fit32[i], sp);
      if (!(p->flags & ORC_FLAG_NO_RECHECK) && fabs((double)ft32 - (double)fit32[i]) <= wt + wp) {
        ++rechecks;
        if (memcmp(u, xi, sizeof(float) * D) == 0) {  /* identical: a tie */
          acc = 1;
          ft64 = fit64[i];
        } else {
          ft64 = orc_eval64(t, u, NULL, NULL);
          if (isnan(fit64[i])) fit64[i] = orc_eval64(t, xi, NULL, NULL);
          acc = ft64 <= fit64[i];
        }
      } else {
        acc = ft32 <= fit32[i];
      }
    }
    if (accepted) accepted[i] = (uint8_t)acc;
    if (acc) {
      memcpy(xi, u, sizeof(float) * D);
      fit64[i] = ft64;
      fit32[i] = mode == 0 ? (float)ft64 : ft32;
    }
  }
  free(U);
  return rechecks;
}

void orc_rank(const float* fit, int NP, int* rank) {
  for (int i = 0; i < NP; ++i) {
    int r = 0;
    for (int j = 0; j < NP; ++j)
      if (fit[j] < fit[i] || (fit[j] == fit[i] && j < i)) ++r;
    rank[i] = r;
  }
}

/* ------------------------------------------------------------------ */
/* elite transfer (SG-EMTF.cu:1514-1591, launched per partner choice   */
/* :1694-1721): candidate c starts from the receiver's c-th best member */
/* and takes each gene, with probability transfer_mix, from the         */
/* partner's c-th best, remapped linearly from the partner's box to the */
/* receiver's (:1554-1556); it replaces the receiver's member of rank   */
/* NP-k+c when strictly better (:1566-1589).                            */
/* ------------------------------------------------------------------ */
int orc_transfer_partner(const orc_params* p, uint32_t t, uint32_t n_tasks, uint32_t gen) {
  uint32_t w[4];
  orc_draw(p->seed, t, gen, 0, ORC_P_TRANSFER_PARTNER, 0, w);
  if (n_tasks < 2) return (int)t;
  uint32_t q = w[0] % (n_tasks - 1);
  if (q >= t) ++q;
  return (int)q;
}

int orc_transfer_in(const orc_params* p, const orc_task* t, const orc_task* pt,
                    const float* elites, int k, float* X, float* fit32, double* fit64,
                    uint32_t gen, int mode) {
  int D = t->D, NP = t->NP, replaced = 0;
  int* rank = (int*)malloc(sizeof(int) * NP);
  int* byrank = (int*)malloc(sizeof(int) * NP);
  orc_rank(fit32, NP, rank);
  for (int i = 0; i < NP; ++i) byrank[rank[i]] = i;
  float rp = pt->hi - pt->lo, rt = t->hi - t->lo;
  /* candidates are built from the pre-transfer population */
  float* C = (float*)malloc(sizeof(float) * (size_t)k * D);
  uint32_t w[4];
  for (int c = 0; c < k; ++c) {
    const float* own = X + (size_t)byrank[c] * D;
    const float* el = elites + (size_t)c * pt->D;
    for (int j = 0; j < D; ++j) {
      if ((j & 3) == 0) orc_draw(p->seed, t->id, gen, (uint32_t)c, ORC_P_TRANSFER_MIX, (uint32_t)(j >> 2), w);
      float v = own[j];
      if (j < pt->D && orc_u01(w[j & 3]) < p->transfer_mix) {
        float r = (el[j] - pt->lo) / rp;
        v = clampf_box(fmaf(r, rt, t->lo), t->lo, t->hi);
      }
      C[(size_t)c * D + j] = v;
    }
  }
  for (int c = 0; c < k; ++c) {
    int m = byrank[NP - k + c];
    float* cv = C + (size_t)c * D;
    float* xm = X + (size_t)m * D;
    int acc;
    double f64 = NAN;
    float f32 = NAN;
    if (mode == 0) {
      double sc;
      f64 = orc_eval64(t, cv, &sc, NULL);
      if (isnan(fit64[m])) fit64[m] = orc_eval64(t, xm, NULL, NULL);
      acc = decide_exact(t, cv, f64, sc, xm, fit64[m], 1);
    } else {
      float sc, sm;
      f32 = orc_eval32(t, cv, &sc);
      orc_eval32(t, xm, &sm);
      double win = recheck_window(p, t, cv, f32, sc) + recheck_window(p, t, xm, fit32[m], sm);
      if (!(p->flags & ORC_FLAG_NO_RECHECK) && fabs((double)f32 - (double)fit32[m]) <= win) {
        f64 = orc_eval64(t, cv, NULL, NULL);
        if (isnan(fit64[m])) fit64[m] = orc_eval64(t, xm, NULL, NULL);
        acc = f64 < fit64[m];
      } else {
        acc = f32 < fit32[m];
      }
    }
    if (acc) {
      memcpy(xm, cv, sizeof(float) * D);
      fit64[m] = f64;
      fit32[m] = mode == 0 ? (float)f64 : f32;
      ++replaced;
    }
  }
  free(C);
  free(rank);
  free(byrank);
  return replaced;
}

/* ------------------------------------------------------------------ */
/* ring migration between sub-islands                                   */
/* ------------------------------------------------------------------ */
int orc_migration_due(const orc_params* p, uint32_t gen) {
  return p->subislands > 1 && p->mig_interval > 0 && gen > 1u &&
         (gen - 1u) % (uint32_t)p->mig_interval == 0u;
}

int orc_migration_count(const orc_params* p, int NP) {
  const int NPs = NP / (p->subislands > 1 ? p->subislands : 1);
  if (p->mig_count > 0) return p->mig_count;
  const int m = NPs / 8;
  return m < 1 ? 1 : m;
}

int orc_migrate(const orc_params* p, const orc_task* t, float* X, float* fit32, double* fit64,
                int mode) {
  const int D = t->D, NP = t->NP, S = p->subislands > 1 ? p->subislands : 1;
  const int NPs = NP / S, m = orc_migration_count(p, NP), k = S * m;
  int replaced = 0;
  int* byrank = (int*)malloc(sizeof(int) * NP);
  for (int i = 0; i < NP; ++i) { /* rank within the member's sub-island */
    const int base = (i / NPs) * NPs;
    int r = 0;
    for (int j = base; j < base + NPs; ++j)
      if (fit32[j] < fit32[i] || (fit32[j] == fit32[i] && j < i)) ++r;
    byrank[base + r] = i;
  }
  /* candidates are the pre-migration members: c = s * m + r is the r-th best
   * of sub-island s, sent to the r-th worst of sub-island s + 1 (mod S) */
  float* C = (float*)malloc(sizeof(float) * (size_t)k * D);
  int* target = (int*)malloc(sizeof(int) * k);
  for (int c = 0; c < k; ++c) {
    const int s = c / m, r = c - s * m, d = (s + 1) % S;
    memcpy(C + (size_t)c * D, X + (size_t)byrank[s * NPs + r] * D, sizeof(float) * D);
    target[c] = byrank[d * NPs + NPs - 1 - r];
  }
  for (int c = 0; c < k; ++c) {
    const int tm = target[c];
    float* cv = C + (size_t)c * D;
    float* xm = X + (size_t)tm * D;
    int acc;
    double f64 = NAN;
    float f32 = NAN;
    if (mode == 0) {
      double sc;
      f64 = orc_eval64(t, cv, &sc, NULL);
      if (isnan(fit64[tm])) fit64[tm] = orc_eval64(t, xm, NULL, NULL);
      acc = decide_exact(t, cv, f64, sc, xm, fit64[tm], 1);
    } else {
      float sc, sm;
      f32 = orc_eval32(t, cv, &sc);
      orc_eval32(t, xm, &sm);
      double win = recheck_window(p, t, cv, f32, sc) + recheck_window(p, t, xm, fit32[tm], sm);
      if (!(p->flags & ORC_FLAG_NO_RECHECK) && fabs((double)f32 - (double)fit32[tm]) <= win) {
        if (memcmp(cv, xm, sizeof(float) * D) == 0) {
          acc = 0; /* identical: a tie, and migration needs strictly better */
        } else {
          f64 = orc_eval64(t, cv, NULL, NULL);
          if (isnan(fit64[tm])) fit64[tm] = orc_eval64(t, xm, NULL, NULL);
          acc = f64 < fit64[tm];
        }
      } else {
        acc = f32 < fit32[tm];
      }
    }
    if (acc) {
      memcpy(xm, cv, sizeof(float) * D);
      fit64[tm] = f64;
      fit32[tm] = mode == 0 ? (float)f64 : f32;
      ++replaced;
    }
  }
  free(C);
  free(target);
  free(byrank);
  return replaced;
}

/* ------------------------------------------------------------------ */
/* multi-threaded CPU run over tasks                                    */
/* ------------------------------------------------------------------ */
typedef struct {
  const orc_params* p;
  const orc_task* tasks;
  int n;
  float** X;
  float** f32;
  double** f64;
  uint32_t gen0;
  int gens, mode;
  int next;
  pthread_mutex_t mu;
} run_ctx;

static void* run_worker(void* arg) {
  run_ctx* c = (run_ctx*)arg;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int t = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (t >= c->n) break;
    for (int g = 0; g < c->gens; ++g) {
      const uint32_t G = c->gen0 + (uint32_t)g + 1u;
      if (orc_migration_due(c->p, G))
        orc_migrate(c->p, &c->tasks[t], c->X[t], c->f32[t], c->f64[t], c->mode);
      orc_generation(c->p, &c->tasks[t], c->X[t], c->f32[t], c->f64[t], G, c->mode, NULL);
    }
  }
  return NULL;
}

double orc_run_threads(const orc_params* p, const orc_task* tasks, int n, float** X,
                       float** fit32, double** fit64, uint32_t gen0, int gens, int mode,
                       int threads) {
  run_ctx c;
  c.p = p; c.tasks = tasks; c.n = n; c.X = X; c.f32 = fit32; c.f64 = fit64;
  c.gen0 = gen0; c.gens = gens; c.mode = mode; c.next = 0;
  pthread_mutex_init(&c.mu, NULL);
  if (threads < 1) threads = 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, run_worker, &c);
  for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
  clock_gettime(CLOCK_MONOTONIC, &b);
  free(th);
  pthread_mutex_destroy(&c.mu);
  return (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
}
