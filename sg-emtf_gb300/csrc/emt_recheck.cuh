// emt_recheck.cuh -- differential re-check of a near-tie selection, FP32/INT
// pipes only.
//
// A selection is re-decided when the FP32 fitness gap of trial u and parent x
// lies inside the rounding window.  In converged islands that is most of them,
// and u and x differ by a few ulps, so what decides is the sign of
// f(u) - f(x), a quantity far smaller than f itself.  This file computes that
// difference directly rather than the two fitness values:
//
//   z  = Q (x - o)       the parent's rotation, by the compensated dot product
//                        (Ogita, Rump, Oishi 2005) kept as float-float z_h + z_l
//                        with a bound on its error; it is cached per member in
//                        HBM and carried forward (z + dz) when a trial replaces
//                        the member;
//   dz = Q (u - x)       from the exact split u - x = d_h + d_l, plain FP32
//                        dot products, error at most gamma_2D |q_n|_2 |u - x|_2;
//   f(u) - f(x) = sum over genes of g(z + dz) - g(z), each difference written
//   in a form without cancellation:
//     z^2:          (2z + dz) dz
//     sin^2(pi z):  sin(pi (2z + dz)) sin(pi dz)      (2z reduced mod 2 exactly)
//     cos(t):       cos(t + dt) / cos(t) = 1 - 2 sin^2(dt/2) - tan(t) sin(dt)
//     z sin sqrt|z|: dz sin r' + 2 z cos((r + r')/2) sin((r' - r)/2),
//                    r' - r = (|z'| - |z|) / (r + r')
//   and the composite functions (Ackley, Griewank) through exp/expm1/log1p of
//   those sums.
//
// Every quantity carries a first-order bound on its distance from the exact
// real value (rounding of each FP32 operation, the library functions' ulp
// error, the error of z and dz).  If |f(u) - f(x)| exceeds the summed bound
// the sign is certain and the selection is decided; otherwise the caller falls
// back to the FP64-class values.  The decision is the exact-arithmetic one,
// so it agrees with any evaluation accurate enough to resolve the same gap.
#pragma once

#include "emt_functions.cuh"

namespace emt {

constexpr uint32_t FLAG_NO_DIFF_RECHECK = 0x40u;

// Functions whose converged islands re-check faster through the differential
// form (measured on GB300, 2000-generation runs of D = 50 islands): Rastrigin,
// Ackley, Griewank, Rosenbrock, Schwefel.  Sphere's near ties are almost all
// bit-identical trials; Weierstrass amplifies dz by 3^k, beyond a first-order
// bound.  Schwefel's converged islands, which otherwise decide every tie with
// double-precision sines on the FP64 pipe, set the length of a Schwefel-only
// launch: 129 -> 113 ms with the differential form (304 islands, TF32X3).
__device__ __forceinline__ bool diff_pays(int fid) {
  return fid == F_RASTRIGIN || fid == F_ACKLEY || fid == F_GRIEWANK || fid == F_ROSENBROCK ||
         fid == F_SCHWEFEL;
}

namespace diffck {

constexpr float kU = 0x1p-24f;   // unit roundoff of FP32
constexpr float kFn = 4.f * kU;  // relative error of a library function (2 ulp)

// sin(pi (h + l)) for a float-float argument: h is reduced mod 2 exactly
// (h - rint(h) is exact), the remainder rounded once.  *r receives the reduced
// argument, whose rounding error is below u (|r| + |l|).
__device__ __forceinline__ float sinpi_ff(float h, float l, float* r) {
  const float n = rintf(h);
  const float rr = __fadd_rn(__fsub_rn(h, n), l);
  *r = rr;
  const float s = sinpif(rr);
  return (__float2int_rn(fmodf(n, 2.f)) != 0) ? -s : s;
}

struct Acc {
  float d = 0.f;  // sum of difference terms
  float e = 0.f;  // sum of their error bounds
  float m = 0.f;  // sum of their magnitudes (summation error)
  __device__ __forceinline__ void add(float t, float et) {
    d += t;
    e += et;
    m += fabsf(t);
  }
};

// w = 2z + dz with its bound; t2 = 2 z_l + dz is returned for the reductions.
__device__ __forceinline__ float twice_plus(float zh, float zl, float dz, float ez, float edz,
                                            float* t2, float* ew) {
  const float t = __fmaf_rn(2.f, zl, dz);
  const float w = __fmaf_rn(2.f, zh, t);
  *t2 = t;
  *ew = kU * (fabsf(t) + fabsf(w)) + 2.f * ez + edz;
  return w;
}

// (2z + dz) dz, the difference of z^2
__device__ __forceinline__ void sq_diff(float w, float ew, float dz, float edz, float* v,
                                        float* e) {
  const float p = __fmul_rn(w, dz);
  *v = p;
  *e = kU * fabsf(p) + ew * fabsf(dz) + (fabsf(w) + ew) * edz;
}

// sin^2(pi z') - sin^2(pi z) = sin(pi (2z + dz)) sin(pi dz)
__device__ __forceinline__ void sin2_diff(float zh, float t2, float ez, float edz, float dz,
                                          float* v, float* e) {
  float r;
  const float sw = sinpi_ff(2.f * zh, t2, &r);
  const float esw =
      3.1415927f * (kU * (fabsf(r) + fabsf(t2)) + 2.f * ez + edz) + kFn * fabsf(sw);
  const float sd = sinpif(dz);
  const float esd = 3.1415927f * edz + kFn * fabsf(sd);
  const float p = __fmul_rn(sw, sd);
  *v = p;
  *e = kU * fabsf(p) + fabsf(sw) * esd + fabsf(sd) * esw + esw * esd;
}

}  // namespace diffck

// Row differences a - b split exactly, a_k - b_k = h_k + l_k (pairs in pr),
// by the calling warp; returns sqrt(sum (|h_k| + |l_k|)^2), rounded up, on
// every lane.  It serves the Cauchy-Schwarz error bounds below:
// sum_k |q_nk| (|h_k| + |l_k|) <= |q_n|_2 * that.
__device__ __forceinline__ float split_rows(const float* __restrict__ a,
                                            const float* __restrict__ b, int D, float2* pr) {
  const int lane = threadIdx.x & 31;
  float ss = 0.f;
  for (int k = lane; k < D; k += 32) {
    float h, l;
    two_sum(a[k], -b[k], h, l);
    pr[k] = make_float2(h, l);
    const float m = __fadd_ru(fabsf(h), fabsf(l));
    ss = __fmaf_ru(m, m, ss);
  }
  ss = warp_sum(ss);
  __syncwarp();
  return __fsqrt_ru(ss * (1.f + 0x1p-18f));
}

// The calling warp writes the compensated rotation z = Q (x - o) of row x as
// float-float (zh, zl, D entries each, any memory) and returns a bound on
// max_n |z_n - z_exact,n|, the same on every lane: the Dot2 bound over 2D + 2
// terms, gamma^2 sum_k |q_nk| |x_k - o_k| <= gamma^2 qnorm |x - o|_2, doubled.
// *zmax receives max_n |z_n|; pr is D float2 of scratch.
__device__ __noinline__ float anchor_rotation(const float* __restrict__ x, const float* __restrict__ o,
                                 const float* __restrict__ qt, int DP, int D, float qnorm,
                                 float* zh, float* zl, float* zmax, float2* pr) {
  using namespace diffck;
  const int lane = threadIdx.x & 31;
  const float gz = (float)(2 * D + 2) * kU;
  const float cz = 2.f * (gz * gz + (float)(D + 1) * kU * kU);
  const float sn = split_rows(x, o, D, pr);
  float zm = 0.f;
  for (int n = lane; n < D; n += 64) {
    const bool two = n + 32 < D;
    const int m = two ? n + 32 : n;
    float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
    for (int k = 0; k < D; ++k) {
      const float2 hl = pr[k];
      const float q0 = qt[k * DP + n], q1 = qt[k * DP + m];
      const float p0 = __fmul_rn(q0, hl.x), p1 = __fmul_rn(q1, hl.x);
      const float e0 = __fmaf_rn(q0, hl.x, -p0), e1 = __fmaf_rn(q1, hl.x, -p1);
      float t0, te0, t1, te1;
      two_sum(S0, p0, t0, te0);
      two_sum(S1, p1, t1, te1);
      S0 = t0;
      S1 = t1;
      C0 = __fmaf_rn(q0, hl.y, __fadd_rn(C0, __fadd_rn(te0, e0)));
      C1 = __fmaf_rn(q1, hl.y, __fadd_rn(C1, __fadd_rn(te1, e1)));
    }
    float h, l;
    two_sum(S0, C0, h, l);
    zh[n] = h;
    zl[n] = l;
    zm = fmaxf(zm, fabsf(h));
    if (two) {
      two_sum(S1, C1, h, l);
      zh[m] = h;
      zl[m] = l;
      zm = fmaxf(zm, fabsf(h));
    }
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) zm = fmaxf(zm, __shfl_xor_sync(0xFFFFFFFFu, zm, s));
  *zmax = zm;
  __syncwarp();
  return cz * qnorm * sn * 1.0625f + 1e-37f;
}

// dz = Q (to - from) into buf[0..D), its error bound into buf[DP..DP+D):
// gamma_2D sum_k |q_nk| |to_k - from_k| <= gamma_2D qnorm |to - from|_2 (one
// value for every n).  pr: D float2 of scratch.  Calling warp.
__device__ __forceinline__ void row_offset(const float* __restrict__ from,
                                           const float* __restrict__ to,
                                           const float* __restrict__ qt, int DP, int D,
                                           float qnorm, float* buf, float2* pr) {
  using namespace diffck;
  const int lane = threadIdx.x & 31;
  const float g2d = (float)(2 * D) * kU / (1.f - (float)(2 * D) * kU);
  const float dn = split_rows(to, from, D, pr);
  const float ed = g2d * qnorm * dn * (1.f + 16.f * kU) + 1e-37f;
  for (int n = lane; n < D; n += 64) {
    const bool two = n + 32 < D;
    const int m = two ? n + 32 : n;
    float d0 = 0.f, d1 = 0.f;
    for (int k = 0; k < D; ++k) {
      const float2 hl = pr[k];
      const float q0 = qt[k * DP + n], q1 = qt[k * DP + m];
      d0 = __fmaf_rn(q0, hl.x, __fmaf_rn(q0, hl.y, d0));
      d1 = __fmaf_rn(q1, hl.x, __fmaf_rn(q1, hl.y, d1));
    }
    buf[n] = d0;
    buf[DP + n] = ed;
    if (two) {
      buf[m] = d1;
      buf[DP + m] = ed;
    }
  }
  __syncwarp();
}

// Sign of f(to) - f(from) by the calling warp, from the anchor z = Q (from - o)
// (bzh/bzl, error at most ez).  Returns 1 when f(to) < f(from) is certain, 0
// when f(to) > f(from) is certain, -1 when the bound cannot separate them or
// the function has no difference form here.  buf: 4 * DP floats of per-warp
// scratch; its first 2 * DP receive dz = Q (to - from) and its bound, for the
// caller's cache update.
__device__ __noinline__ int diff_decide(const FnConst& fc, const float* __restrict__ bzh,
                           const float* __restrict__ bzl, float ez, const float* __restrict__ from,
                           const float* __restrict__ to, const float* __restrict__ qt, int DP,
                           float* buf) {
  using namespace diffck;
  if (fc.fid == F_WEIERSTRASS) return -1;
  const int lane = threadIdx.x & 31, D = fc.D;
  const float* bdz = buf;
  const float* bed = buf + DP;
  row_offset(from, to, qt, DP, D, fc.qnorm * (1.f + 0x1p-20f), buf,
             reinterpret_cast<float2*>(buf + 2 * DP));

  // ---- per-gene differences g(z + dz) - g(z) ----
  Acc P, S;                  // primary sum; secondary (Ackley: sin^2 part)
  float A = 0.f, B = 0.f;    // Ackley: anchor sums of z^2 and sin^2(pi z)
  float Lm = 0.f, Ls = 0.f, Le = 0.f, rP = 0.f, Pt = 1.f;  // Griewank log-ratio sums
  int bad = 0;
  for (int j = lane; j < D; j += 32) {
    const float zh = bzh[j], zl = bzl[j], dz = bdz[j], edz = bed[j];
    float t2, ew, v, e;
    const float w = twice_plus(zh, zl, dz, ez, edz, &t2, &ew);
    switch (fc.fid) {
      case F_SPHERE:
        sq_diff(w, ew, dz, edz, &v, &e);
        P.add(v, e);
        break;
      case F_RASTRIGIN: {
        sq_diff(w, ew, dz, edz, &v, &e);
        P.add(v, e);
        sin2_diff(zh, t2, ez, edz, dz, &v, &e);
        P.add(20.f * v, 20.f * e + 20.f * kU * fabsf(v));
        break;
      }
      case F_ACKLEY: {
        sq_diff(w, ew, dz, edz, &v, &e);
        P.add(v, e);
        sin2_diff(zh, t2, ez, edz, dz, &v, &e);
        S.add(v, e);
        A = __fmaf_rn(zh, zh, A);
        const float sp = sinpif(zh);
        B = __fmaf_rn(sp, sp, B);
        break;
      }
      case F_GRIEWANK: {
        sq_diff(w, ew, dz, edz, &v, &e);
        P.add(v, e);
        if (!(fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT)) {
          const float rs = __frsqrt_rn((float)(j + 1));
          const float th = __fmaf_rn(zh, rs, __fmul_rn(zl, rs));
          const float eth = 3.f * kU * fabsf(th) + ez * rs;
          const float dt = __fmul_rn(dz, rs);
          const float edt = edz * rs + 2.f * kU * fabsf(dt);
          float st, ct;
          sincosf(th, &st, &ct);
          if (fabsf(ct) < 0x1p-8f) {
            bad = 1;
            break;
          }
          const float tn = __fdiv_rn(st, ct);
          const float sd = sinf(dt), hh = sinf(0.5f * dt);
          const float q2 = __fmul_rn(2.f, __fmul_rn(hh, hh));
          const float tsd = __fmul_rn(tn, sd);
          const float vv = __fsub_rn(-q2, tsd);
          if (vv <= -1.f + 0x1p-8f) {
            bad = 1;
            break;
          }
          // rounding and library errors: q2 ~ 10u, tan * sin ~ 14u relative
          const float ev = 16.f * kU * (q2 + fabsf(tsd)) + kU * fabsf(vv) +
                           (fabsf(sd) + fabsf(tn)) * edt + fabsf(sd) / (ct * ct) * eth;
          const float L = log1pf(vv);
          Ls += L;
          Lm += fabsf(L);
          Le += ev / (1.f + vv) * 1.0625f + kFn * fabsf(L);
          Pt *= ct;
          rP += fabsf(tn) * eth;
        }
        break;
      }
      case F_SCHWEFEL: {
        // h(z) = z sin(sqrt|z|); f = const - sum h, so the difference is -sum dh
        const float sg = zh < 0.f ? -1.f : 1.f;
        const float azh = fabsf(zh), azl = sg * zl, ad = sg * dz;
        const float az2 = __fadd_rn(azh, __fadd_rn(azl, ad));  // |z'| if the sign holds
        if (azh < 0x1p-4f || az2 < 0x1p-5f) {
          bad = 1;
          break;
        }
        const float r0 = sqrtf(azh);
        const float r = __fmaf_rn(azl, __fdiv_rn(0.5f, r0), r0);
        const float er = 3.f * kU * r + (ez + fabsf(azl) * fabsf(azl) / azh) / (2.f * r0);
        const float rp0 = sqrtf(az2);
        const float den = __fadd_rn(r, rp0);
        const float dr = __fdiv_rn(ad, den);
        const float edr =
            fabsf(dr) * 8.f * kU + (edz + 4.f * kU * (fabsf(azl) + fabsf(ad))) / den;
        const float rp = __fadd_rn(r, dr);
        const float erp = er + edr + kU * rp;
        const float mm = __fmaf_rn(0.5f, dr, r);
        const float em = er + 0.5f * edr + kU * mm;
        const float srp = sinf(rp);
        const float t1 = __fmul_rn(dz, srp);
        const float et1 =
            fabsf(srp) * edz + fabsf(dz) * (kFn * fabsf(srp) + erp) + kU * fabsf(t1);
        float sm, cm;
        sincosf(mm, &sm, &cm);
        const float sh2 = sinf(0.5f * dr);
        const float zz = __fadd_rn(zh, zl);
        const float t2v = __fmul_rn(__fmul_rn(2.f * zz, cm), sh2);
        const float et2 =
            fabsf(t2v) * (3.f * kU + 2.f * kFn + (ez + kU * fabsf(zz)) / fabsf(zz)) +
            fabsf(2.f * zz * sh2) * fabsf(sm) * em + fabsf(zz * cm) * edr;
        P.add(-t1, et1);
        P.add(-t2v, et2);
        break;
      }
      case F_ROSENBROCK: {
        if (j + 1 >= D) break;
        const float zh1 = bzh[j + 1], zl1 = bzl[j + 1], dz1 = bdz[j + 1], edz1 = bed[j + 1];
        // t = z_j^2 - z_{j+1} in float-float
        const float p = __fmul_rn(zh, zh), pe = __fmaf_rn(zh, zh, -p);
        float th, te;
        two_sum(p, -zh1, th, te);
        const float cr = __fmul_rn(2.f * zh, zl);
        const float small = __fadd_rn(__fadd_rn(te, pe), __fsub_rn(cr, zl1));
        const float t = __fadd_rn(th, small);
        const float et = kU * fabsf(t) +
                         4.f * kU * (fabsf(te) + fabsf(pe) + fabsf(cr) + fabsf(zl1)) +
                         2.f * kU * kU * zh * zh + (2.f * fabsf(zh) + 1.f) * ez + ez * ez;
        // dt = (2 z_j + dz_j) dz_j - dz_{j+1}
        const float dt = __fmaf_rn(w, dz, -dz1);
        const float edt = kU * fabsf(dt) + ew * fabsf(dz) + (fabsf(w) + ew) * edz + edz1;
        const float s2 = __fmaf_rn(2.f, t, dt);
        const float es2 = kU * fabsf(s2) + 2.f * et + edt;
        const float q = __fmul_rn(s2, dt);
        const float eq = kU * fabsf(q) + fabsf(s2) * edt + fabsf(dt) * es2 + es2 * edt;
        P.add(100.f * q, 100.f * eq + 100.f * kU * fabsf(q));
        // (z_j - 1)^2 difference: (2 (z_j - 1) + dz_j) dz_j
        const float c1 = __fsub_rn(zh, 1.f);
        const float tt = __fmaf_rn(2.f, zl, dz);
        const float y = __fmaf_rn(2.f, c1, tt);
        const float ey = 2.f * kU * fabsf(c1) + kU * (fabsf(y) + fabsf(tt)) + 2.f * ez + edz;
        const float r2 = __fmul_rn(y, dz);
        P.add(r2, kU * fabsf(r2) + ey * fabsf(dz) + (fabsf(y) + ey) * edz);
        break;
      }
      default:
        bad = 1;
        break;
    }
  }
  if (__any_sync(0xFFFFFFFFu, bad)) return -1;
  // ---- reduce and combine ----
  const float g9 = 9.f * kU;
  const float Dp = warp_sum(P.d), Ep = warp_sum(P.e), Mp = warp_sum(P.m);
  float delta = Dp, err = Ep + g9 * Mp;
  if (fc.fid == F_ACKLEY) {
    // f = -20 expm1(-0.2 sqrt(A/D)) - e expm1(-2B/D) + const
    const float dA = Dp, eA = err;
    const float dB = warp_sum(S.d), eB = warp_sum(S.e) + g9 * warp_sum(S.m);
    A = warp_sum(A);
    B = warp_sum(B);
    const float Df = (float)D;
    const float at = sqrtf(A / Df), ap = sqrtf(fmaxf(A + dA, 0.f) / Df);
    if (!(at + ap > 1e-30f)) return -1;
    const float da = (dA / Df) / (at + ap);
    const float EA = expf(-0.2f * at), EB = expf(-2.f * B / Df);
    const float TA = -20.f * EA * expm1f(-0.2f * da);
    const float TB = -2.7182817f * EB * expm1f(-2.f * dB / Df);
    const float sA = 20.f * EA * 0.2f / (Df * (at + ap)) * expf(0.2f * fabsf(da)) * 1.0625f;
    const float sB = 2.7182817f * EB * (2.f / Df) * expf(2.f * fabsf(dB) / Df) * 1.0625f;
    const float rel = 32.f * kU + Df * kU * (2.f + 0.2f * at + 2.f * B / Df);
    delta = TA + TB;
    err = sA * eA + fabsf(TA) * rel + sB * eB + fabsf(TB) * rel + 2.f * kU * fabsf(delta);
  } else if (fc.fid == F_GRIEWANK) {
    // f = 1 - prod cos + A/4000: the difference is -P expm1(sum L) + dA/4000
    const float TA = Dp / 4000.f, eTA = err / 4000.f + kU * fabsf(TA);
    float TP = 0.f, eTP = 0.f;
    if (!(fc.flags & FLAG_REF_GRIEWANK_NO_PRODUCT)) {
      const float Lsum = warp_sum(Ls), Lerr = warp_sum(Le) + g9 * warp_sum(Lm);
      const float Pp = warp_prod(Pt), rp = warp_sum(rP) + 6.f * (float)(D + 2) * kU;
      TP = -Pp * expm1f(Lsum);
      eTP = fabsf(Pp) * expf(fabsf(Lsum)) * Lerr * 1.0625f + fabsf(TP) * (rp + 8.f * kU);
    }
    delta = TA + TP;
    err = eTA + eTP + kU * fabsf(delta);
  }
  err = err * 1.125f + 1e-30f;
  if (!isfinite(delta) || !isfinite(err)) return -1;
  if (delta < -err) return 1;  // f(to) < f(from)
  if (delta > err) return 0;   // f(to) > f(from)
  return -1;
}

// Carries a cached anchor forward to the row that just replaced it:
// z <- z + dz (dz and its bound from row_offset in buf) as float-float, in
// place.  Returns the new error bound: ez plus the largest dz bound plus the
// renormalisation.
__device__ float anchor_advance(float* zh, float* zl, const float* buf, int DP, int D, float ez) {
  using namespace diffck;
  const int lane = threadIdx.x & 31;
  float em = 0.f;
  for (int n = lane; n < D; n += 32) {
    float s1, e1, h, l;
    two_sum(zh[n], buf[n], s1, e1);
    const float e2 = __fadd_rn(e1, zl[n]);
    two_sum(s1, e2, h, l);
    zh[n] = h;
    zl[n] = l;
    em = fmaxf(em, buf[DP + n] + 2.f * kU * fabsf(e2));
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) em = fmaxf(em, __shfl_xor_sync(0xFFFFFFFFu, em, s));
  __syncwarp();
  return (ez + em) * 1.0625f;
}

}  // namespace emt
