// Double-float ("FF") arithmetic: a value is the unevaluated sum hi + lo of
// two floats (about 48 significant bits).  Built from the classical
// error-free transformations (Knuth two-sum, Dekker fast-two-sum, FMA-based
// two-product).  Used by the mixed-precision Jacobi so that its rotations run
// on the FP32 pipe at close to FP64 accuracy.
#pragma once

#include "common.cuh"

namespace otb {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(float h, float l) {
  ff r;
  r.hi = h;
  r.lo = l;
  return r;
}
__device__ __forceinline__ ff ff_from(double d) {
  const float h = (float)d;
  return ff_make(h, (float)(d - (double)h));
}
__device__ __forceinline__ double ff_to(ff a) { return (double)a.hi + (double)a.lo; }

// Knuth: s + e == a + b exactly
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff_make(s, e);
}
// Dekker, |a| >= |b|
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return ff_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_make(-b.hi, -b.lo)); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
// acc + a * b
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff acc) { return ff_add(acc, ff_mul(a, b)); }

// 1/sqrt(u) for u > 0: float estimate refined by one Newton step in FF
__device__ __forceinline__ ff ff_rsqrt(ff u) {
  const float y0 = rsqrtf(u.hi);
  const ff y = ff_make(y0, 0.f);
  const ff e = ff_sub(ff_make(1.f, 0.f), ff_mul(u, ff_mul(y, y)));
  return ff_add(y, ff_mul(ff_make(0.5f * y0, 0.f), e));
}

// sqrt(u) for u >= 0: the IEEE float square root refined by one Newton step
// in FF (y + (u - y^2) / (2 y)); 0 for u <= 0
__device__ __forceinline__ ff ff_sqrt(ff u) {
  if (!(u.hi > 0.f)) return ff_make(0.f, 0.f);
  const float y = __fsqrt_rn(u.hi);
  const ff e = ff_sub(u, ff_mul(ff_make(y, 0.f), ff_make(y, 0.f)));
  return ff_add(ff_make(y, 0.f), ff_make(__fdiv_rn(e.hi, 2.f * y), 0.f));
}

// 1 / b for b != 0: the IEEE float reciprocal refined by one Newton step in
// FF (y + y (1 - b y))
__device__ __forceinline__ ff ff_recip(ff b) {
  const float y = __fdiv_rn(1.f, b.hi);
  const ff e = ff_sub(ff_make(1.f, 0.f), ff_mul(b, ff_make(y, 0.f)));
  return ff_add(ff_make(y, 0.f), ff_mul(ff_make(y, 0.f), e));
}

__device__ __forceinline__ ff ff_shfl_xor(ff v, int off) {
  return ff_make(__shfl_xor_sync(0xffffffffu, v.hi, off, 32), __shfl_xor_sync(0xffffffffu, v.lo, off, 32));
}

// complex double-float (16 bytes, one vector load)
struct __align__(16) cff {
  ff x, y;
};

__device__ __forceinline__ cff cff_from(cx<double> z) {
  cff r;
  r.x = ff_from(z.x);
  r.y = ff_from(z.y);
  return r;
}
__device__ __forceinline__ cx<double> cff_to(cff z) { return mk<double>(ff_to(z.x), ff_to(z.y)); }

// Compensated complex multiply-accumulate for contractions: the running sum
// is kept as (hi, lo) per component; every FF x FF product contributes its
// exact leading product through an error-free two-sum into hi and all error
// terms (product and sum errors, cross terms) into lo.  Relative accuracy
// ~n * 2^-47 over an n-term sum, on the FP32 pipe only.
struct ccacc {
  float xh, xl, yh, yl;
};

__device__ __forceinline__ void ffp_acc(float ah, float al, float bh, float bl, float& sh, float& sl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float t = __fadd_rn(sh, p);
  const float bb = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// A compensated accumulator (h, l) -- the exact leading terms through
// two-sum in h, every rounding error and cross term in l (ffp_acc) -- as a
// normalised double-float value.
__device__ __forceinline__ ff ffacc_norm(float h, float l) { return two_sum(h, l); }

__device__ __forceinline__ ccacc ccacc_zero() {
  ccacc a;
  a.xh = a.xl = a.yh = a.yl = 0.f;
  return a;
}

// acc += a * b
__device__ __forceinline__ void ccacc_fma(ccacc& acc, const cff& a, const cff& b) {
  ffp_acc(a.x.hi, a.x.lo, b.x.hi, b.x.lo, acc.xh, acc.xl);
  ffp_acc(-a.y.hi, -a.y.lo, b.y.hi, b.y.lo, acc.xh, acc.xl);
  ffp_acc(a.x.hi, a.x.lo, b.y.hi, b.y.lo, acc.yh, acc.yl);
  ffp_acc(a.y.hi, a.y.lo, b.x.hi, b.x.lo, acc.yh, acc.yl);
}

// acc += conj(a) * b
__device__ __forceinline__ void ccacc_fmaj(ccacc& acc, const cff& a, const cff& b) {
  ffp_acc(a.x.hi, a.x.lo, b.x.hi, b.x.lo, acc.xh, acc.xl);
  ffp_acc(a.y.hi, a.y.lo, b.y.hi, b.y.lo, acc.xh, acc.xl);
  ffp_acc(a.x.hi, a.x.lo, b.y.hi, b.y.lo, acc.yh, acc.yl);
  ffp_acc(-a.y.hi, -a.y.lo, b.x.hi, b.x.lo, acc.yh, acc.yl);
}

// The accumulated value as a double-float complex (no FP64 instruction).
__device__ __forceinline__ cff ccacc_cff(const ccacc& a) {
  cff r;
  r.x = two_sum(a.xh, a.xl);
  r.y = two_sum(a.yh, a.yl);
  return r;
}

__device__ __forceinline__ cff cff_add(const cff& a, const cff& b) {
  cff r;
  r.x = ff_add(a.x, b.x);
  r.y = ff_add(a.y, b.y);
  return r;
}

// a * s for a real double-float s
__device__ __forceinline__ cff cff_scale(const cff& a, ff s) {
  cff r;
  r.x = ff_mul(a.x, s);
  r.y = ff_mul(a.y, s);
  return r;
}

__device__ __forceinline__ cff cff_conj(cff a) {
  a.y.hi = -a.y.hi;
  a.y.lo = -a.y.lo;
  return a;
}

__device__ __forceinline__ cff cff_mul(const cff& a, const cff& b) {
  ccacc f = ccacc_zero();
  ccacc_fma(f, a, b);
  return ccacc_cff(f);
}

__device__ __forceinline__ cx<double> ccacc_value(const ccacc& a) {
  return mk<double>((double)a.xh + (double)a.xl, (double)a.yh + (double)a.yl);
}

}  // namespace otb
