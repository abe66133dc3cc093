// Double-float arithmetic on the FP32 pipes (error-free transformations):
// a value is hi + lo with |lo| <= ulp(hi) / 2, about 2^-46 of relative
// precision.  Products: a*b = ph + pl exactly (ph = fl(a*b), pl = fma(a, b,
// -ph)); sums: TwoSum of the high parts (Knuth), with the low parts and the
// cross terms a_hi*b_lo + a_lo*b_hi accumulated in FP32.  Used by the
// exact precision mode's working states (exact.cu) and by the refinement
// products of stage (a)'s blocked eigensolver (ttsvd_wide.cu).
#pragma once

#include "device_common.cuh"
#include "exact.h"

__device__ __forceinline__ xc xc_from_d(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, ih, __double2float_rn(v.x - (double)rh), __double2float_rn(v.y - (double)ih));
}

__device__ __forceinline__ double2 xc_to_d(xc v) { return cd((double)v.x + (double)v.z, (double)v.y + (double)v.w); }

// s += (ah + al)(bh + bl): the high product exactly (ph + pl), TwoSum into
// s.hi, everything of lower order into s.lo.  Explicitly rounded
// intrinsics keep the compiler from contracting the error terms.
__device__ __forceinline__ void df_mac(DF& s, float ah, float al, float bh, float bl) {
  const float ph = __fmul_rn(ah, bh);
  const float pl = __fmaf_rn(ah, bh, -ph);
  const float t = __fadd_rn(s.hi, ph);
  const float bv = __fsub_rn(t, s.hi);
  const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bv)), __fsub_rn(ph, bv));
  s.hi = t;
  s.lo = __fadd_rn(s.lo, __fadd_rn(err, __fmaf_rn(ah, bl, __fmaf_rn(al, bh, pl))));
}

struct XA {
  DF re, im;
};

__device__ __forceinline__ XA xa_zero() {
  XA a;
  a.re = DF{0.f, 0.f};
  a.im = DF{0.f, 0.f};
  return a;
}

// a += g x
__device__ __forceinline__ void xa_mac(XA& a, xc g, xc x) {
  df_mac(a.re, g.x, g.z, x.x, x.z);
  df_mac(a.re, -g.y, -g.w, x.y, x.w);
  df_mac(a.im, g.x, g.z, x.y, x.w);
  df_mac(a.im, g.y, g.w, x.x, x.z);
}

// a += conj(u) v
__device__ __forceinline__ void xa_macc(XA& a, xc u, xc v) {
  df_mac(a.re, u.x, u.z, v.x, v.z);
  df_mac(a.re, u.y, u.w, v.y, v.w);
  df_mac(a.im, u.x, u.z, v.y, v.w);
  df_mac(a.im, -u.y, -u.w, v.x, v.z);
}

__device__ __forceinline__ float2 df_norm(DF s) {
  const float h = __fadd_rn(s.hi, s.lo);
  return make_float2(h, __fsub_rn(s.lo, __fsub_rn(h, s.hi)));
}

__device__ __forceinline__ xc xa_round(const XA& a) {
  const float2 r = df_norm(a.re), i = df_norm(a.im);
  return make_float4(r.x, i.x, r.y, i.y);
}

__device__ __forceinline__ double2 xa_to_d(const XA& a) {
  return cd((double)a.re.hi + (double)a.re.lo, (double)a.im.hi + (double)a.im.lo);
}

__device__ __forceinline__ xc xc_conj(xc a) { return make_float4(a.x, -a.y, a.z, -a.w); }
