// Pair arithmetic shared by the force kernels and the ensemble kernel.
#pragma once

#include "sol_internal.cuh"

// ---- float-float arithmetic (pairs of FP32 numbers, ~48-bit significand) ------
// Error-free transformations (Knuth's TwoSum, Dekker's FastTwoSum, TwoProduct
// by FMA); the library is built with --fmad=false, so no other contraction
// disturbs them.
__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void ff_fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
  s = a + b;
  e = b - (s - a);
}
__device__ __forceinline__ void ff_two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = __fmaf_rn(a, b, -p);
}

// FP64 -> (hi, lo) floats by integer operations on the bit pattern (no F2F,
// which would occupy the FP64 pipe): hi keeps the leading 24 significant bits
// (truncated), lo the next 24 of the remaining 29 (rounded by I2F).
// |d| outside [2^-126, 2^128) maps to (0, 0); displacements between distinct
// bodies are far inside that range.
__device__ __forceinline__ void ff_from_double(double d, float& h, float& l) {
  const unsigned hi = (unsigned)__double2hiint(d);
  const unsigned lo = (unsigned)__double2loint(d);
  const int e = (int)((hi >> 20) & 0x7FFu);
  const unsigned sign = hi & 0x80000000u;
  const bool in_range = (e >= 897) & (e <= 1150);
  const unsigned hbits = sign | ((unsigned)(e - 896) << 23) | ((hi & 0x000FFFFFu) << 3) | (lo >> 29);
  h = in_range ? __uint_as_float(hbits) : 0.0f;
  const int es = e - 1023 - 52 + 127;  // biased exponent of 2^(E-52)
  const float scale = (es >= 1 && in_range) ? __uint_as_float((unsigned)es << 23) : 0.0f;
  const float m = __uint2float_rn(lo & 0x1FFFFFFFu) * scale;
  l = __uint_as_float(__float_as_uint(m) | sign);
}

// Float-float pair: FP64 displacement (3 DADD, the only FP64 instructions),
// r^2 with exact squares and sums, FP32 rsqrt seed and one Newton correction
// r^-3 = y^3 (1 + 3/2 e + 15/8 e^2) with e = 1 - r^2 y^2 evaluated from exact
// products, G m r^-3 d and the accumulation in float-float.  Pairs closer
// than 1e-12 AU (where r^-3 would leave the FP32 range) take FP64 arithmetic
// and are summed into (fbx, fby, fbz) instead.  Returns r^2 as (hi, lo).
struct FFAcc {
  float h[3], l[3];
};

__device__ __forceinline__ void ff_pair_accumulate(double dxd, double dyd, double dzd, float2 g, FFAcc& A,
                                                   double& fbx, double& fby, double& fbz, float& r2h_out,
                                                   float& r2l_out) {
  float dh[3], dl[3];
  ff_from_double(dxd, dh[0], dl[0]);
  ff_from_double(dyd, dh[1], dl[1]);
  ff_from_double(dzd, dh[2], dl[2]);
  float p1, e1, p2, e2, p3, e3;
  ff_two_prod(dh[0], dh[0], p1, e1);
  ff_two_prod(dh[1], dh[1], p2, e2);
  ff_two_prod(dh[2], dh[2], p3, e3);
  float s12, t12, s3, t3;
  ff_two_sum(p1, p2, s12, t12);
  ff_two_sum(s12, p3, s3, t3);
  float lo = ((t12 + t3) + (e1 + e2)) + e3;
  lo = __fmaf_rn(dh[0] + dh[0], dl[0], lo);
  lo = __fmaf_rn(dh[1] + dh[1], dl[1], lo);
  lo = __fmaf_rn(dh[2] + dh[2], dl[2], lo);
  float r2h, r2l;
  ff_fast_two_sum(s3, lo, r2h, r2l);
  if (r2h < 1.0e-24f && r2h > 0.0f) {  // extremely close pair: FP64 arithmetic
    double r2 = __fma_rn(dxd, dxd, __fma_rn(dyd, dyd, dzd * dzd));
    double rinv = __drcp_rn(__dsqrt_rn(r2));
    double sd = ((double)g.x + (double)g.y) * (rinv * rinv * rinv);
    fbx = __fma_rn(sd, dxd, fbx);
    fby = __fma_rn(sd, dyd, fby);
    fbz = __fma_rn(sd, dzd, fbz);
  } else {
    const float y = rsqrtf(fmaxf(r2h, 1.0e-24f));  // the sink itself: r2 = 0, contribution 0 * d = 0
    float y2, y2e, q, qe;
    ff_two_prod(y, y, y2, y2e);
    ff_two_prod(r2h, y2, q, qe);
    const float e = ((1.0f - q) - qe) - __fmaf_rn(r2h, y2e, r2l * y2);
    float y3h, y3e;
    ff_two_prod(y2, y, y3h, y3e);
    y3e = __fmaf_rn(y2e, y, y3e);
    const float c = e * __fmaf_rn(1.875f, e, 1.5f);
    float Rh, Rl;
    ff_fast_two_sum(y3h, __fmaf_rn(y3h, c, y3e), Rh, Rl);
    float sh, se;
    ff_two_prod(g.x, Rh, sh, se);
    se = __fmaf_rn(g.x, Rl, __fmaf_rn(g.y, Rh, se));
    ff_fast_two_sum(sh, se, sh, se);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float ah, ae;
      ff_two_prod(sh, dh[k], ah, ae);
      ae = __fmaf_rn(sh, dl[k], __fmaf_rn(se, dh[k], ae));
      float s1, s2;
      ff_two_sum(A.h[k], ah, s1, s2);
      s2 = s2 + (A.l[k] + ae);
      ff_fast_two_sum(s1, s2, A.h[k], A.l[k]);
    }
  }
  r2h_out = r2h;
  r2l_out = r2l;
}
