// Pair arithmetic shared by the force kernels and the ensemble kernel.
#pragma once

#include "sol_internal.cuh"

// MUFU reciprocal square root of a positive normal float: rsqrt.approx.ftz
// gives rsqrtf's approximation without its scaling of subnormal inputs (one
// instruction instead of a test, two multiplies and a selection).  Every
// caller passes a normal argument.
__device__ __forceinline__ float sol_rsqrt_normal(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

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
    const float y = sol_rsqrt_normal(fmaxf(r2h, 1.0e-24f));  // the sink itself: r2 = 0, contribution 0 * d = 0
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

// ---- FP32 seed, FP64 Newton step: the pieces that stay off the FP64 pipe ----
// The FP32 seed y (positive, normal) as a double (exact), y^2 and y^3 in FP64
// without FP64 instructions: from y's 24-bit significand m by integer
// multiplies, y^2 = m^2 (48 bits, exact) and y^3 = m^3 (72 bits, truncated to
// 53), with the exponents set directly.
__device__ __forceinline__ double sol_seed_double(float yf) {
  const int b = __float_as_int(yf);
  return __hiloint2double((b >> 3) + 0x38000000, b << 29);
}
__device__ __forceinline__ void sol_seed_square_cube(float yf, double& u, double& y3) {
  const unsigned b = __float_as_uint(yf);
  const int E = (int)(b >> 23) - 127;  // yf = 2^E m 2^-23
  const unsigned long long m = (b & 0x7FFFFFu) | 0x800000u;
  const unsigned long long m2 = m * m;  // [2^46, 2^48)
  const int c2 = (int)(m2 >> 47);       // m^2 >= 2^47: one more binade
  u = __longlong_as_double(((long long)(2 * E + c2 + 1023) << 52) | ((m2 << (6 - c2)) & 0xFFFFFFFFFFFFFull));
  // m^3 / 2^16 = (m2_hi m) 2^16 + (m2_lo m) / 2^16, in [2^53, 2^56)
  const unsigned long long t = (((m2 >> 32) * m) << 16) + (((m2 & 0xFFFFFFFFull) * m) >> 16);
  const int p = 63 - __clzll((long long)t);  // 53, 54 or 55
  y3 = __longlong_as_double(((long long)(3 * E + p - 53 + 1023) << 52) | ((t >> (p - 52)) & 0xFFFFFFFFFFFFFull));
}
__device__ __forceinline__ double sol_seed_square(float yf) {
  const unsigned b = __float_as_uint(yf);
  const int E = (int)(b >> 23) - 127;
  const unsigned long long m = (b & 0x7FFFFFu) | 0x800000u;
  const unsigned long long m2 = m * m;
  const int c2 = (int)(m2 >> 47);
  return __longlong_as_double(((long long)(2 * E + c2 + 1023) << 52) | ((m2 << (6 - c2)) & 0xFFFFFFFFFFFFFull));
}

// 1 + c e^2 in FP64 (0 <= c <= 2) from e's high word: for a Newton residual
// (|e| < 2^-20) the term is below 2^-37 and is needed to 2^-53, i.e. to 16 of
// its own bits, which FP32 gives; it is placed in the low bits of 1.0 by an
// integer addition.  Larger |e| (only a pair at r^2 = 0, whose seed is
// clamped) is clamped so that the result stays finite.
__device__ __forceinline__ double sol_one_plus_ce2(double e, float c) {
  const int eh = __double2hiint(e);
  const int ex = (eh >> 20) & 0x7FF;
  const int fx = min(ex, 0x47E) - 0x380;  // float exponent field of |e|
  const float ef = fx > 0 ? __int_as_float((fx << 23) | ((eh & 0xFFFFF) << 3)) : 0.0f;
  const float q = fminf(c * ef * ef, 4.656612873077393e-10f);  // <= 2^-31
  const float t = __fmaf_rn(q, 4503599627370496.0f, 12582912.0f);  // q 2^52 + 1.5 2^23: rounds to an integer
  return __longlong_as_double(0x3FF0000000000000LL + (long long)(__float_as_int(t) - 0x4B400000));
}

// t = 3/2 e + 15/8 e^2 in FP64 without FP64 instructions, for the Newton
// correction r^-3 = y^3 (1 + t) of a residual e (|e| < 2^-20 for a seed of
// r^2; e = 1 for r^2 = 0, whose displacement is 0).  3/2 e is 3 M exactly,
// M e's 53-bit significand, in units of half e's last place; 15/8 e^2
// (below 2^-37, from e's high word in FP32) is shifted into the same units
// and added as an integer, and the sum is normalised to 53 bits
// (truncated): t is needed to 2^-53 absolute, i.e. to ~32 of its own bits,
// and carries ~2^-52 relative.  No special cases, since a test of e's bits
// for zero or infinity is turned back into an FP64 comparison by the
// compiler (measured: one FP64 instruction per pair): e = 0 or subnormal
// gives |t| < 2^-1020, which leaves y^3 (1 + t) = y^3, and a non-finite e
// comes with a non-finite displacement that the accumulation carries.
__device__ __forceinline__ double sol_split_t(double e) {
  const long long eb = __double_as_longlong(e);
  const int ex = (int)((eb >> 52) & 0x7FF);
  const long long M = (eb & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  long long S = 3 * M;  // 3/2 e in units of 2^(ex - 1076)
  if (eb < 0) S = -S;
  // 15/8 e^2 from e's high word (as sol_one_plus_ce2), clamped to 2^-31
  const int eh = (int)(eb >> 32);
  const int fx = min(ex, 0x47E) - 0x380;
  const float ef = fx > 0 ? __int_as_float((fx << 23) | ((eh & 0xFFFFF) << 3)) : 0.0f;
  const float q = fminf(1.875f * ef * ef, 4.656612873077393e-10f);
  const int qb = __float_as_int(q);
  const long long mq = (long long)((qb & 0x7FFFFF) | 0x800000);
  const int sq = ((qb >> 23) & 0xFF) + 926 - ex;  // q = mq 2^(eq - 150), in units of 2^(ex - 1076)
  const long long Q = qb == 0 ? 0 : (sq >= 0 ? (mq << min(sq, 38)) : (mq >> min(-sq, 62)));
  S += Q;
  const unsigned long long A = (unsigned long long)(S < 0 ? -S : S);
  const int p = 63 - __clzll((long long)A);  // leading bit (A > 0 when e != 0)
  const unsigned long long mant = p >= 52 ? (A >> (p - 52)) : (A << (52 - p));
  const long long bits = ((S < 0 ? 1LL : 0LL) << 63) | ((long long)(p + ex - 53) << 52) |
                         (long long)(mant & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double(bits);
}

// FP64 r^2 -> FP32 by truncation of the high word, clamped to the normal FP32
// range (r^2 == 0 gives a finite seed), and its rsqrt seed.
__device__ __forceinline__ float sol_rsqrt_seed(double r2) {
  int hi = __double2hiint(r2);
  hi = min(max(hi, 0x38100000), 0x47EFFFFF);
  return sol_rsqrt_normal(__int_as_float((hi - 0x38000000) << 3));
}

// ---- paired FP32 (f32x2): one instruction computes two lanes ----------------
// Blackwell's paired FP32 arithmetic (add / sub / mul / fma .f32x2, round to
// nearest even per lane) halves the instruction count of float-float code
// that processes two sources at once.
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(r)
      : "l"(*reinterpret_cast<const unsigned long long*>(&a)), "l"(*reinterpret_cast<const unsigned long long*>(&b)));
  return *reinterpret_cast<const float2*>(&r);
}
__device__ __forceinline__ float2 f2_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2_splat(float v) { return make_float2(v, v); }
// TwoSum (Knuth), FastTwoSum (Dekker, |a| >= |b| or a == 0), TwoProduct by FMA
__device__ __forceinline__ void f2_two_sum(float2 a, float2 b, float2& s, float2& e) {
  s = f2_add(a, b);
  const float2 bb = f2_sub(s, a);
  e = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
}
__device__ __forceinline__ void f2_fast_two_sum(float2 a, float2 b, float2& s, float2& e) {
  s = f2_add(a, b);
  e = f2_sub(b, f2_sub(s, a));
}
__device__ __forceinline__ void f2_two_prod(float2 a, float2 b, float2& p, float2& e) {
  p = f2_mul(a, b);
  e = f2_fma(a, b, f2_neg(p));
}

// ---- displacement from grid triples (the SPLIT_FF 2-D kernel) ----------------
// Every coordinate is stored as x = a + b + c: a a multiple of the grid G1
// (|a| <= 2^23 G1), b a multiple of G2 = G1 2^-24 (|b| <= G1 / 2), c the
// float nearest the rest (|c| <= G2 / 2), G1 a power of two with every |x|
// below 2^23 G1.  Then a_j - a_i and b_j - b_i are exact in FP32 (multiples
// of one grid, at most 2^24 of it), and
//   d = (a_j - a_i) + (b_j - b_i) + (c_j - c_i)
// is formed as a float-float (h, l) with an absolute error below ~2^-22 G2,
// i.e. 2^-46 |d| for |d| >= G1 / 2: the FastTwoSum of the two exact parts
// (|a_j - a_i| >= G1 >= |b_j - b_i| unless a_j = a_i) and the rounded c part
// added to its low word.  For |d| >= G1 (every pair this form serves) the
// low word stays below 2^-23 |h| (half an ulp of h plus |c_j - c_i| <= G2),
// close enough to normalised for the products that follow.  No FP64
// instruction.
__device__ __forceinline__ void f2_grid_disp(float2 aj, float2 bj, float2 cj, float ai, float bi, float ci, float2& h,
                                             float2& l) {
  const float2 s1 = f2_sub(aj, f2_splat(ai));
  const float2 s2 = f2_sub(bj, f2_splat(bi));
  const float2 s3 = f2_sub(cj, f2_splat(ci));
  float2 l0;
  f2_fast_two_sum(s1, s2, h, l0);
  l = f2_add(l0, s3);
}

// TwoSum of two non-negative numbers: FastTwoSum with the larger first (the
// ordering by max / min runs on the integer pipe).
__device__ __forceinline__ void f2_two_sum_pos(float2 a, float2 b, float2& s, float2& e) {
  const float2 big = make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y));
  const float2 small = make_float2(fminf(a.x, b.x), fminf(a.y, b.y));
  s = f2_add(a, b);
  e = f2_add(f2_sub(big, s), small);
}

// r^2 = sum_k (h_k + l_k)^2 as a float-float (exact squares of the high
// words, TwoSum of the three non-negative squares, the cross terms
// 2 sum_k h_k l_k and the squares' errors in the low word).
__device__ __forceinline__ void f2_ff_r2(const float2* h, const float2* l, float2& r2h, float2& r2l) {
  float2 p[3], e[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) f2_two_prod(h[k], h[k], p[k], e[k]);
  float2 s12, t12, s3, t3;
  f2_two_sum_pos(p[0], p[1], s12, t12);
  f2_two_sum_pos(s12, p[2], s3, t3);
  float2 lo = f2_add(f2_add(t12, t3), f2_add(f2_add(e[0], e[1]), e[2]));
  const float2 cross = f2_fma(h[0], l[0], f2_fma(h[1], l[1], f2_mul(h[2], l[2])));
  lo = f2_fma(f2_splat(2.0f), cross, lo);
  f2_fast_two_sum(s3, lo, r2h, r2l);
}

// G m r^-3 as a float-float from r^2 = (qh, ql): the FP32 rsqrt seed y, the
// residual e = 1 - r^2 y^2 from exact products, r^-3 = y^3 (1 + 3/2 e +
// 15/8 e^2) (|e| < 2^-21: truncation ~2^-60), times G m = (gh, gl).  The
// product is left unnormalised: its low word, the TwoProduct error and the
// two cross terms, stays within 3 2^-24 of the high word, and the
// accumulation that takes it multiplies it by the displacement with one
// rounding (f2_ff_accumulate).
__device__ __forceinline__ void f2_ff_gm_rinv3(float2 qh, float2 ql, float2 gh, float2 gl, float2& sh, float2& se) {
  const float2 y = make_float2(sol_rsqrt_normal(qh.x), sol_rsqrt_normal(qh.y));
  float2 y2, y2e, q, qe;
  f2_two_prod(y, y, y2, y2e);
  f2_two_prod(qh, y2, q, qe);
  const float2 e = f2_sub(f2_sub(f2_sub(f2_splat(1.0f), q), qe), f2_fma(qh, y2e, f2_mul(ql, y2)));
  float2 y3h, y3e;
  f2_two_prod(y2, y, y3h, y3e);
  y3e = f2_fma(y2e, y, y3e);
  const float2 c = f2_mul(e, f2_fma(f2_splat(1.875f), e, f2_splat(1.5f)));
  float2 Rh, Rl;
  f2_fast_two_sum(y3h, f2_fma(y3h, c, y3e), Rh, Rl);
  f2_two_prod(gh, Rh, sh, se);
  se = f2_fma(gh, Rl, f2_fma(gl, Rh, se));
}

// A += s d without the final renormalisation: the caller renormalises
// (FastTwoSum of (Ah, Al)) after every second accumulation, so Al holds at
// most two steps' errors (|Al| <= ~4 2^-24 |Ah|) and the rounding of its
// additions stays at ~2^-46 of |A| per step, as with a renormalisation
// after every step (f2_ff_accumulate), for 3 fewer FP32 operations.
__device__ __forceinline__ void f2_ff_accumulate_lazy(float2& Ah, float2& Al, float2 sh, float2 se, float2 dh,
                                                      float2 dl) {
  float2 ah, ae;
  f2_two_prod(sh, dh, ah, ae);
  ae = f2_fma(sh, dl, f2_fma(se, dh, ae));
  float2 s1, s2;
  f2_two_sum(Ah, ah, s1, s2);
  Ah = s1;
  Al = f2_add(Al, f2_add(s2, ae));
}

// A += s d for one component, float-float (s and d float-float, |s_lo| <=
// 3 2^-24 |s_hi|; A kept normalised).
__device__ __forceinline__ void f2_ff_accumulate(float2& Ah, float2& Al, float2 sh, float2 se, float2 dh, float2 dl) {
  float2 ah, ae;
  f2_two_prod(sh, dh, ah, ae);
  ae = f2_fma(sh, dl, f2_fma(se, dh, ae));
  float2 s1, s2;
  // (Knuth's TwoSum: ordering the pair by magnitude instead put a compare and
  // two selections on this accumulator's serial chain and measured 4% slower)
  f2_two_sum(Ah, ah, s1, s2);
  s2 = f2_add(s2, f2_add(Al, ae));
  f2_fast_two_sum(s1, s2, Ah, Al);
}
