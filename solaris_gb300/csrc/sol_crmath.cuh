// Correctly rounded r = sqrt(a) and r^-3 = 1 / (a * r) for the reference-form
// pair (GravityAC, Acceleration.cpp:294-317: rij = sqrt(rij2),
// rijm3 = 1.0 / (rij2 * rij)) with two FP64 instructions besides the product
// a * r, bit-identical to IEEE sqrt and division.
//
// The GPU's FP64 pipe issues one warp instruction per 64 cycles per
// sub-partition; IEEE square root and division take about sixteen of them
// per pair, so they, not the twenty-one additions and multiplications of the
// pair, bound the reference form.  Here the approximations come from the FP32
// and integer pipes and FP64 only measures the remainders:
//
//  1. a = m 4^k with m in [1, 4).  From an FP32 rsqrt seed y and one Newton
//     correction evaluated with exact products (TwoProduct by FMA) come
//     float-float approximations (relative error ~2^-45) of m^-1/2, of
//     m^1/2 and of m^-3/2.
//  2. Integer operations on the bit patterns turn them into doubles
//     q0 ~ sqrt(a) and z0 ~ 1/d (d = RN(a r)), a few hundred ulps at most
//     from the exact values.
//  3. One FMA gives each remainder, a - q0^2 and 1 - d z0, to full
//     precision (its rounding error is 2^-53 of itself).  The remainder over
//     the derivative, in float-float, is the distance of the exact result
//     from q0 (z0) in units in the last place, to ~2^-35 ulp; rounding it to
//     the nearest integer and adding that to the bit pattern gives the
//     correctly rounded result.  This is the remainder-based rounding
//     decision of Markstein (IA-64 and Elementary Functions, 2000, ch. 8;
//     Tuckerman's test for the square root), with the remainder measured
//     rather than only its sign.
//
// Neither quotient can fall exactly on a midpoint between doubles (a
// midpoint needs 54 significant bits; its square, or its product with a
// 53-bit d, cannot be a double, resp. 1).  Where the measured distance lies
// within 2^-16 ulp of a midpoint (probability ~2^-15 per function), where
// it exceeds 2^20 ulp (an approximation gone astray), where the result would
// land on or cross a power of two, or where a is outside [2^-600, 2^600]
// (zero, denormal, infinite or NaN included) the fast path reports failure
// and the caller takes IEEE sqrt and division, so the result is the
// correctly rounded one in every case.
#pragma once

#include "sol_pair.cuh"

namespace solcr {

constexpr float kMidTol = 0.5f - 1.52587890625e-05f;  // 0.5 - 2^-16: beyond it the rounding is decided exactly

// (h, l) floats, h > 0 normal, |l| <= ulp(h)/2, scaled by 2^escale -> the bit
// pattern of a double within one ulp of (h + l) 2^escale.  The 53-bit
// significand is built as an integer; when a negative l takes it below 2^52
// (h a power of two) it is shifted up one place and the exponent lowered, and
// |l| <= ulp(h)/2 keeps the sum below the next power of two.
__device__ __forceinline__ long long ff_to_double_bits(float h, float l, int escale) {
  const unsigned hb = __float_as_uint(h);
  const int eh = (int)(hb >> 23);  // h > 0
  const unsigned mh = (hb & 0x7FFFFFu) | 0x800000u;
  const unsigned lb = __float_as_uint(l);
  const int el = (int)((lb >> 23) & 0xFFu);
  const unsigned ml = el ? ((lb & 0x7FFFFFu) | 0x800000u) : 0u;
  const int sh = el - eh + 29;  // l's unit in units of 2^(E_h - 52); <= 5
  unsigned long long add = 0;
  if (sh >= 0)
    add = (unsigned long long)ml << sh;
  else if (sh > -32)
    add = (unsigned long long)(ml >> (-sh));
  long long m = ((long long)mh << 29);
  m = (lb & 0x80000000u) ? m - (long long)add : m + (long long)add;
  const bool low = m < (1LL << 52);
  m = low ? (m << 1) : m;
  return ((long long)(eh - 127 + 1023 + escale - (low ? 1 : 0)) << 52) + (m - (1LL << 52));
}

// d 2^sh -> (h, l) floats from the bit pattern (h: the leading 24 bits
// truncated, l: the next 29 rounded to 24).  Scaled values below 2^-74 give
// 0 (the callers scale remainders to distances in ulps, where 2^-74 is
// nothing); ok turns false if the scaled value is too large.
__device__ __forceinline__ void double_to_ff_scaled(double d, int sh, float& h, float& l, bool& ok) {
  const unsigned hi = (unsigned)__double2hiint(d);
  const unsigned lo = (unsigned)__double2loint(d);
  const int e = (int)((hi >> 20) & 0x7FFu);
  const unsigned sign = hi & 0x80000000u;
  const int ef = e - 1023 + sh + 127;  // biased float exponent of h
  ok = ok && (ef < 200);
  const bool live = (e != 0) && (ef >= 53);
  h = live ? __uint_as_float(sign | ((unsigned)ef << 23) | ((hi & 0x000FFFFFu) << 3) | (lo >> 29)) : 0.0f;
  const float scale = live ? __uint_as_float((unsigned)(ef - 52) << 23) : 0.0f;
  l = __uint_as_float(__float_as_uint(__uint2float_rn(lo & 0x1FFFFFFFu) * scale) | sign);
}

// Nearest integer n to (h + l), and whether it is decided: |h| < 2^20 (the
// approximations are within a few hundred ulps; anything else goes to the
// IEEE path) and |h + l - n| <= 0.5 - 2^-16.
__device__ __forceinline__ int round_ff(float h, float l, bool& ok) {
  const float t = h + 12582912.0f;  // 1.5 * 2^23: the sum rounds h to an integer
  const int n = __float_as_int(t) - 0x4B400000;
  const float frac = (h - (t - 12582912.0f)) + l;
  ok = ok && (fabsf(frac) <= kMidTol) && (fabsf(h) < 1048576.0f);
  return n;
}

// The correctly rounded neighbour q0 + n ulp, unless that needs another
// binade (the ulp used for n is q0's) or is a power of two.
__device__ __forceinline__ long long step_ulps(long long qb, int n, bool& ok) {
  const long long rb = qb + (long long)n;
  ok = ok && (((rb ^ qb) >> 52) == 0) && ((rb & 0xFFFFFFFFFFFFFLL) != 0);
  return rb;
}

// The correctly rounded 1/d from the bit pattern zb of an approximation
// z0 within a few hundred ulps of it: the distance (1/d - z0) / ulp(z0) =
// (1 - d z0) z0 / ulp(z0) (1 + O(2^-40)), z0 / ulp(z0) being its significand
// in [1, 2) times 2^52.
__device__ __forceinline__ long long rcp_from_approx(double d, long long zb, bool& ok) {
  const double z0 = __longlong_as_double(zb);
  const double er = __fma_rn(-d, z0, 1.0);
  const unsigned hiZ = (unsigned)(zb >> 32);
  const unsigned loZ = (unsigned)zb;
  const float zh = __uint_as_float(0x3F800000u | ((hiZ & 0x000FFFFFu) << 3) | (loZ >> 29));
  const float zl = __uint2float_rn(loZ & 0x1FFFFFFFu) * 2.220446049250313e-16f;  // 2^-52
  float eh, el;
  double_to_ff_scaled(er, 52, eh, el, ok);
  const float ph = eh * zh;
  const float pl = __fmaf_rn(eh, zh, -ph) + __fmaf_rn(eh, zl, el * zh);
  return step_ulps(zb, round_ff(ph, pl, ok), ok);
}

}  // namespace solcr

// Fast path: returns false where the caller must use IEEE sqrt and division.
__device__ __forceinline__ bool sol_ref_rinv3_fast(double a, double& rij, double& rijm3) {
  using namespace solcr;
  const unsigned hiA = (unsigned)__double2hiint(a);
  const unsigned loA = (unsigned)__double2loint(a);
  const int E = (int)(hiA >> 20);  // the sign bit of a sum of squares is clear, NaN aside
  bool ok = (E >= 1023 - 600) & (E <= 1023 + 600);
  const int e2 = E - 1023;
  const int k = e2 >> 1;   // floor(e2 / 2)
  const int p = e2 - 2 * k;  // 0 or 1: m = a 4^-k in [1, 4)
  // m as float-float (mh exact to 24 bits, ml the rest rounded)
  const float mh = __uint_as_float(((unsigned)(127 + p) << 23) | ((hiA & 0x000FFFFFu) << 3) | (loA >> 29));
  const float ml = __uint2float_rn(loA & 0x1FFFFFFFu) * __uint_as_float((unsigned)(127 + p - 52) << 23);
  // seed and residual e = 1 - m y^2 from exact products
  const float y = sol_rsqrt_normal(mh);  // mh in [1, 4)
  float y2, y2e, q, qe;
  ff_two_prod(y, y, y2, y2e);
  ff_two_prod(mh, y2, q, qe);
  const float e = ((1.0f - q) - qe) - __fmaf_rn(mh, y2e, ml * y2);
  // m^-1/2 = y (1 - e)^-1/2 = y (1 + e/2 + 3/8 e^2 + ...)
  float yh, yl;
  ff_fast_two_sum(y, y * (e * __fmaf_rn(0.375f, e, 0.5f)), yh, yl);
  // m^1/2 = m m^-1/2
  float sh, sl;
  {
    float sp, spe;
    ff_two_prod(mh, yh, sp, spe);
    ff_fast_two_sum(sp, spe + __fmaf_rn(mh, yl, ml * yh), sh, sl);
  }
  // m^-3/2 = y^3 (1 - e)^-3/2 = y^3 (1 + 3/2 e + 15/8 e^2 + ...)
  float Rh, Rl;
  {
    float y3h, y3e;
    ff_two_prod(y2, y, y3h, y3e);
    y3e = __fmaf_rn(y2e, y, y3e);
    const float c3 = e * __fmaf_rn(1.875f, e, 1.5f);
    ff_fast_two_sum(y3h, __fmaf_rn(y3h, c3, y3e), Rh, Rl);
  }

  // ---- sqrt(a): q0 ~ m^1/2 2^k; distance = (a - q0^2) / (2 q0 ulp(q0)) ----
  const long long qb = ff_to_double_bits(sh, sl, k);
  const double q0 = __longlong_as_double(qb);
  const double ea = __fma_rn(-q0, q0, a);
  const int Eq = (int)(qb >> 52) - 1023;
  // (a - q0^2) / (2 q0 2^(Eq-52)) = ea 2^(51-Eq-k) / (q0 2^-k) ~ ea 2^(51-Eq-k) m^-1/2
  float eh, el;
  double_to_ff_scaled(ea, 51 - Eq - k, eh, el, ok);
  const float ph = eh * yh;
  const float pl = __fmaf_rn(eh, yh, -ph) + __fmaf_rn(eh, yl, el * yh);
  const long long rb = step_ulps(qb, round_ff(ph, pl, ok), ok);
  const double r = __longlong_as_double(rb);

  // ---- 1/d, d = RN(a r): z0 ~ m^-3/2 2^-3k ----
  const double d = a * r;
  const long long wb = rcp_from_approx(d, ff_to_double_bits(Rh, Rl, -3 * k), ok);

  rij = r;
  rijm3 = __longlong_as_double(wb);
  return ok;
}

static __device__ __noinline__ void sol_ref_rinv3_slow(double a, double& rij, double& rijm3) {
  rij = __dsqrt_rn(a);
  rijm3 = __ddiv_rn(1.0, a * rij);
}

// rij = RN(sqrt(a)), rijm3 = RN(1 / RN(a * rij)), bit-identical to IEEE
// sqrt and division for every a.
__device__ __forceinline__ void sol_ref_rinv3(double a, double& rij, double& rijm3) {
  if (!sol_ref_rinv3_fast(a, rij, rijm3)) sol_ref_rinv3_slow(a, rij, rijm3);
}

// ---- IEEE double multiplication on the integer pipe ----------------------------
// Round-to-nearest-even product of two doubles from 32-bit integer
// multiplies of the significands (the 106-bit product in three words, the
// leading 53 bits, guard and sticky bits): the textbook IEEE 754 multiply.
// It is exact wherever the inputs are finite and normal or zero and the
// product is normal or zero; ok turns false elsewhere (the caller then takes
// the FP64 instruction).  A pair's term multiplies move here from the FP64
// pipe, which binds the reference form, to the integer pipe, which it leaves
// mostly idle.
__device__ __forceinline__ double sol_exact_dmul(double a, double b, bool& ok) {
  const unsigned ah = (unsigned)__double2hiint(a), al = (unsigned)__double2loint(a);
  const unsigned bh = (unsigned)__double2hiint(b), bl = (unsigned)__double2loint(b);
  const int ea = (int)((ah >> 20) & 0x7FFu), eb = (int)((bh >> 20) & 0x7FFu);
  const unsigned sign = (ah ^ bh) & 0x80000000u;
  const unsigned mah = (ah & 0xFFFFFu) | 0x100000u, mbh = (bh & 0xFFFFFu) | 0x100000u;
  // Ma Mb in [2^104, 2^106): bits 64.. in t3, 32..63 in w1, 0..31 in w0
  const unsigned long long t0 = (unsigned long long)al * bl;
  const unsigned long long t1 = (unsigned long long)mah * bl + (t0 >> 32);
  const unsigned long long t2 = (unsigned long long)al * mbh + (t1 & 0xFFFFFFFFull);
  const unsigned long long t3 = (unsigned long long)mah * mbh + (t1 >> 32) + (t2 >> 32);
  const unsigned w1 = (unsigned)t2, w0 = (unsigned)t0;
  const int n = (int)(t3 >> 41);  // product >= 2^105: one more place to drop
  const int s = 20 + n;
  const unsigned long long m = (t3 << (32 - s)) | (unsigned long long)(w1 >> s);  // the leading 53 bits
  const unsigned guard = (w1 >> (s - 1)) & 1u;
  const unsigned sticky = (w1 & ((1u << (s - 1)) - 1u)) | w0;
  const unsigned long long rnd = guard & ((sticky != 0u) | (unsigned)(m & 1ull));
  const int e = ea + eb - 1023 + n;
  const bool za = (ea == 0) & (((ah & 0xFFFFFu) | al) == 0u);
  const bool zb = (eb == 0) & (((bh & 0xFFFFFu) | bl) == 0u);
  const bool zero = za | zb;
  ok = ok && ((ea != 0) | za) && ((eb != 0) | zb) && (ea != 0x7FF) && (eb != 0x7FF) && (zero | ((e >= 1) & (e <= 2045)));
  // a rounding carry out of the significand moves into the exponent field
  const unsigned long long bits = zero ? 0ull : ((unsigned long long)e << 52) + (m - (1ull << 52)) + rnd;
  return __longlong_as_double((long long)(bits | ((unsigned long long)sign << 32)));
}

// The reference's pair term gm (d rijm3 - p) per component
// (Acceleration.cpp:306-308), its six multiplications on the integer pipe;
// bit-identical to the FP64 expression.
__device__ __forceinline__ void sol_ref_terms(double gm, double rijm3, double dx, double dy, double dz, double px,
                                              double py, double pz, double& tx, double& ty, double& tz) {
  bool ok = true;
  const double ux = sol_exact_dmul(dx, rijm3, ok) - px;
  const double uy = sol_exact_dmul(dy, rijm3, ok) - py;
  const double uz = sol_exact_dmul(dz, rijm3, ok) - pz;
  tx = sol_exact_dmul(gm, ux, ok);
  ty = sol_exact_dmul(gm, uy, ok);
  tz = sol_exact_dmul(gm, uz, ok);
  if (!ok) {
    tx = gm * (dx * rijm3 - px);
    ty = gm * (dy * rijm3 - py);
    tz = gm * (dz * rijm3 - pz);
  }
}

// Two independent pairs in one basic block (their dependency chains
// interleave), the rare IEEE fallbacks after both.
__device__ __forceinline__ void sol_ref_rinv3_x2(double a0, double a1, double& r0, double& w0, double& r1,
                                                 double& w1) {
  const bool ok0 = sol_ref_rinv3_fast(a0, r0, w0);
  const bool ok1 = sol_ref_rinv3_fast(a1, r1, w1);
  if (!(ok0 && ok1)) {
    if (!ok0) sol_ref_rinv3_slow(a0, r0, w0);
    if (!ok1) sol_ref_rinv3_slow(a1, r1, w1);
  }
}
