// Deterministic, nearly correctly rounded double-precision functions for the
// CA capture geometry, usable from host and device code.
//
// Why: the reference evaluates atan2, cos, sin, acos and pow with glibc
// (VoxelsCA.C:415-424, 548-591; SampleOrientation.C:72-149). glibc is not
// correctly rounded (about 0.1% of its results differ from the correctly
// rounded value), and CUDA's own functions differ from it far more often. The
// GPU path therefore evaluates these functions in double-double arithmetic
// (relative error below about 2^-80 before the final rounding), which returns
// the correctly rounded result except when the exact value lies within that
// error of a rounding boundary. Every routine uses only IEEE +, -, *, /, sqrt
// and fma with explicit evaluation order, so host and device produce the same
// bits; compile with FP contraction off (-ffp-contract=off, nvcc --fmad=false).
//
// Each of atan2, sin and cos first runs a short evaluation whose result is a
// double plus a correction with relative error below 2^-63, and returns it when
// rounding the result plus or minus that bound gives the same double (Ziv's
// rounding test; about one call in 500 fails it); otherwise the accurate
// double-double evaluation below decides.
//
// Methods: Dekker/Knuth error-free transformations (two_sum, two_prod via fma);
// arctangent by table reduction atan(t) = atan(c) + atan((t-c)/(1+tc)) with
// c = k/64 and a Taylor series; sine/cosine by Cody-Waite reduction by pi/2
// (four-part constant) and the addition formula around c = j/128 with Taylor
// series; arccos via atan2(sqrt(1-x^2), x) with the square root refined by one
// Newton step in double-double. Tables come from gen_crmath_tables.py.
#ifndef CAFE_CRMATH_H
#define CAFE_CRMATH_H

#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define CRM_HD __host__ __device__ __forceinline__
// the double-double paths, taken rarely: one out-of-line copy each keeps the
// inlined fast paths compact
#define CRM_COLD __host__ __device__ __noinline__
#ifdef __CUDA_ARCH__
#define CRM_TAB(name) name##_d
#else
#define CRM_TAB(name) name##_h
#endif
#else
#define CRM_HD static inline
#define CRM_COLD static inline
#define CRM_TAB(name) name##_h
#endif

// Host copies of the tables.
#define CRM_TABLE_DECL(type, name, dims) static const type name##_h dims
#include "cafe_crmath_tables.h"
#undef CRM_TABLE_DECL
#if defined(__CUDACC__)
// Device copies (same initialisers; the constant macros are redefined identically).
#undef CAFE_CRMATH_TABLES_H
#define CRM_TABLE_DECL(type, name, dims) static __device__ const type name##_d dims
#include "cafe_crmath_tables.h"
#undef CRM_TABLE_DECL
#endif

// Profiling builds count the calls that leave the fast paths.
#if defined(CAFE_DETAIL_CYCLES) && defined(__CUDACC__)
__device__ unsigned long long crm_fallback_calls, crm_special_calls;
#ifdef __CUDA_ARCH__
#define CRM_COUNT(c) atomicAdd(&(c), 1ULL)
#else
#define CRM_COUNT(c) ((void)0)
#endif
#else
#define CRM_COUNT(c) ((void)0)
#endif

struct crm_dd {
  double hi, lo;
};

// Bit patterns of doubles (integer tests are cheaper than floating-point
// compares on this hardware; for non-negative doubles the bit order is the
// numeric order).
CRM_HD long long crm_bits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
CRM_HD double crm_from_bits(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}
// Correctly rounded single-precision reciprocal (same bits on host and device).
CRM_HD float crm_rcp_f32(float x) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}
#define CRM_ABS_MASK 0x7fffffffffffffffLL
#define CRM_BITS_INF 0x7ff0000000000000LL
#define CRM_BITS_2P20 0x4130000000000000LL    // 2^20
#define CRM_BITS_PIO4 0x3fe921fb54442d18LL    // CRM_PIO2_1 / 2
#define CRM_BITS_3PIO4 0x4002d97c7f3321d2LL   // 3 CRM_PIO2_1 / 2

CRM_HD crm_dd crm_two_sum(double a, double b) {
  double s = a + b;
  double bp = s - a;
  double e = (a - (s - bp)) + (b - bp);
  crm_dd r = {s, e};
  return r;
}
CRM_HD crm_dd crm_fast_two_sum(double a, double b) {  // |a| >= |b| or a == 0
  double s = a + b;
  double e = b - (s - a);
  crm_dd r = {s, e};
  return r;
}
CRM_HD crm_dd crm_two_prod(double a, double b) {
  double p = a * b;
  double e = fma(a, b, -p);
  crm_dd r = {p, e};
  return r;
}
CRM_HD crm_dd crm_dd_add(crm_dd a, crm_dd b) {
  crm_dd s = crm_two_sum(a.hi, b.hi);
  crm_dd t = crm_two_sum(a.lo, b.lo);
  double lo = s.lo + t.hi;
  s = crm_fast_two_sum(s.hi, lo);
  lo = s.lo + t.lo;
  return crm_fast_two_sum(s.hi, lo);
}
CRM_HD crm_dd crm_dd_neg(crm_dd a) {
  crm_dd r = {-a.hi, -a.lo};
  return r;
}
CRM_HD crm_dd crm_dd_mul(crm_dd a, crm_dd b) {
  crm_dd p = crm_two_prod(a.hi, b.hi);
  double lo = p.lo + (a.hi * b.lo + a.lo * b.hi);
  return crm_fast_two_sum(p.hi, lo);
}
CRM_HD crm_dd crm_dd_mul_d(crm_dd a, double b) {
  crm_dd p = crm_two_prod(a.hi, b);
  double lo = p.lo + a.lo * b;
  return crm_fast_two_sum(p.hi, lo);
}
CRM_HD crm_dd crm_dd_div(crm_dd a, crm_dd b) {
  double q1 = a.hi / b.hi;
  crm_dd r = crm_dd_add(a, crm_dd_neg(crm_dd_mul_d(b, q1)));
  double q2 = r.hi / b.hi;
  r = crm_dd_add(r, crm_dd_neg(crm_dd_mul_d(b, q2)));
  double q3 = r.hi / b.hi;
  crm_dd q = crm_fast_two_sum(q1, q2);
  return crm_dd_add(q, crm_dd{q3, 0.0});
}
CRM_HD double crm_dd_round(crm_dd a) { return a.hi + a.lo; }

// atan(t) for t = num/den with 0 <= t <= 1, num and den double-double.
CRM_HD crm_dd crm_atan_unit(crm_dd num, crm_dd den) {
  crm_dd t = crm_dd_div(num, den);
  int k = (int)(t.hi * (double)CRM_ATAN_STEPS + 0.5);
  if (k > CRM_ATAN_STEPS) k = CRM_ATAN_STEPS;
  if (k < 0) k = 0;
  double c = (double)k * (1.0 / CRM_ATAN_STEPS);
  // u = (t - c) / (1 + t c); t.hi - c is exact (Sterbenz) for k >= 1 and trivially for k = 0
  crm_dd un = crm_two_sum(t.hi - c, t.lo);
  crm_dd tc = crm_dd_mul_d(t, c);
  crm_dd ud = crm_dd_add(crm_dd{1.0, 0.0}, tc);
  crm_dd u = crm_dd_div(un, ud);
  // atan(u) = u (1 - w/3 + w^2/5 - w^3/7 + ... ), w = u^2 <= 2^-14
  crm_dd w = crm_dd_mul(u, u);
  double wh = w.hi;
  double tail = wh * wh * (1.0 / 5 - wh * (1.0 / 7 - wh * (1.0 / 9 - wh * (1.0 / 11 - wh * (1.0 / 13)))));
  crm_dd w3 = crm_dd_div(w, crm_dd{3.0, 0.0});
  crm_dd q = crm_dd_add(crm_dd{1.0, 0.0}, crm_dd_neg(w3));
  q = crm_dd_add(q, crm_dd{tail, 0.0});
  crm_dd au = crm_dd_mul(u, q);
  crm_dd base = {CRM_TAB(crm_atan_tab)[k][0], CRM_TAB(crm_atan_tab)[k][1]};
  return crm_dd_add(base, au);
}

// atan2 on double-double magnitudes ay, ax >= 0 (not both zero), then sign
// handling for the original signs.
CRM_HD double crm_atan2_dd(crm_dd ay, crm_dd ax, int y_neg, int x_neg) {
  const crm_dd pio2 = {CRM_PIO2_1, CRM_PIO2_2};
  const crm_dd pi = {CRM_PI_HI, CRM_PI_LO};
  crm_dd r;
  if (ay.hi <= ax.hi) {
    r = crm_atan_unit(ay, ax);
  } else {
    r = crm_dd_add(pio2, crm_dd_neg(crm_atan_unit(ax, ay)));
  }
  if (x_neg) r = crm_dd_add(pi, crm_dd_neg(r));
  double v = crm_dd_round(r);
  return y_neg ? -v : v;
}

CRM_COLD double crm_atan2_acc(double y, double x) {
  if (y != y || x != x) return y + x;
  int yn = signbit(y) ? 1 : 0, xn = signbit(x) ? 1 : 0;
  double ay = fabs(y), ax = fabs(x);
  const double pio2 = CRM_PIO2_1, pi = CRM_PI_HI;
  if (ay == 0.0) {
    double v = xn ? pi : 0.0;
    return yn ? -v : v;
  }
  if (ax == INFINITY || ay == INFINITY) {
    double v;
    if (ax == INFINITY && ay == INFINITY)
      v = xn ? 3.0 * (pi / 4.0) : pi / 4.0;
    else if (ax == INFINITY)
      v = xn ? pi : 0.0;
    else
      v = pio2;
    return yn ? -v : v;
  }
  if (ax == 0.0) return yn ? -pio2 : pio2;
  return crm_atan2_dd(crm_dd{ay, 0.0}, crm_dd{ax, 0.0}, yn, xn);
}

// Cody-Waite reduction x = k pi/2 + r for |x| < 2^20, r in double-double.
CRM_COLD crm_dd crm_reduce_pio2(double x, int *quadrant) {
  double kd = x * CRM_TWO_OVER_PI;
  kd = (kd >= 0.0) ? (double)(long long)(kd + 0.5) : -(double)(long long)(-kd + 0.5);
  crm_dd a = crm_two_prod(kd, CRM_PIO2_1);  // exact
  crm_dd s = crm_two_sum(x, -a.hi);         // exact
  crm_dd r = crm_fast_two_sum(s.hi, s.lo - a.lo);
  crm_dd b = crm_two_prod(kd, CRM_PIO2_2);
  r = crm_dd_add(r, crm_dd_neg(b));
  crm_dd c = crm_two_prod(kd, CRM_PIO2_3);
  r = crm_dd_add(r, crm_dd_neg(c));
  r = crm_dd_add(r, crm_dd{-kd * CRM_PIO2_4, 0.0});
  long long k = (long long)kd;
  *quadrant = (int)(k & 3);
  return r;
}

// sin and cos of a double-double r with |r| <= pi/4 + 2^-20.
CRM_HD void crm_sincos_small(crm_dd r, crm_dd *sn, crm_dd *cs) {
  int neg = r.hi < 0.0;
  if (neg) r = crm_dd_neg(r);
  int j = (int)(r.hi * (double)CRM_SC_STEPS + 0.5);
  if (j > 103) j = 103;
  double c = (double)j * (1.0 / CRM_SC_STEPS);
  crm_dd s = crm_two_sum(r.hi - c, r.lo);  // |s| <= 2^-8
  crm_dd w = crm_dd_mul(s, s);
  double wh = w.hi;
  // sin s = s (1 - w/6 + w^2/120 - w^3/5040 + w^4/362880 - w^5/39916800)
  double st = wh * wh * (1.0 / 120 - wh * (1.0 / 5040 - wh * (1.0 / 362880 - wh * (1.0 / 39916800))));
  crm_dd sq = crm_dd_add(crm_dd{1.0, 0.0}, crm_dd_neg(crm_dd_div(w, crm_dd{6.0, 0.0})));
  sq = crm_dd_add(sq, crm_dd{st, 0.0});
  crm_dd ss = crm_dd_mul(s, sq);
  // cos s = 1 - w/2 + w^2/24 - w^3/720 + w^4/40320 - w^5/3628800
  double ct = wh * wh * (1.0 / 24 - wh * (1.0 / 720 - wh * (1.0 / 40320 - wh * (1.0 / 3628800))));
  crm_dd cq = crm_dd_add(crm_dd{1.0, 0.0}, crm_dd{-0.5 * w.hi, -0.5 * w.lo});
  crm_dd csv = crm_dd_add(cq, crm_dd{ct, 0.0});
  crm_dd sc = {CRM_TAB(crm_sincos_tab)[j][0], CRM_TAB(crm_sincos_tab)[j][1]};
  crm_dd cc = {CRM_TAB(crm_sincos_tab)[j][2], CRM_TAB(crm_sincos_tab)[j][3]};
  crm_dd sv = crm_dd_add(crm_dd_mul(sc, csv), crm_dd_mul(cc, ss));
  crm_dd cv = crm_dd_add(crm_dd_mul(cc, csv), crm_dd_neg(crm_dd_mul(sc, ss)));
  *sn = neg ? crm_dd_neg(sv) : sv;
  *cs = cv;
}

// Supported domain |x| < 2^20 (the CA evaluates arguments in [-2 pi, 2 pi]);
// outside it the result is NaN.
CRM_COLD double crm_sin_acc(double x) {
  if (!(fabs(x) < 1048576.0)) return NAN;
  if (x == 0.0) return x;
  int q;
  crm_dd r = crm_reduce_pio2(x, &q);
  crm_dd s, c;
  crm_sincos_small(r, &s, &c);
  switch (q) {
    case 0: return crm_dd_round(s);
    case 1: return crm_dd_round(c);
    case 2: return -crm_dd_round(s);
    default: return -crm_dd_round(c);
  }
}
CRM_COLD double crm_cos_acc(double x) {
  if (!(fabs(x) < 1048576.0)) return NAN;
  int q;
  crm_dd r = crm_reduce_pio2(x, &q);
  crm_dd s, c;
  crm_sincos_small(r, &s, &c);
  switch (q) {
    case 0: return crm_dd_round(c);
    case 1: return -crm_dd_round(s);
    case 2: return -crm_dd_round(c);
    default: return crm_dd_round(s);
  }
}

CRM_HD double crm_acos(double x) {
  if (x != x) return x;
  if (fabs(x) > 1.0) return (x - x) / (x - x);
  if (x == 1.0) return 0.0;
  if (x == -1.0) return CRM_PI_HI;
  // d = 1 - x^2 in double-double, then sqrt(d) refined by one Newton step
  crm_dd p = crm_two_prod(x, x);
  crm_dd s = crm_two_sum(1.0, -p.hi);
  crm_dd d = crm_fast_two_sum(s.hi, s.lo - p.lo);
  double s0 = sqrt(d.hi);
  crm_dd s0sq = crm_two_prod(s0, s0);
  double rem = ((d.hi - s0sq.hi) - s0sq.lo) + d.lo;
  crm_dd sq = crm_fast_two_sum(s0, rem / (2.0 * s0));
  int xn = signbit(x) ? 1 : 0;
  return crm_atan2_dd(sq, crm_dd{fabs(x), 0.0}, 0, xn);
}

// ---------------------------------------------------------------- fast paths
// Returns 1 and the rounded value when s + lo is within err of the exact
// result and both s + lo - err and s + lo + err round to the same double.
CRM_HD int crm_round_test(double s, double lo, double err, double *out) {
  double a = s + (lo - err), b = s + (lo + err);
  if (a == b) {
    *out = s + lo;
    return 1;
  }
  return 0;
}

// atan(num/den) for 0 < num <= den, both finite, as hi + lo; returns 0 (no
// result) for subnormal operands or num/den < 2^-1000. Both operands are first
// scaled by the same power of two (den to [1,2)), which is exact. The table
// point c = k/64 comes from a single-precision estimate of num/den (|t - c|
// stays within 1/128 + 2^-23, inside the series' range), and
// u = (num - c den)/(den + c num) = (t - c)/(1 + t c) is formed from
// double-double numerator and denominator with one division; the remainder
// term uses a single-precision reciprocal (relative error 2^-23 on a term below
// 2^-53 |u|).
CRM_HD int crm_atan_unit_fast(double num, double den, double *hi, double *lo) {
  long long nb = crm_bits(num), db = crm_bits(den);
  long long en = nb >> 52, ed = db >> 52;
  if (en == 0 || ed == 0 || en - ed < -1000) return 0;
  long long sh = (ed - 1023) << 52;
  double dens = crm_from_bits(db - sh), nums = crm_from_bits(nb - sh);
  float tf = (float)nums / (float)dens;
  int k = (int)(tf * (float)CRM_ATAN_STEPS + 0.5f);
  if (k > CRM_ATAN_STEPS) k = CRM_ATAN_STEPS;
  double c = (double)k * (1.0 / CRM_ATAN_STEPS);
  double p = c * dens, pe = fma(c, dens, -p);
  crm_dd a = crm_two_sum(nums, -p);
  double alo = a.lo - pe;
  double qv = c * nums, qe = fma(c, nums, -qv);
  crm_dd bd = crm_two_sum(dens, qv);
  double blo = bd.lo + qe;
  double uh = a.hi / bd.hi;
  double rr = (fma(-uh, bd.hi, a.hi) + alo) - uh * blo;
  double ul = rr * (double)crm_rcp_f32((float)bd.hi);
  double w = uh * uh;
  // u^3 (-1/3 + w/5 - w^2/7 + w^3/9 - w^4/11), Horner with explicit fma
  double q = fma(w, -1.0 / 11, 1.0 / 9);
  q = fma(w, q, -1.0 / 7);
  q = fma(w, q, 1.0 / 5);
  q = fma(w, q, -1.0 / 3);
  double poly = uh * w * q;
  double th = CRM_TAB(crm_atan_tab)[k][0], tlo = CRM_TAB(crm_atan_tab)[k][1];
  crm_dd sm = crm_two_sum(th, uh);
  *hi = sm.hi;
  *lo = sm.lo + (tlo + (ul + poly));
  return 1;
}

CRM_HD double crm_atan2(double y, double x) {
  long long yb = crm_bits(y), xb = crm_bits(x);
  long long ayb = yb & CRM_ABS_MASK, axb = xb & CRM_ABS_MASK;
  if (ayb == 0 || axb == 0 || ayb >= CRM_BITS_INF || axb >= CRM_BITS_INF) {
    CRM_COUNT(crm_special_calls);
    return crm_atan2_acc(y, x);
  }
  double ay = crm_from_bits(ayb), ax = crm_from_bits(axb);
  double h, l;
  if (ayb <= axb) {
    if (!crm_atan_unit_fast(ay, ax, &h, &l)) return crm_atan2_acc(y, x);
  } else {
    double h0, l0;
    if (!crm_atan_unit_fast(ax, ay, &h0, &l0)) return crm_atan2_acc(y, x);
    crm_dd d = crm_two_sum(CRM_PIO2_1, -h0);
    h = d.hi;
    l = d.lo + (CRM_PIO2_2 - l0);
  }
  if (xb < 0) {
    crm_dd d = crm_two_sum(CRM_PI_HI, -h);
    h = d.hi;
    l = d.lo + (CRM_PI_LO - l);
  }
  double v;
  if (crm_round_test(h, l, crm_from_bits(crm_bits(h) & CRM_ABS_MASK) * 0x1p-63, &v)) return yb < 0 ? -v : v;
  CRM_COUNT(crm_fallback_calls);
  return crm_atan2_acc(y, x);
}

// Addition-formula cores around the table point c = j/128 nearest to rh, for
// 0 <= rh <= pi/4 + 2^-20 and s = (rh - c) + rl: sin(c+s) = sin c + cos c s +
// cos c (sin s - s) + sin c (cos s - 1) and cos(c+s) = cos c - sin c s -
// sin c (sin s - s) + cos c (cos s - 1), as hi + lo.
CRM_HD void crm_sc_core(double rh, double rl, int want_sin, double *h, double *l) {
  int j = (int)(rh * (double)CRM_SC_STEPS + 0.5);
  if (j > 103) j = 103;
  double c = (double)j * (1.0 / CRM_SC_STEPS);
  double sh0 = rh - c;  // exact (Sterbenz)
  double w = sh0 * sh0;
  // Horner with explicit fma
  double qs = fma(w, -1.0 / 5040, 1.0 / 120);
  qs = fma(w, qs, -1.0 / 6);
  double sm = sh0 * w * qs;  // sin s - s
  double qc = fma(w, 1.0 / 40320, -1.0 / 720);
  qc = fma(w, qc, 1.0 / 24);
  qc = fma(w, qc, -0.5);
  double cm = fma(w, qc, -(sh0 * rl));  // cos s - 1
  double sc = CRM_TAB(crm_sincos_tab)[j][0], scl = CRM_TAB(crm_sincos_tab)[j][1];
  double cc = CRM_TAB(crm_sincos_tab)[j][2], ccl = CRM_TAB(crm_sincos_tab)[j][3];
  if (want_sin) {
    crm_dd p = crm_two_prod(cc, sh0);
    crm_dd t = crm_two_sum(sc, p.hi);
    *h = t.hi;
    *l = t.lo + (scl + (p.lo + fma(cc, rl, fma(ccl, sh0, fma(cc, sm, sc * cm)))));
  } else {
    crm_dd p2 = crm_two_prod(sc, sh0);
    crm_dd t2 = crm_two_sum(cc, -p2.hi);
    *h = t2.hi;
    *l = t2.lo + (ccl + (-p2.lo + fma(-sc, rl, fma(-scl, sh0, fma(-sc, sm, cc * cm)))));
  }
}

// sin(x) (want_sin) or cos(x) for 0 < |x| < 2^20 as hi + lo. |x| <= pi/4 needs
// no reduction; for pi/4 < |x| <= 3 pi/4 the reduction by pi/2 is
// |x| - PIO2_1 (exact by Sterbenz) minus PIO2_2 and PIO2_3 (the remainder is at
// least 6e-17 in magnitude, so the dropped PIO2_4 costs under 2^-100
// relative); larger |x| use the Cody-Waite reduction.
CRM_HD void crm_sincos1_fast(double x, int want_sin, double *h, double *l) {
  long long b = crm_bits(x);
  long long ab = b & CRM_ABS_MASK;
  double ax = crm_from_bits(ab);
  double rh, rl;
  int q;
  if (ab <= CRM_BITS_PIO4) {
    rh = ax;
    rl = 0.0;
    q = 0;
  } else if (ab <= CRM_BITS_3PIO4) {
    crm_dd t = crm_two_sum(ax - CRM_PIO2_1, -CRM_PIO2_2);
    crm_dd u = crm_fast_two_sum(t.hi, t.lo - CRM_PIO2_3);
    rh = u.hi;
    rl = u.lo;
    q = 1;
  } else {
    crm_dd r = crm_reduce_pio2(ax, &q);
    rh = r.hi;
    rl = r.lo;
  }
  // |x| = q pi/2 + r; sin|x| is (sin r, cos r, -sin r, -cos r) and cos|x| is
  // (cos r, -sin r, -cos r, sin r) for q = 0..3
  int rneg = crm_bits(rh) < 0;
  if (rneg) {
    rh = -rh;
    rl = -rl;
  }
  int sin_core = want_sin ? !(q & 1) : (q & 1);
  double hh, ll;
  crm_sc_core(rh, rl, sin_core, &hh, &ll);
  int neg = (sin_core && rneg) ^ (want_sin ? ((q & 2) != 0) : (((q + 1) & 2) != 0)) ^ (want_sin && b < 0);
  *h = neg ? -hh : hh;
  *l = neg ? -ll : ll;
}

CRM_HD double crm_sin(double x) {
  long long ab = crm_bits(x) & CRM_ABS_MASK;
  if (ab >= CRM_BITS_2P20 || ab == 0) return crm_sin_acc(x);
  double sh, sl, v;
  crm_sincos1_fast(x, 1, &sh, &sl);
  if (crm_round_test(sh, sl, crm_from_bits(crm_bits(sh) & CRM_ABS_MASK) * 0x1p-63 + 0x1p-1000, &v)) return v;
  CRM_COUNT(crm_fallback_calls);
  return crm_sin_acc(x);
}
CRM_HD double crm_cos(double x) {
  long long ab = crm_bits(x) & CRM_ABS_MASK;
  if (ab >= CRM_BITS_2P20) return crm_cos_acc(x);
  double ch, cl, v;
  crm_sincos1_fast(x, 0, &ch, &cl);
  if (crm_round_test(ch, cl, crm_from_bits(crm_bits(ch) & CRM_ABS_MASK) * 0x1p-63 + 0x1p-1000, &v)) return v;
  CRM_COUNT(crm_fallback_calls);
  return crm_cos_acc(x);
}

// pow(x, 0.5) as glibc's pow defines it; the correctly rounded value is sqrt
// except for the sign of zero and -inf.
CRM_HD double crm_pow_half(double x) {
  if (x == 0.0) return 0.0;
  if (x == -INFINITY) return INFINITY;
  return sqrt(x);
}

// x^e for integer e >= 1, evaluated in double-double by binary powering.
CRM_HD double crm_pow_int(double x, int e) {
  if (x != x) return x;
  if (x == 0.0 || fabs(x) == INFINITY || e == 1) {
    double r = x;
    for (int i = 1; i < e; ++i) r = r * x;
    return r;
  }
  crm_dd base = {x, 0.0}, acc = {1.0, 0.0};
  int first = 1;
  while (e > 0) {
    if (e & 1) {
      acc = first ? base : crm_dd_mul(acc, base);
      first = 0;
    }
    e >>= 1;
    if (e) base = crm_dd_mul(base, base);
  }
  return crm_dd_round(acc);
}

// ---- exp ----------------------------------------------------------------
// exp(x) = 2^m * 2^(j/128) * exp(r), k = 128 m + j = round(x * 128/ln2),
// r = x - k ln2/128 with ln2/128 in three parts (the first two of 35 bits, so
// k times them is exact for |k| < 2^18) and |r| <= ln2/256 + 2^-60. The fast
// evaluation takes exp(r) - 1 = r + r^2/2 + ... + r^6/720 with the quadratic
// tail in double (relative error below 2^-67 overall); the accurate one takes
// the terms to r^4/24 in double-double and the rest to r^10 in double (error
// below about 2^-100). Results below the normal range are rounded once, on the
// subnormal grid, from the double-double value.

// Rounds (h + l) * 2^m to the nearest double (ties to even) for m <= -1022
// and h + l in [0.99, 2]: results on the subnormal grid (step 2^-1074, which is
// also the step of the lowest normal binade), rounded once from the
// double-double value. `err` bounds the absolute error of h + l. Returns 0 when
// the rounding is not decided within it, unless `force` (then the value itself
// decides).
CRM_HD int crm_round_scaled_sub(double h, double l, double err, int m, int force, double *out) {
  int sh = m + 1074;  // the grid step becomes 1; sh <= 52
  if (sh < -2) {      // below a quarter of the smallest subnormal
    *out = 0.0;
    return 1;
  }
  double sc = crm_from_bits((long long)(1023 + sh) << 52);
  double uh = h * sc, ul = l * sc;                 // exact: powers of two, normal range
  double ue = err * sc + 0x1p-53;                  // + the rounding of f below
  double n0 = uh >= 0x1p52 ? uh : (uh + 0x1p52) - 0x1p52;  // nearest integer, 0 <= uh < 2^53
  double f = (uh - n0) + ul;                       // uh - n0 is exact, |f| <~ 1/2
  double n;
  if (f - ue > 0.5) {
    n = n0 + 1.0;
  } else if (f + ue < -0.5) {
    n = n0 - 1.0;
  } else if (f - ue > -0.5 && f + ue < 0.5) {
    n = n0;
  } else if (!force) {
    return 0;
  } else if (f > 0.5 || f < -0.5) {
    n = f > 0.5 ? n0 + 1.0 : n0 - 1.0;
  } else if (f == 0.5 || f == -0.5) {  // tie: the even neighbour
    double o = f > 0.0 ? n0 + 1.0 : n0 - 1.0;
    n = (n0 * 0.5 == (double)(long long)(n0 * 0.5)) ? n0 : o;
  } else {
    n = n0;
  }
  *out = (n * 0x1p-1022) * 0x1p-52;  // n 2^-1074, exact in two steps
  return 1;
}

// Reduction shared by both evaluations: k, and r as rh + rl.
CRM_HD void crm_exp_reduce(double x, long long *k, double *rh, double *rl) {
  const double MAGIC = 0x1.8p52;
  double kd = (x * CRM_INV_LN2_128 + MAGIC) - MAGIC;
  *k = (long long)kd;
  double a = x - kd * CRM_LN2_128_1;  // exact
  crm_dd t = crm_two_sum(a, -(kd * CRM_LN2_128_2));
  double c = kd * CRM_LN2_128_3;
  crm_dd r = crm_fast_two_sum(t.hi, t.lo - c);
  *rh = r.hi;
  *rl = r.lo;
}

// Final scaling of T (1 + p) = s + lo by 2^m; returns 0 if undecided.
CRM_HD int crm_exp_finish(double s, double lo, double err, int m, int force, double *out) {
  if (m >= -1021) {
    double v;
    if (!crm_round_test(s, lo, err, &v)) return 0;
    if (m > 1023) {  // v * 2^m in two exact-or-overflowing steps
      *out = (v * 0x1p1023) * crm_from_bits((long long)(1023 + m - 1023) << 52);
    } else {
      *out = v * crm_from_bits((long long)(1023 + m) << 52);
    }
    return 1;
  }
  return crm_round_scaled_sub(s, lo, err, m, force, out);
}

CRM_COLD double crm_exp_acc(double x) {
  long long k;
  double rh, rl;
  crm_exp_reduce(x, &k, &rh, &rl);
  int j = (int)(k & (CRM_EXP_STEPS - 1));
  int m = (int)((k - j) / CRM_EXP_STEPS);
  // tail r^5/120 + ... + r^10/10! in double
  double c5 = 1.0 / 120 + rh * (1.0 / 720 + rh * (1.0 / 5040 + rh * (1.0 / 40320 + rh * (1.0 / 362880 + rh * (1.0 / 3628800)))));
  crm_dd r = {rh, rl};
  crm_dd t = crm_dd_add(crm_dd{CRM_INV_FACT24_HI, CRM_INV_FACT24_LO}, crm_dd{rh * c5, 0.0});
  t = crm_dd_add(crm_dd{CRM_INV_FACT6_HI, CRM_INV_FACT6_LO}, crm_dd_mul(r, t));
  t = crm_dd_add(crm_dd{0.5, 0.0}, crm_dd_mul(r, t));
  t = crm_dd_add(crm_dd{1.0, 0.0}, crm_dd_mul(r, t));
  crm_dd p = crm_dd_mul(r, t);  // exp(r) - 1
  crm_dd T = {CRM_TAB(crm_exp2_tab)[j][0], CRM_TAB(crm_exp2_tab)[j][1]};
  crm_dd y = crm_dd_add(T, crm_dd_mul(T, p));
  double v;
  crm_exp_finish(y.hi, y.lo, 0.0, m, 1, &v);
  return v;
}

// exp(x), nearly correctly rounded (see above); same bits on host and device.
CRM_HD double crm_exp(double x) {
  if (x != x) return x + x;
  if (x > 709.8) return INFINITY;
  if (x < -745.2) return 0.0;
  long long k;
  double rh, rl;
  crm_exp_reduce(x, &k, &rh, &rl);
  int j = (int)(k & (CRM_EXP_STEPS - 1));
  int m = (int)((k - j) / CRM_EXP_STEPS);
  double q = rh * rh * (0.5 + rh * (1.0 / 6 + rh * (1.0 / 24 + rh * (1.0 / 120 + rh * (1.0 / 720)))));
  crm_dd p = crm_fast_two_sum(rh, rl + q);  // exp(r) - 1, |rh| > |rl + q| or rh = 0
  double th = CRM_TAB(crm_exp2_tab)[j][0], tl = CRM_TAB(crm_exp2_tab)[j][1];
  crm_dd a = crm_two_prod(th, p.hi);
  crm_dd s = crm_fast_two_sum(th, a.hi);
  double lo = s.lo + (a.lo + (th * p.lo + (tl + tl * p.hi)));
  double v;
  if (crm_exp_finish(s.hi, lo, s.hi * 0x1p-66, m, 0, &v)) return v;
  CRM_COUNT(crm_fallback_calls);
  return crm_exp_acc(x);
}

// ---- pow(x, -0.5) ------------------------------------------------------------
// Sign of the exact sum of n doubles (n <= 8), by Shewchuk's expansion growth.
CRM_HD int crm_sum_sign(const double *t, int n) {
  double e[9];
  int len = 0;
  for (int i = 0; i < n; ++i) {
    double q = t[i];
    int nl = 0;
    for (int k = 0; k < len; ++k) {
      crm_dd s = crm_two_sum(q, e[k]);
      q = s.hi;
      if (s.lo != 0.0) e[nl++] = s.lo;
    }
    if (q != 0.0) e[nl++] = q;
    len = nl;
  }
  // components are non-overlapping and ascending: the last one has the sign
  if (len == 0) return 0;
  return e[len - 1] > 0.0 ? 1 : -1;
}

// x^(-1/2) as pow(x, -0.5) defines it, correctly rounded. x = x' 4^h with x'
// in [1, 4) (subnormal x first scaled by 2^108); y = 1/sqrt(x') is refined
// with the residual 1 - x' y^2 (double-double, error below 2^-100), and when
// that does not decide the rounding, x' m^2 is compared with 1 exactly at the
// midpoint m between the two candidate doubles. (An exact result needs x' = 1
// and a tie is impossible, so the comparison always decides.)
CRM_HD double crm_pow_mhalf(double x) {
  if (x != x) return x + x;
  if (x == 0.0) return INFINITY;
  if (x < 0.0) return (x - x) / (x - x);  // NaN (also for -inf)
  if (x == INFINITY) return 0.0;
  int post = 0;  // result exponent adjustment
  if (x < 0x1p-1022) {
    x = x * 0x1p108;
    post = 54;
  }
  int ex = (int)((crm_bits(x) >> 52) & 0x7ff) - 1023;
  int h2 = ex >> 1;  // floor(ex / 2)
  double xs = x * crm_from_bits((long long)(1023 - 2 * h2) << 52);  // in [1, 4)
  post -= h2;
  double y = 1.0 / sqrt(xs);
  crm_dd y2 = crm_two_prod(y, y);
  crm_dd b = crm_two_prod(xs, y2.hi);
  double c = xs * y2.lo;
  double e = ((1.0 - b.hi) - b.lo) - c;       // 1 - x' y^2
  double corr = y * (e * (0.5 + 0.375 * e));  // y ((1 - e)^(-1/2) - 1) to O(e^3)
  double v;
  if (!crm_round_test(y, corr, y * 0x1p-98, &v)) {
    double v0 = y + corr;
    long long vb = crm_bits(v0);
    double resid = (y - v0) + corr;  // the side of v0 the exact value lies on
    double nb = crm_from_bits(resid >= 0.0 ? vb + 1 : vb - 1);
    double hh = (nb - v0) * 0.5;     // half the gap, a power of two
    // x' (v0 + hh)^2 - 1 as an exact sum
    crm_dd v2 = crm_two_prod(v0, v0);
    crm_dd t1 = crm_two_prod(xs, v2.hi);
    crm_dd t2 = crm_two_prod(xs, v2.lo);
    crm_dd t3 = crm_two_prod(xs, 2.0 * v0 * hh);
    double terms[8] = {-1.0, t1.hi, t1.lo, t2.hi, t2.lo, t3.hi, t3.lo, xs * (hh * hh)};
    int sg = crm_sum_sign(terms, 8);  // > 0: the midpoint lies above the exact value
    if (resid >= 0.0)
      v = sg > 0 ? v0 : nb;
    else
      v = sg < 0 ? v0 : nb;
    CRM_COUNT(crm_fallback_calls);
  }
  return v * crm_from_bits((long long)(1023 + post) << 52);
}

#endif
