// Device-side numerics and tightening rules of SCIP's linear-constraint propagation.
//
// Everything here is FP64 and is compiled with --fmad=false, so each expression rounds exactly like the
// plain C restatement used as the test oracle; integer bounds, cutoff verdicts and (for rows summed in
// the same order) activities are bit-identical.  The rule each function restates is cited beside it
// (paths relative to the SCIP source tree).
#pragma once

#include <cstdint>
#include <cstring>

namespace gbp {

struct Num {
  double inf, eps, sumeps, feastol, huge, bstreps, recomp, maxeasy;
  int nosort;  // constraints/linear/sortvars = FALSE: every entry of a row is tried (no binary skip)
};

// ------------------------------------------------------------------------------------------ comparisons
// A double instruction on this part is a long FP64-pipe issue (the same cost with one lane active as with 32), so
// the tests below decide on a double's IEEE bit pattern in the integer pipe wherever that is exact.  For the
// finite, non-NaN values they see: a pattern read as a signed integer orders like the value for x >= +0 (every
// negative value and -0 read as negative); the pattern without the sign bit is the magnitude, ordered like |x|.
// The numerics in Num are >= +0 (gbp_set_params stores -0 as +0), which the one-sided tests rely on.
__host__ __device__ __forceinline__ long long dbits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ double bitsd(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}
constexpr long long DMAG = 0x7fffffffffffffffLL;
__host__ __device__ __forceinline__ long long dmag(double x) { return dbits(x) & DMAG; }
// x > c and x >= c for c >= +0
__host__ __device__ __forceinline__ bool gtc(double x, double c) { return dbits(x) > dbits(c); }
__host__ __device__ __forceinline__ bool gec(double x, double c) { return dbits(x) >= dbits(c); }
// x < -c and x <= -c for c >= +0
__host__ __device__ __forceinline__ bool ltnc(double x, double c) { return dbits(x) < 0 && dmag(x) > dbits(c); }
__host__ __device__ __forceinline__ bool lenc(double x, double c) { return dbits(x) < 0 && dmag(x) >= dbits(c); }
// x > 0 and x < 0
__host__ __device__ __forceinline__ bool dpos(double x) { return dbits(x) > 0; }
__host__ __device__ __forceinline__ bool dneg(double x) { return dbits(x) < 0 && dmag(x) != 0; }
// a key ordered like the value, -0 and +0 equal: a < b, a > b on keys
__host__ __device__ __forceinline__ long long okey(double x) {
  const long long b = dbits(x);
  return b >= 0 ? b : -(b & DMAG);
}
__host__ __device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }
__host__ __device__ __forceinline__ bool dgt(double a, double b) { return okey(a) > okey(b); }
__host__ __device__ __forceinline__ double dmax(double a, double b) { return dgt(a, b) ? a : b; }  // a > b ? a : b
__host__ __device__ __forceinline__ double dmin(double a, double b) { return dlt(a, b) ? a : b; }  // a < b ? a : b
__host__ __device__ __forceinline__ double dabs(double x) { return bitsd(dmag(x)); }

__host__ __device__ __forceinline__ bool isInf(const Num& s, double x) { return gec(x, s.inf); }   // set.c:6824
__host__ __device__ __forceinline__ bool isNegInf(const Num& s, double x) { return lenc(x, s.inf); }  // isInf(-x)
__host__ __device__ __forceinline__ bool isHuge(const Num& s, double x) { return gec(x, s.huge); }  // set.c:6835
__host__ __device__ __forceinline__ bool isNegHuge(const Num& s, double x) { return lenc(x, s.huge); }  // isHuge(-x)
__host__ __device__ __forceinline__ bool lt(const Num& s, double a, double b) { return ltnc(a - b, s.eps); }  // def.h:193
__host__ __device__ __forceinline__ bool le(const Num& s, double a, double b) { return !gtc(a - b, s.eps); }
__host__ __device__ __forceinline__ bool gt(const Num& s, double a, double b) { return gtc(a - b, s.eps); }
__host__ __device__ __forceinline__ bool ge(const Num& s, double a, double b) { return !ltnc(a - b, s.eps); }
__host__ __device__ __forceinline__ bool eq(const Num& s, double a, double b) { return dmag(a - b) <= dbits(s.eps); }
__host__ __device__ __forceinline__ bool sumGt(const Num& s, double a, double b) { return gtc(a - b, s.sumeps); }
__host__ __device__ __forceinline__ bool positive(const Num& s, double a) { return gtc(a, s.eps); }
__host__ __device__ __forceinline__ bool feasZero(const Num& s, double a) { return dmag(a) <= dbits(s.feastol); }

// SCIPrelDiff, misc.c:11162-11176
__host__ __device__ __forceinline__ double relDiff(double a, double b) {
  double q = fabs(a);
  if (fabs(b) > q) q = fabs(b);
  if (1.0 > q) q = 1.0;
  return (a - b) / q;
}

// A rounded quotient fl(d/q), q > 0, against a double t, decided from the three exponents where they settle it:
// -1 when fl(d/q) < t, 1 when fl(d/q) > t, 0 when the exponents leave it open.  With |d| in [2^a, 2^(a+1)) and q in
// [2^b, 2^(b+1)), |d|/q lies in (2^(a-b-1), 2^(a-b+1)); |t| lies in [2^c, 2^(c+1)).  If a-b >= c+2 the quotient
// exceeds 2^(c+1) and so does its rounding (a power of two is a double and rounding is monotone); if a-b <= c-2
// it stays below 2^(c-1) and so does its rounding.  Signs decide when they differ (fl(-x) = -fl(x)); subnormal or
// non-finite operands are left open.
__host__ __device__ __forceinline__ int quotCmp(double d, double q, double t) {
  const long long bd = dbits(d), bt = dbits(t);
  const long long md = bd & DMAG, mt = bt & DMAG;
  if (md == 0) return mt == 0 ? 0 : (bt < 0 ? 1 : -1);
  if (mt == 0) return 0;  // a zero threshold: the quotient may round to zero
  if ((bd < 0) != (bt < 0)) return bd < 0 ? -1 : 1;
  const int ea = (int)(md >> 52), eb = (int)(dbits(q) >> 52), ec = (int)(mt >> 52);
  if (ea == 0 || eb == 0 || ec == 0 || ea == 0x7ff || eb == 0x7ff || ec == 0x7ff) return 0;
  const int e = ea - eb + 1023;  // biased exponent of 2^(a-b)
  const int mag = e >= ec + 2 ? 1 : (e <= ec - 2 ? -1 : 0);
  return bd < 0 ? -mag : mag;
}

// Tests of a rounded quotient against a threshold, decided like the division itself but mostly without it
// (a double division is a long FP64 instruction sequence on this part).  The exponents settle most cases
// (quotCmp).  Otherwise, for q > 0, fl(d/q) < t holds when the exact d/q < t by more than the rounding of
// fl(d/q), and fails when the exact d/q >= t (rounding is monotone and t is a double).  Comparing d with the
// rounded product t*q decides both cases whenever d lies outside a band of 2^-40 (relative) around t*q -- far
// wider than the product's own rounding (2^-53) -- and the division decides inside the band.  The 1e-290 floor
// covers a zero or subnormal product; callers keep d/q away from the subnormal range (q <= 1e30, |d| above
// 1e-290 outside the band).
__host__ __device__ __forceinline__ bool quotLt(double d, double q, double t) {
  const int c = quotCmp(d, q, t);
  if (c != 0) return c < 0;
  const double tq = t * q;
  const double m = fabs(tq) * 0x1p-40 + 1e-290;
  if (d < tq - m) return true;
  if (d > tq + m) return false;
  return d / q < t;
}
__host__ __device__ __forceinline__ bool quotGt(double d, double q, double t) {
  const int c = quotCmp(d, q, t);
  if (c != 0) return c > 0;
  const double tq = t * q;
  const double m = fabs(tq) * 0x1p-40 + 1e-290;
  if (d > tq + m) return true;
  if (d < tq - m) return false;
  return d / q > t;
}
// the denominator of SCIPrelDiff: max(|a|, |b|, 1), on magnitudes
__host__ __device__ __forceinline__ double relDen(double a, double b) {
  long long q = dmag(a);
  const long long mb = dmag(b);
  if (mb > q) q = mb;
  if (0x3ff0000000000000LL > q) q = 0x3ff0000000000000LL;  // 1.0
  return bitsd(q);
}
// SCIPisFeasLT / SCIPisFeasGT / SCIPisFeasEQ (set.c:7025-7050): relDiff(a, b) against -feastol / feastol
__host__ __device__ __forceinline__ bool feasLt(const Num& s, double a, double b) { return quotLt(a - b, relDen(a, b), -s.feastol); }
__host__ __device__ __forceinline__ bool feasGt(const Num& s, double a, double b) { return quotGt(a - b, relDen(a, b), s.feastol); }
__host__ __device__ __forceinline__ bool feasEq(const Num& s, double a, double b) {
  const double d = a - b, q = relDen(a, b);
  return !quotGt(d, q, s.feastol) && !quotLt(d, q, -s.feastol);
}
// EPSEQ(num / den, 1.0, eps) for |den| >= 1 - eps, the residual guard of tightenVarBounds
// (cons_linear.c:6766): |fl(num/den) - 1| is within 2^-52 of |num - den| / |den|, so a difference clearly
// above or below eps * |den| decides it; the division decides the rest.  The exponents of the difference, of eps
// and of den bound eps * |den| (in [2^(e+f), 2^(e+f+2)]) and settle most cases without the product.
__host__ __device__ __forceinline__ bool quotNear1(double num, double den, double eps) {
  if (eps < 1e-12) return fabs(num / den - 1.0) <= eps;  // the margins below need eps >> 2^-52
  const double diffs = num - den;
  const long long md = dmag(diffs);
  if (md == 0) return true;
  const int ed = (int)(md >> 52), ee = (int)(dbits(eps) >> 52), ef = (int)(dmag(den) >> 52);
  if (ed != 0 && ee != 0 && ef != 0 && ed != 0x7ff && ef != 0x7ff) {
    const int ef2 = ee + ef - 1023;  // biased exponent of 2^(e+f)
    if (ed >= ef2 + 4) return false;  // diff >= 2^(e+f+4) > 2 * eps * |den|
    if (ed <= ef2 - 2) return true;   // diff < 2^(e+f-1) <= eps * |den| / 2
  }
  const double diff = fabs(diffs), scale = eps * fabs(den);
  if (diff > 2.0 * scale) return false;
  if (diff < 0.5 * scale) return true;
  return fabs(num / den - 1.0) <= eps;
}
__host__ __device__ __forceinline__ double feasFloor(const Num& s, double x) { return floor(x + s.feastol); }
__host__ __device__ __forceinline__ double feasCeil(const Num& s, double x) { return ceil(x - s.feastol); }

// SCIPsetIsLbBetter / SCIPsetIsUbBetter, set.c:7711-7753 (minimal improvement "boundstreps").  A new bound that
// does not move past the old one fails at once: its difference is <= 0 and the threshold is >= 0.
__host__ __device__ __forceinline__ bool lbBetter(const Num& s, double nl, double ol, double ou) {
  if (dneg(ol) && !dneg(nl)) return true;
  if (!dgt(nl, ol)) return false;
  return dgt(nl - ol, s.bstreps * dmax(dmin(ou - ol, dabs(ol)), 1e-3));
}
__host__ __device__ __forceinline__ bool ubBetter(const Num& s, double nu, double ol, double ou) {
  if (dpos(ou) && !dpos(nu)) return true;
  if (!dlt(nu, ou)) return false;
  return dlt(nu - ou, -(s.bstreps * dmax(dmin(ou - ol, dabs(ou)), 1e-3)));
}

// SCIPsetIsUpdateUnreliable, set.c:8032-8046
__host__ __device__ __forceinline__ bool updateUnreliable(const Num& s, double nv, double ov) {
  return !quotLt(dabs(ov), dmax(dabs(nv), s.eps), s.recomp);  // fabs(ov) / max(|nv|, eps) >= recompfac
}

// adjustedLb / adjustedUb, var.c:1957-2020 (integral columns are rounded within feastol)
__host__ __device__ __forceinline__ double adjLb(const Num& s, bool isint, double lb) {
  if (isNegInf(s, lb)) return -s.inf;
  if (isInf(s, lb)) return s.inf;
  if (isint) return feasCeil(s, lb);
  if (dpos(lb) && !gec(lb, s.eps)) return 0.0;
  return lb;
}
__host__ __device__ __forceinline__ double adjUb(const Num& s, bool isint, double ub) {
  if (isInf(s, ub)) return s.inf;
  if (isNegInf(s, ub)) return -s.inf;
  if (isint) return feasFloor(s, ub);
  if (dneg(ub) && !lenc(ub, s.eps)) return 0.0;
  return ub;
}

// Compensated accumulation (hi, lo) += b: Knuth's TwoSum on the high word, low words added without
// renormalisation -- the accumulation SCIP applies to activities (dbldblarith.h SCIPdbldblSum21).
__host__ __device__ __forceinline__ void sum21(double& hi, double& lo, double b) {
  double s = hi + b;
  double bb = s - hi;
  double err = (hi - (s - bb)) + (b - bb);
  lo = err + lo;
  hi = s;
}

// The same accumulation for a nonzero summand b added to a high word that is not -0 (every per-entry
// contribution and every partial merge): the rounding error of hi + b is computed with Dekker's Fast2Sum
// after ordering the operands by magnitude, compared as integer bit patterns off the FP64 pipe.  Fast2Sum
// and TwoSum both return the exact rounding error (an exact zero as +0 in both), so (hi, lo) is bit for bit
// what sum21 gives, with 4 FP64 operations instead of 7.
__device__ __forceinline__ void sum21f(double& hi, double& lo, double b) {
  const double s = hi + b;
  const bool hbig = (__double_as_longlong(hi) & 0x7fffffffffffffffLL) >= (__double_as_longlong(b) & 0x7fffffffffffffffLL);
  const double x = hbig ? hi : b;
  const double y = hbig ? b : hi;
  const double err = y - (s - x);
  lo = err + lo;
  hi = s;
}

// Order-preserving int64 key of a double, for atomicMin / atomicMax on candidate bounds.
__device__ __forceinline__ long long dkey(double x) {
  long long i = __double_as_longlong(x);
  return i >= 0 ? i : (i ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double keyd(long long k) {
  return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffLL));
}

// Activity of one row: double-double finite parts plus infinity/huge counters
// (struct SCIP_ConsData minactivity/maxactivity and the eight counters, cons_linear.c:187-266).
struct Act {
  double minhi, minlo, maxhi, maxlo;
  int minposinf, minneginf, minposhuge, minneghuge;
  int maxposinf, maxneginf, maxposhuge, maxneghuge;
};

__device__ __forceinline__ void actZero(Act& a) {
  a.minhi = a.minlo = a.maxhi = a.maxlo = 0.0;
  a.minposinf = a.minneginf = a.minposhuge = a.minneghuge = 0;
  a.maxposinf = a.maxneginf = a.maxposhuge = a.maxneghuge = 0;
}

// One contribution val*bound (consdataUpdateActivities with old bound 0, cons_linear.c:1772-1945).
__device__ __forceinline__ void addContribution(const Num& s, double val, double bound, double& hi, double& lo,
                                                int& posinf, int& neginf, int& poshuge, int& neghuge) {
  if (isInf(s, dabs(bound))) {
    if (dpos(val) == dpos(bound)) ++posinf; else ++neginf;
  } else {
    double c = val * bound;
    if (isHuge(s, dabs(c))) {
      if (dpos(c)) ++poshuge; else ++neghuge;
    } else if (dmag(c) != 0) {
      sum21f(hi, lo, c);
    }
  }
}

__device__ __forceinline__ void addTerm(const Num& s, Act& a, double val, double lb, double ub) {
  addContribution(s, val, dpos(val) ? lb : ub, a.minhi, a.minlo, a.minposinf, a.minneginf, a.minposhuge,
                  a.minneghuge);
  addContribution(s, val, dpos(val) ? ub : lb, a.maxhi, a.maxlo, a.maxposinf, a.maxneginf, a.maxposhuge,
                  a.maxneghuge);
}

// Combination of two partial activities (lane partials of long rows): b's high word enters through the
// compensated sum, its low word is added to the low word.
__device__ __forceinline__ void actMerge(Act& a, const Act& b) {
  sum21f(a.minhi, a.minlo, b.minhi);
  a.minlo = a.minlo + b.minlo;
  sum21f(a.maxhi, a.maxlo, b.maxhi);
  a.maxlo = a.maxlo + b.maxlo;
  a.minposinf += b.minposinf; a.minneginf += b.minneginf; a.minposhuge += b.minposhuge; a.minneghuge += b.minneghuge;
  a.maxposinf += b.maxposinf; a.maxneginf += b.maxneginf; a.maxposhuge += b.maxposhuge; a.maxneghuge += b.maxneghuge;
}

// getMinActivity / getMaxActivity, cons_linear.c:2345-2529
__device__ __forceinline__ void getMinAct(const Num& s, const Act& a, int posinf, int neginf, int poshuge,
                                          int neghuge, double delta, bool goodrelax, double& val, bool& tight,
                                          bool& settoinf) {
  if (neginf > 0) { val = -s.inf; settoinf = true; tight = (posinf == 0); }
  else if (posinf > 0) { val = s.inf; settoinf = true; tight = true; }
  else if (neghuge > 0 || (poshuge > 0 && !goodrelax)) { val = -s.inf; settoinf = true; tight = false; }
  else {
    double hi = a.minhi, lo = a.minlo;
    // subtracting a zero delta leaves (hi, lo) as they are: hi is never -0 and the sum's error is +0
    if ((__double_as_longlong(delta) & 0x7fffffffffffffffLL) != 0) sum21f(hi, lo, -delta);
    if (poshuge > 0) { sum21(hi, lo, poshuge * s.huge); tight = false; }
    else tight = true;
    val = hi + lo;
    settoinf = false;
  }
}
__device__ __forceinline__ void getMaxAct(const Num& s, const Act& a, int posinf, int neginf, int poshuge,
                                          int neghuge, double delta, bool goodrelax, double& val, bool& tight,
                                          bool& settoinf) {
  if (posinf > 0) { val = s.inf; settoinf = true; tight = (neginf == 0); }
  else if (neginf > 0) { val = -s.inf; settoinf = true; tight = true; }
  else if (poshuge > 0 || (neghuge > 0 && !goodrelax)) { val = s.inf; settoinf = true; tight = false; }
  else {
    double hi = a.maxhi, lo = a.maxlo;
    if ((__double_as_longlong(delta) & 0x7fffffffffffffffLL) != 0) sum21f(hi, lo, -delta);
    if (neghuge > 0) { sum21(hi, lo, -neghuge * s.huge); tight = false; }
    else tight = true;
    val = hi + lo;
    settoinf = false;
  }
}

// consdataGetActivityResiduals, cons_linear.c:2661-2806 (goodrelax FALSE, as tightenVarBounds asks)
__device__ __forceinline__ void residuals(const Num& s, const Act& a, double val, double lb, double ub,
                                          double& minres, double& maxres, bool& mintight, bool& maxtight,
                                          bool& mininf, bool& maxinf) {
  double minb, maxb, absval;
  if (dpos(val)) { minb = lb; maxb = ub; absval = val; }
  else { minb = -ub; maxb = -lb; absval = -val; }
  if (isInf(s, minb))
    getMinAct(s, a, a.minposinf - 1, a.minneginf, a.minposhuge, a.minneghuge, 0.0, false, minres, mintight, mininf);
  else if (isNegInf(s, minb))
    getMinAct(s, a, a.minposinf, a.minneginf - 1, a.minposhuge, a.minneghuge, 0.0, false, minres, mintight, mininf);
  else if (isHuge(s, minb * absval))
    getMinAct(s, a, a.minposinf, a.minneginf, a.minposhuge - 1, a.minneghuge, 0.0, false, minres, mintight, mininf);
  else if (isNegHuge(s, minb * absval))
    getMinAct(s, a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge - 1, 0.0, false, minres, mintight, mininf);
  else
    getMinAct(s, a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, absval * minb, false, minres, mintight,
              mininf);

  if (isNegInf(s, maxb))
    getMaxAct(s, a, a.maxposinf, a.maxneginf - 1, a.maxposhuge, a.maxneghuge, 0.0, false, maxres, maxtight, maxinf);
  else if (isInf(s, maxb))
    getMaxAct(s, a, a.maxposinf - 1, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, false, maxres, maxtight, maxinf);
  else if (isHuge(s, absval * maxb))
    getMaxAct(s, a, a.maxposinf, a.maxneginf, a.maxposhuge - 1, a.maxneghuge, 0.0, false, maxres, maxtight, maxinf);
  else if (isNegHuge(s, absval * maxb))
    getMaxAct(s, a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge - 1, 0.0, false, maxres, maxtight, maxinf);
  else
    getMaxAct(s, a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, absval * maxb, false, maxres, maxtight,
              maxinf);
}

}  // namespace gbp
