// Host-side check of the decision helpers of gbp_rules.cuh: the division-free quotient tests must decide exactly
// like the division they replace, and the bit-pattern comparisons exactly like the double comparisons they
// replace, including inputs placed within a few units in the last place of a threshold and signed zeros.
// Built and run by tests/test_rules_cpu.py (nvcc, host code only).  Prints "ok <cases>" or the first
// disagreement and exits non-zero.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../../scip_gb300/csrc/gbp_rules.cuh"

using namespace gbp;

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next() {
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}
static double unit() { return (double)(next() >> 11) * 0x1p-53; }
static double logu(double lo, double hi) { return std::exp(std::log(lo) + unit() * (std::log(hi) - std::log(lo))); }
static double nudge(double x, int k) {  // x moved by k units in the last place (through zero as well)
  int64_t b;
  std::memcpy(&b, &x, 8);
  int64_t key = b >= 0 ? b : -(b & 0x7fffffffffffffffLL);  // ordered like the value
  key += k;
  b = key >= 0 ? key : ((-key) | (int64_t)0x8000000000000000ULL);
  double y;
  std::memcpy(&y, &b, 8);
  return y;
}

// the tests of gbp_rules.cuh as plain double comparisons (SCIP's definitions), for the bit-pattern versions
namespace ref {
static bool lt(const Num& s, double a, double b) { return a - b < -s.eps; }
static bool le(const Num& s, double a, double b) { return a - b <= s.eps; }
static bool gt(const Num& s, double a, double b) { return a - b > s.eps; }
static bool ge(const Num& s, double a, double b) { return a - b >= -s.eps; }
static bool eq(const Num& s, double a, double b) { return std::fabs(a - b) <= s.eps; }
static bool sumGt(const Num& s, double a, double b) { return a - b > s.sumeps; }
static bool positive(const Num& s, double a) { return a > s.eps; }
static bool feasZero(const Num& s, double a) { return std::fabs(a) <= s.feastol; }
static bool isInf(const Num& s, double x) { return x >= s.inf; }
static bool isHuge(const Num& s, double x) { return x >= s.huge; }
static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }
static bool lbBetter(const Num& s, double nl, double ol, double ou) {
  if (ol < 0.0 && nl >= 0.0) return true;
  return nl - ol > s.bstreps * ref::dmax(ref::dmin(ou - ol, std::fabs(ol)), 1e-3);
}
static bool ubBetter(const Num& s, double nu, double ol, double ou) {
  if (ou > 0.0 && nu <= 0.0) return true;
  return nu - ou < -(s.bstreps * ref::dmax(ref::dmin(ou - ol, std::fabs(ou)), 1e-3));
}
static double adjLb(const Num& s, bool isint, double lb) {
  if (lb < 0.0 && ref::isInf(s, -lb)) return -s.inf;
  if (lb > 0.0 && ref::isInf(s, lb)) return s.inf;
  if (isint) return std::ceil(lb - s.feastol);
  if (lb > 0.0 && lb < s.eps) return 0.0;
  return lb;
}
static double adjUb(const Num& s, bool isint, double ub) {
  if (ub > 0.0 && ref::isInf(s, ub)) return s.inf;
  if (ub < 0.0 && ref::isInf(s, -ub)) return -s.inf;
  if (isint) return std::floor(ub + s.feastol);
  if (ub < 0.0 && ub > -s.eps) return 0.0;
  return ub;
}
}  // namespace ref

static bool same(double a, double b) { return std::memcmp(&a, &b, 8) == 0; }

static int fails = 0;
static void report(const char* what, double a, double b, double c, int got, int want) {
  if (fails++ < 5) std::printf("%s(%.17g, %.17g, %.17g): got %d want %d\n", what, a, b, c, got, want);
}

int main() {
  Num s{1e20, 1e-9, 1e-6, 1e-6, 1e15, 0.05, 1e6, 1e6, 0};
  const double ts[] = {1e-6, -1e-6, 1e6, 0.0, -0.0, 1.0, -1.0, 0.05};
  long cases = 0;
  for (int it = 0; it < 4000000; ++it) {
    const double t = ts[next() % 8];
    const double q = (next() & 1) ? 1.0 : logu(1.0, 1e20);
    double d;
    switch (next() % 4) {
      case 0: d = t * q; break;                                    // on the boundary product
      case 1: d = nudge(t * q, (int)(next() % 9) - 4); break;       // a few ulps around it
      case 2: d = (next() & 1 ? 1 : -1) * logu(1e-300, 1e25); break;
      default: d = t * q * (1.0 + (unit() - 0.5) * 1e-11); break;  // inside the 2^-40 band
    }
    ++cases;
    if (quotLt(d, q, t) != (d / q < t)) report("quotLt", d, q, t, quotLt(d, q, t), d / q < t);
    if (quotGt(d, q, t) != (d / q > t)) report("quotGt", d, q, t, quotGt(d, q, t), d / q > t);
    // feasibility comparisons against their relDiff definitions
    const double a = (next() & 1 ? 1 : -1) * logu(1e-8, 1e19);
    double b;
    switch (next() % 3) {
      case 0: b = a * (1.0 + (unit() - 0.5) * 4e-6); break;
      case 1: b = nudge(a - s.feastol * relDen(a, a), (int)(next() % 9) - 4); break;
      default: b = (next() & 1 ? 1 : -1) * logu(1e-8, 1e19); break;
    }
    const double r = relDiff(a, b);
    if (feasLt(s, a, b) != (r < -s.feastol)) report("feasLt", a, b, 0, feasLt(s, a, b), r < -s.feastol);
    if (feasGt(s, a, b) != (r > s.feastol)) report("feasGt", a, b, 0, feasGt(s, a, b), r > s.feastol);
    if (feasEq(s, a, b) != (std::fabs(r) <= s.feastol)) report("feasEq", a, b, 0, feasEq(s, a, b), std::fabs(r) <= s.feastol);
    // the residual guard EPSEQ(num/den, 1, eps) for |den| >= 1
    const double den = (next() & 1 ? 1 : -1) * logu(1.0, 1e12);
    double num;
    switch (next() % 3) {
      case 0: num = den * (1.0 + (next() & 1 ? 1 : -1) * s.eps * (1.0 + (unit() - 0.5) * 1e-6)); break;
      case 1: num = nudge(den, (int)(next() % 2001) - 1000); break;
      default: num = den * (unit() * 3.0 - 1.0); break;
    }
    const bool want1 = std::fabs(num / den - 1.0) <= s.eps;
    if (quotNear1(num, den, s.eps) != want1) report("quotNear1", num, den, s.eps, quotNear1(num, den, s.eps), want1);
    // updateUnreliable: |ov| / max(|nv|, eps) >= recompfac
    const double ov = (next() & 1 ? 1 : -1) * logu(1e-6, 1e19);
    const double nv = (next() % 3 == 0) ? nudge(ov / s.recomp, (int)(next() % 9) - 4) : (next() & 1 ? 1 : -1) * logu(1e-12, 1e19);
    const bool wantu = std::fabs(ov) / dmax(std::fabs(nv), s.eps) >= s.recomp;
    if (updateUnreliable(s, nv, ov) != wantu) report("updateUnreliable", nv, ov, 0, updateUnreliable(s, nv, ov), wantu);
  }
  // the bit-pattern comparisons against their plain definitions, with tolerances of 0 too: values near every
  // threshold, signed zeros, infinities and huge values
  const Num nums[2] = {s, Num{1e20, 0.0, 0.0, 0.0, 1e15, 0.0, 1e6, 1e6, 0}};
  const double specials[] = {0.0, -0.0, 1e-9, -1e-9, 1e-6, -1e-6, 1.0, -1.0, 0.5, -0.5, 1e15, -1e15, 1e20, -1e20, 1e-3, 3.0};
  for (int it = 0; it < 2000000; ++it) {
    const Num& n = nums[it & 1];
    auto draw = [&]() {
      switch (next() % 5) {
        case 0: return specials[next() % 16];
        case 1: return nudge(specials[next() % 16], (int)(next() % 9) - 4);
        case 2: return (next() & 1 ? 1 : -1) * logu(1e-12, 1e21);
        case 3: return (double)((int64_t)(next() % 21) - 10);
        default: return (next() & 1 ? 1 : -1) * logu(1e-3, 1e3);
      }
    };
    double a = draw(), b = draw(), c = draw();
    if (next() % 4 == 0) b = nudge(a + ((next() & 1) ? n.eps : -n.eps), (int)(next() % 5) - 2);  // a - b near +-eps
    ++cases;
#define CMP(f, ...) if (f(__VA_ARGS__) != ref::f(__VA_ARGS__)) report(#f, a, b, c, f(__VA_ARGS__), ref::f(__VA_ARGS__))
    CMP(lt, n, a, b); CMP(le, n, a, b); CMP(gt, n, a, b); CMP(ge, n, a, b); CMP(eq, n, a, b); CMP(sumGt, n, a, b);
    CMP(positive, n, a); CMP(feasZero, n, a); CMP(isInf, n, a); CMP(isHuge, n, a);
#undef CMP
    if (isNegInf(n, a) != ref::isInf(n, -a)) report("isNegInf", a, 0, 0, isNegInf(n, a), ref::isInf(n, -a));
    if (isNegHuge(n, a) != ref::isHuge(n, -a)) report("isNegHuge", a, 0, 0, isNegHuge(n, a), ref::isHuge(n, -a));
    if (dpos(a) != (a > 0.0) || dneg(a) != (a < 0.0)) report("dpos/dneg", a, 0, 0, dpos(a), a > 0.0);
    if (!same(dmax(a, b), ref::dmax(a, b))) report("dmax", a, b, 0, 0, 1);
    if (!same(dmin(a, b), ref::dmin(a, b))) report("dmin", a, b, 0, 0, 1);
    if (!same(dabs(a), std::fabs(a))) report("dabs", a, 0, 0, 0, 1);
    // bounds: ol <= ou
    const double ol = ref::dmin(b, c), ou = ref::dmax(b, c);
    if (lbBetter(n, a, ol, ou) != ref::lbBetter(n, a, ol, ou)) report("lbBetter", a, ol, ou, lbBetter(n, a, ol, ou), ref::lbBetter(n, a, ol, ou));
    if (ubBetter(n, a, ol, ou) != ref::ubBetter(n, a, ol, ou)) report("ubBetter", a, ol, ou, ubBetter(n, a, ol, ou), ref::ubBetter(n, a, ol, ou));
    const bool isint = next() & 1;
    if (!same(adjLb(n, isint, a), ref::adjLb(n, isint, a))) report("adjLb", a, isint, 0, 0, 1);
    if (!same(adjUb(n, isint, a), ref::adjUb(n, isint, a))) report("adjUb", a, isint, 0, 0, 1);
  }
  if (fails) {
    std::printf("%d disagreements in %ld cases\n", fails, cases);
    return 1;
  }
  std::printf("ok %ld\n", cases);
  return 0;
}
