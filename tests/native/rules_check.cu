// Host-side check of the division-free decision helpers of gbp_rules.cuh: each must decide exactly like the
// division it replaces, including inputs placed within a few units in the last place of the threshold.
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
static double nudge(double x, int k) {  // x moved by k units in the last place
  int64_t b;
  std::memcpy(&b, &x, 8);
  if (x == 0.0) return k * 4.9406564584124654e-324;
  b += (x > 0 ? k : -k);
  double y;
  std::memcpy(&y, &b, 8);
  return y;
}

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
  if (fails) {
    std::printf("%d disagreements in %ld cases\n", fails, cases);
    return 1;
  }
  std::printf("ok %ld\n", cases);
  return 0;
}
