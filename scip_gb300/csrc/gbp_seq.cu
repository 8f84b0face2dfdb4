// Branch-and-bound nodes propagated in SCIP's own order (GBP_FLAG_SCIPORDER): marked rows one at a time, every
// tightening applied at once, activities updated incrementally by the bound-change events -- the order
// consPropLinear, tightenBounds and eventExecLinear produce (src/scip/cons_linear.c, src/scip/cons.c), so that the
// final bounds equal SCIP's, not only a valid fixpoint of the same rules.
//
// One warp runs one node at a time.  The node's logic is sequential, so every lane executes it identically (all
// decisions are warp-uniform), and the work inside a step is spread over the lanes:
//   - a row's activities, its reliable residual and its largest activity delta: the lanes load 32 entries at a
//     time; sums are then accumulated in the row's order through shuffles, so they round exactly as the scalar
//     loop does;
//   - a bound change's events: the lanes take the column's rows (ascending, the order the rows caught the column's
//     events) and update each row's state; the rows they mark are appended in that order through a ballot;
//   - tightenBounds' visit of a row's entries: the lanes evaluate 32 consecutive entries without changing any
//     state, and the first entry that would change something (a tightening, a cutoff, the recomputation of an
//     activity) or ends the visit of the binaries is then run for real; the entries before it change nothing, so
//     the outcome is the sequential one.  The evaluation may also report an entry it cannot settle cheaply (an
//     unreliable residual, which SCIP recomputes from scratch): running an entry that then changes nothing
//     advances the visit exactly as skipping it does.
// Per-node state lives in per-warp slots in HBM: a state record per row (stamped with the node's epoch, so a new
// node needs no clearing), the column bounds that differ from the base, and the marked-row and update lists.
//
// Every function restates the one of oracle/linprop_seq.c with the same name (which cites the SCIP source); the
// two are bit-identical (libgbp is compiled with --fmad=false).
#include <cub/device/device_radix_sort.cuh>

#include "gbp_internal.h"

namespace gbp {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double SEQ_INVALID = 1e99;  // SCIP_INVALID
__device__ __forceinline__ bool isInvalid(double x) { return dbits(x) == dbits(SEQ_INVALID); }
constexpr int MAXTIGHTENROUNDS = 10;  // cons_linear.c:6976

// SeqRow::flags
constexpr unsigned RS_VALID = 1u, RS_VMIN = 2u, RS_VMAX = 4u;
constexpr unsigned RS_BTSHIFT = 3u, RS_BTMASK = 3u << 3;  // boundstightened
constexpr unsigned RS_MP = 1u << 5, RS_EN = 1u << 6, RS_DEL = 1u << 7;
constexpr unsigned RS_UM = 1u << 8, RS_UU = 1u << 9, RS_UD = 1u << 10, RS_INUPD = 1u << 11;
constexpr unsigned RS_NBV = 1u << 12, RS_HNB = 1u << 13;  // nonbinvalid, hasnonbin

__device__ __forceinline__ unsigned btOf(unsigned f) { return (f & RS_BTMASK) >> RS_BTSHIFT; }
__device__ __forceinline__ unsigned withBt(unsigned f, unsigned bt) { return (f & ~RS_BTMASK) | (bt << RS_BTSHIFT); }

// Warp-uniform context of the node a warp runs.
struct W {
  const SeqArgs* A;
  SeqRow* rs;
  double2* ovl;
  int* ost;
  int* M;
  int* U;
  int* dirty;
  int epoch;
  int nm;         // marked rows
  int nu;         // rows with delayed updates
  int ndirty;     // columns changed since the base
  bool indelay;   // inside consPropLinear: marks, unmarks and deletions are delayed
  long long nchg; // tightenings of the current consPropLinear call
  int lane;
  long long rows, nnz, cands, live, changes;
};

__device__ __forceinline__ double2 bnd(const W& w, int j) {
  return w.ost[j] == w.epoch ? w.ovl[j] : w.A->base[j];
}

__device__ __forceinline__ bool isBinaryCol(const W& w, int j) {  // SCIPvarIsBinary on the base domain
  const double2 b = w.A->base[j];
  return w.A->P.isint[j] != 0 && !dneg(b.x) && !gtc(b.y, 1.0);
}

// rowSt: the row's record, initialised on the node's first touch
__device__ __forceinline__ SeqRow loadRow(const W& w, int i) {
  SeqRow r = w.rs[i];
  if (r.stamp != w.epoch) {
    r.minhi = r.minlo = r.maxhi = r.maxlo = 0.0;
    r.lastmin = r.lastmax = 0.0;
    r.maxdelta = SEQ_INVALID;
    r.minposinf = r.minneginf = r.minposhuge = r.minneghuge = 0;
    r.maxposinf = r.maxneginf = r.maxposhuge = r.maxneghuge = 0;
    r.maxdeltacol = -1;
    r.mpos = -1;
    r.evc = 0;
    r.stamp = w.epoch;
    // a node starts from the root's fixpoint: rows count as tightened there (tightenmode 2)
    r.flags = RS_EN | (2u << RS_BTSHIFT);
    if (w.A->prep[i] < 0) r.flags = (r.flags & ~RS_EN) | RS_DEL;  // deleted at the root
  }
  return r;
}
__device__ __forceinline__ void storeRow(const W& w, int i, const SeqRow& r) {
  if (w.lane == 0) w.rs[i] = r;
  __syncwarp();
}
__device__ __forceinline__ int nbinOf(const W& w, int i) { return w.A->prep[i] & 0x7fffffff; }

__device__ __forceinline__ Act actOf(const SeqRow& r) {
  Act a;
  a.minhi = r.minhi; a.minlo = r.minlo; a.maxhi = r.maxhi; a.maxlo = r.maxlo;
  a.minposinf = r.minposinf; a.minneginf = r.minneginf; a.minposhuge = r.minposhuge; a.minneghuge = r.minneghuge;
  a.maxposinf = r.maxposinf; a.maxneginf = r.maxneginf; a.maxposhuge = r.maxposhuge; a.maxneghuge = r.maxneghuge;
  return a;
}

// ------------------------------------------------------------------------------------------ activities
// calcActivities: every entry in the row's order through the counters or the compensated sum
__device__ __noinline__ void calcActivities(const W& w, int i, SeqRow& r) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p0 = P.rowptr[i];
  const int len = (int)(P.rowptr[i + 1] - p0);
  Act a;
  actZero(a);
  for (int k0 = 0; k0 < len; k0 += 32) {
    const int k = k0 + w.lane;
    double cmin = 0.0, cmax = 0.0;
    Act mine;
    actZero(mine);
    if (k < len) {
      const double v = P.vals[p0 + k];
      const double2 b = bnd(w, P.colidx[p0 + k]);
      // the counters of this entry, and its finite contributions (added below in order)
      double hi = 0.0, lo = 0.0;
      addContribution(s, v, dpos(v) ? b.x : b.y, hi, lo, mine.minposinf, mine.minneginf, mine.minposhuge,
                      mine.minneghuge);
      cmin = hi;
      hi = 0.0;
      addContribution(s, v, dpos(v) ? b.y : b.x, hi, lo, mine.maxposinf, mine.maxneginf, mine.maxposhuge,
                      mine.maxneghuge);
      cmax = hi;
    }
#define SEQ_CNT(f) a.f += __reduce_add_sync(FULL, (unsigned)mine.f)
    SEQ_CNT(minposinf); SEQ_CNT(minneginf); SEQ_CNT(minposhuge); SEQ_CNT(minneghuge);
    SEQ_CNT(maxposinf); SEQ_CNT(maxneginf); SEQ_CNT(maxposhuge); SEQ_CNT(maxneghuge);
#undef SEQ_CNT
    const int cnt = min(32, len - k0);
    for (int t = 0; t < cnt; ++t) {
      const double x = __shfl_sync(FULL, cmin, t);
      const double y = __shfl_sync(FULL, cmax, t);
      if (dmag(x) != 0) sum21f(a.minhi, a.minlo, x);
      if (dmag(y) != 0) sum21f(a.maxhi, a.maxlo, y);
    }
  }
  r.minhi = a.minhi; r.minlo = a.minlo; r.maxhi = a.maxhi; r.maxlo = a.maxlo;
  r.minposinf = a.minposinf; r.minneginf = a.minneginf; r.minposhuge = a.minposhuge; r.minneghuge = a.minneghuge;
  r.maxposinf = a.maxposinf; r.maxneginf = a.maxneginf; r.maxposhuge = a.maxposhuge; r.maxneghuge = a.maxneghuge;
  r.flags |= RS_VALID | RS_VMIN | RS_VMAX;
  r.lastmin = r.minhi + r.minlo;
  r.lastmax = r.maxhi + r.maxlo;
}

// recomputeSide: the finite non-huge part of one side, last entry first
__device__ __noinline__ void recomputeSide(const W& w, int i, SeqRow& r, bool ismin) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p0 = P.rowptr[i];
  const int len = (int)(P.rowptr[i + 1] - p0);
  double hi = 0.0, lo = 0.0;
  for (int k1 = len; k1 > 0; k1 -= 32) {
    // lanes take entries k1-1-lane (lane 0 the last of the chunk), summed in that order
    const int k = k1 - 1 - w.lane;
    double c = 0.0;
    bool use = false;
    if (k >= 0) {
      const double v = P.vals[p0 + k];
      const double2 b = bnd(w, P.colidx[p0 + k]);
      const double bb = (dpos(v)) == ismin ? b.x : b.y;
      if (!isInf(s, bb) && !isNegInf(s, bb) && !isHuge(s, v * bb) && !isNegHuge(s, v * bb)) {
        c = v * bb;
        use = true;
      }
    }
    const unsigned um = __ballot_sync(FULL, use);
    const int cnt = min(32, k1);
    for (int t = 0; t < cnt; ++t) {
      const double x = __shfl_sync(FULL, c, t);
      if (um & (1u << t)) sum21(hi, lo, x);
    }
  }
  if (ismin) {
    r.minhi = hi; r.minlo = lo; r.flags |= RS_VMIN; r.lastmin = hi + lo;
  } else {
    r.maxhi = hi; r.maxlo = lo; r.flags |= RS_VMAX; r.lastmax = hi + lo;
  }
}

__device__ __forceinline__ void ensureAct(const W& w, int i, SeqRow& r) {
  if (!(r.flags & RS_VALID)) calcActivities(w, i, r);
}

// the finite branch of getMinActivity / getMaxActivity recomputes an invalid side first
__device__ __forceinline__ bool minRecomputes(const SeqRow& r, int posinf, int neginf, int poshuge, int neghuge,
                                              bool goodrelax) {
  return neginf == 0 && posinf == 0 && !(neghuge > 0 || (poshuge > 0 && !goodrelax)) && !(r.flags & RS_VMIN);
}
__device__ __forceinline__ bool maxRecomputes(const SeqRow& r, int posinf, int neginf, int poshuge, int neghuge,
                                              bool goodrelax) {
  return posinf == 0 && neginf == 0 && !(poshuge > 0 || (neghuge > 0 && !goodrelax)) && !(r.flags & RS_VMAX);
}

// seqMin / seqMax (uniform: may recompute)
__device__ void seqMin(const W& w, int i, SeqRow& r, int posinf, int neginf, int poshuge, int neghuge, double delta,
                       bool goodrelax, double& val, bool& tight, bool& settoinf) {
  if (minRecomputes(r, posinf, neginf, poshuge, neghuge, goodrelax)) recomputeSide(w, i, r, true);
  getMinAct(w.A->s, actOf(r), posinf, neginf, poshuge, neghuge, delta, goodrelax, val, tight, settoinf);
}
__device__ void seqMax(const W& w, int i, SeqRow& r, int posinf, int neginf, int poshuge, int neghuge, double delta,
                       bool goodrelax, double& val, bool& tight, bool& settoinf) {
  if (maxRecomputes(r, posinf, neginf, poshuge, neghuge, goodrelax)) recomputeSide(w, i, r, false);
  getMaxAct(w.A->s, actOf(r), posinf, neginf, poshuge, neghuge, delta, goodrelax, val, tight, settoinf);
}

// activityBounds (uniform)
__device__ void activityBounds(const W& w, int i, SeqRow& r, bool goodrelax, double& minact, double& maxact,
                               bool& mint, bool& maxt, bool& mininf, bool& maxinf) {
  ensureAct(w, i, r);
  seqMin(w, i, r, r.minposinf, r.minneginf, r.minposhuge, r.minneghuge, 0.0, goodrelax, minact, mint, mininf);
  seqMax(w, i, r, r.maxposinf, r.maxneginf, r.maxposhuge, r.maxneghuge, 0.0, goodrelax, maxact, maxt, maxinf);
}

// the counters getMinActivity / getMaxActivity are called with for the residual of an entry (minb/maxb: the
// entry's min/max bound with the coefficient's sign folded in), and the delta to subtract
struct ResArgs {
  int mp, mn, mph, mnh;
  double md;
  int xp, xn, xph, xnh;
  double xd;
};
__device__ __forceinline__ ResArgs resArgs(const Num& s, const SeqRow& r, double val, double l, double u) {
  double minb, maxb, absval;
  if (dpos(val)) { minb = l; maxb = u; absval = val; }
  else { minb = -u; maxb = -l; absval = -val; }
  ResArgs a{r.minposinf, r.minneginf, r.minposhuge, r.minneghuge, 0.0,
            r.maxposinf, r.maxneginf, r.maxposhuge, r.maxneghuge, 0.0};
  if (isInf(s, minb)) a.mp -= 1;
  else if (isNegInf(s, minb)) a.mn -= 1;
  else if (isHuge(s, minb * absval)) a.mph -= 1;
  else if (isNegHuge(s, minb * absval)) a.mnh -= 1;
  else a.md = absval * minb;
  if (isNegInf(s, maxb)) a.xn -= 1;
  else if (isInf(s, maxb)) a.xp -= 1;
  else if (isHuge(s, absval * maxb)) a.xph -= 1;
  else if (isNegHuge(s, absval * maxb)) a.xnh -= 1;
  else a.xd = absval * maxb;
  return a;
}

// reliableRes: plain double sum in the row's order, skipping the column (uniform: lanes load, lane order sums)
__device__ __noinline__ double reliableResWarp(const W& w, int i, int skipcol, bool ismin) {
  const Prob& P = w.A->P;
  const int64_t p0 = P.rowptr[i];
  const int len = (int)(P.rowptr[i + 1] - p0);
  double res = 0.0;
  for (int k0 = 0; k0 < len; k0 += 32) {
    const int k = k0 + w.lane;
    double c = 0.0;
    bool use = false;
    if (k < len) {
      const int j = P.colidx[p0 + k];
      if (j != skipcol) {
        const double v = P.vals[p0 + k];
        const double2 b = bnd(w, j);
        c = dpos(v) ? (ismin ? v * b.x : v * b.y) : (ismin ? v * b.y : v * b.x);
        use = true;
      }
    }
    const unsigned um = __ballot_sync(FULL, use);
    const int cnt = min(32, len - k0);
    for (int t = 0; t < cnt; ++t) {
      const double x = __shfl_sync(FULL, c, t);
      if (um & (1u << t)) res += x;
    }
  }
  return res;
}
// recomputeMaxDelta, last entry first (uniform)
__device__ __noinline__ void recomputeMaxDelta(const W& w, int i, SeqRow& r) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p0 = P.rowptr[i];
  const int len = (int)(P.rowptr[i + 1] - p0);
  r.maxdelta = 0.0;
  if (!(r.flags & RS_NBV)) {
    bool nonbin = false;
    for (int k = w.lane; k < len; k += 32) nonbin |= !isBinaryCol(w, P.colidx[p0 + k]);
    if (__any_sync(FULL, nonbin)) r.flags |= RS_HNB;
    else r.flags &= ~RS_HNB;
    r.flags |= RS_NBV;
  }
  const bool binonly = !(r.flags & RS_HNB);
  // the reverse scan keeps the first maximum it meets, i.e. the largest position among equal deltas; without
  // binaries only, the first infinite domain it meets (the largest such position) ends it with infinity
  double best = 0.0;
  int bestk = -1, infk = -1;
  for (int k = w.lane; k < len; k += 32) {
    const int j = P.colidx[p0 + k];
    const double2 b = bnd(w, j);
    double d;
    if (binonly) {
      if (gec(b.x, 0.5) || !gtc(b.y, 0.5)) continue;  // not b.x < 0.5 < b.y
      d = dabs(P.vals[p0 + k]);
    } else {
      if (isNegInf(s, b.x) || isInf(s, b.y)) {
        infk = k;  // k grows within the lane: the lane's largest
        continue;
      }
      d = dabs(P.vals[p0 + k]) * (b.y - b.x);
    }
    if (dgt(d, best) || (!dlt(d, best) && dpos(d))) {  // later positions win ties
      best = d;
      bestk = k;
    }
  }
  const int inf_any = __reduce_max_sync(FULL, (unsigned)(infk + 1)) - 1;
  if (inf_any >= 0) {
    r.maxdelta = s.inf;
    r.maxdeltacol = P.colidx[p0 + inf_any];
    return;
  }
  for (int off = 16; off > 0; off >>= 1) {
    const double ob = __shfl_xor_sync(FULL, best, off);
    const int ok = __shfl_xor_sync(FULL, bestk, off);
    if (ob > best || (ob == best && ok > bestk)) {
      best = ob;
      bestk = ok;
    }
  }
  if (bestk >= 0) {
    r.maxdelta = best;
    r.maxdeltacol = P.colidx[p0 + bestk];
  }
}

// consdataUpdateActivities for a local bound change, checkreliability TRUE (one lane, one row)
__device__ void updateActivities(const Num& s, SeqRow& r, double val, double oldb, double newb, bool islb) {
  const bool ismin = islb == (dpos(val));
  double *hi, *lo, *last;
  int *posinf, *neginf, *poshuge, *neghuge;
  bool validact;
  if (ismin) {
    hi = &r.minhi; lo = &r.minlo; last = &r.lastmin; validact = (r.flags & RS_VMIN) != 0;
    poshuge = &r.minposhuge; neghuge = &r.minneghuge;
    posinf = dpos(val) ? &r.minposinf : &r.minneginf;
    neginf = dpos(val) ? &r.minneginf : &r.minposinf;
  } else {
    hi = &r.maxhi; lo = &r.maxlo; last = &r.lastmax; validact = (r.flags & RS_VMAX) != 0;
    poshuge = &r.maxposhuge; neghuge = &r.maxneghuge;
    posinf = dpos(val) ? &r.maxposinf : &r.maxneginf;
    neginf = dpos(val) ? &r.maxneginf : &r.maxposinf;
  }
  double dhi = 0.0, dlo = 0.0;
  const double oldc = val * oldb, newc = val * newb;
  const bool hugenew = isHuge(s, dabs(newc));
  const bool finnew = !isInf(s, dabs(newb));
  if (isInf(s, dabs(oldb))) {
    if (dpos(oldb)) {
      if (finnew || dneg(newb)) {
        (*posinf)--;
        if (!finnew && dneg(newb)) (*neginf)++;
        else if (hugenew) { if (dpos(newc)) (*poshuge)++; else (*neghuge)++; }
        else dhi = newc;
      }
    } else {
      if (finnew || dpos(newb)) {
        (*neginf)--;
        if (!finnew && dpos(newb)) (*posinf)++;
        else if (hugenew) { if (dpos(newc)) (*poshuge)++; else (*neghuge)++; }
        else dhi = newc;
      }
    }
  } else if (isHuge(s, dabs(oldc))) {
    if (dpos(oldc)) (*poshuge)--; else (*neghuge)--;
    if (!finnew) { if (dpos(newb)) (*posinf)++; else (*neginf)++; }
    else if (hugenew) { if (dpos(newc)) (*poshuge)++; else (*neghuge)++; }
    else dhi = newc;
  } else {
    if (!finnew) {
      if (dpos(newb)) (*posinf)++; else (*neginf)++;
      dhi = -oldc;
    } else if (hugenew) {
      if (dpos(newc)) (*poshuge)++; else (*neghuge)++;
      dhi = -oldc;
    } else {
      dhi = newc;
      sum21(dhi, dlo, -oldc);
    }
  }
  const double dsum = dhi + dlo;
  if (validact && dmag(dsum) != 0) {
    sum21(*hi, *lo, dsum);
    const double cur = *hi + *lo;
    if (dmag(*last) < dmag(cur)) *last = cur;
    else if (updateUnreliable(s, cur, *last)) r.flags &= ismin ? ~RS_VMIN : ~RS_VMAX;
  }
}

// ------------------------------------------------------------------------------------------ marked rows
__device__ __forceinline__ void addUpdate(W& w, int i, SeqRow& r) {
  if (r.flags & RS_INUPD) return;
  r.flags |= RS_INUPD;
  if (w.lane == 0) w.U[w.nu] = i;
  w.nu += 1;
}
// SCIPconsUnmarkPropagate inside the call
__device__ __forceinline__ void unmarkProp(W& w, int i, SeqRow& r) {
  if ((r.flags & RS_UU) || (!(r.flags & RS_MP) && !(r.flags & RS_UM))) return;
  r.flags = (r.flags & ~RS_UM) | RS_UU;
  addUpdate(w, i, r);
}
// SCIPconsDisable inside the call
__device__ __forceinline__ void disableRow(W& w, int i, SeqRow& r) {
  if ((r.flags & RS_UD) || !(r.flags & RS_EN)) return;
  r.flags |= RS_UD;
  addUpdate(w, i, r);
}
// conshdlrProcessUpdates: the delayed updates, the last added first
__device__ __noinline__ void processUpdates(W& w) {
  // scalar list work on two fields of each record (flags, list position): one lane does it, the others wait
  int nm = w.nm;
  if (w.lane == 0) {
    for (int k = w.nu - 1; k >= 0; --k) {
      const int i = w.U[k];
      unsigned f = w.rs[i].flags;
      int mpos = w.rs[i].mpos;  // an earlier unmark in this loop may have moved the row
      auto unmark = [&]() {     // conshdlrUnmarkConsPropagate: the last marked row moves into the hole
        if (!(f & RS_EN) || !(f & RS_MP)) return;
        f &= ~RS_MP;
        const int pos = mpos;
        mpos = -1;
        nm -= 1;
        if (pos < nm) {
          const int last = w.M[nm];
          w.M[pos] = last;
          w.rs[last].mpos = pos;
        }
      };
      if (f & RS_UD) {
        unmark();
        f &= ~(RS_EN | RS_UD);
      }
      if (f & RS_UM) {  // conshdlrMarkConsPropagate: append
        if ((f & RS_EN) && !(f & RS_MP)) {
          f |= RS_MP;
          mpos = nm;
          w.M[nm] = i;
          nm += 1;
        }
      } else if (f & RS_UU) {
        unmark();
      }
      w.rs[i].flags = f & ~(RS_UM | RS_UU | RS_INUPD);
      w.rs[i].mpos = mpos;
    }
  }
  __syncwarp();
  w.nm = __shfl_sync(FULL, nm, 0);
  w.nu = 0;
}

// ------------------------------------------------------------------------------------------ bound changes
// the column's overlay entry and the dirty list (uniform)
__device__ __forceinline__ void setBound(W& w, int j, double l, double u) {
  const bool fresh = w.ost[j] != w.epoch;
  __syncwarp();
  if (w.lane == 0) {
    if (fresh) {
      w.ost[j] = w.epoch;
      w.dirty[w.ndirty] = j;
    }
    w.ovl[j] = make_double2(l, u);
  }
  if (fresh) w.ndirty += 1;
  __syncwarp();
}

// boundEvent: eventExecLinear for every row of column j, in row order (uniform; the lanes take the rows)
__device__ __noinline__ void boundEvent(W& w, int j, bool islb, double oldb, double newb) {
  const SeqArgs& A = *w.A;
  const Num& s = A.s;
  const int64_t q0 = A.ccolptr[j], q1 = A.ccolptr[j + 1];
  for (int64_t qb = q0; qb < q1; qb += 32) {
    const int64_t q = qb + w.lane;
    bool appM = false, appU = false;
    int i = -1;
    SeqRow r;
    if (q < q1) {
      i = A.crow[q];
      const double a = A.cval[q];
      r = loadRow(w, i);
      if (!(r.flags & RS_DEL)) {
        if (r.flags & RS_VALID) updateActivities(s, r, a, oldb, newb, islb);
        // SCIPconsMarkPropagate: delayed inside the call, at once outside it
        if (!((r.flags & RS_UM) || ((r.flags & RS_MP) && !(r.flags & RS_UU)))) {
          if (w.indelay) {
            r.flags = (r.flags & ~RS_UU) | RS_UM;
            if (!(r.flags & RS_INUPD)) {
              r.flags |= RS_INUPD;
              appU = true;
            }
          } else if ((r.flags & RS_EN) && !(r.flags & RS_MP)) {
            r.flags |= RS_MP;
            appM = true;
          }
        }
        r.evc += 1;
        if (r.maxdeltacol == j) {
          r.maxdelta = SEQ_INVALID;
          r.maxdeltacol = -1;
        }
        if (btOf(r.flags) > 0) {
          const bool rhsfin = !isInf(s, A.P.rhs[i]), lhsfin = !isNegInf(s, A.P.lhs[i]);
          if (islb ? (dpos(a) ? rhsfin : lhsfin) : (dpos(a) ? lhsfin : rhsfin)) r.flags = withBt(r.flags, 0);
        }
      }
    }
    const unsigned bm = __ballot_sync(FULL, appM), bu = __ballot_sync(FULL, appU);
    const unsigned below = (1u << w.lane) - 1u;
    if (appM) {
      r.mpos = w.nm + __popc(bm & below);
      w.M[r.mpos] = i;
    }
    if (appU) w.U[w.nu + __popc(bu & below)] = i;
    if (q < q1 && !(r.flags & RS_DEL)) w.rs[i] = r;
    w.nm += __popc(bm);
    w.nu += __popc(bu);
    __syncwarp();
  }
}

// inferUb / inferLb (uniform); return true on infeasibility, *tightened when the bound moved
__device__ __noinline__ bool inferUb(W& w, int j, double newub, bool force, bool& tightened) {
  const Num& s = w.A->s;
  const bool isint = w.A->P.isint[j] != 0;
  const double2 b = bnd(w, j);
  tightened = false;
  newub = adjUb(s, isint, newub);
  if (isNegInf(s, newub) || feasLt(s, newub, b.x)) return true;
  newub = dmax(newub, b.x);
  if ((force && ge(s, newub, b.y)) || (!force && !ubBetter(s, newub, b.x, b.y))) return false;
  if (!lt(s, newub, b.y)) return false;
  setBound(w, j, b.x, newub);
  w.nchg += 1;
  w.changes += 1;
  boundEvent(w, j, false, b.y, newub);
  tightened = true;
  return false;
}
__device__ __noinline__ bool inferLb(W& w, int j, double newlb, bool force, bool& tightened) {
  const Num& s = w.A->s;
  const bool isint = w.A->P.isint[j] != 0;
  const double2 b = bnd(w, j);
  tightened = false;
  newlb = adjLb(s, isint, newlb);
  if (isInf(s, newlb) || feasGt(s, newlb, b.y)) return true;
  newlb = dmin(newlb, b.y);
  if ((force && le(s, newlb, b.x)) || (!force && !lbBetter(s, newlb, b.x, b.y))) return false;
  if (!gt(s, newlb, b.x)) return false;
  setBound(w, j, newlb, b.y);
  w.nchg += 1;
  w.changes += 1;
  boundEvent(w, j, true, b.x, newlb);
  tightened = true;
  return false;
}
// what inferUb / inferLb would do, without doing it: 0 nothing, 1 a change or infeasibility
__device__ __forceinline__ bool wouldInferUb(const Num& s, bool isint, double l, double u, double newub, bool force) {
  newub = adjUb(s, isint, newub);
  if (isNegInf(s, newub) || feasLt(s, newub, l)) return true;
  newub = dmax(newub, l);
  if ((force && ge(s, newub, u)) || (!force && !ubBetter(s, newub, l, u))) return false;
  return lt(s, newub, u);
}
__device__ __forceinline__ bool wouldInferLb(const Num& s, bool isint, double l, double u, double newlb, bool force) {
  newlb = adjLb(s, isint, newlb);
  if (isInf(s, newlb) || feasGt(s, newlb, u)) return true;
  newlb = dmin(newlb, u);
  if ((force && le(s, newlb, l)) || (!force && !lbBetter(s, newlb, l, u))) return false;
  return gt(s, newlb, l);
}

// ------------------------------------------------------------------------------------------ one entry
// the side guard of the residual rule (cons_linear.c:6765-6766): a small side, or a residual not equal to it
__device__ __forceinline__ bool sideOk(const Num& s, double side, double res) {
  return lt(s, dabs(side), 1.0) || !quotNear1(res, side, s.eps);
}

// tightenVarBounds without effects (one lane, entry k of the row in r): true if running it might change anything
// -- recompute an activity, tighten a bound, or find the node infeasible.  A true answer only sends the entry to
// the real run, so cases it cannot settle cheaply (a zero coefficient) answer true.
//
// Both sides are tested as upper bounds on z = x or z = -x: a lower bound nl on x is the upper bound -nl on -x
// over [-u, -l], and every test of tightenVarBounds on a lower bound (gt, feasGt, lbBetter, the inference) is its
// upper-bound test on the negated values, bit for bit (negation is exact and the rules are symmetric).  The
// candidate is then fl(num / |a|) with num = rhs - minres (z = x when a > 0) or maxres - lhs (z = x when a < 0),
// so lanes with coefficients of either sign run the same instructions.  A candidate that does not undercut the
// upper bound of z passes none of the tests; that is decided on the quotient before dividing.
__device__ bool residualWould(const W& w, int i, const SeqRow& r, int k, bool force) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p = P.rowptr[i] + k;
  const int j = P.colidx[p];
  const double val = P.vals[p];
  if (dmag(val) == 0) return true;
  const double lhs = P.lhs[i], rhs = P.rhs[i];
  const bool isint = P.isint[j] != 0;
  const double2 b = bnd(w, j);
  const double l = b.x, u = b.y;
  const ResArgs ra = resArgs(s, r, val, l, u);
  if (minRecomputes(r, ra.mp, ra.mn, ra.mph, ra.mnh, false) || maxRecomputes(r, ra.xp, ra.xn, ra.xph, ra.xnh, false))
    return true;
  const Act a = actOf(r);
  double minres, maxres;
  bool mint, maxt, mininf, maxinf;
  getMinAct(s, a, ra.mp, ra.mn, ra.mph, ra.mnh, ra.md, false, minres, mint, mininf);
  getMaxAct(s, a, ra.xp, ra.xn, ra.xph, ra.xnh, ra.xd, false, maxres, maxt, maxinf);
  const bool pos = dpos(val);
  const double aval = dabs(val);
#pragma unroll 1
  for (int side = 0; side < 2; ++side) {
    const bool rs = side == 0;  // the right-hand side with the minimal residual, else the left with the maximal
    if (rs ? (mininf || isInf(s, rhs) || !mint) : (maxinf || isNegInf(s, lhs) || !maxt)) continue;
    const double sd = rs ? rhs : lhs, res = rs ? minres : maxres;
    if (!sideOk(s, sd, res)) continue;
    const bool zx = rs == pos;
    const double lz = zx ? l : -u, uz = zx ? u : -l;
    const double num = rs ? rhs - minres : maxres - lhs;
    if (!quotLt(num, aval, uz)) continue;
    const double nu = num / aval;
    if (isInf(s, nu)) continue;
    if (!((force && lt(s, nu, uz)) || (isint && feasLt(s, nu, uz)) || ubBetter(s, nu, lz, uz))) continue;
    // an unreliable residual is recomputed from scratch: the entry counts as a hit, run for real
    if (updateUnreliable(s, res, rs ? r.lastmin : r.lastmax)) return true;
    if (wouldInferUb(s, isint, lz, uz, nu, force)) return true;
  }
  return false;
}

// tightenVarBounds, run for real (uniform); returns true on cutoff.  r is reloaded after every change.
__device__ __noinline__ bool residualRun(W& w, int i, SeqRow& r, int k, bool force) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p = P.rowptr[i] + k;
  const int j = P.colidx[p];
  const double val = P.vals[p];
  const double lhs = P.lhs[i], rhs = P.rhs[i];
  const bool isint = P.isint[j] != 0;
  double2 b = bnd(w, j);
  double minres, maxres;
  bool mint, maxt, mininf, maxinf, tightened;
  {
    const ResArgs ra = resArgs(s, r, val, b.x, b.y);
    seqMin(w, i, r, ra.mp, ra.mn, ra.mph, ra.mnh, ra.md, false, minres, mint, mininf);
    seqMax(w, i, r, ra.xp, ra.xn, ra.xph, ra.xnh, ra.xd, false, maxres, maxt, maxinf);
    storeRow(w, i, r);
  }
  double l = b.x, u = b.y;
  if (dpos(val)) {
    if (!mininf && !isInf(s, rhs) && mint && sideOk(s, rhs, minres)) {
      double newub = (rhs - minres) / val;
      if (!isInf(s, newub) && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u))) {
        bool unrel = updateUnreliable(s, minres, r.lastmin);
        if (unrel) {
          minres = reliableResWarp(w, i, j, true);
          newub = (rhs - minres) / val;
          unrel = isNegInf(s, minres) || (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) || !isint) && (!force || !lt(s, newub, u)));
        }
        if (!unrel) {
          if (inferUb(w, j, newub, force, tightened)) return true;
          r = loadRow(w, i);
          if (tightened) u = bnd(w, j).y;
        }
      }
    }
    if (!maxinf && !isNegInf(s, lhs) && maxt && sideOk(s, lhs, maxres)) {
      double newlb = (lhs - maxres) / val;
      if (!isNegInf(s, newlb) && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u))) {
        if (updateUnreliable(s, maxres, r.lastmax)) {
          maxres = reliableResWarp(w, i, j, false);
          newlb = (lhs - maxres) / val;
          if (isInf(s, maxres) || (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint) && (!force || !gt(s, newlb, l))))
            return false;
        }
        if (inferLb(w, j, newlb, force, tightened)) return true;
        r = loadRow(w, i);
      }
    }
  } else {
    if (!mininf && !isInf(s, rhs) && mint && sideOk(s, rhs, minres)) {
      double newlb = (rhs - minres) / val;
      if (!isNegInf(s, newlb) && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u))) {
        bool unrel = updateUnreliable(s, minres, r.lastmin);
        if (unrel) {
          minres = reliableResWarp(w, i, j, true);
          newlb = (rhs - minres) / val;
          unrel = isNegInf(s, minres) || (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint) && (!force || !gt(s, newlb, l)));
        }
        if (!unrel) {
          if (inferLb(w, j, newlb, force, tightened)) return true;
          r = loadRow(w, i);
          if (tightened) l = bnd(w, j).x;
        }
      }
    }
    if (!maxinf && !isNegInf(s, lhs) && maxt && sideOk(s, lhs, maxres)) {
      double newub = (lhs - maxres) / val;
      if (!isInf(s, newub) && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u))) {
        if (updateUnreliable(s, maxres, r.lastmax)) {
          maxres = reliableResWarp(w, i, j, false);
          newub = (lhs - maxres) / val;
          if (isInf(s, maxres) || (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) && !isint) && (!force || !lt(s, newub, u))))
            return false;
        }
        if (inferUb(w, j, newub, force, tightened)) return true;
        r = loadRow(w, i);
      }
    }
  }
  return false;
}

// tightenVarBoundsEasy without effects (one lane)
__device__ bool easyWould(const W& w, int i, const SeqRow& r, int k, bool force) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p = P.rowptr[i] + k;
  const int j = P.colidx[p];
  const double val = P.vals[p];
  const double lhs = P.lhs[i], rhs = P.rhs[i];
  const bool isint = P.isint[j] != 0;
  const double2 b = bnd(w, j);
  const double l = b.x, u = b.y;
  if (!(r.flags & RS_VMIN)) return true;
  if (dpos(val)) {
    if (!isInf(s, rhs)) {
      const double minact = r.minhi + r.minlo;
      if (feasLt(s, rhs, minact)) return true;
      double slack = rhs - minact;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (u - l);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        const double nu = adjUb(s, isint, l + slack / val);
        if ((force || ubBetter(s, nu, l, u)) && wouldInferUb(s, isint, l, u, nu, force)) return true;
      }
    }
    if (!isNegInf(s, lhs)) {
      if (!(r.flags & RS_VMAX)) return true;
      const double maxact = r.maxhi + r.maxlo;
      if (feasLt(s, maxact, lhs)) return true;
      double slack = maxact - lhs;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (u - l);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        const double nl = adjLb(s, isint, u - slack / val);
        if ((force || lbBetter(s, nl, l, u)) && wouldInferLb(s, isint, l, u, nl, force)) return true;
      }
    }
  } else {
    if (!isInf(s, rhs)) {
      const double minact = r.minhi + r.minlo;
      if (feasLt(s, rhs, minact)) return true;
      double slack = rhs - minact;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (l - u);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        const double nl = adjLb(s, isint, u + slack / val);
        if ((force || lbBetter(s, nl, l, u)) && wouldInferLb(s, isint, l, u, nl, force)) return true;
      }
    }
    if (!isNegInf(s, lhs)) {
      if (!(r.flags & RS_VMAX)) return true;
      const double maxact = r.maxhi + r.maxlo;
      if (feasLt(s, maxact, lhs)) return true;
      double slack = maxact - lhs;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (l - u);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        const double nu = adjUb(s, isint, l - slack / val);
        if ((force || ubBetter(s, nu, l, u)) && wouldInferUb(s, isint, l, u, nu, force)) return true;
      }
    }
  }
  return false;
}

// easyUb / easyLb (tightenVarUb / tightenVarLb)
__device__ __forceinline__ bool easyUb(W& w, int j, double newub, double oldub, bool force) {
  bool t;
  newub = adjUb(w.A->s, w.A->P.isint[j] != 0, newub);
  if (force || ubBetter(w.A->s, newub, bnd(w, j).x, oldub)) return inferUb(w, j, newub, force, t);
  return false;
}
__device__ __forceinline__ bool easyLb(W& w, int j, double newlb, double oldlb, bool force) {
  bool t;
  newlb = adjLb(w.A->s, w.A->P.isint[j] != 0, newlb);
  if (force || lbBetter(w.A->s, newlb, oldlb, bnd(w, j).y)) return inferLb(w, j, newlb, force, t);
  return false;
}

// tightenVarBoundsEasy, run for real (uniform); returns true on cutoff
__device__ __noinline__ bool easyRun(W& w, int i, SeqRow& r, int k, bool force) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p = P.rowptr[i] + k;
  const int j = P.colidx[p];
  const double val = P.vals[p];
  const double lhs = P.lhs[i], rhs = P.rhs[i];
  double2 b = bnd(w, j);
  double l = b.x, u = b.y;
  ensureAct(w, i, r);
  if (!(r.flags & RS_VMIN)) recomputeSide(w, i, r, true);
  storeRow(w, i, r);
  if (dpos(val)) {
    if (!isInf(s, rhs)) {
      const double minact = r.minhi + r.minlo;
      if (feasLt(s, rhs, minact)) return true;
      double slack = rhs - minact;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (u - l);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        if (easyUb(w, j, l + slack / val, u, force)) return true;
        r = loadRow(w, i);
        u = bnd(w, j).y;
      }
    }
    if (!isNegInf(s, lhs)) {
      if (!(r.flags & RS_VMAX)) {
        recomputeSide(w, i, r, false);
        storeRow(w, i, r);
      }
      const double maxact = r.maxhi + r.maxlo;
      if (feasLt(s, maxact, lhs)) return true;
      double slack = maxact - lhs;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (u - l);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        if (easyLb(w, j, u - slack / val, l, force)) return true;
        r = loadRow(w, i);
      }
    }
  } else {
    if (!isInf(s, rhs)) {
      const double minact = r.minhi + r.minlo;
      if (feasLt(s, rhs, minact)) return true;
      double slack = rhs - minact;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (l - u);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        if (easyLb(w, j, u + slack / val, l, force)) return true;
        r = loadRow(w, i);
        l = bnd(w, j).x;
      }
    }
    if (!isNegInf(s, lhs)) {
      if (!(r.flags & RS_VMAX)) {
        recomputeSide(w, i, r, false);
        storeRow(w, i, r);
      }
      const double maxact = r.maxhi + r.maxlo;
      if (feasLt(s, maxact, lhs)) return true;
      double slack = maxact - lhs;
      if (!positive(s, slack)) slack = 0.0;
      const double alpha = val * (l - u);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        if (easyUb(w, j, l - slack / val, u, force)) return true;
        r = loadRow(w, i);
      }
    }
  }
  return false;
}

// ------------------------------------------------------------------------------------------ one row, one lane
// Most marked rows never reach tightenBounds' visit of their entries: SCIP's own tests (a tightened row, a largest
// activity delta within the slack) end them after a few activity computations.  The lanes run those computations
// for 32 consecutive rows of a call at once, each on a private copy of its row's record; a row that changes no bound
// changes nothing but its own record, so the rows before the first one that changes a bound end exactly as running
// them one after the other leaves them.  Every function restates its counterpart of oracle/linprop_seq.c step for
// step, one lane alone.

__device__ __noinline__ void laneCalc(const W& w, int i, SeqRow& r) {  // calcActivities
  const Prob& P = w.A->P;
  Act a;
  actZero(a);
  for (int64_t p = P.rowptr[i]; p < P.rowptr[i + 1]; ++p) {
    const double2 b = bnd(w, P.colidx[p]);
    addTerm(w.A->s, a, P.vals[p], b.x, b.y);
  }
  r.minhi = a.minhi; r.minlo = a.minlo; r.maxhi = a.maxhi; r.maxlo = a.maxlo;
  r.minposinf = a.minposinf; r.minneginf = a.minneginf; r.minposhuge = a.minposhuge; r.minneghuge = a.minneghuge;
  r.maxposinf = a.maxposinf; r.maxneginf = a.maxneginf; r.maxposhuge = a.maxposhuge; r.maxneghuge = a.maxneghuge;
  r.flags |= RS_VALID | RS_VMIN | RS_VMAX;
  r.lastmin = r.minhi + r.minlo;
  r.lastmax = r.maxhi + r.maxlo;
}

__device__ __noinline__ void laneRecompute(const W& w, int i, SeqRow& r, bool ismin) {  // recomputeSide
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  double hi = 0.0, lo = 0.0;
  for (int64_t p = P.rowptr[i + 1] - 1; p >= P.rowptr[i]; --p) {
    const double v = P.vals[p];
    const double2 b = bnd(w, P.colidx[p]);
    const double bb = (dpos(v)) == ismin ? b.x : b.y;
    if (!isInf(s, bb) && !isNegInf(s, bb) && !isHuge(s, v * bb) && !isNegHuge(s, v * bb)) sum21(hi, lo, v * bb);
  }
  if (ismin) {
    r.minhi = hi; r.minlo = lo; r.flags |= RS_VMIN; r.lastmin = hi + lo;
  } else {
    r.maxhi = hi; r.maxlo = lo; r.flags |= RS_VMAX; r.lastmax = hi + lo;
  }
}

__device__ __forceinline__ void laneMin(const W& w, int i, SeqRow& r, int posinf, int neginf, int poshuge,
                                        int neghuge, double delta, bool goodrelax, double& val, bool& tight,
                                        bool& settoinf) {
  if (minRecomputes(r, posinf, neginf, poshuge, neghuge, goodrelax)) laneRecompute(w, i, r, true);
  getMinAct(w.A->s, actOf(r), posinf, neginf, poshuge, neghuge, delta, goodrelax, val, tight, settoinf);
}
__device__ __forceinline__ void laneMax(const W& w, int i, SeqRow& r, int posinf, int neginf, int poshuge,
                                        int neghuge, double delta, bool goodrelax, double& val, bool& tight,
                                        bool& settoinf) {
  if (maxRecomputes(r, posinf, neginf, poshuge, neghuge, goodrelax)) laneRecompute(w, i, r, false);
  getMaxAct(w.A->s, actOf(r), posinf, neginf, poshuge, neghuge, delta, goodrelax, val, tight, settoinf);
}
__device__ __forceinline__ void laneBounds(const W& w, int i, SeqRow& r, bool goodrelax, double& minact,
                                           double& maxact, bool& mint, bool& maxt, bool& mininf, bool& maxinf) {
  if (!(r.flags & RS_VALID)) laneCalc(w, i, r);
  laneMin(w, i, r, r.minposinf, r.minneginf, r.minposhuge, r.minneghuge, 0.0, goodrelax, minact, mint, mininf);
  laneMax(w, i, r, r.maxposinf, r.maxneginf, r.maxposhuge, r.maxneghuge, 0.0, goodrelax, maxact, maxt, maxinf);
}

// The largest activity delta of a row as recomputeMaxDelta finds it, gathered in one forward pass: the reverse scan
// keeps the first maximum it meets (the largest position among equal deltas, a delta > 0), and without binaries
// only the first infinite domain it meets (the largest such position) ends it with infinity.
struct MaxDeltaScan {
  double bbest, gbest;  // over the unfixed binaries (|a|), over all entries (|a| * (u - l))
  int bcol, gcol, infcol;
  bool nonbin;
};

// One pass over a row's entries for laneHead: calcActivities (calc) and the candidates of recomputeMaxDelta (md).
// The loads of an entry (its column, coefficient, bounds, base domain and type) are independent of the sums, so
// the pass is unrolled to keep several entries' loads in flight.
__device__ __noinline__ void laneScan(const W& w, int i, SeqRow& r, bool calc, bool md, MaxDeltaScan& m) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int64_t p0 = P.rowptr[i], p1 = P.rowptr[i + 1];
  Act a;
  actZero(a);
  m.bbest = m.gbest = 0.0;
  m.bcol = m.gcol = m.infcol = -1;
  m.nonbin = false;
#pragma unroll 4
  for (int64_t p = p0; p < p1; ++p) {
    const int j = P.colidx[p];
    const double v = P.vals[p];
    const int st = w.ost[j];
    const double2 o = w.ovl[j];
    const double2 base = w.A->base[j];
    const bool isint = P.isint[j] != 0;
    const double2 b = st == w.epoch ? o : base;
    if (calc) addTerm(s, a, v, b.x, b.y);
    if (md) {
      m.nonbin |= !(isint && !dneg(base.x) && !gtc(base.y, 1.0));
      if (!gec(b.x, 0.5) && gtc(b.y, 0.5)) {
        const double d = dabs(v);
        if (!dlt(d, m.bbest) && dpos(d)) {
          m.bbest = d;
          m.bcol = j;
        }
      }
      if (isNegInf(s, b.x) || isInf(s, b.y)) {
        m.infcol = j;
      } else {
        const double d = dabs(v) * (b.y - b.x);
        if (!dlt(d, m.gbest) && dpos(d)) {
          m.gbest = d;
          m.gcol = j;
        }
      }
    }
  }
  if (calc) {
    r.minhi = a.minhi; r.minlo = a.minlo; r.maxhi = a.maxhi; r.maxlo = a.maxlo;
    r.minposinf = a.minposinf; r.minneginf = a.minneginf; r.minposhuge = a.minposhuge; r.minneghuge = a.minneghuge;
    r.maxposinf = a.maxposinf; r.maxneginf = a.maxneginf; r.maxposhuge = a.maxposhuge; r.maxneghuge = a.maxneghuge;
    r.flags |= RS_VALID | RS_VMIN | RS_VMAX;
    r.lastmin = r.minhi + r.minlo;
    r.lastmax = r.maxhi + r.maxlo;
  }
}

// recomputeMaxDelta from the pass's candidates
__device__ __forceinline__ void laneMaxDelta(const Num& s, SeqRow& r, const MaxDeltaScan& m) {
  r.maxdelta = 0.0;
  if (!(r.flags & RS_NBV)) r.flags = (r.flags & ~RS_HNB) | (m.nonbin ? RS_HNB : 0u) | RS_NBV;
  if (!(r.flags & RS_HNB)) {
    if (m.bcol >= 0) {
      r.maxdelta = m.bbest;
      r.maxdeltacol = m.bcol;
    }
  } else if (m.infcol >= 0) {
    r.maxdelta = s.inf;
    r.maxdeltacol = m.infcol;
  } else if (m.gcol >= 0) {
    r.maxdelta = m.gbest;
    r.maxdeltacol = m.gcol;
  }
}

// The head and tail of propagateCons, one lane: tightenBounds up to its visit of the entries, and -- for a row
// that does not reach the visit -- the infeasibility and redundancy tests.  Returns
//   ROW_DONE  the row changes nothing but its own record (r holds it; RS_INUPD set if it joined the update list);
//   ROW_LIVE  the row reaches the visit of its entries (r holds the record the visit starts from);
//   ROW_CUT   the row finds the node infeasible (it is then run for real).
constexpr int ROW_DONE = 0, ROW_LIVE = 1, ROW_CUT = 2;

__device__ __noinline__ int laneHead(const W& w, int i, SeqRow& r) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int len = (int)(P.rowptr[i + 1] - P.rowptr[i]);
  const bool force = (len == 1);
  const unsigned tightenmode = 1;
  // tightenBounds
  bool skip = false;
  // the activities, and the largest delta's candidates in the same pass (used only if the tests reach it)
  const bool calc = !(r.flags & RS_VALID), md = isInvalid(r.maxdelta);
  MaxDeltaScan m;
  if (calc || md) laneScan(w, i, r, calc, md, m);
  if (r.minneginf + r.minposinf + r.minneghuge + r.minposhuge > 1 &&
      r.maxneginf + r.maxposinf + r.maxneghuge + r.maxposhuge > 1)
    skip = true;
  if (!skip && !force && btOf(r.flags) >= tightenmode) skip = true;
  if (!skip && md) laneMaxDelta(s, r, m);
  if (!skip && feasZero(s, r.maxdelta)) skip = true;
  if (!skip && !isInf(s, r.maxdelta)) {
    double minact, maxact;
    bool t1, t2, f1, f2;
    laneBounds(w, i, r, false, minact, maxact, t1, t2, f1, f2);
    const double slack = (isInf(s, P.rhs[i]) || f1) ? s.inf : P.rhs[i] - minact;
    const double surplus = (isNegInf(s, P.lhs[i]) || f2) ? s.inf : maxact - P.lhs[i];
    if (le(s, r.maxdelta, dmin(slack, surplus))) skip = true;
  }
  if (!skip) return ROW_LIVE;
  // propagateCons: the infeasibility and redundancy tests
  double minact, maxact;
  bool t1, t2, f1, f2;
  laneBounds(w, i, r, true, minact, maxact, t1, t2, f1, f2);
  if (feasGt(s, minact, P.rhs[i]) || feasLt(s, maxact, P.lhs[i])) return ROW_CUT;
  // a redundant row is deleted locally (disableRow: joins the update list unless it is there)
  if (ge(s, minact, P.lhs[i]) && le(s, maxact, P.rhs[i]) && !(r.flags & RS_UD) && (r.flags & RS_EN))
    r.flags |= RS_UD | RS_INUPD;
  return ROW_DONE;
}

// ------------------------------------------------------------------------------------------ one row
__device__ __noinline__ bool tightenVisit(W& w, int i, SeqRow r);

// tightenBounds (uniform); returns true on cutoff
__device__ __noinline__ bool tightenBounds(W& w, int i) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int len = (int)(P.rowptr[i + 1] - P.rowptr[i]);
  const bool force = (len == 1);
  const unsigned tightenmode = 1;  // below the root
  SeqRow r = loadRow(w, i);
  ensureAct(w, i, r);
  storeRow(w, i, r);
  if (r.minneginf + r.minposinf + r.minneghuge + r.minposhuge > 1 &&
      r.maxneginf + r.maxposinf + r.maxneghuge + r.maxposhuge > 1)
    return false;
  if (!force && btOf(r.flags) >= tightenmode) return false;
  if (isInvalid(r.maxdelta)) {
    recomputeMaxDelta(w, i, r);
    storeRow(w, i, r);
  }
  if (feasZero(s, r.maxdelta)) return false;
  if (!isInf(s, r.maxdelta)) {
    double minact, maxact;
    bool t1, t2, f1, f2;
    activityBounds(w, i, r, false, minact, maxact, t1, t2, f1, f2);
    storeRow(w, i, r);
    const double slack = (isInf(s, P.rhs[i]) || f1) ? s.inf : P.rhs[i] - minact;
    const double surplus = (isNegInf(s, P.lhs[i]) || f2) ? s.inf : maxact - P.lhs[i];
    if (le(s, r.maxdelta, dmin(slack, surplus))) return false;
  }
  return tightenVisit(w, i, r);
}

// tightenBounds from its visit of the entries on (the row passed the tests before it; r is its record then)
__device__ __noinline__ bool tightenVisit(W& w, int i, SeqRow r) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  const int len = (int)(P.rowptr[i + 1] - P.rowptr[i]);
  const bool force = (len == 1);
  const unsigned tightenmode = 1;
  const bool easy = lt(s, r.maxdelta, s.maxeasy);
  const bool sorted = !s.nosort;
  const int nbin = nbinOf(w, i);
  w.live += 1;
  int lastchange = -1;
  for (int nrounds = 0; (force || btOf(r.flags) < tightenmode) && nrounds < MAXTIGHTENROUNDS; ++nrounds) {
    r.flags = withBt(r.flags, tightenmode);
    storeRow(w, i, r);
    int v = 0;
    while (v < len && v != lastchange) {
      const int end = lastchange > v ? lastchange : len;
      // the first entry in [v, end) that changes something or ends the visit of the binaries
      int hit = -1;
      bool effect = false;
      for (int k0 = v; k0 < end && hit < 0; k0 += 32) {
        const int k = k0 + w.lane;
        bool eff = false, jump = false;
        if (k < end) {
          eff = easy ? easyWould(w, i, r, k, force) : residualWould(w, i, r, k, force);
          if (!eff && sorted && k < nbin - 1) {
            const double2 b = bnd(w, P.colidx[P.rowptr[i] + k]);
            jump = !feasEq(s, b.y, b.x);
          }
        }
        const unsigned m = __ballot_sync(FULL, eff || jump);
        if (m) {
          const int t = __ffs(m) - 1;
          hit = k0 + t;
          effect = __shfl_sync(FULL, eff, t);
        }
      }
      if (hit < 0) {
        w.cands += end - v;
        v = end;
        continue;
      }
      w.cands += hit - v + 1;
      if (!effect) {  // an unfixed binary that does not tighten ends the visit of the binaries
        v = nbin;
        continue;
      }
      const long long old = w.nchg;
      if (easy ? easyRun(w, i, r, hit, force) : residualRun(w, i, r, hit, force)) return true;
      r = loadRow(w, i);
      if (w.nchg > old) {
        lastchange = hit;
        v = hit + 1;
      } else if (sorted && hit < nbin - 1) {
        const double2 b = bnd(w, P.colidx[P.rowptr[i] + hit]);
        v = !feasEq(s, b.y, b.x) ? nbin : hit + 1;
      } else {
        v = hit + 1;
      }
    }
  }
  return false;
}

__device__ __noinline__ bool propagateTail(W& w, int i);

// propagateCons without ranged rows (uniform); returns true on cutoff
__device__ __noinline__ bool propagateCons(W& w, int i) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  w.rows += 1;
  w.nnz += P.rowptr[i + 1] - P.rowptr[i];
  if (tightenBounds(w, i)) return true;
  return propagateTail(w, i);
}

// propagateCons after tightenBounds: the infeasibility and redundancy tests (uniform); returns true on cutoff
__device__ __noinline__ bool propagateTail(W& w, int i) {
  const Prob& P = w.A->P;
  const Num& s = w.A->s;
  SeqRow r = loadRow(w, i);
  double minact, maxact;
  bool t1, t2, f1, f2;
  activityBounds(w, i, r, true, minact, maxact, t1, t2, f1, f2);
  if (feasGt(s, minact, P.rhs[i]) || feasLt(s, maxact, P.lhs[i])) {
    storeRow(w, i, r);
    return true;
  }
  // a redundant row is deleted locally (SCIPdelConsLocal below the root)
  if (ge(s, minact, P.lhs[i]) && le(s, maxact, P.rhs[i])) disableRow(w, i, r);
  storeRow(w, i, r);
  return false;
}

// propagateRounds: consPropLinear over the marked rows until a call changes nothing (uniform);
// 0 fixpoint, 1 cutoff, 2 round limit.  The rows of a call are taken 32 at a time, one per lane, through laneHead;
// walking them in order, the rows it ends are committed as they stand, a row that reaches the visit of its entries
// is visited by the warp, and a row that finds the node infeasible is run for real.  A bound change reaches only the
// rows of its column (their records count the events): after one, the rows still ahead whose records changed are
// taken afresh, and the others' outcomes stand.
__device__ int propagateRounds(W& w, int maxrounds, int& rounds) {
  const Prob& P = w.A->P;
  rounds = 0;
  for (int round = 0; round < maxrounds; ++round) {
    const int nmarked = w.nm;
    if (nmarked == 0) return 0;
    w.nchg = 0;
    w.indelay = true;
    bool cut = false;
    for (int k = 0; k < nmarked && !cut;) {
      const int cnt = min(32, nmarked - k);
      const bool has = w.lane < cnt;
      int i = -1, cls = ROW_DONE;
      bool wasin = false;
      SeqRow r;
      if (has) {
        i = w.M[k + w.lane];
        r = loadRow(w, i);
        wasin = (r.flags & RS_INUPD) != 0;
        // unmarkProp
        if (!((r.flags & RS_UU) || (!(r.flags & RS_MP) && !(r.flags & RS_UM))))
          r.flags = (r.flags & ~RS_UM) | RS_UU | RS_INUPD;
        cls = laneHead(w, i, r);
      }
      const unsigned below = (1u << w.lane) - 1u;
      int pos = 0;
      while (pos < cnt && !cut) {
        const unsigned stop = __ballot_sync(FULL, has && cls != ROW_DONE);
        const unsigned rest = stop & ~((1u << pos) - 1u);
        const int q = rest ? __ffs(rest) - 1 : cnt;
        // rows [pos, q) are committed as they stand, and row q's unmark and head too when it is live
        const int qcls = __shfl_sync(FULL, cls, q & 31);
        const int upto = (q < cnt && qcls == ROW_LIVE) ? q + 1 : q;
        const bool commit = w.lane >= pos && w.lane < upto;
        const bool app = commit && !wasin && (r.flags & RS_INUPD);
        const unsigned am = __ballot_sync(FULL, app);
        if (app) w.U[w.nu + __popc(am & below)] = i;
        if (commit) w.rs[i] = r;
        w.nu += __popc(am);
        const unsigned cm = __ballot_sync(FULL, commit);
        w.rows += __popc(cm);
        w.nnz += __reduce_add_sync(FULL, commit ? (unsigned)(P.rowptr[i + 1] - P.rowptr[i]) : 0u);
        __syncwarp();
        if (q >= cnt) {
          pos = cnt;
          break;
        }
        const int iq = __shfl_sync(FULL, i, q);
        const long long old = w.nchg;
        if (qcls == ROW_LIVE) {
          cut = tightenVisit(w, iq, w.rs[iq]) || propagateTail(w, iq);
        } else {
          SeqRow rr = loadRow(w, iq);
          unmarkProp(w, iq, rr);
          storeRow(w, iq, rr);
          cut = propagateCons(w, iq);
        }
        pos = q + 1;
        if (!cut && w.nchg > old && has && w.lane > q && w.rs[i].evc != r.evc) {
          r = loadRow(w, i);
          wasin = (r.flags & RS_INUPD) != 0;
          if (!((r.flags & RS_UU) || (!(r.flags & RS_MP) && !(r.flags & RS_UM))))
            r.flags = (r.flags & ~RS_UM) | RS_UU | RS_INUPD;
          cls = laneHead(w, i, r);
        }
        __syncwarp();
      }
      k += pos;
    }
    w.indelay = false;
    processUpdates(w);
    rounds = round + 1;
    if (cut) return 1;
    if (w.nchg == 0) return 0;
  }
  return w.nm > 0 ? 2 : 0;
}

}  // namespace

// one warp per node; WPB warps per CTA, each with its own slot
template <int WPB>
__global__ void __launch_bounds__(WPB * 32) k_nodes_seq(const __grid_constant__ SeqArgs A) {
  const int lane = threadIdx.x & 31;
  const int slot = blockIdx.x * WPB + (threadIdx.x >> 5);
  const SeqSlots& S = A.S;
  if (slot >= S.nslots) return;
  W w;
  w.A = &A;
  w.rs = S.rows + (size_t)slot * S.mstride;
  w.ovl = S.ovl + (size_t)slot * S.nstride;
  w.ost = S.ost + (size_t)slot * S.nstride;
  w.M = S.M + (size_t)slot * S.mstride;
  w.U = S.U + (size_t)slot * S.mstride;
  w.dirty = S.dirty + (size_t)slot * S.nstride;
  w.lane = lane;
  w.rows = w.nnz = w.cands = w.live = w.changes = 0;
  int epoch = S.counter[slot];
  unsigned long long mycut = 0, mymaxr = 0;
  const Num& s = A.s;

  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(A.next_item, 1);
    q = __shfl_sync(FULL, q, 0);
    if (q >= A.nnodes) break;
    const int item = A.order != nullptr ? A.order[q] : q;
    w.epoch = ++epoch;
    w.nm = w.nu = w.ndirty = 0;
    w.indelay = false;
    w.nchg = 0;
    bool cut = false;
    int rounds = 0;
    // the node's changes, as SCIPchgVarLbProbing / SCIPchgVarUbProbing make them, each followed by its events
    for (int64_t c = A.ptr[item]; c < A.ptr[item + 1] && !cut; ++c) {
      const int j = A.chg_col[c];
      if (j < 0 || j >= (int)A.P.n) {  // not a column: the call fails, the node is given up
        if (lane == 0) atomicOr(A.status, 4);
        cut = true;
        break;
      }
      const bool isint = A.P.isint[j] != 0;
      const double nl = A.chg_lb[c], nu = A.chg_ub[c];
      double2 b = bnd(w, j);
      if (nl > b.y || nu < b.x) {
        cut = true;
        break;
      }
      if (nl > b.x) {
        double v = adjLb(s, isint, nl);
        if (!isInf(s, v)) {
          v = dmin(v, b.y);
          if (gt(s, v, b.x)) {
            setBound(w, j, v, b.y);
            boundEvent(w, j, true, b.x, v);
          }
        }
      }
      b = bnd(w, j);
      if (nu < b.y) {
        double v = adjUb(s, isint, nu);
        if (!isNegInf(s, v)) {
          v = dmax(v, b.x);
          if (lt(s, v, b.y)) {
            setBound(w, j, b.x, v);
            boundEvent(w, j, false, b.y, v);
          }
        }
      }
    }
    if (!cut) {
      const int st = propagateRounds(w, A.maxrounds, rounds);
      cut = st == 1;
      if (st == 2 && lane == 0) atomicOr(A.status, 1);
    }
    // results: columns whose final bounds differ from the base, packed at a reserved offset
    int cnt = 0;
    if (!cut) {
      for (int t = lane; t < w.ndirty; t += 32) {
        const int j = w.dirty[t];
        const double2 o = w.ovl[j], bb = A.base[j];
        cnt += (o.x != bb.x || o.y != bb.y) ? 1 : 0;
      }
      cnt = __reduce_add_sync(FULL, (unsigned)cnt);
    }
    long long off = 0;
    if (lane == 0 && cnt > 0) off = (long long)atomicAdd(A.out_used, (unsigned long long)cnt);
    off = __shfl_sync(FULL, off, 0);
    const bool fits = off + cnt <= A.out_cap;
    if (lane == 0) {
      if (!fits) atomicOr(A.status, 2);
      A.out_off[item] = fits ? off : 0;
      A.out_n[item] = fits ? cnt : -1;
      A.out_cutoff[item] = cut ? 1 : 0;
      A.out_rounds[item] = rounds;
    }
    if (!cut && fits && cnt > 0) {
      int pos = 0;
      for (int t0 = 0; t0 < w.ndirty; t0 += 32) {
        const int t = t0 + lane;
        bool d = false;
        int j = 0;
        double2 o = make_double2(0.0, 0.0);
        if (t < w.ndirty) {
          j = w.dirty[t];
          o = w.ovl[j];
          const double2 bb = A.base[j];
          d = o.x != bb.x || o.y != bb.y;
        }
        const unsigned m = __ballot_sync(FULL, d);
        if (d) {
          const long long at = off + pos + __popc(m & ((1u << lane) - 1u));
          A.out_col[at] = j;
          A.out_lb[at] = o.x;
          A.out_ub[at] = o.y;
        }
        pos += __popc(m);
      }
    }
    mycut += cut ? 1 : 0;
    if ((unsigned long long)rounds > mymaxr) mymaxr = rounds;
    __syncwarp();
  }
  if (lane == 0) {
    S.counter[slot] = epoch;
    if (mycut) atomicAdd(&A.stats[4], mycut);
    atomicMax(&A.stats[5], mymaxr);
    if (w.rows) atomicAdd(&A.stats[0], (unsigned long long)w.rows);
    if (w.nnz) atomicAdd(&A.stats[1], (unsigned long long)w.nnz);
    if (w.cands) atomicAdd(&A.stats[2], (unsigned long long)w.cands);
    if (w.changes) atomicAdd(&A.stats[3], (unsigned long long)w.changes);
    if (w.live) atomicAdd(&A.stats[6], (unsigned long long)w.live);
  }
}

// per row: the number of leading binaries of its order under the base domain, and whether it is redundant there
// (then it was deleted at the root: prep < 0).  One thread per row, the activity summed in the row's order.
__global__ void k_seq_prepare(Num s, Prob P, const double2* base, int* prep) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = P.rowptr[i], p1 = P.rowptr[i + 1];
    int nbin = 0;
    bool lead = true;
    Act a;
    actZero(a);
    for (int64_t p = p0; p < p1; ++p) {
      const int j = P.colidx[p];
      const double2 b = base[j];
      if (lead && P.isint[j] != 0 && !dneg(b.x) && !gtc(b.y, 1.0)) ++nbin;
      else lead = false;
      addTerm(s, a, P.vals[p], b.x, b.y);
    }
    double minact, maxact;
    bool t1, t2, f1, f2;
    getMinAct(s, a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, 0.0, true, minact, t1, f1);
    getMaxAct(s, a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, true, maxact, t2, f2);
    const bool del = ge(s, minact, P.lhs[i]) && le(s, maxact, P.rhs[i]);
    prep[i] = del ? (int)(0x80000000u | (unsigned)nbin) : nbin;
  }
}

// column-major copy with each column's rows in ascending order (the order the rows caught the column's bound-change
// events, which SCIP processes in that order): CSR positions sorted by column with a stable radix sort keep their
// row order within a column; each sorted position then gives its row (binary search of rowptr) and coefficient
__global__ void k_iota(int64_t nnz, int32_t* out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    out[p] = (int32_t)p;
}
__global__ void k_seq_csc_fill(int64_t nnz, int64_t m, const int32_t* perm, const int64_t* rowptr, const double* vals,
                               int32_t* crow, double* cval) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[q];
    int64_t lo = 0, hi = m - 1;  // the row holding position p: the last i with rowptr[i] <= p
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (rowptr[mid] <= p) lo = mid;
      else hi = mid - 1;
    }
    crow[q] = (int32_t)lo;
    cval[q] = vals[p];
  }
}

cudaError_t launchSeqCsc(cudaStream_t st, int grid, int64_t m, int64_t n, int64_t nnz, const int64_t* rowptr,
                         const int32_t* colidx, const double* vals, int32_t* crow, double* cval) {
  if (nnz == 0) return cudaSuccess;
  int bits = 1;
  while (bits < 31 && (int64_t(1) << bits) < n) ++bits;
  int32_t *keys = nullptr, *iota = nullptr, *perm = nullptr;
  void* tmp = nullptr;
  size_t tmpb = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, tmpb, colidx, keys, iota, perm, (int)nnz, 0, bits, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&keys, nnz * sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&iota, nnz * sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&perm, nnz * sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&tmp, tmpb, st);
  if (e == cudaSuccess) {
    k_iota<<<grid, 256, 0, st>>>(nnz, iota);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cub::DeviceRadixSort::SortPairs(tmp, tmpb, colidx, keys, iota, perm, (int)nnz, 0, bits, st);
  if (e == cudaSuccess) {
    k_seq_csc_fill<<<grid, 256, 0, st>>>(nnz, m, perm, rowptr, vals, crow, cval);
    e = cudaGetLastError();
  }
  if (keys) cudaFreeAsync(keys, st);
  if (iota) cudaFreeAsync(iota, st);
  if (perm) cudaFreeAsync(perm, st);
  if (tmp) cudaFreeAsync(tmp, st);
  return e;
}

cudaError_t launchSeqPrepare(cudaStream_t st, int grid, const Num& s, const Prob& P, const double2* base, int* prep) {
  k_seq_prepare<<<grid, 128, 0, st>>>(s, P, base, prep);
  return cudaGetLastError();
}

cudaError_t launchNodesSeq(cudaStream_t st, int grid, const SeqArgs& A) {
  k_nodes_seq<SEQ_WARPS><<<grid, SEQ_WARPS * 32, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t nodesSeqOccupancy(int* blocksPerSm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, k_nodes_seq<SEQ_WARPS>, SEQ_WARPS * 32, 0);
}

}  // namespace gbp
