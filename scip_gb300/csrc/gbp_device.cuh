// Device procedures shared by the plain (one problem per launch sequence) and the batched (persistent,
// one CTA per node) propagation paths.
//
// One propagation round, for the rows of the current frontier and the bounds B_r at its start:
//   rowThread / rowWarp   activity + cutoff test + candidate bounds of every frontier row
//                         (propagateCons -> tightenBounds -> tightenVarBounds[Easy], cons_linear.c)
//   applyColumn           per touched column, SCIP's acceptance of the best candidates against B_r
//                         (SCIPinferVarUbCons / SCIPinferVarLbCons, scip_var.c:7071 / 6965)
//   expandColumn          rows that the accepted change makes worth re-tightening
//                         (eventExecLinear, cons_linear.c:17226-17255)
// Candidate bounds meet in per-column slots through atomicMin / atomicMax on order-preserving int64 keys,
// so the result does not depend on the order in which rows run.
#pragma once

#include "gbp_rules.cuh"

namespace gbp {

constexpr int LONGROW = 64;  // rows longer than this are summed as 32 interleaved partials (warp per row)
constexpr long long KEY_NONE_UB = 0x7fffffffffffffffLL;       // empty upper-bound candidate slot
constexpr long long KEY_NONE_LB = (long long)0x8000000000000000ULL;  // empty lower-bound candidate slot
constexpr uint32_t CSC_LBUP = 1u << 30;    // row uses a raised lower bound of this column
constexpr uint32_t CSC_UBDOWN = 1u << 31;  // row uses a lowered upper bound of this column
constexpr uint32_t CSC_ROW = (1u << 30) - 1u;

struct Prob {
  int64_t m, n;
  const int64_t* rowptr;
  const int32_t* colidx;
  const double* vals;
  const double* lhs;
  const double* rhs;
  const int8_t* isint;
  const int64_t* colptr;
  const uint32_t* cscrow;  // row index | CSC_LBUP | CSC_UBDOWN; null: use rowidx/cvals below
  const int32_t* rowidx;   // plain CSC (only read when cscrow is null)
  const double* cvals;
  double inf;              // infinity threshold for the relevance test on plain CSC
  // several independent instances in one block-diagonal problem (all null for a single problem)
  const int32_t* rowinst;  // instance of each row
  const int32_t* colinst;  // instance of each column
  int* instcut;            // per-instance cutoff flags
  // global domain for the binary test of the plain path (null: the bounds being propagated, as at the root)
  const double* glb;
  const double* gub;
  // ranged rows (relig null: the rule is off).  relig[i] = 1 for a row the gcd rule can act on; rperm holds
  // each such row's entry order (rperm[p0 + k] = offset of its k-th entry), rtmp is merge scratch beside it.
  // rlive: the order is computed where the row is evaluated, from the global domain of the bounds accessor
  // (the bounds being propagated at the root); otherwise it was computed before the call.  rsorted: the
  // order of constraints/linear/sortvars, else the index order.
  const uint8_t* relig;
  int32_t* rperm;
  int32_t* rtmp;
  const long long* rcoef;  // per entry of such a row: >= 0 (long long)(|a| + feastol) of an integral column with an
                           // integral coefficient other than +-1; -1 another entry with |a| = 1; -2 any other entry
  int rlive;
  int rsorted;
};

// rows of an instance that is already infeasible are skipped
__device__ __forceinline__ bool rowDead(const Prob& P, int i) {
  return P.instcut != nullptr && P.instcut[P.rowinst[i]] != 0;
}
// infeasibility found by row i: the row's instance (instances) or the whole problem (*cut)
__device__ __forceinline__ void cutRow(const Prob& P, int i, int* cut) {
  if (P.instcut != nullptr) atomicExch(&P.instcut[P.rowinst[i]], 1);
  else *cut = 1;
}

// Ranged-row records of the plain path (row null: off): each row whose ranged rule proposed bounds for a column
// (col) or found itself infeasible (col -1), with the round -- the rows conflict analysis needs as reasons
struct RangedLog {
  int* n;          // records written (may exceed cap)
  int64_t cap;
  int32_t* row;
  int32_t* col;
  int32_t* round;
};

struct Cands {
  long long* cub;   // best non-forced upper bound candidate (key), KEY_NONE_UB when empty
  long long* clb;   // best non-forced lower bound candidate (key), KEY_NONE_LB when empty
  long long* cubf;  // forced candidates (single-entry rows, ranged rows)
  long long* clbf;
  int* cflag;       // bit0 ub, bit1 ubf, bit2 lb, bit3 lbf; 0 when the column is untouched this round
  int* touched;     // list of touched columns
  int* ntouched;    // its length (global or shared counter)
  RangedLog rlog;   // ranged-row records (plain path with a change log), else row == nullptr
  int round;        // the round the candidates are for (ranged-row records)
};
__device__ __forceinline__ void logRanged(const Cands& C, int row, int col) {
  if (C.rlog.row == nullptr) return;
  const int k = atomicAdd(C.rlog.n, 1);
  if (k < C.rlog.cap) {
    C.rlog.row[k] = row;
    C.rlog.col[k] = col;
    C.rlog.round[k] = C.round;
  }
}

struct Stats {
  long long rows, nnz, cands, live;  // live: rows that passed the skip tests
};

// Change log of the plain path: every accepted bound change with the round that made it (col null: off).
// SCIP's conflict analysis needs tightenings in an order where each one's reasons already hold; applying the
// log round by round gives that order.
struct ChangeLog {
  int* n;          // entries written (may exceed cap: the log overflowed)
  int64_t cap;
  int32_t* col;
  int32_t* round;
  double* lb;      // the column's bounds after the change
  double* ub;
};
__device__ __forceinline__ void logChange(const ChangeLog& G, int j, int round, double l, double u) {
  if (G.col == nullptr) return;
  const int k = atomicAdd(G.n, 1);
  if (k < G.cap) {
    G.col[k] = j;
    G.round[k] = round;
    G.lb[k] = l;
    G.ub[k] = u;
  }
}

// state of the graph-driven fixpoint loop (device memory): which list holds the frontier (0, 1, or 2 = the
// all-rows list), the lists' sizes, stamps, flags and the bound vectors being propagated
struct LoopState {
  int cur;
  int nshort[3];
  int nlong[3];
  int ntouched;
  int cutoff;
  int round;
  int worked;     // rounds that processed a non-empty frontier
  int maxrounds;
  int stamp;      // row stamp of the list being filled
  int status;     // 2: round limit reached
  int more;       // the cooperative loop: another round follows
  double* lb;
  double* ub;
  ChangeLog log;
};
// the first move of each column in a sparse call (stamp[j] == epoch once recorded) and its bounds before it
struct MovedLog {
  int* stamp = nullptr;
  int epoch = 0;
  int* count = nullptr;
  int32_t* col = nullptr;
  double* lb = nullptr;
  double* ub = nullptr;
};
struct ListSet {
  int* list[3];
  int* rowstamp;
  int cap;        // m: long rows are stored from the back of each list
};

// frontier lists: short rows from the front of `list`, long rows from the back
struct Front {
  int* list;
  int* nshort;
  int* nlong;
  int* rowstamp;
  int cap;  // = m
};

__device__ __forceinline__ long long absBitsOf(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffLL; }

__device__ __forceinline__ void emitUb(Cands& C, int j, double v, bool force) {
  atomicMin(force ? &C.cubf[j] : &C.cub[j], dkey(v));
  int old = atomicOr(&C.cflag[j], force ? 2 : 1);
  if (old == 0) C.touched[atomicAdd(C.ntouched, 1)] = j;
}
__device__ __forceinline__ void emitLb(Cands& C, int j, double v, bool force) {
  atomicMax(force ? &C.clbf[j] : &C.clb[j], dkey(v));
  int old = atomicOr(&C.cflag[j], force ? 8 : 4);
  if (old == 0) C.touched[atomicAdd(C.ntouched, 1)] = j;
}

// candidate sinks for columnCandidates: into the column slots (counted), or only noted
struct EmitTo {
  Cands* C;
  int j;
  long long* n;
  __device__ __forceinline__ void operator()(bool isub, double v, bool force) const {
    if (isub) emitUb(*C, j, v, force);
    else emitLb(*C, j, v, force);
    ++*n;
  }
};
struct Probe {
  bool* hit;
  __device__ __forceinline__ void operator()(bool, double, bool) const { *hit = true; }
};

// SCIPvarIsBinary (var.c:23801-23810): integral with a global domain inside [0,1]; the accessor supplies
// the global domain (base bounds of a node batch, explicit global bounds, or the bounds being propagated)
template <class BND>
__device__ __forceinline__ bool isBinaryCol(const Prob& P, const BND& B, int j) {
  if (P.isint[j] == 0) return false;
  double gl, gu;
  B.glob(P, j, gl, gu);
  return gl >= 0.0 && gu <= 1.0;
}

// Order of a row's binaries during solving (consdataCompVarProp, cons_linear.c:3229-3254): larger |a| first,
// ties by column index.  |a| is compared exactly (SCIP's 1e-9 tie tolerance is not transitive); the two
// orders agree whenever a row's distinct binary coefficients differ by more than 1e-9.
__device__ __forceinline__ bool binBefore(const Prob& P, int64_t p, int64_t q) {
  const long long a1 = absBitsOf(P.vals[p]), a2 = absBitsOf(P.vals[q]);
  if (a1 != a2) return a1 > a2;
  return P.colidx[p] < P.colidx[q];
}

__device__ __forceinline__ void pushRow(const Prob& P, Front& F, int row, int stamp) {
  if (atomicExch(&F.rowstamp[row], stamp) != stamp) {
    int64_t len = P.rowptr[row + 1] - P.rowptr[row];
    if (len <= LONGROW) F.list[atomicAdd(F.nshort, 1)] = row;
    else F.list[F.cap - 1 - atomicAdd(F.nlong, 1)] = row;
  }
}

// rows of column j made relevant by a raised lower bound (lbup) and/or a lowered upper bound (ubdown).  The stamp
// exchanges, length reads and list appends of up to 8 rows are issued together: each is a dependent round trip to
// memory, and one thread expands a column
__device__ __forceinline__ void expandColumn(const Prob& P, Front& F, int j, bool lbup, bool ubdown, int stamp) {
  if (P.cscrow != nullptr) {
    const uint32_t need = (lbup ? CSC_LBUP : 0u) | (ubdown ? CSC_UBDOWN : 0u);
    const int64_t q0 = P.colptr[j], q1 = P.colptr[j + 1];
    for (int64_t qb = q0; qb < q1; qb += 8) {
      int rows[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        rows[t] = -1;
        if (qb + t < q1) {
          const uint32_t e = P.cscrow[qb + t];
          if (e & need) rows[t] = (int)(e & CSC_ROW);
        }
      }
      bool fresh[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) fresh[t] = rows[t] >= 0 && atomicExch(&F.rowstamp[rows[t]], stamp) != stamp;
      bool shortrow[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) shortrow[t] = fresh[t] && P.rowptr[rows[t] + 1] - P.rowptr[rows[t]] <= LONGROW;
      int slot[8];
#pragma unroll
      for (int t = 0; t < 8; ++t)
        slot[t] = !fresh[t] ? -1 : (shortrow[t] ? atomicAdd(F.nshort, 1) : F.cap - 1 - atomicAdd(F.nlong, 1));
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (slot[t] >= 0) F.list[slot[t]] = rows[t];
    }
  } else {
    for (int64_t q = P.colptr[j]; q < P.colptr[j + 1]; ++q) {
      const int i = P.rowidx[q];
      const double a = P.cvals[q];
      const bool rhsfin = !(P.rhs[i] >= P.inf), lhsfin = !(-P.lhs[i] >= P.inf);
      const bool rel = (lbup && (a > 0.0 ? rhsfin : lhsfin)) || (ubdown && (a > 0.0 ? lhsfin : rhsfin));
      if (rel) pushRow(P, F, i, stamp);
    }
  }
}

// Candidate bounds of one entry (value val, column bounds [l,u]) in a row with activity a:
// tightenVarBoundsEasy (cons_linear.c:5380-5653) when `easy`, else tightenVarBounds (:6700-6974).
// Each candidate goes to emit(isub, value, force).  `relres` recomputes a residual in plain double
// (consdataGetReliableResidualActivity, :2580-2657).  Returns true if the row proves infeasibility (easy
// rule only).
template <class EMIT, class RELRES>
__device__ __forceinline__ bool columnCandidates(const Num& s, const Act& a, double lhs, double rhs, bool easy,
                                                 bool force, double val, double l, double u, bool isint,
                                                 const EMIT& emit, const RELRES& relres) {
  if (easy) {
    double minact = a.minhi + a.minlo;
    double maxact = a.maxhi + a.maxlo;
    if (!isInf(s, rhs)) {
      if (feasLt(s, rhs, minact)) return true;
      double slack = rhs - minact;
      if (!positive(s, slack)) slack = 0.0;
      double alpha = val > 0.0 ? val * (u - l) : val * (l - u);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        if (val > 0.0) {
          double nb = adjUb(s, isint, l + slack / val);  // tightenVarUb, cons_linear.c:5242
          if (force || ubBetter(s, nb, l, u)) emit(true, nb, force);
        } else {
          double nb = adjLb(s, isint, u + slack / val);  // tightenVarLb, cons_linear.c:5307
          if (force || lbBetter(s, nb, l, u)) emit(false, nb, force);
        }
      }
    }
    if (!isNegInf(s, lhs)) {
      if (feasLt(s, maxact, lhs)) return true;
      double slack = maxact - lhs;
      if (!positive(s, slack)) slack = 0.0;
      double alpha = val > 0.0 ? val * (u - l) : val * (l - u);
      if (sumGt(s, alpha, slack) || (force && gt(s, alpha, slack))) {
        if (val > 0.0) {
          double nb = adjLb(s, isint, u - slack / val);
          if (force || lbBetter(s, nb, l, u)) emit(false, nb, force);
        } else {
          double nb = adjUb(s, isint, l - slack / val);
          if (force || ubBetter(s, nb, l, u)) emit(true, nb, force);
        }
      }
    }
    return false;
  }

  double minres, maxres;
  bool mintight, maxtight, mininf, maxinf;
  residuals(s, a, val, l, u, minres, maxres, mintight, maxtight, mininf, maxinf);
  bool rhsok = !mininf && !isInf(s, rhs) && mintight && (lt(s, fabs(rhs), 1.0) || !quotNear1(minres, rhs, s.eps));
  bool lhsok = !maxinf && !isNegInf(s, lhs) && maxtight && (lt(s, fabs(lhs), 1.0) || !quotNear1(maxres, lhs, s.eps));
  // Every acceptance test of a new upper bound (forced LT, integral FeasLT, UbBetter) needs newub < u, and of a
  // new lower bound newlb > l.  A side whose exact quotient misses that by more than the rounding of the
  // product bound*val is skipped before its division (the quotient would round to the same side of the
  // bound); the reliable recomputation is only reached when these tests pass, so nothing else changes.
  auto beyond = [](double num, double bv) {  // num > bound*val, decided with margin: +1, -1, or 0 if unsure
    const double m = fabs(bv) * 0x1p-40 + 1e-290;
    return num > bv + m ? 1 : (num < bv - m ? -1 : 0);
  };
  if (rhsok) {
    const int c = beyond(rhs - minres, (val > 0.0 ? u : l) * val);
    if (c > 0) rhsok = false;  // a > 0: newub >= u; a < 0: newlb <= l
  }
  if (lhsok) {
    const int c = beyond(lhs - maxres, (val > 0.0 ? l : u) * val);
    if (c < 0) lhsok = false;  // a > 0: newlb <= l; a < 0: newub >= u
  }
  if (val > 0.0) {
    if (rhsok) {
      double newub = (rhs - minres) / val;
      if (!isInf(s, newub) && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u))) {
        bool unrel = updateUnreliable(s, minres, a.minhi + a.minlo);
        if (unrel) {
          minres = relres(true);
          newub = (rhs - minres) / val;
          unrel = isNegInf(s, minres) ||
                  (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) || !isint) && (!force || !lt(s, newub, u)));
        }
        if (!unrel) emit(true, newub, force);
      }
    }
    if (lhsok) {
      double newlb = (lhs - maxres) / val;
      if (!isNegInf(s, newlb) && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u))) {
        bool skip = false;
        if (updateUnreliable(s, maxres, a.maxhi + a.maxlo)) {
          maxres = relres(false);
          newlb = (lhs - maxres) / val;
          skip = isInf(s, maxres) ||
                 (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint) && (!force || !gt(s, newlb, l)));
        }
        if (!skip) emit(false, newlb, force);
      }
    }
  } else {
    if (rhsok) {
      double newlb = (rhs - minres) / val;
      if (!isNegInf(s, newlb) && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u))) {
        bool unrel = updateUnreliable(s, minres, a.minhi + a.minlo);
        if (unrel) {
          minres = relres(true);
          newlb = (rhs - minres) / val;
          unrel = isNegInf(s, minres) ||
                  (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint) && (!force || !gt(s, newlb, l)));
        }
        if (!unrel) emit(false, newlb, force);
      }
    }
    if (lhsok) {
      double newub = (lhs - maxres) / val;
      if (!isInf(s, newub) && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u))) {
        bool skip = false;
        if (updateUnreliable(s, maxres, a.maxhi + a.maxlo)) {
          maxres = relres(false);
          newub = (lhs - maxres) / val;
          // this branch of SCIP joins its conditions with && (cons_linear.c:6936-6938)
          skip = isInf(s, maxres) ||
                 (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) && !isint) && (!force || !lt(s, newub, u)));
        }
        if (!skip) emit(true, newub, force);
      }
    }
  }
  return false;
}

// Row-level tests before candidates: infeasibility with relaxed huge contributions (propagateCons,
// cons_linear.c:7718-7740), canTightenBounds (:5214-5238), all-fixed and maximal-activity-delta skips
// (tightenBounds, :7050-7083).  Returns 1 = cutoff, 0 = skip row, 2 = generate candidates.
__device__ __forceinline__ int rowTests(const Num& s, const Act& a, double lhs, double rhs, double maxactdelta,
                                        bool& easy) {
  double minact, maxact;
  bool t1, t2, f1, f2;
  getMinAct(s, a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, 0.0, true, minact, t1, f1);
  getMaxAct(s, a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, true, maxact, t2, f2);
  if (feasGt(s, minact, rhs) || feasLt(s, maxact, lhs)) return 1;
  if (a.minneginf + a.minposinf + a.minneghuge + a.minposhuge > 1 &&
      a.maxneginf + a.maxposinf + a.maxneghuge + a.maxposhuge > 1)
    return 0;
  if (feasZero(s, maxactdelta)) return 0;
  if (!isInf(s, maxactdelta)) {
    // without huge contributions the relaxed (goodrelax) activities above are already the plain ones
    if (a.minposhuge + a.minneghuge + a.maxposhuge + a.maxneghuge != 0) {
      getMinAct(s, a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, 0.0, false, minact, t1, f1);
      getMaxAct(s, a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, false, maxact, t2, f2);
    }
    double slack = (isInf(s, rhs) || f1) ? s.inf : rhs - minact;
    double surplus = (isNegInf(s, lhs) || f2) ? s.inf : maxact - lhs;
    if (le(s, maxactdelta, dmin(slack, surplus))) return 0;
  }
  easy = lt(s, maxactdelta, s.maxeasy);
  return 2;
}

// maximal activity contribution of one entry (consdataRecomputeMaxActivityDelta, cons_linear.c:1542-1599);
// returns -1 for an infinite bound
__device__ __forceinline__ double entryDelta(const Num& s, double val, double l, double u) {
  if (isNegInf(s, l) || isInf(s, u)) return -1.0;
  return fabs(val) * (u - l);
}

// ------------------------------------------------------------------------------------------------------
// Short rows (<= LONGROW entries) are processed by a CTA in batches of NT rows:
//   1. the batch is sorted by row length (so a warp's lanes run loops of similar length),
//   2. two lanes per row (one when the batch has more than NT/2 rows) sum the activity as two halves in row
//      order (the oracle's order) and run the row tests,
//   3. each live row selects the few entries that can possibly yield a candidate bound (see selectEntries),
//   4. the CTA evaluates the selected (row, entry) pairs with all lanes busy -- SCIP's full rule, so the
//      result is exactly the oracle's.
// FP64 instructions on GB300 cost the same with 1 or 32 active lanes, so keeping lanes converged is what
// sets the speed of this phase.
constexpr int CHUNK = 4;
constexpr int TOPK = 4;          // largest entry deltas remembered per row
constexpr int MAXSEL = TOPK + 2;  // + the single infinite/huge contributor of each activity

template <int NT>
struct RowBatch {
  Act act[NT];
  double lhs[NT];
  double rhs[NT];
  long long p0[NT];
  int len[NT];
  int nsel[NT];          // entries to evaluate (len when the whole row is selected)
  int full[NT];
  unsigned char sel[NT][MAXSEL];
  unsigned char easy[NT];
  int prefix[NT + 1];
  int order[NT];         // batch position -> row, sorted by length
  int hist[LONGROW + 2];
  int bpos[NT];          // first binary in propagation order that gets no candidate (entry position, -1: none)
  // second-half scan state handed from the odd to the even lane of a pair (its activity goes to act[NT/2 + pair])
  long long htopd[NT / 2][TOPK];
  int htopp[NT / 2][TOPK];
  int hspec[NT / 2][2];
  long long hmaxabs[NT / 2];
  long long hmad[NT / 2];
};

// Load entries [pb, min(pb+CHUNK, p1)) of a row: column indices and values first, then all bound gathers,
// so a chunk costs two memory round trips instead of two per entry.
template <class BND>
__device__ __forceinline__ void loadChunk(const Prob& P, const BND& B, int64_t pb, int64_t p1, int (&jj)[CHUNK],
                                          double (&vv)[CHUNK], double (&ll)[CHUNK], double (&uu)[CHUNK]) {
#pragma unroll
  for (int k = 0; k < CHUNK; ++k) {
    const bool ok = pb + k < p1;
    jj[k] = ok ? P.colidx[pb + k] : 0;
    vv[k] = ok ? P.vals[pb + k] : 0.0;
  }
#pragma unroll
  for (int k = 0; k < CHUNK; ++k)
    if (pb + k < p1) B.get(jj[k], ll[k], uu[k]);
}

// bit pattern of a non-negative double (order-preserving as a signed integer); +inf for an entry with an
// infinite bound
__device__ __forceinline__ long long deltaBits(const Num& s, double val, double l, double u) {
  if (isNegInf(s, l) || isInf(s, u)) return 0x7ff0000000000000LL;
  return __double_as_longlong(fabs(val) * (u - l));
}
__device__ __forceinline__ long long absBits(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffLL; }

// Which entries of a live row can produce a candidate (necessary conditions, never sufficient):
// * residual rule, rhs side: the residual minimal activity of entry j is finite only if the row's minimal
//   activity has no infinite/huge contribution (then newub < ub needs delta_j > slack, up to rounding, where
//   delta_j = |a_j|(ub_j - lb_j) and slack = rhs - minact), or exactly one (then only that entry); lhs side
//   likewise with the maximal activity and the surplus maxact - lhs;
// * easy rule: a candidate needs alpha_j = delta_j > max(slack, 0) (tightenVarBoundsEasy), exactly;
// * a row of one entry is always evaluated (forced tightening).
// `margin` covers every rounding difference between this estimate and the exact rule: the exact residual
// path differs from slack - delta_j by a few units in the last place of the row's largest magnitudes, and
// the plain-double recomputation of consdataGetReliableResidualActivity by at most len such units.
struct ScanOut {
  long long topd[TOPK];
  int topp[TOPK];
  int minspec, maxspec;  // entry holding an infinite or huge contribution (last one seen)
  long long maxabs;      // largest |contribution| and |a_j|*|bound| seen, as bits
};

__device__ __forceinline__ int selectEntries(const Num& s, const Act& a, const ScanOut& so, double lhs, double rhs,
                                             int len, bool easy, unsigned char (&sel)[MAXSEL], bool& full) {
  full = false;
  if (len == 1) {
    full = true;
    return 1;
  }
  const bool rhsfin = !isInf(s, rhs), lhsfin = !isNegInf(s, lhs);
  const int mintot = a.minposinf + a.minneginf + a.minposhuge + a.minneghuge;
  const int maxtot = a.maxposinf + a.maxneginf + a.maxposhuge + a.maxneghuge;
  double thrR = s.inf, thrL = s.inf;  // entries with delta > thr qualify
  bool useR = false, useL = false;
  int n = 0;
  if (easy) {
    if (rhsfin) {
      double slack = rhs - (a.minhi + a.minlo);
      if (!positive(s, slack)) slack = 0.0;
      thrR = slack;
      useR = true;
    }
    if (lhsfin) {
      double surplus = (a.maxhi + a.maxlo) - lhs;
      if (!positive(s, surplus)) surplus = 0.0;
      thrL = surplus;
      useL = true;
    }
  } else {
    const double big = __longlong_as_double(so.maxabs);
    const double margin = 1e-9 * ((rhsfin ? fabs(rhs) : 0.0) + (lhsfin ? fabs(lhs) : 0.0) + (double)(len + 2) * big) +
                          1e-300;
    if (rhsfin) {
      if (mintot == 0) {
        thrR = (rhs - (a.minhi + a.minlo)) - margin;
        useR = true;
      } else if (mintot == 1) {
        sel[n++] = (unsigned char)so.minspec;
      }
    }
    if (lhsfin) {
      if (maxtot == 0) {
        thrL = ((a.maxhi + a.maxlo) - lhs) - margin;
        useL = true;
      } else if (maxtot == 1) {
        if (n == 0 || sel[0] != (unsigned char)so.maxspec) sel[n++] = (unsigned char)so.maxspec;
      }
    }
  }
  if (useR || useL) {
    const double thr = dmin(useR ? thrR : s.inf, useL ? thrL : s.inf);
    int k = 0;
    for (; k < TOPK; ++k) {
      if (so.topp[k] < 0) break;
      const double d = __longlong_as_double(so.topd[k]);
      if (!(d > thr)) break;
      bool dup = false;
      for (int q = 0; q < n; ++q) dup |= (sel[q] == (unsigned char)so.topp[k]);
      if (!dup) sel[n++] = (unsigned char)so.topp[k];
    }
    if (k == TOPK) {  // the TOPK largest all qualify: more may, so evaluate the whole row
      full = true;
      return len;
    }
  }
  return n;
}

// Pass 1 of a short row.  Its activity is summed as two halves, entries [p0, ph) and [ph, p1) with
// ph = p0 + ceil(len/2), each in row order, the second merged into the first (the oracle's order), so that two
// lanes can scan a row together; one lane scanning both halves gets the same bits.
__device__ __forceinline__ void scanInit(Act& a, ScanOut& so, long long& mad) {
  actZero(a);
#pragma unroll
  for (int k = 0; k < TOPK; ++k) {
    so.topd[k] = -1;
    so.topp[k] = -1;
  }
  so.minspec = so.maxspec = 0;
  so.maxabs = 0;
  mad = 0;  // max delta as bits (non-negative doubles order as integers)
}

// Entries [pb0, pb1) of the row that starts at p0: contributions into a, the largest deltas, the special
// (infinite/huge) entries and the largest magnitude into so, the maximal delta into mad.
template <class BND>
__device__ __forceinline__ void scanEntries(const Num& s, const Prob& P, const BND& B, int64_t p0, int64_t pb0,
                                            int64_t pb1, Act& a, ScanOut& so, long long& mad) {
  const long long infb = __double_as_longlong(s.inf), hugeb = __double_as_longlong(s.huge);
  for (int64_t pb = pb0; pb < pb1; pb += CHUNK) {
    int jj[CHUNK];
    double vv[CHUNK], ll[CHUNK], uu[CHUNK];
    loadChunk(P, B, pb, pb1, jj, vv, ll, uu);
#pragma unroll
    for (int k = 0; k < CHUNK; ++k) {
      if (pb + k < pb1) {
        const double v = vv[k], l = ll[k], u = uu[k];
        const int pos = (int)(pb + k - p0);
        // the two contributions of the entry (addContribution semantics; classification on bit patterns so
        // that only the products and sums occupy the FP64 pipe)
        const bool vpos = __double_as_longlong(v) >= 0;
        const double bmin = vpos ? l : u, bmax = vpos ? u : l;
        const long long ibmin = __double_as_longlong(bmin), ibmax = __double_as_longlong(bmax);
        const bool minInf = (ibmin & 0x7fffffffffffffffLL) >= infb, maxInf = (ibmax & 0x7fffffffffffffffLL) >= infb;
        if (minInf) {
          if (vpos == (ibmin >= 0)) ++a.minposinf; else ++a.minneginf;
          so.minspec = pos;
        }
        if (maxInf) {
          if (vpos == (ibmax >= 0)) ++a.maxposinf; else ++a.maxneginf;
          so.maxspec = pos;
        }
        // a finite contribution v * b enters the side's compensated sum (a zero bound contributes nothing)
        auto contribute = [&](bool tomax, double c) {
          const long long cb = __double_as_longlong(c), ca = cb & 0x7fffffffffffffffLL;
          if (ca >= hugeb) {
            if (tomax) {
              if (cb >= 0) ++a.maxposhuge; else ++a.maxneghuge;
              so.maxspec = pos;
            } else {
              if (cb >= 0) ++a.minposhuge; else ++a.minneghuge;
              so.minspec = pos;
            }
          } else if (ca != 0) {
            double hi = tomax ? a.maxhi : a.minhi, lo = tomax ? a.maxlo : a.minlo;
            sum21f(hi, lo, c);
            if (tomax) {
              a.maxhi = hi;
              a.maxlo = lo;
            } else {
              a.minhi = hi;
              a.minlo = lo;
            }
          }
          if (ca > so.maxabs) so.maxabs = ca;
        };
        const bool needMin = !minInf && (ibmin & 0x7fffffffffffffffLL) != 0;
        const bool needMax = !maxInf && (ibmax & 0x7fffffffffffffffLL) != 0;
        // Usually one bound is zero or infinite and the entry has a single product; choosing its side per lane
        // lets the warp issue one multiplication and one compensated sum for all lanes.  Each side still
        // receives its contributions in row order.
        if (needMin || needMax) contribute(needMax, v * (needMax ? bmax : bmin));
        if (needMin && needMax) contribute(false, v * bmin);
        // maximal activity delta of the entry (consdataRecomputeMaxActivityDelta): infinite if a bound is
        const long long il = __double_as_longlong(l), iu = __double_as_longlong(u);
        const bool linf = il < 0 && (il & 0x7fffffffffffffffLL) >= infb;   // -l >= inf
        const bool uinf = iu >= 0 && iu >= infb;                            // u >= inf
        long long d = 0x7ff0000000000000LL;
        if (!(linf || uinf)) {
          double width = u;  // u - (+0) is u bit for bit
          if (il != 0) width = u - l;
          d = __double_as_longlong(fabs(v) * width);
        }
        if (d > mad) mad = d;
        // keep the TOPK largest deltas (ties keep the earlier entry)
        if (d > so.topd[TOPK - 1]) {
          long long cd = d;
          int cp = pos;
#pragma unroll
          for (int q = 0; q < TOPK; ++q) {
            if (cd > so.topd[q]) {
              long long td = so.topd[q];
              int tp = so.topp[q];
              so.topd[q] = cd;
              so.topp[q] = cp;
              cd = td;
              cp = tp;
            }
          }
        }
      }
    }
  }
}

// The second half's results merged into the first's: its entries all come after the first half's, so the
// largest-delta list takes them after equal deltas of the first half (the sequential scan's tie rule), and its
// special entries are the later ones.
__device__ __forceinline__ void scanMerge(Act& a, ScanOut& so, long long& mad, const Act& b, const ScanOut& sb,
                                          long long madb) {
  const bool bmin = b.minposinf + b.minneginf + b.minposhuge + b.minneghuge != 0;
  const bool bmax = b.maxposinf + b.maxneginf + b.maxposhuge + b.maxneghuge != 0;
  actMerge(a, b);
  if (bmin) so.minspec = sb.minspec;
  if (bmax) so.maxspec = sb.maxspec;
  if (sb.maxabs > so.maxabs) so.maxabs = sb.maxabs;
  if (madb > mad) mad = madb;
#pragma unroll
  for (int r = 0; r < TOPK; ++r) {
    long long cd = sb.topd[r];
    int cp = sb.topp[r];
    if (cp < 0 || !(cd > so.topd[TOPK - 1])) continue;
#pragma unroll
    for (int q = 0; q < TOPK; ++q) {
      if (cd > so.topd[q]) {
        long long td = so.topd[q];
        int tp = so.topp[q];
        so.topd[q] = cd;
        so.topp[q] = cp;
        cd = td;
        cp = tp;
      }
    }
  }
}

// End of pass 1 once the row's scan is complete: row tests, the slack rule's infeasibility test, entry
// selection.  Returns 1 on cutoff, else 0; *nsel/full describe the selected entries of a live row.
__device__ __forceinline__ int finishRow(const Num& s, int len, double lhs, double rhs, const Act& a,
                                         const ScanOut& so, long long mad, bool& easy, unsigned char (&sel)[MAXSEL],
                                         int& nsel, bool& full, Stats& st, bool count) {
  if (count) {
    st.rows += 1;
    st.nnz += len;
  }
  const double maxactdelta = (mad == 0x7ff0000000000000LL) ? s.inf : __longlong_as_double(mad);
  int t = rowTests(s, a, lhs, rhs, maxactdelta, easy);
  nsel = 0;
  full = false;
  if (t == 1) return 1;
  if (t == 0) return 0;
  if (count) st.live += 1;
  if (easy) {
    // the slack rule's own infeasibility test (tightenVarBoundsEasy), independent of the entry
    if ((!isInf(s, rhs) && feasLt(s, rhs, a.minhi + a.minlo)) || (!isNegInf(s, lhs) && feasLt(s, a.maxhi + a.maxlo, lhs)))
      return 1;
  }
  nsel = selectEntries(s, a, so, lhs, rhs, len, easy, sel, full);
  return 0;
}

// work item w of a batch belongs to the last batch row o with prefix[o] <= w
template <int NT>
__device__ __forceinline__ int itemOwner(const RowBatch<NT>& rb, int w) {
  int lo = 0, hi = NT - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (rb.prefix[mid] <= w) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// consdataGetReliableResidualActivity (cons_linear.c:2580-2657): the residual activity of entry p summed
// again in plain double, in row order
template <class BND>
__device__ __forceinline__ double reliableResidual(const Prob& P, const BND& B, int64_t p0, int64_t p1, int64_t p,
                                                   bool ismin) {
  double r = 0.0;
  for (int64_t q = p0; q < p1; ++q) {
    if (q == p) continue;
    const int jj = P.colidx[q];
    const double vv = P.vals[q];
    double ll, uu;
    B.get(jj, ll, uu);
    if (vv > 0.0) r += ismin ? vv * ll : vv * uu;
    else r += ismin ? vv * uu : vv * ll;
  }
  return r;
}

// ------------------------------------------------------------------------------------------------------
// Ranged rows: rangedRowPropagation (cons_linear.c:5715-6695) with constraints/linear/rangedrowartcons off.
// One thread evaluates a row, walking its entries in the order SCIP holds them; the rule is sequential by
// nature (running gcd, plain double sums in a fixed order) and acts on few rows, so the thread restates it
// step for step, which keeps it bit-identical with the oracle.

// The order of a row's entries on a global domain D(j, l, u): sorted (consdataCompVarProp,
// cons_linear.c:3191-3254) -- binaries by larger |a| then column, integers by larger |a|*(ub-lb) then column,
// continuous columns by column -- or the index order (consdataCompVar, :3152-3187): binaries, integers,
// continuous columns, each by column.  Keys are compared exactly, so the order is a strict total order.
template <class DOM>
__device__ __forceinline__ bool entryBefore(const Prob& P, const DOM& D, bool sorted, int64_t p, int64_t q) {
  const int jp = P.colidx[p], jq = P.colidx[q];
  double lp, up, lq, uq;
  D(jp, lp, up);
  D(jq, lq, uq);
  const bool ip = P.isint[jp] != 0, iq = P.isint[jq] != 0;
  const bool bp = ip && lp >= 0.0 && up <= 1.0, bq = iq && lq >= 0.0 && uq <= 1.0;
  if (bp != bq) return bp;
  if (bp && sorted) {
    const long long a1 = absBitsOf(P.vals[p]), a2 = absBitsOf(P.vals[q]);
    if (a1 != a2) return a1 > a2;
    return jp < jq;
  }
  if (ip != iq) return ip;
  if (!ip || !sorted) return jp < jq;
  const double kp = fabs(P.vals[p] * (up - lp)), kq = fabs(P.vals[q] * (uq - lq));
  if (kp != kq) return kp > kq;
  return jp < jq;
}

// writes row i's order to P.rperm[p0 ..) by a bottom-up merge sort through P.rtmp (one thread)
template <class DOM>
__device__ void rowOrder(const Prob& P, const DOM& D, bool sorted, int i) {
  const int64_t p0 = P.rowptr[i];
  const int len = (int)(P.rowptr[i + 1] - p0);
  int32_t* src = P.rperm + p0;
  int32_t* dst = P.rtmp + p0;
  for (int k = 0; k < len; ++k) src[k] = k;
  for (int w = 1; w < len; w *= 2) {
    for (int lo = 0; lo < len; lo += 2 * w) {
      const int mid = min(lo + w, len), hi = min(lo + 2 * w, len);
      int x = lo, y = mid;
      for (int k = lo; k < hi; ++k) {
        if (y >= hi || (x < mid && !entryBefore(P, D, sorted, p0 + src[y], p0 + src[x]))) dst[k] = src[x++];
        else dst[k] = src[y++];
      }
    }
    int32_t* t = src;
    src = dst;
    dst = t;
  }
  if (src != P.rperm + p0)
    for (int k = 0; k < len; ++k) P.rperm[p0 + k] = src[k];
}

// (SCIP_Longint)(REALABS(val) + feastol), cons_linear.c:5903/5944/6057, saturated where the cast would overflow
__device__ __forceinline__ long long coefInt(const Num& s, double v) {
  const double x = fabs(v) + s.feastol;
  return x >= 4.0e18 ? 4000000000000000000LL : (long long)x;
}
// greatest common divisor of non-negative integers (the value SCIPcalcGreComDiv, misc.c:9197, computes), by the
// binary method: shifts and subtractions instead of 64-bit divisions, which the GPU emulates in software
__device__ __forceinline__ long long gcd64(long long a, long long b) {
  unsigned long long u = (unsigned long long)a, v = (unsigned long long)b;
  if (u == 0) return (long long)v;
  if (v == 0) return (long long)u;
  const int shift = __ffsll((long long)(u | v)) - 1;
  u >>= __ffsll((long long)u) - 1;
  do {
    v >>= __ffsll((long long)v) - 1;
    if (u > v) {
      const unsigned long long t = u;
      u = v;
      v = t;
    }
    v -= u;
  } while (v != 0);
  return (long long)(u << shift);
}
__device__ __forceinline__ bool epsIntegral(const Num& s, double x) { return x - floor(x + s.eps) <= s.eps; }
__device__ __forceinline__ double epsFloor(const Num& s, double x) { return floor(x + s.eps); }
__device__ __forceinline__ double epsCeil(const Num& s, double x) { return ceil(x - s.eps); }

// each solution-enumeration loop runs at most this often; a row that needs more yields no deduction
constexpr long long RANGED_MAXIT = 1LL << 20;
// the running gcd of the partition changes at most 62 times (it at least halves each time)
constexpr int RANGED_MAXCHG = 64;

// what an entry is to the ranged-row rule (the per-entry values of Prob::rcoef)
__device__ __forceinline__ long long rangedCoef(const Num& s, bool isint, double v) {
  if (isint && epsIntegral(s, v) && !eq(s, fabs(v), 1.0)) return coefInt(s, v);
  return eq(s, fabs(v), 1.0) ? -1 : -2;
}

// Row i's ranged-row deductions from the bounds B (forced candidates, as SCIP's come with force = TRUE);
// returns true on cutoff.  One thread.  The entries' classification comes precomputed (P.rcoef); which entries are
// fixed is kept as bits for the first 64 positions, so that the passes after the first read bounds only where they
// need the values.
template <class BND>
__device__ bool rangedRow(const Num& s, const Prob& P, const BND& B, int i, Cands& C, Stats& st) {
  const int64_t p0 = P.rowptr[i];
  const int len = (int)(P.rowptr[i + 1] - p0);
  if (P.rlive) {
    auto dom = [&](int j, double& l, double& u) { B.glob(P, j, l, u); };
    rowOrder(P, dom, P.rsorted != 0, i);
  }
  const int32_t* ord = P.rperm + p0;
  auto fixedAt = [&](int k, int64_t& p, int& j, double& v, double& l, double& u) {
    p = p0 + ord[k];
    j = P.colidx[p];
    v = P.vals[p];
    B.get(j, l, u);
    return eq(s, l, u);
  };

  // fixed activity, last entry first (cons_linear.c:5803-5814)
  double fixedact = 0.0;
  int nfixed = 0;
  unsigned long long fixm = 0ull;  // fixed entries among the first 64 positions
  for (int k = len - 1; k >= 0; --k) {
    int64_t p;
    int j;
    double v, l, u;
    if (fixedAt(k, p, j, v, l, u)) {
      fixedact += l * v;
      ++nfixed;
      if (k < 64) fixm |= 1ull << k;
    }
  }
  if (isHuge(s, fabs(fixedact))) return false;
  const double lhs = P.lhs[i] - fixedact, rhs = P.rhs[i] - fixedact;
  auto isFixed = [&](int k) {
    if (k < 64) return ((fixm >> k) & 1ull) != 0;
    double l, u;
    B.get(P.colidx[p0 + ord[k]], l, u);
    return eq(s, l, u);
  };
  auto coefAt = [&](int k) { return P.rcoef[p0 + ord[k]]; };
  auto contAt = [&](int k) { return P.isint[P.colidx[p0 + ord[k]]] == 0; };

  // partition (cons_linear.c:5839-5958); membership of position k is kept as a bit for the first 64 positions and
  // recomputed beyond from the running gcd, whose changes are recorded as (position, gcd after it)
  int ninf = 0, ncont = 0, first = -1, kstart;
  bool gcdisone = true, possiblegcd = true;
  unsigned long long memb = 0ull;  // membership of the first 64 positions
  int k = -1;
  do {
    ++k;
    while (k < len && coefAt(k) < 0) {
      if (!isFixed(k)) {
        if (contAt(k)) ++ncont;
        gcdisone = gcdisone && coefAt(k) == -1;
        possiblegcd = false;
        ++ninf;
        if (first < 0) first = k;
        if (k < 64) memb |= 1ull << k;
      }
      ++k;
    }
  } while (k < len && isFixed(k));
  if (k >= len || ncont + 2 > len - nfixed) return false;
  kstart = k;
  const long long g0 = coefAt(k);
  int chgpos[RANGED_MAXCHG];
  long long chgval[RANGED_MAXCHG];
  int nchg = 0;
  long long gcd = g0;
  for (; k < len; ++k) {
    if (isFixed(k)) continue;
    const long long ck = coefAt(k);
    if (ck < 0) {
      if (contAt(k)) ++ncont;
      gcdisone = gcdisone && ck == -1;
      possiblegcd = false;
      ++ninf;
      if (first < 0) first = k;
      if (k < 64) memb |= 1ull << k;
    } else {
      const long long t = gcd64(gcd, ck);
      if (t == 1) {
        ++ninf;
        if (first < 0) first = k;
        if (k < 64) memb |= 1ull << k;
      } else if (t != gcd) {
        if (nchg < RANGED_MAXCHG) {
          chgpos[nchg] = k;
          chgval[nchg] = t;
          ++nchg;
        }
        gcd = t;
      }
    }
  }
  if (ninf == 0) return false;
  // is position kk (unfixed) one of the entries that may lead to infeasibility?
  auto member = [&](int kk) {
    if (kk < 64) return ((memb >> kk) & 1ull) != 0;
    const long long ck = coefAt(kk);
    if (kk < kstart || ck < 0) return true;
    long long gb = g0;
    for (int t = 0; t < nchg && chgpos[t] < kk; ++t) gb = chgval[t];
    return gcd64(gb, ck) == 1;
  };

  // activity bounds of those entries, last first (cons_linear.c:5975-6015)
  double minact = 0.0, maxact = 0.0;
  for (k = len - 1; k >= 0; --k) {
    int64_t p;
    int j;
    double v, l, u;
    if (isFixed(k) || !member(k)) continue;
    fixedAt(k, p, j, v, l, u);
    bool mininv = false, maxinv = false;
    if (isNegInf(s, l)) {
      if (v < 0.0) maxinv = true;
      else mininv = true;
    } else if (v < 0.0) {
      maxact += v * l;
    } else {
      minact += v * l;
    }
    if (isInf(s, u)) {
      if (v > 0.0) maxinv = true;
      else mininv = true;
    } else if (v > 0.0) {
      maxact += v * u;
    } else {
      minact += v * u;
    }
    if (isNegHuge(s, minact)) mininv = true;
    if (isHuge(s, maxact)) maxinv = true;
    if (mininv || maxinv) return false;
  }

  // no multiple of gcd between the sides (cons_linear.c:6033-6045)
  const double g = (double)gcd;
  if (!epsIntegral(s, (lhs - maxact) / g) && gt(s, epsCeil(s, (lhs - maxact) / g) * g, rhs - minact)) {
    logRanged(C, i, -1);
    return true;
  }
  if (ncont != 0) return false;

  // gcd of the other entries (cons_linear.c:6051-6064)
  long long gcdinf = -1;
  if (possiblegcd) {
    for (k = len - 1; k >= 0; --k) {
      if (isFixed(k) || !member(k)) continue;
      gcdinf = gcdinf < 0 ? coefAt(k) : gcd64(gcdinf, coefAt(k));
      if (gcdinf < 2) break;
    }
  } else if (gcdisone) {
    gcdinf = 1;
  }
  if (gcdinf < 1) return false;

  // feasible values of the other entries' activity (cons_linear.c:6076-6139)
  double minvalue = 0.0, maxvalue = 0.0;
  int nsols = 0;
  double value = epsCeil(s, minact - s.feastol);
  for (long long it = 0; le(s, value, maxact); ++it) {
    if (it >= RANGED_MAXIT) return false;
    double value2 = value + g * epsCeil(s, (lhs - value) / g);
    if (!ge(s, value2, lhs)) value2 += g;
    if (le(s, value2, rhs)) {
      ++nsols;
      if (nsols == 3) break;
      if (nsols == 1) minvalue = value;
      maxvalue = value;
    }
    value += (double)gcdinf;
  }
  if (nsols == 3) {
    value = epsFloor(s, maxact + s.feastol);
    for (long long it = 0; ge(s, value, minact); ++it) {
      if (it >= RANGED_MAXIT) return false;
      double value2 = value + g * epsFloor(s, (rhs - value) / g);
      if (!le(s, value2, rhs)) value2 -= g;
      if (ge(s, value2, lhs)) {
        maxvalue = value;
        break;
      }
      value -= (double)gcdinf;
    }
  }
  if (nsols == 0) {
    logRanged(C, i, -1);
    return true;
  }

  int target = -1;
  if (ninf == 1) {
    target = first;  // the single other entry (fixed :6160-6183, bounded :6296-6352)
  } else if (ninf == len - nfixed - 1) {
    // the one unfixed entry outside them (fixed :6184-6283, bounded :6354-6552)
    for (k = 0; k < len; ++k) {
      if (!isFixed(k) && !member(k)) {
        target = k;
        break;
      }
    }
  }
  if (target < 0) return false;
  int64_t p;
  int j;
  double v, l, u;
  fixedAt(target, p, j, v, l, u);
  double newlb, newub;
  bool fix = nsols == 1;
  if (ninf == 1) {
    if (fix) {
      newlb = newub = maxvalue / v;
    } else {
      newlb = v < 0.0 ? maxvalue / v : minvalue / v;
      newub = v < 0.0 ? minvalue / v : maxvalue / v;
    }
  } else if (fix) {
    newlb = newub = v < 0.0 ? epsFloor(s, (lhs - maxvalue) / v) : epsCeil(s, (lhs - maxvalue) / v);
  } else {
    newlb = v < 0.0 ? epsFloor(s, (rhs - minvalue) / v) : epsCeil(s, (lhs - maxvalue) / v);
    newub = v < 0.0 ? epsFloor(s, (lhs - maxvalue) / v) : epsCeil(s, (rhs - minvalue) / v);
  }
  const EmitTo emit{&C, j, &st.cands};
  if (fix || newlb > l) emit(false, newlb, true);
  if (fix || newub < u) emit(true, newub, true);
  if (fix || newlb > l || newub < u) logRanged(C, i, j);
  return false;
}

// The CTA processes rows[0..nrows) (all <= LONGROW entries).  All threads of the CTA must call it with the
// same arguments.  Sets *cut on infeasibility.
// RANGED: the ranged-row rule runs for rows that carry it (P.relig); false compiles it out
template <int NT, bool RANGED = true, class BND>
__device__ void processShortRows(const Num& s, const Prob& P, const BND& B, const int* rows, int nrows, Cands& C,
                                 Stats& st, RowBatch<NT>& rb, int* cut) {
  const int tid = threadIdx.x;
  for (int base = 0; base < nrows; base += NT) {
    const int cnt = (nrows - base) < NT ? (nrows - base) : NT;
    // counting sort of the batch by row length (descending)
    for (int b = tid; b < LONGROW + 2; b += NT) rb.hist[b] = 0;
    __syncthreads();
    int myrow = -1, mylen = 0;
    if (tid < cnt) {
      myrow = rows[base + tid];
      mylen = (int)(P.rowptr[myrow + 1] - P.rowptr[myrow]);
      atomicAdd(&rb.hist[LONGROW - mylen], 1);
    }
    __syncthreads();
    if (tid == 0) {
      int acc = 0;
      for (int b = 0; b <= LONGROW; ++b) {
        int h = rb.hist[b];
        rb.hist[b] = acc;
        acc += h;
      }
    }
    __syncthreads();
    if (tid < cnt) rb.order[atomicAdd(&rb.hist[LONGROW - mylen], 1)] = myrow;
    __syncthreads();

    int nsel = 0;
    bool full = false;
    {
      // Batches of up to NT/2 rows give each row two adjacent lanes, one half each: the odd lane hands its half
      // to the even lane through shared memory.  Larger batches give each row one lane that scans both halves
      // in turn, parking the first half's activity in the row's slot.  Either way the even lane (or the single
      // lane) merges first-then-second and finishes the row; the scan loop has one call site.
      const bool pairs = cnt <= NT / 2;
      const int pos = pairs ? (tid >> 1) : tid;
      const bool second = pairs && (tid & 1) != 0;
      const bool live = pos < cnt && !rowDead(P, rb.order[pos]);
      Act a;
      ScanOut so;
      long long mad;
      scanInit(a, so, mad);
      int64_t p0 = 0;
      int len = 0;
      if (live) {
        const int i = rb.order[pos];
        p0 = P.rowptr[i];
        len = (int)(P.rowptr[i + 1] - p0);
        const int64_t ph = p0 + (len + 1) / 2;
        const int nr = pairs ? 1 : 2;
#pragma unroll 1
        for (int r = 0; r < nr; ++r) {
          const bool h2 = pairs ? second : (r == 1);
          if (!pairs && r == 1) {
            rb.act[pos] = a;  // the first half's activity waits in the row's slot
            actZero(a);
          }
          scanEntries(s, P, B, p0, h2 ? ph : p0, h2 ? p0 + len : ph, a, so, mad);
        }
        if (!pairs) {
          Act whole = rb.act[pos];
          actMerge(whole, a);
          a = whole;
        } else if (second) {
          rb.act[NT / 2 + pos] = a;
#pragma unroll
          for (int k = 0; k < TOPK; ++k) {
            rb.htopd[pos][k] = so.topd[k];
            rb.htopp[pos][k] = so.topp[k];
          }
          rb.hspec[pos][0] = so.minspec;
          rb.hspec[pos][1] = so.maxspec;
          rb.hmaxabs[pos] = so.maxabs;
          rb.hmad[pos] = mad;
        }
      }
      __syncwarp();
      if (live && !second) {
        const int i = rb.order[pos];
        if (pairs) {
          ScanOut sb;
#pragma unroll
          for (int k = 0; k < TOPK; ++k) {
            sb.topd[k] = rb.htopd[pos][k];
            sb.topp[k] = rb.htopp[pos][k];
          }
          sb.minspec = rb.hspec[pos][0];
          sb.maxspec = rb.hspec[pos][1];
          sb.maxabs = rb.hmaxabs[pos];
          scanMerge(a, so, mad, rb.act[NT / 2 + pos], sb, rb.hmad[pos]);
        }
        const double lhs = P.lhs[i], rhs = P.rhs[i];
        bool easy = false;
        unsigned char sel[MAXSEL];
        if (finishRow(s, len, lhs, rhs, a, so, mad, easy, sel, nsel, full, st, true)) cutRow(P, i, cut);
        rb.act[pos] = a;
        rb.lhs[pos] = lhs;
        rb.rhs[pos] = rhs;
        rb.p0[pos] = p0;
        rb.len[pos] = len;
        rb.easy[pos] = easy ? 1 : 0;
        rb.full[pos] = full ? 1 : 0;
#pragma unroll
        for (int q = 0; q < MAXSEL; ++q) rb.sel[pos][q] = sel[q];
      }
      const int slot = second ? NT / 2 + pos : pos;  // in pairs the odd lanes clear the upper half of the slots
      rb.nsel[slot] = (live && !second) ? nsel : 0;
      rb.bpos[slot] = -1;
    }
    __syncthreads();
    // exclusive prefix of the selection counts
    if (tid < 32) {
      int carry = 0;
      for (int c0 = 0; c0 < NT; c0 += 32) {
        int v = rb.nsel[c0 + tid];
        int x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, x, off);
          if (tid >= off) x += y;
        }
        rb.prefix[c0 + tid] = carry + x - v;
        carry += __shfl_sync(0xffffffffu, x, 31);
      }
      if (tid == 0) rb.prefix[NT] = carry;
    }
    __syncthreads();
    const int total = rb.prefix[NT];
    // Binary columns follow tightenBounds' visit (cons_linear.c:7110-7138): the row's binaries are tried in
    // the order of binBefore and the first unfixed one without a candidate ends the visit.  So the candidates
    // of binaries are held back (bit `it` of candm: this thread's it-th work item) until every binary of the
    // batch has been tried and each row knows its first such binary (rb.bpos); then the ones before it are
    // evaluated again and emitted.  A thread has at most LONGROW work items (total <= NT * LONGROW).
    unsigned long long candm = 0ull;
    int it = 0;
    for (int w = tid; w < total; w += NT, ++it) {
      const int o = itemOwner(rb, w);
      const int k = w - rb.prefix[o];
      const int64_t p0 = rb.p0[o];
      const int64_t p1 = p0 + rb.len[o];
      const int64_t p = p0 + (rb.full[o] ? k : (int)rb.sel[o][k]);
      const int j = P.colidx[p];
      const double v = P.vals[p];
      double l, u;
      B.get(j, l, u);
      const Act a = rb.act[o];
      const bool force = p1 - p0 == 1;
      auto relres = [&](bool ismin) { return reliableResidual(P, B, p0, p1, p, ismin); };
      if (s.nosort || force || !isBinaryCol(P, B, j)) {
        if (columnCandidates(s, a, rb.lhs[o], rb.rhs[o], rb.easy[o] != 0, force, v, l, u, P.isint[j] != 0,
                             EmitTo{&C, j, &st.cands}, relres))
          cutRow(P, rb.order[o], cut);
        continue;
      }
      bool hit = false;
      if (columnCandidates(s, a, rb.lhs[o], rb.rhs[o], rb.easy[o] != 0, false, v, l, u, true, Probe{&hit}, relres))
        cutRow(P, rb.order[o], cut);
      if (hit) {
        candm |= 1ull << it;
      } else if (!feasEq(s, u, l)) {
        // keep the earliest such binary of the row
        const int mine = (int)(p - p0);
        int cur = rb.bpos[o];
        while (cur < 0 || binBefore(P, p, p0 + cur)) {
          const int prev = atomicCAS(&rb.bpos[o], cur, mine);
          if (prev == cur) break;
          cur = prev;
        }
      }
    }
    if (__syncthreads_or(candm != 0ull)) {
      it = 0;
      for (int w = tid; w < total; w += NT, ++it) {
        if (!((candm >> it) & 1ull)) continue;
        const int o = itemOwner(rb, w);
        const int k = w - rb.prefix[o];
        const int64_t p0 = rb.p0[o];
        const int64_t p1 = p0 + rb.len[o];
        const int64_t p = p0 + (rb.full[o] ? k : (int)rb.sel[o][k]);
        const int b = rb.bpos[o];
        if (b >= 0 && binBefore(P, p0 + b, p)) continue;  // visited after the end of the binaries
        const int j = P.colidx[p];
        const double v = P.vals[p];
        double l, u;
        B.get(j, l, u);
        const Act a = rb.act[o];
        auto relres = [&](bool ismin) { return reliableResidual(P, B, p0, p1, p, ismin); };
        columnCandidates(s, a, rb.lhs[o], rb.rhs[o], rb.easy[o] != 0, false, v, l, u, true, EmitTo{&C, j, &st.cands},
                         relres);
      }
    }
    // ranged rows of the batch, one thread each, after the activity rules (propagateCons, cons_linear.c:7694-7711)
    if (RANGED && P.relig != nullptr) {
      for (int o = tid; o < cnt; o += NT) {
        const int i = rb.order[o];
        if (P.relig[i] != 0 && !rowDead(P, i) && rangedRow(s, P, B, i, C, st)) cutRow(P, i, cut);
      }
    }
    __syncthreads();
  }
}

// One frontier row longer than LONGROW, processed by a whole warp: lane k sums entries k, k+32, ... and the
// 32 partials are merged pairwise (k absorbs k+16, k+8, ..., k+1) -- the same order the oracle uses.
// Returns true (on every lane) on cutoff.
template <class BND>
__device__ bool rowWarpCore(const Num& s, const Prob& P, const BND& B, int i, Cands& C, Stats& st) {
  const int lane = threadIdx.x & 31;
  const int64_t p0 = P.rowptr[i], p1 = P.rowptr[i + 1];
  const double lhs = P.lhs[i], rhs = P.rhs[i];
  Act a;
  actZero(a);
  double mad = 0.0;
  bool madinf = false;
  long long maxabs = 0;  // largest |contribution| of the lane's entries, as bits
  for (int64_t p = p0 + lane; p < p1; p += 32) {
    int j = P.colidx[p];
    double v = P.vals[p];
    double l, u;
    B.get(j, l, u);
    addTerm(s, a, v, l, u);
    if (!isInf(s, fabs(l))) {
      long long b = absBits(v * l);
      if (b > maxabs) maxabs = b;
    }
    if (!isInf(s, fabs(u))) {
      long long b = absBits(v * u);
      if (b > maxabs) maxabs = b;
    }
    double d = entryDelta(s, v, l, u);
    if (d < 0.0) madinf = true;
    else if (d > mad) mad = d;
  }
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    Act b;
    b.minhi = __shfl_down_sync(0xffffffffu, a.minhi, off);
    b.minlo = __shfl_down_sync(0xffffffffu, a.minlo, off);
    b.maxhi = __shfl_down_sync(0xffffffffu, a.maxhi, off);
    b.maxlo = __shfl_down_sync(0xffffffffu, a.maxlo, off);
    b.minposinf = __shfl_down_sync(0xffffffffu, a.minposinf, off);
    b.minneginf = __shfl_down_sync(0xffffffffu, a.minneginf, off);
    b.minposhuge = __shfl_down_sync(0xffffffffu, a.minposhuge, off);
    b.minneghuge = __shfl_down_sync(0xffffffffu, a.minneghuge, off);
    b.maxposinf = __shfl_down_sync(0xffffffffu, a.maxposinf, off);
    b.maxneginf = __shfl_down_sync(0xffffffffu, a.maxneginf, off);
    b.maxposhuge = __shfl_down_sync(0xffffffffu, a.maxposhuge, off);
    b.maxneghuge = __shfl_down_sync(0xffffffffu, a.maxneghuge, off);
    double dm = __shfl_down_sync(0xffffffffu, mad, off);
    if (lane < off) {
      actMerge(a, b);
      if (dm > mad) mad = dm;
    }
  }
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    long long o = __shfl_xor_sync(0xffffffffu, maxabs, off);
    if (o > maxabs) maxabs = o;
  }
  a.minhi = __shfl_sync(0xffffffffu, a.minhi, 0);
  a.minlo = __shfl_sync(0xffffffffu, a.minlo, 0);
  a.maxhi = __shfl_sync(0xffffffffu, a.maxhi, 0);
  a.maxlo = __shfl_sync(0xffffffffu, a.maxlo, 0);
  a.minposinf = __shfl_sync(0xffffffffu, a.minposinf, 0);
  a.minneginf = __shfl_sync(0xffffffffu, a.minneginf, 0);
  a.minposhuge = __shfl_sync(0xffffffffu, a.minposhuge, 0);
  a.minneghuge = __shfl_sync(0xffffffffu, a.minneghuge, 0);
  a.maxposinf = __shfl_sync(0xffffffffu, a.maxposinf, 0);
  a.maxneginf = __shfl_sync(0xffffffffu, a.maxneginf, 0);
  a.maxposhuge = __shfl_sync(0xffffffffu, a.maxposhuge, 0);
  a.maxneghuge = __shfl_sync(0xffffffffu, a.maxneghuge, 0);
  mad = __shfl_sync(0xffffffffu, mad, 0);
  madinf = __any_sync(0xffffffffu, madinf);
  if (lane == 0) {
    st.rows += 1;
    st.nnz += p1 - p0;
  }
  bool easy = false;
  int t = rowTests(s, a, lhs, rhs, madinf ? s.inf : mad, easy);
  if (t == 1) return true;
  if (t == 0) return false;
  if (lane == 0) st.live += 1;
  const bool rhsfin = !isInf(s, rhs), lhsfin = !isNegInf(s, lhs);
  if (easy && ((rhsfin && feasLt(s, rhs, a.minhi + a.minlo)) || (lhsfin && feasLt(s, a.maxhi + a.maxlo, lhs))))
    return true;  // the slack rule's own infeasibility test (tightenVarBoundsEasy)

  // which entries can produce a candidate (the necessary conditions of selectEntries, per entry)
  const int mintot = a.minposinf + a.minneginf + a.minposhuge + a.minneghuge;
  const int maxtot = a.maxposinf + a.maxneginf + a.maxposhuge + a.maxneghuge;
  bool useR = false, useL = false;
  double thrR = 0.0, thrL = 0.0;
  const bool specMin = !easy && rhsfin && mintot == 1, specMax = !easy && lhsfin && maxtot == 1;
  if (easy) {
    if (rhsfin) {
      double slack = rhs - (a.minhi + a.minlo);
      thrR = positive(s, slack) ? slack : 0.0;
      useR = true;
    }
    if (lhsfin) {
      double surplus = (a.maxhi + a.maxlo) - lhs;
      thrL = positive(s, surplus) ? surplus : 0.0;
      useL = true;
    }
  } else {
    const double margin = 1e-9 * ((rhsfin ? fabs(rhs) : 0.0) + (lhsfin ? fabs(lhs) : 0.0) +
                                  (double)(p1 - p0 + 2) * __longlong_as_double(maxabs)) + 1e-300;
    if (rhsfin && mintot == 0) {
      thrR = (rhs - (a.minhi + a.minlo)) - margin;
      useR = true;
    }
    if (lhsfin && maxtot == 0) {
      thrL = ((a.maxhi + a.maxlo) - lhs) - margin;
      useL = true;
    }
  }
  const long long infb = __double_as_longlong(s.inf), hugeb = __double_as_longlong(s.huge);
  // entry p can produce a candidate (the necessary conditions above)
  auto selected = [&](double v, double l, double u) {
    const double d = __longlong_as_double(deltaBits(s, v, l, u));  // +inf for an infinite bound
    bool go = (useR && d > thrR) || (useL && d > thrL);
    if (!go && (specMin || specMax)) {
      const bool vpos = __double_as_longlong(v) >= 0;
      const double bmin = vpos ? l : u, bmax = vpos ? u : l;
      if (specMin) go |= (absBits(bmin) >= infb) || (absBits(v * bmin) >= hugeb);
      if (specMax) go |= (absBits(bmax) >= infb) || (absBits(v * bmax) >= hugeb);
    }
    return go;
  };
  // Binary columns follow tightenBounds' visit (cons_linear.c:7110-7138), as in processShortRows: their
  // candidates wait until the warp knows the row's first binary (in binBefore order) that gets none.  Bit it
  // of candm marks the lane's it-th entry; entries past the 64th of a lane are tried again afterwards.
  bool cut = false;
  unsigned long long candm = 0ull;
  bool later = false;                 // a binary candidate beyond the 64th entry of this lane
  long long blkA = -1;                // the lane's first candidate-free unfixed binary: |a| bits, column
  int blkC = 0x7fffffff;
  int it = 0;
  for (int64_t p = p0 + lane; p < p1; p += 32, ++it) {
    int j = P.colidx[p];
    double v = P.vals[p];
    double l, u;
    B.get(j, l, u);
    if (!selected(v, l, u)) continue;
    auto relres = [&](bool ismin) { return reliableResidual(P, B, p0, p1, p, ismin); };
    if (s.nosort || !isBinaryCol(P, B, j)) {
      if (columnCandidates(s, a, lhs, rhs, easy, false, v, l, u, P.isint[j] != 0, EmitTo{&C, j, &st.cands},
                           relres)) {
        cut = true;
        break;
      }
      continue;
    }
    bool hit = false;
    if (columnCandidates(s, a, lhs, rhs, easy, false, v, l, u, true, Probe{&hit}, relres)) {
      cut = true;
      break;
    }
    if (hit) {
      if (it < 64) candm |= 1ull << it;
      else later = true;
    } else if (!feasEq(s, u, l)) {
      const long long ab = absBitsOf(v);
      if (ab > blkA || (ab == blkA && j < blkC)) {
        blkA = ab;
        blkC = j;
      }
    }
  }
  if (__any_sync(0xffffffffu, cut)) return true;
  if (!__any_sync(0xffffffffu, candm != 0ull || later)) return false;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const long long oa = __shfl_xor_sync(0xffffffffu, blkA, off);
    const int oc = __shfl_xor_sync(0xffffffffu, blkC, off);
    if (oa > blkA || (oa == blkA && oc < blkC)) {
      blkA = oa;
      blkC = oc;
    }
  }
  // a binary is visited if it comes before the first candidate-free one
  auto visited = [&](double v, int j) {
    const long long ab = absBitsOf(v);
    return blkA < 0 || ab > blkA || (ab == blkA && j < blkC);
  };
  it = 0;
  for (int64_t p = p0 + lane; p < p1; p += 32, ++it) {
    if (it < 64) {
      if (!((candm >> it) & 1ull)) continue;
    } else if (!later) {
      break;
    }
    const int j = P.colidx[p];
    const double v = P.vals[p];
    if (!visited(v, j)) continue;
    double l, u;
    B.get(j, l, u);
    if (it >= 64 && (!selected(v, l, u) || !isBinaryCol(P, B, j))) continue;
    auto relres = [&](bool ismin) { return reliableResidual(P, B, p0, p1, p, ismin); };
    columnCandidates(s, a, lhs, rhs, easy, false, v, l, u, true, EmitTo{&C, j, &st.cands}, relres);
  }
  return false;
}

// the activity rules of a long row, then (lane 0) its ranged-row rule; true on every lane on cutoff
template <bool RANGED = true, class BND>
__device__ bool rowWarp(const Num& s, const Prob& P, const BND& B, int i, Cands& C, Stats& st) {
  const bool cut = rowWarpCore(s, P, B, i, C, st);
  if (!RANGED || P.relig == nullptr || P.relig[i] == 0) return cut;
  bool rcut = false;
  if ((threadIdx.x & 31) == 0) rcut = rangedRow(s, P, B, i, C, st);
  return cut || __shfl_sync(0xffffffffu, rcut ? 1 : 0, 0) != 0;
}

// Acceptance of column j's best candidates against its round-start bounds [l,u]: upper bound first
// (SCIPinferVarUbCons: adjust, infeasible if FeasLT(new, lb), clamp, accept if UbBetter or forced), then the
// lower bound against the new upper bound (SCIPinferVarLbCons).  Resets the candidate slots.
// Returns true on cutoff; nl/nu receive the new bounds.
__device__ __forceinline__ bool applyColumn(const Num& s, bool isint, double l, double u, Cands& C, int j,
                                            double& nl, double& nu) {
  const int f = C.cflag[j];
  const long long kub = C.cub[j], kubf = C.cubf[j], klb = C.clb[j], klbf = C.clbf[j];
  C.cflag[j] = 0;
  C.cub[j] = KEY_NONE_UB;
  C.cubf[j] = KEY_NONE_UB;
  C.clb[j] = KEY_NONE_LB;
  C.clbf[j] = KEY_NONE_LB;
  nu = u;
  nl = l;
  bool cut = false;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool force = (k == 1);
    if (!(f & (force ? 2 : 1))) continue;
    double c = adjUb(s, isint, keyd(force ? kubf : kub));
    if (isNegInf(s, c) || feasLt(s, c, l)) { cut = true; continue; }
    c = dmax(c, l);
    if (force ? !ge(s, c, u) : ubBetter(s, c, l, u)) nu = dmin(nu, c);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool force = (k == 1);
    if (!(f & (force ? 8 : 4))) continue;
    double c = adjLb(s, isint, keyd(force ? klbf : klb));
    if (isInf(s, c) || feasGt(s, c, nu)) { cut = true; continue; }
    c = dmin(c, nu);
    if (force ? !le(s, c, l) : lbBetter(s, c, l, nu)) nl = dmax(nl, c);
  }
  return cut;
}

}  // namespace gbp
