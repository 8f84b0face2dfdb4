// Propagation kernels for sm_103a (FP64, sparse, no tensor cores).
//
// Plain path (one problem, one launch sequence per round):
//   k_rows_short  one thread per frontier row of <= LONGROW entries
//   k_rows_long   one warp per longer frontier row
//   k_apply       one thread per touched column: acceptance, bound write, frontier expansion
// Batched path:
//   k_nodes       persistent; each CTA takes branch-and-bound nodes off a queue and runs a node's whole
//                 fixpoint with CTA-wide barriers between the phases of a round.  A node's bounds are the
//                 shared base vector plus a per-CTA overlay (ovl/ostamp), so nodes cost what they touch.
#include <cooperative_groups.h>

#include "gbp_nodes.cuh"

namespace gbp {

namespace cg = cooperative_groups;

struct PlainBnd {
  const double* lb;
  const double* ub;
  __device__ __forceinline__ void get(int j, double& l, double& u) const {
    l = lb[j];
    u = ub[j];
  }
  // global domain: the problem's explicit global bounds, else the bounds being propagated (root)
  __device__ __forceinline__ void glob(const Prob& P, int j, double& l, double& u) const {
    l = P.glb != nullptr ? P.glb[j] : lb[j];
    u = P.gub != nullptr ? P.gub[j] : ub[j];
  }
};

// ------------------------------------------------------------------------------------------ plain path
constexpr int ROW_THREADS = 128;

// ---- bodies shared by the host-driven kernels and the graph-driven loop
__device__ __forceinline__ void rowsShortBody(const Num& s, const Prob& P, const PlainBnd& B, const int* list, int n,
                                              Cands& C, int* cutoff, unsigned long long* stats,
                                              RowBatch<ROW_THREADS>& rb, int* s_cut) {
  if (threadIdx.x == 0) *s_cut = 0;
  __syncthreads();
  Stats st{0, 0, 0, 0};
  // a frontier smaller than the grid's threads is spread over every block (a batch's latency grows with its rows:
  // each row's scan is sequential, and its candidates share the block's threads); larger ones go in full batches
  const int per = n < (int)gridDim.x * ROW_THREADS ? (n + (int)gridDim.x - 1) / (int)gridDim.x : ROW_THREADS;
  for (int base = blockIdx.x * per; base < n; base += gridDim.x * per) {
    const int cnt = (n - base) < per ? (n - base) : per;
    processShortRows<ROW_THREADS>(s, P, B, list + base, cnt, C, st, rb, s_cut);
  }
  __syncthreads();
  if (threadIdx.x == 0 && *s_cut) atomicExch(cutoff, 1);
  flushStats(stats, st);
}

__device__ __forceinline__ void rowsLongBody(const Num& s, const Prob& P, const PlainBnd& B, const int* list, int n,
                                             int cap, Cands& C, int* cutoff, unsigned long long* stats) {
  Stats st{0, 0, 0, 0};
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int w = warp; w < n; w += nwarps) {
    const int row = list[cap - 1 - w];
    if (rowDead(P, row)) continue;
    if (rowWarp(s, P, B, row, C, st) && lane == 0) {
      if (P.instcut != nullptr) atomicExch(&P.instcut[P.rowinst[row]], 1);
      else atomicExch(cutoff, 1);
    }
  }
  flushStats(stats, st);
}

__device__ __forceinline__ void applyBody(const Num& s, const Prob& P, double* lb, double* ub, Cands& C, Front& F,
                                          int stamp, int* cutoff, unsigned long long* stats, const ChangeLog& G,
                                          int round, const MovedLog& M = MovedLog{}) {
  const int n = *C.ntouched;
  unsigned long long changes = 0;
  bool cut = false;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int j = C.touched[t];
    double l = lb[j], u = ub[j], nl, nu;
    const bool c = applyColumn(s, P.isint[j] != 0, l, u, C, j, nl, nu);
    if (P.instcut != nullptr) {
      int* flag = &P.instcut[P.colinst[j]];
      if (c) atomicExch(flag, 1);
      if (c || *flag) continue;
    } else if (c) {
      cut = true;
      continue;
    }
    bool lbup = nl > l, ubdown = nu < u;
    if (lbup || ubdown) {
      // the sparse call's record of a column's first move: its bounds before the call's propagation
      if (M.stamp != nullptr && atomicExch(&M.stamp[j], M.epoch) != M.epoch) {
        const int k = atomicAdd(M.count, 1);
        M.col[k] = j;
        M.lb[k] = l;
        M.ub[k] = u;
      }
      lb[j] = nl;
      ub[j] = nu;
      changes += (unsigned long long)lbup + (unsigned long long)ubdown;
      logChange(G, j, round, nl, nu);
      expandColumn(P, F, j, lbup, ubdown, stamp);
    }
  }
  if (cut) atomicExch(cutoff, 1);
  if (changes) atomicAdd(&stats[3], changes);
}

// ---- host-driven round (the host reads the frontier sizes after each round)
__global__ void __launch_bounds__(ROW_THREADS) k_rows_short(Num s, Prob P, PlainBnd B, const int* list,
                                                           const int* nshort, Cands C, int* cutoff,
                                                           unsigned long long* stats) {
  __shared__ RowBatch<ROW_THREADS> rb;
  __shared__ int s_cut;
  rowsShortBody(s, P, B, list, *nshort, C, cutoff, stats, rb, &s_cut);
}

// two CTAs per SM (at most 128 registers a thread): one warp walks a long row with a dependent chain per lane, so
// the SM needs the second CTA's warps to hide it (cfg1's Zipf root: 146.5 -> 116.3 ms)
__global__ void __launch_bounds__(256, 2) k_rows_long(Num s, Prob P, PlainBnd B, const int* list, const int* nlong,
                                                   int cap, Cands C, int* cutoff, unsigned long long* stats) {
  rowsLongBody(s, P, B, list, *nlong, cap, C, cutoff, stats);
}

__global__ void __launch_bounds__(256) k_apply(Num s, Prob P, double* lb, double* ub, Cands C, Front F, int stamp,
                                               int* cutoff, unsigned long long* stats, ChangeLog G, int round) {
  applyBody(s, P, lb, ub, C, F, stamp, cutoff, stats, G, round);
}

// ---- graph-driven rounds: the frontier sizes, list parity, stamps and bound pointers live in LoopState
__global__ void __launch_bounds__(ROW_THREADS) k_rows_short_g(Num s, Prob P, Cands C, ListSet L, LoopState* S,
                                                             unsigned long long* stats) {
  __shared__ RowBatch<ROW_THREADS> rb;
  __shared__ int s_cut;
  const int cur = S->cur;
  C.round = S->round;
  rowsShortBody(s, P, PlainBnd{S->lb, S->ub}, L.list[cur], S->nshort[cur], C, &S->cutoff, stats, rb, &s_cut);
}

__global__ void __launch_bounds__(256, 2) k_rows_long_g(Num s, Prob P, Cands C, ListSet L, LoopState* S,
                                                     unsigned long long* stats) {
  const int cur = S->cur;
  C.round = S->round;
  rowsLongBody(s, P, PlainBnd{S->lb, S->ub}, L.list[cur], S->nlong[cur], L.cap, C, &S->cutoff, stats);
}

__global__ void __launch_bounds__(256) k_apply_g(Num s, Prob P, Cands C, ListSet L, LoopState* S,
                                                 unsigned long long* stats) {
  const int nxt = S->cur == 1 ? 0 : 1;
  Front F{L.list[nxt], &S->nshort[nxt], &S->nlong[nxt], L.rowstamp, L.cap};
  applyBody(s, P, S->lb, S->ub, C, F, S->stamp, &S->cutoff, stats, S->log, S->round);
}

// end of a round: switch to the list just filled, clear the other one; returns whether another round follows
__device__ __forceinline__ int advanceRound(LoopState* S) {
  const int ran = S->nshort[S->cur] + S->nlong[S->cur];
  if (ran > 0) S->worked += 1;
  S->round += 1;
  const int nxt = S->cur == 1 ? 0 : 1;
  S->cur = nxt;
  const int other = nxt ^ 1;
  S->nshort[other] = 0;
  S->nlong[other] = 0;
  S->ntouched = 0;
  S->stamp += 1;
  int more = (S->nshort[nxt] + S->nlong[nxt] > 0) && !S->cutoff;
  if (more && S->worked >= S->maxrounds) {
    S->status = 2;
    more = 0;
  }
  return more;
}
__global__ void k_advance_g(LoopState* S, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, advanceRound(S) ? 1u : 0u);
}

// ---- all rounds in one cooperative launch: the graph's round body, with grid-wide barriers (cooperative groups,
// the launch guarantees every block is resident) between its phases instead of kernel boundaries.  For seeded
// calls, whose frontiers are small, the launch and per-kernel costs of the graph dominate.
__global__ void __launch_bounds__(ROW_THREADS) k_plain_coop(Num s, Prob P, Cands C, ListSet L, LoopState* S,
                                                           unsigned long long* stats) {
  __shared__ RowBatch<ROW_THREADS> rb;
  __shared__ int s_cut;
  cg::grid_group grid = cg::this_grid();
  volatile LoopState* V = S;
  for (;;) {
    const int cur = V->cur;
    C.round = V->round;
    const PlainBnd B{S->lb, S->ub};
    rowsShortBody(s, P, B, L.list[cur], V->nshort[cur], C, &S->cutoff, stats, rb, &s_cut);
    rowsLongBody(s, P, B, L.list[cur], V->nlong[cur], L.cap, C, &S->cutoff, stats);
    grid.sync();
    const int nxt = cur == 1 ? 0 : 1;
    Front F{L.list[nxt], &S->nshort[nxt], &S->nlong[nxt], L.rowstamp, L.cap};
    applyBody(s, P, S->lb, S->ub, C, F, V->stamp, &S->cutoff, stats, S->log, V->round);
    grid.sync();
    if (blockIdx.x == 0 && threadIdx.x == 0) S->more = advanceRound(S);
    grid.sync();
    if (!V->more) break;
  }
}

__global__ void k_seed(Prob P, const double* lb, const double* ub, int64_t nseed, const int32_t* cols,
                       const double* oldlb, const double* oldub, Front F, int stamp) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nseed; k += (int64_t)gridDim.x * blockDim.x) {
    int j = cols[k];
    expandColumn(P, F, j, lb[j] > oldlb[k], ub[j] < oldub[k], stamp);
  }
}

__global__ void __launch_bounds__(256) k_activities(Num s, Prob P, PlainBnd B, double* act, int32_t* cnt) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  // warp per 32 rows for short rows (one lane each), warp per row for long rows -- the summation orders
  // of the short-row scan and of rowWarp
  for (int64_t base = (int64_t)warp * 32; base < P.m; base += (int64_t)nwarps * 32) {
    int64_t i = base + lane;
    bool mine = i < P.m && (P.rowptr[i + 1] - P.rowptr[i]) <= LONGROW;
    Act a;
    actZero(a);
    if (mine) {
      // two halves in row order, the second merged into the first (the order of the row scan)
      const int64_t p0 = P.rowptr[i], p1 = P.rowptr[i + 1], ph = p0 + (p1 - p0 + 1) / 2;
      Act second;
      actZero(second);
      for (int64_t p = p0; p < p1; ++p) {
        int j = P.colidx[p];
        double l, u;
        B.get(j, l, u);
        addTerm(s, p < ph ? a : second, P.vals[p], l, u);
      }
      actMerge(a, second);
    }
    unsigned longmask = __ballot_sync(0xffffffffu, i < P.m && !mine);
    while (longmask) {
      int src = __ffs(longmask) - 1;
      longmask &= longmask - 1;
      int64_t r = base + src;
      Act b;
      actZero(b);
      for (int64_t p = P.rowptr[r] + lane; p < P.rowptr[r + 1]; p += 32) {
        int j = P.colidx[p];
        double l, u;
        B.get(j, l, u);
        addTerm(s, b, P.vals[p], l, u);
      }
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) {
        Act c;
        c.minhi = __shfl_down_sync(0xffffffffu, b.minhi, off);
        c.minlo = __shfl_down_sync(0xffffffffu, b.minlo, off);
        c.maxhi = __shfl_down_sync(0xffffffffu, b.maxhi, off);
        c.maxlo = __shfl_down_sync(0xffffffffu, b.maxlo, off);
        c.minposinf = __shfl_down_sync(0xffffffffu, b.minposinf, off);
        c.minneginf = __shfl_down_sync(0xffffffffu, b.minneginf, off);
        c.minposhuge = __shfl_down_sync(0xffffffffu, b.minposhuge, off);
        c.minneghuge = __shfl_down_sync(0xffffffffu, b.minneghuge, off);
        c.maxposinf = __shfl_down_sync(0xffffffffu, b.maxposinf, off);
        c.maxneginf = __shfl_down_sync(0xffffffffu, b.maxneginf, off);
        c.maxposhuge = __shfl_down_sync(0xffffffffu, b.maxposhuge, off);
        c.maxneghuge = __shfl_down_sync(0xffffffffu, b.maxneghuge, off);
        if (lane < off) actMerge(b, c);
      }
      if (lane == 0) {
        act[4 * r + 0] = b.minhi; act[4 * r + 1] = b.minlo; act[4 * r + 2] = b.maxhi; act[4 * r + 3] = b.maxlo;
        cnt[8 * r + 0] = b.minposinf; cnt[8 * r + 1] = b.minneginf; cnt[8 * r + 2] = b.minposhuge;
        cnt[8 * r + 3] = b.minneghuge; cnt[8 * r + 4] = b.maxposinf; cnt[8 * r + 5] = b.maxneginf;
        cnt[8 * r + 6] = b.maxposhuge; cnt[8 * r + 7] = b.maxneghuge;
      }
    }
    if (mine) {
      act[4 * i + 0] = a.minhi; act[4 * i + 1] = a.minlo; act[4 * i + 2] = a.maxhi; act[4 * i + 3] = a.maxlo;
      cnt[8 * i + 0] = a.minposinf; cnt[8 * i + 1] = a.minneginf; cnt[8 * i + 2] = a.minposhuge;
      cnt[8 * i + 3] = a.minneghuge; cnt[8 * i + 4] = a.maxposinf; cnt[8 * i + 5] = a.maxneginf;
      cnt[8 * i + 6] = a.maxposhuge; cnt[8 * i + 7] = a.maxneghuge;
    }
  }
}

__global__ void k_pack(const double* lb, const double* ub, double2* out, int64_t n) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    out[j] = make_double2(lb[j], ub[j]);
}

// the sparse plain call (gbp_propagate_changes): column cols[k] takes bounds [nlb[k], nub[k]]; its previous
// bounds become the call's seeds
// (keepold: the seeds' old bounds are already in oldlb/oldub)
__global__ void k_set_changes(int64_t nchg, const int32_t* cols, const double* nlb, const double* nub, double* lb,
                              double* ub, double* oldlb, double* oldub, int keepold) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nchg; k += (int64_t)gridDim.x * blockDim.x) {
    const int j = cols[k];
    if (!keepold) {
      oldlb[k] = lb[j];
      oldub[k] = ub[j];
    }
    lb[j] = nlb[k];
    ub[j] = nub[k];
  }
}

// columns whose bounds differ from the snapshot, appended in no particular order while they fit cap; count
// reaches the number of such columns
__global__ void k_moved(int64_t n, const double* lb, const double* ub, const double* slb, const double* sub,
                        unsigned long long* count, int64_t cap, int32_t* cols, double* olb, double* oub) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const double l = lb[j], u = ub[j];
    if (l != slb[j] || u != sub[j]) {
      const unsigned long long pos = atomicAdd(count, 1ull);
      if ((int64_t)pos < cap) {
        cols[pos] = (int32_t)j;
        olb[pos] = l;
        oub[pos] = u;
      }
    }
  }
}

__global__ void k_flags8(const int* in, int8_t* out, int64_t n) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    out[j] = in[j] != 0 ? 1 : 0;
}

__global__ void k_fill64(long long* p, int64_t n, long long v) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    p[j] = v;
}

// column-major copy built on the device: count entries per column, then scatter each row's entries to its
// columns' next free slots (the order inside a column does not matter to any result)
__global__ void k_csc_count(int64_t nnz, const int32_t* colidx, int64_t n, unsigned long long* count, int* bad) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
    const int j = colidx[p];
    if (j < 0 || j >= n) {
      atomicExch(bad, 1);
      continue;
    }
    atomicAdd(&count[j], 1ull);
  }
}

__global__ void k_csc_scatter(int64_t m, const int64_t* rowptr, const int32_t* colidx, const double* vals,
                              const double* lhs, const double* rhs, double inf, unsigned long long* cursor,
                              uint32_t* cscrow) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const bool rhsfin = !(rhs[i] >= inf), lhsfin = !(-lhs[i] >= inf);
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p) {
      const double a = vals[p];
      uint32_t e = (uint32_t)i;
      if (a > 0.0 ? rhsfin : lhsfin) e |= CSC_LBUP;
      if (a > 0.0 ? lhsfin : rhsfin) e |= CSC_UBDOWN;
      const unsigned long long q = atomicAdd(&cursor[colidx[p]], 1ull);
      cscrow[q] = e;
    }
  }
}

// Instances uploaded part by part (gbp_upload_instance_list): each part's row pointers and column indices are
// local to the part; shift them by the part's offsets, record each row's and column's instance, and flag column
// indices outside their part.  off = [row_off | col_off | nnz_off], each ninst + 1 entries.
__device__ __forceinline__ int64_t partOf(const int64_t* o, int64_t ninst, int64_t x) {
  int64_t lo = 0, hi = ninst - 1;  // last k with o[k] <= x
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (o[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
__global__ void k_fix_parts(int64_t ninst, const int64_t* off, int64_t m, int64_t n, int64_t nnz, int64_t* rowptr,
                            int32_t* colidx, int32_t* rowinst, int32_t* colinst, int* bad) {
  const int64_t* row_off = off;
  const int64_t* col_off = off + ninst + 1;
  const int64_t* nnz_off = off + 2 * (ninst + 1);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) {
    const int64_t k = partOf(row_off, ninst, i);
    rowptr[i] += nnz_off[k];
    rowinst[i] = (int32_t)k;
  }
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += stride)
    colinst[j] = (int32_t)partOf(col_off, ninst, j);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += stride) {
    const int64_t k = partOf(nnz_off, ninst, p);
    const int64_t c = colidx[p];
    if (c < 0 || c >= col_off[k + 1] - col_off[k]) {
      atomicExch(bad, 1);
      colidx[p] = 0;
    } else {
      colidx[p] = (int32_t)(c + col_off[k]);
    }
  }
}

// Ranged rows: the rows the gcd rule can act on -- three or more entries, both sides finite, and an integral
// column with an integral coefficient other than +-1 (rangedRowPropagation returns at once for any other row,
// cons_linear.c:5770-5777, :5839-5869) -- flagged and compacted into list (any order), with the classification of
// their entries (coef, see Prob::rcoef).
__global__ void k_ranged_elig(Num s, Prob P, uint8_t* elig, int* list, int* count, long long* coef) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.m; i += stride) {
    const int64_t p0 = P.rowptr[i], p1 = P.rowptr[i + 1];
    bool ok = false;
    if (p1 - p0 >= 3 && !isNegInf(s, P.lhs[i]) && !isInf(s, P.rhs[i])) {
      for (int64_t p = p0; p < p1; ++p) {
        const long long c = rangedCoef(s, P.isint[P.colidx[p]] != 0, P.vals[p]);
        coef[p] = c;
        ok = ok || c >= 0;
      }
    }
    elig[i] = ok ? 1 : 0;
    if (ok) list[atomicAdd(count, 1)] = (int)i;
  }
}

// the domain the rows' order was last computed on (saved) against this call's: *changed becomes nonzero if any
// column differs, and saved takes the new values
__global__ void k_ranged_domain(const double* dl, const double* du, double2* saved, int64_t n, int* changed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool diff = false;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += stride) {
    const double2 o = saved[j];
    const double l = dl[j], u = du[j];
    if (__double_as_longlong(o.x) != __double_as_longlong(l) || __double_as_longlong(o.y) != __double_as_longlong(u)) {
      diff = true;
      saved[j] = make_double2(l, u);
    }
  }
  if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(changed, 1);
}

// the entry order of the listed rows on a global domain fixed for the call (one thread per row), when that domain
// changed since the order was last computed
__global__ void k_ranged_order(Prob P, const int* list, int n, const double* dl, const double* du, int sorted,
                               const int* changed) {
  if (*changed == 0) return;
  auto dom = [&](int j, double& l, double& u) {
    l = dl[j];
    u = du[j];
  };
  const int stride = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) rowOrder(P, dom, sorted != 0, list[t]);
}

// rows of instance k may only reference columns of instance k
__global__ void k_check_blocks(int64_t m, const int64_t* rowptr, const int32_t* colidx, const int32_t* rowinst,
                               const int32_t* colinst, int* bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p)
      if (colinst[colidx[p]] != rowinst[i]) atomicExch(bad, 1);
}

// relevance flags of each CSC entry (which bound moves of the column the row can use)
__global__ void k_csc_flags(int64_t nnz, const double* cvals, const int32_t* rowidx, const double* lhs,
                            const double* rhs, double inf, uint32_t* out) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
    int i = rowidx[q];
    double a = cvals[q];
    bool rhsfin = !(rhs[i] >= inf);
    bool lhsfin = !(-lhs[i] >= inf);
    uint32_t e = (uint32_t)i;
    if (a > 0.0 ? rhsfin : lhsfin) e |= CSC_LBUP;
    if (a > 0.0 ? lhsfin : rhsfin) e |= CSC_UBDOWN;
    out[q] = e;
  }
}

// ------------------------------------------------------------------------------------------ node order
__device__ __forceinline__ int orderBucket(const int64_t* ptr, int64_t k) {
  const int64_t c = ptr[k + 1] - ptr[k];
  return ORDER_BUCKETS - 1 - (int)(c < ORDER_BUCKETS - 1 ? c : ORDER_BUCKETS - 1);  // bucket 0: most changes
}
__global__ void __launch_bounds__(256) k_order_hist(int64_t nnodes, const int64_t* ptr, int* hist) {
  __shared__ int h[ORDER_BUCKETS];
  for (int b = threadIdx.x; b < ORDER_BUCKETS; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnodes; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[orderBucket(ptr, k)], 1);
  __syncthreads();
  for (int b = threadIdx.x; b < ORDER_BUCKETS; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}
__global__ void __launch_bounds__(256) k_order_scatter(int64_t nnodes, const int64_t* ptr, const int* hist,
                                                       int* cursor, int* order) {
  __shared__ int start[ORDER_BUCKETS];
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < ORDER_BUCKETS; ++b) {
      start[b] = acc;
      acc += hist[b];
    }
  }
  __syncthreads();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnodes; k += (int64_t)gridDim.x * blockDim.x) {
    const int b = orderBucket(ptr, k);
    order[start[b] + atomicAdd(&cursor[b], 1)] = (int)k;
  }
}

// ------------------------------------------------------------------------------------------ launchers
cudaError_t launchRangedElig(cudaStream_t st, int grid, const Num& s, const Prob& P, uint8_t* elig, int* list,
                             int* count, long long* coef) {
  k_ranged_elig<<<grid, 256, 0, st>>>(s, P, elig, list, count, coef);
  return cudaGetLastError();
}
cudaError_t launchRangedOrder(cudaStream_t st, int grid, const Prob& P, const int* list, int n, const double* dl,
                              const double* du, int sorted, double2* saved, int* changed, int dgrid) {
  if (n <= 0) return cudaSuccess;
  k_ranged_domain<<<dgrid, 256, 0, st>>>(dl, du, saved, P.n, changed);
  k_ranged_order<<<grid, 128, 0, st>>>(P, list, n, dl, du, sorted, changed);
  return cudaGetLastError();
}
cudaError_t launchFixParts(cudaStream_t st, int grid, int64_t ninst, const int64_t* off, int64_t m, int64_t n,
                           int64_t nnz, int64_t* rowptr, int32_t* colidx, int32_t* rowinst, int32_t* colinst, int* bad) {
  k_fix_parts<<<grid, 256, 0, st>>>(ninst, off, m, n, nnz, rowptr, colidx, rowinst, colinst, bad);
  return cudaGetLastError();
}
cudaError_t launchNodeOrder(cudaStream_t st, int grid, int64_t nnodes, const int64_t* ptr, int* hist, int* order) {
  k_order_hist<<<grid, 256, 0, st>>>(nnodes, ptr, hist);
  k_order_scatter<<<grid, 256, 0, st>>>(nnodes, ptr, hist, hist + ORDER_BUCKETS, order);
  return cudaGetLastError();
}
cudaError_t launchRowsShort(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                            const double* ub, const int* list, const int* nshort, Cands C, int* cutoff,
                            unsigned long long* stats) {
  k_rows_short<<<grid, ROW_THREADS, 0, st>>>(s, P, PlainBnd{lb, ub}, list, nshort, C, cutoff, stats);
  return cudaGetLastError();
}
cudaError_t launchRowsLong(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                           const double* ub, const int* list, const int* nlong, int cap, Cands C, int* cutoff,
                           unsigned long long* stats) {
  k_rows_long<<<grid, 256, 0, st>>>(s, P, PlainBnd{lb, ub}, list, nlong, cap, C, cutoff, stats);
  return cudaGetLastError();
}
cudaError_t launchApply(cudaStream_t st, int grid, const Num& s, const Prob& P, double* lb, double* ub, Cands C,
                        Front F, int stamp, int* cutoff, unsigned long long* stats, const ChangeLog& G, int round) {
  k_apply<<<grid, 256, 0, st>>>(s, P, lb, ub, C, F, stamp, cutoff, stats, G, round);
  return cudaGetLastError();
}
// ---- gbp_propagate_changes in one cooperative launch: the caller's changes, the seeds, every round, and the moved
// columns (restored when the call ends in a cutoff or overflows the caller's capacity), so that the call costs one
// copy in, one launch and one copy out
__global__ void __launch_bounds__(ROW_THREADS) k_sparse_coop(const __grid_constant__ SparseArgs A) {
  __shared__ RowBatch<ROW_THREADS> rb;
  __shared__ int s_cut;
  cg::grid_group grid = cg::this_grid();
  LoopState* S = A.S;
  volatile LoopState* V = S;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  if (tid == 0) {
    *S = A.init;
    for (int k = 0; k < 8; ++k) A.stats[k] = 0;
    *A.moved.count = 0;
    if (A.init.log.n != nullptr) *A.init.log.n = 0;
    if (A.C.rlog.n != nullptr) *A.C.rlog.n = 0;
  }
  // the caller's changes, with the bounds they replace (or the caller's seed bounds)
  for (int64_t k = tid; k < A.nchg; k += nth) {
    const int j = A.cols[k];
    if (!A.keepold) {
      A.oldlb[k] = A.lb[j];
      A.oldub[k] = A.ub[j];
    }
    A.lb[j] = A.nlb[k];
    A.ub[j] = A.nub[k];
  }
  grid.sync();
  {
    Front F0{A.L.list[0], &S->nshort[0], &S->nlong[0], A.L.rowstamp, A.L.cap};
    for (int64_t k = tid; k < A.nchg; k += nth) {
      const int j = A.cols[k];
      expandColumn(A.P, F0, j, A.lb[j] > A.oldlb[k], A.ub[j] < A.oldub[k], A.seedstamp);
    }
  }
  grid.sync();
  Cands C = A.C;
  const bool any = A.nchg > 0;
  while (any) {
    const int cur = V->cur;
    C.round = V->round;
    const PlainBnd B{A.lb, A.ub};
    rowsShortBody(A.s, A.P, B, A.L.list[cur], V->nshort[cur], C, &S->cutoff, A.stats, rb, &s_cut);
    rowsLongBody(A.s, A.P, B, A.L.list[cur], V->nlong[cur], A.L.cap, C, &S->cutoff, A.stats);
    grid.sync();
    const int nxt = cur == 1 ? 0 : 1;
    Front F{A.L.list[nxt], &S->nshort[nxt], &S->nlong[nxt], A.L.rowstamp, A.L.cap};
    applyBody(A.s, A.P, A.lb, A.ub, C, F, V->stamp, &S->cutoff, A.stats, A.init.log, V->round, A.moved);
    grid.sync();
    if (tid == 0) S->more = advanceRound(S);
    grid.sync();
    if (!V->more) break;
  }
  // a cutoff, or more moved columns than the caller has room for: back to the bounds after the caller's changes
  const int cnt = *(volatile int*)A.moved.count;
  const bool back = V->cutoff || cnt > A.cap;
  for (int64_t k = tid; k < cnt; k += nth) {
    const int j = A.moved.col[k];
    if (back) {
      A.lb[j] = A.moved.lb[k];
      A.ub[j] = A.moved.ub[k];
    } else {
      SparseOut o;
      o.col = j;
      o.pad = 0;
      o.lb = A.lb[j];
      o.ub = A.ub[j];
      A.out[k] = o;
    }
  }
  if (tid == 0) {
    A.header[0] = V->cutoff;
    A.header[1] = V->status;
    A.header[2] = V->worked;
    A.header[3] = V->stamp;
    A.header[4] = cnt;
    unsigned long long* hs = (unsigned long long*)(A.header + 8);
    for (int k = 0; k < 8; ++k) hs[k] = ((volatile unsigned long long*)A.stats)[k];
  }
}
cudaError_t launchSparseCoop(cudaStream_t st, int grid, const SparseArgs& A) {
  SparseArgs a = A;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_sparse_coop, dim3(grid), dim3(ROW_THREADS), args, 0, st);
}
cudaError_t sparseCoopOccupancy(int* blocksPerSm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, k_sparse_coop, ROW_THREADS, 0);
}

cudaError_t launchPlainCoop(cudaStream_t st, int grid, const Num& s, const Prob& P, const Cands& C, const ListSet& L,
                            LoopState* S, unsigned long long* stats) {
  Num a0 = s;
  Prob a1 = P;
  Cands a2 = C;
  ListSet a3 = L;
  LoopState* a4 = S;
  unsigned long long* a5 = stats;
  void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5};
  return cudaLaunchCooperativeKernel((const void*)k_plain_coop, dim3(grid), dim3(ROW_THREADS), args, 0, st);
}
cudaError_t plainCoopOccupancy(int* blocksPerSm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, k_plain_coop, ROW_THREADS, 0);
}
const void* graphKernel(int which) {
  switch (which) {
    case 0: return (const void*)k_rows_short_g;
    case 1: return (const void*)k_rows_long_g;
    case 2: return (const void*)k_apply_g;
    case 3: return (const void*)k_advance_g;
    default: return nullptr;
  }
}
cudaError_t launchSeed(cudaStream_t st, int grid, const Prob& P, const double* lb, const double* ub, int64_t nseed,
                       const int32_t* cols, const double* oldlb, const double* oldub, Front F, int stamp) {
  k_seed<<<grid, 256, 0, st>>>(P, lb, ub, nseed, cols, oldlb, oldub, F, stamp);
  return cudaGetLastError();
}
cudaError_t launchActivities(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                             const double* ub, double* act, int32_t* cnt) {
  k_activities<<<grid, 256, 0, st>>>(s, P, PlainBnd{lb, ub}, act, cnt);
  return cudaGetLastError();
}
cudaError_t launchSetChanges(cudaStream_t st, int grid, int64_t nchg, const int32_t* cols, const double* nlb,
                             const double* nub, double* lb, double* ub, double* oldlb, double* oldub, int keepold) {
  k_set_changes<<<grid, 256, 0, st>>>(nchg, cols, nlb, nub, lb, ub, oldlb, oldub, keepold);
  return cudaGetLastError();
}
cudaError_t launchMoved(cudaStream_t st, int grid, int64_t n, const double* lb, const double* ub, const double* slb,
                        const double* sub, unsigned long long* count, int64_t cap, int32_t* cols, double* olb,
                        double* oub) {
  k_moved<<<grid, 256, 0, st>>>(n, lb, ub, slb, sub, count, cap, cols, olb, oub);
  return cudaGetLastError();
}
cudaError_t launchPack(cudaStream_t st, int grid, const double* lb, const double* ub, double2* out, int64_t n) {
  k_pack<<<grid, 256, 0, st>>>(lb, ub, out, n);
  return cudaGetLastError();
}
cudaError_t launchCscCount(cudaStream_t st, int grid, int64_t nnz, const int32_t* colidx, int64_t n,
                           unsigned long long* count, int* bad) {
  k_csc_count<<<grid, 256, 0, st>>>(nnz, colidx, n, count, bad);
  return cudaGetLastError();
}
cudaError_t launchCscScatter(cudaStream_t st, int grid, int64_t m, const int64_t* rowptr, const int32_t* colidx,
                             const double* vals, const double* lhs, const double* rhs, double inf,
                             unsigned long long* cursor, uint32_t* cscrow) {
  k_csc_scatter<<<grid, 256, 0, st>>>(m, rowptr, colidx, vals, lhs, rhs, inf, cursor, cscrow);
  return cudaGetLastError();
}
cudaError_t launchCheckBlocks(cudaStream_t st, int grid, int64_t m, const int64_t* rowptr, const int32_t* colidx,
                              const int32_t* rowinst, const int32_t* colinst, int* bad) {
  k_check_blocks<<<grid, 256, 0, st>>>(m, rowptr, colidx, rowinst, colinst, bad);
  return cudaGetLastError();
}
cudaError_t launchFlags8(cudaStream_t st, int grid, const int* in, int8_t* out, int64_t n) {
  k_flags8<<<grid, 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}
cudaError_t launchFill64(cudaStream_t st, int grid, long long* p, int64_t n, long long v) {
  k_fill64<<<grid, 256, 0, st>>>(p, n, v);
  return cudaGetLastError();
}
cudaError_t launchCscFlags(cudaStream_t st, int grid, int64_t nnz, const double* cvals, const int32_t* rowidx,
                           const double* lhs, const double* rhs, double inf, uint32_t* out) {
  k_csc_flags<<<grid, 256, 0, st>>>(nnz, cvals, rowidx, lhs, rhs, inf, out);
  return cudaGetLastError();
}
cudaError_t launchNodes(cudaStream_t st, int grid, int nt, const NodesArgs& A) {
  if (A.P.relig != nullptr) return launchNodesRanged(st, grid, nt, A);
  return launchNodesT<false>(st, grid, nt, A);
}
// the slots are sized for the smaller residency of the two variants
cudaError_t nodesOccupancy(int nt, int minb, int* blocksPerSm) {
  int a = 0, b = 0;
  cudaError_t e = nodesOccupancyT<false>(nt, minb, &a);
  if (e != cudaSuccess) return e;
  e = nodesOccupancyRanged(nt, minb, &b);
  if (e != cudaSuccess) return e;
  *blocksPerSm = a < b ? a : b;
  return cudaSuccess;
}
}  // namespace gbp

// exclusive prefix sum of the per-column counts (n + 1 entries, count[n] = 0): the CSC column pointers
#include <cub/device/device_scan.cuh>
namespace gbp {
cudaError_t columnPointers(cudaStream_t st, const unsigned long long* count, unsigned long long* colptr, int64_t n) {
  size_t tmp = 0;
  cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, tmp, count, colptr, n + 1, st);
  if (e != cudaSuccess) return e;
  void* buf = nullptr;
  e = cudaMallocAsync(&buf, tmp, st);
  if (e != cudaSuccess) return e;
  e = cub::DeviceScan::ExclusiveSum(buf, tmp, count, colptr, n + 1, st);
  cudaError_t f = cudaFreeAsync(buf, st);
  return e != cudaSuccess ? e : f;
}
}  // namespace gbp
