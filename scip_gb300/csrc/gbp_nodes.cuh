// The batched node kernel (k_nodes) and the bound accessor it reads through, shared by the translation units
// that instantiate it: gbp_kernels.cu without ranged rows, gbp_nodes_ranged.cu with them (GBP_FLAG_RANGEDROW),
// so that the common configuration runs code that carries nothing of that rule.
#pragma once

#include "gbp_internal.h"

namespace gbp {

// A node's changed columns are also kept in a small open-addressing table in shared memory, so that the
// bound lookup of every row entry costs a shared-memory probe plus a read of the (L2-resident) base bounds
// instead of a read of the per-CTA global stamp array.  A node that changes more than OVL_HASH_MAX columns
// switches to the global overlay, which is always maintained.
constexpr int OVL_HASH = 512;
constexpr int OVL_HASH_MAX = OVL_HASH / 2;
__device__ __forceinline__ unsigned ovlSlot(int j) { return ((unsigned)j * 2654435761u) >> (32 - 9); }
static_assert((1 << 9) == OVL_HASH, "ovlSlot hashes to 9 bits");

// node bounds: the per-CTA overlay where this node changed a column, else the shared base (packed pairs,
// or two separate arrays when `base` is null)
struct OvlBnd {
  const double2* base;
  const double* baselb;
  const double* baseub;
  double2* ovl;
  int* ostamp;
  int epoch;
  int* hkey;      // shared table: column or -1
  double2* hval;  // its bounds
  int* hstate;    // [0] entries, [1] nonzero once the node uses the global overlay only
  __device__ __forceinline__ double2 getBase(int j) const {
    return base != nullptr ? base[j] : make_double2(baselb[j], baseub[j]);
  }
  __device__ __forceinline__ void get(int j, double& l, double& u) const {
    double2 b;
    bool found = false;
    if (hstate[1] == 0) {
      unsigned h = ovlSlot(j);
      for (int t = 0; t < OVL_HASH; ++t) {
        const int k = hkey[h];
        if (k == j) {
          b = hval[h];
          found = true;
          break;
        }
        if (k < 0) {
          b = getBase(j);
          found = true;
          break;
        }
        h = (h + 1) & (OVL_HASH - 1);
      }
    }
    if (!found) b = (ostamp[j] == epoch) ? ovl[j] : getBase(j);
    l = b.x;
    u = b.y;
  }
  // global domain of every node of the batch: the base bounds
  __device__ __forceinline__ void glob(const Prob&, int j, double& l, double& u) const {
    double2 b = getBase(j);
    l = b.x;
    u = b.y;
  }
};

__device__ __forceinline__ void flushStats(unsigned long long* stats, const Stats& st) {
  if (st.rows) atomicAdd(&stats[0], (unsigned long long)st.rows);
  if (st.nnz) atomicAdd(&stats[1], (unsigned long long)st.nnz);
  if (st.cands) atomicAdd(&stats[2], (unsigned long long)st.cands);
  if (st.live) atomicAdd(&stats[6], (unsigned long long)st.live);
}

// ------------------------------------------------------------------------------------------ batched path
// Column j of the node gets bounds [l,u].  Only the thread that owns j in the current phase reads or writes
// j's entry, so the table needs atomics only to claim free slots.
__device__ __forceinline__ void ovlSet(const OvlBnd& B, int* dirty, int* ndirty, int j, double l, double u) {
  if (B.ostamp[j] != B.epoch) {
    B.ostamp[j] = B.epoch;
    dirty[atomicAdd(ndirty, 1)] = j;
  }
  B.ovl[j] = make_double2(l, u);
  if (B.hstate[1] != 0) return;
  unsigned h = ovlSlot(j);
  for (int t = 0; t < OVL_HASH; ++t) {
    const int k = atomicCAS(&B.hkey[h], -1, j);
    if (k == -1 || k == j) {
      B.hval[h] = make_double2(l, u);
      if (k == -1 && atomicAdd(&B.hstate[0], 1) + 1 > OVL_HASH_MAX) atomicExch(&B.hstate[1], 1);
      return;
    }
    h = (h + 1) & (OVL_HASH - 1);
  }
  atomicExch(&B.hstate[1], 1);
}

// RANGED: rows run the ranged-row rule when the problem carries it (P.relig); false compiles it out
template <int NT, int MINB, bool RANGED>
__global__ void __launch_bounds__(NT, MINB) k_nodes(NodesArgs A) {
  __shared__ RowBatch<NT> rb;
  __shared__ int s_item, s_cut, s_ns[2], s_nl[2], s_ntouched, s_ndirty, s_nout, s_rounds, s_epoch, s_rstamp;
  __shared__ long long s_off;
  __shared__ unsigned long long s_changes;
  __shared__ int s_hkey[OVL_HASH];
  __shared__ double2 s_hval[OVL_HASH];
  __shared__ int s_hstate[2];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  constexpr int NW = NT / 32;
  const SlotArrays& S = A.S;
  const int64_t ns = S.nstride, ms = S.mstride;
  const size_t slot = blockIdx.x;
  double2* ovl = S.ovl + slot * ns;
  int* ostamp = S.ostamp + slot * ns;
  int* touched = S.touched + slot * ns;
  int* dirty = S.dirty + slot * ns;
  int* lists[2] = {S.listA + slot * ms, S.listB + slot * ms};
  int* rowstamp = S.rowstamp + slot * ms;
  Cands C;
  C.cub = S.cub + slot * ns;
  C.clb = S.clb + slot * ns;
  C.cubf = S.cubf + slot * ns;
  C.clbf = S.clbf + slot * ns;
  C.cflag = S.cflag + slot * ns;
  C.touched = touched;
  C.ntouched = &s_ntouched;
  C.rlog = RangedLog{nullptr, 0, nullptr, nullptr, nullptr};
  C.round = 0;
  const int m = (int)A.P.m;

  if (A.abort_flag != nullptr && (*A.abort_flag & 8)) {
    // the caller's arrays failed the input checks: no node runs, each reports that its result was not written
    for (int64_t k = (int64_t)blockIdx.x * NT + tid; k < A.nnodes; k += (int64_t)gridDim.x * NT) {
      A.out_n[k] = -1;
      A.out_off[k] = 0;
      A.out_cutoff[k] = 0;
      A.out_rounds[k] = 0;
    }
    return;
  }
  int counter = 0;
  if (tid == 0) counter = S.counter[slot];
  Stats st{0, 0, 0, 0};
  unsigned long long mycut = 0, mymaxr = 0;

  for (;;) {
    for (int t = tid; t < OVL_HASH; t += NT) s_hkey[t] = -1;
    if (tid == 0) {
      s_hstate[0] = 0;
      s_hstate[1] = 0;
      const int q = atomicAdd(A.next_item, 1);
      s_item = (q < A.nnodes && A.order != nullptr) ? A.order[q] : q;
      s_epoch = ++counter;
      s_cut = 0;
      s_ns[0] = s_nl[0] = s_ns[1] = s_nl[1] = 0;
      s_ndirty = 0;
      s_nout = 0;
      s_rounds = 0;
      s_changes = 0;
    }
    __syncthreads();
    const int item = s_item;
    if (item >= A.nnodes) break;
    OvlBnd B{A.base, A.baselb, A.baseub, ovl, ostamp, s_epoch, s_hkey, s_hval, s_hstate};

    // branching bound changes of the node, then the rows they make relevant
    {
      Front F{lists[0], &s_ns[0], &s_nl[0], rowstamp, m};
      for (int64_t q = A.ptr[item] + tid; q < A.ptr[item + 1]; q += NT) {
        int j = A.chg_col[q];
        if (j < 0 || j >= (int)A.P.n) {  // not a column: the call fails, the node is given up
          atomicOr(A.status, 4);
          s_cut = 1;
          continue;
        }
        // a column named more than once: its first occurrence applies them all (the tightest bounds), which is
        // what applying them one after the other gives
        const int64_t q0 = A.ptr[item], q1 = A.ptr[item + 1];
        bool first = true;
        for (int64_t r2 = q0; r2 < q && first; ++r2) first = A.chg_col[r2] != j;
        if (!first) continue;
        double nl = A.chg_lb[q], nu = A.chg_ub[q];
        for (int64_t r2 = q + 1; r2 < q1; ++r2)
          if (A.chg_col[r2] == j) {
            nl = fmax(nl, A.chg_lb[r2]);
            nu = fmin(nu, A.chg_ub[r2]);
          }
        double l0, u0;
        B.get(j, l0, u0);
        if (nl > u0 || nu < l0 || nl > nu) {
          s_cut = 1;
        } else if (nl > l0 || nu < u0) {
          ovlSet(B, dirty, &s_ndirty, j, nl > l0 ? nl : l0, nu < u0 ? nu : u0);
          expandColumn(A.P, F, j, nl > l0, nu < u0, B.epoch);
        }
      }
    }
    __syncthreads();

    int r = 0;
    while (!s_cut) {
      const int cur = r & 1, nxt = cur ^ 1;
      const int nsh = s_ns[cur], nlo = s_nl[cur];
      if (nsh + nlo == 0) break;
      if (r >= A.maxrounds) {
        if (tid == 0) atomicOr(A.status, 1);
        break;
      }
      __syncthreads();
      if (tid == 0) {
        s_ns[nxt] = 0;
        s_nl[nxt] = 0;
        s_ntouched = 0;
        s_rstamp = ++counter;
        s_rounds = r + 1;
      }
      __syncthreads();
      const int* list = lists[cur];
      processShortRows<NT, RANGED>(A.s, A.P, B, list, nsh, C, st, rb, &s_cut);
      bool cut = false;
      for (int w = warp; w < nlo; w += NW) cut |= rowWarp<RANGED>(A.s, A.P, B, list[m - 1 - w], C, st);
      if (cut) s_cut = 1;
      __syncthreads();
      // acceptance; runs even after a cutoff so that every candidate slot is reset
      Front F{lists[nxt], &s_ns[nxt], &s_nl[nxt], rowstamp, m};
      const int nt = s_ntouched;
      const bool alive = !s_cut;
      unsigned long long ch = 0;
      for (int t = tid; t < nt; t += NT) {
        int j = touched[t];
        double l, u, nl, nu;
        B.get(j, l, u);
        if (applyColumn(A.s, A.P.isint[j] != 0, l, u, C, j, nl, nu)) {
          s_cut = 1;
          continue;
        }
        bool lbup = nl > l, ubdown = nu < u;
        if (alive && (lbup || ubdown)) {
          ovlSet(B, dirty, &s_ndirty, j, nl, nu);
          ch += (unsigned long long)lbup + (unsigned long long)ubdown;
          expandColumn(A.P, F, j, lbup, ubdown, s_rstamp);
        }
      }
      if (ch) atomicAdd(&s_changes, ch);
      __syncthreads();
      ++r;
    }
    __syncthreads();

    // results: columns whose final bounds differ from the base, packed at a reserved offset
    const bool cutoff = s_cut != 0;
    const int nd = s_ndirty;
    int mine = 0;
    if (!cutoff) {
      for (int t = tid; t < nd; t += NT) {
        int j = dirty[t];
        double2 o = ovl[j], b = B.getBase(j);
        if (o.x != b.x || o.y != b.y) ++mine;
      }
      if (mine) atomicAdd(&s_nout, mine);
    }
    __syncthreads();
    if (tid == 0) {
      long long off = 0;
      int cnt = s_nout;
      if (cnt > 0) {
        off = (long long)atomicAdd(A.out_used, (unsigned long long)cnt);
        if (off + cnt > A.out_cap) {
          atomicOr(A.status, 2);
          cnt = -1;
        }
      }
      s_off = cnt < 0 ? -1 : off;
      A.out_off[item] = cnt < 0 ? 0 : off;
      A.out_n[item] = cnt;
      A.out_cutoff[item] = cutoff ? 1 : 0;
      A.out_rounds[item] = s_rounds;
      s_nout = 0;
      mycut += cutoff ? 1 : 0;
      if ((unsigned long long)s_rounds > mymaxr) mymaxr = s_rounds;
      if (s_changes) atomicAdd(&A.stats[3], s_changes);
    }
    __syncthreads();
    if (!cutoff && s_off >= 0) {
      for (int t = tid; t < nd; t += NT) {
        int j = dirty[t];
        double2 o = ovl[j], b = B.getBase(j);
        if (o.x != b.x || o.y != b.y) {
          long long pos = s_off + atomicAdd(&s_nout, 1);
          A.out_col[pos] = j;
          A.out_lb[pos] = o.x;
          A.out_ub[pos] = o.y;
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    S.counter[slot] = counter;
    if (mycut) atomicAdd(&A.stats[4], mycut);
    atomicMax(&A.stats[5], mymaxr);
  }
  flushStats(A.stats, st);
}

// launch shapes: threads per node CTA x register budget (MINB resident CTAs per SM requested from ptxas)
#define GBP_NODE_SHAPES(X) X(32, 16) X(64, 8) X(128, 4) X(256, 2) X(128, 6) X(64, 12) X(32, 24)

template <bool RANGED>
cudaError_t launchNodesT(cudaStream_t st, int grid, int nt, const NodesArgs& A) {
  const int minb = A.minblocks;
#define GBP_LAUNCH(T, B)                             \
  if (nt == T && minb == B) {                        \
    k_nodes<T, B, RANGED><<<grid, T, 0, st>>>(A);    \
    return cudaGetLastError();                       \
  }
  GBP_NODE_SHAPES(GBP_LAUNCH)
#undef GBP_LAUNCH
  return cudaErrorInvalidValue;
}
template <bool RANGED>
cudaError_t nodesOccupancyT(int nt, int minb, int* blocksPerSm) {
#define GBP_OCC(T, B)       \
  if (nt == T && minb == B) \
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, k_nodes<T, B, RANGED>, T, 0);
  GBP_NODE_SHAPES(GBP_OCC)
#undef GBP_OCC
  return cudaErrorInvalidValue;
}

}  // namespace gbp
