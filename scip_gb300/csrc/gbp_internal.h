// Internal interface between the C ABI (gbp_api.cu) and the kernels (gbp_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gbp_device.cuh"

namespace gbp {

// per-CTA scratch of the batched kernel: `slots` copies of column- and row-sized arrays
struct SlotArrays {
  int64_t nstride;     // columns per slot
  int64_t mstride;     // rows per slot
  double2* ovl;        // node bounds that differ from the base (valid where ostamp == node epoch)
  int* ostamp;
  long long* cub;
  long long* clb;
  long long* cubf;
  long long* clbf;
  int* cflag;
  int* touched;        // [nstride]
  int* dirty;          // [nstride] columns written in the current node
  int* rowstamp;       // [mstride]
  int* listA;          // [mstride] frontier (short rows from the front, long rows from the back)
  int* listB;          // [mstride]
  int* counter;        // [slots] stamp counter of each slot (persists across launches)
};

// Carves the per-CTA scratch of `nslots` slots out of one block starting at `base` (null: only measure).
// Returns the bytes needed.
inline size_t slotLayout(int64_t ns, int64_t ms, int64_t nslots, char* base, SlotArrays* out) {
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t S = (size_t)nslots, N = (size_t)ns, M = (size_t)ms;
  size_t off = 0;
  const size_t o_ovl = off; off = align(off + S * N * sizeof(double2));
  const size_t o_ost = off; off = align(off + S * N * sizeof(int));
  const size_t o_cand = off; off = align(off + 4 * S * N * sizeof(long long));
  const size_t o_cflag = off; off = align(off + S * N * sizeof(int));
  const size_t o_touch = off; off = align(off + S * N * sizeof(int));
  const size_t o_dirty = off; off = align(off + S * N * sizeof(int));
  const size_t o_rst = off; off = align(off + S * M * sizeof(int));
  const size_t o_la = off; off = align(off + S * M * sizeof(int));
  const size_t o_lb = off; off = align(off + S * M * sizeof(int));
  const size_t o_ctr = off; off = align(off + S * sizeof(int));
  if (base != nullptr && out != nullptr) {
    out->nstride = ns;
    out->mstride = ms;
    out->ovl = (double2*)(base + o_ovl);
    out->ostamp = (int*)(base + o_ost);
    out->cub = (long long*)(base + o_cand);
    out->clb = out->cub + S * N;
    out->cubf = out->clb + S * N;
    out->clbf = out->cubf + S * N;
    out->cflag = (int*)(base + o_cflag);
    out->touched = (int*)(base + o_touch);
    out->dirty = (int*)(base + o_dirty);
    out->rowstamp = (int*)(base + o_rst);
    out->listA = (int*)(base + o_la);
    out->listB = (int*)(base + o_lb);
    out->counter = (int*)(base + o_ctr);
  }
  return off;
}

struct NodesArgs {
  Num s;
  Prob P;
  const double2* base;     // packed base bounds, or null to read baselb/baseub
  const double* baselb;
  const double* baseub;
  int64_t nnodes;
  const int64_t* ptr;
  const int32_t* chg_col;
  const double* chg_lb;
  const double* chg_ub;
  int8_t* out_cutoff;
  int32_t* out_rounds;
  int64_t* out_off;
  int32_t* out_n;
  int32_t* out_col;
  double* out_lb;
  double* out_ub;
  int64_t out_cap;
  unsigned long long* out_used;  // packed result entries allocated so far
  int maxrounds;
  int* next_item;                // work queue head
  const int* order;              // queue position -> node (longest expected work first), or null: identity
  SlotArrays S;
  unsigned long long* stats;     // rows, nnz, candidates, changes, cutoffs, max rounds
  int* status;                   // bit0 round limit, bit1 output overflow, bit2 a change column out of range
  int minblocks;                 // register-budget variant of the kernel (1 = unconstrained)
  const int* abort_flag;         // null, or a status word whose bit 3 (set by an input check) means: run no node
};


// ------------------------------------------------------------------------------------------ SCIP's own order
// State of one row in one node of the sequential kernel (gbp_seq.cu): struct SCIP_ConsData's activities, counters,
// maxactdelta and flags, plus the node's marking bookkeeping; valid while stamp equals the node's epoch.
struct SeqRow {
  double minhi, minlo, maxhi, maxlo;
  double lastmin, lastmax, maxdelta;
  int minposinf, minneginf, minposhuge, minneghuge;
  int maxposinf, maxneginf, maxposhuge, maxneghuge;
  int maxdeltacol, mpos, stamp;
  unsigned flags;
  int evc;  // bound-change events that reached the row in this node (lanes detect records that changed under them)
};
static_assert(sizeof(SeqRow) == 112, "SeqRow layout");

// warps (one node each) per CTA of the sequential kernel
constexpr int SEQ_WARPS = 4;

// per-warp scratch of the sequential kernel: `nslots` copies of row- and column-sized arrays
struct SeqSlots {
  int64_t nslots;
  int64_t nstride;     // columns per slot
  int64_t mstride;     // rows per slot
  SeqRow* rows;        // [mstride]
  double2* ovl;        // [nstride] node bounds that differ from the base (valid where ost == the node's epoch)
  int* ost;
  int* M;              // [mstride] marked rows, in propagation order
  int* U;              // [mstride] rows with delayed updates
  int* dirty;          // [nstride] columns changed in the node
  int* counter;        // [nslots] epoch counter of each slot (persists across launches)
};

inline size_t seqSlotLayout(int64_t ns, int64_t ms, int64_t nslots, char* base, SeqSlots* out) {
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t S = (size_t)nslots, N = (size_t)ns, M = (size_t)ms;
  size_t off = 0;
  const size_t o_rows = off; off = align(off + S * M * sizeof(SeqRow));
  const size_t o_ovl = off; off = align(off + S * N * sizeof(double2));
  const size_t o_ost = off; off = align(off + S * N * sizeof(int));
  const size_t o_m = off; off = align(off + S * M * sizeof(int));
  const size_t o_u = off; off = align(off + S * M * sizeof(int));
  const size_t o_dirty = off; off = align(off + S * N * sizeof(int));
  const size_t o_ctr = off; off = align(off + S * sizeof(int));
  if (base != nullptr && out != nullptr) {
    out->nslots = nslots;
    out->nstride = ns;
    out->mstride = ms;
    out->rows = (SeqRow*)(base + o_rows);
    out->ovl = (double2*)(base + o_ovl);
    out->ost = (int*)(base + o_ost);
    out->M = (int*)(base + o_m);
    out->U = (int*)(base + o_u);
    out->dirty = (int*)(base + o_dirty);
    out->counter = (int*)(base + o_ctr);
  }
  return off;
}

struct SeqArgs {
  Num s;
  Prob P;                  // rows (CSR) and sides; the entries of a row in the order SCIP holds them
  const int64_t* ccolptr;  // column-major copy with each column's rows ascending
  const int32_t* crow;
  const double* cval;
  const int* prep;         // per row: leading binaries under the base domain; negative: deleted at the root
  const double2* base;     // packed base bounds
  int64_t nnodes;
  const int64_t* ptr;
  const int32_t* chg_col;
  const double* chg_lb;
  const double* chg_ub;
  int8_t* out_cutoff;
  int32_t* out_rounds;
  int64_t* out_off;
  int32_t* out_n;
  int32_t* out_col;
  double* out_lb;
  double* out_ub;
  int64_t out_cap;
  unsigned long long* out_used;
  int maxrounds;
  int* next_item;
  const int* order;
  SeqSlots S;
  unsigned long long* stats;     // rows, nnz, entries visited, changes, cutoffs, max rounds, live rows
  int* status;                   // bit0 round limit, bit1 output overflow, bit2 a change column out of range
};

cudaError_t launchSeqCsc(cudaStream_t st, int grid, int64_t m, int64_t n, int64_t nnz, const int64_t* rowptr,
                         const int32_t* colidx, const double* vals, int32_t* crow, double* cval);
cudaError_t launchSeqPrepare(cudaStream_t st, int grid, const Num& s, const Prob& P, const double2* base, int* prep);
cudaError_t launchNodesSeq(cudaStream_t st, int grid, const SeqArgs& A);
cudaError_t nodesSeqOccupancy(int* blocksPerSm);

// Node order for the queue: more branching changes first (a node's work grows with its changes), so that the
// longest nodes start early and the batch does not end waiting for one of them.  Counting sort on the change
// count (clamped to 255) in two launches; hist holds 2 * ORDER_BUCKETS zeroed ints (counts, cursors).
constexpr int ORDER_BUCKETS = 256;
cudaError_t launchNodeOrder(cudaStream_t st, int grid, int64_t nnodes, const int64_t* ptr, int* hist, int* order);
// ranged rows: flag the rows the gcd rule can act on and list them (count must be zeroed); the entry order of
// listed rows on the global domain dl/du
cudaError_t launchRangedElig(cudaStream_t st, int grid, const Num& s, const Prob& P, uint8_t* elig, int* list,
                             int* count, long long* coef);
// (saved: the domain of the last order, *changed preset to 1 to force the sort; both kernels on st)
cudaError_t launchRangedOrder(cudaStream_t st, int grid, const Prob& P, const int* list, int n, const double* dl,
                              const double* du, int sorted, double2* saved, int* changed, int dgrid);
// instance parts: shift local row pointers / column indices by the parts' offsets, fill the instance maps
cudaError_t launchFixParts(cudaStream_t st, int grid, int64_t ninst, const int64_t* off, int64_t m, int64_t n,
                           int64_t nnz, int64_t* rowptr, int32_t* colidx, int32_t* rowinst, int32_t* colinst, int* bad);

// launchers (return the cudaError_t of the launch)
cudaError_t launchRowsShort(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                            const double* ub, const int* list, const int* nshort, Cands C, int* cutoff,
                            unsigned long long* stats);
cudaError_t launchRowsLong(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                           const double* ub, const int* list, const int* nlong, int cap, Cands C, int* cutoff,
                           unsigned long long* stats);
cudaError_t launchApply(cudaStream_t st, int grid, const Num& s, const Prob& P, double* lb, double* ub, Cands C,
                        Front F, int stamp, int* cutoff, unsigned long long* stats, const ChangeLog& G, int round);
cudaError_t launchSeed(cudaStream_t st, int grid, const Prob& P, const double* lb, const double* ub, int64_t nseed,
                       const int32_t* cols, const double* oldlb, const double* oldub, Front F, int stamp);
cudaError_t launchActivities(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                             const double* ub, double* act, int32_t* cnt);
cudaError_t launchPack(cudaStream_t st, int grid, const double* lb, const double* ub, double2* out, int64_t n);
cudaError_t launchSetChanges(cudaStream_t st, int grid, int64_t nchg, const int32_t* cols, const double* nlb,
                             const double* nub, double* lb, double* ub, double* oldlb, double* oldub, int keepold);
cudaError_t launchMoved(cudaStream_t st, int grid, int64_t n, const double* lb, const double* ub, const double* slb,
                        const double* sub, unsigned long long* count, int64_t cap, int32_t* cols, double* olb,
                        double* oub);
cudaError_t launchNodes(cudaStream_t st, int grid, int threads, const NodesArgs& A);
cudaError_t nodesOccupancy(int threads, int minblocks, int* blocksPerSm);
// the node kernel with the ranged-row rule compiled in (gbp_nodes_ranged.cu); launchNodes picks it when the
// problem carries ranged rows
cudaError_t launchNodesRanged(cudaStream_t st, int grid, int threads, const NodesArgs& A);
cudaError_t nodesOccupancyRanged(int threads, int minblocks, int* blocksPerSm);
cudaError_t launchCscFlags(cudaStream_t st, int grid, int64_t nnz, const double* cvals, const int32_t* rowidx,
                           const double* lhs, const double* rhs, double inf, uint32_t* out);
cudaError_t launchFill64(cudaStream_t st, int grid, long long* p, int64_t n, long long v);
cudaError_t launchFlags8(cudaStream_t st, int grid, const int* in, int8_t* out, int64_t n);
cudaError_t launchCscCount(cudaStream_t st, int grid, int64_t nnz, const int32_t* colidx, int64_t n,
                           unsigned long long* count, int* bad);
cudaError_t launchCscScatter(cudaStream_t st, int grid, int64_t m, const int64_t* rowptr, const int32_t* colidx,
                             const double* vals, const double* lhs, const double* rhs, double inf,
                             unsigned long long* cursor, uint32_t* cscrow);
cudaError_t launchCheckBlocks(cudaStream_t st, int grid, int64_t m, const int64_t* rowptr, const int32_t* colidx,
                              const int32_t* rowinst, const int32_t* colinst, int* bad);
// kernels of the graph-driven loop: 0 rows (short), 1 rows (long), 2 apply, 3 advance
const void* graphKernel(int which);
struct SparseOut {
  int32_t col, pad;
  double lb, ub;
};
// gbp_propagate_changes in one cooperative launch (k_sparse_coop).  Header (SPARSE_HEADER bytes): int cutoff, status,
// rounds, last row stamp, moved columns, 3 unused; then the 8 statistics counters; then the moved columns.
constexpr size_t SPARSE_HEADER = 8 * sizeof(int) + 8 * sizeof(unsigned long long);
struct SparseArgs {
  Num s;
  Prob P;
  Cands C;
  ListSet L;
  LoopState* S;
  LoopState init;  // the loop state the call starts from (its log, bounds, stamps and round limit)
  unsigned long long* stats;
  double* lb;
  double* ub;
  int64_t nchg;
  const int32_t* cols;
  const double* nlb;
  const double* nub;
  double* oldlb;  // the bounds each change replaces (filled unless keepold: then the caller's seed bounds)
  double* oldub;
  int keepold;
  int seedstamp;
  MovedLog moved;
  int64_t cap;
  SparseOut* out;  // the moved columns with their bounds, right after the header
  int* header;
};
cudaError_t launchSparseCoop(cudaStream_t st, int grid, const SparseArgs& A);
cudaError_t sparseCoopOccupancy(int* blocksPerSm);
// all rounds of a seeded plain call in one cooperative launch (grid <= co-resident blocks)
cudaError_t launchPlainCoop(cudaStream_t st, int grid, const Num& s, const Prob& P, const Cands& C, const ListSet& L,
                            LoopState* S, unsigned long long* stats);
cudaError_t plainCoopOccupancy(int* blocksPerSm);
constexpr int ROW_THREADS_G = 128;
cudaError_t columnPointers(cudaStream_t st, const unsigned long long* count, unsigned long long* colptr, int64_t n);

}  // namespace gbp
