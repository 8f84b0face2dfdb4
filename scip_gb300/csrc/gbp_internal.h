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

struct NodesArgs {
  Num s;
  Prob P;
  const double2* base;
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
  SlotArrays S;
  unsigned long long* stats;     // rows, nnz, candidates, changes, cutoffs, max rounds
  int* status;                   // bit0 round limit, bit1 output overflow
};


// launchers (return the cudaError_t of the launch)
cudaError_t launchRowsShort(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                            const double* ub, const int* list, const int* nshort, Cands C, int* cutoff,
                            unsigned long long* stats);
cudaError_t launchRowsLong(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                           const double* ub, const int* list, const int* nlong, int cap, Cands C, int* cutoff,
                           unsigned long long* stats);
cudaError_t launchApply(cudaStream_t st, int grid, const Num& s, const Prob& P, double* lb, double* ub, Cands C,
                        Front F, int stamp, int* cutoff, unsigned long long* stats);
cudaError_t launchSeed(cudaStream_t st, int grid, const Prob& P, const double* lb, const double* ub, int64_t nseed,
                       const int32_t* cols, const double* oldlb, const double* oldub, Front F, int stamp);
cudaError_t launchActivities(cudaStream_t st, int grid, const Num& s, const Prob& P, const double* lb,
                             const double* ub, double* act, int32_t* cnt);
cudaError_t launchPack(cudaStream_t st, int grid, const double* lb, const double* ub, double2* out, int64_t n);
cudaError_t launchNodes(cudaStream_t st, int grid, int threads, const NodesArgs& A);
cudaError_t nodesOccupancy(int threads, int* blocksPerSm);
cudaError_t launchCscFlags(cudaStream_t st, int grid, int64_t nnz, const double* cvals, const int32_t* rowidx,
                           const double* lhs, const double* rhs, double inf, uint32_t* out);
cudaError_t launchFill64(cudaStream_t st, int grid, long long* p, int64_t n, long long v);

}  // namespace gbp
