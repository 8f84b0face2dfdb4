// C ABI of libgbp (declarations and contract: include/gbp.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbp.h"
#include "gbp_internal.h"

using namespace gbp;

namespace {
constexpr int GBP_ABI_VERSION = 1;
}

struct gbp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sms = 0;
  int coop_grid = -1;  // blocks of the cooperative all-rounds kernel (-1 not yet known, 0 unavailable)
  gbp_params par{};
  Num num{};
  std::string err;

  // problem (device arrays are kept and reused by later uploads that fit their capacities)
  bool has_problem = false;
  int64_t m = 0, n = 0, nnz = 0;
  int64_t cap_m = 0, cap_n = 0, cap_nnz = 0, cap_inst = 0;
  int64_t* d_rowptr = nullptr;
  int32_t* d_colidx = nullptr;
  double* d_vals = nullptr;
  double* d_lhs = nullptr;
  double* d_rhs = nullptr;
  int8_t* d_isint = nullptr;
  int64_t* d_colptr = nullptr;
  uint32_t* d_cscrow = nullptr;
  // change log of the plain path (gbp_set_change_log): device arrays and the entry counter, and the ranged-row
  // records kept beside it (same capacity)
  ChangeLog log{};
  int64_t log_cap = 0;
  RangedLog rlog{};
  // explicit global bounds of the plain path (gbp_set_global_bounds)
  bool has_global = false;
  double* d_glb = nullptr;
  double* d_gub = nullptr;
  int64_t cap_glob = 0;

  // ranged rows (GBP_FLAG_RANGEDROW): per-row eligibility, the eligible rows' list, their entry order and merge
  // scratch (per CSR position); valid until the next upload or parameter change
  bool ranged_ready = false;
  uint8_t* d_relig = nullptr;
  int* d_rlist = nullptr;
  int32_t* d_rperm = nullptr;
  int32_t* d_rtmp = nullptr;
  int nranged = 0;
  long long* d_rcoef = nullptr;  // per entry of a ranged row: its classification (Prob::rcoef)
  double2* d_rdom = nullptr;   // the domain d_rperm was sorted on (a fixed-domain order is reused while it holds)
  int* d_rchanged = nullptr;
  bool rdom_valid = false;

  // plain path
  double* d_lb = nullptr;
  double* d_ub = nullptr;
  long long* d_cand = nullptr;  // 4*n keys: cub, clb, cubf, clbf
  int* d_cflag = nullptr;
  int* d_touched = nullptr;
  int* d_list[2] = {nullptr, nullptr};
  int* d_rowstamp = nullptr;
  int* d_allrows = nullptr;
  int nshort_all = 0, nlong_all = 0;
  int* d_ctr = nullptr;  // nshort[2], nlong[2], ntouched, cutoff
  unsigned long long* d_stats = nullptr;  // rows, nnz, cands, changes, cutoffs, maxrounds
  int stamp = 0;
  int32_t* d_seedcols = nullptr;
  double* d_seedold = nullptr;  // 2*cap: oldlb, oldub
  int64_t seedcap = 0;
  int* h_ctr = nullptr;  // pinned

  // several instances uploaded as one block-diagonal problem
  int64_t ninst = 0;
  int32_t* d_rowinst = nullptr;
  int32_t* d_colinst = nullptr;
  int* d_instcut = nullptr;
  bool instmode = false;  // propagateCore works per instance

  // batched path
  int ctas_per_sm = 4;     // register budget / residency of the node kernel variant
  int node_threads = 128;
  int nslots = 0;
  SlotArrays slots{};
  void* slot_mem = nullptr;
  int64_t slot_stamp_budget = 0;
  double2* d_base = nullptr;
  int* d_order = nullptr;     // node order of the queue (capacity order_cap) and its counting-sort buckets
  int* d_orderhist = nullptr;
  int64_t order_cap = 0;
  int* d_next_item = nullptr;
  int* d_status = nullptr;
  unsigned long long* d_out_used = nullptr;
  unsigned long long last_out_used = 0;  // packed entries the last batched call wrote (read with its statistics)
  // sparse plain calls (gbp_set_bounds / gbp_propagate_changes): d_lb/d_ub hold the caller's bounds between calls
  bool bounds_set = false;
  double* d_snap = nullptr;      // [2n] bounds after the caller's changes
  double* d_chgb = nullptr;      // [2 chgcap] new bounds of the changes
  int64_t chgcap = 0;
  char* d_moved = nullptr;       // moved columns: cols [movedcap], lb [movedcap], ub [movedcap]
  int64_t movedcap = 0;
  unsigned long long* d_count = nullptr;
  // staging for the host-pointer node API
  void* stage = nullptr;
  size_t stage_bytes = 0;

  // device-driven fixpoint loop: one CUDA graph per mode (0 single problem, 1 instances) whose conditional
  // while-node repeats rows -> apply -> advance until the frontier is empty, cut off or at the round cap
  LoopState* d_state = nullptr;
  LoopState* h_state = nullptr;  // pinned

  // gbp_propagate_changes in one cooperative launch: per-column first-move stamps and the moved log (n entries),
  // the changes in (device and pinned host), the header and moved columns out (device and pinned host)
  int sparse_grid = -1;
  int* d_mstamp = nullptr;
  int64_t mcap = 0;  // columns the stamps and the moved log hold
  int mepoch = 0;
  int* d_mcount = nullptr;
  int32_t* d_mcol = nullptr;
  double* d_mlb = nullptr;
  double* d_mub = nullptr;
  char* d_sin = nullptr;
  char* h_sin = nullptr;
  size_t sin_bytes = 0;
  char* d_sout = nullptr;
  char* h_sout = nullptr;
  int64_t sout_cap = 0;
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  bool graph_failed = false;

  // SCIP's own order for batched nodes (GBP_FLAG_SCIPORDER): the column-major copy with each column's rows ascending
  // (built on first use after an upload), the per-row preparation of a call, and per-warp slots
  bool seq_csc_ready = false;
  int32_t* d_sq_crow = nullptr;
  double* d_sq_cval = nullptr;
  int64_t sq_cap_nnz = 0;
  int* d_sq_prep = nullptr;
  int64_t sq_cap_m = 0;
  void* seq_mem = nullptr;
  SeqSlots seqslots{};
  int64_t seq_epoch_budget = 0;

  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void destroyGraphs(gbp_ctx* ctx) {
  for (int k = 0; k < 2; ++k) {
    if (ctx->gexec[k]) cudaGraphExecDestroy(ctx->gexec[k]);
    if (ctx->graph[k]) cudaGraphDestroy(ctx->graph[k]);
    ctx->gexec[k] = nullptr;
    ctx->graph[k] = nullptr;
  }
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
      return e_ == cudaErrorMemoryAllocation ? GBP_ERR_NOMEM : GBP_ERR_CUDA;             \
    }                                                                                    \
  } while (0)

static int fail(gbp_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

static void freeProblem(gbp_ctx* ctx) {
  destroyGraphs(ctx);
  void* ptrs[] = {ctx->d_rowptr, ctx->d_colidx, ctx->d_vals, ctx->d_lhs, ctx->d_rhs, ctx->d_isint, ctx->d_colptr,
                  ctx->d_cscrow, ctx->d_lb, ctx->d_ub, ctx->d_cand, ctx->d_cflag, ctx->d_touched, ctx->d_list[0],
                  ctx->d_list[1], ctx->d_rowstamp, ctx->d_allrows, ctx->d_base, ctx->slot_mem, ctx->stage,
                  ctx->d_rowinst, ctx->d_colinst, ctx->d_instcut, ctx->d_glb, ctx->d_gub, ctx->d_relig,
                  ctx->d_rlist, ctx->d_rperm, ctx->d_rtmp, ctx->d_rdom, ctx->d_rchanged, ctx->d_rcoef, ctx->d_snap,
                  ctx->d_sq_crow, ctx->d_sq_cval, ctx->d_sq_prep, ctx->seq_mem};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  ctx->d_rowptr = nullptr; ctx->d_colidx = nullptr; ctx->d_vals = nullptr; ctx->d_lhs = nullptr;
  ctx->d_rhs = nullptr; ctx->d_isint = nullptr; ctx->d_colptr = nullptr; ctx->d_cscrow = nullptr;
  ctx->d_lb = nullptr; ctx->d_ub = nullptr; ctx->d_cand = nullptr; ctx->d_cflag = nullptr;
  ctx->d_touched = nullptr; ctx->d_list[0] = ctx->d_list[1] = nullptr; ctx->d_rowstamp = nullptr;
  ctx->d_allrows = nullptr; ctx->d_base = nullptr; ctx->slot_mem = nullptr; ctx->stage = nullptr;
  ctx->d_rowinst = nullptr; ctx->d_colinst = nullptr; ctx->d_instcut = nullptr; ctx->ninst = 0;
  ctx->d_glb = nullptr; ctx->d_gub = nullptr; ctx->cap_glob = 0; ctx->has_global = false;
  ctx->d_relig = nullptr; ctx->d_rlist = nullptr; ctx->d_rperm = nullptr; ctx->d_rtmp = nullptr;
  ctx->ranged_ready = false; ctx->nranged = 0;
  ctx->d_rdom = nullptr; ctx->d_rchanged = nullptr; ctx->rdom_valid = false; ctx->d_rcoef = nullptr;
  ctx->cap_m = ctx->cap_n = ctx->cap_nnz = ctx->cap_inst = 0;
  ctx->stage_bytes = 0;
  ctx->d_snap = nullptr;
  ctx->bounds_set = false;
  ctx->nslots = 0;
  ctx->d_sq_crow = nullptr; ctx->d_sq_cval = nullptr; ctx->sq_cap_nnz = 0; ctx->seq_csc_ready = false;
  ctx->d_sq_prep = nullptr; ctx->sq_cap_m = 0;
  ctx->seq_mem = nullptr; ctx->seqslots = SeqSlots{};
  ctx->has_problem = false;
}

static bool rangedOn(const gbp_ctx* ctx) { return (ctx->par.flags & GBP_FLAG_RANGEDROW) != 0; }

// nodes: the batch's global domain is its base bounds, so the ranged rows' order is computed before the call
static Prob devProb(const gbp_ctx* ctx, bool instances = false, bool nodes = false) {
  Prob P{ctx->m, ctx->n, ctx->d_rowptr, ctx->d_colidx, ctx->d_vals, ctx->d_lhs, ctx->d_rhs, ctx->d_isint,
         ctx->d_colptr, ctx->d_cscrow, nullptr, nullptr, ctx->par.infinity,
         instances ? ctx->d_rowinst : nullptr, instances ? ctx->d_colinst : nullptr,
         instances ? ctx->d_instcut : nullptr, (!instances && ctx->has_global) ? ctx->d_glb : nullptr,
         (!instances && ctx->has_global) ? ctx->d_gub : nullptr};
  if (rangedOn(ctx) && ctx->ranged_ready) {
    const bool sorted = !(ctx->par.flags & GBP_FLAG_NOSORTVARS);
    P.relig = ctx->d_relig;
    P.rperm = ctx->d_rperm;
    P.rtmp = ctx->d_rtmp;
    P.rcoef = ctx->d_rcoef;
    P.rsorted = sorted ? 1 : 0;
    // the sorted order follows the bounds being propagated when there is no other global domain (at the root
    // SCIP re-sorts a row whenever one of its columns becomes binary); every other order is fixed for a call
    P.rlive = (sorted && !nodes && (instances || !ctx->has_global)) ? 1 : 0;
  }
  return P;
}

static int gridFor(const gbp_ctx* ctx, int64_t work, int per_block = 256, int cap_per_sm = 16) {
  int64_t g = (work + per_block - 1) / per_block;
  int64_t cap = (int64_t)ctx->sms * cap_per_sm;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

extern "C" {

int gbp_version(void) { return GBP_ABI_VERSION; }

const char* gbp_error_string(int code) {
  switch (code) {
    case GBP_OK: return "ok";
    case GBP_ERR_INVALID: return "invalid argument";
    case GBP_ERR_CUDA: return "CUDA error";
    case GBP_ERR_NOMEM: return "out of memory";
    case GBP_ERR_NODEVICE: return "no suitable CUDA device";
    case GBP_ERR_LIMIT: return "round limit reached";
    case GBP_ERR_OVERFLOW: return "output list too small";
    case GBP_ERR_STATE: return "inconsistent device state";
    case GBP_ERR_TOO_LARGE: return "problem too large for the no-alloc scratch";
    case GBP_ERR_BUSY: return "reply not ready";
    default: return "unknown error";
  }
}

const char* gbp_last_error(const gbp_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

void gbp_default_params(gbp_params* p) {
  if (!p) return;
  p->infinity = 1e20;
  p->epsilon = 1e-9;
  p->sumepsilon = 1e-6;
  p->feastol = 1e-6;
  p->hugeval = 1e15;
  p->boundstreps = 0.05;
  p->recompfac = 1e6;
  p->maxeasyactivitydelta = 1e6;
  p->maxrounds = 0;
  p->flags = 0;
}

int gbp_set_params(gbp_ctx* ctx, const gbp_params* p) {
  if (!ctx || !p) return GBP_ERR_INVALID;
  if (!(p->infinity > 0) || !(p->epsilon >= 0) || !(p->sumepsilon >= 0) || !(p->feastol >= 0) ||
      !(p->hugeval > 0) || !(p->boundstreps >= 0) || !(p->recompfac > 0))
    return fail(ctx, GBP_ERR_INVALID, "invalid numerics");
  ctx->par = *p;
  // + 0.0 stores a -0 as +0: the device tests compare the tolerances' bit patterns, which needs them >= +0
  ctx->num = Num{p->infinity, p->epsilon + 0.0, p->sumepsilon + 0.0, p->feastol + 0.0, p->hugeval,
                 p->boundstreps + 0.0, p->recompfac, p->maxeasyactivitydelta, (p->flags & GBP_FLAG_NOSORTVARS) ? 1 : 0};
  destroyGraphs(ctx);  // the numerics are baked into the graphs' kernel arguments
  ctx->ranged_ready = false;  // eligibility depends on epsilon and infinity
  return GBP_OK;
}

int gbp_create(gbp_ctx** out, int device, void* stream) {
  if (!out) return GBP_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
    cudaGetLastError();
    return GBP_ERR_NODEVICE;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return GBP_ERR_NODEVICE;
  if (prop.major != 10 || prop.minor != 3) return GBP_ERR_NODEVICE;  // built for sm_103a only
  gbp_ctx* ctx = new (std::nothrow) gbp_ctx();
  if (!ctx) return GBP_ERR_NOMEM;
  ctx->device = device;
  ctx->sms = prop.multiProcessorCount;
  gbp_params p;
  gbp_default_params(&p);
  gbp_set_params(ctx, &p);
  if (cudaSetDevice(device) != cudaSuccess) {
    delete ctx;
    return GBP_ERR_NODEVICE;
  }
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return GBP_ERR_CUDA;
    }
    ctx->own_stream = true;
  }
  if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
      cudaMalloc(&ctx->d_ctr, 8 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_stats, 8 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&ctx->d_next_item, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_orderhist, 2 * ORDER_BUCKETS * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_out_used, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_ctr, 16 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_state, sizeof(LoopState)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_state, sizeof(LoopState)) != cudaSuccess) {
    gbp_destroy(ctx);
    return GBP_ERR_CUDA;
  }
  *out = ctx;
  return GBP_OK;
}

int gbp_destroy(gbp_ctx* ctx) {
  if (!ctx) return GBP_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  freeProblem(ctx);
  if (ctx->d_seedcols) cudaFree(ctx->d_seedcols);
  if (ctx->d_seedold) cudaFree(ctx->d_seedold);
  if (ctx->d_ctr) cudaFree(ctx->d_ctr);
  if (ctx->d_stats) cudaFree(ctx->d_stats);
  if (ctx->d_next_item) cudaFree(ctx->d_next_item);
  if (ctx->d_chgb) cudaFree(ctx->d_chgb);
  if (ctx->d_moved) cudaFree(ctx->d_moved);
  if (ctx->d_count) cudaFree(ctx->d_count);
  if (ctx->d_orderhist) cudaFree(ctx->d_orderhist);
  {
    void* lp[] = {ctx->log.n, ctx->log.col, ctx->log.round, ctx->log.lb, ctx->log.ub,
                  ctx->rlog.n, ctx->rlog.row, ctx->rlog.col, ctx->rlog.round};
    for (void* p : lp)
      if (p) cudaFree(p);
  }
  if (ctx->d_order) cudaFree(ctx->d_order);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->d_out_used) cudaFree(ctx->d_out_used);
  if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
  if (ctx->d_state) cudaFree(ctx->d_state);
  if (ctx->h_state) cudaFreeHost(ctx->h_state);
  {
    void* dp[] = {ctx->d_mstamp, ctx->d_mcount, ctx->d_mcol, ctx->d_mlb, ctx->d_mub, ctx->d_sin, ctx->d_sout};
    for (void* p : dp)
      if (p) cudaFree(p);
    if (ctx->h_sin) cudaFreeHost(ctx->h_sin);
    if (ctx->h_sout) cudaFreeHost(ctx->h_sout);
  }
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GBP_OK;
}

int gbp_get_stream(const gbp_ctx* ctx, void** stream) {
  if (!ctx || !stream) return GBP_ERR_INVALID;
  *stream = (void*)ctx->stream;
  return GBP_OK;
}

// compiled register budgets of the node kernel: (threads per node, resident CTAs per SM)
static bool shapeCompiled(int t, int b) {
  static const int shapes[][2] = {{32, 16}, {64, 8}, {128, 4}, {256, 2}, {128, 6}, {64, 12}, {32, 24}};
  for (const auto& sh : shapes)
    if (sh[0] == t && sh[1] == b) return true;
  return false;
}
static int defaultBudget(int t) { return t == 32 ? 16 : t == 64 ? 8 : t == 128 ? 4 : 2; }

int gbp_set_batch_shape(gbp_ctx* ctx, int32_t threads_per_node, int32_t ctas_per_sm) {
  if (!ctx) return GBP_ERR_INVALID;
  if (threads_per_node != 32 && threads_per_node != 64 && threads_per_node != 128 && threads_per_node != 256)
    return fail(ctx, GBP_ERR_INVALID, "threads per node must be 32, 64, 128 or 256");
  if (ctas_per_sm == 0) ctas_per_sm = defaultBudget(threads_per_node);
  if (!shapeCompiled(threads_per_node, ctas_per_sm))
    return fail(ctx, GBP_ERR_INVALID, "no compiled variant for this (threads per node, CTAs per SM) shape");
  if (ctas_per_sm != ctx->ctas_per_sm || threads_per_node != ctx->node_threads) {
    ctx->ctas_per_sm = ctas_per_sm;
    ctx->node_threads = threads_per_node;
    if (ctx->slot_mem) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->slot_mem);
      ctx->slot_mem = nullptr;
      ctx->nslots = 0;
    }
  }
  return GBP_OK;
}

// Upload, part 1: drop the previous problem and make the device arrays large enough for m rows, n columns and nnz
// entries.
static int prepareUpload(gbp_ctx* ctx, int64_t m, int64_t n, int64_t nnz) {
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->has_problem = false;
  ctx->has_global = false;
  ctx->ninst = 0;
  destroyGraphs(ctx);
  // the sparse calls' bounds and snapshot belong to the previous problem (the snapshot is sized for its n, and
  // the arrays below may be reused for a larger one)
  ctx->bounds_set = false;
  if (ctx->d_snap) {
    cudaFree(ctx->d_snap);
    ctx->d_snap = nullptr;
  }
  const size_t mm = (size_t)std::max<int64_t>(m, 1), nn = (size_t)std::max<int64_t>(n, 1),
               zz = (size_t)std::max<int64_t>(nnz, 1);
  if ((int64_t)mm > ctx->cap_m || (int64_t)nn > ctx->cap_n || (int64_t)zz > ctx->cap_nnz) {
    // grow (a quarter of headroom, so that a stream of similar uploads reuses the arrays; freeing and
    // allocating synchronise the device, reuse does not)
    const int64_t cm = std::max<int64_t>(mm, ctx->cap_m + ctx->cap_m / 4);
    const int64_t cn = std::max<int64_t>(nn, ctx->cap_n + ctx->cap_n / 4);
    const int64_t cz = std::max<int64_t>(zz, ctx->cap_nnz + ctx->cap_nnz / 4);
    freeProblem(ctx);
    CK(cudaMalloc(&ctx->d_rowptr, (cm + 1) * sizeof(int64_t)));
    CK(cudaMalloc(&ctx->d_colidx, cz * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->d_vals, cz * sizeof(double)));
    CK(cudaMalloc(&ctx->d_lhs, cm * sizeof(double)));
    CK(cudaMalloc(&ctx->d_rhs, cm * sizeof(double)));
    CK(cudaMalloc(&ctx->d_isint, cn));
    CK(cudaMalloc(&ctx->d_colptr, (cn + 1) * sizeof(int64_t)));
    CK(cudaMalloc(&ctx->d_cscrow, cz * sizeof(uint32_t)));
    CK(cudaMalloc(&ctx->d_lb, cn * sizeof(double)));
    CK(cudaMalloc(&ctx->d_ub, cn * sizeof(double)));
    CK(cudaMalloc(&ctx->d_cand, 4 * cn * sizeof(long long)));
    CK(cudaMalloc(&ctx->d_cflag, cn * sizeof(int)));
    CK(cudaMalloc(&ctx->d_touched, cn * sizeof(int)));
    CK(cudaMalloc(&ctx->d_list[0], cm * sizeof(int)));
    CK(cudaMalloc(&ctx->d_list[1], cm * sizeof(int)));
    CK(cudaMalloc(&ctx->d_rowstamp, cm * sizeof(int)));
    CK(cudaMalloc(&ctx->d_allrows, cm * sizeof(int)));
    CK(cudaMalloc(&ctx->d_base, cn * sizeof(double2)));
    ctx->cap_m = cm;
    ctx->cap_n = cn;
    ctx->cap_nnz = cz;
  } else if (ctx->slot_mem && (ctx->slots.nstride < (int64_t)nn || ctx->slots.mstride < (int64_t)mm)) {
    CK(cudaFree(ctx->slot_mem));
    ctx->slot_mem = nullptr;
    ctx->nslots = 0;
  }
  ctx->seq_csc_ready = false;
  if (ctx->seq_mem && (ctx->seqslots.nstride < (int64_t)nn || ctx->seqslots.mstride < (int64_t)mm)) {
    CK(cudaFree(ctx->seq_mem));
    ctx->seq_mem = nullptr;
    ctx->seqslots = SeqSlots{};
  }
  return GBP_OK;
}

// the instance maps (row -> instance, column -> instance) and the per-instance cutoff flags
static int prepareInstanceMaps(gbp_ctx* ctx, int64_t ninst) {
  if (!ctx->d_rowinst || ninst > ctx->cap_inst) {
    if (ctx->d_rowinst) cudaFree(ctx->d_rowinst);
    if (ctx->d_colinst) cudaFree(ctx->d_colinst);
    if (ctx->d_instcut) cudaFree(ctx->d_instcut);
    ctx->d_rowinst = ctx->d_colinst = nullptr;
    ctx->d_instcut = nullptr;
    CK(cudaMalloc(&ctx->d_rowinst, ctx->cap_m * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->d_colinst, ctx->cap_n * sizeof(int32_t)));
    const int64_t ci = std::max<int64_t>(ninst, ctx->cap_inst + ctx->cap_inst / 4);
    CK(cudaMalloc(&ctx->d_instcut, ci * sizeof(int)));
    ctx->cap_inst = ci;
  }
  return GBP_OK;
}

// Upload, part 3 (after the CSR, sides, integrality and the all-rows frontier are on the device): column view,
// candidate keys, flags.
static int finishUpload(gbp_ctx* ctx, int64_t m, int64_t n, int64_t nnz, int ns, int nl) {
  const size_t mm = (size_t)std::max<int64_t>(m, 1), nn = (size_t)std::max<int64_t>(n, 1);
// CSC with relevance flags, built on the device: count per column, prefix sum, scatter
  {
    unsigned long long* count = nullptr;
    unsigned long long* cursor = nullptr;
    CK(cudaMallocAsync((void**)&count, (nn + 1) * sizeof(unsigned long long), ctx->stream));
    CK(cudaMallocAsync((void**)&cursor, (nn + 1) * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(count, 0, (nn + 1) * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_ctr, 0, 8 * sizeof(int), ctx->stream));
    if (nnz) CK(launchCscCount(ctx->stream, gridFor(ctx, nnz), nnz, ctx->d_colidx, n, count, ctx->d_ctr + 7));
    CK(columnPointers(ctx->stream, count, (unsigned long long*)ctx->d_colptr, n));
    CK(cudaMemcpyAsync(cursor, ctx->d_colptr, (nn + 1) * sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                       ctx->stream));
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, ctx->d_ctr + 7, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (bad) {
      cudaFreeAsync(count, ctx->stream);
      cudaFreeAsync(cursor, ctx->stream);
      freeProblem(ctx);
      return fail(ctx, GBP_ERR_INVALID, "column index out of range");
    }
    if (m) CK(launchCscScatter(ctx->stream, gridFor(ctx, m), m, ctx->d_rowptr, ctx->d_colidx, ctx->d_vals, ctx->d_lhs,
                               ctx->d_rhs, ctx->par.infinity, cursor, ctx->d_cscrow));
    CK(cudaFreeAsync(count, ctx->stream));
    CK(cudaFreeAsync(cursor, ctx->stream));
  }
  const size_t cn = (size_t)ctx->cap_n;
  CK(launchFill64(ctx->stream, gridFor(ctx, nn), ctx->d_cand, nn, KEY_NONE_UB));
  CK(launchFill64(ctx->stream, gridFor(ctx, nn), ctx->d_cand + cn, nn, KEY_NONE_LB));
  CK(launchFill64(ctx->stream, gridFor(ctx, nn), ctx->d_cand + 2 * cn, nn, KEY_NONE_UB));
  CK(launchFill64(ctx->stream, gridFor(ctx, nn), ctx->d_cand + 3 * cn, nn, KEY_NONE_LB));
  CK(cudaMemsetAsync(ctx->d_cflag, 0, nn * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_rowstamp, 0, mm * sizeof(int), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->ranged_ready = false;
  ctx->m = m;
  ctx->n = n;
  ctx->nnz = nnz;
  ctx->nshort_all = ns;
  ctx->nlong_all = nl;
  ctx->stamp = 0;
  ctx->has_problem = true;
  return GBP_OK;
}

int gbp_upload_problem(gbp_ctx* ctx, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
                       const double* vals, const double* lhs, const double* rhs, const int8_t* isint) {
  if (!ctx || m < 0 || n < 0 || !rowptr || (m > 0 && (!lhs || !rhs)) || (n > 0 && !isint))
    return fail(ctx, GBP_ERR_INVALID, "null argument or negative size");
  if (m >= (int64_t(1) << 30) || n >= (int64_t(1) << 31) - 1)
    return fail(ctx, GBP_ERR_INVALID, "problem too large (m < 2^30, n < 2^31 required)");
  if (rowptr[0] != 0) return fail(ctx, GBP_ERR_INVALID, "rowptr[0] must be 0");
  for (int64_t i = 0; i < m; ++i)
    if (rowptr[i + 1] < rowptr[i]) return fail(ctx, GBP_ERR_INVALID, "rowptr not monotone");
  const int64_t nnz = rowptr[m];
  if (nnz > 0 && (!colidx || !vals)) return fail(ctx, GBP_ERR_INVALID, "null colidx/vals");

  int rc = prepareUpload(ctx, m, n, nnz);
  if (rc != GBP_OK) return rc;
  // all-rows frontier: short rows from the front, long rows from the back
  std::vector<int> allrows(std::max<int64_t>(m, 1));
  int ns = 0, nl = 0;
  for (int64_t i = 0; i < m; ++i) {
    if (rowptr[i + 1] - rowptr[i] <= LONGROW) allrows[ns++] = (int)i;
    else allrows[m - 1 - nl++] = (int)i;
  }
  CK(cudaMemcpyAsync(ctx->d_rowptr, rowptr, (m + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  if (nnz) {
    CK(cudaMemcpyAsync(ctx->d_colidx, colidx, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_vals, vals, nnz * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  if (m) {
    CK(cudaMemcpyAsync(ctx->d_lhs, lhs, m * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_rhs, rhs, m * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_allrows, allrows.data(), m * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  }
  if (n) CK(cudaMemcpyAsync(ctx->d_isint, isint, n, cudaMemcpyHostToDevice, ctx->stream));
  return finishUpload(ctx, m, n, nnz, ns, nl);
}

// ------------------------------------------------------------------------------------------ plain path
static Cands plainCands(gbp_ctx* ctx) {
  const size_t n = (size_t)ctx->cap_n;
  return Cands{ctx->d_cand, ctx->d_cand + n, ctx->d_cand + 2 * n, ctx->d_cand + 3 * n, ctx->d_cflag,
               ctx->d_touched, ctx->d_ctr + 4, ctx->rlog, 0};
}

static int nextStamp(gbp_ctx* ctx) {
  if (ctx->stamp >= 0x7ffffff0) {
    cudaMemsetAsync(ctx->d_rowstamp, 0, (size_t)std::max<int64_t>(ctx->m, 1) * sizeof(int), ctx->stream);
    ctx->stamp = 0;
  }
  return ++ctx->stamp;
}

// blocks of the cooperative all-rounds kernel: every co-resident block (0: cooperative launches unavailable)
static int coopGrid(gbp_ctx* ctx) {
  if (ctx->coop_grid < 0) {
    int ok = 0, per = 0;
    if (cudaDeviceGetAttribute(&ok, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !ok ||
        plainCoopOccupancy(&per) != cudaSuccess || per < 1) {
      cudaGetLastError();
      ctx->coop_grid = 0;
    } else {
      ctx->coop_grid = per * ctx->sms;
    }
  }
  return ctx->coop_grid;
}

static int buildGraph(gbp_ctx* ctx, int mode) {
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  ctx->graph[mode] = g;
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cn;
  CK(cudaGraphAddNode(&cn, g, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];

  Num s = ctx->num;
  Prob P = devProb(ctx, mode == 1);
  Cands C = plainCands(ctx);
  C.ntouched = &ctx->d_state->ntouched;
  ListSet L{{ctx->d_list[0], ctx->d_list[1], ctx->d_allrows}, ctx->d_rowstamp, (int)ctx->m};
  LoopState* S = ctx->d_state;
  unsigned long long* stats = ctx->d_stats;
  void* args[] = {&s, &P, &C, &L, &S, &stats};
  void* advargs[] = {&S, &h};
  const dim3 grids[4] = {dim3(ctx->sms * 16), dim3(ctx->sms * 8), dim3(ctx->sms * 8), dim3(1)};
  const dim3 blocks[4] = {dim3(ROW_THREADS_G), dim3(256), dim3(256), dim3(1)};
  cudaGraphNode_t prev = nullptr;
  for (int k = 0; k < 4; ++k) {
    cudaKernelNodeParams kp = {};
    kp.func = (void*)graphKernel(k);
    kp.gridDim = grids[k];
    kp.blockDim = blocks[k];
    kp.kernelParams = k == 3 ? advargs : args;
    cudaGraphNode_t node;
    CK(cudaGraphAddKernelNode(&node, body, prev ? &prev : nullptr, prev ? 1 : 0, &kp));
    prev = node;
  }
  CK(cudaGraphInstantiate(&ctx->gexec[mode], g, 0));
  return GBP_OK;
}

// one fixpoint through the graph: seeds (if any) on the stream, then one graph launch for all rounds
// Ranged rows: flags and list of the rows the gcd rule can act on (once per upload and parameter set), then, when
// the entry order is fixed for the call (domain dl/du: explicit global bounds, a node batch's base bounds, or
// the bounds the call starts from for the index order), that order.  Adds its launches to *launches.
static int prepareRanged(gbp_ctx* ctx, bool instances, bool nodes, const double* dl, const double* du,
                         int* launches) {
  if (!rangedOn(ctx)) return GBP_OK;
  if (!ctx->ranged_ready) {
    if (!ctx->d_relig) {
      CK(cudaStreamSynchronize(ctx->stream));
      CK(cudaMalloc(&ctx->d_relig, (size_t)ctx->cap_m));
      CK(cudaMalloc(&ctx->d_rlist, (size_t)ctx->cap_m * sizeof(int)));
      CK(cudaMalloc(&ctx->d_rperm, (size_t)ctx->cap_nnz * sizeof(int32_t)));
      CK(cudaMalloc(&ctx->d_rtmp, (size_t)ctx->cap_nnz * sizeof(int32_t)));
      CK(cudaMalloc(&ctx->d_rdom, (size_t)ctx->cap_n * sizeof(double2)));
      CK(cudaMalloc(&ctx->d_rcoef, (size_t)ctx->cap_nnz * sizeof(long long)));
      CK(cudaMalloc(&ctx->d_rchanged, sizeof(int)));
    }
    ctx->rdom_valid = false;
    destroyGraphs(ctx);  // the graphs hold the ranged rows' pointers
    int* count = ctx->d_ctr + 6;
    CK(cudaMemsetAsync(count, 0, sizeof(int), ctx->stream));
    if (ctx->m) {
      const Prob P = devProb(ctx, instances, nodes);
      CK(launchRangedElig(ctx->stream, gridFor(ctx, ctx->m), ctx->num, P, ctx->d_relig, ctx->d_rlist, count,
                          ctx->d_rcoef));
      *launches += 1;
    }
    int h = 0;
    CK(cudaMemcpyAsync(&h, count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->nranged = h;
    ctx->ranged_ready = true;
  }
  const Prob P = devProb(ctx, instances, nodes);
  if (P.rlive) {
    ctx->rdom_valid = false;  // the rows' order is rewritten where they are evaluated
  } else if (ctx->nranged > 0) {
    // the order is sorted again only if the domain differs from the one it was sorted on
    CK(cudaMemsetAsync(ctx->d_rchanged, ctx->rdom_valid ? 0 : 0xff, sizeof(int), ctx->stream));
    CK(launchRangedOrder(ctx->stream, gridFor(ctx, ctx->nranged, 128, 8), P, ctx->d_rlist, ctx->nranged, dl, du,
                         P.rsorted, ctx->d_rdom, ctx->d_rchanged, gridFor(ctx, ctx->n, 256, 8)));
    ctx->rdom_valid = true;
    *launches += 2;
  }
  return GBP_OK;
}

static int propagateGraph(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* d_seedcols,
                          const double* d_oldlb, const double* d_oldub, int32_t* cutoff, gbp_result* res) {
  const int mode = ctx->instmode ? 1 : 0;
  if (!ctx->gexec[mode]) {
    int rc = buildGraph(ctx, mode);
    if (rc != GBP_OK) {
      destroyGraphs(ctx);
      return rc;
    }
  }
  const int maxrounds = ctx->par.maxrounds > 0 ? ctx->par.maxrounds : 1000000;
  if ((int64_t)ctx->stamp > (int64_t)0x7fffffff - maxrounds - 16) {
    CK(cudaMemsetAsync(ctx->d_rowstamp, 0, (size_t)std::max<int64_t>(ctx->m, 1) * sizeof(int), ctx->stream));
    ctx->stamp = 0;
  }
  LoopState& hs = *ctx->h_state;
  std::memset(&hs, 0, sizeof(hs));
  hs.maxrounds = maxrounds;
  hs.lb = lb;
  hs.ub = ub;
  hs.log = ctx->log;
  if (ctx->log.n) CK(cudaMemsetAsync(ctx->log.n, 0, sizeof(int), ctx->stream));
  if (ctx->rlog.n) CK(cudaMemsetAsync(ctx->rlog.n, 0, sizeof(int), ctx->stream));
  int seedstamp = 0;
  if (nseed < 0) {
    hs.cur = 2;
    hs.nshort[2] = ctx->nshort_all;
    hs.nlong[2] = ctx->nlong_all;
  } else {
    hs.cur = 0;
    seedstamp = ++ctx->stamp;
  }
  hs.stamp = ++ctx->stamp;
  CK(cudaMemsetAsync(ctx->d_stats, 0, 8 * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_state, &hs, sizeof(LoopState), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  int launches = 0;
  if (nseed > 0) {
    const Prob P = devProb(ctx, ctx->instmode);
    Front F{ctx->d_list[0], &ctx->d_state->nshort[0], &ctx->d_state->nlong[0], ctx->d_rowstamp, (int)ctx->m};
    CK(launchSeed(ctx->stream, gridFor(ctx, nseed), P, lb, ub, nseed, d_seedcols, d_oldlb, d_oldub, F, seedstamp));
    ++launches;
  }
  if (nseed > 0 && coopGrid(ctx) > 0) {
    // a seeded call: all rounds in one cooperative launch (the graph's per-kernel costs dominate small frontiers)
    Cands C = plainCands(ctx);
    C.ntouched = &ctx->d_state->ntouched;
    const ListSet L{{ctx->d_list[0], ctx->d_list[1], ctx->d_allrows}, ctx->d_rowstamp, (int)ctx->m};
    CK(launchPlainCoop(ctx->stream, coopGrid(ctx), ctx->num, devProb(ctx, ctx->instmode), C, L, ctx->d_state,
                       ctx->d_stats));
    ++launches;
  } else if (nseed != 0) {
    CK(cudaGraphLaunch(ctx->gexec[mode], ctx->stream));
    ++launches;
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  unsigned long long st[8];
  CK(cudaMemcpyAsync(&hs, ctx->d_state, sizeof(LoopState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(st, ctx->d_stats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (nseed != 0) ctx->stamp = std::max(ctx->stamp, hs.stamp);
  const bool cut = !ctx->instmode && hs.cutoff != 0;
  const int status = cut ? 1 : (hs.status == 2 ? 2 : 0);
  if (cutoff) *cutoff = cut ? 1 : 0;
  if (res) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->cutoff = cut ? 1 : 0;
    res->rounds = hs.worked;
    res->status = status;
    res->launches = launches;
    res->rows = (int64_t)st[0];
    res->nnz = (int64_t)st[1];
    res->candidates = (int64_t)st[2];
    res->changes = (int64_t)st[3];
    res->live_rows = (int64_t)st[6];
    res->kernel_ms = ms;
  }
  return status == 2 ? GBP_ERR_LIMIT : GBP_OK;
}

static int propagateHostLoop(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* d_seedcols,
                             const double* d_oldlb, const double* d_oldub, int32_t* cutoff, gbp_result* res);

static int propagateCore(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* d_seedcols,
                         const double* d_oldlb, const double* d_oldub, int32_t* cutoff, gbp_result* res) {
  int pre = 0;
  const bool glob = !ctx->instmode && ctx->has_global;
  int rc = prepareRanged(ctx, ctx->instmode, false, glob ? ctx->d_glb : lb, glob ? ctx->d_gub : ub, &pre);
  if (rc != GBP_OK) return rc;
  if (!(ctx->par.flags & GBP_FLAG_HOSTLOOP) && !ctx->graph_failed) {
    rc = propagateGraph(ctx, lb, ub, nseed, d_seedcols, d_oldlb, d_oldub, cutoff, res);
    if (rc != GBP_ERR_CUDA || ctx->gexec[ctx->instmode ? 1 : 0] != nullptr) {
      if (res) res->launches += pre;
      return rc;
    }
    // graphs unavailable: fall back to the host-driven rounds for the rest of the context's life
    ctx->graph_failed = true;
    cudaGetLastError();
  }
  rc = propagateHostLoop(ctx, lb, ub, nseed, d_seedcols, d_oldlb, d_oldub, cutoff, res);
  if (res) res->launches += pre;
  return rc;
}

static int propagateHostLoop(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* d_seedcols,
                             const double* d_oldlb, const double* d_oldub, int32_t* cutoff, gbp_result* res) {
  const Prob P = devProb(ctx, ctx->instmode);
  const Num s = ctx->num;
  Cands C = plainCands(ctx);
  const int maxrounds = ctx->par.maxrounds > 0 ? ctx->par.maxrounds : 1000000;
  int launches = 0;
  CK(cudaMemsetAsync(ctx->d_stats, 0, 8 * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_ctr, 0, 8 * sizeof(int), ctx->stream));
  if (ctx->log.n) CK(cudaMemsetAsync(ctx->log.n, 0, sizeof(int), ctx->stream));
  if (ctx->rlog.n) CK(cudaMemsetAsync(ctx->rlog.n, 0, sizeof(int), ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));

  int* cur = nullptr;
  int curidx = 0;
  int ns = 0, nl = 0;
  if (nseed < 0) {
    cur = ctx->d_allrows;
    ns = ctx->nshort_all;
    nl = ctx->nlong_all;
    ctx->h_ctr[0] = ns;
    ctx->h_ctr[1] = 0;
    ctx->h_ctr[2] = nl;
    ctx->h_ctr[3] = 0;
    CK(cudaMemcpyAsync(ctx->d_ctr, ctx->h_ctr, 4 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  } else {
    cur = ctx->d_list[0];
    if (nseed > 0) {
      Front F{cur, ctx->d_ctr + 0, ctx->d_ctr + 2, ctx->d_rowstamp, (int)ctx->m};
      CK(launchSeed(ctx->stream, gridFor(ctx, nseed), P, lb, ub, nseed, d_seedcols, d_oldlb, d_oldub, F,
                    nextStamp(ctx)));
      ++launches;
    }
    CK(cudaMemcpyAsync(ctx->h_ctr, ctx->d_ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ns = ctx->h_ctr[0];
    nl = ctx->h_ctr[2];
  }

  int rounds = 0, status = 0;
  bool cut = false;
  while (ns + nl > 0) {
    if (rounds >= maxrounds) {
      status = 2;
      break;
    }
    const int nxt = curidx ^ 1;
    int* nextlist = ctx->d_list[nxt];  // the current list is d_list[curidx] or the all-rows list
    // reset next counters and the touched count
    CK(cudaMemsetAsync(ctx->d_ctr + nxt, 0, sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_ctr + 2 + nxt, 0, sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_ctr + 4, 0, sizeof(int), ctx->stream));
    C.round = rounds;
    if (ns > 0) {
      CK(launchRowsShort(ctx->stream, gridFor(ctx, ns, 128), s, P, lb, ub, cur, ctx->d_ctr + curidx, C, ctx->d_ctr + 5,
                         ctx->d_stats));
      ++launches;
    }
    if (nl > 0) {
      CK(launchRowsLong(ctx->stream, gridFor(ctx, (int64_t)nl * 32), s, P, lb, ub, cur, ctx->d_ctr + 2 + curidx,
                        (int)ctx->m, C, ctx->d_ctr + 5, ctx->d_stats));
      ++launches;
    }
    Front F{nextlist, ctx->d_ctr + nxt, ctx->d_ctr + 2 + nxt, ctx->d_rowstamp, (int)ctx->m};
    CK(launchApply(ctx->stream, gridFor(ctx, ctx->n, 256, 8), s, P, lb, ub, C, F, nextStamp(ctx), ctx->d_ctr + 5,
                   ctx->d_stats, ctx->log, rounds));
    ++launches;
    CK(cudaMemcpyAsync(ctx->h_ctr, ctx->d_ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ++rounds;
    if (ctx->h_ctr[5]) {
      cut = true;
      status = 1;
      break;
    }
    cur = nextlist;
    curidx = nxt;
    ns = ctx->h_ctr[nxt];
    nl = ctx->h_ctr[2 + nxt];
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  unsigned long long st[8];
  CK(cudaMemcpyAsync(st, ctx->d_stats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (cutoff) *cutoff = cut ? 1 : 0;
  if (res) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->cutoff = cut ? 1 : 0;
    res->rounds = rounds;
    res->status = status;
    res->launches = launches;
    res->rows = (int64_t)st[0];
    res->nnz = (int64_t)st[1];
    res->candidates = (int64_t)st[2];
    res->changes = (int64_t)st[3];
    res->live_rows = (int64_t)st[6];
    res->kernel_ms = ms;
  }
  return status == 2 ? GBP_ERR_LIMIT : GBP_OK;
}

static int ensureSeedBuf(gbp_ctx* ctx, int64_t nseed) {
  if (nseed <= ctx->seedcap) return GBP_OK;
  if (ctx->d_seedcols) cudaFree(ctx->d_seedcols);
  if (ctx->d_seedold) cudaFree(ctx->d_seedold);
  ctx->d_seedcols = nullptr;
  ctx->d_seedold = nullptr;
  ctx->seedcap = 0;
  CK(cudaMalloc(&ctx->d_seedcols, nseed * sizeof(int32_t)));
  CK(cudaMalloc(&ctx->d_seedold, 2 * nseed * sizeof(double)));
  ctx->seedcap = nseed;
  return GBP_OK;
}

static int checkSeeds(gbp_ctx* ctx, int64_t nseed, const int32_t* cols, const double* oldlb, const double* oldub) {
  if (nseed > 0 && (!cols || !oldlb || !oldub)) return fail(ctx, GBP_ERR_INVALID, "null seed arrays");
  return GBP_OK;
}

int gbp_propagate(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* seedcols, const double* oldlb,
                  const double* oldub, int32_t* cutoff, gbp_result* res) {
  if (!ctx || !ctx->has_problem || !lb || !ub) return fail(ctx, GBP_ERR_INVALID, "no problem or null bounds");
  int rc = checkSeeds(ctx, nseed, seedcols, oldlb, oldub);
  if (rc) return rc;
  for (int64_t k = 0; k < nseed; ++k)
    if (seedcols[k] < 0 || seedcols[k] >= ctx->n) return fail(ctx, GBP_ERR_INVALID, "seed column out of range");
  CK(cudaSetDevice(ctx->device));
  ctx->bounds_set = false;  // the device bound arrays are this call's scratch
  const size_t nb = (size_t)ctx->n * sizeof(double);
  if (nb) {
    CK(cudaMemcpyAsync(ctx->d_lb, lb, nb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_ub, ub, nb, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (nseed > 0) {
    rc = ensureSeedBuf(ctx, nseed);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_seedcols, seedcols, nseed * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_seedold, oldlb, nseed * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_seedold + nseed, oldub, nseed * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  rc = propagateCore(ctx, ctx->d_lb, ctx->d_ub, nseed, ctx->d_seedcols, ctx->d_seedold,
                     ctx->d_seedold + (nseed > 0 ? nseed : 0), cutoff, res);
  if (rc != GBP_OK && rc != GBP_ERR_LIMIT) return rc;
  if (nb) {
    CK(cudaMemcpyAsync(lb, ctx->d_lb, nb, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ub, ctx->d_ub, nb, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return rc;
}

// ------------------------------------------------------------------------------------------ sparse plain path
int gbp_set_bounds(gbp_ctx* ctx, const double* lb, const double* ub) {
  if (!ctx || !ctx->has_problem || ctx->instmode) return fail(ctx, GBP_ERR_INVALID, "no single problem uploaded");
  if (ctx->n > 0 && (!lb || !ub)) return fail(ctx, GBP_ERR_INVALID, "null bounds");
  CK(cudaSetDevice(ctx->device));
  const size_t nb = (size_t)ctx->n * sizeof(double);
  if (nb) {
    CK(cudaMemcpyAsync(ctx->d_lb, lb, nb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_ub, ub, nb, cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->bounds_set = true;
  return GBP_OK;
}

// moved-column lists of capacity cap: columns, then (256-byte aligned) lower and upper bounds
static size_t movedLbOffset(int64_t cap) { return ((size_t)cap * sizeof(int32_t) + 255) & ~size_t(255); }

// scratch of the sparse call: snapshot, change bounds, moved-column lists and their counter
static int ensureSparseBufs(gbp_ctx* ctx, int64_t nchg, int64_t cap) {
  if (!ctx->d_snap && ctx->n > 0) CK(cudaMalloc(&ctx->d_snap, 2 * (size_t)ctx->n * sizeof(double)));
  if (!ctx->d_count) CK(cudaMalloc(&ctx->d_count, sizeof(unsigned long long)));
  if (nchg > ctx->chgcap) {
    if (ctx->d_chgb) cudaFree(ctx->d_chgb);
    ctx->d_chgb = nullptr;
    ctx->chgcap = 0;
    CK(cudaMalloc(&ctx->d_chgb, 2 * (size_t)nchg * sizeof(double)));
    ctx->chgcap = nchg;
  }
  if (cap > ctx->movedcap) {
    if (ctx->d_moved) cudaFree(ctx->d_moved);
    ctx->d_moved = nullptr;
    ctx->movedcap = 0;
    CK(cudaMalloc(&ctx->d_moved, movedLbOffset(cap) + 2 * (size_t)cap * sizeof(double)));
    ctx->movedcap = cap;
  }
  return ensureSeedBuf(ctx, std::max<int64_t>(nchg, 1));
}

static int sparseGrid(gbp_ctx* ctx) {
  if (ctx->sparse_grid < 0) {
    int ok = 0, per = 0;
    if (cudaDeviceGetAttribute(&ok, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !ok ||
        sparseCoopOccupancy(&per) != cudaSuccess || per < 1) {
      cudaGetLastError();
      ctx->sparse_grid = 0;
    } else {
      ctx->sparse_grid = per * ctx->sms;
    }
  }
  return ctx->sparse_grid;
}

// gbp_propagate_changes as one copy in, one cooperative launch (k_sparse_coop) and one copy out: the same changes,
// seeds, rounds and moved-column report as the multi-launch path below, without its snapshot of every bound
static int propagateChangesCoop(gbp_ctx* ctx, int64_t nchg, const int32_t* cols, const double* newlb,
                                const double* newub, const double* seedlb, const double* seedub, int64_t cap,
                                int64_t* nout, int32_t* outcols, double* outlb, double* outub, int32_t* cutoff,
                                gbp_result* res) {
  const int64_t n = ctx->n;
  if (!ctx->d_mcount) CK(cudaMalloc(&ctx->d_mcount, sizeof(int)));
  if (n > ctx->mcap) {  // sized by the problem's columns: a later, larger upload grows them
    void* dp[] = {ctx->d_mstamp, ctx->d_mcol, ctx->d_mlb, ctx->d_mub};
    for (void* q : dp)
      if (q) cudaFree(q);
    ctx->d_mstamp = nullptr;
    ctx->d_mcol = nullptr;
    ctx->d_mlb = ctx->d_mub = nullptr;
    ctx->mcap = 0;
    CK(cudaMalloc(&ctx->d_mstamp, (size_t)n * sizeof(int)));
    CK(cudaMemsetAsync(ctx->d_mstamp, 0, (size_t)n * sizeof(int), ctx->stream));
    CK(cudaMalloc(&ctx->d_mcol, (size_t)n * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->d_mlb, (size_t)n * sizeof(double)));
    CK(cudaMalloc(&ctx->d_mub, (size_t)n * sizeof(double)));
    ctx->mcap = n;
    ctx->mepoch = 0;
  }
  const size_t inb = (size_t)nchg * (4 * sizeof(double) + sizeof(int32_t));
  if (inb > ctx->sin_bytes) {
    if (ctx->d_sin) cudaFree(ctx->d_sin);
    if (ctx->h_sin) cudaFreeHost(ctx->h_sin);
    ctx->d_sin = ctx->h_sin = nullptr;
    ctx->sin_bytes = 0;
    const size_t want = std::max<size_t>(inb, 64 << 10);
    CK(cudaMalloc(&ctx->d_sin, want));
    CK(cudaMallocHost(&ctx->h_sin, want));
    ctx->sin_bytes = want;
  }
  const int64_t outcap = std::max<int64_t>(cap, 1);
  if (outcap > ctx->sout_cap) {
    if (ctx->d_sout) cudaFree(ctx->d_sout);
    if (ctx->h_sout) cudaFreeHost(ctx->h_sout);
    ctx->d_sout = ctx->h_sout = nullptr;
    ctx->sout_cap = 0;
    const size_t bytes = SPARSE_HEADER + (size_t)outcap * sizeof(SparseOut);
    CK(cudaMalloc(&ctx->d_sout, bytes));
    CK(cudaMallocHost(&ctx->h_sout, bytes));
    ctx->sout_cap = outcap;
  }
  // the changes: lb, ub, seed (or scratch for the replaced bounds) lb, ub, columns -- one copy
  double* hd = (double*)ctx->h_sin;
  if (nchg > 0) {
    std::memcpy(hd, newlb, nchg * sizeof(double));
    std::memcpy(hd + nchg, newub, nchg * sizeof(double));
    if (seedlb) {
      std::memcpy(hd + 2 * nchg, seedlb, nchg * sizeof(double));
      std::memcpy(hd + 3 * nchg, seedub, nchg * sizeof(double));
    }
    std::memcpy(hd + 4 * nchg, cols, nchg * sizeof(int32_t));
    CK(cudaMemcpyAsync(ctx->d_sin, ctx->h_sin, inb, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (++ctx->mepoch >= 0x7ffffff0) {
    if (ctx->mcap > 0) CK(cudaMemsetAsync(ctx->d_mstamp, 0, (size_t)ctx->mcap * sizeof(int), ctx->stream));
    ctx->mepoch = 1;
  }
  const int maxrounds = ctx->par.maxrounds > 0 ? ctx->par.maxrounds : 1000000;
  if ((int64_t)ctx->stamp > (int64_t)0x7fffffff - maxrounds - 16) {
    CK(cudaMemsetAsync(ctx->d_rowstamp, 0, (size_t)std::max<int64_t>(ctx->m, 1) * sizeof(int), ctx->stream));
    ctx->stamp = 0;
  }
  SparseArgs A{};
  A.s = ctx->num;
  A.P = devProb(ctx, false);
  A.C = plainCands(ctx);
  A.C.ntouched = &ctx->d_state->ntouched;
  A.L = ListSet{{ctx->d_list[0], ctx->d_list[1], ctx->d_allrows}, ctx->d_rowstamp, (int)ctx->m};
  A.S = ctx->d_state;
  std::memset(&A.init, 0, sizeof(A.init));
  A.init.maxrounds = maxrounds;
  A.init.lb = ctx->d_lb;
  A.init.ub = ctx->d_ub;
  A.init.log = ctx->log;
  A.seedstamp = ++ctx->stamp;
  A.init.stamp = ++ctx->stamp;
  A.stats = ctx->d_stats;
  A.lb = ctx->d_lb;
  A.ub = ctx->d_ub;
  A.nchg = nchg;
  double* dd = (double*)ctx->d_sin;
  A.nlb = dd;
  A.nub = dd + nchg;
  A.oldlb = dd + 2 * nchg;
  A.oldub = dd + 3 * nchg;
  A.cols = (const int32_t*)(dd + 4 * nchg);
  A.keepold = seedlb != nullptr;
  A.moved = MovedLog{ctx->d_mstamp, ctx->mepoch, ctx->d_mcount, ctx->d_mcol, ctx->d_mlb, ctx->d_mub};
  A.cap = cap;
  A.header = (int*)ctx->d_sout;
  A.out = (SparseOut*)(ctx->d_sout + SPARSE_HEADER);
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launchSparseCoop(ctx->stream, sparseGrid(ctx), A));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  // the header and a first stretch of moved columns in one copy; the rest (rare) in a second
  const int64_t first = std::min<int64_t>(cap, 2048);
  CK(cudaMemcpyAsync(ctx->h_sout, ctx->d_sout, SPARSE_HEADER + (size_t)first * sizeof(SparseOut),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const int* h = (const int*)ctx->h_sout;
  const unsigned long long* st = (const unsigned long long*)(ctx->h_sout + 8 * sizeof(int));
  const bool cut = h[0] != 0;
  const int status = cut ? 1 : (h[1] == 2 ? 2 : 0);
  const int64_t cnt = h[4];
  ctx->stamp = std::max(ctx->stamp, h[3]);
  if (res) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->cutoff = cut ? 1 : 0;
    res->rounds = h[2];
    res->status = status;
    res->launches = 1;
    res->rows = (int64_t)st[0];
    res->nnz = (int64_t)st[1];
    res->candidates = (int64_t)st[2];
    res->changes = (int64_t)st[3];
    res->live_rows = (int64_t)st[6];
    res->kernel_ms = ms;
  }
  const int rc = status == 2 ? GBP_ERR_LIMIT : GBP_OK;
  if (cut) {  // the kernel put the bounds back to the caller's changes
    *cutoff = 1;
    return rc;
  }
  *nout = cnt;
  if (cnt > cap) return fail(ctx, GBP_ERR_OVERFLOW, "moved-column arrays too small (nout is the count needed)");
  const SparseOut* o = (const SparseOut*)(ctx->h_sout + SPARSE_HEADER);
  if (cnt > first) {
    CK(cudaMemcpyAsync(ctx->h_sout + SPARSE_HEADER + (size_t)first * sizeof(SparseOut),
                       ctx->d_sout + SPARSE_HEADER + (size_t)first * sizeof(SparseOut),
                       (size_t)(cnt - first) * sizeof(SparseOut), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  std::vector<int32_t> idx((size_t)cnt);
  for (int64_t q = 0; q < cnt; ++q) idx[q] = (int32_t)q;
  std::sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return o[a].col < o[b].col; });
  for (int64_t q = 0; q < cnt; ++q) {
    outcols[q] = o[idx[q]].col;
    outlb[q] = o[idx[q]].lb;
    outub[q] = o[idx[q]].ub;
  }
  return rc;
}

int gbp_propagate_changes(gbp_ctx* ctx, int64_t nchg, const int32_t* cols, const double* newlb, const double* newub,
                          const double* seedlb, const double* seedub, int64_t cap, int64_t* nout, int32_t* outcols,
                          double* outlb, double* outub, int32_t* cutoff, gbp_result* res) {
  if (!ctx || !ctx->has_problem || ctx->instmode) return fail(ctx, GBP_ERR_INVALID, "no single problem uploaded");
  if (!ctx->bounds_set) return fail(ctx, GBP_ERR_INVALID, "gbp_set_bounds first");
  if (nchg < 0 || cap < 0 || !nout || !cutoff) return fail(ctx, GBP_ERR_INVALID, "bad sizes or null outputs");
  if (nchg > 0 && (!cols || !newlb || !newub)) return fail(ctx, GBP_ERR_INVALID, "null change arrays");
  if ((seedlb == nullptr) != (seedub == nullptr)) return fail(ctx, GBP_ERR_INVALID, "give both seed arrays or neither");
  if (cap > 0 && (!outcols || !outlb || !outub)) return fail(ctx, GBP_ERR_INVALID, "null output arrays");
  *nout = 0;
  *cutoff = 0;
  if (res) std::memset(res, 0, sizeof(*res));
  for (int64_t k = 0; k < nchg; ++k) {
    if (cols[k] < 0 || cols[k] >= ctx->n) return fail(ctx, GBP_ERR_INVALID, "change column out of range");
    if (newlb[k] > newub[k]) {  // an empty domain: infeasible before any row is looked at
      *cutoff = 1;
      if (res) res->cutoff = 1, res->status = 1;
      return GBP_OK;
    }
  }
  CK(cudaSetDevice(ctx->device));
  if (!rangedOn(ctx) && !(ctx->par.flags & GBP_FLAG_HOSTLOOP) && sparseGrid(ctx) > 0)
    return propagateChangesCoop(ctx, nchg, cols, newlb, newub, seedlb, seedub, cap, nout, outcols, outlb, outub,
                                cutoff, res);
  int rc = ensureSparseBufs(ctx, nchg, cap);
  if (rc) return rc;
  const int64_t n = ctx->n;
  const size_t nb = (size_t)n * sizeof(double);
  double* slb = ctx->d_snap;
  double* sub = ctx->d_snap + n;
  if (nchg > 0) {
    CK(cudaMemcpyAsync(ctx->d_seedcols, cols, nchg * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_chgb, newlb, nchg * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_chgb + nchg, newub, nchg * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (seedlb) {
      CK(cudaMemcpyAsync(ctx->d_seedold, seedlb, nchg * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaMemcpyAsync(ctx->d_seedold + nchg, seedub, nchg * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(launchSetChanges(ctx->stream, gridFor(ctx, nchg), nchg, ctx->d_seedcols, ctx->d_chgb, ctx->d_chgb + nchg,
                        ctx->d_lb, ctx->d_ub, ctx->d_seedold, ctx->d_seedold + nchg, seedlb != nullptr));
  }
  if (nb) {
    CK(cudaMemcpyAsync(slb, ctx->d_lb, nb, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(sub, ctx->d_ub, nb, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  auto restore = [&]() -> int {  // back to the bounds after the caller's changes
    if (nb) {
      CK(cudaMemcpyAsync(ctx->d_lb, slb, nb, cudaMemcpyDeviceToDevice, ctx->stream));
      CK(cudaMemcpyAsync(ctx->d_ub, sub, nb, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return GBP_OK;
  };
  rc = propagateCore(ctx, ctx->d_lb, ctx->d_ub, nchg, ctx->d_seedcols, ctx->d_seedold, ctx->d_seedold + nchg, cutoff,
                     res);
  if (rc != GBP_OK && rc != GBP_ERR_LIMIT) {
    restore();
    return rc;
  }
  if (*cutoff) {
    const int r2 = restore();
    return r2 ? r2 : rc;
  }
  // the columns that propagation moved, against the snapshot
  int32_t* mcols = (int32_t*)ctx->d_moved;
  double* mlb = (double*)(ctx->d_moved + movedLbOffset(ctx->movedcap));
  double* mub = mlb + ctx->movedcap;
  CK(cudaMemsetAsync(ctx->d_count, 0, sizeof(unsigned long long), ctx->stream));
  if (n > 0)
    CK(launchMoved(ctx->stream, gridFor(ctx, n), n, ctx->d_lb, ctx->d_ub, slb, sub, ctx->d_count, cap, mcols, mlb,
                   mub));
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, ctx->d_count, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *nout = (int64_t)cnt;
  if ((int64_t)cnt > cap) {  // the caller retries with room for *nout columns from the same state
    const int r2 = restore();
    return r2 ? r2 : fail(ctx, GBP_ERR_OVERFLOW, "moved-column arrays too small (nout is the count needed)");
  }
  if (cnt > 0) {
    std::vector<int32_t> c(cnt);
    std::vector<double> l(cnt), u(cnt);
    CK(cudaMemcpyAsync(c.data(), mcols, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(l.data(), mlb, cnt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(u.data(), mub, cnt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::vector<int64_t> idx(cnt);
    for (size_t q = 0; q < cnt; ++q) idx[q] = (int64_t)q;
    std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return c[a] < c[b]; });
    for (size_t q = 0; q < cnt; ++q) {
      outcols[q] = c[idx[q]];
      outlb[q] = l[idx[q]];
      outub[q] = u[idx[q]];
    }
  }
  return rc;
}

int gbp_propagate_device(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* seedcols,
                         const double* oldlb, const double* oldub, int32_t* cutoff, gbp_result* res) {
  if (!ctx || !ctx->has_problem || (ctx->n > 0 && (!lb || !ub)))
    return fail(ctx, GBP_ERR_INVALID, "no problem or null bounds");
  int rc = checkSeeds(ctx, nseed, seedcols, oldlb, oldub);
  if (rc) return rc;
  CK(cudaSetDevice(ctx->device));
  return propagateCore(ctx, lb, ub, nseed, seedcols, oldlb, oldub, cutoff, res);
}

int gbp_row_activities(gbp_ctx* ctx, const double* lb, const double* ub, double* act, int32_t* cnt) {
  if (!ctx || !ctx->has_problem || !lb || !ub || !act || !cnt) return fail(ctx, GBP_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  const size_t nb = (size_t)ctx->n * sizeof(double);
  const size_t m = (size_t)ctx->m;
  double* d_act = nullptr;
  int32_t* d_cnt = nullptr;
  CK(cudaMalloc(&d_act, std::max<size_t>(m, 1) * 4 * sizeof(double)));
  CK(cudaMalloc(&d_cnt, std::max<size_t>(m, 1) * 8 * sizeof(int32_t)));
  ctx->bounds_set = false;  // the device bound arrays are this call's scratch
  if (nb) {
    CK(cudaMemcpyAsync(ctx->d_lb, lb, nb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_ub, ub, nb, cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(launchActivities(ctx->stream, gridFor(ctx, (int64_t)m, 256, 8), ctx->num, devProb(ctx), ctx->d_lb, ctx->d_ub,
                      d_act, d_cnt));
  if (m) {
    CK(cudaMemcpyAsync(act, d_act, m * 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(cnt, d_cnt, m * 8 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(d_act);
  cudaFree(d_cnt);
  return GBP_OK;
}

int gbp_set_global_bounds(gbp_ctx* ctx, const double* glb, const double* gub) {
  if (!ctx || !ctx->has_problem) return fail(ctx, GBP_ERR_INVALID, "no problem uploaded");
  if ((glb == nullptr) != (gub == nullptr)) return fail(ctx, GBP_ERR_INVALID, "give both global bound arrays or none");
  CK(cudaSetDevice(ctx->device));
  destroyGraphs(ctx);  // the graphs hold the problem's pointers, including these
  if (glb == nullptr) {
    ctx->has_global = false;
    return GBP_OK;
  }
  const int64_t nn = std::max<int64_t>(ctx->n, 1);
  if (nn > ctx->cap_glob) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->d_glb) cudaFree(ctx->d_glb);
    if (ctx->d_gub) cudaFree(ctx->d_gub);
    ctx->d_glb = ctx->d_gub = nullptr;
    ctx->cap_glob = 0;
    CK(cudaMalloc(&ctx->d_glb, nn * sizeof(double)));
    CK(cudaMalloc(&ctx->d_gub, nn * sizeof(double)));
    ctx->cap_glob = nn;
  }
  if (ctx->n) {
    CK(cudaMemcpyAsync(ctx->d_glb, glb, ctx->n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_gub, gub, ctx->n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));  // the host arrays may go away after the call
  ctx->has_global = true;
  return GBP_OK;
}

int gbp_set_change_log(gbp_ctx* ctx, int64_t capacity) {
  if (!ctx || capacity < 0 || capacity >= (int64_t(1) << 31)) return fail(ctx, GBP_ERR_INVALID, "bad log capacity");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  destroyGraphs(ctx);  // the graphs hold the ranged-row records' pointers
  void* lp[] = {ctx->log.n, ctx->log.col, ctx->log.round, ctx->log.lb, ctx->log.ub,
                ctx->rlog.n, ctx->rlog.row, ctx->rlog.col, ctx->rlog.round};
  for (void* p : lp)
    if (p) cudaFree(p);
  ctx->log = ChangeLog{};
  ctx->rlog = RangedLog{};
  ctx->log_cap = 0;
  if (capacity == 0) return GBP_OK;
  ChangeLog G{};
  G.cap = capacity;
  CK(cudaMalloc(&G.n, sizeof(int)));
  CK(cudaMalloc(&G.col, capacity * sizeof(int32_t)));
  CK(cudaMalloc(&G.round, capacity * sizeof(int32_t)));
  CK(cudaMalloc(&G.lb, capacity * sizeof(double)));
  CK(cudaMalloc(&G.ub, capacity * sizeof(double)));
  CK(cudaMemset(G.n, 0, sizeof(int)));
  ctx->log = G;
  RangedLog R{};
  R.cap = capacity;
  CK(cudaMalloc(&R.n, sizeof(int)));
  CK(cudaMalloc(&R.row, capacity * sizeof(int32_t)));
  CK(cudaMalloc(&R.col, capacity * sizeof(int32_t)));
  CK(cudaMalloc(&R.round, capacity * sizeof(int32_t)));
  CK(cudaMemset(R.n, 0, sizeof(int)));
  ctx->rlog = R;
  ctx->log_cap = capacity;
  return GBP_OK;
}

int gbp_get_ranged_log(gbp_ctx* ctx, int64_t cap, int32_t* round, int32_t* col, int32_t* row, int64_t* n) {
  if (!ctx || !n || cap < 0 || (cap > 0 && (!round || !col || !row))) return fail(ctx, GBP_ERR_INVALID, "null argument");
  *n = 0;
  if (!ctx->rlog.n) return fail(ctx, GBP_ERR_STATE, "no change log (gbp_set_change_log)");
  CK(cudaSetDevice(ctx->device));
  int cnt = 0;
  CK(cudaMemcpyAsync(&cnt, ctx->rlog.n, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *n = cnt;
  const int64_t have = std::min<int64_t>(cnt, ctx->log_cap);
  std::vector<int32_t> w(have), c(have), r(have);
  if (have > 0) {
    CK(cudaMemcpyAsync(w.data(), ctx->rlog.round, have * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(c.data(), ctx->rlog.col, have * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(r.data(), ctx->rlog.row, have * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  // records in (round, column, row) order: the threads of a round append in any order
  std::vector<int64_t> ord(have);
  for (int64_t k = 0; k < have; ++k) ord[k] = k;
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
    if (w[a] != w[b]) return w[a] < w[b];
    if (c[a] != c[b]) return c[a] < c[b];
    return r[a] < r[b];
  });
  const int64_t out = std::min<int64_t>(have, cap);
  for (int64_t k = 0; k < out; ++k) {
    round[k] = w[ord[k]];
    col[k] = c[ord[k]];
    row[k] = r[ord[k]];
  }
  if (cnt > ctx->log_cap) return fail(ctx, GBP_ERR_OVERFLOW, "change log capacity exceeded");
  if (cnt > cap) return fail(ctx, GBP_ERR_OVERFLOW, "output arrays too small for the ranged-row records");
  return GBP_OK;
}

int gbp_get_change_log(gbp_ctx* ctx, int64_t cap, int32_t* col, int32_t* round, double* lb, double* ub, int64_t* n) {
  if (!ctx || !n || cap < 0 || (cap > 0 && (!col || !round || !lb || !ub)))
    return fail(ctx, GBP_ERR_INVALID, "null argument");
  *n = 0;
  if (!ctx->log.n) return fail(ctx, GBP_ERR_STATE, "no change log (gbp_set_change_log)");
  CK(cudaSetDevice(ctx->device));
  int cnt = 0;
  CK(cudaMemcpyAsync(&cnt, ctx->log.n, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *n = cnt;
  const int64_t have = std::min<int64_t>(cnt, ctx->log_cap);
  std::vector<int32_t> c(have), r(have);
  std::vector<double> l(have), u(have);
  if (have > 0) {
    CK(cudaMemcpyAsync(c.data(), ctx->log.col, have * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(r.data(), ctx->log.round, have * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(l.data(), ctx->log.lb, have * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(u.data(), ctx->log.ub, have * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  // device order within a round depends on scheduling: report by (round, column)
  std::vector<int64_t> ord(have);
  for (int64_t k = 0; k < have; ++k) ord[k] = k;
  std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return r[a] != r[b] ? r[a] < r[b] : c[a] < c[b]; });
  const int64_t out = std::min<int64_t>(have, cap);
  for (int64_t k = 0; k < out; ++k) {
    col[k] = c[ord[k]];
    round[k] = r[ord[k]];
    lb[k] = l[ord[k]];
    ub[k] = u[ord[k]];
  }
  if (cnt > ctx->log_cap) return fail(ctx, GBP_ERR_OVERFLOW, "change log capacity exceeded");
  if (cnt > cap) return fail(ctx, GBP_ERR_OVERFLOW, "output arrays too small for the change log");
  return GBP_OK;
}

// ------------------------------------------------------------------------------------------ instances
int gbp_upload_instances(gbp_ctx* ctx, int64_t ninst, const int64_t* row_off, const int64_t* col_off,
                         const int64_t* rowptr, const int32_t* colidx, const double* vals, const double* lhs,
                         const double* rhs, const int8_t* isint) {
  if (!ctx || ninst < 1 || !row_off || !col_off || !rowptr) return fail(ctx, GBP_ERR_INVALID, "null argument");
  if (ninst >= (int64_t(1) << 31) - 1) return fail(ctx, GBP_ERR_INVALID, "too many instances");
  if (row_off[0] != 0 || col_off[0] != 0) return fail(ctx, GBP_ERR_INVALID, "offsets must start at 0");
  for (int64_t k = 0; k < ninst; ++k)
    if (row_off[k + 1] < row_off[k] || col_off[k + 1] < col_off[k])
      return fail(ctx, GBP_ERR_INVALID, "instance offsets not monotone");
  const int64_t m = row_off[ninst], n = col_off[ninst];
  std::vector<int32_t> rowinst(std::max<int64_t>(m, 1)), colinst(std::max<int64_t>(n, 1));
  for (int64_t k = 0; k < ninst; ++k) {
    for (int64_t i = row_off[k]; i < row_off[k + 1]; ++i) rowinst[i] = (int32_t)k;
    for (int64_t j = col_off[k]; j < col_off[k + 1]; ++j) colinst[j] = (int32_t)k;
  }
  int rc = gbp_upload_problem(ctx, m, n, rowptr, colidx, vals, lhs, rhs, isint);
  if (rc != GBP_OK) return rc;
  rc = prepareInstanceMaps(ctx, ninst);
  if (rc != GBP_OK) return rc;
  CK(cudaMemcpyAsync(ctx->d_rowinst, rowinst.data(), rowinst.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_colinst, colinst.data(), colinst.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  // rows may only reference columns of their own instance (checked on the device)
  CK(cudaMemsetAsync(ctx->d_ctr + 7, 0, sizeof(int), ctx->stream));
  if (m) CK(launchCheckBlocks(ctx->stream, gridFor(ctx, m), m, ctx->d_rowptr, ctx->d_colidx, ctx->d_rowinst,
                              ctx->d_colinst, ctx->d_ctr + 7));
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, ctx->d_ctr + 7, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (bad) {
    freeProblem(ctx);
    return fail(ctx, GBP_ERR_INVALID, "a row references a column of another instance");
  }
  ctx->ninst = ninst;
  return GBP_OK;
}

int gbp_upload_instance_list(gbp_ctx* ctx, int64_t ninst, const int64_t* m_k, const int64_t* n_k,
                             const int64_t* const* rowptr_k, const int32_t* const* colidx_k,
                             const double* const* vals_k, const double* const* lhs_k, const double* const* rhs_k,
                             const int8_t* const* isint_k) {
  if (!ctx || ninst < 1 || !m_k || !n_k || !rowptr_k || !colidx_k || !vals_k || !lhs_k || !rhs_k || !isint_k)
    return fail(ctx, GBP_ERR_INVALID, "null argument");
  if (ninst >= (int64_t(1) << 31) - 1) return fail(ctx, GBP_ERR_INVALID, "too many instances");
  // offsets: [row_off | col_off | nnz_off], ninst + 1 entries each
  std::vector<int64_t> off(3 * (ninst + 1) + 1);
  int64_t* row_off = off.data();
  int64_t* col_off = row_off + ninst + 1;
  int64_t* nnz_off = col_off + ninst + 1;
  row_off[0] = col_off[0] = nnz_off[0] = 0;
  for (int64_t k = 0; k < ninst; ++k) {
    const int64_t mk = m_k[k], nk = n_k[k];
    const int64_t* rp = rowptr_k[k];
    if (mk < 0 || nk < 0 || !rp || (mk > 0 && (!lhs_k[k] || !rhs_k[k])) || (nk > 0 && !isint_k[k]))
      return fail(ctx, GBP_ERR_INVALID, "null part or negative part size");
    if (rp[0] != 0) return fail(ctx, GBP_ERR_INVALID, "a part's rowptr[0] must be 0");
    for (int64_t i = 0; i < mk; ++i)
      if (rp[i + 1] < rp[i]) return fail(ctx, GBP_ERR_INVALID, "a part's rowptr is not monotone");
    if (rp[mk] > 0 && (!colidx_k[k] || !vals_k[k])) return fail(ctx, GBP_ERR_INVALID, "null part colidx/vals");
    row_off[k + 1] = row_off[k] + mk;
    col_off[k + 1] = col_off[k] + nk;
    nnz_off[k + 1] = nnz_off[k] + rp[mk];
  }
  const int64_t m = row_off[ninst], n = col_off[ninst], nnz = nnz_off[ninst];
  if (m >= (int64_t(1) << 30) || n >= (int64_t(1) << 31) - 1)
    return fail(ctx, GBP_ERR_INVALID, "problem too large (m < 2^30, n < 2^31 required)");

  int rc = prepareUpload(ctx, m, n, nnz);
  if (rc != GBP_OK) return rc;
  rc = prepareInstanceMaps(ctx, ninst);
  if (rc != GBP_OK) return rc;
  std::vector<int> allrows(std::max<int64_t>(m, 1));
  int ns = 0, nl = 0;
  for (int64_t k = 0; k < ninst; ++k) {
    const int64_t* rp = rowptr_k[k];
    for (int64_t i = 0; i < m_k[k]; ++i) {
      if (rp[i + 1] - rp[i] <= LONGROW) allrows[ns++] = (int)(row_off[k] + i);
      else allrows[m - 1 - nl++] = (int)(row_off[k] + i);
    }
  }
  // each part straight to its place; the last row pointer is the total
  for (int64_t k = 0; k < ninst; ++k) {
    const int64_t mk = m_k[k], nk = n_k[k], zk = nnz_off[k + 1] - nnz_off[k];
    if (mk) {
      CK(cudaMemcpyAsync(ctx->d_rowptr + row_off[k], rowptr_k[k], mk * sizeof(int64_t), cudaMemcpyHostToDevice,
                         ctx->stream));
      CK(cudaMemcpyAsync(ctx->d_lhs + row_off[k], lhs_k[k], mk * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaMemcpyAsync(ctx->d_rhs + row_off[k], rhs_k[k], mk * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    if (zk) {
      CK(cudaMemcpyAsync(ctx->d_colidx + nnz_off[k], colidx_k[k], zk * sizeof(int32_t), cudaMemcpyHostToDevice,
                         ctx->stream));
      CK(cudaMemcpyAsync(ctx->d_vals + nnz_off[k], vals_k[k], zk * sizeof(double), cudaMemcpyHostToDevice,
                         ctx->stream));
    }
    if (nk) CK(cudaMemcpyAsync(ctx->d_isint + col_off[k], isint_k[k], nk, cudaMemcpyHostToDevice, ctx->stream));
  }
  CK(cudaMemcpyAsync(ctx->d_rowptr + m, &nnz_off[ninst], sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  if (m) CK(cudaMemcpyAsync(ctx->d_allrows, allrows.data(), m * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  int64_t* d_off = nullptr;
  const size_t offbytes = off.size() * sizeof(int64_t);
  CK(cudaMallocAsync((void**)&d_off, offbytes, ctx->stream));
  CK(cudaMemcpyAsync(d_off, off.data(), offbytes, cudaMemcpyHostToDevice, ctx->stream));
  int* d_bad = (int*)(d_off + 3 * (ninst + 1));
  CK(cudaMemsetAsync(d_bad, 0, sizeof(int64_t), ctx->stream));
  CK(launchFixParts(ctx->stream, gridFor(ctx, std::max(std::max(m, n), nnz)), ninst, d_off, m, n, nnz, ctx->d_rowptr,
                    ctx->d_colidx, ctx->d_rowinst, ctx->d_colinst, d_bad));
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaFreeAsync(d_off, ctx->stream));
  rc = finishUpload(ctx, m, n, nnz, ns, nl);  // synchronises the stream
  if (rc != GBP_OK) return rc;
  if (bad) {
    freeProblem(ctx);
    return fail(ctx, GBP_ERR_INVALID, "a part's column index is outside its part");
  }
  ctx->ninst = ninst;
  return GBP_OK;
}

static int propagateInstances(gbp_ctx* ctx, double* lb, double* ub, int8_t* inst_cutoff, bool host, gbp_result* res) {
  if (!ctx || !ctx->has_problem || ctx->ninst < 1 || !lb || !ub || !inst_cutoff)
    return fail(ctx, GBP_ERR_INVALID, "no instances uploaded or null argument");
  CK(cudaSetDevice(ctx->device));
  const size_t nb = (size_t)ctx->n * sizeof(double);
  double* dlb = lb;
  double* dub = ub;
  if (host) {
    ctx->bounds_set = false;  // the device bound arrays are this call's scratch
    dlb = ctx->d_lb;
    dub = ctx->d_ub;
    if (nb) {
      CK(cudaMemcpyAsync(dlb, lb, nb, cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaMemcpyAsync(dub, ub, nb, cudaMemcpyHostToDevice, ctx->stream));
    }
  }
  CK(cudaMemsetAsync(ctx->d_instcut, 0, ctx->ninst * sizeof(int), ctx->stream));
  ctx->instmode = true;
  int32_t anycut = 0;
  int rc = propagateCore(ctx, dlb, dub, -1, nullptr, nullptr, nullptr, &anycut, res);
  ctx->instmode = false;
  if (rc != GBP_OK && rc != GBP_ERR_LIMIT) return rc;
  std::vector<int> cut(ctx->ninst);
  CK(cudaMemcpyAsync(cut.data(), ctx->d_instcut, ctx->ninst * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (host && nb) {
    CK(cudaMemcpyAsync(lb, dlb, nb, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ub, dub, nb, cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (!host)  // inst_cutoff is a device array: convert the flags on the device
    CK(launchFlags8(ctx->stream, gridFor(ctx, ctx->ninst), ctx->d_instcut, inst_cutoff, ctx->ninst));
  CK(cudaStreamSynchronize(ctx->stream));
  int ncut = 0;
  for (int64_t k = 0; k < ctx->ninst; ++k) {
    if (host) inst_cutoff[k] = cut[k] ? 1 : 0;
    ncut += cut[k] ? 1 : 0;
  }
  if (res) {
    res->cutoff = ncut;
    res->status = rc == GBP_ERR_LIMIT ? 2 : 0;
  }
  return rc;
}

int gbp_propagate_instances(gbp_ctx* ctx, double* lb, double* ub, int8_t* inst_cutoff, gbp_result* res) {
  return propagateInstances(ctx, lb, ub, inst_cutoff, true, res);
}

int gbp_propagate_instances_device(gbp_ctx* ctx, double* lb, double* ub, int8_t* inst_cutoff, gbp_result* res) {
  return propagateInstances(ctx, lb, ub, inst_cutoff, false, res);
}

// ------------------------------------------------------------------------------------------ batched path
// per-CTA scratch for min(resident CTAs, nnodes) slots; grown when a later call has more nodes
static int ensureSlots(gbp_ctx* ctx, int64_t nnodes) {
  int occ = 0;
  CK(nodesOccupancy(ctx->node_threads, ctx->ctas_per_sm, &occ));
  int per_sm = std::max(occ, 1);
  const int64_t want = std::min<int64_t>((int64_t)ctx->sms * per_sm, std::max<int64_t>(nnodes, 1));
  if (ctx->slot_mem && ctx->nslots >= want) return GBP_OK;
  if (ctx->slot_mem) {
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->slot_mem);
    ctx->slot_mem = nullptr;
    ctx->nslots = 0;
  }
  const int64_t ns = std::max<int64_t>(ctx->n, 1), ms = std::max<int64_t>(ctx->m, 1);
  const size_t per_slot = slotLayout(ns, ms, 1, nullptr, nullptr);
  size_t freeb = 0, totalb = 0;
  CK(cudaMemGetInfo(&freeb, &totalb));
  int64_t nslots = want;
  const size_t budget = freeb / 3;
  while (nslots > 1 && (size_t)nslots * per_slot > budget) nslots -= 1;
  if ((size_t)nslots * per_slot > budget) return fail(ctx, GBP_ERR_NOMEM, "not enough device memory for one slot");
  const size_t bytes = slotLayout(ns, ms, nslots, nullptr, nullptr);
  char* base = nullptr;
  CK(cudaMalloc(&base, bytes));
  ctx->slot_mem = base;
  SlotArrays& A = ctx->slots;
  slotLayout(ns, ms, nslots, base, &A);
  const size_t S = (size_t)nslots;
  CK(cudaMemsetAsync(A.ostamp, 0, S * ns * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(A.cflag, 0, S * ns * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(A.rowstamp, 0, S * ms * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(A.counter, 0, S * sizeof(int), ctx->stream));
  CK(launchFill64(ctx->stream, ctx->sms * 8, A.cub, (int64_t)(S * ns), KEY_NONE_UB));
  CK(launchFill64(ctx->stream, ctx->sms * 8, A.clb, (int64_t)(S * ns), KEY_NONE_LB));
  CK(launchFill64(ctx->stream, ctx->sms * 8, A.cubf, (int64_t)(S * ns), KEY_NONE_UB));
  CK(launchFill64(ctx->stream, ctx->sms * 8, A.clbf, (int64_t)(S * ns), KEY_NONE_LB));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->nslots = (int)nslots;
  ctx->slot_stamp_budget = 0;
  return GBP_OK;
}

// ------------------------------------------------------------------------------------------ SCIP's own order
// the column-major copy with each column's rows ascending and their coefficients (once per upload)
static int ensureSeqCsc(gbp_ctx* ctx) {
  if (ctx->seq_csc_ready) return GBP_OK;
  const int64_t zz = std::max<int64_t>(ctx->nnz, 1);
  if (zz > ctx->sq_cap_nnz) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->d_sq_crow) cudaFree(ctx->d_sq_crow);
    if (ctx->d_sq_cval) cudaFree(ctx->d_sq_cval);
    ctx->d_sq_crow = nullptr;
    ctx->d_sq_cval = nullptr;
    ctx->sq_cap_nnz = 0;
    CK(cudaMalloc(&ctx->d_sq_crow, ctx->cap_nnz * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->d_sq_cval, ctx->cap_nnz * sizeof(double)));
    ctx->sq_cap_nnz = ctx->cap_nnz;
  }
  if (ctx->cap_m > ctx->sq_cap_m) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->d_sq_prep) cudaFree(ctx->d_sq_prep);
    ctx->d_sq_prep = nullptr;
    CK(cudaMalloc(&ctx->d_sq_prep, ctx->cap_m * sizeof(int)));
    ctx->sq_cap_m = ctx->cap_m;
  }
  CK(launchSeqCsc(ctx->stream, gridFor(ctx, ctx->nnz), ctx->m, ctx->n, ctx->nnz, ctx->d_rowptr, ctx->d_colidx,
                  ctx->d_vals, ctx->d_sq_crow, ctx->d_sq_cval));
  ctx->seq_csc_ready = true;
  return GBP_OK;
}

// per-warp scratch for min(resident warps, nnodes) nodes at a time; grown when a later call has more nodes
static int ensureSeqSlots(gbp_ctx* ctx, int64_t nnodes) {
  int occ = 0;
  CK(nodesSeqOccupancy(&occ));
  const int64_t want = std::min<int64_t>((int64_t)ctx->sms * std::max(occ, 1) * SEQ_WARPS, std::max<int64_t>(nnodes, 1));
  if (ctx->seq_mem && ctx->seqslots.nslots >= want) return GBP_OK;
  if (ctx->seq_mem) {
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->seq_mem);
    ctx->seq_mem = nullptr;
    ctx->seqslots = SeqSlots{};
  }
  const int64_t ns = std::max<int64_t>(ctx->n, 1), ms = std::max<int64_t>(ctx->m, 1);
  const size_t per_slot = seqSlotLayout(ns, ms, 1, nullptr, nullptr);
  size_t freeb = 0, totalb = 0;
  CK(cudaMemGetInfo(&freeb, &totalb));
  int64_t nslots = want;
  const size_t budget = freeb / 3;
  while (nslots > 1 && (size_t)nslots * per_slot > budget) nslots -= 1;
  if ((size_t)nslots * per_slot > budget) return fail(ctx, GBP_ERR_NOMEM, "not enough device memory for one slot");
  const size_t bytes = seqSlotLayout(ns, ms, nslots, nullptr, nullptr);
  char* base = nullptr;
  CK(cudaMalloc(&base, bytes));
  ctx->seq_mem = base;
  SeqSlots& A = ctx->seqslots;
  seqSlotLayout(ns, ms, nslots, base, &A);
  const size_t S = (size_t)nslots;
  CK(cudaMemsetAsync(A.rows, 0, S * ms * sizeof(SeqRow), ctx->stream));
  CK(cudaMemsetAsync(A.ost, 0, S * ns * sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(A.counter, 0, S * sizeof(int), ctx->stream));
  ctx->seq_epoch_budget = 0;
  return GBP_OK;
}

static int propagateNodesSeq(gbp_ctx* ctx, const double* baselb, const double* baseub, int64_t nnodes,
                             const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
                             int8_t* out_cutoff, int32_t* out_rounds, int64_t* out_off, int32_t* out_n,
                             int32_t* out_col, double* out_lb, double* out_ub, int64_t out_cap, gbp_result* res) {
  if (rangedOn(ctx)) return fail(ctx, GBP_ERR_INVALID, "GBP_FLAG_SCIPORDER does not combine with GBP_FLAG_RANGEDROW");
  int rc = ensureSeqCsc(ctx);
  if (rc) return rc;
  // one CTA of SEQ_WARPS warps per SM: a node's logic is a long chain of dependent steps, and a warp that shares its
  // SM sub-partition with others waits on their FP64 and memory traffic -- the batch ends with its longest node,
  // so fewer, faster warps finish it sooner (and need fewer slots)
  const int64_t maxwarps = (int64_t)ctx->sms * SEQ_WARPS;
  rc = ensureSeqSlots(ctx, std::min<int64_t>(nnodes, maxwarps));
  if (rc) return rc;
  const SeqSlots& SL = ctx->seqslots;
  // every node takes a new epoch in its slot; re-zero the stamps long before a counter wraps
  if (ctx->seq_epoch_budget + nnodes > (int64_t(1) << 30)) {
    CK(cudaMemsetAsync(SL.rows, 0, (size_t)SL.nslots * SL.mstride * sizeof(SeqRow), ctx->stream));
    CK(cudaMemsetAsync(SL.ost, 0, (size_t)SL.nslots * SL.nstride * sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(SL.counter, 0, (size_t)SL.nslots * sizeof(int), ctx->stream));
    ctx->seq_epoch_budget = 0;
  }
  CK(cudaMemsetAsync(ctx->d_stats, 0, 8 * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_next_item, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_out_used, 0, sizeof(unsigned long long), ctx->stream));
  if (nnodes > ctx->order_cap) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->d_order) cudaFree(ctx->d_order);
    ctx->d_order = nullptr;
    ctx->order_cap = 0;
    const int64_t cap = std::max<int64_t>(nnodes, 4096);
    CK(cudaMalloc(&ctx->d_order, cap * sizeof(int)));
    ctx->order_cap = cap;
  }
  CK(cudaMemsetAsync(ctx->d_orderhist, 0, 2 * ORDER_BUCKETS * sizeof(int), ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launchNodeOrder(ctx->stream, gridFor(ctx, nnodes, 256, 2), nnodes, ptr, ctx->d_orderhist, ctx->d_order));
  CK(launchPack(ctx->stream, gridFor(ctx, ctx->n), baselb, baseub, ctx->d_base, ctx->n));
  const Prob P = devProb(ctx, false, true);
  CK(launchSeqPrepare(ctx->stream, gridFor(ctx, ctx->m), ctx->num, P, ctx->d_base, ctx->d_sq_prep));
  SeqArgs A;
  A.s = ctx->num;
  A.P = P;
  A.ccolptr = ctx->d_colptr;
  A.crow = ctx->d_sq_crow;
  A.cval = ctx->d_sq_cval;
  A.prep = ctx->d_sq_prep;
  A.base = ctx->d_base;
  A.nnodes = nnodes;
  A.ptr = ptr;
  A.chg_col = chg_col;
  A.chg_lb = chg_lb;
  A.chg_ub = chg_ub;
  A.out_cutoff = out_cutoff;
  A.out_rounds = out_rounds;
  A.out_off = out_off;
  A.out_n = out_n;
  A.out_col = out_col;
  A.out_lb = out_lb;
  A.out_ub = out_ub;
  A.out_cap = out_cap;
  A.out_used = ctx->d_out_used;
  A.maxrounds = ctx->par.maxrounds > 0 ? ctx->par.maxrounds : 1000000;
  A.next_item = ctx->d_next_item;
  A.order = ctx->d_order;
  A.S = SL;
  A.stats = ctx->d_stats;
  A.status = ctx->d_status;
  const int64_t warps = std::min<int64_t>(std::min<int64_t>(SL.nslots, nnodes), maxwarps);
  const int grid = (int)((warps + SEQ_WARPS - 1) / SEQ_WARPS);
  CK(launchNodesSeq(ctx->stream, grid, A));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  unsigned long long st[8];
  int status = 0;
  CK(cudaMemcpyAsync(st, ctx->d_stats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&ctx->last_out_used, ctx->d_out_used, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // the queue is dynamic: one slot may have run every node of the call
  ctx->seq_epoch_budget += nnodes;
  if (res) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->cutoff = (int32_t)st[4];
    res->rounds = (int32_t)st[5];
    res->status = (status & 1) ? 2 : 0;
    res->launches = 5;  // order (2), pack, row preparation, nodes
    res->rows = (int64_t)st[0];
    res->nnz = (int64_t)st[1];
    res->candidates = (int64_t)st[2];
    res->changes = (int64_t)st[3];
    res->live_rows = (int64_t)st[6];
    res->kernel_ms = ms;
  }
  if (status & 4) return fail(ctx, GBP_ERR_INVALID, "change column out of range");
  if (status & 2) return fail(ctx, GBP_ERR_OVERFLOW, "node output arrays too small");
  if (status & 1) return GBP_ERR_LIMIT;
  return GBP_OK;
}

int gbp_propagate_nodes_device(gbp_ctx* ctx, const double* baselb, const double* baseub, int64_t nnodes,
                               const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
                               int8_t* out_cutoff, int32_t* out_rounds, int64_t* out_off, int32_t* out_n,
                               int32_t* out_col, double* out_lb, double* out_ub, int64_t out_cap, gbp_result* res) {
  if (!ctx || !ctx->has_problem) return fail(ctx, GBP_ERR_INVALID, "no problem uploaded");
  if (nnodes < 0 || nnodes >= (int64_t(1) << 31) - 1 || out_cap < 0) return fail(ctx, GBP_ERR_INVALID, "bad sizes");
  if (nnodes == 0) {
    if (res) std::memset(res, 0, sizeof(*res));
    return GBP_OK;
  }
  if (!baselb || !baseub || !ptr || !out_cutoff || !out_rounds || !out_off || !out_n ||
      (out_cap > 0 && (!out_col || !out_lb || !out_ub)))
    return fail(ctx, GBP_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  if (ctx->par.flags & GBP_FLAG_SCIPORDER)
    return propagateNodesSeq(ctx, baselb, baseub, nnodes, ptr, chg_col, chg_lb, chg_ub, out_cutoff, out_rounds,
                             out_off, out_n, out_col, out_lb, out_ub, out_cap, res);
  int rc = ensureSlots(ctx, nnodes);
  if (rc) return rc;
  const int maxrounds = ctx->par.maxrounds > 0 ? ctx->par.maxrounds : 1000000;
  // stamp counters grow by (rounds + 1) per node and slot; re-zero the stamps long before they wrap
  if (ctx->slot_stamp_budget > (int64_t(1) << 30)) {
    const size_t S = (size_t)ctx->nslots;
    CK(cudaMemsetAsync(ctx->slots.ostamp, 0, S * ctx->slots.nstride * sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->slots.rowstamp, 0, S * ctx->slots.mstride * sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->slots.counter, 0, S * sizeof(int), ctx->stream));
    ctx->slot_stamp_budget = 0;
  }
  CK(cudaMemsetAsync(ctx->d_stats, 0, 8 * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_next_item, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_out_used, 0, sizeof(unsigned long long), ctx->stream));
  if (nnodes > ctx->order_cap) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->d_order) cudaFree(ctx->d_order);
    ctx->d_order = nullptr;
    ctx->order_cap = 0;
    const int64_t cap = std::max<int64_t>(nnodes, 4096);
    CK(cudaMalloc(&ctx->d_order, cap * sizeof(int)));
    ctx->order_cap = cap;
  }
  CK(cudaMemsetAsync(ctx->d_orderhist, 0, 2 * ORDER_BUCKETS * sizeof(int), ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  CK(launchNodeOrder(ctx->stream, gridFor(ctx, nnodes, 256, 2), nnodes, ptr, ctx->d_orderhist, ctx->d_order));
  CK(launchPack(ctx->stream, gridFor(ctx, ctx->n), baselb, baseub, ctx->d_base, ctx->n));
  int pre = 0;
  rc = prepareRanged(ctx, false, true, baselb, baseub, &pre);
  if (rc) return rc;
  NodesArgs A;
  A.s = ctx->num;
  A.P = devProb(ctx, false, true);
  A.base = ctx->d_base;
  A.baselb = nullptr;
  A.baseub = nullptr;
  A.nnodes = nnodes;
  A.ptr = ptr;
  A.chg_col = chg_col;
  A.chg_lb = chg_lb;
  A.chg_ub = chg_ub;
  A.out_cutoff = out_cutoff;
  A.out_rounds = out_rounds;
  A.out_off = out_off;
  A.out_n = out_n;
  A.out_col = out_col;
  A.out_lb = out_lb;
  A.out_ub = out_ub;
  A.out_cap = out_cap;
  A.out_used = ctx->d_out_used;
  A.maxrounds = maxrounds;
  A.next_item = ctx->d_next_item;
  A.order = ctx->d_order;
  A.S = ctx->slots;
  A.stats = ctx->d_stats;
  A.status = ctx->d_status;
  A.minblocks = ctx->ctas_per_sm;
  A.abort_flag = nullptr;  // uploads checked the rows and columns
  const int grid = (int)std::min<int64_t>(ctx->nslots, nnodes);
  CK(launchNodes(ctx->stream, grid, ctx->node_threads, A));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  unsigned long long st[8];
  int status = 0;
  CK(cudaMemcpyAsync(st, ctx->d_stats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&ctx->last_out_used, ctx->d_out_used, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // the queue is dynamic: one slot may have run every node of the call, not just its average share
  ctx->slot_stamp_budget += (nnodes + 1) * ((int64_t)st[5] + 2);
  if (res) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->cutoff = (int32_t)st[4];
    res->rounds = (int32_t)st[5];
    res->status = (status & 1) ? 2 : 0;
    res->launches = 4 + pre;  // order (2), pack, nodes, and the ranged rows' preparation
    res->rows = (int64_t)st[0];
    res->nnz = (int64_t)st[1];
    res->candidates = (int64_t)st[2];
    res->changes = (int64_t)st[3];
    res->live_rows = (int64_t)st[6];
    res->kernel_ms = ms;
  }
  if (status & 4) return fail(ctx, GBP_ERR_INVALID, "change column out of range");
  if (status & 2) return fail(ctx, GBP_ERR_OVERFLOW, "node output arrays too small");
  if (status & 1) return GBP_ERR_LIMIT;
  return GBP_OK;
}

int gbp_propagate_nodes(gbp_ctx* ctx, const double* baselb, const double* baseub, int64_t nnodes, const int64_t* ptr,
                        const int32_t* chg_col, const double* chg_lb, const double* chg_ub, int8_t* out_cutoff,
                        int32_t* out_rounds, int64_t* out_off, int32_t* out_n, int32_t* out_col, double* out_lb,
                        double* out_ub, int64_t out_cap, gbp_result* res) {
  if (!ctx || !ctx->has_problem) return fail(ctx, GBP_ERR_INVALID, "no problem uploaded");
  if (nnodes < 0 || out_cap < 0) return fail(ctx, GBP_ERR_INVALID, "bad sizes");
  if (nnodes == 0) {
    if (res) std::memset(res, 0, sizeof(*res));
    return GBP_OK;
  }
  if (!baselb || !baseub || !ptr || !out_cutoff || !out_rounds || !out_off || !out_n ||
      (out_cap > 0 && (!out_col || !out_lb || !out_ub)))
    return fail(ctx, GBP_ERR_INVALID, "null argument");
  if (ptr[0] != 0) return fail(ctx, GBP_ERR_INVALID, "ptr[0] must be 0");
  for (int64_t k = 0; k < nnodes; ++k)
    if (ptr[k + 1] < ptr[k]) return fail(ctx, GBP_ERR_INVALID, "ptr not monotone");
  const int64_t nchg = ptr[nnodes];
  if (nchg > 0 && (!chg_col || !chg_lb || !chg_ub)) return fail(ctx, GBP_ERR_INVALID, "null change arrays");
  // change columns are checked by the kernel (GBP_ERR_INVALID)
  CK(cudaSetDevice(ctx->device));
  // one staging allocation for inputs and outputs
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t n = (size_t)ctx->n;
  size_t off = 0;
  const size_t o_blb = off; off = al(off + n * 8);
  const size_t o_bub = off; off = al(off + n * 8);
  const size_t o_ptr = off; off = al(off + (nnodes + 1) * 8);
  const size_t o_col = off; off = al(off + nchg * 4);
  const size_t o_clb = off; off = al(off + nchg * 8);
  const size_t o_cub = off; off = al(off + nchg * 8);
  const size_t o_cut = off; off = al(off + nnodes);
  const size_t o_rnd = off; off = al(off + nnodes * 4);
  const size_t o_off = off; off = al(off + nnodes * 8);
  const size_t o_n = off; off = al(off + nnodes * 4);
  const size_t o_ocol = off; off = al(off + out_cap * 4);
  const size_t o_olb = off; off = al(off + out_cap * 8);
  const size_t o_oub = off; off = al(off + out_cap * 8);
  if (off > ctx->stage_bytes) {
    if (ctx->stage) cudaFree(ctx->stage);
    ctx->stage = nullptr;
    ctx->stage_bytes = 0;
    CK(cudaMalloc(&ctx->stage, off));
    ctx->stage_bytes = off;
  }
  char* b = (char*)ctx->stage;
  CK(cudaMemcpyAsync(b + o_blb, baselb, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(b + o_bub, baseub, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(b + o_ptr, ptr, (nnodes + 1) * 8, cudaMemcpyHostToDevice, ctx->stream));
  if (nchg) {
    CK(cudaMemcpyAsync(b + o_col, chg_col, nchg * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(b + o_clb, chg_lb, nchg * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(b + o_cub, chg_ub, nchg * 8, cudaMemcpyHostToDevice, ctx->stream));
  }
  int rc = gbp_propagate_nodes_device(ctx, (double*)(b + o_blb), (double*)(b + o_bub), nnodes, (int64_t*)(b + o_ptr),
                                      (int32_t*)(b + o_col), (double*)(b + o_clb), (double*)(b + o_cub),
                                      (int8_t*)(b + o_cut), (int32_t*)(b + o_rnd), (int64_t*)(b + o_off),
                                      (int32_t*)(b + o_n), (int32_t*)(b + o_ocol), (double*)(b + o_olb),
                                      (double*)(b + o_oub), out_cap, res);
  if (rc != GBP_OK && rc != GBP_ERR_LIMIT && rc != GBP_ERR_OVERFLOW) return rc;
  // the device call has waited for the kernels and read how many packed entries they wrote
  CK(cudaMemcpyAsync(out_cutoff, b + o_cut, nnodes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out_rounds, b + o_rnd, nnodes * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out_off, b + o_off, nnodes * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(out_n, b + o_n, nnodes * 4, cudaMemcpyDeviceToHost, ctx->stream));
  const size_t cnt = (size_t)std::min<unsigned long long>(ctx->last_out_used, (unsigned long long)out_cap);
  if (cnt) {
    CK(cudaMemcpyAsync(out_col, b + o_ocol, cnt * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(out_lb, b + o_olb, cnt * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(out_ub, b + o_oub, cnt * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return rc;
}

}  // extern "C"
