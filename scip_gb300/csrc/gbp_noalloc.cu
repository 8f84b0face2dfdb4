// gbp_propagate_nodes_noalloc: batched node propagation without any device memory allocation.
//
// Some callers cannot let a library call cudaMalloc:
//   * applications that hand all device memory to their own pool allocator at start-up (a cudaMalloc from a
//     library either fails or fragments the pool they manage), and
//   * callers that must not trigger the implicit device-wide synchronisation of cudaMalloc/cudaFree, e.g. a
//     propagation callback that runs while other streams of the host application keep working.
// For them this entry point takes every input and output as a device pointer from the caller and keeps its
// scratch in one file-scope __device__ array of GBP_NOALLOC_SCRATCH_BYTES (64 MiB), which every GPU that
// loads libgbp holds until the process exits.  Nothing here calls cudaMalloc, cudaFree, cudaMallocAsync or
// an allocating library routine.
//
// Set-up: the first call on a device (with that device current) looks up the array's device address with
// cudaGetSymbolAddress and caches it together with the device's current driver context; make that first call
// before any stream capture.  A later call in another context of the device (after a cudaDeviceReset, whose new
// primary context maps the array elsewhere) looks the address up again.
// Input checks: the caller's arrays are device memory the library cannot check on the host, so two kernels check
// them first (row and column pointers start at 0, never decrease and describe the same number of entries; every
// column index lies in [0, n), every row index in [0, m)) and set a bit in the scratch header; when it is set no
// node runs, every node reports out_n[k] = -1, and the call returns GBP_ERR_INVALID (with res) -- never a read out
// of bounds.  The arrays must hold the entries their pointers describe: rowptr[m] column indices and values,
// colptr[n] row indices and values.
// Sharing: every call on a device uses the same array and leaves its contents behind; each call clears what
// must start at zero before it launches.  Calls whose work overlaps on the GPU (two streams, two host
// threads) race on the array and must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/gbp.h"
#include "gbp_internal.h"

using namespace gbp;

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GBP_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
CUcontext g_scratch_ctx[kMaxDevices] = {nullptr};  // the driver context the cached address belongs to

// header at the start of the array: work-queue head, status bits, packed-output counter, statistics
struct Header {
  int next_item;
  int status;
  unsigned long long out_used;
  unsigned long long stats[8];
};
constexpr size_t kHeaderBytes = 256;
static_assert(sizeof(Header) <= kHeaderBytes, "header too large");
constexpr int kThreads = 128;
constexpr int kBudget = 4;  // compiled variant: 128 threads per node, 4 resident CTAs per SM

int scratchAddress(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return GBP_ERR_NODEVICE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  // the driver's cuCtxGetCurrent through the runtime (libgbp links no driver library)
  static CUresult (*ctxGetCurrent)(CUcontext*) = nullptr;
  if (ctxGetCurrent == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || fn == nullptr) {
      cudaGetLastError();
      return GBP_ERR_CUDA;
    }
    ctxGetCurrent = (CUresult(*)(CUcontext*))fn;
  }
  // before the runtime has made a context current, cuCtxGetCurrent reports none: the lookup below then
  // initialises the device's primary context
  CUcontext cur = nullptr;
  if (ctxGetCurrent(&cur) != CUDA_SUCCESS) cur = nullptr;
  if (g_scratch_ptr[device] == nullptr || cur == nullptr || g_scratch_ctx[device] != cur) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return GBP_ERR_CUDA;
    }
    if (ctxGetCurrent(&cur) != CUDA_SUCCESS || cur == nullptr) return GBP_ERR_CUDA;
    g_scratch_ptr[device] = p;
    g_scratch_ctx[device] = cur;
  }
  *out = g_scratch_ptr[device];
  return GBP_OK;
}

// input checks (status bit 3): the pointer arrays first, reading only their m + 1 and n + 1 entries
__global__ void k_check_pointers(int64_t m, int64_t n, const int64_t* rowptr, const int64_t* colptr, int* status) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t0 == 0 && (rowptr[0] != 0 || colptr[0] != 0 || rowptr[m] != colptr[n])) atomicOr(status, 8);
  for (int64_t i = t0; i < m; i += stride)
    if (rowptr[i + 1] < rowptr[i]) atomicOr(status, 8);
  for (int64_t j = t0; j < n; j += stride)
    if (colptr[j + 1] < colptr[j]) atomicOr(status, 8);
}
// then, when the pointers hold, the indices they describe
__global__ void k_check_indices(int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
                                const int32_t* rowidx, int* status) {
  if (*status & 8) return;
  const int64_t nnz = rowptr[m];
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t j = colidx[p], i = rowidx[p];
    if (j < 0 || j >= n || i < 0 || i >= m) atomicOr(status, 8);
  }
}

}  // namespace

extern "C" int gbp_propagate_nodes_noalloc(int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
                                           const double* vals, const double* lhs, const double* rhs,
                                           const int8_t* isint, const int64_t* colptr, const int32_t* rowidx,
                                           const double* cvals, const double* baselb, const double* baseub,
                                           int64_t nnodes, const int64_t* ptr, const int32_t* chg_col,
                                           const double* chg_lb, const double* chg_ub, int8_t* out_cutoff,
                                           int32_t* out_rounds, int64_t* out_off, int32_t* out_n, int32_t* out_col,
                                           double* out_lb, double* out_ub, int64_t out_cap, const gbp_params* params,
                                           void* stream, gbp_result* res) {
  if (m < 0 || n < 0 || nnodes < 0 || out_cap < 0) return GBP_ERR_INVALID;
  // ranged rows need a context's row order, and SCIP's own order the context's row-ordered column copy
  if (params && (params->flags & (GBP_FLAG_RANGEDROW | GBP_FLAG_SCIPORDER))) return GBP_ERR_INVALID;
  if (m >= (int64_t(1) << 30) || n >= (int64_t(1) << 31) - 1 || nnodes >= (int64_t(1) << 31) - 1)
    return GBP_ERR_TOO_LARGE;
  if (nnodes == 0) {
    if (res) std::memset(res, 0, sizeof(*res));
    return GBP_OK;
  }
  if (!rowptr || !lhs || !rhs || !isint || !colptr || !baselb || !baseub || !ptr || !out_cutoff || !out_rounds ||
      !out_off || !out_n || (out_cap > 0 && (!out_col || !out_lb || !out_ub)) ||
      (n > 0 && (!colidx || !vals || !rowidx || !cvals)))
    return GBP_ERR_INVALID;

  // one slot (the per-CTA scratch of one node at a time) must fit next to the header
  const int64_t ns = std::max<int64_t>(n, 1), ms = std::max<int64_t>(m, 1);
  const size_t per_slot = slotLayout(ns, ms, 1, nullptr, nullptr);
  if (kHeaderBytes + per_slot > GBP_NOALLOC_SCRATCH_BYTES) return GBP_ERR_TOO_LARGE;

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return GBP_ERR_NODEVICE;
  void* scratch = nullptr;
  int rc = scratchAddress(device, &scratch);
  if (rc != GBP_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  int sms = 0, occ = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return GBP_ERR_CUDA;
  if (nodesOccupancy(kThreads, kBudget, &occ) != cudaSuccess) return GBP_ERR_CUDA;
  int64_t nslots = std::min<int64_t>((int64_t)sms * std::max(occ, 1), nnodes);
  while (nslots > 1 && kHeaderBytes + slotLayout(ns, ms, nslots, nullptr, nullptr) > GBP_NOALLOC_SCRATCH_BYTES)
    --nslots;

  char* base = (char*)scratch;
  Header* hdr = (Header*)base;
  SlotArrays S;
  const size_t slot_bytes = slotLayout(ns, ms, nslots, base + kHeaderBytes, &S);
  const size_t NS = (size_t)nslots;
  // the node order of the queue, when it fits behind the slots (else nodes run in index order)
  const size_t order_off = (kHeaderBytes + slot_bytes + 255) & ~size_t(255);
  const size_t order_bytes = (2 * ORDER_BUCKETS + (size_t)nnodes) * sizeof(int);
  int* orderhist = order_off + order_bytes <= GBP_NOALLOC_SCRATCH_BYTES ? (int*)(base + order_off) : nullptr;

  // clear what must start at zero (the array keeps the previous call's contents)
  if (cudaMemsetAsync(hdr, 0, sizeof(Header), st) != cudaSuccess ||
      cudaMemsetAsync(S.ostamp, 0, NS * ns * sizeof(int), st) != cudaSuccess ||
      cudaMemsetAsync(S.cflag, 0, NS * ns * sizeof(int), st) != cudaSuccess ||
      cudaMemsetAsync(S.rowstamp, 0, NS * ms * sizeof(int), st) != cudaSuccess ||
      cudaMemsetAsync(S.counter, 0, NS * sizeof(int), st) != cudaSuccess)
    return GBP_ERR_CUDA;
  const int fillgrid = sms * 4;
  if (orderhist != nullptr) {
    if (cudaMemsetAsync(orderhist, 0, 2 * ORDER_BUCKETS * sizeof(int), st) != cudaSuccess ||
        launchNodeOrder(st, sms * 2, nnodes, ptr, orderhist, orderhist + 2 * ORDER_BUCKETS) != cudaSuccess)
      return GBP_ERR_CUDA;
  }
  if (launchFill64(st, fillgrid, S.cub, (int64_t)(NS * ns), KEY_NONE_UB) != cudaSuccess ||
      launchFill64(st, fillgrid, S.clb, (int64_t)(NS * ns), KEY_NONE_LB) != cudaSuccess ||
      launchFill64(st, fillgrid, S.cubf, (int64_t)(NS * ns), KEY_NONE_UB) != cudaSuccess ||
      launchFill64(st, fillgrid, S.clbf, (int64_t)(NS * ns), KEY_NONE_LB) != cudaSuccess)
    return GBP_ERR_CUDA;

  gbp_params p;
  if (params) p = *params;
  else gbp_default_params(&p);
  NodesArgs A;
  A.s = Num{p.infinity, p.epsilon, p.sumepsilon, p.feastol, p.hugeval, p.boundstreps, p.recompfac,
            p.maxeasyactivitydelta, (p.flags & GBP_FLAG_NOSORTVARS) ? 1 : 0};
  A.P = Prob{m, n, rowptr, colidx, vals, lhs, rhs, isint, colptr, nullptr, rowidx, cvals, p.infinity};
  A.base = nullptr;
  A.baselb = baselb;
  A.baseub = baseub;
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
  A.out_used = &hdr->out_used;
  A.maxrounds = p.maxrounds > 0 ? p.maxrounds : 1000000;
  A.next_item = &hdr->next_item;
  A.order = orderhist != nullptr ? orderhist + 2 * ORDER_BUCKETS : nullptr;
  A.S = S;
  A.stats = hdr->stats;
  A.status = &hdr->status;
  A.minblocks = kBudget;
  A.abort_flag = &hdr->status;
  k_check_pointers<<<sms, 256, 0, st>>>(m, n, rowptr, colptr, &hdr->status);
  k_check_indices<<<sms * 4, 256, 0, st>>>(m, n, rowptr, colidx, rowidx, &hdr->status);
  if (cudaGetLastError() != cudaSuccess) return GBP_ERR_CUDA;
  if (launchNodes(st, (int)nslots, kThreads, A) != cudaSuccess) return GBP_ERR_CUDA;
  if (res == nullptr) return GBP_OK;

  // with a result struct the call waits for the stream and reports statistics and status
  Header h;
  if (cudaMemcpyAsync(&h, hdr, sizeof(Header), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return GBP_ERR_CUDA;
  res->cutoff = (int32_t)h.stats[4];
  res->rounds = (int32_t)h.stats[5];
  res->status = (h.status & 1) ? 2 : 0;
  // kernels of the call: the four candidate-slot fills, the node order (two, when it fits), the two input
  // checks and the node kernel (the context path fills its slots once, when it allocates them)
  res->launches = orderhist != nullptr ? 9 : 7;
  res->rows = (int64_t)h.stats[0];
  res->nnz = (int64_t)h.stats[1];
  res->candidates = (int64_t)h.stats[2];
  res->changes = (int64_t)h.stats[3];
  res->live_rows = (int64_t)h.stats[6];
  res->kernel_ms = 0.0;
  if (h.status & (4 | 8)) return GBP_ERR_INVALID;
  if (h.status & 2) return GBP_ERR_OVERFLOW;
  if (h.status & 1) return GBP_ERR_LIMIT;
  return GBP_OK;
}
