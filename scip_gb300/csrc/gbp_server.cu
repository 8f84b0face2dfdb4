// The serving loop of libgbp (gbp_server_*): node requests against one resident problem and its root bounds, merged
// by node workers into batched launches (gbp_propagate_nodes), and instance requests (problems of their own),
// merged by instance workers into block-diagonal launches (gbp_propagate_instances); each worker has its own
// context and stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gbp.h"

namespace {

struct Req {
  int kind = 0;  // 0 node, 1 instance
  std::vector<int32_t> cols;
  std::vector<double> lb, ub;
  // an instance request: its rows (CSR over local columns), integrality and bounds, borrowed from the caller
  // until the reply has been polled
  int64_t m = 0, n = 0;
  const int64_t* rowptr = nullptr;
  const int32_t* colidx = nullptr;
  const double *vals = nullptr, *lhs = nullptr, *rhs = nullptr, *ilb = nullptr, *iub = nullptr;
  const int8_t* isint = nullptr;
  int64_t t_submit = 0, t_done = 0;
  int done = 0;
  int rc = GBP_OK;
  int32_t cutoff = 0;
  std::vector<int32_t> ocols;
  std::vector<double> olb, oub;
  int64_t bytes = 0;
};

// pinned host buffers of one worker, grown as needed
template <class T>
struct Pinned {
  T* p = nullptr;
  size_t cap = 0;
  bool grow(size_t n) {
    if (n <= cap) return true;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if (cudaMallocHost(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    cap = std::max<size_t>(n, 1);
    return true;
  }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

struct Worker {
  gbp_ctx* ctx = nullptr;
  int kind = 0;  // 0 node requests, 1 instance requests
  std::thread th;
  Pinned<int64_t> ptr, off;
  Pinned<int32_t> col, rounds, n, ocol;
  Pinned<double> lb, ub, olb, oub;
  Pinned<int8_t> cut;
};

}  // namespace

struct gbp_server {
  int device = 0;
  int64_t m = 0, n = 0;
  int64_t max_batch = 0;
  std::vector<double> rootlb, rootub;
  std::vector<Worker> workers;
  mutable std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> queue;   // node requests
  std::deque<int64_t> iqueue;  // instance requests
  std::unordered_map<int64_t, Req> reqs;
  int64_t next_ticket = 1;
  bool stop = false;
  int64_t budget = 0, inflight = 0;
  int64_t batches = 0, served = 0, max_seen = 0;
  std::chrono::steady_clock::time_point t0;

  int64_t now() const {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

// device bytes of a request inside a batch: its changes in, its share of the packed output (one entry per column it
// may move, bounded by 256 as the batch reserves), the per-node outputs
int64_t requestBytes(int64_t nchg) { return 20 * nchg + 256 * 20 + 32; }

// propagate one batch of requests on a worker; fills each request's reply
void runBatch(gbp_server* S, Worker& W, std::vector<Req*>& batch) {
  const int64_t nb = (int64_t)batch.size();
  int64_t nchg = 0;
  for (Req* r : batch) nchg += (int64_t)r->cols.size();
  int64_t cap = 256 * nb;
  bool ok = W.ptr.grow(nb + 1) && W.off.grow(nb) && W.col.grow(nchg) && W.rounds.grow(nb) && W.n.grow(nb) &&
            W.lb.grow(nchg) && W.ub.grow(nchg) && W.cut.grow(nb) && W.ocol.grow(cap) && W.olb.grow(cap) &&
            W.oub.grow(cap);
  if (!ok) {
    for (Req* r : batch) r->rc = GBP_ERR_NOMEM;
    return;
  }
  int64_t at = 0;
  W.ptr.p[0] = 0;
  for (int64_t k = 0; k < nb; ++k) {
    const Req* r = batch[k];
    const size_t c = r->cols.size();
    std::memcpy(W.col.p + at, r->cols.data(), c * sizeof(int32_t));
    std::memcpy(W.lb.p + at, r->lb.data(), c * sizeof(double));
    std::memcpy(W.ub.p + at, r->ub.data(), c * sizeof(double));
    at += (int64_t)c;
    W.ptr.p[k + 1] = at;
  }
  gbp_result res;
  int rc = gbp_propagate_nodes(W.ctx, S->rootlb.data(), S->rootub.data(), nb, W.ptr.p, W.col.p, W.lb.p, W.ub.p,
                               W.cut.p, W.rounds.p, W.off.p, W.n.p, W.ocol.p, W.olb.p, W.oub.p, cap, &res);
  std::vector<Req*> again;  // nodes whose results did not fit the batch's packed output
  for (int64_t k = 0; k < nb; ++k) {
    Req* r = batch[k];
    if (rc != GBP_OK && rc != GBP_ERR_LIMIT && rc != GBP_ERR_OVERFLOW) {
      r->rc = rc;
      continue;
    }
    if (W.n.p[k] < 0) {
      again.push_back(r);
      continue;
    }
    r->cutoff = W.cut.p[k];
    const int64_t cnt = r->cutoff ? 0 : W.n.p[k];
    std::vector<int64_t> idx((size_t)cnt);
    for (int64_t q = 0; q < cnt; ++q) idx[q] = W.off.p[k] + q;
    std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return W.ocol.p[a] < W.ocol.p[b]; });
    r->ocols.resize((size_t)cnt);
    r->olb.resize((size_t)cnt);
    r->oub.resize((size_t)cnt);
    for (int64_t q = 0; q < cnt; ++q) {
      r->ocols[q] = W.ocol.p[idx[q]];
      r->olb[q] = W.olb.p[idx[q]];
      r->oub[q] = W.oub.p[idx[q]];
    }
  }
  for (Req* r : again) {  // alone, with room for every column
    if (!W.ocol.grow((size_t)S->n) || !W.olb.grow((size_t)S->n) || !W.oub.grow((size_t)S->n)) {
      r->rc = GBP_ERR_NOMEM;
      continue;
    }
    std::vector<Req*> one{r};
    const int64_t c = (int64_t)r->cols.size();
    W.ptr.p[0] = 0;
    W.ptr.p[1] = c;
    std::memcpy(W.col.p, r->cols.data(), c * sizeof(int32_t));
    std::memcpy(W.lb.p, r->lb.data(), c * sizeof(double));
    std::memcpy(W.ub.p, r->ub.data(), c * sizeof(double));
    int rc2 = gbp_propagate_nodes(W.ctx, S->rootlb.data(), S->rootub.data(), 1, W.ptr.p, W.col.p, W.lb.p, W.ub.p,
                                  W.cut.p, W.rounds.p, W.off.p, W.n.p, W.ocol.p, W.olb.p, W.oub.p, S->n, &res);
    if (rc2 != GBP_OK && rc2 != GBP_ERR_LIMIT) {
      r->rc = rc2;
      continue;
    }
    r->cutoff = W.cut.p[0];
    const int64_t cnt = r->cutoff ? 0 : W.n.p[0];
    std::vector<int64_t> idx((size_t)cnt);
    for (int64_t q = 0; q < cnt; ++q) idx[q] = W.off.p[0] + q;
    std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return W.ocol.p[a] < W.ocol.p[b]; });
    r->ocols.resize((size_t)cnt);
    r->olb.resize((size_t)cnt);
    r->oub.resize((size_t)cnt);
    for (int64_t q = 0; q < cnt; ++q) {
      r->ocols[q] = W.ocol.p[idx[q]];
      r->olb[q] = W.olb.p[idx[q]];
      r->oub[q] = W.oub.p[idx[q]];
    }
  }
}

// propagate a batch of instance requests on an instance worker: one upload of the instances as parts of a
// block-diagonal problem, one batched root fixpoint, each request's bounds back.  The upload checks every part
// (row pointers on the host, column indices on the device) and refuses the whole batch for one bad part: the
// batch then runs again one request at a time, so that only the bad request is answered GBP_ERR_INVALID.
int runInstanceList(Worker& W, Req* const* batch, size_t k) {
  std::vector<int64_t> mk(k), nk(k);
  std::vector<const int64_t*> rp(k);
  std::vector<const int32_t*> ci(k);
  std::vector<const double*> va(k), lh(k), rh(k);
  std::vector<const int8_t*> it(k);
  std::vector<double> lb, ub;
  for (size_t q = 0; q < k; ++q) {
    const Req* r = batch[q];
    mk[q] = r->m;
    nk[q] = r->n;
    rp[q] = r->rowptr;
    ci[q] = r->colidx;
    va[q] = r->vals;
    lh[q] = r->lhs;
    rh[q] = r->rhs;
    it[q] = r->isint;
    lb.insert(lb.end(), r->ilb, r->ilb + r->n);
    ub.insert(ub.end(), r->iub, r->iub + r->n);
  }
  std::vector<int8_t> cut(k, 0);
  gbp_result res;
  int rc = gbp_upload_instance_list(W.ctx, (int64_t)k, mk.data(), nk.data(), rp.data(), ci.data(), va.data(),
                                    lh.data(), rh.data(), it.data());
  if (rc == GBP_ERR_INVALID) return rc;
  if (rc == GBP_OK) rc = gbp_propagate_instances(W.ctx, lb.data(), ub.data(), cut.data(), &res);
  int64_t at = 0;
  for (size_t q = 0; q < k; ++q) {
    Req* r = batch[q];
    const int64_t n = r->n;
    if (rc != GBP_OK && rc != GBP_ERR_LIMIT) {
      r->rc = rc;
    } else {
      r->cutoff = cut[q];
      if (!r->cutoff) {  // the whole bound vector: every column in order
        r->ocols.resize((size_t)n);
        for (int64_t j = 0; j < n; ++j) r->ocols[j] = (int32_t)j;
        r->olb.assign(lb.begin() + at, lb.begin() + at + n);
        r->oub.assign(ub.begin() + at, ub.begin() + at + n);
      }
    }
    at += n;
  }
  return GBP_OK;
}

void runInstances(Worker& W, std::vector<Req*>& batch) {
  if (runInstanceList(W, batch.data(), batch.size()) != GBP_ERR_INVALID) return;
  for (Req* r : batch)
    if (runInstanceList(W, &r, 1) == GBP_ERR_INVALID) r->rc = GBP_ERR_INVALID;
}

void workerLoop(gbp_server* S, Worker* W) {
  cudaSetDevice(S->device);
  std::deque<int64_t>& Q = W->kind == 0 ? S->queue : S->iqueue;
  const int64_t maxb = W->kind == 0 ? S->max_batch : std::max<int64_t>(1, S->max_batch / 8);
  std::vector<Req*> batch;
  std::vector<int64_t> tickets;
  for (;;) {
    int64_t bytes = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      // a stopping server still serves what is queued; every request fits the budget alone (submission refuses
      // the rest), so the front fits once the other workers' batches have finished
      S->cv_work.wait(lk, [&] {
        return (S->stop && Q.empty()) || (!Q.empty() && S->inflight + S->reqs[Q.front()].bytes <= S->budget);
      });
      if (Q.empty()) return;
      batch.clear();
      tickets.clear();
      while (!Q.empty() && (int64_t)batch.size() < maxb) {
        Req& r = S->reqs[Q.front()];
        if (S->inflight + bytes + r.bytes > S->budget) break;
        bytes += r.bytes;
        batch.push_back(&r);
        tickets.push_back(Q.front());
        Q.pop_front();
      }
      S->inflight += bytes;
    }
    // Req objects stay put: only this worker and the pollers of done tickets touch them
    if (W->kind == 0)
      runBatch(S, *W, batch);
    else
      runInstances(*W, batch);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      const int64_t t = S->now();
      for (Req* r : batch) {
        r->t_done = t;
        r->done = 1;
      }
      S->inflight -= bytes;
      S->batches += 1;
      S->served += (int64_t)batch.size();
      S->max_seen = std::max<int64_t>(S->max_seen, (int64_t)batch.size());
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int gbp_server_create(gbp_server** out, int device, int nworkers, int ninstworkers, int64_t max_batch,
                      int64_t hbm_cap, const gbp_params* params, int64_t m, int64_t n, const int64_t* rowptr,
                      const int32_t* colidx, const double* vals, const double* lhs, const double* rhs,
                      const int8_t* isint, const double* rootlb, const double* rootub) {
  if (!out || nworkers < 1 || ninstworkers < 0 || max_batch < 1 || hbm_cap < 0 || m < 0 || n < 0 ||
      (n > 0 && (!rootlb || !rootub)))
    return GBP_ERR_INVALID;
  *out = nullptr;
  gbp_server* S = new (std::nothrow) gbp_server();
  if (!S) return GBP_ERR_NOMEM;
  S->device = device;
  S->m = m;
  S->n = n;
  S->max_batch = max_batch;
  S->rootlb.assign(rootlb, rootlb + n);
  S->rootub.assign(rootub, rootub + n);
  S->t0 = std::chrono::steady_clock::now();
  S->workers.resize((size_t)(nworkers + ninstworkers));
  int rc = GBP_OK;
  for (size_t q = 0; q < S->workers.size(); ++q) {
    Worker& W = S->workers[q];
    W.kind = (int)q < nworkers ? 0 : 1;
    rc = gbp_create(&W.ctx, device, nullptr);
    if (rc == GBP_OK && params) rc = gbp_set_params(W.ctx, params);
    if (rc != GBP_OK) break;
    if (W.kind == 1) continue;  // an instance worker uploads each batch's instances
    rc = gbp_upload_problem(W.ctx, m, n, rowptr, colidx, vals, lhs, rhs, isint);
    if (rc != GBP_OK) break;
    // a first batch (a node without changes) allocates the worker's slots before the budget is measured
    std::vector<Req> warm(1);
    std::vector<Req*> wb{&warm[0]};
    runBatch(S, W, wb);
    if (warm[0].rc != GBP_OK) {
      rc = warm[0].rc;
      break;
    }
  }
  if (rc != GBP_OK) {
    for (Worker& W : S->workers)
      if (W.ctx) gbp_destroy(W.ctx);
    delete S;
    return rc;
  }
  size_t freeb = 0, totalb = 0;
  cudaSetDevice(device);
  if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) {
    for (Worker& W : S->workers) gbp_destroy(W.ctx);
    delete S;
    return GBP_ERR_CUDA;
  }
  const int64_t cap = hbm_cap > 0 ? hbm_cap : (int64_t)150 << 30;
  S->budget = std::min<int64_t>(cap, (int64_t)freeb);
  for (Worker& W : S->workers) W.th = std::thread(workerLoop, S, &W);
  *out = S;
  return GBP_OK;
}

int gbp_server_submit(gbp_server* S, int64_t nchg, const int32_t* cols, const double* lb, const double* ub,
                      int64_t* ticket) {
  if (!S || !ticket || nchg < 0 || (nchg > 0 && (!cols || !lb || !ub))) return GBP_ERR_INVALID;
  for (int64_t k = 0; k < nchg; ++k)
    if (cols[k] < 0 || cols[k] >= S->n) return GBP_ERR_INVALID;
  const int64_t bytes = requestBytes(nchg);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return GBP_ERR_INVALID;
    if (bytes > S->budget) return GBP_ERR_NOMEM;
    const int64_t t = S->next_ticket++;
    Req& r = S->reqs[t];
    r.cols.assign(cols, cols + nchg);
    r.lb.assign(lb, lb + nchg);
    r.ub.assign(ub, ub + nchg);
    r.bytes = bytes;
    r.t_submit = S->now();
    S->queue.push_back(t);
    *ticket = t;
  }
  S->cv_work.notify_all();
  return GBP_OK;
}

int gbp_server_submit_instance(gbp_server* S, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
                               const double* vals, const double* lhs, const double* rhs, const int8_t* isint,
                               const double* lb, const double* ub, int64_t* ticket) {
  if (!S || !ticket || m < 0 || n < 0 || !rowptr || (m > 0 && (!lhs || !rhs)) || (n > 0 && (!isint || !lb || !ub)))
    return GBP_ERR_INVALID;
  // the rest of the checks (row pointers non-decreasing, column indices inside the instance) run on the worker,
  // off the submitting thread, when the batch is uploaded
  const int64_t nnz = rowptr[m];
  if (rowptr[0] != 0 || nnz < 0 || (nnz > 0 && (!colidx || !vals))) return GBP_ERR_INVALID;
  const int64_t bytes = 28 * nnz + 64 * m + 64 * n + 4096;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return GBP_ERR_INVALID;
    bool any = false;
    for (const Worker& W : S->workers) any |= W.kind == 1;
    if (!any) return GBP_ERR_INVALID;  // the server has no instance workers
    if (bytes > S->budget) return GBP_ERR_NOMEM;
    const int64_t t = S->next_ticket++;
    Req& r = S->reqs[t];
    r.kind = 1;
    r.m = m;
    r.n = n;
    r.rowptr = rowptr;
    r.colidx = colidx;
    r.vals = vals;
    r.lhs = lhs;
    r.rhs = rhs;
    r.isint = isint;
    r.ilb = lb;
    r.iub = ub;
    r.bytes = bytes;
    r.t_submit = S->now();
    S->iqueue.push_back(t);
    *ticket = t;
  }
  S->cv_work.notify_all();
  return GBP_OK;
}

int gbp_server_poll(gbp_server* S, int64_t ticket, int wait_ms, int32_t* cutoff, int64_t cap, int64_t* nout,
                    int32_t* cols, double* lb, double* ub, int64_t* t_submit_ns, int64_t* t_done_ns) {
  if (!S || !cutoff || !nout || cap < 0 || (cap > 0 && (!cols || !lb || !ub))) return GBP_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return GBP_ERR_INVALID;
  auto ready = [&] { return it->second.done != 0; };
  if (wait_ms < 0)
    S->cv_done.wait(lk, ready);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready))
    return GBP_ERR_BUSY;
  Req& r = it->second;
  if (t_submit_ns) *t_submit_ns = r.t_submit;
  if (t_done_ns) *t_done_ns = r.t_done;
  if (r.rc != GBP_OK) {
    const int rc = r.rc;
    S->reqs.erase(it);
    return rc;
  }
  *cutoff = r.cutoff;
  *nout = (int64_t)r.ocols.size();
  if (*nout > cap) return GBP_ERR_OVERFLOW;
  std::memcpy(cols, r.ocols.data(), r.ocols.size() * sizeof(int32_t));
  std::memcpy(lb, r.olb.data(), r.olb.size() * sizeof(double));
  std::memcpy(ub, r.oub.data(), r.oub.size() * sizeof(double));
  S->reqs.erase(it);
  return GBP_OK;
}

int gbp_server_stats(const gbp_server* S, int64_t* batches, int64_t* requests, int64_t* max_batch_seen,
                     int64_t* budget) {
  if (!S) return GBP_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  if (batches) *batches = S->batches;
  if (requests) *requests = S->served;
  if (max_batch_seen) *max_batch_seen = S->max_seen;
  if (budget) *budget = S->budget;
  return GBP_OK;
}

int gbp_server_destroy(gbp_server* S) {
  if (!S) return GBP_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (Worker& W : S->workers)
    if (W.th.joinable()) W.th.join();
  for (Worker& W : S->workers)
    if (W.ctx) gbp_destroy(W.ctx);
  delete S;
  return GBP_OK;
}

}  // extern "C"
