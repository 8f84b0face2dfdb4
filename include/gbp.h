/* gbp.h -- C ABI of the GB300 linear-constraint bound propagator (libgbp.so).
 *
 * The library replaces the propagation work of SCIP's linear constraint handler
 *   consPropLinear -> propagateCons -> tightenBounds -> tightenVarBounds / tightenVarBoundsEasy
 *   (src/scip/cons_linear.c:16126-16195, 7621-7758, 6980-7154, 6700-6974, 5380-5653)
 * for a propagator plugin registered through SCIPincludePropBasic (src/scip/scip_prop.c:118-140) whose
 * SCIP_DECL_PROPEXEC callback (src/scip/type_prop.h:217) hands the transformed problem's rows and local
 * bounds to these entry points and writes the returned bounds back with SCIPinferVarLbProp/UbProp
 * (src/scip/scip_var.c:7589/7705) or reports SCIP_CUTOFF.  scip_gb300/plugin/prop_gpulinear.c is that plugin.
 *
 * Conventions: plain C types only; sizes are int64_t; every function returns GBP_OK (0) or a negative
 * GBP_ERR_* code (no exceptions cross the boundary; gbp_error_string() names the code and
 * gbp_last_error() gives the context's last message).  Host pointers are ordinary CPU memory unless the
 * function name ends in _device, in which case every array argument is a device pointer on the context's
 * GPU; scalar out-parameters (cutoff, res) are always host pointers.  Infinite sides and bounds are +-params.infinity (1e20 by default), as in SCIP.
 *
 * Rows are stored once on the device in CSR and CSC form; bound vectors, node bound changes and results
 * are the only per-call traffic.  One context = one GPU = one CUDA stream; calls on a context must not
 * overlap from several host threads.
 */
#ifndef GBP_H
#define GBP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBP_OK              0
#define GBP_ERR_INVALID    -1   /* bad argument (sizes, indices, null pointers, problem not uploaded) */
#define GBP_ERR_CUDA       -2   /* a CUDA runtime call failed (message in gbp_last_error) */
#define GBP_ERR_NOMEM      -3   /* device or host allocation failed */
#define GBP_ERR_NODEVICE   -4   /* no CUDA device, or the device is not an sm_103 GPU */
#define GBP_ERR_LIMIT      -5   /* the round limit was reached before the fixpoint (results are valid bounds) */
#define GBP_ERR_OVERFLOW   -6   /* an output list was too small (out_n reports -1 for that node) */
#define GBP_ERR_STATE      -7   /* the device reported an inconsistent state (a bounded loop gave up) */
#define GBP_ERR_TOO_LARGE  -8   /* the problem does not fit the fixed scratch of gbp_propagate_nodes_noalloc */
#define GBP_ERR_BUSY       -9   /* gbp_server_poll: the reply is not ready within the wait */

typedef struct gbp_ctx gbp_ctx;

/* numerics of SCIP's set.c / def.h and the two parameters of cons_linear propagation that matter here */
typedef struct
{
   double infinity;             /* numerics/infinity (1e20) */
   double epsilon;              /* numerics/epsilon (1e-9) */
   double sumepsilon;           /* numerics/sumepsilon (1e-6) */
   double feastol;              /* numerics/feastol (1e-6) */
   double hugeval;              /* numerics/hugeval (1e15) */
   double boundstreps;          /* numerics/boundstreps (0.05), minimal relative bound improvement */
   double recompfac;            /* numerics/recompfac (1e6) */
   double maxeasyactivitydelta; /* constraints/linear/maxeasyactivitydelta; SCIP's default is 1e6, 0 selects the
                                 * residual rule (cons_linear.c:6700) for every row */
   int32_t maxrounds;           /* propagation round cap per problem or node; <= 0 means 1,000,000 */
   int32_t flags;               /* GBP_FLAG_* bits, 0 by default */
} gbp_params;

/* plain path: drive the rounds from the host (one synchronisation per round) instead of the device-side loop
 * (a CUDA graph whose conditional while-node repeats the round until the frontier is empty) */
#define GBP_FLAG_HOSTLOOP 1
/* constraints/linear/sortvars = FALSE: every entry of a row is tried.  By default (SCIP's default, TRUE) the
 * binary columns of a row are tried in decreasing |a| (ties: lower column index first) and the first unfixed
 * binary that yields no tightening ends the visit of the binaries, as tightenBounds does
 * (cons_linear.c:7110-7138; order of consdataCompVarProp, cons_linear.c:3229-3254). */
#define GBP_FLAG_NOSORTVARS 2
/* constraints/linear/rangedrowpropagation = TRUE (SCIP's default) with rangedrowartcons = FALSE: after its
 * activity rules, every frontier row with both sides finite runs the gcd-based ranged-row rule
 * (rangedRowPropagation, cons_linear.c:5715-6695) from the same round-start bounds.  Its bound changes are forced
 * (SCIPinferVarFixCons / SCIPinferVarLb/UbCons with force = TRUE), and it may declare the row infeasible.  It
 * walks a row's entries in the order SCIP holds them: with sortvars, consdataCompVarProp on the global domain;
 * without, the index order (binaries, integers, continuous columns, each by column).  Not available in
 * gbp_propagate_nodes_noalloc. */
#define GBP_FLAG_RANGEDROW 4
/* batched nodes (gbp_propagate_nodes / gbp_propagate_nodes_device) in SCIP's own order instead of rounds: the rows
 * marked for propagation one at a time in SCIP's order (SCIPconshdlrPropagate, cons.c:3905-4080, with
 * conshdlrProcessUpdates, cons.c:1689), every tightening applied at once and the other rows' activities updated
 * incrementally by its bound-change event (consPropLinear, cons_linear.c:16126; tightenBounds :6976-7154;
 * eventExecLinear :17162-17363), so that a node's final bounds are the ones SCIP's own propagation reaches, not only
 * a valid fixpoint of the same rules.  Each row's entries are visited in storage order, which must be the order
 * SCIP holds the row in (SCIPgetVarsLinear during solving; consdataCompVarProp, cons_linear.c:3191-3254, on the
 * base bounds for rows SCIP has not re-sorted); with sortvars a row's leading binaries under the base bounds are its
 * nbinvars.  Rows are marked in ascending row index for each changed column, so the rows must be uploaded in the
 * order a variable's bound-change events reach SCIP's constraints: the order SCIP created them (its handler array
 * loses that order once constraints are deleted).  The base bounds must be a propagated fixpoint (SCIP's root):
 * rows redundant under them are the rows
 * SCIP's root deleted and take no part, and every row counts as already tightened there until a change that one of
 * its finite sides can use.  Does not combine with GBP_FLAG_RANGEDROW. */
#define GBP_FLAG_SCIPORDER 8

typedef struct
{
   int32_t cutoff;      /* number of problems/nodes found infeasible */
   int32_t rounds;      /* largest number of rounds any problem/node took */
   int32_t status;      /* 0 fixpoint, 1 cutoff (single problem), 2 round limit */
   int32_t launches;    /* kernels launched by the call */
   int64_t rows;        /* frontier rows processed, summed over rounds and nodes */
   int64_t nnz;         /* nonzeros of those rows */
   int64_t candidates;  /* candidate bounds emitted */
   int64_t changes;     /* accepted bound changes (lower and upper counted separately) */
   int64_t live_rows;   /* frontier rows that passed the skip tests and produced candidate work */
   double kernel_ms;    /* device time of the propagation kernels (CUDA events on the context's stream) */
} gbp_result;

/* ---------------------------------------------------------------- context */
int gbp_version(void);
const char* gbp_error_string(int code);
const char* gbp_last_error(const gbp_ctx* ctx);

/* device: CUDA ordinal; stream: a cudaStream_t to run on, or NULL for a stream the context creates */
int gbp_create(gbp_ctx** ctx, int device, void* stream);
int gbp_destroy(gbp_ctx* ctx);
void gbp_default_params(gbp_params* params);
int gbp_set_params(gbp_ctx* ctx, const gbp_params* params);
int gbp_get_stream(const gbp_ctx* ctx, void** stream);

/* ---------------------------------------------------------------- problem (SCIP_ConsData of all linear rows)
 * Replaces the per-row vars/vals/lhs/rhs that cons_linear keeps in struct SCIP_ConsData (cons_linear.c:187-266)
 * and the column-major view of SCIPmatrixCreate (src/scip/matrix.c:703); the CSC copy is built here.
 * rowptr[m+1] (int64), colidx[nnz] (0..n-1, no repeats inside a row), vals[nnz] (nonzero), lhs/rhs[m],
 * isint[n] (nonzero = integral column, SCIPvarIsIntegral).  m must be below 2^30. */
int gbp_upload_problem(gbp_ctx* ctx, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
   const double* vals, const double* lhs, const double* rhs, const int8_t* isint);

/* ---------------------------------------------------------------- plain path: one problem per call
 * Propagates lb/ub (length n, in place) to the fixpoint.  The first frontier is every row (nseed < 0), or
 * the rows that the listed column changes make relevant: seedcols[k] moved from [oldlb[k], oldub[k]] to its
 * current bounds (SCIP marks exactly those rows through its bound-change events, cons_linear.c:17162-17255).
 * *cutoff is set to 1 if the problem is infeasible (SCIP_CUTOFF). */
int gbp_propagate(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* seedcols,
   const double* oldlb, const double* oldub, int32_t* cutoff, gbp_result* res);
int gbp_propagate_device(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* seedcols,
   const double* oldlb, const double* oldub, int32_t* cutoff, gbp_result* res);

/* row activities from scratch (min/max activity as double-double plus the eight infinity/huge counters of
 * struct SCIP_ConsData): act[4*i] = minhi, minlo, maxhi, maxlo; cnt[8*i] = minposinf, minneginf,
 * minposhuge, minneghuge, maxposinf, maxneginf, maxposhuge, maxneghuge; for all m rows. */
int gbp_row_activities(gbp_ctx* ctx, const double* lb, const double* ub, double* act, int32_t* cnt);

/* global domain of the plain path, for the binary test of GBP_FLAG_NOSORTVARS (a column is binary when it is
 * integral and its global bounds lie inside [0,1], SCIPvarIsBinary, var.c:23801-23810).  glb/gub (host arrays
 * of length n) are copied and used by later gbp_propagate calls until cleared with NULL or until the next upload;
 * without them a call treats the bounds it propagates as global, as SCIP does at the root (depth 0).  The
 * plugin passes SCIPvarGetLbGlobal/SCIPvarGetUbGlobal.  Batched nodes use their base bounds. */
int gbp_set_global_bounds(gbp_ctx* ctx, const double* glb, const double* gub);

/* change log of the plain path, for conflict analysis.  With a capacity > 0, every later gbp_propagate /
 * gbp_propagate_device / gbp_propagate_instances call records each accepted bound change: the column, the round
 * that made it, and the column's bounds after it (a column that moves in several rounds appears once per round).
 * Each change follows from the bounds at the start of its round, so applying the log round by round through
 * SCIPinferVarLbProp / SCIPinferVarUbProp lets SCIP explain every change from bounds it already holds (the
 * propagator's resolve callback, type_prop.h:258, as cons_linear's resolvePropagation does, cons_linear.c:5097).
 * Capacity 0 switches the log off. */
int gbp_set_change_log(gbp_ctx* ctx, int64_t capacity);
/* the last call's log sorted by (round, column): up to cap entries into col/round/lb/ub (host arrays), *n = the
 * number of changes the call made.  GBP_ERR_OVERFLOW if the log capacity or cap was smaller than *n. */
int gbp_get_change_log(gbp_ctx* ctx, int64_t cap, int32_t* col, int32_t* round, double* lb, double* ub, int64_t* n);
/* with GBP_FLAG_RANGEDROW, the rows whose ranged-row rule proposed bounds for a column (col) or found the row
 * infeasible (col = -1) in the last call, with the round: up to cap records sorted by (round, col, row), *n = the
 * number recorded.  Kept beside the change log (same capacity).  A change that no row's activities explain was
 * proposed by one of these rows, whose other columns' bounds at that time imply it (cons_linear explains its
 * ranged-row changes by the bounds of the row's fixed columns, addConflictFixedVars, cons_linear.c:4981). */
int gbp_get_ranged_log(gbp_ctx* ctx, int64_t cap, int32_t* round, int32_t* col, int32_t* row, int64_t* n);

/* ---------------------------------------------------------------- batched path: distinct instances
 * Uneven independent instances (each a set of linear rows with its own columns) propagated together: instance k
 * owns rows [row_off[k], row_off[k+1]) and columns [col_off[k], col_off[k+1]) of one block-diagonal problem whose
 * rows reference only their own instance's columns (global column indices).  gbp_propagate_instances runs every
 * instance's root fixpoint from the given bounds -- what SCIP's root propagation does per instance -- with the
 * frontier rows of all instances in the same launches; inst_cutoff[k] = 1 marks an infeasible instance (its
 * bounds are then meaningless).  The upload replaces any problem uploaded before. */
int gbp_upload_instances(gbp_ctx* ctx, int64_t ninst, const int64_t* row_off, const int64_t* col_off,
   const int64_t* rowptr, const int32_t* colidx, const double* vals, const double* lhs, const double* rhs,
   const int8_t* isint);
/* the same upload from the instances as separate parts, with no host-side concatenation: part k has m_k[k] rows
 * and n_k[k] columns, its own CSR (rowptr_k[k] with m_k[k] + 1 entries from 0; colidx_k[k] LOCAL column indices in
 * [0, n_k[k])), sides and integrality.  Each part is copied straight to its place on the device, where one kernel
 * shifts the row pointers and column indices and fills the instance maps.  The result equals gbp_upload_instances
 * of the concatenation. */
int gbp_upload_instance_list(gbp_ctx* ctx, int64_t ninst, const int64_t* m_k, const int64_t* n_k,
   const int64_t* const* rowptr_k, const int32_t* const* colidx_k, const double* const* vals_k,
   const double* const* lhs_k, const double* const* rhs_k, const int8_t* const* isint_k);
int gbp_propagate_instances(gbp_ctx* ctx, double* lb, double* ub, int8_t* inst_cutoff, gbp_result* res);
int gbp_propagate_instances_device(gbp_ctx* ctx, double* lb, double* ub, int8_t* inst_cutoff, gbp_result* res);

/* ---------------------------------------------------------------- plain path, sparse form
 * For a host that keeps its bounds on the device between calls, as a SCIP propagator does from node to node:
 * gbp_set_bounds copies lb/ub (length n) to the context once; each gbp_propagate_changes then sends only the
 * columns whose bounds the host changed since (cols[k] takes [newlb[k], newub[k]]; tightening or loosening; a
 * column at most once) and propagates from them as gbp_propagate does with seeds: a change marks the rows for
 * which it tightens a bound relative to seedlb[k]/seedub[k], or, when those are NULL, relative to the device's
 * bounds before the call.  (Moving from one search node to another, SCIP relaxes to the common ancestor and
 * tightens from there; a host that passes the ancestor's or the global bounds as seeds marks the rows SCIP marks,
 * or more, with the same results.)  Returns the columns whose bounds propagation moved, sorted by column, with
 * their bounds: *nout of them in outcols/outlb/outub (capacity cap).  The device copy then holds the propagated
 * bounds.  On a cutoff (*cutoff = 1, also when a change has newlb > newub) or when more than cap columns moved
 * (GBP_ERR_OVERFLOW, *nout = the capacity needed) it holds the bounds after the host's changes, so that the call
 * can be repeated.  gbp_propagate, gbp_row_activities and the instance calls use the same device arrays: after
 * them, gbp_set_bounds again. */
int gbp_set_bounds(gbp_ctx* ctx, const double* lb, const double* ub);
int gbp_propagate_changes(gbp_ctx* ctx, int64_t nchg, const int32_t* cols, const double* newlb, const double* newub,
   const double* seedlb, const double* seedub, int64_t cap, int64_t* nout, int32_t* outcols, double* outlb,
   double* outub, int32_t* cutoff, gbp_result* res);

/* ---------------------------------------------------------------- batched path: branch-and-bound nodes
 * nnodes nodes share the uploaded rows and the base bounds baselb/baseub (length n); node k applies the
 * bound changes chg_col/chg_lb/chg_ub[ptr[k] .. ptr[k+1]) (tightenings, as SCIPchgVarLb/UbProbing; a column named
 * more than once in a node takes the tightest of its bounds, and a node whose bounds for a column cross is cut off)
 * and propagates to its own fixpoint -- the per-node work SCIP does in
 * SCIPpropagateProbing (src/scip/scip_probing.c:581) or at each branch-and-bound node.  All nodes run in one
 * persistent launch.  Per node: out_cutoff[k], out_rounds[k] and the columns whose final bounds differ from
 * the base: out_n[k] entries at out_col/out_lb/out_ub[out_off[k] ..].  Node results are packed in completion
 * order into arrays of out_cap entries; a node that does not fit gets out_n[k] = -1 and the call returns
 * GBP_ERR_OVERFLOW.  A change column outside [0, n) is caught by the kernel: that node is given up
 * (out_cutoff[k] = 1) and the call returns GBP_ERR_INVALID. */
int gbp_propagate_nodes(gbp_ctx* ctx, const double* baselb, const double* baseub, int64_t nnodes,
   const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
   int8_t* out_cutoff, int32_t* out_rounds, int64_t* out_off, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int64_t out_cap, gbp_result* res);
int gbp_propagate_nodes_device(gbp_ctx* ctx, const double* baselb, const double* baseub, int64_t nnodes,
   const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
   int8_t* out_cutoff, int32_t* out_rounds, int64_t* out_off, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int64_t out_cap, gbp_result* res);

/* launch shape of the batched kernel -- what the autotuner sets: threads that work on one node (one CTA per node
 * at a time) and the register budget the kernel variant was compiled for, given as resident CTAs per SM.
 * Compiled shapes: (32,16) (32,24) (64,8) (64,12) (128,4) (128,6) (256,2); ctas_per_sm = 0 picks the first
 * listed budget for that width.  Results never depend on the shape. */
int gbp_set_batch_shape(gbp_ctx* ctx, int32_t threads_per_node, int32_t ctas_per_sm);

/* ---------------------------------------------------------------- batched path without allocation
 * No counterpart in the reference: an addition for callers that cannot let a library allocate device memory
 * -- applications that give all device memory to their own pool allocator at start-up, and callers that must
 * not trigger the implicit device-wide synchronisation of cudaMalloc/cudaFree (for example a propagation
 * callback running while other streams of the host application are busy).  It computes what
 * gbp_propagate_nodes_device computes in rounds (GBP_FLAG_SCIPORDER and GBP_FLAG_RANGEDROW are refused with
 * GBP_ERR_INVALID; the binary test of sortvars reads the base bounds, as the batched path does), without a context:
 * every array argument is a device pointer supplied by the caller (the rows in CSR and plain CSC form:
 * colptr[n+1], rowidx[nnz], cvals[nnz]; the arrays must hold the entries their pointers describe), and the scratch
 * is one fixed __device__ array of GBP_NOALLOC_SCRATCH_BYTES inside libgbp that every GPU loading the library
 * holds until exit.  The call allocates nothing (no cudaMalloc, cudaFree or allocating library routine).
 * Limits: one node slot needs about 64*n + 12*m bytes; the call uses as many slots as fit (at most one per
 * resident CTA) and returns GBP_ERR_TOO_LARGE when not even one fits (about n <= 900,000 for m = n/2), so
 * only problems far below that limit run with useful parallelism.
 * The first call on a device (with that device current) looks up the array's address; make it before any
 * stream capture.  All calls on a device share the array, so calls that overlap on the GPU race and must be
 * serialised by the caller.  Before any node runs, two kernels check the pointers (starting at 0, monotone, the same
 * number of entries) and the indices (columns in [0, n), rows in [0, m)); if a check fails no node runs, every
 * node reports out_n[k] = -1 and the call returns GBP_ERR_INVALID.  stream: a cudaStream_t or NULL.  With
 * res == NULL the call only enqueues work and returns GBP_OK: the outputs are then the only report (a node that
 * did not fit the output or whose arrays failed the checks shows out_n[k] = -1; a node with a change column outside
 * [0, n) shows out_cutoff[k] = 1; a node stopped at the round limit holds valid bounds); with res != NULL it waits
 * for the stream, fills res and returns GBP_ERR_INVALID / GBP_ERR_LIMIT / GBP_ERR_OVERFLOW like
 * gbp_propagate_nodes_device.  params == NULL uses the defaults of gbp_default_params. */
/* ---------------------------------------------------------------- serving
 * A request loop inside libgbp for branch-and-bound node requests against one resident problem and its root bounds
 * (the served form of the batched path), and for instance requests (below).  A client thread submits a node -- bound
 * changes, as one node of gbp_propagate_nodes -- and gets a ticket at once; the node's arrays are copied.  nworkers worker threads, each with its own context and stream,
 * take everything queued (up to max_batch nodes) and propagate it in one batched launch, so that requests arriving
 * together share a launch and the batches of different workers overlap on the device.  Admission: at creation every
 * worker runs a first batch (its slot memory is allocated then); the budget for the device bytes of batches in flight
 * is the smaller of hbm_cap (bytes, 0: 150 GB) and the free device memory that remains (cudaMemGetInfo).  A worker
 * takes requests only while its batch's bytes fit what the budget has left; a request that alone exceeds the budget is
 * refused at submission (GBP_ERR_NOMEM).  A node change column outside [0, n) is refused at submission
 * (GBP_ERR_INVALID).  gbp_server_poll waits up to wait_ms (negative: without limit) for a ticket's reply: GBP_OK with
 * *cutoff and the columns whose bounds moved against the root bounds (sorted, *nout of them in cols/lb/ub of capacity
 * cap), GBP_ERR_OVERFLOW with *nout the capacity needed (the reply stays available), GBP_ERR_BUSY when the wait ended
 * first.  A reply is released once read.  t_submit_ns / t_done_ns (may be NULL): when the server took the request and
 * when its batch finished (ns of a steady clock started with the server). */
typedef struct gbp_server gbp_server;
int gbp_server_create(gbp_server** out, int device, int nworkers, int ninstworkers, int64_t max_batch,
   int64_t hbm_cap, const gbp_params* params, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
   const double* vals, const double* lhs, const double* rhs, const int8_t* isint, const double* rootlb,
   const double* rootub);
int gbp_server_submit(gbp_server* srv, int64_t nchg, const int32_t* cols, const double* lb, const double* ub,
   int64_t* ticket);
/* an instance request: a problem of its own (m rows in CSR over its n local columns, sides, integrality, bounds),
 * answered with its root fixpoint -- the reply's columns are 0..n-1 in order with their final bounds, or a cutoff.
 * ninstworkers worker threads (each with its own context) upload everything queued as parts of one block-diagonal
 * problem (gbp_upload_instance_list) and propagate it in one batched launch (gbp_propagate_instances), taking up to
 * max_batch / 8 instances at once.  The instance's arrays are BORROWED, not copied: they must stay valid and
 * unchanged until gbp_server_poll has returned this ticket's reply (or an error other than GBP_ERR_BUSY and
 * GBP_ERR_OVERFLOW).  Submission checks the pointers and rowptr[0] == 0; the upload checks that the row pointers do
 * not decrease and that every column index lies in [0, n), and a request that fails them is answered
 * GBP_ERR_INVALID by gbp_server_poll while the rest of its batch is served.  A server created without instance
 * workers refuses instance requests (GBP_ERR_INVALID).  The device memory an instance worker's context holds for
 * its largest batch stays allocated until gbp_server_destroy and is not counted against the admission budget. */
int gbp_server_submit_instance(gbp_server* srv, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
   const double* vals, const double* lhs, const double* rhs, const int8_t* isint, const double* lb,
   const double* ub, int64_t* ticket);
int gbp_server_poll(gbp_server* srv, int64_t ticket, int wait_ms, int32_t* cutoff, int64_t cap, int64_t* nout,
   int32_t* cols, double* lb, double* ub, int64_t* t_submit_ns, int64_t* t_done_ns);
/* batches launched, requests served, the largest batch, the admission budget in bytes */
int gbp_server_stats(const gbp_server* srv, int64_t* batches, int64_t* requests, int64_t* max_batch_seen,
   int64_t* budget);
/* finishes the queued requests, stops the workers and frees everything */
int gbp_server_destroy(gbp_server* srv);

#define GBP_NOALLOC_SCRATCH_BYTES (64ull << 20)
int gbp_propagate_nodes_noalloc(int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
   const double* vals, const double* lhs, const double* rhs, const int8_t* isint, const int64_t* colptr,
   const int32_t* rowidx, const double* cvals, const double* baselb, const double* baseub, int64_t nnodes,
   const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub, int8_t* out_cutoff,
   int32_t* out_rounds, int64_t* out_off, int32_t* out_n, int32_t* out_col, double* out_lb, double* out_ub,
   int64_t out_cap, const gbp_params* params, void* stream, gbp_result* res);

#ifdef __cplusplus
}
#endif

#endif
