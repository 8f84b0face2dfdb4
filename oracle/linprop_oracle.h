/* Test infrastructure only: CPU restatement of SCIP's cons_linear activity-based bound propagation,
 * used by tests/, smoke() and the CPU-baseline leg of bench.py as the checker of the CUDA path.
 * It is never linked into the product library (scip_gb300/_lib/libgbp.so).
 *
 * Round semantics (shared with the CUDA path, so that both produce bit-identical integer bounds):
 *   a round takes the current frontier of rows and the bounds B_r at the start of the round;
 *   every frontier row computes its activities from B_r and emits candidate bounds with SCIP's rules;
 *   per column the best candidates (min upper / max lower) are accepted with SCIP's acceptance rules
 *   against B_r (upper bound first, then lower bound against the new upper bound); the next frontier
 *   is every row holding a column whose bound moved in a direction that row's finite sides can use.
 * SCIP itself (cons_linear.c consPropLinear) walks marked rows one at a time and applies each
 * tightening at once; because of the minimal-improvement test (set.c:7711-7753) the two orders can stop
 * at different, equally valid fixpoints.  tests/golden holds SCIP's own results to measure that.
 */
#ifndef LINPROP_ORACLE_H
#define LINPROP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
   double infinity;             /* numerics/infinity, def.h:172 */
   double epsilon;              /* numerics/epsilon */
   double sumepsilon;           /* numerics/sumepsilon */
   double feastol;              /* numerics/feastol */
   double hugeval;              /* numerics/hugeval */
   double boundstreps;          /* numerics/boundstreps */
   double recompfac;            /* numerics/recompfac */
   double maxeasyactivitydelta; /* constraints/linear/maxeasyactivitydelta (0 = residual rule everywhere) */
   int32_t maxrounds;           /* round cap; <= 0 means 1,000,000 */
   int32_t flags;               /* LPO_FLAG_* */
} lpo_params;

/* constraints/linear/sortvars = FALSE: every entry of a row is tried (no skipping of the binaries that
 * follow one that cannot be tightened, cons_linear.c:7131-7136) */
#define LPO_FLAG_NOSORTVARS 1
/* constraints/linear/rangedrowpropagation = TRUE with rangedrowartcons = FALSE: the gcd-based propagation of
 * ranged rows and equations (rangedRowPropagation, cons_linear.c:5715-6695) runs after each frontier row's
 * activity rules, from the same round-start bounds; its bound changes are forced ones, as SCIP's are */
#define LPO_FLAG_RANGEDROW 2

typedef struct
{
   int64_t m;
   int64_t n;
   const int64_t* rowptr;
   const int32_t* colidx;
   const double* vals;
   const double* lhs;
   const double* rhs;
   const int8_t* isint;
   const int64_t* colptr;
   const int32_t* rowidx;
   const double* cvals;
   const int32_t* varidx;   /* SCIP's problem index of each column (ties of consdataCompVarProp), NULL: the column */
} lpo_problem;

typedef struct
{
   int32_t cutoff;
   int32_t rounds;
   int32_t status;      /* 0 fixpoint, 1 cutoff, 2 round limit */
   int32_t reserved;
   int64_t rows;        /* frontier rows processed over all rounds */
   int64_t nnz;         /* nonzeros of those rows */
   int64_t candidates;  /* candidate bounds emitted (sequential order: entries evaluated) */
   int64_t changes;     /* accepted bound changes (lower and upper counted separately) */
   int64_t live_rows;   /* sequential order: rows whose tightenBounds got past its skip tests */
} lpo_result;

void lpo_default_params(lpo_params* p);

/* activities of rows[0..nrows) (all rows if rows == NULL) from scratch under [lb,ub]:
 * act[4*k..] = minhi, minlo, maxhi, maxlo (double-double), cnt[8*k..] = minposinf, minneginf, minposhuge,
 * minneghuge, maxposinf, maxneginf, maxposhuge, maxneghuge. */
void lpo_row_activities(const lpo_problem* prob, const lpo_params* par, const double* lb, const double* ub,
   const int32_t* rows, int64_t nrows, double* act, int32_t* cnt);

/* propagate to fixpoint in place; the first frontier is every row (seedcols == NULL) or the rows that the
 * listed column changes make relevant (seedcols[k] moved from [oldlb[k],oldub[k]] to the bounds in lb/ub).
 * glb/gub: the global domain that decides which integer columns count as binary (SCIPvarIsBinary); NULL
 * means the current bounds (propagation at the root, where local and global bounds coincide). */
int lpo_propagate(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub,
   int64_t nseed, const int32_t* seedcols, const double* oldlb, const double* oldub, const double* glb,
   const double* gub, lpo_result* res);

/* change log: every accepted bound change with the round that made it and the column's bounds after it,
 * entries grouped by round in the order they are accepted; n counts all changes, at most cap are stored.
 * With LPO_FLAG_RANGEDROW also the ranged-row records: each row whose ranged rule proposed bounds for a column
 * (rcol) or found itself infeasible (rcol = -1), with the round; rn counts them, at most rcap are stored
 * (rrow NULL: not recorded) */
typedef struct
{
   int64_t cap;
   int64_t n;
   int32_t* col;
   int32_t* round;
   double* lb;
   double* ub;
   int64_t rcap;
   int64_t rn;
   int32_t* rrow;
   int32_t* rcol;
   int32_t* rround;
} lpo_log;

/* lpo_propagate that also fills *log (log may be NULL) */
int lpo_propagate_logged(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub,
   int64_t nseed, const int32_t* seedcols, const double* oldlb, const double* oldub, const double* glb,
   const double* gub, lpo_result* res, lpo_log* log);

/* batch of nodes sharing base bounds, which are also every node's global domain: node k applies bound
 * changes chg_col/chg_lb/chg_ub[ptr[k]..ptr[k+1]) and propagates; outputs per node the cutoff flag, rounds, and up to cap changed columns
 * (out_col/out_lb/out_ub[k*cap..]) whose final bounds differ from the base; out_n[k] = count (or -1 if
 * more than cap).  nthreads <= 0 uses one thread. Returns 0. */
int lpo_propagate_nodes(const lpo_problem* prob, const lpo_params* par, const double* baselb, const double* baseub,
   int64_t nnodes, const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
   int8_t* out_cutoff, int32_t* out_rounds, int32_t* out_n, int32_t* out_col, double* out_lb, double* out_ub,
   int32_t cap, int32_t nthreads, lpo_result* total);

/* ------------------------------------------------------------------ SCIP's own order (linprop_seq.c)
 * SCIP walks the rows marked for propagation one at a time and applies every tightening at once; the bound-change
 * events update the other rows' activities incrementally and mark them.  These entry points restate that order:
 *   - marked rows are processed in SCIP's propconss order: a newly marked row is appended; unmarking moves the last
 *     marked row into the freed place; marks, unmarks and deletions made while consPropLinear runs are applied
 *     after it, the last one first;
 *   - per row, tightenBounds visits the entries in the row's order (up to 10 passes, stopping at the entry of the
 *     last change, binaries skipped after the first unfixed binary that did not tighten);
 *   - activities are computed on first use in the row's order and then updated incrementally by every bound change
 *     of the row's columns, with SCIP's reliability test (recomputed last entry first when unreliable);
 *   - a propagation round is one pass over the rows marked at its start; rounds repeat until one changes nothing.
 *
 * lpo_propagate_seq: the root (depth 0).  Every row starts marked, in row order; bound changes are global, so a
 * column that turns into an unfixed binary unsorts its rows; rows are sorted (consdataCompVarProp on the current
 * bounds) when tightenBounds first needs them; a redundant row is deleted.  out_order (nnz entries, or NULL)
 * receives each row's final order: out_order[rowptr[i] + k] = CSR position of the row's k-th entry.
 *
 * lpo_propagate_nodes_seq: branch-and-bound nodes (depth >= 1) on top of base bounds that are a fixpoint (SCIP's
 * root).  Each row's entries are taken in storage order, which must be the order SCIP holds the row in (out_order
 * of lpo_propagate_seq, or SCIP's own, or consdataCompVarProp on the base bounds); with sortvars its leading
 * binaries (under the base bounds) are SCIP's nbinvars.  A node applies its changes as SCIPchgVarLb/UbProbing do
 * (each change's events mark rows at once), then propagates; a row counts as tightened at the root until a change
 * that its finite sides can use.  Rows redundant under the base bounds are the rows SCIP's root deleted
 * (lpo_root_deleted_rows): they take no part.  Outputs as lpo_propagate_nodes. */
int lpo_propagate_seq(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub, int32_t* out_order,
   lpo_result* res);
void lpo_root_deleted_rows(const lpo_problem* prob, const lpo_params* par, const double* lb, const double* ub,
   uint8_t* del);
int lpo_propagate_nodes_seq(const lpo_problem* prob, const lpo_params* par, const double* baselb,
   const double* baseub, int64_t nnodes, const int64_t* ptr, const int32_t* chg_col, const double* chg_lb,
   const double* chg_ub, int8_t* out_cutoff, int32_t* out_rounds, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int32_t cap, int32_t nthreads, lpo_result* total);

/* Carrying the root's activities into the nodes, as SCIP does.  lpo_propagate_nodes_seq starts each row of a node
 * with activities computed afresh on first use; SCIP's node rows keep the activities the root's incremental updates
 * left (consdataUpdateActivities, cons_linear.c:1604-1992, run by the root's bound-change events, with validity
 * flags and reliability references that survive into the probing node).  The two differ only in the last bits of
 * those activities, which a row with coefficients of very different magnitudes can amplify past the continuous
 * tolerance.  lpo_propagate_seq_states is lpo_propagate_seq that also copies the final row states into out_states
 * (lpo_seq_state_bytes(m) bytes; an opaque record per row); lpo_propagate_nodes_seq_from is lpo_propagate_nodes_seq
 * whose rows start from those states (root_states NULL: afresh), and whose rows deleted at the root are the rows
 * the root restatement deleted (lpo_seq_states_deleted) instead of the rows redundant under the base bounds
 * (lpo_root_deleted_rows, which differs from SCIP's deletions both ways on some instances: SCIP deletes a redundant
 * row only when it propagates the row again after its last column change, and a change that only lowers a
 * one-sided row's slack does not mark it; and SCIP's redundancy test reads incrementally updated activities, which
 * can pass by a last-bit margin where activities computed afresh do not).  The rows of
 * prob may be stored in another order than the root's problem (the order SCIP holds them in after the root); row
 * indices must be the same. */
size_t lpo_seq_state_bytes(int64_t m);
void lpo_seq_states_deleted(const void* states, int64_t m, uint8_t* del);
int lpo_propagate_seq_states(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub,
   int32_t* out_order, lpo_result* res, void* out_states);
int lpo_propagate_nodes_seq_from(const lpo_problem* prob, const lpo_params* par, const double* baselb,
   const double* baseub, int64_t nnodes, const int64_t* ptr, const int32_t* chg_col, const double* chg_lb,
   const double* chg_ub, int8_t* out_cutoff, int32_t* out_rounds, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int32_t cap, int32_t nthreads, lpo_result* total, const void* root_states);

#ifdef __cplusplus
}
#endif

#endif
