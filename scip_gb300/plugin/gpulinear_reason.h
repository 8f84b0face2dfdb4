/* Reasons for the bound changes of the gpulinear propagator, for SCIP's conflict analysis.
 *
 * The device accepts, per column and round, the best candidate over all rows, so it does not say which row made a
 * change.  When SCIP asks for the reason of a change (the propagator's resolve callback, type_prop.h:258), this
 * module finds a row of the column whose other columns' bounds at that time imply the change, and adds the bounds
 * of that row that cons_linear's addConflictBounds (cons_linear.c:4799-4970) would add for it.
 *
 * The module is plain C without SCIP: bounds come in and reason bounds go out through callbacks, so that SCIP's
 * bound-change history (SCIPgetVarLb/UbAtIndex, SCIPaddConflictLb/Ub) plugs in from the propagator and a test
 * harness can drive it with arrays. */
#ifndef GPULINEAR_REASON_H
#define GPULINEAR_REASON_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* the rows as the propagator uploads them (CSR) and their column view (CSC) */
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
   const int64_t* colptr;   /* CSC: rows of column j at rowidx[colptr[j] .. colptr[j+1]) */
   const int32_t* rowidx;
   const int64_t* rowpos;   /* position of that entry inside its row's CSR range */
} gpl_rows;

typedef struct
{
   void* ud;
   double (*lb)(void* ud, int32_t col);    /* local bound when the change was made (before it) */
   double (*ub)(void* ud, int32_t col);
   double (*glb)(void* ud, int32_t col);   /* global bound */
   double (*gub)(void* ud, int32_t col);
   double (*lbafter)(void* ud, int32_t col);  /* the inferred column's bounds just after the change */
   double (*ubafter)(void* ud, int32_t col);
   int (*addlb)(void* ud, int32_t col);    /* add the column's local lower / upper bound to the reason; 0 = ok */
   int (*addub)(void* ud, int32_t col);
} gpl_io;

typedef struct
{
   double infinity;
   double feastol;
   double epsilon;
} gpl_num;

/* Explains "column col has lower (islower) or upper bound bound" with one row.  Returns the row used (>= 0), -1 if
 * no row implies the bound (then nothing was added), or -2 if an add callback failed. */
int64_t gpl_explain(const gpl_rows* R, const gpl_num* num, const gpl_io* io, int32_t col, int islower, double bound);

/* A row that the bounds io->lb/io->ub make infeasible (minimal activity above rhs or maximal below lhs, beyond
 * feastol), explained as cons_linear's analyzeConflict does for an infeasible row (addConflictBounds without an
 * inferred column, cons_linear.c:4799): returns the row (>= 0) after adding its reason bounds, -1 if no row is
 * infeasible, -2 if an add callback failed. */
int64_t gpl_explain_infeasible(const gpl_rows* R, const gpl_num* num, const gpl_io* io);

/* Reason of a change made by row `row`'s ranged-row rule (col = the inferred column), or of that row found
 * infeasible by it (col = -1): every bound of the row's columns that differs from the column's global bound --
 * cons_linear's addConflictFixedVars (cons_linear.c:4981-5037) widened from the fixed columns to all, since the rule
 * reads the bounds of every unfixed column too.  The inferred column's own bounds before the change are included.
 * Valid whenever the bounds io reads are at least as tight as those the rule ran on.  Returns 0, or -2 if an add
 * callback failed. */
int gpl_explain_ranged(const gpl_rows* R, const gpl_num* num, const gpl_io* io, int64_t row, int32_t col);

/* builds colptr/rowidx/rowpos of R from its CSR part; the arrays have n+1, nnz and nnz entries */
void gpl_build_columns(int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx, int64_t* colptr,
   int32_t* rowidx, int64_t* rowpos);

#ifdef __cplusplus
}
#endif

#endif
