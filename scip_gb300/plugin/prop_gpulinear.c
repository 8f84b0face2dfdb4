/* prop_gpulinear.c -- SCIP propagator plugin over libgbp (see prop_gpulinear.h).
 *
 * Call path: SCIPpropExec (src/scip/prop.c:646) -> propExecGpulinear -> gbp_propagate_changes (C ABI, one device
 * round trip per call: the columns whose local bounds differ from the device's copy in, the columns propagation
 * moved and the cutoff flag out; the first call after an upload or a cutoff sends every bound through
 * gbp_propagate) -> SCIPinferVarLb/UbProp or SCIPtightenVarLb/Ub for every moved bound.
 */
#include <float.h>
#include <limits.h>
#include <stdint.h>
#include <string.h>

#include "prop_gpulinear.h"
#include "gpulinear_reason.h"
#include "scip/cons_linear.h"
#include "scip/cons_knapsack.h"
#include "scip/cons_logicor.h"
#include "scip/cons_setppc.h"
#include "scip/cons_varbound.h"
#include "gbp.h"

#define PROP_NAME     "gpulinear"
#define PROP_DESC     "linear-constraint bound propagation on a GB300 GPU (cons_linear rules, libgbp)"
#define PROP_PRIORITY 1000 /* >= 0: runs before the constraint handlers' propagation (solve.c:481-591) */
#define PROP_FREQ     1
#define PROP_DELAY    FALSE
#define PROP_TIMING   SCIP_PROPTIMING_BEFORELP

struct SCIP_PropData
{
   gbp_ctx*              ctx;                /**< libgbp context (NULL while inactive) */
   int                   device;             /**< CUDA device ordinal */
   SCIP_Bool             replacelinear;      /**< switch cons_linear's propagation off at include time */
   SCIP_Bool             failed;             /**< the GPU path failed or is unavailable: do not run */
   int                   nconss;             /**< number of constraints the matrix was built from */
   SCIP_Bool             specialised;        /**< also the rows of setppc, logicor, knapsack, varbound constraints */
   SCIP_Bool             replacespecialised; /**< switch those handlers' propagation off at include time */
   SCIP_Bool             inprobing;          /**< also propagate in probing nodes */
   SCIP_Bool             sciporder;          /**< batched nodes in SCIP's own order (GBP_FLAG_SCIPORDER) */
   int                   nspecialrows;       /**< rows of the matrix from handlers other than linear */
   int                   nrows;              /**< rows in the matrix */
   int                   ncols;              /**< columns = transformed variables */
   SCIP_VAR**            vars;               /**< column -> variable */
   int64_t*              rowptr;
   int32_t*              colidx;
   double*               vals;
   double*               lhs;
   double*               rhs;
   int8_t*               isint;
   double*               lb;                 /**< bounds handed to the device / returned from it */
   double*               ub;
   double*               snaplb;             /**< the device's copy of the bounds after the previous call */
   double*               snapub;
   double*               chglb;              /**< bounds of the columns sent to the device (gbp_propagate_changes) */
   double*               chgub;
   int32_t*              outcols;            /**< columns the device moved, with their bounds */
   double*               outlb;
   double*               outub;
   SCIP_Bool             havesnap;
   double*               glb;                /**< global bounds last passed to the device (binary test) */
   double*               gub;
   SCIP_Bool             haveglobal;
   int64_t*              colptr;             /**< column view of the rows, for the reasons of conflict analysis */
   int32_t*              rowidx;
   int64_t*              rowpos;
   int64_t               logcap;             /**< change log of the last call: column, round, bounds after */
   int32_t*              logcol;
   int32_t*              loground;
   double*               loglb;
   double*               logub;
   int32_t*              seeds;
   double*               seedlo;
   double*               seedhi;
   SCIP_Bool             ranged;             /**< the device runs the ranged-row rule (GBP_FLAG_RANGEDROW) */
   int64_t               rcap;               /**< ranged-row records of the recent calls, sorted by (call, round,
                                              *   column, row): the rows that explain ranged-row changes */
   int64_t               rn;
   SCIP_Longint*         rcall;
   int32_t*              rround;
   int32_t*              rcol;              /**< -1: the row was found infeasible */
   int32_t*              rrow;
   int32_t*              tround;             /**< one call's records as fetched (logcap entries) */
   int32_t*              tcol;
   int32_t*              trow;
   SCIP_Longint          ncalls;
   SCIP_Longint          nchgbds;
   SCIP_Longint          ncutoffs;
   SCIP_Longint          nresolves;          /**< conflict-resolution requests for this propagator's changes */
   SCIP_Longint          nresolved;          /**< ... explained with a row */
   SCIP_Longint          nconflicts;         /**< cutoffs handed to conflict analysis with an infeasible row */
   SCIP_Longint          nrangedreasons;     /**< ... of the resolved changes and analysed cutoffs: by a ranged row */
};

static void freeMatrix(SCIP* scip, SCIP_PROPDATA* pd)
{
   SCIPfreeMemoryArrayNull(scip, &pd->vars);
   SCIPfreeMemoryArrayNull(scip, &pd->rowptr);
   SCIPfreeMemoryArrayNull(scip, &pd->colidx);
   SCIPfreeMemoryArrayNull(scip, &pd->vals);
   SCIPfreeMemoryArrayNull(scip, &pd->lhs);
   SCIPfreeMemoryArrayNull(scip, &pd->rhs);
   SCIPfreeMemoryArrayNull(scip, &pd->isint);
   SCIPfreeMemoryArrayNull(scip, &pd->lb);
   SCIPfreeMemoryArrayNull(scip, &pd->ub);
   SCIPfreeMemoryArrayNull(scip, &pd->snaplb);
   SCIPfreeMemoryArrayNull(scip, &pd->snapub);
   SCIPfreeMemoryArrayNull(scip, &pd->chglb);
   SCIPfreeMemoryArrayNull(scip, &pd->chgub);
   SCIPfreeMemoryArrayNull(scip, &pd->outcols);
   SCIPfreeMemoryArrayNull(scip, &pd->outlb);
   SCIPfreeMemoryArrayNull(scip, &pd->outub);
   SCIPfreeMemoryArrayNull(scip, &pd->glb);
   SCIPfreeMemoryArrayNull(scip, &pd->gub);
   pd->haveglobal = FALSE;
   SCIPfreeMemoryArrayNull(scip, &pd->colptr);
   SCIPfreeMemoryArrayNull(scip, &pd->rowidx);
   SCIPfreeMemoryArrayNull(scip, &pd->rowpos);
   SCIPfreeMemoryArrayNull(scip, &pd->logcol);
   SCIPfreeMemoryArrayNull(scip, &pd->loground);
   SCIPfreeMemoryArrayNull(scip, &pd->loglb);
   SCIPfreeMemoryArrayNull(scip, &pd->logub);
   pd->logcap = 0;
   SCIPfreeMemoryArrayNull(scip, &pd->seeds);
   SCIPfreeMemoryArrayNull(scip, &pd->seedlo);
   SCIPfreeMemoryArrayNull(scip, &pd->seedhi);
   SCIPfreeMemoryArrayNull(scip, &pd->rcall);
   SCIPfreeMemoryArrayNull(scip, &pd->rround);
   SCIPfreeMemoryArrayNull(scip, &pd->rcol);
   SCIPfreeMemoryArrayNull(scip, &pd->rrow);
   SCIPfreeMemoryArrayNull(scip, &pd->tround);
   SCIPfreeMemoryArrayNull(scip, &pd->tcol);
   SCIPfreeMemoryArrayNull(scip, &pd->trow);
   pd->rcap = 0;
   pd->rn = 0;
   pd->nrows = 0;
   pd->ncols = 0;
   pd->havesnap = FALSE;
}

/* the linear-constraint handlers whose rows the propagator reads: cons_linear always, and with `specialised` the
 * handlers SCIP's presolving upgrades linear rows to (cons_setppc, cons_logicor, cons_knapsack, cons_varbound),
 * whose rows are linear too */
static const char* const HDLRS[] = {"linear", "setppc", "logicor", "knapsack", "varbound"};
#define NHDLRS 5

static int numHandlers(SCIP_PROPDATA* pd) { return pd->specialised ? NHDLRS : 1; }

/** whether the propagator reads constraint cons: globally valid rows only -- not local constraints (valid in a
 *  subtree), not conflict constraints (SCIP adds and deletes them all the time; their handler propagates them),
 *  not modifiable ones */
static SCIP_Bool readsCons(SCIP_CONS* cons)
{
   return !SCIPconsIsLocal(cons) && !SCIPconsIsConflict(cons) && !SCIPconsIsModifiable(cons);
}

/** the constraints of the handlers the propagator reads (rebuild test) */
static int countConss(SCIP* scip, SCIP_PROPDATA* pd)
{
   int h;
   int n = 0;
   for( h = 0; h < numHandlers(pd); ++h )
   {
      SCIP_CONSHDLR* c = SCIPfindConshdlr(scip, HDLRS[h]);
      SCIP_CONS** conss = c == NULL ? NULL : SCIPconshdlrGetConss(c);
      int nc = c == NULL ? 0 : SCIPconshdlrGetNConss(c);
      int k;
      for( k = 0; k < nc; ++k )
         n += readsCons(conss[k]) ? 1 : 0;
   }
   return n;
}

/** the row of constraint cons of handler h as coefficients of (possibly non-active) variables and sides: vars and
 *  vals receive at most size entries (*n = the number needed) */
static SCIP_RETCODE consRow(SCIP* scip, int h, SCIP_CONS* cons, SCIP_VAR** vars, SCIP_Real* vals, int size, int* n,
   SCIP_Real* lhs, SCIP_Real* rhs)
{
   int k;
   SCIP_VAR** cv = NULL;
   *n = 0;
   switch( h )
   {
   case 0:   /* linear: lhs <= sum a x <= rhs */
      *n = SCIPgetNVarsLinear(scip, cons);
      if( *n <= size && *n > 0 )
      {
         memcpy(vars, SCIPgetVarsLinear(scip, cons), sizeof(SCIP_VAR*) * (size_t)*n);
         memcpy(vals, SCIPgetValsLinear(scip, cons), sizeof(SCIP_Real) * (size_t)*n);
      }
      *lhs = SCIPgetLhsLinear(scip, cons);
      *rhs = SCIPgetRhsLinear(scip, cons);
      return SCIP_OKAY;
   case 1:   /* setppc: sum x = 1 (partitioning), <= 1 (packing), >= 1 (covering), cons_setppc.h:47-52 */
      *n = SCIPgetNVarsSetppc(scip, cons);
      cv = SCIPgetVarsSetppc(scip, cons);
      *lhs = SCIPgetTypeSetppc(scip, cons) == SCIP_SETPPCTYPE_PACKING ? -SCIPinfinity(scip) : 1.0;
      *rhs = SCIPgetTypeSetppc(scip, cons) == SCIP_SETPPCTYPE_COVERING ? SCIPinfinity(scip) : 1.0;
      break;
   case 2:   /* logicor: sum x >= 1 */
      *n = SCIPgetNVarsLogicor(scip, cons);
      cv = SCIPgetVarsLogicor(scip, cons);
      *lhs = 1.0;
      *rhs = SCIPinfinity(scip);
      break;
   case 3:   /* knapsack: sum w x <= capacity */
   {
      SCIP_Longint* w = SCIPgetWeightsKnapsack(scip, cons);
      *n = SCIPgetNVarsKnapsack(scip, cons);
      if( *n <= size && *n > 0 )
      {
         memcpy(vars, SCIPgetVarsKnapsack(scip, cons), sizeof(SCIP_VAR*) * (size_t)*n);
         for( k = 0; k < *n; ++k )
            vals[k] = (SCIP_Real)w[k];
      }
      *lhs = -SCIPinfinity(scip);
      *rhs = (SCIP_Real)SCIPgetCapacityKnapsack(scip, cons);
      return SCIP_OKAY;
   }
   default:  /* varbound: lhs <= x + c y <= rhs */
      *n = 2;
      if( size >= 2 )
      {
         vars[0] = SCIPgetVarVarbound(scip, cons);
         vals[0] = 1.0;
         vars[1] = SCIPgetVbdvarVarbound(scip, cons);
         vals[1] = SCIPgetVbdcoefVarbound(scip, cons);
      }
      *lhs = SCIPgetLhsVarbound(scip, cons);
      *rhs = SCIPgetRhsVarbound(scip, cons);
      return SCIP_OKAY;
   }
   if( *n <= size && *n > 0 )
   {
      memcpy(vars, cv, sizeof(SCIP_VAR*) * (size_t)*n);
      for( k = 0; k < *n; ++k )
         vals[k] = 1.0;
   }
   return SCIP_OKAY;
}

/** the constraints of a handler in the order SCIP created them, which is the order a variable's bound-change events
 *  reach them (each constraint catches its variables' events when it is transformed): the transformed constraints
 *  of the original ones in the original order, then the others in the handler's order.  The handler's array loses
 *  that order once constraints are deleted (the last entry moves into the hole, conshdlrDelCons in cons.c). */
static SCIP_RETCODE creationOrder(SCIP* scip, SCIP_CONS** conss, int nc, SCIP_CONS** out)
{
   SCIP_CONS** orig = SCIPgetOrigConss(scip);
   int norig = SCIPgetNOrigConss(scip);
   SCIP_HASHMAP* rank;
   int* key;
   int k;
   SCIP_CALL( SCIPhashmapCreate(&rank, SCIPblkmem(scip), MAX(norig, 1)) );
   SCIP_CALL( SCIPallocBufferArray(scip, &key, MAX(nc, 1)) );
   for( k = 0; k < norig; ++k )
   {
      SCIP_CONS* t = NULL;
      SCIP_CALL( SCIPgetTransformedCons(scip, orig[k], &t) );
      if( t != NULL && !SCIPhashmapExists(rank, (void*)t) )
         SCIP_CALL( SCIPhashmapInsertInt(rank, (void*)t, k) );
   }
   for( k = 0; k < nc; ++k )
   {
      out[k] = conss[k];
      key[k] = SCIPhashmapExists(rank, (void*)conss[k]) ? SCIPhashmapGetImageInt(rank, (void*)conss[k]) : norig + k;
   }
   SCIPsortIntPtr(key, (void**)out, nc);
   SCIPfreeBufferArray(scip, &key);
   SCIPhashmapFree(&rank);
   return SCIP_OKAY;
}

/** a variable's type as SCIP's row orders see it: implied integers between integers and continuous variables */
static int typeRank(SCIP_VAR* v)
{
   return SCIPvarIsImpliedIntegral(v) ? (int)SCIP_DEPRECATED_VARTYPE_IMPLINT : (int)SCIPvarGetType(v);
}

/** whether a comes before b in the order SCIP gives a row's variables before solving (consdataCompVar,
 *  cons_linear.c:3152-3187): binaries first, then by type, ties by the variables' unique index */
static SCIP_Bool indexBefore(SCIP_VAR* a, SCIP_VAR* b)
{
   if( SCIPvarIsBinary(a) != SCIPvarIsBinary(b) )
      return SCIPvarIsBinary(a);
   if( !SCIPvarIsBinary(a) && typeRank(a) != typeRank(b) )
      return typeRank(a) < typeRank(b);
   return SCIPvarCompare(a, b) < 0;
}

/** whether (a, va) comes before (b, vb) in the order tightenBounds sorts a row into (consdataCompVarProp,
 *  cons_linear.c:3191-3254): binaries first by decreasing |coefficient|, then by type, integers by decreasing
 *  |coefficient| * (global domain width), ties by problem index */
static SCIP_Bool propBefore(SCIP_VAR* a, SCIP_Real va, SCIP_VAR* b, SCIP_Real vb)
{
   SCIP_Real ka;
   SCIP_Real kb;
   if( SCIPvarIsBinary(a) != SCIPvarIsBinary(b) )
      return SCIPvarIsBinary(a);
   if( SCIPvarIsBinary(a) )
   {
      ka = REALABS(va);
      kb = REALABS(vb);
   }
   else
   {
      if( typeRank(a) != typeRank(b) )
         return typeRank(a) < typeRank(b);
      if( !SCIPvarIsIntegral(a) )
         return SCIPvarGetProbindex(a) < SCIPvarGetProbindex(b);
      ka = REALABS(va * (SCIPvarGetUbGlobal(a) - SCIPvarGetLbGlobal(a)));
      kb = REALABS(vb * (SCIPvarGetUbGlobal(b) - SCIPvarGetLbGlobal(b)));
   }
   if( EPSGT(ka, kb, 1e-9) )
      return TRUE;
   if( EPSGT(kb, ka, 1e-9) )
      return FALSE;
   return SCIPvarGetProbindex(a) < SCIPvarGetProbindex(b);
}

/** the order SCIP's propagation of a node visits a linear row in.  tightenBounds sorts a row the first time it
 *  visits it during solving (cons_linear.c:7041-7046); until then SCIP holds it in the order of presolving, by
 *  index.  A row whose variables are in that index order is therefore sorted here as tightenBounds will sort it;
 *  a row in any other order has been sorted already and keeps it. */
static SCIP_RETCODE propagationOrder(SCIP* scip, SCIP_VAR** vars, SCIP_Real* vals, int n)
{
   SCIP_VAR** tv;
   SCIP_Real* tc;
   int w;
   int k;
   for( k = 0; k + 1 < n; ++k )
      if( indexBefore(vars[k + 1], vars[k]) )
         return SCIP_OKAY;
   SCIP_CALL( SCIPallocBufferArray(scip, &tv, MAX(n, 1)) );
   SCIP_CALL( SCIPallocBufferArray(scip, &tc, MAX(n, 1)) );
   for( w = 1; w < n; w *= 2 )  /* bottom-up merge sort */
   {
      for( k = 0; k < n; k += 2 * w )
      {
         int m = MIN(k + w, n);
         int e = MIN(k + 2 * w, n);
         int x = k;
         int y = m;
         int t = k;
         while( t < e )
         {
            if( y >= e || (x < m && !propBefore(vars[y], vals[y], vars[x], vals[x])) )
            {
               tv[t] = vars[x];
               tc[t++] = vals[x++];
            }
            else
            {
               tv[t] = vars[y];
               tc[t++] = vals[y++];
            }
         }
      }
      memcpy(vars, tv, sizeof(SCIP_VAR*) * (size_t)n);
      memcpy(vals, tc, sizeof(SCIP_Real) * (size_t)n);
   }
   SCIPfreeBufferArray(scip, &tc);
   SCIPfreeBufferArray(scip, &tv);
   return SCIP_OKAY;
}

/** copies the rows of the handlers into CSR form over the active variables (columns = SCIPvarGetProbindex): fixed,
 *  aggregated, multi-aggregated and negated variables are replaced by their active variables
 *  (SCIPgetProbvarLinearSum), constants move into the sides; modifiable constraints are left to their handler */
static SCIP_RETCODE buildMatrix(SCIP* scip, SCIP_PROPDATA* pd)
{
   int nvars = SCIPgetNVars(scip);
   SCIP_VAR** vars = SCIPgetVars(scip);
   int64_t nnz = 0;
   int64_t cap;
   int ntotal = 0;
   int bufsize = 16;
   SCIP_VAR** bv;
   SCIP_Real* bc;
   int64_t* where;   /* position of a column's entry in the row being built (< the row's start: none) */
   SCIP_Bool sortvars = TRUE;
   int h;
   int j;

   if( SCIPgetBoolParam(scip, "constraints/linear/sortvars", &sortvars) != SCIP_OKAY )
      sortvars = TRUE;
   freeMatrix(scip, pd);
   pd->ncols = nvars;
   pd->nconss = countConss(scip, pd);

   SCIP_CALL( SCIPduplicateMemoryArray(scip, &pd->vars, vars, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->isint, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->lb, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->ub, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->snaplb, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->snapub, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->chglb, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->chgub, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->outcols, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->outlb, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->outub, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->glb, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->gub, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->seeds, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->seedlo, nvars > 0 ? nvars : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->seedhi, nvars > 0 ? nvars : 1) );
   for( j = 0; j < nvars; ++j )
      pd->isint[j] = SCIPvarIsIntegral(vars[j]) ? 1 : 0;

   /* sizes: constraints and their entries before mapping to active variables */
   for( h = 0; h < numHandlers(pd); ++h )
   {
      SCIP_CONSHDLR* hdlr = SCIPfindConshdlr(scip, HDLRS[h]);
      SCIP_CONS** conss = hdlr == NULL ? NULL : SCIPconshdlrGetConss(hdlr);
      int nc = hdlr == NULL ? 0 : SCIPconshdlrGetNConss(hdlr);
      int c;
      ntotal += nc;
      for( c = 0; c < nc; ++c )
      {
         int n = 0;
         SCIP_Real l;
         SCIP_Real r;
         SCIP_CALL( consRow(scip, h, conss[c], NULL, NULL, 0, &n, &l, &r) );
         nnz += n;
      }
   }
   cap = nnz > 0 ? nnz : 1;
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rowptr, ntotal + 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->lhs, ntotal > 0 ? ntotal : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rhs, ntotal > 0 ? ntotal : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->vals, cap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->colidx, cap) );
   SCIP_CALL( SCIPallocBufferArray(scip, &bv, bufsize) );
   SCIP_CALL( SCIPallocBufferArray(scip, &bc, bufsize) );
   SCIP_CALL( SCIPallocBufferArray(scip, &where, nvars > 0 ? nvars : 1) );
   for( j = 0; j < nvars; ++j )
      where[j] = -1;

   pd->rowptr[0] = 0;
   pd->nrows = 0;
   pd->nspecialrows = 0;
   for( h = 0; h < numHandlers(pd); ++h )
   {
      SCIP_CONSHDLR* hdlr = SCIPfindConshdlr(scip, HDLRS[h]);
      SCIP_CONS** conss = hdlr == NULL ? NULL : SCIPconshdlrGetConss(hdlr);
      SCIP_CONS** ordered = NULL;
      int nc = hdlr == NULL ? 0 : SCIPconshdlrGetNConss(hdlr);
      int c;
      if( pd->sciporder && nc > 0 )
      {
         /* SCIP's order marks a variable's rows in the order its bound-change events reach them */
         SCIP_CALL( SCIPallocBufferArray(scip, &ordered, nc) );
         SCIP_CALL( creationOrder(scip, conss, nc, ordered) );
         conss = ordered;
      }
      for( c = 0; c < nc; ++c )
      {
         SCIP_CONS* cons = conss[c];
         SCIP_Real l;
         SCIP_Real r;
         SCIP_Real constant = 0.0;
         int n = 0;
         int need = 0;
         int q;
         int64_t start = pd->rowptr[pd->nrows];
         int64_t p = start;
         if( !readsCons(cons) )
            continue;
         SCIP_CALL( consRow(scip, h, cons, bv, bc, bufsize, &n, &l, &r) );
         if( n > bufsize )
         {
            bufsize = 2 * n;
            SCIP_CALL( SCIPreallocBufferArray(scip, &bv, bufsize) );
            SCIP_CALL( SCIPreallocBufferArray(scip, &bc, bufsize) );
            SCIP_CALL( consRow(scip, h, cons, bv, bc, bufsize, &n, &l, &r) );
         }
         if( pd->sciporder && h == 0 && sortvars )
            SCIP_CALL( propagationOrder(scip, bv, bc, n) );
         SCIP_CALL( SCIPgetProbvarLinearSum(scip, bv, bc, &n, bufsize, &constant, &need) );
         if( need > bufsize )
         {
            bufsize = 2 * need;
            SCIP_CALL( SCIPreallocBufferArray(scip, &bv, bufsize) );
            SCIP_CALL( SCIPreallocBufferArray(scip, &bc, bufsize) );
            SCIP_CALL( consRow(scip, h, cons, bv, bc, bufsize, &n, &l, &r) );
            constant = 0.0;
            SCIP_CALL( SCIPgetProbvarLinearSum(scip, bv, bc, &n, bufsize, &constant, &need) );
         }
         if( p + n > cap )
         {
            cap = 2 * (p + n);
            SCIP_CALL( SCIPreallocMemoryArray(scip, &pd->vals, cap) );
            SCIP_CALL( SCIPreallocMemoryArray(scip, &pd->colidx, cap) );
         }
         /* one entry per column: a variable that several entries map to gets their sum */
         for( q = 0; q < n; ++q )
         {
            const int32_t col = (int32_t)SCIPvarGetProbindex(bv[q]);
            if( bc[q] == 0.0 || col < 0 )
               continue;
            if( where[col] >= start )
               pd->vals[where[col]] += bc[q];
            else
            {
               where[col] = p;
               pd->colidx[p] = col;
               pd->vals[p] = bc[q];
               ++p;
            }
         }
         {
            /* drop entries that cancelled */
            int64_t w = start;
            int64_t t;
            for( t = start; t < p; ++t )
            {
               if( pd->vals[t] != 0.0 )
               {
                  pd->colidx[w] = pd->colidx[t];
                  pd->vals[w] = pd->vals[t];
                  ++w;
               }
            }
            p = w;
         }
         if( p == start )
            continue;
         if( !SCIPisInfinity(scip, -l) )
            l -= constant;
         if( !SCIPisInfinity(scip, r) )
            r -= constant;
         pd->lhs[pd->nrows] = SCIPisInfinity(scip, -l) ? -SCIPinfinity(scip) : l;
         pd->rhs[pd->nrows] = SCIPisInfinity(scip, r) ? SCIPinfinity(scip) : r;
         pd->nrows++;
         pd->nspecialrows += h > 0 ? 1 : 0;
         pd->rowptr[pd->nrows] = p;
      }
      if( ordered != NULL )
         SCIPfreeBufferArray(scip, &ordered);
   }
   SCIPfreeBufferArray(scip, &where);
   SCIPfreeBufferArray(scip, &bc);
   SCIPfreeBufferArray(scip, &bv);
   /* the column view for resolving conflicts, and room for the change log (columns times a few rounds) */
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->colptr, nvars + 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rowidx, pd->rowptr[pd->nrows] > 0 ? pd->rowptr[pd->nrows] : 1) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rowpos, pd->rowptr[pd->nrows] > 0 ? pd->rowptr[pd->nrows] : 1) );
   gpl_build_columns(pd->nrows, nvars, pd->rowptr, pd->colidx, pd->colptr, pd->rowidx, pd->rowpos);
   pd->logcap = 4 * (int64_t)nvars + 4096;
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->logcol, pd->logcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->loground, pd->logcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->loglb, pd->logcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->logub, pd->logcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->tround, pd->logcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->tcol, pd->logcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->trow, pd->logcap) );
   pd->rcap = 4 * pd->logcap;
   pd->rn = 0;
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rcall, pd->rcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rround, pd->rcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rcol, pd->rcap) );
   SCIP_CALL( SCIPallocMemoryArray(scip, &pd->rrow, pd->rcap) );
   return SCIP_OKAY;
}

static void disable(SCIP* scip, SCIP_PROPDATA* pd, const char* why, int rc)
{
   SCIPwarningMessage(scip, "propagator <%s> disabled: %s (%s%s%s); cons_linear keeps propagating\n", PROP_NAME, why,
      gbp_error_string(rc), pd->ctx != NULL ? ": " : "", pd->ctx != NULL ? gbp_last_error(pd->ctx) : "");
   pd->failed = TRUE;
}

/** numerics of the running SCIP (set.c / def.h) for the device rules, plus the mode flags in extraflags */
static SCIP_RETCODE setDeviceParamsWith(SCIP* scip, SCIP_PROPDATA* pd, int32_t extraflags)
{
   gbp_params p;
   SCIP_Real v;
   gbp_default_params(&p);
   p.flags |= extraflags;
   p.infinity = SCIPinfinity(scip);
   p.epsilon = SCIPepsilon(scip);
   p.sumepsilon = SCIPsumepsilon(scip);
   p.feastol = SCIPfeastol(scip);
   p.hugeval = SCIPgetHugeValue(scip);
   SCIP_CALL( SCIPgetRealParam(scip, "numerics/boundstreps", &v) );
   p.boundstreps = v;
   SCIP_CALL( SCIPgetRealParam(scip, "numerics/recomputefac", &v) );
   p.recompfac = v;
   if( SCIPgetRealParam(scip, "constraints/linear/maxeasyactivitydelta", &v) == SCIP_OKAY )
      p.maxeasyactivitydelta = v;
   {
      SCIP_Bool sortvars = TRUE;
      if( SCIPgetBoolParam(scip, "constraints/linear/sortvars", &sortvars) == SCIP_OKAY && !sortvars )
         p.flags |= GBP_FLAG_NOSORTVARS;
   }
   if( pd->ranged )
      p.flags |= GBP_FLAG_RANGEDROW;
   if( gbp_set_params(pd->ctx, &p) != GBP_OK )
      return SCIP_INVALIDDATA;
   return SCIP_OKAY;
}

static SCIP_RETCODE setDeviceParams(SCIP* scip, SCIP_PROPDATA* pd)
{
   return setDeviceParamsWith(scip, pd, 0);
}

/** whether cons_linear would run ranged-row propagation now (consPropLinear, cons_linear.c:16159-16170): its
 *  parameter, the depth limit and frequency, not in repropagation -- and not in probing, where SCIP keeps the
 *  rows' rangedrowpropagated marks (cons_linear.c:17222-17224) so that rows already ranged-propagated are not
 *  visited again */
static SCIP_Bool wantRanged(SCIP* scip)
{
   SCIP_Bool on = TRUE;
   int maxdepth = INT_MAX;
   int freq = 1;
   int depth = SCIPgetDepth(scip);
   if( SCIPgetBoolParam(scip, "constraints/linear/rangedrowpropagation", &on) != SCIP_OKAY )
      on = FALSE;
   (void)SCIPgetIntParam(scip, "constraints/linear/rangedrowmaxdepth", &maxdepth);
   (void)SCIPgetIntParam(scip, "constraints/linear/rangedrowfreq", &freq);
   if( !on || SCIPinProbing(scip) || SCIPinRepropagation(scip) || depth > maxdepth || freq < 0 )
      return FALSE;
   return (freq == 0 && depth == 0) || (freq >= 1 && depth % freq == 0);
}

/* inference information of a logged change: the call (its low 20 bits) and the device round (rounds from 2047 on
 * share the last value, which no ranged-row record matches) */
#define INFO_ROUNDBITS 11
#define INFO_CALLMASK 0xfffff
static int encodeInfo(SCIP_Longint call, int32_t round)
{
   const int32_t r = round < (1 << INFO_ROUNDBITS) - 1 ? round : (1 << INFO_ROUNDBITS) - 1;
   return (int)(((call & INFO_CALLMASK) << INFO_ROUNDBITS) | r);
}

/** keeps the last call's ranged-row records (call id pd->ncalls) behind those of earlier calls */
static void storeRanged(SCIP_PROPDATA* pd)
{
   int64_t nr = 0;
   int64_t k;
   if( !pd->ranged || gbp_get_ranged_log(pd->ctx, pd->logcap, pd->tround, pd->tcol, pd->trow, &nr) != GBP_OK )
      return;
   if( nr > pd->rcap )
      return;
   /* the oldest records go when the room is used up, or before their call numbers could alias in the inference
    * information; their changes are then not explained */
   if( pd->rn + nr > pd->rcap || (pd->rn > 0 && pd->ncalls - pd->rcall[0] > INFO_CALLMASK / 2) )
      pd->rn = 0;
   for( k = 0; k < nr; ++k )
   {
      pd->rcall[pd->rn] = pd->ncalls;
      pd->rround[pd->rn] = pd->tround[k];
      pd->rcol[pd->rn] = pd->tcol[k];
      pd->rrow[pd->rn] = pd->trow[k];
      pd->rn++;
   }
}

/** the row of a ranged-row record (call, round, col), or -1: binary search over the sorted records */
static int64_t findRanged(SCIP_PROPDATA* pd, SCIP_Longint call, int32_t round, int32_t col)
{
   int64_t lo = 0;
   int64_t hi = pd->rn;
   while( lo < hi )
   {
      int64_t mid = (lo + hi) / 2;
      SCIP_Bool before = pd->rcall[mid] < call || (pd->rcall[mid] == call && (pd->rround[mid] < round
         || (pd->rround[mid] == round && pd->rcol[mid] < col)));
      if( before )
         lo = mid + 1;
      else
         hi = mid;
   }
   if( lo < pd->rn && pd->rcall[lo] == call && pd->rround[lo] == round && pd->rcol[lo] == col )
      return pd->rrow[lo];
   return -1;
}

static SCIP_RETCODE upload(SCIP* scip, SCIP_PROPDATA* pd)
{
   int rc;
   SCIP_CALL( buildMatrix(scip, pd) );
   pd->ranged = FALSE;   /* switched on by the first call that wants it */
   SCIP_CALL( setDeviceParams(scip, pd) );
   rc = gbp_upload_problem(pd->ctx, pd->nrows, pd->ncols, pd->rowptr, pd->colidx, pd->vals, pd->lhs, pd->rhs, pd->isint);
   if( rc == GBP_OK )
      rc = gbp_set_change_log(pd->ctx, pd->logcap);
   if( rc != GBP_OK )
      disable(scip, pd, "uploading the rows failed", rc);
   pd->havesnap = FALSE;
   return SCIP_OKAY;
}

/** replacelinear = TRUE switches cons_linear's propagation off (constraints/linear/propfreq, cons.c:2247) */
static SCIP_DECL_PARAMCHGD(paramChgdReplacelinear)
{
   if( SCIPparamGetBool(param) )
   {
      SCIP_CALL( SCIPsetIntParam(scip, "constraints/linear/propfreq", -1) );
   }
   return SCIP_OKAY;
}

/** replacespecialised = TRUE switches the propagation of setppc, logicor, knapsack and varbound off (their rows are
 *  then propagated here, with `specialised` on) */
static SCIP_DECL_PARAMCHGD(paramChgdReplacespecialised)
{
   if( SCIPparamGetBool(param) )
   {
      int h;
      for( h = 1; h < NHDLRS; ++h )
      {
         char name[SCIP_MAXSTRLEN];
         (void)SCIPsnprintf(name, SCIP_MAXSTRLEN, "constraints/%s/propfreq", HDLRS[h]);
         SCIP_CALL( SCIPsetIntParam(scip, name, -1) );
      }
   }
   return SCIP_OKAY;
}

/** copies the propagator into sub-SCIPs (heuristics' sub-MIPs, concurrent solvers): they copy the parameters,
 *  including constraints/linear/propfreq = -1 when replacelinear is set, so they need the propagator as well; each
 *  copy opens its own context on the device */
static SCIP_DECL_PROPCOPY(propCopyGpulinear)
{
   SCIP_CALL( SCIPincludePropGpulinear(scip) );
   return SCIP_OKAY;
}

static SCIP_DECL_PROPFREE(propFreeGpulinear)
{
   SCIP_PROPDATA* pd = SCIPpropGetData(prop);
   freeMatrix(scip, pd);
   if( pd->ctx != NULL )
      (void)gbp_destroy(pd->ctx);
   SCIPfreeMemory(scip, &pd);
   SCIPpropSetData(prop, NULL);
   return SCIP_OKAY;
}

static SCIP_DECL_PROPINITSOL(propInitsolGpulinear)
{
   SCIP_PROPDATA* pd = SCIPpropGetData(prop);
   int rc;
   pd->failed = FALSE;
   if( pd->ctx == NULL )
   {
      rc = gbp_create(&pd->ctx, pd->device, NULL);
      if( rc != GBP_OK )
      {
         pd->ctx = NULL;
         disable(scip, pd, "no usable GB300 device", rc);
         SCIP_CALL( buildMatrix(scip, pd) );
         return SCIP_OKAY;
      }
   }
   SCIP_CALL( upload(scip, pd) );
   return SCIP_OKAY;
}

static SCIP_DECL_PROPEXITSOL(propExitsolGpulinear)
{
   SCIP_PROPDATA* pd = SCIPpropGetData(prop);
   freeMatrix(scip, pd);
   return SCIP_OKAY;
}

/* SCIP's bound history behind the reason module's callbacks */
typedef struct
{
   SCIP* scip;
   SCIP_VAR** vars;
   SCIP_BDCHGIDX* bdchgidx;
} ReasonCtx;

/** the last call's change log as inferences of this propagator, round by round */
static SCIP_RETCODE applyLog(SCIP* scip, SCIP_PROP* prop, SCIP_PROPDATA* pd, SCIP_Bool* reduced, SCIP_Bool* infeasible)
{
   int64_t nlog = 0;
   int64_t k;
   *infeasible = FALSE;
   if( gbp_get_change_log(pd->ctx, pd->logcap, pd->logcol, pd->loground, pd->loglb, pd->logub, &nlog) != GBP_OK )
      return SCIP_OKAY;
   for( k = 0; k < nlog && !*infeasible; ++k )
   {
      SCIP_VAR* var = pd->vars[pd->logcol[k]];
      SCIP_Bool tightened = FALSE;
      if( pd->logub[k] < SCIPvarGetUbLocal(var) )
      {
         SCIP_CALL( SCIPinferVarUbProp(scip, var, pd->logub[k], prop, encodeInfo(pd->ncalls, pd->loground[k]), TRUE,
               infeasible, &tightened) );
         *reduced = *reduced || tightened;
         pd->nchgbds += tightened ? 1 : 0;
      }
      if( !*infeasible && pd->loglb[k] > SCIPvarGetLbLocal(var) )
      {
         SCIP_CALL( SCIPinferVarLbProp(scip, var, pd->loglb[k], prop, encodeInfo(pd->ncalls, pd->loground[k]), TRUE,
               infeasible, &tightened) );
         *reduced = *reduced || tightened;
         pd->nchgbds += tightened ? 1 : 0;
      }
   }
   return SCIP_OKAY;
}

/* forward declarations of the reason callbacks (below) */
static double rLb(void* ud, int32_t k);
static double rUb(void* ud, int32_t k);
static double rGlb(void* ud, int32_t k);
static double rGub(void* ud, int32_t k);
static double rLbAfter(void* ud, int32_t k);
static double rUbAfter(void* ud, int32_t k);
static int rAddLb(void* ud, int32_t k);
static int rAddUb(void* ud, int32_t k);
static void reasonSetup(SCIP* scip, SCIP_PROPDATA* pd, SCIP_BDCHGIDX* bdchgidx, void* ctx, gpl_rows* R, gpl_num* num,
   gpl_io* io);

/** conflict analysis of a cutoff the device found: cons_linear analyses the row that became infeasible
 *  (analyzeConflict, cons_linear.c:5190); with the logged changes applied, such a row holds under the local bounds */
static SCIP_RETCODE analyzeCutoff(SCIP* scip, SCIP_PROPDATA* pd)
{
   ReasonCtx c;
   gpl_rows R;
   gpl_num num;
   gpl_io io;
   int64_t r;
   if( !SCIPisConflictAnalysisApplicable(scip) )
      return SCIP_OKAY;
   SCIP_CALL( SCIPinitConflictAnalysis(scip, SCIP_CONFTYPE_PROPAGATION, FALSE) );
   reasonSetup(scip, pd, NULL, &c, &R, &num, &io);
   r = gpl_explain_infeasible(&R, &num, &io);
   if( r == -1 )
   {
      /* no row's activities show it: a ranged row of the last call did (its records with column -1) */
      int64_t k;
      for( k = pd->rn - 1; k >= 0 && pd->rcall[k] == pd->ncalls && r == -1; --k )
         if( pd->rcol[k] == -1 )
         {
            r = gpl_explain_ranged(&R, &num, &io, pd->rrow[k], -1) == 0 ? pd->rrow[k] : -2;
            pd->nrangedreasons++;
         }
   }
   if( r == -2 )
      return SCIP_ERROR;
   if( r >= 0 )
   {
      SCIP_CALL( SCIPanalyzeConflict(scip, 0, NULL) );
      pd->nconflicts++;
   }
   return SCIP_OKAY;
}

static SCIP_DECL_PROPEXEC(propExecGpulinear)
{
   SCIP_PROPDATA* pd = SCIPpropGetData(prop);
   int64_t nseed = -1;
   int32_t cutoff = 0;
   gbp_result res;
   int rc;
   int j;
   SCIP_Bool reduced = FALSE;

   *result = SCIP_DIDNOTRUN;
   if( pd->failed || pd->ctx == NULL || (!pd->inprobing && SCIPinProbing(scip)) )
      return SCIP_OKAY;

   /* constraints added or removed since the upload: rebuild */
   if( countConss(scip, pd) != pd->nconss || SCIPgetNVars(scip) != pd->ncols )
   {
      SCIP_CALL( upload(scip, pd) );
      if( pd->failed )
         return SCIP_OKAY;
   }

   for( j = 0; j < pd->ncols; ++j )
   {
      pd->lb[j] = SCIPvarGetLbLocal(pd->vars[j]);
      pd->ub[j] = SCIPvarGetUbLocal(pd->vars[j]);
   }
   /* the binary test of the device reads the global domain (SCIPvarIsBinary); at the root the local bounds are
    * the global ones, below it the global bounds go to the device whenever they changed */
   if( SCIPgetDepth(scip) > 0 )
   {
      SCIP_Bool changed = !pd->haveglobal;
      for( j = 0; j < pd->ncols; ++j )
      {
         double gl = SCIPvarGetLbGlobal(pd->vars[j]);
         double gu = SCIPvarGetUbGlobal(pd->vars[j]);
         if( changed || gl != pd->glb[j] || gu != pd->gub[j] )
         {
            changed = TRUE;
            pd->glb[j] = gl;
            pd->gub[j] = gu;
         }
      }
      if( changed )
      {
         rc = gbp_set_global_bounds(pd->ctx, pd->glb, pd->gub);
         if( rc != GBP_OK )
         {
            disable(scip, pd, "passing the global bounds failed", rc);
            return SCIP_OKAY;
         }
         pd->haveglobal = TRUE;
      }
   }
   else if( pd->haveglobal )
   {
      rc = gbp_set_global_bounds(pd->ctx, NULL, NULL);
      if( rc != GBP_OK )
      {
         disable(scip, pd, "clearing the global bounds failed", rc);
         return SCIP_OKAY;
      }
      pd->haveglobal = FALSE;
   }
   if( pd->havesnap )
   {
      /* columns whose local bounds differ from the device's copy: only they are sent, and their rows are
       * re-propagated in both directions (a relaxed column can be re-tightened by its own rows after SCIP switched
       * to another node) */
      nseed = 0;
      for( j = 0; j < pd->ncols; ++j )
      {
         if( pd->lb[j] != pd->snaplb[j] || pd->ub[j] != pd->snapub[j] )
         {
            pd->seeds[nseed] = j;
            pd->chglb[nseed] = pd->lb[j];
            pd->chgub[nseed] = pd->ub[j];
            pd->seedlo[nseed] = -DBL_MAX;
            pd->seedhi[nseed] = DBL_MAX;
            ++nseed;
         }
      }
      if( nseed == 0 )
      {
         *result = SCIP_DIDNOTFIND;
         return SCIP_OKAY;
      }
   }

   /* ranged-row propagation where cons_linear would run it (switching it rebuilds the device's loop) */
   if( wantRanged(scip) != pd->ranged )
   {
      pd->ranged = !pd->ranged;
      if( setDeviceParams(scip, pd) != SCIP_OKAY )
      {
         disable(scip, pd, "setting the ranged-row rule failed", GBP_ERR_INVALID);
         return SCIP_OKAY;
      }
   }
   if( pd->havesnap )
   {
      /* the device keeps the bounds between calls: the changed columns go in, the moved ones come back */
      int64_t nout = 0;
      int64_t q;
      rc = gbp_propagate_changes(pd->ctx, nseed, pd->seeds, pd->chglb, pd->chgub, pd->seedlo, pd->seedhi,
         (int64_t)pd->ncols, &nout, pd->outcols, pd->outlb, pd->outub, &cutoff, &res);
      if( (rc == GBP_OK || rc == GBP_ERR_LIMIT) && !cutoff )
      {
         for( q = 0; q < nout; ++q )
         {
            pd->lb[pd->outcols[q]] = pd->outlb[q];
            pd->ub[pd->outcols[q]] = pd->outub[q];
         }
      }
   }
   else
   {
      /* every row from the current bounds, which then stay on the device */
      rc = gbp_propagate(pd->ctx, pd->lb, pd->ub, -1, NULL, NULL, NULL, &cutoff, &res);
      if( (rc == GBP_OK || rc == GBP_ERR_LIMIT) && !cutoff )
      {
         int rc2 = gbp_set_bounds(pd->ctx, pd->lb, pd->ub);
         if( rc2 != GBP_OK )
            rc = rc2;
      }
   }
   pd->ncalls++;
   if( rc != GBP_OK && rc != GBP_ERR_LIMIT )
   {
      disable(scip, pd, "propagation call failed", rc);
      return SCIP_OKAY;
   }
   storeRanged(pd);
   if( cutoff )
   {
      /* the changes the rounds before the infeasibility made, then conflict analysis on the infeasible row */
      SCIP_Bool infeasible = FALSE;
      pd->ncutoffs++;
      pd->havesnap = FALSE;
      SCIP_CALL( applyLog(scip, prop, pd, &reduced, &infeasible) );
      if( !infeasible )
         SCIP_CALL( analyzeCutoff(scip, pd) );
      *result = SCIP_CUTOFF;
      return SCIP_OKAY;
   }

   /* The device applied cons_linear's acceptance rules already: force the moves through.  The change log hands
    * them over round by round as inferences of this propagator, so each one's reasons already hold when conflict
    * analysis asks for them (propRespropGpulinear).  The final loop below then finds nothing left to do, or, when
    * the log overflowed, moves the final bounds in without reasons. */
   {
      SCIP_Bool infeasible = FALSE;
      SCIP_CALL( applyLog(scip, prop, pd, &reduced, &infeasible) );
      if( infeasible )
      {
         pd->havesnap = FALSE;
         *result = SCIP_CUTOFF;
         return SCIP_OKAY;
      }
   }
   for( j = 0; j < pd->ncols; ++j )
   {
      SCIP_VAR* var = pd->vars[j];
      SCIP_Bool infeasible = FALSE;
      SCIP_Bool tightened = FALSE;
      if( pd->lb[j] > SCIPvarGetLbLocal(var) )
      {
         SCIP_CALL( SCIPtightenVarLb(scip, var, pd->lb[j], TRUE, &infeasible, &tightened) );
         if( infeasible )
         {
            pd->havesnap = FALSE;
            *result = SCIP_CUTOFF;
            return SCIP_OKAY;
         }
         reduced = reduced || tightened;
         pd->nchgbds += tightened ? 1 : 0;
      }
      if( pd->ub[j] < SCIPvarGetUbLocal(var) )
      {
         SCIP_CALL( SCIPtightenVarUb(scip, var, pd->ub[j], TRUE, &infeasible, &tightened) );
         if( infeasible )
         {
            pd->havesnap = FALSE;
            *result = SCIP_CUTOFF;
            return SCIP_OKAY;
         }
         reduced = reduced || tightened;
         pd->nchgbds += tightened ? 1 : 0;
      }
   }
   /* the device's copy: a column whose local bound SCIP did not take as proposed differs from it and is sent
    * again at the next call */
   for( j = 0; j < pd->ncols; ++j )
   {
      pd->snaplb[j] = pd->lb[j];
      pd->snapub[j] = pd->ub[j];
   }
   pd->havesnap = TRUE;
   *result = reduced ? SCIP_REDUCEDDOM : SCIP_DIDNOTFIND;
   return SCIP_OKAY;
}


static double rLb(void* ud, int32_t k)
{
   ReasonCtx* c = (ReasonCtx*)ud;
   return SCIPgetVarLbAtIndex(c->scip, c->vars[k], c->bdchgidx, FALSE);
}
static double rUb(void* ud, int32_t k)
{
   ReasonCtx* c = (ReasonCtx*)ud;
   return SCIPgetVarUbAtIndex(c->scip, c->vars[k], c->bdchgidx, FALSE);
}
static double rGlb(void* ud, int32_t k) { return SCIPvarGetLbGlobal(((ReasonCtx*)ud)->vars[k]); }
static double rGub(void* ud, int32_t k) { return SCIPvarGetUbGlobal(((ReasonCtx*)ud)->vars[k]); }
static double rLbAfter(void* ud, int32_t k)
{
   ReasonCtx* c = (ReasonCtx*)ud;
   return SCIPgetVarLbAtIndex(c->scip, c->vars[k], c->bdchgidx, TRUE);
}
static double rUbAfter(void* ud, int32_t k)
{
   ReasonCtx* c = (ReasonCtx*)ud;
   return SCIPgetVarUbAtIndex(c->scip, c->vars[k], c->bdchgidx, TRUE);
}
static int rAddLb(void* ud, int32_t k)
{
   ReasonCtx* c = (ReasonCtx*)ud;
   return SCIPaddConflictLb(c->scip, c->vars[k], c->bdchgidx) == SCIP_OKAY ? 0 : 1;
}
static int rAddUb(void* ud, int32_t k)
{
   ReasonCtx* c = (ReasonCtx*)ud;
   return SCIPaddConflictUb(c->scip, c->vars[k], c->bdchgidx) == SCIP_OKAY ? 0 : 1;
}

/* the rows, numerics and SCIP's bound history (at bdchgidx; NULL: now) for the reason module */
static void reasonSetup(SCIP* scip, SCIP_PROPDATA* pd, SCIP_BDCHGIDX* bdchgidx, void* ctx, gpl_rows* R, gpl_num* num,
   gpl_io* io)
{
   ReasonCtx* c = (ReasonCtx*)ctx;
   c->scip = scip;
   c->vars = pd->vars;
   c->bdchgidx = bdchgidx;
   R->m = pd->nrows;
   R->n = pd->ncols;
   R->rowptr = pd->rowptr;
   R->colidx = pd->colidx;
   R->vals = pd->vals;
   R->lhs = pd->lhs;
   R->rhs = pd->rhs;
   R->isint = pd->isint;
   R->colptr = pd->colptr;
   R->rowidx = pd->rowidx;
   R->rowpos = pd->rowpos;
   num->infinity = SCIPinfinity(scip);
   num->feastol = SCIPfeastol(scip);
   num->epsilon = SCIPepsilon(scip);
   io->ud = c;
   io->lb = rLb;
   io->ub = rUb;
   io->glb = rGlb;
   io->gub = rGub;
   io->lbafter = rLbAfter;
   io->ubafter = rUbAfter;
   io->addlb = rAddLb;
   io->addub = rAddUb;
}

/** reason of one of this propagator's bound changes (type_prop.h:258): the bounds of a row that implies it, chosen
 *  as cons_linear's resolvePropagation / addConflictBounds would for that row (cons_linear.c:5097, :4799) */
static SCIP_DECL_PROPRESPROP(propRespropGpulinear)
{
   SCIP_PROPDATA* pd = SCIPpropGetData(prop);
   int32_t col = (int32_t)SCIPvarGetProbindex(infervar);
   ReasonCtx c;
   gpl_rows R;
   gpl_num num;
   gpl_io io;
   int64_t r;

   *result = SCIP_DIDNOTFIND;
   pd->nresolves++;
   if( pd->colptr == NULL || col < 0 || col >= pd->ncols || pd->vars[col] != infervar )
      return SCIP_OKAY;
   reasonSetup(scip, pd, bdchgidx, &c, &R, &num, &io);
   r = gpl_explain(&R, &num, &io, col, boundtype == SCIP_BOUNDTYPE_LOWER, relaxedbd);
   if( r == -1 )
   {
      /* no row's activities imply it: the ranged row that proposed it in that call and round, if still on record */
      const SCIP_Longint lo = ((SCIP_Longint)inferinfo >> INFO_ROUNDBITS) & INFO_CALLMASK;
      const SCIP_Longint call = pd->ncalls - ((pd->ncalls - lo) & INFO_CALLMASK);
      const int32_t round = inferinfo & ((1 << INFO_ROUNDBITS) - 1);
      const int64_t row = round < (1 << INFO_ROUNDBITS) - 1 ? findRanged(pd, call, round, col) : -1;
      if( row >= 0 )
      {
         r = gpl_explain_ranged(&R, &num, &io, row, col) == 0 ? row : -2;
         pd->nrangedreasons++;
      }
   }
   if( r == -2 )
      return SCIP_ERROR;
   if( r >= 0 )
   {
      *result = SCIP_SUCCESS;
      pd->nresolved++;
   }
   return SCIP_OKAY;
}

SCIP_RETCODE SCIPincludePropGpulinear(SCIP* scip)
{
   SCIP_PROPDATA* pd;
   SCIP_PROP* prop = NULL;

   SCIP_CALL( SCIPallocMemory(scip, &pd) );
   memset(pd, 0, sizeof(*pd));
   SCIP_CALL( SCIPincludePropBasic(scip, &prop, PROP_NAME, PROP_DESC, PROP_PRIORITY, PROP_FREQ, PROP_DELAY,
         PROP_TIMING, propExecGpulinear, pd) );
   SCIP_CALL( SCIPsetPropCopy(scip, prop, propCopyGpulinear) );
   SCIP_CALL( SCIPsetPropFree(scip, prop, propFreeGpulinear) );
   SCIP_CALL( SCIPsetPropInitsol(scip, prop, propInitsolGpulinear) );
   SCIP_CALL( SCIPsetPropExitsol(scip, prop, propExitsolGpulinear) );
   SCIP_CALL( SCIPsetPropResprop(scip, prop, propRespropGpulinear) );
   SCIP_CALL( SCIPaddIntParam(scip, "propagating/" PROP_NAME "/device", "CUDA device ordinal of the GPU",
         &pd->device, FALSE, 0, 0, 1024, NULL, NULL) );
   SCIP_CALL( SCIPaddBoolParam(scip, "propagating/" PROP_NAME "/replacelinear",
         "switch off cons_linear's own propagation (constraints/linear/propfreq = -1) when included",
         &pd->replacelinear, FALSE, FALSE, paramChgdReplacelinear, NULL) );
   SCIP_CALL( SCIPaddBoolParam(scip, "propagating/" PROP_NAME "/specialised",
         "also propagate the rows of setppc, logicor, knapsack and varbound constraints (presolving upgrades linear "
         "rows to these handlers)", &pd->specialised, FALSE, TRUE, NULL, NULL) );
   SCIP_CALL( SCIPaddBoolParam(scip, "propagating/" PROP_NAME "/probing",
         "also propagate in probing nodes (SCIPpropagateProbing); SCIPpropagateGpulinearNodes serves many probing "
         "candidates at once", &pd->inprobing, FALSE, TRUE, NULL, NULL) );
   SCIP_CALL( SCIPaddBoolParam(scip, "propagating/" PROP_NAME "/sciporder",
         "SCIPpropagateGpulinearNodes propagates its nodes in SCIP's own order (one marked row at a time, every "
         "tightening applied at once) instead of rounds, with the rows re-read in the order SCIP holds them; only "
         "for matrices of linear rows alone", &pd->sciporder, FALSE, FALSE, NULL, NULL) );
   SCIP_CALL( SCIPaddBoolParam(scip, "propagating/" PROP_NAME "/replacespecialised",
         "switch off the propagation of setppc, logicor, knapsack and varbound (constraints/<handler>/propfreq = -1)",
         &pd->replacespecialised, FALSE, FALSE, paramChgdReplacespecialised, NULL) );
   return SCIP_OKAY;
}

SCIP_RETCODE SCIPgetGpulinearMatrix(SCIP* scip, int* nrows, int* ncols, const int64_t** rowptr, const int32_t** colidx,
   const double** vals, const double** lhs, const double** rhs)
{
   SCIP_PROP* prop = SCIPfindProp(scip, PROP_NAME);
   SCIP_PROPDATA* pd;
   if( prop == NULL )
      return SCIP_PLUGINNOTFOUND;
   pd = SCIPpropGetData(prop);
   *nrows = pd->nrows;
   *ncols = pd->ncols;
   *rowptr = pd->rowptr;
   *colidx = pd->colidx;
   *vals = pd->vals;
   *lhs = pd->lhs;
   *rhs = pd->rhs;
   return SCIP_OKAY;
}

SCIP_Bool SCIPgpulinearIsActive(SCIP* scip)
{
   SCIP_PROP* prop = SCIPfindProp(scip, PROP_NAME);
   SCIP_PROPDATA* pd;
   if( prop == NULL )
      return FALSE;
   pd = SCIPpropGetData(prop);
   return pd->ctx != NULL && !pd->failed;
}

SCIP_RETCODE SCIPgetGpulinearStats(SCIP* scip, SCIP_Longint* ncalls, SCIP_Longint* nchgbds, SCIP_Longint* ncutoffs,
   SCIP_Longint* nconflicts, SCIP_Longint* nresolves, SCIP_Longint* nresolved)
{
   SCIP_PROP* prop = SCIPfindProp(scip, PROP_NAME);
   SCIP_PROPDATA* pd;
   if( prop == NULL )
      return SCIP_PLUGINNOTFOUND;
   pd = SCIPpropGetData(prop);
   *ncalls = pd->ncalls;
   *nchgbds = pd->nchgbds;
   *ncutoffs = pd->ncutoffs;
   *nconflicts = pd->nconflicts;
   *nresolves = pd->nresolves;
   *nresolved = pd->nresolved;
   return SCIP_OKAY;
}

SCIP_Longint SCIPgetGpulinearRangedReasons(SCIP* scip)
{
   SCIP_PROP* prop = SCIPfindProp(scip, PROP_NAME);
   return prop == NULL ? 0 : SCIPpropGetData(prop)->nrangedreasons;
}

/* Many nodes at once on top of the current local bounds (the batched path of libgbp, gbp_propagate_nodes): for
 * callers that hold many candidate nodes -- probing, strong branching, a lookahead of open nodes.  Below the root the
 * global bounds go to the device for the binary test, as in PROPEXEC. */
SCIP_RETCODE SCIPpropagateGpulinearNodes(SCIP* scip, int nnodes, const int* nodebeg, SCIP_VAR** vars,
   const SCIP_Real* lbs, const SCIP_Real* ubs, int outcap, SCIP_Bool* cutoff, int* outbeg, SCIP_VAR** outvars,
   SCIP_Real* outlbs, SCIP_Real* outubs, SCIP_Bool* success)
{
   SCIP_PROP* prop = SCIPfindProp(scip, PROP_NAME);
   SCIP_PROPDATA* pd;
   int64_t* ptr = NULL;
   int32_t* col = NULL;
   int8_t* ocut = NULL;
   int32_t* orounds = NULL;
   int64_t* ooff = NULL;
   int32_t* on = NULL;
   int32_t* ocol = NULL;
   double* olb = NULL;
   double* oub = NULL;
   gbp_result res;
   SCIP_Bool wasranged;
   int nchg;
   int rc;
   int j;
   int k;
   int at;

   if( prop == NULL )
      return SCIP_PLUGINNOTFOUND;
   if( nnodes < 0 || nodebeg == NULL || cutoff == NULL || outbeg == NULL || success == NULL || outcap < 0 )
      return SCIP_INVALIDDATA;
   *success = FALSE;
   pd = SCIPpropGetData(prop);
   if( pd->failed || pd->ctx == NULL || nnodes == 0 )
      return SCIP_OKAY;
   if( pd->sciporder )
   {
      /* SCIP's order visits a row's entries in the order SCIP holds them now (consdataSort has sorted the rows it
       * propagated since the matrix was built): read the rows again */
      SCIP_CALL( upload(scip, pd) );
      if( pd->failed )
         return SCIP_OKAY;
      /* ranged-row propagation needs no refusal: a probing node keeps every row's rangedrowpropagated mark
       * (cons_linear.c:17222-17224), and a row propagated at the base after its last change carries it, so SCIP's
       * own probing of these nodes runs no ranged-row rule either */
      if( pd->nspecialrows > 0 )
      {
         SCIPwarningMessage(scip, "propagator <%s>: SCIP's order needs linear rows alone; batched nodes not "
            "propagated\n", PROP_NAME);
         return SCIP_OKAY;
      }
      /* the device takes a row's leading binaries under the base (local) bounds; SCIP's are binary in the global
       * domain (SCIPvarIsBinary).  Below the root they differ for an integer column whose local domain lies in
       * [0,1] and whose global domain does not. */
      for( j = 0; j < pd->ncols && SCIPgetDepth(scip) > 0; ++j )
      {
         SCIP_VAR* v = pd->vars[j];
         if( pd->isint[j] && SCIPvarGetLbLocal(v) >= 0.0 && SCIPvarGetUbLocal(v) <= 1.0
            && (SCIPvarGetLbGlobal(v) < 0.0 || SCIPvarGetUbGlobal(v) > 1.0) )
         {
            SCIPwarningMessage(scip, "propagator <%s>: <%s> is binary in the local domain only; SCIP's order "
               "not available at this node\n", PROP_NAME, SCIPvarGetName(v));
            return SCIP_OKAY;
         }
      }
   }
   nchg = nodebeg[nnodes];
   for( j = 0; j < pd->ncols; ++j )
   {
      pd->lb[j] = SCIPvarGetLbLocal(pd->vars[j]);
      pd->ub[j] = SCIPvarGetUbLocal(pd->vars[j]);
   }
   if( SCIPgetDepth(scip) > 0 )
   {
      for( j = 0; j < pd->ncols; ++j )
      {
         pd->glb[j] = SCIPvarGetLbGlobal(pd->vars[j]);
         pd->gub[j] = SCIPvarGetUbGlobal(pd->vars[j]);
      }
      rc = gbp_set_global_bounds(pd->ctx, pd->glb, pd->gub);
      pd->haveglobal = rc == GBP_OK;
   }
   else
   {
      rc = gbp_set_global_bounds(pd->ctx, NULL, NULL);
      pd->haveglobal = FALSE;
   }
   if( rc != GBP_OK )
      return SCIP_OKAY;
   SCIP_CALL( SCIPallocBufferArray(scip, &ptr, nnodes + 1) );
   SCIP_CALL( SCIPallocBufferArray(scip, &col, MAX(nchg, 1)) );
   SCIP_CALL( SCIPallocBufferArray(scip, &ocut, nnodes) );
   SCIP_CALL( SCIPallocBufferArray(scip, &orounds, nnodes) );
   SCIP_CALL( SCIPallocBufferArray(scip, &ooff, nnodes) );
   SCIP_CALL( SCIPallocBufferArray(scip, &on, nnodes) );
   SCIP_CALL( SCIPallocBufferArray(scip, &ocol, MAX(outcap, 1)) );
   SCIP_CALL( SCIPallocBufferArray(scip, &olb, MAX(outcap, 1)) );
   SCIP_CALL( SCIPallocBufferArray(scip, &oub, MAX(outcap, 1)) );
   rc = GBP_OK;
   for( k = 0; k <= nnodes; ++k )
      ptr[k] = nodebeg[k];
   /* a node's variables are columns: active problem variables (column j is SCIPgetVars(scip)[j]) */
   for( k = 0; k < nchg && rc == GBP_OK; ++k )
   {
      j = SCIPvarGetProbindex(vars[k]);
      if( j < 0 || j >= pd->ncols || pd->vars[j] != vars[k] )
         rc = GBP_ERR_INVALID;
      else
         col[k] = j;
   }
   /* the nodes run as SCIP's probing runs them: without the ranged-row rule, since a probing node keeps every
    * row's rangedrowpropagated mark (cons_linear.c:17222-17224) and a row propagated at the base after its last
    * change carries it; in SCIP's order or in rounds */
   wasranged = pd->ranged;
   pd->ranged = FALSE;
   if( rc == GBP_OK && (pd->sciporder || wasranged)
      && setDeviceParamsWith(scip, pd, pd->sciporder ? GBP_FLAG_SCIPORDER : 0) != SCIP_OKAY )
      rc = GBP_ERR_CUDA;
   if( rc == GBP_OK )
      rc = gbp_propagate_nodes(pd->ctx, pd->lb, pd->ub, nnodes, ptr, col, lbs, ubs, ocut, orounds, ooff, on, ocol, olb,
         oub, outcap, &res);
   /* the propagator's own calls: rounds, and the ranged-row rule where it was on */
   pd->ranged = wasranged;
   if( (pd->sciporder || wasranged) && setDeviceParams(scip, pd) != SCIP_OKAY )
      disable(scip, pd, "restoring the device parameters failed", GBP_ERR_INVALID);
   if( rc == GBP_OK || rc == GBP_ERR_LIMIT )
   {
      at = 0;
      for( k = 0; k < nnodes; ++k )
      {
         int t;
         cutoff[k] = ocut[k] != 0;
         outbeg[k] = at;
         if( cutoff[k] )
            continue;
         for( t = 0; t < on[k]; ++t, ++at )
         {
            outvars[at] = pd->vars[ocol[ooff[k] + t]];
            outlbs[at] = olb[ooff[k] + t];
            outubs[at] = oub[ooff[k] + t];
         }
      }
      outbeg[nnodes] = at;
      *success = TRUE;
   }
   SCIPfreeBufferArray(scip, &oub);
   SCIPfreeBufferArray(scip, &olb);
   SCIPfreeBufferArray(scip, &ocol);
   SCIPfreeBufferArray(scip, &on);
   SCIPfreeBufferArray(scip, &ooff);
   SCIPfreeBufferArray(scip, &orounds);
   SCIPfreeBufferArray(scip, &ocut);
   SCIPfreeBufferArray(scip, &col);
   SCIPfreeBufferArray(scip, &ptr);
   if( rc == GBP_ERR_INVALID )
      return SCIP_INVALIDDATA;
   return SCIP_OKAY;
}

