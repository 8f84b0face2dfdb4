/* Test infrastructure only (oracle): runs SCIP 11's own cons_linear propagation on an instance file and
 * writes the resulting bounds, so that fixtures under tests/golden can pin the C restatement
 * (oracle/linprop_oracle.c) and the CUDA path against the reference itself.
 *
 * Usage:  scip_oracle <instance.bin> <nodes.bin|-> <out.bin> [--easy] [--ranged] [--nosort] [--repeat R]
 *                      [--fresh] [--order order.bin] [--unmark]
 *
 * Pattern (the probing-in-heuristic recipe; see src/scip/scip_probing.c:120-690 and
 * tests/include/scip_test.c:121-133 for the interrupt idiom):
 *   - parameters switch off presolving (presolving/maxrounds=0), every linear upgrade
 *     (constraints/linear/upgrade/<x>=FALSE, cons_linear.c:17752-17757), ranged-row propagation
 *     (constraints/linear/rangedrowpropagation=FALSE, cons_linear.c:155), every other propagator
 *     (propagating/<x>/freq=-1), heuristics, separation, conflict analysis and LP solving, and lift
 *     the propagation round limits (propagating/maxrounds[root]=-1);
 *   - --ranged switches ranged-row propagation (cons_linear.c:5715) back on, without its artificial
 *     constraints (constraints/linear/rangedrowartcons=FALSE); --nosort sets constraints/linear/sortvars=FALSE;
 *   - constraints/linear/maxeasyactivitydelta=0 selects the residual rule (cons_linear.c:6700) for
 *     every row; --easy keeps SCIP's default (1e6), i.e. the slack rule of cons_linear.c:5380 for
 *     rows whose largest activity contribution is below 1e6;
 *   - the root fixpoint is what SCIP's root propagation (solve.c:723) leaves in the local bounds when
 *     the BEFORENODE heuristic runs (solve.c:5296-5303);
 *   - each node: SCIPnewProbingNode, SCIPchgVarLb/UbProbing for its bound changes,
 *     SCIPpropagateProbing(-1) (scip_probing.c:581), read SCIPvarGetLb/UbLocal, SCIPbacktrackProbing(0);
 *   - --fresh: every node starts from a newly transformed problem (SCIPfreeTransform, then the root again), so a
 *     node's result does not depend on the nodes before it (SCIP keeps activities, which drift under incremental
 *     updates, marks left by a cut-off node, and per-row flags across the nodes of one probing session);
 *   - --unmark: before each node (in one probing session), unmark the linear rows a cut-off node left marked, so
 *     that every node starts from the root's marks (none) -- the part of --fresh that is cheap for large problems;
 *   - --order: after the (first) root, each row's variables in the order SCIP holds them (SCIPgetVarsLinear on the
 *     transformed constraint), the order the next propagation visits them in: int64 m, then per row int32 len and
 *     int32 columns[len] (len = -1 for a row deleted at the root).
 *
 * Instance file (little endian): "LPINST01", int64 m, n, nnz, flags; int64 rowptr[m+1]; int32 col[nnz];
 * f64 val[nnz]; f64 lhs[m]; f64 rhs[m]; f64 lb[n]; f64 ub[n]; int8 vartype[n] (0 continuous, 1 integer).
 * Node file: "LPNODE01", int64 nnodes, nchg; int64 ptr[nnodes+1]; int32 col[nchg]; f64 lb[nchg]; f64 ub[nchg].
 * Output: "LPOUT001", int64 n, nnodes; int8 rootcutoff; f64 roottime; f64 rootlb[n]; f64 rootub[n];
 *         per node: int8 cutoff; f64 seconds; int32 nchanged; {int32 col; f64 lb; f64 ub}[nchanged]
 *         (columns whose local bounds differ from the root fixpoint).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <time.h>

#include "scip/scip.h"
#include "scip/scipdefplugins.h"

typedef struct
{
   int64_t m, n, nnz;
   int64_t* rowptr;
   int32_t* col;
   double* val;
   double* lhs;
   double* rhs;
   double* lb;
   double* ub;
   int8_t* vartype;
   int64_t nnodes, nchg;
   int64_t* nptr;
   int32_t* ncol;
   double* nlb;
   double* nub;
} Inst;

typedef struct
{
   Inst* inst;
   SCIP_VAR** vars;
   SCIP_CONS** conss;
   FILE* out;
   int done;
   int repeat;
   int64_t k0;          /* nodes [k0, k1) are propagated in this solve */
   int64_t k1;
   int rootdone;        /* the root record was written */
   double* rootlb;
   double* rootub;
   const char* orderpath;
   int unmark;
} Run;

static void die(const char* msg)
{
   fprintf(stderr, "scip_oracle: %s\n", msg);
   exit(2);
}

static void* readn(FILE* f, size_t sz, int64_t cnt)
{
   void* p = malloc(sz * (size_t)(cnt > 0 ? cnt : 1));
   if( p == NULL )
      die("out of memory");
   if( cnt > 0 && fread(p, sz, (size_t)cnt, f) != (size_t)cnt )
      die("short read");
   return p;
}

static double now(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void loadInstance(const char* path, Inst* in)
{
   char magic[8];
   int64_t hdr[4];
   FILE* f = fopen(path, "rb");
   if( f == NULL )
      die("cannot open instance");
   if( fread(magic, 1, 8, f) != 8 || memcmp(magic, "LPINST01", 8) != 0 )
      die("bad instance magic");
   if( fread(hdr, sizeof(int64_t), 4, f) != 4 )
      die("short header");
   in->m = hdr[0]; in->n = hdr[1]; in->nnz = hdr[2];
   in->rowptr = readn(f, 8, in->m + 1);
   in->col = readn(f, 4, in->nnz);
   in->val = readn(f, 8, in->nnz);
   in->lhs = readn(f, 8, in->m);
   in->rhs = readn(f, 8, in->m);
   in->lb = readn(f, 8, in->n);
   in->ub = readn(f, 8, in->n);
   in->vartype = readn(f, 1, in->n);
   fclose(f);
}

static void loadNodes(const char* path, Inst* in)
{
   char magic[8];
   int64_t hdr[2];
   FILE* f;
   in->nnodes = 0;
   in->nchg = 0;
   if( strcmp(path, "-") == 0 )
      return;
   f = fopen(path, "rb");
   if( f == NULL )
      die("cannot open node file");
   if( fread(magic, 1, 8, f) != 8 || memcmp(magic, "LPNODE01", 8) != 0 )
      die("bad node magic");
   if( fread(hdr, sizeof(int64_t), 2, f) != 2 )
      die("short node header");
   in->nnodes = hdr[0]; in->nchg = hdr[1];
   in->nptr = readn(f, 8, in->nnodes + 1);
   in->ncol = readn(f, 4, in->nchg);
   in->nlb = readn(f, 8, in->nchg);
   in->nub = readn(f, 8, in->nchg);
   fclose(f);
}

/* each row's variables in the order the transformed constraint holds them (columns), -1 for a deleted row */
static SCIP_RETCODE writeOrder(SCIP* scip, Run* run)
{
   Inst* in = run->inst;
   FILE* f = fopen(run->orderpath, "wb");
   int64_t i;
   if( f == NULL )
      die("cannot open order output");
   fwrite(&in->m, 8, 1, f);
   for( i = 0; i < in->m; ++i )
   {
      SCIP_CONS* tc = NULL;
      int32_t len = -1;
      SCIP_CALL( SCIPgetTransformedCons(scip, run->conss[i], &tc) );
      if( tc != NULL && !SCIPconsIsDeleted(tc) )
      {
         SCIP_VAR** vars = SCIPgetVarsLinear(scip, tc);
         int q;
         len = SCIPgetNVarsLinear(scip, tc);
         fwrite(&len, 4, 1, f);
         for( q = 0; q < len; ++q )
         {
            /* transformed variables are named t_<original name>, and the original names are x<column> */
            int32_t c = (int32_t)strtol(SCIPvarGetName(vars[q]) + 3, NULL, 10);
            fwrite(&c, 4, 1, f);
         }
      }
      else
         fwrite(&len, 4, 1, f);
   }
   fclose(f);
   return SCIP_OKAY;
}

/* the work happens the first time SCIP calls the heuristic, right after the root propagation loop */
static SCIP_DECL_HEUREXEC(heurExecOracle)
{
   Run* run = (Run*)SCIPheurGetData(heur);
   Inst* in = run->inst;
   int64_t j;
   int64_t k;
   int8_t flag = 0;
   double roottime = 0.0;
   double* rootlb;
   double* rootub;

   *result = SCIP_DIDNOTRUN;
   if( run->done )
      return SCIP_OKAY;
   run->done = 1;

   rootlb = run->rootlb;
   rootub = run->rootub;
   if( !run->rootdone )
   {
      for( j = 0; j < in->n; ++j )
      {
         SCIP_VAR* tv;
         SCIP_CALL( SCIPgetTransformedVar(scip, run->vars[j], &tv) );
         rootlb[j] = SCIPvarGetLbLocal(tv);
         rootub[j] = SCIPvarGetUbLocal(tv);
      }
      fwrite(&flag, 1, 1, run->out);
      fwrite(&roottime, 8, 1, run->out);
      fwrite(rootlb, 8, (size_t)in->n, run->out);
      fwrite(rootub, 8, (size_t)in->n, run->out);
      if( run->orderpath != NULL )
         SCIP_CALL( writeOrder(scip, run) );
      run->rootdone = 1;
   }

   SCIP_CALL( SCIPstartProbing(scip) );
   for( k = run->k0; k < run->k1; ++k )
   {
      SCIP_Bool cutoff = FALSE;
      SCIP_Longint ndomreds = 0;
      int32_t nchanged = 0;
      int8_t co;
      double t0;
      double t1;
      double best = 1e300;
      int rep;

      if( run->unmark )
      {
         /* rows a cut-off node left marked for propagation (its loop stopped before reaching them) */
         SCIP_CONSHDLR* lin = SCIPfindConshdlr(scip, "linear");
         SCIP_CONS** lc = SCIPconshdlrGetConss(lin);
         int nlc = SCIPconshdlrGetNConss(lin);
         int c;
         for( c = 0; c < nlc; ++c )
            if( SCIPconsIsMarkedPropagate(lc[c]) )
               SCIP_CALL( SCIPunmarkConsPropagate(scip, lc[c]) );
      }
      for( rep = 0; rep < run->repeat; ++rep )
      {
         int64_t q;
         cutoff = FALSE;
         SCIP_CALL( SCIPnewProbingNode(scip) );
         for( q = in->nptr[k]; q < in->nptr[k + 1] && !cutoff; ++q )
         {
            SCIP_VAR* tv;
            SCIP_CALL( SCIPgetTransformedVar(scip, run->vars[in->ncol[q]], &tv) );
            if( in->nlb[q] > SCIPvarGetUbLocal(tv) || in->nub[q] < SCIPvarGetLbLocal(tv) )
               cutoff = TRUE;
            else
            {
               if( in->nlb[q] > SCIPvarGetLbLocal(tv) )
                  SCIP_CALL( SCIPchgVarLbProbing(scip, tv, in->nlb[q]) );
               if( in->nub[q] < SCIPvarGetUbLocal(tv) )
                  SCIP_CALL( SCIPchgVarUbProbing(scip, tv, in->nub[q]) );
            }
         }
         t0 = now();
         if( !cutoff )
            SCIP_CALL( SCIPpropagateProbing(scip, -1, &cutoff, &ndomreds) );
         t1 = now();
         if( t1 - t0 < best )
            best = t1 - t0;
         if( rep + 1 < run->repeat )
            SCIP_CALL( SCIPbacktrackProbing(scip, 0) );
      }

      co = cutoff ? 1 : 0;
      fwrite(&co, 1, 1, run->out);
      fwrite(&best, 8, 1, run->out);
      if( !cutoff )
      {
         for( j = 0; j < in->n; ++j )
         {
            SCIP_VAR* tv;
            SCIP_CALL( SCIPgetTransformedVar(scip, run->vars[j], &tv) );
            if( SCIPvarGetLbLocal(tv) != rootlb[j] || SCIPvarGetUbLocal(tv) != rootub[j] )
               ++nchanged;
         }
      }
      fwrite(&nchanged, 4, 1, run->out);
      if( !cutoff )
      {
         for( j = 0; j < in->n; ++j )
         {
            SCIP_VAR* tv;
            double lb;
            double ub;
            int32_t c = (int32_t)j;
            SCIP_CALL( SCIPgetTransformedVar(scip, run->vars[j], &tv) );
            lb = SCIPvarGetLbLocal(tv);
            ub = SCIPvarGetUbLocal(tv);
            if( lb != rootlb[j] || ub != rootub[j] )
            {
               fwrite(&c, 4, 1, run->out);
               fwrite(&lb, 8, 1, run->out);
               fwrite(&ub, 8, 1, run->out);
            }
         }
      }
      SCIP_CALL( SCIPbacktrackProbing(scip, 0) );
   }
   SCIP_CALL( SCIPendProbing(scip) );

   SCIP_CALL( SCIPinterruptSolve(scip) );
   *result = SCIP_DIDNOTFIND;
   return SCIP_OKAY;
}

static SCIP_RETCODE setParams(SCIP* scip, int easy, int ranged, int nosort)
{
   SCIP_PARAM** params = SCIPgetParams(scip);
   int nparams = SCIPgetNParams(scip);
   SCIP_PROP** props = SCIPgetProps(scip);
   int nprops = SCIPgetNProps(scip);
   int i;

   for( i = 0; i < nparams; ++i )
   {
      const char* name = SCIPparamGetName(params[i]);
      if( strncmp(name, "constraints/linear/upgrade/", 27) == 0 )
         SCIP_CALL( SCIPsetBoolParam(scip, name, FALSE) );
   }
   for( i = 0; i < nprops; ++i )
   {
      char pname[SCIP_MAXSTRLEN];
      (void)SCIPsnprintf(pname, SCIP_MAXSTRLEN, "propagating/%s/freq", SCIPpropGetName(props[i]));
      SCIP_CALL( SCIPsetIntParam(scip, pname, -1) );
   }
   SCIP_CALL( SCIPsetIntParam(scip, "presolving/maxrounds", 0) );
   SCIP_CALL( SCIPsetBoolParam(scip, "constraints/linear/rangedrowpropagation", ranged ? TRUE : FALSE) );
   SCIP_CALL( SCIPsetBoolParam(scip, "constraints/linear/rangedrowartcons", FALSE) );
   if( nosort )
      SCIP_CALL( SCIPsetBoolParam(scip, "constraints/linear/sortvars", FALSE) );
   if( !easy )
      SCIP_CALL( SCIPsetRealParam(scip, "constraints/linear/maxeasyactivitydelta", 0.0) );
   SCIP_CALL( SCIPsetIntParam(scip, "propagating/maxrounds", -1) );
   SCIP_CALL( SCIPsetIntParam(scip, "propagating/maxroundsroot", -1) );
   SCIP_CALL( SCIPsetHeuristics(scip, SCIP_PARAMSETTING_OFF, TRUE) );
   SCIP_CALL( SCIPsetSeparating(scip, SCIP_PARAMSETTING_OFF, TRUE) );
   SCIP_CALL( SCIPsetBoolParam(scip, "conflict/enable", FALSE) );
   SCIP_CALL( SCIPsetIntParam(scip, "lp/solvefreq", -1) );
   SCIP_CALL( SCIPsetIntParam(scip, "display/verblevel", 0) );
   return SCIP_OKAY;
}

static SCIP_RETCODE run(const char* instpath, const char* nodepath, const char* outpath, int easy, int ranged,
   int nosort, int repeat, int fresh, const char* orderpath, int unmark)
{
   SCIP* scip = NULL;
   Inst in;
   Run r;
   SCIP_HEUR* heur = NULL;
   int64_t i;
   int64_t j;
   const char magic[8] = { 'L', 'P', 'O', 'U', 'T', '0', '0', '1' };
   int64_t hdr[2];

   memset(&in, 0, sizeof(in));
   loadInstance(instpath, &in);
   loadNodes(nodepath, &in);

   SCIP_CALL( SCIPcreate(&scip) );
   SCIP_CALL( SCIPincludeDefaultPlugins(scip) );
   SCIP_CALL( SCIPcreateProbBasic(scip, "oracle") );

   memset(&r, 0, sizeof(r));
   r.inst = &in;
   r.repeat = repeat;
   r.orderpath = orderpath;
   r.unmark = unmark;
   r.k0 = 0;
   r.k1 = fresh ? (in.nnodes > 0 ? 1 : 0) : in.nnodes;
   r.rootlb = malloc(sizeof(double) * (size_t)(in.n + 1));
   r.rootub = malloc(sizeof(double) * (size_t)(in.n + 1));
   r.conss = malloc(sizeof(SCIP_CONS*) * (size_t)(in.m + 1));
   r.vars = malloc(sizeof(SCIP_VAR*) * (size_t)in.n);
   r.out = fopen(outpath, "wb");
   if( r.out == NULL )
      die("cannot open output");
   hdr[0] = in.n;
   hdr[1] = in.nnodes;
   fwrite(magic, 1, 8, r.out);
   fwrite(hdr, 8, 2, r.out);

   SCIP_CALL( SCIPincludeHeurBasic(scip, &heur, "oracle", "propagation oracle driver", 'o', 1000000, 1, 0, -1,
         SCIP_HEURTIMING_BEFORENODE, FALSE, heurExecOracle, (SCIP_HEURDATA*)&r) );
   SCIP_CALL( setParams(scip, easy, ranged, nosort) );
   /* SCIPsetHeuristics(OFF) above switched the oracle heuristic off as well: switch it back on */
   SCIP_CALL( SCIPsetIntParam(scip, "heuristics/oracle/freq", 1) );

   for( j = 0; j < in.n; ++j )
   {
      char name[32];
      (void)SCIPsnprintf(name, 32, "x%lld", (long long)j);
      SCIP_CALL( SCIPcreateVarBasic(scip, &r.vars[j], name, in.lb[j], in.ub[j], 0.0,
            in.vartype[j] ? SCIP_VARTYPE_INTEGER : SCIP_VARTYPE_CONTINUOUS) );
      SCIP_CALL( SCIPaddVar(scip, r.vars[j]) );
   }
   {
      SCIP_VAR** rowvars = malloc(sizeof(SCIP_VAR*) * 8192);
      for( i = 0; i < in.m; ++i )
      {
         SCIP_CONS* cons;
         char name[32];
         int64_t p0 = in.rowptr[i];
         int len = (int)(in.rowptr[i + 1] - p0);
         int q;
         if( len > 8192 )
            die("row too long");
         for( q = 0; q < len; ++q )
            rowvars[q] = r.vars[in.col[p0 + q]];
         (void)SCIPsnprintf(name, 32, "r%lld", (long long)i);
         SCIP_CALL( SCIPcreateConsBasicLinear(scip, &cons, name, len, rowvars, &in.val[p0], in.lhs[i], in.rhs[i]) );
         SCIP_CALL( SCIPaddCons(scip, cons) );
         r.conss[i] = cons;   /* kept captured, for the order output */
      }
      free(rowvars);
   }

   SCIP_CALL( SCIPsolve(scip) );
   /* --fresh: every further node gets a newly transformed problem and its own root */
   while( fresh && r.done && r.k1 < in.nnodes )
   {
      SCIP_CALL( SCIPfreeTransform(scip) );
      r.done = 0;
      r.k0 = r.k1;
      r.k1 = r.k0 + 1;
      SCIP_CALL( SCIPsolve(scip) );
   }

   if( !r.done )
   {
      /* the root propagation cut the problem off before any heuristic ran */
      int8_t flag = 1;
      double zero = 0.0;
      fwrite(&flag, 1, 1, r.out);
      fwrite(&zero, 8, 1, r.out);
      for( j = 0; j < 2 * in.n; ++j )
         fwrite(&zero, 8, 1, r.out);
   }
   fclose(r.out);

   for( i = 0; i < in.m; ++i )
      SCIP_CALL( SCIPreleaseCons(scip, &r.conss[i]) );
   for( j = 0; j < in.n; ++j )
      SCIP_CALL( SCIPreleaseVar(scip, &r.vars[j]) );
   free(r.vars);
   free(r.conss);
   free(r.rootlb);
   free(r.rootub);
   SCIP_CALL( SCIPfree(&scip) );
   return SCIP_OKAY;
}

int main(int argc, char** argv)
{
   int easy = 0;
   int ranged = 0;
   int nosort = 0;
   int repeat = 1;
   int fresh = 0;
   const char* orderpath = NULL;
   int unmark = 0;
   int a;
   SCIP_RETCODE rc;
   if( argc < 4 )
   {
      fprintf(stderr, "usage: %s instance.bin nodes.bin|- out.bin [--easy] [--ranged] [--nosort] [--repeat R] [--fresh]"
         " [--order order.bin] [--unmark]\n", argv[0]);
      return 2;
   }
   for( a = 4; a < argc; ++a )
   {
      if( strcmp(argv[a], "--easy") == 0 )
         easy = 1;
      else if( strcmp(argv[a], "--ranged") == 0 )
         ranged = 1;
      else if( strcmp(argv[a], "--nosort") == 0 )
         nosort = 1;
      else if( strcmp(argv[a], "--repeat") == 0 && a + 1 < argc )
         repeat = atoi(argv[++a]);
      else if( strcmp(argv[a], "--fresh") == 0 )
         fresh = 1;
      else if( strcmp(argv[a], "--order") == 0 && a + 1 < argc )
         orderpath = argv[++a];
      else if( strcmp(argv[a], "--unmark") == 0 )
         unmark = 1;
   }
   if( repeat < 1 )
      repeat = 1;
   rc = run(argv[1], argv[2], argv[3], easy, ranged, nosort, repeat, fresh, orderpath, unmark);
   if( rc != SCIP_OKAY )
   {
      fprintf(stderr, "scip_oracle: SCIP error %d\n", (int)rc);
      return 1;
   }
   return 0;
}
