/* Test driver for the SCIP propagator plugin (scip_gb300/plugin/prop_gpulinear.c), linked with SCIP built
 * from the reference sources (oracle/_ref) and libgbp.  Reads an instance file (format of
 * oracle/scip_driver.c), includes the plugin, runs SCIP's root propagation and prints, one item per line:
 *   active <0|1>          whether the plugin runs on a GPU
 *   matrix <m> <n> <nnz> <ok>   the rows the plugin extracted and whether they equal the file's rows
 *   root <cutoff> <sum lb> <sum ub>   root fixpoint summary (finite bounds)
 * Usage: plugin_driver <instance.bin> [--replace]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include "scip/scip.h"
#include "scip/scipdefplugins.h"
#include "prop_gpulinear.h"

static int64_t m, n, nnz;
static int64_t* rowptr;
static int32_t* colidx;
static double *vals, *lhs, *rhs, *lb, *ub;
static int8_t* vt;
static int done;
static SCIP_VAR** origvars;

static void* rd(FILE* f, size_t sz, int64_t cnt)
{
   void* p = malloc(sz * (size_t)(cnt > 0 ? cnt : 1));
   if( cnt > 0 && fread(p, sz, (size_t)cnt, f) != (size_t)cnt )
      exit(3);
   return p;
}

static SCIP_DECL_HEUREXEC(heurExecReport)
{
   int nr, nc, ok = 1, i, j;
   const int64_t *rp;
   const int32_t *ci;
   const double *va, *lh, *rh;
   double slb = 0.0, sub = 0.0;
   SCIP_VAR** vars = SCIPgetVars(scip);
   *result = SCIP_DIDNOTRUN;
   if( done )
      return SCIP_OKAY;
   done = 1;
   printf("active %d\n", SCIPgpulinearIsActive(scip) ? 1 : 0);
   SCIP_CALL( SCIPgetGpulinearMatrix(scip, &nr, &nc, &rp, &ci, &va, &lh, &rh) );
   if( nr != m || nc != n || rp[nr] != nnz )
      ok = 0;
   for( i = 0; ok && i < nr; ++i )
   {
      if( rp[i + 1] != rowptr[i + 1] || lh[i] != lhs[i] || rh[i] != rhs[i] )
      {
         fprintf(stderr, "row %lld differs: len %lld/%lld lhs %.17g/%.17g rhs %.17g/%.17g\n", (long long)i,
            (long long)(rp[i + 1] - rp[i]), (long long)(rowptr[i + 1] - rowptr[i]), lh[i], lhs[i], rh[i], rhs[i]);
         ok = 0;
      }
   }
   /* SCIP orders the transformed variables by type and may reorder the entries inside a row (cons_linear
    * sorts its variables), so the file's column c is SCIPvarGetProbindex of its transformed variable and rows
    * are compared as sets of (column, value) pairs */
   for( i = 0; ok && i < nr; ++i )
   {
      int64_t p, q;
      for( p = rowptr[i]; ok && p < rowptr[i + 1]; ++p )
      {
         int found = 0;
         SCIP_VAR* tv = NULL;
         SCIP_CALL( SCIPgetTransformedVar(scip, origvars[colidx[p]], &tv) );
         for( q = rp[i]; q < rp[i + 1]; ++q )
            if( ci[q] == SCIPvarGetProbindex(tv) && va[q] == vals[p] )
               found = 1;
         ok = found;
      }
   }
   printf("matrix %d %d %lld %d\n", nr, nc, (long long)(nr > 0 ? rp[nr] : 0), ok);
   for( j = 0; j < SCIPgetNVars(scip); ++j )
   {
      double l = SCIPvarGetLbLocal(vars[j]), u = SCIPvarGetUbLocal(vars[j]);
      if( !SCIPisInfinity(scip, -l) )
         slb += l;
      if( !SCIPisInfinity(scip, u) )
         sub += u;
   }
   printf("root 0 %.17g %.17g\n", slb, sub);
   SCIP_CALL( SCIPinterruptSolve(scip) );
   return SCIP_OKAY;
}

int main(int argc, char** argv)
{
   SCIP* scip = NULL;
   SCIP_VAR** vars;
   SCIP_HEUR* heur = NULL;
   char magic[8];
   int64_t hdr[4];
   int64_t i, j;
   FILE* f;
   if( argc < 2 )
      return 2;
   f = fopen(argv[1], "rb");
   if( f == NULL || fread(magic, 1, 8, f) != 8 || fread(hdr, 8, 4, f) != 4 )
      return 2;
   m = hdr[0]; n = hdr[1]; nnz = hdr[2];
   rowptr = rd(f, 8, m + 1); colidx = rd(f, 4, nnz); vals = rd(f, 8, nnz); lhs = rd(f, 8, m); rhs = rd(f, 8, m);
   lb = rd(f, 8, n); ub = rd(f, 8, n); vt = rd(f, 1, n);
   fclose(f);

   if( SCIPcreate(&scip) != SCIP_OKAY || SCIPincludeDefaultPlugins(scip) != SCIP_OKAY
      || SCIPincludePropGpulinear(scip) != SCIP_OKAY )
      return 1;
   SCIPcreateProbBasic(scip, "plugin");
   SCIPincludeHeurBasic(scip, &heur, "report", "test report", 'r', 1000000, 1, 0, -1, SCIP_HEURTIMING_BEFORENODE,
      FALSE, heurExecReport, NULL);
   /* the settings of the SCIP oracle (oracle/scip_driver.c): only linear propagation acts at the root */
   {
      SCIP_PARAM** params = SCIPgetParams(scip);
      SCIP_PROP** props = SCIPgetProps(scip);
      int np = SCIPgetNParams(scip), k;
      for( k = 0; k < np; ++k )
         if( strncmp(SCIPparamGetName(params[k]), "constraints/linear/upgrade/", 27) == 0 )
            SCIPsetBoolParam(scip, SCIPparamGetName(params[k]), FALSE);
      for( k = 0; k < SCIPgetNProps(scip); ++k )
      {
         char pn[SCIP_MAXSTRLEN];
         if( strcmp(SCIPpropGetName(props[k]), "gpulinear") == 0 )
            continue;
         snprintf(pn, SCIP_MAXSTRLEN, "propagating/%s/freq", SCIPpropGetName(props[k]));
         SCIPsetIntParam(scip, pn, -1);
      }
   }
   SCIPsetIntParam(scip, "presolving/maxrounds", 0);
   SCIPsetBoolParam(scip, "constraints/linear/rangedrowpropagation", FALSE);
   SCIPsetRealParam(scip, "constraints/linear/maxeasyactivitydelta", 0.0);
   SCIPsetIntParam(scip, "propagating/maxrounds", -1);
   SCIPsetIntParam(scip, "propagating/maxroundsroot", -1);
   SCIPsetHeuristics(scip, SCIP_PARAMSETTING_OFF, TRUE);
   SCIPsetSeparating(scip, SCIP_PARAMSETTING_OFF, TRUE);
   SCIPsetIntParam(scip, "heuristics/report/freq", 1);
   SCIPsetBoolParam(scip, "conflict/enable", FALSE);
   SCIPsetIntParam(scip, "display/verblevel", 0);
   SCIPsetIntParam(scip, "lp/solvefreq", -1);
   if( argc > 2 && strcmp(argv[2], "--replace") == 0 )
      SCIPsetBoolParam(scip, "propagating/gpulinear/replacelinear", TRUE);
   vars = malloc(sizeof(SCIP_VAR*) * (size_t)n);
   origvars = vars;
   for( j = 0; j < n; ++j )
   {
      char name[32];
      snprintf(name, 32, "x%lld", (long long)j);
      SCIPcreateVarBasic(scip, &vars[j], name, lb[j], ub[j], 0.0, vt[j] ? SCIP_VARTYPE_INTEGER : SCIP_VARTYPE_CONTINUOUS);
      SCIPaddVar(scip, vars[j]);
   }
   for( i = 0; i < m; ++i )
   {
      SCIP_CONS* cons;
      SCIP_VAR* rv[4096];
      char name[32];
      int len = (int)(rowptr[i + 1] - rowptr[i]), q;
      for( q = 0; q < len; ++q )
         rv[q] = vars[colidx[rowptr[i] + q]];
      snprintf(name, 32, "r%lld", (long long)i);
      SCIPcreateConsBasicLinear(scip, &cons, name, len, rv, &vals[rowptr[i]], lhs[i], rhs[i]);
      SCIPaddCons(scip, cons);
      SCIPreleaseCons(scip, &cons);
   }
   {
      int pf = 0;
      SCIPgetIntParam(scip, "constraints/linear/propfreq", &pf);
      printf("propfreq %d\n", pf);
   }
   if( SCIPsolve(scip) != SCIP_OKAY )
      return 1;
   if( !done )
      printf("root 1 0 0\n");
   for( j = 0; j < n; ++j )
      SCIPreleaseVar(scip, &vars[j]);
   free(vars);
   SCIPfree(&scip);
   return 0;
}
