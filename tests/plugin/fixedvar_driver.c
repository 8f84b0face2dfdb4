/* The scenario of SCIP's own test tests/src/cons/linear/fixedvar.c with the gpulinear propagator in place (over the
 * oracle test double tests/plugin/gbp_oracle_shim.c): bell5 is solved to its root with cons_linear's propagation
 * delayed to depth 3, then a new variable fixed to 0 and a linear constraint over it and five more variables are
 * added, and the search continues to node 5.  The propagator must take up the new row (the fixed variable turns
 * into a constant of the row) and keep running.  Prints:
 *   rows <before> <after> nnz <after> active <0|1> calls <propagator calls> status <SCIP status code>
 * Usage: fixedvar_driver <bell5.mps> */
#include <stdio.h>

#include "scip/scip.h"
#include "scip/scipdefplugins.h"
#include "scip/cons_linear.h"
#include "prop_gpulinear.h"

int main(int argc, char** argv)
{
   SCIP* scip = NULL;
   SCIP_VAR* fixed = NULL;
   SCIP_CONS* cons = NULL;
   const int64_t* rowptr;
   const int32_t* colidx;
   const double* vals;
   const double* lhs;
   const double* rhs;
   SCIP_Longint ncalls = 0, nchg = 0, ncut = 0, nconfl = 0, nres = 0, nresd = 0;
   int rows0 = -1, rows1 = -1, ncols = 0;
   int i;

   if( argc < 2 )
      return 2;
   if( SCIPcreate(&scip) != SCIP_OKAY || SCIPincludeDefaultPlugins(scip) != SCIP_OKAY
      || SCIPincludePropGpulinear(scip) != SCIP_OKAY )
      return 1;
   SCIPsetEmphasis(scip, SCIP_PARAMEMPHASIS_EASYCIP, TRUE);
   SCIPsetIntParam(scip, "display/verblevel", 0);
   SCIPsetIntParam(scip, "constraints/linear/propfreq", 3);
   if( SCIPreadProb(scip, argv[1], NULL) != SCIP_OKAY )
      return 3;
   if( SCIPcreateVarBasic(scip, &fixed, "fixedzero", 0.0, 0.0, 1.0, SCIP_VARTYPE_CONTINUOUS) != SCIP_OKAY
      || SCIPaddVar(scip, fixed) != SCIP_OKAY )
      return 4;

   /* the root */
   SCIPsetLongintParam(scip, "limits/nodes", 1);
   if( SCIPsolve(scip) != SCIP_OKAY )
      return 5;
   if( SCIPgetGpulinearMatrix(scip, &rows0, &ncols, &rowptr, &colidx, &vals, &lhs, &rhs) != SCIP_OKAY )
      rows0 = -1;

   /* a constraint over the fixed variable and the first five original variables, added while solving */
   if( SCIPcreateConsBasicLinear(scip, &cons, "withfixed", 0, NULL, NULL, 0.0, SCIPinfinity(scip)) != SCIP_OKAY )
      return 6;
   for( i = 0; i < SCIPgetNOrigVars(scip) && i < 5; ++i )
      if( SCIPaddCoefLinear(scip, cons, SCIPgetOrigVars(scip)[i], i + 1.0) != SCIP_OKAY )
         return 7;
   if( SCIPaddCoefLinear(scip, cons, fixed, 1.0) != SCIP_OKAY || SCIPaddCons(scip, cons) != SCIP_OKAY
      || SCIPreleaseCons(scip, &cons) != SCIP_OKAY )
      return 8;

   /* on to node 5 */
   SCIPsetLongintParam(scip, "limits/nodes", 5);
   if( SCIPsolve(scip) != SCIP_OKAY )
      return 9;
   if( SCIPgetGpulinearMatrix(scip, &rows1, &ncols, &rowptr, &colidx, &vals, &lhs, &rhs) != SCIP_OKAY )
      rows1 = -1;
   SCIPgetGpulinearStats(scip, &ncalls, &nchg, &ncut, &nconfl, &nres, &nresd);
   printf("rows %d %d nnz %lld active %d calls %lld status %d\n", rows0, rows1,
      rows1 >= 0 ? (long long)rowptr[rows1] : -1LL, SCIPgpulinearIsActive(scip) ? 1 : 0, (long long)ncalls,
      (int)SCIPgetStatus(scip));
   SCIPreleaseVar(scip, &fixed);
   SCIPfree(&scip);
   return 0;
}
