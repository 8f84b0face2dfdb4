/* Solves an MPS instance with SCIP (built from the reference sources), either with cons_linear's own propagation
 * ("plain") or with the gpulinear propagator replacing it ("gpulinear", linked against the oracle test double
 * tests/plugin/gbp_oracle_shim.c).  Presolving, linear upgrades, ranged-row propagation (unless asked for) and LP
 * solving are off in both modes, so the search runs on propagation and conflict analysis alone.  Prints, one item
 * per line:
 *   status <SCIP status>    obj <primal bound>    nodes <n>
 *   gpulinear <calls> <bound changes> <cutoffs> <cutoffs analysed> <resolve requests> <resolved> active <0|1>
 *   conflicts <conflicts found>    rangedreasons <changes and cutoffs explained by a ranged row>
 * Flags after the node limit: "ranged" switches ranged-row propagation on in both modes (without artificial
 * constraints); "presolve" keeps SCIP's presolving and its upgrades of linear rows to the specialised handlers
 * (setppc, logicor, knapsack, varbound), whose propagation the plugin then replaces as well.
 * Usage: solve_driver <instance file> <plain|gpulinear> [node limit] [ranged] [presolve] */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "scip/scip.h"
#include "scip/scipdefplugins.h"
#include "prop_gpulinear.h"

int main(int argc, char** argv)
{
   SCIP* scip = NULL;
   int gpulinear;
   long long nodelimit;
   int ranged = 0;
   int presolve = 0;
   int k;
   if( argc < 3 )
      return 2;
   gpulinear = strcmp(argv[2], "gpulinear") == 0;
   nodelimit = argc > 3 ? atoll(argv[3]) : 200000;
   for( k = 4; k < argc; ++k )
   {
      ranged = ranged || strcmp(argv[k], "ranged") == 0;
      presolve = presolve || strcmp(argv[k], "presolve") == 0;
   }
   if( SCIPcreate(&scip) != SCIP_OKAY || SCIPincludeDefaultPlugins(scip) != SCIP_OKAY )
      return 1;
   if( gpulinear )
   {
      if( SCIPincludePropGpulinear(scip) != SCIP_OKAY )
         return 1;
      SCIPsetBoolParam(scip, "propagating/gpulinear/replacelinear", TRUE);
      if( presolve )
         SCIPsetBoolParam(scip, "propagating/gpulinear/replacespecialised", TRUE);
   }
   if( SCIPreadProb(scip, argv[1], NULL) != SCIP_OKAY )
      return 3;
   if( !presolve )
   {
      SCIP_PARAM** params = SCIPgetParams(scip);
      int np = SCIPgetNParams(scip);
      for( k = 0; k < np; ++k )
         if( strncmp(SCIPparamGetName(params[k]), "constraints/linear/upgrade/", 27) == 0 )
            SCIPsetBoolParam(scip, SCIPparamGetName(params[k]), FALSE);
      SCIPsetIntParam(scip, "presolving/maxrounds", 0);
   }
   SCIPsetBoolParam(scip, "constraints/linear/rangedrowpropagation", ranged);
   SCIPsetBoolParam(scip, "constraints/linear/rangedrowartcons", FALSE);
   SCIPsetIntParam(scip, "lp/solvefreq", -1);
   SCIPsetBoolParam(scip, "conflict/enable", TRUE);
   SCIPsetLongintParam(scip, "limits/nodes", nodelimit);
   SCIPsetRealParam(scip, "limits/time", 120.0);
   SCIPsetIntParam(scip, "display/verblevel", 0);
   if( SCIPsolve(scip) != SCIP_OKAY )
      return 4;
   {
      const char* st;
      switch( SCIPgetStatus(scip) )
      {
      case SCIP_STATUS_OPTIMAL: st = "optimal"; break;
      case SCIP_STATUS_INFEASIBLE: st = "infeasible"; break;
      case SCIP_STATUS_NODELIMIT: st = "nodelimit"; break;
      case SCIP_STATUS_TIMELIMIT: st = "timelimit"; break;
      default: st = "other"; break;
      }
      printf("status %s\n", st);
   }
   printf("obj %.10g\n", SCIPgetPrimalbound(scip));
   printf("nodes %lld\n", (long long)SCIPgetNNodes(scip));
   printf("conflicts %lld\n", (long long)SCIPgetNConflictConssFound(scip));
   if( gpulinear )
   {
      SCIP_Longint c, b, x, a, q, r;
      if( SCIPgetGpulinearStats(scip, &c, &b, &x, &a, &q, &r) != SCIP_OKAY )
         return 5;
      printf("gpulinear %lld %lld %lld %lld %lld %lld active %d\n", (long long)c, (long long)b, (long long)x,
         (long long)a, (long long)q, (long long)r, SCIPgpulinearIsActive(scip) ? 1 : 0);
      printf("rangedreasons %lld\n", (long long)SCIPgetGpulinearRangedReasons(scip));
   }
   SCIPfree(&scip);
   return 0;
}
