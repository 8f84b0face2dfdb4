/* Test infrastructure only (oracle): reads an instance file with SCIP's own readers (SCIPreadProb) and prints the
 * problem as SCIP holds it, so that tests can compare the repository's readers (scip_gb300/mps.py, lpfile.py) with
 * SCIP's (src/scip/reader_mps.c, reader_lp.c).  One line per item:
 *   var <name> <integral 0|1> <lb> <ub> <obj>
 *   row <name> <lhs> <rhs> <n> <var> <coef> ...       (linear constraints only)
 *   other <constraint handler>                          (any other constraint)
 * Usage: scip_dump <file> */
#include <stdio.h>
#include <string.h>

#include "scip/scip.h"
#include "scip/scipdefplugins.h"
#include "scip/cons_linear.h"

int main(int argc, char** argv)
{
   SCIP* scip = NULL;
   SCIP_VAR** vars;
   SCIP_CONS** conss;
   int nvars;
   int nconss;
   int k;
   if( argc < 2 )
      return 2;
   if( SCIPcreate(&scip) != SCIP_OKAY || SCIPincludeDefaultPlugins(scip) != SCIP_OKAY )
      return 1;
   SCIPsetIntParam(scip, "display/verblevel", 0);
   if( SCIPreadProb(scip, argv[1], NULL) != SCIP_OKAY )
      return 3;
   vars = SCIPgetVars(scip);
   nvars = SCIPgetNVars(scip);
   for( k = 0; k < nvars; ++k )
      printf("var %s %d %.17g %.17g %.17g\n", SCIPvarGetName(vars[k]), SCIPvarIsIntegral(vars[k]) ? 1 : 0,
         SCIPvarGetLbOriginal(vars[k]), SCIPvarGetUbOriginal(vars[k]), SCIPvarGetObj(vars[k]));
   conss = SCIPgetConss(scip);
   nconss = SCIPgetNConss(scip);
   for( k = 0; k < nconss; ++k )
   {
      const char* h = SCIPconshdlrGetName(SCIPconsGetHdlr(conss[k]));
      if( strcmp(h, "linear") == 0 )
      {
         SCIP_VAR** cv = SCIPgetVarsLinear(scip, conss[k]);
         SCIP_Real* cc = SCIPgetValsLinear(scip, conss[k]);
         int n = SCIPgetNVarsLinear(scip, conss[k]);
         int q;
         printf("row %s %.17g %.17g %d", SCIPconsGetName(conss[k]), SCIPgetLhsLinear(scip, conss[k]),
            SCIPgetRhsLinear(scip, conss[k]), n);
         for( q = 0; q < n; ++q )
            printf(" %s %.17g", SCIPvarGetName(cv[q]), cc[q]);
         printf("\n");
      }
      else
         printf("other %s\n", h);
   }
   SCIPfree(&scip);
   return 0;
}
