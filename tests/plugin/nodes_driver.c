/* Checks SCIPpropagateGpulinearNodes (the plugin's batched entry) inside SCIP against SCIP's own probing: reads an
 * MPS instance (SCIP built from the reference sources, the plugin linked against the oracle test double
 * tests/plugin/gbp_oracle_shim.c), propagates at the root, then in a heuristic draws nodes of 1..4 integer fixings,
 * propagates all of them with one SCIPpropagateGpulinearNodes call, and each of them again through SCIP's
 * SCIPpropagateProbing with cons_linear's propagation (the plugin does not run in probing:
 * propagating/gpulinear/probing = FALSE).  Prints:
 *   nodes <n> success <0|1> cutoffs <batched> <probing> cutoffmismatch <k> intmismatch <k> moved <total>
 *   ... contmismatch <k>   (nodes with a continuous bound outside 1e-9 relative / feastol absolute)
 * With "sciporder" after the node count the batched call runs in SCIP's own order
 * (propagating/gpulinear/sciporder), and before each probing node the rows a cut-off node left marked are unmarked,
 * so that every node starts with no row marked, as that mode assumes.
 * With "easy" last, cons_linear and the plugin use SCIP's default rule choice (maxeasyactivitydelta 1e6) instead of
 * the residual rule everywhere (0).
 * The fifth argument lists options: "ranged" turns ranged-row propagation on (constraints/linear/
 * rangedrowpropagation, without artificial constraints) for SCIP and the plugin, "nosort" sets
 * constraints/linear/sortvars to FALSE ("plain": neither).
 * With a depth last, the check runs at the first search node of that depth instead of the root: the nodes' base
 * is that node's local bounds, below SCIP's global ones.
 * With "presolve" after the depth, SCIP presolves first (its rows stay linear: every upgrade is off).
 * Usage: nodes_driver <instance.mps> [nodes] [sciporder|rounds] [easy|res] [ranged|plain] [depth] [presolve] */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "scip/scip.h"
#include "scip/scipdefplugins.h"
#include "prop_gpulinear.h"

static int nwant = 200;
static int done = 0;
static int sciporder = 0;
static int easyrule = 0;
static int ranged = 0;
static int atdepth = 0;
static int presolve = 0;
static int nosort = 0;

static unsigned long long lcg = 0x2545f4914f6cdd1dull;
static unsigned long long nextRand(void)
{
   lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
   return lcg >> 33;
}

static SCIP_DECL_HEUREXEC(heurExecCheck)
{
   SCIP_VAR** vars = SCIPgetVars(scip);
   int nvars = SCIPgetNVars(scip);
   SCIP_VAR** cand;
   int ncand = 0;
   int* beg;
   SCIP_VAR** nv;
   SCIP_Real* nl;
   SCIP_Real* nu;
   SCIP_Bool* cut;
   int* obeg;
   SCIP_VAR** ov;
   SCIP_Real* ol;
   SCIP_Real* ou;
   SCIP_Bool success = FALSE;
   int outcap;
   int k;
   int j;
   int ncutb = 0, ncutp = 0, cutmis = 0, intmis = 0, contmis = 0;

   (void)heur;
   (void)nodeinfeasible;
   (void)heurtiming;
   *result = SCIP_DIDNOTRUN;
   if( done || SCIPgetDepth(scip) < atdepth )
      return SCIP_OKAY;
   done = 1;
   SCIP_CALL( SCIPallocBufferArray(scip, &cand, nvars) );
   for( j = 0; j < nvars; ++j )
      if( SCIPvarGetType(vars[j]) != SCIP_VARTYPE_CONTINUOUS && SCIPvarGetUbLocal(vars[j]) > SCIPvarGetLbLocal(vars[j])
         && !SCIPisInfinity(scip, SCIPvarGetUbLocal(vars[j])) && !SCIPisInfinity(scip, -SCIPvarGetLbLocal(vars[j])) )
         cand[ncand++] = vars[j];
   if( ncand == 0 )
   {
      SCIPfreeBufferArray(scip, &cand);
      printf("nodes 0 success 0\n");
      return SCIP_OKAY;
   }
   SCIP_CALL( SCIPallocBufferArray(scip, &beg, nwant + 1) );
   SCIP_CALL( SCIPallocBufferArray(scip, &nv, 4 * nwant) );
   SCIP_CALL( SCIPallocBufferArray(scip, &nl, 4 * nwant) );
   SCIP_CALL( SCIPallocBufferArray(scip, &nu, 4 * nwant) );
   beg[0] = 0;
   for( k = 0; k < nwant; ++k )
   {
      int nf = 1 + (int)(nextRand() % 4);
      int t;
      beg[k + 1] = beg[k];
      for( t = 0; t < nf; ++t )
      {
         SCIP_VAR* v = cand[nextRand() % (unsigned long long)ncand];
         SCIP_Real lo = SCIPvarGetLbLocal(v), hi = SCIPvarGetUbLocal(v);
         SCIP_Real x = lo + (SCIP_Real)(nextRand() % (unsigned long long)(hi - lo + 1.0));
         int q;
         for( q = beg[k]; q < beg[k + 1]; ++q )
            if( nv[q] == v )
               break;
         if( q < beg[k + 1] )
            continue;
         nv[beg[k + 1]] = v;
         nl[beg[k + 1]] = x;
         nu[beg[k + 1]] = x;
         beg[k + 1]++;
      }
   }
   outcap = nwant * nvars;
   SCIP_CALL( SCIPallocBufferArray(scip, &cut, nwant) );
   SCIP_CALL( SCIPallocBufferArray(scip, &obeg, nwant + 1) );
   SCIP_CALL( SCIPallocBufferArray(scip, &ov, outcap) );
   SCIP_CALL( SCIPallocBufferArray(scip, &ol, outcap) );
   SCIP_CALL( SCIPallocBufferArray(scip, &ou, outcap) );
   SCIP_CALL( SCIPpropagateGpulinearNodes(scip, nwant, beg, nv, nl, nu, outcap, cut, obeg, ov, ol, ou, &success) );
   if( success )
   {
      SCIP_Real* elb;
      SCIP_Real* eub;
      SCIP_Real* rlb;
      SCIP_Real* rub;
      SCIP_CALL( SCIPallocBufferArray(scip, &elb, nvars) );
      SCIP_CALL( SCIPallocBufferArray(scip, &eub, nvars) );
      SCIP_CALL( SCIPallocBufferArray(scip, &rlb, nvars) );
      SCIP_CALL( SCIPallocBufferArray(scip, &rub, nvars) );
      for( j = 0; j < nvars; ++j )  /* the nodes' base: the local bounds the batched call started from */
      {
         rlb[j] = SCIPvarGetLbLocal(vars[j]);
         rub[j] = SCIPvarGetUbLocal(vars[j]);
      }
      SCIP_CALL( SCIPstartProbing(scip) );
      for( k = 0; k < nwant; ++k )
      {
         SCIP_Bool pcut = FALSE;
         int q;
         if( sciporder )
         {
            /* rows a cut-off node left marked (its propagation stopped before reaching them) */
            SCIP_CONSHDLR* lin = SCIPfindConshdlr(scip, "linear");
            SCIP_CONS** lc = SCIPconshdlrGetConss(lin);
            int nlc = SCIPconshdlrGetNConss(lin);
            int c;
            for( c = 0; c < nlc; ++c )
               if( SCIPconsIsMarkedPropagate(lc[c]) )
                  SCIP_CALL( SCIPunmarkConsPropagate(scip, lc[c]) );
         }
         SCIP_CALL( SCIPnewProbingNode(scip) );
         for( q = beg[k]; q < beg[k + 1] && !pcut; ++q )
         {
            if( nl[q] > SCIPvarGetUbLocal(nv[q]) || nu[q] < SCIPvarGetLbLocal(nv[q]) )
               pcut = TRUE;
            else
            {
               if( nl[q] > SCIPvarGetLbLocal(nv[q]) )
                  SCIP_CALL( SCIPchgVarLbProbing(scip, nv[q], nl[q]) );
               if( nu[q] < SCIPvarGetUbLocal(nv[q]) )
                  SCIP_CALL( SCIPchgVarUbProbing(scip, nv[q], nu[q]) );
            }
         }
         if( !pcut )
            SCIP_CALL( SCIPpropagateProbing(scip, -1, &pcut, NULL) );
         ncutb += cut[k] ? 1 : 0;
         ncutp += pcut ? 1 : 0;
         if( (pcut != 0) != (cut[k] != 0) )
            cutmis++;
         else if( !pcut )
         {
            /* the batched bounds: the root's local bounds (outside probing), moved by the node's outputs */
            for( j = 0; j < nvars; ++j )
            {
               elb[j] = rlb[j];
               eub[j] = rub[j];
            }
            for( q = obeg[k]; q < obeg[k + 1]; ++q )
            {
               j = SCIPvarGetProbindex(ov[q]);
               elb[j] = ol[q];
               eub[j] = ou[q];
            }
            for( j = 0; j < nvars; ++j )
               if( SCIPvarGetType(vars[j]) != SCIP_VARTYPE_CONTINUOUS
                  && (elb[j] != SCIPvarGetLbLocal(vars[j]) || eub[j] != SCIPvarGetUbLocal(vars[j])) )
               {
                  intmis++;
                  break;
               }
            for( j = 0; j < nvars; ++j )
            {
               SCIP_Real sl = SCIPvarGetLbLocal(vars[j]);
               SCIP_Real su = SCIPvarGetUbLocal(vars[j]);
               if( SCIPvarGetType(vars[j]) == SCIP_VARTYPE_CONTINUOUS
                  && (REALABS(elb[j] - sl) > MAX(1e-9 * REALABS(sl), 1e-6)
                     || REALABS(eub[j] - su) > MAX(1e-9 * REALABS(su), 1e-6)) )
               {
                  int last = k - 1;  /* the last cut-off node before this one */
                  while( last >= 0 && !cut[last] )
                     --last;
                  fprintf(stderr, "node %d column %d: batched [%.17g, %.17g] probing [%.17g, %.17g] base [%.17g, "
                     "%.17g]; last cut-off node before it: %d\n", k, j, elb[j], eub[j], sl, su, rlb[j], rub[j], last);
                  contmis++;
                  break;
               }
            }
         }
         SCIP_CALL( SCIPbacktrackProbing(scip, 0) );
      }
      SCIP_CALL( SCIPendProbing(scip) );
      SCIPfreeBufferArray(scip, &rub);
      SCIPfreeBufferArray(scip, &rlb);
      SCIPfreeBufferArray(scip, &eub);
      SCIPfreeBufferArray(scip, &elb);
   }
   printf("nodes %d success %d cutoffs %d %d cutoffmismatch %d intmismatch %d contmismatch %d moved %d\n", nwant,
      success ? 1 : 0, ncutb, ncutp, cutmis, intmis, contmis, success ? obeg[nwant] : -1);
   SCIPfreeBufferArray(scip, &ou);
   SCIPfreeBufferArray(scip, &ol);
   SCIPfreeBufferArray(scip, &ov);
   SCIPfreeBufferArray(scip, &obeg);
   SCIPfreeBufferArray(scip, &cut);
   SCIPfreeBufferArray(scip, &nu);
   SCIPfreeBufferArray(scip, &nl);
   SCIPfreeBufferArray(scip, &nv);
   SCIPfreeBufferArray(scip, &beg);
   SCIPfreeBufferArray(scip, &cand);
   SCIP_CALL( SCIPinterruptSolve(scip) );
   return SCIP_OKAY;
}

int main(int argc, char** argv)
{
   SCIP* scip = NULL;
   SCIP_HEUR* heur = NULL;
   SCIP_PARAM** params;
   int np;
   int k;
   if( argc < 2 )
      return 2;
   if( argc > 2 )
      nwant = atoi(argv[2]);
   if( argc > 3 && strcmp(argv[3], "sciporder") == 0 )
      sciporder = 1;
   if( argc > 4 && strcmp(argv[4], "easy") == 0 )
      easyrule = 1;
   if( argc > 5 && strstr(argv[5], "ranged") != NULL )
      ranged = 1;
   if( argc > 5 && strstr(argv[5], "nosort") != NULL )
      nosort = 1;
   if( argc > 6 )
      atdepth = atoi(argv[6]);
   if( argc > 7 && strcmp(argv[7], "presolve") == 0 )
      presolve = 1;
   if( SCIPcreate(&scip) != SCIP_OKAY || SCIPincludeDefaultPlugins(scip) != SCIP_OKAY )
      return 1;
   if( SCIPincludePropGpulinear(scip) != SCIP_OKAY )
      return 1;
   SCIPsetBoolParam(scip, "propagating/gpulinear/probing", FALSE);
   SCIPsetBoolParam(scip, "propagating/gpulinear/sciporder", sciporder ? TRUE : FALSE);
   if( SCIPincludeHeurBasic(scip, &heur, "nodecheck", "batched-node check", 'c', 1000000, 1, 0, -1,
         SCIP_HEURTIMING_BEFORENODE, FALSE, heurExecCheck, NULL) != SCIP_OKAY )
      return 1;
   if( SCIPreadProb(scip, argv[1], NULL) != SCIP_OKAY )
      return 3;
   params = SCIPgetParams(scip);
   np = SCIPgetNParams(scip);
   for( k = 0; k < np; ++k )
   {
      const char* name = SCIPparamGetName(params[k]);
      size_t len = strlen(name);
      if( strncmp(name, "constraints/linear/upgrade/", 27) == 0 )
         SCIPsetBoolParam(scip, name, FALSE);
      /* probing propagates with cons_linear alone: every other propagator off */
      if( strncmp(name, "propagating/", 12) == 0 && len > 5 && strcmp(name + len - 5, "/freq") == 0
         && strcmp(name, "propagating/gpulinear/freq") != 0 )
         SCIPsetIntParam(scip, name, -1);
   }
   /* with "presolve": SCIP's presolving runs (aggregations, fixings, negated variables in rows), the rows stay
    * linear (no upgrade) */
   SCIPsetIntParam(scip, "presolving/maxrounds", presolve ? -1 : 0);
   SCIPsetBoolParam(scip, "constraints/linear/rangedrowpropagation", ranged ? TRUE : FALSE);
   SCIPsetBoolParam(scip, "constraints/linear/sortvars", nosort ? FALSE : TRUE);
   SCIPsetBoolParam(scip, "constraints/linear/rangedrowartcons", FALSE);
   SCIPsetIntParam(scip, "lp/solvefreq", -1);
   SCIPsetRealParam(scip, "constraints/linear/maxeasyactivitydelta", easyrule ? 1e6 : 0.0);
   /* an infeasible probing node must not tighten the root's bounds for the nodes after it (conflict analysis of
    * a cutoff can fix a variable globally) */
   SCIPsetBoolParam(scip, "conflict/enable", FALSE);
   SCIPsetIntParam(scip, "display/verblevel", 0);
   if( SCIPsolve(scip) != SCIP_OKAY )
      return 4;
   SCIPfree(&scip);
   return 0;
}
