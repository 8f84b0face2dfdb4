/* prop_gpulinear.h -- SCIP propagator that runs linear-constraint bound propagation on a GB300 GPU.
 *
 * Registered through SCIPincludePropBasic (src/scip/scip_prop.c:118-140) with a SCIP_DECL_PROPEXEC callback
 * (src/scip/type_prop.h:217).  At PROPINITSOL it copies every linear constraint of the transformed problem
 * (SCIPgetVarsLinear/SCIPgetValsLinear/SCIPgetLhsLinear/SCIPgetRhsLinear, src/scip/cons_linear.h:263-307) into
 * libgbp's device-resident CSR/CSC; each PROPEXEC hands the current local bounds and the columns that changed
 * since its last call to gbp_propagate (include/gbp.h), then writes the tightened bounds back with
 * SCIPtightenVarLb/SCIPtightenVarUb (src/scip/scip_var.c:6402/6652) or reports SCIP_CUTOFF.  The device runs
 * the propagation rules of cons_linear (tightenVarBounds / tightenVarBoundsEasy) to a fixpoint.
 *
 * Parameters (propagating/gpulinear/...): device (CUDA ordinal, default 0), replacelinear (default FALSE:
 * if TRUE, SCIPincludePropGpulinear sets constraints/linear/propfreq = -1 so that the GPU replaces
 * cons_linear's own propagation; cons_linear keeps checking, enforcing and presolving) and probing (default TRUE:
 * also propagate in probing nodes).
 * Without a usable GPU the propagator disables itself with a warning and SCIP continues with cons_linear.
 */
#ifndef PROP_GPULINEAR_H
#define PROP_GPULINEAR_H

#include "scip/scip.h"

#ifdef __cplusplus
extern "C" {
#endif

/** includes the GPU linear propagator in SCIP */
SCIP_RETCODE SCIPincludePropGpulinear(SCIP* scip);

/** the rows the propagator uploads (valid after PROPINITSOL, i.e. once solving has started): CSR arrays owned
 *  by the propagator; column j is SCIPgetVars(scip)[j].  Rows with a variable that is neither active nor
 *  fixed (aggregated, multi-aggregated) are left to cons_linear and are not part of the matrix. */
SCIP_RETCODE SCIPgetGpulinearMatrix(SCIP* scip, int* nrows, int* ncols, const int64_t** rowptr, const int32_t** colidx,
   const double** vals, const double** lhs, const double** rhs);

/** whether the propagator runs on a GPU (FALSE before PROPINITSOL or after it disabled itself) */
SCIP_Bool SCIPgpulinearIsActive(SCIP* scip);

/** counters of the propagator: calls, bounds it changed, cutoffs, cutoffs it handed to conflict analysis with an
 *  infeasible row, conflict-resolution requests for its changes and how many of them it explained with a row */
SCIP_RETCODE SCIPgetGpulinearStats(SCIP* scip, SCIP_Longint* ncalls, SCIP_Longint* nchgbds, SCIP_Longint* ncutoffs,
   SCIP_Longint* nconflicts, SCIP_Longint* nresolves, SCIP_Longint* nresolved);

/** how many of the explained changes and analysed cutoffs were explained by a ranged row's record
 *  (constraints/linear/rangedrowpropagation) */
SCIP_Longint SCIPgetGpulinearRangedReasons(SCIP* scip);

/** propagates nnodes nodes at once on the GPU (libgbp's batched path, gbp_propagate_nodes), each on top of the
 *  current local bounds -- for callers that hold many candidate nodes (probing, strong branching, a lookahead of open
 *  nodes).  Node k tightens the bounds of vars[nodebeg[k] .. nodebeg[k+1]) to [lbs, ubs] (active problem
 *  variables; SCIP_INVALIDDATA otherwise) and runs linear propagation to its fixpoint; SCIP's bounds are not
 *  changed.  Per node: cutoff[k], and the variables whose bounds propagation moved against the local bounds, with
 *  their bounds, at outvars/outlbs/outubs[outbeg[k] .. outbeg[k+1]) (outcap entries in all; a cut-off node has
 *  none).  *success is FALSE when the propagator is inactive (no GPU) or the outputs did not fit.
 *  With propagating/gpulinear/sciporder the nodes run in SCIP's own order (GBP_FLAG_SCIPORDER): the call reads the
 *  rows again in the order SCIP holds them and uploads them, and each node starts from the local bounds with no row
 *  marked, so that its cutoff verdict and integer bounds are the ones SCIP's own propagation of the node reaches
 *  (continuous bounds within 1e-9 relative or feastol absolute).  That mode needs a matrix of linear rows alone
 *  (no rows of setppc, logicor, knapsack or varbound constraints), and below the root no integer variable that is
 *  binary in its local domain only (the device takes a row's binaries under the local bounds, SCIP under the global
 *  ones); otherwise *success is FALSE.
 *  In both modes the nodes run without the ranged-row rule, as SCIP's probing does: a probing node keeps every
 *  row's rangedrowpropagated mark, so rows propagated at the base after their last change are not ranged-propagated
 *  again. */
SCIP_RETCODE SCIPpropagateGpulinearNodes(SCIP* scip, int nnodes, const int* nodebeg, SCIP_VAR** vars,
   const SCIP_Real* lbs, const SCIP_Real* ubs, int outcap, SCIP_Bool* cutoff, int* outbeg, SCIP_VAR** outvars,
   SCIP_Real* outlbs, SCIP_Real* outubs, SCIP_Bool* success);

#ifdef __cplusplus
}
#endif

#endif
