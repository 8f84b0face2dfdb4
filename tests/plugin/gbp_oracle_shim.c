/* Test double of libgbp for the plugin's SCIP-side tests: the C-ABI calls the propagator plugin makes, answered by
 * the oracle (oracle/linprop_oracle.c) on the host.  It exists so that SCIP (which builds only where its sources
 * are) can run the plugin end to end -- write-back of the change log and conflict resolution -- without a GPU.  It
 * is linked only into the SCIP-side test drivers (tests/plugin/*_driver.c); the product library libgbp has no host
 * path. */
#include <stdlib.h>
#include <string.h>

#include "gbp.h"
#include "linprop_oracle.h"

struct gbp_ctx
{
   lpo_problem P;
   int64_t* rowptr;
   int32_t* colidx;
   double* vals;
   double* lhs;
   double* rhs;
   int8_t* isint;
   int64_t* colptr;
   int32_t* rowidx;
   double* cvals;
   lpo_params par;
   double* glb;
   double* gub;
   int has_global;
   lpo_log log;
   int logon;
   double* dlb;   /* bounds kept between sparse calls (gbp_set_bounds / gbp_propagate_changes) */
   double* dub;
   int bset;
   int sciporder;  /* GBP_FLAG_SCIPORDER: batched nodes through the restatement of SCIP's order */
   int64_t ninst;  /* gbp_upload_instance_list: the parts' offsets into the block-diagonal problem */
   int64_t* row_off;
   int64_t* col_off;
};

int gbp_version(void) { return 0; }

const char* gbp_error_string(int code) { return code == GBP_OK ? "ok" : "error (oracle test double)"; }

const char* gbp_last_error(const gbp_ctx* ctx) { (void)ctx; return "oracle test double"; }

void gbp_default_params(gbp_params* p)
{
   p->infinity = 1e20;
   p->epsilon = 1e-9;
   p->sumepsilon = 1e-6;
   p->feastol = 1e-6;
   p->hugeval = 1e15;
   p->boundstreps = 0.05;
   p->recompfac = 1e6;
   p->maxeasyactivitydelta = 1e6;
   p->maxrounds = 0;
   p->flags = 0;
}

int gbp_create(gbp_ctx** ctx, int device, void* stream)
{
   (void)device;
   (void)stream;
   *ctx = calloc(1, sizeof(gbp_ctx));
   if( *ctx == NULL )
      return GBP_ERR_NOMEM;
   lpo_default_params(&(*ctx)->par);
   return GBP_OK;
}

static void freeProblem(gbp_ctx* c)
{
   free(c->rowptr); free(c->colidx); free(c->vals); free(c->lhs); free(c->rhs); free(c->isint);
   free(c->colptr); free(c->rowidx); free(c->cvals); free(c->glb); free(c->gub);
   c->rowptr = NULL; c->colidx = NULL; c->vals = NULL; c->lhs = NULL; c->rhs = NULL; c->isint = NULL;
   c->colptr = NULL; c->rowidx = NULL; c->cvals = NULL; c->glb = NULL; c->gub = NULL;
   c->has_global = 0;
   free(c->dlb); free(c->dub);
   c->dlb = NULL; c->dub = NULL; c->bset = 0;
   free(c->row_off); free(c->col_off);
   c->row_off = NULL; c->col_off = NULL; c->ninst = 0;
}

int gbp_destroy(gbp_ctx* ctx)
{
   if( ctx == NULL )
      return GBP_ERR_INVALID;
   freeProblem(ctx);
   free(ctx->log.col); free(ctx->log.round); free(ctx->log.lb); free(ctx->log.ub);
   free(ctx->log.rrow); free(ctx->log.rcol); free(ctx->log.rround);
   free(ctx);
   return GBP_OK;
}

int gbp_set_params(gbp_ctx* ctx, const gbp_params* p)
{
   ctx->par.infinity = p->infinity;
   ctx->par.epsilon = p->epsilon;
   ctx->par.sumepsilon = p->sumepsilon;
   ctx->par.feastol = p->feastol;
   ctx->par.hugeval = p->hugeval;
   ctx->par.boundstreps = p->boundstreps;
   ctx->par.recompfac = p->recompfac;
   ctx->par.maxeasyactivitydelta = p->maxeasyactivitydelta;
   ctx->par.maxrounds = p->maxrounds;
   ctx->par.flags = ((p->flags & GBP_FLAG_NOSORTVARS) ? LPO_FLAG_NOSORTVARS : 0)
      | ((p->flags & GBP_FLAG_RANGEDROW) ? LPO_FLAG_RANGEDROW : 0);
   if( (p->flags & GBP_FLAG_SCIPORDER) && (p->flags & GBP_FLAG_RANGEDROW) )
      return GBP_ERR_INVALID;
   ctx->sciporder = (p->flags & GBP_FLAG_SCIPORDER) != 0;
   return GBP_OK;
}

#define DUP(dst, src, cnt, T) do { dst = malloc(sizeof(T) * (size_t)((cnt) > 0 ? (cnt) : 1)); \
      if( (cnt) > 0 ) memcpy(dst, src, sizeof(T) * (size_t)(cnt)); } while( 0 )

int gbp_upload_problem(gbp_ctx* ctx, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
   const double* vals, const double* lhs, const double* rhs, const int8_t* isint)
{
   int64_t nnz = rowptr[m];
   int64_t i;
   int64_t p;
   int64_t* fill;
   freeProblem(ctx);
   DUP(ctx->rowptr, rowptr, m + 1, int64_t);
   DUP(ctx->colidx, colidx, nnz, int32_t);
   DUP(ctx->vals, vals, nnz, double);
   DUP(ctx->lhs, lhs, m, double);
   DUP(ctx->rhs, rhs, m, double);
   DUP(ctx->isint, isint, n, int8_t);
   ctx->colptr = calloc((size_t)n + 1, sizeof(int64_t));
   ctx->rowidx = malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
   ctx->cvals = malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
   fill = malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
   for( p = 0; p < nnz; ++p )
      ctx->colptr[colidx[p] + 1]++;
   for( i = 0; i < n; ++i )
      ctx->colptr[i + 1] += ctx->colptr[i];
   for( i = 0; i < n; ++i )
      fill[i] = ctx->colptr[i];
   for( i = 0; i < m; ++i )
      for( p = rowptr[i]; p < rowptr[i + 1]; ++p )
      {
         int64_t q = fill[colidx[p]]++;
         ctx->rowidx[q] = (int32_t)i;
         ctx->cvals[q] = vals[p];
      }
   free(fill);
   ctx->P.m = m; ctx->P.n = n; ctx->P.rowptr = ctx->rowptr; ctx->P.colidx = ctx->colidx; ctx->P.vals = ctx->vals;
   ctx->P.lhs = ctx->lhs; ctx->P.rhs = ctx->rhs; ctx->P.isint = ctx->isint; ctx->P.colptr = ctx->colptr;
   ctx->P.rowidx = ctx->rowidx; ctx->P.cvals = ctx->cvals;
   return GBP_OK;
}

int gbp_set_global_bounds(gbp_ctx* ctx, const double* glb, const double* gub)
{
   free(ctx->glb);
   free(ctx->gub);
   ctx->glb = NULL;
   ctx->gub = NULL;
   ctx->has_global = 0;
   if( glb == NULL )
      return GBP_OK;
   DUP(ctx->glb, glb, ctx->P.n, double);
   DUP(ctx->gub, gub, ctx->P.n, double);
   ctx->has_global = 1;
   return GBP_OK;
}

int gbp_set_change_log(gbp_ctx* ctx, int64_t capacity)
{
   free(ctx->log.col); free(ctx->log.round); free(ctx->log.lb); free(ctx->log.ub);
   free(ctx->log.rrow); free(ctx->log.rcol); free(ctx->log.rround);
   memset(&ctx->log, 0, sizeof(ctx->log));
   ctx->logon = capacity > 0;
   if( !ctx->logon )
      return GBP_OK;
   ctx->log.cap = capacity;
   ctx->log.col = malloc(sizeof(int32_t) * (size_t)capacity);
   ctx->log.round = malloc(sizeof(int32_t) * (size_t)capacity);
   ctx->log.lb = malloc(sizeof(double) * (size_t)capacity);
   ctx->log.ub = malloc(sizeof(double) * (size_t)capacity);
   ctx->log.rcap = capacity;
   ctx->log.rrow = malloc(sizeof(int32_t) * (size_t)capacity);
   ctx->log.rcol = malloc(sizeof(int32_t) * (size_t)capacity);
   ctx->log.rround = malloc(sizeof(int32_t) * (size_t)capacity);
   return GBP_OK;
}

int gbp_propagate(gbp_ctx* ctx, double* lb, double* ub, int64_t nseed, const int32_t* seedcols,
   const double* oldlb, const double* oldub, int32_t* cutoff, gbp_result* res)
{
   lpo_result r;
   ctx->log.n = 0;
   *cutoff = 0;
   if( res != NULL )
      memset(res, 0, sizeof(*res));
   if( nseed == 0 )
      return GBP_OK;
   if( lpo_propagate_logged(&ctx->P, &ctx->par, lb, ub, nseed < 0 ? 0 : nseed, nseed < 0 ? NULL : seedcols, oldlb,
         oldub, ctx->has_global ? ctx->glb : NULL, ctx->has_global ? ctx->gub : NULL, &r,
         ctx->logon ? &ctx->log : NULL) != 0 )
      return GBP_ERR_NOMEM;
   *cutoff = r.cutoff;
   if( res != NULL )
   {
      res->cutoff = r.cutoff;
      res->rounds = r.rounds;
      res->status = r.status;
      res->rows = r.rows;
      res->nnz = r.nnz;
      res->candidates = r.candidates;
      res->changes = r.changes;
   }
   return r.status == 2 ? GBP_ERR_LIMIT : GBP_OK;
}

int gbp_set_bounds(gbp_ctx* ctx, const double* lb, const double* ub)
{
   size_t nb = sizeof(double) * (size_t)(ctx->P.n > 0 ? ctx->P.n : 1);
   if( ctx->dlb == NULL )
   {
      ctx->dlb = malloc(nb);
      ctx->dub = malloc(nb);
      if( ctx->dlb == NULL || ctx->dub == NULL )
         return GBP_ERR_NOMEM;
   }
   if( ctx->P.n > 0 )
   {
      memcpy(ctx->dlb, lb, sizeof(double) * (size_t)ctx->P.n);
      memcpy(ctx->dub, ub, sizeof(double) * (size_t)ctx->P.n);
   }
   ctx->bset = 1;
   return GBP_OK;
}

/* the sparse call as include/gbp.h states it: changes applied to the kept bounds, propagation from them, the
 * columns it moved returned by column; the kept bounds are left after the changes on a cutoff or an overflow */
int gbp_propagate_changes(gbp_ctx* ctx, int64_t nchg, const int32_t* cols, const double* newlb, const double* newub,
   const double* seedlb, const double* seedub, int64_t cap, int64_t* nout, int32_t* outcols, double* outlb,
   double* outub, int32_t* cutoff, gbp_result* res)
{
   int64_t n = ctx->P.n;
   int64_t k;
   int64_t j;
   int64_t cnt = 0;
   double* lb;
   double* ub;
   double* olb;
   double* oub;
   int rc;
   if( !ctx->bset )
      return GBP_ERR_INVALID;
   *nout = 0;
   *cutoff = 0;
   for( k = 0; k < nchg; ++k )
   {
      if( cols[k] < 0 || cols[k] >= n )
         return GBP_ERR_INVALID;
      if( newlb[k] > newub[k] )
      {
         *cutoff = 1;
         if( res != NULL )
         {
            memset(res, 0, sizeof(*res));
            res->cutoff = 1;
            res->status = 1;
         }
         return GBP_OK;
      }
   }
   olb = malloc(sizeof(double) * (size_t)(nchg > 0 ? nchg : 1));
   oub = malloc(sizeof(double) * (size_t)(nchg > 0 ? nchg : 1));
   lb = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
   ub = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
   if( olb == NULL || oub == NULL || lb == NULL || ub == NULL )
   {
      free(olb); free(oub); free(lb); free(ub);
      return GBP_ERR_NOMEM;
   }
   for( k = 0; k < nchg; ++k )
   {
      olb[k] = seedlb != NULL ? seedlb[k] : ctx->dlb[cols[k]];
      oub[k] = seedub != NULL ? seedub[k] : ctx->dub[cols[k]];
      ctx->dlb[cols[k]] = newlb[k];
      ctx->dub[cols[k]] = newub[k];
   }
   if( n > 0 )
   {
      memcpy(lb, ctx->dlb, sizeof(double) * (size_t)n);
      memcpy(ub, ctx->dub, sizeof(double) * (size_t)n);
   }
   rc = gbp_propagate(ctx, lb, ub, nchg, cols, olb, oub, cutoff, res);
   if( (rc == GBP_OK || rc == GBP_ERR_LIMIT) && !*cutoff )
   {
      for( j = 0; j < n; ++j )
         cnt += (lb[j] != ctx->dlb[j] || ub[j] != ctx->dub[j]) ? 1 : 0;
      *nout = cnt;
      if( cnt > cap )
         rc = GBP_ERR_OVERFLOW;
      else
      {
         cnt = 0;
         for( j = 0; j < n; ++j )
         {
            if( lb[j] != ctx->dlb[j] || ub[j] != ctx->dub[j] )
            {
               outcols[cnt] = (int32_t)j;
               outlb[cnt] = lb[j];
               outub[cnt] = ub[j];
               ++cnt;
            }
         }
         memcpy(ctx->dlb, lb, sizeof(double) * (size_t)n);
         memcpy(ctx->dub, ub, sizeof(double) * (size_t)n);
      }
   }
   free(olb); free(oub); free(lb); free(ub);
   return rc;
}

static const lpo_log* sortlog;
static int byRoundCol(const void* a, const void* b)
{
   int64_t x = *(const int64_t*)a;
   int64_t y = *(const int64_t*)b;
   if( sortlog->round[x] != sortlog->round[y] )
      return sortlog->round[x] < sortlog->round[y] ? -1 : 1;
   return sortlog->col[x] < sortlog->col[y] ? -1 : (sortlog->col[x] > sortlog->col[y] ? 1 : 0);
}

int gbp_get_change_log(gbp_ctx* ctx, int64_t cap, int32_t* col, int32_t* round, double* lb, double* ub, int64_t* n)
{
   int64_t have;
   int64_t k;
   int64_t* ord;
   *n = ctx->log.n;
   if( !ctx->logon )
      return GBP_ERR_STATE;
   have = ctx->log.n < ctx->log.cap ? ctx->log.n : ctx->log.cap;
   ord = malloc(sizeof(int64_t) * (size_t)(have > 0 ? have : 1));
   for( k = 0; k < have; ++k )
      ord[k] = k;
   sortlog = &ctx->log;
   qsort(ord, (size_t)have, sizeof(int64_t), byRoundCol);
   for( k = 0; k < have && k < cap; ++k )
   {
      col[k] = ctx->log.col[ord[k]];
      round[k] = ctx->log.round[ord[k]];
      lb[k] = ctx->log.lb[ord[k]];
      ub[k] = ctx->log.ub[ord[k]];
   }
   free(ord);
   return (ctx->log.n > ctx->log.cap || ctx->log.n > cap) ? GBP_ERR_OVERFLOW : GBP_OK;
}

static int byRoundColRow(const void* a, const void* b)
{
   int64_t x = *(const int64_t*)a;
   int64_t y = *(const int64_t*)b;
   if( sortlog->rround[x] != sortlog->rround[y] )
      return sortlog->rround[x] < sortlog->rround[y] ? -1 : 1;
   if( sortlog->rcol[x] != sortlog->rcol[y] )
      return sortlog->rcol[x] < sortlog->rcol[y] ? -1 : 1;
   return sortlog->rrow[x] < sortlog->rrow[y] ? -1 : (sortlog->rrow[x] > sortlog->rrow[y] ? 1 : 0);
}

int gbp_get_ranged_log(gbp_ctx* ctx, int64_t cap, int32_t* round, int32_t* col, int32_t* row, int64_t* n)
{
   int64_t have;
   int64_t k;
   int64_t* ord;
   *n = ctx->log.rn;
   if( !ctx->logon )
      return GBP_ERR_STATE;
   have = ctx->log.rn < ctx->log.rcap ? ctx->log.rn : ctx->log.rcap;
   ord = malloc(sizeof(int64_t) * (size_t)(have > 0 ? have : 1));
   for( k = 0; k < have; ++k )
      ord[k] = k;
   sortlog = &ctx->log;
   qsort(ord, (size_t)have, sizeof(int64_t), byRoundColRow);
   for( k = 0; k < have && k < cap; ++k )
   {
      round[k] = ctx->log.rround[ord[k]];
      col[k] = ctx->log.rcol[ord[k]];
      row[k] = ctx->log.rrow[ord[k]];
   }
   free(ord);
   return (ctx->log.rn > ctx->log.rcap || ctx->log.rn > cap) ? GBP_ERR_OVERFLOW : GBP_OK;
}

/* the batched-node call: the oracle's nodes (binary test on the base bounds), packed in node order */
int gbp_propagate_nodes(gbp_ctx* ctx, const double* baselb, const double* baseub, int64_t nnodes,
   const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
   int8_t* out_cutoff, int32_t* out_rounds, int64_t* out_off, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int64_t out_cap, gbp_result* res)
{
   const int64_t n = ctx->P.n > 0 ? ctx->P.n : 1;
   int32_t* tn = malloc(sizeof(int32_t) * (size_t)(nnodes > 0 ? nnodes : 1));
   int32_t* tc = malloc(sizeof(int32_t) * (size_t)(nnodes * n + 1));
   double* tl = malloc(sizeof(double) * (size_t)(nnodes * n + 1));
   double* tu = malloc(sizeof(double) * (size_t)(nnodes * n + 1));
   lpo_result tot;
   int64_t at = 0;
   int64_t k;
   int over = 0;
   int rc;
   if( res != NULL )
      memset(res, 0, sizeof(*res));
   if( tn == NULL || tc == NULL || tl == NULL || tu == NULL )
      rc = GBP_ERR_NOMEM;
   else if( (ctx->sciporder ? lpo_propagate_nodes_seq : lpo_propagate_nodes)(&ctx->P, &ctx->par, baselb, baseub, nnodes,
               ptr, chg_col, chg_lb, chg_ub, out_cutoff, out_rounds, tn, tc, tl, tu, (int32_t)n, 1, &tot) != 0 )
      rc = GBP_ERR_NOMEM;
   else
   {
      for( k = 0; k < nnodes; ++k )
      {
         int64_t t;
         out_off[k] = at;
         if( at + tn[k] > out_cap )
         {
            out_n[k] = -1;
            over = 1;
            continue;
         }
         for( t = 0; t < tn[k]; ++t, ++at )
         {
            out_col[at] = tc[k * n + t];
            out_lb[at] = tl[k * n + t];
            out_ub[at] = tu[k * n + t];
         }
         out_n[k] = tn[k];
      }
      if( res != NULL )
      {
         res->cutoff = tot.cutoff;
         res->rounds = tot.rounds;
         res->rows = tot.rows;
         res->nnz = tot.nnz;
         res->candidates = tot.candidates;
         res->changes = tot.changes;
      }
      rc = over ? GBP_ERR_OVERFLOW : GBP_OK;
   }
   free(tn);
   free(tc);
   free(tl);
   free(tu);
   return rc;
}

/* the instances as parts of one block-diagonal problem; the checks of the library: row pointers from 0 and not
 * decreasing, every column index inside its part */
int gbp_upload_instance_list(gbp_ctx* ctx, int64_t ninst, const int64_t* m_k, const int64_t* n_k,
   const int64_t* const* rowptr_k, const int32_t* const* colidx_k, const double* const* vals_k,
   const double* const* lhs_k, const double* const* rhs_k, const int8_t* const* isint_k)
{
   int64_t m = 0, n = 0, nnz = 0;
   int64_t k;
   int64_t* rowptr;
   int32_t* colidx;
   double* vals;
   double* lhs;
   double* rhs;
   int8_t* isint;
   int rc;
   if( ctx == NULL || ninst < 1 || m_k == NULL || n_k == NULL || rowptr_k == NULL )
      return GBP_ERR_INVALID;
   for( k = 0; k < ninst; ++k )
   {
      int64_t i;
      const int64_t* rp = rowptr_k[k];
      if( m_k[k] < 0 || n_k[k] < 0 || rp == NULL || rp[0] != 0 )
         return GBP_ERR_INVALID;
      for( i = 0; i < m_k[k]; ++i )
         if( rp[i + 1] < rp[i] )
            return GBP_ERR_INVALID;
      for( i = 0; i < rp[m_k[k]]; ++i )
         if( colidx_k[k][i] < 0 || colidx_k[k][i] >= n_k[k] )
            return GBP_ERR_INVALID;
      m += m_k[k];
      n += n_k[k];
      nnz += rp[m_k[k]];
   }
   rowptr = malloc(sizeof(int64_t) * (size_t)(m + 1));
   colidx = malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
   vals = malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
   lhs = malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
   rhs = malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
   isint = malloc((size_t)(n > 0 ? n : 1));
   {
      int64_t r = 0, c = 0, z = 0;
      rowptr[0] = 0;
      for( k = 0; k < ninst; ++k )
      {
         int64_t i;
         const int64_t* rp = rowptr_k[k];
         for( i = 0; i < m_k[k]; ++i )
         {
            rowptr[r + i + 1] = z + rp[i + 1];
            lhs[r + i] = lhs_k[k][i];
            rhs[r + i] = rhs_k[k][i];
         }
         for( i = 0; i < rp[m_k[k]]; ++i )
         {
            colidx[z + i] = (int32_t)(colidx_k[k][i] + c);
            vals[z + i] = vals_k[k][i];
         }
         if( n_k[k] > 0 )
            memcpy(isint + c, isint_k[k], (size_t)n_k[k]);
         r += m_k[k];
         c += n_k[k];
         z += rp[m_k[k]];
      }
   }
   rc = gbp_upload_problem(ctx, m, n, rowptr, colidx, vals, lhs, rhs, isint);
   free(rowptr); free(colidx); free(vals); free(lhs); free(rhs); free(isint);
   if( rc != GBP_OK )
      return rc;
   ctx->ninst = ninst;
   ctx->row_off = malloc(sizeof(int64_t) * (size_t)(ninst + 1));
   ctx->col_off = malloc(sizeof(int64_t) * (size_t)(ninst + 1));
   ctx->row_off[0] = ctx->col_off[0] = 0;
   for( k = 0; k < ninst; ++k )
   {
      ctx->row_off[k + 1] = ctx->row_off[k] + m_k[k];
      ctx->col_off[k + 1] = ctx->col_off[k] + n_k[k];
   }
   return GBP_OK;
}

/* every part to its own root fixpoint (the oracle on the part alone), a cutoff flag per part */
int gbp_propagate_instances(gbp_ctx* ctx, double* lb, double* ub, int8_t* inst_cutoff, gbp_result* res)
{
   int64_t k;
   int32_t ncut = 0;
   if( ctx == NULL || ctx->ninst < 1 || lb == NULL || ub == NULL )
      return GBP_ERR_INVALID;
   if( res != NULL )
      memset(res, 0, sizeof(*res));
   for( k = 0; k < ctx->ninst; ++k )
   {
      const int64_t r0 = ctx->row_off[k], c0 = ctx->col_off[k];
      lpo_problem part = ctx->P;
      lpo_result r;
      int64_t* rp = malloc(sizeof(int64_t) * (size_t)(ctx->row_off[k + 1] - r0 + 1));
      int32_t* ci;
      int64_t i;
      const int64_t z0 = ctx->rowptr[r0];
      const int64_t nz = ctx->rowptr[ctx->row_off[k + 1]] - z0;
      ci = malloc(sizeof(int32_t) * (size_t)(nz > 0 ? nz : 1));
      for( i = 0; i <= ctx->row_off[k + 1] - r0; ++i )
         rp[i] = ctx->rowptr[r0 + i] - z0;
      for( i = 0; i < nz; ++i )
         ci[i] = (int32_t)(ctx->colidx[z0 + i] - c0);
      part.m = ctx->row_off[k + 1] - r0;
      part.n = ctx->col_off[k + 1] - c0;
      part.rowptr = rp;
      part.colidx = ci;
      part.vals = ctx->vals + z0;
      part.lhs = ctx->lhs + r0;
      part.rhs = ctx->rhs + r0;
      part.isint = ctx->isint + c0;
      part.colptr = NULL;  /* built below: the column view of the part */
      {
         int64_t* cp = calloc((size_t)part.n + 1, sizeof(int64_t));
         int32_t* ri = malloc(sizeof(int32_t) * (size_t)(nz > 0 ? nz : 1));
         double* cv = malloc(sizeof(double) * (size_t)(nz > 0 ? nz : 1));
         int64_t* fill = malloc(sizeof(int64_t) * (size_t)(part.n > 0 ? part.n : 1));
         int64_t p;
         for( p = 0; p < nz; ++p )
            cp[ci[p] + 1]++;
         for( i = 0; i < part.n; ++i )
            cp[i + 1] += cp[i];
         for( i = 0; i < part.n; ++i )
            fill[i] = cp[i];
         for( i = 0; i < part.m; ++i )
            for( p = rp[i]; p < rp[i + 1]; ++p )
            {
               int64_t q = fill[ci[p]]++;
               ri[q] = (int32_t)i;
               cv[q] = part.vals[p];
            }
         part.colptr = cp;
         part.rowidx = ri;
         part.cvals = cv;
         memset(&r, 0, sizeof(r));
         lpo_propagate(&part, &ctx->par, lb + c0, ub + c0, 0, NULL, NULL, NULL, NULL, NULL, &r);
         free(fill); free(cp); free(ri); free(cv);
      }
      free(rp);
      free(ci);
      inst_cutoff[k] = (int8_t)(r.cutoff != 0);
      ncut += inst_cutoff[k];
      if( res != NULL && r.rounds > res->rounds )
         res->rounds = r.rounds;
   }
   if( res != NULL )
      res->cutoff = ncut;
   return GBP_OK;
}

