/* Test infrastructure only: CPU restatement of SCIP 11's cons_linear propagation in SCIP's own order -- marked rows
 * one at a time, every tightening applied at once, activities updated incrementally by bound-change events.  The
 * tests and bench.py's CPU legs use it as the checker of the CUDA sequential node kernel; the product library never
 * links it.  The semantics are described in linprop_oracle.h (lpo_propagate_seq / lpo_propagate_nodes_seq).
 *
 * Every step restates the SCIP function cited beside it (paths relative to the SCIP source tree):
 *   propagation rounds            propagateDomains / propagationRound, solve.c:723-795, 437-719
 *   marked rows                   SCIPconshdlrPropagate, cons.c:3905-4080; conshdlrMarkConsPropagate /
 *                                 conshdlrUnmarkConsPropagate, cons.c:623-760; delayed updates processed last-in
 *                                 first-out, conshdlrProcessUpdates, cons.c:1689-1860; SCIPconsMarkPropagate /
 *                                 SCIPconsUnmarkPropagate, cons.c:7309-7365
 *   one row                       consPropLinear, cons_linear.c:16126-16195; propagateCons, :7621-7758
 *   tightenBounds                 cons_linear.c:6976-7154 (MAXTIGHTENROUNDS, lastchange, the binary skip)
 *   residual rule                 tightenVarBounds, cons_linear.c:6700-6974
 *   slack rule                    tightenVarBoundsEasy / tightenVarUb / tightenVarLb, cons_linear.c:5242-5653
 *   acceptance                    SCIPinferVarUbCons / LbCons, scip_var.c:6965-7175; SCIPnodeAddBoundinfer,
 *                                 tree.c:1912-2215
 *   events                        eventExecLinear, cons_linear.c:17162-17363
 *   activities                    consdataCalcActivities :2283, consdataUpdateActivities :1604-1992,
 *                                 consdataRecomputeMin/Maxactivity :1307-1358, getMin/MaxActivity :2345-2529,
 *                                 consdataGetActivityResiduals :2661-2806, consdataGetReliableResidualActivity
 *                                 :2580-2657, consdataRecomputeMaxActivityDelta :1542-1599
 *   row order                     consdataSort / consdataCompVarProp, cons_linear.c:3191-3254, 3337-3400
 */
#define _POSIX_C_SOURCE 200809L
#include "lpo_common.h"

#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef LPO_SEQ_TRACE
#include <stdio.h>
#endif

#define SEQ_INVALID 1e99          /* SCIP_INVALID, def.h */
#define MAXTIGHTENROUNDS 10       /* cons_linear.c:6976 */

typedef struct
{
   Act a;                 /* QUAD min/max activity and the eight counters */
   double lastmin;
   double lastmax;
   double maxdelta;       /* maxactdelta, SEQ_INVALID when invalid */
   int32_t maxdeltacol;   /* column of maxactdeltavar, -1 for none */
   int32_t mpos;          /* position in the marked list */
   int32_t nbin;          /* leading binaries of the row's order (nbinvars) */
   int32_t stamp;
   uint8_t valid;         /* validactivities */
   uint8_t validmin;
   uint8_t validmax;
   uint8_t bt;            /* boundstightened */
   uint8_t mp;            /* markpropagate */
   uint8_t en;            /* enabled */
   uint8_t del;           /* deleted (globally, at the root) */
   uint8_t um, uu, ud;    /* delayed mark / unmark / disable */
   uint8_t inupd;
   uint8_t coefsorted;
   uint8_t nonbinvalid;
   uint8_t hasnonbin;
} RowSt;

typedef struct
{
   const lpo_problem* P;
   Num s;
   int root;              /* depth 0: global bound changes, tightenmode 2, redundant rows deleted globally */
   int sortvars;
   int32_t maxrounds;
   double* lb;
   double* ub;
   const double* glb;     /* global domain: the base bounds of a node, the current bounds at the root */
   const double* gub;
   RowSt* rs;
   int32_t stamp;
   int32_t* ord;          /* ord[rowptr[i] + k]: CSR position of the k-th entry of row i in its current order */
   int32_t* tmp;
   int32_t* M;            /* marked rows in propconss order */
   int64_t nm;
   int32_t* U;            /* rows with delayed updates, in the order they were added */
   int64_t nu;
   int indelay;           /* inside consPropLinear: mark, unmark and disable are delayed */
   int64_t nchg;          /* tightenings of the current consPropLinear call (nchgbds) */
   /* node bookkeeping: columns changed since the base bounds */
   uint8_t* dirty;
   int32_t* dirtylist;
   int64_t ndirty;
   const uint8_t* rowdel; /* nodes: rows deleted at the root (redundant under the base bounds) */
   const RowSt* rootst;   /* nodes: the root's final row states, whose activities a node starts from (or NULL) */
   lpo_result* res;
} Seq;

/* ------------------------------------------------------------------ row state */
static int isBinaryCol(const Seq* q, int32_t j)   /* SCIPvarIsBinary, var.c:23801-23810 */
{
   return q->P->isint[j] != 0 && q->glb[j] >= 0.0 && q->gub[j] <= 1.0;
}

static RowSt* rowSt(Seq* q, int32_t i)
{
   RowSt* r = &q->rs[i];
   if( r->stamp != q->stamp )
   {
      memset(r, 0, sizeof(*r));
      r->stamp = q->stamp;
      r->maxdelta = SEQ_INVALID;
      r->maxdeltacol = -1;
      r->en = 1;
      r->mpos = -1;
      /* a node starts from the root's fixpoint: every row counts as already tightened there (tightenmode 2), so a
       * node re-tightens a row only after a bound change that one of the row's finite sides can use */
      r->bt = q->root ? 0 : 2;
      if( q->rowdel != NULL && q->rowdel[i] )
      {
         r->del = 1;
         r->en = 0;
      }
      if( q->rootst != NULL )
      {
         /* SCIP keeps a row's activities across the root and into a node: the node starts from the values the
          * root's incremental updates left (with their reliability references and the largest activity delta)
          * instead of recomputing them on first use */
         const RowSt* o = &q->rootst[i];
         r->a = o->a;
         r->lastmin = o->lastmin;
         r->lastmax = o->lastmax;
         r->maxdelta = o->maxdelta;
         r->maxdeltacol = o->maxdeltacol;
         r->valid = o->valid;
         r->validmin = o->validmin;
         r->validmax = o->validmax;
      }
      if( !q->root && q->sortvars )
      {
         /* rows are stored in SCIP's propagation order: binaries first */
         const lpo_problem* P = q->P;
         int64_t p0 = P->rowptr[i];
         int64_t len = P->rowptr[i + 1] - p0;
         int64_t k = 0;
         while( k < len && isBinaryCol(q, P->colidx[p0 + k]) )
            ++k;
         r->nbin = (int32_t)k;
         r->coefsorted = 1;
      }
   }
   return r;
}

static inline int64_t ordPos(const Seq* q, int32_t i, int64_t k)
{
   return q->ord[q->P->rowptr[i] + k];
}

/* consdataSort with consdataCompVarProp (cons_linear.c:3191-3254, 3337-3400) on the global domain: binaries first by
 * decreasing |a|, then integers by decreasing |a|*(ub-lb), then continuous columns; ties by SCIP's problem index
 * (lpo_problem.varidx).  Keys are compared exactly (SCIP treats values within 1e-9 as ties). */
static inline int32_t varIdx(const lpo_problem* P, int32_t j)
{
   return P->varidx != NULL ? P->varidx[j] : j;
}

static int propBefore(const Seq* q, int64_t p, int64_t r)
{
   const lpo_problem* P = q->P;
   int32_t jp = P->colidx[p];
   int32_t jr = P->colidx[r];
   int bp = isBinaryCol(q, jp);
   int br = isBinaryCol(q, jr);
   double kp;
   double kr;
   if( bp != br )
      return bp;
   if( bp )
   {
      kp = fabs(P->vals[p]);
      kr = fabs(P->vals[r]);
   }
   else
   {
      if( (P->isint[jp] != 0) != (P->isint[jr] != 0) )
         return P->isint[jp] != 0;
      if( P->isint[jp] == 0 )
         return varIdx(P, jp) < varIdx(P, jr);
      kp = fabs(P->vals[p] * (q->gub[jp] - q->glb[jp]));
      kr = fabs(P->vals[r] * (q->gub[jr] - q->glb[jr]));
   }
   if( kp != kr )
      return kp > kr;
   return varIdx(P, jp) < varIdx(P, jr);
}

static void sortRow(Seq* q, int32_t i, RowSt* r)
{
   const lpo_problem* P = q->P;
   int64_t p0 = P->rowptr[i];
   int64_t n = P->rowptr[i + 1] - p0;
   int32_t* a = q->ord + p0;
   int64_t w;
   int64_t k;
   /* bottom-up merge sort (stable, so equal keys could never reorder; the comparison is a total order anyway) */
   for( w = 1; w < n; w *= 2 )
   {
      for( k = 0; k < n; k += 2 * w )
      {
         int64_t m = k + w < n ? k + w : n;
         int64_t e = k + 2 * w < n ? k + 2 * w : n;
         int64_t x = k;
         int64_t y = m;
         int64_t t = k;
         while( t < e )
         {
            if( y >= e || (x < m && !propBefore(q, a[y], a[x])) )
               q->tmp[t++] = a[x++];
            else
               q->tmp[t++] = a[y++];
         }
      }
      memcpy(a, q->tmp, sizeof(int32_t) * (size_t)n);
   }
   r->coefsorted = 1;
   for( k = 0; k < n && isBinaryCol(q, P->colidx[a[k]]); ++k )
      ;
   r->nbin = (int32_t)k;
}

/* consdataCalcActivities (cons_linear.c:2283-2339): every entry in the row's current order through
 * consdataUpdateAddCoef, i.e. the counters or the compensated sum */
static void calcActivities(Seq* q, int32_t i, RowSt* r)
{
   const lpo_problem* P = q->P;
   int64_t len = P->rowptr[i + 1] - P->rowptr[i];
   int64_t k;
   memset(&r->a, 0, sizeof(r->a));
   for( k = 0; k < len; ++k )
   {
      int64_t p = ordPos(q, i, k);
      int32_t j = P->colidx[p];
      addTerm(&q->s, &r->a, P->vals[p], q->lb[j], q->ub[j]);
   }
   r->valid = r->validmin = r->validmax = 1;
   r->lastmin = r->a.minhi + r->a.minlo;
   r->lastmax = r->a.maxhi + r->a.maxlo;
}

/* consdataRecomputeMinactivity / Maxactivity (cons_linear.c:1307-1358): finite non-huge part, last entry first */
static void recomputeSide(Seq* q, int32_t i, RowSt* r, int ismin)
{
   const lpo_problem* P = q->P;
   int64_t len = P->rowptr[i + 1] - P->rowptr[i];
   int64_t k;
   double hi = 0.0;
   double lo = 0.0;
   for( k = len - 1; k >= 0; --k )
   {
      int64_t p = ordPos(q, i, k);
      int32_t j = P->colidx[p];
      double v = P->vals[p];
      double b = (v > 0.0) == (ismin != 0) ? q->lb[j] : q->ub[j];
      if( !isInf(&q->s, b) && !isInf(&q->s, -b) && !isHuge(&q->s, v * b) && !isHuge(&q->s, -v * b) )
         sum21(&hi, &lo, v * b);
   }
   if( ismin )
   {
      r->a.minhi = hi;
      r->a.minlo = lo;
      r->validmin = 1;
      r->lastmin = hi + lo;
   }
   else
   {
      r->a.maxhi = hi;
      r->a.maxlo = lo;
      r->validmax = 1;
      r->lastmax = hi + lo;
   }
}

static void ensureAct(Seq* q, int32_t i, RowSt* r)
{
   if( !r->valid )
      calcActivities(q, i, r);
}

/* getMinActivity (cons_linear.c:2345-2436) with the recomputation of an invalid finite part */
static void seqMin(Seq* q, int32_t i, RowSt* r, int posinf, int neginf, int poshuge, int neghuge, double delta,
   int goodrelax, double* val, int* tight, int* settoinf)
{
   if( neginf == 0 && posinf == 0 && !(neghuge > 0 || (poshuge > 0 && !goodrelax)) && !r->validmin )
      recomputeSide(q, i, r, 1);
   getMinAct(&q->s, &r->a, posinf, neginf, poshuge, neghuge, delta, goodrelax, val, tight, settoinf);
}

/* getMaxActivity (cons_linear.c:2441-2529) with the recomputation of an invalid finite part */
static void seqMax(Seq* q, int32_t i, RowSt* r, int posinf, int neginf, int poshuge, int neghuge, double delta,
   int goodrelax, double* val, int* tight, int* settoinf)
{
   if( posinf == 0 && neginf == 0 && !(poshuge > 0 || (neghuge > 0 && !goodrelax)) && !r->validmax )
      recomputeSide(q, i, r, 0);
   getMaxAct(&q->s, &r->a, posinf, neginf, poshuge, neghuge, delta, goodrelax, val, tight, settoinf);
}

/* consdataGetActivityBounds (cons_linear.c:2533-2576) */
static void activityBounds(Seq* q, int32_t i, RowSt* r, int goodrelax, double* minact, double* maxact, int* mintight,
   int* maxtight, int* mininf, int* maxinf)
{
   const Act* a = &r->a;
   ensureAct(q, i, r);
   seqMin(q, i, r, a->minposinf, a->minneginf, a->minposhuge, a->minneghuge, 0.0, goodrelax, minact, mintight, mininf);
   seqMax(q, i, r, a->maxposinf, a->maxneginf, a->maxposhuge, a->maxneghuge, 0.0, goodrelax, maxact, maxtight, maxinf);
}

/* consdataGetActivityResiduals (cons_linear.c:2661-2806), goodrelax FALSE as tightenVarBounds asks */
static void seqResiduals(Seq* q, int32_t i, RowSt* r, double val, double l, double u, double* minres, double* maxres,
   int* mintight, int* maxtight, int* mininf, int* maxinf)
{
   const Num* s = &q->s;
   const Act* a = &r->a;
   double minb;
   double maxb;
   double absval;
   ensureAct(q, i, r);
   if( val > 0.0 )
   {
      minb = l;
      maxb = u;
      absval = val;
   }
   else
   {
      minb = -u;
      maxb = -l;
      absval = -val;
   }
   if( isInf(s, minb) )
      seqMin(q, i, r, a->minposinf - 1, a->minneginf, a->minposhuge, a->minneghuge, 0.0, 0, minres, mintight, mininf);
   else if( isInf(s, -minb) )
      seqMin(q, i, r, a->minposinf, a->minneginf - 1, a->minposhuge, a->minneghuge, 0.0, 0, minres, mintight, mininf);
   else if( isHuge(s, minb * absval) )
      seqMin(q, i, r, a->minposinf, a->minneginf, a->minposhuge - 1, a->minneghuge, 0.0, 0, minres, mintight, mininf);
   else if( isHuge(s, -minb * absval) )
      seqMin(q, i, r, a->minposinf, a->minneginf, a->minposhuge, a->minneghuge - 1, 0.0, 0, minres, mintight, mininf);
   else
      seqMin(q, i, r, a->minposinf, a->minneginf, a->minposhuge, a->minneghuge, absval * minb, 0, minres, mintight,
         mininf);

   if( isInf(s, -maxb) )
      seqMax(q, i, r, a->maxposinf, a->maxneginf - 1, a->maxposhuge, a->maxneghuge, 0.0, 0, maxres, maxtight, maxinf);
   else if( isInf(s, maxb) )
      seqMax(q, i, r, a->maxposinf - 1, a->maxneginf, a->maxposhuge, a->maxneghuge, 0.0, 0, maxres, maxtight, maxinf);
   else if( isHuge(s, absval * maxb) )
      seqMax(q, i, r, a->maxposinf, a->maxneginf, a->maxposhuge - 1, a->maxneghuge, 0.0, 0, maxres, maxtight, maxinf);
   else if( isHuge(s, -absval * maxb) )
      seqMax(q, i, r, a->maxposinf, a->maxneginf, a->maxposhuge, a->maxneghuge - 1, 0.0, 0, maxres, maxtight, maxinf);
   else
      seqMax(q, i, r, a->maxposinf, a->maxneginf, a->maxposhuge, a->maxneghuge, absval * maxb, 0, maxres, maxtight,
         maxinf);
}

/* consdataGetReliableResidualActivity (cons_linear.c:2580-2657): plain double sum in the row's order */
static double reliableRes(Seq* q, int32_t i, int32_t skipcol, int ismin)
{
   const lpo_problem* P = q->P;
   int64_t len = P->rowptr[i + 1] - P->rowptr[i];
   int64_t k;
   double res = 0.0;
   for( k = 0; k < len; ++k )
   {
      int64_t p = ordPos(q, i, k);
      int32_t j = P->colidx[p];
      double v = P->vals[p];
      if( j == skipcol )
         continue;
      if( v > 0.0 )
         res += ismin ? v * q->lb[j] : v * q->ub[j];
      else
         res += ismin ? v * q->ub[j] : v * q->lb[j];
   }
   return res;
}

/* consdataRecomputeMaxActivityDelta (cons_linear.c:1542-1599), last entry first */
static void recomputeMaxDelta(Seq* q, int32_t i, RowSt* r)
{
   const lpo_problem* P = q->P;
   int64_t len = P->rowptr[i + 1] - P->rowptr[i];
   int64_t k;
   r->maxdelta = 0.0;
   if( !r->nonbinvalid )
   {
      /* consdataCheckNonbinvar */
      r->hasnonbin = 0;
      for( k = 0; k < len; ++k )
         if( !isBinaryCol(q, P->colidx[ordPos(q, i, k)]) )
            r->hasnonbin = 1;
      r->nonbinvalid = 1;
   }
   if( !r->hasnonbin )
   {
      for( k = len - 1; k >= 0; --k )
      {
         int64_t p = ordPos(q, i, k);
         int32_t j = P->colidx[p];
         if( q->lb[j] < 0.5 && q->ub[j] > 0.5 )
         {
            double d = fabs(P->vals[p]);
            if( d > r->maxdelta )
            {
               r->maxdelta = d;
               r->maxdeltacol = j;
            }
         }
      }
      return;
   }
   for( k = len - 1; k >= 0; --k )
   {
      int64_t p = ordPos(q, i, k);
      int32_t j = P->colidx[p];
      double d;
      if( isInf(&q->s, -q->lb[j]) || isInf(&q->s, q->ub[j]) )
      {
         r->maxdelta = q->s.inf;
         r->maxdeltacol = j;
         break;
      }
      d = fabs(P->vals[p]) * (q->ub[j] - q->lb[j]);
      if( d > r->maxdelta )
      {
         r->maxdelta = d;
         r->maxdeltacol = j;
      }
   }
}

/* consdataUpdateActivities (cons_linear.c:1604-1992) for a local bound change, checkreliability TRUE */
static void updateActivities(Seq* q, RowSt* r, double val, double oldb, double newb, int islb)
{
   const Num* s = &q->s;
   Act* a = &r->a;
   double* hi;
   double* lo;
   double* last;
   int* posinf;
   int* neginf;
   int* poshuge;
   int* neghuge;
   int validact;
   int ismin = (islb != 0) == (val > 0.0);
   double dhi = 0.0;
   double dlo = 0.0;
   double oldc = val * oldb;
   double newc = val * newb;
   int hugenew = isHuge(s, fabs(newc));
   int finnew = !isInf(s, fabs(newb));

   if( ismin )
   {
      hi = &a->minhi; lo = &a->minlo; last = &r->lastmin; validact = r->validmin;
      poshuge = &a->minposhuge; neghuge = &a->minneghuge;
      /* with a negative coefficient the infinity counters swap */
      posinf = val > 0.0 ? &a->minposinf : &a->minneginf;
      neginf = val > 0.0 ? &a->minneginf : &a->minposinf;
   }
   else
   {
      hi = &a->maxhi; lo = &a->maxlo; last = &r->lastmax; validact = r->validmax;
      poshuge = &a->maxposhuge; neghuge = &a->maxneghuge;
      posinf = val > 0.0 ? &a->maxposinf : &a->maxneginf;
      neginf = val > 0.0 ? &a->maxneginf : &a->maxposinf;
   }

   if( isInf(s, fabs(oldb)) )
   {
      if( oldb > 0.0 )
      {
         if( finnew || newb < 0.0 )
         {
            (*posinf)--;
            if( !finnew && newb < 0.0 )
               (*neginf)++;
            else if( hugenew )
            {
               if( newc > 0.0 )
                  (*poshuge)++;
               else
                  (*neghuge)++;
            }
            else
               dhi = newc;
         }
      }
      else
      {
         if( finnew || newb > 0.0 )
         {
            (*neginf)--;
            if( !finnew && newb > 0.0 )
               (*posinf)++;
            else if( hugenew )
            {
               if( newc > 0.0 )
                  (*poshuge)++;
               else
                  (*neghuge)++;
            }
            else
               dhi = newc;
         }
      }
   }
   else if( isHuge(s, fabs(oldc)) )
   {
      if( oldc > 0.0 )
         (*poshuge)--;
      else
         (*neghuge)--;
      if( !finnew )
      {
         if( newb > 0.0 )
            (*posinf)++;
         else
            (*neginf)++;
      }
      else if( hugenew )
      {
         if( newc > 0.0 )
            (*poshuge)++;
         else
            (*neghuge)++;
      }
      else
         dhi = newc;
   }
   else
   {
      if( !finnew )
      {
         if( newb > 0.0 )
            (*posinf)++;
         else
            (*neginf)++;
         dhi = -oldc;
      }
      else if( hugenew )
      {
         if( newc > 0.0 )
            (*poshuge)++;
         else
            (*neghuge)++;
         dhi = -oldc;
      }
      else
      {
         dhi = newc;
         sum21(&dhi, &dlo, -oldc);
      }
   }

   if( validact && dhi + dlo != 0.0 )
   {
      double cur;
      sum21(hi, lo, dhi + dlo);
      cur = *hi + *lo;
      if( fabs(*last) < fabs(cur) )
         *last = cur;
      else if( updateUnreliable(s, cur, *last) )
      {
         if( ismin )
            r->validmin = 0;
         else
            r->validmax = 0;
      }
   }
}

/* ------------------------------------------------------------------ marked rows (cons.c) */
static void hdlrMark(Seq* q, int32_t i, RowSt* r)          /* conshdlrMarkConsPropagate */
{
   if( !r->en || r->mp )
      return;
   r->mp = 1;
   r->mpos = (int32_t)q->nm;
   q->M[q->nm++] = i;
}

static void hdlrUnmark(Seq* q, RowSt* r)                   /* conshdlrUnmarkConsPropagate */
{
   int32_t pos;
   if( !r->en || !r->mp )
      return;
   r->mp = 0;
   pos = r->mpos;
   r->mpos = -1;
   q->nm--;
   if( pos < q->nm )
   {
      int32_t last = q->M[q->nm];
      q->M[pos] = last;
      q->rs[last].mpos = pos;
   }
}

static void addUpdate(Seq* q, int32_t i, RowSt* r)         /* conshdlrAddUpdateCons */
{
   if( !r->inupd )
   {
      r->inupd = 1;
      q->U[q->nu++] = i;
   }
}

static void markProp(Seq* q, int32_t i, RowSt* r)          /* SCIPconsMarkPropagate */
{
   if( r->um || (r->mp && !r->uu) )
      return;
   if( q->indelay )
   {
      r->uu = 0;
      r->um = 1;
      addUpdate(q, i, r);
   }
   else
      hdlrMark(q, i, r);
}

static void unmarkProp(Seq* q, int32_t i, RowSt* r)        /* SCIPconsUnmarkPropagate (always inside the call) */
{
   if( r->uu || (!r->mp && !r->um) )
      return;
   r->um = 0;
   r->uu = 1;
   addUpdate(q, i, r);
}

static void disableRow(Seq* q, int32_t i, RowSt* r)        /* SCIPconsDisable (inside the call) */
{
   if( r->ud || !r->en )
      return;
   r->ud = 1;
   addUpdate(q, i, r);
}

/* conshdlrProcessUpdates (cons.c:1689-1860): the delayed updates, the last added first */
static void processUpdates(Seq* q)
{
   int64_t k;
   for( k = q->nu - 1; k >= 0; --k )
   {
      int32_t i = q->U[k];
      RowSt* r = &q->rs[i];
      if( r->ud )
      {
         hdlrUnmark(q, r);
         r->en = 0;
         r->ud = 0;
      }
      if( r->um )
         hdlrMark(q, i, r);
      else if( r->uu )
         hdlrUnmark(q, r);
      r->um = r->uu = 0;
      r->inupd = 0;
   }
   q->nu = 0;
}

/* ------------------------------------------------------------------ bound changes */
static void markDirty(Seq* q, int32_t j)
{
   if( q->dirty != NULL && !q->dirty[j] )
   {
      q->dirty[j] = 1;
      q->dirtylist[q->ndirty++] = j;
   }
}

/* eventExecLinear (cons_linear.c:17162-17363) for a tightened local bound of column j, in the order the rows caught
 * the column's events (the row order) */
static void boundEvent(Seq* q, int32_t j, int islb, double oldb, double newb)
{
   const lpo_problem* P = q->P;
   int64_t p;
   markDirty(q, j);
   for( p = P->colptr[j]; p < P->colptr[j + 1]; ++p )
   {
      int32_t i = P->rowidx[p];
      double a = P->cvals[p];
      RowSt* r = rowSt(q, i);
      if( r->del )
         continue;
      if( r->valid )
         updateActivities(q, r, a, oldb, newb, islb);
      markProp(q, i, r);
      if( r->maxdeltacol == j )
      {
         r->maxdelta = SEQ_INVALID;
         r->maxdeltacol = -1;
      }
      if( r->bt > 0 )
      {
         int rhsfin = !isInf(&q->s, P->rhs[i]);
         int lhsfin = !isInf(&q->s, -P->lhs[i]);
         if( islb ? (a > 0.0 ? rhsfin : lhsfin) : (a > 0.0 ? lhsfin : rhsfin) )
            r->bt = 0;
      }
   }
   /* at the root every change is global: a column that became an unfixed binary unsorts its rows
    * (GBDCHANGED branch of eventExecLinear) */
   if( q->root && isBinaryCol(q, j) && gt(&q->s, q->gub[j], q->glb[j]) )
   {
      for( p = P->colptr[j]; p < P->colptr[j + 1]; ++p )
      {
         RowSt* r = rowSt(q, P->rowidx[p]);
         if( !r->del )
            r->coefsorted = 0;
      }
   }
}

/* SCIPinferVarUbCons (scip_var.c:7071-7175) followed by SCIPnodeAddBoundinfer (tree.c:1912-2215): returns 1 if
 * infeasible; *tightened when the bound moved */
static int inferUb(Seq* q, int32_t j, double newub, int force, int* tightened)
{
   const Num* s = &q->s;
   int isint = q->P->isint[j] != 0;
   double l = q->lb[j];
   double u = q->ub[j];
   *tightened = 0;
   newub = adjUb(s, isint, newub);
   if( isInf(s, -newub) || feasLt(s, newub, l) )
      return 1;
   newub = dmax(newub, l);
   if( (force && ge(s, newub, u)) || (!force && !ubBetter(s, newub, l, u)) )
      return 0;
   /* SCIPnodeAddBoundinfer ignores a change that is not below the bound by more than epsilon */
   if( !lt(s, newub, u) )
      return 0;
   q->ub[j] = newub;
   q->nchg++;
   q->res->changes++;
#ifdef LPO_SEQ_TRACE
   fprintf(stderr, "TRACE ub x%d %.17g -> %.17g\n", j, u, newub);
#endif
   boundEvent(q, j, 0, u, newub);
   *tightened = 1;
   return 0;
}

/* SCIPinferVarLbCons (scip_var.c:6965-7069) followed by SCIPnodeAddBoundinfer */
static int inferLb(Seq* q, int32_t j, double newlb, int force, int* tightened)
{
   const Num* s = &q->s;
   int isint = q->P->isint[j] != 0;
   double l = q->lb[j];
   double u = q->ub[j];
   *tightened = 0;
   newlb = adjLb(s, isint, newlb);
   if( isInf(s, newlb) || feasGt(s, newlb, u) )
      return 1;
   newlb = dmin(newlb, u);
   if( (force && le(s, newlb, l)) || (!force && !lbBetter(s, newlb, l, u)) )
      return 0;
   if( !gt(s, newlb, l) )
      return 0;
   q->lb[j] = newlb;
   q->nchg++;
   q->res->changes++;
#ifdef LPO_SEQ_TRACE
   fprintf(stderr, "TRACE lb x%d %.17g -> %.17g\n", j, l, newlb);
#endif
   boundEvent(q, j, 1, l, newlb);
   *tightened = 1;
   return 0;
}

/* ------------------------------------------------------------------ tightening of one entry */
/* tightenVarBounds (cons_linear.c:6700-6974), the residual rule; returns 1 on cutoff */
static int tightenVarBounds(Seq* q, int32_t i, RowSt* r, int64_t k, int force)
{
   const lpo_problem* P = q->P;
   const Num* s = &q->s;
   int64_t p = ordPos(q, i, k);
   int32_t j = P->colidx[p];
   double val = P->vals[p];
   double lhs = P->lhs[i];
   double rhs = P->rhs[i];
   double minres, maxres, l, u;
   int mintight, maxtight, mininf, maxinf, tightened;
   int isint = P->isint[j] != 0;

   seqResiduals(q, i, r, val, q->lb[j], q->ub[j], &minres, &maxres, &mintight, &maxtight, &mininf, &maxinf);
   l = q->lb[j];
   u = q->ub[j];
   q->res->candidates++;

   if( val > 0.0 )
   {
      if( !mininf && !isInf(s, rhs) && mintight && (lt(s, fabs(rhs), 1.0) || !eq(s, minres / rhs, 1.0)) )
      {
         double newub = (rhs - minres) / val;
         if( !isInf(s, newub) && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u)) )
         {
            int unrel = updateUnreliable(s, minres, r->lastmin);
            if( unrel )
            {
               minres = reliableRes(q, i, j, 1);
               newub = (rhs - minres) / val;
               unrel = isInf(s, -minres) || (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) || !isint)
                  && (!force || !lt(s, newub, u)));
            }
            if( !unrel )
            {
               if( inferUb(q, j, newub, force, &tightened) )
                  return 1;
               if( tightened )
                  u = q->ub[j];
            }
         }
      }
      if( !maxinf && !isInf(s, -lhs) && maxtight && (lt(s, fabs(lhs), 1.0) || !eq(s, maxres / lhs, 1.0)) )
      {
         double newlb = (lhs - maxres) / val;
         if( !isInf(s, -newlb) && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u)) )
         {
            if( updateUnreliable(s, maxres, r->lastmax) )
            {
               maxres = reliableRes(q, i, j, 0);
               newlb = (lhs - maxres) / val;
               if( isInf(s, maxres) || (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint)
                     && (!force || !gt(s, newlb, l))) )
                  return 0;
            }
            if( inferLb(q, j, newlb, force, &tightened) )
               return 1;
         }
      }
   }
   else
   {
      if( !mininf && !isInf(s, rhs) && mintight && (lt(s, fabs(rhs), 1.0) || !eq(s, minres / rhs, 1.0)) )
      {
         double newlb = (rhs - minres) / val;
         if( !isInf(s, -newlb) && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u)) )
         {
            int unrel = updateUnreliable(s, minres, r->lastmin);
            if( unrel )
            {
               minres = reliableRes(q, i, j, 1);
               newlb = (rhs - minres) / val;
               unrel = isInf(s, -minres) || (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint)
                  && (!force || !gt(s, newlb, l)));
            }
            if( !unrel )
            {
               if( inferLb(q, j, newlb, force, &tightened) )
                  return 1;
               if( tightened )
                  l = q->lb[j];
            }
         }
      }
      if( !maxinf && !isInf(s, -lhs) && maxtight && (lt(s, fabs(lhs), 1.0) || !eq(s, maxres / lhs, 1.0)) )
      {
         double newub = (lhs - maxres) / val;
         if( !isInf(s, newub) && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u)) )
         {
            if( updateUnreliable(s, maxres, r->lastmax) )
            {
               maxres = reliableRes(q, i, j, 0);
               newub = (lhs - maxres) / val;
               /* cons_linear.c:6936 joins the middle condition with && where the other three branches use || */
               if( isInf(s, maxres) || (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) && !isint)
                     && (!force || !lt(s, newub, u))) )
                  return 0;
            }
            if( inferUb(q, j, newub, force, &tightened) )
               return 1;
         }
      }
   }
   return 0;
}

/* tightenVarUb / tightenVarLb (cons_linear.c:5242-5376) */
static int easyUb(Seq* q, int32_t j, double newub, double oldub, int force)
{
   int tightened;
   newub = adjUb(&q->s, q->P->isint[j] != 0, newub);
   if( force || ubBetter(&q->s, newub, q->lb[j], oldub) )
      return inferUb(q, j, newub, force, &tightened);
   return 0;
}

static int easyLb(Seq* q, int32_t j, double newlb, double oldlb, int force)
{
   int tightened;
   newlb = adjLb(&q->s, q->P->isint[j] != 0, newlb);
   if( force || lbBetter(&q->s, newlb, oldlb, q->ub[j]) )
      return inferLb(q, j, newlb, force, &tightened);
   return 0;
}

/* tightenVarBoundsEasy (cons_linear.c:5380-5653), the slack rule; returns 1 on cutoff */
static int tightenVarBoundsEasy(Seq* q, int32_t i, RowSt* r, int64_t k, int force)
{
   const lpo_problem* P = q->P;
   const Num* s = &q->s;
   int64_t p = ordPos(q, i, k);
   int32_t j = P->colidx[p];
   double val = P->vals[p];
   double lhs = P->lhs[i];
   double rhs = P->rhs[i];
   double l = q->lb[j];
   double u = q->ub[j];

   ensureAct(q, i, r);
   if( !r->validmin )
      recomputeSide(q, i, r, 1);
   q->res->candidates++;

   if( val > 0.0 )
   {
      if( !isInf(s, rhs) )
      {
         double minact = r->a.minhi + r->a.minlo;
         double slack, alpha;
         if( feasLt(s, rhs, minact) )
            return 1;
         slack = rhs - minact;
         if( !positive(s, slack) )
            slack = 0.0;
         alpha = val * (u - l);
         if( sumGt(s, alpha, slack) || (force && gt(s, alpha, slack)) )
         {
            if( easyUb(q, j, l + slack / val, u, force) )
               return 1;
            u = q->ub[j];
         }
      }
      if( !isInf(s, -lhs) )
      {
         double maxact, slack, alpha;
         if( !r->validmax )
            recomputeSide(q, i, r, 0);
         maxact = r->a.maxhi + r->a.maxlo;
         if( feasLt(s, maxact, lhs) )
            return 1;
         slack = maxact - lhs;
         if( !positive(s, slack) )
            slack = 0.0;
         alpha = val * (u - l);
         if( sumGt(s, alpha, slack) || (force && gt(s, alpha, slack)) )
         {
            if( easyLb(q, j, u - slack / val, l, force) )
               return 1;
         }
      }
   }
   else
   {
      if( !isInf(s, rhs) )
      {
         double minact = r->a.minhi + r->a.minlo;
         double slack, alpha;
         if( feasLt(s, rhs, minact) )
            return 1;
         slack = rhs - minact;
         if( !positive(s, slack) )
            slack = 0.0;
         alpha = val * (l - u);
         if( sumGt(s, alpha, slack) || (force && gt(s, alpha, slack)) )
         {
            if( easyLb(q, j, u + slack / val, l, force) )
               return 1;
            l = q->lb[j];
         }
      }
      if( !isInf(s, -lhs) )
      {
         double maxact, slack, alpha;
         if( !r->validmax )
            recomputeSide(q, i, r, 0);
         maxact = r->a.maxhi + r->a.maxlo;
         if( feasLt(s, maxact, lhs) )
            return 1;
         slack = maxact - lhs;
         if( !positive(s, slack) )
            slack = 0.0;
         alpha = val * (l - u);
         if( sumGt(s, alpha, slack) || (force && gt(s, alpha, slack)) )
         {
            if( easyUb(q, j, l - slack / val, u, force) )
               return 1;
         }
      }
   }
   return 0;
}

/* tightenBounds (cons_linear.c:6976-7154); returns 1 on cutoff */
static int tightenBounds(Seq* q, int32_t i, RowSt* r)
{
   const lpo_problem* P = q->P;
   const Num* s = &q->s;
   int64_t len = P->rowptr[i + 1] - P->rowptr[i];
   int force = (len == 1);
   int tightenmode = q->root ? 2 : 1;
   int easy;
   int nrounds;
   int64_t lastchange = -1;

   /* canTightenBounds reads the counters as they are: at the root, before the first computation, they are -1 (the
    * test passes); below the root SCIP's activities are always valid, computed here on first use */
   if( !q->root )
      ensureAct(q, i, r);
   if( r->valid )
   {
      const Act* a = &r->a;
      if( a->minneginf + a->minposinf + a->minneghuge + a->minposhuge > 1
         && a->maxneginf + a->maxposinf + a->maxneghuge + a->maxposhuge > 1 )
         return 0;
   }
   if( !force && r->bt >= tightenmode )
      return 0;
   if( q->sortvars && !r->coefsorted )
      sortRow(q, i, r);
   if( r->maxdelta == SEQ_INVALID )
      recomputeMaxDelta(q, i, r);
   if( feasZero(s, r->maxdelta) )
      return 0;
   if( !isInf(s, r->maxdelta) )
   {
      double minact, maxact, slack, surplus;
      int t1, t2, f1, f2;
      activityBounds(q, i, r, 0, &minact, &maxact, &t1, &t2, &f1, &f2);
      slack = (isInf(s, P->rhs[i]) || f1) ? s->inf : P->rhs[i] - minact;
      surplus = (isInf(s, -P->lhs[i]) || f2) ? s->inf : maxact - P->lhs[i];
      if( le(s, r->maxdelta, dmin(slack, surplus)) )
         return 0;
   }
   easy = lt(s, r->maxdelta, s->maxeasy);
   q->res->live_rows++;

   for( nrounds = 0; (force || r->bt < tightenmode) && nrounds < MAXTIGHTENROUNDS; ++nrounds )
   {
      int64_t v = 0;
      if( q->sortvars && !r->coefsorted )
         sortRow(q, i, r);
      r->bt = (uint8_t)tightenmode;
      while( v < len && v != lastchange )
      {
         int64_t old = q->nchg;
         if( easy ? tightenVarBoundsEasy(q, i, r, v, force) : tightenVarBounds(q, i, r, v, force) )
            return 1;
         if( q->nchg > old )
         {
            lastchange = v;
            ++v;
         }
         else if( r->coefsorted && v < r->nbin - 1 )
         {
            int32_t j = P->colidx[ordPos(q, i, v)];
            if( !(fabs(relDiff(q->ub[j], q->lb[j])) <= s->feastol) )   /* !SCIPisFeasEQ(ub, lb) */
               v = r->nbin;
            else
               ++v;
         }
         else
            ++v;
      }
   }
   return 0;
}

/* propagateCons (cons_linear.c:7621-7758) without ranged rows; returns 1 on cutoff */
static int propagateCons(Seq* q, int32_t i)
{
   const lpo_problem* P = q->P;
   const Num* s = &q->s;
   RowSt* r = rowSt(q, i);
   double minact, maxact;
   int t1, t2, f1, f2;
   q->res->rows++;
   q->res->nnz += P->rowptr[i + 1] - P->rowptr[i];
#ifdef LPO_SEQ_TRACE
   fprintf(stderr, "TRACE row r%d\n", i);
#endif
   if( tightenBounds(q, i, r) )
      return 1;
   activityBounds(q, i, r, 1, &minact, &maxact, &t1, &t2, &f1, &f2);
   if( feasGt(s, minact, P->rhs[i]) || feasLt(s, maxact, P->lhs[i]) )
      return 1;
   if( ge(s, minact, P->lhs[i]) && le(s, maxact, P->rhs[i]) )
   {
      /* redundant: deleted locally below the root (SCIPdelConsLocal -> SCIPnodeDelCons), globally at the root
       * (SCIPconsDelete marks it deleted at once, so its events are ignored from then on) */
      if( q->root )
         r->del = 1;
      disableRow(q, i, r);
   }
   return 0;
}

/* propagateDomains (solve.c:723-795): consPropLinear over the marked rows until a call finds no reduction */
static int propagateRounds(Seq* q, int32_t* rounds)
{
   int32_t round;
   int cutoff = 0;
   *rounds = 0;
   for( round = 0; round < q->maxrounds; ++round )
   {
      int64_t nmarked = q->nm;
      int64_t k;
      if( nmarked == 0 )
         return 0;
      q->nchg = 0;
      q->indelay = 1;
      for( k = 0; k < nmarked && !cutoff; ++k )
      {
         int32_t i = q->M[k];
         unmarkProp(q, i, &q->rs[i]);
         cutoff = propagateCons(q, i);
      }
      q->indelay = 0;
      processUpdates(q);
      *rounds = round + 1;
      if( cutoff )
         return 1;
      if( q->nchg == 0 )
         return 0;
   }
   return q->nm > 0 ? 2 : 0;
}

/* The order in which SCIP created the transformed variables, i.e. their unique index (SCIPvarGetIndex): the host
 * adds the columns in column order to a problem that keeps its variables grouped by type -- binaries, integers,
 * continuous -- and makes room for a new variable by moving the first variable of each later group to that group's
 * end (prob.c probInsertVar); an integral column with bounds in {0,1} is a binary variable; transforming the problem
 * creates the transformed variables in that array's order (SCIPprobTransform).  pos[j] = column j's rank. */
static void creationRank(const lpo_problem* P, const double* lb, const double* ub, int32_t* arr, int32_t* pos)
{
   int64_t nb = 0, ni = 0, nv = 0, j;
   for( j = 0; j < P->n; ++j )
   {
      int64_t at = nv;
      int bin = P->isint[j] != 0 && (lb[j] == 0.0 || lb[j] == 1.0) && (ub[j] == 0.0 || ub[j] == 1.0);
      if( P->isint[j] != 0 )
      {
         if( at > nb + ni )
         {
            arr[at] = arr[nb + ni];
            at = nb + ni;
         }
         if( bin && at > nb )
         {
            arr[at] = arr[nb];
            at = nb;
         }
         if( bin )
            ++nb;
         else
            ++ni;
      }
      arr[at] = (int32_t)j;
      ++nv;
   }
   for( j = 0; j < P->n; ++j )
      pos[arr[j]] = (int32_t)j;
}

/* Before solving SCIP sorts every row by consdataCompVar (cons_linear.c:3152-3187; consdataSort below
 * SCIP_STAGE_INITSOLVE, :3355-3360): binaries first, then by type, ties by the variables' unique index -- together
 * the creation rank.  Rows keep that order until tightenBounds sorts them for propagation (with sortvars). */
static void indexSortRows(Seq* q, const double* lb, const double* ub)
{
   const lpo_problem* P = q->P;
   int32_t* arr = malloc(sizeof(int32_t) * (size_t)(P->n + 1));
   int32_t* pos = malloc(sizeof(int32_t) * (size_t)(P->n + 1));
   int64_t i;
   if( arr == NULL || pos == NULL )
   {
      free(arr);
      free(pos);
      return;
   }
   creationRank(P, lb, ub, arr, pos);
   for( i = 0; i < P->m; ++i )
   {
      int32_t* a = q->ord + P->rowptr[i];
      int64_t len = P->rowptr[i + 1] - P->rowptr[i];
      int64_t k;
      for( k = 1; k < len; ++k )  /* insertion sort: rows are short and the ranks distinct */
      {
         int32_t x = a[k];
         int64_t t = k;
         while( t > 0 && pos[P->colidx[a[t - 1]]] > pos[P->colidx[x]] )
         {
            a[t] = a[t - 1];
            --t;
         }
         a[t] = x;
      }
   }
   free(arr);
   free(pos);
}

static int seqInit(Seq* q, const lpo_problem* P, const lpo_params* par, int root, int track)
{
   int64_t m = P->m;
   int64_t p;
   int64_t maxlen = 1;
   int64_t i;
   memset(q, 0, sizeof(*q));
   q->P = P;
   numFrom(par, &q->s);
   q->root = root;
   q->sortvars = !(par->flags & LPO_FLAG_NOSORTVARS);
   q->maxrounds = par->maxrounds > 0 ? par->maxrounds : 1000000;
   for( i = 0; i < m; ++i )
      if( P->rowptr[i + 1] - P->rowptr[i] > maxlen )
         maxlen = P->rowptr[i + 1] - P->rowptr[i];
   q->rs = calloc((size_t)(m + 1), sizeof(RowSt));
   q->ord = malloc(sizeof(int32_t) * (size_t)(P->rowptr[m] + 1));
   q->tmp = malloc(sizeof(int32_t) * (size_t)maxlen);
   q->M = malloc(sizeof(int32_t) * (size_t)(m + 1));
   q->U = malloc(sizeof(int32_t) * (size_t)(m + 1));
   if( track )
   {
      q->dirty = calloc((size_t)(P->n + 1), 1);
      q->dirtylist = malloc(sizeof(int32_t) * (size_t)(P->n + 1));
   }
   if( q->rs == NULL || q->ord == NULL || q->tmp == NULL || q->M == NULL || q->U == NULL
      || (track && (q->dirty == NULL || q->dirtylist == NULL)) )
      return -1;
   for( p = 0; p < P->rowptr[m]; ++p )
      q->ord[p] = (int32_t)p;
   q->stamp = 1;
   return 0;
}

static void seqFree(Seq* q)
{
   free(q->rs); free(q->ord); free(q->tmp); free(q->M); free(q->U); free(q->dirty); free(q->dirtylist);
}

int lpo_propagate_seq(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub, int32_t* out_order,
   lpo_result* res)
{
   return lpo_propagate_seq_states(prob, par, lb, ub, out_order, res, NULL);
}

size_t lpo_seq_state_bytes(int64_t m)
{
   return sizeof(RowSt) * (size_t)(m + 1);
}

void lpo_seq_states_deleted(const void* states, int64_t m, uint8_t* del)
{
   const RowSt* rs = states;
   int64_t i;
   for( i = 0; i < m; ++i )
      del[i] = rs[i].del;
}

int lpo_propagate_seq_states(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub,
   int32_t* out_order, lpo_result* res, void* out_states)
{
   Seq q;
   int64_t i;
   int st;
   memset(res, 0, sizeof(*res));
   if( seqInit(&q, prob, par, 1, 0) != 0 )
   {
      seqFree(&q);
      return -1;
   }
   q.lb = lb;
   q.ub = ub;
   q.glb = lb;
   q.gub = ub;
   q.res = res;
   indexSortRows(&q, lb, ub);
   /* every row is marked on activation, in the order the rows were added */
   for( i = 0; i < prob->m; ++i )
      hdlrMark(&q, (int32_t)i, rowSt(&q, (int32_t)i));
   st = propagateRounds(&q, &res->rounds);
   res->status = st;
   res->cutoff = st == 1;
   if( out_order != NULL )
      memcpy(out_order, q.ord, sizeof(int32_t) * (size_t)prob->rowptr[prob->m]);
   if( out_states != NULL )
      memcpy(out_states, q.rs, lpo_seq_state_bytes(prob->m));
   seqFree(&q);
   return 0;
}

/* ------------------------------------------------------------------ batched nodes */
typedef struct
{
   const lpo_problem* P;
   const lpo_params* par;
   const uint8_t* rowdel;
   const RowSt* rootst;
   const double* baselb;
   const double* baseub;
   const int64_t* ptr;
   const int32_t* chg_col;
   const double* chg_lb;
   const double* chg_ub;
   int8_t* out_cutoff;
   int32_t* out_rounds;
   int32_t* out_n;
   int32_t* out_col;
   double* out_lb;
   double* out_ub;
   int32_t cap;
   int64_t k0;
   int64_t k1;
   lpo_result tot;
   int err;
} SeqJob;

static void* seqNodeWorker(void* arg)
{
   SeqJob* J = arg;
   const lpo_problem* P = J->P;
   const Num* s;
   Seq q;
   double* lb = malloc(sizeof(double) * (size_t)(P->n + 1));
   double* ub = malloc(sizeof(double) * (size_t)(P->n + 1));
   int64_t k;

   memset(&J->tot, 0, sizeof(J->tot));
   if( lb == NULL || ub == NULL || seqInit(&q, P, J->par, 0, 1) != 0 )
   {
      J->err = -1;
      free(lb);
      free(ub);
      return NULL;
   }
   s = &q.s;
   q.rowdel = J->rowdel;
   q.rootst = J->rootst;
   memcpy(lb, J->baselb, sizeof(double) * (size_t)P->n);
   memcpy(ub, J->baseub, sizeof(double) * (size_t)P->n);
   q.lb = lb;
   q.ub = ub;
   q.glb = J->baselb;
   q.gub = J->baseub;

   for( k = J->k0; k < J->k1; ++k )
   {
      lpo_result r;
      int64_t c;
      int cut = 0;
      int32_t rounds = 0;
      memset(&r, 0, sizeof(r));
      q.res = &r;
      if( ++q.stamp == INT32_MAX )
      {
         memset(q.rs, 0, sizeof(RowSt) * (size_t)(P->m + 1));
         q.stamp = 1;
      }
      q.nm = 0;
      q.nu = 0;
      q.indelay = 0;
      /* the node's branching changes, as SCIPchgVarLbProbing / SCIPchgVarUbProbing make them (scip_probing.c:302-380:
       * adjusted to integrality, ignored unless they tighten by more than epsilon), each followed by its events */
      for( c = J->ptr[k]; c < J->ptr[k + 1] && !cut; ++c )
      {
         int32_t j = J->chg_col[c];
         int isint = P->isint[j] != 0;
         double nl = J->chg_lb[c];
         double nu = J->chg_ub[c];
         if( nl > ub[j] || nu < lb[j] )
         {
            cut = 1;
            break;
         }
         if( nl > lb[j] )
         {
            double v = adjLb(s, isint, nl);
            if( !isInf(s, v) )
            {
               v = dmin(v, ub[j]);
               if( gt(s, v, lb[j]) )
               {
                  double old = lb[j];
                  lb[j] = v;
                  boundEvent(&q, j, 1, old, v);
               }
            }
         }
         if( nu < ub[j] )
         {
            double v = adjUb(s, isint, nu);
            if( !isInf(s, -v) )
            {
               v = dmax(v, lb[j]);
               if( lt(s, v, ub[j]) )
               {
                  double old = ub[j];
                  ub[j] = v;
                  boundEvent(&q, j, 0, old, v);
               }
            }
         }
      }
      if( !cut )
      {
         int st = propagateRounds(&q, &rounds);
         cut = st == 1;
         if( st == 2 )
            r.status = 2;
      }
      J->out_cutoff[k] = (int8_t)cut;
      J->out_rounds[k] = rounds;
      {
         int32_t cnt = 0;
         int64_t d;
         if( !cut )
         {
            for( d = 0; d < q.ndirty; ++d )
            {
               int32_t j = q.dirtylist[d];
               if( lb[j] != J->baselb[j] || ub[j] != J->baseub[j] )
               {
                  if( cnt < J->cap )
                  {
                     int64_t o = k * (int64_t)J->cap + cnt;
                     J->out_col[o] = j;
                     J->out_lb[o] = lb[j];
                     J->out_ub[o] = ub[j];
                  }
                  ++cnt;
               }
            }
         }
         J->out_n[k] = cnt > J->cap ? -1 : cnt;
      }
      for( c = 0; c < q.ndirty; ++c )
      {
         int32_t j = q.dirtylist[c];
         lb[j] = J->baselb[j];
         ub[j] = J->baseub[j];
         q.dirty[j] = 0;
      }
      q.ndirty = 0;
      J->tot.rows += r.rows;
      J->tot.nnz += r.nnz;
      J->tot.candidates += r.candidates;
      J->tot.changes += r.changes;
      J->tot.live_rows += r.live_rows;
      J->tot.cutoff += cut;
      if( rounds > J->tot.rounds )
         J->tot.rounds = rounds;
      if( r.status == 2 )
         J->tot.status = 2;
   }
   seqFree(&q);
   free(lb);
   free(ub);
   return NULL;
}

/* the rows SCIP's root deleted: a row redundant under the root's final bounds was re-propagated after its last
 * column change and found redundant (propagateCons, cons_linear.c:7741-7753; SCIPconsDelete at depth 0), and a
 * deleted row takes no part in any node */
void lpo_root_deleted_rows(const lpo_problem* prob, const lpo_params* par, const double* lb, const double* ub,
   uint8_t* del)
{
   Num s;
   int64_t i;
   numFrom(par, &s);
   for( i = 0; i < prob->m; ++i )
   {
      Act a;
      double minact, maxact;
      int t1, t2, f1, f2;
      int64_t p;
      memset(&a, 0, sizeof(a));
      for( p = prob->rowptr[i]; p < prob->rowptr[i + 1]; ++p )
         addTerm(&s, &a, prob->vals[p], lb[prob->colidx[p]], ub[prob->colidx[p]]);
      getMinAct(&s, &a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, 0.0, 1, &minact, &t1, &f1);
      getMaxAct(&s, &a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, 1, &maxact, &t2, &f2);
      del[i] = (uint8_t)(ge(&s, minact, prob->lhs[i]) && le(&s, maxact, prob->rhs[i]));
   }
}

int lpo_propagate_nodes_seq(const lpo_problem* prob, const lpo_params* par, const double* baselb,
   const double* baseub, int64_t nnodes, const int64_t* ptr, const int32_t* chg_col, const double* chg_lb,
   const double* chg_ub, int8_t* out_cutoff, int32_t* out_rounds, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int32_t cap, int32_t nthreads, lpo_result* total)
{
   return lpo_propagate_nodes_seq_from(prob, par, baselb, baseub, nnodes, ptr, chg_col, chg_lb, chg_ub, out_cutoff,
      out_rounds, out_n, out_col, out_lb, out_ub, cap, nthreads, total, NULL);
}

int lpo_propagate_nodes_seq_from(const lpo_problem* prob, const lpo_params* par, const double* baselb,
   const double* baseub, int64_t nnodes, const int64_t* ptr, const int32_t* chg_col, const double* chg_lb,
   const double* chg_ub, int8_t* out_cutoff, int32_t* out_rounds, int32_t* out_n, int32_t* out_col, double* out_lb,
   double* out_ub, int32_t cap, int32_t nthreads, lpo_result* total, const void* root_states)
{
   SeqJob* jobs;
   pthread_t* th;
   uint8_t* rowdel;
   int32_t t;
   int err = 0;
   if( nthreads < 1 )
      nthreads = 1;
   if( nthreads > nnodes )
      nthreads = nnodes > 0 ? (int32_t)nnodes : 1;
   jobs = calloc((size_t)nthreads, sizeof(SeqJob));
   th = calloc((size_t)nthreads, sizeof(pthread_t));
   rowdel = malloc((size_t)(prob->m + 1));
   if( jobs == NULL || th == NULL || rowdel == NULL )
   {
      free(jobs);
      free(th);
      free(rowdel);
      return -1;
   }
   if( root_states != NULL )
      lpo_seq_states_deleted(root_states, prob->m, rowdel);  /* the rows the root itself deleted */
   else
      lpo_root_deleted_rows(prob, par, baselb, baseub, rowdel);
   for( t = 0; t < nthreads; ++t )
   {
      SeqJob* J = &jobs[t];
      J->P = prob; J->par = par; J->rowdel = rowdel; J->rootst = (const RowSt*)root_states; J->baselb = baselb; J->baseub = baseub; J->ptr = ptr; J->chg_col = chg_col;
      J->chg_lb = chg_lb; J->chg_ub = chg_ub; J->out_cutoff = out_cutoff; J->out_rounds = out_rounds;
      J->out_n = out_n; J->out_col = out_col; J->out_lb = out_lb; J->out_ub = out_ub; J->cap = cap;
      J->k0 = nnodes * t / nthreads;
      J->k1 = nnodes * (t + 1) / nthreads;
   }
   if( nthreads == 1 )
      seqNodeWorker(&jobs[0]);
   else
   {
      for( t = 0; t < nthreads; ++t )
         if( pthread_create(&th[t], NULL, seqNodeWorker, &jobs[t]) != 0 )
         {
            jobs[t].err = -1;
            th[t] = 0;
         }
      for( t = 0; t < nthreads; ++t )
         if( jobs[t].err == 0 )
            pthread_join(th[t], NULL);
   }
   if( total != NULL )
      memset(total, 0, sizeof(*total));
   for( t = 0; t < nthreads; ++t )
   {
      if( jobs[t].err )
         err = -1;
      if( total != NULL )
      {
         total->rows += jobs[t].tot.rows;
         total->nnz += jobs[t].tot.nnz;
         total->candidates += jobs[t].tot.candidates;
         total->changes += jobs[t].tot.changes;
         total->live_rows += jobs[t].tot.live_rows;
         total->cutoff += jobs[t].tot.cutoff;
         if( jobs[t].tot.rounds > total->rounds )
            total->rounds = jobs[t].tot.rounds;
         if( jobs[t].tot.status == 2 )
            total->status = 2;
      }
   }
   free(jobs);
   free(th);
   free(rowdel);
   return err;
}
