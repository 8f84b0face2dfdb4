/* Test infrastructure only: CPU restatement of SCIP 11's cons_linear activity-based bound propagation.
 * The tests, smoke() and the CPU-baseline leg of bench.py use it as the checker of the CUDA path; the
 * product library never links it.  Round semantics are described in linprop_oracle.h.
 *
 * Every rule below restates the SCIP function cited beside it (paths relative to the SCIP source tree).
 */
#define _POSIX_C_SOURCE 200809L
#include "linprop_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "lpo_common.h"

void lpo_default_params(lpo_params* p)
{
   p->infinity = 1e20;
   p->epsilon = 1e-9;
   p->sumepsilon = 1e-6;
   p->feastol = 1e-6;
   p->hugeval = 1e15;
   p->boundstreps = 0.05;
   p->recompfac = 1e6;
   p->maxeasyactivitydelta = 0.0;
   p->maxrounds = 0;
   p->flags = 0;
}

/* Activities are summed in a fixed order that does not depend on how the GPU schedules the row: rows of
 * up to LONGROW entries as two halves (entries [0, ceil(len/2)) and the rest), each in row order
 * (consdataCalcActivities order), the second merged into the first; longer rows as 32 interleaved partial
 * sums (entry p goes to partial (p - rowstart) mod 32, each summed in row order) merged pairwise
 * (partial k absorbs partial k + 16, then k + 8, 4, 2, 1).  A merge adds the other partial's high word through
 * the compensated sum and its low word to the low word. */
#define LONGROW 64
static void rowActivity(const Num* s, const lpo_problem* P, const double* lb, const double* ub, int64_t i, Act* a)
{
   int64_t p;
   int64_t p0 = P->rowptr[i];
   int64_t p1 = P->rowptr[i + 1];
   memset(a, 0, sizeof(*a));
   if( p1 - p0 <= LONGROW )
   {
      /* two halves, each in row order, the second merged into the first */
      Act second;
      int64_t ph = p0 + (p1 - p0 + 1) / 2;
      memset(&second, 0, sizeof(second));
      for( p = p0; p < ph; ++p )
      {
         int32_t j = P->colidx[p];
         addTerm(s, a, P->vals[p], lb[j], ub[j]);
      }
      for( p = ph; p < p1; ++p )
      {
         int32_t j = P->colidx[p];
         addTerm(s, &second, P->vals[p], lb[j], ub[j]);
      }
      actMerge(a, &second);
   }
   else
   {
      Act part[32];
      int k;
      int off;
      memset(part, 0, sizeof(part));
      for( k = 0; k < 32; ++k )
      {
         for( p = p0 + k; p < p1; p += 32 )
         {
            int32_t j = P->colidx[p];
            addTerm(s, &part[k], P->vals[p], lb[j], ub[j]);
         }
      }
      for( off = 16; off >= 1; off /= 2 )
         for( k = 0; k < off; ++k )
            actMerge(&part[k], &part[k + off]);
      *a = part[0];
   }
}

/* consdataGetReliableResidualActivity, cons_linear.c:2580-2657: plain double sum in row order */
static double reliableResidual(const lpo_problem* P, const double* lb, const double* ub, int64_t i, int64_t skip,
   int ismin)
{
   double r = 0.0;
   int64_t p;
   for( p = P->rowptr[i]; p < P->rowptr[i + 1]; ++p )
   {
      double v = P->vals[p];
      int32_t j = P->colidx[p];
      if( p == skip )
         continue;
      if( v > 0.0 )
         r += ismin ? v * lb[j] : v * ub[j];
      else
         r += ismin ? v * ub[j] : v * lb[j];
   }
   return r;
}

void lpo_row_activities(const lpo_problem* prob, const lpo_params* par, const double* lb, const double* ub,
   const int32_t* rows, int64_t nrows, double* act, int32_t* cnt)
{
   Num s;
   int64_t k;
   numFrom(par, &s);
   if( rows == NULL )
      nrows = prob->m;
   for( k = 0; k < nrows; ++k )
   {
      Act a;
      rowActivity(&s, prob, lb, ub, rows == NULL ? k : rows[k], &a);
      act[4 * k + 0] = a.minhi;
      act[4 * k + 1] = a.minlo;
      act[4 * k + 2] = a.maxhi;
      act[4 * k + 3] = a.maxlo;
      cnt[8 * k + 0] = a.minposinf;
      cnt[8 * k + 1] = a.minneginf;
      cnt[8 * k + 2] = a.minposhuge;
      cnt[8 * k + 3] = a.minneghuge;
      cnt[8 * k + 4] = a.maxposinf;
      cnt[8 * k + 5] = a.maxneginf;
      cnt[8 * k + 6] = a.maxposhuge;
      cnt[8 * k + 7] = a.maxneghuge;
   }
}

/* ------------------------------------------------------------------ propagation work space */
typedef struct
{
   const lpo_problem* P;
   Num s;
   int32_t maxrounds;
   /* candidates per column: best non-forced / forced upper and lower bound */
   double* cub;
   double* clb;
   double* cubf;
   double* clbf;
   uint8_t* cflag;      /* bit0 ub, bit1 ubf, bit2 lb, bit3 lbf */
   int32_t* touched;
   int64_t ntouched;
   int32_t* front;      /* current frontier */
   int32_t* next;       /* next frontier */
   int64_t nfront;
   int64_t nnext;
   int32_t* rowstamp;
   int32_t stamp;
   double* oldlb;       /* per changed column: bounds at round start */
   double* oldub;
   int32_t* chg;
   int64_t nchg;
   /* node bookkeeping: columns modified since the base bounds */
   uint8_t* dirty;
   int32_t* dirtylist;
   int64_t ndirty;
   double* savelb;
   double* saveub;
   /* binary skip: global domain for the binary test (NULL = current bounds) and the candidates of the
    * row being processed, per entry position */
   int binskip;
   const double* glb;
   const double* gub;
   double* rub;
   double* rlb;
   uint8_t* rflag;      /* bit0 ub, bit1 forced ub, bit2 lb, bit3 forced lb */
   lpo_log* log;        /* change log, or NULL */
   /* ranged rows: on/off, and for the row being processed its propagation order (rord[k] = offset of the k-th
    * entry), merge scratch and gcd membership per order position */
   int ranged;
   int32_t round;       /* the round being processed (ranged-row records) */
   double* startlb;     /* the bounds the call started from (sortvars off, no global domain), else NULL */
   double* startub;
   int32_t* rord;
   int32_t* rtmp;
   uint8_t* rmem;
} Work;

static int workInit(Work* w, const lpo_problem* P, const lpo_params* par)
{
   int64_t n = P->n;
   int64_t m = P->m;
   int64_t maxlen = 1;
   int64_t i;
   memset(w, 0, sizeof(*w));
   for( i = 0; i < m; ++i )
      if( P->rowptr[i + 1] - P->rowptr[i] > maxlen )
         maxlen = P->rowptr[i + 1] - P->rowptr[i];
   w->binskip = !(par->flags & LPO_FLAG_NOSORTVARS);
   w->ranged = (par->flags & LPO_FLAG_RANGEDROW) != 0;
   w->rmem = calloc((size_t)maxlen, 1);
   w->rord = malloc(sizeof(int32_t) * (size_t)maxlen);
   w->rtmp = malloc(sizeof(int32_t) * (size_t)maxlen);
   w->rub = malloc(sizeof(double) * (size_t)maxlen);
   w->rlb = malloc(sizeof(double) * (size_t)maxlen);
   w->rflag = calloc((size_t)maxlen, 1);
   w->P = P;
   numFrom(par, &w->s);
   w->maxrounds = par->maxrounds > 0 ? par->maxrounds : 1000000;
   w->cub = malloc(sizeof(double) * (size_t)(n + 1));
   w->clb = malloc(sizeof(double) * (size_t)(n + 1));
   w->cubf = malloc(sizeof(double) * (size_t)(n + 1));
   w->clbf = malloc(sizeof(double) * (size_t)(n + 1));
   w->cflag = calloc((size_t)(n + 1), 1);
   w->touched = malloc(sizeof(int32_t) * (size_t)(n + 1));
   w->front = malloc(sizeof(int32_t) * (size_t)(m + 1));
   w->next = malloc(sizeof(int32_t) * (size_t)(m + 1));
   w->rowstamp = calloc((size_t)(m + 1), sizeof(int32_t));
   w->oldlb = malloc(sizeof(double) * (size_t)(n + 1));
   w->oldub = malloc(sizeof(double) * (size_t)(n + 1));
   w->chg = malloc(sizeof(int32_t) * (size_t)(n + 1));
   w->dirty = calloc((size_t)(n + 1), 1);
   w->dirtylist = malloc(sizeof(int32_t) * (size_t)(n + 1));
   w->savelb = malloc(sizeof(double) * (size_t)(n + 1));
   w->saveub = malloc(sizeof(double) * (size_t)(n + 1));
   return (w->cub && w->clb && w->cubf && w->clbf && w->cflag && w->touched && w->front && w->next && w->rowstamp
      && w->oldlb && w->oldub && w->chg && w->dirty && w->dirtylist && w->savelb && w->saveub && w->rub && w->rlb
      && w->rflag && w->rmem && w->rord && w->rtmp) ? 0 : -1;
}

static void workFree(Work* w)
{
   free(w->cub); free(w->clb); free(w->cubf); free(w->clbf); free(w->cflag); free(w->touched);
   free(w->front); free(w->next); free(w->rowstamp); free(w->oldlb); free(w->oldub); free(w->chg);
   free(w->dirty); free(w->dirtylist); free(w->savelb); free(w->saveub);
   free(w->rub); free(w->rlb); free(w->rflag); free(w->rmem); free(w->rord); free(w->rtmp); free(w->startlb); free(w->startub);
}

static void newStamp(Work* w)
{
   if( ++w->stamp == INT32_MAX )
   {
      memset(w->rowstamp, 0, sizeof(int32_t) * (size_t)(w->P->m + 1));
      w->stamp = 1;
   }
}

static void pushNext(Work* w, int32_t row)
{
   if( w->rowstamp[row] != w->stamp )
   {
      w->rowstamp[row] = w->stamp;
      w->next[w->nnext++] = row;
   }
}

/* rows that a bound move of column j makes worth re-tightening: the boundstightened reset of
 * eventExecLinear, cons_linear.c:17239-17255 (lower bound up with a > 0 needs a finite rhs, with a < 0 a
 * finite lhs; upper bound down with a > 0 needs a finite lhs, with a < 0 a finite rhs) */
static void expandColumn(Work* w, int32_t j, int lbup, int ubdown)
{
   const lpo_problem* P = w->P;
   int64_t p;
   for( p = P->colptr[j]; p < P->colptr[j + 1]; ++p )
   {
      int32_t i = P->rowidx[p];
      double a = P->cvals[p];
      int rhsfin = !isInf(&w->s, P->rhs[i]);
      int lhsfin = !isInf(&w->s, -P->lhs[i]);
      int rel = 0;
      if( lbup )
         rel |= a > 0.0 ? rhsfin : lhsfin;
      if( ubdown )
         rel |= a > 0.0 ? lhsfin : rhsfin;
      if( rel )
         pushNext(w, i);
   }
}

static void candUb(Work* w, int32_t j, double v, int force)
{
   uint8_t bit = force ? 2 : 1;
   double* arr = force ? w->cubf : w->cub;
   if( w->cflag[j] == 0 )
      w->touched[w->ntouched++] = j;
   if( !(w->cflag[j] & bit) || v < arr[j] )
      arr[j] = v;
   w->cflag[j] |= bit;
}

static void candLb(Work* w, int32_t j, double v, int force)
{
   uint8_t bit = force ? 8 : 4;
   double* arr = force ? w->clbf : w->clb;
   if( w->cflag[j] == 0 )
      w->touched[w->ntouched++] = j;
   if( !(w->cflag[j] & bit) || v > arr[j] )
      arr[j] = v;
   w->cflag[j] |= bit;
}

/* candidate of the row being processed for its entry at position k */
static void rowUb(Work* w, int64_t k, double v, int force)
{
   uint8_t bit = force ? 2 : 1;
   if( !(w->rflag[k] & 3) || v < w->rub[k] )
      w->rub[k] = v;
   w->rflag[k] |= bit;
}

static void rowLb(Work* w, int64_t k, double v, int force)
{
   uint8_t bit = force ? 8 : 4;
   if( !(w->rflag[k] & 12) || v > w->rlb[k] )
      w->rlb[k] = v;
   w->rflag[k] |= bit;
}

/* SCIPvarIsBinary (var.c:23801-23810): integral with a global domain inside [0,1] */
static int isBinary(const Work* w, int32_t j, const double* lb, const double* ub)
{
   const double* gl = w->glb != NULL ? w->glb : lb;
   const double* gu = w->gub != NULL ? w->gub : ub;
   return w->P->isint[j] != 0 && gl[j] >= 0.0 && gu[j] <= 1.0;
}

/* order of a row's binaries during solving, consdataCompVarProp (cons_linear.c:3229-3254): larger |a| first, ties
 * by problem index (the column index).  SCIP counts |a| values within 1e-9 of each other as a tie; here |a| is
 * compared exactly, which orders the same whenever a row's distinct binary coefficients differ by more than
 * 1e-9 (a tolerance-based tie is not transitive, so it cannot define the order of a parallel reduction). */
static int binBefore(const lpo_problem* P, int64_t p, int64_t q)
{
   double a1 = fabs(P->vals[p]);
   double a2 = fabs(P->vals[q]);
   if( a1 != a2 )
      return a1 > a2;
   return P->colidx[p] < P->colidx[q];
}

/* the candidates of one row reach the columns as tightenBounds would apply them (cons_linear.c:7110-7138):
 * with the row's binaries visited in the order above, the first unfixed binary that gets no candidate ends
 * the visit of the binaries, so candidates of the binaries after it are dropped; other columns keep theirs */
static void commitRow(Work* w, const double* lb, const double* ub, int64_t p0, int64_t p1, lpo_result* res)
{
   const lpo_problem* P = w->P;
   int64_t blocker = -1;
   int64_t p;
   if( w->binskip )
   {
      for( p = p0; p < p1; ++p )
      {
         int32_t j = P->colidx[p];
         if( w->rflag[p - p0] != 0 || !isBinary(w, j, lb, ub) )
            continue;
         if( fabs(relDiff(ub[j], lb[j])) <= w->s.feastol )   /* SCIPisFeasEQ: fixed binaries never end it */
            continue;
         if( blocker < 0 || binBefore(P, p, blocker) )
            blocker = p;
      }
   }
   for( p = p0; p < p1; ++p )
   {
      uint8_t f = w->rflag[p - p0];
      int32_t j = P->colidx[p];
      if( f == 0 )
         continue;
      if( blocker >= 0 && binBefore(P, blocker, p) && isBinary(w, j, lb, ub) )
         continue;
      if( f & 3 )
      {
         candUb(w, j, w->rub[p - p0], (f & 2) != 0);
         res->candidates++;
      }
      if( f & 12 )
      {
         candLb(w, j, w->rlb[p - p0], (f & 8) != 0);
         res->candidates++;
      }
   }
}

/* ------------------------------------------------------------------ ranged rows (rangedRowPropagation,
 * cons_linear.c:5715-6695, with constraints/linear/rangedrowartcons = FALSE) */

/* the order of a row's entries on the global domain dl/du.  sorted (constraints/linear/sortvars, the order
 * tightenBounds sorts rows into, consdataCompVarProp, cons_linear.c:3191-3254): binaries first (larger |a| first,
 * ties by column), then integers (larger |a|*(ub-lb) first, ties by column), then continuous columns by column;
 * keys are compared exactly, as in binBefore.  Not sorted (the index order rows keep from presolving,
 * consdataCompVar, cons_linear.c:3152-3187): binaries, integers, continuous columns, each by column.  The column
 * index stands for SCIP's variable index, which follows it when the columns of each type come in index order. */
static int propBefore(const lpo_problem* P, const double* dl, const double* du, int sorted, int64_t p, int64_t q)
{
   int32_t jp = P->colidx[p];
   int32_t jq = P->colidx[q];
   int bp = P->isint[jp] != 0 && dl[jp] >= 0.0 && du[jp] <= 1.0;
   int bq = P->isint[jq] != 0 && dl[jq] >= 0.0 && du[jq] <= 1.0;
   double kp;
   double kq;
   if( bp != bq )
      return bp;
   if( bp && sorted )
      return binBefore(P, p, q);
   if( (P->isint[jp] != 0) != (P->isint[jq] != 0) )
      return P->isint[jp] != 0;
   if( P->isint[jp] == 0 || !sorted )
      return jp < jq;
   kp = fabs(P->vals[p] * (du[jp] - dl[jp]));
   kq = fabs(P->vals[q] * (du[jq] - dl[jq]));
   if( kp != kq )
      return kp > kq;
   return jp < jq;
}

static void orderMerge(const lpo_problem* P, const double* dl, const double* du, int sorted, int64_t p0, int32_t* a,
   int32_t* tmp, int64_t n)
{
   int64_t h;
   int64_t x;
   int64_t y;
   int64_t k;
   if( n < 2 )
      return;
   h = n / 2;
   orderMerge(P, dl, du, sorted, p0, a, tmp, h);
   orderMerge(P, dl, du, sorted, p0, a + h, tmp, n - h);
   for( x = 0, y = h, k = 0; k < n; ++k )
   {
      if( y >= n || (x < h && !propBefore(P, dl, du, sorted, p0 + a[y], p0 + a[x])) )
         tmp[k] = a[x++];
      else
         tmp[k] = a[y++];
   }
   memcpy(a, tmp, sizeof(int32_t) * (size_t)n);
}

static int64_t gcdLL(int64_t a, int64_t b)   /* SCIPcalcGreComDiv (misc.c:9197) computes the same value */
{
   while( b != 0 )
   {
      int64_t t = a % b;
      a = b;
      b = t;
   }
   return a;
}
/* (SCIP_Longint)(REALABS(val) + feastol) of cons_linear.c:5903/5944/6057; saturated where the cast would
 * overflow */
static int64_t coefInt(const Num* s, double v)
{
   double x = fabs(v) + s->feastol;
   return x >= 4.0e18 ? (int64_t)4000000000000000000LL : (int64_t)x;
}
static int isIntegral(const Num* s, double x) { return x - floor(x + s->eps) <= s->eps; }  /* EPSISINT */
static double epsFloor(const Num* s, double x) { return floor(x + s->eps); }              /* SCIPfloor */
static double epsCeil(const Num* s, double x) { return ceil(x - s->eps); }                /* SCIPceil */

/* each of the two solution-enumeration loops of cons_linear.c:6087-6139 runs at most this many times; a row
 * that needs more (its residual activity range spans over a million steps) yields no deduction */
#define RANGED_MAXIT (1 << 20)

static void logRanged(Work* w, int64_t row, int32_t col)
{
   lpo_log* g = w->log;
   if( g == NULL || g->rrow == NULL )
      return;
   if( g->rn < g->rcap )
   {
      g->rrow[g->rn] = (int32_t)row;
      g->rcol[g->rn] = col;
      g->rround[g->rn] = w->round;
   }
   g->rn++;
}

/* rangedRowPropagation for frontier row i from the round-start bounds; bound changes become forced
 * candidates (SCIPinferVarFixCons / SCIPinferVarLb/UbCons with force = TRUE).  Returns 1 on cutoff. */
static int rangedRow(Work* w, const double* lb, const double* ub, int64_t i, lpo_result* res)
{
   const lpo_problem* P = w->P;
   const Num* s = &w->s;
   const int64_t p0 = P->rowptr[i];
   const int64_t len = P->rowptr[i + 1] - p0;
   double fixedact = 0.0;
   int64_t nfixed = 0;
   int64_t ninf = 0;
   int64_t ncont = 0;
   int64_t first = -1;
   int gcdisone = 1;
   int possiblegcd = 1;
   double lhs;
   double rhs;
   int64_t k;
   int64_t gcd;
   double minact = 0.0;
   double maxact = 0.0;
   double g;
   double value;
   double minvalue = 0.0;
   double maxvalue = 0.0;
   int nsols = 0;
   int64_t gcdinf;
   int64_t it;
#define RPOS(k) (p0 + w->rord[k])
#define RFIXED(p) eq(s, lb[P->colidx[p]], ub[P->colidx[p]])
#define RQUAL(p) (P->isint[P->colidx[p]] != 0 && isIntegral(s, P->vals[p]) && !eq(s, fabs(P->vals[p]), 1.0))

   if( len < 3 || isInf(s, -P->lhs[i]) || isInf(s, P->rhs[i]) )
      return 0;
   /* the row in the order SCIP holds it when this runs (after tightenBounds, cons_linear.c:7042-7046), on the
    * global domain: with sortvars the round-start bounds at the root, where SCIP re-sorts a row whenever one of
    * its columns becomes binary (cons_linear.c:17327-17333); without, the bounds the call started from, which
    * the index order of presolving saw */
   for( k = 0; k < len; ++k )
      w->rord[k] = (int32_t)k;
   if( w->glb != NULL )
      orderMerge(P, w->glb, w->gub, w->binskip, p0, w->rord, w->rtmp, len);
   else if( w->startlb != NULL )
      orderMerge(P, w->startlb, w->startub, 0, p0, w->rord, w->rtmp, len);
   else
      orderMerge(P, lb, ub, w->binskip, p0, w->rord, w->rtmp, len);
   /* fixed activity, last entry first (cons_linear.c:5803-5814) */
   for( k = len - 1; k >= 0; --k )
   {
      int64_t p = RPOS(k);
      if( RFIXED(p) )
      {
         fixedact += lb[P->colidx[p]] * P->vals[p];
         ++nfixed;
      }
   }
   if( isHuge(s, fabs(fixedact)) )
      return 0;
   lhs = P->lhs[i] - fixedact;
   rhs = P->rhs[i] - fixedact;

   /* partition (cons_linear.c:5839-5958): rmem[k] = 1 for the entries that may lead to infeasibility */
   memset(w->rmem, 0, (size_t)len);
   k = -1;
   do
   {
      ++k;
      while( k < len && !RQUAL(RPOS(k)) )
      {
         int64_t p = RPOS(k);
         if( !RFIXED(p) )
         {
            if( P->isint[P->colidx[p]] == 0 )
               ++ncont;
            gcdisone = gcdisone && eq(s, fabs(P->vals[p]), 1.0);
            possiblegcd = 0;
            w->rmem[k] = 1;
            ++ninf;
            if( first < 0 )
               first = k;
         }
         ++k;
      }
   }
   while( k < len && RFIXED(RPOS(k)) );
   if( k == len || ncont + 2 > len - nfixed )
      return 0;
   gcd = coefInt(s, P->vals[RPOS(k)]);
   for( ; k < len; ++k )
   {
      int64_t p = RPOS(k);
      if( RFIXED(p) )
         continue;
      if( !RQUAL(p) )
      {
         if( P->isint[P->colidx[p]] == 0 )
            ++ncont;
         gcdisone = gcdisone && eq(s, fabs(P->vals[p]), 1.0);
         possiblegcd = 0;
         w->rmem[k] = 1;
         ++ninf;
         if( first < 0 )
            first = k;
      }
      else
      {
         int64_t t = gcdLL(gcd, coefInt(s, P->vals[p]));
         if( t == 1 )
         {
            w->rmem[k] = 1;
            ++ninf;
            if( first < 0 )
               first = k;
         }
         else
            gcd = t;
      }
   }
   if( ninf == 0 )
      return 0;

   /* activity bounds of those entries, last first (cons_linear.c:5975-6015) */
   for( k = len - 1; k >= 0; --k )
   {
      int64_t p;
      double v;
      double l;
      double u;
      int mininv = 0;
      int maxinv = 0;
      if( !w->rmem[k] )
         continue;
      p = RPOS(k);
      v = P->vals[p];
      l = lb[P->colidx[p]];
      u = ub[P->colidx[p]];
      if( isInf(s, -l) )
      {
         if( v < 0.0 )
            maxinv = 1;
         else
            mininv = 1;
      }
      else if( v < 0.0 )
         maxact += v * l;
      else
         minact += v * l;
      if( isInf(s, u) )
      {
         if( v > 0.0 )
            maxinv = 1;
         else
            mininv = 1;
      }
      else if( v > 0.0 )
         maxact += v * u;
      else
         minact += v * u;
      if( isHuge(s, -minact) )
         mininv = 1;
      if( isHuge(s, maxact) )
         maxinv = 1;
      if( mininv || maxinv )
         return 0;
   }

   /* no multiple of gcd between the sides (cons_linear.c:6033-6045) */
   g = (double)gcd;
   if( !isIntegral(s, (lhs - maxact) / g) && gt(s, epsCeil(s, (lhs - maxact) / g) * g, rhs - minact) )
   {
      logRanged(w, i, -1);
      return 1;
   }
   if( ncont != 0 )
      return 0;

   /* gcd of the other entries (cons_linear.c:6051-6064) */
   gcdinf = -1;
   if( possiblegcd )
   {
      for( k = len - 1; k >= 0; --k )
      {
         if( !w->rmem[k] )
            continue;
         gcdinf = gcdinf < 0 ? coefInt(s, P->vals[RPOS(k)]) : gcdLL(gcdinf, coefInt(s, P->vals[RPOS(k)]));
         if( gcdinf < 2 )
            break;
      }
   }
   else if( gcdisone )
      gcdinf = 1;
   if( gcdinf < 1 )
      return 0;

   /* feasible values of the other entries' activity (cons_linear.c:6076-6139) */
   value = epsCeil(s, minact - s->feastol);
   for( it = 0; le(s, value, maxact); ++it )
   {
      double value2;
      if( it >= RANGED_MAXIT )
         return 0;
      value2 = value + g * epsCeil(s, (lhs - value) / g);
      if( !ge(s, value2, lhs) )
         value2 += g;
      if( le(s, value2, rhs) )
      {
         ++nsols;
         if( nsols == 3 )
            break;
         if( nsols == 1 )
            minvalue = value;
         maxvalue = value;
      }
      value += (double)gcdinf;
   }
   if( nsols == 3 )
   {
      value = epsFloor(s, maxact + s->feastol);
      for( it = 0; ge(s, value, minact); ++it )
      {
         double value2;
         if( it >= RANGED_MAXIT )
            return 0;
         value2 = value + g * epsFloor(s, (rhs - value) / g);
         if( !le(s, value2, rhs) )
            value2 -= g;
         if( ge(s, value2, lhs) )
         {
            maxvalue = value;
            break;
         }
         value -= (double)gcdinf;
      }
   }
   if( nsols == 0 )
   {
      logRanged(w, i, -1);
      return 1;
   }

   if( ninf == 1 )
   {
      /* the single other entry (cons_linear.c:6160-6183 fixes it, :6296-6352 bounds it) */
      int64_t p = RPOS(first);
      int32_t j = P->colidx[p];
      double v = P->vals[p];
      if( nsols == 1 )
      {
         candLb(w, j, maxvalue / v, 1);
         candUb(w, j, maxvalue / v, 1);
         res->candidates += 2;
         logRanged(w, i, j);
      }
      else
      {
         double newlb = v < 0.0 ? maxvalue / v : minvalue / v;
         double newub = v < 0.0 ? minvalue / v : maxvalue / v;
         if( newlb > lb[j] )
         {
            candLb(w, j, newlb, 1);
            res->candidates++;
         }
         if( newub < ub[j] )
         {
            candUb(w, j, newub, 1);
            res->candidates++;
         }
         if( newlb > lb[j] || newub < ub[j] )
            logRanged(w, i, j);
      }
   }
   else if( ninf == len - nfixed - 1 )
   {
      /* the one unfixed entry outside them (cons_linear.c:6184-6283 fixes it, :6354-6552 bounds it) */
      int64_t p = -1;
      int32_t j;
      double v;
      for( k = 0; k < len; ++k )
         if( !w->rmem[k] && !RFIXED(RPOS(k)) )
         {
            p = RPOS(k);
            break;
         }
      if( p < 0 )
         return 0;
      j = P->colidx[p];
      v = P->vals[p];
      if( nsols == 1 )
      {
         double bound = v < 0.0 ? epsFloor(s, (lhs - maxvalue) / v) : epsCeil(s, (lhs - maxvalue) / v);
         candLb(w, j, bound, 1);
         candUb(w, j, bound, 1);
         res->candidates += 2;
         logRanged(w, i, j);
      }
      else
      {
         double newlb = v < 0.0 ? epsFloor(s, (rhs - minvalue) / v) : epsCeil(s, (lhs - maxvalue) / v);
         double newub = v < 0.0 ? epsFloor(s, (lhs - maxvalue) / v) : epsCeil(s, (rhs - minvalue) / v);
         if( newlb > lb[j] )
         {
            candLb(w, j, newlb, 1);
            res->candidates++;
         }
         if( newub < ub[j] )
         {
            candUb(w, j, newub, 1);
            res->candidates++;
         }
         if( newlb > lb[j] || newub < ub[j] )
            logRanged(w, i, j);
      }
   }
#undef RPOS
#undef RFIXED
#undef RQUAL
   return 0;
}

/* one frontier row: cutoff check of propagateCons (cons_linear.c:7718-7753), skip tests of tightenBounds
 * (cons_linear.c:7017-7083, canTightenBounds :5214-5238) and candidate bounds of tightenVarBounds
 * (:6700-6974, residual rule) or tightenVarBoundsEasy (:5380-5653, slack rule).  Returns 1 on cutoff. */
static int processRow(Work* w, const double* lb, const double* ub, int64_t i, lpo_result* res)
{
   const lpo_problem* P = w->P;
   const Num* s = &w->s;
   Act a;
   double lhs = P->lhs[i];
   double rhs = P->rhs[i];
   int64_t p0 = P->rowptr[i];
   int64_t p1 = P->rowptr[i + 1];
   int64_t p;
   int force;
   double maxactdelta;
   int easy;

   rowActivity(s, P, lb, ub, i, &a);
   res->rows++;
   res->nnz += p1 - p0;

   /* infeasibility with relaxed huge contributions (goodrelax TRUE), cons_linear.c:7718-7740 */
   {
      double minact, maxact;
      int t1, t2, f1, f2;
      getMinAct(s, &a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, 0.0, 1, &minact, &t1, &f1);
      getMaxAct(s, &a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, 1, &maxact, &t2, &f2);
      if( feasGt(s, minact, rhs) || feasLt(s, maxact, lhs) )
         return 1;
   }

   /* ranged rows (propagateCons, cons_linear.c:7694-7711): runs whatever tightenBounds' own tests decide */
   if( w->ranged && rangedRow(w, lb, ub, i, res) )
      return 1;

   /* canTightenBounds */
   if( a.minneginf + a.minposinf + a.minneghuge + a.minposhuge > 1
      && a.maxneginf + a.maxposinf + a.maxneghuge + a.maxposhuge > 1 )
      return 0;

   /* consdataRecomputeMaxActivityDelta, cons_linear.c:1542-1599 */
   maxactdelta = 0.0;
   for( p = p0; p < p1; ++p )
   {
      int32_t j = P->colidx[p];
      double d;
      if( isInf(s, -lb[j]) || isInf(s, ub[j]) )
      {
         maxactdelta = s->inf;
         break;
      }
      d = fabs(P->vals[p]) * (ub[j] - lb[j]);
      if( d > maxactdelta )
         maxactdelta = d;
   }
   if( feasZero(s, maxactdelta) )
      return 0;
   if( !isInf(s, maxactdelta) )
   {
      double minact, maxact, slack, surplus;
      int t1, t2, f1, f2;
      getMinAct(s, &a, a.minposinf, a.minneginf, a.minposhuge, a.minneghuge, 0.0, 0, &minact, &t1, &f1);
      getMaxAct(s, &a, a.maxposinf, a.maxneginf, a.maxposhuge, a.maxneghuge, 0.0, 0, &maxact, &t2, &f2);
      slack = (isInf(s, rhs) || f1) ? s->inf : rhs - minact;
      surplus = (isInf(s, -lhs) || f2) ? s->inf : maxact - lhs;
      if( le(s, maxactdelta, dmin(slack, surplus)) )
         return 0;
   }
   easy = lt(s, maxactdelta, s->maxeasy);
   force = (p1 - p0 == 1);
   memset(w->rflag, 0, (size_t)(p1 - p0));

   for( p = p0; p < p1; ++p )
   {
      int32_t j = P->colidx[p];
      double val = P->vals[p];
      double l = lb[j];
      double u = ub[j];
      int isint = P->isint[j] != 0;

      if( easy )
      {
         /* tightenVarBoundsEasy; the finite part of the activity is QUAD_TO_DBL(minactivity) */
         double minact = a.minhi + a.minlo;
         double maxact = a.maxhi + a.maxlo;
         if( !isInf(s, rhs) )
         {
            double slack, alpha;
            if( feasLt(s, rhs, minact) )
               return 1;
            slack = rhs - minact;
            if( !positive(s, slack) )
               slack = 0.0;
            alpha = val > 0.0 ? val * (u - l) : val * (l - u);
            if( sumGt(s, alpha, slack) || (force && gt(s, alpha, slack)) )
            {
               if( val > 0.0 )
               {
                  /* tightenVarUb, cons_linear.c:5242-5304 */
                  double nb = adjUb(s, isint, l + slack / val);
                  if( force || ubBetter(s, nb, l, u) )
                  {
                     rowUb(w, p - p0, nb, force);
                  }
               }
               else
               {
                  /* tightenVarLb, cons_linear.c:5307-5376 */
                  double nb = adjLb(s, isint, u + slack / val);
                  if( force || lbBetter(s, nb, l, u) )
                  {
                     rowLb(w, p - p0, nb, force);
                  }
               }
            }
         }
         if( !isInf(s, -lhs) )
         {
            double slack, alpha;
            if( feasLt(s, maxact, lhs) )
               return 1;
            slack = maxact - lhs;
            if( !positive(s, slack) )
               slack = 0.0;
            alpha = val > 0.0 ? val * (u - l) : val * (l - u);
            if( sumGt(s, alpha, slack) || (force && gt(s, alpha, slack)) )
            {
               if( val > 0.0 )
               {
                  double nb = adjLb(s, isint, u - slack / val);
                  if( force || lbBetter(s, nb, l, u) )
                  {
                     rowLb(w, p - p0, nb, force);
                  }
               }
               else
               {
                  double nb = adjUb(s, isint, l - slack / val);
                  if( force || ubBetter(s, nb, l, u) )
                  {
                     rowUb(w, p - p0, nb, force);
                  }
               }
            }
         }
         continue;
      }

      {
         /* tightenVarBounds, residual rule */
         double minres, maxres;
         int mintight, maxtight, mininf, maxinf;
         residuals(s, &a, val, l, u, &minres, &maxres, &mintight, &maxtight, &mininf, &maxinf);

         if( val > 0.0 )
         {
            if( !mininf && !isInf(s, rhs) && mintight && (lt(s, fabs(rhs), 1.0) || !eq(s, minres / rhs, 1.0)) )
            {
               double newub = (rhs - minres) / val;
               if( !isInf(s, newub)
                  && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u)) )
               {
                  int unreliable = updateUnreliable(s, minres, a.minhi + a.minlo);
                  if( unreliable )
                  {
                     minres = reliableResidual(P, lb, ub, i, p, 1);
                     newub = (rhs - minres) / val;
                     unreliable = isInf(s, -minres) || (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) || !isint)
                        && (!force || !lt(s, newub, u)));
                  }
                  if( !unreliable )
                  {
                     rowUb(w, p - p0, newub, force);
                  }
               }
            }
            if( !maxinf && !isInf(s, -lhs) && maxtight && (lt(s, fabs(lhs), 1.0) || !eq(s, maxres / lhs, 1.0)) )
            {
               double newlb = (lhs - maxres) / val;
               if( !isInf(s, -newlb)
                  && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u)) )
               {
                  int skip = 0;
                  if( updateUnreliable(s, maxres, a.maxhi + a.maxlo) )
                  {
                     maxres = reliableResidual(P, lb, ub, i, p, 0);
                     newlb = (lhs - maxres) / val;
                     skip = isInf(s, maxres) || (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint)
                        && (!force || !gt(s, newlb, l)));
                  }
                  if( !skip )
                  {
                     rowLb(w, p - p0, newlb, force);
                  }
               }
            }
         }
         else
         {
            if( !mininf && !isInf(s, rhs) && mintight && (lt(s, fabs(rhs), 1.0) || !eq(s, minres / rhs, 1.0)) )
            {
               double newlb = (rhs - minres) / val;
               if( !isInf(s, -newlb)
                  && ((force && gt(s, newlb, l)) || (isint && feasGt(s, newlb, l)) || lbBetter(s, newlb, l, u)) )
               {
                  int unreliable = updateUnreliable(s, minres, a.minhi + a.minlo);
                  if( unreliable )
                  {
                     minres = reliableResidual(P, lb, ub, i, p, 1);
                     newlb = (rhs - minres) / val;
                     unreliable = isInf(s, -minres) || (!lbBetter(s, newlb, l, u) && (!feasGt(s, newlb, l) || !isint)
                        && (!force || !gt(s, newlb, l)));
                  }
                  if( !unreliable )
                  {
                     rowLb(w, p - p0, newlb, force);
                  }
               }
            }
            if( !maxinf && !isInf(s, -lhs) && maxtight && (lt(s, fabs(lhs), 1.0) || !eq(s, maxres / lhs, 1.0)) )
            {
               double newub = (lhs - maxres) / val;
               if( !isInf(s, newub)
                  && ((force && lt(s, newub, u)) || (isint && feasLt(s, newub, u)) || ubBetter(s, newub, l, u)) )
               {
                  int skip = 0;
                  if( updateUnreliable(s, maxres, a.maxhi + a.maxlo) )
                  {
                     maxres = reliableResidual(P, lb, ub, i, p, 0);
                     newub = (lhs - maxres) / val;
                     /* the upper-bound branch for a < 0 combines its conditions with && (cons_linear.c:6936-6938) */
                     skip = isInf(s, maxres) || (!ubBetter(s, newub, l, u) && (!feasLt(s, newub, u) && !isint)
                        && (!force || !lt(s, newub, u)));
                  }
                  if( !skip )
                  {
                     rowUb(w, p - p0, newub, force);
                  }
               }
            }
         }
      }
   }
   commitRow(w, lb, ub, p0, p1, res);
   return 0;
}

/* acceptance of the best candidates of one column: SCIPinferVarUbCons / SCIPinferVarLbCons
 * (scip_var.c:7071-7112 / 6965-7006) against the round-start bounds, upper bound first and the lower
 * bound against the new upper bound.  Returns 1 on cutoff. */
static int applyColumn(Work* w, int32_t j, double* lb, double* ub, int* lbup, int* ubdown)
{
   const Num* s = &w->s;
   const lpo_problem* P = w->P;
   int isint = P->isint[j] != 0;
   double l = lb[j];
   double u = ub[j];
   double nu = u;
   double nl = l;
   uint8_t f = w->cflag[j];
   int k;

   for( k = 0; k < 2; ++k )
   {
      int force = (k == 1);
      double c;
      if( !(f & (force ? 2 : 1)) )
         continue;
      c = adjUb(s, isint, force ? w->cubf[j] : w->cub[j]);
      if( isInf(s, -c) || feasLt(s, c, l) )
         return 1;
      c = dmax(c, l);
      if( force ? !ge(s, c, u) : ubBetter(s, c, l, u) )
         nu = dmin(nu, c);
   }
   for( k = 0; k < 2; ++k )
   {
      int force = (k == 1);
      double c;
      if( !(f & (force ? 8 : 4)) )
         continue;
      c = adjLb(s, isint, force ? w->clbf[j] : w->clb[j]);
      if( isInf(s, c) || feasGt(s, c, nu) )
         return 1;
      c = dmin(c, nu);
      if( force ? !le(s, c, l) : lbBetter(s, c, l, nu) )
         nl = dmax(nl, c);
   }
   *lbup = nl > l;
   *ubdown = nu < u;
   lb[j] = nl;
   ub[j] = nu;
   return 0;
}

static void markDirty(Work* w, int32_t j, double l, double u)
{
   if( !w->dirty[j] )
   {
      w->dirty[j] = 1;
      w->dirtylist[w->ndirty++] = j;
      w->savelb[j] = l;
      w->saveub[j] = u;
   }
}

/* the fixpoint loop over the frontier in w->next (already stamped) */
static int fixpoint(Work* w, double* lb, double* ub, lpo_result* res, int track)
{
   int32_t round;
   res->cutoff = 0;
   res->status = 0;
   res->rounds = 0;
   for( round = 0; w->nnext > 0; ++round )
   {
      int64_t k;
      int32_t* t;
      if( round >= w->maxrounds )
      {
         res->status = 2;
         return 0;
      }
      t = w->front; w->front = w->next; w->next = t;
      w->nfront = w->nnext;
      w->nnext = 0;
      res->rounds = round + 1;
      w->round = round;

      w->ntouched = 0;
      for( k = 0; k < w->nfront; ++k )
      {
         if( processRow(w, lb, ub, w->front[k], res) )
         {
            int64_t q;
            for( q = 0; q < w->ntouched; ++q )
               w->cflag[w->touched[q]] = 0;
            res->cutoff = 1;
            res->status = 1;
            return 1;
         }
      }

      newStamp(w);
      for( k = 0; k < w->ntouched; ++k )
      {
         int32_t j = w->touched[k];
         int lbup = 0, ubdown = 0;
         double l0 = lb[j], u0 = ub[j];
         if( applyColumn(w, j, lb, ub, &lbup, &ubdown) )
         {
            int64_t q;
            for( q = 0; q < w->ntouched; ++q )
               w->cflag[w->touched[q]] = 0;
            res->cutoff = 1;
            res->status = 1;
            return 1;
         }
         w->cflag[j] = 0;
         if( lbup || ubdown )
         {
            if( track )
               markDirty(w, j, l0, u0);
            res->changes += lbup + ubdown;
            if( w->log != NULL )
            {
               lpo_log* g = w->log;
               if( g->n < g->cap )
               {
                  g->col[g->n] = j;
                  g->round[g->n] = round;
                  g->lb[g->n] = lb[j];
                  g->ub[g->n] = ub[j];
               }
               g->n++;
            }
            expandColumn(w, j, lbup, ubdown);
         }
      }
   }
   return 0;
}

int lpo_propagate(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub,
   int64_t nseed, const int32_t* seedcols, const double* oldlb, const double* oldub, const double* glb,
   const double* gub, lpo_result* res)
{
   return lpo_propagate_logged(prob, par, lb, ub, nseed, seedcols, oldlb, oldub, glb, gub, res, NULL);
}

int lpo_propagate_logged(const lpo_problem* prob, const lpo_params* par, double* lb, double* ub,
   int64_t nseed, const int32_t* seedcols, const double* oldlb, const double* oldub, const double* glb,
   const double* gub, lpo_result* res, lpo_log* log)
{
   Work w;
   int64_t k;
   memset(res, 0, sizeof(*res));
   if( workInit(&w, prob, par) != 0 )
   {
      workFree(&w);
      return -1;
   }
   w.glb = glb;
   w.gub = gub;
   w.log = log;
   /* without a global domain, rows keep the index order of the bounds the call starts from */
   if( glb == NULL && w.ranged && !w.binskip )
   {
      w.startlb = malloc(sizeof(double) * (size_t)(prob->n > 0 ? prob->n : 1));
      w.startub = malloc(sizeof(double) * (size_t)(prob->n > 0 ? prob->n : 1));
      if( w.startlb == NULL || w.startub == NULL )
      {
         workFree(&w);
         return -1;
      }
      memcpy(w.startlb, lb, sizeof(double) * (size_t)prob->n);
      memcpy(w.startub, ub, sizeof(double) * (size_t)prob->n);
   }

   if( log != NULL )
   {
      log->n = 0;
      log->rn = 0;
   }
   newStamp(&w);
   w.nnext = 0;
   if( seedcols == NULL )
   {
      for( k = 0; k < prob->m; ++k )
         pushNext(&w, (int32_t)k);
   }
   else
   {
      for( k = 0; k < nseed; ++k )
      {
         int32_t j = seedcols[k];
         expandColumn(&w, j, lb[j] > oldlb[k], ub[j] < oldub[k]);
      }
   }
   fixpoint(&w, lb, ub, res, 0);
   workFree(&w);
   return 0;
}

typedef struct
{
   const lpo_problem* P;
   const lpo_params* par;
   const double* baselb;
   const double* baseub;
   int64_t k0, k1;
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
   lpo_result tot;
   int err;
} NodeJob;

static void* nodeWorker(void* arg)
{
   NodeJob* J = arg;
   const lpo_problem* P = J->P;
   Work w;
   double* lb;
   double* ub;
   int64_t k;

   memset(&J->tot, 0, sizeof(J->tot));
   lb = malloc(sizeof(double) * (size_t)P->n);
   ub = malloc(sizeof(double) * (size_t)P->n);
   if( lb == NULL || ub == NULL || workInit(&w, P, J->par) != 0 )
   {
      J->err = -1;
      free(lb);
      free(ub);
      return NULL;
   }
   memcpy(lb, J->baselb, sizeof(double) * (size_t)P->n);
   memcpy(ub, J->baseub, sizeof(double) * (size_t)P->n);
   w.glb = J->baselb;
   w.gub = J->baseub;

   for( k = J->k0; k < J->k1; ++k )
   {
      lpo_result r;
      int64_t q;
      int cut = 0;
      memset(&r, 0, sizeof(r));
      newStamp(&w);
      w.nnext = 0;
      w.ndirty = 0;
      for( q = J->ptr[k]; q < J->ptr[k + 1]; ++q )
      {
         int32_t j = J->chg_col[q];
         double nl = J->chg_lb[q];
         double nu = J->chg_ub[q];
         double l0 = lb[j], u0 = ub[j];
         if( nl > u0 || nu < l0 || nl > nu )
            cut = 1;
         else
         {
            /* branching bound changes tighten only (SCIPchgVarLb/UbProbing semantics); a column named again
             * tightens further, and its bounds crossing cuts the node off */
            if( nl > l0 || nu < u0 )
            {
               markDirty(&w, j, l0, u0);
               if( nl > l0 )
                  lb[j] = nl;
               if( nu < u0 )
                  ub[j] = nu;
               if( lb[j] > ub[j] )
                  cut = 1;
            }
         }
      }
      if( !cut )
      {
         for( q = J->ptr[k]; q < J->ptr[k + 1]; ++q )
         {
            int32_t j = J->chg_col[q];
            if( w.dirty[j] )
               expandColumn(&w, j, lb[j] > w.savelb[j], ub[j] < w.saveub[j]);
         }
         cut = fixpoint(&w, lb, ub, &r, 1);
      }
      else
      {
         r.cutoff = 1;
         r.status = 1;
      }
      J->out_cutoff[k] = (int8_t)cut;
      J->out_rounds[k] = r.rounds;
      {
         int32_t cnt = 0;
         if( !cut )
         {
            for( q = 0; q < w.ndirty; ++q )
            {
               int32_t j = w.dirtylist[q];
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
      /* restore the base bounds */
      for( q = 0; q < w.ndirty; ++q )
      {
         int32_t j = w.dirtylist[q];
         lb[j] = J->baselb[j];
         ub[j] = J->baseub[j];
         w.dirty[j] = 0;
      }
      w.ndirty = 0;
      J->tot.rows += r.rows;
      J->tot.nnz += r.nnz;
      J->tot.candidates += r.candidates;
      J->tot.changes += r.changes;
      J->tot.cutoff += cut;
      if( r.rounds > J->tot.rounds )
         J->tot.rounds = r.rounds;
   }
   workFree(&w);
   free(lb);
   free(ub);
   return NULL;
}

int lpo_propagate_nodes(const lpo_problem* prob, const lpo_params* par, const double* baselb, const double* baseub,
   int64_t nnodes, const int64_t* ptr, const int32_t* chg_col, const double* chg_lb, const double* chg_ub,
   int8_t* out_cutoff, int32_t* out_rounds, int32_t* out_n, int32_t* out_col, double* out_lb, double* out_ub,
   int32_t cap, int32_t nthreads, lpo_result* total)
{
   NodeJob* jobs;
   pthread_t* th;
   int t;
   int err = 0;
   if( nthreads <= 0 )
      nthreads = 1;
   if( nthreads > nnodes && nnodes > 0 )
      nthreads = (int32_t)nnodes;
   jobs = calloc((size_t)nthreads, sizeof(NodeJob));
   th = calloc((size_t)nthreads, sizeof(pthread_t));
   if( jobs == NULL || th == NULL )
   {
      free(jobs);
      free(th);
      return -1;
   }
   for( t = 0; t < nthreads; ++t )
   {
      NodeJob* J = &jobs[t];
      J->P = prob; J->par = par; J->baselb = baselb; J->baseub = baseub;
      J->k0 = nnodes * t / nthreads;
      J->k1 = nnodes * (t + 1) / nthreads;
      J->ptr = ptr; J->chg_col = chg_col; J->chg_lb = chg_lb; J->chg_ub = chg_ub;
      J->out_cutoff = out_cutoff; J->out_rounds = out_rounds; J->out_n = out_n;
      J->out_col = out_col; J->out_lb = out_lb; J->out_ub = out_ub; J->cap = cap;
   }
   if( nthreads == 1 )
      nodeWorker(&jobs[0]);
   else
   {
      for( t = 0; t < nthreads; ++t )
         pthread_create(&th[t], NULL, nodeWorker, &jobs[t]);
      for( t = 0; t < nthreads; ++t )
         pthread_join(th[t], NULL);
   }
   if( total != NULL )
      memset(total, 0, sizeof(*total));
   for( t = 0; t < nthreads; ++t )
   {
      if( jobs[t].err )
         err = jobs[t].err;
      if( total != NULL )
      {
         total->rows += jobs[t].tot.rows;
         total->nnz += jobs[t].tot.nnz;
         total->candidates += jobs[t].tot.candidates;
         total->changes += jobs[t].tot.changes;
         total->cutoff += jobs[t].tot.cutoff;
         if( jobs[t].tot.rounds > total->rounds )
            total->rounds = jobs[t].tot.rounds;
      }
   }
   free(jobs);
   free(th);
   return err;
}
