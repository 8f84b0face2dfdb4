/* Test infrastructure only: numerics and activity helpers shared by the two CPU restatements of SCIP's
 * cons_linear propagation (linprop_oracle.c: rounds; linprop_seq.c: SCIP's own one-row-at-a-time order).
 * Every function restates the SCIP function cited beside it. */
#ifndef LPO_COMMON_H
#define LPO_COMMON_H

#include "linprop_oracle.h"

#include <math.h>
#include <string.h>
/* ------------------------------------------------------------------ numerics (src/scip/def.h:192-204,
 * set.c:6824-6845, 7025-7050, 7425-7460, 7705-7753, 8032-8046, misc.c:11162-11176) */
typedef struct
{
   double inf, eps, sumeps, feastol, huge, bstreps, recomp, maxeasy;
} Num;

static inline int isInf(const Num* s, double x) { return x >= s->inf; }                    /* SCIPsetIsInfinity */
static inline int isHuge(const Num* s, double x) { return x >= s->huge; }                  /* SCIPsetIsHugeValue */
static inline int lt(const Num* s, double a, double b) { return a - b < -s->eps; }         /* EPSLT */
static inline int le(const Num* s, double a, double b) { return a - b <= s->eps; }         /* EPSLE */
static inline int gt(const Num* s, double a, double b) { return a - b > s->eps; }          /* EPSGT */
static inline int ge(const Num* s, double a, double b) { return a - b >= -s->eps; }        /* EPSGE */
static inline int eq(const Num* s, double a, double b) { return fabs(a - b) <= s->eps; }   /* EPSEQ */
static inline int sumGt(const Num* s, double a, double b) { return a - b > s->sumeps; }    /* SCIPsetIsSumGT */
static inline int positive(const Num* s, double a) { return a > s->eps; }                  /* SCIPsetIsPositive */
static inline int feasZero(const Num* s, double a) { return fabs(a) <= s->feastol; }       /* SCIPsetIsFeasZero */

static inline double relDiff(double a, double b)                                           /* SCIPrelDiff */
{
   double q = fabs(a);
   if( fabs(b) > q )
      q = fabs(b);
   if( 1.0 > q )
      q = 1.0;
   return (a - b) / q;
}
static inline int feasLt(const Num* s, double a, double b) { return relDiff(a, b) < -s->feastol; }
static inline int feasGt(const Num* s, double a, double b) { return relDiff(a, b) > s->feastol; }
static inline double feasFloor(const Num* s, double x) { return floor(x + s->feastol); }  /* EPSFLOOR */
static inline double feasCeil(const Num* s, double x) { return ceil(x - s->feastol); }    /* EPSCEIL */

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* SCIPsetIsLbBetter / SCIPsetIsUbBetter, set.c:7711-7753 */
static inline int lbBetter(const Num* s, double newlb, double oldlb, double oldub)
{
   if( oldlb < 0.0 && newlb >= 0.0 )
      return 1;
   return newlb - oldlb > s->bstreps * dmax(dmin(oldub - oldlb, fabs(oldlb)), 1e-3);
}
static inline int ubBetter(const Num* s, double newub, double oldlb, double oldub)
{
   if( oldub > 0.0 && newub <= 0.0 )
      return 1;
   return newub - oldub < -(s->bstreps * dmax(dmin(oldub - oldlb, fabs(oldub)), 1e-3));
}

/* SCIPsetIsUpdateUnreliable, set.c:8032-8046 */
static inline int updateUnreliable(const Num* s, double newvalue, double oldvalue)
{
   double quot = fabs(oldvalue) / dmax(fabs(newvalue), s->eps);
   return quot >= s->recomp;
}

/* adjustedLb / adjustedUb, var.c:1957-2020 */
static inline double adjLb(const Num* s, int isint, double lb)
{
   if( lb < 0.0 && isInf(s, -lb) )
      return -s->inf;
   if( lb > 0.0 && isInf(s, lb) )
      return s->inf;
   if( isint )
      return feasCeil(s, lb);
   if( lb > 0.0 && lb < s->eps )
      return 0.0;
   return lb;
}
static inline double adjUb(const Num* s, int isint, double ub)
{
   if( ub > 0.0 && isInf(s, ub) )
      return s->inf;
   if( ub < 0.0 && isInf(s, -ub) )
      return -s->inf;
   if( isint )
      return feasFloor(s, ub);
   if( ub < 0.0 && ub > -s->eps )
      return 0.0;
   return ub;
}

/* SCIPdbldblSum21 (dbldblarith.h:154-190): (hi,lo) + b, TwoSum on the high part, low parts added */
static inline void sum21(double* hi, double* lo, double b)
{
   double s = *hi + b;
   double bb = s - *hi;
   double err = (*hi - (s - bb)) + (b - bb);
   *lo = err + *lo;
   *hi = s;
}

static inline void numFrom(const lpo_params* p, Num* s)
{
   s->inf = p->infinity;
   s->eps = p->epsilon;
   s->sumeps = p->sumepsilon;
   s->feastol = p->feastol;
   s->huge = p->hugeval;
   s->bstreps = p->boundstreps;
   s->recomp = p->recompfac;
   s->maxeasy = p->maxeasyactivitydelta;
}


/* ------------------------------------------------------------------ row activity */
typedef struct
{
   double minhi, minlo, maxhi, maxlo;
   int minposinf, minneginf, minposhuge, minneghuge;
   int maxposinf, maxneginf, maxposhuge, maxneghuge;
} Act;

/* one contribution val*bound to an activity: infinite bounds and huge products are counted, the rest
 * summed (consdataUpdateActivities with oldbound 0, cons_linear.c:1772-1945, as used by
 * consdataCalcActivities/consdataUpdateAddCoef, cons_linear.c:2092-2339) */
static inline void addContribution(const Num* s, double val, double bound, double* hi, double* lo, int* posinf,
   int* neginf, int* poshuge, int* neghuge)
{
   if( isInf(s, fabs(bound)) )
   {
      if( (val > 0.0) == (bound > 0.0) )
         ++(*posinf);
      else
         ++(*neginf);
   }
   else
   {
      double c = val * bound;
      if( isHuge(s, fabs(c)) )
      {
         if( c > 0.0 )
            ++(*poshuge);
         else
            ++(*neghuge);
      }
      else if( c != 0.0 )
         sum21(hi, lo, c);
   }
}

static inline void addTerm(const Num* s, Act* a, double v, double l, double u)
{
   addContribution(s, v, v > 0.0 ? l : u, &a->minhi, &a->minlo, &a->minposinf, &a->minneginf, &a->minposhuge,
      &a->minneghuge);
   addContribution(s, v, v > 0.0 ? u : l, &a->maxhi, &a->maxlo, &a->maxposinf, &a->maxneginf, &a->maxposhuge,
      &a->maxneghuge);
}

/* partial activity b merged into a: b's high word through the compensated sum, low words added */
static inline void actMerge(Act* a, const Act* b)
{
   sum21(&a->minhi, &a->minlo, b->minhi);
   a->minlo = a->minlo + b->minlo;
   sum21(&a->maxhi, &a->maxlo, b->maxhi);
   a->maxlo = a->maxlo + b->maxlo;
   a->minposinf += b->minposinf; a->minneginf += b->minneginf;
   a->minposhuge += b->minposhuge; a->minneghuge += b->minneghuge;
   a->maxposinf += b->maxposinf; a->maxneginf += b->maxneginf;
   a->maxposhuge += b->maxposhuge; a->maxneghuge += b->maxneghuge;
}

/* getMinActivity, cons_linear.c:2345-2436 */
static inline void getMinAct(const Num* s, const Act* a, int posinf, int neginf, int poshuge, int neghuge, double delta,
   int goodrelax, double* val, int* tight, int* settoinf)
{
   if( neginf > 0 )
   {
      *val = -s->inf; *settoinf = 1; *tight = (posinf == 0);
   }
   else if( posinf > 0 )
   {
      *val = s->inf; *settoinf = 1; *tight = 1;
   }
   else if( neghuge > 0 || (poshuge > 0 && !goodrelax) )
   {
      *val = -s->inf; *settoinf = 1; *tight = 0;
   }
   else
   {
      double hi = a->minhi;
      double lo = a->minlo;
      sum21(&hi, &lo, -delta);
      if( poshuge > 0 )
      {
         sum21(&hi, &lo, poshuge * s->huge);
         *tight = 0;
      }
      else
         *tight = 1;
      *val = hi + lo;
      *settoinf = 0;
   }
}

/* getMaxActivity, cons_linear.c:2441-2529 */
static inline void getMaxAct(const Num* s, const Act* a, int posinf, int neginf, int poshuge, int neghuge, double delta,
   int goodrelax, double* val, int* tight, int* settoinf)
{
   if( posinf > 0 )
   {
      *val = s->inf; *settoinf = 1; *tight = (neginf == 0);
   }
   else if( neginf > 0 )
   {
      *val = -s->inf; *settoinf = 1; *tight = 1;
   }
   else if( poshuge > 0 || (neghuge > 0 && !goodrelax) )
   {
      *val = s->inf; *settoinf = 1; *tight = 0;
   }
   else
   {
      double hi = a->maxhi;
      double lo = a->maxlo;
      sum21(&hi, &lo, -delta);
      if( neghuge > 0 )
      {
         sum21(&hi, &lo, -neghuge * s->huge);
         *tight = 0;
      }
      else
         *tight = 1;
      *val = hi + lo;
      *settoinf = 0;
   }
}

/* consdataGetActivityResiduals, cons_linear.c:2661-2806 (goodrelax FALSE as in tightenVarBounds) */
static inline void residuals(const Num* s, const Act* a, double val, double lb, double ub, double* minres, double* maxres,
   int* mintight, int* maxtight, int* mininf, int* maxinf)
{
   double minb, maxb, absval;
   if( val > 0.0 )
   {
      minb = lb; maxb = ub; absval = val;
   }
   else
   {
      minb = -ub; maxb = -lb; absval = -val;
   }
   if( isInf(s, minb) )
      getMinAct(s, a, a->minposinf - 1, a->minneginf, a->minposhuge, a->minneghuge, 0.0, 0, minres, mintight, mininf);
   else if( isInf(s, -minb) )
      getMinAct(s, a, a->minposinf, a->minneginf - 1, a->minposhuge, a->minneghuge, 0.0, 0, minres, mintight, mininf);
   else if( isHuge(s, minb * absval) )
      getMinAct(s, a, a->minposinf, a->minneginf, a->minposhuge - 1, a->minneghuge, 0.0, 0, minres, mintight, mininf);
   else if( isHuge(s, -minb * absval) )
      getMinAct(s, a, a->minposinf, a->minneginf, a->minposhuge, a->minneghuge - 1, 0.0, 0, minres, mintight, mininf);
   else
      getMinAct(s, a, a->minposinf, a->minneginf, a->minposhuge, a->minneghuge, absval * minb, 0, minres, mintight, mininf);

   if( isInf(s, -maxb) )
      getMaxAct(s, a, a->maxposinf, a->maxneginf - 1, a->maxposhuge, a->maxneghuge, 0.0, 0, maxres, maxtight, maxinf);
   else if( isInf(s, maxb) )
      getMaxAct(s, a, a->maxposinf - 1, a->maxneginf, a->maxposhuge, a->maxneghuge, 0.0, 0, maxres, maxtight, maxinf);
   else if( isHuge(s, absval * maxb) )
      getMaxAct(s, a, a->maxposinf, a->maxneginf, a->maxposhuge - 1, a->maxneghuge, 0.0, 0, maxres, maxtight, maxinf);
   else if( isHuge(s, -absval * maxb) )
      getMaxAct(s, a, a->maxposinf, a->maxneginf, a->maxposhuge, a->maxneghuge - 1, 0.0, 0, maxres, maxtight, maxinf);
   else
      getMaxAct(s, a, a->maxposinf, a->maxneginf, a->maxposhuge, a->maxneghuge, absval * maxb, 0, maxres, maxtight, maxinf);
}

#endif
