/* Reasons for the gpulinear propagator's bound changes (see gpulinear_reason.h). */
#include "gpulinear_reason.h"

#include <math.h>
#include <stdlib.h>

void gpl_build_columns(int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx, int64_t* colptr,
   int32_t* rowidx, int64_t* rowpos)
{
   int64_t i;
   int64_t p;
   int64_t j;
   for( j = 0; j <= n; ++j )
      colptr[j] = 0;
   for( p = 0; p < rowptr[m]; ++p )
      colptr[colidx[p] + 1]++;
   for( j = 0; j < n; ++j )
      colptr[j + 1] += colptr[j];
   /* rows in increasing order within each column: a stable pass over the rows */
   {
      int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
      for( j = 0; j < n; ++j )
         fill[j] = colptr[j];
      for( i = 0; i < m; ++i )
      {
         for( p = rowptr[i]; p < rowptr[i + 1]; ++p )
         {
            int64_t q = fill[colidx[p]]++;
            rowidx[q] = (int32_t)i;
            rowpos[q] = p - rowptr[i];
         }
      }
      free(fill);
   }
}

/* addConflictBounds (cons_linear.c:4799-4970) for row r, whose entry at CSR position pinf is the inferred column
 * (pinf < 0: no inferred column, the row itself is infeasible): for an integral column, or none, bounds are added in
 * row order only until the residual capacity left by the other columns' global bounds is used up; otherwise every
 * other column's responsible bound is added. */
static int addBounds(const gpl_rows* R, const gpl_num* num, const gpl_io* io, int64_t r, int64_t pinf, int32_t col,
   int reasonisrhs)
{
   const double a = pinf >= 0 ? R->vals[pinf] : 0.0;
   int64_t p;
   /* without an inferred column (an infeasible row) the capacity logic applies as for an integral one */
   if( pinf < 0 || R->isint[col] )
   {
      double gres = 0.0;
      int finite = 1;
      for( p = R->rowptr[r]; p < R->rowptr[r + 1]; ++p )
      {
         double v = R->vals[p];
         int32_t k = R->colidx[p];
         double b;
         if( p == pinf )
            continue;
         b = (reasonisrhs == (v > 0.0)) ? io->glb(io->ud, k) : io->gub(io->ud, k);
         if( fabs(b) >= num->infinity )
         {
            finite = 0;
            break;
         }
         gres += v * b;
      }
      if( finite )
      {
         double rescap = (reasonisrhs ? R->rhs[r] : R->lhs[r]) - gres;
         if( pinf >= 0 )
         {
            if( reasonisrhs == (a > 0.0) )
               rescap -= a * (io->ubafter(io->ud, col) + 1.0);
            else
               rescap -= a * (io->lbafter(io->ud, col) - 1.0);
         }
         for( p = R->rowptr[r]; p < R->rowptr[r + 1]; ++p )
         {
            double v = R->vals[p];
            int32_t k = R->colidx[p];
            if( p == pinf || fabs(v) <= num->epsilon )
               continue;
            if( (reasonisrhs && rescap < -num->feastol) || (!reasonisrhs && rescap > num->feastol) )
               break;
            if( reasonisrhs == (v > 0.0) )
            {
               if( io->addlb(io->ud, k) )
                  return -1;
               rescap -= v * (io->lb(io->ud, k) - io->glb(io->ud, k));
            }
            else
            {
               if( io->addub(io->ud, k) )
                  return -1;
               rescap -= v * (io->ub(io->ud, k) - io->gub(io->ud, k));
            }
         }
         return 0;
      }
   }
   for( p = R->rowptr[r]; p < R->rowptr[r + 1]; ++p )
   {
      double v = R->vals[p];
      int32_t k = R->colidx[p];
      if( p == pinf || fabs(v) <= num->epsilon )
         continue;
      if( (reasonisrhs == (v > 0.0)) ? io->addlb(io->ud, k) : io->addub(io->ud, k) )
         return -1;
   }
   return 0;
}

int64_t gpl_explain(const gpl_rows* R, const gpl_num* num, const gpl_io* io, int32_t col, int islower, double bound)
{
   int64_t q;
   const double tol = num->feastol * (fabs(bound) > 1.0 ? fabs(bound) : 1.0);
   for( q = R->colptr[col]; q < R->colptr[col + 1]; ++q )
   {
      const int64_t r = R->rowidx[q];
      const int64_t pinf = R->rowptr[r] + R->rowpos[q];
      const double a = R->vals[pinf];
      /* a lower bound comes from the lhs for a > 0 and from the rhs for a < 0; an upper bound the other way */
      const int reasonisrhs = islower ? (a < 0.0) : (a > 0.0);
      const double side = reasonisrhs ? R->rhs[r] : R->lhs[r];
      double res = 0.0;
      double implied;
      int finite = 1;
      int64_t p;
      if( fabs(side) >= num->infinity || fabs(a) <= num->epsilon )
         continue;
      /* residual activity of the other columns at the time of the change: minimal for the rhs, maximal for the lhs */
      for( p = R->rowptr[r]; p < R->rowptr[r + 1]; ++p )
      {
         double v = R->vals[p];
         int32_t k = R->colidx[p];
         double b;
         if( p == pinf )
            continue;
         b = (reasonisrhs == (v > 0.0)) ? io->lb(io->ud, k) : io->ub(io->ud, k);
         if( fabs(b) >= num->infinity )
         {
            finite = 0;
            break;
         }
         res += v * b;
      }
      if( !finite )
         continue;
      implied = (side - res) / a;
      if( R->isint[col] )
         implied = islower ? ceil(implied - num->feastol) : floor(implied + num->feastol);
      if( islower ? implied < bound - tol : implied > bound + tol )
         continue;
      return addBounds(R, num, io, r, pinf, col, reasonisrhs) == 0 ? r : -2;
   }
   return -1;
}

int64_t gpl_explain_infeasible(const gpl_rows* R, const gpl_num* num, const gpl_io* io)
{
   int64_t r;
   for( r = 0; r < R->m; ++r )
   {
      double minact = 0.0;
      double maxact = 0.0;
      int mininf = 0;
      int maxinf = 0;
      int64_t p;
      for( p = R->rowptr[r]; p < R->rowptr[r + 1]; ++p )
      {
         const double v = R->vals[p];
         const double l = io->lb(io->ud, R->colidx[p]);
         const double u = io->ub(io->ud, R->colidx[p]);
         const double bmin = v > 0.0 ? l : u;
         const double bmax = v > 0.0 ? u : l;
         if( fabs(bmin) >= num->infinity )
            mininf = 1;
         else
            minact += v * bmin;
         if( fabs(bmax) >= num->infinity )
            maxinf = 1;
         else
            maxact += v * bmax;
      }
      if( !mininf && fabs(R->rhs[r]) < num->infinity
         && minact - R->rhs[r] > num->feastol * (fabs(R->rhs[r]) > 1.0 ? fabs(R->rhs[r]) : 1.0) )
         return addBounds(R, num, io, r, -1, -1, 1) == 0 ? r : -2;
      if( !maxinf && fabs(R->lhs[r]) < num->infinity
         && R->lhs[r] - maxact > num->feastol * (fabs(R->lhs[r]) > 1.0 ? fabs(R->lhs[r]) : 1.0) )
         return addBounds(R, num, io, r, -1, -1, 0) == 0 ? r : -2;
   }
   return -1;
}

int gpl_explain_ranged(const gpl_rows* R, const gpl_num* num, const gpl_io* io, int64_t row, int32_t col)
{
   int64_t p;
   (void)col;
   for( p = R->rowptr[row]; p < R->rowptr[row + 1]; ++p )
   {
      const int32_t k = R->colidx[p];
      if( fabs(io->lb(io->ud, k) - io->glb(io->ud, k)) > num->epsilon && io->addlb(io->ud, k) )
         return -2;
      if( fabs(io->ub(io->ud, k) - io->gub(io->ud, k)) > num->epsilon && io->addub(io->ud, k) )
         return -2;
   }
   return 0;
}
