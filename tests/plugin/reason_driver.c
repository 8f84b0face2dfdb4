/* Test harness of the gpulinear reason module (scip_gb300/plugin/gpulinear_reason.c): array-backed bounds, prints
 * for each case the row used and the reason bounds added ("L<col>" lower, "U<col>" upper). */
#include <stdio.h>
#include <string.h>

#include "gpulinear_reason.h"

#define MAXN 16

typedef struct
{
   double lb[MAXN], ub[MAXN], glb[MAXN], gub[MAXN], lbafter[MAXN], ubafter[MAXN];
   char added[256];
} Bounds;

static double fLb(void* u, int32_t k) { return ((Bounds*)u)->lb[k]; }
static double fUb(void* u, int32_t k) { return ((Bounds*)u)->ub[k]; }
static double fGlb(void* u, int32_t k) { return ((Bounds*)u)->glb[k]; }
static double fGub(void* u, int32_t k) { return ((Bounds*)u)->gub[k]; }
static double fLbA(void* u, int32_t k) { return ((Bounds*)u)->lbafter[k]; }
static double fUbA(void* u, int32_t k) { return ((Bounds*)u)->ubafter[k]; }
static int fAddLb(void* u, int32_t k)
{
   char t[16];
   snprintf(t, sizeof t, " L%d", (int)k);
   strcat(((Bounds*)u)->added, t);
   return 0;
}
static int fAddUb(void* u, int32_t k)
{
   char t[16];
   snprintf(t, sizeof t, " U%d", (int)k);
   strcat(((Bounds*)u)->added, t);
   return 0;
}

static void run(const char* name, int64_t m, int64_t n, const int64_t* rowptr, const int32_t* colidx,
   const double* vals, const double* lhs, const double* rhs, const int8_t* isint, Bounds* B, int32_t col, int islower,
   double bound)
{
   int64_t colptr[MAXN + 1];
   int32_t rowidx[64];
   int64_t rowpos[64];
   gpl_rows R;
   gpl_num num = {1e20, 1e-6, 1e-9};
   gpl_io io = {B, fLb, fUb, fGlb, fGub, fLbA, fUbA, fAddLb, fAddUb};
   int64_t r;
   gpl_build_columns(m, n, rowptr, colidx, colptr, rowidx, rowpos);
   R.m = m; R.n = n; R.rowptr = rowptr; R.colidx = colidx; R.vals = vals; R.lhs = lhs; R.rhs = rhs; R.isint = isint;
   R.colptr = colptr; R.rowidx = rowidx; R.rowpos = rowpos;
   B->added[0] = '\0';
   r = gpl_explain(&R, &num, &io, col, islower, bound);
   printf("%s row %lld adds%s\n", name, (long long)r, B->added);
}

static void binaries(Bounds* B, int n)
{
   int k;
   for( k = 0; k < n; ++k )
   {
      B->lb[k] = B->glb[k] = 0.0;
      B->ub[k] = B->gub[k] = 1.0;
      B->lbafter[k] = 0.0;
      B->ubafter[k] = 1.0;
   }
}

int main(void)
{
   const double INF = 1e20;
   /* packing: x0 + x1 + x2 + x3 <= 1 with x0 = 1: x3 <= 0 needs only x0's lower bound */
   {
      int64_t rowptr[] = {0, 4};
      int32_t colidx[] = {0, 1, 2, 3};
      double vals[] = {1, 1, 1, 1}, lhs[] = {-INF}, rhs[] = {1};
      int8_t isint[] = {1, 1, 1, 1};
      Bounds B;
      binaries(&B, 4);
      B.lb[0] = 1.0;
      B.ubafter[3] = 0.0;
      run("packing", 1, 4, rowptr, colidx, vals, lhs, rhs, isint, &B, 3, 0, 0.0);
   }
   /* two rows: row 0 (x0 + x2 <= 5) cannot imply x2 <= 0, row 1 (x1 + x2 <= 1, x1 = 1) can */
   {
      int64_t rowptr[] = {0, 2, 4};
      int32_t colidx[] = {0, 2, 1, 2};
      double vals[] = {1, 1, 1, 1}, lhs[] = {-INF, -INF}, rhs[] = {5, 1};
      int8_t isint[] = {1, 1, 1};
      Bounds B;
      binaries(&B, 3);
      B.lb[1] = 1.0;
      B.ubafter[2] = 0.0;
      run("second_row", 2, 3, rowptr, colidx, vals, lhs, rhs, isint, &B, 2, 0, 0.0);
   }
   /* continuous: 2 y + x0 - x1 <= 4 with x0 = 1, x1 = 0: y <= 1.5; all responsible bounds (L0, U1) */
   {
      int64_t rowptr[] = {0, 3};
      int32_t colidx[] = {2, 0, 1};
      double vals[] = {2, 1, -1}, lhs[] = {-INF}, rhs[] = {4};
      int8_t isint[] = {1, 1, 0};
      Bounds B;
      binaries(&B, 3);
      B.lb[0] = 1.0;
      B.ub[1] = 0.0;
      B.glb[2] = B.lb[2] = B.lbafter[2] = 0.0;
      B.gub[2] = B.ub[2] = 10.0;
      B.ubafter[2] = 1.5;
      run("continuous", 1, 3, rowptr, colidx, vals, lhs, rhs, isint, &B, 2, 0, 1.5);
   }
   /* lhs side, negative coefficient: -x2 + x0 + x1 >= 1 with x0 = x1 = 0 gives x2 <= -1: infeasible for a
    * binary, so use an integer x2 in [-5, 5]: x2 <= -1 needs U0 and U1 */
   {
      int64_t rowptr[] = {0, 3};
      int32_t colidx[] = {2, 0, 1};
      double vals[] = {-1, 1, 1}, lhs[] = {1}, rhs[] = {INF};
      int8_t isint[] = {1, 1, 1};
      Bounds B;
      binaries(&B, 3);
      B.ub[0] = 0.0;
      B.ub[1] = 0.0;
      B.glb[2] = B.lb[2] = B.lbafter[2] = -5.0;
      B.gub[2] = B.ub[2] = 5.0;
      B.ubafter[2] = -1.0;
      run("lhs_negative", 1, 3, rowptr, colidx, vals, lhs, rhs, isint, &B, 2, 0, -1.0);
   }
   /* no implying row: x0 + x1 <= 2 says nothing about x1 <= 0 */
   {
      int64_t rowptr[] = {0, 2};
      int32_t colidx[] = {0, 1};
      double vals[] = {1, 1}, lhs[] = {-INF}, rhs[] = {2};
      int8_t isint[] = {1, 1};
      Bounds B;
      binaries(&B, 2);
      B.lb[0] = 1.0;
      B.ubafter[1] = 0.0;
      run("none", 1, 2, rowptr, colidx, vals, lhs, rhs, isint, &B, 1, 0, 0.0);
   }
   /* lower bound from the rhs with a negative coefficient: x0 + x1 - y <= 1 with x0 = x1 = 1 gives y >= 1 */
   {
      int64_t rowptr[] = {0, 3};
      int32_t colidx[] = {0, 1, 2};
      double vals[] = {1, 1, -1}, lhs[] = {-INF}, rhs[] = {1};
      int8_t isint[] = {1, 1, 1};
      Bounds B;
      binaries(&B, 3);
      B.lb[0] = 1.0;
      B.lb[1] = 1.0;
      B.lbafter[2] = 1.0;
      run("indicator", 1, 3, rowptr, colidx, vals, lhs, rhs, isint, &B, 2, 1, 1.0);
   }
   return 0;
}
