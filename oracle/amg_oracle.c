/* CPU oracle for the BoomerAMG-preconditioned Krylov path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference library's
 * serial CPU algorithms, used as the parity checker and as the timed CPU
 * baseline.  The product library never links it.  Every function cites the
 * reference file:line (paths relative to the reference project's root) whose
 * behaviour it restates.  Integer results (strength pattern, C/F splitting,
 * interpolation pattern, coarse-operator pattern) are meant to be identical to
 * the reference's, and floating-point results are computed with the same
 * operation order (build with -ffp-contract=off so no a*b+c is fused).
 */
#include "amg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define C_PT   1
#define F_PT  -1
#define SF_PT -3

static int g_threads = 1;

void or_set_threads(int nthreads)
{
   g_threads = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
   omp_set_num_threads(g_threads);
#endif
}

static void *xmalloc(size_t n) { void *p = malloc(n ? n : 1); if (!p) { abort(); } return p; }
static void *xcalloc(size_t n, size_t s) { void *p = calloc(n ? n : 1, s ? s : 1); if (!p) { abort(); } return p; }
static void *xrealloc(void *q, size_t n) { void *p = realloc(q, n ? n : 1); if (!p) { abort(); } return p; }

void or_csr_free(or_csr *A)
{
   if (!A) { return; }
   free(A->i); free(A->j); free(A->v);
   A->i = NULL; A->j = NULL; A->v = NULL;
}

void or_default_params(or_amg_params *p)
{
   /* defaults of hypre_BoomerAMGCreate, src/parcsr_ls/par_amg.c:162-304, with the
    * device-path overrides of :306-313 (PMIS, l1-Jacobi) */
   memset(p, 0, sizeof(*p));
   p->strong_threshold = 0.25;
   p->max_row_sum = 0.9;
   p->trunc_factor = 0.0;
   p->p_max_elmts = 4;
   p->interp_type = 6;
   p->coarsen_type = 8;
   p->agg_num_levels = 0;
   p->agg_interp_type = 4;
   p->num_paths = 1;
   p->max_levels = 25;
   p->max_coarse_size = 9;
   p->relax_down = 18;
   p->relax_up = 18;
   p->relax_coarse = 9;
   p->num_sweeps = 1;
   p->relax_weight = 1.0;
   p->cheby_order = 2;
   p->cheby_fraction = 0.3;
   p->cheby_scale = 1;
   p->cheby_eig_est = 10;
   p->cycle_type = 1;
   p->outer_weight = 1.0;
}

/* ------------------------------------------------------------------------ */
/* Park-Miller minimal standard generator, src/utilities/random.c:25-95      */
/* ------------------------------------------------------------------------ */

static int pm_next(int seed)
{
   /* Schrage's method with a=16807, m=2^31-1, q=127773, r=2836 (random.c:68-82) */
   int high = seed / 127773;
   int low = seed % 127773;
   int test = 16807 * low - 2836 * high;
   return test > 0 ? test : test + 2147483647;
}

static int pm_clamp_seed(int seed)
{
   /* hypre_SeedRand, random.c:41-54 */
   if (seed < 1) { return 1; }
   if (seed >= 2147483647) { return 2147483646; }
   return seed;
}

double or_park_miller_nth(int seed, long long k)
{
   /* a^k * seed mod m by square-and-multiply; equals k applications of pm_next */
   unsigned long long m = 2147483647ULL, a = 16807ULL, r = 1ULL, x = (unsigned long long) pm_clamp_seed(seed);
   long long e = k;
   while (e > 0) { if (e & 1) { r = (r * a) % m; } a = (a * a) % m; e >>= 1; }
   return (double) ((r * x) % m) / (double) 2147483647;
}

void or_rand_uniform(int n, int seed, double *out)
{
   /* hypre_SeqVectorSetRandomValues, src/seq_mv/vector.c:615-640 */
   int s = pm_clamp_seed(seed);
   for (int i = 0; i < n; i++)
   {
      s = pm_next(s);
      out[i] = 2.0 * ((double) s / (double) 2147483647) - 1.0;
   }
}

/* ------------------------------------------------------------------------ */
/* Generators                                                               */
/* ------------------------------------------------------------------------ */

int or_gen_stencil(int kind, int nx, int ny, int nz, or_csr *A)
{
   /* GenerateLaplacian (src/parcsr_ls/par_laplace.c:15, values src/test/ij.c:10454)
    * and GenerateLaplacian27pt (src/parcsr_ls/par_laplace_27pt.c:15, values
    * src/test/ij.c:11901): diagonal first, off-diagonals in ascending column order. */
   long long n = (long long) nx * ny * nz;
   int maxrow = kind == 27 ? 27 : 7;
   A->nr = A->nc = (int) n;
   A->i = xmalloc(sizeof(int) * (n + 1));
   A->j = xmalloc(sizeof(int) * n * maxrow);
   A->v = xmalloc(sizeof(double) * n * maxrow);
   long long cnt = 0;
   for (int iz = 0; iz < nz; iz++)
      for (int iy = 0; iy < ny; iy++)
         for (int ix = 0; ix < nx; ix++)
         {
            long long row = ix + (long long) nx * (iy + (long long) ny * iz);
            A->i[row] = (int) cnt;
            A->j[cnt] = (int) row; A->v[cnt] = kind == 27 ? 26.0 : 6.0; cnt++;
            for (int dz = -1; dz <= 1; dz++)
               for (int dy = -1; dy <= 1; dy++)
                  for (int dx = -1; dx <= 1; dx++)
                  {
                     int m = abs(dx) + abs(dy) + abs(dz);
                     if (m == 0 || (kind == 7 && m != 1)) { continue; }
                     int jx = ix + dx, jy = iy + dy, jz = iz + dz;
                     if (jx < 0 || jy < 0 || jz < 0 || jx >= nx || jy >= ny || jz >= nz) { continue; }
                     A->j[cnt] = jx + nx * (jy + ny * jz); A->v[cnt] = -1.0; cnt++;
                  }
         }
   A->i[n] = (int) cnt;
   return 0;
}

int or_gen_aniso2d(int n, double eps, or_csr *A)
{
   /* -eps*u_xx - u_yy on an n x n grid, 5-point, Dirichlet, diagonal first */
   int N = n * n;
   A->nr = A->nc = N;
   A->i = xmalloc(sizeof(int) * (N + 1));
   A->j = xmalloc(sizeof(int) * N * 5);
   A->v = xmalloc(sizeof(double) * N * 5);
   int cnt = 0;
   for (int iy = 0; iy < n; iy++)
      for (int ix = 0; ix < n; ix++)
      {
         int row = ix + n * iy;
         A->i[row] = cnt;
         A->j[cnt] = row; A->v[cnt] = 2.0 * eps + 2.0; cnt++;
         if (iy > 0) { A->j[cnt] = row - n; A->v[cnt] = -1.0; cnt++; }
         if (ix > 0) { A->j[cnt] = row - 1; A->v[cnt] = -eps; cnt++; }
         if (ix < n - 1) { A->j[cnt] = row + 1; A->v[cnt] = -eps; cnt++; }
         if (iy < n - 1) { A->j[cnt] = row + n; A->v[cnt] = -1.0; cnt++; }
      }
   A->i[N] = cnt;
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Strength of connection, hypre_BoomerAMGCreateSHost                        */
/* src/parcsr_ls/par_strength.c:75-527 (num_functions == 1, offd empty)     */
/* ------------------------------------------------------------------------ */

int or_strength(const or_csr *A, double theta, double max_row_sum, or_csr *S)
{
   int n = A->nr;
   int *mark = xmalloc(sizeof(int) * (size_t) (A->i[n] > 0 ? A->i[n] : 1));
   int *cnt = xcalloc(n + 1, sizeof(int));
   #pragma omp parallel for schedule(static)
   for (int i = 0; i < n; i++)
   {
      int b = A->i[i], e = A->i[i + 1];
      double diag = A->v[b];                      /* diagonal assumed first, :245 */
      double row_scale = 0.0, row_sum = diag;
      if (diag < 0)
      {
         for (int k = b + 1; k < e; k++) { row_scale = row_scale > A->v[k] ? row_scale : A->v[k]; row_sum += A->v[k]; }
      }
      else
      {
         for (int k = b + 1; k < e; k++) { row_scale = row_scale < A->v[k] ? row_scale : A->v[k]; row_sum += A->v[k]; }
      }
      int c = 0;
      mark[b] = 0;
      if ((fabs(row_sum) > fabs(diag) * max_row_sum) && (max_row_sum < 1.0))
      {
         for (int k = b + 1; k < e; k++) { mark[k] = 0; }   /* all weak, :326-340 */
      }
      else
      {
         double thr = theta * row_scale;
         for (int k = b + 1; k < e; k++)
         {
            int strong = diag < 0 ? !(A->v[k] <= thr) : !(A->v[k] >= thr);
            mark[k] = strong;
            c += strong;
         }
      }
      cnt[i + 1] = c;
   }
   S->nr = S->nc = n;
   S->i = xmalloc(sizeof(int) * (n + 1));
   S->i[0] = 0;
   for (int i = 0; i < n; i++) { S->i[i + 1] = S->i[i] + cnt[i + 1]; }
   S->j = xmalloc(sizeof(int) * (size_t) (S->i[n] ? S->i[n] : 1));
   S->v = NULL;
   #pragma omp parallel for schedule(static)
   for (int i = 0; i < n; i++)
   {
      int p = S->i[i];
      for (int k = A->i[i] + 1; k < A->i[i + 1]; k++) { if (mark[k]) { S->j[p++] = A->j[k]; } }
   }
   free(mark); free(cnt);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* PMIS, hypre_BoomerAMGCoarsenPMISHost src/parcsr_ls/par_coarsen.c:2094-2806 */
/* with hypre_BoomerAMGIndepSetInit src/parcsr_ls/par_indepset.c:33-63       */
/* ------------------------------------------------------------------------ */

int or_pmis(const or_csr *S, int CF_init, int *CF)
{
   int n = S->nr;
   double *measure = xcalloc(n, sizeof(double));
   int *graph = xmalloc(sizeof(int) * (n ? n : 1));
   int *graph2 = xmalloc(sizeof(int) * (n ? n : 1));
   /* measures: column counts of S (:2232-2288) */
   for (int k = 0; k < S->i[n]; k++) { measure[S->j[k]] += 1.0; }
   /* plus one Park-Miller draw per row, seed 2747, in row order (par_indepset.c:45-60) */
   {
      int s = 2747;
      for (int i = 0; i < n; i++) { s = pm_next(s); measure[i] += (double) s / (double) 2147483647; }
   }
   int gsize = 0;
   for (int i = 0; i < n; i++)
   {
      CF[i] = 0;
      if (S->i[i + 1] - S->i[i] == 0)
      {
         CF[i] = (CF_init == 3 || CF_init == 4) ? C_PT : SF_PT;    /* :2383-2400 */
         measure[i] = 0;
      }
      else { graph[gsize++] = i; }
   }
   int iter = 0;
   while (gsize > 0)
   {
      if (!CF_init || iter)
      {
         for (int g = 0; g < gsize; g++) { int i = graph[g]; if (measure[i] > 1) { CF[i] = 1; } }
         for (int g = 0; g < gsize; g++)
         {
            int i = graph[g];
            if (measure[i] > 1)
            {
               for (int k = S->i[i]; k < S->i[i + 1]; k++)
               {
                  int j = S->j[k];
                  if (measure[j] > 1)
                  {
                     if (measure[i] > measure[j]) { CF[j] = 0; }
                     else if (measure[j] > measure[i]) { CF[i] = 0; }
                  }
               }
            }
         }
      }
      iter++;
      for (int g = 0; g < gsize; g++)   /* :2610-2662 */
      {
         int i = graph[g];
         if (measure[i] < 1) { CF[i] = F_PT; }
         if (CF[i] > 0) { CF[i] = C_PT; }
         else
         {
            for (int k = S->i[i]; k < S->i[i + 1]; k++) { if (CF[S->j[k]] > 0) { CF[i] = F_PT; } }
         }
      }
      int ng = 0;
      for (int g = 0; g < gsize; g++)
      {
         int i = graph[g];
         if (CF[i] != 0) { measure[i] = 0; } else { graph2[ng++] = i; }
      }
      int *t = graph; graph = graph2; graph2 = t;
      gsize = ng;
   }
   free(measure); free(graph); free(graph2);
   return 0;
}

int or_coarse_count(int n, const int *CF)
{
   /* hypre_BoomerAMGCoarseParms, src/parcsr_ls/par_coarse_parms.c:45-106 */
   int c = 0;
   for (int i = 0; i < n; i++) { if (CF[i] == 1) { c++; } }
   return c;
}

/* ------------------------------------------------------------------------ */
/* Direct interpolation (interp_type 3), hypre_BoomerAMGBuildDirInterpHost   */
/* src/parcsr_ls/par_interp.c:1873-2575 (one process, one thread)           */
/* ------------------------------------------------------------------------ */

/* F point i interpolates from the C points of its S row (S order); weight
 * a_ij summed per column, then scaled by -alfa (weights <= 0) or -beta
 * (> 0) with alfa = sum of negative off-diagonals / sum of negative C-point
 * couplings / a_ii and beta likewise for the positive ones (:2362-2455).
 * alfa and beta start at 1 once and keep the last value set: a row whose
 * C-point couplings have no negative (positive) entry reuses the previous
 * row's alfa (beta) (:2240-2245, :2445-2446).  Points with CF -3 become F
 * afterwards (:2560-2563). */
int or_dir_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P)
{
   int n = A->nr;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1));
   int nc = 0;
   for (int i = 0; i < n; i++) { f2c[i] = CF[i] >= 0 ? nc++ : -1; }
   int *Pi = xcalloc(n + 1, sizeof(int));
   for (int i = 0; i < n; i++)
   {
      int c = 0;
      if (CF[i] >= 0) { c = 1; }
      else { for (int k = S->i[i]; k < S->i[i + 1]; k++) { if (CF[S->j[k]] > 0) { c++; } } }
      Pi[i + 1] = Pi[i] + c;
   }
   int *Pj = xmalloc(sizeof(int) * (Pi[n] ? Pi[n] : 1));
   double *Pv = xmalloc(sizeof(double) * (Pi[n] ? Pi[n] : 1));
   int *mark = xmalloc(sizeof(int) * (n ? n : 1));
   for (int i = 0; i < n; i++) { mark[i] = -1; }
   double alfa = 1.0, beta = 1.0;
   for (int i = 0; i < n; i++)
   {
      int c = Pi[i];
      if (CF[i] >= 0) { Pj[c] = f2c[i]; Pv[c] = 1.0; continue; }
      const int jb = c;
      for (int k = S->i[i]; k < S->i[i + 1]; k++)
      {
         int i1 = S->j[k];
         if (CF[i1] >= 0) { mark[i1] = c; Pj[c] = f2c[i1]; Pv[c] = 0.0; c++; }
      }
      const int je = c;
      double diagonal = A->v[A->i[i]];
      double sNp = 0, sNn = 0, sPp = 0, sPn = 0;
      for (int jj = A->i[i] + 1; jj < A->i[i + 1]; jj++)
      {
         int i1 = A->j[jj];
         double a = A->v[jj];
         if (a > 0) { sNp += a; } else { sNn += a; }
         if (mark[i1] >= jb)
         {
            Pv[mark[i1]] += a;
            if (a > 0) { sPp += a; } else { sPn += a; }
         }
      }
      if (sPn != 0.0) { alfa = sNn / sPn / diagonal; }
      if (sPp != 0.0) { beta = sNp / sPp / diagonal; }
      for (int jj = jb; jj < je; jj++)
      {
         if (Pv[jj] > 0) { Pv[jj] *= -beta; }
         else { Pv[jj] *= -alfa; }
      }
   }
   for (int i = 0; i < n; i++) { if (CF[i] == SF_PT) { CF[i] = F_PT; } }
   P->nr = n; P->nc = nc; P->i = Pi; P->j = Pj; P->v = Pv;
   free(f2c); free(mark);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Extended+i interpolation, hypre_BoomerAMGBuildExtPIInterpHost             */
/* src/parcsr_ls/par_lr_interp.c:1024-1924 (one process, offd empty)        */
/* ------------------------------------------------------------------------ */

static int ext_interp(const or_csr *A, const or_csr *S, int *CF, int iterm, or_csr *P);

int or_extpi_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P) { return ext_interp(A, S, CF, 1, P); }

/* Extended interpolation (interp_type 14), hypre_BoomerAMGBuildExtInterpHost
 * src/parcsr_ls/par_lr_interp.c:4777-5515: the same pattern and weights
 * without the point's own term -- the sums and the distribution over a strong
 * F neighbour's row leave i out (:5279-5325 against :1649-1700). */
int or_ext_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P) { return ext_interp(A, S, CF, 0, P); }

static int ext_interp(const or_csr *A, const or_csr *S, int *CF, int iterm, or_csr *P)
{
   int n = A->nr;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1));
   int nc = 0;
   for (int i = 0; i < n; i++) { f2c[i] = CF[i] >= 0 ? nc++ : -1; }   /* :1261-1266 */

   /* pass 1: row sizes, with a per-row marker (:1267-1380) */
   int *Pi = xcalloc(n + 1, sizeof(int));
   int *marker = xmalloc(sizeof(int) * (n ? n : 1));
   for (int i = 0; i < n; i++) { marker[i] = -1; }
   for (int i = 0; i < n; i++)
   {
      int cnt = 0;
      if (CF[i] >= 0) { cnt = 1; }
      else if (CF[i] != SF_PT)
      {
         for (int k = S->i[i]; k < S->i[i + 1]; k++)
         {
            int i1 = S->j[k];
            if (CF[i1] >= 0) { if (marker[i1] != i) { marker[i1] = i; cnt++; } }
            else if (CF[i1] != SF_PT)
            {
               for (int kk = S->i[i1]; kk < S->i[i1 + 1]; kk++)
               {
                  int k1 = S->j[kk];
                  if (CF[k1] >= 0 && marker[k1] != i) { marker[k1] = i; cnt++; }
               }
            }
         }
      }
      Pi[i + 1] = cnt;
   }
   for (int i = 0; i < n; i++) { Pi[i + 1] += Pi[i]; }
   int nnz = Pi[n];
   int *Pj = xmalloc(sizeof(int) * (nnz ? nnz : 1));
   double *Pv = xmalloc(sizeof(double) * (nnz ? nnz : 1));

   /* pass 2: columns in first-discovery order and weights (:1500-1810).
    * pmark[x] >= row_begin: x is a C column of this row at that position;
    * pmark[x] == strong_f: x is a strong F neighbour of this row. */
   int *pmark = xmalloc(sizeof(int) * (n ? n : 1));
   for (int i = 0; i < n; i++) { pmark[i] = -1; }
   int strong_f = -2;
   for (int i = 0; i < n; i++)
   {
      int begin = Pi[i], c = begin;
      if (CF[i] >= 0)
      {
         Pj[c] = f2c[i]; Pv[c] = 1.0; c++;
      }
      else if (CF[i] != SF_PT)
      {
         strong_f--;
         for (int k = S->i[i]; k < S->i[i + 1]; k++)
         {
            int i1 = S->j[k];
            if (CF[i1] >= 0)
            {
               if (pmark[i1] < begin) { pmark[i1] = c; Pj[c] = f2c[i1]; Pv[c] = 0.0; c++; }
            }
            else if (CF[i1] != SF_PT)
            {
               pmark[i1] = strong_f;
               for (int kk = S->i[i1]; kk < S->i[i1 + 1]; kk++)
               {
                  int k1 = S->j[kk];
                  if (CF[k1] >= 0 && pmark[k1] < begin) { pmark[k1] = c; Pj[c] = f2c[k1]; Pv[c] = 0.0; c++; }
               }
            }
         }
         int end = c;
         double diagonal = A->v[A->i[i]];
         for (int jj = A->i[i] + 1; jj < A->i[i + 1]; jj++)
         {
            int i1 = A->j[jj];
            if (pmark[i1] >= begin) { Pv[pmark[i1]] += A->v[jj]; }
            else if (pmark[i1] == strong_f)
            {
               double sum = 0.0;
               int sgn = A->v[A->i[i1]] < 0 ? -1 : 1;
               for (int jj1 = A->i[i1] + 1; jj1 < A->i[i1 + 1]; jj1++)
               {
                  int i2 = A->j[jj1];
                  if ((pmark[i2] >= begin || (iterm && i2 == i)) && (sgn * A->v[jj1]) < 0) { sum += A->v[jj1]; }
               }
               if (sum != 0)
               {
                  double distribute = A->v[jj] / sum;
                  for (int jj1 = A->i[i1] + 1; jj1 < A->i[i1 + 1]; jj1++)
                  {
                     int i2 = A->j[jj1];
                     if (pmark[i2] >= begin && (sgn * A->v[jj1]) < 0) { Pv[pmark[i2]] += distribute * A->v[jj1]; }
                     if (iterm && i2 == i && (sgn * A->v[jj1]) < 0) { diagonal += distribute * A->v[jj1]; }
                  }
               }
               else { diagonal += A->v[jj]; }
            }
            else if (CF[i1] != SF_PT) { diagonal += A->v[jj]; }
         }
         if (diagonal != 0.0)
         {
            for (int k = begin; k < end; k++) { Pv[k] /= -diagonal; }
         }
      }
      strong_f--;
   }
   /* SF points are reported as F points afterwards (:1896-1902) */
   for (int i = 0; i < n; i++) { if (CF[i] == SF_PT) { CF[i] = F_PT; } }
   P->nr = n; P->nc = nc; P->i = Pi; P->j = Pj; P->v = Pv;
   free(f2c); free(marker); free(pmark);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Truncation, hypre_ParCSRMatrixTruncate src/parcsr_mv/par_csr_matrix.c     */
/* :2943-3300 (rescale = 1, infinity-norm), sorting with hypre_qsort2_abs    */
/* src/utilities/qsort.c:452-474                                            */
/* ------------------------------------------------------------------------ */

static void swap2(int *v, double *w, int a, int b)
{
   int t = v[a]; v[a] = v[b]; v[b] = t;
   double u = w[a]; w[a] = w[b]; w[b] = u;
}

static void qsort2_abs(int *v, double *w, int left, int right)
{
   if (left >= right) { return; }
   swap2(v, w, left, (left + right) / 2);
   int last = left;
   for (int i = left + 1; i <= right; i++)
   {
      if (fabs(w[i]) > fabs(w[left])) { swap2(v, w, ++last, i); }
   }
   swap2(v, w, left, last);
   qsort2_abs(v, w, left, last - 1);
   qsort2_abs(v, w, last + 1, right);
}

int or_truncate(or_csr *P, double tol, int max_elmts)
{
   int n = P->nr;
   if (tol <= 0.0 && max_elmts == 0) { return 0; }
   int *Pi = P->i, *Pj = P->j;
   double *Pv = P->v;
   if (tol > 0)
   {
      /* drop |p| < tol * max|p_row|, then rescale to keep the row sum (:3038-3120) */
      int next_open = 0, now = 0;
      int *newi = xmalloc(sizeof(int) * (n + 1));
      newi[0] = 0;
      for (int i = 0; i < n; i++)
      {
         double row_nrm = 0;
         for (int k = Pi[i]; k < Pi[i + 1]; k++) { row_nrm = row_nrm < fabs(Pv[k]) ? fabs(Pv[k]) : row_nrm; }
         double drop = tol * row_nrm;
         double row_sum = 0, scale = 0;
         int rb = next_open;
         for (now = Pi[i]; now < Pi[i + 1]; now++)
         {
            row_sum += Pv[now];
            if (!(fabs(Pv[now]) < drop))
            {
               scale += Pv[now];
               Pv[next_open] = Pv[now]; Pj[next_open] = Pj[now]; next_open++;
            }
         }
         if (scale != 0. && scale != row_sum)
         {
            scale = row_sum / scale;
            for (int k = rb; k < next_open; k++) { Pv[k] *= scale; }
         }
         newi[i + 1] = next_open;
      }
      memcpy(Pi, newi, sizeof(int) * (n + 1));
      free(newi);
   }
   if (max_elmts > 0)
   {
      int mx = 0;
      for (int i = 0; i < n; i++) { int c = Pi[i + 1] - Pi[i]; if (c > mx) { mx = c; } }
      if (mx > max_elmts)
      {
         int *aj = xmalloc(sizeof(int) * mx);
         double *av = xmalloc(sizeof(double) * mx);
         int cntd = 0;
         int prev_end = Pi[0];
         for (int i = 0; i < n; i++)
         {
            int b = prev_end, e = Pi[i + 1];
            prev_end = e;
            int num = e - b;
            Pi[i] = cntd;
            if (max_elmts < num)
            {
               double row_sum = 0;
               int c = 0;
               for (int k = b; k < e; k++) { aj[c] = Pj[k]; av[c] = Pv[k]; row_sum += Pv[k]; c++; }
               qsort2_abs(aj, av, 0, c - 1);
               double scale = 0;
               int rb = cntd;
               for (int k = 0; k < max_elmts; k++)
               {
                  scale += av[k];
                  Pj[cntd] = aj[k]; Pv[cntd] = av[k]; cntd++;
               }
               if (scale != 0. && scale != row_sum)
               {
                  scale = row_sum / scale;
                  for (int k = rb; k < cntd; k++) { Pv[k] *= scale; }
               }
            }
            else
            {
               for (int k = b; k < e; k++) { Pj[cntd] = Pj[k]; Pv[cntd] = Pv[k]; cntd++; }
            }
         }
         Pi[n] = cntd;
         free(aj); free(av);
      }
   }
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Transpose by counting sort (stable: rows of A^T list A's rows ascending),  */
/* hypre_CSRMatrixTransposeHost src/seq_mv/csr_matop.c:1071                  */
/* ------------------------------------------------------------------------ */

int or_transpose(const or_csr *A, or_csr *AT)
{
   int nr = A->nr, nc = A->nc, nnz = A->i[nr];
   AT->nr = nc; AT->nc = nr;
   AT->i = xcalloc(nc + 1, sizeof(int));
   AT->j = xmalloc(sizeof(int) * (nnz ? nnz : 1));
   AT->v = A->v ? xmalloc(sizeof(double) * (nnz ? nnz : 1)) : NULL;
   for (int k = 0; k < nnz; k++) { AT->i[A->j[k] + 1]++; }
   for (int c = 0; c < nc; c++) { AT->i[c + 1] += AT->i[c]; }
   int *pos = xmalloc(sizeof(int) * (nc ? nc : 1));
   memcpy(pos, AT->i, sizeof(int) * nc);
   for (int r = 0; r < nr; r++)
   {
      for (int k = A->i[r]; k < A->i[r + 1]; k++)
      {
         int p = pos[A->j[k]]++;
         AT->j[p] = r;
         if (A->v) { AT->v[p] = A->v[k]; }
      }
   }
   free(pos);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Galerkin product, hypre_BoomerAMGBuildCoarseOperatorKT                    */
/* src/parcsr_ls/par_rap.c:30 (numeric pass :1640-1880): per coarse row ic,  */
/* diagonal first, then RA row in discovery order, then RAP in discovery     */
/* order over (RA entries x P rows).                                         */
/* ------------------------------------------------------------------------ */

int or_rap(const or_csr *P, const or_csr *A, or_csr *Ac)
{
   or_csr R;
   or_transpose(P, &R);
   int nc = P->nc, nf = A->nr;
   /* pass 1: sizes */
   int *Ci = xcalloc(nc + 1, sizeof(int));
   int nthr = 1;
#ifdef _OPENMP
   nthr = g_threads;
#endif
   #pragma omp parallel num_threads(nthr)
   {
      int *pm = xmalloc(sizeof(int) * (nc ? nc : 1));
      int *am = xmalloc(sizeof(int) * (nf ? nf : 1));
      for (int k = 0; k < nc; k++) { pm[k] = -1; }
      for (int k = 0; k < nf; k++) { am[k] = -1; }
      #pragma omp for schedule(static)
      for (int ic = 0; ic < nc; ic++)
      {
         int cnt = 1;
         pm[ic] = ic;
         for (int k1 = R.i[ic]; k1 < R.i[ic + 1]; k1++)
         {
            int i1 = R.j[k1];
            for (int k2 = A->i[i1]; k2 < A->i[i1 + 1]; k2++)
            {
               int i2 = A->j[k2];
               if (am[i2] != ic)
               {
                  am[i2] = ic;
                  for (int k3 = P->i[i2]; k3 < P->i[i2 + 1]; k3++)
                  {
                     int i3 = P->j[k3];
                     if (pm[i3] != ic) { pm[i3] = ic; cnt++; }
                  }
               }
            }
         }
         Ci[ic + 1] = cnt;
      }
      free(pm); free(am);
   }
   for (int ic = 0; ic < nc; ic++) { Ci[ic + 1] += Ci[ic]; }
   int nnz = Ci[nc];
   int *Cj = xmalloc(sizeof(int) * (nnz ? nnz : 1));
   double *Cv = xmalloc(sizeof(double) * (nnz ? nnz : 1));
   /* pass 2: values */
   #pragma omp parallel num_threads(nthr)
   {
      int *pm = xmalloc(sizeof(int) * (nc ? nc : 1));
      int *am = xmalloc(sizeof(int) * (nf ? nf : 1));
      int *raj = xmalloc(sizeof(int) * (nf ? nf : 1));
      double *rav = xmalloc(sizeof(double) * (nf ? nf : 1));
      for (int k = 0; k < nc; k++) { pm[k] = -1; }
      for (int k = 0; k < nf; k++) { am[k] = -1; }
      #pragma omp for schedule(static)
      for (int ic = 0; ic < nc; ic++)
      {
         int begin = Ci[ic], c = begin;
         pm[ic] = c; Cj[c] = ic; Cv[c] = 0.0; c++;
         int nra = 0;
         for (int k1 = R.i[ic]; k1 < R.i[ic + 1]; k1++)
         {
            int i1 = R.j[k1];
            double r = R.v[k1];
            for (int k2 = A->i[i1]; k2 < A->i[i1 + 1]; k2++)
            {
               int i2 = A->j[k2];
               double a = A->v[k2];
               /* am[i2] holds ic*? no: use a row-local check via position */
               int m = am[i2];
               if (m < 0 || m >= nra || raj[m] != i2) { am[i2] = nra; raj[nra] = i2; rav[nra] = r * a; nra++; }
               else { rav[m] += r * a; }
            }
         }
         for (int t = 0; t < nra; t++)
         {
            int i1 = raj[t];
            double ra = rav[t];
            for (int k3 = P->i[i1]; k3 < P->i[i1 + 1]; k3++)
            {
               int i2 = P->j[k3];
               double p = P->v[k3];
               int m = pm[i2];
               if (m < begin) { pm[i2] = c; Cj[c] = i2; Cv[c] = ra * p; c++; }
               else { Cv[m] += ra * p; }
            }
         }
      }
      free(pm); free(am); free(raj); free(rav);
   }
   Ac->nr = nc; Ac->nc = nc; Ac->i = Ci; Ac->j = Cj; Ac->v = Cv;
   or_csr_free(&R);
   return 0;
}

/* general product C = A*B with columns in discovery order (row-wise marker
 * SpGEMM, the order hypre_ParMatmul's diag part produces) */
static int matmul_ex(const or_csr *A, const or_csr *B, or_csr *C, int square);

int or_matmul(const or_csr *A, const or_csr *B, or_csr *C)
{
   /* hypre_ParMatmul, src/parcsr_mv/par_csr_matop.c:348 (one process): row-wise
    * marker product, columns in discovery order, first contribution stored,
    * later ones added; a square product places its diagonal first (:688-697). */
   return matmul_ex(A, B, C, A->nr == B->nc);
}

static int matmul_ex(const or_csr *A, const or_csr *B, or_csr *C, int square)
{
   int n = A->nr, m = B->nc;
   int *Ci = xcalloc(n + 1, sizeof(int));
   int *mk = xmalloc(sizeof(int) * (m ? m : 1));
   for (int k = 0; k < m; k++) { mk[k] = -1; }
   for (int i = 0; i < n; i++)
   {
      int cnt = 0;
      if (square) { mk[i] = i; cnt++; }
      for (int ka = A->i[i]; ka < A->i[i + 1]; ka++)
      {
         int r = A->j[ka];
         for (int kb = B->i[r]; kb < B->i[r + 1]; kb++) { int c = B->j[kb]; if (mk[c] != i) { mk[c] = i; cnt++; } }
      }
      Ci[i + 1] = Ci[i] + cnt;
   }
   int nnz = Ci[n];
   int *Cj = xmalloc(sizeof(int) * (nnz ? nnz : 1));
   double *Cv = xmalloc(sizeof(double) * (nnz ? nnz : 1));
   for (int k = 0; k < m; k++) { mk[k] = -1; }
   for (int i = 0; i < n; i++)
   {
      int begin = Ci[i], c = begin;
      if (square) { mk[i] = c; Cj[c] = i; Cv[c] = 0.0; c++; }
      for (int ka = A->i[i]; ka < A->i[i + 1]; ka++)
      {
         int r = A->j[ka];
         double a = A->v[ka];
         for (int kb = B->i[r]; kb < B->i[r + 1]; kb++)
         {
            int col = B->j[kb];
            if (mk[col] < begin) { mk[col] = c; Cj[c] = col; Cv[c] = a * B->v[kb]; c++; }
            else { Cv[mk[col]] += a * B->v[kb]; }
         }
      }
   }
   C->nr = n; C->nc = m; C->i = Ci; C->j = Cj; C->v = Cv;
   free(mk);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Aggressive coarsening (agg_num_levels > 0, agg_interp_type 6)             */
/* ------------------------------------------------------------------------ */

/* Second-order strength between C points, hypre_BoomerAMGCreate2ndSHost
 * src/parcsr_ls/par_strength.c:1795-3030 (num_paths = 1): row ic (the ic-th C
 * point i1) holds, in discovery order, the coarse index of every C neighbour
 * i2 of i1 in S and of every C point i3 != i1 in S_i2 for each neighbour i2.
 * C points with an empty row are marked CF = 2 (:2701-2723). */
int or_strength2(const or_csr *S, int *CF, int num_paths, or_csr *S2)
{
   (void) num_paths;
   int n = S->nr;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1));
   int nc = 0;
   for (int i = 0; i < n; i++) { f2c[i] = CF[i] > 0 ? nc++ : -1; }
   int *c2f = xmalloc(sizeof(int) * (nc ? nc : 1));
   for (int i = 0; i < n; i++) { if (CF[i] > 0) { c2f[f2c[i]] = i; } }
   int *mark = xmalloc(sizeof(int) * (nc ? nc : 1));
   for (int k = 0; k < nc; k++) { mark[k] = -1; }
   int *Ci = xcalloc(nc + 1, sizeof(int));
   /* pass 1: counts */
   for (int ic = 0; ic < nc; ic++)
   {
      int i1 = c2f[ic], cnt = 0;
      for (int k1 = S->i[i1]; k1 < S->i[i1 + 1]; k1++)
      {
         int i2 = S->j[k1];
         if (CF[i2] > 0) { int idx = f2c[i2]; if (mark[idx] != ic) { mark[idx] = ic; cnt++; } }
         for (int k2 = S->i[i2]; k2 < S->i[i2 + 1]; k2++)
         {
            int i3 = S->j[k2];
            if (CF[i3] > 0) { int idx = f2c[i3]; if (idx != ic && mark[idx] != ic) { mark[idx] = ic; cnt++; } }
         }
      }
      Ci[ic + 1] = cnt;
   }
   for (int ic = 0; ic < nc; ic++)
   {
      if (Ci[ic + 1] == 0) { CF[c2f[ic]] = 2; }
      Ci[ic + 1] += Ci[ic];
   }
   int *Cj = xmalloc(sizeof(int) * (Ci[nc] ? Ci[nc] : 1));
   for (int k = 0; k < nc; k++) { mark[k] = -1; }
   for (int ic = 0; ic < nc; ic++)
   {
      int i1 = c2f[ic], c = Ci[ic];
      for (int k1 = S->i[i1]; k1 < S->i[i1 + 1]; k1++)
      {
         int i2 = S->j[k1];
         if (CF[i2] > 0) { int idx = f2c[i2]; if (mark[idx] < Ci[ic]) { mark[idx] = c; Cj[c++] = idx; } }
         for (int k2 = S->i[i2]; k2 < S->i[i2 + 1]; k2++)
         {
            int i3 = S->j[k2];
            if (CF[i3] > 0) { int idx = f2c[i3]; if (idx != ic && mark[idx] < Ci[ic]) { mark[idx] = c; Cj[c++] = idx; } }
         }
      }
   }
   S2->nr = S2->nc = nc; S2->i = Ci; S2->j = Cj; S2->v = NULL;
   free(f2c); free(c2f); free(mark);
   return 0;
}

/* hypre_BoomerAMGCorrectCFMarkerHost src/parcsr_ls/par_strength.c:3068-3090:
 * C points take the second coarsening's marker (CF 2, isolated in S2, stays C). */
void or_correct_cf(int n, int *CF, const int *CFN)
{
   int cnt = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] > 0)
      {
         if (CF[i] == 1) { CF[i] = CFN[cnt++]; }
         else { CF[i] = 1; cnt++; }
      }
   }
}

/* Multipass interpolation (agg_interp_type 4), hypre_BoomerAMGBuildMultipassHost
 * src/parcsr_ls/par_multi_interp.c:16-2130 on one process with one thread and
 * the default weights (sep_weight 0, :1600-1960).  Passes (:310-512): F points
 * with a strong C neighbour are pass 1; pass p (< 10) takes the F points with a
 * strong neighbour of pass p-1; the points are visited in the order the
 * reference's pass_array reaches them.  Pattern (:540-1105): pass 1 rows hold
 * their strong C neighbours; a row of pass p the union, in S order, of the rows
 * of its strong neighbours of pass p-1.  Weights: pass 1 row i takes a_ij of
 * its strong C neighbours (A order), pass p row i the sums of a_ij p_jk over
 * its strong neighbours j of pass p-1 (A order); sum_C sums those terms,
 * sum_N the same plus the row's other off-diagonals (CF != -3), and the row
 * is scaled by alfa = -sum_N / (sum_C a_ii) -- alfa keeps its last value when
 * sum_C a_ii is zero (in passes >= 2 that is the row's last product).
 * Truncated with (trunc_factor, max_elmts); CF -3 becomes -1 (:2098-2104). */
int or_multipass_interp(const or_csr *A, const or_csr *S, int *CF, double trunc_factor, int max_elmts, or_csr *P)
{
   const int n = A->nr, max_passes = 10;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1)), *assigned = xmalloc(sizeof(int) * (n ? n : 1));
   int nf = 0, nc = 0;
   for (int i = 0; i < n; i++) { if (CF[i] == -1) { nf++; } }
   int *pass_array = xmalloc(sizeof(int) * (nf ? nf : 1));
   int p_cnt = nf - 1;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] == 1) { f2c[i] = nc++; assigned[i] = 0; }
      else if (CF[i] == -1) { pass_array[p_cnt--] = i; assigned[i] = -1; f2c[i] = -1; }
      else { assigned[i] = -1; f2c[i] = -1; }
   }
   int pass_ptr[12] = {0};
   int cnt = 0;
   for (int i = nf - 1; i > cnt - 1; i--)
   {
      int i1 = pass_array[i];
      for (int j = S->i[i1]; j < S->i[i1 + 1]; j++) { if (CF[S->j[j]] == 1) { assigned[i1] = 1; } }
      if (assigned[i1] == 1) { pass_array[i++] = pass_array[cnt]; pass_array[cnt++] = i1; }
   }
   pass_ptr[2] = cnt;
   int pass = 2;
   while (nf - cnt > 0 && pass < max_passes)
   {
      for (int i = nf - 1; i > cnt - 1; i--)
      {
         int i1 = pass_array[i];
         for (int j = S->i[i1]; j < S->i[i1 + 1]; j++)
         {
            if (assigned[S->j[j]] == pass - 1)
            {
               pass_array[i++] = pass_array[cnt];
               pass_array[cnt++] = i1;
               assigned[i1] = pass;
               break;
            }
         }
      }
      pass++;
      pass_ptr[pass] = cnt;
   }
   const int num_passes = pass;
   /* rows: C identity, pass rows built pass by pass (each from the finished
    * rows of the previous pass) */
   int **rj = xcalloc(n ? n : 1, sizeof(int *));
   double **rv = xcalloc(n ? n : 1, sizeof(double *));
   int *rl = xcalloc(n ? n : 1, sizeof(int));
   for (int i = 0; i < n; i++)
   {
      if (CF[i] == 1) { rj[i] = xmalloc(sizeof(int)); rv[i] = xmalloc(sizeof(double)); rj[i][0] = f2c[i]; rv[i][0] = 1.0; rl[i] = 1; }
   }
   int *mark = xmalloc(sizeof(int) * (n ? n : 1)), *pos = xmalloc(sizeof(int) * (nc ? nc : 1));
   for (int i = 0; i < n; i++) { mark[i] = -1; }
   double alfa = 1.0;
   for (int ps = 1; ps < num_passes; ps++)
   {
      if (ps >= 2) { alfa = 1.0; }   /* a fresh parallel region per pass (:1757) */
      for (int t = pass_ptr[ps]; t < pass_ptr[ps + 1]; t++)
      {
         int i1 = pass_array[t];
         /* pattern: pass 1, the strong C neighbours in A order (:1665-1672);
          * pass p, the union of the strong pass p-1 neighbours' rows taken
          * in S order (:1048-1072) */
         int len = 0, cap = 16;
         int *cj = xmalloc(sizeof(int) * cap);
         for (int k = 0; k < nc; k++) { pos[k] = -1; }
         for (int j = S->i[i1]; j < S->i[i1 + 1]; j++)
         {
            int j1 = S->j[j];
            if (assigned[j1] != ps - 1) { continue; }
            mark[j1] = i1;
            if (ps == 1) { continue; }
            for (int k = 0; k < rl[j1]; k++)
            {
               int k1 = rj[j1][k];
               if (pos[k1] < 0)
               {
                  if (len == cap) { cap *= 2; cj = xrealloc(cj, sizeof(int) * cap); }
                  pos[k1] = len; cj[len++] = k1;
               }
            }
         }
         if (ps == 1)
         {
            for (int j = A->i[i1] + 1; j < A->i[i1 + 1]; j++)
            {
               int j1 = A->j[j];
               if (mark[j1] == i1 && pos[f2c[j1]] < 0)
               {
                  if (len == cap) { cap *= 2; cj = xrealloc(cj, sizeof(int) * cap); }
                  pos[f2c[j1]] = len; cj[len++] = f2c[j1];
               }
            }
         }
         double *cv = xcalloc(len ? len : 1, sizeof(double));
         double sum_C = 0.0, sum_N = 0.0;
         for (int j = A->i[i1] + 1; j < A->i[i1 + 1]; j++)
         {
            int j1 = A->j[j];
            double a = A->v[j];
            if (ps == 1)
            {
               /* :1646-1660: every off-diagonal (CF != -3) in sum_N, strong C in P and sum_C */
               if (CF[j1] != -3) { sum_N += a; }
               if (mark[j1] == i1) { cv[pos[f2c[j1]]] = a; sum_C += a; }
            }
            else if (mark[j1] == i1)
            {
               for (int k = 0; k < rl[j1]; k++)
               {
                  alfa = a * rv[j1][k];
                  cv[pos[rj[j1][k]]] += alfa;
                  sum_C += alfa;
                  sum_N += alfa;
               }
            }
            else if (CF[j1] != -3) { sum_N += a; }
         }
         double diagonal = A->v[A->i[i1]];
         if (sum_C * diagonal != 0) { alfa = -sum_N / (sum_C * diagonal); }
         for (int k = 0; k < len; k++) { cv[k] *= alfa; }
         rj[i1] = cj; rv[i1] = cv; rl[i1] = len;
      }
   }
   int *Pi = xcalloc(n + 1, sizeof(int));
   for (int i = 0; i < n; i++) { Pi[i + 1] = Pi[i] + rl[i]; }
   int *Pj = xmalloc(sizeof(int) * (Pi[n] ? Pi[n] : 1));
   double *Pv = xmalloc(sizeof(double) * (Pi[n] ? Pi[n] : 1));
   for (int i = 0; i < n; i++)
   {
      if (rl[i]) { memcpy(Pj + Pi[i], rj[i], sizeof(int) * rl[i]); memcpy(Pv + Pi[i], rv[i], sizeof(double) * rl[i]); }
      free(rj[i]); free(rv[i]);
   }
   P->nr = n; P->nc = nc; P->i = Pi; P->j = Pj; P->v = Pv;
   if (trunc_factor != 0.0 || max_elmts != 0) { or_truncate(P, trunc_factor, max_elmts); }
   for (int i = 0; i < n; i++) { if (CF[i] == SF_PT) { CF[i] = F_PT; } }
   free(rj); free(rv); free(rl); free(mark); free(pos); free(f2c); free(assigned); free(pass_array);
   return 0;
}

/* One pass block of the product-form multipass interpolation:
 * hypre_GenerateMultipassPi src/parcsr_ls/par_mod_multi_interp.c:530-838
 * (type 8, and the first block of type 9) and the Q part of
 * hypre_GenerateMultiPi :841-1277 (type 9, Q unscaled plus w).  Rows: the m
 * points pts[] (a pass, in row order); columns: the points of pass `color`
 * numbered in row order (col[]).  Entries: the strong neighbours of pass
 * `color`, in S order, with A's value.  Type 8: w == NULL, the row is scaled
 * by -rs / (sum * a_ii) with rs = rsum[i1] (sum of the row's off-diagonals),
 * or by -rs when sum * a_ii is zero.  Type 9: w[r] receives, in A order, the
 * off-diagonals that did not enter Q; the row is not scaled. */
static void mmp_block(const or_csr *A, const or_csr *S, const int *pass, const int *col, const int *pts, int m,
                      int color, double *rsum, double *w, or_csr *Q, int ncols)
{
   int *Qi = xcalloc(m + 1, sizeof(int));
   for (int r = 0; r < m; r++)
   {
      const int i1 = pts[r];
      int c = 0;
      for (int j = S->i[i1]; j < S->i[i1 + 1]; j++) { if (pass[S->j[j]] == color) { c++; } }
      Qi[r + 1] = Qi[r] + c;
   }
   const int nnz = Qi[m];
   int *Qj = xmalloc(sizeof(int) * (nnz ? nnz : 1));
   double *Qv = xmalloc(sizeof(double) * (nnz ? nnz : 1));
   for (int r = 0; r < m; r++)
   {
      const int i1 = pts[r];
      int q = Qi[r];
      if (!w)
      {
         /* :766-786: S's columns are found in A by a forward walk from the
          * row start */
         int j2 = A->i[i1];
         for (int j = S->i[i1]; j < S->i[i1 + 1]; j++)
         {
            const int j1 = S->j[j];
            while (A->j[j2] != j1) { j2++; }
            if (pass[j1] == color) { Qj[q] = col[j1]; Qv[q] = A->v[j2]; q++; }
         }
         /* :790-823 */
         double sum = 0.0;
         for (int k = Qi[r]; k < Qi[r + 1]; k++) { sum += Qv[k]; }
         const double value = sum * A->v[A->i[i1]];
         if (value != 0) { rsum[i1] /= value; }
         for (int k = Qi[r]; k < Qi[r + 1]; k++) { Qv[k] = -Qv[k] * rsum[i1]; }
      }
      else
      {
         /* :1100-1140: every off-diagonal of A that is not a Q entry goes
          * to w, in A order */
         double ws = 0.0;
         int j2 = A->i[i1] + 1;
         for (int j = S->i[i1]; j < S->i[i1 + 1]; j++)
         {
            const int j1 = S->j[j];
            while (A->j[j2] != j1) { ws += A->v[j2]; j2++; }
            if (pass[j1] == color) { Qj[q] = col[j1]; Qv[q] = A->v[j2]; q++; }
            else { ws += A->v[j2]; }
            j2++;
         }
         while (j2 < A->i[i1 + 1]) { ws += A->v[j2]; j2++; }
         w[r] = ws;
      }
   }
   Q->nr = m; Q->nc = ncols; Q->i = Qi; Q->j = Qj; Q->v = Qv;
}

/* Multipass interpolation expressed with sparse products (agg_interp_type 8
 * and 9), hypre_BoomerAMGBuildModMultipassHost
 * src/parcsr_ls/par_mod_multi_interp.c:17-525 on one process.  Passes
 * (:123-270): the C points are pass 1; each round visits the points still
 * unassigned in row order and gives pass p+1 to those with a strong neighbour
 * of pass p (the marks of a round do not affect the same round); rounds stop
 * when none are left, when a round assigns none, or after 9 passes.  Row sums
 * (:272-312): the off-diagonals of every F row.  Pi[0] interpolates pass 2
 * from the C points (mmp_block); type 8: Pi[p] = Q_p Pi[p-1] with Q_p the
 * scaled block of pass p+2 from pass p+1 (hypre_ParMatmul); type 9: Pi[p] =
 * Q_p Pi[p-1] with Q_p unscaled, then each row r scaled by -(s + w_r) /
 * (s a_ii) with s the row's sum (-(s + w_r) when s a_ii is zero;
 * :1236-1265).  P: C rows identity, a pass row the matching row of its Pi;
 * truncated with (trunc_factor, max_elmts); CF -3 becomes -1 (:507-510).
 * More than 9 passes is an error (-1), as is an assignment that stalls. */
int or_mod_multipass_interp(const or_csr *A, const or_csr *S, int *CF, int type, double trunc_factor,
                            int max_elmts, or_csr *P)
{
   const int n = A->nr;
   int *pass = xcalloc(n ? n : 1, sizeof(int));
   int *left = xmalloc(sizeof(int) * (n ? n : 1));
   int *order = xmalloc(sizeof(int) * (n ? n : 1));
   int starts[12] = {0};
   int nleft = 0, cnt = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] == 1) { pass[i] = 1; order[cnt++] = i; }
      else { left[nleft++] = i; }
   }
   const int nc = cnt;
   starts[1] = cnt;
   int num_passes = 1, cur = 1, rc = 0;
   while (nleft > 0)
   {
      const int old = nleft;
      int keep = 0;
      for (int t = 0; t < old; t++)
      {
         const int i1 = left[t];
         int hit = 0;
         for (int j = S->i[i1]; j < S->i[i1 + 1]; j++) { if (pass[S->j[j]] == cur) { hit = 1; break; } }
         if (hit) { pass[i1] = cur + 1; order[cnt++] = i1; }
         else { left[keep++] = i1; }
      }
      nleft = keep;
      cur++;
      num_passes++;
      if (num_passes > 9) { rc = -1; break; }
      starts[num_passes] = cnt;
      if (nleft == old) { break; }
   }
   free(left);
   if (rc) { free(pass); free(order); return -1; }
   double *rsum = xcalloc(n ? n : 1, sizeof(double));
   for (int i = 0; i < n; i++)
   {
      if (CF[i] < 0) { for (int j = A->i[i] + 1; j < A->i[i + 1]; j++) { rsum[i] += A->v[j]; } }
   }
   /* column numbering of each pass: row order among its points */
   int *col = xmalloc(sizeof(int) * (n ? n : 1));
   {
      int pc[12] = {0};
      for (int i = 0; i < n; i++) { col[i] = pass[i] > 0 ? pc[pass[i]]++ : -1; }
   }
   const int nblk = num_passes - 1;
   or_csr *Pi = xcalloc(nblk > 0 ? nblk : 1, sizeof(or_csr));
   for (int b = 0; b < nblk; b++)
   {
      const int m = starts[b + 2] - starts[b + 1];
      const int *pts = order + starts[b + 1];
      if (b == 0) { mmp_block(A, S, pass, col, pts, m, 1, rsum, NULL, &Pi[0], nc); continue; }
      const int prev_m = starts[b + 1] - starts[b];
      or_csr Q;
      double *w = type == 9 ? xmalloc(sizeof(double) * (m ? m : 1)) : NULL;
      mmp_block(A, S, pass, col, pts, m, b + 1, rsum, w, &Q, prev_m);
      or_matmul(&Q, &Pi[b - 1], &Pi[b]);
      if (type == 9)
      {
         for (int r = 0; r < m; r++)
         {
            const int i1 = pts[r];
            double s = 0.0;
            for (int k = Pi[b].i[r]; k < Pi[b].i[r + 1]; k++) { s += Pi[b].v[k]; }
            const double value = s * A->v[A->i[i1]];
            s += w[r];
            if (value != 0) { s /= value; }
            for (int k = Pi[b].i[r]; k < Pi[b].i[r + 1]; k++) { Pi[b].v[k] = -Pi[b].v[k] * s; }
         }
      }
      free(w);
      or_csr_free(&Q);
   }
   /* assembly (:316-380) */
   int *Pp = xcalloc(n + 1, sizeof(int));
   int *blk = xmalloc(sizeof(int) * (n ? n : 1));
   for (int i = 0; i < n; i++)
   {
      blk[i] = -1;
      if (CF[i] == 1) { Pp[i + 1] = 1; }
      else if (pass[i] >= 2 && pass[i] - 2 < nblk)
      {
         blk[i] = pass[i] - 2;
         const or_csr *B = &Pi[blk[i]];
         Pp[i + 1] = B->i[col[i] + 1] - B->i[col[i]];
      }
   }
   for (int i = 0; i < n; i++) { Pp[i + 1] += Pp[i]; }
   int *Pj = xmalloc(sizeof(int) * (Pp[n] ? Pp[n] : 1));
   double *Pv = xmalloc(sizeof(double) * (Pp[n] ? Pp[n] : 1));
   for (int i = 0; i < n; i++)
   {
      if (CF[i] == 1) { Pj[Pp[i]] = col[i]; Pv[Pp[i]] = 1.0; }
      else if (blk[i] >= 0)
      {
         const or_csr *B = &Pi[blk[i]];
         const int k0 = B->i[col[i]], l = Pp[i + 1] - Pp[i];
         memcpy(Pj + Pp[i], B->j + k0, sizeof(int) * (size_t) l);
         memcpy(Pv + Pp[i], B->v + k0, sizeof(double) * (size_t) l);
      }
   }
   P->nr = n; P->nc = nc; P->i = Pp; P->j = Pj; P->v = Pv;
   if (trunc_factor != 0.0 || max_elmts > 0) { or_truncate(P, trunc_factor, max_elmts); }
   for (int i = 0; i < n; i++) { if (CF[i] == SF_PT) { CF[i] = F_PT; } }
   for (int b = 0; b < nblk; b++) { or_csr_free(&Pi[b]); }
   free(Pi); free(blk); free(col); free(rsum); free(pass); free(order);
   return 0;
}

/* hypre_BoomerAMGCorrectCFMarker2Host src/parcsr_ls/par_strength.c:3096:
 * C points that the second coarsening made F become -2, the others 1. */
void or_correct_cf2(int n, int *CF, const int *CFN)
{
   int cnt = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] > 0) { CF[i] = CFN[cnt] == -1 ? -2 : 1; cnt++; }
   }
}

/* Modified extended+i interpolation, hypre_BoomerAMGBuildModExtPIInterpHost
 * src/parcsr_ls/par_mod_lr_interp.c:585-1215 with the F/C blocks of
 * hypre_ParCSRMatrixGenerateFFFCHost src/parcsr_mv/gen_fffc.c:18-530:
 * As_FF / As_FC are A restricted to strong connections (FF with the diagonal
 * first), W = As_FF As_FC after the D_q, D_w, D_theta scaling, P = [I; W]. */
static int mod_interp(const or_csr *A, const or_csr *S, const int *CF, int variant, or_csr *P);

int or_mod_extpi_interp(const or_csr *A, const or_csr *S, const int *CF, or_csr *P)
{
   return mod_interp(A, S, CF, 17, P);
}

/* The modified ("MM") interpolations (hypre_BoomerAMGBuildModExtInterpHost
 * :16-540, ModExtPIInterpHost :585-1215, ModExtPEInterpHost :1260-1855 of
 * src/parcsr_ls/par_mod_lr_interp.c): variant 16 extended, 17 extended+i,
 * 18 extended+e.  They share As_FF / As_FC, W = As_FF As_FC and P = [I; W];
 * they differ in the row scalings applied before the product. */
static int mod_interp(const or_csr *A, const or_csr *S, const int *CF, int variant, or_csr *P)
{
   int n = A->nr;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1)), *f2f = xmalloc(sizeof(int) * (n ? n : 1));
   int nc = 0, nf = 0;
   for (int i = 0; i < n; i++) { if (CF[i] > 0) { f2c[i] = nc++; f2f[i] = -1; } else { f2f[i] = nf++; f2c[i] = -1; } }
   /* As_FF, As_FC */
   int *FFi = xcalloc(nf + 1, sizeof(int)), *FCi = xcalloc(nf + 1, sizeof(int));
   int row = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] >= 0 && CF[i] > 0) { continue; }
      if (CF[i] > 0) { continue; }
      int ff = 0, fc = 0;
      if (A->i[i] < A->i[i + 1] && A->j[A->i[i]] == i) { ff++; }
      for (int k = S->i[i]; k < S->i[i + 1]; k++) { if (CF[S->j[k]] > 0) { fc++; } else { ff++; } }
      FFi[row + 1] = FFi[row] + ff; FCi[row + 1] = FCi[row] + fc; row++;
   }
   int *FFj = xmalloc(sizeof(int) * (FFi[nf] ? FFi[nf] : 1)), *FCj = xmalloc(sizeof(int) * (FCi[nf] ? FCi[nf] : 1));
   double *FFv = xmalloc(sizeof(double) * (FFi[nf] ? FFi[nf] : 1)), *FCv = xmalloc(sizeof(double) * (FCi[nf] ? FCi[nf] : 1));
   row = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] > 0) { continue; }
      int pf = FFi[row], pc = FCi[row];
      int jA = A->i[i];
      if (jA < A->i[i + 1] && A->j[jA] == i) { FFj[pf] = f2f[i]; FFv[pf++] = A->v[jA]; }
      for (int k = S->i[i]; k < S->i[i + 1]; k++)
      {
         jA = A->i[i];
         if (jA < A->i[i + 1] && A->j[jA] == i) { jA++; }
         int jS = S->j[k];
         while (A->j[jA] != jS) { jA++; }
         if (CF[jS] > 0) { FCj[pc] = f2c[jS]; FCv[pc++] = A->v[jA]; }
         else { FFj[pf] = f2f[jS]; FFv[pf++] = A->v[jA]; }
      }
      row++;
   }
   double *Dq = xcalloc(nf, sizeof(double)), *Dw = xcalloc(nf, sizeof(double)), *Dt = xcalloc(nf, sizeof(double));
   double *tmp = xmalloc(sizeof(double) * (FFi[nf] ? FFi[nf] : 1));
   if (variant == 16 || variant == 18)
   {
      /* D_w = A row sum - FF off-diagonals - FC row sum (:240-310, :1570-1627) */
      double *Dl = xcalloc(nf, sizeof(double)), *Dx = xcalloc(nf, sizeof(double));
      for (int r = 0; r < nf; r++)
      {
         if (variant == 18)
         {
            for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { Dl[r] += FFv[k]; }
            double number = (double) (FFi[r + 1] - FFi[r] - 1);
            if (number != 0.0) { Dl[r] /= number; }
         }
         for (int k = FCi[r]; k < FCi[r + 1]; k++) { Dq[r] += FCv[k]; }
         if (variant == 18 && Dl[r] + Dq[r] != 0.0) { Dx[r] = Dl[r] / (Dq[r] + Dl[r]); }
      }
      row = 0;
      for (int i = 0; i < n; i++)
      {
         if (CF[i] > 0) { continue; }
         for (int k = A->i[i]; k < A->i[i + 1]; k++) { Dw[row] += A->v[k]; }
         for (int k = FFi[row] + 1; k < FFi[row + 1]; k++) { Dw[row] -= FFv[k]; }
         Dw[row] -= Dq[row];
         row++;
      }
      for (int r = 0; r < nf; r++)
      {
         if (variant == 16)
         {
            /* :316-354 */
            double beta = Dw[r] != 0.0 ? 1.0 / Dw[r] : 1.0;
            FFv[FFi[r]] = beta * Dq[r];
            double gamma = Dq[r] != 0.0 ? -1.0 / Dq[r] : 1.0;
            for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { FFv[k] *= beta; }
            for (int k = FCi[r]; k < FCi[r + 1]; k++) { FCv[k] *= gamma; }
         }
         else
         {
            /* D_tau and the scalings, :1629-1662 */
            for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { Dt[r] += FFv[k] * Dx[FFj[k]]; }
         }
      }
      if (variant == 18)
      {
         for (int r = 0; r < nf; r++)
         {
            double value = Dw[r] + Dt[r];
            if (value != 0.0) { value = -1.0 / value; }
            double theta = Dq[r] + Dl[r];
            FFv[FFi[r]] = value * theta;
            if (theta != 0.0) { theta = 1.0 / theta; }
            for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { FFv[k] *= value; }
            for (int k = FCi[r]; k < FCi[r + 1]; k++) { FCv[k] *= theta; }
         }
      }
      free(Dl); free(Dx);
      goto product;
   }
   for (int r = 0; r < nf; r++) { for (int k = FCi[r]; k < FCi[r + 1]; k++) { Dq[r] += FCv[k]; } }
   memcpy(tmp, FFv, sizeof(double) * FFi[nf]);
   row = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] >= 0) { if (CF[i] > 0) { continue; } }
      if (CF[i] > 0) { continue; }
      for (int k = A->i[i]; k < A->i[i + 1]; k++) { Dw[row] += A->v[k]; }
      for (int k = FFi[row] + 1; k < FFi[row + 1]; k++) { Dw[row] -= FFv[k]; }
      Dw[row] -= Dq[row];
      row++;
   }
   for (int r = 0; r < nf; r++)
   {
      for (int j = FFi[r] + 1; j < FFi[r + 1]; j++)
      {
         int jj = FFj[j];
         double value = Dq[jj];
         for (int k = FFi[jj] + 1; k < FFi[jj + 1]; k++)
         {
            if (FFj[k] == r)
            {
               double value1 = tmp[k];
               value += value1;
               Dt[r] += FFv[j] * value1 / value;
               break;
            }
         }
         if (value != 0.0) { FFv[j] /= value; }
      }
      FFv[FFi[r]] = 1.0;
   }
   for (int r = 0; r < nf; r++)
   {
      double theta = Dt[r] + Dw[r];
      if (theta != 0.0)
      {
         theta = -1.0 / theta;
         for (int j = FFi[r]; j < FFi[r + 1]; j++) { FFv[j] *= theta; }
      }
   }
product:;
   or_csr FF = { nf, nf, FFi, FFj, FFv }, FC = { nf, nc, FCi, FCj, FCv }, W;
   or_matmul(&FF, &FC, &W);
   /* P = [I; W] in fine order */
   int *Pi = xcalloc(n + 1, sizeof(int));
   row = 0;
   for (int i = 0; i < n; i++)
   {
      int len = CF[i] > 0 ? 1 : W.i[row + 1] - W.i[row];
      if (CF[i] <= 0) { row++; }
      Pi[i + 1] = Pi[i] + len;
   }
   int *Pj = xmalloc(sizeof(int) * (Pi[n] ? Pi[n] : 1));
   double *Pv = xmalloc(sizeof(double) * (Pi[n] ? Pi[n] : 1));
   row = 0;
   for (int i = 0; i < n; i++)
   {
      int c = Pi[i];
      if (CF[i] > 0) { Pj[c] = f2c[i]; Pv[c] = 1.0; }
      else
      {
         for (int k = W.i[row]; k < W.i[row + 1]; k++) { Pj[c] = W.j[k]; Pv[c] = W.v[k]; c++; }
         row++;
      }
   }
   P->nr = n; P->nc = nc; P->i = Pi; P->j = Pj; P->v = Pv;
   or_csr_free(&FF); or_csr_free(&FC); or_csr_free(&W);
   free(f2c); free(f2f); free(Dq); free(Dw); free(Dt); free(tmp);
   return 0;
}

/* Modified partial interpolations of the second stage:
 * variant 5 extended, hypre_BoomerAMGBuildModPartialExtInterpHost
 * src/parcsr_ls/par_2s_interp.c:15-620; variant 7 extended+e,
 * hypre_BoomerAMGBuildModPartialExtPEInterpHost :662-1320.  Blocks
 * (hypre_ParCSRMatrixGenerateFFFC3 / FFFCD3, src/parcsr_mv/gen_fffc.c:568-1105
 * / 1108-1560): FC over every non-C point (its strong C neighbours in S order),
 * FF over the CF -2 points (the diagonal, then the strong non-C neighbours in
 * S order; columns number the non-C points), and for variant 7 D_lambda =
 * the mean of each non-C row's strong non-C values.  D_q = FC row sums.
 * Variant 5 (:261-417): D_w = A row sum - FF off-diagonals whose column has
 * D_q != 0 - D_q; FF's diagonal becomes D_q / D_w and its off-diagonals are
 * divided by D_w (when D_w != 0); FC rows are scaled by -1 / D_q (0 when D_q
 * is zero).  Variant 7 (:897-1055): D_inv = 1 / (D_q + D_lambda) (0 when that
 * is zero), D_tau = sum FF_ij D_lambda_j D_inv_j, D_w = A row sum - FF
 * off-diagonals whose column has D_inv != 0 + (D_tau - D_q); with beta =
 * -1 / D_w FF's diagonal becomes beta (D_q + D_lambda) and its off-diagonals
 * are scaled by beta; FC rows by D_inv.  W = FF FC (hypre_ParMatmul); P over
 * the old C points in row order (CF 1 identity, CF -2 the row of W), columns
 * the new C points.  CF is not changed. */
int or_mod_partial_interp(const or_csr *A, const or_csr *S, const int *CF, int variant, or_csr *P)
{
   const int n = A->nr;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1)), *f2f = xmalloc(sizeof(int) * (n ? n : 1));
   int nc = 0, nf = 0, nn = 0;
   for (int i = 0; i < n; i++)
   {
      f2c[i] = f2f[i] = -1;
      if (CF[i] > 0) { f2c[i] = nc++; }
      else { f2f[i] = nf++; if (CF[i] == -2) { nn++; } }
   }
   int *nlist = xmalloc(sizeof(int) * (nn ? nn : 1));
   int *FCi = xcalloc(nf + 1, sizeof(int)), *FFi = xcalloc(nn + 1, sizeof(int));
   for (int i = 0, t = 0; i < n; i++)
   {
      if (CF[i] > 0) { continue; }
      int c = 0, f = 0;
      for (int k = S->i[i]; k < S->i[i + 1]; k++) { if (CF[S->j[k]] > 0) { c++; } else { f++; } }
      FCi[f2f[i] + 1] = c;
      if (CF[i] == -2) { nlist[t] = i; FFi[t + 1] = f + 1; t++; }
   }
   for (int r = 0; r < nf; r++) { FCi[r + 1] += FCi[r]; }
   for (int t = 0; t < nn; t++) { FFi[t + 1] += FFi[t]; }
   int *FCj = xmalloc(sizeof(int) * (FCi[nf] ? FCi[nf] : 1)), *FFj = xmalloc(sizeof(int) * (FFi[nn] ? FFi[nn] : 1));
   double *FCv = xmalloc(sizeof(double) * (FCi[nf] ? FCi[nf] : 1));
   double *FFv = xmalloc(sizeof(double) * (FFi[nn] ? FFi[nn] : 1));
   double *lam = xcalloc(nf ? nf : 1, sizeof(double));
   for (int i = 0, t = 0; i < n; i++)
   {
      if (CF[i] > 0) { continue; }
      const int r = f2f[i], isnew = CF[i] == -2;
      int qc = FCi[r], qf = isnew ? FFi[t] : 0;
      if (isnew) { FFj[qf] = f2f[A->j[A->i[i]]]; FFv[qf] = A->v[A->i[i]]; qf++; }
      double sum = 0;
      for (int k = S->i[i]; k < S->i[i + 1]; k++)
      {
         const int js = S->j[k];
         int ja = A->i[i] + 1;
         while (A->j[ja] != js) { ja++; }
         if (CF[js] > 0) { FCj[qc] = f2c[js]; FCv[qc] = A->v[ja]; qc++; }
         else
         {
            sum += 1;
            lam[r] += A->v[ja];
            if (isnew) { FFj[qf] = f2f[js]; FFv[qf] = A->v[ja]; qf++; }
         }
      }
      if (sum != 0.0) { lam[r] = lam[r] / sum; }
      if (isnew) { t++; }
   }
   double *Dq = xcalloc(nf ? nf : 1, sizeof(double)), *Dinv = xcalloc(nf ? nf : 1, sizeof(double));
   for (int r = 0; r < nf; r++)
   {
      for (int k = FCi[r]; k < FCi[r + 1]; k++) { Dq[r] += FCv[k]; }
      if (variant == 7 && Dq[r] + lam[r] != 0.0) { Dinv[r] = 1.0 / (Dq[r] + lam[r]); }
   }
   for (int t = 0; t < nn; t++)
   {
      const int i = nlist[t], self = f2f[i];
      double tau = 0.0, w = 0.0;
      if (variant == 7)
      {
         for (int k = FFi[t] + 1; k < FFi[t + 1]; k++) { tau += FFv[k] * lam[FFj[k]] * Dinv[FFj[k]]; }
      }
      for (int k = A->i[i]; k < A->i[i + 1]; k++) { w += A->v[k]; }
      if (variant == 7)
      {
         for (int k = FFi[t] + 1; k < FFi[t + 1]; k++) { if (Dinv[FFj[k]] != 0.0) { w -= FFv[k]; } }
         w += tau - Dq[self];
         if (w != 0.0)
         {
            const double beta = -1.0 / w;
            FFv[FFi[t]] = beta * (Dq[self] + lam[self]);
            for (int k = FFi[t] + 1; k < FFi[t + 1]; k++) { FFv[k] *= beta; }
         }
      }
      else
      {
         for (int k = FFi[t] + 1; k < FFi[t + 1]; k++) { if (Dq[FFj[k]] != 0.0) { w -= FFv[k]; } }
         w -= Dq[self];
         if (w != 0.0)
         {
            const double beta = 1.0 / w;
            FFv[FFi[t]] = beta * Dq[self];
            for (int k = FFi[t] + 1; k < FFi[t + 1]; k++) { FFv[k] *= beta; }
         }
      }
   }
   for (int r = 0; r < nf; r++)
   {
      double gamma;
      if (variant == 7) { gamma = Dinv[r]; }
      else { gamma = Dq[r] != 0.0 ? -1.0 / Dq[r] : 0.0; }
      for (int k = FCi[r]; k < FCi[r + 1]; k++) { FCv[k] *= gamma; }
   }
   or_csr FF = {nn, nf, FFi, FFj, FFv}, FC = {nf, nc, FCi, FCj, FCv}, W;
   or_matmul(&FF, &FC, &W);
   int nco = nc + nn;
   int *Pi = xcalloc(nco + 1, sizeof(int));
   int *Pj = xmalloc(sizeof(int) * (size_t) (nc + W.i[nn] ? nc + W.i[nn] : 1));
   double *Pv = xmalloc(sizeof(double) * (size_t) (nc + W.i[nn] ? nc + W.i[nn] : 1));
   int c = 0, rowp = 0, t = 0;
   for (int i = 0; i < n; i++)
   {
      if (CF[i] > 0) { Pj[c] = f2c[i]; Pv[c] = 1.0; c++; Pi[++rowp] = c; }
      else if (CF[i] == -2)
      {
         for (int k = W.i[t]; k < W.i[t + 1]; k++) { Pj[c] = W.j[k]; Pv[c] = W.v[k]; c++; }
         t++;
         Pi[++rowp] = c;
      }
   }
   P->nr = nco; P->nc = nc; P->i = Pi; P->j = Pj; P->v = Pv;
   or_csr_free(&FF); or_csr_free(&FC); or_csr_free(&W);
   free(f2c); free(f2f); free(nlist); free(lam); free(Dq); free(Dinv);
   return 0;
}

/* Partial extended+i interpolation, hypre_BoomerAMGBuildPartialExtPIInterp
 * src/parcsr_ls/partial.c:16-720: extended+i weights (as
 * or_extpi_interp) for the rows of the old C points only (CF == 1 identity,
 * CF == -2 interpolated); rows numbered by old coarse index, columns by new.
 * Afterwards CF values below -1 become -1 (:700). */
static int partial_ext_interp(const or_csr *A, const or_csr *S, int *CF, int iterm, or_csr *P);

int or_partial_extpi_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P)
{
   return partial_ext_interp(A, S, CF, 1, P);
}

/* Partial extended interpolation, hypre_BoomerAMGBuildPartialExtInterp
 * src/parcsr_ls/partial.c:1902-2635: the same rows, pattern and weights as
 * the partial extended+i interpolation without the i terms (a strong F
 * neighbour's connection back to i takes no share of the distribution). */
int or_partial_ext_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P)
{
   return partial_ext_interp(A, S, CF, 0, P);
}

static int partial_ext_interp(const or_csr *A, const or_csr *S, int *CF, int iterm, or_csr *P)
{
   int n = A->nr;
   int *f2c = xmalloc(sizeof(int) * (n ? n : 1));
   int nco = 0, nc = 0;
   for (int i = 0; i < n; i++) { f2c[i] = -1; if (CF[i] == 1) { f2c[i] = nc++; nco++; } else if (CF[i] == -2) { nco++; } }
   int *oc2f = xmalloc(sizeof(int) * (nco ? nco : 1));
   nco = 0;
   for (int i = 0; i < n; i++) { if (CF[i] == 1 || CF[i] == -2) { oc2f[nco++] = i; } }
   int *Pi = xcalloc(nco + 1, sizeof(int));
   int *marker = xmalloc(sizeof(int) * (n ? n : 1));
   for (int i = 0; i < n; i++) { marker[i] = -1; }
   for (int ii = 0; ii < nco; ii++)
   {
      int i = oc2f[ii], cnt = 0;
      if (CF[i] > 0) { cnt = 1; }
      else if (CF[i] == -2)
      {
         for (int k = S->i[i]; k < S->i[i + 1]; k++)
         {
            int i1 = S->j[k];
            if (CF[i1] > 0) { if (marker[i1] != i) { marker[i1] = i; cnt++; } }
            else if (CF[i1] != SF_PT)
            {
               for (int kk = S->i[i1]; kk < S->i[i1 + 1]; kk++)
               {
                  int k1 = S->j[kk];
                  if (CF[k1] > 0 && marker[k1] != i) { marker[k1] = i; cnt++; }
               }
            }
         }
      }
      Pi[ii + 1] = Pi[ii] + cnt;
   }
   int nnz = Pi[nco];
   int *Pj = xmalloc(sizeof(int) * (nnz ? nnz : 1));
   double *Pv = xmalloc(sizeof(double) * (nnz ? nnz : 1));
   int *pmark = xmalloc(sizeof(int) * (n ? n : 1));
   for (int i = 0; i < n; i++) { pmark[i] = -1; }
   int strong_f = -2;
   for (int ii = 0; ii < nco; ii++)
   {
      int i = oc2f[ii];
      int begin = Pi[ii], c = begin;
      if (CF[i] > 0) { Pj[c] = f2c[i]; Pv[c] = 1.0; c++; }
      else if (CF[i] == -2)
      {
         strong_f--;
         for (int k = S->i[i]; k < S->i[i + 1]; k++)
         {
            int i1 = S->j[k];
            if (CF[i1] >= 0)
            {
               if (pmark[i1] < begin) { pmark[i1] = c; Pj[c] = f2c[i1]; Pv[c] = 0.0; c++; }
            }
            else if (CF[i1] != SF_PT)
            {
               pmark[i1] = strong_f;
               for (int kk = S->i[i1]; kk < S->i[i1 + 1]; kk++)
               {
                  int k1 = S->j[kk];
                  if (CF[k1] >= 0 && pmark[k1] < begin) { pmark[k1] = c; Pj[c] = f2c[k1]; Pv[c] = 0.0; c++; }
               }
            }
         }
         int end = c;
         double diagonal = A->v[A->i[i]];
         for (int jj = A->i[i] + 1; jj < A->i[i + 1]; jj++)
         {
            int i1 = A->j[jj];
            if (pmark[i1] >= begin) { Pv[pmark[i1]] += A->v[jj]; }
            else if (pmark[i1] == strong_f)
            {
               double sum = 0.0;
               int sgn = A->v[A->i[i1]] < 0 ? -1 : 1;
               for (int jj1 = A->i[i1] + 1; jj1 < A->i[i1 + 1]; jj1++)
               {
                  int i2 = A->j[jj1];
                  if ((pmark[i2] >= begin || (iterm && i2 == i)) && (sgn * A->v[jj1]) < 0) { sum += A->v[jj1]; }
               }
               if (sum != 0)
               {
                  double distribute = A->v[jj] / sum;
                  for (int jj1 = A->i[i1] + 1; jj1 < A->i[i1 + 1]; jj1++)
                  {
                     int i2 = A->j[jj1];
                     if (pmark[i2] >= begin && (sgn * A->v[jj1]) < 0) { Pv[pmark[i2]] += distribute * A->v[jj1]; }
                     if (iterm && i2 == i && (sgn * A->v[jj1]) < 0) { diagonal += distribute * A->v[jj1]; }
                  }
               }
               else { diagonal += A->v[jj]; }
            }
            else if (CF[i1] != SF_PT) { diagonal += A->v[jj]; }
         }
         if (diagonal != 0.0) { for (int k = begin; k < end; k++) { Pv[k] /= -diagonal; } }
      }
      strong_f--;
   }
   for (int i = 0; i < n; i++) { if (CF[i] < -1) { CF[i] = -1; } }
   P->nr = nco; P->nc = nc; P->i = Pi; P->j = Pj; P->v = Pv;
   free(f2c); free(oc2f); free(marker); free(pmark);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* l1 norms, hypre_ParCSRComputeL1Norms src/parcsr_ls/ams.c:517-790          */
/* option 1: sum |a_ij| (relax 18); option 4: |a_ii| on one process (relax  */
/* 8/13/14); option 5: diagonal, 0 -> 1 (relax 7/11/12)                      */
/* ------------------------------------------------------------------------ */

int or_l1_norms(const or_csr *A, int option, double *l1)
{
   return or_l1_norms_cf(A, option, NULL, l1);
}

/* CF != NULL (option 1 with relax_order 1, par_amg_setup.c:3352-3360): the
 * row sum takes only the columns of the row's own CF value
 * (hypre_CSRMatrixComputeRowSumHost src/seq_mv/csr_matop.c:1866-1905) */
int or_l1_norms_cf(const or_csr *A, int option, const int *CF, double *l1)
{
   int n = A->nr;
   #pragma omp parallel for schedule(static)
   for (int i = 0; i < n; i++)
   {
      double d = 0.0, s = 0.0;
      for (int k = A->i[i]; k < A->i[i + 1]; k++)
      {
         if (A->j[k] == i) { d = A->v[k]; }
         if (CF && CF[i] != CF[A->j[k]]) { continue; }
         s += fabs(A->v[k]);
      }
      double v;
      if (option == 1) { v = s; }
      else if (option == 4) { v = fabs(d); }   /* one process: |a_ii| (ams.c:649-684) */
      else { v = d != 0.0 ? d : 1.0; }
      if (d < 0.0) { v = -v; }   /* negative-definite rows, :747-770 */
      l1[i] = v;
   }
   return 0;
}

/* ------------------------------------------------------------------------ */
/* Vectors and SpMV (hypre_CSRMatrixMatvecOutOfPlaceHost csr_matvec.c:22)    */
/* ------------------------------------------------------------------------ */

void or_matvec(double alpha, const or_csr *A, const double *x, double beta, const double *b, double *y)
{
   int n = A->nr;
   #pragma omp parallel for schedule(static)
   for (int i = 0; i < n; i++)
   {
      double s = 0.0;
      for (int k = A->i[i]; k < A->i[i + 1]; k++) { s += A->v[k] * x[A->j[k]]; }
      y[i] = alpha * s + (beta != 0.0 ? beta * b[i] : 0.0);
   }
}

static void matvecT(const or_csr *A, const double *x, double *y)
{
   /* y = A^T x (restriction), hypre_CSRMatrixMatvecTHost csr_matvec.c:914 */
   for (int c = 0; c < A->nc; c++) { y[c] = 0.0; }
   for (int r = 0; r < A->nr; r++)
   {
      for (int k = A->i[r]; k < A->i[r + 1]; k++) { y[A->j[k]] += A->v[k] * x[r]; }
   }
}

double or_dot(int n, const double *x, const double *y)
{
   double s = 0.0;
   #pragma omp parallel for reduction(+ : s) schedule(static)
   for (int i = 0; i < n; i++) { s += x[i] * y[i]; }
   return s;
}

/* ------------------------------------------------------------------------ */
/* Coarsest solve: hypre_gselim (src/utilities/gselim.h) on a dense copy,    */
/* as hypre_GaussElimSolve type 9 (src/parcsr_ls/par_gauss_elim.c:642-646)   */
/* ------------------------------------------------------------------------ */

static void gselim(double *A, double *x, int n)
{
   if (n == 1) { if (A[0] != 0.0) { x[0] = x[0] / A[0]; } return; }
   for (int k = 0; k < n - 1; k++)
   {
      if (A[k * n + k] != 0.0)
      {
         double divA = 1.0 / A[k * n + k];
         for (int j = k + 1; j < n; j++)
         {
            if (A[j * n + k] != 0.0)
            {
               double factor = A[j * n + k] * divA;
               for (int m = k + 1; m < n; m++) { A[j * n + m] -= factor * A[k * n + m]; }
               x[j] -= factor * x[k];
            }
         }
      }
   }
   for (int k = n - 1; k > 0; --k)
   {
      if (A[k * n + k] != 0.0)
      {
         x[k] /= A[k * n + k];
         for (int j = 0; j < k; j++) { if (A[j * n + k] != 0.0) { x[j] -= x[k] * A[j * n + k]; } }
      }
   }
   if (A[0] != 0.0) { x[0] /= A[0]; }
}

/* ------------------------------------------------------------------------ */
/* Smoothers                                                                */
/* ------------------------------------------------------------------------ */

static void relax_l1_jacobi(const or_csr *A, const double *f, const double *l1, double w,
                            double *u, double *V, int u_zero, const int *CF, int pts)
{
   /* hypre_BoomerAMGRelax7Jacobi src/parcsr_ls/par_relax.c:1178 (relax 18 calls it
    * for relax_points == 0, :338-365): V = w(f - Au); u += V / l1, with
    * relax_points != 0 only where CF == relax_points (:1237-1240) */
   int n = A->nr;
   if (u_zero) { for (int i = 0; i < n; i++) { V[i] = w * f[i]; } }
   else { or_matvec(-w, A, u, w, f, V); }
   for (int i = 0; i < n; i++) { if (!pts || CF[i] == pts) { u[i] += V[i] / l1[i]; } }
}

static void relax_jacobi_cf(const or_csr *A, const double *f, const double *l1, double w, double *u, double *V,
                            const int *CF, int pts)
{
   /* relax 18 with relax_points != 0 on the host,
    * hypre_BoomerAMGRelaxWeightedJacobi_core src/parcsr_ls/par_relax.c:180-320
    * (Skip_diag 0): over the values from before the relaxation, rows with
    * CF == relax_points and l1 != 0 take u += w * (f - A u) / l1, the
    * residual summed in row order */
   int n = A->nr;
   memcpy(V, u, sizeof(double) * (size_t) n);
   for (int i = 0; i < n; i++)
   {
      if (CF[i] != pts || l1[i] == 0.0) { continue; }
      double res = f[i];
      for (int jj = A->i[i]; jj < A->i[i + 1]; jj++) { res -= A->v[jj] * V[A->j[jj]]; }
      u[i] += w * res / l1[i];
   }
}

static void relax_two_stage_gs(const or_csr *A, const double *f, double w, int inner,
                               double *u, double *V, int u_zero)
{
   /* hypre_BoomerAMGRelaxTwoStageGaussSeidelHost src/parcsr_ls/par_relax.c:1506-1590 */
   int n = A->nr;
   if (u_zero) { for (int i = 0; i < n; i++) { V[i] = w * f[i]; } }
   else { or_matvec(-w, A, u, w, f, V); }
   double mult = 1.0;
   for (int i = 0; i < n; i++) { V[i] /= A->v[A->i[i]]; u[i] += mult * V[i]; }
   mult *= -1.0;
   for (int k = 0; k < inner; k++)
   {
      for (int i = n - 1; i >= 0; i--)
      {
         double res = 0.0;
         for (int jj = A->i[i]; jj < A->i[i + 1]; jj++) { if (A->j[jj] < i) { res += A->v[jj] * V[A->j[jj]]; } }
         V[i] = res / A->v[A->i[i]];
         u[i] += mult * V[i];
      }
      mult *= -1.0;
   }
}

/* ------------------------------------------------------------------------ */
/* Chebyshev smoother (relax 16)                                             */
/* ------------------------------------------------------------------------ */

static double pythag(double a, double b)
{
   /* sqrt(a^2 + b^2) without overflow: the iteration of Moler and Morrison
    * (IBM J. Res. Dev. 27, 1983) as used by EISPACK's PYTHAG */
   double aa = fabs(a), ab = fabs(b);
   double p = aa > ab ? aa : ab;
   if (p == 0.0) { return p; }
   double q = (aa < ab ? aa : ab) / p;
   double r = q * q;
   for (;;)
   {
      double t = r + 4.0;
      if (t == 4.0) { break; }
      double sr = r / t;
      double u = sr * 2.0 + 1.0;
      p = u * p;
      double v = sr / u;
      r = v * v * r;
   }
   return p;
}

int or_eig_tridiag(int n, double *d, double *e)
{
   /* Eigenvalues (ascending, in d) of the symmetric tridiagonal matrix with
    * diagonal d[0..n-1] and sub-diagonal e[1..n-1] (e[0] unused), by the
    * implicit QL method TQL1 of Bowdler, Martin, Reinsch and Wilkinson
    * (Numer. Math. 11, 293-306, 1968), as the reference calls it through
    * hypre_LINPACKcgtql1 (src/parcsr_ls/par_relax_more.c:507).  Returns the
    * 1-based index of an eigenvalue that did not converge in 30 steps, else 0. */
   if (n <= 1) { return 0; }
   for (int i = 1; i < n; i++) { e[i - 1] = e[i]; }
   e[n - 1] = 0.0;
   double f = 0.0, tst1 = 0.0;
   for (int l = 0; l < n; l++)
   {
      double h = fabs(d[l]) + fabs(e[l]);
      if (tst1 < h) { tst1 = h; }
      int m = l;
      while (tst1 + fabs(e[m]) != tst1) { m++; }   /* e[n-1] == 0 ends the search */
      if (m > l)
      {
         int steps = 0;
         do
         {
            if (steps == 30) { return l + 1; }
            steps++;
            /* Wilkinson-type shift from the leading 2x2 block */
            double g = d[l];
            double p = (d[l + 1] - g) / (e[l] * 2.0);
            double r = pythag(p, 1.0);
            double sg = p < 0.0 ? -1.0 : 1.0;
            d[l] = e[l] / (p + sg * r);
            d[l + 1] = e[l] * (p + sg * r);
            double dl1 = d[l + 1];
            h = g - d[l];
            for (int i = l + 2; i < n; i++) { d[i] -= h; }
            f += h;
            /* QL sweep from m-1 up to l */
            p = d[m];
            double c = 1.0, c2 = 1.0, c3 = 0.0, sn = 0.0, s2 = 0.0;
            double el1 = e[l + 1];
            for (int i = m - 1; i >= l; i--)
            {
               c3 = c2;
               c2 = c;
               s2 = sn;
               g = c * e[i];
               h = c * p;
               r = pythag(p, e[i]);
               e[i + 1] = sn * r;
               sn = e[i] / r;
               c = p / r;
               p = c * d[i] - sn * g;
               d[i + 1] = h + sn * (c * g + sn * d[i]);
            }
            p = -sn * s2 * c3 * el1 * e[l] / dl1;
            e[l] = sn * p;
            d[l] = c * p;
         } while (tst1 + fabs(e[l]) > tst1);
      }
      /* place d[l] + f among the already ordered d[0..l-1] */
      double p = d[l] + f;
      int i = l;
      while (i > 0 && p < d[i - 1]) { d[i] = d[i - 1]; i--; }
      d[i] = p;
   }
   return 0;
}

static void diag_inv_sqrt(const or_csr *A, double *ds)
{
   /* hypre_CSRMatrixExtractDiagonal type 4 (src/seq_mv/csr_matop.c:2100-2150):
    * 1/sqrt(|a_ii|) of the first entry in row i whose column is i, else 0 */
   for (int i = 0; i < A->nr; i++)
   {
      double di = 0.0;
      for (int k = A->i[i]; k < A->i[i + 1]; k++)
      {
         if (A->j[k] == i)
         {
            if (A->v[k] != 0.0) { di = 1.0 / sqrt(fabs(A->v[k])); }
            break;
         }
      }
      ds[i] = di;
   }
}

int or_max_eig_cg(const or_csr *A, int scale, int max_iter, double *max_eig, double *min_eig)
{
   /* hypre_ParCSRMaxEigEstimateCGHost src/parcsr_ls/par_relax_more.c:203-390:
    * max_iter steps of CG on D^{-1/2} A D^{-1/2} (or A) from a random start
    * (seed 1); the Lanczos tridiagonal built from the CG coefficients gives the
    * extreme eigenvalue estimates. */
   int n = A->nr;
   if (n < max_iter) { max_iter = n; }
   double *r = xmalloc(sizeof(double) * (n ? n : 1)), *p = xcalloc(n, sizeof(double));
   double *sv = xcalloc(n, sizeof(double)), *ds = xmalloc(sizeof(double) * (n ? n : 1));
   double *u = xcalloc(n, sizeof(double));
   double *td = xcalloc(max_iter + 1, sizeof(double)), *te = xcalloc(max_iter + 1, sizeof(double));
   or_rand_uniform(n, 1, r);
   if (scale) { diag_inv_sqrt(A, ds); }
   else { for (int i = 0; i < n; i++) { ds[i] = 1.0; } }
   double gamma = or_dot(n, r, p), gamma_old, beta = 1.0;
   int it = 0;
   while (it < max_iter)
   {
      memcpy(sv, r, sizeof(double) * n);
      gamma_old = gamma;
      gamma = or_dot(n, r, sv);
      if (gamma < 2.220446049250313e-16) { break; }
      if (it == 0) { beta = 1.0; memcpy(p, sv, sizeof(double) * n); }
      else
      {
         beta = gamma / gamma_old;
         for (int i = 0; i < n; i++) { p[i] = sv[i] + beta * p[i]; }
      }
      if (scale)
      {
         for (int i = 0; i < n; i++) { u[i] = ds[i] * p[i]; }
         or_matvec(1.0, A, u, 0.0, NULL, sv);
         for (int i = 0; i < n; i++) { sv[i] = ds[i] * sv[i]; }
      }
      else { or_matvec(1.0, A, p, 0.0, NULL, sv); }
      double sdotp = or_dot(n, sv, p);
      double alpha = gamma / sdotp;
      double ainv = 1.0 / alpha;
      td[it + 1] = ainv;
      td[it] *= beta;
      td[it] += ainv;
      te[it + 1] = ainv;
      te[it] *= sqrt(beta);
      for (int i = 0; i < n; i++) { r[i] += -alpha * sv[i]; }
      it++;
   }
   or_eig_tridiag(it, td, te);
   *max_eig = it > 0 ? td[it - 1] : 0.0;
   *min_eig = td[0];
   free(r); free(p); free(sv); free(ds); free(u); free(td); free(te);
   return 0;
}

int or_cheby_setup(const or_csr *A, double max_eig, double min_eig, double fraction, int order,
                   int scale, int variant, double *coefs, double *ds)
{
   /* hypre_ParCSRRelax_Cheby_Setup src/parcsr_ls/par_cheby_setup.c: the
    * coefficients of s(t), u <- u + s(A) r, where 1 - t s(t) is the Chebyshev
    * residual polynomial of the given order on [lower, upper] (upper = 1.1 *
    * max_eig, lower = min_eig + fraction * (upper - min_eig)); ds = D^{-1/2} */
   if (order > 4) { order = 4; }
   if (order < 1) { order = 1; }
   int co = order - 1;
   double upper, lower;
   if (max_eig <= 0.0)
   {
      upper = min_eig * 1.1;
      lower = max_eig - (max_eig - upper) * fraction;
   }
   else
   {
      upper = max_eig * 1.1;
      lower = (upper - min_eig) * fraction + min_eig;
   }
   double th = (upper + lower) / 2, de = (upper - lower) / 2, den;
   for (int k = 0; k <= co; k++) { coefs[k] = 0.0; }
   if (variant == 1)
   {
      if (co == 0) { coefs[0] = fabs(th) > 0.0 ? 1.0 / th : 0.0; }
      else if (co == 1)
      {
         den = th * th + de * th;
         if (fabs(den) > 0.0) { coefs[0] = (de + 2 * th) / den; coefs[1] = -1.0 / den; }
      }
      else if (co == 2)
      {
         den = 2 * de * th * th - de * de * th - pow(de, 3) + 2 * pow(th, 3);
         if (fabs(den) > 0.0)
         {
            coefs[0] = (4 * de * th - pow(de, 2) + 6 * pow(th, 2)) / den;
            coefs[1] = -(2 * de + 6 * th) / den;
            coefs[2] = 2 / den;
         }
      }
      else
      {
         den = -4 * de * pow(th, 3) + 3 * pow(de, 2) * pow(th, 2) + 3 * pow(de, 3) * th - 4 * pow(th, 4);
         if (fabs(den) > 0.0)
         {
            coefs[0] = (6 * pow(de, 2) * th - 12 * de * pow(th, 2) + 3 * pow(de, 3) - 16 * pow(th, 3)) / den;
            coefs[1] = (12 * de * th - 3 * pow(de, 2) + 24 * pow(th, 2)) / den;
            coefs[2] = -(4 * de + 16 * th) / den;
            coefs[3] = 4 / den;
         }
      }
   }
   else
   {
      if (co == 0) { coefs[0] = fabs(th) > 0.0 ? 1.0 / th : 0.0; }
      else if (co == 1)
      {
         den = de * de - 2 * th * th;
         if (fabs(den) > 0.0) { coefs[0] = -4 * th / den; coefs[1] = 2 / den; }
      }
      else if (co == 2)
      {
         den = 3 * (de * de) * th - 4 * (th * th * th);
         if (fabs(den) > 0.0)
         {
            coefs[0] = (3 * de * de - 12 * th * th) / den;
            coefs[1] = 12 * th / den;
            coefs[2] = -4 / den;
         }
      }
      else
      {
         den = pow(de, 4) - 8 * ((de * th) * (de * th)) + pow(th, 4) * 8;
         if (fabs(den) > 0.0)
         {
            coefs[0] = (32 * pow(th, 3) - 16 * de * de * th) / den;
            coefs[1] = (8 * de * de - 48 * th * th) / den;
            coefs[2] = 32 * th / den;
            coefs[3] = -8 / den;
         }
      }
   }
   if (scale) { diag_inv_sqrt(A, ds); }
   else { for (int i = 0; i < A->nr; i++) { ds[i] = 1.0; } }
   return 0;
}

static void relax_cheby(const or_csr *A, const double *f, const double *ds, const double *coefs, int order,
                        int scale, double *u, double *r, double *o, double *v, double *tmp)
{
   /* hypre_ParCSRRelax_Cheby_SolveHost src/parcsr_ls/par_cheby_solve.c:194-330 */
   int n = A->nr;
   if (order > 4) { order = 4; }
   if (order < 1) { order = 1; }
   int co = order - 1;
   if (!scale)
   {
      or_matvec(-1.0, A, u, 1.0, f, r);
      for (int i = 0; i < n; i++) { o[i] = u[i]; u[i] = r[i] * coefs[co]; }
      for (int k = co - 1; k >= 0; k--)
      {
         or_matvec(1.0, A, u, 0.0, NULL, v);
         for (int i = 0; i < n; i++) { u[i] = coefs[k] * r[i] + v[i]; }
      }
      for (int i = 0; i < n; i++) { u[i] = o[i] + u[i]; }
      return;
   }
   or_matvec(-1.0, A, u, 0.0, NULL, tmp);
   for (int i = 0; i < n; i++) { r[i] = ds[i] * (f[i] + tmp[i]); }
   for (int i = 0; i < n; i++) { o[i] = u[i]; u[i] = r[i] * coefs[co]; }
   for (int k = co - 1; k >= 0; k--)
   {
      for (int i = 0; i < n; i++) { tmp[i] = ds[i] * u[i]; }
      or_matvec(1.0, A, tmp, 0.0, NULL, v);
      for (int i = 0; i < n; i++) { u[i] = coefs[k] * r[i] + ds[i] * v[i]; }
   }
   for (int i = 0; i < n; i++) { u[i] = o[i] + ds[i] * u[i]; }
}

/* Hybrid Gauss-Seidel on one process (relax 3/4/6 and 8/13/14):
 * hypre_BoomerAMGRelaxHybridGaussSeidel_core src/parcsr_ls/par_relax.c:692-945
 * with one thread, whose sweeps are hypre_HybridGaussSeidelNS (unscaled,
 * src/parcsr_ls/par_relax.h:13-108) and hypre_HybridGaussSeidel (scaled,
 * :222-330).  dir0: direction of the first sweep; nsw: 1, or 2 for the
 * symmetric types (a forward then a backward sweep); d: l1 norms or NULL
 * (the row's first entry, the diagonal); skip: leave the first entry out of
 * the sums.  Vt: the values before the relaxation (the scaled form's Vtemp). */
static void relax_hybrid_gs(const or_csr *A, const double *f, const double *d, double w, double omega, int dir0,
                            int nsw, int skip, double *u, double *Vt, const int *CF, int pts)
{
   int n = A->nr;
   const int non_scale = w == 1.0 && omega == 1.0;
   const double prod = 1.0 - w * omega, one_minus_omega = 1.0 - omega;
   if (!non_scale) { memcpy(Vt, u, sizeof(double) * (size_t) n); }
   for (int sw = 0; sw < nsw; sw++)
   {
      const int dir = sw == 0 ? dir0 : -dir0;
      const int ib = dir > 0 ? 0 : n - 1, ie = dir > 0 ? n : -1;
      for (int i = ib; i != ie; i += dir)
      {
         const double di = d ? d[i] : A->v[A->i[i]];
         if (di == 0.0 || (pts && CF[i] != pts)) { continue; }
         if (non_scale)
         {
            double res = f[i];
            for (int jj = A->i[i] + skip; jj < A->i[i + 1]; jj++) { res -= A->v[jj] * u[A->j[jj]]; }
            if (skip) { u[i] = res / di; }
            else { u[i] += res / di; }
         }
         else
         {
            double res = f[i], res0 = 0.0, res2 = 0.0;
            for (int jj = A->i[i] + skip; jj < A->i[i + 1]; jj++)
            {
               res0 -= A->v[jj] * u[A->j[jj]];
               res2 += A->v[jj] * Vt[A->j[jj]];
            }
            if (skip) { u[i] *= prod; }
            u[i] += w * (omega * res + res0 + one_minus_omega * res2) / di;
         }
      }
   }
}

static int hybrid_gs_type(int t) { return t == 3 || t == 4 || t == 6 || t == 8 || t == 13 || t == 14; }

/* One relaxation (hypre_BoomerAMGRelax src/parcsr_ls/par_relax.c:20-172);
 * pts: relax_points (0 all points; 1 / -1 only the points with that CF value,
 * for the smoothers that look at it: Jacobi and hybrid Gauss-Seidel) */
static void relax(or_hierarchy *H, int lvl, int type, const double *f, double *u, int u_zero, int pts)
{
   const int *CF = pts ? H->CF[lvl] : NULL;
   const or_csr *A = &H->A[lvl];
   double w = H->prm.relax_weight;
   if (type == 16)
   {
      int n = A->nr;
      double *r = xmalloc(sizeof(double) * (n ? n : 1)), *o = xmalloc(sizeof(double) * (n ? n : 1));
      double *tmp = xmalloc(sizeof(double) * (n ? n : 1));
      relax_cheby(A, f, H->cheby_ds[lvl], H->cheby_coefs[lvl], H->prm.cheby_order, H->prm.cheby_scale, u, r, o,
                  H->Vtmp, tmp);
      free(r); free(o); free(tmp);
      return;
   }
   if (hybrid_gs_type(type))
   {
      /* par_relax.c:954-1377: 3 forward, 4 backward, 6 symmetric (diagonal);
       * 13 forward, 14 backward, 8 symmetric (l1 norms; the diagonal term
       * stays in the sum unless weighted) */
      const int l1 = type == 8 || type == 13 || type == 14;
      const double omega = H->prm.outer_weight;   /* hypre_BoomerAMGSetOuterWt, par_amg.c:2611-2634 */
      const int skip = l1 ? !(w == 1.0 && omega == 1.0) : 1;
      relax_hybrid_gs(A, f, l1 ? H->l1[lvl] : NULL, w, omega, (type == 4 || type == 14) ? -1 : 1,
                      (type == 6 || type == 8) ? 2 : 1, skip, u, H->Ztmp, CF, pts);
   }
   else if (type == 18 && pts)
   {
      relax_jacobi_cf(A, f, H->l1[lvl], w, u, H->Vtmp, CF, pts);
   }
   else if (type == 18 || type == 7)
   {
      relax_l1_jacobi(A, f, H->l1[lvl], w, u, H->Vtmp, u_zero, CF, pts);
   }
   else if (type == 11 || type == 12)
   {
      relax_two_stage_gs(A, f, w, type == 11 ? 1 : 2, u, H->Vtmp, u_zero);
   }
   else
   {
      relax_l1_jacobi(A, f, H->l1[lvl], w, u, H->Vtmp, u_zero, CF, pts);
   }
}

/* hypre_BoomerAMGRelaxIF src/parcsr_ls/par_relax_interface.c:20-64: with
 * relax_order 1 a relaxation of the down (up) cycle is two, over the C then
 * the F points (F then C); the coarsest level and a single-level hierarchy
 * relax all points (par_cycle.c:441-452).  Smoothers that ignore the points
 * (two-stage Gauss-Seidel) then simply run twice; Chebyshev is not routed
 * through it (:545-556). */
static void relax_if(or_hierarchy *H, int lvl, int type, int cycle_param, const double *f, double *u, int u_zero)
{
   if (H->prm.relax_order == 1 && cycle_param < 3 && H->num_levels > 1 && type != 16)
   {
      const int p0 = cycle_param < 2 ? 1 : -1;
      relax(H, lvl, type, f, u, u_zero, p0);
      relax(H, lvl, type, f, u, 0, -p0);
   }
   else { relax(H, lvl, type, f, u, u_zero, 0); }
}

/* ------------------------------------------------------------------------ */
/* Setup driver, hypre_BoomerAMGSetup src/parcsr_ls/par_amg_setup.c:29       */
/* (non-aggressive levels: strength -> PMIS -> ext+i + truncation -> RAP)    */
/* ------------------------------------------------------------------------ */

static void csr_copy(const or_csr *A, or_csr *B)
{
   int nnz = A->i[A->nr];
   B->nr = A->nr; B->nc = A->nc;
   B->i = xmalloc(sizeof(int) * (A->nr + 1)); memcpy(B->i, A->i, sizeof(int) * (A->nr + 1));
   B->j = xmalloc(sizeof(int) * (nnz ? nnz : 1)); memcpy(B->j, A->j, sizeof(int) * nnz);
   B->v = NULL;
   if (A->v) { B->v = xmalloc(sizeof(double) * (nnz ? nnz : 1)); memcpy(B->v, A->v, sizeof(double) * nnz); }
}

int or_amg_setup(const or_csr *A0, const or_amg_params *prm, or_hierarchy *H)
{
   memset(H, 0, sizeof(*H));
   H->prm = *prm;
   prm = &H->prm;
   int maxl = prm->max_levels;
   H->A = xcalloc(maxl, sizeof(or_csr));
   H->P = xcalloc(maxl, sizeof(or_csr));
   H->S = xcalloc(maxl, sizeof(or_csr));
   H->CF = xcalloc(maxl, sizeof(int *));
   H->l1 = xcalloc(maxl, sizeof(double *));
   csr_copy(A0, &H->A[0]);
   int level = 0;
   int max_thresh = prm->max_coarse_size;
   while (1)
   {
      or_csr *A = &H->A[level];
      int n = A->nr;
      /* the size test comes after each coarsening (par_amg_setup.c:3136-3143):
       * the finest level is coarsened even when it is within max_coarse_size */
      if (level == maxl - 1) { break; }
      or_csr S;
      or_strength(A, prm->strong_threshold, prm->max_row_sum, &S);
      int *CF = xmalloc(sizeof(int) * (n ? n : 1));
      or_pmis(&S, 0, CF);
      or_csr P;
      int nc;
      if (level < prm->agg_num_levels)
      {
         /* par_amg_setup.c:1311-1358 and :1778-1915 (agg_interp_type 1, 3-9) */
         or_csr S2;
         or_strength2(&S, CF, prm->num_paths, &S2);
         int *CFN = xmalloc(sizeof(int) * (S2.nr ? S2.nr : 1));
         or_pmis(&S2, 3, CFN);
         if (prm->agg_interp_type == 4)
         {
            /* :1799-1815: CF corrected by the second coarsening, then
             * multipass interpolation on S */
            or_correct_cf(n, CF, CFN);
            or_multipass_interp(A, &S, CF, prm->agg_trunc_factor, prm->agg_p_max_elmts, &P);
         }
         else if (prm->agg_interp_type == 8 || prm->agg_interp_type == 9)
         {
            /* :1799-1824: the same correction, then the product form */
            or_correct_cf(n, CF, CFN);
            if (or_mod_multipass_interp(A, &S, CF, prm->agg_interp_type, prm->agg_trunc_factor,
                                        prm->agg_p_max_elmts, &P))
            {
               or_csr_free(&S2); free(CFN); or_csr_free(&S); free(CF);
               return -1;
            }
         }
         else
         {
            /* :1778-1915: P1 over the first coarsening, the CF correction,
             * P2 over the old C points, P = P1 P2 */
            or_csr P1, P2;
            const int t = prm->agg_interp_type;
            if (t == 1) { or_extpi_interp(A, &S, CF, &P1); }
            else if (t == 3) { or_ext_interp(A, &S, CF, &P1); }
            else { mod_interp(A, &S, CF, t == 5 ? 16 : t == 7 ? 18 : 17, &P1); }
            or_truncate(&P1, prm->agg_p12_trunc_factor, prm->agg_p12_max_elmts);
            or_correct_cf2(n, CF, CFN);
            if (t == 1 || t == 6) { or_partial_extpi_interp(A, &S, CF, &P2); }
            else if (t == 3) { or_partial_ext_interp(A, &S, CF, &P2); }
            else { or_mod_partial_interp(A, &S, CF, t, &P2); }
            or_truncate(&P2, prm->agg_p12_trunc_factor, prm->agg_p12_max_elmts);
            or_matmul(&P1, &P2, &P);
            or_truncate(&P, prm->agg_trunc_factor, prm->agg_p_max_elmts);
            or_csr_free(&P1); or_csr_free(&P2);
         }
         nc = P.nc;
         or_csr_free(&S2); free(CFN);
      }
      else
      {
         nc = or_coarse_count(n, CF);
         if (nc == 0 || nc == n || nc < prm->min_coarse_size)
         {
            or_csr_free(&S); free(CF);
            break;
         }
         if (prm->interp_type == 6) { or_extpi_interp(A, &S, CF, &P); }
         else if (prm->interp_type == 3 || prm->interp_type == 15) { or_dir_interp(A, &S, CF, &P); }   /* par_interp.c:2580-2610 */
         else if (prm->interp_type == 14) { or_ext_interp(A, &S, CF, &P); }
         else { mod_interp(A, &S, CF, prm->interp_type, &P); }   /* 16, 17, 18 */
         or_truncate(&P, prm->trunc_factor, prm->p_max_elmts);
      }
      or_csr Ac;
      or_rap(&P, A, &Ac);
      H->S[level] = S;
      H->CF[level] = CF;
      H->P[level] = P;
      level++;
      H->A[level] = Ac;
      if (nc <= max_thresh) { break; }
   }
   H->num_levels = level + 1;
   int nl = H->num_levels;
   /* par_amg_setup.c:3162-3178: Gaussian elimination only when the coarsest
    * level is within max_coarse_size (coarsening can stop above it); else
    * the coarsest level relaxes with the down-cycle type */
   {
      const int t = H->prm.relax_coarse;
      if ((t == 9 || t == 19 || t == 98 || t == 99 || t == 198 || t == 199) && H->A[nl - 1].nr > max_thresh)
      {
         H->prm.relax_coarse = H->prm.relax_down;
      }
   }
   H->F = xcalloc(nl, sizeof(double *));
   H->U = xcalloc(nl, sizeof(double *));
   for (int l = 0; l < nl; l++)
   {
      int n = H->A[l].nr;
      H->F[l] = xcalloc(n, sizeof(double));
      H->U[l] = xcalloc(n, sizeof(double));
      /* the l1 option of a level (par_amg_setup.c:3298-3496): its relax
       * types (down and up, or the coarsest's) choose, later rules
       * overriding earlier ones: 8/13/14 -> 4, 18 -> 1, 7/11/12 -> 5 */
      const int last = l == nl - 1;
      const int ta = last ? prm->relax_coarse : prm->relax_down, tb = last ? prm->relax_coarse : prm->relax_up;
      int opt = 5;
      if (ta == 8 || ta == 13 || ta == 14 || tb == 8 || tb == 13 || tb == 14) { opt = 4; }
      if (ta == 18 || tb == 18) { opt = 1; }
      const int t1 = prm->relax_down, t2 = prm->relax_up, t3 = prm->relax_coarse;
      if (t1 == 7 || t2 == 7 || (t3 == 7 && last) || t1 == 11 || t2 == 11 || (t3 == 11 && last) ||
          t1 == 12 || t2 == 12 || (t3 == 12 && last)) { opt = 5; }
      H->l1[l] = xmalloc(sizeof(double) * (n ? n : 1));
      or_l1_norms_cf(&H->A[l], opt, (opt == 1 && !last && prm->relax_order) ? H->CF[l] : NULL, H->l1[l]);
   }
   H->Vtmp = xcalloc(H->A[0].nr, sizeof(double));
   H->Ztmp = xcalloc(H->A[0].nr, sizeof(double));
   /* Chebyshev data per level (par_amg_setup.c:3496-3536) */
   H->cheby_coefs = xcalloc(nl, sizeof(double *));
   H->cheby_ds = xcalloc(nl, sizeof(double *));
   H->cheby_eig = xcalloc(2 * nl, sizeof(double));
   for (int l = 0; l < nl; l++)
   {
      if (prm->relax_down == 16 || prm->relax_up == 16 || (prm->relax_coarse == 16 && l == nl - 1))
      {
         double mx = 0.0, mn = 0.0;
         if (prm->cheby_eig_est > 0) { or_max_eig_cg(&H->A[l], prm->cheby_scale, prm->cheby_eig_est, &mx, &mn); }
         H->cheby_eig[2 * l] = mx;
         H->cheby_eig[2 * l + 1] = mn;
         H->cheby_coefs[l] = xcalloc(5, sizeof(double));
         H->cheby_ds[l] = xmalloc(sizeof(double) * (H->A[l].nr ? H->A[l].nr : 1));
         or_cheby_setup(&H->A[l], mx, mn, prm->cheby_fraction, prm->cheby_order, prm->cheby_scale,
                        prm->cheby_variant, H->cheby_coefs[l], H->cheby_ds[l]);
      }
   }
   /* coarse dense matrix (hypre_GaussElimSetup par_gauss_elim.c:33) */
   if (prm->relax_coarse == 9 || prm->relax_coarse == 99 || prm->relax_coarse == 19 || prm->relax_coarse == 98)
   {
      or_csr *Ac = &H->A[nl - 1];
      int nn = Ac->nr;
      H->coarse_n = nn;
      H->coarse_lu = xcalloc((size_t) nn * nn, sizeof(double));
      for (int r = 0; r < nn; r++)
         for (int k = Ac->i[r]; k < Ac->i[r + 1]; k++) { H->coarse_lu[(size_t) r * nn + Ac->j[k]] = Ac->v[k]; }
   }
   return 0;
}

void or_amg_free(or_hierarchy *H)
{
   for (int l = 0; l < H->num_levels; l++)
   {
      or_csr_free(&H->A[l]);
      if (l < H->num_levels - 1) { or_csr_free(&H->P[l]); or_csr_free(&H->S[l]); free(H->CF[l]); }
      free(H->l1[l]); free(H->F[l]); free(H->U[l]);
   }
   if (H->cheby_coefs)
   {
      for (int l = 0; l < H->num_levels; l++) { free(H->cheby_coefs[l]); free(H->cheby_ds[l]); }
   }
   free(H->cheby_coefs); free(H->cheby_ds); free(H->cheby_eig);
   free(H->A); free(H->P); free(H->S); free(H->CF); free(H->l1); free(H->F); free(H->U);
   free(H->Vtmp); free(H->Ztmp); free(H->coarse_lu);
   memset(H, 0, sizeof(*H));
}

/* ------------------------------------------------------------------------ */
/* One cycle, hypre_BoomerAMGCycle src/parcsr_ls/par_cycle.c:23-889: the     */
/* reference's level counters choose the next level (V, W and F cycles)      */
/* ------------------------------------------------------------------------ */

int or_amg_vcycle(or_hierarchy *H, const double *f, double *u)
{
   const int nl = H->num_levels;
   const int n0 = H->A[0].nr;
   const int ct = H->prm.cycle_type, fcycle = H->prm.fcycle;
   memcpy(H->F[0], f, sizeof(double) * n0);
   memcpy(H->U[0], u, sizeof(double) * n0);
   int *counter = xcalloc(nl, sizeof(int)), *zero = xcalloc(nl, sizeof(int));
   zero[0] = 1;
   for (int i = 0; i < n0; i++) { if (u[i] != 0.0) { zero[0] = 0; break; } }
   /* :227-238 */
   counter[0] = 1;
   for (int k = 1; k < nl; k++) { counter[k] = fcycle ? 1 : ct; }
   int fcycle_lev = nl - 2, level = 0, cycle_param = nl == 1 ? 3 : 1;
   for (;;)
   {
      /* relaxation (:430-660): the coarsest level's direct solve, or
       * num_sweeps relaxations of the cycle part's type */
      if (level == nl - 1)
      {
         const int nn = H->A[level].nr;
         if (H->coarse_lu)
         {
            double *work = xmalloc(sizeof(double) * (size_t) nn * nn);
            memcpy(work, H->coarse_lu, sizeof(double) * (size_t) nn * nn);
            memcpy(H->U[level], H->F[level], sizeof(double) * nn);
            gselim(work, H->U[level], nn);
            free(work);
         }
         else { relax(H, level, H->prm.relax_coarse, H->F[level], H->U[level], nl > 1 || zero[level], 0); }
      }
      else
      {
         const int type = cycle_param == 1 ? H->prm.relax_down : H->prm.relax_up;
         for (int s = 0; s < H->prm.num_sweeps; s++)
         {
            relax_if(H, level, type, cycle_param, H->F[level], H->U[level], zero[level] && s == 0);
            zero[level] = 0;
         }
      }
      zero[level] = 0;
      --counter[level];
      if (counter[level] >= 0 && level != nl - 1)
      {
         /* down (:730-807): residual, restriction, zero coarse guess */
         or_matvec(-1.0, &H->A[level], H->U[level], 1.0, H->F[level], H->Vtmp);
         matvecT(&H->P[level], H->Vtmp, H->F[level + 1]);
         memset(H->U[level + 1], 0, sizeof(double) * H->A[level + 1].nr);
         zero[level + 1] = 1;
         ++level;
         counter[level] = counter[level] > ct ? counter[level] : ct;
         cycle_param = level == nl - 1 ? 3 : 1;
      }
      else if (level != 0)
      {
         /* up (:808-860): u_f += P u_c */
         or_matvec(1.0, &H->P[level - 1], H->U[level], 1.0, H->U[level - 1], H->U[level - 1]);
         --level;
         cycle_param = 2;
         if (fcycle && fcycle_lev == level)
         {
            counter[level] = counter[level] > 1 ? counter[level] : 1;
            fcycle_lev--;
         }
      }
      else { break; }
   }
   memcpy(u, H->U[0], sizeof(double) * n0);
   free(counter); free(zero);
   return 0;
}

/* ------------------------------------------------------------------------ */
/* PCG, hypre_PCGSolve src/krylov/pcg.c:313-1015 (two_norm = 1,             */
/* recompute_residual 0, as the reference's ij driver configures it; the     */
/* relative-change test when the hierarchy's pcg_rel_change is set)          */
/* ------------------------------------------------------------------------ */

int or_pcg(const or_csr *A, or_hierarchy *H, const double *b, double *x,
           double tol, int maxit, double *relres, int *iters)
{
   int n = A->nr;
   double *r = xmalloc(sizeof(double) * n), *p = xcalloc(n, sizeof(double));
   double *s = xcalloc(n, sizeof(double));
   double bi_prod = or_dot(n, b, b);
   int i = 0;
   if (bi_prod == 0.0)
   {
      memcpy(x, b, sizeof(double) * n);
      if (relres) { relres[0] = 0.0; }
      *iters = 0;
      free(r); free(p); free(s);
      return 0;
   }
   double eps = tol * tol;
   or_matvec(-1.0, A, x, 1.0, b, r);
   memset(p, 0, sizeof(double) * n);
   or_amg_vcycle(H, r, p);
   double gamma = or_dot(n, r, p);
   double i_prod = or_dot(n, r, r);
   if (relres) { relres[0] = sqrt(i_prod / bi_prod); }
   int conv = 0;
   while (i + 1 <= maxit)
   {
      i++;
      or_matvec(1.0, A, p, 0.0, NULL, s);
      double sdotp = or_dot(n, s, p);
      if (sdotp == 0.0) { break; }
      double alpha = gamma / sdotp;
      if (alpha <= 0.0) { break; }
      double gamma_old = gamma;
      for (int k = 0; k < n; k++) { x[k] += alpha * p[k]; }
      for (int k = 0; k < n; k++) { r[k] += -alpha * s[k]; }
      memset(s, 0, sizeof(double) * n);
      or_amg_vcycle(H, r, s);
      gamma = or_dot(n, r, s);
      i_prod = or_dot(n, r, r);
      if (relres) { relres[i] = sqrt(i_prod / bi_prod); }
      if (i_prod / bi_prod < eps)
      {
         int tentative = 1;
         if (H->prm.pcg_rel_change && i_prod > 0.0)
         {
            /* :836-843: x must also have changed little, alpha^2 <p,p> / <x,x> < eps */
            const double pi_prod = or_dot(n, p, p), xi_prod = or_dot(n, x, x);
            if (alpha * alpha * pi_prod / xi_prod >= eps) { tentative = 0; }
         }
         if (tentative) { conv = 1; break; }
      }
      double beta = gamma / gamma_old;
      for (int k = 0; k < n; k++) { p[k] = s[k] + beta * p[k]; }
   }
   *iters = i;
   free(r); free(p); free(s);
   return conv ? 0 : 256;
}

/* ------------------------------------------------------------------------ */
/* Flexible GMRES, hypre_FlexGMRESSolve src/krylov/flexgmres.c:288            */
/* ------------------------------------------------------------------------ */

int or_fgmres(const or_csr *A, or_hierarchy *H, const double *b, double *x,
              double tol, int maxit, int kdim, double *resnorms, int *iters)
{
   /* hypre_FlexGMRESSolve, src/krylov/flexgmres.c:288-800 (a_tol 0, no
    * rel_change, min_iter 0): right preconditioning, modified Gram-Schmidt,
    * Givens rotations, restart residual rebuilt from the Krylov basis */
   int n = A->nr;
   double **p = xmalloc(sizeof(double *) * (kdim + 1));
   double **pre = xmalloc(sizeof(double *) * (kdim + 1));
   for (int k = 0; k <= kdim; k++) { p[k] = xcalloc(n, sizeof(double)); pre[k] = xcalloc(n, sizeof(double)); }
   double *r = xcalloc(n, sizeof(double)), *w = xcalloc(n, sizeof(double));
   double *hh = xcalloc((size_t) (kdim + 1) * kdim, sizeof(double));
   double *c = xcalloc(kdim, sizeof(double)), *s = xcalloc(kdim, sizeof(double));
   double *rs = xcalloc(kdim + 1, sizeof(double));
#define HH(i, j) hh[(size_t) (i) * kdim + (j)]
   or_matvec(-1.0, A, x, 1.0, b, p[0]);
   double b_norm = sqrt(or_dot(n, b, b));
   double r_norm = sqrt(or_dot(n, p[0], p[0]));
   if (resnorms) { resnorms[0] = r_norm; }
   double den = b_norm > 0.0 ? b_norm : r_norm;
   double epsilon = tol * den;
   int iter = 0, conv = 0, i = 0;
   while (iter < maxit)
   {
      rs[0] = r_norm;
      if (r_norm == 0.0) { conv = 1; break; }
      if (r_norm <= epsilon)
      {
         or_matvec(-1.0, A, x, 1.0, b, r);
         r_norm = sqrt(or_dot(n, r, r));
         if (r_norm <= epsilon) { conv = 1; break; }
      }
      double t = 1.0 / r_norm;
      for (int k = 0; k < n; k++) { p[0][k] *= t; }
      i = 0;
      while (i < kdim && iter < maxit)
      {
         i++;
         iter++;
         memset(pre[i - 1], 0, sizeof(double) * n);
         or_amg_vcycle(H, p[i - 1], pre[i - 1]);
         or_matvec(1.0, A, pre[i - 1], 0.0, NULL, p[i]);
         for (int j = 0; j < i; j++)
         {
            HH(j, i - 1) = or_dot(n, p[j], p[i]);
            double h = -HH(j, i - 1);
            for (int k = 0; k < n; k++) { p[i][k] += h * p[j][k]; }
         }
         t = sqrt(or_dot(n, p[i], p[i]));
         HH(i, i - 1) = t;
         if (t != 0.0) { t = 1.0 / t; for (int k = 0; k < n; k++) { p[i][k] *= t; } }
         for (int j = 1; j < i; j++)
         {
            t = HH(j - 1, i - 1);
            HH(j - 1, i - 1) = s[j - 1] * HH(j, i - 1) + c[j - 1] * t;
            HH(j, i - 1) = -s[j - 1] * t + c[j - 1] * HH(j, i - 1);
         }
         t = HH(i, i - 1) * HH(i, i - 1);
         t += HH(i - 1, i - 1) * HH(i - 1, i - 1);
         double gamma = sqrt(t);
         if (gamma == 0.0) { gamma = 1.0e-16; }
         c[i - 1] = HH(i - 1, i - 1) / gamma;
         s[i - 1] = HH(i, i - 1) / gamma;
         rs[i] = -HH(i, i - 1) * rs[i - 1];
         rs[i] /= gamma;
         rs[i - 1] = c[i - 1] * rs[i - 1];
         HH(i - 1, i - 1) = s[i - 1] * HH(i, i - 1) + c[i - 1] * HH(i - 1, i - 1);
         r_norm = fabs(rs[i]);
         if (resnorms) { resnorms[iter] = r_norm; }
         if (r_norm <= epsilon) { break; }
      }
      rs[i - 1] = rs[i - 1] / HH(i - 1, i - 1);
      for (int k = i - 2; k >= 0; k--)
      {
         t = 0.0;
         for (int j = k + 1; j < i; j++) { t -= HH(k, j) * rs[j]; }
         t += rs[k];
         rs[k] = t / HH(k, k);
      }
      for (int k = 0; k < n; k++) { w[k] = pre[i - 1][k] * rs[i - 1]; }
      for (int j = i - 2; j >= 0; j--) { for (int k = 0; k < n; k++) { w[k] += rs[j] * pre[j][k]; } }
      for (int k = 0; k < n; k++) { x[k] += w[k]; }
      if (r_norm <= epsilon)
      {
         or_matvec(-1.0, A, x, 1.0, b, r);
         r_norm = sqrt(or_dot(n, r, r));
         if (r_norm <= epsilon) { conv = 1; break; }
         memcpy(p[0], r, sizeof(double) * n);
         i = 0;
      }
      for (int j = i; j > 0; j--)
      {
         rs[j - 1] = -s[j - 1] * rs[j];
         rs[j] = c[j - 1] * rs[j];
      }
      if (i) { double a1 = rs[i] - 1.0; for (int k = 0; k < n; k++) { p[i][k] += a1 * p[i][k]; } }
      for (int j = i - 1; j > 0; j--) { for (int k = 0; k < n; k++) { p[i][k] += rs[j] * p[j][k]; } }
      if (i)
      {
         double a0 = rs[0] - 1.0;
         for (int k = 0; k < n; k++) { p[0][k] += a0 * p[0][k]; }
         for (int k = 0; k < n; k++) { p[0][k] += p[i][k]; }
      }
   }
#undef HH
   *iters = iter;
   for (int k = 0; k <= kdim; k++) { free(p[k]); free(pre[k]); }
   free(p); free(pre); free(r); free(w); free(hh); free(c); free(s); free(rs);
   return conv ? 0 : 256;
}

/* ------------------------------------------------------------------------ */
/* Flat accessors for the ctypes wrapper (oracle/oracle.py)                  */
/* ------------------------------------------------------------------------ */

or_hierarchy *or_h_new(void) { return xcalloc(1, sizeof(or_hierarchy)); }
void or_h_delete(or_hierarchy *H) { if (H) { or_amg_free(H); free(H); } }
int or_h_num_levels(const or_hierarchy *H) { return H->num_levels; }

/* which: 0 = A, 1 = P, 2 = S */
int or_h_csr(const or_hierarchy *H, int which, int l, int *nr, int *nc, int **i, int **j, double **v)
{
   const or_csr *M = which == 0 ? &H->A[l] : which == 1 ? &H->P[l] : &H->S[l];
   *nr = M->nr; *nc = M->nc; *i = M->i; *j = M->j; *v = M->v;
   return M->i ? M->i[M->nr] : 0;
}
int *or_h_cf(const or_hierarchy *H, int l) { return H->CF[l]; }
double *or_h_l1(const or_hierarchy *H, int l) { return H->l1[l]; }
double *or_h_cheby_coefs(const or_hierarchy *H, int l) { return H->cheby_coefs ? H->cheby_coefs[l] : NULL; }
double *or_h_cheby_ds(const or_hierarchy *H, int l) { return H->cheby_ds ? H->cheby_ds[l] : NULL; }
double *or_h_cheby_eig(const or_hierarchy *H) { return H->cheby_eig; }

int or_setup_flat(int n, const int *Ai, const int *Aj, const double *Av, const or_amg_params *prm, or_hierarchy *H)
{
   or_csr A = { n, n, (int *) Ai, (int *) Aj, (double *) Av };
   return or_amg_setup(&A, prm, H);
}
int or_pcg_flat(int n, const int *Ai, const int *Aj, const double *Av, or_hierarchy *H, const double *b, double *x,
                double tol, int maxit, double *relres, int *iters)
{
   or_csr A = { n, n, (int *) Ai, (int *) Aj, (double *) Av };
   return or_pcg(&A, H, b, x, tol, maxit, relres, iters);
}
int or_fgmres_flat(int n, const int *Ai, const int *Aj, const double *Av, or_hierarchy *H, const double *b, double *x,
                   double tol, int maxit, int kdim, double *resn, int *iters)
{
   or_csr A = { n, n, (int *) Ai, (int *) Aj, (double *) Av };
   return or_fgmres(&A, H, b, x, tol, maxit, kdim, resn, iters);
}
int or_vcycle_flat(or_hierarchy *H, const double *f, double *u) { return or_amg_vcycle(H, f, u); }

/* BoomerAMG as the solver, hypre_BoomerAMGSolve src/parcsr_ls/par_amg_solve.c:
 * 150-351 (one process, print level and logging 0, convergence type 0): the
 * relative residual ||b - A x|| / ||b|| (the absolute one when b = 0) before
 * the loop; V-cycles on (b, x) in place while it is >= tol (1 when tol = 0)
 * and fewer than maxit cycles ran, the residual after each.  relres[k]: after
 * k cycles (relres[0] the initial one). */
int or_amg_solve_flat(int n, const int *Ai, const int *Aj, const double *Av, or_hierarchy *H, const double *b,
                      double *x, double tol, int maxit, double *relres, int *iters)
{
   or_csr A = { n, n, (int *) Ai, (int *) Aj, (double *) Av };
   double *r = xmalloc(sizeof(double) * (n ? n : 1));
   double rel = 1.0, rhs = 0.0;
   if (tol > 0.0)
   {
      or_matvec(-1.0, &A, x, 1.0, b, r);
      double res = sqrt(or_dot(n, r, r));
      rhs = sqrt(or_dot(n, b, b));
      rel = rhs != 0.0 ? res / rhs : res;
   }
   if (relres) { relres[0] = rel; }
   int it = 0;
   while (rel >= tol && it < maxit)
   {
      or_amg_vcycle(H, b, x);
      if (tol > 0.0)
      {
         or_matvec(-1.0, &A, x, 1.0, b, r);
         double res = sqrt(or_dot(n, r, r));
         rel = rhs != 0.0 ? res / rhs : res;
      }
      it++;
      if (relres) { relres[it] = rel; }
   }
   free(r);
   *iters = it;
   return 0;
}
void or_free_ptr(void *p) { free(p); }

/* C = A*B as HYPRE_ParCSRMatrixMatmat computes it on one process
 * (src/parcsr_mv/HYPRE_parcsr_matrix.c:457 -> par_csr_triplemat.c:20 ->
 * hypre_CSRMatrixMultiplyHost, src/seq_mv/csr_matop.c:693-933): an empty A or
 * B gives an empty C (:745-752); a square product reserves each row's
 * diagonal first (stored as 0, then summed into, :900-909) unless A has a
 * row-nonzero list, which IJ assembly sets when some but not all rows of A
 * are empty (src/IJ_mv/IJMatrix_parcsr.c:3053, src/seq_mv/csr_matrix.c:354-400);
 * then each non-empty row takes columns in first-discovery order only.
 * Returns nnz(C); *Ci (nra+1), *Cj, *Cv are malloc'd (or_free_ptr). */
int or_matmat_flat(int nra, int nca, int ncb, const int *Ai, const int *Aj, const double *Av,
                   const int *Bi, const int *Bj, const double *Bv, int **Ci, int **Cj, double **Cv)
{
   or_csr A = { nra, nca, (int *) Ai, (int *) Aj, (double *) Av };
   or_csr B = { nca, ncb, (int *) Bi, (int *) Bj, (double *) Bv };
   or_csr C;
   int empty_rows = 0;
   for (int i = 0; i < nra; i++) { empty_rows += Ai[i + 1] == Ai[i]; }
   if (Ai[nra] == 0 || Bi[nca] == 0)
   {
      *Ci = xcalloc(nra + 1, sizeof(int));
      *Cj = xmalloc(sizeof(int));
      *Cv = xmalloc(sizeof(double));
      return 0;
   }
   matmul_ex(&A, &B, &C, nra == ncb && empty_rows == 0);
   *Ci = C.i; *Cj = C.j; *Cv = C.v;
   return C.i[nra];
}
int or_gen_stencil_flat(int kind, int nx, int ny, int nz, int **i, int **j, double **v)
{
   or_csr A;
   or_gen_stencil(kind, nx, ny, nz, &A);
   *i = A.i; *j = A.j; *v = A.v;
   return A.i[A.nr];
}
