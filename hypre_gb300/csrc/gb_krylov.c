/* Krylov drivers (host C over fused device vector kernels): preconditioned
 * CG and flexible GMRES, plus the diagonal-scaling preconditioner.
 * Reference: hypre_PCGSolve src/krylov/pcg.c:313-1015 (defaults :97-127),
 * hypre_FlexGMRESSolve src/krylov/flexgmres.c:288-800, ParCSR front ends
 * src/parcsr_ls/HYPRE_parcsr_pcg.c, HYPRE_parcsr_flexgmres.c,
 * HYPRE_ParCSRDiagScale src/parcsr_ls/HYPRE_parcsr_pcg.c. */
#include "gb_internal.h"

#include <math.h>

int gb_amg_precond(HYPRE_Solver solver, const double *b, double *x);

static gb_krylov *kry_of(HYPRE_Solver s, int arg)
{
   gb_krylov *k = (gb_krylov *) s;
   if (!k || (k->magic != GB_MAGIC_PCG && k->magic != GB_MAGIC_GMR)) { gb_error_in_arg(arg); return NULL; }
   return k;
}

static void kry_free_work(gb_krylov *k)
{
   gb_krylov_multi_free(k);
   gb_dfree(k->r); gb_dfree(k->p); gb_dfree(k->s); gb_dfree(k->w);
   k->r = k->p = k->s = k->w = NULL;
   for (int i = 0; i < k->nV; i++) { gb_dfree(k->V[i]); gb_dfree(k->Z[i]); }
   free(k->V); free(k->Z);
   k->V = k->Z = NULL;
   gb_dfree(k->hdev);
   gb_hfree_pinned(k->hhost);
   k->hdev = k->hhost = NULL;
   k->nV = 0;
   k->n = 0;
}

static void hist_push(gb_krylov *k, int i, double v)
{
   if (i >= k->hist_cap)
   {
      int nc = (i + 1) * 2;
      k->hist = (double *) realloc(k->hist, sizeof(double) * (size_t) nc);
      k->hist_cap = nc;
   }
   k->hist[i] = v;
   if (i + 1 > k->hist_n) { k->hist_n = i + 1; }
}

/* preconditioner application: x = C b (x is cleared first, as the reference
 * does with ClearVector before calling precond) */
static void apply_precond(gb_krylov *k, gb_parcsr *A, gb_parvec *bv, gb_parvec *xv)
{
   if (!k->precond)
   {
      cudaMemcpyAsync(xv->d, bv->d, sizeof(double) * (size_t) bv->n, cudaMemcpyDeviceToDevice, gb_stream());
      return;
   }
   if ((void *) k->precond == (void *) HYPRE_BoomerAMGSolve)
   {
      /* fast path: one graph-captured V-cycle from a zero guess */
      gb_amg_precond(k->precond_solver, bv->d, xv->d);
      return;
   }
   gb_fill_d(xv->n, xv->d, 0.0, gb_stream());
   k->precond(k->precond_solver, (HYPRE_Matrix) A, (HYPRE_Vector) bv, (HYPRE_Vector) xv);
}

static gb_parvec wrap_vec(double *d, int n)
{
   gb_parvec v;
   v.magic = GB_MAGIC_VEC;
   v.n = n;
   v.num_vectors = 1;
   v.d = d;
   v.owns = 0;
   return v;
}

static void ensure_work(gb_krylov *k, int n, int nbasis)
{
   if (k->n == n && k->nV >= nbasis && k->r) { return; }
   kry_free_work(k);
   size_t nb = sizeof(double) * (size_t) (n > 0 ? n : 1);
   k->r = (double *) gb_dcalloc(nb); k->p = (double *) gb_dcalloc(nb);
   k->s = (double *) gb_dcalloc(nb); k->w = (double *) gb_dcalloc(nb);
   if (nbasis > 0)
   {
      k->V = (double **) calloc((size_t) nbasis, sizeof(double *));
      k->Z = (double **) calloc((size_t) nbasis, sizeof(double *));
      for (int i = 0; i < nbasis; i++) { k->V[i] = (double *) gb_dcalloc(nb); k->Z[i] = (double *) gb_dcalloc(nb); }
      k->nV = nbasis;
      k->hdev = (double *) gb_dcalloc(sizeof(double) * (size_t) (nbasis + 1));
      k->hhost = (double *) gb_hmalloc_pinned(sizeof(double) * (size_t) (nbasis + 1));
   }
   k->n = n;
}

/* --------------------------------------------------------------------------
 * PCG
 * ------------------------------------------------------------------------ */
static int pcg_solve(gb_krylov *k, gb_parcsr *A, gb_parvec *b, gb_parvec *x)
{
   int n = A->A.nr;
   cudaStream_t st = gb_stream();
   ensure_work(k, n, 0);
   gb_parvec rv = wrap_vec(k->r, n), pv = wrap_vec(k->p, n), sv = wrap_vec(k->s, n);
   const gb_spmv_desc *Ad = gb_solve_desc(A, GB_PREC_F64);
   double *part = gb_red_part(), *out = gb_red_out(), *h = gb_red_host();
   k->hist_n = 0;
   double bi_prod;
   if (k->two_norm) { bi_prod = gb_dot(n, b->d, b->d); }
   else
   {
      apply_precond(k, A, b, &pv);
      bi_prod = gb_dot(n, k->p, b->d);
   }
   if (bi_prod != bi_prod) { gb_error(HYPRE_ERROR_GENERIC, "NaN or Inf in right-hand side"); return gb_error_flag; }
   double eps = k->tol * k->tol;
   if (bi_prod > 0.0) { double e2 = k->a_tol * k->a_tol / bi_prod; eps = eps > e2 ? eps : e2; }
   else
   {
      cudaMemcpyAsync(x->d, b->d, sizeof(double) * (size_t) n, cudaMemcpyDeviceToDevice, st);
      k->num_iterations = 0;
      k->rel_resid = 0.0;
      hist_push(k, 0, 0.0);
      return gb_error_flag;
   }
   /* r = b - A x */
   gb_spmv_d(Ad, x->d, k->r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, st);
   apply_precond(k, A, &rv, &pv);
   /* gamma = <r,p>, i_prod = <r,r> */
   gb_dot2_d(n, k->r, k->p, k->r, part, out, st);
   cudaMemcpyAsync(h, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
   gb_sync();
   double gamma = h[0];
   double i_prod = k->two_norm ? h[1] : gamma;
   if (gamma != gamma) { gb_error(HYPRE_ERROR_GENERIC, "NaN or Inf in preconditioned residual"); return gb_error_flag; }
   hist_push(k, 0, sqrt(i_prod / bi_prod));
   int i = 0, converged = 0;
   while (i + 1 <= k->max_iter)
   {
      i++;
      /* s = A p and <s,p> in one pass */
      gb_spmv_d(Ad, k->p, k->s, 0, 1.0, 0.0, NULL, NULL, 0.0, k->p, part, st);
      gb_final_sum(GB_RED_BLOCKS, 1, part, out, st);
      cudaMemcpyAsync(h, out, sizeof(double), cudaMemcpyDeviceToHost, st);
      gb_sync();
      double sdotp = h[0];
      if (sdotp == 0.0)
      {
         gb_error(HYPRE_ERROR_CONV, "zero sdotp in PCG");
         break;
      }
      double alpha = gamma / sdotp;
      if (alpha <= 0.0)
      {
         gb_error(HYPRE_ERROR_CONV, "negative or zero alpha in PCG");
         break;
      }
      double gamma_old = gamma;
      /* x += alpha p ; r -= alpha s */
      gb_pcg_xr_d(n, alpha, k->p, k->s, x->d, k->r, part, out, st);
      /* s = C r */
      apply_precond(k, A, &rv, &sv);
      gb_dot2_d(n, k->r, k->s, k->r, part, out, st);
      cudaMemcpyAsync(h, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
      gb_sync();
      gamma = h[0];
      i_prod = k->two_norm ? h[1] : gamma;
      hist_push(k, i, sqrt(i_prod / bi_prod));
      /* the convergence tests of pcg.c:808-849: the basic test, then (on
       * request) the recomputed residual and the relative change of x,
       * alpha^2 <p,p> / <x,x> < eps */
      if (i_prod / bi_prod < eps)
      {
         int tentative = 1;
         if (k->recompute_residual)
         {
            gb_spmv_d(Ad, x->d, k->r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, st);
            if (k->two_norm) { i_prod = gb_dot(n, k->r, k->r); }
            else
            {
               apply_precond(k, A, &rv, &sv);
               i_prod = gb_dot(n, k->r, k->s);
               gamma = i_prod;
            }
            if (i_prod / bi_prod >= eps) { tentative = 0; }
         }
         if (tentative && k->rel_change && i_prod > 0.0)
         {
            const double pi_prod = gb_dot(n, k->p, k->p), xi_prod = gb_dot(n, x->d, x->d);
            if (alpha * alpha * pi_prod / xi_prod >= eps) { tentative = 0; }
         }
         if (tentative) { converged = 1; break; }
      }
      /* p = s + beta p */
      double beta = gamma / gamma_old;
      gb_xpay_d(n, k->s, beta, k->p, st);
   }
   gb_sync();
   k->num_iterations = i;
   k->rel_resid = sqrt(i_prod / bi_prod);
   if (!converged && k->tol > 0.0) { gb_error(HYPRE_ERROR_CONV, NULL); }
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * FlexGMRES (right preconditioning, modified Gram-Schmidt, Givens)
 * ------------------------------------------------------------------------ */
static int fgmres_solve(gb_krylov *k, gb_parcsr *A, gb_parvec *b, gb_parvec *x)
{
   int n = A->A.nr;
   int kd = k->k_dim;
   cudaStream_t st = gb_stream();
   ensure_work(k, n, kd + 1);
   const gb_spmv_desc *Ad = gb_solve_desc(A, GB_PREC_F64);
   double **p = k->V, **pre = k->Z;
   k->hist_n = 0;
   double *hh = (double *) calloc((size_t) (kd + 1) * kd, sizeof(double));
   double *c = (double *) calloc((size_t) kd, sizeof(double)), *s = (double *) calloc((size_t) kd, sizeof(double));
   double *rs = (double *) calloc((size_t) kd + 1, sizeof(double));
#define HH(i, j) hh[(size_t) (i) * kd + (j)]
   gb_spmv_d(Ad, x->d, p[0], 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, st);
   double b_norm = sqrt(gb_dot(n, b->d, b->d));
   if (b_norm != b_norm) { gb_error(HYPRE_ERROR_GENERIC, "NaN or Inf in right-hand side"); free(hh); free(c); free(s); free(rs); return gb_error_flag; }
   double r_norm = sqrt(gb_dot(n, p[0], p[0]));
   hist_push(k, 0, b_norm > 0 ? r_norm / b_norm : r_norm);
   double den = b_norm > 0.0 ? b_norm : r_norm;
   double epsilon = k->a_tol > k->tol * den ? k->a_tol : k->tol * den;
   int iter = 0, converged = 0, i = 0;
   while (iter < k->max_iter)
   {
      rs[0] = r_norm;
      if (r_norm == 0.0) { converged = 1; break; }
      if (r_norm <= epsilon)
      {
         gb_spmv_d(Ad, x->d, k->r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, st);
         r_norm = sqrt(gb_dot(n, k->r, k->r));
         if (r_norm <= epsilon) { converged = 1; break; }
      }
      gb_scale_d(n, 1.0 / r_norm, p[0], st);
      i = 0;
      while (i < kd && iter < k->max_iter)
      {
         i++;
         iter++;
         gb_parvec pin = wrap_vec(p[i - 1], n), zout = wrap_vec(pre[i - 1], n);
         apply_precond(k, A, &pin, &zout);
         gb_spmv_d(Ad, pre[i - 1], p[i], 0, 1.0, 0.0, NULL, NULL, 0.0, NULL, NULL, st);
         /* modified Gram-Schmidt on the device: h_0 = (p_0, p_i), then each
          * update p_i -= h_j p_j (h_j read from device memory) is fused with
          * the next inner product (with p_{j+1}, or p_i's own norm at the
          * end); the column comes back to the host once */
         gb_dot_d(n, p[0], p[i], gb_red_part(), gb_red_count(), k->hdev, st);
         for (int j = 0; j < i; j++)
         {
            gb_axpy_dot_dev_d(n, k->hdev + j, p[j], p[i], j + 1 < i ? p[j + 1] : p[i], gb_red_part(),
                              gb_red_count(), k->hdev + j + 1, st);
         }
         cudaMemcpyAsync(k->hhost, k->hdev, sizeof(double) * (size_t) (i + 1), cudaMemcpyDeviceToHost, st);
         gb_sync();
         for (int j = 0; j < i; j++) { HH(j, i - 1) = k->hhost[j]; }
         double t = sqrt(k->hhost[i]);
         HH(i, i - 1) = t;
         if (t != 0.0) { gb_scale_d(n, 1.0 / t, p[i], st); }
         for (int j = 1; j < i; j++)
         {
            t = HH(j - 1, i - 1);
            HH(j - 1, i - 1) = s[j - 1] * HH(j, i - 1) + c[j - 1] * t;
            HH(j, i - 1) = -s[j - 1] * t + c[j - 1] * HH(j, i - 1);
         }
         t = HH(i, i - 1) * HH(i, i - 1);
         t += HH(i - 1, i - 1) * HH(i - 1, i - 1);
         double gamma = sqrt(t);
         if (gamma == 0.0) { gamma = 1.e-16; }
         c[i - 1] = HH(i - 1, i - 1) / gamma;
         s[i - 1] = HH(i, i - 1) / gamma;
         rs[i] = -HH(i, i - 1) * rs[i - 1];
         rs[i] /= gamma;
         rs[i - 1] = c[i - 1] * rs[i - 1];
         HH(i - 1, i - 1) = s[i - 1] * HH(i, i - 1) + c[i - 1] * HH(i - 1, i - 1);
         r_norm = fabs(rs[i]);
         hist_push(k, iter, b_norm > 0 ? r_norm / b_norm : r_norm);
         if (r_norm <= epsilon) { break; }
      }
      rs[i - 1] = rs[i - 1] / HH(i - 1, i - 1);
      for (int kk = i - 2; kk >= 0; kk--)
      {
         double t = 0.0;
         for (int j = kk + 1; j < i; j++) { t -= HH(kk, j) * rs[j]; }
         t += rs[kk];
         rs[kk] = t / HH(kk, kk);
      }
      /* w = sum rs[j] pre[j]; x += w */
      cudaMemcpyAsync(k->w, pre[i - 1], sizeof(double) * (size_t) n, cudaMemcpyDeviceToDevice, st);
      gb_scale_d(n, rs[i - 1], k->w, st);
      for (int j = i - 2; j >= 0; j--) { gb_axpy_d(n, rs[j], pre[j], k->w, st); }
      gb_axpy_d(n, 1.0, k->w, x->d, st);
      if (r_norm <= epsilon)
      {
         gb_spmv_d(Ad, x->d, k->r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, st);
         r_norm = sqrt(gb_dot(n, k->r, k->r));
         if (r_norm <= epsilon) { converged = 1; break; }
         cudaMemcpyAsync(p[0], k->r, sizeof(double) * (size_t) n, cudaMemcpyDeviceToDevice, st);
         i = 0;
      }
      /* residual vector of the restart from the Krylov basis */
      for (int j = i; j > 0; j--)
      {
         rs[j - 1] = -s[j - 1] * rs[j];
         rs[j] = c[j - 1] * rs[j];
      }
      if (i) { gb_axpy_d(n, rs[i] - 1.0, p[i], p[i], st); }
      for (int j = i - 1; j > 0; j--) { gb_axpy_d(n, rs[j], p[j], p[i], st); }
      if (i)
      {
         gb_axpy_d(n, rs[0] - 1.0, p[0], p[0], st);
         gb_axpy_d(n, 1.0, p[i], p[0], st);
      }
   }
#undef HH
   gb_sync();
   k->num_iterations = iter;
   k->rel_resid = b_norm > 0.0 ? r_norm / b_norm : r_norm;
   if (iter >= k->max_iter && r_norm > epsilon && epsilon > 0) { gb_error(HYPRE_ERROR_CONV, NULL); }
   (void) converged;
   free(hh); free(c); free(s); free(rs);
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * Public API
 * ------------------------------------------------------------------------ */
static gb_krylov *kry_new(int magic)
{
   gb_runtime_init();
   gb_krylov *k = (gb_krylov *) calloc(1, sizeof(gb_krylov));
   k->magic = magic;
   if (magic == GB_MAGIC_PCG)
   {
      /* pcg.c:97-127 */
      k->tol = 1.0e-6; k->a_tol = 0.0; k->max_iter = 1000; k->two_norm = 0; k->rel_change = 0;
   }
   else
   {
      /* flexgmres.c defaults */
      k->tol = 1.0e-6; k->a_tol = 0.0; k->max_iter = 1000; k->k_dim = 5;
   }
   return k;
}

HYPRE_Int HYPRE_ParCSRPCGCreate(MPI_Comm comm, HYPRE_Solver *solver)
{
   (void) comm;
   if (!solver) { gb_error_in_arg(2); return gb_error_flag; }
   *solver = (HYPRE_Solver) kry_new(GB_MAGIC_PCG);
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRFlexGMRESCreate(MPI_Comm comm, HYPRE_Solver *solver)
{
   (void) comm;
   if (!solver) { gb_error_in_arg(2); return gb_error_flag; }
   *solver = (HYPRE_Solver) kry_new(GB_MAGIC_GMR);
   return gb_error_flag;
}

static HYPRE_Int kry_destroy(HYPRE_Solver solver)
{
   gb_krylov *k = (gb_krylov *) solver;
   if (!k || (k->magic != GB_MAGIC_PCG && k->magic != GB_MAGIC_GMR)) { return gb_error_flag; }
   kry_free_work(k);
   free(k->hist);
   k->magic = 0;
   free(k);
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRPCGDestroy(HYPRE_Solver solver) { return kry_destroy(solver); }
HYPRE_Int HYPRE_ParCSRFlexGMRESDestroy(HYPRE_Solver solver) { return kry_destroy(solver); }

static HYPRE_Int kry_setup(HYPRE_Solver solver, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x)
{
   gb_krylov *k = kry_of(solver, 1);
   if (!k) { return gb_error_flag; }
   gb_parcsr *M = (gb_parcsr *) A;
   if (!M || M->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   ensure_work(k, M->A.nr, k->magic == GB_MAGIC_GMR ? k->k_dim + 1 : 0);
   if (k->precond_setup) { k->precond_setup(k->precond_solver, A, b, x); }
   return gb_error_flag;
}

static HYPRE_Int kry_solve(HYPRE_Solver solver, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x)
{
   gb_krylov *k = kry_of(solver, 1);
   if (!k) { return gb_error_flag; }
   gb_parcsr *M = (gb_parcsr *) A;
   gb_parvec *bv = (gb_parvec *) b, *xv = (gb_parvec *) x;
   if (!M || M->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   if (!bv || bv->magic != GB_MAGIC_VEC || bv->n != M->A.nr) { gb_error_in_arg(3); return gb_error_flag; }
   if (!xv || xv->magic != GB_MAGIC_VEC || xv->n != M->A.nr) { gb_error_in_arg(4); return gb_error_flag; }
   k->last_multi = bv->num_vectors > 1 || xv->num_vectors > 1;
   if (k->last_multi)
   {
      if (k->magic == GB_MAGIC_PCG) { return gb_pcg_multi(k, M, bv, xv); }
      gb_error(HYPRE_ERROR_GENERIC, "multi-vector right-hand sides: PCG only");
      gb_error_in_arg(3);
      return gb_error_flag;
   }
   HYPRE_Int r = k->magic == GB_MAGIC_PCG ? pcg_solve(k, M, bv, xv) : fgmres_solve(k, M, bv, xv);
   if (gb_amg_check_sweeps()) { r = gb_error_flag; }
   return r;
}

HYPRE_Int HYPRE_PCGSetup(HYPRE_Solver s, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x) { return kry_setup(s, A, b, x); }
HYPRE_Int HYPRE_PCGSolve(HYPRE_Solver s, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x) { return kry_solve(s, A, b, x); }
HYPRE_Int HYPRE_FlexGMRESSetup(HYPRE_Solver s, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x) { return kry_setup(s, A, b, x); }
HYPRE_Int HYPRE_FlexGMRESSolve(HYPRE_Solver s, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x) { return kry_solve(s, A, b, x); }
HYPRE_Int HYPRE_ParCSRPCGSetup(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{ return kry_setup(s, (HYPRE_Matrix) A, (HYPRE_Vector) b, (HYPRE_Vector) x); }
HYPRE_Int HYPRE_ParCSRPCGSolve(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{ return kry_solve(s, (HYPRE_Matrix) A, (HYPRE_Vector) b, (HYPRE_Vector) x); }
HYPRE_Int HYPRE_ParCSRFlexGMRESSetup(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{ return kry_setup(s, (HYPRE_Matrix) A, (HYPRE_Vector) b, (HYPRE_Vector) x); }
HYPRE_Int HYPRE_ParCSRFlexGMRESSolve(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{ return kry_solve(s, (HYPRE_Matrix) A, (HYPRE_Vector) b, (HYPRE_Vector) x); }

#define KSET(name, field, type)                                  \
   HYPRE_Int name(HYPRE_Solver solver, type v)                    \
   {                                                              \
      gb_krylov *k = kry_of(solver, 1);                           \
      if (k) { k->field = v; }                                    \
      return gb_error_flag;                                       \
   }
KSET(HYPRE_PCGSetTol, tol, HYPRE_Real)
KSET(HYPRE_PCGSetAbsoluteTol, a_tol, HYPRE_Real)
KSET(HYPRE_PCGSetMaxIter, max_iter, HYPRE_Int)
KSET(HYPRE_PCGSetTwoNorm, two_norm, HYPRE_Int)
KSET(HYPRE_PCGSetRelChange, rel_change, HYPRE_Int)
KSET(HYPRE_PCGSetRecomputeResidual, recompute_residual, HYPRE_Int)
KSET(HYPRE_PCGSetLogging, logging, HYPRE_Int)
KSET(HYPRE_PCGSetPrintLevel, print_level, HYPRE_Int)
KSET(HYPRE_ParCSRPCGSetTol, tol, HYPRE_Real)
KSET(HYPRE_ParCSRPCGSetMaxIter, max_iter, HYPRE_Int)
KSET(HYPRE_ParCSRPCGSetTwoNorm, two_norm, HYPRE_Int)
KSET(HYPRE_FlexGMRESSetTol, tol, HYPRE_Real)
KSET(HYPRE_FlexGMRESSetAbsoluteTol, a_tol, HYPRE_Real)
KSET(HYPRE_FlexGMRESSetMaxIter, max_iter, HYPRE_Int)
KSET(HYPRE_FlexGMRESSetLogging, logging, HYPRE_Int)
KSET(HYPRE_FlexGMRESSetPrintLevel, print_level, HYPRE_Int)
KSET(HYPRE_ParCSRFlexGMRESSetTol, tol, HYPRE_Real)
KSET(HYPRE_ParCSRFlexGMRESSetMaxIter, max_iter, HYPRE_Int)

static HYPRE_Int set_kdim(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_krylov *k = kry_of(solver, 1);
   if (!k) { return gb_error_flag; }
   if (v < 1) { gb_error_in_arg(2); return gb_error_flag; }
   k->k_dim = v;
   return gb_error_flag;
}
HYPRE_Int HYPRE_FlexGMRESSetKDim(HYPRE_Solver s, HYPRE_Int v) { return set_kdim(s, v); }
HYPRE_Int HYPRE_ParCSRFlexGMRESSetKDim(HYPRE_Solver s, HYPRE_Int v) { return set_kdim(s, v); }

static HYPRE_Int set_precond(HYPRE_Solver solver, HYPRE_PtrToSolverFcn pc, HYPRE_PtrToSolverFcn pcs, HYPRE_Solver ps)
{
   gb_krylov *k = kry_of(solver, 1);
   if (!k) { return gb_error_flag; }
   k->precond = pc;
   k->precond_setup = pcs;
   k->precond_solver = ps;
   return gb_error_flag;
}
HYPRE_Int HYPRE_PCGSetPrecond(HYPRE_Solver s, HYPRE_PtrToSolverFcn pc, HYPRE_PtrToSolverFcn pcs, HYPRE_Solver ps)
{ return set_precond(s, pc, pcs, ps); }
HYPRE_Int HYPRE_FlexGMRESSetPrecond(HYPRE_Solver s, HYPRE_PtrToSolverFcn pc, HYPRE_PtrToSolverFcn pcs, HYPRE_Solver ps)
{ return set_precond(s, pc, pcs, ps); }
HYPRE_Int HYPRE_ParCSRPCGSetPrecond(HYPRE_Solver s, HYPRE_PtrToParSolverFcn pc, HYPRE_PtrToParSolverFcn pcs, HYPRE_Solver ps)
{ return set_precond(s, (HYPRE_PtrToSolverFcn) pc, (HYPRE_PtrToSolverFcn) pcs, ps); }
HYPRE_Int HYPRE_ParCSRFlexGMRESSetPrecond(HYPRE_Solver s, HYPRE_PtrToParSolverFcn pc, HYPRE_PtrToParSolverFcn pcs,
                                          HYPRE_Solver ps)
{ return set_precond(s, (HYPRE_PtrToSolverFcn) pc, (HYPRE_PtrToSolverFcn) pcs, ps); }

HYPRE_Int HYPRE_PCGGetPrecond(HYPRE_Solver solver, HYPRE_Solver *p)
{
   gb_krylov *k = kry_of(solver, 1);
   if (k && p) { *p = k->precond_solver; }
   return gb_error_flag;
}

static HYPRE_Int get_iters(HYPRE_Solver solver, HYPRE_Int *n)
{
   gb_krylov *k = kry_of(solver, 1);
   if (k && n) { *n = k->num_iterations; }
   return gb_error_flag;
}
static HYPRE_Int get_res(HYPRE_Solver solver, HYPRE_Real *r)
{
   gb_krylov *k = kry_of(solver, 1);
   if (k && r) { *r = k->rel_resid; }
   return gb_error_flag;
}
HYPRE_Int HYPRE_PCGGetNumIterations(HYPRE_Solver s, HYPRE_Int *n) { return get_iters(s, n); }
HYPRE_Int HYPRE_PCGGetFinalRelativeResidualNorm(HYPRE_Solver s, HYPRE_Real *r) { return get_res(s, r); }
HYPRE_Int HYPRE_ParCSRPCGGetNumIterations(HYPRE_Solver s, HYPRE_Int *n) { return get_iters(s, n); }
HYPRE_Int HYPRE_ParCSRPCGGetFinalRelativeResidualNorm(HYPRE_Solver s, HYPRE_Real *r) { return get_res(s, r); }
HYPRE_Int HYPRE_FlexGMRESGetNumIterations(HYPRE_Solver s, HYPRE_Int *n) { return get_iters(s, n); }
HYPRE_Int HYPRE_FlexGMRESGetFinalRelativeResidualNorm(HYPRE_Solver s, HYPRE_Real *r) { return get_res(s, r); }
HYPRE_Int HYPRE_ParCSRFlexGMRESGetNumIterations(HYPRE_Solver s, HYPRE_Int *n) { return get_iters(s, n); }
HYPRE_Int HYPRE_ParCSRFlexGMRESGetFinalRelativeResidualNorm(HYPRE_Solver s, HYPRE_Real *r) { return get_res(s, r); }

HYPRE_Int HYPRE_GB300_KrylovGetResidualHistory(HYPRE_Solver solver, HYPRE_Int maxn, HYPRE_Real *relres, HYPRE_Int *n)
{
   gb_krylov *k = kry_of(solver, 1);
   if (!k) { return gb_error_flag; }
   int m = k->hist_n < maxn ? k->hist_n : maxn;
   if (relres) { for (int i = 0; i < m; i++) { relres[i] = k->hist[i]; } }
   if (n) { *n = k->hist_n; }
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * Diagonal scaling preconditioner: x = b ./ diag(A)
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_ParCSRDiagScaleSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector y, HYPRE_ParVector x)
{
   (void) solver; (void) y; (void) x;
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   if (!A->diag)
   {
      A->diag = (double *) gb_dmalloc(sizeof(double) * (size_t) (A->A.nr ? A->A.nr : 1));
      /* option 5 of the l1-norm kernel: the diagonal, 0 -> 1 (sign kept) */
      gb_l1_norms(A->A.nr, A->A.i, A->A.j, A->A.v, 5, NULL, A->diag, gb_stream());
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRDiagScale(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector y, HYPRE_ParVector x)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   if (!A->diag) { HYPRE_ParCSRDiagScaleSetup(solver, A, y, x); }
   gb_scaled_div_d(A->A.nr, 1.0, y->d, A->diag, x->d, gb_stream());
   return gb_error_flag;
}
