/* Multiple right-hand sides through one hierarchy: HYPRE_ParCSRPCGSolve with
 * multi-vectors (HYPRE_GB300_ParVectorCreateMulti, nv <= 64 columns stored
 * interleaved) runs an independent FP64 PCG per column -- its own scalars,
 * stopping test and history, as HYPRE_ParCSRPCGSolve on that column alone
 * (src/krylov/pcg.c:313, two-norm test) -- while every matrix product and the
 * V-cycle (FP64 or FP32) serve all columns in one SpMM pass.  The reference
 * has multi-vectors for its SpMV only; this extends its PCG column-wise.
 * Converged columns are frozen (step length 0). */
#include "gb_internal.h"

#include <math.h>

int gb_mdot_blocks(void);
void gb_spmm_d(int n, int nv, const int *Ai, const int *Aj, const double *Av, const double *x, double *y, int mode,
               double alpha, double beta, const double *b, const double *d, double w, int T, int U, cudaStream_t s);
void gb_spmm_f(int n, int nv, const int *Ai, const int *Aj, const float *Av, const float *x, float *y, int mode,
               float alpha, float beta, const float *b, const float *d, float w, int T, int U, cudaStream_t s);
void gb_mscaled_div_d(long long n, int nv, double w, const double *f, const double *d, double *u, cudaStream_t s);
void gb_mscaled_div_f(long long n, int nv, float w, const float *f, const float *d, float *u, cudaStream_t s);
void gb_mdense_d(int nc, int nv, const double *D, const double *f, double *u, cudaStream_t s);
void gb_mdense_f(int nc, int nv, const double *D, const float *f, float *u, cudaStream_t s);
void gb_mdot2(int n, int nv, const double *x, const double *y, const double *z, double *part, double *out,
              cudaStream_t s);
void gb_mpcg_xr(long long n, int nv, const double *a, const double *p, const double *sv, double *x, double *r,
                cudaStream_t s);
void gb_mxpay(long long n, int nv, const double *sv, const double *bc, double *p, cudaStream_t s);
void gb_d2f_n(long long n, const double *a, float *b, cudaStream_t s);
void gb_f2d_n(long long n, const float *a, double *b, cudaStream_t s);

#define MAXNV 64

typedef struct
{
   int     nv;
   double *F[32], *U[32], *U2[32], *V[32];
   float  *Ff[32], *Uf[32], *U2f[32], *Vf[32];
   float  *Avf[32], *Pvf[32], *Rvf[32];
   /* SpMM launch shapes (block size, rows of x in flight) per level of the
    * operands A, R, P in FP64 [0] and FP32 [1] */
   int     shA[32][2][2], shR[32][2][2], shP[32][2][2];
} gb_multi_ws;

void gb_multi_free(gb_amg *amg)
{
   gb_multi_ws *w = (gb_multi_ws *) amg->multi_ws;
   if (!w) { return; }
   for (int l = 0; l < 32; l++)
   {
      gb_dfree(w->F[l]); gb_dfree(w->U[l]); gb_dfree(w->U2[l]); gb_dfree(w->V[l]);
      gb_dfree(w->Ff[l]); gb_dfree(w->Uf[l]); gb_dfree(w->U2f[l]); gb_dfree(w->Vf[l]);
      gb_dfree(w->Avf[l]); gb_dfree(w->Pvf[l]); gb_dfree(w->Rvf[l]);
   }
   free(w);
   amg->multi_ws = NULL;
}

static gb_multi_ws *multi_ws(gb_amg *amg, int nv)
{
   gb_multi_ws *w = (gb_multi_ws *) amg->multi_ws;
   if (w && w->nv == nv) { return w; }
   gb_multi_free(amg);
   w = (gb_multi_ws *) calloc(1, sizeof(gb_multi_ws));
   w->nv = nv;
   cudaStream_t s = gb_stream();
   for (int l = 0; l < amg->num_levels; l++)
   {
      gb_level *L = &amg->lev[l];
      size_t m = (size_t) (L->n > 0 ? L->n : 1) * (size_t) nv;
      w->F[l] = (double *) gb_dcalloc(sizeof(double) * m);
      w->U[l] = (double *) gb_dcalloc(sizeof(double) * m);
      w->U2[l] = (double *) gb_dcalloc(sizeof(double) * m);
      w->V[l] = (double *) gb_dcalloc(sizeof(double) * m);
      w->Ff[l] = (float *) gb_dcalloc(sizeof(float) * m);
      w->Uf[l] = (float *) gb_dcalloc(sizeof(float) * m);
      w->U2f[l] = (float *) gb_dcalloc(sizeof(float) * m);
      w->Vf[l] = (float *) gb_dcalloc(sizeof(float) * m);
      gb_csr *A = &L->A->A;
      w->Avf[l] = (float *) gb_dmalloc(sizeof(float) * (size_t) (A->nnz > 0 ? A->nnz : 1));
      gb_d2f_n(A->nnz, A->v, w->Avf[l], s);
      if (L->P)
      {
         gb_csr *P = &L->P->A, *R = &L->R->A;
         w->Pvf[l] = (float *) gb_dmalloc(sizeof(float) * (size_t) (P->nnz > 0 ? P->nnz : 1));
         w->Rvf[l] = (float *) gb_dmalloc(sizeof(float) * (size_t) (R->nnz > 0 ? R->nnz : 1));
         gb_d2f_n(P->nnz, P->v, w->Pvf[l], s);
         gb_d2f_n(R->nnz, R->v, w->Rvf[l], s);
      }
   }
   /* launch shapes of every operand, timed on the workspace's vectors */
   for (int l = 0; l < amg->num_levels; l++)
   {
      gb_level *L = &amg->lev[l];
      gb_csr *A = &L->A->A;
      for (int pr = 0; pr < 2; pr++)
      {
         const int prec = pr ? GB_PREC_F32 : GB_PREC_F64;
         void *x = pr ? (void *) w->Uf[l] : (void *) w->U[l], *y = pr ? (void *) w->Vf[l] : (void *) w->V[l];
         gb_spmm_autotune(prec, L->n, L->n, A->nnz, nv, A->i, A->j, pr ? (const void *) w->Avf[l] : (const void *) A->v,
                          x, y, &w->shA[l][pr][0], &w->shA[l][pr][1]);
         if (L->P)
         {
            gb_csr *P = &L->P->A, *R = &L->R->A;
            void *xc = pr ? (void *) w->Uf[l + 1] : (void *) w->U[l + 1];
            void *yc = pr ? (void *) w->Ff[l + 1] : (void *) w->F[l + 1];
            gb_spmm_autotune(prec, R->nr, L->n, R->nnz, nv, R->i, R->j, pr ? (const void *) w->Rvf[l] : (const void *) R->v,
                             y, yc, &w->shR[l][pr][0], &w->shR[l][pr][1]);
            gb_spmm_autotune(prec, P->nr, R->nr, P->nnz, nv, P->i, P->j, pr ? (const void *) w->Pvf[l] : (const void *) P->v,
                             xc, x, &w->shP[l][pr][0], &w->shP[l][pr][1]);
         }
      }
   }
   amg->multi_ws = w;
   return w;
}

static int multi_cycle_supported(gb_amg *amg)
{
   gb_amg_params *p = &amg->prm;
   for (int k = 1; k <= 2; k++)
   {
      if (p->relax_type[k] != 18 && p->relax_type[k] != 7) { return 0; }
   }
   if ((p->relax_order != 0 || p->cycle_type != 1 || p->fcycle) && amg->num_levels > 1) { return 0; }
   return amg->coarse_inv != NULL || amg->num_levels == 1;
}

/* one V-cycle on nv columns from a zero guess, FP64 */
static void mcycle_d(gb_amg *amg, gb_multi_ws *w, int nv, const double *f0, double *u0)
{
   gb_amg_params *prm = &amg->prm;
   cudaStream_t s = gb_stream();
   int nl = amg->num_levels;
   for (int l = 0; l < nl - 1; l++)
   {
      gb_level *L = &amg->lev[l];
      gb_csr *A = &L->A->A, *R = &L->R->A;
      const double *F = l ? w->F[l] : f0;
      double *U = l ? w->U[l] : u0;
      gb_mscaled_div_d(L->n, nv, L->relax_w, F, L->l1, U, s);
      for (int sw = 1; sw < prm->num_sweeps[1]; sw++)
      {
         gb_spmm_d(L->n, nv, A->i, A->j, A->v, U, w->U2[l], 1, 0.0, 0.0, F, L->l1, L->relax_w, w->shA[l][0][0], w->shA[l][0][1], s);
         cudaMemcpyAsync(U, w->U2[l], sizeof(double) * (size_t) L->n * nv, cudaMemcpyDeviceToDevice, s);
      }
      gb_spmm_d(L->n, nv, A->i, A->j, A->v, U, w->V[l], 2, -1.0, 1.0, F, NULL, 0.0, w->shA[l][0][0], w->shA[l][0][1], s);
      gb_spmm_d(R->nr, nv, R->i, R->j, R->v, w->V[l], w->F[l + 1], 0, 1.0, 0.0, NULL, NULL, 0.0, w->shR[l][0][0], w->shR[l][0][1], s);
   }
   {
      int l = nl - 1;
      gb_level *L = &amg->lev[l];
      const double *F = l ? w->F[l] : f0;
      double *U = l ? w->U[l] : u0;
      if (amg->coarse_inv) { gb_mdense_d(amg->coarse_n, nv, amg->coarse_inv, F, U, s); }
      else { gb_mscaled_div_d(L->n, nv, L->relax_w, F, L->l1, U, s); }
   }
   for (int l = nl - 2; l >= 0; l--)
   {
      gb_level *L = &amg->lev[l];
      gb_csr *A = &L->A->A, *P = &L->P->A;
      const double *F = l ? w->F[l] : f0;
      double *U = l ? w->U[l] : u0;
      gb_spmm_d(P->nr, nv, P->i, P->j, P->v, w->U[l + 1], w->U2[l], 0, 1.0, 1.0, U, NULL, 0.0, w->shP[l][0][0], w->shP[l][0][1], s);
      if (prm->num_sweeps[2] == 0)
      {
         cudaMemcpyAsync(U, w->U2[l], sizeof(double) * (size_t) L->n * nv, cudaMemcpyDeviceToDevice, s);
      }
      for (int sw = 0; sw < prm->num_sweeps[2]; sw++)
      {
         if (sw == 0) { gb_spmm_d(L->n, nv, A->i, A->j, A->v, w->U2[l], U, 1, 0.0, 0.0, F, L->l1, L->relax_w, w->shA[l][0][0], w->shA[l][0][1], s); }
         else
         {
            gb_spmm_d(L->n, nv, A->i, A->j, A->v, U, w->U2[l], 1, 0.0, 0.0, F, L->l1, L->relax_w, w->shA[l][0][0], w->shA[l][0][1], s);
            cudaMemcpyAsync(U, w->U2[l], sizeof(double) * (size_t) L->n * nv, cudaMemcpyDeviceToDevice, s);
         }
      }
   }
}

/* the same cycle with FP32 vectors and level values; f0/u0 FP64 */
static void mcycle_f(gb_amg *amg, gb_multi_ws *w, int nv, const double *f0, double *u0)
{
   gb_amg_params *prm = &amg->prm;
   cudaStream_t s = gb_stream();
   int nl = amg->num_levels;
   gb_d2f_n((long long) amg->lev[0].n * nv, f0, w->Ff[0], s);
   for (int l = 0; l < nl - 1; l++)
   {
      gb_level *L = &amg->lev[l];
      gb_csr *A = &L->A->A, *R = &L->R->A;
      float *F = w->Ff[l], *U = w->Uf[l];
      float wt = (float) L->relax_w;
      gb_mscaled_div_f(L->n, nv, wt, F, L->l1f, U, s);
      for (int sw = 1; sw < prm->num_sweeps[1]; sw++)
      {
         gb_spmm_f(L->n, nv, A->i, A->j, w->Avf[l], U, w->U2f[l], 1, 0.f, 0.f, F, L->l1f, wt, w->shA[l][1][0], w->shA[l][1][1], s);
         cudaMemcpyAsync(U, w->U2f[l], sizeof(float) * (size_t) L->n * nv, cudaMemcpyDeviceToDevice, s);
      }
      gb_spmm_f(L->n, nv, A->i, A->j, w->Avf[l], U, w->Vf[l], 2, -1.f, 1.f, F, NULL, 0.f, w->shA[l][1][0], w->shA[l][1][1], s);
      gb_spmm_f(R->nr, nv, R->i, R->j, w->Rvf[l], w->Vf[l], w->Ff[l + 1], 0, 1.f, 0.f, NULL, NULL, 0.f, w->shR[l][1][0], w->shR[l][1][1], s);
   }
   {
      int l = nl - 1;
      gb_level *L = &amg->lev[l];
      if (amg->coarse_inv) { gb_mdense_f(amg->coarse_n, nv, amg->coarse_inv, w->Ff[l], w->Uf[l], s); }
      else { gb_mscaled_div_f(L->n, nv, (float) L->relax_w, w->Ff[l], L->l1f, w->Uf[l], s); }
   }
   for (int l = nl - 2; l >= 0; l--)
   {
      gb_level *L = &amg->lev[l];
      gb_csr *A = &L->A->A, *P = &L->P->A;
      float *F = w->Ff[l], *U = w->Uf[l];
      float wt = (float) L->relax_w;
      gb_spmm_f(P->nr, nv, P->i, P->j, w->Pvf[l], w->Uf[l + 1], w->U2f[l], 0, 1.f, 1.f, U, NULL, 0.f, w->shP[l][1][0], w->shP[l][1][1], s);
      if (prm->num_sweeps[2] == 0)
      {
         cudaMemcpyAsync(U, w->U2f[l], sizeof(float) * (size_t) L->n * nv, cudaMemcpyDeviceToDevice, s);
      }
      for (int sw = 0; sw < prm->num_sweeps[2]; sw++)
      {
         if (sw == 0) { gb_spmm_f(L->n, nv, A->i, A->j, w->Avf[l], w->U2f[l], U, 1, 0.f, 0.f, F, L->l1f, wt, w->shA[l][1][0], w->shA[l][1][1], s); }
         else
         {
            gb_spmm_f(L->n, nv, A->i, A->j, w->Avf[l], U, w->U2f[l], 1, 0.f, 0.f, F, L->l1f, wt, w->shA[l][1][0], w->shA[l][1][1], s);
            cudaMemcpyAsync(U, w->U2f[l], sizeof(float) * (size_t) L->n * nv, cudaMemcpyDeviceToDevice, s);
         }
      }
   }
   gb_f2d_n((long long) amg->lev[0].n * nv, w->Uf[0], u0, s);
}

static void mprecond(gb_krylov *k, gb_amg *amg, int n, int nv, const double *r, double *z)
{
   if (!amg)
   {
      cudaMemcpyAsync(z, r, sizeof(double) * (size_t) n * nv, cudaMemcpyDeviceToDevice, gb_stream());
      return;
   }
   gb_multi_ws *w = multi_ws(amg, nv);
   if (amg->prm.cycle_prec == GB_PREC_F64) { mcycle_d(amg, w, nv, r, z); }
   else { mcycle_f(amg, w, nv, r, z); }
   (void) k;
}

void gb_krylov_multi_free(gb_krylov *k)
{
   gb_dfree(k->m_r); gb_dfree(k->m_p); gb_dfree(k->m_s); gb_dfree(k->m_dev);
   k->m_r = k->m_p = k->m_s = k->m_dev = NULL;
   free(k->m_iters); free(k->m_relres); free(k->m_hist);
   k->m_iters = NULL; k->m_relres = NULL; k->m_hist = NULL;
   k->m_nv = 0;
   k->m_n = 0;
}

int gb_pcg_multi(gb_krylov *k, gb_parcsr *A, gb_parvec *b, gb_parvec *x)
{
   int n = A->A.nr, nv = b->num_vectors;
   if (nv < 1 || nv > MAXNV || x->num_vectors != nv)
   {
      gb_error(HYPRE_ERROR_GENERIC, "multi-vector PCG: 1..64 columns, b and x alike");
      gb_error_in_arg(3);
      return gb_error_flag;
   }
   gb_amg *amg = NULL;
   if (k->precond)
   {
      if ((void *) k->precond != (void *) HYPRE_BoomerAMGSolve)
      {
         gb_error(HYPRE_ERROR_GENERIC, "multi-vector PCG: the preconditioner must be BoomerAMG");
         return gb_error_flag;
      }
      amg = (gb_amg *) k->precond_solver;
      if (!amg->setup_done || !multi_cycle_supported(amg))
      {
         gb_error(HYPRE_ERROR_GENERIC, "multi-vector PCG: BoomerAMG needs setup, V-cycles, relax 18 or 7 in lexicographic order, direct coarsest");
         return gb_error_flag;
      }
   }
   cudaStream_t st = gb_stream();
   size_t nb = sizeof(double) * (size_t) (n > 0 ? n : 1) * (size_t) nv;
   int nbl = gb_mdot_blocks();
   if (k->m_nv != nv || k->m_n != n)
   {
      gb_krylov_multi_free(k);
      k->m_r = (double *) gb_dcalloc(nb);
      k->m_p = (double *) gb_dcalloc(nb);
      k->m_s = (double *) gb_dcalloc(nb);
      /* device scratch: dot partials, dot results, step lengths */
      k->m_dev = (double *) gb_dcalloc(sizeof(double) * ((size_t) nbl * 2 * nv + 4 * (size_t) nv));
      k->m_iters = (int *) calloc((size_t) nv, sizeof(int));
      k->m_relres = (double *) calloc((size_t) nv, sizeof(double));
      k->m_nv = nv;
      k->m_n = n;
      gb_spmm_autotune(GB_PREC_F64, n, n, A->A.nnz, nv, A->A.i, A->A.j, A->A.v, k->m_p, k->m_s, &k->m_shT,
                       &k->m_shU);
   }
   free(k->m_hist);
   k->m_hist = (double *) calloc((size_t) nv * (size_t) (k->max_iter + 1), sizeof(double));
   double *part = k->m_dev, *out = part + (size_t) nbl * 2 * nv, *da = out + 2 * nv, *db = da + nv;
   double *h = (double *) malloc(sizeof(double) * 2 * nv);
   double bi[MAXNV], gamma[MAXNV], gold[MAXNV], iprod[MAXNV], ha[MAXNV], hb[MAXNV];
   int active[MAXNV];
   const double *Av = A->A.v;
   /* <b, b> per column */
   gb_mdot2(n, nv, b->d, b->d, NULL, part, out, st);
   cudaMemcpyAsync(h, out, sizeof(double) * nv, cudaMemcpyDeviceToHost, st);
   gb_sync();
   for (int c = 0; c < nv; c++) { bi[c] = h[c]; active[c] = bi[c] > 0.0; k->m_iters[c] = 0; k->m_relres[c] = 0.0; }
   /* r = b - A x ; p = M r */
   gb_spmm_d(n, nv, A->A.i, A->A.j, Av, x->d, k->m_r, 2, -1.0, 1.0, b->d, NULL, 0.0, k->m_shT, k->m_shU, st);
   mprecond(k, amg, n, nv, k->m_r, k->m_p);
   gb_mdot2(n, nv, k->m_r, k->m_p, k->m_r, part, out, st);
   cudaMemcpyAsync(h, out, sizeof(double) * 2 * nv, cudaMemcpyDeviceToHost, st);
   gb_sync();
   const int stride = k->max_iter + 1;
   for (int c = 0; c < nv; c++)
   {
      gamma[c] = h[c];
      iprod[c] = h[nv + c];
      if (active[c]) { k->m_hist[(size_t) c * stride] = sqrt(iprod[c] / bi[c]); }
   }
   double eps = k->tol * k->tol;
   int any = 0;
   for (int c = 0; c < nv; c++) { any |= active[c]; }
   int it = 0;
   while (any && it + 1 <= k->max_iter)
   {
      it++;
      gb_spmm_d(n, nv, A->A.i, A->A.j, Av, k->m_p, k->m_s, 0, 1.0, 0.0, NULL, NULL, 0.0, k->m_shT, k->m_shU, st);
      gb_mdot2(n, nv, k->m_s, k->m_p, NULL, part, out, st);
      cudaMemcpyAsync(h, out, sizeof(double) * nv, cudaMemcpyDeviceToHost, st);
      gb_sync();
      for (int c = 0; c < nv; c++)
      {
         ha[c] = 0.0;
         if (!active[c]) { continue; }
         double sdotp = h[c];
         double al = sdotp != 0.0 ? gamma[c] / sdotp : 0.0;
         if (!(al > 0.0)) { active[c] = 0; gb_error(HYPRE_ERROR_CONV, "multi-vector PCG breakdown"); continue; }
         ha[c] = al;
      }
      cudaMemcpyAsync(da, ha, sizeof(double) * nv, cudaMemcpyHostToDevice, st);
      gb_mpcg_xr(n, nv, da, k->m_p, k->m_s, x->d, k->m_r, st);
      mprecond(k, amg, n, nv, k->m_r, k->m_s);
      gb_mdot2(n, nv, k->m_r, k->m_s, k->m_r, part, out, st);
      cudaMemcpyAsync(h, out, sizeof(double) * 2 * nv, cudaMemcpyDeviceToHost, st);
      gb_sync();
      any = 0;
      for (int c = 0; c < nv; c++)
      {
         hb[c] = 0.0;
         if (!active[c]) { continue; }
         gold[c] = gamma[c];
         gamma[c] = h[c];
         iprod[c] = h[nv + c];
         k->m_hist[(size_t) c * stride + it] = sqrt(iprod[c] / bi[c]);
         k->m_iters[c] = it;
         double e = eps;
         if (k->a_tol > 0.0 && k->a_tol * k->a_tol / bi[c] > e) { e = k->a_tol * k->a_tol / bi[c]; }
         if (iprod[c] / bi[c] < e) { active[c] = 0; continue; }
         hb[c] = gamma[c] / gold[c];
         any = 1;
      }
      cudaMemcpyAsync(db, hb, sizeof(double) * nv, cudaMemcpyHostToDevice, st);
      gb_mxpay(n, nv, k->m_s, db, k->m_p, st);
   }
   gb_sync();
   int conv = 1;
   for (int c = 0; c < nv; c++)
   {
      k->m_relres[c] = bi[c] > 0.0 ? sqrt(iprod[c] / bi[c]) : 0.0;
      if (active[c]) { conv = 0; }
   }
   free(h);
   k->num_iterations = it;
   double mx = 0.0;
   for (int c = 0; c < nv; c++) { mx = k->m_relres[c] > mx ? k->m_relres[c] : mx; }
   k->rel_resid = mx;
   if (!conv && k->tol > 0.0) { gb_error(HYPRE_ERROR_CONV, NULL); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_ParVectorCreateMulti(HYPRE_BigInt n, HYPRE_Int num_vectors, HYPRE_ParVector *vector)
{
   if (!vector) { gb_error_in_arg(3); return gb_error_flag; }
   if (n < 0) { gb_error_in_arg(1); return gb_error_flag; }
   if (num_vectors < 1 || num_vectors > MAXNV) { gb_error_in_arg(2); return gb_error_flag; }
   if (gb_runtime_init()) { return gb_error_flag; }
   gb_parvec *v = (gb_parvec *) calloc(1, sizeof(gb_parvec));
   v->magic = GB_MAGIC_VEC;
   v->n = n;
   v->num_vectors = num_vectors;
   v->d = (double *) gb_dcalloc(sizeof(double) * (size_t) (n > 0 ? n : 1) * (size_t) num_vectors);
   v->owns = 1;
   *vector = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_KrylovGetMultiNumIterations(HYPRE_Solver solver, HYPRE_Int *iterations)
{
   gb_krylov *k = (gb_krylov *) solver;
   if (!k || (k->magic != GB_MAGIC_PCG && k->magic != GB_MAGIC_GMR)) { gb_error_in_arg(1); return gb_error_flag; }
   if (!iterations) { gb_error_in_arg(2); return gb_error_flag; }
   if (!k->last_multi) { iterations[0] = k->num_iterations; return gb_error_flag; }
   memcpy(iterations, k->m_iters, sizeof(int) * (size_t) k->m_nv);
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_KrylovGetMultiFinalRelativeResidualNorms(HYPRE_Solver solver, HYPRE_Real *relres)
{
   gb_krylov *k = (gb_krylov *) solver;
   if (!k || (k->magic != GB_MAGIC_PCG && k->magic != GB_MAGIC_GMR)) { gb_error_in_arg(1); return gb_error_flag; }
   if (!relres) { gb_error_in_arg(2); return gb_error_flag; }
   if (!k->last_multi) { relres[0] = k->rel_resid; return gb_error_flag; }
   memcpy(relres, k->m_relres, sizeof(double) * (size_t) k->m_nv);
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_KrylovGetMultiResidualHistory(HYPRE_Solver solver, HYPRE_Int column, HYPRE_Int maxn,
                                                    HYPRE_Real *relres, HYPRE_Int *n)
{
   gb_krylov *k = (gb_krylov *) solver;
   if (!k || (k->magic != GB_MAGIC_PCG && k->magic != GB_MAGIC_GMR)) { gb_error_in_arg(1); return gb_error_flag; }
   if (!k->last_multi)
   {
      /* single-vector solve: its history is column 0 */
      if (column != 0 || !relres) { gb_error_in_arg(2); return gb_error_flag; }
      int cnt = k->hist_n < maxn ? k->hist_n : maxn;
      if (cnt > 0) { memcpy(relres, k->hist, sizeof(double) * (size_t) cnt); }
      if (n) { *n = cnt; }
      return gb_error_flag;
   }
   if (column < 0 || column >= k->m_nv || !k->m_hist || !relres) { gb_error_in_arg(2); return gb_error_flag; }
   int cnt = k->m_iters[column] + 1;
   if (cnt > maxn) { cnt = maxn; }
   memcpy(relres, k->m_hist + (size_t) column * (k->max_iter + 1), sizeof(double) * (size_t) cnt);
   if (n) { *n = cnt; }
   return gb_error_flag;
}
