/* Batched AMG-PCG: many independent systems, given as the diagonal blocks of
 * one matrix, solved by one persistent kernel launch (gb_batch.cu).  The
 * reference has no batched solver; this is the GPU-native way to run its
 * BoomerAMG-PCG on hundreds of small systems at once.
 *
 * Setup runs the ordinary BoomerAMG setup on the block-diagonal matrix (one
 * call for the whole batch).  Every level stays block diagonal and the coarse
 * points of a block are numbered consecutively, so the per-system row ranges
 * of level l+1 follow from counting C points inside the ranges of level l.
 * An autotuner picks the lanes per row and the block size of the persistent
 * kernel by timing each variant on the first solve. */
#include "gb_internal.h"

typedef struct
{
   int      magic;
   gb_amg  *amg;          /* borrowed */
   gb_parcsr *A;          /* borrowed */
   int      n, nsys, nlev;
   double   tol;
   int      maxit, prec;
   int      lpr, block, autotune, tuned;
   int     *off_h[32];    /* host per-level offsets (nsys + 1) */
   int     *off_d[32];
   float   *Avf[32], *Pvf[32], *Rvf[32];
   void    *lev_d[2];     /* device gb_blevel arrays: [0] FP64 cycle, [1] FP32 cycle */
   int     *order_d, *counter_d, *iters_d;
   double  *relres_d, *hist_d;
   int      hist_cap;
   int     *iters_h;
   double  *relres_h, *hist_h;
   double  *r, *p, *s;
   double  *opc;          /* per-system operator complexity (host) */
   double  *dinv;         /* coarsest level: inverse of each system's block (device) */
   long long *doff_d;
   int      sms;
   float    tune_ms[4][3];
} gb_batch;

static gb_batch *bat_of(HYPRE_Solver s, int arg)
{
   gb_batch *b = (gb_batch *) s;
   if (!b || b->magic != GB_MAGIC_BAT) { gb_error_in_arg(arg); return NULL; }
   return b;
}

static void batch_free_setup(gb_batch *b)
{
   for (int l = 0; l < 32; l++)
   {
      free(b->off_h[l]); b->off_h[l] = NULL;
      gb_dfree(b->off_d[l]); b->off_d[l] = NULL;
      gb_dfree(b->Avf[l]); gb_dfree(b->Pvf[l]); gb_dfree(b->Rvf[l]);
      b->Avf[l] = b->Pvf[l] = b->Rvf[l] = NULL;
   }
   gb_dfree(b->lev_d[0]); gb_dfree(b->lev_d[1]);
   b->lev_d[0] = b->lev_d[1] = NULL;
   gb_dfree(b->order_d); gb_dfree(b->counter_d); gb_dfree(b->iters_d); gb_dfree(b->relres_d); gb_dfree(b->hist_d);
   b->order_d = b->counter_d = b->iters_d = NULL;
   b->relres_d = b->hist_d = NULL;
   b->hist_cap = 0;
   free(b->iters_h); free(b->relres_h); free(b->hist_h);
   b->iters_h = NULL; b->relres_h = NULL; b->hist_h = NULL;
   gb_dfree(b->r); gb_dfree(b->p); gb_dfree(b->s);
   b->r = b->p = b->s = NULL;
   free(b->opc);
   b->opc = NULL;
   gb_dfree(b->dinv); gb_dfree(b->doff_d);
   b->dinv = NULL;
   b->doff_d = NULL;
   b->nlev = 0;
}

HYPRE_Int HYPRE_GB300_BatchedPCGCreate(HYPRE_Solver *solver)
{
   if (!solver) { gb_error_in_arg(1); return gb_error_flag; }
   if (gb_runtime_init()) { return gb_error_flag; }
   gb_batch *b = (gb_batch *) calloc(1, sizeof(gb_batch));
   b->magic = GB_MAGIC_BAT;
   b->tol = 1e-8;
   b->maxit = 100;
   b->prec = GB_PREC_F32;
   b->lpr = 4;
   b->block = 256;
   b->autotune = 1;
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   b->sms = sms > 0 ? sms : 1;
   *solver = (HYPRE_Solver) b;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGDestroy(HYPRE_Solver solver)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   batch_free_setup(b);
   b->magic = 0;
   free(b);
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGSetTol(HYPRE_Solver solver, HYPRE_Real tol)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (tol < 0.0) { gb_error_in_arg(2); return gb_error_flag; }
   b->tol = tol;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (max_iter < 0) { gb_error_in_arg(2); return gb_error_flag; }
   b->maxit = max_iter;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGSetCyclePrecision(HYPRE_Solver solver, HYPRE_Int precision)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (precision != GB_PREC_F64 && precision != GB_PREC_F32) { gb_error_in_arg(2); return gb_error_flag; }
   b->prec = precision;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGSetKernelShape(HYPRE_Solver solver, HYPRE_Int lanes_per_row, HYPRE_Int block)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (lanes_per_row != 1 && lanes_per_row != 2 && lanes_per_row != 4 && lanes_per_row != 8)
   {
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   if (block != 128 && block != 256 && block != 512) { gb_error_in_arg(3); return gb_error_flag; }
   b->lpr = lanes_per_row;
   b->block = block;
   b->autotune = 0;
   b->tuned = 1;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGSetAutotune(HYPRE_Solver solver, HYPRE_Int autotune)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   b->autotune = autotune ? 1 : 0;
   b->tuned = 0;
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetKernelShape(HYPRE_Solver solver, HYPRE_Int *lanes_per_row, HYPRE_Int *block)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (lanes_per_row) { *lanes_per_row = b->lpr; }
   if (block) { *block = b->block; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetTuningTimes(HYPRE_Solver solver, HYPRE_Real *ms)
{
   /* ms[4][3]: lanes per row 1, 2, 4, 8 x block 128, 256, 512 (0 = not timed) */
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (!ms) { gb_error_in_arg(2); return gb_error_flag; }
   for (int i = 0; i < 4; i++)
      for (int j = 0; j < 3; j++) { ms[i * 3 + j] = b->tune_ms[i][j]; }
   return gb_error_flag;
}

static const int *g_sort_off;
static int cmp_sys(const void *x, const void *y)
{
   int a = *(const int *) x, c = *(const int *) y;
   int la = g_sort_off[a + 1] - g_sort_off[a], lc = g_sort_off[c + 1] - g_sort_off[c];
   if (la != lc) { return lc - la; }
   return a - c;
}

HYPRE_Int HYPRE_GB300_BatchedPCGSetup(HYPRE_Solver solver, HYPRE_Solver amg_solver, HYPRE_ParCSRMatrix A,
                                      HYPRE_Int num_systems, const HYPRE_Int *system_offsets)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   gb_amg *amg = (gb_amg *) amg_solver;
   if (!amg || amg->magic != GB_MAGIC_AMG) { gb_error_in_arg(2); return gb_error_flag; }
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(3); return gb_error_flag; }
   int n = A->A.nr;
   if (num_systems < 1) { gb_error_in_arg(4); return gb_error_flag; }
   if (!system_offsets || system_offsets[0] != 0 || system_offsets[num_systems] != n)
   {
      gb_error_in_arg(5);
      return gb_error_flag;
   }
   for (int s = 0; s < num_systems; s++)
   {
      if (system_offsets[s + 1] < system_offsets[s]) { gb_error_in_arg(5); return gb_error_flag; }
   }
   gb_amg_params *prm = &amg->prm;
   for (int k = 1; k <= 2; k++)
   {
      if (prm->relax_type[k] != 18 && prm->relax_type[k] != 7)
      {
         gb_error(HYPRE_ERROR_GENERIC, "batched PCG: relax type must be 18 (l1-Jacobi) or 7 (Jacobi)");
         return gb_error_flag;
      }
   }
   if (prm->relax_order != 0 || prm->cycle_type != 1 || prm->fcycle)
   {
      gb_error(HYPRE_ERROR_GENERIC, "batched PCG: V-cycles with relax_order 0 (lexicographic)");
      return gb_error_flag;
   }
   if (prm->agg_num_levels > 0)
   {
      gb_error(HYPRE_ERROR_GENERIC, "batched PCG: aggressive coarsening is not supported");
      return gb_error_flag;
   }
   batch_free_setup(b);
   cudaStream_t st = gb_stream();
   b->n = n;
   b->nsys = num_systems;
   b->A = A;
   b->amg = amg;
   /* level-0 offsets and the block-diagonal check */
   size_t ob = sizeof(int) * (size_t) (num_systems + 1);
   b->off_h[0] = (int *) malloc(ob);
   memcpy(b->off_h[0], system_offsets, ob);
   b->off_d[0] = (int *) gb_dmalloc(ob);
   cudaMemcpyAsync(b->off_d[0], b->off_h[0], ob, cudaMemcpyHostToDevice, st);
   int *bad = (int *) gb_dcalloc(sizeof(int));
   gb_check_blockdiag(n, A->A.i, A->A.j, b->off_d[0], num_systems, bad, st);
   int hbad = 0;
   cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
   gb_sync();
   gb_dfree(bad);
   if (hbad)
   {
      gb_error(HYPRE_ERROR_GENERIC, "batched PCG: matrix has entries outside the systems' diagonal blocks");
      gb_error_in_arg(3);
      batch_free_setup(b);
      return gb_error_flag;
   }
   /* one BoomerAMG setup for the whole block-diagonal matrix.  Its coarsest
    * level holds every system's coarsest block and may exceed max_coarse_size,
    * where the single-system setup switches the coarsest relaxation to the
    * down-cycle type; each system's block is solved directly here, so the
    * coarsest type is kept. */
   const int ct = prm->relax_type[3];
   const int setup_rc = gb_amg_setup(amg, A);
   prm->relax_type[3] = ct;
   if (setup_rc) { batch_free_setup(b); return gb_error_flag; }
   int nl = amg->num_levels;
   if (!(ct == 9 || ct == 19 || ct == 98 || ct == 99))
   {
      gb_error(HYPRE_ERROR_GENERIC, "batched PCG: the coarsest level needs a direct solve (relax 9/19/98/99)");
      batch_free_setup(b);
      return gb_error_flag;
   }
   b->nlev = nl;
   /* per-level system offsets from the C points inside each system's range */
   for (int l = 0; l + 1 < nl; l++)
   {
      int nlv = amg->lev[l].n;
      int *cf = (int *) malloc(sizeof(int) * (size_t) (nlv > 0 ? nlv : 1));
      cudaMemcpyAsync(cf, amg->lev[l].CF, sizeof(int) * (size_t) nlv, cudaMemcpyDeviceToHost, st);
      gb_sync();
      int *o = (int *) malloc(ob);
      o[0] = 0;
      int c = 0;
      for (int s = 0; s < num_systems; s++)
      {
         for (int i = b->off_h[l][s]; i < b->off_h[l][s + 1]; i++) { c += cf[i] > 0; }
         o[s + 1] = c;
      }
      free(cf);
      if (c != amg->lev[l + 1].n)
      {
         free(o);
         gb_error(HYPRE_ERROR_GENERIC, "batched PCG: coarse numbering does not follow the systems");
         batch_free_setup(b);
         return gb_error_flag;
      }
      b->off_h[l + 1] = o;
      b->off_d[l + 1] = (int *) gb_dmalloc(ob);
      cudaMemcpyAsync(b->off_d[l + 1], o, ob, cudaMemcpyHostToDevice, st);
   }
   /* coarsest level: the inverse of each system's diagonal block */
   {
      const int *oc = b->off_h[nl - 1];
      long long *doff = (long long *) malloc(sizeof(long long) * (size_t) (num_systems + 1));
      doff[0] = 0;
      int mmax = 0;
      for (int s = 0; s < num_systems; s++)
      {
         long long m = oc[s + 1] - oc[s];
         if (m > mmax) { mmax = (int) m; }
         doff[s + 1] = doff[s] + m * m;
      }
      if (mmax > 2048)
      {
         free(doff);
         gb_error(HYPRE_ERROR_GENERIC, "batched PCG: a system's coarsest block exceeds 2048 rows");
         batch_free_setup(b);
         return gb_error_flag;
      }
      size_t tot = sizeof(double) * (size_t) (doff[num_systems] > 0 ? doff[num_systems] : 1);
      b->dinv = (double *) gb_dmalloc(tot);
      double *W = (double *) gb_dmalloc(tot);
      b->doff_d = (long long *) gb_dmalloc(sizeof(long long) * (size_t) (num_systems + 1));
      cudaMemcpyAsync(b->doff_d, doff, sizeof(long long) * (size_t) (num_systems + 1), cudaMemcpyHostToDevice, st);
      gb_csr *Ac = &amg->lev[nl - 1].A->A;
      gb_block_inverse(num_systems, b->off_d[nl - 1], Ac->i, Ac->j, Ac->v, b->doff_d, b->dinv, W, st);
      gb_sync();
      gb_dfree(W);
      free(doff);
   }
   /* per-system operator complexity: sum over levels of the system's nonzeros / level-0 nonzeros */
   b->opc = (double *) calloc((size_t) num_systems, sizeof(double));
   double *nnz0 = (double *) calloc((size_t) num_systems, sizeof(double));
   for (int l = 0; l < nl; l++)
   {
      int nlv = amg->lev[l].n;
      int *ai = (int *) malloc(sizeof(int) * (size_t) (nlv + 1));
      cudaMemcpyAsync(ai, amg->lev[l].A->A.i, sizeof(int) * (size_t) (nlv + 1), cudaMemcpyDeviceToHost, st);
      gb_sync();
      for (int s = 0; s < num_systems; s++)
      {
         double z = (double) (ai[b->off_h[l][s + 1]] - ai[b->off_h[l][s]]);
         if (l == 0) { nnz0[s] = z; }
         b->opc[s] += z;
      }
      free(ai);
   }
   for (int s = 0; s < num_systems; s++) { b->opc[s] = nnz0[s] > 0 ? b->opc[s] / nnz0[s] : 1.0; }
   free(nnz0);
   /* FP32 values of the level operators and the device level tables */
   size_t lsz = gb_blevel_size();
   void *hl[2];
   hl[0] = calloc((size_t) nl, lsz);
   hl[1] = calloc((size_t) nl, lsz);
   for (int l = 0; l < nl; l++)
   {
      gb_level *L = &amg->lev[l];
      gb_csr *M = &L->A->A;
      b->Avf[l] = (float *) gb_dmalloc(sizeof(float) * (size_t) (M->nnz > 0 ? M->nnz : 1));
      gb_convert_vals(M->nnz, M->v, b->Avf[l], GB_PREC_F32, st);
      const int *Pi = NULL, *Pj = NULL, *Ri = NULL, *Rj = NULL;
      const double *Pv = NULL, *Rv = NULL;
      if (l + 1 < nl)
      {
         gb_csr *P = &L->P->A, *R = &L->R->A;
         Pi = P->i; Pj = P->j; Pv = P->v;
         Ri = R->i; Rj = R->j; Rv = R->v;
         b->Pvf[l] = (float *) gb_dmalloc(sizeof(float) * (size_t) (P->nnz > 0 ? P->nnz : 1));
         b->Rvf[l] = (float *) gb_dmalloc(sizeof(float) * (size_t) (R->nnz > 0 ? R->nnz : 1));
         gb_convert_vals(P->nnz, P->v, b->Pvf[l], GB_PREC_F32, st);
         gb_convert_vals(R->nnz, R->v, b->Rvf[l], GB_PREC_F32, st);
      }
      double w = L->relax_w;
      gb_blevel_set(hl[0], l, L->n, M->i, M->j, M->v, Pi, Pj, Pv, Ri, Rj, Rv, L->l1, L->F, L->U, L->V,
                    b->off_d[l], w);
      gb_blevel_set(hl[1], l, L->n, M->i, M->j, b->Avf[l], Pi, Pj, b->Pvf[l], Ri, Rj, b->Rvf[l], L->l1f, L->Ff,
                    L->Uf, L->Vf, b->off_d[l], w);
   }
   for (int k = 0; k < 2; k++)
   {
      b->lev_d[k] = gb_dmalloc(lsz * (size_t) nl);
      cudaMemcpyAsync(b->lev_d[k], hl[k], lsz * (size_t) nl, cudaMemcpyHostToDevice, st);
   }
   /* work queue, largest systems first */
   int *order = (int *) malloc(sizeof(int) * (size_t) num_systems);
   for (int s = 0; s < num_systems; s++) { order[s] = s; }
   g_sort_off = b->off_h[0];
   qsort(order, (size_t) num_systems, sizeof(int), cmp_sys);
   b->order_d = (int *) gb_dmalloc(sizeof(int) * (size_t) num_systems);
   cudaMemcpyAsync(b->order_d, order, sizeof(int) * (size_t) num_systems, cudaMemcpyHostToDevice, st);
   b->counter_d = (int *) gb_dcalloc(sizeof(int));
   b->iters_d = (int *) gb_dmalloc(sizeof(int) * (size_t) num_systems);
   b->relres_d = (double *) gb_dmalloc(sizeof(double) * (size_t) num_systems);
   b->iters_h = (int *) calloc((size_t) num_systems, sizeof(int));
   b->relres_h = (double *) calloc((size_t) num_systems, sizeof(double));
   size_t nb = sizeof(double) * (size_t) (n > 0 ? n : 1);
   b->r = (double *) gb_dmalloc(nb);
   b->p = (double *) gb_dmalloc(nb);
   b->s = (double *) gb_dmalloc(nb);
   gb_sync();
   free(hl[0]); free(hl[1]); free(order);
   return gb_error_flag;
}

static void ensure_hist(gb_batch *b)
{
   int need = b->nsys * (b->maxit + 1);
   if (need > b->hist_cap)
   {
      gb_dfree(b->hist_d);
      free(b->hist_h);
      b->hist_d = (double *) gb_dcalloc(sizeof(double) * (size_t) need);
      b->hist_h = (double *) calloc((size_t) need, sizeof(double));
      b->hist_cap = need;
   }
}

static void launch(gb_batch *b, const double *bd, double *xd, int lpr, int block)
{
   gb_amg *amg = b->amg;
   int grid = b->sms * (block <= 128 ? 8 : block <= 256 ? 4 : 2);
   if (grid > b->nsys) { grid = b->nsys; }
   gb_batch_pcg(b->lev_d[b->prec == GB_PREC_F64 ? 0 : 1], b->nlev, b->nsys, amg->prm.num_sweeps[1],
                amg->prm.num_sweeps[2], b->A->A.i, b->A->A.j, b->A->A.v, b->order_d, b->counter_d, bd, xd, b->r,
                b->p, b->s, b->dinv, b->doff_d, b->tol, b->maxit, b->iters_d, b->relres_d, b->hist_d,
                b->prec, lpr, grid, block, gb_stream());
}

HYPRE_Int HYPRE_GB300_BatchedPCGSolve(HYPRE_Solver solver, HYPRE_ParVector bv, HYPRE_ParVector xv)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (!b->nlev) { gb_error(HYPRE_ERROR_GENERIC, "batched PCG: setup not done"); return gb_error_flag; }
   if (!bv || bv->magic != GB_MAGIC_VEC || bv->n != b->n) { gb_error_in_arg(2); return gb_error_flag; }
   if (!xv || xv->magic != GB_MAGIC_VEC || xv->n != b->n) { gb_error_in_arg(3); return gb_error_flag; }
   cudaStream_t st = gb_stream();
   ensure_hist(b);
   if (b->autotune && !b->tuned)
   {
      /* time every kernel shape on this right-hand side from the same initial guess */
      size_t nb = sizeof(double) * (size_t) b->n;
      double *x0 = (double *) gb_dmalloc(nb > 0 ? nb : 8);
      cudaMemcpyAsync(x0, xv->d, nb, cudaMemcpyDeviceToDevice, st);
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      const int lprs[4] = {1, 2, 4, 8}, blocks[3] = {128, 256, 512};
      float best = 1e30f;
      for (int i = 0; i < 4; i++)
      {
         for (int j = 0; j < 3; j++)
         {
            cudaMemcpyAsync(xv->d, x0, nb, cudaMemcpyDeviceToDevice, st);
            cudaEventRecord(e0, st);
            launch(b, bv->d, xv->d, lprs[i], blocks[j]);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            b->tune_ms[i][j] = ms;
            if (ms < best) { best = ms; b->lpr = lprs[i]; b->block = blocks[j]; }
         }
      }
      cudaMemcpyAsync(xv->d, x0, nb, cudaMemcpyDeviceToDevice, st);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      gb_dfree(x0);
      b->tuned = 1;
   }
   launch(b, bv->d, xv->d, b->lpr, b->block);
   cudaMemcpyAsync(b->iters_h, b->iters_d, sizeof(int) * (size_t) b->nsys, cudaMemcpyDeviceToHost, st);
   cudaMemcpyAsync(b->relres_h, b->relres_d, sizeof(double) * (size_t) b->nsys, cudaMemcpyDeviceToHost, st);
   gb_sync();
   gb_cuda_ok(cudaGetLastError(), "batched PCG");
   if (b->tol > 0.0)
   {
      for (int s = 0; s < b->nsys; s++)
      {
         if (!(b->relres_h[s] < b->tol)) { gb_error(HYPRE_ERROR_CONV, NULL); break; }
      }
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetNumIterations(HYPRE_Solver solver, HYPRE_Int *iters)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (!iters) { gb_error_in_arg(2); return gb_error_flag; }
   if (b->iters_h) { memcpy(iters, b->iters_h, sizeof(int) * (size_t) b->nsys); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetFinalRelativeResidualNorms(HYPRE_Solver solver, HYPRE_Real *relres)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (!relres) { gb_error_in_arg(2); return gb_error_flag; }
   if (b->relres_h) { memcpy(relres, b->relres_h, sizeof(double) * (size_t) b->nsys); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetResidualHistory(HYPRE_Solver solver, HYPRE_Int system, HYPRE_Int maxn,
                                                   HYPRE_Real *relres, HYPRE_Int *n)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (system < 0 || system >= b->nsys || !b->hist_d) { gb_error_in_arg(2); return gb_error_flag; }
   int cnt = b->iters_h[system] + 1;
   if (cnt > maxn) { cnt = maxn; }
   cudaMemcpyAsync(relres, b->hist_d + (size_t) system * (b->maxit + 1), sizeof(double) * (size_t) cnt,
                   cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   if (n) { *n = cnt; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetLevelOffsets(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int *offsets)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (level < 0 || level >= b->nlev || !offsets) { gb_error_in_arg(2); return gb_error_flag; }
   memcpy(offsets, b->off_h[level], sizeof(int) * (size_t) (b->nsys + 1));
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BatchedPCGGetOperatorComplexities(HYPRE_Solver solver, HYPRE_Real *opc)
{
   gb_batch *b = bat_of(solver, 1);
   if (!b) { return gb_error_flag; }
   if (!opc || !b->opc) { gb_error_in_arg(2); return gb_error_flag; }
   memcpy(opc, b->opc, sizeof(double) * (size_t) b->nsys);
   return gb_error_flag;
}
