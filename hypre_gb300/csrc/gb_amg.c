/* BoomerAMG on one GB300: parameter object, setup driver, V-cycle and the
 * stand-alone solve, in C over the kernels of gb_setup.cu / gb_solve.cu.
 *
 * Reference behaviour followed:
 *   defaults            src/parcsr_ls/par_amg.c:162-313 (device defaults: PMIS,
 *                       l1-Jacobi, kept transpose)
 *   setup level loop    src/parcsr_ls/par_amg_setup.c:1002-3145
 *   coarsest solve      src/parcsr_ls/par_gauss_elim.c (dense, explicit inverse)
 *   smoother setup      src/parcsr_ls/par_amg_setup.c:3242-3545
 *   V-cycle             src/parcsr_ls/par_cycle.c:23-889
 *   stand-alone solve   src/parcsr_ls/par_amg_solve.c:22-424
 */
#include "gb_internal.h"

#include <math.h>

static size_t gb_slab_bytes_c(int cap)
{
   /* per-warp slab of gb_device.cuh: hk[cap] hp[cap] vals/keys/slots[cap/2] */
   return (size_t) cap * 4 * 2 + (size_t) (cap / 2) * (4 + 4 + 8);
}

static int next_pow2(long long x)
{
   long long p = 64;
   while (p < x) { p <<= 1; }
   return p > (1LL << 30) ? (1 << 30) : (int) p;
}

static void amg_defaults(gb_amg_params *p)
{
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
   p->min_coarse_size = 0;
   p->relax_type[0] = 18; p->relax_type[1] = 18; p->relax_type[2] = 18; p->relax_type[3] = 9;
   for (int k = 0; k < 4; k++) { p->num_sweeps[k] = 1; }
   p->relax_weight = 1.0;
   p->cheby_order = 2;
   p->cheby_fraction = 0.3;
   p->cheby_scale = 1;
   p->cheby_eig_est = 10;
   p->cycle_type = 1;
   p->outer_weight = 1.0;
   p->tol = 1.0e-6;
   p->max_iter = 20;
   p->cycle_prec = GB_PREC_F64;
   p->use_graph = 1;
}

static gb_amg *amg_of(HYPRE_Solver s, int arg)
{
   gb_amg *a = (gb_amg *) s;
   if (!a || a->magic != GB_MAGIC_AMG) { gb_error_in_arg(arg); return NULL; }
   return a;
}

/* --------------------------------------------------------------------------
 * hierarchy memory
 * ------------------------------------------------------------------------ */
static void level_free_vectors(gb_level *L)
{
   gb_dfree(L->F); gb_dfree(L->U); gb_dfree(L->U2); gb_dfree(L->V);
   gb_dfree(L->Ff); gb_dfree(L->Uf); gb_dfree(L->U2f); gb_dfree(L->Vf);
   gb_dfree(L->cheb_ds); gb_dfree(L->cheb_dsf); gb_dfree(L->W); gb_dfree(L->Wf);
   gb_dfree(L->hgs_flags); gb_dfree(L->hgs_t); gb_dfree(L->hgs_tf);
   L->hgs_flags = NULL; L->hgs_t = NULL; L->hgs_tf = NULL;
   L->F = L->U = L->U2 = L->V = NULL;
   L->Ff = L->Uf = L->U2f = L->Vf = NULL;
   L->cheb_ds = L->W = NULL;
   L->cheb_dsf = L->Wf = NULL;
}

static void amg_free_hierarchy(gb_amg *amg)
{
   if (amg->graph) { cudaGraphExecDestroy(amg->graph); amg->graph = NULL; }
   gb_multi_free(amg);
   for (int l = 0; l < amg->num_levels; l++)
   {
      gb_level *L = &amg->lev[l];
      if (l > 0 && L->A) { gb_parcsr_free(L->A); }
      if (L->P) { gb_parcsr_free(L->P); }
      if (L->R) { gb_parcsr_free(L->R); }
      gb_csr_free(&L->S);
      gb_dfree(L->CF); gb_dfree(L->l1); gb_dfree(L->l1f);
      level_free_vectors(L);
      memset(L, 0, sizeof(*L));
   }
   gb_dfree(amg->coarse_inv);
   amg->coarse_inv = NULL;
   gb_dfree(amg->r_work);
   amg->r_work = NULL;
   amg->num_levels = 0;
   amg->setup_done = 0;
   amg->uses_hgs = 0;
}

/* --------------------------------------------------------------------------
 * device helpers
 * ------------------------------------------------------------------------ */
static int read_int(const int *d)
{
   int *h = gb_red_ints();
   h[0] = 0;
   cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   return h[0];
}

/* exclusive scan into out (n+1), returns total */
static int scan_total(const int *in, int *out, int n)
{
   int *scr = (int *) gb_scratch(0, sizeof(int) * (size_t) gb_scan_scratch_ints(n > 0 ? n : 1));
   gb_exclusive_scan(in, out, n, scr, gb_stream());
   return read_int(out + n);
}

/* Rewrites a list of distinct rows of 0..n-1 in increasing order (flags,
 * scan, scatter): the warps of the next tier then work on neighbouring rows
 * at the same time, whose B rows share the L2. */
static void sort_row_list_n(int *list, int nlist, const int *dcount, int n)
{
   if (nlist <= 1) { return; }
   cudaStream_t s = gb_stream();
   int *flag = (int *) gb_dcalloc(sizeof(int) * (size_t) (n + 1));
   int *pos = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   if (!flag || !pos) { gb_dfree(flag); gb_dfree(pos); return; }
   gb_list_flags(nlist, dcount, list, flag, s);
   int *scr = (int *) gb_scratch(0, sizeof(int) * (size_t) gb_scan_scratch_ints(n > 0 ? n : 1));
   gb_exclusive_scan(flag, pos, n, scr, s);
   gb_scatter_list(n, flag, pos, list, s);
   gb_dfree(flag); gb_dfree(pos);
}

static void sort_row_list(int *list, int nlist, int n) { sort_row_list_n(list, nlist, NULL, n); }

static int max_of(const int *d, int n)
{
   /* small host reduction of a device array (setup only) */
   if (n <= 0) { return 0; }
   int *h = (int *) malloc(sizeof(int) * (size_t) n);
   cudaMemcpyAsync(h, d, sizeof(int) * (size_t) n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   int m = 0;
   for (int i = 0; i < n; i++) { if (h[i] > m) { m = h[i]; } }
   free(h);
   return m;
}

/* number of persistent warps for slab kernels under a memory budget */
static int slab_warps(size_t slab_bytes, int rows)
{
   size_t budget = (size_t) 2 << 30;   /* 2 GiB of scratch at most */
   long long w = (long long) (budget / (slab_bytes ? slab_bytes : 1));
   long long maxw = (long long) gb_num_sms() * 48;
   if (w > maxw) { w = maxw; }
   if (w > rows) { w = rows; }
   /* launchers use 4-warp blocks: keep the count a multiple of 4 so every
    * launched warp owns an allocated slab */
   w = (w + 3) / 4 * 4;
   if (w < 4) { w = 4; }
   return (int) w;
}

static char *alloc_slabs(int cap, int nwarps)
{
   size_t per = (size_t) cap * 4 * 2 + (size_t) (cap / 2) * (4 + 4 + 8);
   size_t bytes = per * (size_t) nwarps;
   char *p = (char *) gb_dmalloc(bytes);
   if (p) { cudaMemsetAsync(p, 0xff, bytes, gb_stream()); }
   return p;
}

gb_parcsr *gb_transpose(gb_parcsr *M)
{
   gb_csr *A = &M->A;
   gb_csr T;
   T.nr = A->nc; T.nc = A->nr; T.nnz = A->nnz;
   int *cnt = (int *) gb_dcalloc(sizeof(int) * (size_t) (T.nr + 1));
   T.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (T.nr + 1));
   T.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (T.nnz ? T.nnz : 1));
   T.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (T.nnz ? T.nnz : 1));
   if (!cnt || !T.i || !T.j || !T.v) { return NULL; }
   gb_transpose_count(A->nnz, A->j, cnt, gb_stream());
   scan_total(cnt, T.i, T.nr);
   int *fill = (int *) gb_dmalloc(sizeof(int) * (size_t) (T.nr + 1));
   cudaMemcpyAsync(fill, T.i, sizeof(int) * (size_t) (T.nr + 1), cudaMemcpyDeviceToDevice, gb_stream());
   gb_transpose_fill(A->nr, T.nr, A->i, A->j, A->v, fill, T.i, T.j, T.v, gb_stream());
   gb_dfree(fill);
   gb_dfree(cnt);
   return gb_parcsr_wrap(T, 1);
}

/* --------------------------------------------------------------------------
 * Tiered drivers: shared-memory tables first, overflowing rows again with
 * global tables sized from the rows' upper bounds.
 * ------------------------------------------------------------------------ */
typedef struct
{
   int *ovf_list, *ovf_n, *err;
   int  h_ovf;
   int *gtab;
   int  gcap, gwarps;
} gb_tier;

/* one device flag for every tier of a setup: a table that overflows even its
 * last tier sets it; the setup reads it once at its end */
static int *g_tier_err = NULL;
/* the setup's SetupTables mode 1: every row of the ordered kernels in the
 * global-memory tier */
static int g_global_only = 0;

static void tier_begin(gb_tier *t, int nrows)
{
   memset(t, 0, sizeof(*t));
   t->ovf_list = (int *) gb_dmalloc(sizeof(int) * (size_t) (nrows > 0 ? nrows : 1));
   t->ovf_n = (int *) gb_dcalloc(sizeof(int) * 2);
   if (!g_tier_err) { g_tier_err = (int *) gb_dcalloc(sizeof(int) * 2); }
   t->err = g_tier_err;
}

/* after the symbolic shared-memory pass: read the overflow count and, if
 * needed, size the global tables from ub (device, nub entries) */
static void tier_global_n(gb_tier *t, const int *ub, int nub, int count)
{
   t->h_ovf = count;
   if (t->h_ovf <= 0) { return; }
   int m = max_of(ub, nub);
   t->gcap = next_pow2(2LL * (m + 1));
   size_t per = (size_t) 12 * (size_t) t->gcap;
   t->gwarps = slab_warps(per, t->h_ovf);
   t->gtab = (int *) gb_dmalloc(per * (size_t) t->gwarps);
   if (t->gtab) { cudaMemsetAsync(t->gtab, 0xff, per * (size_t) t->gwarps, gb_stream()); }
}

static void tier_global(gb_tier *t, const int *ub, int nub) { tier_global_n(t, ub, nub, read_int(t->ovf_n)); }

static int tier_end(gb_tier *t)
{
   gb_dfree(t->ovf_list); gb_dfree(t->ovf_n); gb_dfree(t->gtab);
   return 0;
}

/* the tiers' overflow flag, read (and cleared) once per setup */
static int tier_errors(void)
{
   if (!g_tier_err) { return 0; }
   int e = read_int(g_tier_err);
   if (e) { cudaMemsetAsync(g_tier_err, 0, sizeof(int), gb_stream()); }
   return e;
}

/* C = A B with hypre_ParMatmul's column order (square: diagonal first) */
/* algorithmic bytes and device time of the sparse products of the current
 * setup (CUDA events on the library stream around each product) */
static double g_sg_bytes, g_sg_seconds;
static int g_sg_calls;
#define GB_SG_EVENTS 96
static cudaEvent_t g_sg_ev[GB_SG_EVENTS][2];
static int g_sg_nev;

/* device time of the products recorded since the setup began (one sync) */
static void spgemm_times_collect(void)
{
   if (g_sg_nev == 0) { return; }
   cudaEventSynchronize(g_sg_ev[g_sg_nev - 1][1]);
   for (int k = 0; k < g_sg_nev; k++)
   {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, g_sg_ev[k][0], g_sg_ev[k][1]);
      g_sg_seconds += ms * 1e-3;
   }
   g_sg_nev = 0;
}

static double csr_bytes(const gb_csr *M) { return 12.0 * (double) M->nnz + 4.0 * ((double) M->nr + 1.0); }

static int spgemm_host_inner(const gb_csr *A, const gb_csr *B, int square, gb_csr *C);

static int spgemm_host(const gb_csr *A, const gb_csr *B, int square, gb_csr *C)
{
   cudaStream_t s = gb_stream();
   if (g_sg_nev == GB_SG_EVENTS) { spgemm_times_collect(); }
   const int k = g_sg_nev++;
   if (!g_sg_ev[k][0]) { cudaEventCreate(&g_sg_ev[k][0]); cudaEventCreate(&g_sg_ev[k][1]); }
   cudaEventRecord(g_sg_ev[k][0], s);
   int r = spgemm_host_inner(A, B, square, C);
   cudaEventRecord(g_sg_ev[k][1], s);
   if (r == 0)
   {
      g_sg_bytes += csr_bytes(A) + csr_bytes(B) + csr_bytes(C);
      g_sg_calls++;
   }
   return r;
}

/* Sparse product with one counting-and-filling pass per shared-memory tier
 * (gb_spgemm / gb_spgemm_rc phase 2): each row goes to a temporary area
 * sized by its product count (capped by the tier-0 table; rows that may
 * overflow it get a tier-1 area), the row counts are scanned into C's row
 * pointers and a gather moves the rows into place.  Rows beyond tier 1 take
 * the global-table tier's two passes.  Returns -2 when the temporary areas
 * would exceed 2^31 entries (the caller runs the two-pass driver). */
#define GB_SPGEMM_LCAP0 768
#define GB_SPGEMM_LCAP1 1536
static int spgemm_fused(const gb_csr *A, const gb_csr *B, int square, gb_csr *C, int rowchunk)
{
   cudaStream_t s = gb_stream();
   int n = A->nr;
   int *ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (n > 0 ? n : 1));
   int *cap = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *over = (int *) gb_dcalloc(sizeof(int) * 2);
   unsigned long long *sum = (unsigned long long *) gb_dcalloc(sizeof(unsigned long long));
   if (!ub || !cap || !over || !sum) { gb_dfree(ub); gb_dfree(cap); gb_dfree(over); gb_dfree(sum); return -1; }
   gb_spgemm_cap(n, B->nc, square, A->i, A->j, B->i, GB_SPGEMM_LCAP0, ub, cap, sum, over, s);
   unsigned long long hsum = 0;
   cudaMemcpyAsync(&hsum, sum, sizeof(hsum), cudaMemcpyDeviceToHost, s);
   int hover = read_int(over);
   gb_dfree(sum); gb_dfree(over);
   long long tot = (long long) hsum + (long long) hover * GB_SPGEMM_LCAP1;
   if (tot > 0x7fffff00LL) { gb_dfree(ub); gb_dfree(cap); return -2; }
   int *tofs = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *tj = (int *) gb_dmalloc(sizeof(int) * (size_t) (tot > 0 ? tot : 1));
   double *tv = (double *) gb_dmalloc(sizeof(double) * (size_t) (tot > 0 ? tot : 1));
   int *src = (int *) gb_dmalloc(sizeof(int) * (size_t) (n > 0 ? n : 1));
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *list2 = NULL, *n2 = (int *) gb_dcalloc(sizeof(int) * 2);
   if (!tofs || !tj || !tv || !src || !cnt || !n2)
   {
      gb_dfree(ub); gb_dfree(cap); gb_dfree(tofs); gb_dfree(tj); gb_dfree(tv); gb_dfree(src); gb_dfree(cnt);
      gb_dfree(n2);
      return -1;
   }
   scan_total(cap, tofs, n);
   gb_dfree(cap);
   gb_tier t;
   tier_begin(&t, n);
   /* tier 0 over every row: areas at tofs[r] */
   if (rowchunk)
   {
      gb_spgemm_rc(n, square, A->i, A->j, A->v, B->i, B->j, B->v, cnt, tofs, tj, tv, t.ovf_list, t.ovf_n, NULL,
                   NULL, n, t.err, ub, src, 0, 2, 0, s);
   }
   else
   {
      gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, tofs, tj, tv, t.ovf_list, t.ovf_n, NULL,
                NULL, n, NULL, 0, 0, t.err, ub, src, 0, 2, 0, s);
   }
   /* tier 1 over the rows that did not fit, in row order: areas of 1536
    * entries after the tier-0 ones.  The list's length stays on the device
    * (the kernels read it); hover bounds it. */
   int h2 = 0;
   if (hover > 0)
   {
      sort_row_list_n(t.ovf_list, hover, t.ovf_n, n);
      list2 = (int *) gb_dmalloc(sizeof(int) * (size_t) hover);
      if (rowchunk)
      {
         gb_spgemm_rc(n, square, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, tj, tv, t.ovf_list, t.ovf_n, list2,
                      n2, hover, t.err, NULL, src, (int) hsum, 2, 1, s);
      }
      else
      {
         gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, tj, tv, t.ovf_list, t.ovf_n, list2,
                   n2, hover, NULL, 0, 0, t.err, NULL, src, (int) hsum, 2, 1, s);
      }
   }
   /* row pointers; the row total and the global tier's row count come back
    * together */
   C->nr = n; C->nc = B->nc;
   C->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   {
      int *scr = (int *) gb_scratch(0, sizeof(int) * (size_t) gb_scan_scratch_ints(n > 0 ? n : 1));
      gb_exclusive_scan(cnt, C->i, n, scr, s);
      int two[2] = {0, 0};
      cudaMemcpyAsync(&two[0], C->i + n, sizeof(int), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(&two[1], n2, sizeof(int), cudaMemcpyDeviceToHost, s);
      gb_sync();
      C->nnz = two[0];
      h2 = two[1];
   }
   if (h2 > 0)
   {
      /* rows beyond tier 1: global tables, count, then the row pointers again */
      tier_global_n(&t, ub, n, h2);
      gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, list2, n2, NULL, NULL, h2,
                t.gtab, t.gcap, t.gwarps, t.err, NULL, NULL, 0, 0, 2, s);
      C->nnz = scan_total(cnt, C->i, n);
   }
   C->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (C->nnz ? C->nnz : 1));
   C->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (C->nnz ? C->nnz : 1));
   gb_spgemm_gather(n, C->nnz, C->i, src, tj, tv, C->j, C->v, s);
   if (h2 > 0)
   {
      gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, list2, n2, NULL, NULL, h2,
                t.gtab, t.gcap, t.gwarps, t.err, NULL, NULL, 0, 1, 2, s);
   }
   int e = tier_end(&t);
   gb_dfree(ub); gb_dfree(tofs); gb_dfree(tj); gb_dfree(tv); gb_dfree(src); gb_dfree(cnt); gb_dfree(list2);
   gb_dfree(n2);
   if (e) { gb_error(HYPRE_ERROR_GENERIC, "sparse product table overflow"); return -1; }
   return 0;
}

/* every row in global-memory tables (count, then fill) */
static int spgemm_global(const gb_csr *A, const gb_csr *B, int square, gb_csr *C)
{
   cudaStream_t s = gb_stream();
   int n = A->nr;
   int *ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (n > 0 ? n : 1));
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_tier t;
   tier_begin(&t, n);
   gb_spgemm_ub(n, B->nc, square, A->i, A->j, B->i, ub, s);
   gb_iota(n, t.ovf_list, t.ovf_n, s);
   tier_global_n(&t, ub, n, n);
   if (n > 0)
   {
      gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, t.ovf_list, t.ovf_n, NULL,
                NULL, n, t.gtab, t.gcap, t.gwarps, t.err, NULL, NULL, 0, 0, 2, s);
   }
   C->nr = n; C->nc = B->nc;
   C->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   C->nnz = scan_total(cnt, C->i, n);
   C->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (C->nnz ? C->nnz : 1));
   C->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (C->nnz ? C->nnz : 1));
   if (n > 0)
   {
      gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, t.ovf_list, t.ovf_n, NULL,
                NULL, n, t.gtab, t.gcap, t.gwarps, t.err, NULL, NULL, 0, 1, 2, s);
   }
   tier_end(&t);
   gb_dfree(ub); gb_dfree(cnt);
   return 0;
}

static int spgemm_host_inner(const gb_csr *A, const gb_csr *B, int square, gb_csr *C)
{
   cudaStream_t s = gb_stream();
   if (g_global_only) { return spgemm_global(A, B, square, C); }
   {
      const int rc = B->nr > 0 && (long long) B->nnz >= 12LL * (long long) B->nr;
      int f = spgemm_fused(A, B, square, C, rc);
      if (f != -2) { return f; }
   }
   int n = A->nr;
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_tier t;
   tier_begin(&t, n);
   int *list2 = NULL, *n2 = (int *) gb_dcalloc(sizeof(int) * 2);
   const int W = 0;   /* no rows skipped by the tier-0 numeric pass */
   int *ub = NULL;
   /* B rows of a dozen entries or more: one B-row chunk per warp step
    * (gb_spgemm_rc); short B rows: products flattened 32 per step */
   const int rowchunk = B->nr > 0 && (long long) B->nnz >= 12LL * (long long) B->nr;
   if (rowchunk)
   {
      /* rows with far more products than a 1024-slot table holds skip
       * tier 0 (they are the long rows of R*A) */
      ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (n > 0 ? n : 1));
      gb_spgemm_ub(n, B->nc, square, A->i, A->j, B->i, ub, s);
   }
   /* symbolic: small shared tables, then compact shared tables for the rows
    * that did not fit, then global tables for the rest.  (Routing rows of
    * the flattened kernel by an upper bound of their length was measured
    * slower: the product count is a poor bound for rows of RA*P, which then
    * leave the fast tier.) */
   if (rowchunk)
   {
      gb_spgemm_rc(n, square, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, t.ovf_list, t.ovf_n, NULL,
                   NULL, n, t.err, ub, NULL, 0, 0, 0, s);
   }
   else
   {
      gb_spgemm(n, square, W, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, t.ovf_list, t.ovf_n, NULL,
                NULL, n, NULL, 0, 0, t.err, NULL, NULL, 0, 0, 0, s);
   }
   int h1 = read_int(t.ovf_n), h2 = 0;
   if (h1 > 0)
   {
      sort_row_list(t.ovf_list, h1, n);
      list2 = (int *) gb_dmalloc(sizeof(int) * (size_t) h1);
      if (rowchunk)
      {
         gb_spgemm_rc(n, square, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, t.ovf_list, t.ovf_n,
                      list2, n2, h1, t.err, NULL, NULL, 0, 0, 1, s);
      }
      else
      {
         gb_spgemm(n, square, W, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, t.ovf_list, t.ovf_n,
                   list2, n2, h1, NULL, 0, 0, t.err, NULL, NULL, 0, 0, 1, s);
      }
      h2 = read_int(n2);
   }
   if (h2 > 0)
   {
      /* global tables for the rows of the second list, sized from upper bounds */
      if (!ub)
      {
         ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (n > 0 ? n : 1));
         gb_spgemm_ub(n, B->nc, square, A->i, A->j, B->i, ub, s);
      }
      tier_global_n(&t, ub, n, h2);
      gb_spgemm(n, square, W, A->i, A->j, A->v, B->i, B->j, B->v, cnt, NULL, NULL, NULL, list2, n2, NULL, NULL, h2,
                t.gtab, t.gcap, t.gwarps, t.err, NULL, NULL, 0, 0, 2, s);
   }
   C->nr = n; C->nc = B->nc;
   C->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   C->nnz = scan_total(cnt, C->i, n);
   C->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (C->nnz ? C->nnz : 1));
   C->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (C->nnz ? C->nnz : 1));
   /* numeric: the same three tiers (each skips rows longer than its tables) */
   if (rowchunk)
   {
      gb_spgemm_rc(n, square, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, t.ovf_list, t.ovf_n, NULL,
                   NULL, n, t.err, NULL, NULL, 0, 1, 0, s);
      if (h1 > 0)
      {
         gb_spgemm_rc(n, square, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, t.ovf_list, t.ovf_n,
                      NULL, NULL, h1, t.err, NULL, NULL, 0, 1, 1, s);
      }
   }
   else
   {
      /* many products per row (RA*P): rows of at most 192 columns accumulate
       * in shared memory (tier 3), the longer ones in tier 0; few products
       * per row (FF*FC, P1*P2): tier 0 alone, where the fixed cost per row
       * is lower */
      const double prods = ((double) A->nnz / (A->nr > 0 ? A->nr : 1)) * ((double) B->nnz / (B->nr > 0 ? B->nr : 1));
      int skip = 0;
      if (prods >= 512.0)
      {
         gb_spgemm(n, square, 0, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, t.ovf_list, t.ovf_n,
                   NULL, NULL, n, NULL, 0, 0, t.err, NULL, NULL, 0, 1, 3, s);
         skip = GB_SPGEMM_TINY_COLS;
      }
      gb_spgemm(n, square, skip, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, t.ovf_list, t.ovf_n,
                NULL, NULL, n, NULL, 0, 0, t.err, NULL, NULL, 0, 1, 0, s);
      if (h1 > 0)
      {
         gb_spgemm(n, square, W, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, t.ovf_list, t.ovf_n,
                   NULL, NULL, h1, NULL, 0, 0, t.err, NULL, NULL, 0, 1, 1, s);
      }
   }
   if (h2 > 0)
   {
      gb_spgemm(n, square, W, A->i, A->j, A->v, B->i, B->j, B->v, cnt, C->i, C->j, C->v, list2, n2, NULL, NULL, h2,
                t.gtab, t.gcap, t.gwarps, t.err, NULL, NULL, 0, 1, 2, s);
   }
   int e = tier_end(&t);
   gb_dfree(ub); gb_dfree(cnt); gb_dfree(list2); gb_dfree(n2);
   if (e) { gb_error(HYPRE_ERROR_GENERIC, "sparse product table overflow"); return -1; }
   return 0;
}

/* --------------------------------------------------------------------------
 * C = A * B (HYPRE_ParCSRMatrixMatmat, src/parcsr_mv/HYPRE_parcsr_matrix.c:457
 * -> hypre_ParCSRMatMatHost, src/parcsr_mv/par_csr_triplemat.c:20 ->
 * hypre_CSRMatrixMultiplyHost, src/seq_mv/csr_matop.c:693 on one process).
 * The reference's product: columns of each row in first-discovery order,
 * each entry's terms summed in product order; when C is square and A has no
 * empty rows (A's row-nonzero list is unset) every row starts with its
 * diagonal, stored as 0 and then summed into; an empty A or B gives an empty
 * C.  The ordered sparse-product kernels of the setup compute it.
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_ParCSRMatrixMatmat(HYPRE_ParCSRMatrix A, HYPRE_ParCSRMatrix B, HYPRE_ParCSRMatrix *C)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(1); return gb_error_flag; }
   if (!B || B->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   if (!C) { gb_error_in_arg(3); return gb_error_flag; }
   *C = NULL;
   if (A->A.nc != B->A.nr)
   {
      gb_error(HYPRE_ERROR_ARG, "Matmat: incompatible matrix dimensions");
      gb_error_in_arg(1);
      return gb_error_flag;
   }
   gb_csr P;
   memset(&P, 0, sizeof(P));
   if (A->A.nnz == 0 || B->A.nnz == 0)
   {
      P.nr = A->A.nr; P.nc = B->A.nc; P.nnz = 0;
      P.i = (int *) gb_dcalloc(sizeof(int) * (size_t) (P.nr + 1));
      P.j = (int *) gb_dmalloc(sizeof(int));
      P.v = (double *) gb_dmalloc(sizeof(double));
      if (!P.i || !P.j || !P.v) { gb_dfree(P.i); gb_dfree(P.j); gb_dfree(P.v); return gb_error_flag; }
   }
   else
   {
      int square = A->A.nr == B->A.nc;
      if (square)
      {
         int *empty = (int *) gb_dcalloc(sizeof(int));
         if (!empty) { return gb_error_flag; }
         gb_count_empty_rows(A->A.nr, A->A.i, empty, gb_stream());
         square = read_int(empty) == 0;
         gb_dfree(empty);
      }
      if (spgemm_host_inner(&A->A, &B->A, square, &P) != 0) { return gb_error_flag; }
   }
   gb_parcsr *out = gb_parcsr_wrap(P, 1);
   if (!out) { gb_dfree(P.i); gb_dfree(P.j); gb_dfree(P.v); return gb_error_flag; }
   *C = out;
   return gb_error_flag;
}

/* extended+i rows for fine points rows[r] (all points when rows == NULL);
 * iterm 0 gives the extended interpolation (interp_type 14,
 * hypre_BoomerAMGBuildExtInterpHost src/parcsr_ls/par_lr_interp.c:4777),
 * whose distribution leaves the point itself out of the sums and of the
 * diagonal (par_lr_interp.c:5279-5325 against :1649-1700).
 * Tier 0: one thread per row (rows with <= 64 candidates); tier 1: one warp
 * per row with shared-memory tables; tier 2: global-memory tables. */
static int extpi_host(const gb_csr *A, const gb_csr *S, const int *CF, const int *f2c, int nrows, const int *rows,
                      int ncols, int iterm, gb_csr *P)
{
   cudaStream_t s = gb_stream();
   int n = A->nr;
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (nrows + 1));
   int *l1 = (int *) gb_dmalloc(sizeof(int) * (size_t) (nrows > 0 ? nrows : 1));
   int *n1 = (int *) gb_dcalloc(sizeof(int) * 2);
   gb_tier t;
   tier_begin(&t, nrows);
   /* thread-per-row: the FP64 sums of 32 rows share each warp instruction
    * (FP64 issue is scarce on this GPU), but only large levels have enough
    * rows to keep the SMs busy (on the 57k-row second level of a 160^3
    * 27-point problem it took 5.1 ms against 1.5 ms for the warp kernels) */
   int use_thread = nrows >= 65536 && ncols < (1 << 25) && !g_global_only;
   int h1;
   if (use_thread)
   {
      gb_extpi_count_t(nrows, rows, S->i, S->j, CF, f2c, cnt, l1, n1, s);
      h1 = read_int(n1);
   }
   else
   {
      gb_iota(nrows, l1, n1, s);
      h1 = nrows;
   }
   int *ub = NULL;
   if (h1 > 0)
   {
      if (g_global_only) { gb_iota(nrows, t.ovf_list, t.ovf_n, s); }
      else
      {
         gb_extpi_count(nrows, rows, S->i, S->j, CF, cnt, l1, n1, h1, t.ovf_list, t.ovf_n, NULL, 0, 0, t.err, 1,
                        s);
      }
      if (read_int(t.ovf_n) > 0)
      {
         ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (n > 0 ? n : 1));
         gb_extpi_ub(n, S->i, S->j, CF, ub, s);
      }
      tier_global(&t, ub, n);
      if (t.h_ovf > 0)
      {
         gb_extpi_count(nrows, rows, S->i, S->j, CF, cnt, t.ovf_list, t.ovf_n, t.h_ovf, NULL, NULL, t.gtab, t.gcap,
                        t.gwarps, t.err, 2, s);
      }
   }
   P->nr = nrows; P->nc = ncols;
   P->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (nrows + 1));
   P->nnz = scan_total(cnt, P->i, nrows);
   P->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (P->nnz ? P->nnz : 1));
   P->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (P->nnz ? P->nnz : 1));
   if (use_thread) { gb_extpi_fill_t(nrows, rows, A->i, A->j, A->v, S->i, S->j, CF, f2c, P->i, P->j, P->v, iterm, s); }
   if (h1 > 0)
   {
      if (!g_global_only)
      {
         gb_extpi_fill(nrows, rows, A->i, A->j, A->v, S->i, S->j, CF, f2c, P->i, P->j, P->v, l1, n1, h1, NULL, 0, 0,
                       t.err, 1, iterm, s);
      }
      if (t.h_ovf > 0)
      {
         gb_extpi_fill(nrows, rows, A->i, A->j, A->v, S->i, S->j, CF, f2c, P->i, P->j, P->v, t.ovf_list, t.ovf_n,
                       t.h_ovf, t.gtab, t.gcap, t.gwarps, t.err, 2, iterm, s);
      }
   }
   int e = tier_end(&t);
   gb_dfree(ub); gb_dfree(cnt); gb_dfree(l1); gb_dfree(n1);
   if (e) { gb_error(HYPRE_ERROR_GENERIC, "interpolation table overflow"); return -1; }
   return 0;
}

/* truncation by tolerance / max elements (par_csr_matrix.c:2943) in place */
static void truncate_host(gb_csr *P, double tol, int max_elmts)
{
   if (!(tol > 0.0 || max_elmts > 0)) { return; }
   cudaStream_t s = gb_stream();
   int n = P->nr;
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_truncate_rows(n, P->i, P->j, P->v, tol, max_elmts, cnt, s);
   int *Ni = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int nnz2 = scan_total(cnt, Ni, n);
   int *Nj = (int *) gb_dmalloc(sizeof(int) * (size_t) (nnz2 ? nnz2 : 1));
   double *Nv = (double *) gb_dmalloc(sizeof(double) * (size_t) (nnz2 ? nnz2 : 1));
   gb_compact_rows(n, P->i, P->j, P->v, Ni, Nj, Nv, s);
   gb_dfree(P->i); gb_dfree(P->j); gb_dfree(P->v);
   P->i = Ni; P->j = Nj; P->v = Nv; P->nnz = nnz2;
   gb_dfree(cnt);
}

/* scanned flag numbering: out[i] = number of flagged points before i; list (optional) */
static int number_points(int n, const int *CF, int kind, int v, int *out, int **list)
{
   cudaStream_t s = gb_stream();
   int *flag = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_flags(n, CF, kind, v, flag, s);
   int tot = scan_total(flag, out, n);
   if (list)
   {
      *list = (int *) gb_dmalloc(sizeof(int) * (size_t) (tot > 0 ? tot : 1));
      gb_scatter_list(n, flag, out, *list, s);
   }
   gb_dfree(flag);
   return tot;
}

/* direct interpolation (interp_type 3, par_interp.c:1873); not truncated here */
static int dir_interp(const gb_csr *A, const gb_csr *S, const int *CF, const int *f2c, int nc, gb_csr *P)
{
   cudaStream_t s = gb_stream();
   int n = A->nr;
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_dir_count(n, S->i, S->j, CF, cnt, s);
   P->nr = n; P->nc = nc;
   P->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   P->nnz = scan_total(cnt, P->i, n);
   P->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (P->nnz ? P->nnz : 1));
   P->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (P->nnz ? P->nnz : 1));
   size_t nb = sizeof(double) * (size_t) (n ? n : 1);
   double *alfa = (double *) gb_dmalloc(nb), *beta = (double *) gb_dmalloc(nb);
   if (!cnt || !P->i || !P->j || !P->v || !alfa || !beta)
   {
      gb_dfree(cnt); gb_dfree(alfa); gb_dfree(beta);
      return -1;
   }
   gb_dir_fill(n, A->i, A->j, A->v, S->i, S->j, CF, f2c, P->i, P->j, P->v, alfa, beta, cnt, s);
   gb_dfree(cnt); gb_dfree(alfa); gb_dfree(beta);
   return 0;
}

/* The modified ("MM") interpolations, P = [I; W] with W = As_FF As_FC
 * (hypre_BoomerAMGBuildModExtInterpHost / ModExtPIInterpHost /
 * ModExtPEInterpHost, src/parcsr_ls/par_mod_lr_interp.c:16, :585, :1260;
 * As_FF / As_FC from hypre_ParCSRMatrixGenerateFFFCHost, src/parcsr_mv/
 * gen_fffc.c:18): variant 16 extended, 17 extended+i, 18 extended+e.  CF:
 * C points > 0; f2c: coarse numbers of the C points (nc of them).  P is not
 * truncated here. */
static int mm_interp(const gb_csr *A, const gb_csr *S, const int *CF, const int *f2c, int nc, int variant,
                     gb_csr *P)
{
   cudaStream_t s = gb_stream();
   int n = A->nr;
   int *f2f = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *fl = NULL;
   int nf = number_points(n, CF, 2, 0, f2f, &fl);
   gb_csr FF, FC;
   FF.nr = FF.nc = nf; FC.nr = nf; FC.nc = nc;
   int *cff = (int *) gb_dmalloc(sizeof(int) * (size_t) (nf + 1));
   int *cfc = (int *) gb_dmalloc(sizeof(int) * (size_t) (nf + 1));
   gb_fffc_count(nf, fl, A->i, A->j, S->i, S->j, CF, cff, cfc, s);
   FF.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (nf + 1));
   FC.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (nf + 1));
   FF.nnz = scan_total(cff, FF.i, nf);
   FC.nnz = scan_total(cfc, FC.i, nf);
   FF.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (FF.nnz ? FF.nnz : 1));
   FF.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (FF.nnz ? FF.nnz : 1));
   FC.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (FC.nnz ? FC.nnz : 1));
   FC.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (FC.nnz ? FC.nnz : 1));
   gb_fffc_fill(nf, n, A->nnz, fl, A->i, A->j, A->v, S->i, S->j, CF, f2c, f2f, FF.i, FF.j, FF.v, FC.i, FC.j, FC.v,
                s);
   {
      double *tmp = (double *) gb_dmalloc(sizeof(double) * (size_t) (FF.nnz ? FF.nnz : 1));
      size_t nb = sizeof(double) * (size_t) (nf ? nf : 1);
      double *D1 = (double *) gb_dmalloc(nb), *D2 = (double *) gb_dmalloc(nb);
      double *D3 = (double *) gb_dmalloc(nb), *D4 = (double *) gb_dmalloc(nb);
      gb_mod_interp_scale(variant, nf, FF.nnz, fl, A->i, A->v, FF.i, FF.j, FF.v, FC.i, FC.v, tmp, D1, D2, D3, D4, s);
      gb_dfree(tmp); gb_dfree(D1); gb_dfree(D2); gb_dfree(D3); gb_dfree(D4);
   }
   gb_csr W;
   if (spgemm_host(&FF, &FC, nf == nc, &W)) { return -1; }
   gb_csr_free(&FF); gb_csr_free(&FC);
   P->nr = n; P->nc = nc;
   int *len = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_p1_len(n, CF, f2f, W.i, len, s);
   P->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   P->nnz = scan_total(len, P->i, n);
   P->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (P->nnz ? P->nnz : 1));
   P->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (P->nnz ? P->nnz : 1));
   gb_p1_fill(n, CF, f2c, f2f, W.i, W.j, W.v, P->i, P->j, P->v, s);
   gb_csr_free(&W);
   gb_dfree(f2f); gb_dfree(fl); gb_dfree(cff); gb_dfree(cfc); gb_dfree(len);
   return 0;
}

/* multipass interpolation (agg_interp_type 4, par_multi_interp.c:16-2130)
 * after the C/F correction by the second coarsening (CFN, numbered by f2c1
 * over the CF > 0 points; par_strength.c:3068-3090), truncated with
 * (agg_trunc_factor, agg_P_max_elmts).  Returns the number of coarse points. */
static int multipass_interp(const gb_amg_params *prm, const gb_csr *A, const gb_csr *S, int *CF, const int *f2c1,
                            const int *CFN, gb_csr *P)
{
   cudaStream_t s = gb_stream();
   const int n = A->nr;
   gb_correct_cf(n, f2c1, CFN, CF, s);
   int *f2c = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   const int nc = number_points(n, CF, 1, 1, f2c, NULL);
   int *fscan = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *fl = NULL;
   const int nf = number_points(n, CF, 1, -1, fscan, &fl);
   gb_dfree(fscan);
   size_t ni = sizeof(int) * (size_t) (n ? n : 1);
   int *assigned = (int *) gb_dmalloc(ni), *rowoff = (int *) gb_dcalloc(ni), *rowlen = (int *) gb_dcalloc(ni);
   int *degen = (int *) gb_dcalloc(ni);
   double *alfa = (double *) gb_dmalloc(sizeof(double) * (size_t) (n ? n : 1));
   int *dcnt = (int *) gb_dcalloc(sizeof(int) * 2);
   unsigned long long *dtot = (unsigned long long *) gb_dcalloc(sizeof(unsigned long long));
   gb_mp_areas areas;
   memset(&areas, 0, sizeof(areas));
   int rc = -1;
   if (!f2c || !assigned || !rowoff || !rowlen || !degen || !alfa || !dcnt || !dtot) { goto done; }
   /* passes: breadth-first distance from the C points in S (< 10) */
   gb_mp_pass(n, S->i, S->j, CF, 1, assigned, dcnt, s);
   int remaining = nf - read_int(dcnt);
   int np = 2;                                   /* rows of passes 1 .. np-1 */
   while (remaining > 0 && np < GB_MP_MAXP)
   {
      cudaMemsetAsync(dcnt, 0, sizeof(int), s);
      gb_mp_pass(n, S->i, S->j, CF, np, assigned, dcnt, s);
      int c = read_int(dcnt);
      if (c == 0) { break; }                    /* later passes would find none */
      remaining -= c;
      np++;
   }
   /* the rows, pass by pass */
   for (int p = 1; p < np; p++)
   {
      int *pscan = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      int *rows = NULL;
      const int m = number_points(n, assigned, 1, p, pscan, &rows);
      gb_dfree(pscan);
      int *ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (m + 1));
      int *off = (int *) gb_dmalloc(sizeof(int) * (size_t) (m + 1));
      cudaMemsetAsync(dtot, 0, sizeof(unsigned long long), s);
      gb_mp_bound(m, rows, S->i, S->j, assigned, p, rowlen, ub, dtot, s);
      unsigned long long tot = 0;
      cudaMemcpyAsync(&tot, dtot, sizeof(tot), cudaMemcpyDeviceToHost, s);
      gb_sync();
      if (tot > 0x7fffff00ULL)
      {
         gb_dfree(rows); gb_dfree(ub); gb_dfree(off);
         gb_error(HYPRE_ERROR_MEMORY, "multipass interpolation: rows of a pass");
         goto done;
      }
      scan_total(ub, off, m);
      areas.j[p] = (int *) gb_dmalloc(sizeof(int) * (size_t) (tot ? tot : 1));
      areas.v[p] = (double *) gb_dmalloc(sizeof(double) * (size_t) (tot ? tot : 1));
      cudaMemsetAsync(dcnt, 0, sizeof(int), s);
      gb_mp_rows(m, rows, off, p, A->i, A->j, A->v, S->i, S->j, CF, f2c, assigned, areas.j[p - 1],
                 areas.v[p - 1], areas.j[p], areas.v[p], rowoff, rowlen, alfa, degen, dcnt, s);
      if (p == 1 && read_int(dcnt) > 0)
      {
         gb_mp_carry1(nf, fl, assigned, degen, alfa, rowoff, rowlen, areas.v[1], s);
      }
      gb_dfree(rows); gb_dfree(ub); gb_dfree(off);
   }
   {
      int *len = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      gb_mp_len(n, CF, assigned, rowlen, len, s);
      P->nr = n; P->nc = nc;
      P->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      P->nnz = scan_total(len, P->i, n);
      P->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (P->nnz ? P->nnz : 1));
      P->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (P->nnz ? P->nnz : 1));
      gb_mp_gather(n, CF, assigned, f2c, rowoff, &areas, P->i, P->j, P->v, s);
      gb_dfree(len);
   }
   truncate_host(P, prm->agg_trunc_factor, prm->agg_p_max_elmts);
   gb_sf_to_f(n, CF, s);
   rc = nc;
done:
   gb_sync();
   for (int p = 0; p < GB_MP_MAXP; p++) { gb_dfree(areas.j[p]); gb_dfree(areas.v[p]); }
   gb_dfree(f2c); gb_dfree(fl); gb_dfree(assigned); gb_dfree(rowoff); gb_dfree(rowlen); gb_dfree(degen);
   gb_dfree(alfa); gb_dfree(dcnt); gb_dfree(dtot);
   return rc;
}

/* an empty CSR block with nc columns */
static void csr_empty(gb_csr *M, int nc)
{
   memset(M, 0, sizeof(*M));
   M->nc = nc;
   M->i = (int *) gb_dcalloc(sizeof(int));
   M->j = (int *) gb_dmalloc(sizeof(int));
   M->v = (double *) gb_dmalloc(sizeof(double));
}

/* the modified partial interpolations of the second stage (agg_interp_type
 * 5 and 7; par_2s_interp.c:15-620, :662-1320): the F/C blocks of every non-C
 * point (FC, and FF for D_lambda) and of the CF -2 points (FF), the D
 * scalings, W = FF FC (hypre_ParMatmul), P over the old C points in row order
 * (CF 1 identity, CF -2 the row of W); f2c / nc number the new C points */
static int mm_partial_interp(const gb_csr *A, const gb_csr *S, const int *CF, const int *f2c, int nc, int variant,
                             gb_csr *P)
{
   cudaStream_t s = gb_stream();
   const int n = A->nr;
   int *f2f = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *nscan = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *fl = NULL, *nl = NULL;
   const int nf = number_points(n, CF, 2, 0, f2f, &fl);
   const int nn = number_points(n, CF, 1, -2, nscan, &nl);
   /* blocks over a row list: FF (diagonal first) and FC */
   gb_csr FF[2], FC[2];
   const int m[2] = {nf, nn};
   const int *lst[2] = {fl, nl};
   for (int b = 0; b < 2; b++)
   {
      const int r = m[b];
      memset(&FF[b], 0, sizeof(gb_csr));
      memset(&FC[b], 0, sizeof(gb_csr));
      FF[b].nr = r; FF[b].nc = nf; FC[b].nr = r; FC[b].nc = nc;
      int *cff = (int *) gb_dmalloc(sizeof(int) * (size_t) (r + 1));
      int *cfc = (int *) gb_dmalloc(sizeof(int) * (size_t) (r + 1));
      if (r > 0) { gb_fffc_count(r, lst[b], A->i, A->j, S->i, S->j, CF, cff, cfc, s); }
      FF[b].i = (int *) gb_dmalloc(sizeof(int) * (size_t) (r + 1));
      FC[b].i = (int *) gb_dmalloc(sizeof(int) * (size_t) (r + 1));
      FF[b].nnz = scan_total(cff, FF[b].i, r);
      FC[b].nnz = scan_total(cfc, FC[b].i, r);
      gb_dfree(cff); gb_dfree(cfc);
      FF[b].j = (int *) gb_dmalloc(sizeof(int) * (size_t) (FF[b].nnz ? FF[b].nnz : 1));
      FF[b].v = (double *) gb_dmalloc(sizeof(double) * (size_t) (FF[b].nnz ? FF[b].nnz : 1));
      FC[b].j = (int *) gb_dmalloc(sizeof(int) * (size_t) (FC[b].nnz ? FC[b].nnz : 1));
      FC[b].v = (double *) gb_dmalloc(sizeof(double) * (size_t) (FC[b].nnz ? FC[b].nnz : 1));
      if (r > 0)
      {
         gb_fffc_fill(r, n, A->nnz, lst[b], A->i, A->j, A->v, S->i, S->j, CF, f2c, f2f, FF[b].i, FF[b].j, FF[b].v,
                      FC[b].i, FC[b].j, FC[b].v, s);
      }
   }
   {
      const size_t nb = sizeof(double) * (size_t) (nf ? nf : 1);
      double *Dq = (double *) gb_dmalloc(nb), *Dl = (double *) gb_dmalloc(nb), *Dinv = (double *) gb_dmalloc(nb);
      gb_modp_scale(variant, nf, nn, nl, f2f, A->i, A->v, FF[0].i, FF[0].v, FC[0].i, FC[0].v, FF[1].i, FF[1].j,
                    FF[1].v, Dq, Dl, Dinv, s);
      gb_dfree(Dq); gb_dfree(Dl); gb_dfree(Dinv);
   }
   gb_csr W;
   int rc = -1;
   if (nn == 0) { csr_empty(&W, nc); }
   else if (spgemm_host(&FF[1], &FC[0], nn == nc, &W)) { goto done; }
   {
      int *oscan = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      int *oc = NULL;
      int *flag = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      gb_flags(n, CF, 3, -2, flag, s);
      const int nco = scan_total(flag, oscan, n);
      oc = (int *) gb_dmalloc(sizeof(int) * (size_t) (nco > 0 ? nco : 1));
      gb_scatter_list(n, flag, oscan, oc, s);
      gb_dfree(flag); gb_dfree(oscan);
      int *len = (int *) gb_dmalloc(sizeof(int) * (size_t) (nco + 1));
      gb_modp_len(nco, oc, CF, nscan, W.i, len, s);
      P->nr = nco; P->nc = nc;
      P->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (nco + 1));
      P->nnz = scan_total(len, P->i, nco);
      P->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (P->nnz ? P->nnz : 1));
      P->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (P->nnz ? P->nnz : 1));
      gb_modp_gather(nco, oc, CF, f2c, nscan, W.i, W.j, W.v, P->i, P->j, P->v, s);
      gb_dfree(len); gb_dfree(oc);
   }
   gb_csr_free(&W);
   rc = 0;
done:
   for (int b = 0; b < 2; b++) { gb_csr_free(&FF[b]); gb_csr_free(&FC[b]); }
   gb_dfree(f2f); gb_dfree(nscan); gb_dfree(fl); gb_dfree(nl);
   return rc;
}

/* multipass interpolation in product form (agg_interp_type 8 and 9,
 * par_mod_multi_interp.c:17-525) after the C/F correction by the second
 * coarsening: passes by rounds (C points 1; a point left takes pass p+1 in
 * the round that finds a strong neighbour of pass p; more than 9 passes is an
 * error), one block of rows per pass (pass 2 from the C points; later passes
 * a sparse product with the previous block), P assembled from the blocks and
 * truncated with (agg_trunc_factor, agg_P_max_elmts).  Returns the number of
 * coarse points. */
static int mod_multipass_interp(const gb_amg_params *prm, const gb_csr *A, const gb_csr *S, int *CF, const int *f2c1,
                                const int *CFN, gb_csr *P)
{
   cudaStream_t s = gb_stream();
   const int n = A->nr, type = prm->agg_interp_type;
   gb_correct_cf(n, f2c1, CFN, CF, s);
   const size_t ni = sizeof(int) * (size_t) (n ? n : 1);
   int *pass = (int *) gb_dmalloc(ni), *col = (int *) gb_dmalloc(ni);
   int *dcnt = (int *) gb_dcalloc(sizeof(int));
   double *rsum = (double *) gb_dmalloc(sizeof(double) * (size_t) (n ? n : 1));
   int *rows[GB_MMP_MAXB + 3];
   int cnt[GB_MMP_MAXB + 3];
   gb_csr B[GB_MMP_MAXB];
   memset(rows, 0, sizeof(rows));
   memset(cnt, 0, sizeof(cnt));
   memset(B, 0, sizeof(B));
   int nblk = 0, rc = -1;
   if (!pass || !col || !dcnt || !rsum) { goto done; }
   gb_mmp_init(n, CF, pass, dcnt, s);
   const int nc = read_int(dcnt);
   int remaining = n - nc, num_passes = 1;
   while (remaining > 0)
   {
      cudaMemsetAsync(dcnt, 0, sizeof(int), s);
      gb_mmp_round(n, S->i, S->j, num_passes, pass, dcnt, s);
      const int c = read_int(dcnt);
      remaining -= c;
      num_passes++;
      if (num_passes > 9)
      {
         gb_error(HYPRE_ERROR_GENERIC, "multipass interpolation: more than 9 passes");
         goto done;
      }
      if (c == 0) { break; }
   }
   for (int p = 1; p <= num_passes; p++)
   {
      int *scan = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      cnt[p] = number_points(n, pass, 1, p, scan, &rows[p]);
      gb_mmp_col(n, pass, p, scan, col, s);
      gb_dfree(scan);
   }
   gb_mmp_rowsum(n, CF, A->i, A->v, rsum, s);
   nblk = num_passes - 1;
   for (int b = 0; b < nblk; b++)
   {
      const int m = cnt[b + 2], color = b + 1;
      const int *rws = rows[b + 2];
      gb_csr Q;
      memset(&Q, 0, sizeof(Q));
      Q.nr = m;
      Q.nc = cnt[b + 1];
      Q.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (m + 1));
      int *qc = (int *) gb_dmalloc(sizeof(int) * (size_t) (m + 1));
      gb_mmp_count(m, rws, S->i, S->j, pass, color, qc, s);
      Q.nnz = scan_total(qc, Q.i, m);
      gb_dfree(qc);
      Q.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (Q.nnz ? Q.nnz : 1));
      Q.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (Q.nnz ? Q.nnz : 1));
      double *w = (type == 9 && b > 0) ? (double *) gb_dmalloc(sizeof(double) * (size_t) (m ? m : 1)) : NULL;
      gb_mmp_fill(m, rws, A->i, A->j, A->v, S->i, S->j, pass, col, color, Q.i, Q.j, Q.v, rsum, w, s);
      if (b == 0) { B[0] = Q; continue; }
      /* hypre_ParMatmul (:354-356): square when Q's rows match the
       * previous block's columns */
      int r = 0;
      if (m == 0) { csr_empty(&B[b], B[b - 1].nc); }
      else { r = spgemm_host(&Q, &B[b - 1], Q.nr == B[b - 1].nc, &B[b]); }
      gb_csr_free(&Q);
      if (!r && w) { gb_mmp_scale9(m, rws, A->i, A->v, B[b].i, B[b].v, w, s); }
      gb_dfree(w);
      if (r) { goto done; }
   }
   {
      gb_mmp_blocks blk;
      memset(&blk, 0, sizeof(blk));
      blk.nblk = nblk;
      for (int b = 0; b < nblk; b++) { blk.i[b] = B[b].i; blk.j[b] = B[b].j; blk.v[b] = B[b].v; }
      int *len = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      gb_mmp_len(n, CF, pass, col, &blk, len, s);
      P->nr = n; P->nc = nc;
      P->i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      P->nnz = scan_total(len, P->i, n);
      P->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (P->nnz ? P->nnz : 1));
      P->v = (double *) gb_dmalloc(sizeof(double) * (size_t) (P->nnz ? P->nnz : 1));
      gb_mmp_gather(n, CF, pass, col, &blk, P->i, P->j, P->v, s);
      gb_dfree(len);
   }
   truncate_host(P, prm->agg_trunc_factor, prm->agg_p_max_elmts);
   gb_sf_to_f(n, CF, s);
   rc = nc;
done:
   gb_sync();
   for (int b = 0; b < GB_MMP_MAXB; b++) { gb_csr_free(&B[b]); }
   for (int p = 0; p < GB_MMP_MAXB + 3; p++) { gb_dfree(rows[p]); }
   gb_dfree(pass); gb_dfree(col); gb_dfree(dcnt); gb_dfree(rsum);
   return rc;
}

/* aggressive level (par_amg_setup.c:1311-1358, :1778-1915): second-order
 * strength and PMIS on it, then multipass interpolation (agg_interp_type 4;
 * 8 and 9 in product form) or a two-stage P = P1 P2 (1: extended+i and
 * partial extended+i; 3: extended and partial extended; 5, 6, 7: modified extended, extended+i, extended+e
 * and the matching partial second stage).  Returns the number of coarse
 * points. */
static int agg_interp(gb_amg *amg, const gb_csr *A, const gb_csr *S, int *CF, gb_csr *P)
{
   gb_amg_params *prm = &amg->prm;
   cudaStream_t s = gb_stream();
   int n = A->nr;
   /* first-pass C numbering and list */
   int *f2c1 = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *c2f1 = NULL;
   int nc1 = number_points(n, CF, 0, 0, f2c1, &c2f1);
   /* S2 (par_strength.c:1795) */
   gb_csr S2;
   memset(&S2, 0, sizeof(S2));
   S2.nr = S2.nc = nc1;
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 + 1));
   gb_tier t;
   tier_begin(&t, nc1);
   /* count and fill in one pass into temporary areas sized by each row's
    * upper bound (capped by the shared-memory table), then the rows that did
    * not fit with global tables (count, then fill in place) */
   /* every point's candidate list: itself when a C point, then the C points
    * of its S row (coarse indices) */
   int *Li = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int *lcnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_s2_lists(n, S->i, S->j, CF, f2c1, lcnt, NULL, NULL, s);
   int nl = scan_total(lcnt, Li, n);
   gb_dfree(lcnt);
   int *Lj = (int *) gb_dmalloc(sizeof(int) * (size_t) (nl > 0 ? nl : 1));
   gb_s2_lists(n, S->i, S->j, CF, f2c1, NULL, Li, Lj, s);
   int *ub = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 > 0 ? nc1 : 1));
   int *cap = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 + 1));
   unsigned long long *dsum = (unsigned long long *) gb_dcalloc(sizeof(unsigned long long));
   gb_strength2_ub(nc1, c2f1, S->i, S->j, Li, ub, s);
   gb_cap_sum(nc1, ub, GB_SPGEMM_LCAP0, cap, dsum, s);
   unsigned long long hsum = 0;
   cudaMemcpyAsync(&hsum, dsum, sizeof(hsum), cudaMemcpyDeviceToHost, s);
   gb_sync();
   gb_dfree(dsum);
   if (hsum > 0x7fffff00ULL) { gb_error(HYPRE_ERROR_MEMORY, "second-order strength: temporary areas"); return -1; }
   int *tofs = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 + 1));
   scan_total(cap, tofs, nc1);
   gb_dfree(cap);
   int *tj = (int *) gb_dmalloc(sizeof(int) * (size_t) (hsum > 0 ? hsum : 1));
   int *src = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 > 0 ? nc1 : 1));
   if (g_global_only)
   {
      gb_iota(nc1, t.ovf_list, t.ovf_n, s);
      cudaMemsetAsync(src, 0xff, sizeof(int) * (size_t) (nc1 > 0 ? nc1 : 1), s);
   }
   else
   {
      gb_strength2(nc1, c2f1, Li, Lj, S->i, S->j, cnt, tofs, tj, t.ovf_list, t.ovf_n, NULL, 0, 0, t.err, src, 2,
                   0, s);
   }
   tier_global(&t, ub, nc1);
   if (t.h_ovf > 0)
   {
      gb_strength2(nc1, c2f1, Li, Lj, S->i, S->j, cnt, NULL, NULL, t.ovf_list, t.ovf_n, t.gtab, t.gcap, t.gwarps,
                   t.err, NULL, 0, 1, s);
   }
   gb_mark_isolated(nc1, c2f1, cnt, CF, s);
   S2.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 + 1));
   S2.nnz = scan_total(cnt, S2.i, nc1);
   S2.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (S2.nnz ? S2.nnz : 1));
   gb_spgemm_gather(nc1, S2.nnz, S2.i, src, tj, NULL, S2.j, NULL, s);
   if (t.h_ovf > 0)
   {
      gb_strength2(nc1, c2f1, Li, Lj, S->i, S->j, cnt, S2.i, S2.j, t.ovf_list, t.ovf_n, t.gtab, t.gcap, t.gwarps,
                   t.err, NULL, 1, 1, s);
   }
   gb_dfree(tofs); gb_dfree(tj); gb_dfree(src); gb_dfree(Li); gb_dfree(Lj);
   if (tier_end(&t)) { gb_error(HYPRE_ERROR_GENERIC, "second-order strength overflow"); return -1; }
   gb_dfree(ub);
   /* PMIS on S2 with CF_init 3 */
   int *CFN = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 ? nc1 : 1));
   {
      double *measure = (double *) gb_dmalloc(sizeof(double) * (size_t) (nc1 ? nc1 : 1));
      int *ingraph = (int *) gb_dmalloc(sizeof(int) * (size_t) (nc1 ? nc1 : 1));
      int *counter = (int *) gb_dmalloc(sizeof(int) * 4);
      int it = gb_pmis(nc1, S2.nnz, S2.i, S2.j, 3, CFN, measure, ingraph, cnt, counter, gb_red_ints() + 4, 10000,
                       s);
      gb_dfree(measure); gb_dfree(ingraph); gb_dfree(counter);
      if (it < 0) { gb_error(HYPRE_ERROR_GENERIC, "PMIS on S2 did not terminate"); return -1; }
   }
   gb_csr_free(&S2);
   if (prm->agg_interp_type == 4 || prm->agg_interp_type == 8 || prm->agg_interp_type == 9)
   {
      int nc = prm->agg_interp_type == 4 ? multipass_interp(prm, A, S, CF, f2c1, CFN, P)
                                         : mod_multipass_interp(prm, A, S, CF, f2c1, CFN, P);
      gb_dfree(f2c1); gb_dfree(c2f1); gb_dfree(cnt); gb_dfree(CFN);
      return nc;
   }
   /* P1 over the first coarsening (par_amg_setup.c:1778-1847): extended+i
    * (agg_interp_type 1) or extended (3), both turning CF -3 into -1;
    * modified extended (5),
    * modified extended+i (6), modified extended+e (7) */
   const int at = prm->agg_interp_type;
   gb_csr P1;
   if (at == 1 || at == 3)
   {
      if (extpi_host(A, S, CF, f2c1, n, NULL, nc1, at == 1, &P1)) { return -1; }
      gb_sf_to_f(n, CF, s);
   }
   else if (mm_interp(A, S, CF, f2c1, nc1, at == 5 ? 16 : at == 7 ? 18 : 17, &P1)) { return -1; }
   truncate_host(&P1, prm->agg_p12_trunc_factor, prm->agg_p12_max_elmts);
   /* CF correction (par_strength.c:3096) and P2 over the old C points: partial
    * extended+i (1, 6; partial.c:16, CF below -1 becomes -1), modified partial
    * extended (5) or extended+e (7; par_2s_interp.c, CF kept) */
   gb_correct_cf2(n, f2c1, CFN, CF, s);
   int *f2c2 = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   int nc2 = number_points(n, CF, 1, 1, f2c2, NULL);
   gb_csr P2;
   if (at == 1 || at == 3 || at == 6)
   {
      /* partial extended+i, or partial extended for 3 (partial.c:1902) */
      if (extpi_host(A, S, CF, f2c2, nc1, c2f1, nc2, at != 3, &P2)) { return -1; }
      gb_cf_clamp(n, CF, s);
   }
   else if (mm_partial_interp(A, S, CF, f2c2, nc2, at, &P2)) { return -1; }
   truncate_host(&P2, prm->agg_p12_trunc_factor, prm->agg_p12_max_elmts);
   if (spgemm_host(&P1, &P2, n == nc2, P)) { return -1; }
   truncate_host(P, prm->agg_trunc_factor, prm->agg_p_max_elmts);
   gb_csr_free(&P1); gb_csr_free(&P2);
   gb_dfree(f2c1); gb_dfree(c2f1); gb_dfree(f2c2); gb_dfree(cnt); gb_dfree(CFN);
   return nc2;
}

/* --------------------------------------------------------------------------
 * one coarsening level: S, CF, P, A_c
 * returns 1 if a coarse level was produced, 0 to stop, -1 on error
 * ------------------------------------------------------------------------ */
static int setup_level(gb_amg *amg, int l, double *t_phase)
{
   gb_amg_params *prm = &amg->prm;
   gb_level *L = &amg->lev[l];
   gb_csr *A = &L->A->A;
   int n = A->nr;
   cudaStream_t s = gb_stream();
   double t0 = gb_wtime();

   /* 1. strength (par_strength.c:75) */
   int *cnt = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   gb_csr S;
   memset(&S, 0, sizeof(S));
   S.nr = S.nc = n;
   S.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   long long *rkey = (long long *) gb_dmalloc(sizeof(long long) * (size_t) (n ? n : 1));
   gb_strength_count(n, A->i, A->v, prm->strong_threshold, prm->max_row_sum, cnt, rkey, s);
   S.nnz = scan_total(cnt, S.i, n);
   S.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (S.nnz ? S.nnz : 1));
   gb_strength_fill(n, A->i, A->j, A->v, rkey, S.i, S.j, s);
   gb_dfree(rkey);
   double t1 = gb_wtime();
   t_phase[0] += t1 - t0;

   /* 2. PMIS (par_coarsen.c:2094) */
   int *CF = (int *) gb_dmalloc(sizeof(int) * (size_t) (n ? n : 1));
   {
      double *measure = (double *) gb_dmalloc(sizeof(double) * (size_t) (n ? n : 1));
      int *ingraph = (int *) gb_dmalloc(sizeof(int) * (size_t) (n ? n : 1));
      int *counter = (int *) gb_dmalloc(sizeof(int) * 4);
      int it = gb_pmis(n, S.nnz, S.i, S.j, 0, CF, measure, ingraph, cnt, counter, gb_red_ints() + 4, 10000, s);
      gb_dfree(measure); gb_dfree(ingraph); gb_dfree(counter);
      if (it < 0) { gb_error(HYPRE_ERROR_GENERIC, "PMIS did not terminate"); return -1; }
   }
   double t2 = gb_wtime();
   t_phase[1] += t2 - t1;

   gb_csr P;
   int nc;
   if (l < prm->agg_num_levels)
   {
      nc = agg_interp(amg, A, &S, CF, &P);
      if (nc < 0) { return -1; }
   }
   else
   {
      /* 3. coarse points and numbering (par_coarse_parms.c:45) */
      int *f2c = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      gb_cpoint_flags(n, CF, cnt, s);
      nc = scan_total(cnt, f2c, n);
      if (nc == 0 || nc == n || nc < prm->min_coarse_size)
      {
         gb_dfree(cnt); gb_dfree(f2c); gb_dfree(CF); gb_csr_free(&S);
         return 0;
      }
      /* 4. extended+i interpolation (par_lr_interp.c:1024) or a modified
       * (MM) interpolation (16/17/18), then truncation */
      if (prm->interp_type == 6 || prm->interp_type == 14)
      {
         if (extpi_host(A, &S, CF, f2c, n, NULL, nc, prm->interp_type == 6, &P)) { return -1; }
      }
      /* 15 (BAMG-direct) is the direct interpolation on the reference's
       * host path, which does not look at interp_type (par_interp.c:2580-2610) */
      else if (prm->interp_type == 3 || prm->interp_type == 15)
      {
         if (dir_interp(A, &S, CF, f2c, nc, &P)) { return -1; }
      }
      else if (mm_interp(A, &S, CF, f2c, nc, prm->interp_type, &P)) { return -1; }
      /* ext(+i) and direct interpolation turn the points without strong
       * couplings (-3) into F points (par_lr_interp.c:1887-1893, :5488-5491,
       * par_interp.c:2560-2563); the modified interpolations keep -3 */
      if (prm->interp_type == 6 || prm->interp_type == 14 || prm->interp_type == 3 || prm->interp_type == 15)
      {
         gb_sf_to_f(n, CF, s);
      }
      truncate_host(&P, prm->trunc_factor, prm->p_max_elmts);
      gb_dfree(f2c);
   }
   double t3 = gb_wtime();
   t_phase[2] += t3 - t2;

   /* 5. R = P^T and A_c = (R A) P (par_rap.c:30) */
   gb_parcsr *Pm = gb_parcsr_wrap(P, 1);
   gb_parcsr *Rm = gb_transpose(Pm);
   if (!Rm) { return -1; }
   gb_csr RA, C;
   if (spgemm_host(&Rm->A, A, 0, &RA)) { return -1; }
   if (spgemm_host(&RA, &P, 1, &C)) { return -1; }
   gb_csr_free(&RA);
   gb_dfree(cnt);
   double t4 = gb_wtime();
   t_phase[3] += t4 - t3;

   L->S = S;
   L->CF = CF;
   L->P = Pm;
   L->R = Rm;
   amg->lev[l + 1].A = gb_parcsr_wrap(C, 1);
   amg->lev[l + 1].n = nc;
   return 1;
}

/* hybrid Gauss-Seidel relax types (gb_hgs.cu) */
static int hgs_type(int t) { return t == 3 || t == 4 || t == 6 || t == 8 || t == 13 || t == 14; }

/* l1-norm option of a level (par_amg_setup.c:3298-3496): the relax types of
 * the level (down and up, or the coarsest's) pick it; later rules override
 * earlier ones as in the reference: 8/13/14 -> option 4, 18 -> 1, and
 * 7/11/12 -> 5 (also the default here) */
static int relax_l1_option_level(const gb_amg_params *prm, int l, int nl)
{
   const int last = l == nl - 1;
   const int a = last ? prm->relax_type[3] : prm->relax_type[1];
   const int b = last ? prm->relax_type[3] : prm->relax_type[2];
   int opt = 5;
   if (a == 8 || a == 13 || a == 14 || b == 8 || b == 13 || b == 14) { opt = 4; }
   if (a == 18 || b == 18) { opt = 1; }
   /* 7/11/12 in any part of the cycle (the coarsest's only on the last level) */
   const int *t = prm->relax_type;
   if (t[1] == 7 || t[2] == 7 || (t[3] == 7 && last) || t[1] == 11 || t[2] == 11 || (t[3] == 11 && last) ||
       t[1] == 12 || t[2] == 12 || (t[3] == 12 && last)) { opt = 5; }
   return opt;
}

/* device flag set by a hybrid Gauss-Seidel sweep whose dependency wait ran
 * out; read back once per solve (only when a hybrid sweep ran) */
static int *g_hgs_err = NULL;
static int g_hgs_used = 0;

/* --------------------------------------------------------------------------
 * Chebyshev smoother setup
 * ------------------------------------------------------------------------ */
static double pythag(double a, double b)
{
   /* sqrt(a^2 + b^2) by the overflow-free iteration of Moler and Morrison
    * (IBM J. Res. Dev. 27, 1983) */
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

/* Eigenvalues (ascending, in d) of the symmetric tridiagonal matrix with
 * diagonal d[0..n-1] and sub-diagonal e[1..n-1], by the implicit QL method
 * TQL1 (Bowdler, Martin, Reinsch, Wilkinson, Numer. Math. 11, 1968), which the
 * reference calls as hypre_LINPACKcgtql1 (src/parcsr_ls/par_relax_more.c:507).
 * Returns nonzero if an eigenvalue needs more than 30 QL steps. */
static int eig_tridiag(int n, double *d, double *e)
{
   if (n <= 1) { return 0; }
   for (int i = 1; i < n; i++) { e[i - 1] = e[i]; }
   e[n - 1] = 0.0;
   double f = 0.0, tst1 = 0.0;
   for (int l = 0; l < n; l++)
   {
      double h = fabs(d[l]) + fabs(e[l]);
      if (tst1 < h) { tst1 = h; }
      int m = l;
      while (tst1 + fabs(e[m]) != tst1) { m++; }
      if (m > l)
      {
         int steps = 0;
         do
         {
            if (steps == 30) { return l + 1; }
            steps++;
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
      double p = d[l] + f;
      int i = l;
      while (i > 0 && p < d[i - 1]) { d[i] = d[i - 1]; i--; }
      d[i] = p;
   }
   return 0;
}

/* Extreme eigenvalue estimates of D^{-1/2} A D^{-1/2} (or A without scaling):
 * max_iter CG steps from the seed-1 random vector, Lanczos tridiagonal from
 * the CG coefficients (hypre_ParCSRMaxEigEstimateCGHost,
 * src/parcsr_ls/par_relax_more.c:203).  ds must already hold the scaling. */
static void cheby_eig_estimate(gb_level *L, int scale, int max_iter, double *max_eig, double *min_eig)
{
   int n = L->n;
   cudaStream_t s = gb_stream();
   if (n < max_iter) { max_iter = n; }
   const gb_spmv_desc *A = gb_solve_desc(L->A, GB_PREC_F64);
   size_t nb = sizeof(double) * (size_t) (n ? n : 1);
   double *r = (double *) gb_dmalloc(nb), *p = (double *) gb_dcalloc(nb);
   double *sv = (double *) gb_dmalloc(nb), *u = (double *) gb_dmalloc(nb);
   double td[34], te[34];
   memset(td, 0, sizeof(td));
   memset(te, 0, sizeof(te));
   gb_rand_uniform(n, 1, r, s);
   double gamma = 0.0, gamma_old, beta = 1.0;   /* <r, p> with p = 0 */
   int it = 0;
   while (it < max_iter)
   {
      cudaMemcpyAsync(sv, r, nb, cudaMemcpyDeviceToDevice, s);
      gamma_old = gamma;
      gamma = gb_dot(n, r, sv);
      if (gamma < 2.220446049250313e-16) { break; }
      if (it == 0) { beta = 1.0; cudaMemcpyAsync(p, sv, nb, cudaMemcpyDeviceToDevice, s); }
      else
      {
         beta = gamma / gamma_old;
         gb_xpay_d(n, sv, beta, p, s);
      }
      if (scale)
      {
         gb_vmul_d(n, L->cheb_ds, p, u, s);
         gb_spmv_d(A, u, sv, GB_EPI_AXPBY, 1.0, 0.0, NULL, NULL, 0.0, NULL, NULL, s);
         gb_vmul_d(n, L->cheb_ds, sv, sv, s);
      }
      else { gb_spmv_d(A, p, sv, GB_EPI_AXPBY, 1.0, 0.0, NULL, NULL, 0.0, NULL, NULL, s); }
      double sdotp = gb_dot(n, sv, p);
      double alpha = gamma / sdotp;
      double ainv = 1.0 / alpha;
      td[it + 1] = ainv;
      td[it] *= beta;
      td[it] += ainv;
      te[it + 1] = ainv;
      te[it] *= sqrt(beta);
      gb_axpy_d(n, -alpha, sv, r, s);
      it++;
   }
   gb_sync();
   gb_dfree(r); gb_dfree(p); gb_dfree(sv); gb_dfree(u);
   eig_tridiag(it, td, te);
   *max_eig = it > 0 ? td[it - 1] : 0.0;
   *min_eig = td[0];
}

/* Coefficients of s(t) with u <- u + s(A) r, 1 - t s(t) the Chebyshev residual
 * polynomial of the given order on [lower, upper] (hypre_ParCSRRelax_Cheby_Setup,
 * src/parcsr_ls/par_cheby_setup.c): upper = 1.1 max_eig, lower = min_eig +
 * fraction (upper - min_eig); variant 1 is the reference's modified form. */
static void cheby_coefs(double max_eig, double min_eig, double fraction, int order, int variant, double *c)
{
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
   for (int k = 0; k < 5; k++) { c[k] = 0.0; }
   if (co == 0) { c[0] = fabs(th) > 0.0 ? 1.0 / th : 0.0; return; }
   if (variant == 1)
   {
      if (co == 1)
      {
         den = th * th + de * th;
         if (fabs(den) > 0.0) { c[0] = (de + 2 * th) / den; c[1] = -1.0 / den; }
      }
      else if (co == 2)
      {
         den = 2 * de * th * th - de * de * th - pow(de, 3) + 2 * pow(th, 3);
         if (fabs(den) > 0.0)
         {
            c[0] = (4 * de * th - pow(de, 2) + 6 * pow(th, 2)) / den;
            c[1] = -(2 * de + 6 * th) / den;
            c[2] = 2 / den;
         }
      }
      else
      {
         den = -4 * de * pow(th, 3) + 3 * pow(de, 2) * pow(th, 2) + 3 * pow(de, 3) * th - 4 * pow(th, 4);
         if (fabs(den) > 0.0)
         {
            c[0] = (6 * pow(de, 2) * th - 12 * de * pow(th, 2) + 3 * pow(de, 3) - 16 * pow(th, 3)) / den;
            c[1] = (12 * de * th - 3 * pow(de, 2) + 24 * pow(th, 2)) / den;
            c[2] = -(4 * de + 16 * th) / den;
            c[3] = 4 / den;
         }
      }
      return;
   }
   if (co == 1)
   {
      den = de * de - 2 * th * th;
      if (fabs(den) > 0.0) { c[0] = -4 * th / den; c[1] = 2 / den; }
   }
   else if (co == 2)
   {
      den = 3 * (de * de) * th - 4 * (th * th * th);
      if (fabs(den) > 0.0)
      {
         c[0] = (3 * de * de - 12 * th * th) / den;
         c[1] = 12 * th / den;
         c[2] = -4 / den;
      }
   }
   else
   {
      den = pow(de, 4) - 8 * ((de * th) * (de * th)) + pow(th, 4) * 8;
      if (fabs(den) > 0.0)
      {
         c[0] = (32 * pow(th, 3) - 16 * de * de * th) / den;
         c[1] = (8 * de * de - 48 * th * th) / den;
         c[2] = 32 * th / den;
         c[3] = -8 / den;
      }
   }
}

static void cheby_level_setup(gb_amg *amg, int l)
{
   gb_amg_params *prm = &amg->prm;
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   int n = L->n;
   int order = prm->cheby_order > 4 ? 4 : (prm->cheby_order < 1 ? 1 : prm->cheby_order);
   L->cheb_order = order;
   size_t nb = sizeof(double) * (size_t) (n ? n : 1), nf = sizeof(float) * (size_t) (n ? n : 1);
   L->cheb_ds = (double *) gb_dmalloc(nb);
   L->cheb_dsf = (float *) gb_dmalloc(nf);
   L->W = (double *) gb_dcalloc(nb);
   L->Wf = (float *) gb_dcalloc(nf);
   if (prm->cheby_scale) { gb_diag_inv_sqrt(n, L->A->A.i, L->A->A.j, L->A->A.v, L->cheb_ds, s); }
   else { gb_fill_d(n, L->cheb_ds, 1.0, s); }
   gb_d2f(n, L->cheb_ds, L->cheb_dsf, s);
   double mx = 0.0, mn = 0.0;
   if (prm->cheby_eig_est > 0)
   {
      int it = prm->cheby_eig_est < 32 ? prm->cheby_eig_est : 32;
      cheby_eig_estimate(L, prm->cheby_scale, it, &mx, &mn);
   }
   L->cheb_eig[0] = mx;
   L->cheb_eig[1] = mn;
   cheby_coefs(mx, mn, prm->cheby_fraction, order, prm->cheby_variant, L->cheb_c);
}

static int amg_setup_inner(gb_amg *amg, gb_parcsr *A0);

/* With a learned model the strength threshold of this setup is the model's
 * prediction from the finest level's rows; the user's value is kept. */
int gb_amg_setup(gb_amg *amg, gb_parcsr *A0)
{
   double user_theta = amg->prm.strong_threshold;
   if (amg->mlp_params)
   {
      amg_free_hierarchy(amg);
      if (gb_learn_theta(amg, A0, &amg->prm.strong_threshold)) { return gb_error_flag; }
   }
   int r = amg_setup_inner(amg, A0);
   amg->prm.strong_threshold = user_theta;
   return r;
}

static int amg_setup_inner(gb_amg *amg, gb_parcsr *A0)
{
   amg_free_hierarchy(amg);
   gb_amg_params *prm = &amg->prm;
   double t_start = gb_wtime();
   g_sg_bytes = g_sg_seconds = 0.0;
   g_sg_calls = 0;
   g_sg_nev = 0;
   g_global_only = amg->prm.setup_tables == 1;

   memset(amg->setup_times, 0, sizeof(amg->setup_times));
   const long long sync0 = gb_sync_calls;
   const double tsync0 = gb_sync_seconds;
   amg->lev[0].A = A0;
   amg->lev[0].n = A0->A.nr;
   int level = 0;
   int maxl = prm->max_levels < 32 ? prm->max_levels : 32;
   if (prm->agg_num_levels > 0 && !(prm->agg_interp_type == 1 || (prm->agg_interp_type >= 3 && prm->agg_interp_type <= 9)))
   {
      gb_error(HYPRE_ERROR_GENERIC, "aggressive coarsening: agg_interp_type 1 and 3-9 are supported");
      return gb_error_flag;
   }
   while (1)
   {
      /* the size test follows each coarsening (par_amg_setup.c:3136-3143):
       * the finest level is coarsened even when it is within max_coarse_size */
      if (level == maxl - 1) { break; }
      int r = setup_level(amg, level, amg->setup_times);
      if (r < 0) { amg->num_levels = level + 1; return gb_error_flag; }
      if (r == 0) { break; }
      level++;
      if (amg->lev[level].n <= prm->max_coarse_size) { break; }
   }
   amg->num_levels = level + 1;
   /* Gaussian elimination only when the coarsest level is within
    * max_coarse_size -- coarsening can stop above it -- else the coarsest
    * level relaxes with the down-cycle type (par_amg_setup.c:3162-3178; the
    * reference also keeps the change in its parameters) */
   {
      const int t = prm->relax_type[3];
      if ((t == 9 || t == 19 || t == 98 || t == 99 || t == 198 || t == 199) &&
          amg->lev[amg->num_levels - 1].n > prm->max_coarse_size)
      {
         prm->relax_type[3] = prm->relax_type[1];
      }
   }
   double t_sm = gb_wtime();
   /* smoother setup: l1 norms or diagonal per level (par_amg_setup.c:3352-3496) */
   cudaStream_t s = gb_stream();
   for (int l = 0; l < amg->num_levels; l++)
   {
      gb_level *L = &amg->lev[l];
      int n = L->n;
      L->l1 = (double *) gb_dmalloc(sizeof(double) * (size_t) (n ? n : 1));
      /* with relax_order the l1-Jacobi norms of the levels above the coarsest
       * sum over the row's own C/F class (par_amg_setup.c:3352-3360) */
      const int opt = relax_l1_option_level(prm, l, amg->num_levels);
      const int *cfl = (opt == 1 && prm->relax_order && l < amg->num_levels - 1) ? L->CF : NULL;
      gb_l1_norms(n, L->A->A.i, L->A->A.j, L->A->A.v, opt, cfl, L->l1, s);
      L->l1f = (float *) gb_dmalloc(sizeof(float) * (size_t) (n ? n : 1));
      gb_d2f(n, L->l1, L->l1f, s);
      L->relax_w = prm->level_relax_weight ? prm->level_relax_weight[l] : prm->relax_weight;
      size_t nb = sizeof(double) * (size_t) (n ? n : 1);
      L->F = (double *) gb_dcalloc(nb); L->U = (double *) gb_dcalloc(nb);
      L->U2 = (double *) gb_dcalloc(nb); L->V = (double *) gb_dcalloc(nb);
      size_t nf = sizeof(float) * (size_t) (n ? n : 1);
      L->Ff = (float *) gb_dcalloc(nf); L->Uf = (float *) gb_dcalloc(nf);
      L->U2f = (float *) gb_dcalloc(nf); L->Vf = (float *) gb_dcalloc(nf);
      const int last = l == amg->num_levels - 1;
      if ((!last && (hgs_type(prm->relax_type[1]) || hgs_type(prm->relax_type[2]))) ||
          (last && hgs_type(prm->relax_type[3])))
      {
         L->hgs_flags = (int *) gb_dcalloc(sizeof(int) * ((size_t) n + 1));
         L->hgs_t = (double *) gb_dcalloc(nb);
         L->hgs_tf = (float *) gb_dcalloc(nf);
         if (!g_hgs_err) { g_hgs_err = (int *) gb_dcalloc(sizeof(int)); }
         amg->uses_hgs = 1;
      }
   }
   /* coarsest grid: dense inverse (par_gauss_elim.c:33) */
   {
      gb_level *L = &amg->lev[amg->num_levels - 1];
      int t = prm->relax_type[3];
      if ((t == 9 || t == 19 || t == 98 || t == 99 || t == 198 || t == 199) && L->n <= 4096)
      {
         int nn = L->n;
         amg->coarse_n = nn;
         amg->coarse_inv = (double *) gb_dmalloc(sizeof(double) * (size_t) nn * nn);
         double *W = (double *) gb_dmalloc(sizeof(double) * (size_t) nn * nn);
         gb_dense_inverse(nn, L->A->A.i, L->A->A.j, L->A->A.v, amg->coarse_inv, W, s);
         gb_sync();
         gb_dfree(W);
      }
   }
   /* solve-phase forms of every level operator in the cycle precision */
   for (int l = 0; l < amg->num_levels; l++)
   {
      gb_level *L = &amg->lev[l];
      int vp = prm->cycle_prec == GB_PREC_F64 ? GB_PREC_F64 : GB_PREC_F32;
      int vp0 = prm->cycle_prec == GB_PREC_F16 && l == 0 ? GB_PREC_F16 : vp;
      gb_solve_desc(L->A, vp0);
      if (vp0 != GB_PREC_F64) { gb_solve_desc(L->A, GB_PREC_F64); }
      /* hybrid Gauss-Seidel in the FP16-finest cycle sweeps FP32 CSR values */
      if (vp0 == GB_PREC_F16 && L->hgs_flags) { gb_solve_desc(L->A, GB_PREC_F32); }
      if (L->P) { gb_solve_desc(L->P, vp); gb_solve_desc(L->R, vp); }
      /* lower-part forms for two-stage Gauss-Seidel (built here, outside any
       * graph capture of the cycle) */
      int ts = 0;
      for (int k = 1; k <= 2; k++) { ts |= prm->relax_type[k] == 11 || prm->relax_type[k] == 12; }
      if (ts && l < amg->num_levels - 1)
      {
         const void *dg = NULL;
         gb_lower_desc(L->A, vp0, &dg);
      }
   }
   if (amg->mlp_params && gb_learn_weights(amg)) { return gb_error_flag; }
   /* Chebyshev data on the levels that relax with it (par_amg_setup.c:3496-3536) */
   for (int l = 0; l < amg->num_levels; l++)
   {
      if (prm->relax_type[1] == 16 || prm->relax_type[2] == 16 ||
          (prm->relax_type[3] == 16 && l == amg->num_levels - 1))
      {
         cheby_level_setup(amg, l);
      }
   }
   gb_sync();
   g_global_only = 0;
   spgemm_times_collect();
   if (tier_errors()) { gb_error(HYPRE_ERROR_GENERIC, "sparse table overflow in setup"); }
   amg->r_work = (double *) gb_dmalloc(sizeof(double) * (size_t) (amg->lev[0].n ? amg->lev[0].n : 1));
   amg->setup_times[4] = gb_wtime() - t_sm;
   amg->spgemm_bytes = g_sg_bytes;
   amg->spgemm_seconds = g_sg_seconds;
   amg->spgemm_calls = g_sg_calls;
   amg->setup_times[5] = gb_wtime() - t_start;
   amg->setup_times[6] = (double) (gb_sync_calls - sync0);
   amg->setup_times[7] = gb_sync_seconds - tsync0;
   amg->setup_done = 1;
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * V(1,1) cycle (par_cycle.c): f, u on level 0; u_zero: u is zero on entry
 * ------------------------------------------------------------------------ */
static void relax_d(gb_amg *amg, int l, int type, const double *f, double *u_in, double *u_out, int u_zero)
{
   /* l1-Jacobi (relax 18 via Relax7Jacobi par_relax.c:1178) and Jacobi (7):
    * u_out = u_in + w (f - A u_in) ./ d ; two-stage GS (11/12, par_relax.c:1506)
    * updates u_in in place and leaves u_out untouched. */
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   const gb_spmv_desc *A = gb_solve_desc(L->A, GB_PREC_F64);
   double w = L->relax_w;
   (void) type;
   if (u_zero) { gb_scaled_div_d(L->n, w, f, L->l1, u_out, s); }
   else { gb_spmv_d(A, u_in, u_out, 1, 0.0, 0.0, f, L->l1, w, NULL, NULL, s); }
}

static void twostage_gs_d(gb_amg *amg, int l, int inner, const double *f, double *u, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   const gb_spmv_desc *A = gb_solve_desc(L->A, GB_PREC_F64);
   double w = L->relax_w;
   double *V = L->V, *Z = L->U2;
   /* V = w (f - A u) */
   if (u_zero) { gb_fill_d(L->n, u, 0.0, s); gb_scaled_copy_d(L->n, w, f, V, s); }
   else { gb_spmv_d(A, u, V, 0, -w, w, f, NULL, 0.0, NULL, NULL, s); }
   /* large levels: the strictly lower part as SELL-32 with the diagonal in
    * a contiguous array (coalesced, half the bytes of the whole rows) */
   const void *diag = NULL;
   const gb_spmv_desc *Lo = gb_lower_desc(L->A, GB_PREC_F64, &diag);
   if (Lo) { gb_gs_first_diag_d(L->n, (const double *) diag, V, u, s); }
   else { gb_gs_first_d(L->n, L->A->A.i, L->A->A.v, V, u, s); }
   double m = -1.0;
   for (int k = 0; k < inner; k++)
   {
      if (Lo) { gb_spmv_d(Lo, V, Z, GB_EPI_GS, m, 0.0, u, (const double *) diag, 0.0, NULL, NULL, s); }
      else { gb_gs_lower_d(L->n, L->A->A.i, L->A->A.j, L->A->A.v, V, Z, u, m, s); }
      double *t = V; V = Z; Z = t;
      m = -m;
   }
}

/* Hybrid Gauss-Seidel relaxation in place on u (relax 3/4: forward/backward,
 * 6: symmetric; 13/14/8: the same with l1 norms; par_relax.c:954-1377):
 * one relaxation is one sweep, or a forward and a backward sweep (6, 8).
 * Unscaled (weight and outer weight 1): 3/4/6 leave the diagonal out of the
 * sum and divide by it, 8/13/14 include it and add res / l1; scaled: the
 * reference's weighted form over the values from before the relaxation. */
static void hybrid_gs_d(gb_amg *amg, int l, int type, const double *f, double *u, int u_zero, int pts)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   const int n = L->n;
   if (u_zero) { gb_fill_d(n, u, 0.0, s); }
   const double w = L->relax_w, omega = amg->prm.outer_weight;
   const int scaled = !(w == 1.0 && omega == 1.0);
   const int l1 = type == 8 || type == 13 || type == 14;
   const int skip = l1 ? scaled : 1;
   double *ut = NULL;
   if (scaled)
   {
      ut = L->hgs_t;
      cudaMemcpyAsync(ut, u, sizeof(double) * (size_t) n, cudaMemcpyDeviceToDevice, s);
   }
   const int dir0 = (type == 4 || type == 14) ? -1 : 1;
   const int nsw = (type == 6 || type == 8) ? 2 : 1;
   const gb_csr *A = &L->A->A;
   for (int k = 0; k < nsw; k++)
   {
      gb_hgs_sweep_d(n, A->nnz, A->i, A->j, A->v, f, u, L->V, ut, l1 ? L->l1 : NULL, k == 0 ? dir0 : -dir0, skip,
                     w, omega, L->CF, pts, L->hgs_flags, g_hgs_err, s);
   }
   g_hgs_used = 1;
}

static void hybrid_gs_f(gb_amg *amg, int l, int type, const float *f, float *u, int u_zero, int pts)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   const int n = L->n;
   if (u_zero) { gb_fill_f(n, u, 0.f, s); }
   const double w = L->relax_w, omega = amg->prm.outer_weight;
   const int scaled = !(w == 1.0 && omega == 1.0);
   const int l1 = type == 8 || type == 13 || type == 14;
   const int skip = l1 ? scaled : 1;
   float *ut = NULL;
   if (scaled)
   {
      ut = L->hgs_tf;
      cudaMemcpyAsync(ut, u, sizeof(float) * (size_t) n, cudaMemcpyDeviceToDevice, s);
   }
   const int dir0 = (type == 4 || type == 14) ? -1 : 1;
   const int nsw = (type == 6 || type == 8) ? 2 : 1;
   const gb_spmv_desc *A = gb_solve_desc(L->A, GB_PREC_F32);
   for (int k = 0; k < nsw; k++)
   {
      gb_hgs_sweep_f(n, L->A->A.nnz, A->i, A->j, (const float *) A->v, f, u, L->Vf, ut, l1 ? L->l1f : NULL,
                     k == 0 ? dir0 : -dir0, skip, w, omega, L->CF, pts, L->hgs_flags, g_hgs_err, s);
   }
   g_hgs_used = 1;
}

/* HYPRE_ERROR_GENERIC when a hybrid Gauss-Seidel sweep since the last check
 * gave up waiting on a dependency (reads one int; only after a sweep ran) */
int gb_amg_check_sweeps(void)
{
   if (!g_hgs_used || !g_hgs_err) { return 0; }
   int h = 0;
   cudaMemcpyAsync(&h, g_hgs_err, sizeof(int), cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   g_hgs_used = 0;
   if (h)
   {
      cudaMemsetAsync(g_hgs_err, 0, sizeof(int), gb_stream());
      gb_error(HYPRE_ERROR_GENERIC, "hybrid Gauss-Seidel sweep: a dependency wait ran out");
      return 1;
   }
   return 0;
}

/* Chebyshev smoother, in place on u (hypre_ParCSRRelax_Cheby_SolveHost,
 * src/parcsr_ls/par_cheby_solve.c:194): r = D^{-1/2}(f - Au), then the
 * polynomial by Horner steps, each one SpMV with a fused epilogue. */
static void cheby_d(gb_amg *amg, int l, const double *f, double *u, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   const gb_spmv_desc *A = gb_solve_desc(L->A, GB_PREC_F64);
   int co = L->cheb_order - 1;
   const double *c = L->cheb_c, *ds = L->cheb_ds;
   double *r = L->V, *q = L->U2, *q2 = L->W;
   if (u_zero) { gb_fill_d(L->n, u, 0.0, s); gb_vmul_d(L->n, ds, f, r, s); }
   else { gb_spmv_d(A, u, r, GB_EPI_CHEB_RES, 0.0, 0.0, f, ds, 0.0, NULL, NULL, s); }
   if (co == 0) { gb_cheb_order1_d(L->n, c[0], r, ds, u, s); return; }
   gb_cheb_start_d(L->n, c[co], r, ds, q, s);
   for (int k = co - 1; k >= 1; k--)
   {
      gb_spmv_d(A, q, q2, GB_EPI_CHEB_STEP, c[k], 0.0, r, ds, 0.0, NULL, NULL, s);
      double *t = q; q = q2; q2 = t;
   }
   gb_spmv_d(A, q, u, GB_EPI_CHEB_LAST, c[0], 0.0, r, ds, 0.0, NULL, NULL, s);
}

static void cheby_f(gb_amg *amg, int l, const float *f, float *u, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   int vp = (amg->prm.cycle_prec == GB_PREC_F16 && l == 0) ? GB_PREC_F16 : GB_PREC_F32;
   const gb_spmv_desc *A = gb_solve_desc(L->A, vp);
   int co = L->cheb_order - 1;
   const double *c = L->cheb_c;
   const float *ds = L->cheb_dsf;
   float *r = L->Vf, *q = L->U2f, *q2 = L->Wf;
   if (u_zero) { gb_fill_f(L->n, u, 0.0f, s); gb_vmul_f(L->n, ds, f, r, s); }
   else { gb_spmv_f(A, u, r, GB_EPI_CHEB_RES, 0.0f, 0.0f, f, ds, 0.0f, NULL, NULL, s); }
   if (co == 0) { gb_cheb_order1_f(L->n, (float) c[0], r, ds, u, s); return; }
   gb_cheb_start_f(L->n, (float) c[co], r, ds, q, s);
   for (int k = co - 1; k >= 1; k--)
   {
      gb_spmv_f(A, q, q2, GB_EPI_CHEB_STEP, (float) c[k], 0.0f, r, ds, 0.0f, NULL, NULL, s);
      float *t = q; q = q2; q2 = t;
   }
   gb_spmv_f(A, q, u, GB_EPI_CHEB_LAST, (float) c[0], 0.0f, r, ds, 0.0f, NULL, NULL, s);
}

/* One relaxation in place on u of the points of class pts (C/F relaxation,
 * hypre_BoomerAMGRelaxIF src/parcsr_ls/par_relax_interface.c:20-64 into
 * hypre_BoomerAMGRelax): the Jacobi types update the rows with CF == pts (and
 * a nonzero divisor) from one Jacobi step over the values from before the
 * relaxation; hybrid Gauss-Seidel sweeps leave the other rows as they are;
 * two-stage Gauss-Seidel ignores the points and relaxes all of them. */
static void relax_points_d(gb_amg *amg, int l, int type, const double *f, double *u, int u_zero, int pts)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   if (type == 11 || type == 12) { twostage_gs_d(amg, l, type == 11 ? 1 : 2, f, u, u_zero); }
   else if (hgs_type(type)) { hybrid_gs_d(amg, l, type, f, u, u_zero, pts); }
   else
   {
      if (u_zero) { gb_fill_d(L->n, u, 0.0, s); }
      relax_d(amg, l, type, f, u, L->U2, u_zero);
      gb_select_points_d(L->n, L->CF, pts, L->l1, L->U2, u, s);
   }
}

/* relax_order 1 above the coarsest level: a relaxation of the down cycle
 * (cycle_param 1) is two, over the C and then the F points; of the up cycle
 * (2) over the F and then the C points (par_relax_interface.c:36-56) */
static void relax_cf_d(gb_amg *amg, int l, int type, int cycle_param, const double *f, double *u, int u_zero)
{
   const int p0 = cycle_param < 2 ? 1 : -1;
   relax_points_d(amg, l, type, f, u, u_zero, p0);
   relax_points_d(amg, l, type, f, u, 0, -p0);
}

/* One relaxation in place on u, for the general cycle: the cycle part's C/F
 * order when it applies, else the smoother of the V-cycle */
static void relax_level_d(gb_amg *amg, int l, int type, int cycle_param, const double *f, double *u, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   if (amg->prm.relax_order == 1 && amg->num_levels > 1 && cycle_param < 3 && type != 16)
   {
      relax_cf_d(amg, l, type, cycle_param, f, u, u_zero);
   }
   else if (type == 11 || type == 12) { twostage_gs_d(amg, l, type == 11 ? 1 : 2, f, u, u_zero); }
   else if (type == 16) { cheby_d(amg, l, f, u, u_zero); }
   else if (hgs_type(type)) { hybrid_gs_d(amg, l, type, f, u, u_zero, 0); }
   else if (u_zero) { relax_d(amg, l, type, f, u, u, 1); }
   else
   {
      relax_d(amg, l, type, f, u, L->U2, 0);
      cudaMemcpyAsync(u, L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
   }
}

/* W- and F-cycles: the reference's level counters (hypre_BoomerAMGCycle
 * src/parcsr_ls/par_cycle.c:225-866) choose the next level -- coarser while
 * the level's counter stays >= 0, else finer -- with the per-level
 * operations of the V-cycle: relaxation of the cycle part (down 1, up 2,
 * coarsest 3), residual and restriction with a zero coarse guess on the way
 * down, u_f += P u_c on the way up.  Host control only: the sequence is
 * captured into the cycle's graph like the V-cycle's. */
static void cycle_gen_d(gb_amg *amg, const double *f0, double *u0, int u0_zero)
{
   gb_amg_params *prm = &amg->prm;
   cudaStream_t s = gb_stream();
   const int nl = amg->num_levels, ct = prm->cycle_type;
   const double *F[32];
   double *U[32];
   int counter[32], zero[32];
   F[0] = f0; U[0] = u0;
   for (int l = 1; l < nl; l++) { F[l] = amg->lev[l].F; U[l] = amg->lev[l].U; }
   counter[0] = 1;
   zero[0] = u0_zero;
   for (int l = 1; l < nl; l++) { counter[l] = prm->fcycle ? 1 : ct; zero[l] = 0; }
   int fl = nl - 2, level = 0, cp = nl == 1 ? 3 : 1;
   for (;;)
   {
      gb_level *L = &amg->lev[level];
      if (level == nl - 1)
      {
         if (amg->coarse_inv) { gb_dense_apply_d(amg->coarse_n, amg->coarse_inv, F[level], U[level], s); }
         else { relax_level_d(amg, level, prm->relax_type[3], 3, F[level], U[level], zero[level]); }
      }
      else
      {
         for (int sw = 0; sw < prm->num_sweeps[cp]; sw++)
         {
            relax_level_d(amg, level, prm->relax_type[cp], cp, F[level], U[level], zero[level] && sw == 0);
         }
      }
      zero[level] = 0;
      --counter[level];
      if (counter[level] >= 0 && level != nl - 1)
      {
         gb_spmv_d(gb_solve_desc(L->A, GB_PREC_F64), U[level], L->V, 2, -1.0, 1.0, F[level], NULL, 0.0, NULL, NULL,
                   s);
         gb_spmv_d(gb_solve_desc(L->R, GB_PREC_F64), L->V, (double *) F[level + 1], 0, 1.0, 0.0, NULL, NULL, 0.0,
                   NULL, NULL, s);
         cudaMemsetAsync(U[level + 1], 0, sizeof(double) * (size_t) amg->lev[level + 1].n, s);
         zero[level + 1] = 1;
         ++level;
         if (counter[level] < ct) { counter[level] = ct; }
         cp = level == nl - 1 ? 3 : 1;
      }
      else if (level != 0)
      {
         gb_level *Lf = &amg->lev[level - 1];
         gb_spmv_d(gb_solve_desc(Lf->P, GB_PREC_F64), U[level], Lf->U2, 0, 1.0, 1.0, U[level - 1], NULL, 0.0, NULL,
                   NULL, s);
         cudaMemcpyAsync(U[level - 1], Lf->U2, sizeof(double) * (size_t) Lf->n, cudaMemcpyDeviceToDevice, s);
         --level;
         cp = 2;
         if (prm->fcycle && fl == level)
         {
            if (counter[level] < 1) { counter[level] = 1; }
            fl--;
         }
      }
      else { break; }
   }
}

static void cycle_d(gb_amg *amg, const double *f0, double *u0, int u0_zero)
{
   gb_amg_params *prm = &amg->prm;
   if (prm->cycle_type != 1 || prm->fcycle) { cycle_gen_d(amg, f0, u0, u0_zero); return; }
   cudaStream_t s = gb_stream();
   int nl = amg->num_levels;
   /* C/F relaxation order above the coarsest level (par_cycle.c:441-452) */
   const int cf = prm->relax_order == 1 && nl > 1;
   const double *F[32];
   double *U[32];
   F[0] = f0; U[0] = u0;
   for (int l = 1; l < nl; l++) { F[l] = amg->lev[l].F; U[l] = amg->lev[l].U; }
   for (int l = 0; l < nl - 1; l++)
   {
      gb_level *L = &amg->lev[l];
      int type = prm->relax_type[1];
      int uz = (l > 0) || u0_zero;
      for (int sw = 0; sw < prm->num_sweeps[1]; sw++)
      {
         if (cf && type != 16) { relax_cf_d(amg, l, type, 1, F[l], U[l], uz && sw == 0); }
         else if (type == 11 || type == 12) { twostage_gs_d(amg, l, type == 11 ? 1 : 2, F[l], U[l], uz && sw == 0); }
         else if (type == 16) { cheby_d(amg, l, F[l], U[l], uz && sw == 0); }
         else if (hgs_type(type)) { hybrid_gs_d(amg, l, type, F[l], U[l], uz && sw == 0, 0); }
         else
         {
            if (uz && sw == 0) { relax_d(amg, l, type, F[l], U[l], U[l], 1); }
            else
            {
               relax_d(amg, l, type, F[l], U[l], L->U2, 0);
               cudaMemcpyAsync(U[l], L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
            }
         }
      }
      /* residual and restriction */
      gb_spmv_d(gb_solve_desc(L->A, GB_PREC_F64), U[l], L->V, 2, -1.0, 1.0, F[l], NULL, 0.0, NULL, NULL, s);
      gb_spmv_d(gb_solve_desc(L->R, GB_PREC_F64), L->V, (double *) F[l + 1], 0, 1.0, 0.0, NULL, NULL, 0.0, NULL,
                NULL, s);
   }
   {
      int l = nl - 1;
      gb_level *L = &amg->lev[l];
      if (amg->coarse_inv) { gb_dense_apply_d(amg->coarse_n, amg->coarse_inv, F[l], U[l], s); }
      else if (nl == 1 && !u0_zero && prm->relax_type[3] == 16) { cheby_d(amg, l, F[l], U[l], 0); }
      else if (nl == 1 && !u0_zero && hgs_type(prm->relax_type[3])) { hybrid_gs_d(amg, l, prm->relax_type[3], F[l], U[l], 0, 0); }
      else if (nl == 1 && !u0_zero)
      {
         relax_d(amg, l, prm->relax_type[3], F[l], U[l], L->U2, 0);
         cudaMemcpyAsync(U[l], L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
      }
      else
      {
         int type = prm->relax_type[3];
         if (type == 11 || type == 12) { twostage_gs_d(amg, l, type == 11 ? 1 : 2, F[l], U[l], 1); }
         else if (type == 16) { cheby_d(amg, l, F[l], U[l], 1); }
         else if (hgs_type(type)) { hybrid_gs_d(amg, l, type, F[l], U[l], 1, 0); }
         else { relax_d(amg, l, type, F[l], U[l], U[l], 1); }
      }
   }
   for (int l = nl - 2; l >= 0; l--)
   {
      gb_level *L = &amg->lev[l];
      int type = prm->relax_type[2];
      /* u_f += P u_c written to U2, then the post-smoother writes back into U */
      gb_spmv_d(gb_solve_desc(L->P, GB_PREC_F64), U[l + 1], L->U2, 0, 1.0, 1.0, U[l], NULL, 0.0, NULL, NULL, s);
      if (cf && type != 16)
      {
         cudaMemcpyAsync(U[l], L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
         for (int sw = 0; sw < prm->num_sweeps[2]; sw++) { relax_cf_d(amg, l, type, 2, F[l], U[l], 0); }
         continue;
      }
      for (int sw = 0; sw < prm->num_sweeps[2]; sw++)
      {
         if (type == 11 || type == 12 || type == 16 || hgs_type(type))
         {
            if (sw == 0) { cudaMemcpyAsync(U[l], L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s); }
            if (type == 16) { cheby_d(amg, l, F[l], U[l], 0); }
            else if (hgs_type(type)) { hybrid_gs_d(amg, l, type, F[l], U[l], 0, 0); }
            else { twostage_gs_d(amg, l, type == 11 ? 1 : 2, F[l], U[l], 0); }
         }
         else
         {
            if (sw == 0) { relax_d(amg, l, type, F[l], L->U2, U[l], 0); }
            else
            {
               relax_d(amg, l, type, F[l], U[l], L->U2, 0);
               cudaMemcpyAsync(U[l], L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
            }
         }
      }
      if (prm->num_sweeps[2] == 0)
      {
         cudaMemcpyAsync(U[l], L->U2, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
      }
   }
}

/* FP32 cycle (FP16 finest values when requested): f0/u0 are FP64 */
static void relax_f(gb_amg *amg, int l, int type, const float *f, float *u_in, float *u_out, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   int vp = (amg->prm.cycle_prec == GB_PREC_F16 && l == 0) ? GB_PREC_F16 : GB_PREC_F32;
   const gb_spmv_desc *A = gb_solve_desc(L->A, vp);
   float w = (float) L->relax_w;
   (void) type;
   if (u_zero) { gb_scaled_div_f(L->n, w, f, L->l1f, u_out, s); }
   else { gb_spmv_f(A, u_in, u_out, 1, 0.f, 0.f, f, L->l1f, w, NULL, NULL, s); }
}

static void twostage_gs_f(gb_amg *amg, int l, int inner, const float *f, float *u, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   int vp = (amg->prm.cycle_prec == GB_PREC_F16 && l == 0) ? GB_PREC_F16 : GB_PREC_F32;
   const gb_spmv_desc *A = gb_solve_desc(L->A, vp);
   float w = (float) L->relax_w;
   float *V = L->Vf, *Z = L->U2f;
   if (u_zero) { gb_fill_f(L->n, u, 0.f, s); gb_scaled_copy_f(L->n, w, f, V, s); }
   else { gb_spmv_f(A, u, V, 0, -w, w, f, NULL, 0.f, NULL, NULL, s); }
   /* large levels: strictly lower part as SELL-32 (see twostage_gs_d); the
    * FP16 form has a unit diagonal in its values and a_ii in rs */
   const void *diag = NULL;
   const gb_spmv_desc *Lo = gb_lower_desc(L->A, vp, &diag);
   const float *d1 = vp == GB_PREC_F16 ? A->rs : (const float *) diag;
   if (Lo) { gb_gs_first_diag_f(L->n, d1, V, u, s); }
   else { gb_gs_first_f(L->n, L->A->A.i, A->v, vp, A->rs, V, u, s); }
   float m = -1.f;
   for (int k = 0; k < inner; k++)
   {
      if (Lo) { gb_spmv_f(Lo, V, Z, GB_EPI_GS, m, 0.f, u, (const float *) diag, 0.f, NULL, NULL, s); }
      else { gb_gs_lower_f(L->n, L->A->A.i, L->A->A.j, A->v, vp, V, Z, u, m, s); }
      float *t = V; V = Z; Z = t;
      m = -m;
   }
}

static void relax_points_f(gb_amg *amg, int l, int type, const float *f, float *u, int u_zero, int pts)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   if (type == 11 || type == 12) { twostage_gs_f(amg, l, type == 11 ? 1 : 2, f, u, u_zero); }
   else if (hgs_type(type)) { hybrid_gs_f(amg, l, type, f, u, u_zero, pts); }
   else
   {
      if (u_zero) { gb_fill_f(L->n, u, 0.f, s); }
      relax_f(amg, l, type, f, u, L->U2f, u_zero);
      gb_select_points_f(L->n, L->CF, pts, L->l1f, L->U2f, u, s);
   }
}

static void relax_cf_f(gb_amg *amg, int l, int type, int cycle_param, const float *f, float *u, int u_zero)
{
   const int p0 = cycle_param < 2 ? 1 : -1;
   relax_points_f(amg, l, type, f, u, u_zero, p0);
   relax_points_f(amg, l, type, f, u, 0, -p0);
}

static void relax_level_f(gb_amg *amg, int l, int type, int cycle_param, const float *f, float *u, int u_zero)
{
   gb_level *L = &amg->lev[l];
   cudaStream_t s = gb_stream();
   if (amg->prm.relax_order == 1 && amg->num_levels > 1 && cycle_param < 3 && type != 16)
   {
      relax_cf_f(amg, l, type, cycle_param, f, u, u_zero);
   }
   else if (type == 11 || type == 12) { twostage_gs_f(amg, l, type == 11 ? 1 : 2, f, u, u_zero); }
   else if (type == 16) { cheby_f(amg, l, f, u, u_zero); }
   else if (hgs_type(type)) { hybrid_gs_f(amg, l, type, f, u, u_zero, 0); }
   else if (u_zero) { relax_f(amg, l, type, f, u, u, 1); }
   else
   {
      relax_f(amg, l, type, f, u, L->U2f, 0);
      cudaMemcpyAsync(u, L->U2f, sizeof(float) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
   }
}

/* the FP32 form of cycle_gen_d, from a zero initial guess (f0d/u0d FP64) */
static void cycle_gen_f(gb_amg *amg, const double *f0d, double *u0d)
{
   gb_amg_params *prm = &amg->prm;
   cudaStream_t s = gb_stream();
   const int nl = amg->num_levels, ct = prm->cycle_type;
   float *F[32] = {0}, *U[32] = {0};
   int counter[32], zero[32];
   for (int l = 0; l < nl; l++) { F[l] = amg->lev[l].Ff; U[l] = amg->lev[l].Uf; }
   gb_d2f(amg->lev[0].n, f0d, F[0], s);
   counter[0] = 1;
   zero[0] = 1;
   for (int l = 1; l < nl; l++) { counter[l] = prm->fcycle ? 1 : ct; zero[l] = 0; }
   int fl = nl - 2, level = 0, cp = nl == 1 ? 3 : 1;
   for (;;)
   {
      gb_level *L = &amg->lev[level];
      const int vp = (prm->cycle_prec == GB_PREC_F16 && level == 0) ? GB_PREC_F16 : GB_PREC_F32;
      if (level == nl - 1)
      {
         if (amg->coarse_inv) { gb_dense_apply_f(amg->coarse_n, amg->coarse_inv, F[level], U[level], s); }
         else { relax_level_f(amg, level, prm->relax_type[3], 3, F[level], U[level], zero[level]); }
      }
      else
      {
         for (int sw = 0; sw < prm->num_sweeps[cp]; sw++)
         {
            relax_level_f(amg, level, prm->relax_type[cp], cp, F[level], U[level], zero[level] && sw == 0);
         }
      }
      zero[level] = 0;
      --counter[level];
      if (counter[level] >= 0 && level != nl - 1)
      {
         gb_spmv_f(gb_solve_desc(L->A, vp), U[level], L->Vf, 2, -1.f, 1.f, F[level], NULL, 0.f, NULL, NULL, s);
         gb_spmv_f(gb_solve_desc(L->R, GB_PREC_F32), L->Vf, F[level + 1], 0, 1.f, 0.f, NULL, NULL, 0.f, NULL, NULL,
                   s);
         cudaMemsetAsync(U[level + 1], 0, sizeof(float) * (size_t) amg->lev[level + 1].n, s);
         zero[level + 1] = 1;
         ++level;
         if (counter[level] < ct) { counter[level] = ct; }
         cp = level == nl - 1 ? 3 : 1;
      }
      else if (level != 0)
      {
         gb_level *Lf = &amg->lev[level - 1];
         gb_spmv_f(gb_solve_desc(Lf->P, GB_PREC_F32), U[level], Lf->U2f, 0, 1.f, 1.f, U[level - 1], NULL, 0.f, NULL,
                   NULL, s);
         cudaMemcpyAsync(U[level - 1], Lf->U2f, sizeof(float) * (size_t) Lf->n, cudaMemcpyDeviceToDevice, s);
         --level;
         cp = 2;
         if (prm->fcycle && fl == level)
         {
            if (counter[level] < 1) { counter[level] = 1; }
            fl--;
         }
      }
      else { break; }
   }
   gb_f2d(amg->lev[0].n, U[0], u0d, s);
}

static void cycle_f(gb_amg *amg, const double *f0d, double *u0d)
{
   gb_amg_params *prm = &amg->prm;
   if (prm->cycle_type != 1 || prm->fcycle) { cycle_gen_f(amg, f0d, u0d); return; }
   cudaStream_t s = gb_stream();
   int nl = amg->num_levels;
   const int cf = prm->relax_order == 1 && nl > 1;
   float *F[32] = {0}, *U[32] = {0};
   for (int l = 0; l < nl; l++) { F[l] = amg->lev[l].Ff; U[l] = amg->lev[l].Uf; }
   gb_d2f(amg->lev[0].n, f0d, F[0], s);
   for (int l = 0; l < nl - 1; l++)
   {
      gb_level *L = &amg->lev[l];
      int type = prm->relax_type[1];
      int vp = (prm->cycle_prec == GB_PREC_F16 && l == 0) ? GB_PREC_F16 : GB_PREC_F32;
      for (int sw = 0; sw < prm->num_sweeps[1]; sw++)
      {
         if (cf && type != 16) { relax_cf_f(amg, l, type, 1, F[l], U[l], sw == 0); }
         else if (type == 11 || type == 12) { twostage_gs_f(amg, l, type == 11 ? 1 : 2, F[l], U[l], sw == 0); }
         else if (type == 16) { cheby_f(amg, l, F[l], U[l], sw == 0); }
         else if (hgs_type(type)) { hybrid_gs_f(amg, l, type, F[l], U[l], sw == 0, 0); }
         else if (sw == 0) { relax_f(amg, l, type, F[l], U[l], U[l], 1); }
         else
         {
            relax_f(amg, l, type, F[l], U[l], L->U2f, 0);
            cudaMemcpyAsync(U[l], L->U2f, sizeof(float) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
         }
      }
      gb_spmv_f(gb_solve_desc(L->A, vp), U[l], L->Vf, 2, -1.f, 1.f, F[l], NULL, 0.f, NULL, NULL, s);
      gb_spmv_f(gb_solve_desc(L->R, GB_PREC_F32), L->Vf, F[l + 1], 0, 1.f, 0.f, NULL, NULL, 0.f, NULL, NULL, s);
   }
   {
      int l = nl - 1;
      if (amg->coarse_inv) { gb_dense_apply_f(amg->coarse_n, amg->coarse_inv, F[l], U[l], s); }
      else
      {
         int type = prm->relax_type[3];
         if (type == 11 || type == 12) { twostage_gs_f(amg, l, type == 11 ? 1 : 2, F[l], U[l], 1); }
         else if (type == 16) { cheby_f(amg, l, F[l], U[l], 1); }
         else if (hgs_type(type)) { hybrid_gs_f(amg, l, type, F[l], U[l], 1, 0); }
         else { relax_f(amg, l, type, F[l], U[l], U[l], 1); }
      }
   }
   for (int l = nl - 2; l >= 0; l--)
   {
      gb_level *L = &amg->lev[l];
      int type = prm->relax_type[2];
      gb_spmv_f(gb_solve_desc(L->P, GB_PREC_F32), U[l + 1], L->U2f, 0, 1.f, 1.f, U[l], NULL, 0.f, NULL, NULL, s);
      if (cf && type != 16)
      {
         cudaMemcpyAsync(U[l], L->U2f, sizeof(float) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
         for (int sw = 0; sw < prm->num_sweeps[2]; sw++) { relax_cf_f(amg, l, type, 2, F[l], U[l], 0); }
         continue;
      }
      for (int sw = 0; sw < prm->num_sweeps[2]; sw++)
      {
         if (type == 11 || type == 12 || type == 16 || hgs_type(type))
         {
            if (sw == 0) { cudaMemcpyAsync(U[l], L->U2f, sizeof(float) * (size_t) L->n, cudaMemcpyDeviceToDevice, s); }
            if (type == 16) { cheby_f(amg, l, F[l], U[l], 0); }
            else if (hgs_type(type)) { hybrid_gs_f(amg, l, type, F[l], U[l], 0, 0); }
            else { twostage_gs_f(amg, l, type == 11 ? 1 : 2, F[l], U[l], 0); }
         }
         else if (sw == 0) { relax_f(amg, l, type, F[l], L->U2f, U[l], 0); }
         else
         {
            relax_f(amg, l, type, F[l], U[l], L->U2f, 0);
            cudaMemcpyAsync(U[l], L->U2f, sizeof(float) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
         }
      }
      if (prm->num_sweeps[2] == 0)
      {
         cudaMemcpyAsync(U[l], L->U2f, sizeof(float) * (size_t) L->n, cudaMemcpyDeviceToDevice, s);
      }
   }
   gb_f2d(amg->lev[0].n, U[0], u0d, s);
}

static long long g_graph_kernels = 0;

/* One V-cycle from a zero initial guess: u = M^{-1} f.  Captured once per
 * (f, u, precision) as a CUDA graph and replayed. */
int gb_amg_cycle(gb_amg *amg, const double *f, double *u)
{
   cudaStream_t s = gb_stream();
   int prec = amg->prm.cycle_prec;
   if (amg->uses_hgs) { g_hgs_used = 1; }
   if (amg->prm.use_graph)
   {
      if (amg->graph && (amg->graph_f != f || amg->graph_u != u || amg->graph_prec != prec))
      {
         cudaGraphExecDestroy(amg->graph);
         amg->graph = NULL;
      }
      if (!amg->graph)
      {
         cudaGraph_t g;
         long long before = 0, after = 0;
         HYPRE_GB300_GetKernelLaunchCount(&before);
         if (!gb_cuda_ok(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture")) { return 1; }
         if (prec == GB_PREC_F64) { cycle_d(amg, f, u, 1); } else { cycle_f(amg, f, u); }
         if (!gb_cuda_ok(cudaStreamEndCapture(s, &g), "capture end")) { return 1; }
         if (!gb_cuda_ok(cudaGraphInstantiate(&amg->graph, g, 0), "graph instantiate")) { cudaGraphDestroy(g); return 1; }
         cudaGraphDestroy(g);
         HYPRE_GB300_GetKernelLaunchCount(&after);
         g_graph_kernels = after - before;
         gb_count_launch((int) -(after - before));   /* counted at replay */
         amg->graph_f = f; amg->graph_u = u; amg->graph_prec = prec;
      }
      gb_cuda_ok(cudaGraphLaunch(amg->graph, s), "graph launch");
      gb_count_launch((int) g_graph_kernels);
      return 0;
   }
   if (prec == GB_PREC_F64) { cycle_d(amg, f, u, 1); } else { cycle_f(amg, f, u); }
   return 0;
}

/* --------------------------------------------------------------------------
 * Public API
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *solver)
{
   if (!solver) { gb_error_in_arg(1); return gb_error_flag; }
   gb_runtime_init();
   gb_amg *a = (gb_amg *) calloc(1, sizeof(gb_amg));
   a->magic = GB_MAGIC_AMG;
   amg_defaults(&a->prm);
   *solver = (HYPRE_Solver) a;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGDestroy(HYPRE_Solver solver)
{
   gb_amg *a = (gb_amg *) solver;
   if (!a || a->magic != GB_MAGIC_AMG) { return gb_error_flag; }
   amg_free_hierarchy(a);
   gb_dfree(a->mlp_params);
   free(a->prm.level_relax_weight);
   a->magic = 0;
   free(a);
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{
   (void) b; (void) x;
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   return gb_amg_setup(a, A);
}

HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   if (!b || b->magic != GB_MAGIC_VEC) { gb_error_in_arg(3); return gb_error_flag; }
   if (!x || x->magic != GB_MAGIC_VEC) { gb_error_in_arg(4); return gb_error_flag; }
   if (!a->setup_done) { gb_error(HYPRE_ERROR_GENERIC, "BoomerAMGSolve before Setup"); return gb_error_flag; }
   int n = A->A.nr;
   cudaStream_t s = gb_stream();
   gb_amg_params *prm = &a->prm;
   /* hypre_BoomerAMGSolve (par_amg_solve.c:150-342): the relative residual
    * ||b - A x|| / ||b|| (absolute when b = 0; 1 when tol = 0) before the
    * loop and after every cycle; cycles while it is >= tol (or fewer than
    * min_iter ran) and fewer than max_iter ran; running into max_iter with
    * tol > 0 is a convergence error */
   const int check = prm->tol > 0.0;
   double *r = a->r_work;
   double rel = 1.0, rhs = 0.0;
   if (check)
   {
      gb_spmv_d(gb_solve_desc(A, GB_PREC_F64), x->d, r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, s);
      const double res = sqrt(gb_dot(n, r, r));
      rhs = sqrt(gb_dot(n, b->d, b->d));
      rel = rhs != 0.0 ? res / rhs : res;
   }
   int iter = 0;
   double *corr = prm->cycle_prec == GB_PREC_F64 ? NULL : (double *) gb_scratch(5, sizeof(double) * (size_t) n);
   while ((rel >= prm->tol || iter < prm->min_iter) && iter < prm->max_iter)
   {
      if (!corr)
      {
         /* FP64: the V-cycle on (b, x) in place, as the reference */
         cycle_d(a, b->d, x->d, 0);
      }
      else
      {
         /* FP32 / FP16 cycles: iterative refinement, x += M^{-1} (b - A x)
          * with the FP64 residual */
         gb_spmv_d(gb_solve_desc(A, GB_PREC_F64), x->d, r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, s);
         gb_amg_cycle(a, r, corr);
         gb_axpy_d(n, 1.0, corr, x->d, s);
      }
      iter++;
      if (check)
      {
         gb_spmv_d(gb_solve_desc(A, GB_PREC_F64), x->d, r, 2, -1.0, 1.0, b->d, NULL, 0.0, NULL, NULL, s);
         const double res = sqrt(gb_dot(n, r, r));
         rel = rhs != 0.0 ? res / rhs : res;
      }
   }
   if (check && iter == prm->max_iter) { gb_error(HYPRE_ERROR_CONV, NULL); }
   a->num_iterations = iter;
   a->rel_resid = rel;
   gb_amg_check_sweeps();
   return gb_error_flag;
}

/* preconditioner entry used by the Krylov drivers: x = M^{-1} b, x zero */
int gb_amg_precond(HYPRE_Solver solver, const double *b, double *x)
{
   gb_amg *a = (gb_amg *) solver;
   return gb_amg_cycle(a, b, x);
}

#define SETTER(name, field, type)                                  \
   HYPRE_Int name(HYPRE_Solver solver, type v)                      \
   {                                                                \
      gb_amg *a = amg_of(solver, 1);                                \
      if (a) { a->prm.field = v; }                                  \
      return gb_error_flag;                                         \
   }

SETTER(HYPRE_BoomerAMGSetTol, tol, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetMinIter, min_iter, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetMaxIter, max_iter, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetMaxCoarseSize, max_coarse_size, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetMinCoarseSize, min_coarse_size, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetStrongThreshold, strong_threshold, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetMaxRowSum, max_row_sum, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetAggNumLevels, agg_num_levels, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetTruncFactor, trunc_factor, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetPMaxElmts, p_max_elmts, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetAggInterpType, agg_interp_type, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetAggTruncFactor, agg_trunc_factor, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetAggPMaxElmts, agg_p_max_elmts, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetAggP12MaxElmts, agg_p12_max_elmts, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetAggP12TruncFactor, agg_p12_trunc_factor, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetChebyOrder, cheby_order, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetChebyFraction, cheby_fraction, HYPRE_Real)
SETTER(HYPRE_BoomerAMGSetChebyScale, cheby_scale, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetChebyVariant, cheby_variant, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetChebyEigEst, cheby_eig_est, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetPrintLevel, print_level, HYPRE_Int)
SETTER(HYPRE_BoomerAMGSetLogging, logging, HYPRE_Int)
SETTER(HYPRE_GB300_BoomerAMGSetUseGraph, use_graph, HYPRE_Int)
SETTER(HYPRE_GB300_BoomerAMGSetSetupTables, setup_tables, HYPRE_Int)

HYPRE_Int HYPRE_BoomerAMGSetMaxLevels(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v < 1) { gb_error_in_arg(2); return gb_error_flag; }
   a->prm.max_levels = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v != 8) { gb_error(HYPRE_ERROR_GENERIC, "coarsen_type: only PMIS (8) is supported"); gb_error_in_arg(2); return gb_error_flag; }
   a->prm.coarsen_type = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetInterpType(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v != 6 && v != 3 && v != 15 && v != 14 && v != 16 && v != 17 && v != 18)
   {
      gb_error(HYPRE_ERROR_GENERIC, "interp_type: extended+i (6), direct (3, 15), extended (14) and the modified "
                                    "16, 17, 18 are supported");
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   a->prm.interp_type = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetCycleType(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v != 1 && v != 2)
   {
      gb_error(HYPRE_ERROR_GENERIC, "cycle_type: V (1) and W (2) cycles are supported");
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   a->prm.cycle_type = v;
   return gb_error_flag;
}

/* second-order strength with one path (par_strength.c:2435-2526); the
 * path-counting form for num_paths > 1 is not built */
HYPRE_Int HYPRE_BoomerAMGSetNumPaths(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v != 1)
   {
      gb_error(HYPRE_ERROR_GENERIC, "num_paths: only 1 is supported");
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   a->prm.num_paths = v;
   return gb_error_flag;
}

/* outer weight omega of the hybrid Gauss-Seidel / SSOR smoothers on every
 * level (par_amg.c:2611-2634); the CG-estimated weights (omega < 0) are not
 * built */
HYPRE_Int HYPRE_BoomerAMGSetOuterWt(HYPRE_Solver solver, HYPRE_Real v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (!(v > 0.0))
   {
      gb_error(HYPRE_ERROR_GENERIC, "outer_wt: positive weights are supported");
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   a->prm.outer_weight = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetFCycle(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   a->prm.fcycle = v != 0;
   return gb_error_flag;
}

static int relax_supported(int t)
{
   return t == 18 || t == 7 || t == 11 || t == 12 || t == 16 || t == 9 || t == 99 || t == 19 || t == 98 ||
          hgs_type(t);
}

HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (!relax_supported(v)) { gb_error(HYPRE_ERROR_GENERIC, "relax_type not supported"); gb_error_in_arg(2); return gb_error_flag; }
   /* hypre_BoomerAMGSetRelaxType sets every cycle part, the coarsest to 9 only
    * when v is not a direct solve (par_amg.c: grid_relax_type[3] = 9 default kept) */
   a->prm.relax_type[0] = a->prm.relax_type[1] = a->prm.relax_type[2] = v;
   a->prm.relax_type[3] = 9;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetCycleRelaxType(HYPRE_Solver solver, HYPRE_Int v, HYPRE_Int k)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (k < 0 || k > 3) { gb_error_in_arg(3); return gb_error_flag; }
   if (!relax_supported(v)) { gb_error(HYPRE_ERROR_GENERIC, "relax_type not supported"); gb_error_in_arg(2); return gb_error_flag; }
   a->prm.relax_type[k] = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetRelaxOrder(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v != 0 && v != 1)
   {
      gb_error(HYPRE_ERROR_GENERIC, "relax_order: 0 (lexicographic) and 1 (C/F) are supported");
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   a->prm.relax_order = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetNumSweeps(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v < 0) { gb_error_in_arg(2); return gb_error_flag; }
   a->prm.num_sweeps[0] = a->prm.num_sweeps[1] = a->prm.num_sweeps[2] = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetCycleNumSweeps(HYPRE_Solver solver, HYPRE_Int v, HYPRE_Int k)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (k < 0 || k > 3) { gb_error_in_arg(3); return gb_error_flag; }
   a->prm.num_sweeps[k] = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetRelaxWt(HYPRE_Solver solver, HYPRE_Real v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   a->prm.relax_weight = v;
   free(a->prm.level_relax_weight);
   a->prm.level_relax_weight = NULL;
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGSetLevelRelaxWt(HYPRE_Solver solver, HYPRE_Real v, HYPRE_Int level)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (level < 0 || level >= 32) { gb_error_in_arg(3); return gb_error_flag; }
   if (!a->prm.level_relax_weight)
   {
      a->prm.level_relax_weight = (double *) malloc(sizeof(double) * 32);
      for (int l = 0; l < 32; l++) { a->prm.level_relax_weight[l] = a->prm.relax_weight; }
   }
   a->prm.level_relax_weight[level] = v;
   return gb_error_flag;
}

/* The coarse operator is the reference's host Galerkin product
 * (hypre_BoomerAMGBuildCoarseOperatorKT, par_amg_setup.c:3055-3066) and the
 * aggressive P1 P2 its hypre_ParMatmul; RAP2 (A P, then P^T (A P)) and the
 * modularized products (ModuleRAP2) sum in other orders and are not built, so
 * they are refused rather than ignored.  KeepTranspose changes nothing the
 * results depend on (the restriction multiplies by a stored P^T whose rows
 * are in the same order as the transposed product's sums). */
static HYPRE_Int refuse_nonzero(HYPRE_Solver solver, HYPRE_Int v, const char *what)
{
   if (!amg_of(solver, 1)) { return gb_error_flag; }
   if (v != 0)
   {
      gb_error(HYPRE_ERROR_GENERIC, what);
      gb_error_in_arg(2);
   }
   return gb_error_flag;
}
HYPRE_Int HYPRE_BoomerAMGSetRAP2(HYPRE_Solver solver, HYPRE_Int v)
{
   return refuse_nonzero(solver, v, "rap2: only the Galerkin triple product (0) is supported");
}
HYPRE_Int HYPRE_BoomerAMGSetModuleRAP2(HYPRE_Solver solver, HYPRE_Int v)
{
   return refuse_nonzero(solver, v, "module_rap2: only the host products (0) are supported");
}
HYPRE_Int HYPRE_BoomerAMGSetKeepTranspose(HYPRE_Solver solver, HYPRE_Int v) { (void) v; amg_of(solver, 1); return gb_error_flag; }

HYPRE_Int HYPRE_GB300_BoomerAMGSetCyclePrecision(HYPRE_Solver solver, HYPRE_Int v)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (v < 0 || v > 2) { gb_error_in_arg(2); return gb_error_flag; }
   a->prm.cycle_prec = v;
   if (a->graph) { cudaGraphExecDestroy(a->graph); a->graph = NULL; }
   if (a->setup_done)
   {
      for (int l = 0; l < a->num_levels; l++)
      {
         gb_level *L = &a->lev[l];
         int vp = v == GB_PREC_F64 ? GB_PREC_F64 : GB_PREC_F32;
         gb_solve_desc(L->A, (v == GB_PREC_F16 && l == 0) ? GB_PREC_F16 : vp);
         if (L->P) { gb_solve_desc(L->P, vp); gb_solve_desc(L->R, vp); }
      }
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGGetNumIterations(HYPRE_Solver solver, HYPRE_Int *n)
{
   gb_amg *a = amg_of(solver, 1);
   if (a && n) { *n = a->num_iterations; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGGetFinalRelativeResidualNorm(HYPRE_Solver solver, HYPRE_Real *r)
{
   gb_amg *a = amg_of(solver, 1);
   if (a && r) { *r = a->rel_resid; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGGetNumLevels(HYPRE_Solver solver, HYPRE_Int *n)
{
   gb_amg *a = amg_of(solver, 1);
   if (a && n) { *n = a->num_levels; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetSetupTimes(HYPRE_Solver solver, HYPRE_Real *t, HYPRE_Int n)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a || !t) { return gb_error_flag; }
   for (int k = 0; k < n && k < 8; k++) { t[k] = a->setup_times[k]; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelCSR(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int which, HYPRE_Int *nrows,
                                           HYPRE_Int *ncols, HYPRE_Int *nnz, HYPRE_Int *rowptr, HYPRE_Int *colidx,
                                           HYPRE_Real *values)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (level < 0 || level >= a->num_levels) { gb_error_in_arg(2); return gb_error_flag; }
   gb_level *L = &a->lev[level];
   gb_csr *M = NULL;
   if (which == 0) { M = &L->A->A; }
   else if (which == 1) { if (!L->P) { gb_error_in_arg(3); return gb_error_flag; } M = &L->P->A; }
   else if (which == 2) { if (!L->S.i) { gb_error_in_arg(3); return gb_error_flag; } M = &L->S; }
   else { gb_error_in_arg(3); return gb_error_flag; }
   if (nrows) { *nrows = M->nr; }
   if (ncols) { *ncols = M->nc; }
   if (nnz) { *nnz = M->nnz; }
   cudaStream_t s = gb_stream();
   if (rowptr) { cudaMemcpyAsync(rowptr, M->i, sizeof(int) * (size_t) (M->nr + 1), cudaMemcpyDeviceToHost, s); }
   if (colidx) { cudaMemcpyAsync(colidx, M->j, sizeof(int) * (size_t) M->nnz, cudaMemcpyDeviceToHost, s); }
   if (values && M->v) { cudaMemcpyAsync(values, M->v, sizeof(double) * (size_t) M->nnz, cudaMemcpyDeviceToHost, s); }
   gb_sync();
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelCF(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int *cf)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (level < 0 || level >= a->num_levels - 1 || !cf) { gb_error_in_arg(2); return gb_error_flag; }
   cudaMemcpyAsync(cf, a->lev[level].CF, sizeof(int) * (size_t) a->lev[level].n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   return gb_error_flag;
}

/* Times the solve-phase SpMV y = A_l x of one level in one value precision
 * (0 FP64, 1 FP32, 2 FP16 values with FP32 vectors): `reps` launches of the
 * level's solve form back to back on the library stream between two CUDA
 * events.  Returns the mean seconds per launch and the algorithmic bytes of
 * one launch: nnz * (value bytes + index bytes), x read once, y written
 * once, and the row pointers (CSR) or slice offsets and widths (SELL-32). */
HYPRE_Int HYPRE_GB300_BoomerAMGLevelSpMVTime(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int prec, HYPRE_Int reps,
                                             HYPRE_Real *seconds, HYPRE_Real *bytes)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (level < 0 || level >= a->num_levels) { gb_error_in_arg(2); return gb_error_flag; }
   if (prec < GB_PREC_F64 || prec > GB_PREC_F16) { gb_error_in_arg(3); return gb_error_flag; }
   if (reps < 1) { gb_error_in_arg(4); return gb_error_flag; }
   gb_level *L = &a->lev[level];
   const gb_spmv_desc *d = gb_solve_desc(L->A, prec);
   if (!d) { return gb_error_flag; }
   const int n = L->A->A.nr;
   const size_t xb = prec == GB_PREC_F64 ? 8 : 4;
   void *x = gb_dcalloc(xb * (size_t) (n > 0 ? n : 1)), *y = gb_dmalloc(xb * (size_t) (n > 0 ? n : 1));
   if (!x || !y) { gb_dfree(x); gb_dfree(y); return gb_error_flag; }
   cudaStream_t s = gb_stream();
   cudaEvent_t e0, e1;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   for (int r = -1; r < reps; r++)
   {
      if (r == 0) { cudaEventRecord(e0, s); }
      if (prec == GB_PREC_F64) { gb_spmv_d(d, (const double *) x, (double *) y, 0, 1.0, 0.0, NULL, NULL, 0.0, NULL, NULL, s); }
      else { gb_spmv_f(d, (const float *) x, (float *) y, 0, 1.0f, 0.0f, NULL, NULL, 0.0f, NULL, NULL, s); }
   }
   cudaEventRecord(e1, s);
   gb_sync();
   float ms = 0.f;
   cudaEventElapsedTime(&ms, e0, e1);
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   gb_dfree(x);
   gb_dfree(y);
   const double nnz = (double) L->A->A.nnz;
   double vb = prec == GB_PREC_F64 ? (d->fmt == GB_FMT_SELL && d->sl_v32 ? 4.0 : 8.0) : prec == GB_PREC_F32 ? 4.0 : 2.0;
   double ib = d->fmt == GB_FMT_SELL && d->sl_j16 ? 2.0 : 4.0;
   double meta = d->fmt == GB_FMT_SELL ? 12.0 * (double) d->nslices : 4.0 * ((double) n + 1.0);
   if (seconds) { *seconds = ms * 1e-3 / reps; }
   if (bytes) { *bytes = nnz * (vb + ib) + 2.0 * (double) xb * n + meta + (d->rs ? 4.0 * n : 0.0); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetSpGEMMStats(HYPRE_Solver solver, HYPRE_Real *bytes, HYPRE_Real *seconds,
                                              HYPRE_Int *calls)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (bytes) { *bytes = a->spgemm_bytes; }
   if (seconds) { *seconds = a->spgemm_seconds; }
   if (calls) { *calls = a->spgemm_calls; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelCheby(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Real *coefs,
                                             HYPRE_Real *eig, HYPRE_Real *ds)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (level < 0 || level >= a->num_levels) { gb_error_in_arg(2); return gb_error_flag; }
   gb_level *L = &a->lev[level];
   if (!L->cheb_ds) { gb_error(HYPRE_ERROR_GENERIC, "level has no Chebyshev smoother data"); return gb_error_flag; }
   if (coefs) { for (int k = 0; k < L->cheb_order; k++) { coefs[k] = L->cheb_c[k]; } }
   if (eig) { eig[0] = L->cheb_eig[0]; eig[1] = L->cheb_eig[1]; }
   if (ds)
   {
      cudaMemcpyAsync(ds, L->cheb_ds, sizeof(double) * (size_t) L->n, cudaMemcpyDeviceToHost, gb_stream());
      gb_sync();
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelL1(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Real *l1)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (level < 0 || level >= a->num_levels || !l1) { gb_error_in_arg(2); return gb_error_flag; }
   cudaMemcpyAsync(l1, a->lev[level].l1, sizeof(double) * (size_t) a->lev[level].n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   return gb_error_flag;
}

/* ------------------------------------------------------------------------
 * Getters of the parameters above (HYPRE_parcsr_ls.h), and settings that
 * have one supported value: anything else is refused, not ignored.
 * Output-only settings (debug flag, sequential threshold of the multi-process
 * coarse solve) are accepted.
 * ------------------------------------------------------------------------ */
#define GETTER(name, field, type)                                  \
   HYPRE_Int name(HYPRE_Solver solver, type *v)                     \
   {                                                                \
      gb_amg *a = amg_of(solver, 1);                                \
      if (!a) { return gb_error_flag; }                             \
      if (!v) { gb_error_in_arg(2); return gb_error_flag; }         \
      *v = (type) a->prm.field;                                     \
      return gb_error_flag;                                         \
   }
GETTER(HYPRE_BoomerAMGGetMaxIter, max_iter, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetTol, tol, HYPRE_Real)
GETTER(HYPRE_BoomerAMGGetCycleType, cycle_type, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetFCycle, fcycle, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetStrongThreshold, strong_threshold, HYPRE_Real)
GETTER(HYPRE_BoomerAMGGetMaxRowSum, max_row_sum, HYPRE_Real)
GETTER(HYPRE_BoomerAMGGetPMaxElmts, p_max_elmts, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetTruncFactor, trunc_factor, HYPRE_Real)
GETTER(HYPRE_BoomerAMGGetMaxLevels, max_levels, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetMaxCoarseSize, max_coarse_size, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetMinCoarseSize, min_coarse_size, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetCoarsenType, coarsen_type, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetPrintLevel, print_level, HYPRE_Int)
GETTER(HYPRE_BoomerAMGGetLogging, logging, HYPRE_Int)
#undef GETTER

/* k: 1 down, 2 up, 3 coarsest (HYPRE_parcsr_ls.h:821, :907) */
HYPRE_Int HYPRE_BoomerAMGGetCycleNumSweeps(HYPRE_Solver solver, HYPRE_Int *num_sweeps, HYPRE_Int k)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (!num_sweeps) { gb_error_in_arg(2); return gb_error_flag; }
   if (k < 1 || k > 3) { gb_error_in_arg(3); return gb_error_flag; }
   *num_sweeps = a->prm.num_sweeps[k];
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGGetCycleRelaxType(HYPRE_Solver solver, HYPRE_Int *relax_type, HYPRE_Int k)
{
   gb_amg *a = amg_of(solver, 1);
   if (!a) { return gb_error_flag; }
   if (!relax_type) { gb_error_in_arg(2); return gb_error_flag; }
   if (k < 1 || k > 3) { gb_error_in_arg(3); return gb_error_flag; }
   *relax_type = a->prm.relax_type[k];
   return gb_error_flag;
}

HYPRE_Int HYPRE_BoomerAMGGetNumFunctions(HYPRE_Solver solver, HYPRE_Int *num_functions)
{
   if (!amg_of(solver, 1)) { return gb_error_flag; }
   if (!num_functions) { gb_error_in_arg(2); return gb_error_flag; }
   *num_functions = 1;
   return gb_error_flag;
}

static HYPRE_Int only_value(HYPRE_Solver solver, HYPRE_Int v, HYPRE_Int ok, const char *what)
{
   if (!amg_of(solver, 1)) { return gb_error_flag; }
   if (v != ok)
   {
      gb_error(HYPRE_ERROR_GENERIC, what);
      gb_error_in_arg(2);
   }
   return gb_error_flag;
}
HYPRE_Int HYPRE_BoomerAMGSetNumFunctions(HYPRE_Solver solver, HYPRE_Int v)
{
   return only_value(solver, v, 1, "num_functions: scalar problems (1) are supported");
}
HYPRE_Int HYPRE_BoomerAMGSetNodal(HYPRE_Solver solver, HYPRE_Int v)
{
   return only_value(solver, v, 0, "nodal: only 0 is supported");
}
HYPRE_Int HYPRE_BoomerAMGSetMeasureType(HYPRE_Solver solver, HYPRE_Int v)
{
   return only_value(solver, v, 0, "measure_type: only local measures (0) are supported");
}
HYPRE_Int HYPRE_BoomerAMGSetRedundant(HYPRE_Solver solver, HYPRE_Int v)
{
   return only_value(solver, v, 0, "redundant: only 0 is supported");
}
HYPRE_Int HYPRE_BoomerAMGSetCoarsenCutFactor(HYPRE_Solver solver, HYPRE_Int v)
{
   return only_value(solver, v, 0, "coarsen_cut_factor: only 0 is supported");
}
HYPRE_Int HYPRE_BoomerAMGSetConvergeType(HYPRE_Solver solver, HYPRE_Int v)
{
   return only_value(solver, v, 0, "converge_type: only the relative residual (0) is supported");
}
HYPRE_Int HYPRE_BoomerAMGSetDebugFlag(HYPRE_Solver solver, HYPRE_Int v)
{
   (void) v;
   amg_of(solver, 1);
   return gb_error_flag;
}
HYPRE_Int HYPRE_BoomerAMGSetSeqThreshold(HYPRE_Solver solver, HYPRE_Int v)
{
   (void) v;
   amg_of(solver, 1);
   return gb_error_flag;
}
