/* Launchers of the sm_103a kernels (gb_setup.cu, gb_solve.cu), called by the
 * C host code.  All pointers are device pointers unless named h_*; every
 * launcher enqueues on the given stream and returns immediately unless it
 * says it synchronises. */
#ifndef GB_KERNELS_H
#define GB_KERNELS_H

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* SpMV epilogue modes: y = alpha*Ax + beta*b (0), Jacobi (1), residual b - Ax (2),
 * Chebyshev: d.*(b - Ax) (3), d.*(alpha*b + d.*Ax) (4), y + d.*(alpha*b + d.*Ax) (5) */
#define GB_EPI_AXPBY 0
#define GB_EPI_JACOBI 1
#define GB_EPI_RESID 2
#define GB_EPI_CHEB_RES 3
#define GB_EPI_CHEB_STEP 4
#define GB_EPI_CHEB_LAST 5
#define GB_EPI_GS 6            /* y = s / d_i (s when d is NULL), b_i += alpha * y_i */
#define GB_PREC_F64 0
#define GB_PREC_F32 1
#define GB_PREC_F16 2

#define GB_FMT_CSR 0
#define GB_FMT_SELL 1

/* blocks of every reduction kernel (fixed so sums are deterministic) */
#define GB_RED_BLOCKS 1216

/* solve-phase view of a sparse matrix */
typedef struct
{
   int        n;         /* rows */
   int        fmt;       /* GB_FMT_* */
   int        vprec;     /* GB_PREC_* of v / sl_v */
   int        K;         /* lanes per row (CSR) */
   const int *i, *j;     /* CSR */
   const void *v;        /* CSR values in vprec */
   int        nslices;   /* SELL-32 */
   const long long *sl_ptr;
   const int *sl_w;
   const int *sl_j;
   const short *sl_j16;  /* 16-bit offsets from the row instead of sl_j (NULL: sl_j) */
   const void *sl_v;
   int        sl_v32;    /* FP64 form whose SELL values are held as FP32 (every value exact in FP32) */
   const float *rs;      /* FP16 forms: values are a_ij / a_ii, rs[i] = a_ii (NULL otherwise) */
   int        tuneT;     /* autotuned block size (0: default 256) */
   int        tuneD;     /* autotuned SELL prefetch depth (0: default 4) */
} gb_spmv_desc;

/* runtime */
void gb_count_launch(int n);
int  gb_num_sms(void);

/* scan / setup */
long long gb_scan_scratch_ints(int n);
void gb_exclusive_scan(const int *in, int *out, int n, int *scratch, cudaStream_t s);
/* rkey: n per-row threshold keys written by the count, read by the fill */
void gb_strength_count(int n, const int *Ai, const double *Av, double theta, double mrs, int *cnt, long long *rkey,
                       cudaStream_t s);
void gb_strength_fill(int n, const int *Ai, const int *Aj, const double *Av, const long long *rkey, const int *Si,
                      int *Sj, cudaStream_t s);
/* nnz = Si[n]; d_counter: 4 device ints; h_counter: 2 pinned host ints */
int  gb_pmis(int n, int nnz, const int *Si, const int *Sj, int CF_init, int *CF, double *measure, int *ingraph,
             int *colcnt, int *d_counter, int *h_counter, int max_iter, cudaStream_t s);   /* synchronises */
void gb_cpoint_flags(int n, const int *CF, int *flag, cudaStream_t s);
void gb_sf_to_f(int n, int *CF, cudaStream_t s);
void gb_extpi_ub(int n, const int *Si, const int *Sj, const int *CF, int *ub, cudaStream_t s);
void gb_extpi_count(int nrows, const int *rows, const int *Si, const int *Sj, const int *CF, int *cnt,
                    const int *in_list, const int *in_n, int n_hint, int *out_list, int *out_n, int *gtab, int gcap,
                    int gwarps, int *err, int tier, cudaStream_t s);
void gb_extpi_fill(int nrows, const int *rows, const int *Ai, const int *Aj, const double *Av, const int *Si,
                   const int *Sj, const int *CF, const int *f2c, const int *Pi, int *Pj, double *Pv,
                   const int *in_list, const int *in_n, int n_hint, int *gtab, int gcap, int gwarps, int *err,
                   int tier, int iterm, cudaStream_t s);
void gb_iota(int n, int *out, int *count, cudaStream_t s);
void gb_count_empty_rows(int n, const int *Ai, int *count, cudaStream_t s);
void gb_dir_count(int n, const int *Si, const int *Sj, const int *CF, int *cnt, cudaStream_t s);
void gb_dir_fill(int n, const int *Ai, const int *Aj, const double *Av, const int *Si, const int *Sj, const int *CF,
                 const int *f2c, const int *Pi, int *Pj, double *Pv, double *alfa, double *beta, int *flags,
                 cudaStream_t s);
void gb_extpi_count_t(int nrows, const int *rows, const int *Si, const int *Sj, const int *CF, const int *f2c,
                      int *cnt, int *ovf_list, int *ovf_n, cudaStream_t s);
void gb_extpi_fill_t(int nrows, const int *rows, const int *Ai, const int *Aj, const double *Av, const int *Si,
                     const int *Sj, const int *CF, const int *f2c, const int *Pi, int *Pj, double *Pv, int iterm,
                     cudaStream_t s);
void gb_truncate_rows(int n, const int *Pi, int *Pj, double *Pv, double tol, int max_elmts, int *newcnt,
                      cudaStream_t s);
void gb_compact_rows(int n, const int *Pi, const int *Pj, const double *Pv, const int *Ni, int *Nj, double *Nv,
                     cudaStream_t s);
void gb_transpose_count(int nnz, const int *Aj, int *cnt, cudaStream_t s);
void gb_transpose_fill(int nr, int nc, const int *Ai, const int *Aj, const double *Av, int *fill, const int *Ti,
                       int *Tj, double *Tv, cudaStream_t s);
void gb_spgemm_ub(int nrows, int ncols, int square, const int *Ai, const int *Aj, const int *Bi, int *ub,
                  cudaStream_t s);
/* ordered sparse product, tier 0 (small shared tables, all rows; with ub,
 * rows whose upper bound exceeds the table go straight to the list), 1 (large
 * shared tables, rows in ovf_list, overflow to out_list) or 2 (global tables,
 * rows in ovf_list); phase 0 symbolic, 1 numeric */
#define GB_SPGEMM_TINY_COLS 192   /* list capacity of numeric tier 3 */
void gb_spgemm(int nrows, int square, int W, const int *Ai, const int *Aj, const double *Av, const int *Bi,
               const int *Bj, const double *Bv, int *cnt, const int *Ci, int *Cj, double *Cv, int *ovf_list,
               int *ovf_n, int *out_list, int *out_n, int nlist, int *gtab, int gcap, int gwarps, int *err,
               const int *ub, int *src, int fbase, int phase, int tier, cudaStream_t s);
/* phase 2 (tiers 0 and 1): count and fill in one pass into temporary areas
 * (tier 0 at Ci[r], tier 1 at fbase + t * 1536), cnt[r] and src[r] set;
 * gb_spgemm_cap sizes the areas, gb_spgemm_gather moves rows into place */
void gb_spgemm_cap(int n, int ncols, int square, const int *Ai, const int *Aj, const int *Bi, int lcap0, int *ub,
                   int *cap, unsigned long long *sum, int *over, cudaStream_t s);
void gb_spgemm_gather(int n, long long nnz, const int *Ci, const int *src, const int *tj, const double *tv, int *Cj,
                      double *Cv, cudaStream_t s);
void gb_spgemm_rc(int nrows, int square, const int *Ai, const int *Aj, const double *Av, const int *Bi, const int *Bj,
                  const double *Bv, int *cnt, const int *Ci, int *Cj, double *Cv, int *ovf_list, int *ovf_n,
                  int *out_list, int *out_n, int nlist, int *err, const int *ub, int *src, int fbase, int phase,
                  int tier, cudaStream_t s);
/* IJ matrix device assembly (gb_ijdev.cu) */
void gb_ij_check(int nrows, const int *start, const int *cols, int ncol, int *flags, cudaStream_t s);
void gb_ij_gather(int n, long long nnz, const long long *off, const int *I, const int *scols, const double *svals,
                  int swap_diag, const int *key, int *J, double *V, cudaStream_t s);
void gb_rowlen_max(int n, const int *Bi, int *out, cudaStream_t s);
/* aggressive coarsening (gb_agg.cu) */
void gb_flags(int n, const int *CF, int kind, int v, int *flag, cudaStream_t s);
void gb_list_flags(int nlist, const int *dcount, const int *list, int *flag, cudaStream_t s);
void gb_scatter_list(int n, const int *flag, const int *scan, int *list, cudaStream_t s);
/* second-order strength: the candidate lists (Lj NULL: counts into cnt;
 * else the lists at Li), then the rows */
void gb_s2_lists(int n, const int *Si, const int *Sj, const int *CF, const int *f2c, int *cnt, const int *Li,
                 int *Lj, cudaStream_t s);
void gb_strength2(int nc, const int *c2f, const int *Li, const int *Lj, const int *Si, const int *Sj, int *cnt,
                  const int *S2i, int *S2j, int *ovf_list, int *ovf_n, int *gtab, int gcap, int gwarps, int *err,
                  int *src, int fill, int tier, cudaStream_t s);
void gb_strength2_ub(int nc, const int *c2f, const int *Si, const int *Sj, const int *Li, int *ub, cudaStream_t s);
void gb_cap_sum(int n, const int *ub, int lcap, int *cap, unsigned long long *sum, cudaStream_t s);
void gb_mark_isolated(int nc, const int *c2f, const int *cnt, int *CF, cudaStream_t s);
void gb_correct_cf2(int n, const int *f2c, const int *CFN, int *CF, cudaStream_t s);
void gb_cf_clamp(int n, int *CF, cudaStream_t s);
/* multipass interpolation (gb_multipass.cu): the areas of the passes' rows */
#define GB_MP_MAXP 10
typedef struct
{
   int    *j[GB_MP_MAXP];
   double *v[GB_MP_MAXP];
} gb_mp_areas;
void gb_correct_cf(int n, const int *f2c, const int *CFN, int *CF, cudaStream_t s);
void gb_mp_pass(int n, const int *Si, const int *Sj, const int *CF, int p, int *assigned, int *count,
                cudaStream_t s);
void gb_mp_bound(int m, const int *rows, const int *Si, const int *Sj, const int *assigned, int p,
                 const int *rowlen, int *ub, unsigned long long *total, cudaStream_t s);
void gb_mp_rows(int m, const int *rows, const int *off, int p, const int *Ai, const int *Aj, const double *Av,
                const int *Si, const int *Sj, const int *CF, const int *f2c, const int *assigned, const int *qj,
                const double *qv, int *pj, double *pv, int *rowoff, int *rowlen, double *alfa, int *degen,
                int *ndegen, cudaStream_t s);
void gb_mp_carry1(int m, const int *fl, const int *assigned, const int *degen, const double *alfa,
                  const int *rowoff, const int *rowlen, double *pv, cudaStream_t s);
void gb_mp_len(int n, const int *CF, const int *assigned, const int *rowlen, int *len, cudaStream_t s);
void gb_mp_gather(int n, const int *CF, const int *assigned, const int *f2c, const int *rowoff,
                  const gb_mp_areas *areas, const int *Pi, int *Pj, double *Pv, cudaStream_t s);
/* multipass interpolation in product form (gb_multipass.cu): the blocks of
 * passes 2 .. nblk+1 (rows: the pass's points in row order) */
#define GB_MMP_MAXB 8
typedef struct
{
   const int    *i[GB_MMP_MAXB];
   const int    *j[GB_MMP_MAXB];
   const double *v[GB_MMP_MAXB];
   int           nblk;
} gb_mmp_blocks;
void gb_mmp_init(int n, const int *CF, int *pass, int *count, cudaStream_t s);
void gb_mmp_round(int n, const int *Si, const int *Sj, int cur, int *pass, int *count, cudaStream_t s);
void gb_mmp_col(int n, const int *pass, int p, const int *scan, int *col, cudaStream_t s);
void gb_mmp_rowsum(int n, const int *CF, const int *Ai, const double *Av, double *rsum, cudaStream_t s);
void gb_mmp_count(int m, const int *rows, const int *Si, const int *Sj, const int *pass, int color, int *cnt,
                  cudaStream_t s);
void gb_mmp_fill(int m, const int *rows, const int *Ai, const int *Aj, const double *Av, const int *Si,
                 const int *Sj, const int *pass, const int *col, int color, const int *Qi, int *Qj, double *Qv,
                 const double *rsum, double *w, cudaStream_t s);
void gb_mmp_scale9(int m, const int *rows, const int *Ai, const double *Av, const int *Bi, double *Bv,
                   const double *w, cudaStream_t s);
void gb_mmp_len(int n, const int *CF, const int *pass, const int *col, const gb_mmp_blocks *B, int *len,
                cudaStream_t s);
void gb_mmp_gather(int n, const int *CF, const int *pass, const int *col, const gb_mmp_blocks *B, const int *Pi,
                   int *Pj, double *Pv, cudaStream_t s);
void gb_fffc_count(int nf, const int *fl, const int *Ai, const int *Aj, const int *Si, const int *Sj, const int *CF,
                   int *cff, int *cfc, cudaStream_t s);
/* nrows, nnz: A's size (the mean row length picks the lanes per row) */
void gb_fffc_fill(int nf, int nrows, long long nnz, const int *fl, const int *Ai, const int *Aj, const double *Av,
                  const int *Si, const int *Sj, const int *CF, const int *f2c, const int *f2f, const int *FFi,
                  int *FFj, double *FFv, const int *FCi, int *FCj, double *FCv, cudaStream_t s);
void gb_mod_extpi_scale(int nf, int nnzff, const int *fl, const int *Ai, const double *Av, const int *FFi,
                        const int *FFj, double *FFv, const int *FCi, const double *FCv, double *tmp, double *Dq,
                        double *Dw, cudaStream_t s);
void gb_modp_scale(int variant, int nf, int nn, const int *nl, const int *f2f, const int *Ai, const double *Av,
                   const int *FFai, const double *FFav, const int *FCi, double *FCv, const int *FFi, const int *FFj,
                   double *FFv, double *Dq, double *Dl, double *Dinv, cudaStream_t s);
void gb_modp_len(int nco, const int *oc, const int *CF, const int *nscan, const int *Wi, int *len, cudaStream_t s);
void gb_modp_gather(int nco, const int *oc, const int *CF, const int *f2c, const int *nscan, const int *Wi,
                    const int *Wj, const double *Wv, const int *Pi, int *Pj, double *Pv, cudaStream_t s);
void gb_mod_interp_scale(int variant, int nf, int nnzff, const int *fl, const int *Ai, const double *Av,
                         const int *FFi, const int *FFj, double *FFv, const int *FCi, double *FCv, double *tmp,
                         double *D1, double *D2, double *D3, double *D4, cudaStream_t s);
void gb_p1_len(int n, const int *CF, const int *f2f, const int *Wi, int *len, cudaStream_t s);
void gb_p1_fill(int n, const int *CF, const int *f2c, const int *f2f, const int *Wi, const int *Wj, const double *Wv,
                const int *Pi, int *Pj, double *Pv, cudaStream_t s);
void gb_l1_norms(int n, const int *Ai, const int *Aj, const double *Av, int option, const int *CF, double *l1,
                 cudaStream_t s);
void gb_block_inverse(int nsys, const int *off, const int *Ai, const int *Aj, const double *Av,
                      const long long *doff, double *D, double *W, cudaStream_t s);
void gb_dense_inverse(int n, const int *Ai, const int *Aj, const double *Av, double *D, double *W, cudaStream_t s);

/* hybrid Gauss-Seidel sweep (gb_hgs.cu): dir +1 forward, -1 backward; uo
 * receives u's values from before the sweep; ut: the scaled form's starting
 * values (NULL: unscaled); dvec: l1 norms or NULL (diagonal); flags: n + 1
 * ints; *err set when a dependency wait ran out */
void gb_hgs_sweep_d(int n, long long nnz, const int *Ai, const int *Aj, const double *Av, const double *f,
                    double *u, double *uo, const double *ut, const double *dvec, int dir, int skip, double w,
                    double omega, const int *cf, int pts, int *flags, int *err, cudaStream_t s);
void gb_hgs_sweep_f(int n, long long nnz, const int *Ai, const int *Aj, const float *Av, const float *f, float *u,
                    float *uo, const float *ut, const float *dvec, int dir, int skip, double w, double omega,
                    const int *cf, int pts, int *flags, int *err, cudaStream_t s);
/* u[i] = t[i] where CF[i] == pts and d[i] != 0 (the points a C/F Jacobi
 * half-relaxation updates) */
void gb_select_points_d(int n, const int *CF, int pts, const double *d, const double *t, double *u, cudaStream_t s);
void gb_select_points_f(int n, const int *CF, int pts, const float *d, const float *t, float *u, cudaStream_t s);

/* solve phase */
void gb_spmv_d(const gb_spmv_desc *A, const double *x, double *y, int mode, double alpha, double beta,
               const double *b, const double *d, double w, const double *dotz, double *dpart, cudaStream_t st);
void gb_spmv_f(const gb_spmv_desc *A, const float *x, float *y, int mode, float alpha, float beta, const float *b,
               const float *d, float w, const float *dotz, double *dpart, cudaStream_t st);
/* stage 0: widths, offsets and *wide (1 when some |j - i| >= 2^15); stage 1:
 * indices into sl_j, or as offsets into sl_j16 when that is given */
void gb_sell_struct(int n, const int *Ai, const int *Aj, int lower, int nslices, int *sl_w, long long *sl_ptr,
                    int *sl_j, short *sl_j16, int *wide, cudaStream_t s, int stage);
void gb_sell_vals(int n, const int *Ai, const int *Aj, const double *Av, int lower, int scaled, int vprec, int nslices,
                  const int *sl_w, const long long *sl_ptr, void *sl_v, cudaStream_t s);
void gb_convert_vals(long long nnz, const double *in, void *out, int vprec, cudaStream_t s);
/* *flag = 1 unless every value is zero or a normal FP32 number exactly */
void gb_exact32(long long nnz, const double *v, int *flag, cudaStream_t s);
void gb_row_scaled_half(int n, const int *Ai, const double *Av, void *out, float *rs, cudaStream_t s);
void gb_gs_first_d(int n, const int *Ai, const double *Av, double *v, double *u, cudaStream_t s);
void gb_gs_first_f(int n, const int *Ai, const void *Av, int vprec, const float *rs, float *v, float *u,
                   cudaStream_t s);
/* diagonal entries, and the first stage of the two-stage Gauss-Seidel sweep
 * with a diagonal array */
void gb_diag_vals(int n, const int *Ai, const double *Av, int vprec, void *out, cudaStream_t s);
void gb_gs_first_diag_d(int n, const double *diag, double *v, double *u, cudaStream_t s);
void gb_gs_first_diag_f(int n, const float *diag, float *v, float *u, cudaStream_t s);
void gb_gs_lower_d(int n, const int *Ai, const int *Aj, const double *Av, const double *z, double *znew, double *u,
                   double m, cudaStream_t s);
void gb_gs_lower_f(int n, const int *Ai, const int *Aj, const void *Av, int vprec, const float *z, float *znew,
                   float *u, float m, cudaStream_t s);

void gb_rand_uniform(int n, int seed, double *v, cudaStream_t s);
void gb_diag_inv_sqrt(int n, const int *Ai, const int *Aj, const double *Av, double *ds, cudaStream_t s);
void gb_cheb_start_d(long long n, double c, const double *r, const double *d, double *q, cudaStream_t s);
void gb_cheb_start_f(long long n, float c, const float *r, const float *d, float *q, cudaStream_t s);
void gb_cheb_order1_d(long long n, double c, const double *r, const double *d, double *u, cudaStream_t s);
void gb_cheb_order1_f(long long n, float c, const float *r, const float *d, float *u, cudaStream_t s);
void gb_vmul_d(long long n, const double *a, const double *b, double *c, cudaStream_t s);
void gb_vmul_f(long long n, const float *a, const float *b, float *c, cudaStream_t s);

void gb_fill_d(long long n, double *x, double v, cudaStream_t s);
/* batched persistent AMG-PCG (gb_batch.cu) */
void gb_check_blockdiag(int n, const int *Ai, const int *Aj, const int *off, int nsys, int *bad, cudaStream_t s);
void gb_batch_pcg(const void *lev_dev, int nlev, int nsys, int sweeps_down, int sweeps_up, const int *Ai,
                  const int *Aj, const double *Av, const int *order, int *counter, const double *b, double *x,
                  double *r, double *p, double *sv, const double *Dinv, const long long *doff, double tol, int maxit,
                  int *iters,
                  double *relres, double *hist, int prec, int lpr, int grid, int block, cudaStream_t s);
size_t gb_blevel_size(void);
/* learned parameters (gb_mlp.cu) */
int gb_mlp_nparam(void);
int gb_mlp_nbw(void);
int gb_mlp_grid(void);
void gb_mlp_pack(const float *P, void *W, cudaStream_t s);
void gb_mlp_forward(long long N, const void *X, const void *W, const float *P, float *out, cudaStream_t s);
int gb_mlp_grad(long long N, const void *X, const float *T, const void *W, const float *P, float *part,
                float *loss_part, float *grad, float *loss, cudaStream_t s);
void gb_mlp_adam(float *P, const float *grad, float *m, float *v, float lr, float b1, float b2, float eps, int step,
                 cudaStream_t s);
void gb_row_features(int n, const int *Ai, const int *Aj, const double *Av, void *X, cudaStream_t s);
void gb_mean2(long long N, const float *out, double *res, cudaStream_t s);
void gb_blevel_set(void *host_array, int l, int n, const int *Ai, const int *Aj, const void *Av, const int *Pi,
                   const int *Pj, const void *Pv, const int *Ri, const int *Rj, const void *Rv, const void *l1,
                   void *F, void *U, void *V, const int *off, double w);
void gb_fill_f(long long n, float *x, float v, cudaStream_t s);
void gb_scale_d(long long n, double a, double *x, cudaStream_t s);
void gb_axpy_d(long long n, double a, const double *x, double *y, cudaStream_t s);
void gb_xpay_d(long long n, const double *x, double a, double *y, cudaStream_t s);
void gb_scaled_div_d(long long n, double w, const double *f, const double *d, double *u, cudaStream_t s);
void gb_scaled_div_f(long long n, float w, const float *f, const float *d, float *u, cudaStream_t s);
void gb_scaled_copy_d(long long n, double w, const double *f, double *v, cudaStream_t s);
void gb_scaled_copy_f(long long n, float w, const float *f, float *v, cudaStream_t s);
void gb_d2f(long long n, const double *a, float *b, cudaStream_t s);
void gb_f2d(long long n, const float *a, double *b, cudaStream_t s);
/* dot products in one launch: the last block to finish sums the partials
 * (count: a zeroed counter, reset by that block) */
void gb_dot_d(long long n, const double *x, const double *y, double *part, unsigned int *count, double *out,
              cudaStream_t s);
void gb_axpy_dot_dev_d(long long n, const double *h, const double *x, double *y, const double *z, double *part,
                       unsigned int *count, double *out, cudaStream_t s);
void gb_axpy_dot_d(long long n, double a, const double *x, double *y, const double *z, double *part, double *out,
                   cudaStream_t s);
void gb_dot2_d(long long n, const double *x, const double *y, const double *z, double *part, double *out,
               cudaStream_t s);
void gb_pcg_xr_d(long long n, double a, const double *p, const double *sv, double *x, double *r, double *part,
                 double *out, cudaStream_t s);
void gb_final_sum(int nparts, int nsums, const double *part, double *out, cudaStream_t s);
void gb_dense_apply_d(int n, const double *D, const double *f, double *u, cudaStream_t s);
void gb_dense_apply_f(int n, const double *D, const float *f, float *u, cudaStream_t s);

#ifdef __cplusplus
}
#endif
#endif
