/* CPU oracle for the BoomerAMG-preconditioned Krylov path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * library's serial CPU algorithms (each function cites the reference file:line
 * it follows).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it, and only as the checker or the timed CPU baseline;
 * the product library never links or calls it.
 *
 * Parity is pinned against the reference library itself, compiled from its
 * sources by oracle/ref/Makefile (golden fixtures under tests/golden/).
 */
#ifndef AMG_ORACLE_H
#define AMG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
   int     nr, nc;
   int    *i;      /* nr+1 */
   int    *j;      /* nnz  */
   double *v;      /* nnz (may be NULL for a pattern) */
} or_csr;

typedef struct
{
   /* setup */
   double strong_threshold;   /* 0.25 */
   double max_row_sum;        /* 0.9 library default, 1.0 as the reference's ij driver sets */
   double trunc_factor;       /* 0.0 */
   int    p_max_elmts;        /* 4 */
   int    interp_type;        /* 6 = extended+i */
   int    coarsen_type;       /* 8 = PMIS */
   int    agg_num_levels;     /* 0 */
   int    agg_interp_type;    /* 4 */
   int    agg_p_max_elmts;    /* 0 */
   int    agg_p12_max_elmts;  /* 0 */
   double agg_trunc_factor;   /* 0 */
   double agg_p12_trunc_factor; /* 0 */
   int    num_paths;          /* 1 */
   int    max_levels;         /* 25 */
   int    max_coarse_size;    /* 9 */
   int    min_coarse_size;    /* 0 */
   /* cycle */
   int    relax_down, relax_up, relax_coarse; /* 18, 18, 9 */
   int    num_sweeps;         /* 1 */
   double relax_weight;       /* 1.0 */
   int    cheby_order;        /* 2 */
   double cheby_fraction;     /* 0.3 */
   int    cheby_scale;        /* 1 */
   int    cheby_variant;      /* 0 */
   int    cheby_eig_est;      /* 10 */
   int    relax_order;        /* 0 lexicographic, 1 C/F (C then F down, F then C up) */
   int    cycle_type;         /* 1 V, 2 W (visits of each coarse level per visit of the finer) */
   int    fcycle;             /* 0, or 1: F-cycle */
   int    pcg_rel_change;     /* PCG driven by this hierarchy: the relative-change test (pcg.c:836-843) */
   double outer_weight;       /* 1.0: outer weight omega of the hybrid Gauss-Seidel / SSOR smoothers */
} or_amg_params;

typedef struct
{
   int      num_levels;
   or_csr  *A;            /* num_levels */
   or_csr  *P;            /* num_levels-1 */
   or_csr  *S;            /* num_levels-1, pattern only (NULL j on aggressive levels) */
   int    **CF;           /* num_levels-1 */
   double **l1;           /* num_levels (l1 norms or diagonal, per the smoother) */
   double **cheby_coefs;  /* num_levels, order+1 coefficients */
   double **cheby_ds;     /* num_levels, D^{-1/2} scaling (ones when cheby_scale is 0) */
   double  *cheby_eig;    /* 2 per level: max, min eigenvalue estimates */
   double  *coarse_lu;    /* dense n_c x n_c row-major copy of the coarsest matrix */
   int      coarse_n;
   or_amg_params prm;
   /* work vectors */
   double **F, **U;
   double  *Vtmp, *Ztmp;
} or_hierarchy;

void   or_default_params(or_amg_params *p);
void   or_set_threads(int nthreads);

/* generators */
void   or_rand_uniform(int n, int seed, double *out);           /* 2*PM-1, hypre_SeqVectorSetRandomValues */
double or_park_miller_nth(int seed, long long k);                /* k-th draw (k>=1) from seed */
int    or_gen_stencil(int kind, int nx, int ny, int nz, or_csr *A);  /* 7 or 27 point, diag first */
int    or_gen_aniso2d(int n, double eps, or_csr *A);             /* -eps*dxx - dyy, 5-point, diag first */

/* setup kernels */
int    or_strength(const or_csr *A, double theta, double max_row_sum, or_csr *S);
int    or_pmis(const or_csr *S, int CF_init, int *CF);
int    or_coarse_count(int n, const int *CF);
int    or_extpi_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P);
int    or_ext_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P);
int    or_dir_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P);
int    or_truncate(or_csr *P, double trunc_factor, int max_elmts);
int    or_transpose(const or_csr *A, or_csr *AT);
int    or_rap(const or_csr *P, const or_csr *A, or_csr *Ac);
int    or_l1_norms(const or_csr *A, int option, double *l1);
int    or_l1_norms_cf(const or_csr *A, int option, const int *CF, double *l1);
int    or_matmul(const or_csr *A, const or_csr *B, or_csr *C);
int    or_matmat_flat(int nra, int nca, int ncb, const int *Ai, const int *Aj, const double *Av,
                      const int *Bi, const int *Bj, const double *Bv, int **Ci, int **Cj, double **Cv);
int    or_strength2(const or_csr *S, int *CF, int num_paths, or_csr *S2);
void   or_correct_cf2(int n, int *CF, const int *CFN);
void   or_correct_cf(int n, int *CF, const int *CFN);
int    or_multipass_interp(const or_csr *A, const or_csr *S, int *CF, double trunc_factor, int max_elmts, or_csr *P);
int    or_mod_multipass_interp(const or_csr *A, const or_csr *S, int *CF, int type, double trunc_factor,
                               int max_elmts, or_csr *P);
int    or_partial_ext_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P);
int    or_mod_partial_interp(const or_csr *A, const or_csr *S, const int *CF, int variant, or_csr *P);
int    or_mod_extpi_interp(const or_csr *A, const or_csr *S, const int *CF, or_csr *P);
int    or_partial_extpi_interp(const or_csr *A, const or_csr *S, int *CF, or_csr *P);
int    or_eig_tridiag(int n, double *d, double *e);
int    or_max_eig_cg(const or_csr *A, int scale, int max_iter, double *max_eig, double *min_eig);
int    or_cheby_setup(const or_csr *A, double max_eig, double min_eig, double fraction, int order,
                      int scale, int variant, double *coefs, double *ds);

/* hierarchy */
int    or_amg_setup(const or_csr *A, const or_amg_params *prm, or_hierarchy *H);
void   or_amg_free(or_hierarchy *H);
int    or_amg_vcycle(or_hierarchy *H, const double *f, double *u);
int    or_amg_solve_flat(int n, const int *Ai, const int *Aj, const double *Av, or_hierarchy *H, const double *b,
                         double *x, double tol, int maxit, double *relres, int *iters);

/* vectors / matvec */
void   or_matvec(double alpha, const or_csr *A, const double *x, double beta, const double *b, double *y);
double or_dot(int n, const double *x, const double *y);

/* Krylov, relative residual history written to relres[0..iters] */
int    or_pcg(const or_csr *A, or_hierarchy *H, const double *b, double *x,
              double tol, int maxit, double *relres, int *iters);
int    or_fgmres(const or_csr *A, or_hierarchy *H, const double *b, double *x,
                 double tol, int maxit, int kdim, double *resnorms, int *iters);

void   or_csr_free(or_csr *A);

#ifdef __cplusplus
}
#endif
#endif
