/* Internal host-side structures of libHYPRE_gb300 (C). */
#ifndef GB_INTERNAL_H
#define GB_INTERNAL_H

#include "HYPRE_gb300.h"
#include "gb_kernels.h"

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- error flag (reference: src/utilities/error.c:13-91) ------------------ */
extern HYPRE_Int gb_error_flag;
extern HYPRE_Int gb_error_arg;
void gb_error(HYPRE_Int code, const char *msg);
void gb_error_in_arg(HYPRE_Int arg);
int  gb_cuda_ok(cudaError_t e, const char *what);   /* records a GENERIC error on failure */

/* --- runtime ------------------------------------------------------------- */
cudaStream_t gb_stream(void);
int   gb_runtime_init(void);
void *gb_dmalloc(size_t bytes);              /* stream-ordered device allocation */
void *gb_dcalloc(size_t bytes);
void  gb_dfree(void *p);
void *gb_hmalloc_pinned(size_t bytes);
void  gb_hfree_pinned(void *p);
int   gb_sync(void);                         /* stream sync + error check */
extern long long gb_sync_calls;              /* gb_sync calls and seconds waited */
extern double    gb_sync_seconds;
double gb_wtime(void);
/* scratch buffers reused across calls (grow-only, stream ordered) */
void *gb_scratch(int slot, size_t bytes);
double *gb_red_part(void);                   /* GB_RED_BLOCKS * 4 doubles */
double *gb_red_out(void);                    /* 8 doubles (device) */
unsigned int *gb_red_count(void);            /* zeroed counter of one-launch reductions */
double *gb_red_host(void);                   /* 8 doubles (pinned host) */
/* 16 ints (pinned host, 64-byte aligned): 0 setup read-backs, 1 IJ read-backs,
 * 2 and 8-9 (one int64) SELL sizing, 3 FP32-exactness flag, 4-5 PMIS counts */
int *gb_red_ints(void);
void  gb_release_scratch(void);

/* --- matrices and vectors -------------------------------------------------- */
#define GB_MAGIC_MAT 0x4d415452
#define GB_MAGIC_VEC 0x56454354
#define GB_MAGIC_AMG 0x414d4731
#define GB_MAGIC_PCG 0x50434731
#define GB_MAGIC_GMR 0x474d5231
#define GB_MAGIC_DS  0x44534331
#define GB_MAGIC_BAT 0x42415431

typedef struct
{
   int     nr, nc, nnz;
   int    *i, *j;        /* device */
   double *v;            /* device, FP64 */
} gb_csr;

/* SELL-32 structure of a matrix (whole rows, or their strictly lower parts):
 * slice widths and offsets and column indices, shared by the solve forms of
 * every precision; state 1 built, -1 not used, 0 not tried.  The indices are
 * kept as 16-bit offsets from the row (j16) when every |j - i| < 2^15 (a
 * banded matrix: 3-D stencils up to 180 points a side), else as j. */
typedef struct
{
   int        state;
   int        nslices;
   long long  tot;
   int       *w;
   long long *ptr;
   int       *j;
   short     *j16;
} gb_sellstruct;

/* cached solve-phase form of a matrix in one precision */
typedef struct
{
   int          valid;
   int          vprec;
   gb_spmv_desc desc;
   void        *vals;      /* CSR values in vprec (NULL when vprec == F64) */
   void        *sl_v;      /* SELL values in vprec (FP64 form: FP32 when exact32) */
   int          exact32;   /* FP64 form: every value is zero or a normal FP32 number */
   float       *rs;        /* FP16 form: row scales a_ii */
   /* strictly lower part as SELL-32 and the diagonal (in the vector
    * precision; none for the unit-diagonal FP16 form), for two-stage
    * Gauss-Seidel sweeps on large levels; lo_valid 1 built, -1 not used */
   int          lo_valid;
   gb_spmv_desc lo;
   void        *lo_diag;
   void        *lo_sl_v;
} gb_solveform;

struct hypre_ParCSRMatrix_struct
{
   int          magic;
   gb_csr       A;
   int          owns;
   gb_solveform sf[3];     /* per precision (GB_PREC_*) */
   gb_sellstruct sell;     /* SELL-32 structure of the rows */
   gb_sellstruct lsell;    /* ... of the strictly lower parts */
   double      *diag;      /* device, for diagonal scaling (lazy) */
   int          row_active;          /* GetRow .. RestoreRow */
   int         *row_cols;            /* host copy of the active row */
   double      *row_vals;
   int          row_cap;
};
typedef struct hypre_ParCSRMatrix_struct gb_parcsr;

struct hypre_ParVector_struct
{
   int     magic;
   int     n;
   int     num_vectors;
   double *d;              /* device */
   int     owns;
};
typedef struct hypre_ParVector_struct gb_parvec;

gb_parcsr *gb_parcsr_wrap(gb_csr A, int owns);
void       gb_parcsr_free(gb_parcsr *M);
void       gb_csr_free(gb_csr *A);
const gb_spmv_desc *gb_solve_desc(gb_parcsr *M, int vprec);   /* builds lazily */
void gb_spmv_autotune(gb_spmv_desc *d, long long nnz);        /* gb_tune.c */
void gb_spmm_autotune(int prec, int nrows, int ncols, long long nnz, int nv, const int *Ai, const int *Aj,
                      const void *Av, void *x, void *y, int *T, int *U);
/* strictly lower part of a large matrix for two-stage Gauss-Seidel (NULL for
 * small or wide-row matrices: the CSR kernel is used there); builds lazily */
const gb_spmv_desc *gb_lower_desc(gb_parcsr *M, int vprec, const void **diag);
gb_parvec *gb_parvec_new(int n);
void       gb_parvec_free(gb_parvec *v);

/* y = alpha*A*x + beta*y on the library stream, FP64 */
void gb_matvec(double alpha, gb_parcsr *A, const double *x, double beta, double *y);
double gb_dot(long long n, const double *x, const double *y);     /* synchronises */

/* --- BoomerAMG ----------------------------------------------------------- */
typedef struct
{
   double strong_threshold, max_row_sum, trunc_factor;
   int    p_max_elmts, interp_type, coarsen_type;
   int    agg_num_levels, agg_interp_type, agg_p_max_elmts, agg_p12_max_elmts, num_paths;
   double agg_trunc_factor, agg_p12_trunc_factor;
   int    max_levels, max_coarse_size, min_coarse_size;
   int    relax_type[4];     /* [1] down, [2] up, [3] coarsest (reference grid_relax_type) */
   int    num_sweeps[4];
   int    relax_order;       /* 0 lexicographic, 1 C/F (C then F down, F then C up) */
   double relax_weight;
   double outer_weight;      /* omega of the hybrid Gauss-Seidel / SSOR smoothers (> 0) */
   double *level_relax_weight;   /* optional, per level */
   int    cheby_order, cheby_scale, cheby_variant, cheby_eig_est;
   double cheby_fraction;
   int    cycle_type;        /* 1 V, 2 W */
   int    fcycle;            /* 1: F-cycle */
   double tol;
   int    max_iter;
   int    min_iter;          /* BoomerAMG as the solver: cycles at least this many */
   int    print_level, logging;
   int    cycle_prec;        /* GB_PREC_F64 / F32 / F16 (finest values) */
   int    use_graph;
   int    setup_tables;      /* 0 automatic tiers, 1 global-memory tables only */
} gb_amg_params;

typedef struct
{
   int        n;
   gb_parcsr *A;          /* level operator (level 0: borrowed from the caller) */
   gb_parcsr *P;          /* interpolation to this level from level+1 (n x n_c) */
   gb_parcsr *R;          /* P^T */
   gb_csr     S;          /* strength pattern (kept for inspection) */
   int       *CF;         /* device */
   double    *l1;         /* device, FP64 */
   float     *l1f;        /* device, FP32 copy */
   double     relax_w;
   /* cycle vectors (FP64 and FP32 sets) */
   double    *F, *U, *U2, *V;
   float     *Ff, *Uf, *U2f, *Vf;
   /* Chebyshev smoother (relax 16): coefficients of s(t), eigenvalue
    * estimates, D^{-1/2} (ones without scaling) and a second work vector */
   int        cheb_order;
   double     cheb_c[5];
   double     cheb_eig[2];
   double    *cheb_ds, *W;
   float     *cheb_dsf, *Wf;
   /* hybrid Gauss-Seidel (relax 3, 4, 6, 8, 13, 14): row flags and counter
    * (n + 1 ints) and the relaxation's starting values (scaled forms) */
   int       *hgs_flags;
   double    *hgs_t;
   float     *hgs_tf;
} gb_level;

typedef struct
{
   int           magic;
   gb_amg_params prm;
   int           num_levels;
   gb_level      lev[32];
   double       *coarse_inv;    /* device, n_c x n_c */
   int           coarse_n;
   int           num_iterations;
   double        rel_resid;
   double        setup_times[8];   /* phases [0..4], total [5], host syncs [6], seconds in them [7] */
   int           setup_done;
   /* CUDA graph of one V-cycle for given (f, u) device pointers */
   cudaGraphExec_t graph;
   const void   *graph_f;
   void         *graph_u;
   int           graph_prec;
   double       *r_work;        /* FP64 residual for stand-alone solve */
   /* learned parameters: MLP weights (device FP32) and what they predicted */
   float        *mlp_params;
   double        learned_theta;
   double        learned_w[32];
   void         *multi_ws;      /* multi-vector cycle work space (gb_multi.c) */
   int           uses_hgs;      /* some level relaxes with hybrid Gauss-Seidel */
   double        spgemm_bytes, spgemm_seconds;   /* sparse products of the last setup */
   int           spgemm_calls;
} gb_amg;

int gb_amg_cycle(gb_amg *amg, const double *f, double *u);   /* one V-cycle, u from zero */
int gb_amg_check_sweeps(void);   /* HYPRE_ERROR_GENERIC after a hybrid Gauss-Seidel wait ran out */
int gb_amg_setup(gb_amg *amg, gb_parcsr *A0);
/* learned parameters (gb_learn.c): strength threshold from the finest level's
 * rows before coarsening, smoother weight per level after the hierarchy */
int gb_learn_theta(gb_amg *amg, gb_parcsr *A0, double *theta);
int gb_learn_weights(gb_amg *amg);

/* --- Krylov -------------------------------------------------------------- */
typedef struct
{
   int                  magic;
   double               tol, a_tol;
   int                  max_iter, two_norm, rel_change, recompute_residual, k_dim;
   int                  print_level, logging;
   HYPRE_PtrToSolverFcn precond, precond_setup;
   HYPRE_Solver         precond_solver;
   int                  num_iterations;
   double               rel_resid;
   double              *hist;
   int                  hist_n, hist_cap;
   /* work vectors */
   int                  n;
   double              *r, *p, *s, *w;
   double             **V, **Z;
   int                  nV;
   double              *hdev, *hhost;   /* one Hessenberg column: device and pinned host */
   /* multi-vector PCG (gb_multi.c); last_multi: the last solve had multi-vectors */
   int                  last_multi;
   int                  m_nv, m_n;
   int                  m_shT, m_shU;     /* SpMM launch shape of the outer products */
   double              *m_r, *m_p, *m_s, *m_dev;
   int                 *m_iters;
   double              *m_relres, *m_hist;
} gb_krylov;

void gb_multi_free(gb_amg *amg);
void gb_krylov_multi_free(gb_krylov *k);
int  gb_pcg_multi(gb_krylov *k, gb_parcsr *A, gb_parvec *b, gb_parvec *x);

#ifdef __cplusplus
}
#endif
#endif
