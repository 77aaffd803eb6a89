/* IJ assembly interface and ParCSR / ParVector objects (one process, device
 * data, empty off-diagonal block).
 * Reference: src/IJ_mv/HYPRE_IJMatrix.c, IJMatrix_parcsr.c (host assembly,
 * diagonal moved to the front of each row :2800-2990), src/IJ_mv/HYPRE_IJVector.c,
 * src/parcsr_mv/HYPRE_parcsr_matrix.c, HYPRE_parcsr_vector.c. */
#include "gb_internal.h"

/* --------------------------------------------------------------------------
 * ParCSR matrix
 * ------------------------------------------------------------------------ */
void gb_csr_free(gb_csr *A)
{
   gb_dfree(A->i); gb_dfree(A->j); gb_dfree(A->v);
   A->i = NULL; A->j = NULL; A->v = NULL;
}

gb_parcsr *gb_parcsr_wrap(gb_csr A, int owns)
{
   gb_parcsr *M = (gb_parcsr *) calloc(1, sizeof(gb_parcsr));
   M->magic = GB_MAGIC_MAT;
   M->A = A;
   M->owns = owns;
   return M;
}

static void solveform_free(gb_solveform *f)
{
   gb_dfree(f->vals); gb_dfree(f->sl_v); gb_dfree(f->rs);
   gb_dfree(f->lo_diag); gb_dfree(f->lo_sl_v);
   memset(f, 0, sizeof(*f));
}

static void sellstruct_free(gb_sellstruct *S)
{
   gb_dfree(S->w); gb_dfree(S->ptr); gb_dfree(S->j); gb_dfree(S->j16);
   memset(S, 0, sizeof(*S));
}

void gb_parcsr_free(gb_parcsr *M)
{
   if (!M) { return; }
   for (int p = 0; p < 3; p++) { solveform_free(&M->sf[p]); }
   sellstruct_free(&M->sell);
   sellstruct_free(&M->lsell);
   if (M->owns) { gb_csr_free(&M->A); }
   gb_dfree(M->diag);
   free(M->row_cols); free(M->row_vals);
   M->magic = 0;
   free(M);
}

/* Lanes per row for the CSR kernel from the average row length (the
 * reference's group-size rule, src/seq_mv/csr_spmv_device.c:302-315). */
static int lanes_for(double avg)
{
   if (avg >= 64) { return 32; }
   if (avg >= 32) { return 16; }
   if (avg >= 16) { return 8; }
   if (avg >= 8) { return 4; }
   return 2;
}

/* SELL-32 structure of M's rows (lower = 0: used when rows are short and
 * near uniform, n >= 4096, 4 <= nnz/row <= 40, padding <= 15%) or of their
 * strictly lower parts (lower = 1: levels of >= 65,536 rows); built once and
 * shared by the forms of every precision.  1 when usable. */
static int sell_struct(gb_parcsr *M, int lower)
{
   gb_sellstruct *S = lower ? &M->lsell : &M->sell;
   if (S->state) { return S->state > 0; }
   gb_csr *A = &M->A;
   double avg = A->nr ? (double) A->nnz / A->nr : 0;
   int nsl = (A->nr + 31) / 32;
   int ok = lower ? (A->nr >= 65536 && avg <= 40 && nsl <= 1024 * 1024)
                  : (A->nr >= 4096 && avg <= 40 && avg >= 4 && nsl <= 1024 * 1024);
   if (!ok) { S->state = -1; return 0; }
   cudaStream_t s = gb_stream();
   S->nslices = nsl;
   S->w = (int *) gb_dmalloc(sizeof(int) * (size_t) nsl);
   S->ptr = (long long *) gb_dmalloc(sizeof(long long) * (size_t) (nsl + 1));
   if (!S->w || !S->ptr) { sellstruct_free(S); S->state = -1; return 0; }
   int *wide = (int *) gb_dmalloc(sizeof(int));
   long long *htot = (long long *) (gb_red_ints() + 8);
   int *hwide = gb_red_ints() + 2;
   gb_sell_struct(A->nr, A->i, A->j, lower, nsl, S->w, S->ptr, NULL, NULL, wide, s, 0);
   cudaMemcpyAsync(htot, S->ptr + nsl, sizeof(long long), cudaMemcpyDeviceToHost, s);
   cudaMemcpyAsync(hwide, wide, sizeof(int), cudaMemcpyDeviceToHost, s);
   gb_sync();
   gb_dfree(wide);
   S->tot = *htot;
   if (!lower && (double) S->tot > 1.15 * (double) A->nnz) { sellstruct_free(S); S->state = -1; return 0; }
   if (*hwide == 0) { S->j16 = (short *) gb_dmalloc(sizeof(short) * (size_t) (S->tot ? S->tot : 1)); }
   else { S->j = (int *) gb_dmalloc(sizeof(int) * (size_t) (S->tot ? S->tot : 1)); }
   if (!S->j && !S->j16) { sellstruct_free(S); S->state = -1; return 0; }
   gb_sell_struct(A->nr, A->i, A->j, lower, nsl, S->w, S->ptr, S->j, S->j16, NULL, s, 1);
   S->state = 1;
   return 1;
}

static size_t vbytes(int vprec) { return vprec == GB_PREC_F64 ? 8 : vprec == GB_PREC_F32 ? 4 : 2; }

const gb_spmv_desc *gb_solve_desc(gb_parcsr *M, int vprec)
{
   gb_solveform *f = &M->sf[vprec];
   if (f->valid) { return &f->desc; }
   cudaStream_t s = gb_stream();
   gb_csr *A = &M->A;
   memset(&f->desc, 0, sizeof(f->desc));
   f->vprec = vprec;
   f->desc.n = A->nr;
   f->desc.vprec = vprec;
   f->desc.i = A->i;
   f->desc.j = A->j;
   double avg = A->nr ? (double) A->nnz / A->nr : 0;
   f->desc.K = lanes_for(avg);
   /* FP16 forms hold row-scaled values a_ij / a_ii (unit diagonal) with the
    * diagonal kept in FP32, so coefficients of any magnitude stay in range */
   const int scaled = vprec == GB_PREC_F16;
   /* CSR values in the requested precision (the CSR SpMV and the small-level
    * Gauss-Seidel kernels read them; FP16: also the row scales) */
   if (vprec == GB_PREC_F64) { f->desc.v = A->v; }
   else
   {
      f->vals = gb_dmalloc(vbytes(vprec) * (size_t) (A->nnz ? A->nnz : 1));
      if (scaled)
      {
         f->rs = (float *) gb_dmalloc(sizeof(float) * (size_t) (A->nr ? A->nr : 1));
         gb_row_scaled_half(A->nr, A->i, A->v, f->vals, f->rs, s);
         f->desc.rs = f->rs;
      }
      else { gb_convert_vals(A->nnz, A->v, f->vals, vprec, s); }
      f->desc.v = f->vals;
   }
   /* SELL-32 values on the shared structure */
   f->desc.fmt = GB_FMT_CSR;
   if (sell_struct(M, 0))
   {
      /* FP64 values that are all exact in FP32 (stencils with small integer
       * coefficients) are held as FP32 and widened exactly in the kernel */
      int svp = vprec;
      if (vprec == GB_PREC_F64)
      {
         int *flag = (int *) gb_dmalloc(sizeof(int));
         int *hflag = gb_red_ints() + 3;
         gb_exact32(A->nnz, A->v, flag, s);
         cudaMemcpyAsync(hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
         gb_sync();
         gb_dfree(flag);
         f->exact32 = *hflag == 0;
         if (f->exact32) { svp = GB_PREC_F32; }
      }
      f->sl_v = gb_dmalloc(vbytes(svp) * (size_t) (M->sell.tot ? M->sell.tot : 1));
      gb_sell_vals(A->nr, A->i, A->j, A->v, 0, scaled, svp, M->sell.nslices, M->sell.w, M->sell.ptr, f->sl_v, s);
      f->desc.sl_v32 = f->exact32;
      f->desc.fmt = GB_FMT_SELL;
      f->desc.nslices = M->sell.nslices;
      f->desc.sl_ptr = M->sell.ptr; f->desc.sl_w = M->sell.w; f->desc.sl_j = M->sell.j; f->desc.sl_v = f->sl_v;
      f->desc.sl_j16 = M->sell.j16;
   }
   f->valid = 1;
   gb_spmv_autotune(&f->desc, A->nnz);
   return &f->desc;
}

const gb_spmv_desc *gb_lower_desc(gb_parcsr *M, int vprec, const void **diag)
{
   gb_solveform *f = &M->sf[vprec];
   if (!f->valid) { gb_solve_desc(M, vprec); }
   if (f->lo_valid) { *diag = f->lo_diag; return f->lo_valid > 0 ? &f->lo : NULL; }
   if (!sell_struct(M, 1)) { f->lo_valid = -1; *diag = NULL; return NULL; }
   cudaStream_t s = gb_stream();
   gb_csr *A = &M->A;
   int n = A->nr;
   const int svp = (vprec == GB_PREC_F64 && f->exact32) ? GB_PREC_F32 : vprec;
   f->lo_sl_v = gb_dmalloc(vbytes(svp) * (size_t) (M->lsell.tot ? M->lsell.tot : 1));
   gb_sell_vals(n, A->i, A->j, A->v, 1, vprec == GB_PREC_F16, svp, M->lsell.nslices, M->lsell.w, M->lsell.ptr,
                f->lo_sl_v, s);
   /* the diagonal in the vector precision (FP16 forms: unit diagonal) */
   if (vprec != GB_PREC_F16)
   {
      f->lo_diag = gb_dmalloc((vprec == GB_PREC_F64 ? 8 : 4) * (size_t) n);
      gb_diag_vals(n, A->i, A->v, vprec, f->lo_diag, s);
   }
   memset(&f->lo, 0, sizeof(f->lo));
   f->lo.n = n;
   f->lo.vprec = vprec;
   f->lo.fmt = GB_FMT_SELL;
   f->lo.nslices = M->lsell.nslices;
   f->lo.sl_ptr = M->lsell.ptr; f->lo.sl_w = M->lsell.w; f->lo.sl_j = M->lsell.j; f->lo.sl_v = f->lo_sl_v;
   f->lo.sl_j16 = M->lsell.j16;
   f->lo.sl_v32 = vprec == GB_PREC_F64 && f->exact32;
   f->lo.K = 8;
   f->lo_valid = 1;
   *diag = f->lo_diag;
   return &f->lo;
}

void gb_matvec(double alpha, gb_parcsr *A, const double *x, double beta, double *y)
{
   const gb_spmv_desc *d = gb_solve_desc(A, GB_PREC_F64);
   gb_spmv_d(d, x, y, 0, alpha, beta, y, NULL, 0.0, NULL, NULL, gb_stream());
}

/* --------------------------------------------------------------------------
 * ParVector
 * ------------------------------------------------------------------------ */
gb_parvec *gb_parvec_new(int n)
{
   gb_parvec *v = (gb_parvec *) calloc(1, sizeof(gb_parvec));
   v->magic = GB_MAGIC_VEC;
   v->n = n;
   v->num_vectors = 1;
   v->d = (double *) gb_dcalloc(sizeof(double) * (size_t) (n > 0 ? n : 1));
   v->owns = 1;
   return v;
}

void gb_parvec_free(gb_parvec *v)
{
   if (!v) { return; }
   if (v->owns) { gb_dfree(v->d); }
   v->magic = 0;
   free(v);
}

static int check_vec(gb_parvec *v, int arg)
{
   if (!v || v->magic != GB_MAGIC_VEC) { gb_error_in_arg(arg); return 0; }
   return 1;
}

static int check_mat(gb_parcsr *A, int arg)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(arg); return 0; }
   return 1;
}

HYPRE_Int HYPRE_ParVectorCreate(MPI_Comm comm, HYPRE_BigInt global_size, HYPRE_BigInt *partitioning,
                                HYPRE_ParVector *vector)
{
   (void) comm; (void) partitioning;
   if (!vector) { gb_error_in_arg(4); return gb_error_flag; }
   if (global_size < 0) { gb_error_in_arg(2); return gb_error_flag; }
   gb_runtime_init();
   gb_parvec *v = (gb_parvec *) calloc(1, sizeof(gb_parvec));
   v->magic = GB_MAGIC_VEC;
   v->n = global_size;
   v->num_vectors = 1;
   *vector = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorInitialize(HYPRE_ParVector v)
{
   if (!check_vec(v, 1)) { return gb_error_flag; }
   if (!v->d)
   {
      v->d = (double *) gb_dcalloc(sizeof(double) * (size_t) (v->n > 0 ? v->n : 1));
      v->owns = 1;
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorDestroy(HYPRE_ParVector v)
{
   if (v && v->magic == GB_MAGIC_VEC) { gb_parvec_free(v); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorSetConstantValues(HYPRE_ParVector v, HYPRE_Complex value)
{
   if (!check_vec(v, 1)) { return gb_error_flag; }
   gb_fill_d(v->n, v->d, value, gb_stream());
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorSetRandomValues(HYPRE_ParVector v, HYPRE_Int seed)
{
   /* hypre_SeqVectorSetRandomValues, src/seq_mv/vector.c:615: 2*PM-1 from the
    * Park-Miller sequence, generated on the host as the reference does */
   if (!check_vec(v, 1)) { return gb_error_flag; }
   double *h = (double *) malloc(sizeof(double) * (size_t) (v->n > 0 ? v->n : 1));
   int s = seed < 1 ? 1 : (seed >= 2147483647 ? 2147483646 : seed);
   for (int i = 0; i < v->n; i++)
   {
      int high = s / 127773, low = s % 127773;
      int test = 16807 * low - 2836 * high;
      s = test > 0 ? test : test + 2147483647;
      h[i] = 2.0 * ((double) s / (double) 2147483647) - 1.0;
   }
   cudaMemcpyAsync(v->d, h, sizeof(double) * (size_t) v->n, cudaMemcpyHostToDevice, gb_stream());
   gb_sync();
   free(h);
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorCopy(HYPRE_ParVector x, HYPRE_ParVector y)
{
   if (!check_vec(x, 1) || !check_vec(y, 2)) { return gb_error_flag; }
   if (x->n != y->n) { gb_error_in_arg(2); return gb_error_flag; }
   cudaMemcpyAsync(y->d, x->d, sizeof(double) * (size_t) x->n, cudaMemcpyDeviceToDevice, gb_stream());
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorScale(HYPRE_Complex a, HYPRE_ParVector x)
{
   if (!check_vec(x, 2)) { return gb_error_flag; }
   gb_scale_d(x->n, a, x->d, gb_stream());
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorAxpy(HYPRE_Complex a, HYPRE_ParVector x, HYPRE_ParVector y)
{
   if (!check_vec(x, 2) || !check_vec(y, 3)) { return gb_error_flag; }
   gb_axpy_d(x->n, a, x->d, y->d, gb_stream());
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorInnerProd(HYPRE_ParVector x, HYPRE_ParVector y, HYPRE_Real *prod)
{
   if (!check_vec(x, 1) || !check_vec(y, 2)) { return gb_error_flag; }
   if (!prod) { gb_error_in_arg(3); return gb_error_flag; }
   *prod = gb_dot(x->n, x->d, y->d);
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_ParVectorGetDevicePointer(HYPRE_ParVector v, void **dptr, HYPRE_Int *n)
{
   if (!check_vec(v, 1)) { return gb_error_flag; }
   if (dptr) { *dptr = v->d; }
   if (n) { *n = v->n; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_ParVectorCopyFromHost(HYPRE_ParVector v, const HYPRE_Real *h, HYPRE_Int n)
{
   if (!check_vec(v, 1)) { return gb_error_flag; }
   if ((long long) n != (long long) v->n * v->num_vectors || !h) { gb_error_in_arg(3); return gb_error_flag; }
   cudaMemcpyAsync(v->d, h, sizeof(double) * (size_t) n, cudaMemcpyHostToDevice, gb_stream());
   gb_sync();
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_ParVectorCopyToHost(HYPRE_ParVector v, HYPRE_Real *h, HYPRE_Int n)
{
   if (!check_vec(v, 1)) { return gb_error_flag; }
   if ((long long) n != (long long) v->n * v->num_vectors || !h) { gb_error_in_arg(3); return gb_error_flag; }
   cudaMemcpyAsync(h, v->d, sizeof(double) * (size_t) n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRMatrixGetDims(HYPRE_ParCSRMatrix A, HYPRE_BigInt *M, HYPRE_BigInt *N)
{
   if (!check_mat(A, 1)) { return gb_error_flag; }
   if (M) { *M = A->A.nr; }
   if (N) { *N = A->A.nc; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRMatrixGetLocalRange(HYPRE_ParCSRMatrix A, HYPRE_BigInt *rs, HYPRE_BigInt *re,
                                          HYPRE_BigInt *cs, HYPRE_BigInt *ce)
{
   if (!check_mat(A, 1)) { return gb_error_flag; }
   if (rs) { *rs = 0; }
   if (re) { *re = A->A.nr - 1; }
   if (cs) { *cs = 0; }
   if (ce) { *ce = A->A.nc - 1; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRMatrixMatvec(HYPRE_Complex alpha, HYPRE_ParCSRMatrix A, HYPRE_ParVector x,
                                   HYPRE_Complex beta, HYPRE_ParVector y)
{
   if (!check_mat(A, 2) || !check_vec(x, 3) || !check_vec(y, 5)) { return gb_error_flag; }
   /* single vectors only (multi-vectors go through the multi-RHS Krylov path) */
   if (x->n != A->A.nc || x->num_vectors != 1) { gb_error_in_arg(3); return gb_error_flag; }
   if (y->n != A->A.nr || y->num_vectors != 1) { gb_error_in_arg(5); return gb_error_flag; }
   gb_matvec(alpha, A, x->d, beta, y->d);
   return gb_error_flag;
}

/* y = alpha*A^T x + beta*y through an explicit transpose built on demand */
HYPRE_Int HYPRE_ParCSRMatrixMatvecT(HYPRE_Complex alpha, HYPRE_ParCSRMatrix A, HYPRE_ParVector x,
                                    HYPRE_Complex beta, HYPRE_ParVector y)
{
   if (!check_mat(A, 2) || !check_vec(x, 3) || !check_vec(y, 5)) { return gb_error_flag; }
   if (x->n != A->A.nr || x->num_vectors != 1) { gb_error_in_arg(3); return gb_error_flag; }
   if (y->n != A->A.nc || y->num_vectors != 1) { gb_error_in_arg(5); return gb_error_flag; }
   extern gb_parcsr *gb_transpose(gb_parcsr *A);
   gb_parcsr *T = gb_transpose(A);
   if (!T) { return gb_error_flag; }
   gb_matvec(alpha, T, x->d, beta, y->d);
   gb_sync();
   gb_parcsr_free(T);
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * Host CSR -> device ParCSR (diagonal moved first with shift semantics)
 * ------------------------------------------------------------------------ */
static gb_parcsr *upload_csr(int n, int nc, const int *I, const int *J, const double *V)
{
   gb_csr A;
   A.nr = n; A.nc = nc; A.nnz = I[n];
   A.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   A.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (A.nnz ? A.nnz : 1));
   A.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (A.nnz ? A.nnz : 1));
   if (!A.i || !A.j || !A.v) { return NULL; }
   cudaStream_t s = gb_stream();
   cudaMemcpyAsync(A.i, I, sizeof(int) * (size_t) (n + 1), cudaMemcpyHostToDevice, s);
   cudaMemcpyAsync(A.j, J, sizeof(int) * (size_t) A.nnz, cudaMemcpyHostToDevice, s);
   cudaMemcpyAsync(A.v, V, sizeof(double) * (size_t) A.nnz, cudaMemcpyHostToDevice, s);
   gb_sync();
   return gb_parcsr_wrap(A, 1);
}

HYPRE_Int HYPRE_GB300_ParCSRMatrixCreateFromHostCSR(HYPRE_Int n, const HYPRE_Int *rowptr, const HYPRE_Int *colidx,
                                                    const HYPRE_Real *values, HYPRE_ParCSRMatrix *Aout)
{
   if (n < 0) { gb_error_in_arg(1); return gb_error_flag; }
   if (!rowptr || !colidx || !values) { gb_error_in_arg(2); return gb_error_flag; }
   if (!Aout) { gb_error_in_arg(5); return gb_error_flag; }
   gb_runtime_init();
   int nnz = rowptr[n];
   int *J = (int *) malloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
   double *V = (double *) malloc(sizeof(double) * (size_t) (nnz ? nnz : 1));
   for (int i = 0; i < n; i++)
   {
      int b = rowptr[i], e = rowptr[i + 1], c = b + 1, dpos = -1;
      for (int k = b; k < e; k++) { if (colidx[k] == i) { dpos = k; break; } }
      if (dpos < 0) { memcpy(J + b, colidx + b, sizeof(int) * (size_t) (e - b)); memcpy(V + b, values + b, sizeof(double) * (size_t) (e - b)); continue; }
      J[b] = i; V[b] = values[dpos];
      for (int k = b; k < e; k++) { if (k != dpos) { J[c] = colidx[k]; V[c] = values[k]; c++; } }
   }
   *Aout = upload_csr(n, n, rowptr, J, V);
   free(J); free(V);
   return gb_error_flag;
}

/* One row of the matrix in host memory (reference: HYPRE_ParCSRMatrixGetRow,
 * src/parcsr_mv/HYPRE_parcsr_matrix.c / par_csr_matrix.c hypre_ParCSRMatrixGetRow):
 * global column indices, diagonal first; one row may be active at a time and
 * RestoreRow releases it. */
HYPRE_Int HYPRE_ParCSRMatrixGetRow(HYPRE_ParCSRMatrix A, HYPRE_BigInt row, HYPRE_Int *size, HYPRE_BigInt **col_ind,
                                   HYPRE_Complex **values)
{
   if (!check_mat(A, 1)) { return gb_error_flag; }
   if (row < 0 || row >= A->A.nr) { gb_error_in_arg(2); return gb_error_flag; }
   if (A->row_active) { gb_error(HYPRE_ERROR_GENERIC, "a row is already active"); return gb_error_flag; }
   int be[2];
   cudaMemcpyAsync(be, A->A.i + row, sizeof(int) * 2, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   int l = be[1] - be[0];
   if (l > A->row_cap)
   {
      free(A->row_cols); free(A->row_vals);
      A->row_cols = (int *) malloc(sizeof(int) * (size_t) l);
      A->row_vals = (double *) malloc(sizeof(double) * (size_t) l);
      A->row_cap = (A->row_cols && A->row_vals) ? l : 0;
      if (!A->row_cap) { gb_error(HYPRE_ERROR_MEMORY, "GetRow"); return gb_error_flag; }
   }
   if (l > 0)
   {
      if (col_ind) { cudaMemcpyAsync(A->row_cols, A->A.j + be[0], sizeof(int) * (size_t) l, cudaMemcpyDeviceToHost, gb_stream()); }
      if (values) { cudaMemcpyAsync(A->row_vals, A->A.v + be[0], sizeof(double) * (size_t) l, cudaMemcpyDeviceToHost, gb_stream()); }
      gb_sync();
   }
   A->row_active = 1;
   if (size) { *size = l; }
   if (col_ind) { *col_ind = A->row_cols; }
   if (values) { *values = A->row_vals; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRMatrixRestoreRow(HYPRE_ParCSRMatrix A, HYPRE_BigInt row, HYPRE_Int *size,
                                       HYPRE_BigInt **col_ind, HYPRE_Complex **values)
{
   (void) row;
   if (!check_mat(A, 1)) { return gb_error_flag; }
   if (!A->row_active) { gb_error_in_arg(1); return gb_error_flag; }
   A->row_active = 0;
   if (size) { *size = 0; }
   if (col_ind) { *col_ind = NULL; }
   if (values) { *values = NULL; }
   return gb_error_flag;
}

/* The whole local CSR (row pointers n+1, columns and values nnz; any of the
 * arrays may be NULL) copied to host memory. */
HYPRE_Int HYPRE_GB300_ParCSRMatrixCopyToHostCSR(HYPRE_ParCSRMatrix A, HYPRE_Int *nrows, HYPRE_Int *nnz,
                                               HYPRE_Int *rowptr, HYPRE_Int *colidx, HYPRE_Real *values)
{
   if (!check_mat(A, 1)) { return gb_error_flag; }
   if (nrows) { *nrows = A->A.nr; }
   if (nnz) { *nnz = A->A.nnz; }
   cudaStream_t s = gb_stream();
   if (rowptr) { cudaMemcpyAsync(rowptr, A->A.i, sizeof(int) * (size_t) (A->A.nr + 1), cudaMemcpyDeviceToHost, s); }
   if (colidx) { cudaMemcpyAsync(colidx, A->A.j, sizeof(int) * (size_t) A->A.nnz, cudaMemcpyDeviceToHost, s); }
   if (values && A->A.v) { cudaMemcpyAsync(values, A->A.v, sizeof(double) * (size_t) A->A.nnz, cudaMemcpyDeviceToHost, s); }
   gb_sync();
   return gb_error_flag;
}

/* A ParCSR matrix from CSR arrays in device memory (copied; the diagonal is
 * moved to the front of each row, shifting the entries before it, as for
 * host arrays). */
HYPRE_Int HYPRE_GB300_ParCSRMatrixCreateFromDeviceCSR(HYPRE_Int n, const HYPRE_Int *rowptr, const HYPRE_Int *colidx,
                                                     const HYPRE_Real *values, HYPRE_ParCSRMatrix *Aout)
{
   if (n < 0) { gb_error_in_arg(1); return gb_error_flag; }
   if (!rowptr || !colidx || !values) { gb_error_in_arg(2); return gb_error_flag; }
   if (!Aout) { gb_error_in_arg(5); return gb_error_flag; }
   gb_runtime_init();
   cudaStream_t s = gb_stream();
   int *hn = gb_red_ints() + 1;
   hn[0] = 0;
   cudaMemcpyAsync(hn, rowptr + n, sizeof(int), cudaMemcpyDeviceToHost, s);
   if (gb_sync()) { return gb_error_flag; }
   int nnz = hn[0];
   gb_csr A;
   A.nr = n; A.nc = n; A.nnz = nnz;
   A.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   A.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
   A.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (nnz ? nnz : 1));
   if (!A.i || !A.j || !A.v) { gb_dfree(A.i); gb_dfree(A.j); gb_dfree(A.v); *Aout = NULL; return gb_error_flag; }
   cudaMemcpyAsync(A.i, rowptr, sizeof(int) * (size_t) (n + 1), cudaMemcpyDeviceToDevice, s);
   gb_ij_gather(n, nnz, NULL, A.i, colidx, values, 0, NULL, A.j, A.v, s);
   *Aout = gb_parcsr_wrap(A, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_ParCSRMatrixDestroy(HYPRE_ParCSRMatrix A)
{
   if (A && A->magic == GB_MAGIC_MAT) { gb_parcsr_free(A); }
   return gb_error_flag;
}

/* src/parcsr_mv/HYPRE_parcsr_matrix.c:39 (matrices the caller owns, such as
 * HYPRE_ParCSRMatrixMatmat's product; a matrix handed out by
 * HYPRE_IJMatrixGetObject belongs to its IJ matrix, as in the reference) */
HYPRE_Int HYPRE_ParCSRMatrixDestroy(HYPRE_ParCSRMatrix matrix)
{
   if (!matrix || matrix->magic != GB_MAGIC_MAT) { gb_error_in_arg(1); return gb_error_flag; }
   gb_parcsr_free(matrix);
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * IJ matrix: host staging rows (arena), assembled into a device ParCSR
 * ------------------------------------------------------------------------ */
struct hypre_IJMatrix_struct
{
   int        magic;
   int        ilower, iupper, jlower, jupper;
   int        nrows;
   int        object_type;
   int        initialized, assembled;
   int        swap_diag;      /* SetDiagOffdSizes used: diagonal swapped to the front */
   int       *row_off, *row_len, *row_cap;
   int       *cols;
   double    *vals;
   long long  arena_len, arena_cap;
   int       *hint;           /* row sizes from SetRowSizes */
   int        hint_zero;      /* some row was given no space */
   gb_parcsr *par;
   /* device staging: rows put by large SetValues calls are copied straight
    * to the device (row_state 2, entries at dev_off[r]); the others live in
    * the host arena (row_state 0/1) */
   unsigned char *row_state;
   long long *dev_off;
   int       *st_cols;
   double    *st_vals;
   long long  st_len, st_cap;
   int       *st_rowptr;      /* device: set when one put holds every row in order */
   int       *st_hstart;      /* host copy of those offsets until per-row state exists */
};

#define GB_MAGIC_IJM 0x494a4d31
#define GB_IJ_ROW_DEVICE 2
#define GB_IJ_ROW_PENDING 3
/* puts with fewer entries stay on the host (one copy per call would cost
 * more than the staging) */
#define GB_IJ_DEVICE_MIN 65536
#define GB_MAGIC_IJV 0x494a5631

static int check_ijm(HYPRE_IJMatrix m, int arg)
{
   if (!m || m->magic != GB_MAGIC_IJM) { gb_error_in_arg(arg); return 0; }
   return 1;
}

/* Host arrays of one entry per row (row sizes, offsets of a put) are reused
 * across IJ objects: a fresh allocation of tens of MB pays a page fault per
 * page on first touch (milliseconds at millions of rows), which a caller that
 * assembles a matrix every time step would pay every step.  Blocks carry
 * their size in a 16-byte header; up to four freed blocks of at least 1 MB
 * are kept (released by HYPRE_Finalize). */
#define GB_IJ_HCACHE 4
static void *g_hcache[GB_IJ_HCACHE];

static void *ij_halloc(size_t bytes)
{
   int best = -1;
   for (int k = 0; k < GB_IJ_HCACHE; k++)
   {
      if (!g_hcache[k]) { continue; }
      size_t have = *(size_t *) g_hcache[k];
      if (have >= bytes && have <= 2 * bytes + (1 << 20) &&
          (best < 0 || have < *(size_t *) g_hcache[best])) { best = k; }
   }
   char *b;
   if (best >= 0) { b = (char *) g_hcache[best]; g_hcache[best] = NULL; }
   else
   {
      b = (char *) malloc(bytes + 16);
      if (!b) { return NULL; }
      *(size_t *) b = bytes;
   }
   return b + 16;
}

static void ij_hfree(void *p)
{
   if (!p) { return; }
   char *b = (char *) p - 16;
   if (*(size_t *) b >= (1 << 20))
   {
      for (int k = 0; k < GB_IJ_HCACHE; k++)
      {
         if (!g_hcache[k]) { g_hcache[k] = b; return; }
      }
   }
   free(b);
}

void gb_ij_release_host_cache(void)
{
   for (int k = 0; k < GB_IJ_HCACHE; k++) { free(g_hcache[k]); g_hcache[k] = NULL; }
}

HYPRE_Int HYPRE_IJMatrixCreate(MPI_Comm comm, HYPRE_BigInt ilower, HYPRE_BigInt iupper, HYPRE_BigInt jlower,
                               HYPRE_BigInt jupper, HYPRE_IJMatrix *matrix)
{
   (void) comm;
   if (!matrix) { gb_error_in_arg(6); return gb_error_flag; }
   if (ilower > iupper + 1 || ilower < 0) { gb_error_in_arg(2); return gb_error_flag; }
   if (jlower > jupper + 1 || jlower < 0) { gb_error_in_arg(4); return gb_error_flag; }
   if (ilower != 0 || jlower != 0 || (iupper - ilower) != (jupper - jlower))
   {
      gb_error(HYPRE_ERROR_GENERIC, "single-GPU build: the matrix must be square and start at row 0");
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   gb_runtime_init();
   struct hypre_IJMatrix_struct *m = calloc(1, sizeof(*m));
   m->magic = GB_MAGIC_IJM;
   m->ilower = ilower; m->iupper = iupper; m->jlower = jlower; m->jupper = jupper;
   m->nrows = iupper - ilower + 1;
   *matrix = m;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetObjectType(HYPRE_IJMatrix m, HYPRE_Int type)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (type != HYPRE_PARCSR) { gb_error_in_arg(2); return gb_error_flag; }
   m->object_type = type;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetRowSizes(HYPRE_IJMatrix m, const HYPRE_Int *sizes)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!sizes) { gb_error_in_arg(2); return gb_error_flag; }
   ij_hfree(m->hint);
   m->hint = (int *) ij_halloc(sizeof(int) * (size_t) (m->nrows ? m->nrows : 1));
   if (!m->hint) { gb_error(HYPRE_ERROR_MEMORY, "IJ row sizes"); return gb_error_flag; }
   int mn = 1;
   int *h = m->hint;
   const int nr = m->nrows;
   #pragma omp parallel for reduction(min : mn) schedule(static) if (nr > 100000)
   for (int r = 0; r < nr; r++)
   {
      h[r] = sizes[r];
      mn = sizes[r] < mn ? sizes[r] : mn;
   }
   m->hint_zero = mn <= 0;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetDiagOffdSizes(HYPRE_IJMatrix m, const HYPRE_Int *diag_sizes, const HYPRE_Int *offd)
{
   (void) offd;
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!diag_sizes) { gb_error_in_arg(2); return gb_error_flag; }
   HYPRE_IJMatrixSetRowSizes(m, diag_sizes);
   m->swap_diag = 1;
   return gb_error_flag;
}

static void ijm_free_stage(HYPRE_IJMatrix m)
{
   free(m->row_off); free(m->row_len); free(m->row_cap); free(m->cols); free(m->vals);
   m->row_off = m->row_len = m->row_cap = NULL; m->cols = NULL; m->vals = NULL;
   m->arena_len = m->arena_cap = 0;
   free(m->row_state); free(m->dev_off);
   m->row_state = NULL; m->dev_off = NULL;
   gb_dfree(m->st_cols); gb_dfree(m->st_vals); gb_dfree(m->st_rowptr);
   m->st_cols = NULL; m->st_vals = NULL; m->st_rowptr = NULL;
   ij_hfree(m->st_hstart);
   m->st_hstart = NULL;
   m->st_len = m->st_cap = 0;
}

/* Per-row host state (arena slots sized from SetRowSizes, row lengths, where
 * each row lives), allocated on first use: a single in-order put of every
 * row never needs it.  Rows of such a put are recorded here when it is
 * first needed. */
static int ijm_host_ready(HYPRE_IJMatrix m)
{
   if (m->row_len) { return 1; }
   int n = m->nrows;
   m->row_off = (int *) malloc(sizeof(int) * (size_t) (n ? n : 1));
   m->row_len = (int *) calloc((size_t) (n ? n : 1), sizeof(int));
   m->row_cap = (int *) malloc(sizeof(int) * (size_t) (n ? n : 1));
   m->row_state = (unsigned char *) calloc((size_t) (n ? n : 1), 1);
   m->dev_off = (long long *) malloc(sizeof(long long) * (size_t) (n ? n : 1));
   if (!m->row_off || !m->row_len || !m->row_cap || !m->row_state || !m->dev_off)
   {
      gb_error(HYPRE_ERROR_MEMORY, "IJ staging");
      return 0;
   }
   long long tot = 0;
   for (int i = 0; i < n; i++)
   {
      int c = m->hint ? m->hint[i] : 8;
      if (c < 1) { c = 1; }
      m->row_off[i] = (int) tot;
      m->row_cap[i] = c;
      tot += c;
   }
   m->arena_cap = tot + tot / 8 + 64;
   m->arena_len = tot;
   m->cols = (int *) malloc(sizeof(int) * (size_t) m->arena_cap);
   m->vals = (double *) malloc(sizeof(double) * (size_t) m->arena_cap);
   if (!m->cols || !m->vals) { gb_error(HYPRE_ERROR_MEMORY, "IJ staging"); return 0; }
   if (m->st_hstart)
   {
      for (int r = 0; r < n; r++)
      {
         m->dev_off[r] = m->st_hstart[r];
         m->row_len[r] = m->st_hstart[r + 1] - m->st_hstart[r];
         m->row_state[r] = GB_IJ_ROW_DEVICE;
      }
      ij_hfree(m->st_hstart);
      m->st_hstart = NULL;
   }
   return 1;
}

HYPRE_Int HYPRE_IJMatrixInitialize(HYPRE_IJMatrix m)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   ijm_free_stage(m);
   m->initialized = 1;
   m->assembled = 0;
   if (m->par) { gb_parcsr_free(m->par); m->par = NULL; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixInitialize_v2(HYPRE_IJMatrix m, HYPRE_MemoryLocation loc)
{
   (void) loc;
   return HYPRE_IJMatrixInitialize(m);
}

static int row_grow(HYPRE_IJMatrix m, int r, int need)
{
   int cap = m->row_cap[r];
   if (need <= cap) { return 1; }
   int ncap = cap * 2;
   while (ncap < need) { ncap *= 2; }
   if (m->arena_len + ncap > m->arena_cap)
   {
      long long nc = (m->arena_cap + ncap) * 2;
      int *c2 = (int *) realloc(m->cols, sizeof(int) * (size_t) nc);
      double *v2 = (double *) realloc(m->vals, sizeof(double) * (size_t) nc);
      if (!c2 || !v2) { gb_error(HYPRE_ERROR_MEMORY, "IJ staging"); return 0; }
      m->cols = c2; m->vals = v2; m->arena_cap = nc;
   }
   int off = (int) m->arena_len;
   memcpy(m->cols + off, m->cols + m->row_off[r], sizeof(int) * (size_t) m->row_len[r]);
   memcpy(m->vals + off, m->vals + m->row_off[r], sizeof(double) * (size_t) m->row_len[r]);
   m->row_off[r] = off;
   m->row_cap[r] = ncap;
   m->arena_len += ncap;
   return 1;
}

static int ij_read_int(const int *d)
{
   int *h = gb_red_ints() + 1;
   h[0] = 0;
   cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   return h[0];
}

/* grows the device staging to hold need entries (stream-ordered copies);
 * 0 when the device memory is not available */
static int ijm_staging_reserve(HYPRE_IJMatrix m, long long need)
{
   if (need <= m->st_cap) { return 1; }
   long long cap = m->st_cap * 2;
   if (cap < need) { cap = need; }
   int *c = (int *) gb_dmalloc(sizeof(int) * (size_t) cap);
   double *v = (double *) gb_dmalloc(sizeof(double) * (size_t) cap);
   if (!c || !v) { gb_dfree(c); gb_dfree(v); return 0; }
   if (m->st_len > 0)
   {
      cudaMemcpyAsync(c, m->st_cols, sizeof(int) * (size_t) m->st_len, cudaMemcpyDeviceToDevice, gb_stream());
      cudaMemcpyAsync(v, m->st_vals, sizeof(double) * (size_t) m->st_len, cudaMemcpyDeviceToDevice, gb_stream());
   }
   gb_dfree(m->st_cols); gb_dfree(m->st_vals);
   m->st_cols = c; m->st_vals = v; m->st_cap = cap;
   return 1;
}

/* Moves every device-staged row into the host arena (before a put that the
 * host path must handle touches one of them, or a GetValues). */
static int ijm_migrate(HYPRE_IJMatrix m)
{
   if (m->st_len == 0) { return 1; }
   if (!ijm_host_ready(m)) { return 0; }
   int *hc = (int *) malloc(sizeof(int) * (size_t) m->st_len);
   double *hv = (double *) malloc(sizeof(double) * (size_t) m->st_len);
   if (!hc || !hv) { free(hc); free(hv); gb_error(HYPRE_ERROR_MEMORY, "IJ staging"); return 0; }
   cudaMemcpyAsync(hc, m->st_cols, sizeof(int) * (size_t) m->st_len, cudaMemcpyDeviceToHost, gb_stream());
   cudaMemcpyAsync(hv, m->st_vals, sizeof(double) * (size_t) m->st_len, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   for (int r = 0; r < m->nrows; r++)
   {
      if (m->row_state[r] != GB_IJ_ROW_DEVICE) { continue; }
      int len = m->row_len[r];
      m->row_len[r] = 0;
      if (!row_grow(m, r, len)) { free(hc); free(hv); return 0; }
      memcpy(m->cols + m->row_off[r], hc + m->dev_off[r], sizeof(int) * (size_t) len);
      memcpy(m->vals + m->row_off[r], hv + m->dev_off[r], sizeof(double) * (size_t) len);
      m->row_len[r] = len;
      m->row_state[r] = 0;
   }
   free(hc); free(hv);
   m->st_len = 0;
   gb_dfree(m->st_rowptr);
   m->st_rowptr = NULL;
   return 1;
}

/* hstart[t] = the offset of the put's row t (an exclusive scan of ncols,
 * hstart[nrows] = the total), in blocks on the host's threads; returns
 * whether the put lists rows ilower, ilower + 1, ... in order */
static int ij_offsets(int nrows, const int *rows, int ilower, const int *ncols, int *hstart)
{
   enum { NB = 64 };
   long long bsum[NB + 1];
   int bord[NB];
   const int nb = nrows > 100000 ? NB : 1;
   #pragma omp parallel for schedule(static) if (nb > 1)
   for (int b = 0; b < nb; b++)
   {
      const int t0 = (int) ((long long) nrows * b / nb), t1 = (int) ((long long) nrows * (b + 1) / nb);
      long long acc = 0;
      int ord = 1;
      for (int t = t0; t < t1; t++)
      {
         ord &= rows[t] - ilower == t;
         acc += ncols[t];
      }
      bsum[b + 1] = acc;
      bord[b] = ord;
   }
   bsum[0] = 0;
   int inorder = 1;
   for (int b = 0; b < nb; b++) { bsum[b + 1] += bsum[b]; inorder &= bord[b]; }
   #pragma omp parallel for schedule(static) if (nb > 1)
   for (int b = 0; b < nb; b++)
   {
      const int t0 = (int) ((long long) nrows * b / nb), t1 = (int) ((long long) nrows * (b + 1) / nb);
      long long acc = bsum[b];
      for (int t = t0; t < t1; t++)
      {
         hstart[t] = (int) acc;
         acc += ncols[t];
      }
   }
   hstart[nrows] = (int) bsum[nb];
   return inorder;
}

/* SetValues of new rows with many entries: copied from the caller's buffers
 * to the device staging and checked there (columns in range, none repeated
 * within a row).  Returns 1 when the put was taken, 0 when the host path must
 * run it (small put, repeated or already-set rows, failed check); nothing is
 * changed in that case. */
static int ijm_put_device(HYPRE_IJMatrix m, int nrows, const int *ncols, const int *rows, const int *cols,
                          const double *values)
{
   if (nrows <= 0) { return 0; }
   /* sizes first, so the copies of the caller's buffers start before the row
    * checks (they overlap when the buffers are pinned) */
   long long tot = 0;
   int mn = 0;
   #pragma omp parallel for reduction(+ : tot) reduction(min : mn) schedule(static) if (nrows > 100000)
   for (int t = 0; t < nrows; t++)
   {
      mn = ncols[t] < mn ? ncols[t] : mn;
      tot += ncols[t];
   }
   if (mn < 0) { return 0; }
   if (tot < GB_IJ_DEVICE_MIN || tot > 0x7fffffffLL) { return 0; }
   int *hstart = (int *) ij_halloc(sizeof(int) * (size_t) (nrows + 1));
   if (!hstart || !ijm_staging_reserve(m, m->st_len + tot)) { ij_hfree(hstart); return 0; }
   cudaStream_t s = gb_stream();
   cudaMemcpyAsync(m->st_cols + m->st_len, cols, sizeof(int) * (size_t) tot, cudaMemcpyHostToDevice, s);
   cudaMemcpyAsync(m->st_vals + m->st_len, values, sizeof(double) * (size_t) tot, cudaMemcpyHostToDevice, s);
   if (!m->row_len && m->st_len == 0 && nrows == m->nrows)
   {
      /* no row holds data yet: a put of every row in order needs no per-row
       * host state (its offsets are the CSR row pointers) */
      const int inorder = ij_offsets(nrows, rows, m->ilower, ncols, hstart);
      if (inorder)
      {
         int *dstart = (int *) gb_dmalloc(sizeof(int) * (size_t) (nrows + 1));
         int *flags = (int *) gb_dcalloc(sizeof(int));
         int f = 1;
         if (dstart && flags)
         {
            cudaMemcpyAsync(dstart, hstart, sizeof(int) * (size_t) (nrows + 1), cudaMemcpyHostToDevice, s);
            gb_ij_check(nrows, dstart, m->st_cols, m->jupper - m->jlower + 1, flags, s);
            f = ij_read_int(flags);   /* also the point after which the caller's buffers are free */
         }
         else { gb_sync(); }
         gb_dfree(flags);
         if (f != 0) { gb_dfree(dstart); ij_hfree(hstart); return 0; }
         m->st_len = tot;
         m->st_rowptr = dstart;
         m->st_hstart = hstart;
         return 1;
      }
   }
   if (!ijm_host_ready(m)) { gb_sync(); ij_hfree(hstart); return 0; }
   /* row offsets within the put; every row valid, new and not repeated in
    * this put (marked pending, unmarked on failure); whether the put is the
    * whole matrix in row order (its offsets are then the CSR row pointers) */
   int t = 0, ok = 1, inorder = m->st_len == 0 && nrows == m->nrows;
   long long acc = 0;
   hstart[0] = 0;
   for (; t < nrows; t++)
   {
      int r = rows[t] - m->ilower;
      if (r < 0 || r >= m->nrows || m->row_state[r] != 0 || m->row_len[r] != 0) { ok = 0; break; }
      m->row_state[r] = GB_IJ_ROW_PENDING;
      inorder &= r == t;
      acc += ncols[t];
      hstart[t + 1] = (int) acc;
   }
   int *dstart = NULL, *flags = NULL;
   if (ok)
   {
      dstart = (int *) gb_dmalloc(sizeof(int) * (size_t) (nrows + 1));
      flags = (int *) gb_dcalloc(sizeof(int));
      ok = dstart && flags;
   }
   int f = 1;
   if (ok)
   {
      cudaMemcpyAsync(dstart, hstart, sizeof(int) * (size_t) (nrows + 1), cudaMemcpyHostToDevice, s);
      gb_ij_check(nrows, dstart, m->st_cols + m->st_len, m->jupper - m->jlower + 1, flags, s);
      f = ij_read_int(flags);   /* also the point after which the caller's buffers are free */
   }
   else { gb_sync(); }          /* the copies read the caller's buffers */
   gb_dfree(flags);
   if (f != 0)
   {
      for (int u = 0; u < (ok ? nrows : t); u++) { m->row_state[rows[u] - m->ilower] = 0; }
      gb_dfree(dstart);
      ij_hfree(hstart);
      return 0;
   }
   for (int u = 0; u < nrows; u++)
   {
      int r = rows[u] - m->ilower;
      m->dev_off[r] = m->st_len + hstart[u];
      m->row_len[r] = ncols[u];
      m->row_state[r] = GB_IJ_ROW_DEVICE;
   }
   m->st_len += tot;
   if (inorder) { m->st_rowptr = dstart; }
   else { gb_dfree(dstart); }
   ij_hfree(hstart);
   return 1;
}

static HYPRE_Int ijm_put(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_Int *ncols, const HYPRE_BigInt *rows,
                         const HYPRE_BigInt *cols, const HYPRE_Complex *values, int add)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!m->initialized) { gb_error(HYPRE_ERROR_GENERIC, "IJ matrix not initialized"); return gb_error_flag; }
   if (nrows < 0) { gb_error_in_arg(2); return gb_error_flag; }
   if (nrows == 0) { return gb_error_flag; }
   if (!ncols) { gb_error_in_arg(3); return gb_error_flag; }
   if (!rows) { gb_error_in_arg(4); return gb_error_flag; }
   if (!cols) { gb_error_in_arg(5); return gb_error_flag; }
   if (!values) { gb_error_in_arg(6); return gb_error_flag; }
   if (!add && ijm_put_device(m, nrows, ncols, rows, cols, values))
   {
      m->assembled = 0;
      return gb_error_flag;
   }
   if (!ijm_host_ready(m)) { return gb_error_flag; }
   if (m->st_len > 0)
   {
      /* the host path edits rows in the arena: bring staged rows back first
       * when this put touches one */
      for (int t = 0; t < nrows; t++)
      {
         int r = rows[t] - m->ilower;
         if (r >= 0 && r < m->nrows && m->row_state[r] == GB_IJ_ROW_DEVICE)
         {
            if (!ijm_migrate(m)) { return gb_error_flag; }
            break;
         }
      }
   }
   long long k = 0;
   for (int t = 0; t < nrows; t++)
   {
      int r = rows[t] - m->ilower;
      int nc = ncols[t];
      if (r < 0 || r >= m->nrows) { gb_error_in_arg(4); k += nc; continue; }
      int len = m->row_len[r];
      if (len == 0 && !add)
      {
         /* fresh row: append, merging repeated columns within the call */
         if (!row_grow(m, r, nc)) { return gb_error_flag; }
         int *rc = m->cols + m->row_off[r];
         double *rv = m->vals + m->row_off[r];
         /* common case: columns in range and ascending after the first entry,
          * the first not repeated later -> no duplicates, copy straight */
         int fast = 1;
         for (int q = 0; q < nc && fast; q++)
         {
            int c = cols[k + q] - m->jlower;
            if (c < 0 || c > m->jupper - m->jlower) { fast = 0; }
            if (q >= 2 && cols[k + q] <= cols[k + q - 1]) { fast = 0; }
         }
         if (fast && nc > 2)
         {
            int c0 = cols[k];
            int lo = 1, hi = nc - 1;
            while (lo <= hi) { int mid = (lo + hi) / 2; if (cols[k + mid] == c0) { fast = 0; break; } if (cols[k + mid] < c0) { lo = mid + 1; } else { hi = mid - 1; } }
         }
         if (fast && nc == 2 && cols[k] == cols[k + 1]) { fast = 0; }
         if (fast)
         {
            for (int q = 0; q < nc; q++) { rc[q] = cols[k + q] - m->jlower; rv[q] = values[k + q]; }
            m->row_len[r] = nc;
            k += nc;
            continue;
         }
         int l = 0;
         for (int q = 0; q < nc; q++, k++)
         {
            int c = cols[k] - m->jlower;
            if (c < 0 || c > m->jupper - m->jlower) { gb_error_in_arg(5); continue; }
            int found = -1;
            if (l <= 32) { for (int z = 0; z < l; z++) { if (rc[z] == c) { found = z; break; } } }
            else { for (int z = l - 1; z >= 0; z--) { if (rc[z] == c) { found = z; break; } } }
            if (found >= 0) { rv[found] = values[k]; }
            else { rc[l] = c; rv[l] = values[k]; l++; }
         }
         m->row_len[r] = l;
         continue;
      }
      for (int q = 0; q < nc; q++, k++)
      {
         int c = cols[k] - m->jlower;
         if (c < 0 || c > m->jupper - m->jlower) { gb_error_in_arg(5); continue; }
         int *rc = m->cols + m->row_off[r];
         int l = m->row_len[r];
         int found = -1;
         for (int z = 0; z < l; z++) { if (rc[z] == c) { found = z; break; } }
         if (found >= 0)
         {
            double *rv = m->vals + m->row_off[r];
            if (add) { rv[found] += values[k]; } else { rv[found] = values[k]; }
         }
         else
         {
            if (!row_grow(m, r, l + 1)) { return gb_error_flag; }
            m->cols[m->row_off[r] + l] = c;
            m->vals[m->row_off[r] + l] = values[k];
            m->row_len[r] = l + 1;
         }
      }
   }
   m->assembled = 0;
   return gb_error_flag;
}

/* ncols NULL: one column per row (the reference accepts it,
 * src/IJ_mv/HYPRE_IJMatrix.c:271-320, and its setters read 1) */
static HYPRE_Int ijm_put_ones(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_Int *ncols, const HYPRE_BigInt *rows,
                              const HYPRE_BigInt *cols, const HYPRE_Complex *values, int add)
{
   if (ncols || nrows <= 0) { return ijm_put(m, nrows, ncols, rows, cols, values, add); }
   int *ones = (int *) malloc(sizeof(int) * (size_t) nrows);
   if (!ones) { gb_error(HYPRE_ERROR_MEMORY, "IJ matrix"); return gb_error_flag; }
   for (int t = 0; t < nrows; t++) { ones[t] = 1; }
   ijm_put(m, nrows, ones, rows, cols, values, add);
   free(ones);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_Int *ncols, const HYPRE_BigInt *rows,
                                  const HYPRE_BigInt *cols, const HYPRE_Complex *values)
{
   return ijm_put_ones(m, nrows, ncols, rows, cols, values, 0);
}

HYPRE_Int HYPRE_IJMatrixAddToValues(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_Int *ncols, const HYPRE_BigInt *rows,
                                    const HYPRE_BigInt *cols, const HYPRE_Complex *values)
{
   return ijm_put_ones(m, nrows, ncols, rows, cols, values, 1);
}

/* The column each row's assembly moves to the front.  The reference's
 * assembly of rows put with SetRowSizes (the auxiliary-row path,
 * src/IJ_mv/IJMatrix_parcsr.c:2800-2930) walks the rows that have space --
 * a size above zero from SetRowSizes, or entries put into the row
 * (src/IJ_mv/aux_parcsr_matrix.c:164-215) -- and moves to the front the entry
 * whose column equals the row's ordinal among those rows (it compares the
 * column with the walk's index, :2843).  Every row has space unless
 * SetRowSizes gave some row zero, so the ordinal is the row itself and the
 * diagonal moves to the front.  Returns a device array of the ordinals when
 * some differ from the row (NULL otherwise, and always after
 * SetDiagOffdSizes, whose assembly swaps the true diagonal, :2974-2995).
 * I: host row pointers of the assembled rows. */
static int *ijm_front_keys(HYPRE_IJMatrix m, const int *I)
{
   if (m->swap_diag || !m->hint) { return NULL; }
   int n = m->nrows, ord = 0, differs = 0;
   int *key = (int *) malloc(sizeof(int) * (size_t) (n ? n : 1));
   if (!key) { gb_error(HYPRE_ERROR_MEMORY, "IJ assembly"); return NULL; }
   for (int r = 0; r < n; r++)
   {
      key[r] = ord;
      differs |= ord != r;
      if (m->hint[r] > 0 || I[r + 1] > I[r]) { ord++; }
   }
   int *d = NULL;
   if (differs)
   {
      d = (int *) gb_dmalloc(sizeof(int) * (size_t) n);
      if (d) { cudaMemcpyAsync(d, key, sizeof(int) * (size_t) n, cudaMemcpyHostToDevice, gb_stream()); gb_sync(); }
   }
   free(key);
   return d;
}

HYPRE_Int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix m)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!m->initialized) { gb_error(HYPRE_ERROR_GENERIC, "IJ matrix not initialized"); return gb_error_flag; }
   int n = m->nrows;
   cudaStream_t s = gb_stream();
   if (m->st_rowptr)
   {
      /* one device put of every row in order: its offsets are the row
       * pointers and the staged rows are gathered in place order */
      int nnz = (int) m->st_len;
      gb_csr A;
      A.nr = n; A.nc = m->jupper - m->jlower + 1; A.nnz = nnz;
      A.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
      A.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
      A.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (nnz ? nnz : 1));
      if (!A.i || !A.j || !A.v) { gb_dfree(A.i); gb_dfree(A.j); gb_dfree(A.v); return gb_error_flag; }
      cudaMemcpyAsync(A.i, m->st_rowptr, sizeof(int) * (size_t) (n + 1), cudaMemcpyDeviceToDevice, s);
      int *key = NULL;
      if (m->hint && !m->swap_diag)
      {
         if (m->hint_zero)
         {
            /* some row was given no space: the front rule needs the row lengths */
            int *hI = (int *) malloc(sizeof(int) * (size_t) (n + 1));
            if (!hI) { gb_error(HYPRE_ERROR_MEMORY, "IJ assembly"); return gb_error_flag; }
            cudaMemcpyAsync(hI, m->st_rowptr, sizeof(int) * (size_t) (n + 1), cudaMemcpyDeviceToHost, s);
            gb_sync();
            key = ijm_front_keys(m, hI);
            free(hI);
         }
      }
      gb_ij_gather(n, nnz, NULL, A.i, m->st_cols, m->st_vals, m->swap_diag, key, A.j, A.v, s);
      gb_dfree(key);
      if (m->par) { gb_parcsr_free(m->par); }
      m->par = gb_parcsr_wrap(A, 1);
      m->assembled = 1;
      return gb_error_flag;
   }
   if (!ijm_host_ready(m)) { return gb_error_flag; }
   /* row pointers; host-arena rows are packed behind the device-staged ones
    * (their offsets point past st_len into a temporary upload) */
   int *I = (int *) malloc(sizeof(int) * (size_t) (n + 1));
   long long *off = (long long *) malloc(sizeof(long long) * (size_t) (n ? n : 1));
   if (!I || !off) { free(I); free(off); gb_error(HYPRE_ERROR_MEMORY, "IJ assembly"); return gb_error_flag; }
   I[0] = 0;
   long long nhost = 0;
   for (int i = 0; i < n; i++)
   {
      int l = m->row_len[i];
      I[i + 1] = I[i] + l;
      if (m->row_state[i] == GB_IJ_ROW_DEVICE) { off[i] = m->dev_off[i]; }
      else { off[i] = m->st_len + nhost; nhost += l; }
   }
   int nnz = I[n];
   long long need = m->st_len + nhost;
   if (!ijm_staging_reserve(m, need > 0 ? need : 1))
   {
      free(I); free(off);
      gb_error(HYPRE_ERROR_MEMORY, "IJ device staging");
      return gb_error_flag;
   }
   int *hc = NULL;
   double *hv = NULL;
   if (nhost > 0)
   {
      hc = (int *) malloc(sizeof(int) * (size_t) nhost);
      hv = (double *) malloc(sizeof(double) * (size_t) nhost);
      if (!hc || !hv) { free(I); free(off); free(hc); free(hv); gb_error(HYPRE_ERROR_MEMORY, "IJ assembly"); return gb_error_flag; }
      for (int i = 0; i < n; i++)
      {
         if (m->row_state[i] == GB_IJ_ROW_DEVICE || m->row_len[i] == 0) { continue; }
         long long o = off[i] - m->st_len;
         memcpy(hc + o, m->cols + m->row_off[i], sizeof(int) * (size_t) m->row_len[i]);
         memcpy(hv + o, m->vals + m->row_off[i], sizeof(double) * (size_t) m->row_len[i]);
      }
      cudaMemcpyAsync(m->st_cols + m->st_len, hc, sizeof(int) * (size_t) nhost, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(m->st_vals + m->st_len, hv, sizeof(double) * (size_t) nhost, cudaMemcpyHostToDevice, s);
   }
   gb_csr A;
   A.nr = n; A.nc = m->jupper - m->jlower + 1; A.nnz = nnz;
   A.i = (int *) gb_dmalloc(sizeof(int) * (size_t) (n + 1));
   A.j = (int *) gb_dmalloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
   A.v = (double *) gb_dmalloc(sizeof(double) * (size_t) (nnz ? nnz : 1));
   long long *doff = (long long *) gb_dmalloc(sizeof(long long) * (size_t) (n ? n : 1));
   if (!A.i || !A.j || !A.v || !doff)
   {
      free(I); free(off); free(hc); free(hv);
      gb_dfree(A.i); gb_dfree(A.j); gb_dfree(A.v); gb_dfree(doff);
      return gb_error_flag;
   }
   cudaMemcpyAsync(A.i, I, sizeof(int) * (size_t) (n + 1), cudaMemcpyHostToDevice, s);
   cudaMemcpyAsync(doff, off, sizeof(long long) * (size_t) (n ? n : 1), cudaMemcpyHostToDevice, s);
   int *key = ijm_front_keys(m, I);
   gb_ij_gather(n, A.nnz, doff, A.i, m->st_cols, m->st_vals, m->swap_diag, key, A.j, A.v, s);
   gb_sync();   /* the host buffers above are read by the copies */
   gb_dfree(doff);
   gb_dfree(key);
   free(I); free(off); free(hc); free(hv);
   if (m->par) { gb_parcsr_free(m->par); }
   m->par = gb_parcsr_wrap(A, 1);
   m->assembled = 1;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixGetValues(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_Int *ncols, HYPRE_BigInt *rows,
                                  HYPRE_BigInt *cols, HYPRE_Complex *values)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!m->initialized) { gb_error(HYPRE_ERROR_GENERIC, "IJ matrix not initialized"); return gb_error_flag; }
   if (!ijm_host_ready(m) || !ijm_migrate(m)) { return gb_error_flag; }
   long long k = 0;
   for (int t = 0; t < nrows; t++)
   {
      int r = rows[t] - m->ilower;
      for (int q = 0; q < ncols[t]; q++, k++)
      {
         int c = cols[k] - m->jlower;
         double v = 0.0;
         if (r >= 0 && r < m->nrows)
         {
            const int *rc = m->cols + m->row_off[r];
            for (int z = 0; z < m->row_len[r]; z++) { if (rc[z] == c) { v = m->vals[m->row_off[r] + z]; break; } }
         }
         values[k] = v;
      }
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixGetLocalRange(HYPRE_IJMatrix m, HYPRE_BigInt *il, HYPRE_BigInt *iu, HYPRE_BigInt *jl,
                                      HYPRE_BigInt *ju)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (il) { *il = m->ilower; }
   if (iu) { *iu = m->iupper; }
   if (jl) { *jl = m->jlower; }
   if (ju) { *ju = m->jupper; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixGetObject(HYPRE_IJMatrix m, void **object)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!object) { gb_error_in_arg(2); return gb_error_flag; }
   if (!m->assembled || !m->par) { gb_error(HYPRE_ERROR_GENERIC, "IJ matrix not assembled"); *object = NULL; return gb_error_flag; }
   *object = m->par;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixDestroy(HYPRE_IJMatrix m)
{
   if (!m || m->magic != GB_MAGIC_IJM) { return gb_error_flag; }
   ijm_free_stage(m);
   ij_hfree(m->hint);
   if (m->par) { gb_parcsr_free(m->par); }
   m->magic = 0;
   free(m);
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * IJ vector
 * ------------------------------------------------------------------------ */
struct hypre_IJVector_struct
{
   int        magic;
   int        jlower, jupper, n;
   int        object_type;
   int        num_components;
   double    *h;        /* host mirror for partial puts */
   int        h_valid;  /* h holds the vector's values (plus pending puts) */
   int        h_dirty;  /* h has puts not yet on the device */
   gb_parvec *par;
   int        initialized;
};

static int check_ijv(HYPRE_IJVector v, int arg)
{
   if (!v || v->magic != GB_MAGIC_IJV) { gb_error_in_arg(arg); return 0; }
   return 1;
}

HYPRE_Int HYPRE_IJVectorCreate(MPI_Comm comm, HYPRE_BigInt jlower, HYPRE_BigInt jupper, HYPRE_IJVector *vector)
{
   (void) comm;
   if (!vector) { gb_error_in_arg(4); return gb_error_flag; }
   if (jlower != 0 || jupper < jlower - 1) { gb_error_in_arg(2); return gb_error_flag; }
   gb_runtime_init();
   struct hypre_IJVector_struct *v = calloc(1, sizeof(*v));
   v->magic = GB_MAGIC_IJV;
   v->jlower = jlower; v->jupper = jupper; v->n = jupper - jlower + 1;
   v->num_components = 1;
   *vector = v;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorGetLocalRange(HYPRE_IJVector v, HYPRE_BigInt *jlower, HYPRE_BigInt *jupper)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!jlower) { gb_error_in_arg(2); return gb_error_flag; }
   if (!jupper) { gb_error_in_arg(3); return gb_error_flag; }
   *jlower = v->jlower;
   *jupper = v->jupper;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorSetObjectType(HYPRE_IJVector v, HYPRE_Int type)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (type != HYPRE_PARCSR) { gb_error_in_arg(2); return gb_error_flag; }
   v->object_type = type;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorSetNumComponents(HYPRE_IJVector v, HYPRE_Int nc)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (nc != 1) { gb_error(HYPRE_ERROR_GENERIC, "multi-component IJ vectors: use the batched solve entry points"); gb_error_in_arg(2); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorInitialize(HYPRE_IJVector v)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!v->par) { v->par = gb_parvec_new(v->n); }
   if (v->par) { gb_fill_d(v->n, v->par->d, 0.0, gb_stream()); }
   v->h_valid = 0;
   v->h_dirty = 0;
   v->initialized = 1;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorInitialize_v2(HYPRE_IJVector v, HYPRE_MemoryLocation loc)
{
   (void) loc;
   return HYPRE_IJVectorInitialize(v);
}

/* host mirror = the device vector's current values */
static int ijv_mirror(HYPRE_IJVector v)
{
   if (v->h_valid) { return 1; }
   if (!v->h) { v->h = (double *) malloc(sizeof(double) * (size_t) (v->n ? v->n : 1)); }
   if (!v->h) { gb_error(HYPRE_ERROR_MEMORY, "IJ vector"); return 0; }
   cudaMemcpyAsync(v->h, v->par->d, sizeof(double) * (size_t) v->n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   v->h_valid = 1;
   return 1;
}

/* Puts write the vector's values (as the reference's, which go straight into
 * the ParVector's data).  A put of all n values in order is copied from the
 * caller's buffer to the device; other puts edit the host mirror, which
 * Assemble uploads. */
static HYPRE_Int ijv_put(HYPRE_IJVector v, HYPRE_Int nvalues, const HYPRE_BigInt *idx, const HYPRE_Complex *vals,
                         int add)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!v->initialized) { gb_error(HYPRE_ERROR_GENERIC, "IJ vector not initialized"); return gb_error_flag; }
   if (nvalues < 0) { gb_error_in_arg(2); return gb_error_flag; }
   if (!vals) { gb_error_in_arg(4); return gb_error_flag; }
   if (!add && !idx && nvalues == v->n)
   {
      cudaMemcpyAsync(v->par->d, vals, sizeof(double) * (size_t) v->n, cudaMemcpyHostToDevice, gb_stream());
      gb_sync();
      v->h_valid = 0;
      v->h_dirty = 0;
      return gb_error_flag;
   }
   if (!ijv_mirror(v)) { return gb_error_flag; }
   for (int k = 0; k < nvalues; k++)
   {
      int i = idx ? idx[k] - v->jlower : k;
      if (i < 0 || i >= v->n) { gb_error_in_arg(3); continue; }
      if (add) { v->h[i] += vals[k]; } else { v->h[i] = vals[k]; }
   }
   v->h_dirty = 1;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorSetValues(HYPRE_IJVector v, HYPRE_Int nvalues, const HYPRE_BigInt *idx,
                                  const HYPRE_Complex *vals)
{
   return ijv_put(v, nvalues, idx, vals, 0);
}

HYPRE_Int HYPRE_IJVectorAddToValues(HYPRE_IJVector v, HYPRE_Int nvalues, const HYPRE_BigInt *idx,
                                    const HYPRE_Complex *vals)
{
   return ijv_put(v, nvalues, idx, vals, 1);
}

HYPRE_Int HYPRE_IJVectorAssemble(HYPRE_IJVector v)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!v->initialized) { gb_error(HYPRE_ERROR_GENERIC, "IJ vector not initialized"); return gb_error_flag; }
   if (v->h_dirty)
   {
      cudaMemcpyAsync(v->par->d, v->h, sizeof(double) * (size_t) v->n, cudaMemcpyHostToDevice, gb_stream());
      gb_sync();
      v->h_dirty = 0;
   }
   /* solves change the device vector from here on */
   v->h_valid = 0;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorGetValues(HYPRE_IJVector v, HYPRE_Int nvalues, const HYPRE_BigInt *idx, HYPRE_Complex *vals)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!vals) { gb_error_in_arg(4); return gb_error_flag; }
   if (!v->initialized || !v->par) { gb_error(HYPRE_ERROR_GENERIC, "IJ vector not initialized"); return gb_error_flag; }
   if (!v->h_dirty && !idx && nvalues == v->n)
   {
      /* the device vector (it may have been changed by a solve) */
      cudaMemcpyAsync(vals, v->par->d, sizeof(double) * (size_t) v->n, cudaMemcpyDeviceToHost, gb_stream());
      gb_sync();
      return gb_error_flag;
   }
   if (!v->h_dirty) { v->h_valid = 0; }
   if (!ijv_mirror(v)) { return gb_error_flag; }
   for (int k = 0; k < nvalues; k++)
   {
      int i = idx ? idx[k] - v->jlower : k;
      if (i < 0 || i >= v->n) { gb_error_in_arg(3); continue; }
      vals[k] = v->h[i];
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorGetObject(HYPRE_IJVector v, void **object)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!object) { gb_error_in_arg(2); return gb_error_flag; }
   *object = v->par;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorDestroy(HYPRE_IJVector v)
{
   if (!v || v->magic != GB_MAGIC_IJV) { return gb_error_flag; }
   free(v->h);
   if (v->par) { gb_parvec_free(v->par); }
   v->magic = 0;
   free(v);
   return gb_error_flag;
}

/* ------------------------------------------------------------------------
 * The rest of the reference's IJ interface for one process
 * (HYPRE_IJ_mv.h:140-750): object types, row counts, constant values, the
 * inner product of two IJ vectors, and the settings that only concern
 * off-process entries, printing, threading or the memory location, which
 * one process holding its data on the device accepts and ignores.
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_IJMatrixGetObjectType(HYPRE_IJMatrix m, HYPRE_Int *type)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!type) { gb_error_in_arg(2); return gb_error_flag; }
   *type = m->object_type;
   return gb_error_flag;
}

/* the assembled rows' lengths (IJMatrix_parcsr.c:449-495: the ParCSR's row
 * pointers; rows outside the local range count 0) */
HYPRE_Int HYPRE_IJMatrixGetRowCounts(HYPRE_IJMatrix m, HYPRE_Int nrows, HYPRE_BigInt *rows, HYPRE_Int *ncols)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (nrows < 0) { gb_error_in_arg(2); return gb_error_flag; }
   if (nrows > 0 && !rows) { gb_error_in_arg(3); return gb_error_flag; }
   if (nrows > 0 && !ncols) { gb_error_in_arg(4); return gb_error_flag; }
   if (!m->assembled || !m->par) { gb_error(HYPRE_ERROR_GENERIC, "IJ matrix not assembled"); return gb_error_flag; }
   const int n = m->par->A.nr;
   int *ptr = (int *) malloc(sizeof(int) * (size_t) (n + 1));
   if (!ptr) { gb_error(HYPRE_ERROR_MEMORY, "row counts"); return gb_error_flag; }
   cudaMemcpyAsync(ptr, m->par->A.i, sizeof(int) * (size_t) (n + 1), cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   for (int t = 0; t < nrows; t++)
   {
      const long long r = (long long) rows[t] - m->ilower;
      ncols[t] = (r >= 0 && r < n) ? ptr[r + 1] - ptr[r] : 0;
   }
   free(ptr);
   return gb_error_flag;
}

/* every stored entry of the assembled matrix takes the value
 * (hypre_IJMatrixSetConstantValuesParCSR, IJMatrix_parcsr.c:1170-1198, which
 * requires assembly); the value-dependent solve forms are rebuilt on use */
HYPRE_Int HYPRE_IJMatrixSetConstantValues(HYPRE_IJMatrix m, HYPRE_Complex value)
{
   if (!check_ijm(m, 1)) { return gb_error_flag; }
   if (!m->assembled || !m->par) { gb_error(HYPRE_ERROR_GENERIC, "IJ matrix not assembled"); return gb_error_flag; }
   gb_parcsr *M = m->par;
   gb_fill_d(M->A.nnz, M->A.v, value, gb_stream());
   for (int p = 0; p < 3; p++) { solveform_free(&M->sf[p]); }
   gb_dfree(M->diag);
   M->diag = NULL;
   free(M->row_vals);
   M->row_vals = NULL;
   free(M->row_cols);
   M->row_cols = NULL;
   /* the host copy of the rows that GetValues reads */
   if (!ijm_host_ready(m) || !ijm_migrate(m)) { return gb_error_flag; }
   for (int r = 0; r < m->nrows; r++)
   {
      for (int z = 0; z < m->row_len[r]; z++) { m->vals[m->row_off[r] + z] = value; }
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetMaxOffProcElmts(HYPRE_IJMatrix m, HYPRE_Int v)
{
   (void) v;
   check_ijm(m, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetPrintLevel(HYPRE_IJMatrix m, HYPRE_Int v)
{
   (void) v;
   check_ijm(m, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixSetOMPFlag(HYPRE_IJMatrix m, HYPRE_Int v)
{
   (void) v;
   check_ijm(m, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixMigrate(HYPRE_IJMatrix m, HYPRE_MemoryLocation loc)
{
   (void) loc;
   check_ijm(m, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorGetObjectType(HYPRE_IJVector v, HYPRE_Int *type)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!type) { gb_error_in_arg(2); return gb_error_flag; }
   *type = v->object_type;
   return gb_error_flag;
}

/* every value of the vector (hypre_IJVectorSetConstantValuesPar) */
HYPRE_Int HYPRE_IJVectorSetConstantValues(HYPRE_IJVector v, HYPRE_Complex value)
{
   if (!check_ijv(v, 1)) { return gb_error_flag; }
   if (!v->initialized || !v->par) { gb_error(HYPRE_ERROR_GENERIC, "IJ vector not initialized"); return gb_error_flag; }
   gb_fill_d(v->n, v->par->d, value, gb_stream());
   v->h_valid = 0;
   v->h_dirty = 0;
   return gb_error_flag;
}

/* <x, y> of the two vectors' current values (hypre_IJVectorInnerProdPar) */
HYPRE_Int HYPRE_IJVectorInnerProd(HYPRE_IJVector x, HYPRE_IJVector y, HYPRE_Real *prod)
{
   if (!check_ijv(x, 1)) { return gb_error_flag; }
   if (!y || y->magic != GB_MAGIC_IJV) { gb_error_in_arg(2); return gb_error_flag; }
   if (!prod) { gb_error_in_arg(3); return gb_error_flag; }
   if (!x->par || !y->par || x->n != y->n) { gb_error_in_arg(2); return gb_error_flag; }
   if (x->h_dirty || y->h_dirty)
   {
      gb_error(HYPRE_ERROR_GENERIC, "IJ vector values put but not assembled");
      return gb_error_flag;
   }
   *prod = gb_dot(x->n, x->par->d, y->par->d);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorSetMaxOffProcElmts(HYPRE_IJVector v, HYPRE_Int n)
{
   (void) n;
   check_ijv(v, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorSetPrintLevel(HYPRE_IJVector v, HYPRE_Int n)
{
   (void) n;
   check_ijv(v, 1);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorMigrate(HYPRE_IJVector v, HYPRE_MemoryLocation loc)
{
   (void) loc;
   check_ijv(v, 1);
   return gb_error_flag;
}
