/* IJ matrix and vector files: the reference's ASCII IJ format, Matrix Market
 * coordinate files and its binary IJ format, for one process (file suffix
 * ".00000", ".00000.bin").
 *
 *   matrix read    src/IJ_mv/IJMatrix.c:110-241 (hypre_IJMatrixRead: IJ and
 *                  Matrix Market), :252-520 (hypre_IJMatrixReadBinary);
 *                  Matrix Market banner and size line src/utilities/mmio.c
 *   matrix print   src/parcsr_mv/par_csr_matrix.c:940-1070 (PrintIJ),
 *                  :1140-1330 (PrintBinaryIJ)
 *   vector read    src/IJ_mv/HYPRE_IJVector.c:785-845, src/IJ_mv/IJVector.c:110-240
 *   vector print   src/IJ_mv/HYPRE_IJVector.c:862-920, src/parcsr_mv/par_vector.c:1360-1440
 *
 * Readers feed the entries through SetValues / AddToValues in file order, as
 * the reference does (entries of rows outside the range go to AddToValues;
 * a repeated entry replaces the earlier one), so the assembled matrix follows
 * the IJ interface's rules.  Consecutive entries of one row are passed in one
 * SetValues call, which gives the same result as one call per entry. */
#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gb_internal.h"

#define GB_IO_NAME 1100

/* --------------------------------------------------------------------------
 * COO entry lists
 * ------------------------------------------------------------------------ */
typedef struct
{
   long long n, cap;
   int      *r, *c;
   double   *v;
} gb_coo;

static int coo_push(gb_coo *e, int r, int c, double v)
{
   if (e->n == e->cap)
   {
      long long nc = e->cap ? 2 * e->cap : 4096;
      int *nr = (int *) realloc(e->r, sizeof(int) * (size_t) nc);
      if (nr) { e->r = nr; }
      int *ncl = (int *) realloc(e->c, sizeof(int) * (size_t) nc);
      if (ncl) { e->c = ncl; }
      double *nv = (double *) realloc(e->v, sizeof(double) * (size_t) nc);
      if (nv) { e->v = nv; }
      if (!nr || !ncl || !nv) { return 0; }
      e->cap = nc;
   }
   e->r[e->n] = r;
   e->c[e->n] = c;
   e->v[e->n] = v;
   e->n++;
   return 1;
}

static void coo_free(gb_coo *e)
{
   free(e->r); free(e->c); free(e->v);
   memset(e, 0, sizeof(*e));
}

/* Matrix Market banner: "%%MatrixMarket matrix coordinate real|integer
 * general|symmetric" (object, format, field and symmetry in any case).
 * Returns 0 and sets *sym, or a message. */
static const char *mm_banner(FILE *f, int *sym)
{
   char line[1030], banner[1030], mtx[1030], crd[1030], field[1030], symm[1030];
   if (!fgets(line, sizeof(line), f)) { return "Could not process Matrix Market banner."; }
   if (sscanf(line, "%1029s %1029s %1029s %1029s %1029s", banner, mtx, crd, field, symm) != 5)
   {
      return "Could not process Matrix Market banner.";
   }
   for (char *p = mtx; *p; p++) { *p = (char) tolower((unsigned char) *p); }
   for (char *p = crd; *p; p++) { *p = (char) tolower((unsigned char) *p); }
   for (char *p = field; *p; p++) { *p = (char) tolower((unsigned char) *p); }
   for (char *p = symm; *p; p++) { *p = (char) tolower((unsigned char) *p); }
   if (strncmp(banner, "%%MatrixMarket", 14) != 0 || strcmp(mtx, "matrix") != 0)
   {
      return "Could not process Matrix Market banner.";
   }
   int dense = strcmp(crd, "array") == 0;
   if (!dense && strcmp(crd, "coordinate") != 0) { return "Could not process Matrix Market banner."; }
   int real = strcmp(field, "real") == 0, integer = strcmp(field, "integer") == 0;
   int complex_ = strcmp(field, "complex") == 0, pattern = strcmp(field, "pattern") == 0;
   if (!real && !integer && !complex_ && !pattern) { return "Could not process Matrix Market banner."; }
   int general = strcmp(symm, "general") == 0, symmetric = strcmp(symm, "symmetric") == 0;
   int herm = strcmp(symm, "hermitian") == 0, skew = strcmp(symm, "skew-symmetric") == 0;
   if (!general && !symmetric && !herm && !skew) { return "Could not process Matrix Market banner."; }
   /* combinations the format itself rules out */
   if ((dense && pattern) || ((real || integer) && herm) || (pattern && (herm || skew)))
   {
      return "Invalid Matrix Market file.";
   }
   if (!((real || integer) && !dense))
   {
      return "Only sparse real-valued/integer coordinate matrices are supported";
   }
   *sym = symmetric;
   return NULL;
}

/* size line after the comment lines */
static int mm_size(FILE *f, int *m, int *n, int *nz)
{
   char line[1030];
   do
   {
      if (!fgets(line, sizeof(line), f)) { return 0; }
   }
   while (line[0] == '%');
   if (sscanf(line, "%d %d %d", m, n, nz) == 3) { return 1; }
   for (;;)
   {
      int k = fscanf(f, "%d %d %d", m, n, nz);
      if (k == EOF) { return 0; }
      if (k == 3) { return 1; }
   }
}

/* Reads the entries of an IJ (is_mm 0) or Matrix Market (is_mm 1) file in
 * file order, 0-based (Matrix Market entries shifted by one, symmetric files
 * mirrored: (j, i) follows (i, j) for i != j), and the index range. */
static const char *read_text(const char *filename, int is_mm, int range[4], gb_coo *e, int *missing)
{
   char name[GB_IO_NAME];
   *missing = 0;
   if (is_mm) { snprintf(name, sizeof(name), "%s", filename); }
   else { snprintf(name, sizeof(name), "%s.%05d", filename, 0); }
   FILE *f = fopen(name, "r");
   if (!f) { *missing = 1; return "could not open the input file"; }
   int sym = 0;
   if (is_mm)
   {
      const char *msg = mm_banner(f, &sym);
      int nr = 0, nc = 0, nz = 0;
      if (!msg && !mm_size(f, &nr, &nc, &nz)) { msg = "MM read size error !"; }
      if (msg) { fclose(f); return msg; }
      range[0] = 0; range[1] = nr - 1; range[2] = 0; range[3] = nc - 1;
   }
   else if (fscanf(f, "%d %d %d %d", &range[0], &range[1], &range[2], &range[3]) != 4)
   {
      fclose(f);
      return "Error in IJ matrix input file.";
   }
   int i, j, ret;
   double v;
   /* whitespace must follow the column index (a line with a single number
    * then fails instead of being read as an index and a value) */
   while ((ret = fscanf(f, "%d %d%*[ \t]%le", &i, &j, &v)) != EOF)
   {
      if (ret != 3) { fclose(f); return "Error in IJ matrix input file."; }
      if (is_mm) { i--; j--; }
      if (!coo_push(e, i, j, v)) { fclose(f); return "out of host memory"; }
      if (sym && i != j && !coo_push(e, j, i, v)) { fclose(f); return "out of host memory"; }
   }
   fclose(f);
   return NULL;
}

/* IJ matrix from entries in order: runs of one in-range row go through one
 * SetValues call, rows outside the range through AddToValues */
static HYPRE_Int build_matrix(const int range[4], const gb_coo *e, HYPRE_Int type, HYPRE_IJMatrix *matrix)
{
   HYPRE_IJMatrix m = NULL;
   HYPRE_IJMatrixCreate(0, range[0], range[1], range[2], range[3], &m);
   if (!m) { return gb_error_flag; }
   HYPRE_IJMatrixSetObjectType(m, type);
   HYPRE_IJMatrixInitialize(m);
   long long k = 0;
   while (k < e->n)
   {
      const int r = e->r[k];
      long long q = k + 1;
      if (r < range[0] || r > range[1])
      {
         int one = 1;
         HYPRE_IJMatrixAddToValues(m, 1, &one, &e->r[k], &e->c[k], &e->v[k]);
      }
      else
      {
         while (q < e->n && e->r[q] == r && q - k < 0x7fffffff) { q++; }
         int nc = (int) (q - k);
         HYPRE_IJMatrixSetValues(m, 1, &nc, &e->r[k], &e->c[k], &e->v[k]);
      }
      k = q;
   }
   HYPRE_IJMatrixAssemble(m);
   *matrix = m;
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixRead(const char *filename, MPI_Comm comm, HYPRE_Int type, HYPRE_IJMatrix *matrix)
{
   (void) comm;
   if (!filename) { gb_error_in_arg(1); return gb_error_flag; }
   if (!matrix) { gb_error_in_arg(4); return gb_error_flag; }
   gb_coo e;
   memset(&e, 0, sizeof(e));
   int range[4], missing = 0;
   const char *msg = read_text(filename, 0, range, &e, &missing);
   if (msg)
   {
      if (missing) { gb_error_in_arg(1); }
      else { gb_error(HYPRE_ERROR_GENERIC, msg); }
      coo_free(&e);
      return gb_error_flag;
   }
   build_matrix(range, &e, type, matrix);
   coo_free(&e);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixReadMM(const char *filename, MPI_Comm comm, HYPRE_Int type, HYPRE_IJMatrix *matrix)
{
   (void) comm;
   if (!filename) { gb_error_in_arg(1); return gb_error_flag; }
   if (!matrix) { gb_error_in_arg(4); return gb_error_flag; }
   gb_coo e;
   memset(&e, 0, sizeof(e));
   int range[4], missing = 0;
   const char *msg = read_text(filename, 1, range, &e, &missing);
   if (msg)
   {
      if (missing) { gb_error_in_arg(1); }
      else { gb_error(HYPRE_ERROR_GENERIC, msg); }
      coo_free(&e);
      return gb_error_flag;
   }
   build_matrix(range, &e, type, matrix);
   coo_free(&e);
   return gb_error_flag;
}

/* binary IJ file: 11 uint64 header (version 1, index bytes, value bytes,
 * global rows, global columns, global nonzeros, local nonzeros, ilower,
 * iupper, jlower, jupper), row indices, column indices, values */
static int read_index_array(FILE *f, size_t ib, long long n, int *out)
{
   if (ib == 4)
   {
      uint32_t *b = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (n ? n : 1));
      if (!b || fread(b, sizeof(uint32_t), (size_t) n, f) != (size_t) n) { free(b); return 0; }
      int ok = 1;
      for (long long k = 0; k < n; k++) { ok &= b[k] <= 0x7fffffffu; out[k] = (int) b[k]; }
      free(b);
      return ok ? 1 : -1;
   }
   uint64_t *b = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (n ? n : 1));
   if (!b || fread(b, sizeof(uint64_t), (size_t) n, f) != (size_t) n) { free(b); return 0; }
   int ok = 1;
   for (long long k = 0; k < n; k++) { ok &= b[k] <= 0x7fffffffULL; out[k] = (int) b[k]; }
   free(b);
   return ok ? 1 : -1;
}

HYPRE_Int HYPRE_IJMatrixReadBinary(const char *filename, MPI_Comm comm, HYPRE_Int type, HYPRE_IJMatrix *matrix)
{
   (void) comm;
   if (!filename) { gb_error_in_arg(1); return gb_error_flag; }
   if (!matrix) { gb_error_in_arg(4); return gb_error_flag; }
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d.bin", filename, 0);
   FILE *f = fopen(name, "rb");
   if (!f) { gb_error(HYPRE_ERROR_GENERIC, "Could not open input file"); return gb_error_flag; }
   uint64_t h[11];
   if (fread(h, sizeof(uint64_t), 11, f) != 11)
   {
      fclose(f);
      gb_error(HYPRE_ERROR_GENERIC, "Could not read header entries");
      return gb_error_flag;
   }
   const char *msg = NULL;
   if (h[0] != 1) { msg = "Unsupported header version"; }
   else if (h[6] > 0x7fffffffULL) { msg = "Detected integer overflow at 7th header entry"; }
   else if (h[1] != 4 && h[1] != 8) { msg = "Unsupported data type for row/column indices"; }
   else if (h[2] != 4 && h[2] != 8) { msg = "Unsupported data type for matrix coefficients"; }
   else if (h[7] > 0x7fffffffULL || h[8] > 0x7fffffffULL || h[9] > 0x7fffffffULL || h[10] > 0x7fffffffULL)
   {
      msg = "index range beyond 32-bit HYPRE_BigInt";
   }
   if (msg) { fclose(f); gb_error(HYPRE_ERROR_GENERIC, msg); return gb_error_flag; }
   const long long nnz = (long long) h[6];
   gb_coo e;
   memset(&e, 0, sizeof(e));
   e.n = e.cap = nnz;
   e.r = (int *) malloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
   e.c = (int *) malloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
   e.v = (double *) malloc(sizeof(double) * (size_t) (nnz ? nnz : 1));
   int ok = e.r && e.c && e.v;
   int ri = ok ? read_index_array(f, (size_t) h[1], nnz, e.r) : 0;
   int ci = ri == 1 ? read_index_array(f, (size_t) h[1], nnz, e.c) : ri;
   if (ci == 1)
   {
      if (h[2] == 4)
      {
         float *b = (float *) malloc(sizeof(float) * (size_t) (nnz ? nnz : 1));
         if (b && fread(b, sizeof(float), (size_t) nnz, f) == (size_t) nnz)
         {
            for (long long k = 0; k < nnz; k++) { e.v[k] = (double) b[k]; }
         }
         else { ci = 0; }
         free(b);
      }
      else if (fread(e.v, sizeof(double), (size_t) nnz, f) != (size_t) nnz) { ci = 0; }
   }
   fclose(f);
   if (ci != 1)
   {
      coo_free(&e);
      gb_error(HYPRE_ERROR_GENERIC, ci < 0 ? "index beyond 32-bit HYPRE_BigInt" : "Could not read all entries");
      return gb_error_flag;
   }
   int range[4] = {(int) h[7], (int) h[8], (int) h[9], (int) h[10]};
   build_matrix(range, &e, type, matrix);
   coo_free(&e);
   return gb_error_flag;
}

/* host copy of the assembled matrix: CSR with the diagonal first */
static int host_csr(HYPRE_IJMatrix matrix, int *n, int **I, int **J, double **V, int range[4])
{
   void *obj = NULL;
   if (HYPRE_IJMatrixGetObject(matrix, &obj) || !obj) { return 0; }
   HYPRE_IJMatrixGetLocalRange(matrix, &range[0], &range[1], &range[2], &range[3]);
   gb_parcsr *M = (gb_parcsr *) obj;
   const gb_csr *A = &M->A;
   *n = A->nr;
   *I = (int *) malloc(sizeof(int) * (size_t) (A->nr + 1));
   *J = (int *) malloc(sizeof(int) * (size_t) (A->nnz ? A->nnz : 1));
   *V = (double *) malloc(sizeof(double) * (size_t) (A->nnz ? A->nnz : 1));
   if (!*I || !*J || !*V) { free(*I); free(*J); free(*V); gb_error(HYPRE_ERROR_MEMORY, "print"); return 0; }
   cudaStream_t s = gb_stream();
   cudaMemcpyAsync(*I, A->i, sizeof(int) * (size_t) (A->nr + 1), cudaMemcpyDeviceToHost, s);
   if (A->nnz)
   {
      cudaMemcpyAsync(*J, A->j, sizeof(int) * (size_t) A->nnz, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(*V, A->v, sizeof(double) * (size_t) A->nnz, cudaMemcpyDeviceToHost, s);
   }
   if (gb_sync()) { free(*I); free(*J); free(*V); return 0; }
   return 1;
}

HYPRE_Int HYPRE_IJMatrixPrint(HYPRE_IJMatrix matrix, const char *filename)
{
   if (!matrix) { gb_error_in_arg(1); return gb_error_flag; }
   if (!filename) { gb_error_in_arg(2); return gb_error_flag; }
   int n = 0, range[4], *I = NULL, *J = NULL;
   double *V = NULL;
   if (!host_csr(matrix, &n, &I, &J, &V, range)) { return gb_error_flag; }
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d", filename, 0);
   FILE *f = fopen(name, "w");
   if (!f) { free(I); free(J); free(V); gb_error_in_arg(2); return gb_error_flag; }
   fprintf(f, "%d %d %d %d\n", range[0], range[1], range[2], range[3]);
   for (int i = 0; i < n; i++)
   {
      for (int k = I[i]; k < I[i + 1]; k++) { fprintf(f, "%d %d %.14e\n", range[0] + i, range[2] + J[k], V[k]); }
   }
   fclose(f);
   free(I); free(J); free(V);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJMatrixPrintBinary(HYPRE_IJMatrix matrix, const char *filename)
{
   if (!matrix) { gb_error_in_arg(1); return gb_error_flag; }
   if (!filename) { gb_error_in_arg(2); return gb_error_flag; }
   int n = 0, range[4], *I = NULL, *J = NULL;
   double *V = NULL;
   if (!host_csr(matrix, &n, &I, &J, &V, range)) { return gb_error_flag; }
   const long long nnz = I[n];
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d.bin", filename, 0);
   FILE *f = fopen(name, "wb");
   uint32_t *rb = (uint32_t *) malloc(sizeof(uint32_t) * (size_t) (nnz ? nnz : 1));
   if (!f || !rb)
   {
      if (f) { fclose(f); }
      free(rb); free(I); free(J); free(V);
      gb_error(HYPRE_ERROR_GENERIC, "Could not open output file!");
      return gb_error_flag;
   }
   uint64_t h[11] = {1, sizeof(HYPRE_BigInt), sizeof(HYPRE_Complex), (uint64_t) (range[1] - range[0] + 1),
                     (uint64_t) (range[3] - range[2] + 1), (uint64_t) nnz, (uint64_t) nnz, (uint64_t) range[0],
                     (uint64_t) range[1], (uint64_t) range[2], (uint64_t) range[3]};
   size_t w = fwrite(h, sizeof(uint64_t), 11, f);
   for (int i = 0; i < n; i++)
   {
      for (int k = I[i]; k < I[i + 1]; k++) { rb[k] = (uint32_t) (range[0] + i); }
   }
   w += fwrite(rb, sizeof(uint32_t), (size_t) nnz, f);
   for (long long k = 0; k < nnz; k++) { rb[k] = (uint32_t) (range[2] + J[k]); }
   w += fwrite(rb, sizeof(uint32_t), (size_t) nnz, f);
   w += fwrite(V, sizeof(double), (size_t) nnz, f);
   fclose(f);
   free(rb); free(I); free(J); free(V);
   if (w != 11 + 3 * (size_t) nnz) { gb_error(HYPRE_ERROR_GENERIC, "Could not write all entries"); }
   return gb_error_flag;
}

/* --------------------------------------------------------------------------
 * vectors
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_IJVectorRead(const char *filename, MPI_Comm comm, HYPRE_Int type, HYPRE_IJVector *vector)
{
   (void) comm;
   if (!filename) { gb_error_in_arg(1); return gb_error_flag; }
   if (!vector) { gb_error_in_arg(4); return gb_error_flag; }
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d", filename, 0);
   FILE *f = fopen(name, "r");
   if (!f) { gb_error_in_arg(1); return gb_error_flag; }
   int jlower = 0, jupper = -1;
   if (fscanf(f, "%d %d", &jlower, &jupper) != 2)
   {
      fclose(f);
      gb_error(HYPRE_ERROR_GENERIC, "Error in IJ vector input file.");
      return gb_error_flag;
   }
   HYPRE_IJVector v = NULL;
   HYPRE_IJVectorCreate(0, jlower, jupper, &v);
   if (!v) { fclose(f); return gb_error_flag; }
   HYPRE_IJVectorSetObjectType(v, type);
   HYPRE_IJVectorInitialize(v);
   gb_coo e;
   memset(&e, 0, sizeof(e));
   int j, ret;
   double x;
   const char *msg = NULL;
   while ((ret = fscanf(f, "%d%*[ \t]%le", &j, &x)) != EOF)
   {
      if (ret != 2) { msg = "Error in IJ vector input file."; break; }
      if (!coo_push(&e, j, 0, x)) { msg = "out of host memory"; break; }
   }
   fclose(f);
   if (msg) { gb_error(HYPRE_ERROR_GENERIC, msg); coo_free(&e); *vector = v; return gb_error_flag; }
   /* in-range entries in runs, rows outside the range through AddToValues */
   long long k = 0;
   while (k < e.n)
   {
      long long q = k;
      if (e.r[k] < jlower || e.r[k] > jupper)
      {
         HYPRE_IJVectorAddToValues(v, 1, &e.r[k], &e.v[k]);
         k++;
         continue;
      }
      while (q < e.n && e.r[q] >= jlower && e.r[q] <= jupper && q - k < 0x7fffffff) { q++; }
      HYPRE_IJVectorSetValues(v, (int) (q - k), &e.r[k], &e.v[k]);
      k = q;
   }
   coo_free(&e);
   HYPRE_IJVectorAssemble(v);
   *vector = v;
   return gb_error_flag;
}

/* binary vector file: 8 uint64 header (version 1, value bytes, first index,
 * last index + 1, global size, local size, components, storage method),
 * then the values (components one after another) */
HYPRE_Int HYPRE_IJVectorReadBinary(const char *filename, MPI_Comm comm, HYPRE_Int type, HYPRE_IJVector *vector)
{
   (void) comm;
   if (!filename) { gb_error_in_arg(1); return gb_error_flag; }
   if (!vector) { gb_error_in_arg(4); return gb_error_flag; }
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d.bin", filename, 0);
   FILE *f = fopen(name, "rb");
   if (!f) { gb_error(HYPRE_ERROR_GENERIC, "Could not open input file"); return gb_error_flag; }
   uint64_t h[8];
   const char *msg = NULL;
   if (fread(h, sizeof(uint64_t), 8, f) != 8) { msg = "Could not read header entries"; }
   else if (h[0] != 1) { msg = "Unsupported header version"; }
   else if (h[7] == 1) { msg = "row-wise ordering is not supported!"; }
   else if (h[5] > h[4] || h[3] < h[2] || h[3] - h[2] != h[5]) { msg = "Invalid vector size!"; }
   else if (h[6] != 1) { msg = "multi-component IJ vectors: use the batched solve entry points"; }
   else if (h[1] != 4 && h[1] != 8) { msg = "Unsupported data type for vector entries"; }
   else if (h[3] > 0x7fffffffULL) { msg = "index range beyond 32-bit HYPRE_BigInt"; }
   if (msg) { fclose(f); gb_error(HYPRE_ERROR_GENERIC, msg); return gb_error_flag; }
   const long long n = (long long) h[5];
   double *x = (double *) malloc(sizeof(double) * (size_t) (n ? n : 1));
   int ok = x != NULL;
   if (ok && h[1] == 4)
   {
      float *b = (float *) malloc(sizeof(float) * (size_t) (n ? n : 1));
      ok = b && fread(b, sizeof(float), (size_t) n, f) == (size_t) n;
      for (long long k = 0; ok && k < n; k++) { x[k] = (double) b[k]; }
      free(b);
   }
   else if (ok) { ok = fread(x, sizeof(double), (size_t) n, f) == (size_t) n; }
   fclose(f);
   if (!ok) { free(x); gb_error(HYPRE_ERROR_GENERIC, "Could not read all vector coefficients"); return gb_error_flag; }
   HYPRE_IJVector v = NULL;
   HYPRE_IJVectorCreate(0, (int) h[2], (int) h[3] - 1, &v);
   if (v)
   {
      HYPRE_IJVectorSetObjectType(v, type);
      HYPRE_IJVectorInitialize(v);
      HYPRE_IJVectorSetValues(v, (int) n, NULL, x);
      HYPRE_IJVectorAssemble(v);
   }
   free(x);
   *vector = v;
   return gb_error_flag;
}

static int vector_host(HYPRE_IJVector vector, int *jlower, int *jupper, double **x)
{
   if (HYPRE_IJVectorGetLocalRange(vector, jlower, jupper)) { return 0; }
   const int n = *jupper - *jlower + 1;
   *x = (double *) malloc(sizeof(double) * (size_t) (n > 0 ? n : 1));
   if (!*x) { gb_error(HYPRE_ERROR_MEMORY, "print"); return 0; }
   if (HYPRE_IJVectorGetValues(vector, n, NULL, *x)) { free(*x); return 0; }
   return 1;
}

HYPRE_Int HYPRE_IJVectorPrint(HYPRE_IJVector vector, const char *filename)
{
   if (!vector) { gb_error_in_arg(1); return gb_error_flag; }
   if (!filename) { gb_error_in_arg(2); return gb_error_flag; }
   int jl = 0, ju = -1;
   double *x = NULL;
   if (!vector_host(vector, &jl, &ju, &x)) { return gb_error_flag; }
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d", filename, 0);
   FILE *f = fopen(name, "w");
   if (!f) { free(x); gb_error_in_arg(2); return gb_error_flag; }
   fprintf(f, "%d %d\n", jl, ju);
   for (int j = 0; j <= ju - jl; j++) { fprintf(f, "%d %.14e\n", jl + j, x[j]); }
   fclose(f);
   free(x);
   return gb_error_flag;
}

HYPRE_Int HYPRE_IJVectorPrintBinary(HYPRE_IJVector vector, const char *filename)
{
   if (!vector) { gb_error_in_arg(1); return gb_error_flag; }
   if (!filename) { gb_error_in_arg(2); return gb_error_flag; }
   int jl = 0, ju = -1;
   double *x = NULL;
   if (!vector_host(vector, &jl, &ju, &x)) { return gb_error_flag; }
   char name[GB_IO_NAME];
   snprintf(name, sizeof(name), "%s.%05d.bin", filename, 0);
   FILE *f = fopen(name, "wb");
   if (!f) { free(x); gb_error(HYPRE_ERROR_GENERIC, "Could not open output file!"); return gb_error_flag; }
   const uint64_t n = (uint64_t) (ju - jl + 1);
   uint64_t h[8] = {1, sizeof(HYPRE_Complex), (uint64_t) jl, (uint64_t) (ju + 1), n, n, 1, 0};
   size_t w = fwrite(h, sizeof(uint64_t), 8, f);
   w += fwrite(x, sizeof(double), (size_t) n, f);
   fclose(f);
   free(x);
   if (w != 8 + (size_t) n) { gb_error(HYPRE_ERROR_GENERIC, "Could not write all entries"); }
   return gb_error_flag;
}

/* ------------------------------------------------------------------------
 * ParVector text files of one process (hypre_ParVectorPrint / Read,
 * src/parcsr_mv/par_vector.c:330-410, with hypre_SeqVectorPrint / Read
 * src/seq_mv/vector.c:420-525): <name>.0 holds the size and then one value
 * per line (%.14e); <name>.INFO.0 the global size and the row range [0, n).
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_ParVectorPrint(HYPRE_ParVector vector, const char *file_name)
{
   gb_parvec *v = (gb_parvec *) vector;
   if (!v || v->magic != GB_MAGIC_VEC || !v->d) { gb_error_in_arg(1); return gb_error_flag; }
   if (!file_name) { gb_error_in_arg(2); return gb_error_flag; }
   const int n = v->n;
   double *h = (double *) malloc(sizeof(double) * (size_t) (n > 0 ? n : 1));
   if (!h) { gb_error(HYPRE_ERROR_MEMORY, "ParVectorPrint"); return gb_error_flag; }
   cudaMemcpyAsync(h, v->d, sizeof(double) * (size_t) n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   char name[4096];
   snprintf(name, sizeof(name), "%s.0", file_name);
   FILE *f = fopen(name, "w");
   if (!f) { free(h); gb_error(HYPRE_ERROR_GENERIC, "ParVectorPrint: cannot open the file"); return gb_error_flag; }
   fprintf(f, "%d\n", n);
   for (int i = 0; i < n; i++) { fprintf(f, "%.14e\n", h[i]); }
   fclose(f);
   free(h);
   snprintf(name, sizeof(name), "%s.INFO.0", file_name);
   f = fopen(name, "w");
   if (!f) { gb_error(HYPRE_ERROR_GENERIC, "ParVectorPrint: cannot open the file"); return gb_error_flag; }
   fprintf(f, "%d\n%d\n%d\n", n, 0, n);
   fclose(f);
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParVectorRead(MPI_Comm comm, const char *file_name, HYPRE_ParVector *vector)
{
   (void) comm;
   if (!file_name) { gb_error_in_arg(2); return gb_error_flag; }
   if (!vector) { gb_error_in_arg(3); return gb_error_flag; }
   *vector = NULL;
   char name[4096];
   snprintf(name, sizeof(name), "%s.INFO.0", file_name);
   FILE *f = fopen(name, "r");
   int gsize = 0, p0 = 0, p1 = 0;
   if (!f || fscanf(f, "%d %d %d", &gsize, &p0, &p1) != 3)
   {
      if (f) { fclose(f); }
      gb_error(HYPRE_ERROR_GENERIC, "ParVectorRead: cannot read the INFO file");
      return gb_error_flag;
   }
   fclose(f);
   snprintf(name, sizeof(name), "%s.0", file_name);
   f = fopen(name, "r");
   int n = 0;
   if (!f || fscanf(f, "%d", &n) != 1 || n < 0 || n != p1 - p0 || n != gsize)
   {
      if (f) { fclose(f); }
      gb_error(HYPRE_ERROR_GENERIC, "ParVectorRead: cannot read the vector file (one process)");
      return gb_error_flag;
   }
   double *h = (double *) malloc(sizeof(double) * (size_t) (n > 0 ? n : 1));
   if (!h) { fclose(f); gb_error(HYPRE_ERROR_MEMORY, "ParVectorRead"); return gb_error_flag; }
   for (int i = 0; i < n; i++)
   {
      if (fscanf(f, "%le", &h[i]) != 1)
      {
         fclose(f); free(h);
         gb_error(HYPRE_ERROR_GENERIC, "ParVectorRead: short vector file");
         return gb_error_flag;
      }
   }
   fclose(f);
   HYPRE_ParVector v = NULL;
   HYPRE_ParVectorCreate(comm, n, NULL, &v);
   HYPRE_ParVectorInitialize(v);
   gb_parvec *pv = (gb_parvec *) v;
   if (pv && pv->d)
   {
      cudaMemcpyAsync(pv->d, h, sizeof(double) * (size_t) n, cudaMemcpyHostToDevice, gb_stream());
      gb_sync();
   }
   free(h);
   *vector = v;
   return gb_error_flag;
}

/* values at the given global indices (all values in order when indices is
 * NULL), copied to the host (HYPRE_parcsr_vector.c, one process) */
HYPRE_Int HYPRE_ParVectorGetValues(HYPRE_ParVector vector, HYPRE_Int num_values, HYPRE_BigInt *indices,
                                   HYPRE_Complex *values)
{
   gb_parvec *v = (gb_parvec *) vector;
   if (!v || v->magic != GB_MAGIC_VEC || !v->d) { gb_error_in_arg(1); return gb_error_flag; }
   if (num_values < 0) { gb_error_in_arg(2); return gb_error_flag; }
   if (num_values > 0 && !values) { gb_error_in_arg(4); return gb_error_flag; }
   if (!indices)
   {
      if (num_values > v->n) { gb_error_in_arg(2); return gb_error_flag; }
      cudaMemcpyAsync(values, v->d, sizeof(double) * (size_t) num_values, cudaMemcpyDeviceToHost, gb_stream());
      gb_sync();
      return gb_error_flag;
   }
   double *h = (double *) malloc(sizeof(double) * (size_t) (v->n > 0 ? v->n : 1));
   if (!h) { gb_error(HYPRE_ERROR_MEMORY, "ParVectorGetValues"); return gb_error_flag; }
   cudaMemcpyAsync(h, v->d, sizeof(double) * (size_t) v->n, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   for (int k = 0; k < num_values; k++)
   {
      if (indices[k] < 0 || indices[k] >= v->n) { gb_error_in_arg(3); continue; }
      values[k] = h[indices[k]];
   }
   free(h);
   return gb_error_flag;
}

/* ------------------------------------------------------------------------
 * ParCSR text files of one process (hypre_ParCSRMatrixPrint / Read,
 * src/parcsr_mv/par_csr_matrix.c:872-930, with hypre_CSRMatrixPrint
 * src/seq_mv/csr_matrix.c:540-610): <name>.D.0 holds the row count, the row
 * pointers, the column indices (both 1-based) and the values (%.14e), one
 * per line; <name>.INFO.0 the global sizes, the number of off-process columns
 * (0) and the row and column ranges.  No <name>.O.0 is written: one process
 * has no off-process block.  Read accepts square matrices.
 * ------------------------------------------------------------------------ */
HYPRE_Int HYPRE_ParCSRMatrixPrint(HYPRE_ParCSRMatrix matrix, const char *file_name)
{
   gb_parcsr *A = (gb_parcsr *) matrix;
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(1); return gb_error_flag; }
   if (!file_name) { gb_error_in_arg(2); return gb_error_flag; }
   const int n = A->A.nr, nnz = A->A.nnz;
   int *I = (int *) malloc(sizeof(int) * (size_t) (n + 1)), *J = (int *) malloc(sizeof(int) * (size_t) (nnz ? nnz : 1));
   double *V = (double *) malloc(sizeof(double) * (size_t) (nnz ? nnz : 1));
   if (!I || !J || !V) { free(I); free(J); free(V); gb_error(HYPRE_ERROR_MEMORY, "ParCSRMatrixPrint"); return gb_error_flag; }
   cudaMemcpyAsync(I, A->A.i, sizeof(int) * (size_t) (n + 1), cudaMemcpyDeviceToHost, gb_stream());
   cudaMemcpyAsync(J, A->A.j, sizeof(int) * (size_t) nnz, cudaMemcpyDeviceToHost, gb_stream());
   cudaMemcpyAsync(V, A->A.v, sizeof(double) * (size_t) nnz, cudaMemcpyDeviceToHost, gb_stream());
   gb_sync();
   char name[4096];
   snprintf(name, sizeof(name), "%s.D.0", file_name);
   FILE *f = fopen(name, "w");
   if (!f) { free(I); free(J); free(V); gb_error(HYPRE_ERROR_GENERIC, "ParCSRMatrixPrint: cannot open the file"); return gb_error_flag; }
   fprintf(f, "%d\n", n);
   for (int r = 0; r <= n; r++) { fprintf(f, "%d\n", I[r] + 1); }
   for (int k = 0; k < nnz; k++) { fprintf(f, "%d\n", J[k] + 1); }
   for (int k = 0; k < nnz; k++) { fprintf(f, "%.14e\n", V[k]); }
   fclose(f);
   free(I); free(J); free(V);
   snprintf(name, sizeof(name), "%s.INFO.0", file_name);
   f = fopen(name, "w");
   if (!f) { gb_error(HYPRE_ERROR_GENERIC, "ParCSRMatrixPrint: cannot open the file"); return gb_error_flag; }
   fprintf(f, "%d\n%d\n%d\n%d %d %d %d\n", n, A->A.nc, 0, 0, n, 0, A->A.nc);
   fclose(f);
   return gb_error_flag;
}

HYPRE_Int HYPRE_ParCSRMatrixRead(MPI_Comm comm, const char *file_name, HYPRE_ParCSRMatrix *matrix)
{
   (void) comm;
   if (!file_name) { gb_error_in_arg(2); return gb_error_flag; }
   if (!matrix) { gb_error_in_arg(3); return gb_error_flag; }
   *matrix = NULL;
   char name[4096];
   snprintf(name, sizeof(name), "%s.INFO.0", file_name);
   FILE *f = fopen(name, "r");
   int gr = 0, gc = 0, noffd = 0, rs = 0, re = 0, cs = 0, ce = 0;
   if (!f || fscanf(f, "%d %d %d %d %d %d %d", &gr, &gc, &noffd, &rs, &re, &cs, &ce) != 7)
   {
      if (f) { fclose(f); }
      gb_error(HYPRE_ERROR_GENERIC, "ParCSRMatrixRead: cannot read the INFO file");
      return gb_error_flag;
   }
   fclose(f);
   if (noffd != 0 || gr != gc || rs != 0 || re != gr || cs != 0 || ce != gc)
   {
      gb_error(HYPRE_ERROR_GENERIC, "ParCSRMatrixRead: one process, square matrices");
      return gb_error_flag;
   }
   snprintf(name, sizeof(name), "%s.D.0", file_name);
   f = fopen(name, "r");
   int n = -1;
   if (!f || fscanf(f, "%d", &n) != 1 || n != gr)
   {
      if (f) { fclose(f); }
      gb_error(HYPRE_ERROR_GENERIC, "ParCSRMatrixRead: cannot read the matrix file");
      return gb_error_flag;
   }
   int *I = (int *) malloc(sizeof(int) * (size_t) (n + 1));
   int ok = I != NULL;
   for (int r = 0; ok && r <= n; r++) { ok = fscanf(f, "%d", &I[r]) == 1; if (ok) { I[r] -= 1; } }
   const int nnz = ok ? I[n] : 0;
   ok = ok && I[0] == 0 && nnz >= 0;
   for (int r = 0; ok && r < n; r++) { ok = I[r + 1] >= I[r]; }
   int *J = ok ? (int *) malloc(sizeof(int) * (size_t) (nnz ? nnz : 1)) : NULL;
   double *V = ok ? (double *) malloc(sizeof(double) * (size_t) (nnz ? nnz : 1)) : NULL;
   ok = ok && J && V;
   for (int k = 0; ok && k < nnz; k++)
   {
      ok = fscanf(f, "%d", &J[k]) == 1;
      if (ok) { J[k] -= 1; ok = J[k] >= 0 && J[k] < n; }
   }
   for (int k = 0; ok && k < nnz; k++) { ok = fscanf(f, "%le", &V[k]) == 1; }
   fclose(f);
   if (!ok)
   {
      free(I); free(J); free(V);
      gb_error(HYPRE_ERROR_GENERIC, "ParCSRMatrixRead: malformed matrix file");
      return gb_error_flag;
   }
   HYPRE_GB300_ParCSRMatrixCreateFromHostCSR(n, I, J, V, matrix);
   free(I); free(J); free(V);
   return gb_error_flag;
}
