/* Autotuner of the solve-phase SpMV launch shape.
 *
 * When a solve form (gb_solve_desc) is built for a matrix of at least
 * GB_TUNE_MIN_ROWS rows, every launch shape is timed on the library stream
 * and the fastest is kept in the form's descriptor:
 *   SELL-32 forms: prefetch depth D in {1, 2, 4, 8} x block size {128, 256, 512}
 *     (every choice sums each row in element order: results are identical);
 *   CSR forms: lanes per row K in {2, 4, 8, 16, 32} x block size {128, 256, 512}
 *     (K splits a row's sum into K partial sums: results differ in rounding).
 * Choices are cached per matrix shape (format, value and vector precision,
 * index width, rows, nonzeros) in memory and in a JSON file --
 * $HYPRE_GB300_TUNE_CACHE, else $HOME/.cache/hypre_gb300/spmv_tune.json -- so
 * a shape is timed once per machine.  HYPRE_GB300_AUTOTUNE=0 (or
 * HYPRE_GB300_SetAutotune(0)) keeps the default shapes (SELL: D 4, 256
 * threads; CSR: K from the mean row length, 256 threads).  Forms built while
 * the stream is being captured into a graph keep the defaults. */
#include "gb_internal.h"

#include <errno.h>
#include <sys/stat.h>
#include <unistd.h>

#define GB_TUNE_MIN_ROWS 20000
#define GB_TUNE_KEY 96

typedef struct
{
   char   key[GB_TUNE_KEY];
   int    T, D, K;
   double us;
} tune_entry;

static tune_entry *g_tab = NULL;
static int g_ntab = 0, g_cap = 0, g_loaded = 0, g_enabled = -1;

static int tune_enabled(void)
{
   if (g_enabled < 0)
   {
      const char *e = getenv("HYPRE_GB300_AUTOTUNE");
      g_enabled = !(e && e[0] == '0');
   }
   return g_enabled;
}

HYPRE_Int HYPRE_GB300_SetAutotune(HYPRE_Int on)
{
   g_enabled = on ? 1 : 0;
   return gb_error_flag;
}

static int cache_path(char *buf, size_t n)
{
   const char *e = getenv("HYPRE_GB300_TUNE_CACHE");
   if (e && e[0]) { snprintf(buf, n, "%s", e); return 1; }
   const char *h = getenv("HOME");
   if (!h || !h[0]) { return 0; }
   char dir[512];
   snprintf(dir, sizeof(dir), "%s/.cache", h);
   mkdir(dir, 0755);
   snprintf(dir, sizeof(dir), "%s/.cache/hypre_gb300", h);
   if (mkdir(dir, 0755) != 0 && errno != EEXIST) { return 0; }
   snprintf(buf, n, "%s/spmv_tune.json", dir);
   return 1;
}

static tune_entry *tab_find(const char *key)
{
   for (int k = 0; k < g_ntab; k++) { if (strcmp(g_tab[k].key, key) == 0) { return &g_tab[k]; } }
   return NULL;
}

static tune_entry *tab_add(const char *key)
{
   tune_entry *e = tab_find(key);
   if (e) { return e; }
   if (g_ntab == g_cap)
   {
      int nc = g_cap ? 2 * g_cap : 64;
      tune_entry *t = (tune_entry *) realloc(g_tab, sizeof(tune_entry) * (size_t) nc);
      if (!t) { return NULL; }
      g_tab = t;
      g_cap = nc;
   }
   e = &g_tab[g_ntab++];
   memset(e, 0, sizeof(*e));
   snprintf(e->key, GB_TUNE_KEY, "%s", key);
   return e;
}

/* the cache file: one entry per line, "key": [T, D, K, microseconds] */
static void cache_load(void)
{
   if (g_loaded) { return; }
   g_loaded = 1;
   char path[600];
   if (!cache_path(path, sizeof(path))) { return; }
   FILE *f = fopen(path, "r");
   if (!f) { return; }
   char line[512];
   while (fgets(line, sizeof(line), f))
   {
      char key[GB_TUNE_KEY];
      int T, D, K;
      double us;
      if (sscanf(line, " \"%95[^\"]\" : [ %d , %d , %d , %lf ]", key, &T, &D, &K, &us) == 5)
      {
         tune_entry *e = tab_add(key);
         if (e) { e->T = T; e->D = D; e->K = K; e->us = us; }
      }
   }
   fclose(f);
}

static void cache_save(void)
{
   char path[600], tmp[620];
   if (!cache_path(path, sizeof(path))) { return; }
   snprintf(tmp, sizeof(tmp), "%s.%d.tmp", path, (int) getpid());
   FILE *f = fopen(tmp, "w");
   if (!f) { return; }
   fprintf(f, "{\n");
   for (int k = 0; k < g_ntab; k++)
   {
      fprintf(f, "  \"%s\": [%d, %d, %d, %.3f]%s\n", g_tab[k].key, g_tab[k].T, g_tab[k].D, g_tab[k].K, g_tab[k].us,
              k + 1 < g_ntab ? "," : "");
   }
   fprintf(f, "}\n");
   fclose(f);
   rename(tmp, path);
}

static void shape_key(const gb_spmv_desc *d, long long nnz, char *key)
{
   const char *vp = d->vprec == GB_PREC_F64 ? (d->fmt == GB_FMT_SELL && d->sl_v32 ? "f64v32" : "f64")
                                            : d->vprec == GB_PREC_F32 ? "f32" : "f16";
   snprintf(key, GB_TUNE_KEY, "%s:%s:%s:%d:%lld", d->fmt == GB_FMT_SELL ? "sell" : "csr", vp,
            d->fmt == GB_FMT_SELL && d->sl_j16 ? "i16" : "i32", d->n, nnz);
}

static void apply(gb_spmv_desc *d, const tune_entry *e)
{
   d->tuneT = e->T;
   if (d->fmt == GB_FMT_SELL) { d->tuneD = e->D; }
   else if (e->K) { d->K = e->K; }
}

/* mean device microseconds of `reps` launches of y = A x */
static double time_shape(gb_spmv_desc *d, void *x, void *y, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1)
{
   const int reps = 5;
   for (int r = -2; r < reps; r++)
   {
      if (r == 0) { cudaEventRecord(e0, s); }
      if (d->vprec == GB_PREC_F64) { gb_spmv_d(d, (const double *) x, (double *) y, 0, 1.0, 0.0, NULL, NULL, 0.0, NULL, NULL, s); }
      else { gb_spmv_f(d, (const float *) x, (float *) y, 0, 1.f, 0.f, NULL, NULL, 0.f, NULL, NULL, s); }
   }
   cudaEventRecord(e1, s);
   cudaEventSynchronize(e1);
   float ms = 0.f;
   cudaEventElapsedTime(&ms, e0, e1);
   return 1e3 * ms / reps;
}

void gb_spmv_autotune(gb_spmv_desc *d, long long nnz)
{
   if (!tune_enabled() || d->n < GB_TUNE_MIN_ROWS) { return; }
   cudaStream_t s = gb_stream();
   enum cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
   if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) { cudaGetLastError(); return; }
   cache_load();
   char key[GB_TUNE_KEY];
   shape_key(d, nnz, key);
   tune_entry *hit = tab_find(key);
   if (hit) { apply(d, hit); return; }
   const size_t xb = d->vprec == GB_PREC_F64 ? 8 : 4;
   void *x = gb_dcalloc(xb * (size_t) d->n), *y = gb_dmalloc(xb * (size_t) d->n);
   if (!x || !y) { gb_dfree(x); gb_dfree(y); return; }
   cudaEvent_t e0, e1;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   static const int Ts[3] = {128, 256, 512}, Ds[4] = {1, 2, 4, 8}, Ks[5] = {2, 4, 8, 16, 32};
   tune_entry best;
   memset(&best, 0, sizeof(best));
   best.us = 1e30;
   const int K0 = d->K;
   for (int a = 0; a < 3; a++)
   {
      const int nb = d->fmt == GB_FMT_SELL ? 4 : 5;
      for (int c = 0; c < nb; c++)
      {
         tune_entry cand;
         memset(&cand, 0, sizeof(cand));
         cand.T = Ts[a];
         if (d->fmt == GB_FMT_SELL) { cand.D = Ds[c]; } else { cand.K = Ks[c]; }
         apply(d, &cand);
         cand.us = time_shape(d, x, y, s, e0, e1);
         if (cand.us < best.us) { best = cand; }
      }
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   gb_dfree(x);
   gb_dfree(y);
   if (cudaGetLastError() != cudaSuccess || best.us >= 1e30)
   {
      d->tuneT = 0; d->tuneD = 0; d->K = K0;
      return;
   }
   apply(d, &best);
   tune_entry *e = tab_add(key);
   if (e) { e->T = best.T; e->D = best.D; e->K = best.K; e->us = best.us; }
   cache_save();
}

void gb_spmm_d(int n, int nv, const int *Ai, const int *Aj, const double *Av, const double *x, double *y, int mode,
               double alpha, double beta, const double *b, const double *d, double w, int T, int U, cudaStream_t s);
void gb_spmm_f(int n, int nv, const int *Ai, const int *Aj, const float *Av, const float *x, float *y, int mode,
               float alpha, float beta, const float *b, const float *d, float w, int T, int U, cudaStream_t s);

/* The launch shape of one sparse operand of the multi-vector cycle (SpMM on
 * nv interleaved columns): block size {128, 256, 512} x neighbour rows in
 * flight per lane {1, 2, 4, 8}, every shape summing each column in element
 * order (identical results).  Timed with x and y as given (their contents
 * are overwritten: y = A x), kept per (precision, nv, rows, columns, nonzeros)
 * in the same cache as the SpMV shapes.  Defaults (256, 2) when tuning is off,
 * the operand is small or the stream is being captured;
 * $HYPRE_GB300_SPMM_SHAPE = "T,U" sets every operand's shape. */
void gb_spmm_autotune(int prec, int nrows, int ncols, long long nnz, int nv, const int *Ai, const int *Aj,
                      const void *Av, void *x, void *y, int *T, int *U)
{
   *T = 256;
   *U = 2;
   /* HYPRE_GB300_SPMM_SHAPE="T,U" sets the shape of every operand (tests) */
   const char *forced = getenv("HYPRE_GB300_SPMM_SHAPE");
   if (forced && forced[0])
   {
      int ft = 0, fu = 0;
      if (sscanf(forced, "%d,%d", &ft, &fu) == 2 && (ft == 128 || ft == 256 || ft == 512) &&
          (fu == 1 || fu == 2 || fu == 4 || fu == 8))
      {
         *T = ft;
         *U = fu;
      }
      return;
   }
   if (!tune_enabled() || nrows < GB_TUNE_MIN_ROWS) { return; }
   cudaStream_t s = gb_stream();
   enum cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
   if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) { cudaGetLastError(); return; }
   cache_load();
   char key[GB_TUNE_KEY];
   snprintf(key, GB_TUNE_KEY, "spmm:%s:nv%d:%d:%d:%lld", prec == GB_PREC_F64 ? "f64" : "f32", nv, nrows, ncols, nnz);
   tune_entry *hit = tab_find(key);
   if (hit) { *T = hit->T; *U = hit->D; return; }
   cudaEvent_t e0, e1;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   static const int Ts[3] = {128, 256, 512}, Us[4] = {1, 2, 4, 8};
   tune_entry best;
   memset(&best, 0, sizeof(best));
   best.us = 1e30;
   for (int a = 0; a < 3; a++)
   {
      for (int c = 0; c < 4; c++)
      {
         const int reps = 5;
         for (int r = -2; r < reps; r++)
         {
            if (r == 0) { cudaEventRecord(e0, s); }
            if (prec == GB_PREC_F64)
            {
               gb_spmm_d(nrows, nv, Ai, Aj, (const double *) Av, (const double *) x, (double *) y, 0, 1.0, 0.0, NULL,
                         NULL, 0.0, Ts[a], Us[c], s);
            }
            else
            {
               gb_spmm_f(nrows, nv, Ai, Aj, (const float *) Av, (const float *) x, (float *) y, 0, 1.f, 0.f, NULL,
                         NULL, 0.f, Ts[a], Us[c], s);
            }
         }
         cudaEventRecord(e1, s);
         cudaEventSynchronize(e1);
         float ms = 0.f;
         cudaEventElapsedTime(&ms, e0, e1);
         const double us = 1e3 * ms / reps;
         if (us < best.us) { best.us = us; best.T = Ts[a]; best.D = Us[c]; }
      }
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   if (cudaGetLastError() != cudaSuccess || best.us >= 1e30) { return; }
   *T = best.T;
   *U = best.D;
   tune_entry *e = tab_add(key);
   if (e) { e->T = best.T; e->D = best.D; e->K = 0; e->us = best.us; }
   cache_save();
}

/* the shape a form was given (tests and diagnostics) */
HYPRE_Int HYPRE_GB300_ParCSRMatrixGetSpMVShape(HYPRE_ParCSRMatrix A, HYPRE_Int precision, HYPRE_Int *format,
                                               HYPRE_Int *block, HYPRE_Int *depth_or_lanes)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(1); return gb_error_flag; }
   if (precision < GB_PREC_F64 || precision > GB_PREC_F16) { gb_error_in_arg(2); return gb_error_flag; }
   const gb_spmv_desc *d = gb_solve_desc(A, precision);
   if (!d) { return gb_error_flag; }
   if (format) { *format = d->fmt; }
   if (block) { *block = d->tuneT ? d->tuneT : 256; }
   if (depth_or_lanes) { *depth_or_lanes = d->fmt == GB_FMT_SELL ? (d->tuneD ? d->tuneD : 4) : d->K; }
   return gb_error_flag;
}

/* sets the shape of a form by hand: block size 0 = 256; SELL prefetch depth
 * 0 = 4; CSR lanes per row 0 = unchanged.  The autotuner's test compares
 * every shape's result with the default's. */
HYPRE_Int HYPRE_GB300_ParCSRMatrixSetSpMVShape(HYPRE_ParCSRMatrix A, HYPRE_Int precision, HYPRE_Int block,
                                               HYPRE_Int depth_or_lanes)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(1); return gb_error_flag; }
   if (precision < GB_PREC_F64 || precision > GB_PREC_F16) { gb_error_in_arg(2); return gb_error_flag; }
   if (block != 0 && block != 128 && block != 256 && block != 512) { gb_error_in_arg(3); return gb_error_flag; }
   gb_spmv_desc *d = (gb_spmv_desc *) gb_solve_desc(A, precision);
   if (!d) { return gb_error_flag; }
   if (d->fmt == GB_FMT_SELL)
   {
      if (depth_or_lanes != 0 && depth_or_lanes != 1 && depth_or_lanes != 2 && depth_or_lanes != 4 &&
          depth_or_lanes != 8) { gb_error_in_arg(4); return gb_error_flag; }
      d->tuneD = depth_or_lanes;
   }
   else
   {
      if (depth_or_lanes != 0 && depth_or_lanes != 2 && depth_or_lanes != 4 && depth_or_lanes != 8 &&
          depth_or_lanes != 16 && depth_or_lanes != 32) { gb_error_in_arg(4); return gb_error_flag; }
      if (depth_or_lanes) { d->K = depth_or_lanes; }
   }
   d->tuneT = block;
   return gb_error_flag;
}
