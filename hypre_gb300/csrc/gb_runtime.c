/* Runtime of libHYPRE_gb300: error flag, stream, stream-ordered device
 * memory, reusable scratch, launch counter.
 * Reference behaviour: error flag src/utilities/error.c:13-91,
 * HYPRE_Initialize/Finalize src/utilities/general.c:436,485. */
#include "gb_internal.h"

#include <time.h>

HYPRE_Int gb_error_flag = 0;
HYPRE_Int gb_error_arg = 0;

static cudaStream_t g_stream = 0;
static int g_own_stream = 0;
static int g_initialized = 0;
static long long g_launches = 0;
static int g_verbose_errors = -1;

#define GB_NSCRATCH 16
static void *g_scratch[GB_NSCRATCH];
static size_t g_scratch_sz[GB_NSCRATCH];
static double *g_red_part = NULL, *g_red_out = NULL, *g_red_host = NULL;
static unsigned int *g_red_count = NULL;
static int *g_red_ints = NULL;

void gb_count_launch(int n) { g_launches += n; }

void gb_error(HYPRE_Int code, const char *msg)
{
   gb_error_flag |= code;
   if (g_verbose_errors < 0)
   {
      const char *e = getenv("HYPRE_GB300_VERBOSE");
      g_verbose_errors = e && e[0] == '1';
   }
   if (g_verbose_errors && msg) { fprintf(stderr, "hypre_gb300 error %d: %s\n", (int) code, msg); }
}

void gb_error_in_arg(HYPRE_Int arg)
{
   gb_error_flag |= HYPRE_ERROR_ARG;
   gb_error_flag |= arg << 3;
   gb_error_arg = arg;
}

int gb_cuda_ok(cudaError_t e, const char *what)
{
   if (e == cudaSuccess) { return 1; }
   char buf[256];
   snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
   gb_error(HYPRE_ERROR_GENERIC, buf);
   return 0;
}

int gb_runtime_init(void)
{
   if (g_initialized) { return 0; }
   int ndev = 0;
   if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
   {
      gb_error(HYPRE_ERROR_GENERIC, "no CUDA device: libHYPRE_gb300 runs on the GPU only");
      return 1;
   }
   if (!g_stream)
   {
      if (!gb_cuda_ok(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking), "stream")) { return 1; }
      g_own_stream = 1;
   }
   /* keep freed blocks in the default pool so stream-ordered allocation is cheap */
   int dev = 0;
   cudaGetDevice(&dev);
   cudaMemPool_t pool;
   if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
   {
      unsigned long long thr = ~0ULL;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
   }
   g_initialized = 1;
   return 0;
}

cudaStream_t gb_stream(void)
{
   if (!g_initialized) { gb_runtime_init(); }
   return g_stream;
}

void *gb_dmalloc(size_t bytes)
{
   void *p = NULL;
   if (bytes == 0) { bytes = 16; }
   if (cudaMallocAsync(&p, bytes, gb_stream()) != cudaSuccess)
   {
      cudaGetLastError();
      gb_error(HYPRE_ERROR_MEMORY, "device allocation failed");
      return NULL;
   }
   return p;
}

void *gb_dcalloc(size_t bytes)
{
   void *p = gb_dmalloc(bytes);
   if (p) { cudaMemsetAsync(p, 0, bytes ? bytes : 16, gb_stream()); }
   return p;
}

void gb_dfree(void *p)
{
   if (p) { cudaFreeAsync(p, gb_stream()); }
}

void *gb_hmalloc_pinned(size_t bytes)
{
   void *p = NULL;
   if (cudaMallocHost(&p, bytes ? bytes : 16) != cudaSuccess) { cudaGetLastError(); return NULL; }
   return p;
}

void gb_hfree_pinned(void *p)
{
   if (p) { cudaFreeHost(p); }
}

/* host waits on the library stream: count and seconds (setup diagnostics) */
long long gb_sync_calls = 0;
double gb_sync_seconds = 0.0;

int gb_sync(void)
{
   const double t0 = gb_wtime();
   cudaError_t e = cudaStreamSynchronize(gb_stream());
   gb_sync_seconds += gb_wtime() - t0;
   gb_sync_calls++;
   if (e == cudaSuccess) { e = cudaGetLastError(); }
   return gb_cuda_ok(e, "kernel") ? 0 : 1;
}

double gb_wtime(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

void *gb_scratch(int slot, size_t bytes)
{
   if (bytes > g_scratch_sz[slot])
   {
      gb_dfree(g_scratch[slot]);
      size_t nb = bytes + bytes / 4 + 256;
      g_scratch[slot] = gb_dmalloc(nb);
      g_scratch_sz[slot] = g_scratch[slot] ? nb : 0;
   }
   return g_scratch[slot];
}

static void red_init(void)
{
   if (!g_red_part)
   {
      g_red_part = (double *) gb_dmalloc(sizeof(double) * GB_RED_BLOCKS * 4);
      g_red_out = (double *) gb_dmalloc(sizeof(double) * 8);
      g_red_host = (double *) gb_hmalloc_pinned(sizeof(double) * 8);
      g_red_count = (unsigned int *) gb_dcalloc(sizeof(unsigned int) * 4);
      g_red_ints = (int *) gb_hmalloc_pinned(sizeof(int) * 16);
   }
}
double *gb_red_part(void) { red_init(); return g_red_part; }
double *gb_red_out(void) { red_init(); return g_red_out; }
double *gb_red_host(void) { red_init(); return g_red_host; }
unsigned int *gb_red_count(void) { red_init(); return g_red_count; }
int *gb_red_ints(void) { red_init(); return g_red_ints; }

void gb_release_scratch(void)
{
   for (int k = 0; k < GB_NSCRATCH; k++) { gb_dfree(g_scratch[k]); g_scratch[k] = NULL; g_scratch_sz[k] = 0; }
}

double gb_dot(long long n, const double *x, const double *y)
{
   cudaStream_t s = gb_stream();
   gb_dot_d(n, x, y, gb_red_part(), gb_red_count(), gb_red_out(), s);
   cudaMemcpyAsync(gb_red_host(), gb_red_out(), sizeof(double), cudaMemcpyDeviceToHost, s);
   gb_sync();
   return gb_red_host()[0];
}

/* ---------------------------------------------------------------------------
 * Public runtime API
 * ------------------------------------------------------------------------- */
HYPRE_Int HYPRE_Initialize(void)
{
   gb_runtime_init();
   return gb_error_flag;
}

void gb_ij_release_host_cache(void);

HYPRE_Int HYPRE_Finalize(void)
{
   gb_ij_release_host_cache();
   if (g_initialized)
   {
      cudaStreamSynchronize(g_stream);
      gb_release_scratch();
      if (g_red_part)
      {
         gb_dfree(g_red_part); gb_dfree(g_red_out); gb_hfree_pinned(g_red_host); gb_dfree(g_red_count);
         gb_hfree_pinned(g_red_ints);
      }
      g_red_part = NULL; g_red_out = NULL; g_red_host = NULL; g_red_count = NULL; g_red_ints = NULL;
      cudaStreamSynchronize(g_stream);
      if (g_own_stream) { cudaStreamDestroy(g_stream); g_stream = 0; g_own_stream = 0; }
      g_initialized = 0;
   }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GetError(void) { return gb_error_flag; }

HYPRE_Int HYPRE_CheckError(HYPRE_Int ierr, HYPRE_Int code) { return ierr & code; }

HYPRE_Int HYPRE_GetErrorArg(void) { return gb_error_arg; }

void HYPRE_DescribeError(HYPRE_Int ierr, char *msg)
{
   if (!msg) { return; }
   msg[0] = 0;
   if (ierr == 0) { strcpy(msg, "[No error] "); return; }
   if (ierr & HYPRE_ERROR_GENERIC) { strcat(msg, "[Generic error] "); }
   if (ierr & HYPRE_ERROR_MEMORY) { strcat(msg, "[Memory error] "); }
   if (ierr & HYPRE_ERROR_ARG) { sprintf(msg + strlen(msg), "[Error in argument %d] ", (int) (ierr >> 3) & 31); }
   if (ierr & HYPRE_ERROR_CONV) { strcat(msg, "[Method did not converge] "); }
}

HYPRE_Int HYPRE_ClearAllErrors(void)
{
   gb_error_flag = 0;
   gb_error_arg = 0;
   return 0;
}

HYPRE_Int HYPRE_SetMemoryLocation(HYPRE_MemoryLocation m)
{
   if (m == HYPRE_MEMORY_HOST) { gb_error(HYPRE_ERROR_GENERIC, "host memory location unsupported: device only"); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GetMemoryLocation(HYPRE_MemoryLocation *m)
{
   if (m) { *m = HYPRE_MEMORY_DEVICE; }
   return gb_error_flag;
}

HYPRE_Int HYPRE_SetExecutionPolicy(HYPRE_ExecutionPolicy p)
{
   if (p == HYPRE_EXEC_HOST) { gb_error(HYPRE_ERROR_GENERIC, "host execution unsupported: device only"); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_SetSpMVUseVendor(HYPRE_Int u) { (void) u; return gb_error_flag; }
HYPRE_Int HYPRE_SetSpGemmUseVendor(HYPRE_Int u) { (void) u; return gb_error_flag; }
HYPRE_Int HYPRE_SetUseGpuRand(HYPRE_Int u) { (void) u; return gb_error_flag; }

HYPRE_Int HYPRE_GB300_SetStream(void *s)
{
   if (g_initialized && g_own_stream)
   {
      cudaStreamSynchronize(g_stream);
      cudaStreamDestroy(g_stream);
      g_own_stream = 0;
   }
   g_stream = (cudaStream_t) s;
   if (!g_initialized) { gb_runtime_init(); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_GetStream(void **s)
{
   if (s) { *s = (void *) gb_stream(); }
   return gb_error_flag;
}

HYPRE_Int HYPRE_GB300_GetKernelLaunchCount(long long *c)
{
   if (c) { *c = g_launches; }
   return 0;
}

HYPRE_Int HYPRE_GB300_ResetKernelLaunchCount(void)
{
   g_launches = 0;
   return 0;
}
