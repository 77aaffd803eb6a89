// Transpose mat-vec that allocates nothing: y = alpha * A^T x + beta * y with
// the transpose of A built in a fixed, file-scope device array instead of
// freshly allocated memory.
//
// Callers that cannot let the library allocate device memory use it: code
// that enqueues work while a stream is being captured into a CUDA graph, and
// hosts whose device memory belongs to another allocator (a framework that
// hands this library raw pointers and forbids it to grow its own pool).
// HYPRE_ParCSRMatrixMatvecT, by contrast, allocates the transpose from the
// library's stream-ordered pool on every call (growing the pool) and
// synchronises the stream before freeing it; this form only enqueues work on
// the library's stream.
//
// Limit: the transpose, its row pointers and the scan workspace must fit in
// GB_NOALLOC_SCRATCH_BYTES (32 MiB, for example about 2.6 million nonzeros
// of a matrix with up to 100,000 columns); larger matrices are rejected with
// HYPRE_ERROR_ARG.  The array is held by every GPU that loads the library
// until the process exits.
//
// The array is shared by all calls: each call overwrites it (the column
// counters are cleared at the start of every call), so calls that may
// overlap on the GPU -- on different streams, or from different host threads
// -- race on it and must be serialised by the caller.
//
// The first call on each device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.  Like every entry point of the library, it runs
// on the library's one stream: the current device must be that stream's
// device, else the call returns HYPRE_ERROR_GENERIC without enqueuing work.
#include "gb_internal.h"

#define GB_NOALLOC_SCRATCH_BYTES (32u << 20)
#define GB_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

static unsigned char *g_noalloc_ptr[GB_NOALLOC_MAX_DEVICES];

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

/* Device address of the scratch array on the current device (looked up once
 * per device).  In host code the symbol itself is only a stand-in, never a
 * device address. */
static unsigned char *noalloc_base(void)
{
   int dev = 0;
   if (!gb_cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) { return NULL; }
   if (dev < 0 || dev >= GB_NOALLOC_MAX_DEVICES)
   {
      gb_error(HYPRE_ERROR_GENERIC, "no-alloc scratch: device index out of range");
      return NULL;
   }
   if (!g_noalloc_ptr[dev])
   {
      void *p = NULL;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (!gb_cuda_ok(e, "cudaGetSymbolAddress(no-alloc scratch)")) { return NULL; }
      g_noalloc_ptr[dev] = (unsigned char *) p;
   }
   return g_noalloc_ptr[dev];
}

extern "C" HYPRE_Int HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(HYPRE_Complex alpha, HYPRE_ParCSRMatrix A,
                                                           HYPRE_ParVector x, HYPRE_Complex beta,
                                                           HYPRE_ParVector y)
{
   if (!A || A->magic != GB_MAGIC_MAT) { gb_error_in_arg(2); return gb_error_flag; }
   if (!x || x->magic != GB_MAGIC_VEC) { gb_error_in_arg(3); return gb_error_flag; }
   if (!y || y->magic != GB_MAGIC_VEC) { gb_error_in_arg(5); return gb_error_flag; }
   const gb_csr *M = &A->A;
   if (x->n != M->nr || x->num_vectors != 1) { gb_error_in_arg(3); return gb_error_flag; }
   if (y->n != M->nc || y->num_vectors != 1) { gb_error_in_arg(5); return gb_error_flag; }
   int nc = M->nc, nr = M->nr, nnz = M->nnz;

   /* layout of the transpose inside the fixed array */
   size_t o_cnt = 0;
   size_t o_ti = o_cnt + align256(sizeof(int) * ((size_t) nc + 1));
   size_t o_fill = o_ti + align256(sizeof(int) * ((size_t) nc + 1));
   size_t o_scan = o_fill + align256(sizeof(int) * ((size_t) nc + 1));
   size_t o_tj = o_scan + align256(sizeof(int) * (size_t) gb_scan_scratch_ints(nc > 0 ? nc : 1));
   size_t o_tv = o_tj + align256(sizeof(int) * (size_t) (nnz > 0 ? nnz : 1));
   size_t need = o_tv + align256(sizeof(double) * (size_t) (nnz > 0 ? nnz : 1));
   if (need > GB_NOALLOC_SCRATCH_BYTES)
   {
      char msg[200];
      snprintf(msg, sizeof(msg),
               "MatvecTNoAlloc: matrix needs %zu bytes of transpose scratch, the fixed array holds %u",
               need, (unsigned) GB_NOALLOC_SCRATCH_BYTES);
      gb_error(HYPRE_ERROR_ARG, msg);
      gb_error_in_arg(2);
      return gb_error_flag;
   }
   cudaStream_t s = gb_stream();
   int dev = 0, sdev = 0;
   if (!gb_cuda_ok(cudaGetDevice(&dev), "cudaGetDevice") ||
       !gb_cuda_ok(cudaStreamGetDevice(s, &sdev), "cudaStreamGetDevice")) { return gb_error_flag; }
   if (dev != sdev)
   {
      gb_error(HYPRE_ERROR_GENERIC, "MatvecTNoAlloc: the current device is not the library stream's device");
      return gb_error_flag;
   }
   unsigned char *base = noalloc_base();
   if (!base) { return gb_error_flag; }
   int *cnt = (int *) (base + o_cnt);
   int *Ti = (int *) (base + o_ti);
   int *fill = (int *) (base + o_fill);
   int *scan = (int *) (base + o_scan);
   int *Tj = (int *) (base + o_tj);
   double *Tv = (double *) (base + o_tv);

   /* counters start at zero on every call (the array keeps the last call's data) */
   cudaMemsetAsync(cnt, 0, sizeof(int) * ((size_t) nc + 1), s);
   gb_transpose_count(nnz, M->j, cnt, s);
   gb_exclusive_scan(cnt, Ti, nc, scan, s);
   cudaMemcpyAsync(fill, Ti, sizeof(int) * ((size_t) nc + 1), cudaMemcpyDeviceToDevice, s);
   gb_transpose_fill(nr, nc, M->i, M->j, M->v, fill, Ti, Tj, Tv, s);

   /* y = alpha * T x + beta * y with the CSR kernel (no solve-form cache, which would allocate) */
   gb_spmv_desc d;
   memset(&d, 0, sizeof(d));
   d.n = nc;
   d.fmt = GB_FMT_CSR;
   d.vprec = GB_PREC_F64;
   double avg = nc ? (double) nnz / nc : 0.0;
   d.K = avg >= 64 ? 32 : avg >= 32 ? 16 : avg >= 16 ? 8 : avg >= 8 ? 4 : 2;
   d.i = Ti;
   d.j = Tj;
   d.v = Tv;
   gb_spmv_d(&d, x->d, y->d, 0, alpha, beta, y->d, NULL, 0.0, NULL, NULL, s);
   gb_cuda_ok(cudaGetLastError(), "MatvecTNoAlloc");
   return gb_error_flag;
}
