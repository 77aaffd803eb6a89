// Solve-phase kernels for sm_103a: SpMV in two layouts (CSR with K lanes per
// row, and SELL-32 with one thread per row for near-uniform rows), fused
// smoother sweeps, Krylov vector operations with deterministic two-stage
// reductions, precision conversions and the dense coarsest-grid apply.
//
// All kernels are HBM-bandwidth bound.  Value and vector types are template
// parameters: FP64 values/vectors (reference arithmetic), FP32 values/vectors
// (mixed-precision cycle) and FP16 values with FP32 vectors and accumulation.
#include "gb_device.cuh"
#include "gb_kernels.h"

#include <cuda_fp16.h>

static int nblk(long long n, int t) { long long b = (n + t - 1) / t; return (int) (b < 1 ? 1 : b); }

template <typename T> __device__ __forceinline__ float tof(T v);
template <> __device__ __forceinline__ float tof<float>(float v) { return v; }
template <> __device__ __forceinline__ float tof<__half>(__half v) { return __half2float(v); }

template <typename VT, typename XT> struct Acc;
template <> struct Acc<double, double>
{
   typedef double T;
   static __device__ __forceinline__ double mul(double a, double x) { return a * x; }
};
template <> struct Acc<float, float>
{
   typedef float T;
   static __device__ __forceinline__ float mul(float a, float x) { return a * x; }
};
template <> struct Acc<__half, float>
{
   typedef float T;
   static __device__ __forceinline__ float mul(__half a, float x) { return __half2float(a) * x; }
};
// FP64 values held as FP32 because every one of them is a normal FP32 number
// or zero (checked when the form is built): widened exactly with integer
// operations (exponent rebiased by 1023 - 127, mantissa shifted by 29 bits),
// so the products and sums are those of the FP64 values, bit for bit
__device__ __forceinline__ double gb_widen_exact(float a)
{
   const unsigned u = __float_as_uint(a);
   const unsigned long long sign = (unsigned long long) (u & 0x80000000u) << 32;
   const unsigned em = u & 0x7fffffffu;
   if (em == 0) { return __longlong_as_double((long long) sign); }
   return __longlong_as_double((long long) (sign | (((unsigned long long) em << 29) + (896ULL << 52))));
}
// FP64 -> FP32, rounded to nearest even, with integer operations when the
// result is a normal FP32 number (biased FP64 exponent 897..1150): the FP64
// pipe is scarce on this GPU and a conversion instruction would use it.  The
// 29 dropped mantissa bits decide the rounding (above half: up; exactly half:
// to the even neighbour); a carry out of the mantissa moves to the exponent
// (to infinity past the largest FP32).  Other values take the conversion.
__device__ __forceinline__ float gb_narrow_rn(double x)
{
   const unsigned long long b = (unsigned long long) __double_as_longlong(x);
   const unsigned long long mag = b & 0x7fffffffffffffffULL;
   const unsigned e = (unsigned) (mag >> 52);
   if (e < 897u || e > 1150u) { return (float) x; }
   const unsigned long long m = mag & 0xfffffffffffffULL;
   unsigned f = ((e - 896u) << 23) | (unsigned) (m >> 29);
   const unsigned rem = (unsigned) (m & 0x1fffffffULL);
   f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
   return __uint_as_float(f | ((unsigned) (b >> 63) << 31));
}

template <typename VT> __device__ __forceinline__ VT gb_to_vt(double x) { return (VT) x; }
template <> __device__ __forceinline__ float gb_to_vt<float>(double x) { return gb_narrow_rn(x); }

template <> struct Acc<float, double>
{
   typedef double T;
   static __device__ __forceinline__ double mul(float a, double x) { return gb_widen_exact(a) * x; }
};

static int num_sms();

// flag = 1 when some value is not zero or a normal FP32 number exactly.
// Integer tests on the bits (FP64 conversions and compares would hold the
// scarce FP64 pipe: 0.81 ms for the 109M values of a 160^3 27-point matrix):
// the biased exponent within FP32's normal range (897..1150) and the 29
// mantissa bits below FP32's precision zero.  Grid-stride, at most one write
// per block.
__global__ void __launch_bounds__(256) k_exact32(long long nnz, const double *__restrict__ v, int *flag)
{
   bool bad = false;
   for (long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < nnz && !bad;
        k += (long long) gridDim.x * blockDim.x)
   {
      const unsigned long long mag = (unsigned long long) __double_as_longlong(v[k]) & 0x7fffffffffffffffULL;
      const unsigned e = (unsigned) (mag >> 52);
      bad = mag != 0 && ((mag & 0x1fffffffULL) != 0 || e < 897u || e > 1150u);
   }
   if (__syncthreads_or(bad) && threadIdx.x == 0) { *flag = 1; }
}

extern "C" void gb_exact32(long long nnz, const double *v, int *flag, cudaStream_t s)
{
   cudaMemsetAsync(flag, 0, sizeof(int), s);
   if (nnz > 0)
   {
      const long long want = (nnz + 255) / 256;
      const int blocks = (int) (want < (long long) num_sms() * 8 ? want : (long long) num_sms() * 8);
      k_exact32<<<blocks, 256, 0, s>>>(nnz, v, flag);
      GB_COUNT(1);
   }
}

// Epilogue of a row: mode 0  y = alpha*s + beta*b
//                    mode 1  y = x_i + w*(b_i - s)/d_i   (l1 / diagonal Jacobi)
//                    mode 2  y = (b_i - s) for residuals   (alpha=-1, beta=1 shortcut)
//                    mode 6  y = s/d_i, and b_i += alpha*y (two-stage Gauss-Seidel)
template <typename XT>
__device__ __forceinline__ XT row_epilogue(int mode, XT s, int i, XT alpha, XT beta, const XT *b, const XT *x,
                                           const XT *d, XT w, const XT *y)
{
   if (mode == 1) { return x[i] + w * (b[i] - s) / d[i]; }
   if (mode == 2) { return b[i] - s; }
   // Chebyshev steps (d = D^{-1/2}, b = scaled residual r, alpha = coefficient)
   if (mode == 3) { return d[i] * (b[i] - s); }
   if (mode == 4) { return d[i] * (alpha * b[i] + d[i] * s); }
   if (mode == 5) { return y[i] + d[i] * (alpha * b[i] + d[i] * s); }
   // two-stage Gauss-Seidel inner sweep over the strictly lower part: the
   // kernel also adds alpha * y_i to b_i
   if (mode == 6) { return d ? s / d[i] : s; }
   XT r = alpha * s;
   if (beta != (XT) 0) { r += beta * b[i]; }
   return r;
}

// Block-level sum of v (fixed reduction tree: deterministic), lane 0 of warp 0
// holds the result.
template <typename T>
__device__ __forceinline__ T block_sum(T v)
{
   __shared__ T red[32];
   for (int o = 16; o > 0; o >>= 1) { v += __shfl_down_sync(GB_FULL, v, o); }
   int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   __syncthreads();
   if (lane == 0) { red[wid] = v; }
   __syncthreads();
   T t = 0;
   if (wid == 0)
   {
      int nw = (blockDim.x + 31) >> 5;
      t = lane < nw ? red[lane] : (T) 0;
      for (int o = 16; o > 0; o >>= 1) { t += __shfl_down_sync(GB_FULL, t, o); }
   }
   return t;
}

// ---------------------------------------------------------------------------
// CSR SpMV, K lanes per row (K in 2..32), rows distributed over the grid.
// dotz (optional): per-block partial sums of y_i * z_i written to dpart.
// ---------------------------------------------------------------------------
template <int K, typename VT, typename XT>
__global__ void __launch_bounds__(512) k_spmv_csr(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                                                  const VT *__restrict__ Av, const XT *__restrict__ x, XT *y,
                                                  int mode, XT alpha, XT beta, const XT *b, const XT *d, XT w,
                                                  const XT *__restrict__ dotz, double *dpart,
                                                  const float *__restrict__ rs)
{
   typedef typename Acc<VT, XT>::T AT;
   const int gpw = 32 / K;                       // row groups per warp
   const int wl = threadIdx.x & 31;
   const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int nwarps = (gridDim.x * blockDim.x) >> 5;
   const int lane = wl % K;
   double dsum = 0.0;
   for (int base = warp * gpw; base < n; base += nwarps * gpw)
   {
      int i = base + wl / K;
      bool valid = i < n;
      AT s = 0;
      if (valid)
      {
         int b0 = __ldg(Ai + i), e0 = __ldg(Ai + i + 1);
         for (int k = b0 + lane; k < e0; k += K) { s += Acc<VT, XT>::mul(__ldg(Av + k), __ldg(x + __ldg(Aj + k))); }
      }
      for (int o = K / 2; o > 0; o >>= 1) { s += __shfl_down_sync(GB_FULL, s, o, K); }
      if (valid && lane == 0)
      {
         XT si = (XT) s;
         if (rs) { si *= (XT) rs[i]; }
         XT yi = row_epilogue<XT>(mode, si, i, alpha, beta, b, x, d, w, y);
         y[i] = yi;
         if (dotz) { dsum += (double) yi * (double) dotz[i]; }
      }
   }
   if (dpart)
   {
      double t = block_sum<double>(dsum);
      if (threadIdx.x == 0) { dpart[blockIdx.x] = t; }
   }
}

// ---------------------------------------------------------------------------
// SELL-32 SpMV: slice s holds rows 32s..32s+31, element k of row 32s+t at
// sl_ptr[s] + 32k + t, so a warp's loads are fully coalesced (256 B values,
// 128 B indices per instruction for FP64).  Padding: a valid column (the
// row itself, or the last row for rows past n), value 0.
// ---------------------------------------------------------------------------
// column of the element stored as IT at Sj[p] for row i: the index itself, or
// (IT = short) the offset from the row
template <typename IT>
__device__ __forceinline__ int sell_col(const IT *__restrict__ Sj, long long p, int i)
{
   if constexpr (sizeof(IT) == 2) { return i + (int) __ldg(Sj + p); }
   else { return __ldg(Sj + p); }
}

// GS: the two-stage Gauss-Seidel epilogue (mode 6), which also updates b.
// D: prefetch depth -- the values, column indices and x entries of D
// consecutive elements are loaded before their products are summed, so each
// warp keeps D times 32 loads of each stream in flight.  The row's terms are
// summed in element order into one accumulator whatever D is, so every depth
// (and block size) gives the same result bit for bit; the autotuner picks D
// and the block size per matrix shape.
template <typename VT, typename XT, bool GS, typename IT, int D>
__global__ void __launch_bounds__(512) k_spmv_sell(int n, int nslices, const long long *__restrict__ sl_ptr,
                                                   const int *__restrict__ sl_w, const IT *__restrict__ Sj,
                                                   const VT *__restrict__ Sv, const XT *__restrict__ x, XT *y,
                                                   int mode, XT alpha, XT beta, const XT *b, const XT *d, XT w,
                                                   const XT *__restrict__ dotz, double *dpart,
                                                   const float *__restrict__ rs)
{
   typedef typename Acc<VT, XT>::T AT;
   const int t = threadIdx.x & 31;
   const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int nwarps = (gridDim.x * blockDim.x) >> 5;
   double dsum = 0.0;
   for (int s = warp; s < nslices; s += nwarps)
   {
      const long long base = __ldg(sl_ptr + s) + t;
      const int width = __ldg(sl_w + s);
      const int i = s * 32 + t;
      AT acc = 0;
      for (int k0 = 0; k0 < width; k0 += D)
      {
         VT a[D];
         int j[D];
#pragma unroll
         for (int u = 0; u < D; u++)
         {
            if (k0 + u < width)
            {
               const long long p = base + (long long) (k0 + u) * 32;
               j[u] = sell_col(Sj, p, i);
               a[u] = __ldg(Sv + p);
            }
         }
         XT xv[D];
#pragma unroll
         for (int u = 0; u < D; u++)
         {
            if (k0 + u < width) { xv[u] = __ldg(x + j[u]); }
         }
#pragma unroll
         for (int u = 0; u < D; u++)
         {
            if (k0 + u < width) { acc += Acc<VT, XT>::mul(a[u], xv[u]); }
         }
      }
      if (i < n)
      {
         XT si = (XT) acc;
         if (rs) { si *= (XT) rs[i]; }
         XT yi = row_epilogue<XT>(mode, si, i, alpha, beta, b, x, d, w, y);
         y[i] = yi;
         if (GS) { const_cast<XT *>(b)[i] += alpha * yi; }
         if (dotz) { dsum += (double) yi * (double) dotz[i]; }
      }
   }
   if (dpart)
   {
      double tt = block_sum<double>(dsum);
      if (threadIdx.x == 0) { dpart[blockIdx.x] = tt; }
   }
}

// SELL-32 construction: slice widths (the longest row of each slice of 32
// rows; lower: only the entries j < i), offsets, then column indices and
// values (values converted to VT, optionally divided by the row's first
// entry for the row-scaled FP16 forms).  One warp per slice, one lane per row.
// *wide = 1 when a kept entry is 2^15 or more columns from its row
__global__ void k_sell_width(int n, int nslices, const int *__restrict__ Ai, const int *__restrict__ Aj, int lower,
                             int *__restrict__ w, int *wide)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const int s = i >> 5;
   if (s >= nslices) { return; }
   int l = 0;
   bool far = false;
   if (i < n)
   {
      const int b = Ai[i], e = Ai[i + 1];
      for (int k = b; k < e; k++)
      {
         const int j = Aj[k];
         if (!lower || j < i)
         {
            l++;
            far |= j - i > 32767 || i - j > 32768;
         }
      }
   }
   for (int o = 16; o > 0; o >>= 1) { l = max(l, __shfl_xor_sync(GB_FULL, l, o)); }
   if ((i & 31) == 0) { w[s] = l; }
   if (__any_sync(GB_FULL, far) && (i & 31) == 0) { *wide = 1; }
}

// slice offsets: block-level scans of width*32 (int64), then block offsets
__global__ void k_sell_ptr_blocks(int nslices, const int *__restrict__ w, long long *__restrict__ ptr,
                                  long long *__restrict__ bsum)
{
   __shared__ long long ws[32];
   int s = blockIdx.x * blockDim.x + threadIdx.x;
   long long v = s < nslices ? (long long) w[s] * 32 : 0;
   int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   long long x = v;
   for (int o = 1; o < 32; o <<= 1) { long long y = __shfl_up_sync(GB_FULL, x, o); if (lane >= o) { x += y; } }
   if (lane == 31) { ws[wid] = x; }
   __syncthreads();
   if (wid == 0)
   {
      long long t = lane < (int) (blockDim.x >> 5) ? ws[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) { long long y = __shfl_up_sync(GB_FULL, t, o); if (lane >= o) { t += y; } }
      ws[lane] = t;
   }
   __syncthreads();
   long long excl = x - v + (wid > 0 ? ws[wid - 1] : 0);
   if (s < nslices) { ptr[s] = excl; }
   if (threadIdx.x == blockDim.x - 1) { bsum[blockIdx.x] = excl + v; }
}

// block b adds the sum of the earlier blocks' totals to its 1024 slice
// offsets; the last block also writes the total
__global__ void k_sell_ptr_fix(int nslices, long long *__restrict__ ptr, const long long *__restrict__ bsum,
                               int nblocks)
{
   __shared__ long long red[32];
   long long a = 0;
   for (int k = threadIdx.x; k < (int) blockIdx.x; k += blockDim.x) { a += bsum[k]; }
   for (int o = 16; o > 0; o >>= 1) { a += __shfl_down_sync(GB_FULL, a, o); }
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   if (lane == 0) { red[wid] = a; }
   __syncthreads();
   if (wid == 0)
   {
      a = lane < (int) (blockDim.x >> 5) ? red[lane] : 0;
      for (int o = 16; o > 0; o >>= 1) { a += __shfl_down_sync(GB_FULL, a, o); }
      if (lane == 0) { red[0] = a; }
   }
   __syncthreads();
   const long long off = red[0];
   const int s = blockIdx.x * 1024 + threadIdx.x;
   if (s < nslices) { ptr[s] += off; }
   if (blockIdx.x == nblocks - 1 && threadIdx.x == 0) { ptr[nslices] = off + bsum[blockIdx.x]; }
}

// IT = short: offsets j - i (checked to fit by k_sell_width)
template <typename IT>
__global__ void k_sell_fill_j(int n, int nslices, const int *__restrict__ Ai, const int *__restrict__ Aj,
                              const long long *__restrict__ ptr, const int *__restrict__ w, int lower,
                              IT *__restrict__ Sj)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const int s = i >> 5;
   if (s >= nslices) { return; }
   const int width = w[s];
   const long long base = ptr[s] + (i & 31);
   const int rel = sizeof(IT) == 2 ? i : 0;
   int k = 0;
   if (i < n)
   {
      for (int q = Ai[i]; q < Ai[i + 1]; q++)
      {
         const int j = Aj[q];
         if (!lower || j < i) { Sj[base + (long long) k * 32] = (IT) (j - rel); k++; }
      }
   }
   // padding: the row's own index (rows past n: the last row, at most 31
   // rows back) with value 0
   const int pad = i < n ? i : (n > 0 ? n - 1 : 0);
   for (; k < width; k++) { Sj[base + (long long) k * 32] = (IT) (pad - rel); }
}

template <typename VT>
__global__ void k_sell_fill_v(int n, int nslices, const int *__restrict__ Ai, const int *__restrict__ Aj,
                              const double *__restrict__ Av, const long long *__restrict__ ptr,
                              const int *__restrict__ w, int lower, int scaled, VT *__restrict__ Sv)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const int s = i >> 5;
   if (s >= nslices) { return; }
   const int width = w[s];
   const long long base = ptr[s] + (i & 31);
   int k = 0;
   if (i < n)
   {
      const int b = Ai[i], e = Ai[i + 1];
      double d = 1.0;
      if (scaled)
      {
         d = e > b ? Av[b] : 1.0;
         if (d == 0.0) { d = 1.0; }
      }
      for (int q = b; q < e; q++)
      {
         if (!lower || Aj[q] < i)
         {
            Sv[base + (long long) k * 32] = gb_to_vt<VT>(scaled ? Av[q] / d : Av[q]);
            k++;
         }
      }
   }
   for (; k < width; k++) { Sv[base + (long long) k * 32] = (VT) 0.0; }
}

template <typename VT>
__global__ void k_convert_vals(long long nnz, const double *__restrict__ in, VT *__restrict__ out)
{
   long long k = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (k < nnz) { out[k] = gb_to_vt<VT>(in[k]); }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
static int g_num_sms = 0;
static int num_sms()
{
   if (!g_num_sms)
   {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
      if (g_num_sms <= 0) { g_num_sms = 148; }
   }
   return g_num_sms;
}

extern "C" int gb_num_sms(void) { return num_sms(); }

extern "C" int gb_reduce_blocks(void) { return GB_RED_BLOCKS; }

template <typename VT, typename XT>
static void spmv_dispatch(const gb_spmv_desc *A, const XT *x, XT *y, int mode, XT alpha, XT beta, const XT *b,
                          const XT *d, XT w, const XT *dotz, double *dpart, cudaStream_t st)
{
   // block size and SELL prefetch depth: the autotuned choice, else 256 / 4;
   // the fused dot products (dpart) need the fixed reduction grid and 256
   const int T = (A->tuneT && !dpart) ? A->tuneT : 256;
   if (A->fmt == GB_FMT_SELL)
   {
      int nsl = A->nslices;
      int blocks = dpart ? GB_RED_BLOCKS : nblk((long long) nsl * 32, T);
      const int D = A->tuneD ? A->tuneD : 4;
#define GB_SELL_D(GS, IT, J, DD)                                                                                  \
   k_spmv_sell<VT, XT, GS, IT, DD><<<blocks, T, 0, st>>>(A->n, nsl, A->sl_ptr, A->sl_w, J, (const VT *) A->sl_v, x, \
                                                         y, mode, alpha, beta, b, d, w, dotz, dpart, A->rs)
#define GB_SELL(GS, IT, J)                                                                                         \
   switch (D)                                                                                                      \
   {                                                                                                               \
      case 1: GB_SELL_D(GS, IT, J, 1); break;                                                                      \
      case 2: GB_SELL_D(GS, IT, J, 2); break;                                                                      \
      case 8: GB_SELL_D(GS, IT, J, 8); break;                                                                      \
      default: GB_SELL_D(GS, IT, J, 4); break;                                                                     \
   }
      if (mode == GB_EPI_GS)
      {
         if (A->sl_j16) { GB_SELL(true, short, A->sl_j16); }
         else { GB_SELL(true, int, A->sl_j); }
      }
      else
      {
         if (A->sl_j16) { GB_SELL(false, short, A->sl_j16); }
         else { GB_SELL(false, int, A->sl_j); }
      }
#undef GB_SELL
#undef GB_SELL_D
   }
   else
   {
      int K = A->K;
      long long threads = (long long) A->n * K;
      int blocks = dpart ? GB_RED_BLOCKS : nblk(threads, T);
      const VT *vals = (const VT *) A->v;
#define LAUNCH_K(KK) k_spmv_csr<KK, VT, XT><<<blocks, T, 0, st>>>(A->n, A->i, A->j, vals, x, y, mode, alpha, beta, b, d, w, dotz, dpart, A->rs)
      switch (K)
      {
         case 2: LAUNCH_K(2); break;
         case 4: LAUNCH_K(4); break;
         case 8: LAUNCH_K(8); break;
         case 16: LAUNCH_K(16); break;
         default: LAUNCH_K(32); break;
      }
#undef LAUNCH_K
   }
   GB_COUNT(1);
}

extern "C" void gb_spmv_d(const gb_spmv_desc *A, const double *x, double *y, int mode, double alpha, double beta,
                          const double *b, const double *d, double w, const double *dotz, double *dpart,
                          cudaStream_t st)
{
   if (A->fmt == GB_FMT_SELL && A->sl_v32)
   {
      spmv_dispatch<float, double>(A, x, y, mode, alpha, beta, b, d, w, dotz, dpart, st);
   }
   else { spmv_dispatch<double, double>(A, x, y, mode, alpha, beta, b, d, w, dotz, dpart, st); }
}

extern "C" void gb_spmv_f(const gb_spmv_desc *A, const float *x, float *y, int mode, float alpha, float beta,
                          const float *b, const float *d, float w, const float *dotz, double *dpart, cudaStream_t st)
{
   if (A->vprec == GB_PREC_F16)
   {
      spmv_dispatch<__half, float>(A, x, y, mode, alpha, beta, b, d, w, dotz, dpart, st);
   }
   else
   {
      spmv_dispatch<float, float>(A, x, y, mode, alpha, beta, b, d, w, dotz, dpart, st);
   }
}

extern "C" void gb_sell_struct(int n, const int *Ai, const int *Aj, int lower, int nslices, int *sl_w,
                               long long *sl_ptr, int *sl_j, short *sl_j16, int *wide, cudaStream_t s, int stage)
{
   // stage 0: widths + offsets (caller then reads sl_ptr[nslices] to size
   // the arrays) and the wide flag; stage 1: column indices or offsets
   const long long nt = (long long) nslices * 32;
   if (stage == 0)
   {
      cudaMemsetAsync(wide, 0, sizeof(int), s);
      k_sell_width<<<nblk(nt, 256), 256, 0, s>>>(n, nslices, Ai, Aj, lower, sl_w, wide);
      int nb = nblk(nslices, 1024);
      long long *bsum = NULL;
      cudaMallocAsync((void **) &bsum, sizeof(long long) * (size_t) nb, s);
      k_sell_ptr_blocks<<<nb, 1024, 0, s>>>(nslices, sl_w, sl_ptr, bsum);
      k_sell_ptr_fix<<<nb, 1024, 0, s>>>(nslices, sl_ptr, bsum, nb);
      cudaFreeAsync(bsum, s);
      GB_COUNT(3);
      return;
   }
   if (sl_j16) { k_sell_fill_j<short><<<nblk(nt, 256), 256, 0, s>>>(n, nslices, Ai, Aj, sl_ptr, sl_w, lower, sl_j16); }
   else { k_sell_fill_j<int><<<nblk(nt, 256), 256, 0, s>>>(n, nslices, Ai, Aj, sl_ptr, sl_w, lower, sl_j); }
   GB_COUNT(1);
}

extern "C" void gb_sell_vals(int n, const int *Ai, const int *Aj, const double *Av, int lower, int scaled, int vprec,
                             int nslices, const int *sl_w, const long long *sl_ptr, void *sl_v, cudaStream_t s)
{
   const long long nt = (long long) nslices * 32;
   if (vprec == GB_PREC_F64)
   {
      k_sell_fill_v<double><<<nblk(nt, 256), 256, 0, s>>>(n, nslices, Ai, Aj, Av, sl_ptr, sl_w, lower, scaled,
                                                          (double *) sl_v);
   }
   else if (vprec == GB_PREC_F32)
   {
      k_sell_fill_v<float><<<nblk(nt, 256), 256, 0, s>>>(n, nslices, Ai, Aj, Av, sl_ptr, sl_w, lower, scaled,
                                                         (float *) sl_v);
   }
   else
   {
      k_sell_fill_v<__half><<<nblk(nt, 256), 256, 0, s>>>(n, nslices, Ai, Aj, Av, sl_ptr, sl_w, lower, scaled,
                                                          (__half *) sl_v);
   }
   GB_COUNT(1);
}

// FP16 CSR values a_ij / a_ii row by row (the diagonal is each row's first
// entry; 1 for an empty row or a zero diagonal) and rs[i] = a_ii: the FP16
// forms store these so their range stays near 1
__global__ void k_row_scaled_half(int n, const int *__restrict__ Ai, const double *__restrict__ Av,
                                  __half *__restrict__ out, float *__restrict__ rs)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int b = Ai[i], e = Ai[i + 1];
   double d = e > b ? Av[b] : 1.0;
   if (d == 0.0) { d = 1.0; }
   rs[i] = (float) d;
   for (int k = b; k < e; k++) { out[k] = (__half) (Av[k] / d); }
}

extern "C" void gb_row_scaled_half(int n, const int *Ai, const double *Av, void *out, float *rs, cudaStream_t s)
{
   if (n > 0) { k_row_scaled_half<<<nblk(n, 256), 256, 0, s>>>(n, Ai, Av, (__half *) out, rs); GB_COUNT(1); }
}

extern "C" void gb_convert_vals(long long nnz, const double *in, void *out, int vprec, cudaStream_t s)
{
   if (nnz <= 0) { return; }
   if (vprec == GB_PREC_F32) { k_convert_vals<float><<<nblk(nnz, 256), 256, 0, s>>>(nnz, in, (float *) out); }
   else { k_convert_vals<__half><<<nblk(nnz, 256), 256, 0, s>>>(nnz, in, (__half *) out); }
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Two-stage Gauss-Seidel inner sweep (reference:
// hypre_BoomerAMGRelaxTwoStageGaussSeidelHost src/parcsr_ls/par_relax.c:1506):
// z_new_i = (sum_{j<i} a_ij z_j) / a_ii ; u_i += m * z_new_i.
// The first entry of each row is the diagonal.
// ---------------------------------------------------------------------------
template <typename VT, typename XT>
__global__ void k_gs_lower(int n, const int *__restrict__ Ai, const int *__restrict__ Aj, const VT *__restrict__ Av,
                           const XT *__restrict__ z, XT *__restrict__ znew, XT *__restrict__ u, XT m)
{
   typedef typename Acc<VT, XT>::T AT;
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid >> 3, lane = tid & 7;
   bool valid = i < n;
   AT s = 0;
   int b0 = 0;
   if (valid)
   {
      b0 = Ai[i];
      int e0 = Ai[i + 1];
      for (int k = b0 + lane; k < e0; k += 8)
      {
         int j = Aj[k];
         if (j < i) { s += Acc<VT, XT>::mul(Av[k], z[j]); }
      }
   }
   for (int o = 4; o > 0; o >>= 1) { s += __shfl_down_sync(GB_FULL, s, o, 8); }
   if (valid && lane == 0)
   {
      XT diag = (XT) Acc<VT, XT>::mul(Av[b0], (XT) 1);
      XT zn = (XT) s / diag;
      znew[i] = zn;
      u[i] += m * zn;
   }
}

template <typename VT, typename XT>
__global__ void k_gs_first(int n, const int *__restrict__ Ai, const VT *__restrict__ Av, XT *__restrict__ v,
                           XT *__restrict__ u, const float *__restrict__ rs)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   // row-scaled FP16 values have a unit diagonal: the diagonal is rs[i]
   XT diag = rs ? (XT) rs[i] : (XT) Acc<VT, XT>::mul(Av[Ai[i]], (XT) 1);
   XT z = v[i] / diag;
   v[i] = z;
   u[i] += z;
}

// a_ii (the first entry of row i; 1 for an empty row) in the given precision
template <typename T>
__global__ void k_diag_vals(int n, const int *__restrict__ Ai, const double *__restrict__ Av, T *__restrict__ out)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int b = Ai[i];
   out[i] = (T) (Ai[i + 1] > b ? Av[b] : 1.0);
}

// first stage with a contiguous diagonal: z = v/d; v = z; u += z
template <typename XT>
__global__ void k_gs_first_diag(int n, const XT *__restrict__ diag, XT *__restrict__ v, XT *__restrict__ u)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   XT z = v[i] / diag[i];
   v[i] = z;
   u[i] += z;
}

extern "C" void gb_diag_vals(int n, const int *Ai, const double *Av, int vprec, void *out, cudaStream_t s)
{
   if (n <= 0) { return; }
   if (vprec == GB_PREC_F64) { k_diag_vals<double><<<nblk(n, 256), 256, 0, s>>>(n, Ai, Av, (double *) out); }
   else { k_diag_vals<float><<<nblk(n, 256), 256, 0, s>>>(n, Ai, Av, (float *) out); }
   GB_COUNT(1);
}

extern "C" void gb_gs_first_diag_d(int n, const double *diag, double *v, double *u, cudaStream_t s)
{
   if (n > 0) { k_gs_first_diag<double><<<nblk(n, 256), 256, 0, s>>>(n, diag, v, u); GB_COUNT(1); }
}

extern "C" void gb_gs_first_diag_f(int n, const float *diag, float *v, float *u, cudaStream_t s)
{
   if (n > 0) { k_gs_first_diag<float><<<nblk(n, 256), 256, 0, s>>>(n, diag, v, u); GB_COUNT(1); }
}

extern "C" void gb_gs_first_d(int n, const int *Ai, const double *Av, double *v, double *u, cudaStream_t s)
{
   k_gs_first<double, double><<<nblk(n, 256), 256, 0, s>>>(n, Ai, Av, v, u, nullptr);
   GB_COUNT(1);
}
extern "C" void gb_gs_first_f(int n, const int *Ai, const void *Av, int vprec, const float *rs, float *v, float *u,
                              cudaStream_t s)
{
   if (vprec == GB_PREC_F16)
   {
      k_gs_first<__half, float><<<nblk(n, 256), 256, 0, s>>>(n, Ai, (const __half *) Av, v, u, rs);
   }
   else { k_gs_first<float, float><<<nblk(n, 256), 256, 0, s>>>(n, Ai, (const float *) Av, v, u, nullptr); }
   GB_COUNT(1);
}
extern "C" void gb_gs_lower_d(int n, const int *Ai, const int *Aj, const double *Av, const double *z, double *znew,
                              double *u, double m, cudaStream_t s)
{
   k_gs_lower<double, double><<<nblk((long long) n * 8, 256), 256, 0, s>>>(n, Ai, Aj, Av, z, znew, u, m);
   GB_COUNT(1);
}
extern "C" void gb_gs_lower_f(int n, const int *Ai, const int *Aj, const void *Av, int vprec, const float *z,
                              float *znew, float *u, float m, cudaStream_t s)
{
   if (vprec == GB_PREC_F16)
   {
      k_gs_lower<__half, float><<<nblk((long long) n * 8, 256), 256, 0, s>>>(n, Ai, Aj, (const __half *) Av, z, znew, u, m);
   }
   else
   {
      k_gs_lower<float, float><<<nblk((long long) n * 8, 256), 256, 0, s>>>(n, Ai, Aj, (const float *) Av, z, znew, u, m);
   }
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Vector operations (FP64 unless suffixed _f)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fill(long long n, T *x, T v)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { x[i] = v; }
}
template <typename T>
__global__ void k_scale(long long n, T a, T *x)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { x[i] *= a; }
}
template <typename T>
__global__ void k_axpy(long long n, T a, const T *__restrict__ x, T *__restrict__ y)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { y[i] += a * x[i]; }
}
template <typename T>
__global__ void k_xpay(long long n, const T *__restrict__ x, T a, T *__restrict__ y)
{
   // y = x + a*y
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { y[i] = x[i] + a * y[i]; }
}
template <typename T>
__global__ void k_scaled_div(long long n, T w, const T *__restrict__ f, const T *__restrict__ d, T *__restrict__ u)
{
   // u = w * f / d   (first Jacobi sweep from a zero guess)
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { u[i] = (w * f[i]) / d[i]; }
}
template <typename T>
__global__ void k_scaled_copy(long long n, T w, const T *__restrict__ f, T *__restrict__ v)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { v[i] = w * f[i]; }
}
__global__ void k_d2f(long long n, const double *__restrict__ a, float *__restrict__ b)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { b[i] = (float) a[i]; }
}
__global__ void k_f2d(long long n, const float *__restrict__ a, double *__restrict__ b)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { b[i] = (double) a[i]; }
}

// dot products: partial sums per block over a fixed grid, then one block.
__global__ void __launch_bounds__(256) k_dot_part(long long n, const double *__restrict__ x,
                                                  const double *__restrict__ y, double *__restrict__ part)
{
   double s = 0.0;
   for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
   {
      s += x[i] * y[i];
   }
   double t = block_sum<double>(s);
   if (threadIdx.x == 0) { part[blockIdx.x] = t; }
}

// y += a*x, then partial sums of z . y (z may be y): one pass for a
// modified Gram-Schmidt step and the next inner product, with the grid,
// loop order and reduction of k_dot_part (identical sums)
__global__ void __launch_bounds__(256) k_axpy_dot_part(long long n, double a, const double *__restrict__ x, double *y,
                                                       const double *z, double *__restrict__ part)
{
   double s = 0.0;
   for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
   {
      double yi = y[i] + a * x[i];
      y[i] = yi;
      s += z[i] * yi;
   }
   double t = block_sum<double>(s);
   if (threadIdx.x == 0) { part[blockIdx.x] = t; }
}

__global__ void __launch_bounds__(256) k_dot2_part(long long n, const double *__restrict__ x,
                                                   const double *__restrict__ y, const double *__restrict__ z,
                                                   double *__restrict__ part)
{
   // part[b] = sum x*y, part[nb + b] = sum x*z
   double s = 0.0, t2 = 0.0;
   for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
   {
      double xi = x[i];
      s += xi * y[i];
      t2 += xi * z[i];
   }
   double a = block_sum<double>(s);
   double c = block_sum<double>(t2);
   if (threadIdx.x == 0) { part[blockIdx.x] = a; part[gridDim.x + blockIdx.x] = c; }
}

// x += a*p ; r -= a*s ; partial (r, r)
__global__ void __launch_bounds__(256) k_pcg_xr(long long n, double a, const double *__restrict__ p,
                                                const double *__restrict__ s, double *__restrict__ x,
                                                double *__restrict__ r, double *__restrict__ part)
{
   double acc = 0.0;
   for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
   {
      x[i] += a * p[i];
      double ri = r[i] + (-a) * s[i];
      r[i] = ri;
      acc += ri * ri;
   }
   double t = block_sum<double>(acc);
   if (threadIdx.x == 0) { part[blockIdx.x] = t; }
}

__global__ void k_final_sum(int nparts, int nsums, const double *__restrict__ part, double *__restrict__ out)
{
   // one block; out[q] = sum_b part[q*nparts + b] in a fixed order
   for (int q = 0; q < nsums; q++)
   {
      double s = 0.0;
      for (int b = threadIdx.x; b < nparts; b += blockDim.x) { s += part[(size_t) q * nparts + b]; }
      double t = block_sum<double>(s);
      if (threadIdx.x == 0) { out[q] = t; }
      __syncthreads();
   }
}

extern "C" void gb_fill_d(long long n, double *x, double v, cudaStream_t s)
{ if (n > 0) { k_fill<double><<<nblk(n, 256), 256, 0, s>>>(n, x, v); GB_COUNT(1); } }
extern "C" void gb_fill_f(long long n, float *x, float v, cudaStream_t s)
{ if (n > 0) { k_fill<float><<<nblk(n, 256), 256, 0, s>>>(n, x, v); GB_COUNT(1); } }
extern "C" void gb_scale_d(long long n, double a, double *x, cudaStream_t s)
{ if (n > 0) { k_scale<double><<<nblk(n, 256), 256, 0, s>>>(n, a, x); GB_COUNT(1); } }
extern "C" void gb_axpy_d(long long n, double a, const double *x, double *y, cudaStream_t s)
{ if (n > 0) { k_axpy<double><<<nblk(n, 256), 256, 0, s>>>(n, a, x, y); GB_COUNT(1); } }
extern "C" void gb_xpay_d(long long n, const double *x, double a, double *y, cudaStream_t s)
{ if (n > 0) { k_xpay<double><<<nblk(n, 256), 256, 0, s>>>(n, x, a, y); GB_COUNT(1); } }
extern "C" void gb_scaled_div_d(long long n, double w, const double *f, const double *d, double *u, cudaStream_t s)
{ if (n > 0) { k_scaled_div<double><<<nblk(n, 256), 256, 0, s>>>(n, w, f, d, u); GB_COUNT(1); } }
extern "C" void gb_scaled_div_f(long long n, float w, const float *f, const float *d, float *u, cudaStream_t s)
{ if (n > 0) { k_scaled_div<float><<<nblk(n, 256), 256, 0, s>>>(n, w, f, d, u); GB_COUNT(1); } }
extern "C" void gb_scaled_copy_d(long long n, double w, const double *f, double *v, cudaStream_t s)
{ if (n > 0) { k_scaled_copy<double><<<nblk(n, 256), 256, 0, s>>>(n, w, f, v); GB_COUNT(1); } }
extern "C" void gb_scaled_copy_f(long long n, float w, const float *f, float *v, cudaStream_t s)
{ if (n > 0) { k_scaled_copy<float><<<nblk(n, 256), 256, 0, s>>>(n, w, f, v); GB_COUNT(1); } }
extern "C" void gb_d2f(long long n, const double *a, float *b, cudaStream_t s)
{ if (n > 0) { k_d2f<<<nblk(n, 256), 256, 0, s>>>(n, a, b); GB_COUNT(1); } }
extern "C" void gb_f2d(long long n, const float *a, double *b, cudaStream_t s)
{ if (n > 0) { k_f2d<<<nblk(n, 256), 256, 0, s>>>(n, a, b); GB_COUNT(1); } }

// Chebyshev smoother vector steps (d = D^{-1/2}):
//   start:   q = d .* (c * r)          (u stays as the original iterate)
//   order 1: u = u + d .* (c * r)
template <typename T>
__global__ void k_cheb_start(long long n, T c, const T *__restrict__ r, const T *__restrict__ d, T *__restrict__ q)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { q[i] = d[i] * (r[i] * c); }
}
template <typename T>
__global__ void k_cheb_order1(long long n, T c, const T *__restrict__ r, const T *__restrict__ d, T *__restrict__ u)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { u[i] = u[i] + d[i] * (r[i] * c); }
}
template <typename T>
__global__ void k_vmul(long long n, const T *__restrict__ a, const T *__restrict__ b, T *c)
{
   long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { c[i] = a[i] * b[i]; }
}

extern "C" void gb_cheb_start_d(long long n, double c, const double *r, const double *d, double *q, cudaStream_t s)
{ if (n > 0) { k_cheb_start<double><<<nblk(n, 256), 256, 0, s>>>(n, c, r, d, q); GB_COUNT(1); } }
extern "C" void gb_cheb_start_f(long long n, float c, const float *r, const float *d, float *q, cudaStream_t s)
{ if (n > 0) { k_cheb_start<float><<<nblk(n, 256), 256, 0, s>>>(n, c, r, d, q); GB_COUNT(1); } }
extern "C" void gb_cheb_order1_d(long long n, double c, const double *r, const double *d, double *u, cudaStream_t s)
{ if (n > 0) { k_cheb_order1<double><<<nblk(n, 256), 256, 0, s>>>(n, c, r, d, u); GB_COUNT(1); } }
extern "C" void gb_cheb_order1_f(long long n, float c, const float *r, const float *d, float *u, cudaStream_t s)
{ if (n > 0) { k_cheb_order1<float><<<nblk(n, 256), 256, 0, s>>>(n, c, r, d, u); GB_COUNT(1); } }
extern "C" void gb_vmul_d(long long n, const double *a, const double *b, double *c, cudaStream_t s)
{ if (n > 0) { k_vmul<double><<<nblk(n, 256), 256, 0, s>>>(n, a, b, c); GB_COUNT(1); } }
extern "C" void gb_vmul_f(long long n, const float *a, const float *b, float *c, cudaStream_t s)
{ if (n > 0) { k_vmul<float><<<nblk(n, 256), 256, 0, s>>>(n, a, b, c); GB_COUNT(1); } }

// Sum of nparts block partials in the order and tree of k_final_sum (1024
// threads: thread v adds part[v], part[v + 1024], ... from 0, then
// block_sum), computed by one block of 256 threads that each carry the
// virtual threads t, t+256, t+512, t+768 -- the same lanes, so every warp
// shuffle pairs the same values and the result is bit for bit k_final_sum's.
// Valid in thread 0.
__device__ double final_sum_1024(const double *part, int nparts)
{
   __shared__ double red[32];
   const int t = threadIdx.x, lane = t & 31, w = t >> 5;
   double sk[4];
#pragma unroll
   for (int k = 0; k < 4; k++)
   {
      double a = 0.0;
      for (int b = t + 256 * k; b < nparts; b += 1024) { a += __ldcg(part + b); }
      sk[k] = a;
   }
#pragma unroll
   for (int k = 0; k < 4; k++)
   {
      for (int o = 16; o > 0; o >>= 1) { sk[k] += __shfl_down_sync(GB_FULL, sk[k], o); }
   }
   __syncthreads();
   if (lane == 0)
   {
#pragma unroll
      for (int k = 0; k < 4; k++) { red[w + 8 * k] = sk[k]; }
   }
   __syncthreads();
   double r = 0.0;
   if (w == 0)
   {
      r = red[lane];
      for (int o = 16; o > 0; o >>= 1) { r += __shfl_down_sync(GB_FULL, r, o); }
   }
   return r;
}

// the block that finishes last (a counter after a fence) sums the partials
// and resets the counter: one launch per reduction
__device__ __forceinline__ void finish_sum(double t, double *part, unsigned int *count, double *out)
{
   __shared__ int last;
   if (threadIdx.x == 0)
   {
      part[blockIdx.x] = t;
      __threadfence();
      last = atomicAdd(count, 1u) == gridDim.x - 1;
   }
   __syncthreads();
   if (!last) { return; }
   __threadfence();
   double r = final_sum_1024(part, gridDim.x);
   if (threadIdx.x == 0) { *out = r; *count = 0u; }
}

// (x, y) in one launch, the sum as k_dot_part + k_final_sum
__global__ void __launch_bounds__(256) k_dot_fin(long long n, const double *__restrict__ x,
                                                 const double *__restrict__ y, double *part, unsigned int *count,
                                                 double *out)
{
   double s = 0.0;
   for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
   {
      s += x[i] * y[i];
   }
   finish_sum(block_sum<double>(s), part, count, out);
}

// y -= (*h) x, then (z, y) in one launch (the sum as k_axpy_dot_part +
// k_final_sum); h is read from device memory (the previous inner product, so
// the Gram-Schmidt chain needs no host round trip)
__global__ void __launch_bounds__(256) k_axpy_dot_dev_fin(long long n, const double *__restrict__ h,
                                                          const double *__restrict__ x, double *y, const double *z,
                                                          double *part, unsigned int *count, double *out)
{
   const double a = -(*h);
   double s = 0.0;
   for (long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
   {
      double yi = y[i] + a * x[i];
      y[i] = yi;
      s += z[i] * yi;
   }
   finish_sum(block_sum<double>(s), part, count, out);
}

extern "C" void gb_dot_d(long long n, const double *x, const double *y, double *part, unsigned int *count,
                         double *out, cudaStream_t s)
{
   k_dot_fin<<<GB_RED_BLOCKS, 256, 0, s>>>(n, x, y, part, count, out);
   GB_COUNT(1);
}

extern "C" void gb_axpy_dot_dev_d(long long n, const double *h, const double *x, double *y, const double *z,
                                  double *part, unsigned int *count, double *out, cudaStream_t s)
{
   k_axpy_dot_dev_fin<<<GB_RED_BLOCKS, 256, 0, s>>>(n, h, x, y, z, part, count, out);
   GB_COUNT(1);
}

extern "C" void gb_axpy_dot_d(long long n, double a, const double *x, double *y, const double *z, double *part,
                              double *out, cudaStream_t s)
{
   k_axpy_dot_part<<<GB_RED_BLOCKS, 256, 0, s>>>(n, a, x, y, z, part);
   k_final_sum<<<1, 1024, 0, s>>>(GB_RED_BLOCKS, 1, part, out);
   GB_COUNT(2);
}
extern "C" void gb_dot2_d(long long n, const double *x, const double *y, const double *z, double *part, double *out,
                          cudaStream_t s)
{
   k_dot2_part<<<GB_RED_BLOCKS, 256, 0, s>>>(n, x, y, z, part);
   k_final_sum<<<1, 1024, 0, s>>>(GB_RED_BLOCKS, 2, part, out);
   GB_COUNT(2);
}
extern "C" void gb_pcg_xr_d(long long n, double a, const double *p, const double *sv, double *x, double *r,
                            double *part, double *out, cudaStream_t s)
{
   k_pcg_xr<<<GB_RED_BLOCKS, 256, 0, s>>>(n, a, p, sv, x, r, part);
   k_final_sum<<<1, 1024, 0, s>>>(GB_RED_BLOCKS, 1, part, out);
   GB_COUNT(2);
}
extern "C" void gb_final_sum(int nparts, int nsums, const double *part, double *out, cudaStream_t s)
{
   k_final_sum<<<1, 1024, 0, s>>>(nparts, nsums, part, out);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Dense coarsest-grid apply: u = Dinv * f (n small)
// ---------------------------------------------------------------------------
template <typename XT>
__global__ void k_dense_apply(int n, const double *__restrict__ D, const XT *__restrict__ f, XT *__restrict__ u)
{
   int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
   int lane = threadIdx.x & 31;
   if (i >= n) { return; }
   double s = 0.0;
   for (int j = lane; j < n; j += 32) { s += D[(size_t) i * n + j] * (double) f[j]; }
   for (int o = 16; o > 0; o >>= 1) { s += __shfl_down_sync(GB_FULL, s, o); }
   if (lane == 0) { u[i] = (XT) s; }
}

extern "C" void gb_dense_apply_d(int n, const double *D, const double *f, double *u, cudaStream_t s)
{
   k_dense_apply<double><<<nblk(n, 8), 256, 0, s>>>(n, D, f, u);
   GB_COUNT(1);
}
extern "C" void gb_dense_apply_f(int n, const double *D, const float *f, float *u, cudaStream_t s)
{
   k_dense_apply<float><<<nblk(n, 8), 256, 0, s>>>(n, D, f, u);
   GB_COUNT(1);
}
