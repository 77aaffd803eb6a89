// Multiple right-hand sides: vectors of nv columns stored interleaved
// (entry (i, c) at i * nv + c), so one pass over a sparse matrix serves every
// column (SpMM).  A warp owns a row: the row's column indices and values are
// read once and broadcast, lane l accumulates columns l and l + 32, and the
// loads of a neighbour's nv values are contiguous (nv * 8 bytes for FP64).
// Inner products are per column with a fixed reduction order.
#include "gb_device.cuh"
#include "gb_internal.h"

namespace
{

inline int nblk(long long n, int b) { return (int) ((n + b - 1) / b); }

__device__ __forceinline__ double mfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Epilogue modes as the single-vector SpMV: 0 y = alpha s + beta b,
// 1 Jacobi y = x + w (b - s) / d_i, 2 residual y = b - s.
// The row's column indices and values are loaded 32 at a time (one
// coalesced load per lane) and broadcast by shuffles; U neighbour rows of x
// are loaded before any of them is used, so U gathers per lane are in flight.
// Each column's sum adds the row's terms in element order whatever U is, so
// every U gives the same result.
template <typename VT, typename XT, int U>
__global__ void __launch_bounds__(512) k_spmm_csr(int n, int nv, const int *__restrict__ Ai,
                                                  const int *__restrict__ Aj, const VT *__restrict__ Av,
                                                  const XT *__restrict__ x, XT *y, int mode, XT alpha, XT beta,
                                                  const XT *b, const XT *d, XT w)
{
   const int lane = threadIdx.x & 31;
   const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int nwarps = (gridDim.x * blockDim.x) >> 5;
   const bool c0 = lane < nv, c1 = lane + 32 < nv;
   for (int i = warp; i < n; i += nwarps)
   {
      XT s0 = 0, s1 = 0;
      const int e = Ai[i + 1];
      for (int c = Ai[i]; c < e; c += 32)
      {
         const int k = c + lane;
         int jl = 0;
         XT al = 0;
         if (k < e)
         {
            jl = __ldg(Aj + k);
            al = (XT) __ldg(Av + k);
         }
         const int m = min(32, e - c);
         for (int t = 0; t < m; t += U)
         {
            XT aa[U], xa[U], xb[U];
#pragma unroll
            for (int u = 0; u < U; u++)
            {
               const int tt = (t + u) & 31;
               const int j = __shfl_sync(GB_FULL, jl, tt);
               aa[u] = __shfl_sync(GB_FULL, al, tt);
               const bool ok = t + u < m;
               const XT *xr = x + (size_t) j * nv;
               xa[u] = ok && c0 ? __ldg(xr + lane) : (XT) 0;
               xb[u] = ok && c1 ? __ldg(xr + lane + 32) : (XT) 0;
            }
#pragma unroll
            for (int u = 0; u < U; u++)
            {
               if (t + u < m)
               {
                  // explicit fused multiply-adds: the same operation whatever
                  // the compiler would contract in each unrolled variant
                  if (c0) { s0 = mfma(aa[u], xa[u], s0); }
                  if (c1) { s1 = mfma(aa[u], xb[u], s1); }
               }
            }
         }
      }
      for (int h = 0; h < 2; h++)
      {
         if (h == 0 ? !c0 : !c1) { continue; }
         const size_t o = (size_t) i * nv + lane + 32 * h;
         const XT s = h == 0 ? s0 : s1;
         XT r;
         if (mode == 1) { r = x[o] + w * (b[o] - s) / d[i]; }
         else if (mode == 2) { r = b[o] - s; }
         else
         {
            r = alpha * s;
            if (beta != (XT) 0) { r += beta * b[o]; }
         }
         y[o] = r;
      }
   }
}

// u = w f / d per row (first Jacobi sweep from zero)
template <typename T>
__global__ void k_mscaled_div(long long n, int nv, T w, const T *__restrict__ f, const T *__restrict__ d,
                              T *__restrict__ u)
{
   long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (e < n * nv) { u[e] = (w * f[e]) / d[e / nv]; }
}

// U (nc x nv) = D (nc x nc, FP64) F
template <typename XT>
__global__ void k_mdense(int nc, int nv, const double *__restrict__ D, const XT *__restrict__ f, XT *__restrict__ u)
{
   int e = blockIdx.x * blockDim.x + threadIdx.x;
   if (e >= nc * nv) { return; }
   int i = e / nv, c = e % nv;
   double s = 0.0;
   for (int j = 0; j < nc; j++) { s += D[(size_t) i * nc + j] * (double) f[(size_t) j * nv + c]; }
   u[e] = (XT) s;
}

// per-column partial sums: part[b * (2 nv) + c] = sum x*y, part[b * (2 nv) + nv + c] = sum x*z
// (z may be NULL); rows of block b: a contiguous range
__global__ void __launch_bounds__(256) k_mdot_part(int n, int nv, const double *__restrict__ x,
                                                   const double *__restrict__ y, const double *__restrict__ z,
                                                   double *__restrict__ part)
{
   __shared__ double s1[256], s2[256];
   const int rows_per_pass = blockDim.x / nv;
   const int c = threadIdx.x % nv, rr = threadIdx.x / nv;
   const long long chunk = ((long long) n + gridDim.x - 1) / gridDim.x;
   const long long r0 = (long long) blockIdx.x * chunk;
   long long r1 = r0 + chunk;
   if (r1 > n) { r1 = n; }
   double a = 0.0, bb = 0.0;
   if (rr < rows_per_pass)
   {
      for (long long i = r0 + rr; i < r1; i += rows_per_pass)
      {
         double xv = x[i * nv + c];
         a += xv * y[i * nv + c];
         if (z) { bb += xv * z[i * nv + c]; }
      }
   }
   s1[threadIdx.x] = a;
   s2[threadIdx.x] = bb;
   __syncthreads();
   if (threadIdx.x < nv)
   {
      double t1 = 0.0, t2 = 0.0;
      for (int q = 0; q < rows_per_pass; q++) { t1 += s1[q * nv + threadIdx.x]; t2 += s2[q * nv + threadIdx.x]; }
      part[(size_t) blockIdx.x * 2 * nv + threadIdx.x] = t1;
      part[(size_t) blockIdx.x * 2 * nv + nv + threadIdx.x] = t2;
   }
}

__global__ void k_mdot_final(int nb, int nv, const double *__restrict__ part, double *__restrict__ out)
{
   int c = threadIdx.x;
   if (c >= 2 * nv) { return; }
   double s = 0.0;
   for (int b = 0; b < nb; b++) { s += part[(size_t) b * 2 * nv + c]; }
   out[c] = s;
}

// x += a_c p ; r -= a_c s  (a per column, device)
__global__ void k_mpcg_xr(long long n, int nv, const double *__restrict__ a, const double *__restrict__ p,
                          const double *__restrict__ s, double *__restrict__ x, double *__restrict__ r)
{
   long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (e >= n * nv) { return; }
   double al = a[e % nv];
   x[e] += al * p[e];
   r[e] = r[e] + (-al) * s[e];
}

// p = s + b_c p
__global__ void k_mxpay(long long n, int nv, const double *__restrict__ s, const double *__restrict__ bc,
                        double *__restrict__ p)
{
   long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (e < n * nv) { p[e] = s[e] + bc[e % nv] * p[e]; }
}

template <typename A, typename B>
__global__ void k_mconvert(long long n, const A *__restrict__ a, B *__restrict__ b)
{
   long long e = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   if (e < n) { b[e] = (B) a[e]; }
}

} // namespace

#define MDOT_BLOCKS 608

extern "C" int gb_mdot_blocks(void) { return MDOT_BLOCKS; }

template <typename VT, typename XT>
static void spmm_launch(int n, int nv, const int *Ai, const int *Aj, const VT *Av, const XT *x, XT *y, int mode,
                        XT alpha, XT beta, const XT *b, const XT *d, XT w, int T, int U, cudaStream_t s)
{
   if (n <= 0) { return; }
   if (T != 128 && T != 512) { T = 256; }
   long long blocks = ((long long) n * 32 + T - 1) / T;
   const long long cap = 152LL * 16 * 256 / T;
   if (blocks > cap) { blocks = cap; }
   const int nb = (int) blocks;
   if (U == 1) { k_spmm_csr<VT, XT, 1><<<nb, T, 0, s>>>(n, nv, Ai, Aj, Av, x, y, mode, alpha, beta, b, d, w); }
   else if (U == 4) { k_spmm_csr<VT, XT, 4><<<nb, T, 0, s>>>(n, nv, Ai, Aj, Av, x, y, mode, alpha, beta, b, d, w); }
   else if (U == 8) { k_spmm_csr<VT, XT, 8><<<nb, T, 0, s>>>(n, nv, Ai, Aj, Av, x, y, mode, alpha, beta, b, d, w); }
   else { k_spmm_csr<VT, XT, 2><<<nb, T, 0, s>>>(n, nv, Ai, Aj, Av, x, y, mode, alpha, beta, b, d, w); }
   GB_COUNT(1);
}

// T: block size (128, 256, 512; 0 = 256), U: neighbour rows of x in flight
// per lane (1, 2, 4, 8; 0 = 2)
extern "C" void gb_spmm_d(int n, int nv, const int *Ai, const int *Aj, const double *Av, const double *x, double *y,
                          int mode, double alpha, double beta, const double *b, const double *d, double w, int T,
                          int U, cudaStream_t s)
{
   spmm_launch<double, double>(n, nv, Ai, Aj, Av, x, y, mode, alpha, beta, b, d, w, T, U, s);
}

extern "C" void gb_spmm_f(int n, int nv, const int *Ai, const int *Aj, const float *Av, const float *x, float *y,
                          int mode, float alpha, float beta, const float *b, const float *d, float w, int T, int U,
                          cudaStream_t s)
{
   spmm_launch<float, float>(n, nv, Ai, Aj, Av, x, y, mode, alpha, beta, b, d, w, T, U, s);
}

extern "C" void gb_mscaled_div_d(long long n, int nv, double w, const double *f, const double *d, double *u,
                                 cudaStream_t s)
{
   if (n > 0) { k_mscaled_div<double><<<nblk(n * nv, 256), 256, 0, s>>>(n, nv, w, f, d, u); GB_COUNT(1); }
}

extern "C" void gb_mscaled_div_f(long long n, int nv, float w, const float *f, const float *d, float *u,
                                 cudaStream_t s)
{
   if (n > 0) { k_mscaled_div<float><<<nblk(n * nv, 256), 256, 0, s>>>(n, nv, w, f, d, u); GB_COUNT(1); }
}

extern "C" void gb_mdense_d(int nc, int nv, const double *D, const double *f, double *u, cudaStream_t s)
{
   if (nc > 0) { k_mdense<double><<<nblk((long long) nc * nv, 128), 128, 0, s>>>(nc, nv, D, f, u); GB_COUNT(1); }
}

extern "C" void gb_mdense_f(int nc, int nv, const double *D, const float *f, float *u, cudaStream_t s)
{
   if (nc > 0) { k_mdense<float><<<nblk((long long) nc * nv, 128), 128, 0, s>>>(nc, nv, D, f, u); GB_COUNT(1); }
}

// out[c] = (x, y)_c and out[nv + c] = (x, z)_c (z may be NULL); nv <= 64
extern "C" void gb_mdot2(int n, int nv, const double *x, const double *y, const double *z, double *part, double *out,
                         cudaStream_t s)
{
   k_mdot_part<<<MDOT_BLOCKS, 256, 0, s>>>(n, nv, x, y, z, part);
   k_mdot_final<<<1, 128, 0, s>>>(MDOT_BLOCKS, nv, part, out);
   GB_COUNT(2);
}

extern "C" void gb_mpcg_xr(long long n, int nv, const double *a, const double *p, const double *sv, double *x,
                           double *r, cudaStream_t s)
{
   if (n > 0) { k_mpcg_xr<<<nblk(n * nv, 256), 256, 0, s>>>(n, nv, a, p, sv, x, r); GB_COUNT(1); }
}

extern "C" void gb_mxpay(long long n, int nv, const double *sv, const double *bc, double *p, cudaStream_t s)
{
   if (n > 0) { k_mxpay<<<nblk(n * nv, 256), 256, 0, s>>>(n, nv, sv, bc, p); GB_COUNT(1); }
}

extern "C" void gb_d2f_n(long long n, const double *a, float *b, cudaStream_t s)
{
   if (n > 0) { k_mconvert<double, float><<<nblk(n, 256), 256, 0, s>>>(n, a, b); GB_COUNT(1); }
}

extern "C" void gb_f2d_n(long long n, const float *a, double *b, cudaStream_t s)
{
   if (n > 0) { k_mconvert<float, double><<<nblk(n, 256), 256, 0, s>>>(n, a, b); GB_COUNT(1); }
}
