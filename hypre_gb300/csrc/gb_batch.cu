// Batched AMG-PCG for many independent systems in one persistent launch.
//
// The systems are the diagonal blocks of one block-diagonal matrix; BoomerAMG
// setup on that matrix keeps every level block diagonal, and the coarse points
// of a block are numbered consecutively, so system s owns the rows
// off_l[s] .. off_l[s+1]-1 of every level l.  Each CTA takes systems from a
// queue (largest first) and runs the whole FP64 PCG -- every SpMV, V-cycle,
// inner product and update of that system -- with only block barriers, so one
// launch solves the batch.  The V-cycle (l1-Jacobi or Jacobi smoothing, coarse
// dense solve) runs in FP64 or FP32 (template CT); the Krylov vectors, inner
// products and the stopping test are FP64.
//
// Same arithmetic as the single-system path: the PCG of src/krylov/pcg.c:313
// (two-norm stopping test), the V(1,1) cycle of src/parcsr_ls/par_cycle.c with
// relaxation from a zero guess on the way down (u = w f / l1) and
// u += w (f - A u) / l1 sweeps on the way up.
#include "gb_device.cuh"
#include "gb_internal.h"

typedef struct
{
   int n;
   const int *Ai, *Aj;
   const void *Av;    // CT
   const int *Pi, *Pj;
   const void *Pv;
   const int *Ri, *Rj;
   const void *Rv;
   const void *l1;    // CT
   void *F, *U, *V;   // CT work vectors of the level
   const int *off;    // nsys + 1 row offsets
   double w;
} gb_blevel;

typedef struct
{
   const gb_blevel *lev;
   int nlev, nsys, sweeps_down, sweeps_up;
   const int *Ai, *Aj;       // FP64 level-0 operator for the Krylov method
   const double *Av;
   const int *order;         // systems, largest first
   int *counter;
   const double *b;
   double *x, *r, *p, *s;
   const double *Dinv;       // coarsest level: inverse of each system's block
   const long long *doff;    // its offset in Dinv (block s is m x m, m its coarsest rows)
   double tol;
   int maxit;
   int *iters;
   double *relres;
   double *hist;             // nsys x (maxit + 1)
} gb_batch_args;

namespace
{

__device__ __forceinline__ double block_sum2(double v, double *red, int nw)
{
   // sum over the block; every thread receives the total (fixed tree: deterministic)
   for (int o = 16; o > 0; o >>= 1) { v += __shfl_down_sync(GB_FULL, v, o); }
   int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   __syncthreads();
   if (lane == 0) { red[wid] = v; }
   __syncthreads();
   if (wid == 0)
   {
      double t = lane < nw ? red[lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) { t += __shfl_down_sync(GB_FULL, t, o); }
      if (lane == 0) { red[32] = t; }
   }
   __syncthreads();
   return red[32];
}

// Row loop over rows [a, b) with LPR lanes per row; op(i, s) gets the row's
// sum s = sum_k A_ik x_k (type AT) on the group's first lane.  The loop count
// is uniform over the block, so the group shuffles see every lane.
template <int LPR, typename AT, typename VT, typename XT, typename Op>
__device__ __forceinline__ void rows_spmv(int a, int b, const int *__restrict__ Ai, const int *__restrict__ Aj,
                                          const VT *__restrict__ Av, const XT *x, Op op)
{
   const int groups = blockDim.x / LPR;
   const int g = threadIdx.x / LPR, lane = threadIdx.x % LPR;
   for (int base = a; base < b; base += groups)
   {
      int i = base + g;
      AT s = 0;
      if (i < b)
      {
         for (int k = Ai[i] + lane; k < Ai[i + 1]; k += LPR) { s += (AT) Av[k] * (AT) x[Aj[k]]; }
      }
      if (LPR > 1)
      {
         for (int o = LPR / 2; o > 0; o >>= 1) { s += __shfl_down_sync(GB_FULL, s, o, LPR); }
      }
      if (i < b && lane == 0) { op(i, s); }
   }
}

template <typename CT, int LPR>
__device__ void vcycle(const gb_batch_args &A, int sys, const double *r0, double *z0)
{
   const gb_blevel *lev = A.lev;
   const int nlev = A.nlev;
   // level 0 right-hand side and iterate
   CT *F0, *U0;
   {
      int a = lev[0].off[sys], b = lev[0].off[sys + 1];
      if constexpr (sizeof(CT) == sizeof(double))
      {
         F0 = (CT *) r0;
         U0 = (CT *) z0;
      }
      else
      {
         F0 = (CT *) lev[0].F;
         U0 = (CT *) lev[0].U;
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { F0[i] = (CT) r0[i]; }
         __syncthreads();
      }
   }
   // down
   for (int l = 0; l < nlev - 1; l++)
   {
      const gb_blevel &L = lev[l];
      int a = L.off[sys], b = L.off[sys + 1];
      CT *F = l ? (CT *) L.F : F0, *U = l ? (CT *) L.U : U0, *V = (CT *) L.V;
      const CT *Av = (const CT *) L.Av, *l1 = (const CT *) L.l1;
      const CT w = (CT) L.w;
      for (int i = a + threadIdx.x; i < b; i += blockDim.x) { U[i] = (w * F[i]) / l1[i]; }
      __syncthreads();
      for (int sw = 1; sw < A.sweeps_down; sw++)
      {
         rows_spmv<LPR, CT>(a, b, L.Ai, L.Aj, Av, U, [&](int i, CT s) { V[i] = U[i] + w * (F[i] - s) / l1[i]; });
         __syncthreads();
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { U[i] = V[i]; }
         __syncthreads();
      }
      // residual, then restriction to the system's coarse rows
      rows_spmv<LPR, CT>(a, b, L.Ai, L.Aj, Av, U, [&](int i, CT s) { V[i] = F[i] - s; });
      __syncthreads();
      const gb_blevel &C = lev[l + 1];
      rows_spmv<LPR, CT>(C.off[sys], C.off[sys + 1], L.Ri, L.Rj, (const CT *) L.Rv, V,
                         [&](int i, CT s) { ((CT *) C.F)[i] = s; });
      __syncthreads();
   }
   // coarsest: dense inverse restricted to the system's block
   {
      const gb_blevel &L = lev[nlev - 1];
      int a = L.off[sys], b = L.off[sys + 1];
      CT *F = nlev > 1 ? (CT *) L.F : F0, *U = nlev > 1 ? (CT *) L.U : U0;
      for (int i = a + threadIdx.x; i < b; i += blockDim.x)
      {
         double s = 0.0;
         const double *Ds = A.Dinv + A.doff[sys] + (size_t) (i - a) * (b - a);
         for (int j = a; j < b; j++) { s += Ds[j - a] * (double) F[j]; }
         U[i] = (CT) s;
      }
      __syncthreads();
   }
   // up
   for (int l = nlev - 2; l >= 0; l--)
   {
      const gb_blevel &L = lev[l];
      const gb_blevel &C = lev[l + 1];
      int a = L.off[sys], b = L.off[sys + 1];
      CT *F = l ? (CT *) L.F : F0, *U = l ? (CT *) L.U : U0, *V = (CT *) L.V;
      const CT *Av = (const CT *) L.Av, *l1 = (const CT *) L.l1;
      const CT w = (CT) L.w;
      const CT *Uc = (const CT *) C.U;   // level l + 1 >= 1
      rows_spmv<LPR, CT>(a, b, L.Pi, L.Pj, (const CT *) L.Pv, Uc, [&](int i, CT s) { U[i] = s + U[i]; });
      __syncthreads();
      for (int sw = 0; sw < A.sweeps_up; sw++)
      {
         rows_spmv<LPR, CT>(a, b, L.Ai, L.Aj, Av, U, [&](int i, CT s) { V[i] = U[i] + w * (F[i] - s) / l1[i]; });
         __syncthreads();
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { U[i] = V[i]; }
         __syncthreads();
      }
   }
   if constexpr (sizeof(CT) != sizeof(double))
   {
      int a = lev[0].off[sys], b = lev[0].off[sys + 1];
      for (int i = a + threadIdx.x; i < b; i += blockDim.x) { z0[i] = (double) U0[i]; }
      __syncthreads();
   }
}

template <typename CT, int LPR>
__global__ void __launch_bounds__(512) k_batch_pcg(gb_batch_args A)
{
   __shared__ double red[33];
   __shared__ int sys_sh;
   const int nw = (blockDim.x + 31) >> 5;
   const int *off0 = A.lev[0].off;
   for (;;)
   {
      if (threadIdx.x == 0)
      {
         int t = atomicAdd(A.counter, 1);
         sys_sh = t < A.nsys ? A.order[t] : -1;
      }
      __syncthreads();
      const int sys = sys_sh;
      __syncthreads();
      if (sys < 0) { break; }
      const int a = off0[sys], b = off0[sys + 1];
      double *hist = A.hist + (size_t) sys * (A.maxit + 1);
      // <b, b>
      double acc = 0.0;
      for (int i = a + threadIdx.x; i < b; i += blockDim.x) { acc += A.b[i] * A.b[i]; }
      const double bi = block_sum2(acc, red, nw);
      if (!(bi > 0.0))
      {
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { A.x[i] = A.b[i]; }
         if (threadIdx.x == 0) { A.iters[sys] = 0; A.relres[sys] = 0.0; hist[0] = 0.0; }
         __syncthreads();
         continue;
      }
      const double eps = A.tol * A.tol;
      // r = b - A x
      rows_spmv<LPR, double>(a, b, A.Ai, A.Aj, A.Av, (const double *) A.x,
                             [&](int i, double s) { A.r[i] = A.b[i] - s; });
      __syncthreads();
      vcycle<CT, LPR>(A, sys, A.r, A.p);
      double g0 = 0.0, g1 = 0.0;
      for (int i = a + threadIdx.x; i < b; i += blockDim.x) { g0 += A.r[i] * A.p[i]; g1 += A.r[i] * A.r[i]; }
      double gamma = block_sum2(g0, red, nw);
      double iprod = block_sum2(g1, red, nw);
      if (threadIdx.x == 0) { hist[0] = sqrt(iprod / bi); }
      int it = 0;
      while (it + 1 <= A.maxit)
      {
         it++;
         double sp = 0.0;
         rows_spmv<LPR, double>(a, b, A.Ai, A.Aj, A.Av, (const double *) A.p, [&](int i, double s) { A.s[i] = s; });
         __syncthreads();
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { sp += A.s[i] * A.p[i]; }
         const double sdotp = block_sum2(sp, red, nw);
         if (sdotp == 0.0) { break; }
         const double alpha = gamma / sdotp;
         if (alpha <= 0.0) { break; }
         const double gamma_old = gamma;
         for (int i = a + threadIdx.x; i < b; i += blockDim.x)
         {
            A.x[i] += alpha * A.p[i];
            A.r[i] = A.r[i] + (-alpha) * A.s[i];
         }
         __syncthreads();
         vcycle<CT, LPR>(A, sys, A.r, A.s);
         g0 = 0.0;
         g1 = 0.0;
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { g0 += A.r[i] * A.s[i]; g1 += A.r[i] * A.r[i]; }
         gamma = block_sum2(g0, red, nw);
         iprod = block_sum2(g1, red, nw);
         if (threadIdx.x == 0) { hist[it] = sqrt(iprod / bi); }
         if (iprod / bi < eps) { break; }
         const double beta = gamma / gamma_old;
         for (int i = a + threadIdx.x; i < b; i += blockDim.x) { A.p[i] = A.s[i] + beta * A.p[i]; }
         __syncthreads();
      }
      if (threadIdx.x == 0)
      {
         A.iters[sys] = it;
         A.relres[sys] = sqrt(iprod / bi);
      }
      __syncthreads();
   }
}

template <typename CT>
void launch_lpr(const gb_batch_args &A, int lpr, int grid, int block, cudaStream_t s)
{
   switch (lpr)
   {
      case 1: k_batch_pcg<CT, 1><<<grid, block, 0, s>>>(A); break;
      case 2: k_batch_pcg<CT, 2><<<grid, block, 0, s>>>(A); break;
      case 4: k_batch_pcg<CT, 4><<<grid, block, 0, s>>>(A); break;
      default: k_batch_pcg<CT, 8><<<grid, block, 0, s>>>(A); break;
   }
}

} // namespace

// Check that every row's columns stay inside its system's diagonal block.
__global__ void k_check_blockdiag(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                                  const int *__restrict__ off, int nsys, int *__restrict__ bad)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int lo = 0, hi = nsys;   // find s with off[s] <= i < off[s+1]
   while (hi - lo > 1)
   {
      int mid = (lo + hi) >> 1;
      if (off[mid] <= i) { lo = mid; } else { hi = mid; }
   }
   int a = off[lo], b = off[lo + 1];
   for (int k = Ai[i]; k < Ai[i + 1]; k++)
   {
      int j = Aj[k];
      if (j < a || j >= b) { atomicExch(bad, 1); return; }
   }
}

extern "C" void gb_check_blockdiag(int n, const int *Ai, const int *Aj, const int *off, int nsys, int *bad,
                                   cudaStream_t s)
{
   if (n > 0) { k_check_blockdiag<<<(n + 255) / 256, 256, 0, s>>>(n, Ai, Aj, off, nsys, bad); GB_COUNT(1); }
}

extern "C" void gb_batch_pcg(const void *lev_dev, int nlev, int nsys, int sweeps_down, int sweeps_up,
                             const int *Ai, const int *Aj, const double *Av, const int *order, int *counter,
                             const double *b, double *x, double *r, double *p, double *sv, const double *Dinv,
                             const long long *doff, double tol, int maxit, int *iters, double *relres, double *hist, int prec,
                             int lpr, int grid, int block, cudaStream_t s)
{
   gb_batch_args A;
   A.lev = (const gb_blevel *) lev_dev;
   A.nlev = nlev;
   A.nsys = nsys;
   A.sweeps_down = sweeps_down;
   A.sweeps_up = sweeps_up;
   A.Ai = Ai; A.Aj = Aj; A.Av = Av;
   A.order = order; A.counter = counter;
   A.b = b; A.x = x; A.r = r; A.p = p; A.s = sv;
   A.Dinv = Dinv; A.doff = doff;
   A.tol = tol; A.maxit = maxit;
   A.iters = iters; A.relres = relres; A.hist = hist;
   cudaMemsetAsync(counter, 0, sizeof(int), s);
   if (prec == GB_PREC_F64) { launch_lpr<double>(A, lpr, grid, block, s); }
   else { launch_lpr<float>(A, lpr, grid, block, s); }
   GB_COUNT(1);
}

extern "C" size_t gb_blevel_size(void) { return sizeof(gb_blevel); }

extern "C" void gb_blevel_set(void *host_array, int l, int n, const int *Ai, const int *Aj, const void *Av,
                              const int *Pi, const int *Pj, const void *Pv, const int *Ri, const int *Rj,
                              const void *Rv, const void *l1, void *F, void *U, void *V, const int *off, double w)
{
   gb_blevel *L = ((gb_blevel *) host_array) + l;
   L->n = n;
   L->Ai = Ai; L->Aj = Aj; L->Av = Av;
   L->Pi = Pi; L->Pj = Pj; L->Pv = Pv;
   L->Ri = Ri; L->Rj = Rj; L->Rv = Rv;
   L->l1 = l1;
   L->F = F; L->U = U; L->V = V;
   L->off = off;
   L->w = w;
}
