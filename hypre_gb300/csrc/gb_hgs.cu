// Hybrid Gauss-Seidel sweeps (relax types 3, 4, 6, 8, 13, 14), bit for bit
// the reference's single-process loops (src/parcsr_ls/par_relax.h:13-330,
// hypre_HybridGaussSeidelNS and hypre_HybridGaussSeidel, driven by
// hypre_BoomerAMGRelaxHybridGaussSeidel_core, par_relax.c:692-945).
//
// A sweep visits the rows in order (forward: 0..n-1, backward: n-1..0).  Row
// i reads the values the sweep already produced for the rows before it and
// the values from before the sweep for the rows after it, and sums its terms
// in CSR order.  On the GPU each warp takes the next row of the sweep from an
// atomic counter; a row waits only for the earlier rows its entries refer to
// (their flags, set with release semantics after the value is stored), so
// rows without such a dependency run at once and the sweep's critical path is
// the dependency depth of the matrix, not its row count.  Rows are handed out
// in sweep order to running warps, so the earliest unfinished row never waits
// on a row that no warp holds: the sweep always progresses.  Every wait is
// bounded (GB_HGS_SPIN polls); a wait that runs out sets *err and the sweep
// finishes with an undefined result, which the host reports.
//
// The products, sums and divisions use explicit round-to-nearest operations
// in the reference's order, so the FP64 sweep equals the sequential loop.
#include "gb_device.cuh"

#define GB_HGS_SPIN (1 << 21)

__device__ __forceinline__ int hgs_ld_acquire(const int *p)
{
   int v;
   asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
   return v;
}

__device__ __forceinline__ void hgs_st_release(int *p, int v)
{
   asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ double hgs_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float hgs_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double hgs_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float hgs_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double hgs_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float hgs_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double hgs_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float hgs_div(float a, float b) { return __fdiv_rn(a, b); }

// Waits until the rows of the lanes with dep set have been written.  One lane
// polls at a time -- the dependency nearest this row in sweep order, usually
// the last to finish -- and then every waiting lane checks its flag once, so
// a warp keeps one poll in flight instead of one per neighbour (thousands of
// warps polling every neighbour's flag saturated the L2).  Polls are acquire
// loads, so a lane that has seen its flag set reads the row's value after the
// writer's release.  Each poll loop is bounded: when it runs out, or another
// warp's did (*err), the wait ends.
__device__ __forceinline__ void hgs_wait(bool dep, int col, const int *flags, int *err, int lane, int dir)
{
   unsigned pending = __ballot_sync(GB_FULL, dep && hgs_ld_acquire(flags + col) == 0);
   while (pending)
   {
      const int L = dir > 0 ? 31 - __clz(pending) : __ffs(pending) - 1;
      int bail = 0;
      if (lane == L)
      {
         int spins = 0;
         unsigned ns = 32;
         while (hgs_ld_acquire(flags + col) == 0)
         {
            if (++spins > GB_HGS_SPIN) { atomicExch(err, 1); bail = 1; break; }
            if ((spins & 1023) == 0 && *(volatile int *) err) { bail = 1; break; }
            __nanosleep(ns);
            if (ns < 256) { ns <<= 1; }
         }
      }
      if (__shfl_sync(GB_FULL, bail, L)) { break; }
      pending = __ballot_sync(GB_FULL, ((pending >> lane) & 1u) && hgs_ld_acquire(flags + col) == 0);
   }
}

// One sweep.  cf / pts: with pts != 0 only the rows with cf == pts relax
// (C/F relaxation; the others keep their values, par_relax.h:45,77).
// u: values updated in place; uo: u as it was when the sweep
// started (read for the rows not yet visited and for the row's own entry);
// ut: u before the first sweep of the relaxation (the scaled form's second
// sum, hypre's Vtemp), NULL when unscaled; dvec: l1 norms (relax 8/13/14) or
// NULL for the diagonal (the row's first entry).  skip: the row's first
// (diagonal) entry is left out of the sums.  flags[0..n-1] and flags[n] (the
// row counter) start at zero.
template <typename T>
__global__ void __launch_bounds__(256) k_hgs(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                                             const T *__restrict__ Av, const T *__restrict__ f, T *u,
                                             const T *__restrict__ uo, const T *__restrict__ ut,
                                             const T *__restrict__ dvec, int dir, int skip, T w, T omega, T prod,
                                             const int *__restrict__ cf, int pts, int *flags, int *err)
{
   const int lane = threadIdx.x & 31;
   int *counter = flags + n;
   for (;;)
   {
      int t = 0;
      if (lane == 0) { t = atomicAdd(counter, 1); }
      t = __shfl_sync(GB_FULL, t, 0);
      if (t >= n) { break; }
      const int i = dir > 0 ? t : n - 1 - t;
      const int b = Ai[i], e = Ai[i + 1];
      const T aii = e > b ? Av[b] : (T) 0;
      const T di = dvec ? dvec[i] : aii;
      T ui = uo[i];
      if (di != (T) 0 && (pts == 0 || cf[i] == pts))
      {
         T res = f[i], res0 = 0, res2 = 0;
         for (int c = b + skip; c < e; c += 32)
         {
            const int k = c + lane;
            int col = 0;
            bool dep = false;
            if (k < e)
            {
               col = Aj[k];
               dep = dir > 0 ? col < i : col > i;   // visited by the sweep before this row
            }
            hgs_wait(dep, col, flags, err, lane, dir);
            T p = 0, p2 = 0;
            if (k < e)
            {
               const T a = Av[k];
               const T v = dep ? __ldcg(u + col) : uo[col];
               p = hgs_mul(a, v);
               if (ut) { p2 = hgs_mul(a, ut[col]); }
            }
            const int cnt = min(32, e - c);
            for (int q = 0; q < cnt; q++)
            {
               const T pq = __shfl_sync(GB_FULL, p, q);
               if (ut)
               {
                  const T p2q = __shfl_sync(GB_FULL, p2, q);
                  res0 = hgs_sub(res0, pq);
                  res2 = hgs_add(res2, p2q);
               }
               else { res = hgs_sub(res, pq); }
            }
         }
         if (ut)
         {
            // u = (skip ? u * prod : u) + w * (omega * f + res0 + (1 - omega) * res2) / d
            const T s = hgs_add(hgs_add(hgs_mul(omega, res), res0), hgs_mul(hgs_sub((T) 1, omega), res2));
            const T upd = hgs_div(hgs_mul(w, s), di);
            ui = hgs_add(skip ? hgs_mul(ui, prod) : ui, upd);
         }
         else if (skip) { ui = hgs_div(res, di); }
         else { ui = hgs_add(ui, hgs_div(res, di)); }
      }
      if (lane == 0)
      {
         u[i] = ui;
         hgs_st_release(flags + i, 1);
      }
      __syncwarp();
   }
}

// One sweep of a level whose matrix and vectors fit in shared memory (the
// coarse levels, whose dependency chains are about as long as their row
// counts, so that waiting on flags in global memory costs more than running
// the loop).  The block stages the rows, u, f, the l1 norms and the starting
// values into shared memory; one warp then runs the reference's loop in sweep
// order -- in place, so an unvisited row's entry still holds its value from
// before the sweep -- and the block writes u back.  The arithmetic is that of
// k_hgs, term for term.
template <typename T>
__global__ void __launch_bounds__(512) k_hgs_seq(int n, int nnz, const int *__restrict__ Ai,
                                                 const int *__restrict__ Aj, const T *__restrict__ Av,
                                                 const T *__restrict__ f, T *u, const T *__restrict__ ut,
                                                 const T *__restrict__ dvec, int dir, int skip, T w, T omega, T prod,
                                                 const int *__restrict__ cf, int pts)
{
   extern __shared__ __align__(16) unsigned char hgs_smem[];
   T *su = (T *) hgs_smem;
   T *sf = su + n;
   T *sut = sf + n;
   T *sd = sut + (ut ? n : 0);
   T *sav = sd + (dvec ? n : 0);
   int *sai = (int *) (sav + nnz);
   int *saj = sai + n + 1;
   const int base = Ai[0];
   for (int k = threadIdx.x; k < n; k += blockDim.x)
   {
      su[k] = u[k];
      sf[k] = f[k];
      if (ut) { sut[k] = ut[k]; }
      if (dvec) { sd[k] = dvec[k]; }
   }
   for (int k = threadIdx.x; k <= n; k += blockDim.x) { sai[k] = Ai[k] - base; }
   for (int k = threadIdx.x; k < nnz; k += blockDim.x)
   {
      saj[k] = Aj[base + k];
      sav[k] = Av[base + k];
   }
   __syncthreads();
   if (threadIdx.x < 32)
   {
      const int lane = threadIdx.x;
      for (int t = 0; t < n; t++)
      {
         const int i = dir > 0 ? t : n - 1 - t;
         const int b = sai[i], e = sai[i + 1];
         const T aii = e > b ? sav[b] : (T) 0;
         const T di = dvec ? sd[i] : aii;
         T ui = su[i];
         if (di != (T) 0 && (pts == 0 || cf[i] == pts))
         {
            T res = sf[i], res0 = 0, res2 = 0;
            for (int c = b + skip; c < e; c += 32)
            {
               const int k = c + lane;
               T p = 0, p2 = 0;
               if (k < e)
               {
                  const int col = saj[k];
                  const T a = sav[k];
                  p = hgs_mul(a, su[col]);
                  if (ut) { p2 = hgs_mul(a, sut[col]); }
               }
               const int cnt = min(32, e - c);
            for (int q = 0; q < cnt; q++)
            {
               const T pq = __shfl_sync(GB_FULL, p, q);
               if (ut)
               {
                  const T p2q = __shfl_sync(GB_FULL, p2, q);
                  res0 = hgs_sub(res0, pq);
                  res2 = hgs_add(res2, p2q);
               }
               else { res = hgs_sub(res, pq); }
            }
            }
            if (ut)
            {
               const T s = hgs_add(hgs_add(hgs_mul(omega, res), res0), hgs_mul(hgs_sub((T) 1, omega), res2));
               const T upd = hgs_div(hgs_mul(w, s), di);
               ui = hgs_add(skip ? hgs_mul(ui, prod) : ui, upd);
            }
            else if (skip) { ui = hgs_div(res, di); }
            else { ui = hgs_add(ui, hgs_div(res, di)); }
         }
         if (lane == 0) { su[i] = ui; }
         __syncwarp();
      }
   }
   __syncthreads();
   for (int k = threadIdx.x; k < n; k += blockDim.x) { u[k] = su[k]; }
}

#define GB_HGS_SEQ_SMEM (200 * 1024)

template <typename T>
static void hgs_sweep(int n, long long nnz, const int *Ai, const int *Aj, const T *Av, const T *f, T *u, T *uo,
                      const T *ut, const T *dvec, int dir, int skip, double w, double omega, const int *cf, int pts,
                      int *flags, int *err, cudaStream_t s)
{
   if (n <= 0) { return; }
   const double prod0 = 1.0 - w * omega;
   const long long smem = (long long) sizeof(T) * (2LL * n + (ut ? n : 0) + (dvec ? n : 0) + nnz) +
                          4LL * ((long long) n + 1 + nnz);
   if (smem <= GB_HGS_SEQ_SMEM)
   {
      static int attr_set = 0;
      if (!attr_set)
      {
         cudaFuncSetAttribute(k_hgs_seq<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_HGS_SEQ_SMEM);
         attr_set = 1;
      }
      k_hgs_seq<T><<<1, 512, (size_t) smem, s>>>(n, (int) nnz, Ai, Aj, Av, f, u, ut, dvec, dir, skip, (T) w,
                                                 (T) omega, (T) prod0, cf, pts);
      GB_COUNT(1);
      return;
   }
   cudaMemsetAsync(flags, 0, sizeof(int) * ((size_t) n + 1), s);
   cudaMemcpyAsync(uo, u, sizeof(T) * (size_t) n, cudaMemcpyDeviceToDevice, s);
   // a warp per row in flight; enough warps to cover a dependency front of a
   // few thousand rows, few enough that the spinning warps leave issue slots
   long long warps = n < 152LL * 16 ? n : 152LL * 16;
   int blocks = (int) ((warps * 32 + 255) / 256);
   k_hgs<T><<<blocks, 256, 0, s>>>(n, Ai, Aj, Av, f, u, uo, ut, dvec, dir, skip, (T) w, (T) omega, (T) prod0, cf,
                                   pts, flags, err);
   GB_COUNT(1);
}

extern "C" void gb_hgs_sweep_d(int n, long long nnz, const int *Ai, const int *Aj, const double *Av,
                               const double *f, double *u, double *uo, const double *ut, const double *dvec, int dir,
                               int skip, double w, double omega, const int *cf, int pts, int *flags, int *err,
                               cudaStream_t s)
{
   hgs_sweep<double>(n, nnz, Ai, Aj, Av, f, u, uo, ut, dvec, dir, skip, w, omega, cf, pts, flags, err, s);
}

extern "C" void gb_hgs_sweep_f(int n, long long nnz, const int *Ai, const int *Aj, const float *Av, const float *f,
                               float *u, float *uo, const float *ut, const float *dvec, int dir, int skip, double w,
                               double omega, const int *cf, int pts, int *flags, int *err, cudaStream_t s)
{
   hgs_sweep<float>(n, nnz, Ai, Aj, Av, f, u, uo, ut, dvec, dir, skip, w, omega, cf, pts, flags, err, s);
}

// C/F Jacobi half-relaxation: the rows of class pts (and a nonzero divisor)
// take the Jacobi value t, the others keep u
template <typename T>
__global__ void k_select_points(int n, const int *__restrict__ cf, int pts, const T *__restrict__ d,
                                const T *__restrict__ t, T *__restrict__ u)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && cf[i] == pts && d[i] != (T) 0) { u[i] = t[i]; }
}

extern "C" void gb_select_points_d(int n, const int *CF, int pts, const double *d, const double *t, double *u,
                                   cudaStream_t s)
{
   if (n <= 0) { return; }
   k_select_points<double><<<(n + 255) / 256, 256, 0, s>>>(n, CF, pts, d, t, u);
   GB_COUNT(1);
}

extern "C" void gb_select_points_f(int n, const int *CF, int pts, const float *d, const float *t, float *u,
                                   cudaStream_t s)
{
   if (n <= 0) { return; }
   k_select_points<float><<<(n + 255) / 256, 256, 0, s>>>(n, CF, pts, d, t, u);
   GB_COUNT(1);
}
