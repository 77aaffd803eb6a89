// AMG setup kernels for sm_103a: strength, PMIS, coarse numbering, extended+i
// interpolation, truncation, transpose, Galerkin product (RAP), l1 norms and
// the dense coarsest-grid inverse.
//
// Every integer result (strength pattern, C/F splitting, interpolation and
// coarse-operator sparsity, column order) is identical to the reference's
// serial CPU algorithms, and floating-point values are accumulated in the same
// order, so the FP64 hierarchy is bit-for-bit the reference's.  This file is
// compiled with --fmad=false: no a*b+c is fused, as in the reference's build.
//
// Column order matters downstream (the strength matrix keeps A's order, the
// interpolation discovers columns in that order, truncation sorts by |value|
// with a non-stable quicksort), so rows are built by one warp each with an
// ordered hash table (gb_warp_insert) that assigns positions in the exact
// discovery order of the reference's sequential loops.
#include "gb_device.cuh"
#include "gb_kernels.h"

#include <stdio.h>

#define C_PT 1
#define F_PT -1
#define SF_PT -3

static int gb_blocks(long long n, int t) { long long b = (n + t - 1) / t; return (int) (b < 1 ? 1 : b); }

// ---------------------------------------------------------------------------
// Exclusive scan of int32 (out[0..n], out[n] = total), three-phase.
// ---------------------------------------------------------------------------
#define SCAN_T 512
#define SCAN_PER 4
#define SCAN_TILE (SCAN_T * SCAN_PER)

// last: where a single-tile scan also writes its total (out + n), else NULL
__global__ void k_scan_tile(const int *__restrict__ in, int *__restrict__ out, int *__restrict__ sums, int n,
                            int *last)
{
   __shared__ int ws[SCAN_T / 32];
   int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
   int v[SCAN_PER];
   int loc = 0;
   for (int k = 0; k < SCAN_PER; k++) { int idx = base + k; v[k] = idx < n ? in[idx] : 0; loc += v[k]; }
   // inclusive warp scan of per-thread totals
   int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   int x = loc;
   for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(GB_FULL, x, o); if (lane >= o) { x += y; } }
   if (lane == 31) { ws[wid] = x; }
   __syncthreads();
   if (wid == 0)
   {
      int w = lane < SCAN_T / 32 ? ws[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(GB_FULL, w, o); if (lane >= o) { w += y; } }
      if (lane < SCAN_T / 32) { ws[lane] = w; }
   }
   __syncthreads();
   int excl = x - loc + (wid > 0 ? ws[wid - 1] : 0);
   for (int k = 0; k < SCAN_PER; k++) { int idx = base + k; if (idx < n) { out[idx] = excl; } excl += v[k]; }
   if (threadIdx.x == SCAN_T - 1)
   {
      sums[blockIdx.x] = excl;
      if (last) { *last = excl; }
   }
}

__global__ void k_scan_add(int *__restrict__ out, const int *__restrict__ sums_scanned, int n)
{
   int idx = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
   int add = sums_scanned[blockIdx.x];
   for (int k = 0; k < SCAN_PER; k++) { if (idx + k < n) { out[idx + k] += add; } }
}

__global__ void k_set_last(int *out, int n, const int *sums_scanned_total)
{
   out[n] = *sums_scanned_total;
}

// out has n+1 entries; scratch must hold gb_scan_scratch_ints(n) ints.
extern "C" long long gb_scan_scratch_ints(int n)
{
   long long tot = 0;
   long long m = n;
   while (1)
   {
      long long nb = (m + SCAN_TILE - 1) / SCAN_TILE;
      if (nb < 1) { nb = 1; }
      tot += nb + 1;
      if (nb == 1) { break; }
      m = nb;
   }
   return 2 * tot + 16;
}

static void scan_rec(const int *in, int *out, int n, int *scratch, cudaStream_t s)
{
   int nb = gb_blocks(n, SCAN_TILE);
   int *sums = scratch;            // nb+1 entries (exclusive-scanned in place below)
   // one tile: the tile kernel writes the total to out[n] itself
   k_scan_tile<<<nb, SCAN_T, 0, s>>>(in, out, sums, n, nb == 1 ? out + n : nullptr);
   GB_COUNT(1);
   if (nb == 1) { return; }
   int *sums_out = scratch + nb + 1;
   scan_rec(sums, sums_out, nb, sums_out + nb + 1, s);
   k_scan_add<<<nb, SCAN_T, 0, s>>>(out, sums_out, n);
   GB_COUNT(1);
   k_set_last<<<1, 1, 0, s>>>(out, n, sums_out + nb);
   GB_COUNT(1);
}

extern "C" void gb_exclusive_scan(const int *in, int *out, int n, int *scratch, cudaStream_t s)
{
   if (n <= 0)
   {
      cudaMemsetAsync(out, 0, sizeof(int), s);
      return;
   }
   scan_rec(in, out, n, scratch, s);
}

// ---------------------------------------------------------------------------
// Strength of connection (reference: src/parcsr_ls/par_strength.c:75-527).
// S keeps A's column order without the diagonal (the first entry of a row).
// ---------------------------------------------------------------------------
// sign tests on the bit pattern (integer ops; x < 0 and x > 0 as IEEE compares,
// false for zeros and NaN)
__device__ __forceinline__ bool gb_lt0(double x)
{
   long long b = __double_as_longlong(x);
   return b < 0 && (b & 0x7fffffffffffffffLL) != 0 && (b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool gb_gt0(double x)
{
   long long b = __double_as_longlong(x);
   return b > 0 && b <= 0x7ff0000000000000LL;
}

// Comparisons of matrix values run on integer keys: key(x) = +|x| or -|x|
// as the integer of the magnitude bits, which orders non-NaN doubles as the
// IEEE comparisons do (-0 and +0 both map to 0).  FP64 compares are scarce on
// this GPU; the row sum stays an FP64 sum in the reference's order.
__device__ __forceinline__ long long gb_okey(double x)
{
   long long b = __double_as_longlong(x);
   return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}

#define GB_WEAK_ROW ((long long) 0x8000000000000000ULL)

// row i's threshold key, or GB_WEAK_ROW when the row-sum test makes every
// connection weak
__device__ __forceinline__ long long strength_row(const int *Ai, const double *Av, int i, double theta, double mrs)
{
   int b = Ai[i], e = Ai[i + 1];
   if (b >= e) { return GB_WEAK_ROW; }   // an empty row has no connections
   double diag = Av[b];
   double row_scale = 0.0, row_sum = diag;
   long long ks = 0;
   if (diag < 0)
   {
      for (int k = b + 1; k < e; k++)
      {
         double v = Av[k];
         long long kv = gb_okey(v);
         if (ks < kv) { ks = kv; row_scale = v; }
         row_sum += v;
      }
   }
   else
   {
      for (int k = b + 1; k < e; k++)
      {
         double v = Av[k];
         long long kv = gb_okey(v);
         if (ks > kv) { ks = kv; row_scale = v; }
         row_sum += v;
      }
   }
   if ((fabs(row_sum) > fabs(diag) * mrs) && (mrs < 1.0)) { return GB_WEAK_ROW; }
   return gb_okey(theta * row_scale);
}

// strong: v > thr for a negative diagonal, v < thr otherwise
__device__ __forceinline__ int strength_test(double v, long long kt, bool dneg)
{
   long long kv = gb_okey(v);
   return dneg ? kv > kt : kv < kt;
}

__global__ void k_strength_count(int n, const int *__restrict__ Ai, const double *__restrict__ Av,
                                 double theta, double mrs, int *__restrict__ cnt, long long *__restrict__ rkey)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   long long kt = strength_row(Ai, Av, i, theta, mrs);
   rkey[i] = kt;
   int c = 0;
   if (kt != GB_WEAK_ROW)
   {
      const bool dneg = gb_lt0(Av[Ai[i]]);
      for (int k = Ai[i] + 1; k < Ai[i + 1]; k++) { c += strength_test(Av[k], kt, dneg); }
   }
   cnt[i] = c;
}

__global__ void k_strength_fill(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                                const double *__restrict__ Av, const long long *__restrict__ rkey,
                                const int *__restrict__ Si, int *__restrict__ Sj)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   long long kt = rkey[i];
   if (kt == GB_WEAK_ROW) { return; }
   const bool dneg = gb_lt0(Av[Ai[i]]);
   int p = Si[i];
   for (int k = Ai[i] + 1; k < Ai[i + 1]; k++)
   {
      if (strength_test(Av[k], kt, dneg)) { Sj[p++] = Aj[k]; }
   }
}

extern "C" void gb_strength_count(int n, const int *Ai, const double *Av, double theta, double mrs, int *cnt,
                                  long long *rkey, cudaStream_t s)
{
   k_strength_count<<<gb_blocks(n, 256), 256, 0, s>>>(n, Ai, Av, theta, mrs, cnt, rkey);
   GB_COUNT(1);
}

extern "C" void gb_strength_fill(int n, const int *Ai, const int *Aj, const double *Av, const long long *rkey,
                                 const int *Si, int *Sj, cudaStream_t s)
{
   k_strength_fill<<<gb_blocks(n, 256), 256, 0, s>>>(n, Ai, Aj, Av, rkey, Si, Sj);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// PMIS (reference: src/parcsr_ls/par_coarsen.c:2094-2806 with the random
// measures of src/parcsr_ls/par_indepset.c:33-63).  The reference's loops only
// write CF=0/1/-1 in ways whose outcome does not depend on the visiting order,
// so each phase is one data-parallel kernel.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pm_draw(long long k)
{
   // k-th Park-Miller draw (k >= 1) from seed 2747: 16807^k * 2747 mod (2^31-1)
   const unsigned long long m = 2147483647ULL;
   unsigned long long a = 16807ULL, r = 1ULL;
   long long e = k;
   while (e > 0) { if (e & 1) { r = (r * a) % m; } a = (a * a) % m; e >>= 1; }
   unsigned long long x = (r * 2747ULL) % m;
   return (double) x / (double) 2147483647;
}

// v[i] = 2 * (i+1)-th Park-Miller draw from seed - 1 (hypre_SeqVectorSetRandomValues,
// src/seq_mv/vector.c), each element computed independently by jump-ahead
__global__ void k_rand_uniform(int n, unsigned long long seed, double *__restrict__ v)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   const unsigned long long m = 2147483647ULL;
   unsigned long long a = 16807ULL, r = 1ULL;
   long long e = (long long) i + 1;
   while (e > 0) { if (e & 1) { r = (r * a) % m; } a = (a * a) % m; e >>= 1; }
   unsigned long long x = (r * seed) % m;
   v[i] = 2.0 * ((double) x / (double) 2147483647) - 1.0;
}

extern "C" void gb_rand_uniform(int n, int seed, double *v, cudaStream_t s)
{
   // seeds are clamped to [1, 2^31 - 2] as hypre_SeedRand does
   long long sd = seed < 1 ? 1 : (seed >= 2147483647 ? 2147483646 : seed);
   if (n > 0) { k_rand_uniform<<<gb_blocks(n, 256), 256, 0, s>>>(n, (unsigned long long) sd, v); GB_COUNT(1); }
}

// ds[i] = 1/sqrt(|a_ii|) for the first entry of row i in column i, 0 when
// there is none or it is zero (hypre_CSRMatrixExtractDiagonal type 4,
// src/seq_mv/csr_matop.c)
__global__ void k_diag_inv_sqrt(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                                const double *__restrict__ Av, double *__restrict__ ds)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   double d = 0.0;
   for (int k = Ai[i]; k < Ai[i + 1]; k++)
   {
      if (Aj[k] == i)
      {
         if (Av[k] != 0.0) { d = 1.0 / sqrt(fabs(Av[k])); }
         break;
      }
   }
   ds[i] = d;
}

extern "C" void gb_diag_inv_sqrt(int n, const int *Ai, const int *Aj, const double *Av, double *ds, cudaStream_t s)
{
   if (n > 0) { k_diag_inv_sqrt<<<gb_blocks(n, 256), 256, 0, s>>>(n, Ai, Aj, Av, ds); GB_COUNT(1); }
}

// (one atomic per entry: grouping a warp's equal columns with
// __match_any_sync first made the level-0 count 2x slower)
__global__ void k_colcount(int nnz, const int *__restrict__ Sj, int *__restrict__ colcnt)
{
   int k = blockIdx.x * blockDim.x + threadIdx.x;
   if (k < nnz) { atomicAdd(&colcnt[Sj[k]], 1); }
}

__global__ void k_pmis_init(int n, const int *__restrict__ Si, const int *__restrict__ colcnt, int CF_init,
                            double *__restrict__ measure, int *__restrict__ CF, int *__restrict__ ingraph)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   double m = (double) colcnt[i];
   m += pm_draw((long long) i + 1);
   int cf = 0, g = 1;
   if (Si[i + 1] - Si[i] == 0)
   {
      cf = (CF_init == 3 || CF_init == 4) ? C_PT : SF_PT;
      m = 0.0;
      g = 0;
   }
   measure[i] = m;
   CF[i] = cf;
   ingraph[i] = g;
}

// Measures are never negative (a column count plus a draw in (0, 1), or
// +0.0 once a point leaves the graph), and for non-negative doubles the
// order of the bit patterns as integers is the numeric order: the passes
// compare measures with integer instructions (FP64 compares are scarce on
// this GPU) and the same outcomes.
#define GB_ONE_BITS 0x3ff0000000000000LL

__device__ __forceinline__ long long gb_mbits(const double *m, int i) { return __double_as_longlong(m[i]); }

__global__ void k_pmis_select(int n, const int *__restrict__ ingraph, const double *__restrict__ measure,
                              int *__restrict__ CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && ingraph[i] && gb_mbits(measure, i) > GB_ONE_BITS) { CF[i] = 1; }
}

__global__ void k_pmis_remove(int n, const int *__restrict__ ingraph, const double *__restrict__ measure,
                              const int *__restrict__ Si, const int *__restrict__ Sj, int *CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n || !ingraph[i]) { return; }
   long long mi = gb_mbits(measure, i);
   if (!(mi > GB_ONE_BITS)) { return; }
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      int j = Sj[k];
      long long mj = gb_mbits(measure, j);
      if (mj > GB_ONE_BITS)
      {
         if (mi > mj) { CF[j] = 0; }
         else if (mj > mi) { CF[i] = 0; }
      }
   }
}

__global__ void k_pmis_setcf(int n, const int *__restrict__ ingraph, const double *__restrict__ measure,
                             const int *__restrict__ Si, const int *__restrict__ Sj, int *CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n || !ingraph[i]) { return; }
   if (gb_mbits(measure, i) < GB_ONE_BITS) { CF[i] = F_PT; }
   if (CF[i] > 0) { CF[i] = C_PT; return; }
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      if (CF[Sj[k]] > 0) { CF[i] = F_PT; break; }
   }
}

__global__ void k_pmis_update(int n, int *__restrict__ ingraph, double *__restrict__ measure,
                              const int *__restrict__ CF, int *__restrict__ remaining)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   int keep = 0;
   if (i < n && ingraph[i])
   {
      if (CF[i] != 0) { measure[i] = 0.0; ingraph[i] = 0; }
      else { keep = 1; }
   }
   unsigned b = __ballot_sync(GB_FULL, keep);
   if ((threadIdx.x & 31) == 0 && b) { atomicAdd(remaining, __popc(b)); }
}

// one PMIS pass (par_coarsen.c:2300-2420): the first pass with CF_init skips the
// selection; the pass's remaining graph size goes to d_counter[slot] and, by
// an asynchronous copy, to h_counter[slot].  A pass over an empty graph
// changes nothing.
static void pmis_pass(int n, int nb, int first, const int *Si, const int *Sj, int CF_init, int *CF,
                      double *measure, int *ingraph, int *d_counter, int *h_counter, int slot, cudaStream_t s)
{
   if (!CF_init || !first)
   {
      k_pmis_select<<<nb, 256, 0, s>>>(n, ingraph, measure, CF);
      k_pmis_remove<<<nb, 256, 0, s>>>(n, ingraph, measure, Si, Sj, CF);
      GB_COUNT(2);
   }
   k_pmis_setcf<<<nb, 256, 0, s>>>(n, ingraph, measure, Si, Sj, CF);
   cudaMemsetAsync(d_counter + slot, 0, sizeof(int), s);
   k_pmis_update<<<nb, 256, 0, s>>>(n, ingraph, measure, CF, d_counter + slot);
   GB_COUNT(2);
   cudaMemcpyAsync(h_counter + slot, d_counter + slot, sizeof(int), cudaMemcpyDeviceToHost, s);
}

// Passes run until the graph is empty.  Two passes are kept in flight: the
// host reads pass k's count while pass k+1 runs, so the GPU does not wait
// for the host between passes; the one pass queued after the last needed
// one finds an empty graph.  Returns the number of passes, -1 past max_iter.
extern "C" int gb_pmis(int n, int nnz, const int *Si, const int *Sj, int CF_init, int *CF, double *measure,
                       int *ingraph, int *colcnt, int *d_counter, int *h_counter, int max_iter, cudaStream_t s)
{
   cudaMemsetAsync(colcnt, 0, sizeof(int) * (size_t) (n > 0 ? n : 1), s);
   if (nnz > 0) { k_colcount<<<gb_blocks(nnz, 256), 256, 0, s>>>(nnz, Sj, colcnt); GB_COUNT(1); }
   int nb = gb_blocks(n, 256);
   k_pmis_init<<<nb, 256, 0, s>>>(n, Si, colcnt, CF_init, measure, CF, ingraph);
   GB_COUNT(1);
   cudaMemsetAsync(d_counter, 0, sizeof(int), s);
   // initial graph size
   k_pmis_update<<<nb, 256, 0, s>>>(n, ingraph, measure, CF, d_counter);
   GB_COUNT(1);
   cudaMemcpyAsync(h_counter, d_counter, sizeof(int), cudaMemcpyDeviceToHost, s);
   cudaStreamSynchronize(s);
   if (h_counter[0] == 0) { return 0; }
   cudaEvent_t ev[2];
   cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
   cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
   int queued = 0, checked = 0, result = -1;
   for (;;)
   {
      while (queued < checked + 2 && queued < max_iter)
      {
         pmis_pass(n, nb, queued == 0, Si, Sj, CF_init, CF, measure, ingraph, d_counter, h_counter, queued & 1, s);
         cudaEventRecord(ev[queued & 1], s);
         queued++;
      }
      if (checked == queued) { break; }
      cudaEventSynchronize(ev[checked & 1]);
      checked++;
      if (h_counter[(checked - 1) & 1] == 0) { result = checked; break; }
   }
   cudaEventDestroy(ev[0]);
   cudaEventDestroy(ev[1]);
   return result;
}

// ---------------------------------------------------------------------------
// Coarse numbering: flags (CF >= 0) for the scan, and counting
// ---------------------------------------------------------------------------
__global__ void k_cflag(int n, const int *__restrict__ CF, int *__restrict__ flag)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { flag[i] = CF[i] >= 0; }
}

extern "C" void gb_cpoint_flags(int n, const int *CF, int *flag, cudaStream_t s)
{
   k_cflag<<<gb_blocks(n, 256), 256, 0, s>>>(n, CF, flag);
   GB_COUNT(1);
}

__global__ void k_sf_to_f(int n, int *CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && CF[i] == SF_PT) { CF[i] = F_PT; }
}

extern "C" void gb_sf_to_f(int n, int *CF, cudaStream_t s)
{
   k_sf_to_f<<<gb_blocks(n, 256), 256, 0, s>>>(n, CF);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Extended+i interpolation (reference: src/parcsr_ls/par_lr_interp.c:1024-1924,
// hypre_BoomerAMGBuildExtPIInterpHost, one process) and its partial form for
// aggressive coarsening (src/parcsr_ls/partial.c:16-720), which builds the same
// rows for a listed subset of points (the old C points) numbered by list
// position.
//
// Tiers: every row is first built with a 1024-slot table in shared memory;
// rows whose candidate set does not fit are listed and rebuilt by a second
// launch with tables in global memory.
// ---------------------------------------------------------------------------

// Upper bound of the candidate C set of each row: |S_i| + sum over strong F
// neighbours of |S_i1| (+1).
__global__ void k_extpi_ub(int n, const int *__restrict__ Si, const int *__restrict__ Sj, const int *__restrict__ CF,
                           int *__restrict__ ub)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int u = 1;
   if (CF[i] < 0 && CF[i] != SF_PT)
   {
      for (int k = Si[i]; k < Si[i + 1]; k++)
      {
         int i1 = Sj[k];
         u += 1;
         if (CF[i1] < 0 && CF[i1] != SF_PT) { u += Si[i1 + 1] - Si[i1]; }
      }
   }
   ub[i] = u;
}

// Discovers the interpolation columns of F row i in the reference's order
// (strong C neighbours, then strong C neighbours of strong F neighbours).
__device__ __forceinline__ void extpi_discover(int i, const int *__restrict__ Si, const int *__restrict__ Sj,
                                               const int *__restrict__ CF, GbTab &T, int &count, int &ovf,
                                               int *Pj_row, const int *f2c, double *Pv_row)
{
   const int lane = gb_lane();
   for (int k = Si[i]; k < Si[i + 1] && !ovf; k++)
   {
      int i1 = Sj[k];
      int cf1 = CF[i1];
      if (cf1 >= 0)
      {
         if (Pj_row)
         {
            bool created;
            int pos = gb_winsert(T, count, i1, lane == 0, created, ovf);
            if (created && pos >= 0) { Pj_row[pos] = f2c[i1]; Pv_row[pos] = 0.0; }
         }
         else { gb_wcount(T, count, i1, lane == 0, ovf); }
      }
      else if (cf1 != SF_PT)
      {
         int b = Si[i1], e = Si[i1 + 1];
         for (int base = b; base < e && !ovf; base += 32)
         {
            int kk = base + lane;
            int k1 = kk < e ? Sj[kk] : -1;
            bool act = kk < e && CF[k1] >= 0;
            if (Pj_row)
            {
               bool created;
               int pos = gb_winsert(T, count, k1, act, created, ovf);
               if (created && pos >= 0) { Pj_row[pos] = f2c[k1]; Pv_row[pos] = 0.0; }
            }
            else { gb_wcount(T, count, k1, act, ovf); }
         }
      }
   }
   __syncwarp();
}

// Row r of the output is point i = rows ? rows[r] : r.
// GLOBAL == false: shared-memory tables, all rows; rows that overflow are
// appended to ovf_list.  GLOBAL == true: global tables, rows from ovf_list.
template <bool GLOBAL>
__global__ void __launch_bounds__(128) k_extpi_count(int nrows, const int *__restrict__ rows,
                                                     const int *__restrict__ Si, const int *__restrict__ Sj,
                                                     const int *__restrict__ CF, int *__restrict__ cnt,
                                                     const int *in_list, const int *in_n, int *ovf_list, int *ovf_n,
                                                     int *gtab, int gcap, int *err)
{
   extern __shared__ __align__(16) int sh[];
   const int lane = gb_lane();
   int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   int nwarps = (gridDim.x * blockDim.x) >> 5;
   GbTab T = GLOBAL ? gb_tab_at(gtab + (size_t) warp * GB_TAB_INTS(gcap), gcap)
                    : gb_tab_at(sh + (threadIdx.x >> 5) * GB_TAB_INTS(GB_SMEM_CAP), GB_SMEM_CAP);
   if (!GLOBAL) { gb_tab_init(T); }
   int total = *in_n;
   for (int t = warp; t < total; t += nwarps)
   {
      int r = in_list[t];
      int i = rows ? rows[r] : r;
      int cf = CF[i];
      if (cf >= 0) { if (lane == 0) { cnt[r] = 1; } continue; }
      if (cf == SF_PT) { if (lane == 0) { cnt[r] = 0; } continue; }
      int count = 0, ovf = 0;
      extpi_discover(i, Si, Sj, CF, T, count, ovf, nullptr, nullptr, nullptr);
      if (lane == 0)
      {
         if (!ovf) { cnt[r] = count; }
         else if (!GLOBAL) { ovf_list[atomicAdd(ovf_n, 1)] = r; cnt[r] = 0; }
         else { atomicExch(err, 1); }
      }
      gb_tab_clear(T, count);
   }
}

template <bool GLOBAL>
__global__ void __launch_bounds__(128) k_extpi_fill(int nrows, const int *__restrict__ rows,
                                                    const int *__restrict__ Ai, const int *__restrict__ Aj,
                                                    const double *__restrict__ Av, const int *__restrict__ Si,
                                                    const int *__restrict__ Sj, const int *__restrict__ CF,
                                                    const int *__restrict__ f2c, const int *__restrict__ Pi,
                                                    int *__restrict__ Pj, double *__restrict__ Pv,
                                                    const int *in_list, const int *in_n, int *gtab, int gcap,
                                                    int *err, int iterm)
{
   extern __shared__ __align__(16) int sh[];
   const int lane = gb_lane();
   int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   int nwarps = (gridDim.x * blockDim.x) >> 5;
   GbTab T = GLOBAL ? gb_tab_at(gtab + (size_t) warp * GB_TAB_INTS(gcap), gcap)
                    : gb_tab_at(sh + (threadIdx.x >> 5) * GB_TAB_INTS(GB_SMEM_CAP), GB_SMEM_CAP);
   if (!GLOBAL) { gb_tab_init(T); }
   int total = *in_n;
   for (int t = warp; t < total; t += nwarps)
   {
      int r = in_list[t];
      int i = rows ? rows[r] : r;
      int cf = CF[i];
      int begin = Pi[r];
      int len = Pi[r + 1] - begin;
      if (cf >= 0)
      {
         if (lane == 0) { Pj[begin] = f2c[i]; Pv[begin] = 1.0; }
         continue;
      }
      if (cf == SF_PT) { continue; }
      if (!GLOBAL && len > T.listcap) { continue; }   // rebuilt by the global tier
      int count = 0, ovf = 0;
      extpi_discover(i, Si, Sj, CF, T, count, ovf, Pj + begin, f2c, Pv + begin);
      if (ovf) { if (lane == 0) { atomicExch(err, 1); } gb_tab_clear(T, count); continue; }
      double *P = Pv + begin;
      double diagonal = Av[Ai[i]];
      int sp = Si[i], se = Si[i + 1];
      for (int jj = Ai[i] + 1; jj < Ai[i + 1]; jj++)
      {
         int i1 = Aj[jj];
         double a = Av[jj];
         bool strong = (sp < se && Sj[sp] == i1);
         if (strong) { sp++; }
         int pos1 = gb_tab_find(T.hk, T.hp, T.cap, i1);
         int cf1 = CF[i1];
         if (pos1 >= 0)
         {
            if (lane == 0) { P[pos1] += a; }
            __syncwarp();
         }
         else if (strong && cf1 < 0 && cf1 != SF_PT)
         {
            int b = Ai[i1], e = Ai[i1 + 1];
            int neg = Av[b] < 0;          // sgn = -1 when the neighbour's diagonal is negative
            double sum = 0.0;
            for (int base = b + 1; base < e; base += 32)
            {
               int k = base + lane;
               bool in = k < e;
               int i2 = in ? Aj[k] : -1;
               double a2 = in ? Av[k] : 0.0;
               bool sgnneg = neg ? (a2 > 0) : (a2 < 0);    // sgn * a2 < 0
               bool cond = in && sgnneg && ((iterm && i2 == i) || gb_tab_find(T.hk, T.hp, T.cap, i2) >= 0);
               sum = gb_warp_ordered_sum(a2, cond, sum);
            }
            if (sum != 0)
            {
               double distribute = a / sum;
               for (int base = b + 1; base < e; base += 32)
               {
                  int k = base + lane;
                  bool in = k < e;
                  int i2 = in ? Aj[k] : -1;
                  double a2 = in ? Av[k] : 0.0;
                  bool sgnneg = neg ? (a2 > 0) : (a2 < 0);
                  int pos2 = (in && sgnneg) ? gb_tab_find(T.hk, T.hp, T.cap, i2) : -1;
                  if (pos2 >= 0) { P[pos2] += distribute * a2; }
                  bool dterm = iterm && in && i2 == i && sgnneg;
                  unsigned dm = __ballot_sync(GB_FULL, dterm);
                  if (dm)
                  {
                     double contrib = __shfl_sync(GB_FULL, distribute * a2, __ffs(dm) - 1);
                     diagonal += contrib;
                  }
               }
               __syncwarp();
            }
            else { diagonal += a; }
         }
         else if (cf1 != SF_PT) { diagonal += a; }
      }
      __syncwarp();
      if (diagonal != 0.0)
      {
         for (int t2 = lane; t2 < count; t2 += 32) { P[t2] /= -diagonal; }
      }
      gb_tab_clear(T, count);
   }
}

extern "C" void gb_extpi_ub(int n, const int *Si, const int *Sj, const int *CF, int *ub, cudaStream_t s)
{
   k_extpi_ub<<<gb_blocks(n, 256), 256, 0, s>>>(n, Si, Sj, CF, ub);
   GB_COUNT(1);
}

static int gb_smem_blocks(int nrows)
{
   int dev = 0, sms = 148;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   long long want = (nrows + GB_SMEM_WARPS - 1) / GB_SMEM_WARPS;
   long long maxb = (long long) sms * 4;
   return (int) (want < maxb ? (want < 1 ? 1 : want) : maxb);
}

// tier 1: shared-memory tables, rows in_list -> overflow to out_list;
// tier 2: global tables, rows in_list.  (Tier 0 is the thread-per-row kernel.)
extern "C" void gb_extpi_count(int nrows, const int *rows, const int *Si, const int *Sj, const int *CF, int *cnt,
                               const int *in_list, const int *in_n, int n_hint, int *out_list, int *out_n, int *gtab,
                               int gcap, int gwarps, int *err, int tier, cudaStream_t s)
{
   if (tier == 1)
   {
      k_extpi_count<false><<<gb_smem_blocks(n_hint), 128, GB_SMEM_BYTES, s>>>(nrows, rows, Si, Sj, CF, cnt, in_list,
                                                                             in_n, out_list, out_n, nullptr, 0, err);
   }
   else
   {
      k_extpi_count<true><<<(gwarps + 3) / 4, 128, 0, s>>>(nrows, rows, Si, Sj, CF, cnt, in_list, in_n, out_list,
                                                           out_n, gtab, gcap, err);
   }
   GB_COUNT(1);
}

extern "C" void gb_extpi_fill(int nrows, const int *rows, const int *Ai, const int *Aj, const double *Av,
                              const int *Si, const int *Sj, const int *CF, const int *f2c, const int *Pi, int *Pj,
                              double *Pv, const int *in_list, const int *in_n, int n_hint, int *gtab, int gcap,
                              int gwarps, int *err, int tier, int iterm, cudaStream_t s)
{
   if (tier == 1)
   {
      k_extpi_fill<false><<<gb_smem_blocks(n_hint), 128, GB_SMEM_BYTES, s>>>(nrows, rows, Ai, Aj, Av, Si, Sj, CF, f2c,
                                                                            Pi, Pj, Pv, in_list, in_n, nullptr, 0,
                                                                            err, iterm);
   }
   else
   {
      k_extpi_fill<true><<<(gwarps + 3) / 4, 128, 0, s>>>(nrows, rows, Ai, Aj, Av, Si, Sj, CF, f2c, Pi, Pj, Pv,
                                                          in_list, in_n, gtab, gcap, err, iterm);
   }
   GB_COUNT(1);
}


// ---------------------------------------------------------------------------
// Thread-per-row extended+i (rows with at most GB_TPR_MAX candidates): each
// thread runs the reference's sequential loops for its row, so the FP64
// additions of 32 rows proceed in parallel on a warp instead of one serial
// chain per warp.  Membership of a fine point in the row's column set is a
// search of the row's coarse columns (only C points can be members).
// Rows with more candidates are listed for the warp-per-row kernels.
// (Key sets in shared memory, 32 KB per 128 threads, made the counting and
// filling about 10 ms slower on the 160^3 27-point problem than these local
// arrays, which stay in L1 and L2.)
// ---------------------------------------------------------------------------
#define GB_TPR_MAX 64
#define GB_TPR_BLOCK 128
typedef int *TprKeys;


/* The row's coarse columns are kept as a sorted set of packed keys
 * (coarse index << 6 | position in discovery order), so a membership test is
 * a binary search; coarse indices stay below 2^25 (checked by the host). */
__device__ __forceinline__ int tpr_lower(TprKeys sk, int len, int c)
{
   int lo = 0, hi = len;
   while (lo < hi)
   {
      int mid = (lo + hi) >> 1;
      if ((sk[mid] >> 6) < c) { lo = mid + 1; }
      else { hi = mid; }
   }
   return lo;
}

__device__ __forceinline__ int tpr_find(TprKeys sk, int len, int c)
{
   int lo = tpr_lower(sk, len, c);
   return (lo < len && (sk[lo] >> 6) == c) ? (sk[lo] & 63) : -1;
}

// adds coarse column c (new columns take the next position; Pj, when given,
// receives the columns in discovery order); false beyond GB_TPR_MAX
__device__ __forceinline__ bool tpr_add(TprKeys sk, int &len, int c, int *Pj)
{
   int lo = tpr_lower(sk, len, c);
   if (lo < len && (sk[lo] >> 6) == c) { return true; }
   if (len == GB_TPR_MAX) { return false; }
   for (int q = len; q > lo; q--) { sk[q] = sk[q - 1]; }
   sk[lo] = (c << 6) | len;
   if (Pj) { Pj[len] = c; }
   len++;
   return true;
}

// counts (or fills Pj, when given) the candidate columns of row i in
// discovery order; returns -1 beyond GB_TPR_MAX
__device__ int tpr_discover(int i, const int *__restrict__ Si, const int *__restrict__ Sj, const int *__restrict__ CF,
                            const int *__restrict__ f2c, TprKeys sk, int *Pj)
{
   int len = 0;
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      int i1 = Sj[k];
      int cf1 = CF[i1];
      if (cf1 >= 0)
      {
         if (!tpr_add(sk, len, f2c[i1], Pj)) { return -1; }
      }
      else if (cf1 != SF_PT)
      {
         for (int kk = Si[i1]; kk < Si[i1 + 1]; kk++)
         {
            int k1 = Sj[kk];
            if (CF[k1] >= 0 && !tpr_add(sk, len, f2c[k1], Pj)) { return -1; }
         }
      }
   }
   return len;
}

__global__ void __launch_bounds__(GB_TPR_BLOCK) k_extpi_count_t(int nrows, const int *__restrict__ rows,
                                                       const int *__restrict__ Si, const int *__restrict__ Sj,
                                                       const int *__restrict__ CF, const int *__restrict__ f2c,
                                                       int *__restrict__ cnt, int *ovf_list, int *ovf_n)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nrows) { return; }
   int i = rows ? rows[r] : r;
   int cf = CF[i];
   if (cf >= 0) { cnt[r] = 1; return; }
   if (cf == SF_PT) { cnt[r] = 0; return; }
   int sk[GB_TPR_MAX];
   int len = tpr_discover(i, Si, Sj, CF, f2c, sk, nullptr);
   if (len < 0) { cnt[r] = 0; ovf_list[atomicAdd(ovf_n, 1)] = r; }
   else { cnt[r] = len; }
}

__global__ void __launch_bounds__(GB_TPR_BLOCK) k_extpi_fill_t(int nrows, const int *__restrict__ rows,
                                                      const int *__restrict__ Ai, const int *__restrict__ Aj,
                                                      const double *__restrict__ Av, const int *__restrict__ Si,
                                                      const int *__restrict__ Sj, const int *__restrict__ CF,
                                                      const int *__restrict__ f2c, const int *__restrict__ Pi,
                                                      int *__restrict__ Pj, double *__restrict__ Pv, int iterm)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nrows) { return; }
   int i = rows ? rows[r] : r;
   int cf = CF[i];
   int begin = Pi[r];
   int len = Pi[r + 1] - begin;
   if (cf >= 0) { Pj[begin] = f2c[i]; Pv[begin] = 1.0; return; }
   if (cf == SF_PT || len > GB_TPR_MAX) { return; }
   int sk[GB_TPR_MAX];
   int l2 = tpr_discover(i, Si, Sj, CF, f2c, sk, Pj + begin);
   (void) l2;
   double *P = Pv + begin;
   for (int k = 0; k < len; k++) { P[k] = 0.0; }
   double diagonal = Av[Ai[i]];
   int sp = Si[i], se = Si[i + 1];
   for (int jj = Ai[i] + 1; jj < Ai[i + 1]; jj++)
   {
      int i1 = Aj[jj];
      double a = Av[jj];
      bool strong = (sp < se && Sj[sp] == i1);
      if (strong) { sp++; }
      int cf1 = CF[i1];
      int pos1 = cf1 >= 0 ? tpr_find(sk, len, f2c[i1]) : -1;
      if (pos1 >= 0) { P[pos1] += a; }
      else if (strong && cf1 < 0 && cf1 != SF_PT)
      {
         int b = Ai[i1], e = Ai[i1 + 1];
         bool neg = gb_lt0(Av[b]);
         double sum = 0.0;
         for (int k = b + 1; k < e; k++)
         {
            int i2 = Aj[k];
            double a2 = Av[k];
            bool sg = neg ? gb_gt0(a2) : gb_lt0(a2);
            if (sg && ((iterm && i2 == i) || (CF[i2] >= 0 && tpr_find(sk, len, f2c[i2]) >= 0))) { sum += a2; }
         }
         if (sum != 0)
         {
            double distribute = a / sum;
            for (int k = b + 1; k < e; k++)
            {
               int i2 = Aj[k];
               double a2 = Av[k];
               bool sg = neg ? gb_gt0(a2) : gb_lt0(a2);
               if (!sg) { continue; }
               int p2 = CF[i2] >= 0 ? tpr_find(sk, len, f2c[i2]) : -1;
               if (p2 >= 0) { P[p2] += distribute * a2; }
               if (iterm && i2 == i) { diagonal += distribute * a2; }
            }
         }
         else { diagonal += a; }
      }
      else if (cf1 != SF_PT) { diagonal += a; }
   }
   if (diagonal != 0.0)
   {
      for (int k = 0; k < len; k++) { P[k] /= -diagonal; }
   }
}

__global__ void k_iota(int n, int *__restrict__ out, int *__restrict__ count)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { out[i] = i; }
   if (i == 0) { *count = n; }
}

// ---------------------------------------------------------------------------
// Direct interpolation (interp_type 3, hypre_BoomerAMGBuildDirInterpHost
// src/parcsr_ls/par_interp.c:1873-2575, one process).  Count: C rows 1, F
// rows the C points of their S row.  Fill (thread per row): F row i takes
// those C points in S order with weight sum a_ij over A's row; alfa =
// (negative off-diagonal sum) / (negative C-point sum) / a_ii and beta the
// same for the positive ones, kept per row with a flag when defined.  Scale:
// the reference keeps alfa and beta from the previous row that defined them
// (starting from 1), so a row without one looks back for it.
// ---------------------------------------------------------------------------
__global__ void k_dir_count(int n, const int *__restrict__ Si, const int *__restrict__ Sj, const int *__restrict__ CF,
                            int *__restrict__ cnt)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int c = 0;
   if (CF[i] >= 0) { c = 1; }
   else { for (int k = Si[i]; k < Si[i + 1]; k++) { c += CF[Sj[k]] > 0; } }
   cnt[i] = c;
}

__global__ void k_dir_fill(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                           const double *__restrict__ Av, const int *__restrict__ Si, const int *__restrict__ Sj,
                           const int *__restrict__ CF, const int *__restrict__ f2c, const int *__restrict__ Pi,
                           int *__restrict__ Pj, double *__restrict__ Pv, double *__restrict__ alfa,
                           double *__restrict__ beta, int *__restrict__ flags)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   const int jb = Pi[i];
   if (CF[i] >= 0)
   {
      Pj[jb] = f2c[i];
      Pv[jb] = 1.0;
      flags[i] = 0;
      return;
   }
   int c = jb;
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      const int i1 = Sj[k];
      if (CF[i1] >= 0) { Pj[c] = f2c[i1]; Pv[c] = 0.0; c++; }
   }
   const double diagonal = Av[Ai[i]];
   double sNp = 0.0, sNn = 0.0, sPp = 0.0, sPn = 0.0;
   for (int jj = Ai[i] + 1; jj < Ai[i + 1]; jj++)
   {
      const int i1 = Aj[jj];
      const double a = Av[jj];
      if (a > 0) { sNp += a; } else { sNn += a; }
      // position of i1 among the row's strong C points (S order)
      int pos = -1, q = jb;
      for (int k = Si[i]; k < Si[i + 1] && pos < 0; k++)
      {
         const int j1 = Sj[k];
         if (CF[j1] >= 0)
         {
            if (j1 == i1) { pos = q; }
            q++;
         }
      }
      if (pos >= 0)
      {
         Pv[pos] += a;
         if (a > 0) { sPp += a; } else { sPn += a; }
      }
   }
   int fl = 0;
   if (sPn != 0.0) { alfa[i] = sNn / sPn / diagonal; fl |= 1; }
   if (sPp != 0.0) { beta[i] = sNp / sPp / diagonal; fl |= 2; }
   flags[i] = fl;
}

__global__ void k_dir_scale(int n, const int *__restrict__ CF, const int *__restrict__ Pi, double *__restrict__ Pv,
                            const double *__restrict__ alfa, const double *__restrict__ beta,
                            const int *__restrict__ flags)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n || CF[i] >= 0) { return; }
   double a = 1.0, b = 1.0;
   int k = i;
   while (k >= 0 && !(flags[k] & 1)) { k--; }
   if (k >= 0) { a = alfa[k]; }
   k = i;
   while (k >= 0 && !(flags[k] & 2)) { k--; }
   if (k >= 0) { b = beta[k]; }
   for (int jj = Pi[i]; jj < Pi[i + 1]; jj++)
   {
      if (Pv[jj] > 0) { Pv[jj] *= -b; }
      else { Pv[jj] *= -a; }
   }
}

extern "C" void gb_dir_count(int n, const int *Si, const int *Sj, const int *CF, int *cnt, cudaStream_t s)
{
   k_dir_count<<<gb_blocks(n, 256), 256, 0, s>>>(n, Si, Sj, CF, cnt);
   GB_COUNT(1);
}

extern "C" void gb_dir_fill(int n, const int *Ai, const int *Aj, const double *Av, const int *Si, const int *Sj,
                            const int *CF, const int *f2c, const int *Pi, int *Pj, double *Pv, double *alfa,
                            double *beta, int *flags, cudaStream_t s)
{
   k_dir_fill<<<gb_blocks(n, 128), 128, 0, s>>>(n, Ai, Aj, Av, Si, Sj, CF, f2c, Pi, Pj, Pv, alfa, beta, flags);
   k_dir_scale<<<gb_blocks(n, 256), 256, 0, s>>>(n, CF, Pi, Pv, alfa, beta, flags);
   GB_COUNT(2);
}

/* number of empty rows (row pointer steps of zero), added into *count */
__global__ void k_count_empty_rows(int n, const int *__restrict__ Ai, int *__restrict__ count)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   int e = (i < n) && (Ai[i + 1] == Ai[i]);
   e = __syncthreads_count(e);
   if (threadIdx.x == 0 && e) { atomicAdd(count, e); }
}

extern "C" void gb_count_empty_rows(int n, const int *Ai, int *count, cudaStream_t s)
{
   if (n > 0)
   {
      k_count_empty_rows<<<gb_blocks(n, 256), 256, 0, s>>>(n, Ai, count);
      GB_COUNT(1);
   }
}

extern "C" void gb_iota(int n, int *out, int *count, cudaStream_t s)
{
   k_iota<<<gb_blocks(n, 256), 256, 0, s>>>(n, out, count);
   GB_COUNT(1);
}

extern "C" void gb_extpi_count_t(int nrows, const int *rows, const int *Si, const int *Sj, const int *CF,
                                 const int *f2c, int *cnt, int *ovf_list, int *ovf_n, cudaStream_t s)
{
   k_extpi_count_t<<<gb_blocks(nrows, GB_TPR_BLOCK), GB_TPR_BLOCK, 0, s>>>(nrows, rows, Si, Sj, CF, f2c, cnt,
                                                                         ovf_list, ovf_n);
   GB_COUNT(1);
}

extern "C" void gb_extpi_fill_t(int nrows, const int *rows, const int *Ai, const int *Aj, const double *Av,
                                const int *Si, const int *Sj, const int *CF, const int *f2c, const int *Pi, int *Pj,
                                double *Pv, int iterm, cudaStream_t s)
{
   k_extpi_fill_t<<<gb_blocks(nrows, GB_TPR_BLOCK), GB_TPR_BLOCK, 0, s>>>(nrows, rows, Ai, Aj, Av, Si, Sj, CF, f2c,
                                                                        Pi, Pj, Pv, iterm);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Truncation (reference: src/parcsr_mv/par_csr_matrix.c:2943-3300, rescale=1,
// infinity norm; hypre_qsort2_abs src/utilities/qsort.c:452-474).
// Works in place on each row, then the rows are compacted.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sw2(int *v, double *w, int a, int b)
{
   int t = v[a]; v[a] = v[b]; v[b] = t;
   double u = w[a]; w[a] = w[b]; w[b] = u;
}

// K&R quicksort by |w| descending (pivot (l+r)/2, strict '>'), iterative.
// Disjoint subranges are independent, so the processing order does not change
// the final arrangement.
__device__ void qsort2_abs_iter(int *v, double *w, int left, int right)
{
   int stl[64], str[64];
   int sp = 0;
   stl[sp] = left; str[sp] = right; sp++;
   while (sp > 0)
   {
      sp--;
      int l = stl[sp], r = str[sp];
      while (l < r)
      {
         sw2(v, w, l, (l + r) / 2);
         int last = l;
         for (int i = l + 1; i <= r; i++) { if (fabs(w[i]) > fabs(w[l])) { sw2(v, w, ++last, i); } }
         sw2(v, w, l, last);
         // ranges [l, last-1] and [last+1, r]: continue with the smaller one
         if (last - l < r - last)
         {
            if (last + 1 < r) { stl[sp] = last + 1; str[sp] = r; sp++; }
            r = last - 1;
         }
         else
         {
            if (l < last - 1) { stl[sp] = l; str[sp] = last - 1; sp++; }
            l = last + 1;
         }
      }
   }
}

__global__ void k_truncate_rows(int n, const int *__restrict__ Pi, int *__restrict__ Pj, double *__restrict__ Pv,
                                double tol, int max_elmts, int *__restrict__ newcnt)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int b = Pi[i], e = Pi[i + 1];
   int len = e - b;
   if (tol > 0)
   {
      double row_nrm = 0;
      for (int k = b; k < e; k++) { double a = fabs(Pv[k]); row_nrm = row_nrm < a ? a : row_nrm; }
      double drop = tol * row_nrm;
      double row_sum = 0, scale = 0;
      int w = b;
      for (int k = b; k < e; k++)
      {
         double v = Pv[k];
         row_sum += v;
         if (!(fabs(v) < drop)) { scale += v; Pv[w] = v; Pj[w] = Pj[k]; w++; }
      }
      if (scale != 0. && scale != row_sum)
      {
         scale = row_sum / scale;
         for (int k = b; k < w; k++) { Pv[k] *= scale; }
      }
      len = w - b;
   }
   if (max_elmts > 0 && max_elmts < len)
   {
      double row_sum = 0;
      for (int k = b; k < b + len; k++) { row_sum += Pv[k]; }
      qsort2_abs_iter(Pj + b, Pv + b, 0, len - 1);
      double scale = 0;
      for (int k = 0; k < max_elmts; k++) { scale += Pv[b + k]; }
      if (scale != 0. && scale != row_sum)
      {
         scale = row_sum / scale;
         for (int k = 0; k < max_elmts; k++) { Pv[b + k] *= scale; }
      }
      len = max_elmts;
   }
   newcnt[i] = len;
}

__global__ void k_compact_rows(int n, const int *__restrict__ Pi, const int *__restrict__ Pj,
                               const double *__restrict__ Pv, const int *__restrict__ Ni, int *__restrict__ Nj,
                               double *__restrict__ Nv)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int b = Pi[i], nb = Ni[i], len = Ni[i + 1] - Ni[i];
   for (int k = 0; k < len; k++) { Nj[nb + k] = Pj[b + k]; Nv[nb + k] = Pv[b + k]; }
}

extern "C" void gb_truncate_rows(int n, const int *Pi, int *Pj, double *Pv, double tol, int max_elmts, int *newcnt,
                                 cudaStream_t s)
{
   k_truncate_rows<<<gb_blocks(n, 128), 128, 0, s>>>(n, Pi, Pj, Pv, tol, max_elmts, newcnt);
   GB_COUNT(1);
}

extern "C" void gb_compact_rows(int n, const int *Pi, const int *Pj, const double *Pv, const int *Ni, int *Nj,
                                double *Nv, cudaStream_t s)
{
   k_compact_rows<<<gb_blocks(n, 128), 128, 0, s>>>(n, Pi, Pj, Pv, Ni, Nj, Nv);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Transpose (reference: hypre_CSRMatrixTransposeHost src/seq_mv/csr_matop.c:1071,
// a counting sort: rows of A^T list A's rows in ascending order).  Scatter with
// atomics, then sort each output row by row index (entries are unique).
// ---------------------------------------------------------------------------
// Lanes of a warp that hit the same column share one atomic (neighbouring
// rows of P share coarse columns); the order within a column is set by the
// sort afterwards.
__global__ void k_tr_count(int nnz, const int *__restrict__ Aj, int *__restrict__ cnt)
{
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   const int lane = threadIdx.x & 31;
   const int c = k < nnz ? Aj[k] : -1 - lane;
   const unsigned m = __match_any_sync(GB_FULL, c);
   if (c >= 0 && lane == __ffs(m) - 1) { atomicAdd(&cnt[c], __popc(m)); }
}

__global__ void k_tr_scatter(int nr, const int *__restrict__ Ai, const int *__restrict__ Aj,
                             const double *__restrict__ Av, int *__restrict__ fill, int *__restrict__ Tj,
                             double *__restrict__ Tv)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   const int lane = threadIdx.x & 31;
   const unsigned lt = (1u << lane) - 1u;
   int k = 0, e = 0;
   if (r < nr) { k = Ai[r]; e = Ai[r + 1]; }
   while (__any_sync(GB_FULL, k < e))
   {
      const bool act = k < e;
      const int c = act ? Aj[k] : -1 - lane;
      const unsigned m = __match_any_sync(GB_FULL, c);
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (act && lane == leader) { base = atomicAdd(&fill[c], __popc(m)); }
      base = __shfl_sync(GB_FULL, base, leader);
      if (act)
      {
         const int p = base + __popc(m & lt);
         Tj[p] = r;
         if (Av) { Tv[p] = Av[k]; }
         k++;
      }
   }
}

__global__ void k_tr_sort(int nc, const int *__restrict__ Ti, int *__restrict__ Tj, double *__restrict__ Tv,
                          int minlen)
{
   // shell sort of one row by a thread (rows of at least minlen entries
   // are left to the block sort)
   int c = blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= nc) { return; }
   int b = Ti[c], e = Ti[c + 1];
   int len = e - b;
   if (len >= minlen && len <= 2048) { return; }
   for (int gap = len / 2; gap > 0; gap /= 2)
   {
      for (int x = b + gap; x < e; x++)
      {
         int kj = Tj[x];
         double kv = Tv ? Tv[x] : 0.0;
         int y = x;
         while (y - gap >= b && Tj[y - gap] > kj)
         {
            Tj[y] = Tj[y - gap];
            if (Tv) { Tv[y] = Tv[y - gap]; }
            y -= gap;
         }
         Tj[y] = kj;
         if (Tv) { Tv[y] = kv; }
      }
   }
}

// merge sort of one row (minlen <= len <= 2048) by a 256-thread block.  Runs
// of width w are merged pairwise; an element's place in the merged run is its
// place in its own run plus the number of smaller keys in the partner run (a
// binary search; the keys of a row are distinct).  Keys carry their original
// position (key << 11 | position), so the values move once, at the end.
__global__ void __launch_bounds__(256) k_tr_sort_block(int nc, const int *__restrict__ Ti, int *__restrict__ Tj,
                                                      double *__restrict__ Tv, int minlen)
{
   __shared__ long long buf[2][2048];
   for (int c = blockIdx.x; c < nc; c += gridDim.x)
   {
      const int b = Ti[c], e = Ti[c + 1];
      const int len = e - b;
      if (len < minlen || len > 2048) { continue; }
      double v[8];
#pragma unroll
      for (int q = 0; q < 8; q++)
      {
         const int t = threadIdx.x + 256 * q;
         v[q] = 0.0;
         if (t < len)
         {
            buf[0][t] = ((long long) Tj[b + t] << 11) | t;
            if (Tv) { v[q] = Tv[b + t]; }
         }
      }
      __syncthreads();
      int src = 0;
      for (int lw = 0; (1 << lw) < len; lw++)
      {
         const int w = 1 << lw;
         const long long *in = buf[src];
         long long *out = buf[src ^ 1];
         for (int t = threadIdx.x; t < len; t += 256)
         {
            const long long x = in[t];
            const int run = t >> lw;
            const int start = run << lw;
            const int pstart = (run ^ 1) << lw;
            int rank = 0;
            if (pstart < len)
            {
               int lo = pstart, hi = min(pstart + w, len);
               while (lo < hi)
               {
                  const int mid = (lo + hi) >> 1;
                  if (in[mid] < x) { lo = mid + 1; }
                  else { hi = mid; }
               }
               rank = lo - pstart;
            }
            out[min(start, pstart) + (t - start) + rank] = x;
         }
         __syncthreads();
         src ^= 1;
      }
      // the other buffer is free: stage the values by original position
      double *vs = reinterpret_cast<double *>(buf[src ^ 1]);
      if (Tv)
      {
#pragma unroll
         for (int q = 0; q < 8; q++)
         {
            const int t = threadIdx.x + 256 * q;
            if (t < len) { vs[t] = v[q]; }
         }
      }
      __syncthreads();
      for (int t = threadIdx.x; t < len; t += 256)
      {
         const long long x = buf[src][t];
         Tj[b + t] = (int) (x >> 11);
         if (Tv) { Tv[b + t] = vs[x & 2047]; }
      }
      __syncthreads();
   }
}

extern "C" void gb_transpose_count(int nnz, const int *Aj, int *cnt, cudaStream_t s)
{
   if (nnz > 0) { k_tr_count<<<gb_blocks(nnz, 256), 256, 0, s>>>(nnz, Aj, cnt); GB_COUNT(1); }
}

extern "C" void gb_transpose_fill(int nr, int nc, const int *Ai, const int *Aj, const double *Av, int *fill,
                                  const int *Ti, int *Tj, double *Tv, cudaStream_t s)
{
   k_tr_scatter<<<gb_blocks(nr, 256), 256, 0, s>>>(nr, Ai, Aj, Av, fill, Tj, Tv);
   const int minlen = 64;
   k_tr_sort<<<gb_blocks(nc, 128), 128, 0, s>>>(nc, Ti, Tj, Tv, minlen);
   int nb = nc < 4096 ? (nc > 0 ? nc : 1) : 4096;
   k_tr_sort_block<<<nb, 256, 0, s>>>(nc, Ti, Tj, Tv, minlen);
   GB_COUNT(3);
}

// ---------------------------------------------------------------------------
// Ordered sparse product C = A B (reference: hypre_ParMatmul
// src/parcsr_mv/par_csr_matop.c:348, one process): row i lists columns in
// the order a loop over A's row and then B's rows first meets them; the first
// contribution is stored, later ones added; a square product starts each row
// with its diagonal (value 0, then accumulated).  The Galerkin product of
// hypre_BoomerAMGBuildCoarseOperatorKT (src/parcsr_ls/par_rap.c:30) is the
// same two products: RA = P^T A (rectangular), then A_c = RA P (square), so
// it is computed with this kernel twice.
//
// One warp per row.  When B's rows are short (at most W <= 32 entries, W a
// power of two) each warp step covers 32/W consecutive entries of A's row,
// lane groups of W lanes each reading one B row; keys repeated within a step
// are merged in lane order (the sequential order), the group leader adding
// the other members' products one by one.  Longer B rows are walked one A
// entry at a time in chunks of 32.
// Tiers: shared-memory tables first, overflowing rows rebuilt with global
// tables.
// ---------------------------------------------------------------------------
// Tiers of the ordered sparse product, by the row's number of distinct
// output columns: MODE 0 every row, compact 1024-slot tables in shared memory
// (rows up to 768 columns, 4 warps per block, 6 KB per warp); MODE 1 the rows MODE 0 could not hold (list in ovf_list),
// compact 2048-slot tables in shared memory (rows up to 1536 columns, 4 warps
// per block, 12 KB per warp); MODE 2 the
// rows MODE 1 could not hold (list in ovf_list), tables in global memory.
// The symbolic pass of MODE 0 / MODE 1 appends the rows it cannot hold to
// ovf_list / out_list; the numeric pass of MODE 0 / 1 skips rows longer than
// its list capacity.
#define GB_BIG_CAP 2048
#define GB_BIG_WARPS 4
#define GB_BIG_BYTES (GB_BIG_WARPS * GB_TABC_BYTES(GB_BIG_CAP))

// tier 0: compact 1024-slot tables (6 KB per warp, rows up to 768 columns)
#define GB_SMALL_BYTES (GB_SMEM_WARPS * GB_TABC_BYTES(GB_SMEM_CAP))

// numeric tier 3: rows of at most 192 columns, 256-slot compact tables with
// the row's FP64 values in shared memory beside them (3 KB per warp)
#define GB_TINY_CAP 256
#define GB_TINY_LCAP (GB_TINY_CAP / 4 * 3)
#define GB_TINY_WBYTES (GB_TABC_BYTES(GB_TINY_CAP) + GB_TINY_LCAP * 8)
#define GB_TINY_BYTES (GB_SMEM_WARPS * GB_TINY_WBYTES)
static_assert(GB_TINY_LCAP == GB_SPGEMM_TINY_COLS, "tier-3 capacity known to the host");

template <int MODE> struct SpgemmTab { typedef GbTabC type; };
template <> struct SpgemmTab<2> { typedef GbTab type; };

template <int MODE>
__device__ __forceinline__ typename SpgemmTab<MODE>::type spgemm_tab(int *sh, int *gtab, int gcap, int warp)
{
   if constexpr (MODE == 1) { return gb_tabc_at((char *) sh + (threadIdx.x >> 5) * GB_TABC_BYTES(GB_BIG_CAP), GB_BIG_CAP); }
   else if constexpr (MODE == 2) { return gb_tab_at(gtab + (size_t) warp * GB_TAB_INTS(gcap), gcap); }
   else if constexpr (MODE == 3) { return gb_tabc_at((char *) sh + (threadIdx.x >> 5) * GB_TINY_WBYTES, GB_TINY_CAP); }
   else { return gb_tabc_at((char *) sh + (threadIdx.x >> 5) * GB_TABC_BYTES(GB_SMEM_CAP), GB_SMEM_CAP); }
}

// FUSED (numeric tiers 0 and 1): one pass instead of count + fill.  Each row
// is written to a temporary area -- at Ci[r] for tier 0 (sized by the row's
// product count, capped by the table), at fbase + t * listcap for the t-th
// listed row of tier 1 -- and its column count and area offset go to cnt[r]
// and src[r]; rows that overflow are listed for the next tier as in the
// symbolic pass (src[r] = -1).  A gather then moves the rows into place.
template <int MODE, bool NUMERIC, bool FUSED = false>
__global__ void __launch_bounds__(128, 8) k_spgemm(int nrows, int square, int W, const int *__restrict__ Ai,
                                                const int *__restrict__ Aj, const double *__restrict__ Av,
                                                const int *__restrict__ Bi, const int *__restrict__ Bj,
                                                const double *__restrict__ Bv, int *__restrict__ cnt,
                                                const int *__restrict__ Ci, int *__restrict__ Cj,
                                                double *__restrict__ Cv, int *ovf_list, int *ovf_n, int *out_list,
                                                int *out_n, int *gtab, int gcap, int *err, const int *__restrict__ ub,
                                                int *__restrict__ src, int fbase)
{
   constexpr bool COUNTING = !NUMERIC || FUSED;
   extern __shared__ __align__(16) int sh[];
   __shared__ double stage_all[128];
   const int lane = gb_lane();
   double *stage = stage_all + (threadIdx.x & ~31);
   int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   int nwarps = (gridDim.x * blockDim.x) >> 5;
   typename SpgemmTab<MODE>::type T = spgemm_tab<MODE>(sh, gtab, gcap, warp);
   if (MODE != 2) { gb_tab_init(T); }
   // tier 3 keeps the row's values in shared memory behind its table
   double *vals = MODE == 3 ? (double *) ((char *) sh + (threadIdx.x >> 5) * GB_TINY_WBYTES +
                                          GB_TABC_BYTES(GB_TINY_CAP))
                            : nullptr;
   constexpr bool LISTED = MODE == 1 || MODE == 2;
   int total = LISTED ? *ovf_n : nrows;
   for (int t = warp; t < total; t += nwarps)
   {
      int r = LISTED ? ovf_list[t] : t;
      int off = 0;
      if (MODE == 0 && COUNTING && ub && ub[r] > 16 * T.listcap)
      {
         // far more products than the table holds (at most 16 per distinct
         // column on average would be needed to fit): straight to the next tier
         if (lane == 0)
         {
            ovf_list[atomicAdd(ovf_n, 1)] = r;
            cnt[r] = 0;
            if (FUSED) { src[r] = -1; }
         }
         continue;
      }
      if (FUSED) { off = MODE == 0 ? Ci[r] : fbase + t * T.listcap; }
      else if (NUMERIC)
      {
         off = Ci[r];
         const int len = Ci[r + 1] - off;
         if (MODE != 2 && len > T.listcap) { continue; }
         // W > 0: rows of at most W columns were done by tier 3
         if (MODE == 0 && W > 0 && len <= W) { continue; }
      }
      int count = 0, ovf = 0;
      bool created;
      if (square)
      {
         int pos = gb_winsert(T, count, r, lane == 0, created, ovf);
         if (NUMERIC && lane == 0 && pos >= 0)
         {
            Cj[off + pos] = r;
            if (MODE == 3) { vals[pos] = 0.0; }
            else { Cv[off + pos] = 0.0; }
         }
         __syncwarp();
      }
      // The row's products a_rk b_kc in sequential order (A entries in
      // order, each B row in order), 32 per step: lane l takes the l-th
      // product after the cursor (entry ka, from its first unused B entry).
      int ka = Ai[r];
      const int ka1 = Ai[r + 1];
      // window: lane i holds entry ka + i -- its remaining products (len),
      // next B index (kb0) and A value; refilled only as entries are used up
      int len = 0, kb0 = 0;
      double av = 0.0;
      if (ka + lane < ka1)
      {
         const int k = Aj[ka + lane];
         kb0 = Bi[k];
         len = Bi[k + 1] - kb0;
         if (NUMERIC) { av = Av[ka + lane]; }
      }
      // maps lane l to its product in the window (inclusive prefix pre over
      // the entries' remaining lengths) and loads its column and B value
      auto map_step = [&](int &pre, int &total, int &col, double &bval, double &aval) {
         pre = len;
         for (int o = 1; o < 32; o <<= 1)
         {
            int y = __shfl_up_sync(GB_FULL, pre, o);
            if (lane >= o) { pre += y; }
         }
         total = __shfl_sync(GB_FULL, pre, 31);
         // entry j of lane's product l = lane: smallest j with pre_j > l
         int lo = 0, hi = 31;
         for (int it = 0; it < 5; it++)
         {
            int mid = (lo + hi) >> 1;
            int pm = __shfl_sync(GB_FULL, pre, mid);
            if (pm > lane) { hi = mid; } else { lo = mid + 1; }
         }
         const int j = lo;
         const int prej = __shfl_sync(GB_FULL, pre, j > 0 ? j - 1 : 0);
         const int kbj = __shfl_sync(GB_FULL, kb0, j);
         aval = NUMERIC ? __shfl_sync(GB_FULL, av, j) : 0.0;
         col = -1;
         bval = 0.0;
         if (lane < total)
         {
            const int kb = kbj + (lane - (j > 0 ? prej : 0));
            col = Bj[kb];
            if (NUMERIC) { bval = Bv[kb]; }
         }
      };
      // drops the products of the step just mapped: the nfull used-up
      // entries leave, the window shifts down and loads the entries that enter
      auto advance = [&](int pre, int total) {
         const int consumed = total < 32 ? total : 32;
         const int nfull = __popc(__ballot_sync(GB_FULL, pre <= consumed));
         if (nfull == 0)
         {
            if (lane == 0) { kb0 += consumed; len -= consumed; }
         }
         else
         {
            const int used = consumed - __shfl_sync(GB_FULL, pre, nfull - 1);   // of entry ka + nfull
            ka += nfull;
            if (nfull < 32)
            {
               len = __shfl_down_sync(GB_FULL, len, nfull);
               kb0 = __shfl_down_sync(GB_FULL, kb0, nfull);
               if (NUMERIC) { av = __shfl_down_sync(GB_FULL, av, nfull); }
            }
            if (lane >= 32 - nfull)
            {
               len = 0;
               if (ka + lane < ka1)
               {
                  const int k = Aj[ka + lane];
                  kb0 = Bi[k];
                  len = Bi[k + 1] - kb0;
                  if (NUMERIC) { av = Av[ka + lane]; }
               }
            }
            if (lane == 0) { kb0 += used; len -= used; }
         }
      };
      int pre = 0, total = 0, col = -1;
      double bval = 0.0, aval = 0.0;
      if (ka < ka1) { map_step(pre, total, col, bval, aval); }
      while (ka < ka1 && !ovf)
      {
         const bool act = lane < total;
         const int ccol = col;
         const double v = aval * bval;
         // map and load the next step before inserting this one
         advance(pre, total);
         if (ka < ka1) { map_step(pre, total, col, bval, aval); }
         if (!NUMERIC)
         {
            gb_wcount(T, count, ccol, act, ovf);
         }
         else
         {
            // lanes with the same column form a group; its first lane finds
            // or inserts the column (new columns numbered in lane order, the
            // order of first discovery) and adds the group's terms in lane
            // order to the row's value
            const unsigned grp = __match_any_sync(GB_FULL, act ? ccol : -(lane + 2));
            const int leader = __ffs(grp) - 1;
            const bool lead = act && lane == leader;
            int pos = lead ? gb_tfind(T, ccol) : -1;
            const bool need = lead && pos < 0;
            const unsigned nm = __ballot_sync(GB_FULL, need);
            bool bad = false, created = false;
            if (need)
            {
               const int p = count + __popc(nm & ((1u << lane) - 1u));
               if (p < T.listcap && gb_tinsert(T, ccol, p)) { pos = p; created = true; }
               else { bad = true; }
            }
            count += __popc(nm);
            if (count > T.listcap) { count = T.listcap; }
            if (__any_sync(GB_FULL, bad)) { ovf = 1; }
            stage[lane] = v;
            __syncwarp();
            if (lead && pos >= 0)
            {
               unsigned rest = grp & (grp - 1u);
               if (MODE == 3)
               {
                  double x;
                  if (created) { Cj[off + pos] = ccol; x = v; }
                  else { x = vals[pos] + v; }
                  while (rest)
                  {
                     int m = __ffs(rest) - 1;
                     rest &= rest - 1u;
                     x += stage[m];
                  }
                  vals[pos] = x;
               }
               else
               {
                  // the first term stored (new column) or added, then the
                  // group's other terms in lane order: fire-and-forget adds
                  // from one thread to one address apply in issue order, and
                  // __syncwarp orders them after the previous steps' adds
                  if (created) { Cj[off + pos] = ccol; Cv[off + pos] = v; }
                  else { atomicAdd(Cv + off + pos, v); }
                  while (rest)
                  {
                     int m = __ffs(rest) - 1;
                     rest &= rest - 1u;
                     atomicAdd(Cv + off + pos, stage[m]);
                  }
               }
            }
            __syncwarp();
         }
      }
      if (MODE == 3 && NUMERIC && !ovf)
      {
         for (int p = lane; p < count; p += 32) { Cv[off + p] = vals[p]; }
         __syncwarp();
      }
      if (lane == 0)
      {
         if (!ovf)
         {
            if (COUNTING) { cnt[r] = count; }
            if (FUSED) { src[r] = off; }
         }
         else if (MODE == 0 && COUNTING)
         {
            ovf_list[atomicAdd(ovf_n, 1)] = r;
            cnt[r] = 0;
            if (FUSED) { src[r] = -1; }
         }
         else if (MODE == 1 && COUNTING)
         {
            out_list[atomicAdd(out_n, 1)] = r;
            cnt[r] = 0;
            if (FUSED) { src[r] = -1; }
         }
         else { atomicExch(err, 1); }
      }
      gb_tab_clear(T, count);
   }
}

// Upper bound of each product row's length: sum over A's row of B row lengths
// (+1 when square), capped by B's column count.
__global__ void k_spgemm_ub(int nrows, int ncols, int square, const int *__restrict__ Ai,
                            const int *__restrict__ Aj, const int *__restrict__ Bi, int *__restrict__ ub)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nrows) { return; }
   long long u = square ? 1 : 0;
   for (int ka = Ai[r]; ka < Ai[r + 1]; ka++) { int k = Aj[ka]; u += Bi[k + 1] - Bi[k]; }
   if (u > ncols) { u = ncols; }
   ub[r] = (int) u;
}

__global__ void k_rowlen_max(int n, const int *__restrict__ Bi, int *__restrict__ out)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   int l = r < n ? Bi[r + 1] - Bi[r] : 0;
   for (int o = 16; o > 0; o >>= 1) { int y = __shfl_down_sync(GB_FULL, l, o); l = y > l ? y : l; }
   if ((threadIdx.x & 31) == 0) { atomicMax(out, l); }
}

extern "C" void gb_rowlen_max(int n, const int *Bi, int *out, cudaStream_t s)
{
   cudaMemsetAsync(out, 0, sizeof(int), s);
   if (n > 0) { k_rowlen_max<<<gb_blocks(n, 256), 256, 0, s>>>(n, Bi, out); GB_COUNT(1); }
}

extern "C" void gb_spgemm_ub(int nrows, int ncols, int square, const int *Ai, const int *Aj, const int *Bi, int *ub,
                             cudaStream_t s)
{
   k_spgemm_ub<<<gb_blocks(nrows, 256), 256, 0, s>>>(nrows, ncols, square, Ai, Aj, Bi, ub);
   GB_COUNT(1);
}

// phase: 0 symbolic, 1 numeric; tier: 0 shared memory (all rows), 1 large shared tables
// (overflow list), 2 global tables (second list), 3 numeric rows of at most GB_TINY_LCAP
// columns with values in shared memory.  W (numeric tier 0): rows of at most W columns
// are skipped (done by tier 3); 0 skips none.
extern "C" void gb_spgemm(int nrows, int square, int W, const int *Ai, const int *Aj, const double *Av,
                          const int *Bi, const int *Bj, const double *Bv, int *cnt, const int *Ci, int *Cj,
                          double *Cv, int *ovf_list, int *ovf_n, int *out_list, int *out_n, int nlist, int *gtab,
                          int gcap, int gwarps, int *err, const int *ub, int *src, int fbase, int phase, int tier,
                          cudaStream_t s)
{
   static int attr_done = 0;
   if (!attr_done)
   {
      /* the tables plus the static staging array exceed the default dynamic
       * shared-memory limit: opt in once */
      cudaFuncSetAttribute(k_spgemm<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_SMALL_BYTES);
      cudaFuncSetAttribute(k_spgemm<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_SMALL_BYTES);
      cudaFuncSetAttribute(k_spgemm<0, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_SMALL_BYTES);
      cudaFuncSetAttribute(k_spgemm<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_BIG_BYTES);
      cudaFuncSetAttribute(k_spgemm<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_BIG_BYTES);
      cudaFuncSetAttribute(k_spgemm<1, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_BIG_BYTES);
      attr_done = 1;
   }
#define GB_SG_ARGS(gt, gc) nrows, square, W, Ai, Aj, Av, Bi, Bj, Bv, cnt, Ci, Cj, Cv, ovf_list, ovf_n, out_list, \
                           out_n, gt, gc, err, ub, src, fbase
   if (tier == 0)
   {
      /* eight blocks of four warps per SM (24 KB of tables each) */
      long long want = ((long long) nrows + GB_SMEM_WARPS - 1) / GB_SMEM_WARPS;
      int blocks = (int) (want < 152 * 8 ? (want > 0 ? want : 1) : 152 * 8);
      if (phase == 0) { k_spgemm<0, false><<<blocks, 128, GB_SMALL_BYTES, s>>>(GB_SG_ARGS(nullptr, 0)); }
      else if (phase == 1) { k_spgemm<0, true><<<blocks, 128, GB_SMALL_BYTES, s>>>(GB_SG_ARGS(nullptr, 0)); }
      else { k_spgemm<0, true, true><<<blocks, 128, GB_SMALL_BYTES, s>>>(GB_SG_ARGS(nullptr, 0)); }
   }
   else if (tier == 3)
   {
      /* numeric only: 3 KB tables per warp, twelve blocks per SM (registers) */
      long long want = ((long long) nrows + GB_SMEM_WARPS - 1) / GB_SMEM_WARPS;
      int blocks = (int) (want < 152 * 12 ? (want > 0 ? want : 1) : 152 * 12);
      k_spgemm<3, true><<<blocks, 128, GB_TINY_BYTES, s>>>(GB_SG_ARGS(nullptr, 0));
   }
   else if (tier == 1)
   {
      /* persistent: four blocks of four warps per SM, grid-stride over the list */
      long long want = ((long long) nlist + GB_BIG_WARPS - 1) / GB_BIG_WARPS;
      int blocks = (int) (want < 152 * 4 ? (want > 0 ? want : 1) : 152 * 4);
      int threads = 32 * GB_BIG_WARPS;
      if (phase == 0) { k_spgemm<1, false><<<blocks, threads, GB_BIG_BYTES, s>>>(GB_SG_ARGS(nullptr, 0)); }
      else if (phase == 1) { k_spgemm<1, true><<<blocks, threads, GB_BIG_BYTES, s>>>(GB_SG_ARGS(nullptr, 0)); }
      else { k_spgemm<1, true, true><<<blocks, threads, GB_BIG_BYTES, s>>>(GB_SG_ARGS(nullptr, 0)); }
   }
   else
   {
      int blocks = (gwarps + 3) / 4;
      if (phase == 0) { k_spgemm<2, false><<<blocks, 128, 0, s>>>(GB_SG_ARGS(gtab, gcap)); }
      else { k_spgemm<2, true><<<blocks, 128, 0, s>>>(GB_SG_ARGS(gtab, gcap)); }
   }
#undef GB_SG_ARGS
   GB_COUNT(1);
}

// temporary areas of the fused products: ub[r] = the row's product count
// (as k_spgemm_ub), cap[r] = min(ub[r], lcap0); *sum accumulates the capped
// sizes, *over counts the rows whose bound exceeds lcap0
__global__ void k_spgemm_cap(int n, int ncols, int square, const int *__restrict__ Ai, const int *__restrict__ Aj,
                             const int *__restrict__ Bi, int lcap0, int *__restrict__ ub, int *__restrict__ cap,
                             unsigned long long *sum, int *over)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   unsigned long long c = 0;
   int o = 0;
   if (r < n)
   {
      long long u = square ? 1 : 0;
      for (int ka = Ai[r]; ka < Ai[r + 1]; ka++) { const int k = Aj[ka]; u += Bi[k + 1] - Bi[k]; }
      if (u > ncols) { u = ncols; }
      ub[r] = (int) u;
      c = (unsigned long long) (u < lcap0 ? u : lcap0);
      o = u > lcap0;
      cap[r] = (int) c;
   }
   for (int d = 16; d > 0; d >>= 1)
   {
      c += __shfl_down_sync(GB_FULL, c, d);
      o += __shfl_down_sync(GB_FULL, o, d);
   }
   if ((threadIdx.x & 31) == 0)
   {
      if (c) { atomicAdd(sum, c); }
      if (o) { atomicAdd(over, o); }
   }
}

extern "C" void gb_spgemm_cap(int n, int ncols, int square, const int *Ai, const int *Aj, const int *Bi, int lcap0,
                              int *ub, int *cap, unsigned long long *sum, int *over, cudaStream_t s)
{
   if (n > 0)
   {
      k_spgemm_cap<<<gb_blocks(n, 256), 256, 0, s>>>(n, ncols, square, Ai, Aj, Bi, lcap0, ub, cap, sum, over);
      GB_COUNT(1);
   }
}

// one warp per row: the row's cnt entries from its temporary area src[r]
// (rows with src[r] < 0 were filled in place by the global-table tier;
// tv NULL: column indices only)
// LPR lanes per row (LPR divides 32): short rows share a warp
template <int LPR>
__global__ void k_spgemm_gather(int n, const int *__restrict__ Ci, const int *__restrict__ src,
                                const int *__restrict__ tj, const double *__restrict__ tv, int *__restrict__ Cj,
                                double *__restrict__ Cv)
{
   const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
   const int r = (int) (g / LPR);
   const int lane = (int) (g % LPR);
   if (r >= n) { return; }
   const int o = src[r];
   if (o < 0) { return; }
   const int d = Ci[r], l = Ci[r + 1] - d;
   for (int q = lane; q < l; q += LPR)
   {
      Cj[d + q] = tj[o + q];
      if (tv) { Cv[d + q] = tv[o + q]; }
   }
}

extern "C" void gb_spgemm_gather(int n, long long nnz, const int *Ci, const int *src, const int *tj, const double *tv,
                                 int *Cj, double *Cv, cudaStream_t s)
{
   if (n <= 0) { return; }
   const long long avg = nnz / n;
   if (avg <= 6)
   {
      k_spgemm_gather<4><<<gb_blocks((long long) n * 4, 256), 256, 0, s>>>(n, Ci, src, tj, tv, Cj, Cv);
   }
   else if (avg <= 12)
   {
      k_spgemm_gather<8><<<gb_blocks((long long) n * 8, 256), 256, 0, s>>>(n, Ci, src, tj, tv, Cj, Cv);
   }
   else if (avg <= 24)
   {
      k_spgemm_gather<16><<<gb_blocks((long long) n * 16, 256), 256, 0, s>>>(n, Ci, src, tj, tv, Cj, Cv);
   }
   else { k_spgemm_gather<32><<<gb_blocks((long long) n * 32, 256), 256, 0, s>>>(n, Ci, src, tj, tv, Cj, Cv); }
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Row-chunk products for B operands with long rows (R*A: A's rows hold tens
// of entries).  A warp step takes one chunk of up to 32 entries of one B
// row; the columns of a B row are distinct, so no two lanes of a step share
// a column and the ordered insertion needs neither lane grouping nor a
// product prefix: new columns take positions in lane order (= product
// order), and each column receives at most one term per step, added in
// product order -- the same positions and sums as the flattened kernel.
// The numeric pass stores a new column's first term and adds later terms
// with fire-and-forget FP64 atomics: a column gets at most one term per step
// and __syncwarp orders one step's memory operations before the next's, so
// the adds to each output entry happen in product order (the sequential sum)
// and no warp waits on them.  Chunk c+1's B entries and the next window of 32
// A entries are loaded while chunk c is inserted.
// MODE 0: 1024-slot tables for all rows; MODE 1: 2048-slot tables for the
// rows listed by MODE 0's symbolic pass.
// ---------------------------------------------------------------------------
template <int MODE, bool NUMERIC> struct RcCfg
{
   static constexpr int CAP = MODE ? GB_BIG_CAP : GB_SMEM_CAP;
   static constexpr int LCAP = CAP / 4 * 3;
   static constexpr int WBYTES = GB_TABC_BYTES(CAP);
   static constexpr int WARPS = 4;
   static constexpr int BYTES = WARPS * WBYTES;
};

// FUSED: one pass into a temporary area, as for k_spgemm
template <int MODE, bool NUMERIC, bool FUSED = false>
__global__ void __launch_bounds__(128, 8) k_spgemm_rc(int nrows, int square, const int *__restrict__ Ai,
                                                   const int *__restrict__ Aj, const double *__restrict__ Av,
                                                   const int *__restrict__ Bi, const int *__restrict__ Bj,
                                                   const double *__restrict__ Bv, int *__restrict__ cnt,
                                                   const int *__restrict__ Ci, int *__restrict__ Cj,
                                                   double *__restrict__ Cv, int *ovf_list, int *ovf_n,
                                                   int *out_list, int *out_n, int *err, const int *__restrict__ ub,
                                                   int *__restrict__ src, int fbase)
{
   constexpr bool COUNTING = !NUMERIC || FUSED;
   typedef RcCfg<MODE, NUMERIC> K;
   extern __shared__ __align__(16) unsigned char shrc[];
   const int lane = gb_lane();
   const unsigned lt = (1u << lane) - 1u;
   unsigned char *mine = shrc + (size_t) (threadIdx.x >> 5) * K::WBYTES;
   GbTabC T = gb_tabc_at((char *) mine, K::CAP);
   gb_tab_init(T);
   const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int nwarps = (gridDim.x * blockDim.x) >> 5;
   const int total = MODE ? *ovf_n : nrows;
   for (int t = warp; t < total; t += nwarps)
   {
      const int r = MODE ? ovf_list[t] : t;
      if (MODE == 0 && COUNTING && ub && ub[r] > 16 * K::LCAP)
      {
         // far more products than the table holds: straight to the next tier
         if (lane == 0)
         {
            ovf_list[atomicAdd(ovf_n, 1)] = r;
            cnt[r] = 0;
            if (FUSED) { src[r] = -1; }
         }
         continue;
      }
      int off = 0;
      if (FUSED) { off = MODE == 0 ? Ci[r] : fbase + t * K::LCAP; }
      else if (NUMERIC)
      {
         off = Ci[r];
         const int len = Ci[r + 1] - off;
         if (len > K::LCAP) { continue; }
         if (MODE == 1 && len <= RcCfg<0, true>::LCAP) { continue; }   // done by MODE 0
      }
      int count = 0, ovf = 0;
      if (square)
      {
         if (lane == 0)
         {
            gb_tabc_insert(T, r, 0);
            if (NUMERIC) { Cv[off] = 0.0; Cj[off] = r; }
         }
         count = 1;
         __syncwarp();
      }
      const int ka1 = Ai[r + 1];
      int wb = Ai[r];
      // window registers: lane l holds entry wb + l (cur) and wb + 32 + l (nxt)
      int cb0 = 0, cb1 = 0, nb0 = 0, nb1 = 0;
      double ca = 0.0, na = 0.0;
      {
         const int e = wb + lane;
         if (e < ka1) { const int k = Aj[e]; cb0 = Bi[k]; cb1 = Bi[k + 1]; if (NUMERIC) { ca = Av[e]; } }
         const int e2 = e + 32;
         if (e2 < ka1) { const int k = Aj[e2]; nb0 = Bi[k]; nb1 = Bi[k + 1]; if (NUMERIC) { na = Av[e2]; } }
      }
      int q = 0;
      int base = __shfl_sync(GB_FULL, cb0, 0), end = __shfl_sync(GB_FULL, cb1, 0);
      double aq = NUMERIC ? __shfl_sync(GB_FULL, ca, 0) : 0.0;
      int col = -1;
      double bv = 0.0;
      {
         const int kb = base + lane;
         if (kb < end) { col = Bj[kb]; if (NUMERIC) { bv = Bv[kb]; } }
      }
      while (wb + q < ka1 && !ovf)
      {
         // descriptor and loads of the next chunk
         int nbase = base + 32, nend = end, nq = q;
         double naq = aq;
         if (nbase >= nend)
         {
            nq = q + 1;
            if (nq < 32)
            {
               nbase = __shfl_sync(GB_FULL, cb0, nq);
               nend = __shfl_sync(GB_FULL, cb1, nq);
               if (NUMERIC) { naq = __shfl_sync(GB_FULL, ca, nq); }
            }
            else
            {
               nbase = __shfl_sync(GB_FULL, nb0, 0);
               nend = __shfl_sync(GB_FULL, nb1, 0);
               if (NUMERIC) { naq = __shfl_sync(GB_FULL, na, 0); }
            }
         }
         int ncol = -1;
         double nbv = 0.0;
         {
            const int kb = nbase + lane;
            if (kb < nend) { ncol = Bj[kb]; if (NUMERIC) { nbv = Bv[kb]; } }
         }
         // insert the current chunk
         const bool act = col >= 0;
         if (!NUMERIC) { gb_wcount(T, count, col, act, ovf); }
         else
         {
            const double v = aq * bv;
            int pos = act ? gb_tabc_find(T, col) : -1;
            const bool need = act && pos < 0;
            const unsigned nm = __ballot_sync(GB_FULL, need);
            bool bad = false;
            if (need)
            {
               const int p = count + __popc(nm & lt);
               if (p < K::LCAP && gb_tabc_insert(T, col, p) >= 0) { Cv[off + p] = v; Cj[off + p] = col; }
               else { bad = true; }
            }
            else if (act) { atomicAdd(Cv + off + pos, v); }
            count += __popc(nm);
            if (__any_sync(GB_FULL, bad)) { ovf = 1; }
            __syncwarp();
         }
         // advance
         base = nbase; end = nend; aq = naq; col = ncol; bv = nbv;
         if (nq == 32)
         {
            q = 0;
            wb += 32;
            cb0 = nb0; cb1 = nb1; ca = na;
            nb0 = nb1 = 0; na = 0.0;
            const int e2 = wb + 32 + lane;
            if (e2 < ka1) { const int k = Aj[e2]; nb0 = Bi[k]; nb1 = Bi[k + 1]; if (NUMERIC) { na = Av[e2]; } }
         }
         else { q = nq; }
      }
      if (lane == 0)
      {
         if (!ovf)
         {
            if (COUNTING) { cnt[r] = count; }
            if (FUSED) { src[r] = off; }
         }
         else if (MODE == 0 && COUNTING)
         {
            ovf_list[atomicAdd(ovf_n, 1)] = r;
            cnt[r] = 0;
            if (FUSED) { src[r] = -1; }
         }
         else if (MODE == 1 && COUNTING)
         {
            out_list[atomicAdd(out_n, 1)] = r;
            cnt[r] = 0;
            if (FUSED) { src[r] = -1; }
         }
         else { atomicExch(err, 1); }
      }
      gb_tab_clear(T, count);
   }
}

// phase: 0 symbolic, 1 numeric; tier 0 (all rows) or 1 (listed rows)
extern "C" void gb_spgemm_rc(int nrows, int square, const int *Ai, const int *Aj, const double *Av, const int *Bi,
                             const int *Bj, const double *Bv, int *cnt, const int *Ci, int *Cj, double *Cv,
                             int *ovf_list, int *ovf_n, int *out_list, int *out_n, int nlist, int *err,
                             const int *ub, int *src, int fbase, int phase, int tier, cudaStream_t s)
{
   static int attr_done = 0;
   if (!attr_done)
   {
      cudaFuncSetAttribute(k_spgemm_rc<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, RcCfg<0, false>::BYTES);
      cudaFuncSetAttribute(k_spgemm_rc<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, RcCfg<0, true>::BYTES);
      cudaFuncSetAttribute(k_spgemm_rc<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, RcCfg<1, false>::BYTES);
      cudaFuncSetAttribute(k_spgemm_rc<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, RcCfg<1, true>::BYTES);
      cudaFuncSetAttribute(k_spgemm_rc<0, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           RcCfg<0, true>::BYTES);
      cudaFuncSetAttribute(k_spgemm_rc<1, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           RcCfg<1, true>::BYTES);
      attr_done = 1;
   }
   int dev = 0, sms = 152;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   const long long rows = tier == 0 ? nrows : nlist;
   const long long want = (rows + 3) / 4;
   /* resident blocks per SM from the shared memory each one takes (about
    * 227 KB usable per SM) */
   int bytes = tier == 0 ? (phase ? RcCfg<0, true>::BYTES : RcCfg<0, false>::BYTES)
                         : (phase ? RcCfg<1, true>::BYTES : RcCfg<1, false>::BYTES);
   int per_sm = (227 * 1024) / (bytes + 1024);
   if (per_sm < 1) { per_sm = 1; }
   if (per_sm > 16) { per_sm = 16; }
   const long long maxb = (long long) sms * per_sm;
   const int blocks = (int) (want < maxb ? (want > 0 ? want : 1) : maxb);
#define GB_RC_ARGS nrows, square, Ai, Aj, Av, Bi, Bj, Bv, cnt, Ci, Cj, Cv, ovf_list, ovf_n, out_list, out_n, err, ub, \
                   src, fbase
   if (tier == 0)
   {
      if (phase == 0) { k_spgemm_rc<0, false><<<blocks, 128, bytes, s>>>(GB_RC_ARGS); }
      else if (phase == 1) { k_spgemm_rc<0, true><<<blocks, 128, bytes, s>>>(GB_RC_ARGS); }
      else { k_spgemm_rc<0, true, true><<<blocks, 128, bytes, s>>>(GB_RC_ARGS); }
   }
   else
   {
      if (phase == 0) { k_spgemm_rc<1, false><<<blocks, 128, bytes, s>>>(GB_RC_ARGS); }
      else if (phase == 1) { k_spgemm_rc<1, true><<<blocks, 128, bytes, s>>>(GB_RC_ARGS); }
      else { k_spgemm_rc<1, true, true><<<blocks, 128, bytes, s>>>(GB_RC_ARGS); }
   }
#undef GB_RC_ARGS
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// l1 norms (reference: hypre_ParCSRComputeL1Norms src/parcsr_ls/ams.c:517-790)
// option 1: sum_j |a_ij|; option 5: a_ii (0 -> 1); rows with a_ii < 0 negated.
// ---------------------------------------------------------------------------
__global__ void k_l1(int n, const int *__restrict__ Ai, const int *__restrict__ Aj, const double *__restrict__ Av,
                     int option, const int *__restrict__ CF, double *__restrict__ l1)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   double d = 0.0, s = 0.0;
   const int ci = CF ? CF[i] : 0;
   for (int k = Ai[i]; k < Ai[i + 1]; k++)
   {
      double v = Av[k];
      if (Aj[k] == i) { d = v; }
      if (CF && CF[Aj[k]] != ci) { continue; }
      s += fabs(v);
   }
   // option 1: sum |a_ij| (with CF: over the columns of the row's own C/F
   // class, hypre_CSRMatrixComputeRowSumHost src/seq_mv/csr_matop.c:1866);
   // 4 (one process): |a_ii|; 5: a_ii, 0 -> 1
   double r = option == 1 ? s : option == 4 ? fabs(d) : (d != 0.0 ? d : 1.0);
   if (d < 0.0) { r = -r; }
   l1[i] = r;
}

extern "C" void gb_l1_norms(int n, const int *Ai, const int *Aj, const double *Av, int option, const int *CF,
                            double *l1, cudaStream_t s)
{
   k_l1<<<gb_blocks(n, 256), 256, 0, s>>>(n, Ai, Aj, Av, option, CF, l1);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Coarsest grid: dense copy and inverse (Gauss-Jordan without pivoting, as the
// reference's unpivoted elimination hypre_gselim, src/utilities/gselim.h).
// ---------------------------------------------------------------------------
__global__ void k_to_dense(int n, const int *__restrict__ Ai, const int *__restrict__ Aj,
                           const double *__restrict__ Av, double *__restrict__ D)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   for (int j = 0; j < n; j++) { D[(size_t) i * n + j] = 0.0; }
   for (int k = Ai[i]; k < Ai[i + 1]; k++) { D[(size_t) i * n + Aj[k]] = Av[k]; }
}

// One block; D (n x n, row major) is replaced by its inverse, W is n x n work.
// Gauss-Jordan inverse of the n x n row-major D by one thread block (W: n x n
// work); D is replaced by its inverse.
__device__ void gj_block(int n, double *D, double *W)
{
   // W = I
   for (int t = threadIdx.x; t < n * n; t += blockDim.x) { W[t] = (t / n == t % n) ? 1.0 : 0.0; }
   __syncthreads();
   __shared__ double piv;
   for (int k = 0; k < n; k++)
   {
      if (threadIdx.x == 0) { piv = D[(size_t) k * n + k]; }
      __syncthreads();
      if (piv != 0.0)
      {
         double inv = 1.0 / piv;
         for (int j = threadIdx.x; j < n; j += blockDim.x)
         {
            D[(size_t) k * n + j] *= inv;
            W[(size_t) k * n + j] *= inv;
         }
         __syncthreads();
         for (int t = threadIdx.x; t < n * n; t += blockDim.x)
         {
            int r = t / n, j = t % n;
            if (r == k) { continue; }
            double f = D[(size_t) r * n + k];
            if (j == k) { continue; }
            if (f != 0.0)
            {
               D[(size_t) r * n + j] -= f * D[(size_t) k * n + j];
               W[(size_t) r * n + j] -= f * W[(size_t) k * n + j];
            }
         }
         __syncthreads();
         // column k: D[r][k] -= f * D[k][k] (=1) -> 0, and W column k
         for (int r = threadIdx.x; r < n; r += blockDim.x)
         {
            if (r == k) { continue; }
            double f = D[(size_t) r * n + k];
            if (f != 0.0)
            {
               W[(size_t) r * n + k] -= f * W[(size_t) k * n + k];
               D[(size_t) r * n + k] = 0.0;
            }
         }
      }
      __syncthreads();
   }
   for (int t = threadIdx.x; t < n * n; t += blockDim.x) { D[t] = W[t]; }
   __syncthreads();
}

__global__ void k_gauss_jordan(int n, double *D, double *W) { gj_block(n, D, W); }

// Inverse of each diagonal block rows off[s]..off[s+1]-1 of a block-diagonal
// CSR matrix (one thread block per system), stored at D + doff[s] (m x m).
__global__ void k_block_inverse(int nsys, const int *__restrict__ off, const int *__restrict__ Ai,
                                const int *__restrict__ Aj, const double *__restrict__ Av,
                                const long long *__restrict__ doff, double *D, double *W)
{
   for (int sys = blockIdx.x; sys < nsys; sys += gridDim.x)
   {
      const int a = off[sys], m = off[sys + 1] - a;
      double *Ds = D + doff[sys], *Ws = W + doff[sys];
      for (int t = threadIdx.x; t < m * m; t += blockDim.x) { Ds[t] = 0.0; }
      __syncthreads();
      for (int r = threadIdx.x; r < m; r += blockDim.x)
      {
         for (int k = Ai[a + r]; k < Ai[a + r + 1]; k++)
         {
            int c = Aj[k] - a;
            if (c >= 0 && c < m) { Ds[(size_t) r * m + c] = Av[k]; }
         }
      }
      __syncthreads();
      if (m > 0) { gj_block(m, Ds, Ws); }
   }
}

extern "C" void gb_block_inverse(int nsys, const int *off, const int *Ai, const int *Aj, const double *Av,
                                 const long long *doff, double *D, double *W, cudaStream_t s)
{
   int grid = nsys < 152 * 8 ? (nsys > 0 ? nsys : 1) : 152 * 8;
   k_block_inverse<<<grid, 256, 0, s>>>(nsys, off, Ai, Aj, Av, doff, D, W);
   GB_COUNT(1);
}

extern "C" void gb_dense_inverse(int n, const int *Ai, const int *Aj, const double *Av, double *D, double *W,
                                 cudaStream_t s)
{
   k_to_dense<<<gb_blocks(n, 128), 128, 0, s>>>(n, Ai, Aj, Av, D);
   k_gauss_jordan<<<1, 1024, 0, s>>>(n, D, W);
   GB_COUNT(2);
}
