// Aggressive-coarsening kernels for sm_103a (agg_interp_type 6): second-order
// strength between C points, C/F marker corrections, the F/C blocks of A and
// the scalings of the modified extended+i interpolation, and the assembly of
// P1 = [I; W].  Results are identical to the reference's serial loops
// (compiled with --fmad=false like the other setup kernels).
#include "gb_device.cuh"
#include "gb_kernels.h"

#define C_PT 1
#define F_PT -1
#define SF_PT -3

static int gb_blocks2(long long n, int t) { long long b = (n + t - 1) / t; return (int) (b < 1 ? 1 : b); }

__global__ void k_flag_pos(int n, const int *__restrict__ CF, int *__restrict__ flag)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { flag[i] = CF[i] > 0; }
}
__global__ void k_flag_eq(int n, const int *__restrict__ CF, int v, int *__restrict__ flag)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { flag[i] = CF[i] == v; }
}
__global__ void k_flag_nonpos(int n, const int *__restrict__ CF, int *__restrict__ flag)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { flag[i] = CF[i] <= 0; }
}
__global__ void k_flag_pos_or(int n, const int *__restrict__ CF, int v, int *__restrict__ flag)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) { flag[i] = CF[i] > 0 || CF[i] == v; }
}
// inverse of a scanned flag: list[scan[i]] = i where flag[i]
__global__ void k_scatter_list(int n, const int *__restrict__ flag, const int *__restrict__ scan, int *__restrict__ list)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && flag[i]) { list[scan[i]] = i; }
}

// flag[list[t]] = 1 for the distinct entries of a row list: nlist of them,
// or *dcount when given (at most nlist)
__global__ void k_list_flags(int nlist, const int *__restrict__ dcount, const int *__restrict__ list,
                             int *__restrict__ flag)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   const int m = dcount ? *dcount : nlist;
   if (t < m) { flag[list[t]] = 1; }
}

extern "C" void gb_list_flags(int nlist, const int *dcount, const int *list, int *flag, cudaStream_t s)
{
   if (nlist <= 0) { return; }
   k_list_flags<<<gb_blocks2(nlist, 256), 256, 0, s>>>(nlist, dcount, list, flag);
   GB_COUNT(1);
}

extern "C" void gb_flags(int n, const int *CF, int kind, int v, int *flag, cudaStream_t s)
{
   // kind 0: CF > 0 ; 1: CF == v ; 2: CF <= 0 ; 3: CF > 0 or CF == v
   if (kind == 0) { k_flag_pos<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF, flag); }
   else if (kind == 1) { k_flag_eq<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF, v, flag); }
   else if (kind == 3) { k_flag_pos_or<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF, v, flag); }
   else { k_flag_nonpos<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF, flag); }
   GB_COUNT(1);
}

extern "C" void gb_scatter_list(int n, const int *flag, const int *scan, int *list, cudaStream_t s)
{
   k_scatter_list<<<gb_blocks2(n, 256), 256, 0, s>>>(n, flag, scan, list);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Second-order strength (reference: hypre_BoomerAMGCreate2ndSHost
// src/parcsr_ls/par_strength.c:1795-3030, num_paths = 1).  Row ic is the
// ic-th C point i1; its columns are, in discovery order, the coarse indices of
// C neighbours i2 of i1 in S and of C points i3 != i1 in S_i2 for every
// neighbour i2.  Shared-memory tables, global tables for overflowing rows.
//
// Each point's part of that sequence is fixed: its own coarse index when it
// is a C point, then the coarse indices of the C points of its S row.  These
// lists (Li, Lj) are built once, so a row's candidates are the concatenation
// of the lists of i1's strong neighbours (the row's own index skipped), taken
// 32 per warp step across list boundaries -- about 3 steps per row of a
// 27-point operator instead of one step per strong neighbour.
// ---------------------------------------------------------------------------
__global__ void k_s2_lists_count(int n, const int *__restrict__ Si, const int *__restrict__ Sj,
                                 const int *__restrict__ CF, int *__restrict__ cnt)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int c = CF[i] > 0;
   for (int k = Si[i]; k < Si[i + 1]; k++) { c += CF[Sj[k]] > 0; }
   cnt[i] = c;
}

__global__ void k_s2_lists_fill(int n, const int *__restrict__ Si, const int *__restrict__ Sj,
                                const int *__restrict__ CF, const int *__restrict__ f2c, const int *__restrict__ Li,
                                int *__restrict__ Lj)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int p = Li[i];
   if (CF[i] > 0) { Lj[p++] = f2c[i]; }
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      const int i3 = Sj[k];
      if (CF[i3] > 0) { Lj[p++] = f2c[i3]; }
   }
}

extern "C" void gb_s2_lists(int n, const int *Si, const int *Sj, const int *CF, const int *f2c, int *cnt,
                            const int *Li, int *Lj, cudaStream_t s)
{
   if (n <= 0) { return; }
   if (!Lj) { k_s2_lists_count<<<gb_blocks2(n, 256), 256, 0, s>>>(n, Si, Sj, CF, cnt); }
   else { k_s2_lists_fill<<<gb_blocks2(n, 256), 256, 0, s>>>(n, Si, Sj, CF, f2c, Li, Lj); }
   GB_COUNT(1);
}

// FUSED (shared-memory tier): count and fill in one pass, each row into a
// temporary area at S2i[ic] (sized by its upper bound, capped by the table);
// the count goes to cnt[ic] and the area to src[ic] (-1 for rows listed for
// the global tier), and a gather then moves the rows into place.
template <bool GLOBAL, bool FILL, bool FUSED = false>
__global__ void __launch_bounds__(128) k_s2(int nc, const int *__restrict__ c2f, const int *__restrict__ Li,
                                            const int *__restrict__ Lj, const int *__restrict__ Si,
                                            const int *__restrict__ Sj, int *__restrict__ cnt,
                                            const int *__restrict__ S2i, int *__restrict__ S2j, int *ovf_list,
                                            int *ovf_n, int *gtab, int gcap, int *err, int *__restrict__ src)
{
   constexpr bool COUNTING = !FILL || FUSED;
   extern __shared__ __align__(16) int sh[];
   const int lane = gb_lane();
   int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   int nwarps = (gridDim.x * blockDim.x) >> 5;
   auto T = gb_tier_tab<GLOBAL>(sh, gtab, gcap, warp);
   if (!GLOBAL) { gb_tab_init(T); }
   int total = GLOBAL ? *ovf_n : nc;
   for (int t = warp; t < total; t += nwarps)
   {
      int ic = GLOBAL ? ovf_list[t] : t;
      int off = 0;
      if (FUSED) { off = S2i[ic]; }
      else if (FILL)
      {
         off = S2i[ic];
         if (!GLOBAL && S2i[ic + 1] - off > T.listcap) { continue; }
      }
      const int i1 = c2f[ic];
      int count = 0, ovf = 0;
      bool created;
      // window: lane q holds strong neighbour ka + q of i1 -- the unused
      // part of its list (next index kb0, remaining length len)
      int ka = Si[i1];
      const int ka1 = Si[i1 + 1];
      int len = 0, kb0 = 0;
      if (ka + lane < ka1)
      {
         const int i2 = Sj[ka + lane];
         kb0 = Li[i2];
         len = Li[i2 + 1] - kb0;
      }
      while (ka < ka1 && !ovf)
      {
         // lane l takes candidate l after the cursor: inclusive prefix over
         // the window's lengths, then the entry whose prefix first exceeds l
         int pre = len;
         for (int o = 1; o < 32; o <<= 1)
         {
            const int y = __shfl_up_sync(GB_FULL, pre, o);
            if (lane >= o) { pre += y; }
         }
         const int avail = __shfl_sync(GB_FULL, pre, 31);
         int lo = 0, hi = 31;
         for (int it = 0; it < 5; it++)
         {
            const int mid = (lo + hi) >> 1;
            if (__shfl_sync(GB_FULL, pre, mid) > lane) { hi = mid; }
            else { lo = mid + 1; }
         }
         const int prej = __shfl_sync(GB_FULL, pre, lo > 0 ? lo - 1 : 0);
         const int kbj = __shfl_sync(GB_FULL, kb0, lo);
         int idx = -1;
         if (lane < avail) { idx = Lj[kbj + lane - (lo > 0 ? prej : 0)]; }
         const bool act = lane < avail && idx != ic;
         if (FILL)
         {
            int pos = gb_winsert(T, count, idx, act, created, ovf);
            if (created && pos >= 0) { S2j[off + pos] = idx; }
         }
         else { gb_wcount(T, count, idx, act, ovf); }
         // drop the candidates just taken: used-up entries leave the window,
         // which shifts down and loads the entries that enter
         const int consumed = avail < 32 ? avail : 32;
         const int nfull = __popc(__ballot_sync(GB_FULL, pre <= consumed));
         if (nfull == 0)
         {
            if (lane == 0) { kb0 += consumed; len -= consumed; }
         }
         else
         {
            const int used = consumed - __shfl_sync(GB_FULL, pre, nfull - 1);
            ka += nfull;
            if (nfull < 32)
            {
               len = __shfl_down_sync(GB_FULL, len, nfull);
               kb0 = __shfl_down_sync(GB_FULL, kb0, nfull);
            }
            if (lane >= 32 - nfull)
            {
               len = 0;
               if (ka + lane < ka1)
               {
                  const int i2 = Sj[ka + lane];
                  kb0 = Li[i2];
                  len = Li[i2 + 1] - kb0;
               }
            }
            if (lane == 0) { kb0 += used; len -= used; }
         }
      }
      if (lane == 0)
      {
         if (!ovf)
         {
            if (COUNTING) { cnt[ic] = count; }
            if (FUSED) { src[ic] = off; }
         }
         else if (!GLOBAL && COUNTING)
         {
            ovf_list[atomicAdd(ovf_n, 1)] = ic;
            cnt[ic] = 0;
            if (FUSED) { src[ic] = -1; }
         }
         else { atomicExch(err, 1); }
      }
      gb_tab_clear(T, count);
   }
}

static int smem_blocks(int nrows)
{
   int dev = 0, sms = 148;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   long long want = (nrows + GB_SMEM_WARPS - 1) / GB_SMEM_WARPS;
   long long maxb = (long long) sms * 8;
   return (int) (want < maxb ? (want < 1 ? 1 : want) : maxb);
}

// fill: 0 count, 1 fill (at S2i), 2 count and fill into temporary areas
// (tier 0 only; src receives each row's area)
extern "C" void gb_strength2(int nc, const int *c2f, const int *Li, const int *Lj, const int *Si, const int *Sj,
                             int *cnt, const int *S2i, int *S2j, int *ovf_list, int *ovf_n, int *gtab, int gcap,
                             int gwarps, int *err, int *src, int fill, int tier, cudaStream_t s)
{
#define GB_S2_ARGS(gt, gc) nc, c2f, Li, Lj, Si, Sj, cnt, S2i, S2j, ovf_list, ovf_n, gt, gc, err, src
   if (tier == 0)
   {
      int blocks = smem_blocks(nc);
      if (fill == 0) { k_s2<false, false><<<blocks, 128, GB_SMEMC_BYTES, s>>>(GB_S2_ARGS(nullptr, 0)); }
      else if (fill == 1) { k_s2<false, true><<<blocks, 128, GB_SMEMC_BYTES, s>>>(GB_S2_ARGS(nullptr, 0)); }
      else { k_s2<false, true, true><<<blocks, 128, GB_SMEMC_BYTES, s>>>(GB_S2_ARGS(nullptr, 0)); }
   }
   else
   {
      int blocks = (gwarps + 3) / 4;
      if (!fill) { k_s2<true, false><<<blocks, 128, 0, s>>>(GB_S2_ARGS(gtab, gcap)); }
      else { k_s2<true, true><<<blocks, 128, 0, s>>>(GB_S2_ARGS(gtab, gcap)); }
   }
#undef GB_S2_ARGS
   GB_COUNT(1);
}

// cap[r] = min(ub[r], lcap); *sum accumulates the capped sizes
__global__ void k_cap_sum(int n, const int *__restrict__ ub, int lcap, int *__restrict__ cap, unsigned long long *sum)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   unsigned long long c = 0;
   if (r < n)
   {
      const int u = ub[r];
      c = (unsigned long long) (u < lcap ? u : lcap);
      cap[r] = (int) c;
   }
   for (int d = 16; d > 0; d >>= 1) { c += __shfl_down_sync(0xffffffffu, c, d); }
   if ((threadIdx.x & 31) == 0 && c) { atomicAdd(sum, c); }
}

extern "C" void gb_cap_sum(int n, const int *ub, int lcap, int *cap, unsigned long long *sum, cudaStream_t s)
{
   if (n > 0) { k_cap_sum<<<gb_blocks2(n, 256), 256, 0, s>>>(n, ub, lcap, cap, sum); GB_COUNT(1); }
}

// upper bound of an S2 row: the candidates, sum over i2 in S_i1 of |L_i2|
__global__ void k_s2_ub(int nc, const int *__restrict__ c2f, const int *__restrict__ Si, const int *__restrict__ Sj,
                        const int *__restrict__ Li, int *__restrict__ ub)
{
   int ic = blockIdx.x * blockDim.x + threadIdx.x;
   if (ic >= nc) { return; }
   int i1 = c2f[ic];
   long long u = 0;
   for (int k = Si[i1]; k < Si[i1 + 1]; k++) { int i2 = Sj[k]; u += Li[i2 + 1] - Li[i2]; }
   ub[ic] = (int) (u > nc ? nc : u);
}

extern "C" void gb_strength2_ub(int nc, const int *c2f, const int *Si, const int *Sj, const int *Li, int *ub,
                                cudaStream_t s)
{
   k_s2_ub<<<gb_blocks2(nc, 256), 256, 0, s>>>(nc, c2f, Si, Sj, Li, ub);
   GB_COUNT(1);
}

// C points whose S2 row is empty become CF = 2 (par_strength.c:2701-2723)
__global__ void k_mark_isolated(int nc, const int *__restrict__ c2f, const int *__restrict__ cnt, int *CF)
{
   int ic = blockIdx.x * blockDim.x + threadIdx.x;
   if (ic < nc && cnt[ic] == 0) { CF[c2f[ic]] = 2; }
}

extern "C" void gb_mark_isolated(int nc, const int *c2f, const int *cnt, int *CF, cudaStream_t s)
{
   k_mark_isolated<<<gb_blocks2(nc, 256), 256, 0, s>>>(nc, c2f, cnt, CF);
   GB_COUNT(1);
}

// hypre_BoomerAMGCorrectCFMarker2Host (par_strength.c:3096): C points made F
// by the second coarsening become -2, the others 1.
__global__ void k_correct_cf2(int n, const int *__restrict__ f2c, const int *__restrict__ CFN, int *CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && CF[i] > 0) { CF[i] = CFN[f2c[i]] == -1 ? -2 : 1; }
}

extern "C" void gb_correct_cf2(int n, const int *f2c, const int *CFN, int *CF, cudaStream_t s)
{
   k_correct_cf2<<<gb_blocks2(n, 256), 256, 0, s>>>(n, f2c, CFN, CF);
   GB_COUNT(1);
}

// CF < -1 -> -1 (partial.c:700)
__global__ void k_cf_clamp(int n, int *CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && CF[i] < -1) { CF[i] = -1; }
}

extern "C" void gb_cf_clamp(int n, int *CF, cudaStream_t s)
{
   k_cf_clamp<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// F/C blocks of A on strong connections (hypre_ParCSRMatrixGenerateFFFCHost
// src/parcsr_mv/gen_fffc.c:18-530): for F row r (fine point i = fl[r]):
// FF = [a_ii, strong F neighbours], FC = strong C neighbours, in S's order.
// ---------------------------------------------------------------------------
__global__ void k_fffc_count(int nf, const int *__restrict__ fl, const int *__restrict__ Ai,
                             const int *__restrict__ Aj, const int *__restrict__ Si, const int *__restrict__ Sj,
                             const int *__restrict__ CF, int *__restrict__ cff, int *__restrict__ cfc)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   int i = fl[r];
   int ff = 0, fc = 0;
   if (Ai[i] < Ai[i + 1] && Aj[Ai[i]] == i) { ff++; }
   for (int k = Si[i]; k < Si[i + 1]; k++) { if (CF[Sj[k]] > 0) { fc++; } else { ff++; } }
   cff[r] = ff;
   cfc[r] = fc;
}

template <int LPR>
__global__ void k_fffc_fill(int nf, const int *__restrict__ fl, const int *__restrict__ Ai,
                            const int *__restrict__ Aj, const double *__restrict__ Av, const int *__restrict__ Si,
                            const int *__restrict__ Sj, const int *__restrict__ CF, const int *__restrict__ f2c,
                            const int *__restrict__ f2f, const int *__restrict__ FFi, int *__restrict__ FFj,
                            double *__restrict__ FFv, const int *__restrict__ FCi, int *__restrict__ FCj,
                            double *__restrict__ FCv)
{
   /* LPR lanes per F row (a segment of the warp).  S_i is A_i's
    * off-diagonal columns filtered in order (the reference looks each S
    * entry up in A_i), and A_i's columns are distinct, so an A entry of a
    * chunk of LPR is strong iff its column occurs among the next LPR
    * unmatched S entries; ballot prefixes keep the A order, which is the S
    * order of the sequential fill */
   const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
   const int r = (int) (g / LPR);
   const int lane = (int) (g % LPR);
   if (r >= nf) { return; }   // whole segments leave together
   const int sbase = (threadIdx.x & 31) & ~(LPR - 1);
   const unsigned seg = LPR == 32 ? 0xffffffffu : (((1u << LPR) - 1u) << sbase);
   int i = fl[r];
   int pf = FFi[r], pc = FCi[r];
   int a0 = Ai[i], a1 = Ai[i + 1];
   int hasdiag = (a0 < a1 && Aj[a0] == i);
   if (hasdiag && lane == 0) { FFj[pf] = f2f[i]; FFv[pf] = Av[a0]; }
   pf += hasdiag;
   int s0 = Si[i], s1 = Si[i + 1];
   unsigned lt = (1u << lane) - 1u;
   for (int base = a0 + hasdiag; base < a1 && s0 < s1; base += LPR)
   {
      int p = base + lane;
      int c = (p < a1) ? Aj[p] : -1;
      int ns = min(LPR, s1 - s0);
      int sj = (lane < ns) ? Sj[s0 + lane] : -2;
      bool in = false;
      for (int t = 0; t < ns; t++) { in |= (c == __shfl_sync(seg, sj, t, LPR)); }
      bool isc = in && CF[c] > 0;
      bool isf = in && !isc;
      unsigned bc = __ballot_sync(seg, isc) >> sbase, bf = __ballot_sync(seg, isf) >> sbase;
      if (isc) { int q = pc + __popc(bc & lt); FCj[q] = f2c[c]; FCv[q] = Av[p]; }
      if (isf) { int q = pf + __popc(bf & lt); FFj[q] = f2f[c]; FFv[q] = Av[p]; }
      pc += __popc(bc);
      pf += __popc(bf);
      s0 += __popc(bc | bf);
   }
}

extern "C" void gb_fffc_count(int nf, const int *fl, const int *Ai, const int *Aj, const int *Si, const int *Sj,
                              const int *CF, int *cff, int *cfc, cudaStream_t s)
{
   k_fffc_count<<<gb_blocks2(nf, 256), 256, 0, s>>>(nf, fl, Ai, Aj, Si, Sj, CF, cff, cfc);
   GB_COUNT(1);
}

extern "C" void gb_fffc_fill(int nf, int nrows, long long nnz, const int *fl, const int *Ai, const int *Aj,
                             const double *Av, const int *Si, const int *Sj, const int *CF, const int *f2c,
                             const int *f2f, const int *FFi, int *FFj, double *FFv, const int *FCi, int *FCj,
                             double *FCv, cudaStream_t s)
{
   // lanes per row from the mean row length of A (27-point: 16)
   const long long avg = nf > 0 ? (long long) nnz / (nrows > 0 ? nrows : 1) : 0;
#define GB_FFFC(L)                                                                                                 \
   k_fffc_fill<L><<<gb_blocks2((long long) nf * L, 256), 256, 0, s>>>(nf, fl, Ai, Aj, Av, Si, Sj, CF, f2c, f2f, FFi, \
                                                                      FFj, FFv, FCi, FCj, FCv)
   if (avg <= 10) { GB_FFFC(8); }
   else if (avg <= 40) { GB_FFFC(16); }
   else { GB_FFFC(32); }
#undef GB_FFFC
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Scalings of the modified extended+i interpolation
// (hypre_BoomerAMGBuildModExtPIInterpHost src/parcsr_ls/par_mod_lr_interp.c
// :690-905, one function): D_q (FC row sums), D_w (A row sum minus the strong
// F and C parts), D_theta, the division of FF's off-diagonals and the final
// row scaling -1/(D_theta + D_w).
// ---------------------------------------------------------------------------
__global__ void k_mod_dq_dw(int nf, const int *__restrict__ fl, const int *__restrict__ Ai,
                            const double *__restrict__ Av, const int *__restrict__ FFi,
                            const double *__restrict__ FFv, const int *__restrict__ FCi,
                            const double *__restrict__ FCv, double *__restrict__ Dq, double *__restrict__ Dw)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double q = 0.0;
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { q += FCv[k]; }
   int i = fl[r];
   double w = 0.0;
   for (int k = Ai[i]; k < Ai[i + 1]; k++) { w += Av[k]; }
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { w -= FFv[k]; }
   w -= q;
   Dq[r] = q;
   Dw[r] = w;
}

__global__ void k_mod_theta(int nf, const int *__restrict__ FFi, const int *__restrict__ FFj,
                            double *__restrict__ FFv, const double *__restrict__ tmp, const double *__restrict__ Dq,
                            const double *__restrict__ Dw)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double dt = 0.0;
   for (int j = FFi[r] + 1; j < FFi[r + 1]; j++)
   {
      int jj = FFj[j];
      double value = Dq[jj];
      for (int k = FFi[jj] + 1; k < FFi[jj + 1]; k++)
      {
         if (FFj[k] == r)
         {
            double value1 = tmp[k];
            value += value1;
            dt += FFv[j] * value1 / value;
            break;
         }
      }
      if (value != 0.0) { FFv[j] /= value; }
   }
   FFv[FFi[r]] = 1.0;
   double theta = dt + Dw[r];
   if (theta != 0.0)
   {
      theta = -1.0 / theta;
      for (int j = FFi[r]; j < FFi[r + 1]; j++) { FFv[j] *= theta; }
   }
}

extern "C" void gb_mod_extpi_scale(int nf, int nnzff, const int *fl, const int *Ai, const double *Av,
                                   const int *FFi, const int *FFj, double *FFv, const int *FCi, const double *FCv,
                                   double *tmp, double *Dq, double *Dw, cudaStream_t s)
{
   cudaMemcpyAsync(tmp, FFv, sizeof(double) * (size_t) nnzff, cudaMemcpyDeviceToDevice, s);
   k_mod_dq_dw<<<gb_blocks2(nf, 256), 256, 0, s>>>(nf, fl, Ai, Av, FFi, FFv, FCi, FCv, Dq, Dw);
   k_mod_theta<<<gb_blocks2(nf, 128), 128, 0, s>>>(nf, FFi, FFj, FFv, tmp, Dq, Dw);
   GB_COUNT(2);
}

// Scalings of the modified extended interpolation (interp_type 16,
// hypre_BoomerAMGBuildModExtInterpHost src/parcsr_ls/par_mod_lr_interp.c:
// 229-355): D_q = FC row sum, D_w = A row sum - FF off-diagonals - D_q;
// FF's diagonal becomes D_q / D_w, its off-diagonals are divided by D_w and
// FC is scaled by -1 / D_q (1 when a divisor is zero).
__global__ void k_modext_scale(int nf, const int *__restrict__ fl, const int *__restrict__ Ai,
                               const double *__restrict__ Av, const int *__restrict__ FFi, double *__restrict__ FFv,
                               const int *__restrict__ FCi, double *__restrict__ FCv)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double q = 0.0;
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { q += FCv[k]; }
   int i = fl[r];
   double w = 0.0;
   for (int k = Ai[i]; k < Ai[i + 1]; k++) { w += Av[k]; }
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { w -= FFv[k]; }
   w -= q;
   const double beta = w != 0.0 ? 1.0 / w : 1.0;
   FFv[FFi[r]] = beta * q;
   const double gamma = q != 0.0 ? -1.0 / q : 1.0;
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { FFv[k] *= beta; }
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { FCv[k] *= gamma; }
}

// Scalings of the modified extended+e interpolation (interp_type 18,
// hypre_BoomerAMGBuildModExtPEInterpHost src/parcsr_ls/par_mod_lr_interp.c:
// 1483-1662).  Pass 1 per F row: D_lambda = mean of FF's off-diagonals,
// D_beta = FC row sum, D_tmp = D_lambda / (D_beta + D_lambda), D_w = A row
// sum - FF off-diagonals - D_beta.  Pass 2: D_tau = sum FF_ij D_tmp_j,
// value = -1 / (D_w + D_tau), theta = D_beta + D_lambda; FF's diagonal
// becomes value * theta, its off-diagonals are scaled by value and FC by
// 1 / theta.
__global__ void k_modpe_rows(int nf, const int *__restrict__ fl, const int *__restrict__ Ai,
                             const double *__restrict__ Av, const int *__restrict__ FFi,
                             const double *__restrict__ FFv, const int *__restrict__ FCi,
                             const double *__restrict__ FCv, double *__restrict__ Dl, double *__restrict__ Db,
                             double *__restrict__ Dt, double *__restrict__ Dw)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double lambda = 0.0;
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { lambda += FFv[k]; }
   const double number = (double) (FFi[r + 1] - FFi[r] - 1);
   if (number != 0.0) { lambda /= number; }
   double beta = 0.0;
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { beta += FCv[k]; }
   Dt[r] = lambda + beta != 0.0 ? lambda / (beta + lambda) : 0.0;
   int i = fl[r];
   double w = 0.0;
   for (int k = Ai[i]; k < Ai[i + 1]; k++) { w += Av[k]; }
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { w -= FFv[k]; }
   w -= beta;
   Dl[r] = lambda;
   Db[r] = beta;
   Dw[r] = w;
}

__global__ void k_modpe_scale(int nf, const int *__restrict__ FFi, const int *__restrict__ FFj,
                              double *__restrict__ FFv, const int *__restrict__ FCi, double *__restrict__ FCv,
                              const double *__restrict__ Dl, const double *__restrict__ Db,
                              const double *__restrict__ Dt, const double *__restrict__ Dw)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double tau = 0.0;
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { tau += FFv[k] * Dt[FFj[k]]; }
   double value = Dw[r] + tau;
   if (value != 0.0) { value = -1.0 / value; }
   double theta = Db[r] + Dl[r];
   FFv[FFi[r]] = value * theta;
   if (theta != 0.0) { theta = 1.0 / theta; }
   for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { FFv[k] *= value; }
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { FCv[k] *= theta; }
}

// the row scalings of the modified interpolations 16, 17 and 18 on FF / FC
// (work: tmp nnz(FF), D1..D4 nf each)
extern "C" void gb_mod_interp_scale(int variant, int nf, int nnzff, const int *fl, const int *Ai, const double *Av,
                                    const int *FFi, const int *FFj, double *FFv, const int *FCi, double *FCv,
                                    double *tmp, double *D1, double *D2, double *D3, double *D4, cudaStream_t s)
{
   if (nf <= 0) { return; }
   if (variant == 16)
   {
      k_modext_scale<<<gb_blocks2(nf, 256), 256, 0, s>>>(nf, fl, Ai, Av, FFi, FFv, FCi, FCv);
      GB_COUNT(1);
   }
   else if (variant == 18)
   {
      k_modpe_rows<<<gb_blocks2(nf, 256), 256, 0, s>>>(nf, fl, Ai, Av, FFi, FFv, FCi, FCv, D1, D2, D3, D4);
      k_modpe_scale<<<gb_blocks2(nf, 256), 256, 0, s>>>(nf, FFi, FFj, FFv, FCi, FCv, D1, D2, D3, D4);
      GB_COUNT(2);
   }
   else { gb_mod_extpi_scale(nf, nnzff, fl, Ai, Av, FFi, FFj, FFv, FCi, FCv, tmp, D1, D2, s); }
}

// P1 = [I; W] in fine order: C points get (f2c[i], 1), F points W's row f2f[i]
__global__ void k_p1_len(int n, const int *__restrict__ CF, const int *__restrict__ f2f, const int *__restrict__ Wi,
                         int *__restrict__ len)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   if (CF[i] > 0) { len[i] = 1; }
   else { int r = f2f[i]; len[i] = Wi[r + 1] - Wi[r]; }
}

__global__ void k_p1_fill(int n, const int *__restrict__ CF, const int *__restrict__ f2c, const int *__restrict__ f2f,
                          const int *__restrict__ Wi, const int *__restrict__ Wj, const double *__restrict__ Wv,
                          const int *__restrict__ Pi, int *__restrict__ Pj, double *__restrict__ Pv)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int c = Pi[i];
   if (CF[i] > 0) { Pj[c] = f2c[i]; Pv[c] = 1.0; }
   else
   {
      int r = f2f[i];
      for (int k = Wi[r]; k < Wi[r + 1]; k++) { Pj[c] = Wj[k]; Pv[c] = Wv[k]; c++; }
   }
}

extern "C" void gb_p1_len(int n, const int *CF, const int *f2f, const int *Wi, int *len, cudaStream_t s)
{
   k_p1_len<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF, f2f, Wi, len);
   GB_COUNT(1);
}

extern "C" void gb_p1_fill(int n, const int *CF, const int *f2c, const int *f2f, const int *Wi, const int *Wj,
                           const double *Wv, const int *Pi, int *Pj, double *Pv, cudaStream_t s)
{
   k_p1_fill<<<gb_blocks2(n, 256), 256, 0, s>>>(n, CF, f2c, f2f, Wi, Wj, Wv, Pi, Pj, Pv);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Modified partial interpolations of the second stage on an aggressive level
// (variant 5 extended: hypre_BoomerAMGBuildModPartialExtInterpHost
// src/parcsr_ls/par_2s_interp.c:15-620; variant 7 extended+e:
// hypre_BoomerAMGBuildModPartialExtPEInterpHost :662-1320).  F rows r (every
// non-C point): D_q = FC row sum; variant 7: D_lambda = the mean of the row's
// strong non-C values (FF's off-diagonals over the full F list, as
// hypre_ParCSRMatrixGenerateFFFCD3 src/parcsr_mv/gen_fffc.c:1497-1560 sums
// them) and D_inv = 1 / (D_q + D_lambda), 0 when that is zero.
// ---------------------------------------------------------------------------
__global__ void k_modp_dq(int variant, int nf, const int *__restrict__ FFi, const double *__restrict__ FFv,
                          const int *__restrict__ FCi, const double *__restrict__ FCv, double *__restrict__ Dq,
                          double *__restrict__ Dl, double *__restrict__ Dinv)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double q = 0.0;
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { q += FCv[k]; }
   Dq[r] = q;
   if (variant == 7)
   {
      double l = 0.0, c = 0.0;
      for (int k = FFi[r] + 1; k < FFi[r + 1]; k++) { c += 1; l += FFv[k]; }
      if (c != 0.0) { l = l / c; }
      Dl[r] = l;
      Dinv[r] = q + l != 0.0 ? 1.0 / (q + l) : 0.0;
   }
}

// the CF -2 rows (t-th: point nl[t], F index f2f[nl[t]]) of FF (:261-393,
// :897-1042): D_w = A row sum - the FF off-diagonals whose column has D_q != 0
// (variant 7: D_inv != 0), minus D_q (variant 7: plus D_tau - D_q, D_tau =
// sum FF_ij D_lambda_j D_inv_j); when D_w != 0 the diagonal becomes
// D_q / D_w and the off-diagonals are divided by D_w (variant 7: with
// beta = -1 / D_w, the diagonal beta (D_q + D_lambda), off-diagonals * beta)
__global__ void k_modp_rows(int variant, int nn, const int *__restrict__ nl, const int *__restrict__ f2f,
                            const int *__restrict__ Ai, const double *__restrict__ Av, const int *__restrict__ FFi,
                            const int *__restrict__ FFj, double *__restrict__ FFv, const double *__restrict__ Dq,
                            const double *__restrict__ Dl, const double *__restrict__ Dinv)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= nn) { return; }
   const int i = nl[t], self = f2f[i];
   const int f0 = FFi[t], f1 = FFi[t + 1];
   double w = 0.0;
   if (variant == 7)
   {
      double tau = 0.0;
      for (int k = f0 + 1; k < f1; k++) { const int c = FFj[k]; tau += FFv[k] * Dl[c] * Dinv[c]; }
      for (int k = Ai[i]; k < Ai[i + 1]; k++) { w += Av[k]; }
      for (int k = f0 + 1; k < f1; k++) { if (Dinv[FFj[k]] != 0.0) { w -= FFv[k]; } }
      w += tau - Dq[self];
      if (w != 0.0)
      {
         const double beta = -1.0 / w;
         FFv[f0] = beta * (Dq[self] + Dl[self]);
         for (int k = f0 + 1; k < f1; k++) { FFv[k] *= beta; }
      }
   }
   else
   {
      for (int k = Ai[i]; k < Ai[i + 1]; k++) { w += Av[k]; }
      for (int k = f0 + 1; k < f1; k++) { if (Dq[FFj[k]] != 0.0) { w -= FFv[k]; } }
      w -= Dq[self];
      if (w != 0.0)
      {
         const double beta = 1.0 / w;
         FFv[f0] = beta * Dq[self];
         for (int k = f0 + 1; k < f1; k++) { FFv[k] *= beta; }
      }
   }
}

// FC rows scaled by -1 / D_q (0 when D_q is zero); variant 7 by D_inv
__global__ void k_modp_fc(int variant, int nf, const int *__restrict__ FCi, double *__restrict__ FCv,
                          const double *__restrict__ Dq, const double *__restrict__ Dinv)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nf) { return; }
   double g;
   if (variant == 7) { g = Dinv[r]; }
   else { g = Dq[r] != 0.0 ? -1.0 / Dq[r] : 0.0; }
   for (int k = FCi[r]; k < FCi[r + 1]; k++) { FCv[k] *= g; }
}

extern "C" void gb_modp_scale(int variant, int nf, int nn, const int *nl, const int *f2f, const int *Ai,
                              const double *Av, const int *FFai, const double *FFav, const int *FCi, double *FCv,
                              const int *FFi, const int *FFj, double *FFv, double *Dq, double *Dl, double *Dinv,
                              cudaStream_t s)
{
   if (nf > 0) { k_modp_dq<<<gb_blocks2(nf, 256), 256, 0, s>>>(variant, nf, FFai, FFav, FCi, FCv, Dq, Dl, Dinv); }
   if (nn > 0)
   {
      k_modp_rows<<<gb_blocks2(nn, 128), 128, 0, s>>>(variant, nn, nl, f2f, Ai, Av, FFi, FFj, FFv, Dq, Dl, Dinv);
   }
   if (nf > 0) { k_modp_fc<<<gb_blocks2(nf, 256), 256, 0, s>>>(variant, nf, FCi, FCv, Dq, Dinv); }
   GB_COUNT(3);
}

// P over the old C points (oc, in row order): CF 1 rows the identity (f2c),
// CF -2 rows the row nscan[i] of W
__global__ void k_modp_len(int nco, const int *__restrict__ oc, const int *__restrict__ CF,
                           const int *__restrict__ nscan, const int *__restrict__ Wi, int *__restrict__ len)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nco) { return; }
   const int i = oc[r];
   len[r] = CF[i] > 0 ? 1 : Wi[nscan[i] + 1] - Wi[nscan[i]];
}

__global__ void k_modp_gather(int nco, const int *__restrict__ oc, const int *__restrict__ CF,
                              const int *__restrict__ f2c, const int *__restrict__ nscan, const int *__restrict__ Wi,
                              const int *__restrict__ Wj, const double *__restrict__ Wv, const int *__restrict__ Pi,
                              int *__restrict__ Pj, double *__restrict__ Pv)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= nco) { return; }
   const int i = oc[r], o = Pi[r];
   if (CF[i] > 0)
   {
      Pj[o] = f2c[i];
      Pv[o] = 1.0;
      return;
   }
   const int k0 = Wi[nscan[i]], l = Pi[r + 1] - o;
   for (int q = 0; q < l; q++)
   {
      Pj[o + q] = Wj[k0 + q];
      Pv[o + q] = Wv[k0 + q];
   }
}

extern "C" void gb_modp_len(int nco, const int *oc, const int *CF, const int *nscan, const int *Wi, int *len,
                            cudaStream_t s)
{
   if (nco <= 0) { return; }
   k_modp_len<<<gb_blocks2(nco, 256), 256, 0, s>>>(nco, oc, CF, nscan, Wi, len);
   GB_COUNT(1);
}

extern "C" void gb_modp_gather(int nco, const int *oc, const int *CF, const int *f2c, const int *nscan, const int *Wi,
                               const int *Wj, const double *Wv, const int *Pi, int *Pj, double *Pv, cudaStream_t s)
{
   if (nco <= 0) { return; }
   k_modp_gather<<<gb_blocks2(nco, 256), 256, 0, s>>>(nco, oc, CF, f2c, nscan, Wi, Wj, Wv, Pi, Pj, Pv);
   GB_COUNT(1);
}
