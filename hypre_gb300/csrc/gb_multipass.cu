// Multipass interpolation (agg_interp_type 4, the reference's default on
// aggressive levels), bit for bit the reference's single-process loops
// (hypre_BoomerAMGBuildMultipassHost, src/parcsr_ls/par_multi_interp.c:16-2130,
// default weights: sep_weight 0, :1600-1960), and the C/F marker correction
// after the second coarsening (hypre_BoomerAMGCorrectCFMarkerHost,
// src/parcsr_ls/par_strength.c:3068-3090).
//
// Passes.  C points are pass 0; F points (CF -1) with a strong C neighbour
// are pass 1; pass p takes the F points left that have a strong neighbour of
// pass p-1 (p < 10).  A point's pass is its breadth-first distance from the C
// points in S, so one data-parallel kernel per pass assigns it, whatever order
// the reference's pass_array visits the points in.
//
// Rows.  A pass 1 row holds its strong C neighbours in A order with the
// values a_ij; a pass p row the union of the rows of its strong pass p-1
// neighbours (taken in S order, each row in its own order) with the sums of
// a_ij p_jk over those neighbours j in A order.  sum_C sums the row's terms,
// sum_N the same plus the row's other off-diagonals (CF != -3), and the row is
// scaled by alfa = -sum_N / (sum_C a_ii).  When sum_C a_ii is zero the
// reference keeps alfa from before: in passes >= 2 that is the row's own last
// product; in pass 1 it is the alfa of the previous pass 1 row in the order
// the reference visits them (1.0 before the first), which a one-thread kernel
// replays only when such rows exist.
//
// One thread per row; S is a subsequence of A's off-diagonals in A's order
// (the strength kernel writes it that way), so walking a row of A and of S
// together tells which entries of A are strong.  Compiled with --fmad=false.
#include "gb_device.cuh"
#include "gb_kernels.h"

#define C_PT 1
#define F_PT -1
#define SF_PT -3

static int mp_blocks(long long n, int t) { long long b = (n + t - 1) / t; return (int) (b < 1 ? 1 : b); }

// CF of the C points from the second coarsening (f2c numbers the CF > 0 points)
__global__ void k_correct_cf(int n, const int *__restrict__ f2c, const int *__restrict__ CFN, int *CF)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && CF[i] > 0) { CF[i] = CF[i] == 1 ? CFN[f2c[i]] : 1; }
}

extern "C" void gb_correct_cf(int n, const int *f2c, const int *CFN, int *CF, cudaStream_t s)
{
   k_correct_cf<<<mp_blocks(n, 256), 256, 0, s>>>(n, f2c, CFN, CF);
   GB_COUNT(1);
}

// pass 0/1: assigned = 0 for C points, 1 for F points with a strong C
// neighbour, -1 otherwise; *count += the pass 1 points
__global__ void k_mp_pass1(int n, const int *__restrict__ Si, const int *__restrict__ Sj,
                           const int *__restrict__ CF, int *__restrict__ assigned, int *count)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int a = -1;
   if (CF[i] == C_PT) { a = 0; }
   else if (CF[i] == F_PT)
   {
      for (int k = Si[i]; k < Si[i + 1]; k++)
      {
         if (CF[Sj[k]] == C_PT) { a = 1; break; }
      }
      if (a == 1) { atomicAdd(count, 1); }
   }
   assigned[i] = a;
}

// pass p >= 2: F points not yet assigned with a strong neighbour of pass
// p-1.  In place: a point changes only from -1 to p, neither equal to p-1.
__global__ void k_mp_pass(int n, const int *__restrict__ Si, const int *__restrict__ Sj,
                          const int *__restrict__ CF, int p, int *assigned, int *count)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n || CF[i] != F_PT || assigned[i] != -1) { return; }
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      if (assigned[Sj[k]] == p - 1)
      {
         assigned[i] = p;
         atomicAdd(count, 1);
         return;
      }
   }
}

extern "C" void gb_mp_pass(int n, const int *Si, const int *Sj, const int *CF, int p, int *assigned, int *count,
                           cudaStream_t s)
{
   if (p == 1) { k_mp_pass1<<<mp_blocks(n, 256), 256, 0, s>>>(n, Si, Sj, CF, assigned, count); }
   else { k_mp_pass<<<mp_blocks(n, 256), 256, 0, s>>>(n, Si, Sj, CF, p, assigned, count); }
   GB_COUNT(1);
}

// upper bound of each row of pass p (listed in rows[0..m)): pass 1, its
// strong C neighbours; pass p, the lengths of its strong pass p-1
// neighbours' rows.  *total (64-bit) += the bounds.
__global__ void k_mp_bound(int m, const int *__restrict__ rows, const int *__restrict__ Si,
                           const int *__restrict__ Sj, const int *__restrict__ assigned, int p,
                           const int *__restrict__ rowlen, int *__restrict__ ub, unsigned long long *total)
{
   int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= m) { return; }
   const int i = rows[t];
   long long b = 0;
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      const int j = Sj[k];
      if (assigned[j] == p - 1) { b += p == 1 ? 1 : rowlen[j]; }
   }
   const int bi = b > 0x7fffffffLL ? 0x7fffffff : (int) b;
   ub[t] = bi;
   atomicAdd(total, (unsigned long long) bi);
}

extern "C" void gb_mp_bound(int m, const int *rows, const int *Si, const int *Sj, const int *assigned, int p,
                            const int *rowlen, int *ub, unsigned long long *total, cudaStream_t s)
{
   if (m <= 0) { return; }
   k_mp_bound<<<mp_blocks(m, 256), 256, 0, s>>>(m, rows, Si, Sj, assigned, p, rowlen, ub, total);
   GB_COUNT(1);
}

// the rows of pass 1, written at off[t] of the pass's area (pj, pv);
// rowoff/rowlen/alfa indexed by point.  A row whose sum_C a_ii is zero is
// left unscaled, flagged in degen[i], and counted in *ndegen.
__global__ void k_mp_rows1(int m, const int *__restrict__ rows, const int *__restrict__ off,
                           const int *__restrict__ Ai, const int *__restrict__ Aj, const double *__restrict__ Av,
                           const int *__restrict__ Si, const int *__restrict__ Sj, const int *__restrict__ CF,
                           const int *__restrict__ f2c, int *__restrict__ pj, double *__restrict__ pv,
                           int *__restrict__ rowoff, int *__restrict__ rowlen, double *__restrict__ alfa_out,
                           int *__restrict__ degen, int *ndegen)
{
   int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= m) { return; }
   const int i = rows[t];
   const int o = off[t];
   int len = 0, sp = Si[i];
   const int se = Si[i + 1];
   double sum_C = 0.0, sum_N = 0.0;
   for (int k = Ai[i] + 1; k < Ai[i + 1]; k++)
   {
      const int j = Aj[k];
      const double a = Av[k];
      const bool strong = sp < se && Sj[sp] == j;
      if (strong) { sp++; }
      if (CF[j] != SF_PT) { sum_N += a; }
      if (strong && CF[j] == C_PT)
      {
         pj[o + len] = f2c[j];
         pv[o + len] = a;
         len++;
         sum_C += a;
      }
   }
   rowoff[i] = o;
   rowlen[i] = len;
   const double diagonal = Av[Ai[i]];
   const double d = sum_C * diagonal;
   if (d != 0.0)
   {
      const double alfa = -sum_N / d;
      for (int q = 0; q < len; q++) { pv[o + q] *= alfa; }
      alfa_out[i] = alfa;
      degen[i] = 0;
   }
   else
   {
      degen[i] = 1;
      atomicAdd(ndegen, 1);
   }
}

// the rows of pass p >= 2 from the finished rows of pass p-1 (area qj, qv)
__global__ void k_mp_rows(int m, const int *__restrict__ rows, const int *__restrict__ off, int p,
                          const int *__restrict__ Ai, const int *__restrict__ Aj, const double *__restrict__ Av,
                          const int *__restrict__ Si, const int *__restrict__ Sj, const int *__restrict__ CF,
                          const int *__restrict__ assigned, const int *__restrict__ qj, const double *__restrict__ qv,
                          int *__restrict__ pj, double *__restrict__ pv, int *__restrict__ rowoff,
                          int *__restrict__ rowlen)
{
   int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= m) { return; }
   const int i = rows[t];
   const int o = off[t];
   // pattern: the union of the strong pass p-1 neighbours' rows, S order
   int len = 0;
   for (int k = Si[i]; k < Si[i + 1]; k++)
   {
      const int j = Sj[k];
      if (assigned[j] != p - 1) { continue; }
      const int b = rowoff[j], e = b + rowlen[j];
      for (int q = b; q < e; q++)
      {
         const int c = qj[q];
         int x = 0;
         while (x < len && pj[o + x] != c) { x++; }
         if (x == len)
         {
            pj[o + len] = c;
            pv[o + len] = 0.0;
            len++;
         }
      }
   }
   // weights: products over the strong pass p-1 neighbours in A order
   double sum_C = 0.0, sum_N = 0.0, alfa = 1.0;
   int sp = Si[i];
   const int se = Si[i + 1];
   for (int k = Ai[i] + 1; k < Ai[i + 1]; k++)
   {
      const int j = Aj[k];
      const double a = Av[k];
      const bool strong = sp < se && Sj[sp] == j;
      if (strong) { sp++; }
      if (strong && assigned[j] == p - 1)
      {
         const int b = rowoff[j], e = b + rowlen[j];
         for (int q = b; q < e; q++)
         {
            const int c = qj[q];
            int x = 0;
            while (x < len && pj[o + x] != c) { x++; }
            if (x == len) { continue; }        // not reached: the pattern holds every column
            alfa = a * qv[q];
            pv[o + x] += alfa;
            sum_C += alfa;
            sum_N += alfa;
         }
      }
      else if (CF[j] != SF_PT) { sum_N += a; }
   }
   const double diagonal = Av[Ai[i]];
   if (sum_C * diagonal != 0.0) { alfa = -sum_N / (sum_C * diagonal); }
   for (int q = 0; q < len; q++) { pv[o + q] *= alfa; }
   rowoff[i] = o;
   rowlen[i] = len;
}

extern "C" void gb_mp_rows(int m, const int *rows, const int *off, int p, const int *Ai, const int *Aj,
                           const double *Av, const int *Si, const int *Sj, const int *CF, const int *f2c,
                           const int *assigned, const int *qj, const double *qv, int *pj, double *pv, int *rowoff,
                           int *rowlen, double *alfa, int *degen, int *ndegen, cudaStream_t s)
{
   if (m <= 0) { return; }
   if (p == 1)
   {
      k_mp_rows1<<<mp_blocks(m, 128), 128, 0, s>>>(m, rows, off, Ai, Aj, Av, Si, Sj, CF, f2c, pj, pv, rowoff,
                                                    rowlen, alfa, degen, ndegen);
   }
   else
   {
      k_mp_rows<<<mp_blocks(m, 128), 128, 0, s>>>(m, rows, off, p, Ai, Aj, Av, Si, Sj, CF, assigned, qj, qv, pj,
                                                   pv, rowoff, rowlen);
   }
   GB_COUNT(1);
}

// Pass 1 rows whose sum_C a_ii is zero take the alfa of the previous pass 1
// row in the reference's visiting order (par_multi_interp.c:466-518, 1626-
// 1715).  Its pass_array starts as the F points in descending order and is
// consumed from both ends: from the back (ascending index) until a point with
// a strong C neighbour is met, then from the front (descending index) while
// the points taken have one, and so on, until the two ends meet; the points
// with a strong C neighbour, in the order taken, are the pass 1 order.  One
// thread replays that merge over the F list fl[0..m).
__global__ void k_mp_carry1(int m, const int *__restrict__ fl, const int *__restrict__ assigned,
                            const int *__restrict__ degen, const double *__restrict__ alfa_row,
                            const int *__restrict__ rowoff, const int *__restrict__ rowlen, double *pv)
{
   if (blockIdx.x != 0 || threadIdx.x != 0) { return; }
   int lo = 0, hi = m - 1;   // next from the back: fl[lo]; from the front: fl[hi]
   bool back = true;
   double alfa = 1.0;
   while (lo <= hi)
   {
      const int i = back ? fl[lo++] : fl[hi--];
      if (assigned[i] == 1)
      {
         if (degen[i])
         {
            for (int q = rowoff[i]; q < rowoff[i] + rowlen[i]; q++) { pv[q] *= alfa; }
         }
         else { alfa = alfa_row[i]; }
         back = false;
      }
      else { back = true; }
   }
}

extern "C" void gb_mp_carry1(int m, const int *fl, const int *assigned, const int *degen, const double *alfa,
                             const int *rowoff, const int *rowlen, double *pv, cudaStream_t s)
{
   if (m <= 0) { return; }
   k_mp_carry1<<<1, 32, 0, s>>>(m, fl, assigned, degen, alfa, rowoff, rowlen, pv);
   GB_COUNT(1);
}

// final row lengths: C points 1, rows of a pass their length, others 0
__global__ void k_mp_len(int n, const int *__restrict__ CF, const int *__restrict__ assigned,
                         const int *__restrict__ rowlen, int *__restrict__ len)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   const int a = assigned[i];
   len[i] = CF[i] == C_PT ? 1 : (a > 0 ? rowlen[i] : 0);
}

extern "C" void gb_mp_len(int n, const int *CF, const int *assigned, const int *rowlen, int *len, cudaStream_t s)
{
   k_mp_len<<<mp_blocks(n, 256), 256, 0, s>>>(n, CF, assigned, rowlen, len);
   GB_COUNT(1);
}

// P from the pass areas: C rows (f2c, 1.0), pass rows copied
__global__ void k_mp_gather(int n, const int *__restrict__ CF, const int *__restrict__ assigned,
                            const int *__restrict__ f2c, const int *__restrict__ rowoff, gb_mp_areas areas,
                            const int *__restrict__ Pi, int *__restrict__ Pj, double *__restrict__ Pv)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   const int b = Pi[i], e = Pi[i + 1];
   if (CF[i] == C_PT)
   {
      Pj[b] = f2c[i];
      Pv[b] = 1.0;
      return;
   }
   const int a = assigned[i];
   if (a <= 0 || e == b) { return; }
   const int *qj = areas.j[a];
   const double *qv = areas.v[a];
   const int o = rowoff[i];
   for (int q = 0; q < e - b; q++)
   {
      Pj[b + q] = qj[o + q];
      Pv[b + q] = qv[o + q];
   }
}

extern "C" void gb_mp_gather(int n, const int *CF, const int *assigned, const int *f2c, const int *rowoff,
                             const gb_mp_areas *areas, const int *Pi, int *Pj, double *Pv, cudaStream_t s)
{
   k_mp_gather<<<mp_blocks(n, 256), 256, 0, s>>>(n, CF, assigned, f2c, rowoff, *areas, Pi, Pj, Pv);
   GB_COUNT(1);
}

// ---------------------------------------------------------------------------
// Multipass interpolation in product form (agg_interp_type 8 and 9,
// hypre_BoomerAMGBuildModMultipassHost src/parcsr_ls/par_mod_multi_interp.c:
// 17-525, hypre_GenerateMultipassPi :530-838, hypre_GenerateMultiPi
// :841-1277).
//
// Passes.  C points are pass 1; in round p the points without a pass that
// have a strong neighbour of pass p take pass p+1 (the reference visits them
// in row order, but a mark of the round, p+1, never equals p, so the result
// does not depend on the order and one kernel per round assigns it).  Within
// a pass the points are numbered in row order: they are the rows of that
// pass's block and the columns of the next pass's Q.
// ---------------------------------------------------------------------------

// pass = 1 for C points, 0 otherwise; *count = the C points
__global__ void k_mmp_init(int n, const int *__restrict__ CF, int *__restrict__ pass, int *count)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   const bool c = i < n && CF[i] == C_PT;
   if (i < n) { pass[i] = c ? 1 : 0; }
   const unsigned b = __ballot_sync(0xffffffffu, c);
   if ((threadIdx.x & 31) == 0 && b) { atomicAdd(count, __popc(b)); }
}

extern "C" void gb_mmp_init(int n, const int *CF, int *pass, int *count, cudaStream_t s)
{
   k_mmp_init<<<mp_blocks(n, 256), 256, 0, s>>>(n, CF, pass, count);
   GB_COUNT(1);
}

// round `cur`: points without a pass and with a strong neighbour of pass cur
// take pass cur+1 (in place); *count += the points marked
__global__ void k_mmp_round(int n, const int *__restrict__ Si, const int *__restrict__ Sj, int cur, int *pass,
                            int *count)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   bool hit = false;
   if (i < n && pass[i] == 0)
   {
      for (int k = Si[i]; k < Si[i + 1]; k++)
      {
         if (pass[Sj[k]] == cur) { hit = true; break; }
      }
      if (hit) { pass[i] = cur + 1; }
   }
   const unsigned b = __ballot_sync(0xffffffffu, hit);
   if ((threadIdx.x & 31) == 0 && b) { atomicAdd(count, __popc(b)); }
}

extern "C" void gb_mmp_round(int n, const int *Si, const int *Sj, int cur, int *pass, int *count, cudaStream_t s)
{
   k_mmp_round<<<mp_blocks(n, 256), 256, 0, s>>>(n, Si, Sj, cur, pass, count);
   GB_COUNT(1);
}

// col[i] = scan[i] for the points of pass p (their number within the pass)
__global__ void k_mmp_col(int n, const int *__restrict__ pass, int p, const int *__restrict__ scan,
                          int *__restrict__ col)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n && pass[i] == p) { col[i] = scan[i]; }
}

extern "C" void gb_mmp_col(int n, const int *pass, int p, const int *scan, int *col, cudaStream_t s)
{
   k_mmp_col<<<mp_blocks(n, 256), 256, 0, s>>>(n, pass, p, scan, col);
   GB_COUNT(1);
}

// rsum[i] = the sum of the off-diagonals of F row i in A order (:272-312;
// the diagonal is the row's first entry), 0 for C rows
__global__ void k_mmp_rowsum(int n, const int *__restrict__ CF, const int *__restrict__ Ai,
                             const double *__restrict__ Av, double *__restrict__ rsum)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   double s = 0.0;
   if (CF[i] < 0)
   {
      for (int k = Ai[i] + 1; k < Ai[i + 1]; k++) { s += Av[k]; }
   }
   rsum[i] = s;
}

extern "C" void gb_mmp_rowsum(int n, const int *CF, const int *Ai, const double *Av, double *rsum, cudaStream_t s)
{
   k_mmp_rowsum<<<mp_blocks(n, 256), 256, 0, s>>>(n, CF, Ai, Av, rsum);
   GB_COUNT(1);
}

// entries of the block rows: strong neighbours of pass `color`
__global__ void k_mmp_count(int m, const int *__restrict__ rows, const int *__restrict__ Si,
                            const int *__restrict__ Sj, const int *__restrict__ pass, int color, int *__restrict__ cnt)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= m) { return; }
   const int i1 = rows[r];
   int c = 0;
   for (int k = Si[i1]; k < Si[i1 + 1]; k++) { c += pass[Sj[k]] == color; }
   cnt[r] = c;
}

extern "C" void gb_mmp_count(int m, const int *rows, const int *Si, const int *Sj, const int *pass, int color,
                             int *cnt, cudaStream_t s)
{
   if (m <= 0) { return; }
   k_mmp_count<<<mp_blocks(m, 256), 256, 0, s>>>(m, rows, Si, Sj, pass, color, cnt);
   GB_COUNT(1);
}

// Block rows (one thread per row).  The row's strong neighbours of pass
// `color` in S order with A's values (S's columns are found in A by a forward
// walk: S is a subsequence of A's off-diagonals).  w == NULL
// (hypre_GenerateMultipassPi :766-823): the row is scaled by -rs with
// rs = rsum / (sum a_ii), or rs = rsum when sum a_ii is zero.  w != NULL (the
// Q of hypre_GenerateMultiPi :1100-1140): the row stays unscaled and w[r]
// sums, in A order, every off-diagonal that is not an entry.
__global__ void k_mmp_fill(int m, const int *__restrict__ rows, const int *__restrict__ Ai,
                           const int *__restrict__ Aj, const double *__restrict__ Av, const int *__restrict__ Si,
                           const int *__restrict__ Sj, const int *__restrict__ pass, const int *__restrict__ col,
                           int color, const int *__restrict__ Qi, int *__restrict__ Qj, double *__restrict__ Qv,
                           const double *__restrict__ rsum, double *__restrict__ w)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= m) { return; }
   const int i1 = rows[r];
   const int a1 = Ai[i1 + 1];
   const int q0 = Qi[r];
   int q = q0;
   if (!w)
   {
      int j2 = Ai[i1];
      for (int k = Si[i1]; k < Si[i1 + 1]; k++)
      {
         const int j1 = Sj[k];
         while (j2 < a1 && Aj[j2] != j1) { j2++; }
         if (j2 == a1) { break; }
         if (pass[j1] == color) { Qj[q] = col[j1]; Qv[q] = Av[j2]; q++; }
      }
      double sum = 0.0;
      for (int k = q0; k < q; k++) { sum += Qv[k]; }
      const double value = sum * Av[Ai[i1]];
      double rs = rsum[i1];
      if (value != 0) { rs /= value; }
      for (int k = q0; k < q; k++) { Qv[k] = -Qv[k] * rs; }
   }
   else
   {
      double ws = 0.0;
      int j2 = Ai[i1] + 1;
      for (int k = Si[i1]; k < Si[i1 + 1]; k++)
      {
         const int j1 = Sj[k];
         while (j2 < a1 && Aj[j2] != j1) { ws += Av[j2]; j2++; }
         if (j2 == a1) { break; }
         if (pass[j1] == color) { Qj[q] = col[j1]; Qv[q] = Av[j2]; q++; }
         else { ws += Av[j2]; }
         j2++;
      }
      while (j2 < a1) { ws += Av[j2]; j2++; }
      w[r] = ws;
   }
}

extern "C" void gb_mmp_fill(int m, const int *rows, const int *Ai, const int *Aj, const double *Av, const int *Si,
                            const int *Sj, const int *pass, const int *col, int color, const int *Qi, int *Qj,
                            double *Qv, const double *rsum, double *w, cudaStream_t s)
{
   if (m <= 0) { return; }
   k_mmp_fill<<<mp_blocks(m, 128), 128, 0, s>>>(m, rows, Ai, Aj, Av, Si, Sj, pass, col, color, Qi, Qj, Qv, rsum,
                                                 w);
   GB_COUNT(1);
}

// type 9 rows after the product (:1236-1265): s = the row's sum,
// value = s a_ii, s += w[r], s /= value when value is not zero, entries *= -s
__global__ void k_mmp_scale9(int m, const int *__restrict__ rows, const int *__restrict__ Ai,
                             const double *__restrict__ Av, const int *__restrict__ Bi, double *__restrict__ Bv,
                             const double *__restrict__ w)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if (r >= m) { return; }
   double s = 0.0;
   for (int k = Bi[r]; k < Bi[r + 1]; k++) { s += Bv[k]; }
   const double value = s * Av[Ai[rows[r]]];
   s += w[r];
   if (value != 0) { s /= value; }
   for (int k = Bi[r]; k < Bi[r + 1]; k++) { Bv[k] = -Bv[k] * s; }
}

extern "C" void gb_mmp_scale9(int m, const int *rows, const int *Ai, const double *Av, const int *Bi, double *Bv,
                              const double *w, cudaStream_t s)
{
   if (m <= 0) { return; }
   k_mmp_scale9<<<mp_blocks(m, 128), 128, 0, s>>>(m, rows, Ai, Av, Bi, Bv, w);
   GB_COUNT(1);
}

// P's row lengths: 1 for C points, the length of the row `col` of the block
// of the point's pass (pass - 2), 0 for points without a pass
__global__ void k_mmp_len(int n, const int *__restrict__ CF, const int *__restrict__ pass,
                          const int *__restrict__ col, gb_mmp_blocks B, int *__restrict__ len)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   int l = 0;
   if (CF[i] == C_PT) { l = 1; }
   else
   {
      const int b = pass[i] - 2;
      if (b >= 0 && b < B.nblk) { l = B.i[b][col[i] + 1] - B.i[b][col[i]]; }
   }
   len[i] = l;
}

__global__ void k_mmp_gather(int n, const int *__restrict__ CF, const int *__restrict__ pass,
                             const int *__restrict__ col, gb_mmp_blocks B, const int *__restrict__ Pi,
                             int *__restrict__ Pj, double *__restrict__ Pv)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) { return; }
   const int o = Pi[i], l = Pi[i + 1] - o;
   if (CF[i] == C_PT)
   {
      Pj[o] = col[i];
      Pv[o] = 1.0;
      return;
   }
   if (l == 0) { return; }
   const int b = pass[i] - 2;
   const int k0 = B.i[b][col[i]];
   for (int q = 0; q < l; q++)
   {
      Pj[o + q] = B.j[b][k0 + q];
      Pv[o + q] = B.v[b][k0 + q];
   }
}

extern "C" void gb_mmp_len(int n, const int *CF, const int *pass, const int *col, const gb_mmp_blocks *B, int *len,
                           cudaStream_t s)
{
   k_mmp_len<<<mp_blocks(n, 256), 256, 0, s>>>(n, CF, pass, col, *B, len);
   GB_COUNT(1);
}

extern "C" void gb_mmp_gather(int n, const int *CF, const int *pass, const int *col, const gb_mmp_blocks *B,
                              const int *Pi, int *Pj, double *Pv, cudaStream_t s)
{
   k_mmp_gather<<<mp_blocks(n, 256), 256, 0, s>>>(n, CF, pass, col, *B, Pi, Pj, Pv);
   GB_COUNT(1);
}
