// Device assembly of IJ matrices (HYPRE_IJMatrixSetValues / Assemble).
//
// Large puts whose rows are new are copied straight from the caller's
// buffers into a device staging area; k_ij_check validates them (columns in
// range, no column repeated within a row) before the put returns, so a put
// that would need the host path's merge or error reporting is handed to it
// instead.  At assembly k_ij_gather builds the CSR arrays from the staged
// rows with the reference's diagonal handling (IJMatrix_parcsr.c:2900-2990):
// the diagonal moves to the front, either by shifting the entries before it
// or (SetDiagOffdSizes) by swapping it with the first entry.
#include <cuda_runtime.h>

#include "gb_device.cuh"
#include "gb_kernels.h"

// one warp per put row t (entries start[t] .. start[t+1]-1 of cols):
// flags |= 1 for a column outside [0, ncol), 2 for a repeated column,
// 4 for a row too long to check here
__global__ void k_ij_check(int nrows, const int *__restrict__ start, const int *__restrict__ cols, int ncol,
                           int *flags)
{
   const int t = (int) ((blockIdx.x * (long long) blockDim.x + threadIdx.x) >> 5);
   const int lane = threadIdx.x & 31;
   if (t >= nrows) { return; }
   const int b = start[t], e = start[t + 1];
   const int l = e - b;
   int f = 0;
   if (l > 4096) { f = 4; }
   else
   {
      for (int ca = b; ca < e; ca += 32)
      {
         const int ka = ca + lane;
         const bool va = ka < e;
         const int ka_col = va ? cols[ka] : -1;
         if (va && (ka_col < 0 || ka_col >= ncol)) { f |= 1; }
         // within the chunk: lanes sharing a column
         const unsigned grp = __match_any_sync(GB_FULL, va ? ka_col : -(lane + 2));
         if (va && __popc(grp) > 1) { f |= 2; }
         // against the later chunks: broadcast each of their columns
         for (int cb = ca + 32; cb < e; cb += 32)
         {
            const int kb = cb + lane;
            const int kb_col = kb < e ? cols[kb] : -1;
            const int nb = min(32, e - cb);
            for (int q = 0; q < nb; q++)
            {
               const int c = __shfl_sync(GB_FULL, kb_col, q);
               if (va && c == ka_col) { f |= 2; }
            }
         }
      }
   }
   f = __reduce_or_sync(GB_FULL, f);
   if (lane == 0 && f) { atomicOr(flags, f); }
}

extern "C" void gb_ij_check(int nrows, const int *start, const int *cols, int ncol, int *flags, cudaStream_t s)
{
   if (nrows <= 0) { return; }
   k_ij_check<<<(int) (((long long) nrows * 32 + 255) / 256), 256, 0, s>>>(nrows, start, cols, ncol, flags);
   GB_COUNT(1);
}

// LPR lanes per row r (LPR divides 32): staged entries off[r] .. off[r]+len
// (len = I[r+1]-I[r]; off NULL: the staging is in row order, off[r] = I[r])
// -> J, V at I[r], diagonal first (shift, or swap when swap_diag).  key
// (optional): the column moved to the front of row r is key[r] instead of r
// (the reference's rule when some rows have no space, see gb_ij.c)
template <int LPR>
__global__ void k_ij_gather(int n, const long long *__restrict__ off, const int *__restrict__ I,
                            const int *__restrict__ scols, const double *__restrict__ svals, int swap_diag,
                            const int *__restrict__ key, int *__restrict__ J, double *__restrict__ V)
{
   const long long g = blockIdx.x * (long long) blockDim.x + threadIdx.x;
   const int r = (int) (g / LPR);
   const int lane = (int) (g % LPR);
   if (r >= n) { return; }   // whole segments leave together
   const int sbase = (threadIdx.x & 31) & ~(LPR - 1);
   const unsigned seg = LPR == 32 ? GB_FULL : (((1u << LPR) - 1u) << sbase);
   const int d = I[r], l = I[r + 1] - d;
   const long long o = off ? off[r] : (long long) d;
   const int front = key ? key[r] : r;
   // first position of the diagonal
   int dpos = -1;
   for (int c = 0; c < l && dpos < 0; c += LPR)
   {
      const int q = c + lane;
      const unsigned m = __ballot_sync(seg, q < l && scols[o + q] == front) >> sbase;
      if (m) { dpos = c + __ffs(m) - 1; }
   }
   for (int q = lane; q < l; q += LPR)
   {
      int src = q;
      if (dpos > 0)
      {
         if (swap_diag) { src = q == 0 ? dpos : (q == dpos ? 0 : q); }
         else { src = q == 0 ? dpos : (q <= dpos ? q - 1 : q); }
      }
      J[d + q] = scols[o + src];
      V[d + q] = svals[o + src];
   }
}

extern "C" void gb_ij_gather(int n, long long nnz, const long long *off, const int *I, const int *scols,
                             const double *svals, int swap_diag, const int *key, int *J, double *V, cudaStream_t s)
{
   if (n <= 0) { return; }
   const long long avg = nnz / n;
#define GB_IJG(L)                                                                                                  \
   k_ij_gather<L><<<(int) (((long long) n * L + 255) / 256), 256, 0, s>>>(n, off, I, scols, svals, swap_diag, key, \
                                                                          J, V)
   if (avg <= 6) { GB_IJG(4); }
   else if (avg <= 12) { GB_IJG(8); }
   else if (avg <= 40) { GB_IJG(16); }
   else { GB_IJG(32); }
#undef GB_IJG
   GB_COUNT(1);
}
