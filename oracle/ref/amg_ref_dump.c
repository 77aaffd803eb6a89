/* Golden dumper: runs the REFERENCE library's CPU BoomerAMG-PCG / FGMRES
 * through its public C API (IJ assembly, BoomerAMG setters, ParCSR PCG or
 * FlexGMRES) and writes the hierarchy and residual history to a binary record
 * file that tests/golden/make_golden.py turns into fixtures.
 *
 * Test infrastructure only: linked against oracle/_ref/libHYPRE_ref.a, which
 * oracle/ref/Makefile compiles from the reference's own sources.
 *
 * Record file format (little endian): repeated
 *   char name[32]; int32 dtype (0=int32, 1=float64); int64 count; data[count]
 *
 * Timing and digest mode (the CPU reference timed by bench.py and the
 * parity record at full size):
 *   -repeat R    R complete setup+solve runs (new solver objects, x0 = 0 each
 *                time), setup and solve timed with CLOCK_MONOTONIC
 *   -threads T   OpenMP threads of the reference's threaded loops (OpenMP build)
 *   -json F      write a JSON summary instead of the record file: per-run
 *                times, iterations, residual history, per level rows and nnz
 *   -matmat      instead of a solve, record C = A*A from HYPRE_ParCSRMatrixMatmat
 *                (C_i, C_j, C_v) and the product's wall time (t_matmat)
 *   -digest      with -json: per level also SHA-256 digests of A's and P's
 *                patterns (row pointers then column indices, int32) and values
 *                (float64), of the CF markers, and the sums of |values|
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <math.h>

#include "_hypre_utilities.h"
#include "HYPRE.h"
#include "HYPRE_parcsr_ls.h"
#include "_hypre_parcsr_ls.h"
#include "_hypre_krylov.h"
#include "HYPRE_krylov.h"
#include "sha256.h"
#ifdef GB_REF_OPENMP
#include <omp.h>
#endif

static FILE *g_out = NULL;

static void rec(const char *name, int dtype, long long count, const void *data)
{
   char nm[32];
   memset(nm, 0, sizeof(nm));
   strncpy(nm, name, 31);
   fwrite(nm, 1, 32, g_out);
   fwrite(&dtype, 4, 1, g_out);
   fwrite(&count, 8, 1, g_out);
   if (count > 0) { fwrite(data, dtype == 0 ? 4 : 8, (size_t) count, g_out); }
}

static double now_s(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* Stencil generators: diagonal first, then off-diagonals in ascending column
 * order (the order GenerateLaplacian / GenerateLaplacian27pt emit). */
static void gen_stencil(int kind, int nx, int ny, int nz,
                        int **ip, int **jp, double **vp, int *nnz_out)
{
   int n = nx * ny * nz;
   int maxrow = (kind == 27) ? 27 : 7;
   int *I = malloc(sizeof(int) * (n + 1));
   int *J = malloc(sizeof(int) * (size_t) n * maxrow);
   double *V = malloc(sizeof(double) * (size_t) n * maxrow);
   int cnt = 0;
   for (int iz = 0; iz < nz; iz++)
      for (int iy = 0; iy < ny; iy++)
         for (int ix = 0; ix < nx; ix++)
         {
            int row = ix + nx * (iy + ny * iz);
            I[row] = cnt;
            J[cnt] = row; V[cnt] = (kind == 27) ? 26.0 : 6.0; cnt++;
            for (int dz = -1; dz <= 1; dz++)
               for (int dy = -1; dy <= 1; dy++)
                  for (int dx = -1; dx <= 1; dx++)
                  {
                     int m = abs(dx) + abs(dy) + abs(dz);
                     if (m == 0) { continue; }
                     if (kind == 7 && m != 1) { continue; }
                     int jx = ix + dx, jy = iy + dy, jz = iz + dz;
                     if (jx < 0 || jy < 0 || jz < 0 || jx >= nx || jy >= ny || jz >= nz) { continue; }
                     J[cnt] = jx + nx * (jy + ny * jz); V[cnt] = -1.0; cnt++;
                  }
         }
   I[n] = cnt;
   *ip = I; *jp = J; *vp = V; *nnz_out = cnt;
}

/* Binary CSR file: int32 n, int32 nnz, int32 rowptr[n+1], int32 col[nnz],
 * float64 val[nnz], then optionally float64 rhs[n]. */
static int read_csr(const char *path, int *n_out, int **ip, int **jp, double **vp, double **rhs)
{
   FILE *f = fopen(path, "rb");
   if (!f) { return 1; }
   int n, nnz;
   if (fread(&n, 4, 1, f) != 1 || fread(&nnz, 4, 1, f) != 1) { fclose(f); return 1; }
   *ip = malloc(sizeof(int) * (n + 1));
   *jp = malloc(sizeof(int) * nnz);
   *vp = malloc(sizeof(double) * nnz);
   if (fread(*ip, 4, n + 1, f) != (size_t)(n + 1)) { fclose(f); return 1; }
   if (fread(*jp, 4, nnz, f) != (size_t) nnz) { fclose(f); return 1; }
   if (fread(*vp, 8, nnz, f) != (size_t) nnz) { fclose(f); return 1; }
   double *b = malloc(sizeof(double) * n);
   if (fread(b, 8, n, f) == (size_t) n) { *rhs = b; } else { free(b); *rhs = NULL; }
   fclose(f);
   *n_out = n;
   return 0;
}

static void dump_csr(const char *pfx, int lvl, hypre_CSRMatrix *M, int with_data)
{
   char nm[32];
   int nr = hypre_CSRMatrixNumRows(M);
   int *I = hypre_CSRMatrixI(M);
   int nnz = I[nr];
   snprintf(nm, 32, "%s%d_i", pfx, lvl); rec(nm, 0, nr + 1, I);
   snprintf(nm, 32, "%s%d_j", pfx, lvl); rec(nm, 0, nnz, hypre_CSRMatrixJ(M));
   if (with_data && hypre_CSRMatrixData(M))
   {
      snprintf(nm, 32, "%s%d_v", pfx, lvl); rec(nm, 1, nnz, hypre_CSRMatrixData(M));
   }
}

static void digest_csr(hypre_CSRMatrix *M, char pat[65], char val[65], double *abs_sum)
{
   int nr = hypre_CSRMatrixNumRows(M);
   int *I = hypre_CSRMatrixI(M);
   int nnz = I[nr];
   double *D = hypre_CSRMatrixData(M);
   sha256_ctx s;
   sha256_init(&s);
   sha256_update(&s, I, sizeof(int) * (size_t)(nr + 1));
   sha256_update(&s, hypre_CSRMatrixJ(M), sizeof(int) * (size_t) nnz);
   sha256_hex(&s, pat);
   sha256_init(&s);
   sha256_update(&s, D, sizeof(double) * (size_t) nnz);
   sha256_hex(&s, val);
   double a = 0.0;
   for (int k = 0; k < nnz; k++) { a += fabs(D[k]); }
   *abs_sum = a;
}

static void json_strs(FILE *f, const char *key, char (*v)[65], int n, int last)
{
   fprintf(f, "\"%s\": [", key);
   for (int i = 0; i < n; i++) { fprintf(f, "%s\"%s\"", i ? ", " : "", v[i]); }
   fprintf(f, "]%s\n", last ? "" : ",");
}

static void json_nums(FILE *f, const char *key, const double *v, int n, int last)
{
   fprintf(f, "\"%s\": [", key);
   for (int i = 0; i < n; i++) { fprintf(f, "%s%.17g", i ? ", " : "", v[i]); }
   fprintf(f, "]%s\n", last ? "" : ",");
}

int main(int argc, char **argv)
{
   int kind = 7, nx = 10, ny = 10, nz = 10;
   const char *matfile = NULL, *outfile = "dump.bin";
   double theta = 0.25, mrs = 1.0, tol = 1e-8, trunc = 0.0, relax_wt = 1.0;
   int pmx = 4, interp = 6, agg_nl = 0, agg_interp = 4, agg_pmx = 0, agg_p12 = 0, num_paths = 1;
   int relax = 18, relax_coarse = 9, coarse_th = 9, maxit = 100, solver = 1, kdim = 30;
   int max_levels = 25, dump_levels = 1, seed = 22775, cheby_order = 2, relax_order = 0;
   int coarsen = 8, precond = 1, keep_t = 0, rhs_ones = 0, cycle_type = 1, fcycle = 0, num_sweeps = 1;
   int rel_change = 0;
   double outer_wt = 1.0;
   int repeat = 1, threads = 0, want_digest = 0, matmat = 0, relax_down = -1, relax_up = -1;
   const char *jsonfile = NULL;
   double cheby_fraction = 0.3;

   for (int a = 1; a < argc; a++)
   {
#define ARG(s) (strcmp(argv[a], s) == 0 && a + 1 < argc)
      if (ARG("-lap7")) { kind = 7; nx = atoi(argv[++a]); ny = atoi(argv[++a]); nz = atoi(argv[++a]); }
      else if (ARG("-lap27")) { kind = 27; nx = atoi(argv[++a]); ny = atoi(argv[++a]); nz = atoi(argv[++a]); }
      else if (ARG("-mat")) { matfile = argv[++a]; }
      else if (ARG("-o")) { outfile = argv[++a]; }
      else if (ARG("-th")) { theta = atof(argv[++a]); }
      else if (ARG("-mxrs")) { mrs = atof(argv[++a]); }
      else if (ARG("-tol")) { tol = atof(argv[++a]); }
      else if (ARG("-tr")) { trunc = atof(argv[++a]); }
      else if (ARG("-w")) { relax_wt = atof(argv[++a]); }
      else if (ARG("-Pmx")) { pmx = atoi(argv[++a]); }
      else if (ARG("-interptype")) { interp = atoi(argv[++a]); }
      else if (ARG("-agg_nl")) { agg_nl = atoi(argv[++a]); }
      else if (ARG("-agg_interp")) { agg_interp = atoi(argv[++a]); }
      else if (ARG("-agg_Pmx")) { agg_pmx = atoi(argv[++a]); }
      else if (ARG("-agg_P12_mx")) { agg_p12 = atoi(argv[++a]); }
      else if (ARG("-np")) { num_paths = atoi(argv[++a]); }
      else if (ARG("-rlx")) { relax = atoi(argv[++a]); }
      else if (ARG("-rlx_coarse")) { relax_coarse = atoi(argv[++a]); }
      else if (ARG("-rlx_down")) { relax_down = atoi(argv[++a]); }
      else if (ARG("-rlx_up")) { relax_up = atoi(argv[++a]); }
      else if (ARG("-coarse_th")) { coarse_th = atoi(argv[++a]); }
      else if (ARG("-maxit")) { maxit = atoi(argv[++a]); }
      else if (ARG("-solver")) { solver = atoi(argv[++a]); }
      else if (ARG("-k")) { kdim = atoi(argv[++a]); }
      else if (ARG("-max_levels")) { max_levels = atoi(argv[++a]); }
      else if (ARG("-dump_levels")) { dump_levels = atoi(argv[++a]); }
      else if (ARG("-seed")) { seed = atoi(argv[++a]); }
      else if (ARG("-cheby_order")) { cheby_order = atoi(argv[++a]); }
      else if (ARG("-cheby_fraction")) { cheby_fraction = atof(argv[++a]); }
      else if (ARG("-coarsen")) { coarsen = atoi(argv[++a]); }
      else if (ARG("-precond")) { precond = atoi(argv[++a]); }
      else if (ARG("-keepT")) { keep_t = atoi(argv[++a]); }
      else if (ARG("-relax_order")) { relax_order = atoi(argv[++a]); }
      else if (ARG("-cycle_type")) { cycle_type = atoi(argv[++a]); }
      else if (ARG("-fcycle")) { fcycle = atoi(argv[++a]); }
      else if (ARG("-ns")) { num_sweeps = atoi(argv[++a]); }
      else if (ARG("-rel_change")) { rel_change = atoi(argv[++a]); }
      else if (ARG("-ow")) { outer_wt = atof(argv[++a]); }
      else if (ARG("-repeat")) { repeat = atoi(argv[++a]); }
      else if (ARG("-threads")) { threads = atoi(argv[++a]); }
      else if (ARG("-json")) { jsonfile = argv[++a]; }
      else if (strcmp(argv[a], "-digest") == 0) { want_digest = 1; }
      else if (strcmp(argv[a], "-matmat") == 0) { matmat = 1; }
      else if (strcmp(argv[a], "-rhsones") == 0) { rhs_ones = 1; }
      else { fprintf(stderr, "unknown/incomplete arg %s\n", argv[a]); return 2; }
#undef ARG
   }

   int n, nnz = 0;
   int *I, *J;
   double *V, *rhs = NULL;
   if (matfile)
   {
      if (read_csr(matfile, &n, &I, &J, &V, &rhs)) { fprintf(stderr, "cannot read %s\n", matfile); return 2; }
      nnz = I[n];
   }
   else
   {
      gen_stencil(kind, nx, ny, nz, &I, &J, &V, &nnz);
      n = nx * ny * nz;
   }

   if (repeat < 1) { repeat = 1; }
#ifdef GB_REF_OPENMP
   if (threads > 0) { omp_set_num_threads(threads); }
   threads = omp_get_max_threads();
#else
   threads = 1;
#endif
   HYPRE_Initialize();
   if (!jsonfile)
   {
      g_out = fopen(outfile, "wb");
      if (!g_out) { return 2; }
   }

   /* --- IJ assembly, one SetValues call per row (user order kept, diagonal first) --- */
   HYPRE_IJMatrix ij_A;
   HYPRE_IJMatrixCreate(hypre_MPI_COMM_WORLD, 0, n - 1, 0, n - 1, &ij_A);
   HYPRE_IJMatrixSetObjectType(ij_A, HYPRE_PARCSR);
   int *rowsz = malloc(sizeof(int) * n);
   for (int i = 0; i < n; i++) { rowsz[i] = I[i + 1] - I[i]; }
   HYPRE_IJMatrixSetRowSizes(ij_A, rowsz);
   HYPRE_IJMatrixInitialize(ij_A);
   for (int i = 0; i < n; i++)
   {
      int nc = rowsz[i];
      HYPRE_BigInt row = i;
      HYPRE_IJMatrixSetValues(ij_A, 1, &nc, &row, (HYPRE_BigInt *) &J[I[i]], &V[I[i]]);
   }
   HYPRE_IJMatrixAssemble(ij_A);
   HYPRE_ParCSRMatrix A;
   HYPRE_IJMatrixGetObject(ij_A, (void **) &A);

   if (matmat)
   {
      HYPRE_ParCSRMatrix Cm = NULL;
      double tm = now_s();
      HYPRE_ParCSRMatrixMatmat(A, A, &Cm);
      tm = now_s() - tm;
      dump_csr("A", 0, hypre_ParCSRMatrixDiag((hypre_ParCSRMatrix *) A), 1);
      dump_csr("C", 0, hypre_ParCSRMatrixDiag((hypre_ParCSRMatrix *) Cm), 1);
      rec("t_matmat", 1, 1, &tm);
      fclose(g_out);
      printf("A*A: %d rows, nnz %d, %.4f s\n", n,
             hypre_CSRMatrixNumNonzeros(hypre_ParCSRMatrixDiag((hypre_ParCSRMatrix *) Cm)), tm);
      return 0;
   }

   /* --- vectors: b = random[-1,1] (seeded), normalised to unit 2-norm; x0 = 0 --- */
   HYPRE_IJVector ij_b, ij_x;
   HYPRE_IJVectorCreate(hypre_MPI_COMM_WORLD, 0, n - 1, &ij_b);
   HYPRE_IJVectorSetObjectType(ij_b, HYPRE_PARCSR);
   HYPRE_IJVectorInitialize(ij_b);
   HYPRE_IJVectorAssemble(ij_b);
   HYPRE_ParVector b, x;
   HYPRE_IJVectorGetObject(ij_b, (void **) &b);
   if (rhs)
   {
      memcpy(hypre_VectorData(hypre_ParVectorLocalVector((hypre_ParVector *) b)), rhs, sizeof(double) * n);
   }
   else if (rhs_ones)
   {
      HYPRE_ParVectorSetConstantValues(b, 1.0);
   }
   else
   {
      double norm;
      HYPRE_ParVectorSetRandomValues(b, seed);
      HYPRE_ParVectorInnerProd(b, b, &norm);
      norm = 1. / sqrt(norm);
      HYPRE_ParVectorScale(norm, b);
   }
   HYPRE_IJVectorCreate(hypre_MPI_COMM_WORLD, 0, n - 1, &ij_x);
   HYPRE_IJVectorSetObjectType(ij_x, HYPRE_PARCSR);
   HYPRE_IJVectorInitialize(ij_x);
   HYPRE_IJVectorAssemble(ij_x);
   HYPRE_IJVectorGetObject(ij_x, (void **) &x);
   HYPRE_ParVectorSetConstantValues(x, 0.0);
   if (!jsonfile) { rec("b", 1, n, hypre_VectorData(hypre_ParVectorLocalVector((hypre_ParVector *) b))); }

   double *run_setup = malloc(sizeof(double) * repeat), *run_solve = malloc(sizeof(double) * repeat);
   HYPRE_Solver amg = NULL, ks = NULL;
   double t0, t_setup = 0, t_solve = 0;
   int iters = 0;
   double final_res = 0;
   const double *hist = NULL;
   for (int r = 0; r < repeat; r++)
   {
   if (r > 0)
   {
      /* the previous run's solver objects; the last run's are kept for the dumps */
      if (solver == 1) { HYPRE_ParCSRPCGDestroy(ks); }
      else if (solver == 61) { HYPRE_ParCSRFlexGMRESDestroy(ks); }
      HYPRE_BoomerAMGDestroy(amg);
      ks = NULL;
      HYPRE_ParVectorSetConstantValues(x, 0.0);
   }
   /* --- BoomerAMG as preconditioner (one V-cycle, tol 0) --- */
   HYPRE_BoomerAMGCreate(&amg);
   HYPRE_BoomerAMGSetCoarsenType(amg, coarsen);
   HYPRE_BoomerAMGSetStrongThreshold(amg, theta);
   HYPRE_BoomerAMGSetMaxRowSum(amg, mrs);
   HYPRE_BoomerAMGSetTruncFactor(amg, trunc);
   HYPRE_BoomerAMGSetPMaxElmts(amg, pmx);
   HYPRE_BoomerAMGSetInterpType(amg, interp);
   HYPRE_BoomerAMGSetAggNumLevels(amg, agg_nl);
   HYPRE_BoomerAMGSetAggInterpType(amg, agg_interp);
   HYPRE_BoomerAMGSetAggPMaxElmts(amg, agg_pmx);
   HYPRE_BoomerAMGSetAggP12MaxElmts(amg, agg_p12);
   HYPRE_BoomerAMGSetNumPaths(amg, num_paths);
   HYPRE_BoomerAMGSetRelaxType(amg, relax);
   if (relax_down >= 0) { HYPRE_BoomerAMGSetCycleRelaxType(amg, relax_down, 1); }
   if (relax_up >= 0) { HYPRE_BoomerAMGSetCycleRelaxType(amg, relax_up, 2); }
   HYPRE_BoomerAMGSetCycleRelaxType(amg, relax_coarse, 3);
   HYPRE_BoomerAMGSetRelaxWt(amg, relax_wt);
   HYPRE_BoomerAMGSetOuterWt(amg, outer_wt);
   HYPRE_BoomerAMGSetRelaxOrder(amg, relax_order);
   HYPRE_BoomerAMGSetNumSweeps(amg, num_sweeps);
   HYPRE_BoomerAMGSetCycleNumSweeps(amg, 1, 3);
   HYPRE_BoomerAMGSetCycleType(amg, cycle_type);
   HYPRE_BoomerAMGSetFCycle(amg, fcycle);
   HYPRE_BoomerAMGSetChebyOrder(amg, cheby_order);
   HYPRE_BoomerAMGSetChebyFraction(amg, cheby_fraction);
   HYPRE_BoomerAMGSetMaxCoarseSize(amg, coarse_th);
   HYPRE_BoomerAMGSetMaxLevels(amg, max_levels);
   HYPRE_BoomerAMGSetKeepTranspose(amg, keep_t);
   HYPRE_BoomerAMGSetPrintLevel(amg, 0);
   if (precond)
   {
      HYPRE_BoomerAMGSetMaxIter(amg, 1);
      HYPRE_BoomerAMGSetTol(amg, 0.0);
   }
   else
   {
      HYPRE_BoomerAMGSetMaxIter(amg, maxit);
      HYPRE_BoomerAMGSetTol(amg, tol);
   }

   if (solver == 1)
   {
      HYPRE_ParCSRPCGCreate(hypre_MPI_COMM_WORLD, &ks);
      HYPRE_PCGSetMaxIter(ks, maxit);
      HYPRE_PCGSetTol(ks, tol);
      HYPRE_PCGSetTwoNorm(ks, 1);
      HYPRE_PCGSetRelChange(ks, rel_change);
      HYPRE_PCGSetPrintLevel(ks, 0);
      HYPRE_PCGSetLogging(ks, 1);
      HYPRE_PCGSetPrecond(ks, (HYPRE_PtrToSolverFcn) HYPRE_BoomerAMGSolve,
                          (HYPRE_PtrToSolverFcn) HYPRE_BoomerAMGSetup, amg);
      t0 = now_s();
      HYPRE_ParCSRPCGSetup(ks, A, b, x);
      t_setup = now_s() - t0;
      t0 = now_s();
      HYPRE_ParCSRPCGSolve(ks, A, b, x);
      t_solve = now_s() - t0;
      HYPRE_PCGGetNumIterations(ks, &iters);
      HYPRE_PCGGetFinalRelativeResidualNorm(ks, &final_res);
      hypre_PCGData *pd = (hypre_PCGData *) ks;
      hist = pd->rel_norms;
   }
   else if (solver == 61)
   {
      HYPRE_ParCSRFlexGMRESCreate(hypre_MPI_COMM_WORLD, &ks);
      HYPRE_FlexGMRESSetKDim(ks, kdim);
      HYPRE_FlexGMRESSetMaxIter(ks, maxit);
      HYPRE_FlexGMRESSetTol(ks, tol);
      /* print level 1 keeps the residual norm of every iteration (norms[]) */
      HYPRE_FlexGMRESSetPrintLevel(ks, 1);
      HYPRE_FlexGMRESSetLogging(ks, 1);
      HYPRE_FlexGMRESSetPrecond(ks, (HYPRE_PtrToSolverFcn) HYPRE_BoomerAMGSolve,
                                (HYPRE_PtrToSolverFcn) HYPRE_BoomerAMGSetup, amg);
      t0 = now_s();
      HYPRE_ParCSRFlexGMRESSetup(ks, A, b, x);
      t_setup = now_s() - t0;
      t0 = now_s();
      HYPRE_ParCSRFlexGMRESSolve(ks, A, b, x);
      t_solve = now_s() - t0;
      HYPRE_FlexGMRESGetNumIterations(ks, &iters);
      HYPRE_FlexGMRESGetFinalRelativeResidualNorm(ks, &final_res);
      hypre_FlexGMRESData *gd = (hypre_FlexGMRESData *) ks;
      hist = gd->norms;
   }
   else
   {
      /* stand-alone AMG */
      HYPRE_BoomerAMGSetPrintLevel(amg, 0);
      HYPRE_BoomerAMGSetLogging(amg, 0);
      t0 = now_s();
      HYPRE_BoomerAMGSetup(amg, A, b, x);
      t_setup = now_s() - t0;
      t0 = now_s();
      HYPRE_BoomerAMGSolve(amg, A, b, x);
      t_solve = now_s() - t0;
      HYPRE_BoomerAMGGetNumIterations(amg, &iters);
      HYPRE_BoomerAMGGetFinalRelativeResidualNorm(amg, &final_res);
   }
   run_setup[r] = t_setup;
   run_solve[r] = t_solve;
   }
   if (jsonfile)
   {
      hypre_ParAMGData *ad = (hypre_ParAMGData *) amg;
      int nl = hypre_ParAMGDataNumLevels(ad);
      char (*apat)[65] = malloc(65 * (size_t) nl), (*aval)[65] = malloc(65 * (size_t) nl);
      char (*ppat)[65] = malloc(65 * (size_t) nl), (*pval)[65] = malloc(65 * (size_t) nl);
      char (*cfd)[65] = malloc(65 * (size_t) nl);
      double *rows = malloc(sizeof(double) * nl), *nzs = malloc(sizeof(double) * nl);
      double *aabs = malloc(sizeof(double) * nl), *pabs = malloc(sizeof(double) * nl);
      for (int l = 0; l < nl; l++)
      {
         hypre_CSRMatrix *Ad = hypre_ParCSRMatrixDiag(hypre_ParAMGDataAArray(ad)[l]);
         rows[l] = hypre_CSRMatrixNumRows(Ad);
         nzs[l] = hypre_CSRMatrixI(Ad)[hypre_CSRMatrixNumRows(Ad)];
         strcpy(apat[l], ""); strcpy(aval[l], ""); aabs[l] = 0.0;
         strcpy(ppat[l], ""); strcpy(pval[l], ""); strcpy(cfd[l], ""); pabs[l] = 0.0;
         if (!want_digest) { continue; }
         digest_csr(Ad, apat[l], aval[l], &aabs[l]);
         if (l < nl - 1)
         {
            digest_csr(hypre_ParCSRMatrixDiag(hypre_ParAMGDataPArray(ad)[l]), ppat[l], pval[l], &pabs[l]);
            hypre_IntArray *cf = hypre_ParAMGDataCFMarkerArray(ad)[l];
            if (cf)
            {
               sha256_ctx sc;
               sha256_init(&sc);
               sha256_update(&sc, hypre_IntArrayData(cf), sizeof(int) * (size_t) hypre_IntArraySize(cf));
               sha256_hex(&sc, cfd[l]);
            }
         }
      }
      FILE *f = fopen(jsonfile, "w");
      if (!f) { return 2; }
      fprintf(f, "{\n\"n\": %d, \"nnz\": %d, \"threads\": %d, \"levels\": %d, \"iterations\": %d,\n",
              n, nnz, threads, nl, iters);
      fprintf(f, "\"final_relres\": %.17g,\n", final_res);
      json_nums(f, "setup_seconds", run_setup, repeat, 0);
      json_nums(f, "solve_seconds", run_solve, repeat, 0);
      if (hist) { json_nums(f, "history", hist, iters + 1, 0); }
      json_nums(f, "rows", rows, nl, 0);
      json_nums(f, "nnz_levels", nzs, nl, 0);
      json_nums(f, "A_abs_sum", aabs, nl, 0);
      json_nums(f, "P_abs_sum", pabs, nl - 1 > 0 ? nl - 1 : 0, 0);
      json_strs(f, "A_pattern", apat, nl, 0);
      json_strs(f, "A_values", aval, nl, 0);
      json_strs(f, "P_pattern", ppat, nl - 1 > 0 ? nl - 1 : 0, 0);
      json_strs(f, "P_values", pval, nl - 1 > 0 ? nl - 1 : 0, 0);
      json_strs(f, "CF", cfd, nl - 1 > 0 ? nl - 1 : 0, 1);
      fprintf(f, "}\n");
      fclose(f);
      printf("levels %d iters %d final_relres %.6e setup %.4f s solve %.4f s (%d threads)\n",
             nl, iters, final_res, t_setup, t_solve, threads);
      return 0;
   }
   if (hist) { rec(solver == 1 ? "relres" : "resnorms", 1, iters + 1, hist); }
   rec("iters", 0, 1, &iters);
   rec("final_relres", 1, 1, &final_res);
   rec("t_setup", 1, 1, &t_setup);
   rec("t_solve", 1, 1, &t_solve);
   rec("x", 1, n, hypre_VectorData(hypre_ParVectorLocalVector((hypre_ParVector *) x)));

   /* --- hierarchy --- */
   hypre_ParAMGData *amg_data = (hypre_ParAMGData *) amg;
   int nlev = hypre_ParAMGDataNumLevels(amg_data);
   rec("nlev", 0, 1, &nlev);
   int *lev_rows = malloc(sizeof(int) * nlev), *lev_nnz = malloc(sizeof(int) * nlev);
   for (int l = 0; l < nlev; l++)
   {
      hypre_ParCSRMatrix *Al = hypre_ParAMGDataAArray(amg_data)[l];
      hypre_CSRMatrix *Ad = hypre_ParCSRMatrixDiag(Al);
      lev_rows[l] = hypre_CSRMatrixNumRows(Ad);
      lev_nnz[l] = hypre_CSRMatrixI(Ad)[lev_rows[l]];
      if (!dump_levels) { continue; }
      dump_csr("A", l, Ad, 1);
      if (l < nlev - 1)
      {
         hypre_ParCSRMatrix *Pl = hypre_ParAMGDataPArray(amg_data)[l];
         dump_csr("P", l, hypre_ParCSRMatrixDiag(Pl), 1);
         hypre_IntArray *cf = hypre_ParAMGDataCFMarkerArray(amg_data)[l];
         if (cf)
         {
            char nm[32];
            snprintf(nm, 32, "CF%d", l);
            rec(nm, 0, hypre_IntArraySize(cf), hypre_IntArrayData(cf));
         }
         if (l >= agg_nl)
         {
            /* strength matrix of this level, recomputed with the setup's parameters */
            hypre_ParCSRMatrix *S = NULL;
            hypre_BoomerAMGCreateS(Al, theta, mrs, 1, NULL, &S);
            dump_csr("S", l, hypre_ParCSRMatrixDiag(S), 0);
            hypre_ParCSRMatrixDestroy(S);
         }
      }
      /* Chebyshev smoother data (relax 16): eigenvalue estimates, coefficients, D^{-1/2} */
      HYPRE_Real **coefs = hypre_ParAMGDataChebyCoefs(amg_data);
      if (coefs && coefs[l])
      {
         char nm[32];
         int ord = cheby_order < 1 ? 1 : (cheby_order > 4 ? 4 : cheby_order);
         snprintf(nm, 32, "CHEB_COEF%d", l);
         rec(nm, 1, ord, coefs[l]);
         double eig[2] = {hypre_ParAMGDataMaxEigEst(amg_data)[l], hypre_ParAMGDataMinEigEst(amg_data)[l]};
         snprintf(nm, 32, "CHEB_EIG%d", l);
         rec(nm, 1, 2, eig);
         hypre_Vector **ds = hypre_ParAMGDataChebyDS(amg_data);
         if (ds && ds[l] && hypre_VectorData(ds[l]))
         {
            snprintf(nm, 32, "CHEB_DS%d", l);
            rec(nm, 1, lev_rows[l], hypre_VectorData(ds[l]));
         }
      }
      hypre_Vector **l1 = hypre_ParAMGDataL1Norms(amg_data);
      if (l1 && l1[l])
      {
         char nm[32];
         snprintf(nm, 32, "L1_%d", l);
         rec(nm, 1, lev_rows[l], hypre_VectorData(l1[l]));
      }
   }
   rec("lev_rows", 0, nlev, lev_rows);
   rec("lev_nnz", 0, nlev, lev_nnz);
   fclose(g_out);
   printf("levels %d iters %d final_relres %.6e setup %.4f s solve %.4f s\n",
          nlev, iters, final_res, t_setup, t_solve);
   for (int l = 0; l < nlev; l++) { printf("  level %d rows %d nnz %d\n", l, lev_rows[l], lev_nnz[l]); }
   return 0;
}
