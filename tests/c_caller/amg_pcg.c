/* A C caller written against the reference's API only (the calls of
 * src/examples/ex5.c:342-400 and src/test/ij.c's AMG-PCG path), compiled
 * with gcc against include/HYPRE_gb300.h and linked with -lHYPRE_gb300 by
 * tests/test_gpu_c_caller.py.
 *
 * Problem: the 3-D 7-point Laplacian on an n^3 grid (diagonal 6, off-diagonals
 * -1, Dirichlet), assembled row by row through HYPRE_IJMatrixSetValues; the
 * right-hand side HYPRE_ParVectorSetRandomValues(b, 22775) scaled to unit
 * 2-norm, x0 = 0.  BoomerAMG (PMIS, threshold 0.25, extended+i with at most 4
 * entries per row, l1-Jacobi, coarsest level of at most 100 rows) as the
 * preconditioner of PCG to relative residual 1e-8.
 *
 * Prints: "iterations K relres R" and exits 0 when no error flag is set. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "HYPRE_gb300.h"

int main(int argc, char **argv)
{
   int nx = argc > 1 ? atoi(argv[1]) : 50;
   int n = nx * nx * nx;
   MPI_Comm comm = hypre_MPI_COMM_WORLD;

   HYPRE_Initialize();

   HYPRE_IJMatrix ij;
   HYPRE_ParCSRMatrix A;
   HYPRE_IJMatrixCreate(comm, 0, n - 1, 0, n - 1, &ij);
   HYPRE_IJMatrixSetObjectType(ij, HYPRE_PARCSR);
   int *sizes = malloc(sizeof(int) * n);
   for (int i = 0; i < n; i++) { sizes[i] = 7; }
   HYPRE_IJMatrixSetRowSizes(ij, sizes);
   HYPRE_IJMatrixInitialize(ij);
   for (int iz = 0; iz < nx; iz++)
      for (int iy = 0; iy < nx; iy++)
         for (int ix = 0; ix < nx; ix++)
         {
            HYPRE_BigInt row = ix + nx * (iy + nx * iz), cols[7];
            double vals[7];
            int nc = 0;
            cols[nc] = row; vals[nc++] = 6.0;
            if (iz > 0) { cols[nc] = row - nx * nx; vals[nc++] = -1.0; }
            if (iy > 0) { cols[nc] = row - nx; vals[nc++] = -1.0; }
            if (ix > 0) { cols[nc] = row - 1; vals[nc++] = -1.0; }
            if (ix < nx - 1) { cols[nc] = row + 1; vals[nc++] = -1.0; }
            if (iy < nx - 1) { cols[nc] = row + nx; vals[nc++] = -1.0; }
            if (iz < nx - 1) { cols[nc] = row + nx * nx; vals[nc++] = -1.0; }
            HYPRE_IJMatrixSetValues(ij, 1, &nc, &row, cols, vals);
         }
   HYPRE_IJMatrixAssemble(ij);
   HYPRE_IJMatrixGetObject(ij, (void **) &A);

   HYPRE_IJVector ijb, ijx;
   HYPRE_ParVector b, x;
   HYPRE_IJVectorCreate(comm, 0, n - 1, &ijb);
   HYPRE_IJVectorSetObjectType(ijb, HYPRE_PARCSR);
   HYPRE_IJVectorInitialize(ijb);
   HYPRE_IJVectorAssemble(ijb);
   HYPRE_IJVectorGetObject(ijb, (void **) &b);
   HYPRE_IJVectorCreate(comm, 0, n - 1, &ijx);
   HYPRE_IJVectorSetObjectType(ijx, HYPRE_PARCSR);
   HYPRE_IJVectorInitialize(ijx);
   HYPRE_IJVectorAssemble(ijx);
   HYPRE_IJVectorGetObject(ijx, (void **) &x);
   double norm;
   HYPRE_ParVectorSetRandomValues(b, 22775);
   HYPRE_ParVectorInnerProd(b, b, &norm);
   HYPRE_ParVectorScale(1.0 / sqrt(norm), b);
   HYPRE_ParVectorSetConstantValues(x, 0.0);

   HYPRE_Solver amg, pcg;
   HYPRE_BoomerAMGCreate(&amg);
   HYPRE_BoomerAMGSetCoarsenType(amg, 8);
   HYPRE_BoomerAMGSetStrongThreshold(amg, 0.25);
   HYPRE_BoomerAMGSetMaxRowSum(amg, 1.0);
   HYPRE_BoomerAMGSetInterpType(amg, 6);
   HYPRE_BoomerAMGSetPMaxElmts(amg, 4);
   HYPRE_BoomerAMGSetRelaxType(amg, 18);
   HYPRE_BoomerAMGSetNumSweeps(amg, 1);
   HYPRE_BoomerAMGSetMaxCoarseSize(amg, 100);
   HYPRE_BoomerAMGSetTol(amg, 0.0);
   HYPRE_BoomerAMGSetMaxIter(amg, 1);

   HYPRE_ParCSRPCGCreate(comm, &pcg);
   HYPRE_PCGSetMaxIter(pcg, 100);
   HYPRE_PCGSetTol(pcg, 1e-8);
   HYPRE_PCGSetTwoNorm(pcg, 1);
   HYPRE_PCGSetRelChange(pcg, 0);
   HYPRE_PCGSetLogging(pcg, 1);
   HYPRE_PCGSetPrecond(pcg, (HYPRE_PtrToSolverFcn) HYPRE_BoomerAMGSolve,
                       (HYPRE_PtrToSolverFcn) HYPRE_BoomerAMGSetup, amg);
   HYPRE_ParCSRPCGSetup(pcg, A, b, x);
   HYPRE_ParCSRPCGSolve(pcg, A, b, x);

   int its = 0;
   double rel = 0.0;
   HYPRE_PCGGetNumIterations(pcg, &its);
   HYPRE_PCGGetFinalRelativeResidualNorm(pcg, &rel);
   printf("iterations %d relres %.6e\n", its, rel);

   HYPRE_ParCSRPCGDestroy(pcg);
   HYPRE_BoomerAMGDestroy(amg);
   HYPRE_IJVectorDestroy(ijx);
   HYPRE_IJVectorDestroy(ijb);
   HYPRE_IJMatrixDestroy(ij);
   free(sizes);
   int err = HYPRE_GetError();
   HYPRE_Finalize();
   return err ? 1 : 0;
}
