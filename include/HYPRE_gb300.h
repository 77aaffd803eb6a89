/* HYPRE_gb300.h -- C ABI of libHYPRE_gb300.so, a single-GPU (GB300, sm_103a)
 * drop-in for the reference library's IJ / ParCSR / BoomerAMG / PCG / FlexGMRES
 * path.  Names, argument meaning, return values (the sticky error flag) and
 * defaults follow the reference headers cited beside each declaration
 * (paths relative to the reference project's root).  Types: HYPRE_Int and
 * HYPRE_BigInt are 32-bit, HYPRE_Real / HYPRE_Complex are double, the default
 * non-mixed-int build of the reference.
 *
 * Scope: one process, one GPU.  MPI_Comm is accepted and ignored (an opaque
 * integer here); every ParCSR matrix has an empty off-diagonal block.  All
 * matrix and vector data handed out as objects live in device memory.
 */
#ifndef HYPRE_GB300_H
#define HYPRE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- basic types: src/utilities/HYPRE_utilities.h:40-120 ----------------- */
typedef int    HYPRE_Int;
typedef int    HYPRE_BigInt;
typedef double HYPRE_Real;
typedef double HYPRE_Complex;
#ifndef HYPRE_GB300_MPI_COMM_DEFINED
#define HYPRE_GB300_MPI_COMM_DEFINED
typedef int    MPI_Comm;           /* stands in for the MPI communicator; ignored */
#endif
#define hypre_MPI_COMM_WORLD 0

/* error codes: src/utilities/HYPRE_utilities.h:273-277 */
#define HYPRE_ERROR_GENERIC  1
#define HYPRE_ERROR_MEMORY   2
#define HYPRE_ERROR_ARG      4
#define HYPRE_ERROR_CONV   256

/* object type tag: src/HYPRE.h:33 */
#define HYPRE_PARCSR 5555

/* src/utilities/HYPRE_utilities.h:461-466 */
typedef enum _HYPRE_MemoryLocation
{
   HYPRE_MEMORY_UNDEFINED = -1,
   HYPRE_MEMORY_HOST,
   HYPRE_MEMORY_DEVICE
} HYPRE_MemoryLocation;

/* src/utilities/HYPRE_utilities.h:493-498 */
typedef enum _HYPRE_ExecutionPolicy
{
   HYPRE_EXEC_UNDEFINED = -1,
   HYPRE_EXEC_HOST,
   HYPRE_EXEC_DEVICE
} HYPRE_ExecutionPolicy;

/* opaque handles: src/utilities/HYPRE_utilities.h:730-738, IJ_mv/HYPRE_IJ_mv.h,
 * parcsr_mv/HYPRE_parcsr_mv.h */
typedef struct hypre_Solver_struct        *HYPRE_Solver;
typedef struct hypre_Matrix_struct        *HYPRE_Matrix;
typedef struct hypre_Vector_struct        *HYPRE_Vector;
typedef struct hypre_IJMatrix_struct      *HYPRE_IJMatrix;
typedef struct hypre_IJVector_struct      *HYPRE_IJVector;
typedef struct hypre_ParCSRMatrix_struct  *HYPRE_ParCSRMatrix;
typedef struct hypre_ParVector_struct     *HYPRE_ParVector;

/* preconditioner plug-in: src/utilities/HYPRE_utilities.h:749 */
typedef HYPRE_Int (*HYPRE_PtrToSolverFcn)(HYPRE_Solver, HYPRE_Matrix, HYPRE_Vector, HYPRE_Vector);
typedef HYPRE_Int (*HYPRE_PtrToParSolverFcn)(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector);

/* --- runtime: src/utilities/HYPRE_utilities.h ----------------------------- */
HYPRE_Int HYPRE_Initialize(void);                                          /* :341 */
HYPRE_Int HYPRE_Finalize(void);                                            /* :357 */
HYPRE_Int HYPRE_GetError(void);                                            /* :289 */
HYPRE_Int HYPRE_CheckError(HYPRE_Int hypre_ierr, HYPRE_Int hypre_error_code); /* :292 */
HYPRE_Int HYPRE_GetErrorArg(void);                                         /* :298 */
void      HYPRE_DescribeError(HYPRE_Int hypre_ierr, char *descr);          /* :301 */
HYPRE_Int HYPRE_ClearAllErrors(void);                                      /* :304 */
HYPRE_Int HYPRE_SetMemoryLocation(HYPRE_MemoryLocation memory_location);   /* :473, accepted, device only */
HYPRE_Int HYPRE_GetMemoryLocation(HYPRE_MemoryLocation *memory_location);  /* :478 */
HYPRE_Int HYPRE_SetExecutionPolicy(HYPRE_ExecutionPolicy exec_policy);     /* :504, accepted, device only */
HYPRE_Int HYPRE_SetSpMVUseVendor(HYPRE_Int use_vendor);                    /* :660, accepted, ignored */
HYPRE_Int HYPRE_SetSpGemmUseVendor(HYPRE_Int use_vendor);                  /* :679, accepted, ignored */
HYPRE_Int HYPRE_SetUseGpuRand(HYPRE_Int use_gpurand);                      /* :699, accepted, ignored */

/* --- IJ matrix: src/IJ_mv/HYPRE_IJ_mv.h ------------------------------------ */
HYPRE_Int HYPRE_IJMatrixCreate(MPI_Comm comm, HYPRE_BigInt ilower, HYPRE_BigInt iupper,
                               HYPRE_BigInt jlower, HYPRE_BigInt jupper, HYPRE_IJMatrix *matrix); /* :70 */
HYPRE_Int HYPRE_IJMatrixDestroy(HYPRE_IJMatrix matrix);                   /* :86 */
HYPRE_Int HYPRE_IJMatrixInitialize(HYPRE_IJMatrix matrix);                /* :93 */
HYPRE_Int HYPRE_IJMatrixInitialize_v2(HYPRE_IJMatrix matrix, HYPRE_MemoryLocation memory_location); /* :101 */
HYPRE_Int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix matrix, HYPRE_Int nrows, HYPRE_Int *ncols,
                                  const HYPRE_BigInt *rows, const HYPRE_BigInt *cols,
                                  const HYPRE_Complex *values);            /* :129 */
HYPRE_Int HYPRE_IJMatrixAddToValues(HYPRE_IJMatrix matrix, HYPRE_Int nrows, HYPRE_Int *ncols,
                                    const HYPRE_BigInt *rows, const HYPRE_BigInt *cols,
                                    const HYPRE_Complex *values);          /* :160 */
HYPRE_Int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix matrix);                  /* :202 */
HYPRE_Int HYPRE_IJMatrixGetValues(HYPRE_IJMatrix matrix, HYPRE_Int nrows, HYPRE_Int *ncols,
                                  HYPRE_BigInt *rows, HYPRE_BigInt *cols, HYPRE_Complex *values); /* :222 */
HYPRE_Int HYPRE_IJMatrixSetObjectType(HYPRE_IJMatrix matrix, HYPRE_Int type); /* :268 */
HYPRE_Int HYPRE_IJMatrixGetLocalRange(HYPRE_IJMatrix matrix, HYPRE_BigInt *ilower, HYPRE_BigInt *iupper,
                                      HYPRE_BigInt *jlower, HYPRE_BigInt *jupper); /* :281 */
HYPRE_Int HYPRE_IJMatrixGetObject(HYPRE_IJMatrix matrix, void **object);  /* :310 */
HYPRE_Int HYPRE_IJMatrixSetRowSizes(HYPRE_IJMatrix matrix, const HYPRE_Int *sizes); /* :321 */
HYPRE_Int HYPRE_IJMatrixSetDiagOffdSizes(HYPRE_IJMatrix matrix, const HYPRE_Int *diag_sizes,
                                         const HYPRE_Int *offdiag_sizes);  /* :336 */
/* files, one process: "<filename>.00000" (IJ text), "<filename>" (Matrix
 * Market coordinate real/integer, general or symmetric), "<filename>.00000.bin"
 * (binary IJ, 32- or 64-bit indices, FP32 or FP64 values); type HYPRE_PARCSR */
HYPRE_Int HYPRE_IJMatrixRead(const char *filename, MPI_Comm comm, HYPRE_Int type,
                             HYPRE_IJMatrix *matrix);                      /* :406 */
HYPRE_Int HYPRE_IJMatrixReadMM(const char *filename, MPI_Comm comm, HYPRE_Int type,
                               HYPRE_IJMatrix *matrix);                    /* :414 */
HYPRE_Int HYPRE_IJMatrixPrint(HYPRE_IJMatrix matrix, const char *filename); /* :422 */
HYPRE_Int HYPRE_IJMatrixPrintBinary(HYPRE_IJMatrix matrix, const char *filename); /* :452 */
HYPRE_Int HYPRE_IJMatrixReadBinary(const char *filename, MPI_Comm comm, HYPRE_Int type,
                                   HYPRE_IJMatrix *matrix);                /* :458 */

/* --- IJ vector: src/IJ_mv/HYPRE_IJ_mv.h ------------------------------------ */
HYPRE_Int HYPRE_IJVectorCreate(MPI_Comm comm, HYPRE_BigInt jlower, HYPRE_BigInt jupper,
                               HYPRE_IJVector *vector);                    /* :499 */
HYPRE_Int HYPRE_IJVectorDestroy(HYPRE_IJVector vector);                   /* :513 */
HYPRE_Int HYPRE_IJVectorInitialize(HYPRE_IJVector vector);                /* :563 */
HYPRE_Int HYPRE_IJVectorInitialize_v2(HYPRE_IJVector vector, HYPRE_MemoryLocation memory_location); /* :571 */
HYPRE_Int HYPRE_IJVectorSetNumComponents(HYPRE_IJVector vector, HYPRE_Int num_components); /* :590 */
HYPRE_Int HYPRE_IJVectorSetValues(HYPRE_IJVector vector, HYPRE_Int nvalues,
                                  const HYPRE_BigInt *indices, const HYPRE_Complex *values); /* :613 */
HYPRE_Int HYPRE_IJVectorAddToValues(HYPRE_IJVector vector, HYPRE_Int nvalues,
                                    const HYPRE_BigInt *indices, const HYPRE_Complex *values); /* :633 */
HYPRE_Int HYPRE_IJVectorAssemble(HYPRE_IJVector vector);                  /* :645 */
HYPRE_Int HYPRE_IJVectorGetValues(HYPRE_IJVector vector, HYPRE_Int nvalues,
                                  const HYPRE_BigInt *indices, HYPRE_Complex *values); /* :667 */
HYPRE_Int HYPRE_IJVectorSetObjectType(HYPRE_IJVector vector, HYPRE_Int type); /* :680 */
HYPRE_Int HYPRE_IJVectorGetObject(HYPRE_IJVector vector, void **object);  /* :701 */
HYPRE_Int HYPRE_IJVectorGetLocalRange(HYPRE_IJVector vector, HYPRE_BigInt *jlower,
                                      HYPRE_BigInt *jupper);               /* :692 */
/* the rest of the IJ interface for one process: object types, row counts,
 * constant values, the inner product of two IJ vectors; the off-process,
 * print, thread and memory-location settings are accepted (one process, data
 * on the device) */
HYPRE_Int HYPRE_IJMatrixGetObjectType(HYPRE_IJMatrix matrix, HYPRE_Int *type); /* HYPRE_IJ_mv.h:274 */
HYPRE_Int HYPRE_IJMatrixGetRowCounts(HYPRE_IJMatrix matrix, HYPRE_Int nrows, HYPRE_BigInt *rows,
                                     HYPRE_Int *ncols); /* :209 */
HYPRE_Int HYPRE_IJMatrixSetConstantValues(HYPRE_IJMatrix matrix, HYPRE_Complex value); /* :140 */
HYPRE_Int HYPRE_IJMatrixSetMaxOffProcElmts(HYPRE_IJMatrix matrix, HYPRE_Int max_off_proc_elmts); /* :348 */
HYPRE_Int HYPRE_IJMatrixSetPrintLevel(HYPRE_IJMatrix matrix, HYPRE_Int print_level); /* :382 */
HYPRE_Int HYPRE_IJMatrixSetOMPFlag(HYPRE_IJMatrix matrix, HYPRE_Int omp_flag); /* :400 */
HYPRE_Int HYPRE_IJMatrixMigrate(HYPRE_IJMatrix matrix, HYPRE_MemoryLocation memory_location); /* :466 */
HYPRE_Int HYPRE_IJVectorGetObjectType(HYPRE_IJVector vector, HYPRE_Int *type); /* :686 */
HYPRE_Int HYPRE_IJVectorSetConstantValues(HYPRE_IJVector vector, HYPRE_Complex value); /* :621 */
HYPRE_Int HYPRE_IJVectorInnerProd(HYPRE_IJVector x, HYPRE_IJVector y, HYPRE_Real *prod); /* :743 */
HYPRE_Int HYPRE_IJVectorSetMaxOffProcElmts(HYPRE_IJVector vector, HYPRE_Int max_off_proc_elmts); /* :582 */
HYPRE_Int HYPRE_IJVectorSetPrintLevel(HYPRE_IJVector vector, HYPRE_Int print_level); /* :709 */
HYPRE_Int HYPRE_IJVectorMigrate(HYPRE_IJVector vector, HYPRE_MemoryLocation memory_location); /* :750 */
HYPRE_Int HYPRE_IJVectorRead(const char *filename, MPI_Comm comm, HYPRE_Int type,
                             HYPRE_IJVector *vector);                      /* :715 */
HYPRE_Int HYPRE_IJVectorReadBinary(const char *filename, MPI_Comm comm, HYPRE_Int type,
                                   HYPRE_IJVector *vector);                /* :723 */
HYPRE_Int HYPRE_IJVectorPrint(HYPRE_IJVector vector, const char *filename); /* :731 */
HYPRE_Int HYPRE_IJVectorPrintBinary(HYPRE_IJVector vector, const char *filename); /* :737 */

/* --- ParCSR matrix / vector: src/parcsr_mv/HYPRE_parcsr_mv.h --------------- */
HYPRE_Int HYPRE_ParCSRMatrixGetDims(HYPRE_ParCSRMatrix matrix, HYPRE_BigInt *M, HYPRE_BigInt *N); /* :105 */
HYPRE_Int HYPRE_ParCSRMatrixGetLocalRange(HYPRE_ParCSRMatrix matrix, HYPRE_BigInt *row_start,
                                          HYPRE_BigInt *row_end, HYPRE_BigInt *col_start,
                                          HYPRE_BigInt *col_end);          /* :123 */
/* one row in host memory, diagonal first; one active row at a time */
HYPRE_Int HYPRE_ParCSRMatrixGetRow(HYPRE_ParCSRMatrix matrix, HYPRE_BigInt row, HYPRE_Int *size,
                                   HYPRE_BigInt **col_ind, HYPRE_Complex **values);   /* :130 */
HYPRE_Int HYPRE_ParCSRMatrixRestoreRow(HYPRE_ParCSRMatrix matrix, HYPRE_BigInt row, HYPRE_Int *size,
                                       HYPRE_BigInt **col_ind, HYPRE_Complex **values); /* :137 */
HYPRE_Int HYPRE_ParCSRMatrixMatvec(HYPRE_Complex alpha, HYPRE_ParCSRMatrix A, HYPRE_ParVector x,
                                   HYPRE_Complex beta, HYPRE_ParVector y); /* :285 */
HYPRE_Int HYPRE_ParCSRMatrixMatvecT(HYPRE_Complex alpha, HYPRE_ParCSRMatrix A, HYPRE_ParVector x,
                                    HYPRE_Complex beta, HYPRE_ParVector y); /* :295 */
/* C = A * B with the reference's column order and summation order (the
 * single-process CSR product); the caller owns C */
HYPRE_Int HYPRE_ParCSRMatrixMatmat(HYPRE_ParCSRMatrix A, HYPRE_ParCSRMatrix B,
                                   HYPRE_ParCSRMatrix *C);                 /* :305 */
HYPRE_Int HYPRE_ParCSRMatrixDestroy(HYPRE_ParCSRMatrix matrix);           /* :75 */
/* ParVector text files of one process (<name>.0 with the size and %.14e values,
 * <name>.INFO.0 with the global size and row range) and values by index */
HYPRE_Int HYPRE_ParVectorPrint(HYPRE_ParVector vector, const char *file_name); /* HYPRE_parcsr_mv.h:209 */
HYPRE_Int HYPRE_ParVectorRead(MPI_Comm comm, const char *file_name, HYPRE_ParVector *vector); /* :201 */
HYPRE_Int HYPRE_ParVectorGetValues(HYPRE_ParVector vector, HYPRE_Int num_values, HYPRE_BigInt *indices,
                                   HYPRE_Complex *values); /* :331 */
/* ParCSR text files of one process (<name>.D.0: row count, 1-based row
 * pointers and columns, %.14e values; <name>.INFO.0: sizes and ranges; Read
 * takes square matrices) */
HYPRE_Int HYPRE_ParCSRMatrixPrint(HYPRE_ParCSRMatrix matrix, const char *file_name); /* HYPRE_parcsr_mv.h:95 */
HYPRE_Int HYPRE_ParCSRMatrixRead(MPI_Comm comm, const char *file_name, HYPRE_ParCSRMatrix *matrix); /* :87 */
HYPRE_Int HYPRE_ParVectorCreate(MPI_Comm comm, HYPRE_BigInt global_size, HYPRE_BigInt *partitioning,
                                HYPRE_ParVector *vector);                  /* :179 */
HYPRE_Int HYPRE_ParVectorDestroy(HYPRE_ParVector vector);                 /* :188 */
HYPRE_Int HYPRE_ParVectorInitialize(HYPRE_ParVector vector);              /* :195 */
HYPRE_Int HYPRE_ParVectorSetConstantValues(HYPRE_ParVector vector, HYPRE_Complex value); /* :226 */
HYPRE_Int HYPRE_ParVectorSetRandomValues(HYPRE_ParVector vector, HYPRE_Int seed); /* :230 */
HYPRE_Int HYPRE_ParVectorCopy(HYPRE_ParVector x, HYPRE_ParVector y);      /* :255 */
HYPRE_Int HYPRE_ParVectorScale(HYPRE_Complex value, HYPRE_ParVector x);   /* :262 */
HYPRE_Int HYPRE_ParVectorAxpy(HYPRE_Complex alpha, HYPRE_ParVector x, HYPRE_ParVector y); /* :269 */
HYPRE_Int HYPRE_ParVectorInnerProd(HYPRE_ParVector x, HYPRE_ParVector y, HYPRE_Real *prod); /* :277 */

/* --- BoomerAMG: src/parcsr_ls/HYPRE_parcsr_ls.h ---------------------------- */
HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *solver);                     /* :71 */
HYPRE_Int HYPRE_BoomerAMGDestroy(HYPRE_Solver solver);                     /* :76 */
HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                               HYPRE_ParVector b, HYPRE_ParVector x);      /* :88 */
HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                               HYPRE_ParVector b, HYPRE_ParVector x);      /* :103 */
HYPRE_Int HYPRE_BoomerAMGGetNumIterations(HYPRE_Solver solver, HYPRE_Int *num_iterations); /* :143 */
HYPRE_Int HYPRE_BoomerAMGGetFinalRelativeResidualNorm(HYPRE_Solver solver, HYPRE_Real *rel_resid_norm); /* :164 */
HYPRE_Int HYPRE_BoomerAMGSetTol(HYPRE_Solver solver, HYPRE_Real tol);      /* :219 */
HYPRE_Int HYPRE_BoomerAMGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter); /* :229 */
HYPRE_Int HYPRE_BoomerAMGSetMaxCoarseSize(HYPRE_Solver solver, HYPRE_Int max_coarse_size); /* :244 */
HYPRE_Int HYPRE_BoomerAMGSetMinCoarseSize(HYPRE_Solver solver, HYPRE_Int min_coarse_size); /* :253 */
HYPRE_Int HYPRE_BoomerAMGSetMaxLevels(HYPRE_Solver solver, HYPRE_Int max_levels); /* :262 */
HYPRE_Int HYPRE_BoomerAMGSetStrongThreshold(HYPRE_Solver solver, HYPRE_Real strong_threshold); /* :286 */
HYPRE_Int HYPRE_BoomerAMGSetMaxRowSum(HYPRE_Solver solver, HYPRE_Real max_row_sum); /* :324 */
HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver solver, HYPRE_Int coarsen_type); /* :351 */
HYPRE_Int HYPRE_BoomerAMGSetAggNumLevels(HYPRE_Solver solver, HYPRE_Int agg_num_levels); /* :415 */
HYPRE_Int HYPRE_BoomerAMGSetNumPaths(HYPRE_Solver solver, HYPRE_Int num_paths); /* :423 */
HYPRE_Int HYPRE_BoomerAMGSetInterpType(HYPRE_Solver solver, HYPRE_Int interp_type); /* :502 */
HYPRE_Int HYPRE_BoomerAMGSetTruncFactor(HYPRE_Solver solver, HYPRE_Real trunc_factor); /* :516 */
HYPRE_Int HYPRE_BoomerAMGSetPMaxElmts(HYPRE_Solver solver, HYPRE_Int P_max_elmts); /* :525 */
HYPRE_Int HYPRE_BoomerAMGSetAggInterpType(HYPRE_Solver solver, HYPRE_Int agg_interp_type); /* :553 */
HYPRE_Int HYPRE_BoomerAMGSetAggTruncFactor(HYPRE_Solver solver, HYPRE_Real agg_trunc_factor); /* :561 */
HYPRE_Int HYPRE_BoomerAMGSetAggPMaxElmts(HYPRE_Solver solver, HYPRE_Int agg_P_max_elmts); /* :577 */
HYPRE_Int HYPRE_BoomerAMGSetAggP12TruncFactor(HYPRE_Solver solver, HYPRE_Real agg_P12_trunc_factor); /* :569 */
HYPRE_Int HYPRE_BoomerAMGSetAggP12MaxElmts(HYPRE_Solver solver, HYPRE_Int agg_P12_max_elmts); /* :585 */
/* getters of the stored parameters, and settings with one supported value
 * (others are refused with HYPRE_ERROR_GENERIC); MinIter bounds the
 * stand-alone solve's cycles from below */
HYPRE_Int HYPRE_BoomerAMGSetMinIter(HYPRE_Solver solver, HYPRE_Int min_iter); /* :237 */
HYPRE_Int HYPRE_BoomerAMGGetMaxIter(HYPRE_Solver solver, HYPRE_Int *max_iter); /* :232 */
HYPRE_Int HYPRE_BoomerAMGGetTol(HYPRE_Solver solver, HYPRE_Real *tol); /* :222 */
HYPRE_Int HYPRE_BoomerAMGGetCycleType(HYPRE_Solver solver, HYPRE_Int *cycle_type); /* :656 */
HYPRE_Int HYPRE_BoomerAMGGetFCycle(HYPRE_Solver solver, HYPRE_Int *fcycle); /* :665 */
HYPRE_Int HYPRE_BoomerAMGGetStrongThreshold(HYPRE_Solver solver, HYPRE_Real *strong_threshold); /* :289 */
HYPRE_Int HYPRE_BoomerAMGGetMaxRowSum(HYPRE_Solver solver, HYPRE_Real *max_row_sum);
HYPRE_Int HYPRE_BoomerAMGGetPMaxElmts(HYPRE_Solver solver, HYPRE_Int *P_max_elmts);
HYPRE_Int HYPRE_BoomerAMGGetTruncFactor(HYPRE_Solver solver, HYPRE_Real *trunc_factor);
HYPRE_Int HYPRE_BoomerAMGGetMaxLevels(HYPRE_Solver solver, HYPRE_Int *max_levels);
HYPRE_Int HYPRE_BoomerAMGGetMaxCoarseSize(HYPRE_Solver solver, HYPRE_Int *max_coarse_size);
HYPRE_Int HYPRE_BoomerAMGGetMinCoarseSize(HYPRE_Solver solver, HYPRE_Int *min_coarse_size);
HYPRE_Int HYPRE_BoomerAMGGetCoarsenType(HYPRE_Solver solver, HYPRE_Int *coarsen_type);
HYPRE_Int HYPRE_BoomerAMGGetPrintLevel(HYPRE_Solver solver, HYPRE_Int *print_level);
HYPRE_Int HYPRE_BoomerAMGGetLogging(HYPRE_Solver solver, HYPRE_Int *logging);
HYPRE_Int HYPRE_BoomerAMGGetCycleNumSweeps(HYPRE_Solver solver, HYPRE_Int *num_sweeps, HYPRE_Int k); /* :821 */
HYPRE_Int HYPRE_BoomerAMGGetCycleRelaxType(HYPRE_Solver solver, HYPRE_Int *relax_type, HYPRE_Int k); /* :907 */
HYPRE_Int HYPRE_BoomerAMGGetNumFunctions(HYPRE_Solver solver, HYPRE_Int *num_functions); /* :174 */
HYPRE_Int HYPRE_BoomerAMGSetNumFunctions(HYPRE_Solver solver, HYPRE_Int num_functions); /* :171 */
HYPRE_Int HYPRE_BoomerAMGSetNodal(HYPRE_Solver solver, HYPRE_Int nodal); /* :446 */
HYPRE_Int HYPRE_BoomerAMGSetMeasureType(HYPRE_Solver solver, HYPRE_Int measure_type); /* :405 */
HYPRE_Int HYPRE_BoomerAMGSetRedundant(HYPRE_Solver solver, HYPRE_Int redundant); /* :785 */
HYPRE_Int HYPRE_BoomerAMGSetCoarsenCutFactor(HYPRE_Solver solver, HYPRE_Int coarsen_cut_factor); /* :274 */
HYPRE_Int HYPRE_BoomerAMGSetConvergeType(HYPRE_Solver solver, HYPRE_Int type); /* :208 */
HYPRE_Int HYPRE_BoomerAMGSetDebugFlag(HYPRE_Solver solver, HYPRE_Int debug_flag); /* :1521 */
HYPRE_Int HYPRE_BoomerAMGSetSeqThreshold(HYPRE_Solver solver, HYPRE_Int seq_threshold); /* :775 */
HYPRE_Int HYPRE_BoomerAMGSetOuterWt(HYPRE_Solver solver, HYPRE_Real omega); /* :991 (omega > 0) */
HYPRE_Int HYPRE_BoomerAMGSetCycleType(HYPRE_Solver solver, HYPRE_Int cycle_type); /* :653 */
HYPRE_Int HYPRE_BoomerAMGSetFCycle(HYPRE_Solver solver, HYPRE_Int fcycle); /* :662 */
HYPRE_Int HYPRE_BoomerAMGSetNumSweeps(HYPRE_Solver solver, HYPRE_Int num_sweeps); /* :806 */
HYPRE_Int HYPRE_BoomerAMGSetCycleNumSweeps(HYPRE_Solver solver, HYPRE_Int num_sweeps, HYPRE_Int k); /* :817 */
HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver solver, HYPRE_Int relax_type); /* :877 */
HYPRE_Int HYPRE_BoomerAMGSetCycleRelaxType(HYPRE_Solver solver, HYPRE_Int relax_type, HYPRE_Int k); /* :903 */
HYPRE_Int HYPRE_BoomerAMGSetRelaxOrder(HYPRE_Solver solver, HYPRE_Int relax_order); /* :923 */
HYPRE_Int HYPRE_BoomerAMGSetRelaxWt(HYPRE_Solver solver, HYPRE_Real relax_weight); /* :957 */
HYPRE_Int HYPRE_BoomerAMGSetLevelRelaxWt(HYPRE_Solver solver, HYPRE_Real relax_weight, HYPRE_Int level); /* :967 */
HYPRE_Int HYPRE_BoomerAMGSetChebyOrder(HYPRE_Solver solver, HYPRE_Int order); /* :1008 */
HYPRE_Int HYPRE_BoomerAMGSetChebyFraction(HYPRE_Solver solver, HYPRE_Real ratio); /* :1014 */
HYPRE_Int HYPRE_BoomerAMGSetChebyScale(HYPRE_Solver solver, HYPRE_Int scale); /* :1020 */
HYPRE_Int HYPRE_BoomerAMGSetChebyVariant(HYPRE_Solver solver, HYPRE_Int variant); /* :1026 */
HYPRE_Int HYPRE_BoomerAMGSetChebyEigEst(HYPRE_Solver solver, HYPRE_Int eig_est); /* :1032 */
HYPRE_Int HYPRE_BoomerAMGSetPrintLevel(HYPRE_Solver solver, HYPRE_Int print_level); /* :1503 */
HYPRE_Int HYPRE_BoomerAMGSetLogging(HYPRE_Solver solver, HYPRE_Int logging); /* :1513 */
HYPRE_Int HYPRE_BoomerAMGSetRAP2(HYPRE_Solver solver, HYPRE_Int rap2);     /* :1541, accepted */
HYPRE_Int HYPRE_BoomerAMGSetModuleRAP2(HYPRE_Solver solver, HYPRE_Int mod_rap2); /* :1549, accepted */
HYPRE_Int HYPRE_BoomerAMGSetKeepTranspose(HYPRE_Solver solver, HYPRE_Int keepTranspose); /* :1557, accepted: P^T is always kept */
HYPRE_Int HYPRE_BoomerAMGGetNumLevels(HYPRE_Solver solver, HYPRE_Int *num_levels); /* no public counterpart: the reference reads hypre_ParAMGDataNumLevels, src/parcsr_ls/par_amg.h */

/* --- generic Krylov: src/krylov/HYPRE_krylov.h ----------------------------- */
HYPRE_Int HYPRE_PCGSetup(HYPRE_Solver solver, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x); /* :63 */
HYPRE_Int HYPRE_PCGSolve(HYPRE_Solver solver, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x); /* :71 */
HYPRE_Int HYPRE_PCGSetTol(HYPRE_Solver solver, HYPRE_Real tol);            /* :79 */
HYPRE_Int HYPRE_PCGSetAbsoluteTol(HYPRE_Solver solver, HYPRE_Real a_tol);  /* :89 */
HYPRE_Int HYPRE_PCGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter);    /* :121 */
HYPRE_Int HYPRE_PCGSetTwoNorm(HYPRE_Solver solver, HYPRE_Int two_norm);    /* :127 */
HYPRE_Int HYPRE_PCGSetRelChange(HYPRE_Solver solver, HYPRE_Int rel_change); /* :134 */
HYPRE_Int HYPRE_PCGSetRecomputeResidual(HYPRE_Solver solver, HYPRE_Int recompute_residual); /* :140 */
HYPRE_Int HYPRE_PCGSetPrecond(HYPRE_Solver solver, HYPRE_PtrToSolverFcn precond,
                              HYPRE_PtrToSolverFcn precond_setup, HYPRE_Solver precond_solver); /* :170 */
HYPRE_Int HYPRE_PCGSetLogging(HYPRE_Solver solver, HYPRE_Int logging);     /* :191 */
HYPRE_Int HYPRE_PCGSetPrintLevel(HYPRE_Solver solver, HYPRE_Int level);    /* :197 */
HYPRE_Int HYPRE_PCGGetNumIterations(HYPRE_Solver solver, HYPRE_Int *num_iterations); /* :203 */
HYPRE_Int HYPRE_PCGGetFinalRelativeResidualNorm(HYPRE_Solver solver, HYPRE_Real *norm); /* :209 */
HYPRE_Int HYPRE_PCGGetPrecond(HYPRE_Solver solver, HYPRE_Solver *precond_data_ptr); /* :273 */

HYPRE_Int HYPRE_FlexGMRESSetup(HYPRE_Solver solver, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x); /* :552 */
HYPRE_Int HYPRE_FlexGMRESSolve(HYPRE_Solver solver, HYPRE_Matrix A, HYPRE_Vector b, HYPRE_Vector x); /* :560 */
HYPRE_Int HYPRE_FlexGMRESSetTol(HYPRE_Solver solver, HYPRE_Real tol);      /* :568 */
HYPRE_Int HYPRE_FlexGMRESSetAbsoluteTol(HYPRE_Solver solver, HYPRE_Real a_tol); /* :579 */
HYPRE_Int HYPRE_FlexGMRESSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter); /* :595 */
HYPRE_Int HYPRE_FlexGMRESSetKDim(HYPRE_Solver solver, HYPRE_Int k_dim);    /* :601 */
HYPRE_Int HYPRE_FlexGMRESSetPrecond(HYPRE_Solver solver, HYPRE_PtrToSolverFcn precond,
                                    HYPRE_PtrToSolverFcn precond_setup, HYPRE_Solver precond_solver); /* :607 */
HYPRE_Int HYPRE_FlexGMRESSetLogging(HYPRE_Solver solver, HYPRE_Int logging); /* :615 */
HYPRE_Int HYPRE_FlexGMRESSetPrintLevel(HYPRE_Solver solver, HYPRE_Int level); /* :621 */
HYPRE_Int HYPRE_FlexGMRESGetNumIterations(HYPRE_Solver solver, HYPRE_Int *num_iterations); /* :627 */
HYPRE_Int HYPRE_FlexGMRESGetFinalRelativeResidualNorm(HYPRE_Solver solver, HYPRE_Real *norm); /* :633 */

/* --- ParCSR Krylov front ends: src/parcsr_ls/HYPRE_parcsr_ls.h ------------- */
HYPRE_Int HYPRE_ParCSRPCGCreate(MPI_Comm comm, HYPRE_Solver *solver);      /* :3162 */
HYPRE_Int HYPRE_ParCSRPCGDestroy(HYPRE_Solver solver);                     /* :3168 */
HYPRE_Int HYPRE_ParCSRPCGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                               HYPRE_ParVector b, HYPRE_ParVector x);      /* :3170 */
HYPRE_Int HYPRE_ParCSRPCGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                               HYPRE_ParVector b, HYPRE_ParVector x);      /* :3175 */
HYPRE_Int HYPRE_ParCSRPCGSetTol(HYPRE_Solver solver, HYPRE_Real tol);      /* :3180 */
HYPRE_Int HYPRE_ParCSRPCGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter); /* :3186 */
HYPRE_Int HYPRE_ParCSRPCGSetTwoNorm(HYPRE_Solver solver, HYPRE_Int two_norm); /* :3195 */
HYPRE_Int HYPRE_ParCSRPCGSetPrecond(HYPRE_Solver solver, HYPRE_PtrToParSolverFcn precond,
                                    HYPRE_PtrToParSolverFcn precond_setup,
                                    HYPRE_Solver precond_solver);           /* :3201 */
HYPRE_Int HYPRE_ParCSRPCGGetNumIterations(HYPRE_Solver solver, HYPRE_Int *num_iterations); /* :3218 */
HYPRE_Int HYPRE_ParCSRPCGGetFinalRelativeResidualNorm(HYPRE_Solver solver, HYPRE_Real *norm); /* :3221 */
HYPRE_Int HYPRE_ParCSRDiagScaleSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                                     HYPRE_ParVector y, HYPRE_ParVector x); /* :3232 */
HYPRE_Int HYPRE_ParCSRDiagScale(HYPRE_Solver solver, HYPRE_ParCSRMatrix HA,
                                HYPRE_ParVector Hy, HYPRE_ParVector Hx);   /* :3240 */

HYPRE_Int HYPRE_ParCSRFlexGMRESCreate(MPI_Comm comm, HYPRE_Solver *solver); /* :3444 */
HYPRE_Int HYPRE_ParCSRFlexGMRESDestroy(HYPRE_Solver solver);               /* :3450 */
HYPRE_Int HYPRE_ParCSRFlexGMRESSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                                     HYPRE_ParVector b, HYPRE_ParVector x); /* :3452 */
HYPRE_Int HYPRE_ParCSRFlexGMRESSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A,
                                     HYPRE_ParVector b, HYPRE_ParVector x); /* :3457 */
HYPRE_Int HYPRE_ParCSRFlexGMRESSetKDim(HYPRE_Solver solver, HYPRE_Int k_dim); /* :3462 */
HYPRE_Int HYPRE_ParCSRFlexGMRESSetTol(HYPRE_Solver solver, HYPRE_Real tol); /* :3465 */
HYPRE_Int HYPRE_ParCSRFlexGMRESSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter); /* :3477 */
HYPRE_Int HYPRE_ParCSRFlexGMRESSetPrecond(HYPRE_Solver solver, HYPRE_PtrToParSolverFcn precond,
                                          HYPRE_PtrToParSolverFcn precond_setup,
                                          HYPRE_Solver precond_solver);     /* :3481 */
HYPRE_Int HYPRE_ParCSRFlexGMRESGetNumIterations(HYPRE_Solver solver, HYPRE_Int *num_iterations); /* :3495 */
HYPRE_Int HYPRE_ParCSRFlexGMRESGetFinalRelativeResidualNorm(HYPRE_Solver solver, HYPRE_Real *norm); /* :3498 */

/* --- Batched AMG-PCG (no counterpart in the reference) ---------------------
 * Many independent systems given as the diagonal blocks of one matrix A
 * (system s owns rows system_offsets[s] .. system_offsets[s+1]-1; entries
 * outside the blocks are rejected).  Setup runs HYPRE_BoomerAMGSetup's
 * algorithm once on A with the given BoomerAMG solver's parameters (relax
 * type 18 or 7, direct coarsest solve, no aggressive levels); Solve runs an
 * FP64 PCG per system (two-norm stopping test, tolerance per system) with the
 * V-cycle in FP64 or FP32, all systems in one persistent kernel launch.  The
 * kernel shape (lanes per row 1/2/4/8, block 128/256/512) is autotuned on the
 * first Solve unless set explicitly.  Errors: HYPRE_ERROR_CONV when a system
 * does not reach the tolerance. */
HYPRE_Int HYPRE_GB300_BatchedPCGCreate(HYPRE_Solver *solver);
HYPRE_Int HYPRE_GB300_BatchedPCGDestroy(HYPRE_Solver solver);
HYPRE_Int HYPRE_GB300_BatchedPCGSetTol(HYPRE_Solver solver, HYPRE_Real tol);
HYPRE_Int HYPRE_GB300_BatchedPCGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter);
HYPRE_Int HYPRE_GB300_BatchedPCGSetCyclePrecision(HYPRE_Solver solver, HYPRE_Int precision); /* 0 FP64, 1 FP32 */
HYPRE_Int HYPRE_GB300_BatchedPCGSetKernelShape(HYPRE_Solver solver, HYPRE_Int lanes_per_row, HYPRE_Int block);
HYPRE_Int HYPRE_GB300_BatchedPCGSetAutotune(HYPRE_Solver solver, HYPRE_Int autotune);
HYPRE_Int HYPRE_GB300_BatchedPCGGetKernelShape(HYPRE_Solver solver, HYPRE_Int *lanes_per_row, HYPRE_Int *block);
HYPRE_Int HYPRE_GB300_BatchedPCGGetTuningTimes(HYPRE_Solver solver, HYPRE_Real *ms); /* 4 x 3 */
HYPRE_Int HYPRE_GB300_BatchedPCGSetup(HYPRE_Solver solver, HYPRE_Solver amg, HYPRE_ParCSRMatrix A,
                                      HYPRE_Int num_systems, const HYPRE_Int *system_offsets);
HYPRE_Int HYPRE_GB300_BatchedPCGSolve(HYPRE_Solver solver, HYPRE_ParVector b, HYPRE_ParVector x);
HYPRE_Int HYPRE_GB300_BatchedPCGGetNumIterations(HYPRE_Solver solver, HYPRE_Int *iterations);
HYPRE_Int HYPRE_GB300_BatchedPCGGetFinalRelativeResidualNorms(HYPRE_Solver solver, HYPRE_Real *relres);
HYPRE_Int HYPRE_GB300_BatchedPCGGetResidualHistory(HYPRE_Solver solver, HYPRE_Int system, HYPRE_Int maxn,
                                                   HYPRE_Real *relres, HYPRE_Int *n);
HYPRE_Int HYPRE_GB300_BatchedPCGGetLevelOffsets(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int *offsets);
/* per system: sum over levels of its nonzeros divided by its level-0 nonzeros */
HYPRE_Int HYPRE_GB300_BatchedPCGGetOperatorComplexities(HYPRE_Solver solver, HYPRE_Real *opc);

/* --- Multiple right-hand sides (extends the reference's PCG column-wise) ----
 * A multi-vector of num_vectors <= 64 columns, stored interleaved (entry
 * (i, c) at i * num_vectors + c); CopyFromHost/CopyToHost take
 * n * num_vectors values.  HYPRE_ParCSRPCGSolve on multi-vectors runs one
 * PCG per column (own scalars, stopping test and history) with every
 * product and the BoomerAMG V-cycle (relax 18 or 7, FP64 or FP32 cycle)
 * applied to all columns in one pass. */
HYPRE_Int HYPRE_GB300_ParVectorCreateMulti(HYPRE_BigInt n, HYPRE_Int num_vectors, HYPRE_ParVector *vector);
HYPRE_Int HYPRE_GB300_KrylovGetMultiNumIterations(HYPRE_Solver solver, HYPRE_Int *iterations);
HYPRE_Int HYPRE_GB300_KrylovGetMultiFinalRelativeResidualNorms(HYPRE_Solver solver, HYPRE_Real *relres);
HYPRE_Int HYPRE_GB300_KrylovGetMultiResidualHistory(HYPRE_Solver solver, HYPRE_Int column, HYPRE_Int maxn,
                                                    HYPRE_Real *relres, HYPRE_Int *n);

/* --- Learned parameters (no counterpart in the reference) ------------------
 * A per-row MLP (16 stencil features -> 64 -> 64 -> 2, ReLU, BF16 tensor-core
 * products with FP32 accumulation) predicts (strength threshold, smoother
 * weight) for each row.  With a model set, BoomerAMG setup uses the mean
 * predicted threshold over the finest level's rows (clamped to [0.1, 0.9]) and
 * sets each level's relaxation weight to the mean predicted weight over its
 * rows (clamped to [0.3, 1.5]); NULL removes the model.  params: the
 * HYPRE_GB300_MLPNumParams() FP32 values W1[64][16] b1[64] W2[64][64] b2[64]
 * W3[2][64] b3[2].  The training primitives take device pointers:
 * features n x 16 BF16, targets and out n x 2 FP32, params/grad/m/v FP32. */
HYPRE_Int HYPRE_GB300_MLPNumParams(HYPRE_Int *n);
HYPRE_Int HYPRE_GB300_BoomerAMGSetLearnedModel(HYPRE_Solver solver, const HYPRE_Real *params);
HYPRE_Int HYPRE_GB300_BoomerAMGGetLearnedParams(HYPRE_Solver solver, HYPRE_Real *theta, HYPRE_Real *weights,
                                                HYPRE_Int max_levels);
HYPRE_Int HYPRE_GB300_MLPRowFeatures(HYPRE_ParCSRMatrix A, void *features);
HYPRE_Int HYPRE_GB300_MLPForward(HYPRE_BigInt n, const void *features, const float *params, float *out);
HYPRE_Int HYPRE_GB300_MLPGradient(HYPRE_BigInt n, const void *features, const float *targets,
                                  const float *params, float *grad, float *loss);
HYPRE_Int HYPRE_GB300_MLPAdamStep(float *params, const float *grad, float *m, float *v, HYPRE_Real lr,
                                  HYPRE_Int step);

/* --- GB300 extensions (no counterpart in the reference) ------------------- */
/* Precision of the AMG V-cycle (hierarchy values, smoothers, level SpMVs);
 * setup and the outer Krylov method stay in FP64.
 *   0 = FP64 (default, reference arithmetic), 1 = FP32,
 *   2 = FP32 with FP16 values on the finest level (FP32 accumulation). */
HYPRE_Int HYPRE_GB300_BoomerAMGSetCyclePrecision(HYPRE_Solver solver, HYPRE_Int precision);
/* Capture each V-cycle as a CUDA graph and replay it (default on). */
HYPRE_Int HYPRE_GB300_BoomerAMGSetUseGraph(HYPRE_Solver solver, HYPRE_Int use_graph);
/* Hash tables of the ordered setup kernels (sparse products, second-order
 * strength, extended+i): 0 = shared-memory tiers first (default), 1 = every
 * row in global-memory tables (the path long rows take; results are the
 * same).  No counterpart in the reference. */
HYPRE_Int HYPRE_GB300_BoomerAMGSetSetupTables(HYPRE_Solver solver, HYPRE_Int mode);
/* Hierarchy inspection (host copies).  which: 0 = A, 1 = P, 2 = S (pattern).
 * nnz/rows/cols returned; arrays may be NULL to query sizes only. */
HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelCSR(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int which,
                                           HYPRE_Int *nrows, HYPRE_Int *ncols, HYPRE_Int *nnz,
                                           HYPRE_Int *rowptr, HYPRE_Int *colidx, HYPRE_Real *values);
HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelCF(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int *cf_marker);
HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelL1(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Real *l1);
/* Sparse matrix products of the last setup (the Galerkin products and the
 * aggressive level's products): algorithmic bytes (inputs read once, output
 * written once, 12 bytes per nonzero + 4 per row pointer), device seconds
 * (CUDA events on the library stream around each product) and their count. */
HYPRE_Int HYPRE_GB300_BoomerAMGGetSpGEMMStats(HYPRE_Solver solver, HYPRE_Real *bytes, HYPRE_Real *seconds,
                                              HYPRE_Int *calls);
/* SpMV launch-shape autotuner: on (1, the default unless the environment sets
 * HYPRE_GB300_AUTOTUNE=0) or off (0).  When on, each solve form of at least
 * 20,000 rows gets the fastest launch shape of its matrix shape, timed once
 * per machine and kept in a JSON cache ($HYPRE_GB300_TUNE_CACHE, else
 * $HOME/.cache/hypre_gb300/spmv_tune.json). */
HYPRE_Int HYPRE_GB300_SetAutotune(HYPRE_Int on);
/* The launch shape of a matrix's solve form in one value precision (0 FP64,
 * 1 FP32, 2 FP16): format (0 CSR, 1 SELL-32), block size, and the SELL
 * prefetch depth or the CSR lanes per row; and setting it by hand (block 0:
 * 256; depth 0: 4; lanes 0: unchanged).  Every SELL shape gives the same
 * result bit for bit; CSR lane counts differ in rounding only. */
HYPRE_Int HYPRE_GB300_ParCSRMatrixGetSpMVShape(HYPRE_ParCSRMatrix A, HYPRE_Int precision, HYPRE_Int *format,
                                               HYPRE_Int *block, HYPRE_Int *depth_or_lanes);
HYPRE_Int HYPRE_GB300_ParCSRMatrixSetSpMVShape(HYPRE_ParCSRMatrix A, HYPRE_Int precision, HYPRE_Int block,
                                               HYPRE_Int depth_or_lanes);
/* Mean device seconds of the solve-phase SpMV y = A_l x of one level in one
 * value precision (0 FP64, 1 FP32, 2 FP16 values with FP32 vectors) over
 * `reps` back-to-back launches, and its algorithmic bytes per launch. */
HYPRE_Int HYPRE_GB300_BoomerAMGLevelSpMVTime(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Int prec, HYPRE_Int reps,
                                             HYPRE_Real *seconds, HYPRE_Real *bytes);
/* Chebyshev smoother data of a level (relax type 16): the ChebyOrder
 * coefficients of s(t) in u <- u + s(A) r, eig[0..1] = max/min eigenvalue
 * estimates, ds = D^{-1/2} (n values); any pointer may be NULL. */
HYPRE_Int HYPRE_GB300_BoomerAMGGetLevelCheby(HYPRE_Solver solver, HYPRE_Int level, HYPRE_Real *coefs,
                                             HYPRE_Real *eig, HYPRE_Real *ds);
/* Relative residual history of the last Krylov solve (entries 0..iters). */
HYPRE_Int HYPRE_GB300_KrylovGetResidualHistory(HYPRE_Solver solver, HYPRE_Int maxn, HYPRE_Real *relres,
                                               HYPRE_Int *n);
/* Device data of a ParVector / sizes, for zero-copy use by callers that own
 * device memory (returns the device pointer as an integer). */
HYPRE_Int HYPRE_GB300_ParVectorGetDevicePointer(HYPRE_ParVector v, void **dptr, HYPRE_Int *n);
HYPRE_Int HYPRE_GB300_ParVectorCopyFromHost(HYPRE_ParVector v, const HYPRE_Real *h, HYPRE_Int n);
HYPRE_Int HYPRE_GB300_ParVectorCopyToHost(HYPRE_ParVector v, HYPRE_Real *h, HYPRE_Int n);
/* Build a ParCSR matrix straight from host CSR arrays (rows in the IJ order:
 * the diagonal is moved to the front of each row). */
HYPRE_Int HYPRE_GB300_ParCSRMatrixCreateFromHostCSR(HYPRE_Int n, const HYPRE_Int *rowptr,
                                                    const HYPRE_Int *colidx, const HYPRE_Real *values,
                                                    HYPRE_ParCSRMatrix *A);
/* The same from CSR arrays in device memory (copied by the library; the
 * caller keeps its arrays). */
HYPRE_Int HYPRE_GB300_ParCSRMatrixCreateFromDeviceCSR(HYPRE_Int n, const HYPRE_Int *rowptr,
                                                      const HYPRE_Int *colidx, const HYPRE_Real *values,
                                                      HYPRE_ParCSRMatrix *A);
HYPRE_Int HYPRE_GB300_ParCSRMatrixDestroy(HYPRE_ParCSRMatrix A);
/* The local CSR arrays copied to host memory (any array may be NULL).  No
 * counterpart in the reference (whose matrices are host-addressable). */
HYPRE_Int HYPRE_GB300_ParCSRMatrixCopyToHostCSR(HYPRE_ParCSRMatrix A, HYPRE_Int *nrows, HYPRE_Int *nnz,
                                               HYPRE_Int *rowptr, HYPRE_Int *colidx, HYPRE_Real *values);
/* Stream used for every kernel (default: a library-owned non-blocking stream). */
HYPRE_Int HYPRE_GB300_SetStream(void *cuda_stream);
HYPRE_Int HYPRE_GB300_GetStream(void **cuda_stream);
/* Count of this library's kernel launches since the counter was reset
 * (graph replays count every kernel node). */
HYPRE_Int HYPRE_GB300_GetKernelLaunchCount(long long *count);
HYPRE_Int HYPRE_GB300_ResetKernelLaunchCount(void);
/* y = alpha * A^T x + beta * y without allocating device memory: the transpose
 * of A is built in a fixed device array of 32 MiB compiled into the library,
 * for callers that cannot let the library allocate (code enqueuing work under
 * CUDA-graph stream capture, or hosts whose device memory is owned by another
 * allocator).  The allocating form grows the library's pool and synchronises
 * its stream; this one only enqueues work on the library's stream, whose
 * device must be the current one (else HYPRE_ERROR_GENERIC).  Matrices whose
 * transpose does not fit are rejected with HYPRE_ERROR_ARG.  All calls share
 * the array, so calls that overlap on the GPU race; the first call on a
 * device looks the array up and should come before any capture.
 * No counterpart in the reference (its MatvecT, HYPRE_ParCSRMatrixMatvecT
 * above, is the allocating form). */
HYPRE_Int HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(HYPRE_Complex alpha, HYPRE_ParCSRMatrix A, HYPRE_ParVector x,
                                                HYPRE_Complex beta, HYPRE_ParVector y);
/* Per-phase timings of the last setup (seconds, host clock; the phases end
 * at host read-backs, so they are close to device time): [0] strength [1] coarsening
 * [2] interpolation [3] RAP [4] smoother setup [5] total; [6] the number of
 * times the host waited for the stream during setup, [7] seconds spent in
 * those waits. */
HYPRE_Int HYPRE_GB300_BoomerAMGGetSetupTimes(HYPRE_Solver solver, HYPRE_Real *times, HYPRE_Int n);

#ifdef __cplusplus
}
#endif
#endif
