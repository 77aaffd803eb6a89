/* Build configuration for compiling the reference library's CPU path directly
 * with gcc (one process, no MPI, internal BLAS/LAPACK, 32-bit ints, double
 * values; the reference's OpenMP loops when GB_REF_OPENMP is defined).
 * Written for this project's oracle recipe; the reference normally generates
 * this header from its own build system. */
#ifndef HYPRE_CONFIG_H
#define HYPRE_CONFIG_H
#define HYPRE_RELEASE_NAME    "HYPRE"
#define HYPRE_RELEASE_VERSION "3.1.0"
#define HYPRE_RELEASE_NUMBER  30100
#define HYPRE_RELEASE_DATE    "2026/01/23"
#define HYPRE_RELEASE_TIME    "00:00:00"
#define HYPRE_RELEASE_BUGS    "none"
#define HYPRE_MAXDIM 3
#define HYPRE_SEQUENTIAL 1
#define HYPRE_USING_HYPRE_BLAS 1
#define HYPRE_USING_HYPRE_LAPACK 1
#define HYPRE_USING_HOST_MEMORY 1
#ifdef GB_REF_OPENMP
#define HYPRE_USING_OPENMP 1
#endif
#define HYPRE_FMANGLE 0
#define HYPRE_FMANGLE_BLAS 0
#define HYPRE_FMANGLE_LAPACK 0
#define HYPRE_F77_FUNC(name,NAME) name ## _
#define HYPRE_F77_FUNC_(name,NAME) name ## __
#endif
