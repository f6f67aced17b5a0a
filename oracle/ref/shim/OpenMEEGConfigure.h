/* Build configuration for compiling the reference CPU path as a test oracle
 * (OpenMP on, OpenBLAS-style CBLAS/LAPACKE). */
#pragma once
static const char version[] = "2.5.16-oracle";
#if defined USE_OMP && defined _OPENMP
    #define STATIC_OMP
#else
    #define STATIC_OMP static
    #define NO_OPENMP
#endif
#define HAVE_BLAS
#define HAVE_LAPACK
#define USE_OPENBLAS
