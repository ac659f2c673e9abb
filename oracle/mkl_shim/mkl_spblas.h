/* mkl_cspblas_dcsrgemv as called at src/solverIm-cpu.cpp:245, served by oracle/mkl_shim.cpp. */
#ifndef NEURITE_MKL_SHIM_SPBLAS_H
#define NEURITE_MKL_SHIM_SPBLAS_H
#include "mkl_rci.h"
void mkl_cspblas_dcsrgemv(const char *transa, const MKL_INT *m, const double *a,
                          const MKL_INT *ia, const MKL_INT *ja, const double *x, double *y);
#endif
