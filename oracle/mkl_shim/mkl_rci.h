/* Declarations of the Intel MKL RCI ISS FGMRES entry points the reference calls
 * (src/solverIm-cpu.cpp:218-267), served by oracle/mkl_shim.cpp.  TEST INFRASTRUCTURE. */
#ifndef NEURITE_MKL_SHIM_RCI_H
#define NEURITE_MKL_SHIM_RCI_H
typedef int MKL_INT;
void dfgmres_init(const MKL_INT *n, const double *x, const double *b, MKL_INT *RCI_request,
                  MKL_INT *ipar, double *dpar, double *tmp);
void dfgmres_check(const MKL_INT *n, const double *x, const double *b, MKL_INT *RCI_request,
                   MKL_INT *ipar, double *dpar, double *tmp);
void dfgmres(const MKL_INT *n, double *x, double *b, MKL_INT *RCI_request, MKL_INT *ipar,
             double *dpar, double *tmp);
void dfgmres_get(const MKL_INT *n, double *x, double *b, MKL_INT *RCI_request,
                 const MKL_INT *ipar, const double *dpar, double *tmp, MKL_INT *itercount);
#endif
