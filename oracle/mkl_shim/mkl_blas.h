/* Placeholder for <mkl_blas.h>; the reference includes it but calls nothing from it. */
#include "mkl_rci.h"
