/* MKL_Free_Buffers as called at src/solverIm-cpu.cpp:267, served by oracle/mkl_shim.cpp. */
#ifndef NEURITE_MKL_SHIM_SERVICE_H
#define NEURITE_MKL_SHIM_SERVICE_H
void MKL_Free_Buffers(void);
#endif
