// Kernels for lpd = 6 (FP32 and FP64).
#include "kernels.cuh"
SESNT_INSTANTIATE_LPD(6)
