// Kernels for lpd = 7 (FP32 and FP64).
#include "kernels.cuh"
SESNT_INSTANTIATE_LPD(7)
