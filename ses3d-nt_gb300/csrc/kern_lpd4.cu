// Kernels for lpd = 4 (FP32 and FP64).
#include "kernels.cuh"
SESNT_INSTANTIATE_LPD(4)
