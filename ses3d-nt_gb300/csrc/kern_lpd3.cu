// Kernels for lpd = 3 (FP32 and FP64).
#include "kernels.cuh"
SESNT_INSTANTIATE_LPD(3)
