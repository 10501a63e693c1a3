// Kernel instantiations for N = 192, 256.
#include "d2z_launch.cuh"
PRC_INSTANTIATE(192)
PRC_INSTANTIATE(256)
