// Kernel instantiations for N = 64, 96, 128.
#include "d2z_launch.cuh"
PRC_INSTANTIATE(64)
PRC_INSTANTIATE(96)
PRC_INSTANTIATE(128)
