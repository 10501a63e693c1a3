// Kernel instantiations for N = 512.
#include "d2z_launch.cuh"
PRC_INSTANTIATE(512)
