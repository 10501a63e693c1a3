// Kernel instantiations for N = 1024.
#include "d2z_launch.cuh"
PRC_INSTANTIATE(1024)
