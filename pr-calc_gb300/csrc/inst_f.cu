// Kernel instantiations for N = 384, 768 (three times a power of two).
#include "d2z_launch.cuh"
PRC_INSTANTIATE(384)
PRC_INSTANTIATE(768)
