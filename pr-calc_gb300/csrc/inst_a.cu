// Kernel instantiations for the small grid sizes (tests and batched boxes).
#include "d2z_launch.cuh"
PRC_INSTANTIATE(8)
PRC_INSTANTIATE(12)
PRC_INSTANTIATE(16)
PRC_INSTANTIATE(24)
PRC_INSTANTIATE(32)
PRC_INSTANTIATE(48)
