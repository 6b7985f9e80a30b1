// Pass-kernel instantiations for axis lengths 64,96.
#include "instantiate.cuh"
WDM_INSTANTIATE(64)
WDM_INSTANTIATE(96)
