// Pass-kernel instantiations for axis lengths 128,192.
#include "instantiate.cuh"
WDM_INSTANTIATE(128)
WDM_INSTANTIATE(192)
