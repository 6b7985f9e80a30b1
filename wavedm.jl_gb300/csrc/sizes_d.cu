// Pass-kernel instantiations for axis lengths 256.
#include "instantiate.cuh"
WDM_INSTANTIATE(256)
