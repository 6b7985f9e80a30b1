// Pass-kernel instantiations for axis lengths 512.
#include "instantiate.cuh"
WDM_INSTANTIATE(512)
