// Pass-kernel instantiations for axis lengths 384.
#include "instantiate.cuh"
WDM_INSTANTIATE(384)
