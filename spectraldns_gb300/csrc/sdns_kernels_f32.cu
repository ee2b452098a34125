// FP32 instantiation of the transform sweeps (single-precision solver).
#include "sdns_kernels.cuh"
template struct sdns::Kernels<float>;
