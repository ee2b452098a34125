// FP64 instantiation of the transform sweeps (double-precision solver).
#include "sdns_kernels.cuh"
template struct sdns::Kernels<double>;
