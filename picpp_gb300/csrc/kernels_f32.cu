// FP32 particle-state instantiation of the particle and Yee kernels.
#include "kernels_impl.cuh"
template struct pic::PK<float>;
