// FP64 particle-state instantiation of the particle and Yee kernels.  Built
// with --fmad=false so that every multiply and add rounds separately, as in
// the oracle: the FP64 push then reproduces the oracle operation by operation.
#include "kernels_impl.cuh"
template struct pic::PK<double>;
