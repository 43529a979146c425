// Instantiates the D*Q27 step, stream, init and codec kernels (one
// translation unit per velocity set keeps the build parallel).
#include "lbm_kernels.cuh"
namespace bf {
BF_INSTANTIATE_Q(27)
}
