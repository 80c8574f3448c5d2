// BF16 offset (f - w) population storage instantiation of the step kernels.
#include "lbmx_kernels.cuh"
namespace lbmx {
LBMX_INSTANTIATE(__nv_bfloat16)
}
