// FP32 population storage instantiation of the step kernels.
#include "lbmx_kernels.cuh"
namespace lbmx {
LBMX_INSTANTIATE(float)
}
