// FP32 population storage instantiation of the batched step kernels.
#include "lbmx_batch_kernels.cuh"
namespace lbmx {
LBMX_INSTANTIATE_BATCH(float)
}
