// BF16 offset (f - w) population storage instantiation of the batched step kernels.
#include "lbmx_batch_kernels.cuh"
namespace lbmx {
LBMX_INSTANTIATE_BATCH(__nv_bfloat16)
}
