// lbmx_ibm.cu -- the size of the IBM kernel's shared-memory state (the
// rounds themselves are ibm_fast_iterate, lbmx_ibm.cuh; the engine runs them
// in ibm_step_kernel, lbmx_kernels.cuh).
#include "lbmx.h"
#include "lbmx_ibm.cuh"

namespace lbmx {

size_t ibm_smem_bytes(int npatch, int nm, int stencil) { return ibm_fast_smem_bytes(npatch, nm, stencil); }

}  // namespace lbmx
