// Instantiates the resident plane kernels for double-word FP64 fields with 1 component(s).
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_PLANE(DWR, 1)
}  // namespace gpe
