// Instantiates the resident plane kernels for FP32 fields with 1 component(s).
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_PLANE(float, 1)
}  // namespace gpe
