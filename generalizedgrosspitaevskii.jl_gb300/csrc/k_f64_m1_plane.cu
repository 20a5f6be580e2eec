// Instantiates the resident plane kernels for native FP64 fields with 1 component(s).
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_PLANE(double, 1)
}  // namespace gpe
