// Instantiates the fine-tiling row kernels (V = 2: 4 points a thread) for FP64
// fields with 2 component(s), used when a field is too small to fill the GPU.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_ROW_V(double, 2, 2)
}  // namespace gpe
