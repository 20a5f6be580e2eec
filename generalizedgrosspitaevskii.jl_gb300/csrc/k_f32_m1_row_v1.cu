// Instantiates the alternative-tiling row kernels (V = 1) for FP32 fields with one
// component: 8 points a thread in the row pass, 16 in the column pass.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_ROW_V(float, 1, 1)
}  // namespace gpe
