// Instantiates the row kernels for FP32 fields with 2 component(s); the
// kernels are split over many small translation units so the build runs in parallel.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_ROW(float, 2)
}  // namespace gpe
