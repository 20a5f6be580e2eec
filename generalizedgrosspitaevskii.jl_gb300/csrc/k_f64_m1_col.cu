// Instantiates the col kernels for native FP64 fields with 1 component(s); the
// kernels are split over many small translation units so the build runs in parallel.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_COL(double, 1)
}  // namespace gpe
