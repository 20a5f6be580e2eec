// Instantiates the other kernels for double-word FP64 fields with 2 component(s); the
// kernels are split over many small translation units so the build runs in parallel.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE_OTHER(DWR, 2)
GPE_INSTANTIATE_MAT(DWR)
}  // namespace gpe
