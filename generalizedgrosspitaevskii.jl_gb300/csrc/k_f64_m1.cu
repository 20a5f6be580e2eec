// Instantiates the line passes for double fields with 1 component(s); one
// translation unit per (precision, M) so the build compiles them in parallel.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE(double, 1)
}  // namespace gpe
