// Instantiates the line passes for float fields with 2 component(s); one
// translation unit per (precision, M) so the build compiles them in parallel.
#include "passes.cuh"
namespace gpe {
GPE_INSTANTIATE(float, 2)
}  // namespace gpe
