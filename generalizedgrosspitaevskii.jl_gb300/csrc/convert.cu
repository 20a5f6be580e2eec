// convert.cu -- small device utilities: FP64 <-> double-word conversion of complex
// arrays, the step-counter advance that ends a captured chunk of steps, and the probe of
// the bounded mbarrier wait.
#include "dw.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace gpe {

// src and dst may be the same buffer: each element is read before it is written.
__global__ void f64_to_dw_kernel(const double2* src, dwc* dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = src[i];
    dst[i] = mk(dw_from(v.x), dw_from(v.y));
  }
}

__global__ void dw_to_f64_kernel(const dwc* __restrict__ src, double2* __restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const dwc v = src[i];
    dst[i] = make_double2(dw_to_double(re(v)), dw_to_double(im(v)));
  }
}

__global__ void advance_kernel(int64_t* k, int64_t n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *k += n;
}

// One CTA waits on an mbarrier of one expected arrival, with the same bounded wait the
// TMA column pass uses.  arrive = 0: nothing arrives, so the wait runs out after limit_ns
// and the kernel stores 1 in *status; arrive = 1: thread 0 arrives first and the wait
// completes at once.
__global__ void wait_probe_kernel(int arrive, uint64_t limit_ns, int32_t* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar)) : "memory");
  const bool ok = mbar_wait(&bar, 0, limit_ns);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(status, 1);
}

int launch_wait_probe(int arrive, uint64_t limit_ns, int32_t* status, cudaStream_t s) {
  wait_probe_kernel<<<1, 32, 0, s>>>(arrive, limit_ns, status);
  return (int)cudaGetLastError();
}

int launch_advance(int64_t* k, int64_t n, cudaStream_t s) {
  advance_kernel<<<1, 32, 0, s>>>(k, n);
  return (int)cudaGetLastError();
}

static unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

// *flag |= 1 when any of n values (FP64 or FP32) is NaN or Inf
template <typename T>
__global__ void nonfinite_kernel(const T* __restrict__ v, int64_t n, int* flag) {
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(v[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

int launch_nonfinite(const void* data, int64_t n, int is_f64, int* flag, cudaStream_t s) {
  if (is_f64)
    nonfinite_kernel<double><<<grid_for(n), 256, 0, s>>>((const double*)data, n, flag);
  else
    nonfinite_kernel<float><<<grid_for(n), 256, 0, s>>>((const float*)data, n, flag);
  return (int)cudaGetLastError();
}

int launch_f64_to_dw(const void* src, void* dst, int64_t n, cudaStream_t s) {
  f64_to_dw_kernel<<<grid_for(n), 256, 0, s>>>((const double2*)src, (dwc*)dst, n);
  return (int)cudaGetLastError();
}

int launch_dw_to_f64(const void* src, void* dst, int64_t n, cudaStream_t s) {
  dw_to_f64_kernel<<<grid_for(n), 256, 0, s>>>((const dwc*)src, (double2*)dst, n);
  return (int)cudaGetLastError();
}

}  // namespace gpe
