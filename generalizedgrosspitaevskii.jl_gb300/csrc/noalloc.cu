// noalloc.cu -- gpe_norms_noalloc: per-trajectory norms with no device allocation.
//
// Some callers cannot call cudaMalloc: their device memory is owned up front by another
// allocator (a framework's caching pool, a fixed budget set at start-up), or they run in
// a loop where cudaMalloc's implicit device synchronisation is not acceptable.  This
// entry point therefore takes the caller's fields and the caller's host output and uses,
// as its only scratch, the file-scope device array below.  Every GPU that loads this
// library holds the array (GPE_NOALLOC_MAX_NORMS doubles, 64 KiB) until the process exits.
//
// Host code must not hand the array's name to a kernel: in host code that name is a
// host-side stand-in, not a device address.  The first call on each device looks up the
// real address with cudaGetSymbolAddress, with that device current, and caches it.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/gpe.h"

namespace {

constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

// One slot per (component, trajectory) norm of the last call.
static __device__ __align__(256) double g_norm_scratch[GPE_NOALLOC_MAX_NORMS];

std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};

// Block (traj, comp) reduces sum |u|^2 over the npoints values of trajectory traj of
// component comp and writes it to slot comp*ntraj + traj.  Every slot of the call is
// overwritten, so nothing has to be cleared between calls.
template <typename C>
__global__ void __launch_bounds__(kThreads)
norms_kernel(const C* __restrict__ f0, const C* __restrict__ f1, int64_t npoints, int64_t ntraj, double* scratch) {
  const int64_t traj = blockIdx.x;
  const int comp = blockIdx.y;
  const C* f = (comp == 0 ? f0 : f1) + traj * npoints;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < npoints; i += kThreads) {
    const C v = f[i];
    acc += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
  }
  __shared__ double red[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) scratch[(int64_t)comp * ntraj + traj] = v;
  }
}

thread_local char g_err[256] = "";

int nerr(int code, const char* msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
  return code;
}

}  // namespace

extern "C" {

const char* gpe_noalloc_last_error(void) { return g_err; }

int gpe_norms_noalloc(const void* const* fields_dev, int ncomp, int64_t npoints, int64_t ntraj, int dtype,
                      double dV, double* out_host) {
  if (!fields_dev || !out_host) return nerr(GPE_ERR_INVALID, "null argument");
  if (ncomp < 1 || ncomp > 2) return nerr(GPE_ERR_INVALID, "ncomp must be 1 or 2");
  if (dtype != GPE_C128 && dtype != GPE_C64) return nerr(GPE_ERR_INVALID, "dtype must be GPE_C128 or GPE_C64");
  if (npoints < 1 || ntraj < 1) return nerr(GPE_ERR_INVALID, "npoints and ntraj must be positive");
  if (ntraj > 65535) return nerr(GPE_ERR_INVALID, "ntraj exceeds 65535");
  if ((int64_t)ncomp * ntraj > GPE_NOALLOC_MAX_NORMS)
    return nerr(GPE_ERR_INVALID, "ncomp * ntraj exceeds GPE_NOALLOC_MAX_NORMS (8192) scratch slots");
  for (int m = 0; m < ncomp; ++m)
    if (!fields_dev[m]) return nerr(GPE_ERR_INVALID, "null field pointer");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return nerr(GPE_ERR_CUDA, "no usable current CUDA device");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      // once per device, with that device current: the device address of the array
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_norm_scratch);
      if (e != cudaSuccess) return nerr(GPE_ERR_CUDA, cudaGetErrorString(e));
      g_scratch_addr[dev] = (double*)p;
    }
    scratch = g_scratch_addr[dev];
  }
  const dim3 grid((unsigned)ntraj, (unsigned)ncomp);
  const void* f1 = fields_dev[ncomp == 2 ? 1 : 0];
  if (dtype == GPE_C128)
    norms_kernel<double2><<<grid, kThreads>>>((const double2*)fields_dev[0], (const double2*)f1, npoints, ntraj, scratch);
  else
    norms_kernel<float2><<<grid, kThreads>>>((const float2*)fields_dev[0], (const float2*)f1, npoints, ntraj, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return nerr(GPE_ERR_CUDA, cudaGetErrorString(e));
  const size_t n = (size_t)ncomp * (size_t)ntraj;
  e = cudaMemcpy(out_host, scratch, n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return nerr(GPE_ERR_CUDA, cudaGetErrorString(e));
  for (size_t i = 0; i < n; ++i) out_host[i] *= dV;
  return GPE_OK;
}

}  // extern "C"
