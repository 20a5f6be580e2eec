// diag.cu -- FP64 energy reductions (gpe_energy).
//
// kinetic     sum_k Re(u~^H D(k) u~) dV / P      (u~ = unnormalised FFT of the state)
// interaction sum_r sum_j [ (1/2) sum_l Re g_jl |u_l|^2 + Re c_j ] |u_j|^2 dV
// potential   sum_r Re(u^H V(r) u) dV
// for the diagonal nonlinearity family and scalar / diagonal / matrix D and V samples
// kept in FP64.  Accumulated in FP64 whatever the field precision.
#include "passes.cuh"

namespace gpe {

__device__ __forceinline__ double2 todd(const double2& v) { return v; }
__device__ __forceinline__ double2 todd(const float2& v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 todd(const dwc& v) { return make_double2(dw_to_double(re(v)), dw_to_double(im(v))); }

__device__ __forceinline__ double re_conj_mul(double2 a, double2 d, double2 b) {
  // Re(conj(a) * d * b)
  const double dbx = d.x * b.x - d.y * b.y, dby = d.x * b.y + d.y * b.x;
  return a.x * dbx + a.y * dby;
}

__device__ __forceinline__ void block_add(double v, double* out) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (threadIdx.x == 0) atomicAdd(out, w);
  }
  __syncthreads();
}

// sum of u^H T u over all points for a table of FP64 samples T (kind scalar / diag / matrix)
template <typename C, int M>
__global__ void __launch_bounds__(256) quad_kernel(const C* u0, const C* u1, int64_t P, int64_t B, const double2* T,
                                                   int kind, double* out) {
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < P * B; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = q % P;
    double2 v[M];
    v[0] = todd(u0[q]);
    if constexpr (M == 2) v[1] = todd(u1[q]);
    if (kind == TAB_SCALAR) {
      for (int m = 0; m < M; ++m) acc += re_conj_mul(v[m], T[p], v[m]);
    } else if (kind == TAB_DIAG) {
      for (int m = 0; m < M; ++m) acc += re_conj_mul(v[m], T[(int64_t)m * P + p], v[m]);
    } else {
      for (int i = 0; i < M; ++i)
        for (int j = 0; j < M; ++j) acc += re_conj_mul(v[i], T[(int64_t)(i * M + j) * P + p], v[j]);
    }
  }
  block_add(acc, out);
}

// sum_j [ (1/2) sum_l Re g_jl |u_l|^2 + Re c_j ] |u_j|^2
template <typename C, int M>
__global__ void __launch_bounds__(256) interaction_kernel(const C* u0, const C* u1, int64_t n, PassArgs a, double* out) {
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double d[M];
    double2 v = todd(u0[q]);
    d[0] = v.x * v.x + v.y * v.y;
    if constexpr (M == 2) {
      v = todd(u1[q]);
      d[M - 1] = v.x * v.x + v.y * v.y;
    }
    for (int j = 0; j < M; ++j) {
      double w = a.c[j][0];
      for (int l = 0; l < M; ++l) w += 0.5 * a.g[j][l][0] * d[l];
      acc += w * d[j];
    }
  }
  block_add(acc, out);
}

template <typename Real, int M>
int energy_sums_t(const void* const* uk, const void* const* ur, int64_t P, int64_t B, const double2* D, int dkind,
                  const double2* V, int vkind, const PassArgs& a, double* out3, cudaStream_t s) {
  using C = typename CT<Real>::T;
  const int64_t n = P * B;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (D) quad_kernel<C, M><<<(unsigned)blocks, 256, 0, s>>>((const C*)uk[0], (const C*)uk[M - 1], P, B, D, dkind, out3);
  interaction_kernel<C, M><<<(unsigned)blocks, 256, 0, s>>>((const C*)ur[0], (const C*)ur[M - 1], n, a, out3 + 1);
  if (V) quad_kernel<C, M><<<(unsigned)blocks, 256, 0, s>>>((const C*)ur[0], (const C*)ur[M - 1], P, B, V, vkind, out3 + 2);
  return (int)cudaGetLastError();
}

int launch_energy_sums(int prec, int M, const void* const* uk, const void* const* ur, int64_t P, int64_t B,
                       const double2* D, int dkind, const double2* V, int vkind, const PassArgs& a, double* out3,
                       cudaStream_t s) {
  if (prec == PREC_F64)
    return M == 1 ? energy_sums_t<double, 1>(uk, ur, P, B, D, dkind, V, vkind, a, out3, s)
                  : energy_sums_t<double, 2>(uk, ur, P, B, D, dkind, V, vkind, a, out3, s);
  if (prec == PREC_DW)
    return M == 1 ? energy_sums_t<DWR, 1>(uk, ur, P, B, D, dkind, V, vkind, a, out3, s)
                  : energy_sums_t<DWR, 2>(uk, ur, P, B, D, dkind, V, vkind, a, out3, s);
  return M == 1 ? energy_sums_t<float, 1>(uk, ur, P, B, D, dkind, V, vkind, a, out3, s)
                : energy_sums_t<float, 2>(uk, ur, P, B, D, dkind, V, vkind, a, out3, s);
}

}  // namespace gpe

namespace gpe {

// nb[b*P + k] = |u~_b(k)|^2 / P^2 for the transformed fields of one component
template <typename C>
__global__ void __launch_bounds__(256) occupation_kernel(const C* uk, int64_t P, int64_t B, double* nb) {
  const double s = 1.0 / ((double)P * (double)P);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < P * B; q += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = todd(uk[q]);
    nb[q] = (v.x * v.x + v.y * v.y) * s;
  }
}

// mean[k] = (1/B) sum_b nb[b][k]
__global__ void __launch_bounds__(256) mean_kernel(const double* nb, int64_t P, int64_t B, double* mean) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < P; k += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int64_t b = 0; b < B; ++b) acc += nb[b * P + k];
    mean[k] = acc / (double)B;
  }
}

// second[k][k'] = (1/B) sum_b nb[b][k] nb[b][k'], 32x32 tiles staged through shared memory
__global__ void __launch_bounds__(256) second_moment_kernel(const double* nb, int64_t P, int64_t B, double* second) {
  __shared__ double a[32][33], c[32][33];
  const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;  // 32 x 8 threads, 4 outputs each
  const int64_t k0 = (int64_t)blockIdx.y * 32, k1 = (int64_t)blockIdx.x * 32;
  double acc[4] = {0, 0, 0, 0};
  for (int64_t b0 = 0; b0 < B; b0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      const int64_t b = b0 + r;
      a[r][tx] = (b < B && k0 + tx < P) ? nb[b * P + k0 + tx] : 0.0;
      c[r][tx] = (b < B && k1 + tx < P) ? nb[b * P + k1 + tx] : 0.0;
    }
    __syncthreads();
    for (int r = 0; r < 32; ++r)
      for (int j = 0; j < 4; ++j) acc[j] += a[r][ty + 8 * j] * c[r][tx];
    __syncthreads();
  }
  for (int j = 0; j < 4; ++j) {
    const int64_t k = k0 + ty + 8 * j, kp = k1 + tx;
    if (k < P && kp < P) second[k * P + kp] = acc[j] / (double)B;
  }
}

int launch_spectral_moments(int prec, const void* uk, int64_t P, int64_t B, double* nb, double* mean, double* second,
                            cudaStream_t s) {
  const int64_t n = P * B;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (prec == PREC_F64) occupation_kernel<double2><<<(unsigned)blocks, 256, 0, s>>>((const double2*)uk, P, B, nb);
  else if (prec == PREC_DW) occupation_kernel<dwc><<<(unsigned)blocks, 256, 0, s>>>((const dwc*)uk, P, B, nb);
  else occupation_kernel<float2><<<(unsigned)blocks, 256, 0, s>>>((const float2*)uk, P, B, nb);
  mean_kernel<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(nb, P, B, mean);
  if (second) {
    const dim3 grid((unsigned)((P + 31) / 32), (unsigned)((P + 31) / 32));
    second_moment_kernel<<<grid, 256, 0, s>>>(nb, P, B, second);
  }
  return (int)cudaGetLastError();
}

}  // namespace gpe
