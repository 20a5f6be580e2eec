// fno.cu -- kernels of the Fourier-neural-operator surrogate (C ABI in include/gpe_fno.h).
//
// Every linear map of the network (lift, the truncated DFTs along x and y, the per-mode
// complex channel mixing, the pointwise channel mixing, the projection) and every
// gradient of it is one call of a strided, batched GEMM on the tensor cores:
// operands are rounded to BF16 while they are staged in shared memory, products
// accumulate in FP32 (mma.sync m16n8k16), results are FP32.  GELU, bias and Adam are
// elementwise kernels.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gpe_fno.h"

namespace {

constexpr int BM = 128, BN = 64, BK = 32;  // CTA tile
constexpr int NTH = 256;                   // 8 warps: 4 along M x 2 along N, warp tile 32 x 32
constexpr int SA = BK + 8;                 // shared row pitch (bf16) of the A tile [BM][SA]
constexpr int SB = BK + 8;                 // shared row pitch of the B tile stored as [BN][SB] (k fastest)

// D = A(16x16, row) * B(16x8, col) + D with BF16 inputs and FP32 accumulators
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[z] = alpha * A[z] B[z] + beta * C[z], element (i, j) of X at X + i*x_r + j*x_c.
__global__ void __launch_bounds__(NTH) gemm_kernel(gpe_gemm_desc g) {
  __shared__ __align__(16) __nv_bfloat16 As[BM * SA];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN * SB];
  const int z = blockIdx.z;
  const float* A = g.A + (int64_t)z * g.a_z;
  const float* B = g.B + (int64_t)z * g.b_z;
  float* C = g.C + (int64_t)z * g.c_z;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp & 3, wn = warp >> 2;  // warp tile origin (wm*32, wn*32)
  const int gq = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  for (int64_t k0 = 0; k0 < g.K; k0 += BK) {
    // stage A[m0:m0+BM, k0:k0+BK] -> As[m][k], zero outside the matrix
    for (int e = tid; e < BM * BK; e += NTH) {
      // consecutive threads walk the operand's contiguous index
      const int mi = g.a_r == 1 ? e % BM : e / BK, ki = g.a_r == 1 ? e / BM : e % BK;
      const int64_t m = m0 + mi, k = k0 + ki;
      const float v = (m < g.M && k < g.K) ? A[m * g.a_r + k * g.a_c] : 0.f;
      As[mi * SA + ki] = __float2bfloat16_rn(v);
    }
    // stage B[k0:k0+BK, n0:n0+BN] -> Bs[n][k]
    for (int e = tid; e < BN * BK; e += NTH) {
      const int ni = g.b_c == 1 ? e % BN : e / BK, ki = g.b_c == 1 ? e / BN : e % BK;
      const int64_t n = n0 + ni, k = k0 + ki;
      const float v = (n < g.N && k < g.K) ? B[k * g.b_r + n * g.b_c] : 0.f;
      Bs[ni * SB + ki] = __float2bfloat16_rn(v);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r0 = wm * 32 + i * 16 + gq;
        const __nv_bfloat16* p = As + r0 * SA + kk + 2 * tq;
        af[i][0] = *reinterpret_cast<const uint32_t*>(p);
        af[i][1] = *reinterpret_cast<const uint32_t*>(p + 8 * SA);
        af[i][2] = *reinterpret_cast<const uint32_t*>(p + 8);
        af[i][3] = *reinterpret_cast<const uint32_t*>(p + 8 * SA + 8);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c0 = wn * 32 + j * 8 + gq;
        const __nv_bfloat16* p = Bs + c0 * SB + kk + 2 * tq;
        bf[j][0] = *reinterpret_cast<const uint32_t*>(p);
        bf[j][1] = *reinterpret_cast<const uint32_t*>(p + 8);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int64_t m = m0 + wm * 32 + i * 16 + gq + (r >= 2 ? 8 : 0);
        const int64_t n = n0 + wn * 32 + j * 8 + 2 * tq + (r & 1);
        if (m < g.M && n < g.N) {
          float* c = C + m * g.c_r + n * g.c_c;
          *c = g.alpha * acc[i][j][r] + (g.beta != 0.f ? g.beta * *c : 0.f);
        }
      }
}

// ---------------------------------------------------------------- elementwise kernels
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }
__device__ __forceinline__ int64_t gidx() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

// dst = src viewed with dims d[0..nd) (row-major) and transposed by perm: dst axis a is
// src axis perm[a].
__global__ void permute_kernel(const float* __restrict__ src, float* __restrict__ dst, gpe_permute_desc p) {
  int64_t n = 1;
  for (int a = 0; a < p.nd; ++a) n *= p.d[a];
  int64_t sstr[6];
  int64_t acc = 1;
  for (int a = p.nd - 1; a >= 0; --a) { sstr[a] = acc; acc *= p.d[a]; }
  for (int64_t i = gidx(); i < n; i += gstride()) {
    // i indexes dst; decompose over dst dims d[perm[a]]
    int64_t r = i, off = 0;
    for (int a = p.nd - 1; a >= 0; --a) {
      const int64_t da = p.d[p.perm[a]];
      const int64_t c = r % da;
      r /= da;
      off += c * sstr[p.perm[a]];
    }
    dst[i] = src[off];
  }
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// x[b][c][p] += bias[c]; pre = x; x = gelu(x) when act != 0
__global__ void bias_act_kernel(float* x, const float* bias, float* pre, int64_t B, int64_t C, int64_t P, int act) {
  const int64_t n = B * C * P;
  for (int64_t i = gidx(); i < n; i += gstride()) {
    const int64_t c = (i / P) % C;
    const float v = x[i] + (bias ? bias[c] : 0.f);
    if (pre) pre[i] = v;
    x[i] = act ? gelu(v) : v;
  }
}

__global__ void gelu_bwd_kernel(float* dy, const float* pre, int64_t n) {
  for (int64_t i = gidx(); i < n; i += gstride()) dy[i] *= gelu_grad(pre[i]);
}

// dbias[c] = sum over b, p of dy[b][c][p] (one block per channel, fixed order)
__global__ void bias_grad_kernel(const float* dy, float* dbias, int64_t B, int64_t C, int64_t P) {
  const int64_t c = blockIdx.x;
  double acc = 0.0;
  for (int64_t b = 0; b < B; ++b)
    for (int64_t p = threadIdx.x; p < P; p += blockDim.x) acc += dy[(b * C + c) * P + p];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) dbias[c] = (float)v;
  }
}

__global__ void axpy_kernel(float* y, const float* x, float alpha, int64_t n, int64_t batch, int64_t ys, int64_t xs) {
  const int64_t total = n * batch;
  for (int64_t q = gidx(); q < total; q += gstride()) {
    const int64_t z = q / n, i = q - z * n;
    y[z * ys + i] += alpha * x[z * xs + i];
  }
}

// grad = 2 (pred - target) / n; partial sums of squares into loss_acc (FP64)
__global__ void mse_kernel(const float* pred, const float* target, float* grad, double* loss_acc, int64_t n) {
  double acc = 0.0;
  for (int64_t i = gidx(); i < n; i += gstride()) {
    const float d = pred[i] - target[i];
    if (grad) grad[i] = 2.f * d / (float)n;
    acc += (double)d * d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc, acc);
}

// Adam (Kingma & Ba, ICLR 2015) with bias correction, step t >= 1
__global__ void adam_kernel(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  for (int64_t i = gidx(); i < n; i += gstride()) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// dst[i] = sum_z src[z * n + i] (split-K partial sums, fixed order)
__global__ void sum_slices_kernel(const float* src, float* dst, int64_t n, int64_t slices) {
  for (int64_t i = gidx(); i < n; i += gstride()) {
    float acc = 0.f;
    for (int64_t z = 0; z < slices; ++z) acc += src[z * n + i];
    dst[i] = acc;
  }
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

}  // namespace

extern "C" {

int gpe_fno_gemm(const gpe_gemm_desc* d, void* stream) {
  if (!d || !d->A || !d->B || !d->C || d->M < 1 || d->N < 1 || d->K < 1 || d->batch < 1 || d->batch > 65535)
    return GPE_ERR_INVALID;
  const dim3 grid((unsigned)((d->N + BN - 1) / BN), (unsigned)((d->M + BM - 1) / BM), (unsigned)d->batch);
  if (grid.y > 65535) return GPE_ERR_INVALID;
  gemm_kernel<<<grid, NTH, 0, (cudaStream_t)stream>>>(*d);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_permute(const float* src, float* dst, const gpe_permute_desc* p, void* stream) {
  if (!src || !dst || !p || p->nd < 1 || p->nd > 6) return GPE_ERR_INVALID;
  int64_t n = 1;
  for (int a = 0; a < p->nd; ++a) n *= p->d[a];
  permute_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(src, dst, *p);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_bias_act(float* x, const float* bias, float* pre, int64_t B, int64_t C, int64_t P, int act, void* stream) {
  bias_act_kernel<<<grid_for(B * C * P), 256, 0, (cudaStream_t)stream>>>(x, bias, pre, B, C, P, act);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_gelu_bwd(float* dy, const float* pre, int64_t n, void* stream) {
  gelu_bwd_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dy, pre, n);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_bias_grad(const float* dy, float* dbias, int64_t B, int64_t C, int64_t P, void* stream) {
  bias_grad_kernel<<<(unsigned)C, 256, 0, (cudaStream_t)stream>>>(dy, dbias, B, C, P);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_axpy(float* y, const float* x, float alpha, int64_t n, int64_t batch, int64_t y_stride, int64_t x_stride,
                 void* stream) {
  if (n < 0 || batch < 0) return GPE_ERR_INVALID;
  if (n == 0 || batch == 0) return GPE_OK;
  axpy_kernel<<<grid_for(n * batch), 256, 0, (cudaStream_t)stream>>>(y, x, alpha, n, batch, y_stride, x_stride);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_mse(const float* pred, const float* target, float* grad, double* loss_acc, int64_t n, void* stream) {
  mse_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(pred, target, grad, loss_acc, n);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_sum_slices(const float* src, float* dst, int64_t n, int64_t slices, void* stream) {
  sum_slices_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(src, dst, n, slices);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

int gpe_fno_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                 int64_t t, void* stream) {
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

}  // extern "C"
