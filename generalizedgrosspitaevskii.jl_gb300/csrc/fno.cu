// fno.cu -- kernels of the Fourier-neural-operator surrogate (C ABI in include/gpe_fno.h).
//
// Every linear map of the network (lift, the truncated DFTs along x and y, the per-mode
// complex channel mixing, the pointwise channel mixing, the projection) and every
// gradient of it is one call of a strided, batched GEMM on the tensor cores: operands
// are rounded to BF16 while they are staged in shared memory, tcgen05.mma accumulates in
// FP32 in tensor memory, results are FP32.  GELU, bias and Adam are elementwise kernels.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gpe_fno.h"

namespace {

// ---------------------------------------------------------------- GEMM on tcgen05
// One CTA computes a TBM x TBN tile of C with the fifth-generation tensor cores: the
// operand tiles are staged into shared memory as BF16 (rounded from FP32 while they are
// loaded, any strides), one thread issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32)
// with the accumulator in tensor memory (TMEM), and the epilogue reads it back with
// tcgen05.ld.  K is walked in TBK-deep stages through two shared-memory buffers: the
// threads fill one while the MMAs of the other run; tcgen05.commit arrives on a
// per-buffer mbarrier when the MMAs reading it are done.
//
// Shared-memory operand layout (both A and B "K-major", no swizzle): 8 x 16-byte core
// matrices (8 rows, 8 BF16 along K each), element (r, k) at byte
//   (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2,  LBO = 128, SBO = TBK * 16,
// so one MMA of K = 16 reads two K-adjacent core matrices and the next one starts 256
// bytes further.
constexpr int TBM = 128, TBK = 64, TNTH = 256;
constexpr uint32_t kLBO = 128, kSBO = TBK * 16;
constexpr uint64_t kTcWaitNs = 1000000000ull;  // 1 s bound on every mbarrier wait

__device__ int32_t g_tc_status;  // set to 1 when a wait of the GEMM ran out (gpe_fno_take_status)

__device__ __forceinline__ uint32_t sptr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait for the given phase parity of the barrier; false after kTcWaitNs
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  while (!mbar_try(bar, parity))
    if (gtimer() - t0 > kTcWaitNs) return false;
  return true;
}

// shared-memory matrix descriptor: start address, leading (K) and stride (M/N) byte
// offsets (all encoded >> 4), the fixed 0b001 at bits 46-48, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((kLBO & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((kSBO & 0x3FFFFu) >> 4) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4
// at bits 24-28
template <int BN>
__device__ __forceinline__ uint32_t instr_desc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
}

__device__ __forceinline__ uint32_t core_off(int r, int k) {
  return (uint32_t)((r >> 3) * kSBO + (k >> 3) * kLBO + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // a in the low half
  return *reinterpret_cast<const uint32_t*>(&h);
}

// Stage an R x TBK tile of an FP32 operand, element (r, k) at G[r * sr + k * sk], into the
// core-matrix layout as BF16 (zero outside r < rlim, k < klim).  A thread takes 8
// consecutive k of one row and writes them as one 16-byte chunk; consecutive threads take
// consecutive rows, so eight of them fill one core matrix's 128 contiguous bytes (no bank
// conflicts).  mode 1 (K contiguous, rows 16-byte aligned): the 8 values are two float4
// loads.  Otherwise, and for the chunks that cross the matrix edge: 8 element loads, which
// are coalesced across the warp when the rows are contiguous (sr = 1).
template <int R>
__device__ __forceinline__ void stage_tile(unsigned char* dst, const float* __restrict__ G, int64_t r0, int64_t k0,
                                           int64_t rlim, int64_t klim, int64_t sr, int64_t sk, int mode, int tid) {
  for (int c = tid; c < R * (TBK / 8); c += TNTH) {
    const int ri = c % R, ki = (c / R) * 8;
    const int64_t r = r0 + ri, k = k0 + ki;
    uint4 q;
    if (mode == 1 && r < rlim && k + 7 < klim) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(G + r * sr + k));
      const float4 b = __ldg(reinterpret_cast<const float4*>(G + r * sr + k + 4));
      q = make_uint4(pack_bf16(a.x, a.y), pack_bf16(a.z, a.w), pack_bf16(b.x, b.y), pack_bf16(b.z, b.w));
    } else {
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = (r < rlim && k + j < klim) ? __ldg(G + r * sr + (k + j) * sk) : 0.f;
      q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
    }
    *reinterpret_cast<uint4*>(dst + core_off(ri, ki)) = q;
  }
}

template <int BN>
struct TcSmem {
  static constexpr uint32_t A_BYTES = TBM * TBK * 2, B_BYTES = BN * TBK * 2;
  static constexpr uint32_t STAGE = A_BYTES + B_BYTES;
  static constexpr uint32_t BAR = 2 * STAGE;   // two mbarriers
  static constexpr uint32_t SLOT = BAR + 16;   // TMEM base address written by tcgen05.alloc
  static constexpr uint32_t BYTES = SLOT + 16 + 1024;  // + alignment slack of the dynamic base
};

// C[z] = alpha * A[z] B[z] + beta * C[z], element (i, j) of X at X + i*x_r + j*x_c.
// vmode: bits 0-1 the staging mode of A (stage_tile), bits 2-3 that of B
template <int BN>
__global__ void __launch_bounds__(TNTH, 2) gemm_tc_kernel(gpe_gemm_desc g, int vmode) {
  using S = TcSmem<BN>;
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  unsigned char* sm = tc_raw + ((1024u - (sptr(tc_raw) & 1023u)) & 1023u);
  const uint32_t sbase = sptr(sm);
  const uint32_t bar0 = sbase + S::BAR, bar1 = bar0 + 8;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + S::SLOT);
  const int z = blockIdx.z;
  const float* A = g.A + (int64_t)z * g.a_z;
  const float* B = g.B + (int64_t)z * g.b_z;
  float* C = g.C + (int64_t)z * g.c_z;
  const int64_t m0 = (int64_t)blockIdx.y * TBM, n0 = (int64_t)blockIdx.x * BN;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    // BN columns of tensor memory (128 lanes x BN FP32 accumulators)
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sptr(tslot)), "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  const int64_t ktiles = (g.K + TBK - 1) / TBK;
  bool ok = true;
  int64_t committed = -1;  // last stage whose MMAs were committed (the same in every thread)
  for (int64_t t = 0; t < ktiles; ++t) {
    const int buf = (int)(t & 1);
    const uint32_t bar = buf ? bar1 : bar0;
    if (t >= 2 && !mbar_wait_bounded(bar, (uint32_t)(((t - 2) >> 1) & 1))) ok = false;  // MMAs of stage t-2 done
    if (__syncthreads_or(!ok)) break;
    unsigned char* As = sm + buf * S::STAGE;
    unsigned char* Bs = As + S::A_BYTES;
    const int64_t k0 = t * TBK;
    // stage A[m0:m0+TBM, k0:k0+TBK] and B[k0:k0+TBK, n0:n0+BN] (as n rows, K-major), zero
    // outside the matrices
    stage_tile<TBM>(As, A, m0, k0, g.M, g.K, g.a_r, g.a_c, vmode & 3, tid);
    stage_tile<BN>(Bs, B, n0, k0, g.N, g.K, g.b_c, g.b_r, (vmode >> 2) & 3, tid);
    // the generic-proxy stores must be visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t idesc = instr_desc<BN>();
#pragma unroll
      for (int kk = 0; kk < TBK / 16; ++kk) {
        const uint64_t ad = smem_desc(sptr(As) + kk * 2 * kLBO);
        const uint64_t bd = smem_desc(sptr(Bs) + kk * 2 * kLBO);
        const uint32_t accum = (t > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
            ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
            : "memory");
      }
      // arrives on this buffer's barrier once every MMA issued so far has completed
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                   : "memory");
    }
    committed = t;
  }
  // the last commit covers every MMA issued (also after a wait that ran out: the tensor
  // memory is freed only once the MMAs writing it are done, or the bound has passed again)
  if (committed >= 0 && !mbar_wait_bounded((committed & 1) ? bar1 : bar0, (uint32_t)((committed >> 1) & 1)))
    ok = false;
  if (!ok && tid == 0) atomicExch(&g_tc_status, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (__syncthreads_and(ok)) {
    // warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows of the tile) and half w / 4 of the columns
    const int q = warp & 3, half = warp >> 2;
    constexpr int NC = BN / 2;
    // rows of C contiguous and 16-byte aligned: vector stores
    const bool cvec = g.c_c == 1 && g.c_r % 4 == 0 && g.c_z % 4 == 0 && (((uintptr_t)g.C) & 15) == 0;
    const int64_t m = m0 + 32 * q + lane;
#pragma unroll
    for (int c0 = 0; c0 < NC; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(half * NC + c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int64_t nb = n0 + half * NC + c0;
      if (m < g.M && cvec && nb + 15 < g.N) {
        // 16 consecutive columns of one row: four 16-byte stores
        float4* c4 = reinterpret_cast<float4*>(C + m * g.c_r + nb);
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) {
          float4 o = make_float4(g.alpha * __uint_as_float(r[4 * q4]), g.alpha * __uint_as_float(r[4 * q4 + 1]),
                                 g.alpha * __uint_as_float(r[4 * q4 + 2]), g.alpha * __uint_as_float(r[4 * q4 + 3]));
          if (g.beta != 0.f) {
            const float4 old = c4[q4];
            o.x += g.beta * old.x; o.y += g.beta * old.y; o.z += g.beta * old.z; o.w += g.beta * old.w;
          }
          c4[q4] = o;
        }
      } else if (m < g.M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int64_t n = n0 + half * NC + c0 + j;
          if (n < g.N) {
            float* c = C + m * g.c_r + n * g.c_c;
            const float acc = __uint_as_float(r[j]);
            *c = g.alpha * acc + (g.beta != 0.f ? g.beta * *c : 0.f);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
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

template <int BN>
int launch_gemm_tc(const gpe_gemm_desc* d, cudaStream_t s) {
  static_assert(TcSmem<BN>::BYTES <= 227 * 1024, "shared memory");
  const dim3 grid((unsigned)((d->N + BN - 1) / BN), (unsigned)((d->M + TBM - 1) / TBM), (unsigned)d->batch);
  if (grid.y > 65535) return GPE_ERR_INVALID;
  static bool attr = false;  // idempotent: every caller sets the same value
  if (!attr) {
    if (cudaFuncSetAttribute(gemm_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)TcSmem<BN>::BYTES) != cudaSuccess)
      return GPE_ERR_CUDA;
    attr = true;
  }
  // float4 staging loads where an operand's K index is contiguous and 16-byte aligned
  auto mode = [](const float* X, int64_t sr, int64_t sk, int64_t sz) {
    return (((uintptr_t)X & 15) == 0 && sz % 4 == 0 && sk == 1 && sr % 4 == 0) ? 1 : 0;
  };
  const int vmode = mode(d->A, d->a_r, d->a_c, d->a_z) | (mode(d->B, d->b_c, d->b_r, d->b_z) << 2);
  gemm_tc_kernel<BN><<<grid, TNTH, TcSmem<BN>::BYTES, s>>>(*d, vmode);
  return cudaGetLastError() == cudaSuccess ? GPE_OK : GPE_ERR_CUDA;
}

}  // namespace

extern "C" {

int gpe_fno_gemm(const gpe_gemm_desc* d, void* stream) {
  if (!d || !d->A || !d->B || !d->C || d->M < 1 || d->N < 1 || d->K < 1 || d->batch < 1 || d->batch > 65535)
    return GPE_ERR_INVALID;
  // N tiles of 32 for the narrow products (channel counts, retained modes), else 64
  return d->N <= 32 ? launch_gemm_tc<32>(d, (cudaStream_t)stream) : launch_gemm_tc<64>(d, (cudaStream_t)stream);
}

int gpe_fno_take_status(void) {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_status, sizeof v) != cudaSuccess) return GPE_ERR_CUDA;
  if (v && cudaMemcpyToSymbol(g_tc_status, &zero, sizeof zero) != cudaSuccess) return GPE_ERR_CUDA;
  return v ? GPE_ERR_TIMEOUT : GPE_OK;
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
