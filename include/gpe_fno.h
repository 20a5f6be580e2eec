/*
 * gpe_fno.h -- kernels of the Fourier-neural-operator surrogate of the StrangSplitting
 * solver (no counterpart in the reference: a learned model trained on trajectories the
 * solver generates, with the solver as its fallback and the measure of its error).
 *
 * All entry points take caller-owned device pointers (FP32) and an optional CUDA stream
 * (NULL = legacy default stream); they enqueue work and return GPE_OK (0) or a negative
 * GPE_ERR_* code.
 */
#ifndef GPE_FNO_H
#define GPE_FNO_H

#include <stdint.h>

#include "gpe.h"

#ifdef __cplusplus
extern "C" {
#endif

/* C[z] = alpha * A[z] * B[z] + beta * C[z] for z < batch; element (i, j) of a matrix X is
 * X + i * x_r + j * x_c, matrix z starts at X + z * x_z.  A is M x K, B is K x N.  The
 * operands are rounded to BF16 as they are staged in shared memory and multiplied on the
 * fifth-generation tensor cores (tcgen05.mma, kind::f16) with FP32 accumulation in tensor
 * memory.  Every wait of the kernel is bounded (1 s); gpe_fno_take_status reports one that
 * ran out. */
typedef struct gpe_gemm_desc {
  const float* A;
  const float* B;
  float* C;
  int64_t M, N, K;
  int64_t a_r, a_c, a_z;
  int64_t b_r, b_c, b_z;
  int64_t c_r, c_c, c_z;
  int64_t batch;
  float alpha, beta;
} gpe_gemm_desc;
int gpe_fno_gemm(const gpe_gemm_desc* d, void* stream);
/* GPE_ERR_TIMEOUT (and clears it) when a GEMM's bounded wait has run out since the last
 * call, else GPE_OK; synchronises with the device. */
int gpe_fno_take_status(void);

/* dst = src (row-major dims d[0..nd)) transposed so that dst axis a is src axis perm[a]. */
typedef struct gpe_permute_desc {
  int32_t nd;
  int32_t perm[6];
  int64_t d[6];
} gpe_permute_desc;
int gpe_fno_permute(const float* src, float* dst, const gpe_permute_desc* p, void* stream);

/* x[b][c][p] += bias[c] (bias may be NULL); pre (may be NULL) <- x; x <- GELU(x) if act. */
int gpe_fno_bias_act(float* x, const float* bias, float* pre, int64_t B, int64_t C, int64_t P, int act, void* stream);
/* dy *= GELU'(pre) */
int gpe_fno_gelu_bwd(float* dy, const float* pre, int64_t n, void* stream);
/* dbias[c] = sum_{b,p} dy[b][c][p] */
int gpe_fno_bias_grad(const float* dy, float* dbias, int64_t B, int64_t C, int64_t P, void* stream);
/* y[z * y_stride + i] += alpha * x[z * x_stride + i] for z < batch, i < n */
int gpe_fno_axpy(float* y, const float* x, float alpha, int64_t n, int64_t batch, int64_t y_stride, int64_t x_stride,
                 void* stream);
/* *loss_acc += sum (pred - target)^2 (FP64); grad (may be NULL) = 2 (pred - target) / n */
int gpe_fno_mse(const float* pred, const float* target, float* grad, double* loss_acc, int64_t n, void* stream);
/* dst[i] = sum over z < slices of src[z*n + i] (split-K reduction) */
int gpe_fno_sum_slices(const float* src, float* dst, int64_t n, int64_t slices, void* stream);
/* Adam step t >= 1 on n parameters */
int gpe_fno_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                 int64_t t, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GPE_FNO_H */
