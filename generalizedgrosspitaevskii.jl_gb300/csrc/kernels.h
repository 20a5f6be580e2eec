// kernels.h -- argument block shared by the host driver and the pass kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gpe {

struct DWR;  // double-word precision tag (defined in fft.cuh)

enum TableKind { TAB_NONE = 0, TAB_SCALAR = 1, TAB_DIAG = 2, TAB_MATRIX = 3 };
enum NoiseMode { NOISE_OFF = 0, NOISE_PHILOX = 1, NOISE_REPLAY = 2 };
// Half-step families with a compile-time specialisation (every precision; no potential, no noise,
// real nonlinearity, real non-uniform pump profiles): G = components whose nonlinearity is
// on, D = the densities it reads, P = pumped components.
enum LeanKind {
  LEAN_OFF = 0,
  LEAN_M1_G = 1,    // one component: G from |u|^2 (Kerr)
  LEAN_M1_GP = 2,   // one component: G from |u|^2, pumped (driven Kerr)
  LEAN_M2_G1P0 = 3, // two components: G_2 from |u_2|^2, pump on component 1 (exciton-polariton)
  LEAN_M2_GG = 4    // two components: G_1, G_2 from both densities, no pump (two-component condensate)
};

// One launch of a line pass.  Plain data only: it is copied to the kernel's
// parameter space by value.
struct PassArgs {
  // geometry: n[0] = x (fastest); P = n0*n1*n2 spatial points; B trajectories
  int32_t n0, n1, n2;
  int64_t P, B;
  int32_t nsm;  // streaming multiprocessors of the device (launch shapes)
  // fields (M planes of B*P complex numbers in the pass precision)
  void* u[2];
  // optional copy of the real-space state after the first half step of the pass
  void* save[2];
  // k-space table exp(-i dt D)/P (col pass / 1D) and real-space table exp(-i dt/2 V)
  const void* ktab;
  int32_t kkind;
  // FP64 passes with block floating point transforms: the k-space table in Q62 fixed point
  // ({re.hi, re.lo, im.hi, im.lo} 32-bit halves, entries times P 2^-kexp), kq_exp = kexp - log2 P
  const void* ktab_q;
  int32_t kq_exp;
  const void* vtab;
  int32_t vkind;
  // twiddles w_N^k, k < N, for the transformed line length (tw2: y lines of the
  // resident plane kernel)
  const void* tw;
  const void* tw2;
  // nonlinearity G_j = sum_l g[j][l] |u_l|^2 + c[j] (complex).  FP64 values, their FP32
  // roundings (gf, cf) and the FP32 remainders (gl, cl) that make (gf + gl) the
  // double-word form, so no pass converts per point.
  int32_t nl_on[2], nl_imag[2];
  int32_t dens_mask;  // bit l: some active G_j depends on |u_l|^2
  int32_t g_nz;       // bit j*4 + l*2 + r: g[j][l][r] != 0 (tested on the integer pipe)
  double g[2][2][2];
  double c[2][2];
  // the same times dt/2 (FP64 passes form the phase dt/2 G with one FMA a term) and the
  // nonzero c terms, bit j*2 + r
  double gd[2][2][2];
  double cd[2][2];
  int32_t c_nz;
  float gf[2][2][2], gl[2][2][2];
  float cf[2][2], cl[2][2];
  // matrix nonlinearity (M = 2), null when off: 24 doubles on the device, g[a][b][l] (re, im)
  // then c[a][b] (re, im), G_ab = sum_l g[a][b][l] |u_l|^2 + c[a][b]; the per-point phase
  // exp(-i delta G) is a 2x2 matrix exponential
  const double* nlm;
  // pump F_m = a_m(t) p_m(r): profile (real or complex) and the per-boundary
  // coefficients (dt/4) a_m(t_h), both stored in the pass precision
  const void* pprof[2];
  int32_t pprof_cplx;
  int32_t pump_uniform;  // bit m: profile m is 1 everywhere (its value is in the coefficients)
  const void* pcoef[2];
  int64_t pcoef_n[2];
  // noise: -i sqrt(dt/2) eta_m (host-formed) [* eta profile] * xi
  int32_t noise;
  uint32_t seed_lo, seed_hi;
  int64_t traj0;  // global index of this handle's first trajectory (Philox counter word 1)
  double nfac[2][2];
  float nfacf[2][2], nfacl[2][2];
  const void* etaprof[2];
  const void* xi;     // replay: [half - xi_h0][m][b][p]
  int64_t xi_h0;
  double dt;
  float dthf, dthl;  // dt/2 as FP32 and its double-word remainder
  // row pass program: [iFFT] [half hA] [save] [half hB] [FFT]; h < 0 skips a half
  int32_t do_ifft, do_fft;
  int64_t hA, hB;
  // graph replay: when set, step indices (step0, hA, hB) are relative to the step count
  // stored here on the device, so a captured chunk of steps replays at any position
  const int64_t* kbase;
  // 1D resident program: nsteps full steps from step0, save every save_every steps
  // into save[m] + slot*save_stride
  int64_t nsteps, step0, save_every, save_stride;
  // column pass: lines of length N with stride ld; a tile is CC consecutive x
  // columns at outer index o (offset o*ostride) of trajectory b
  int64_t ld, ostride, nouter;
  int32_t col_fwd, col_inv;
  // TMA staging of 2D column tiles: 0 never, 1 wherever the shape and shared memory
  // allow, 2 by the measured rule (one-component lines of at most 512 points)
  int32_t col_tma;
  // FP64 line transforms of the row and column passes in block floating point on the
  // integer pipes (Q62 twiddles after the FP64 ones in the table)
  int32_t fx;
  // half steps of the common families specialised at compile time (LeanKind; 0 = the
  // generic half step)
  int32_t lean;
  // host-mapped status word: a device wait that ran out of time stores 1 here
  int32_t* status;
};

// Pass precisions: native FP64, FP32, double-word FP64 on the FP32 pipes.
enum PassPrec { PREC_F64 = 0, PREC_F32 = 1, PREC_DW = 2 };

// Launchers: return 0 or a cudaError_t value.  logn = log2 of the line length.
// variant: line tiling (0 default; 1 = the alternative FP32 one-component tiling)
int launch_row(int dtype, int M, int logn, const PassArgs& a, int64_t nlines, cudaStream_t s, int variant = 0);
int launch_col(int dtype, int M, int logn, const PassArgs& a, cudaStream_t s, int variant = 0);
int launch_line1d(int dtype, int M, int logn, const PassArgs& a, cudaStream_t s);
int launch_nl_only(int dtype, int M, const PassArgs& a, cudaStream_t s);
// pointwise pass of the 2x2 matrix nonlinearity family (M = 2, a.nlm set)
int launch_mat(int dtype, const PassArgs& a, cudaStream_t s);
// whole-trajectory resident 2D kernel (square grids of side 2^logn that fit in shared memory)
int launch_plane(int dtype, int M, int logn, const PassArgs& a, cudaStream_t s);
bool plane_fits(int dtype, int M, int logn);
// FP64 reductions: out[m] += sum |u_m|^2 (device double array of M entries)
int launch_norm(int dtype, int M, const PassArgs& a, double* out, cudaStream_t s);
// FP64 energy sums into out3[0..2] (kinetic on the transformed fields uk with D samples,
// interaction on ur, potential on ur with V samples); D or V may be null
int launch_energy_sums(int prec, int M, const void* const* uk, const void* const* ur, int64_t P, int64_t B,
                       const double2* D, int dkind, const double2* V, int vkind, const PassArgs& a, double* out3,
                       cudaStream_t s);
// per-trajectory occupations nb = |u~|^2/P^2, their trajectory mean, and (second != null)
// the matrix (1/B) sum_b nb[b][k] nb[b][k']
int launch_spectral_moments(int prec, const void* uk, int64_t P, int64_t B, double* nb, double* mean, double* second,
                            cudaStream_t s);
// bounded-wait probe: one CTA waits on an mbarrier that (arrive = 0) nothing completes;
// *status = 1 when the wait ran out after limit_ns
int launch_wait_probe(int arrive, uint64_t limit_ns, int32_t* status, cudaStream_t s);
// *k += n on the device (end of a captured chunk of n steps)
int launch_advance(int64_t* k, int64_t n, cudaStream_t s);
// FP64 <-> double-word conversion of n complex numbers
int launch_f64_to_dw(const void* src, void* dst, int64_t n, cudaStream_t s);
// *flag |= 1 if any of n FP64 (is_f64) or FP32 values is NaN or Inf
int launch_nonfinite(const void* data, int64_t n, int is_f64, int* flag, cudaStream_t s);
int launch_dw_to_f64(const void* src, void* dst, int64_t n, cudaStream_t s);

}  // namespace gpe
