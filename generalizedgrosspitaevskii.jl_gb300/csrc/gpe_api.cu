// gpe_api.cu -- the C ABI of include/gpe.h: handle lifetime, host-side table
// construction in FP64 and the launch sequence of gpe_run.
//
// Reference correspondence (paths in GeneralizedGrossPitaevskii.jl):
//   gpe_create            init(prob, StrangSplitting(), ...)   src/strang_splitting.jl:32-67
//   gpe_set_dispersion    get_exponential(dispersion, ..., dt)  src/misc.jl:12-20, :53 (1/P of inv(plan))
//   gpe_set_potential     get_exponential(potential, ..., dt/2) src/strang_splitting.jl:54
//   gpe_set_pump          get_pump_buffer / evaluate_pump!      src/misc.jl:22-42
//   gpe_set_noise         sample_noise! + noise term            src/misc.jl:44-51, src/kernels.jl:42
//   gpe_run               solve! host loop + step!              src/fixed_time_stepping.jl:26-54,
//                                                              src/strang_splitting.jl:69-90
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gpe.h"
#include "kernels.h"

using cd = std::complex<double>;

namespace gpe {
template <typename Real, int M, int V> int launch_row_t(int, const PassArgs&, int64_t, cudaStream_t);
template <typename Real, int M, int V> int launch_col_t(int, const PassArgs&, cudaStream_t);
template <typename Real, int M> int launch_line1d_t(int, const PassArgs&, cudaStream_t);
template <typename Real, int M> int launch_nl_only_t(const PassArgs&, cudaStream_t);
template <typename Real, int M> int launch_plane_t(int, const PassArgs&, cudaStream_t);
template <typename Real, int M> bool plane_fits_t(int);
template <typename Real, int M> int launch_norm_t(const PassArgs&, double*, cudaStream_t);
template <typename Real> int launch_mat_t(const PassArgs&, cudaStream_t);

// dtype here is the pass precision (PREC_F64, PREC_F32, PREC_DW)
#define GPE_DISPATCH(FN, ...)                                                                  \
  if (dtype == PREC_F64) return M == 1 ? FN<double, 1>(__VA_ARGS__) : FN<double, 2>(__VA_ARGS__); \
  if (dtype == PREC_DW) return M == 1 ? FN<DWR, 1>(__VA_ARGS__) : FN<DWR, 2>(__VA_ARGS__);        \
  return M == 1 ? FN<float, 1>(__VA_ARGS__) : FN<float, 2>(__VA_ARGS__);

// variant 1 (alternative line tiling) exists for FP32 one-component fields only;
// variant 2 (fine tiling) for every precision and component count
#define GPE_DISPATCH_V2(FN, ...)                                                                        \
  if (variant == 2) {                                                                                   \
    if (dtype == PREC_F64) return M == 1 ? FN<double, 1, 2>(__VA_ARGS__) : FN<double, 2, 2>(__VA_ARGS__); \
    if (dtype == PREC_DW) return M == 1 ? FN<DWR, 1, 2>(__VA_ARGS__) : FN<DWR, 2, 2>(__VA_ARGS__);       \
    return M == 1 ? FN<float, 1, 2>(__VA_ARGS__) : FN<float, 2, 2>(__VA_ARGS__);                         \
  }
int launch_row(int dtype, int M, int logn, const PassArgs& a, int64_t nl, cudaStream_t s, int variant) {
  GPE_DISPATCH_V2(launch_row_t, logn, a, nl, s)
  if (variant == 1 && dtype == PREC_F32 && M == 1) return launch_row_t<float, 1, 1>(logn, a, nl, s);
  if (dtype == PREC_F64) return M == 1 ? launch_row_t<double, 1, 0>(logn, a, nl, s) : launch_row_t<double, 2, 0>(logn, a, nl, s);
  if (dtype == PREC_DW) return M == 1 ? launch_row_t<DWR, 1, 0>(logn, a, nl, s) : launch_row_t<DWR, 2, 0>(logn, a, nl, s);
  return M == 1 ? launch_row_t<float, 1, 0>(logn, a, nl, s) : launch_row_t<float, 2, 0>(logn, a, nl, s);
}
int launch_col(int dtype, int M, int logn, const PassArgs& a, cudaStream_t s, int variant) {
  GPE_DISPATCH_V2(launch_col_t, logn, a, s)
  if (variant == 1 && dtype == PREC_F32 && M == 1) return launch_col_t<float, 1, 1>(logn, a, s);
  if (dtype == PREC_F64) return M == 1 ? launch_col_t<double, 1, 0>(logn, a, s) : launch_col_t<double, 2, 0>(logn, a, s);
  if (dtype == PREC_DW) return M == 1 ? launch_col_t<DWR, 1, 0>(logn, a, s) : launch_col_t<DWR, 2, 0>(logn, a, s);
  return M == 1 ? launch_col_t<float, 1, 0>(logn, a, s) : launch_col_t<float, 2, 0>(logn, a, s);
}
int launch_line1d(int dtype, int M, int logn, const PassArgs& a, cudaStream_t s) { GPE_DISPATCH(launch_line1d_t, logn, a, s) }
int launch_nl_only(int dtype, int M, const PassArgs& a, cudaStream_t s) { GPE_DISPATCH(launch_nl_only_t, a, s) }
int launch_norm(int dtype, int M, const PassArgs& a, double* out, cudaStream_t s) { GPE_DISPATCH(launch_norm_t, a, out, s) }
int launch_mat(int dtype, const PassArgs& a, cudaStream_t s) {
  if (dtype == PREC_F64) return launch_mat_t<double>(a, s);
  if (dtype == PREC_DW) return launch_mat_t<DWR>(a, s);
  return launch_mat_t<float>(a, s);
}
int launch_plane(int dtype, int M, int logn, const PassArgs& a, cudaStream_t s) { GPE_DISPATCH(launch_plane_t, logn, a, s) }
bool plane_fits(int dtype, int M, int logn) { GPE_DISPATCH(plane_fits_t, logn) }
}  // namespace gpe

using gpe::PassArgs;

struct gpe_handle {
  gpe_desc d{};
  int dev = 0;
  int nsm = 152;  // multiprocessors of dev
  int M = 1, dtype = GPE_C128, ndim = 2;
  int prec = gpe::PREC_F64;  // pass precision: FP64 fields run native FP64 unless GPE_FLAG_FP64_DW
  size_t rsz = 8, csz = 16;  // device bytes per real / complex number
  int64_t n[3] = {1, 1, 1};
  int logn[3] = {0, 0, 0};
  int64_t P = 1, B = 1;
  double dV = 1.0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_ext = nullptr;  // orders the handle's stream after the legacy default stream
  void* u[2] = {nullptr, nullptr};
  void* tw[3] = {nullptr, nullptr, nullptr};
  void* ktab = nullptr;
  int kkind = GPE_TABLE_NONE;
  void* ktab_q = nullptr;  // Q62 copy for block floating point column passes (FP64 fields)
  int kq_exp = 0;
  std::vector<cd> Dsamples;  // dispersion samples kept for gpe_energy
  int dkind = GPE_TABLE_NONE;
  void* vtab = nullptr;
  int vkind = GPE_TABLE_NONE;
  std::vector<cd> Vsamples;
  int vskind = GPE_TABLE_NONE;
  void* pprof[2] = {nullptr, nullptr};
  int pprof_cplx = 0;
  int pump_uniform = 0;  // bit m: component m's profile is one value everywhere, folded into its coefficients
  std::vector<cd> pprof_host[2];
  void* pcoef[2] = {nullptr, nullptr};  // (dt/4) a(t_h) per half-step boundary, pass precision
  int64_t pcoef_n[2] = {0, 0};
  void* etaprof[2] = {nullptr, nullptr};
  int noise = GPE_NOISE_OFF;
  uint64_t seed = 0;
  int64_t traj0 = 0;  // global index of the first trajectory (gpe_set_noise_offset)
  double eta[2][2] = {{0, 0}, {0, 0}};
  double g[2][2][2] = {};
  double c[2][2] = {};
  int nl_on[2] = {0, 0};
  int variant = -1;  // line tiling of the two-pass passes (gpe_set_variant); -1 = by size
  int nl_matrix = 0;
  double* nlm = nullptr;  // device copy of the matrix nonlinearity coefficients
  double t = 0.0;
  int64_t steps = 0;
  void* save_buf = nullptr;
  size_t save_cap = 0;
  // save ring: pinned host staging, copy stream and per-slot events (see SaveRing)
  void* pinned = nullptr;
  size_t pinned_cap = 0;
  cudaStream_t cstream = nullptr;
  std::vector<cudaEvent_t> ring_ready, ring_done;
  void* xi_buf = nullptr;
  size_t xi_cap = 0;
  void* conv_buf = nullptr;  // FP64 staging of double-word fields on their way to the host
  size_t conv_cap = 0;
  double* red = nullptr;  // reduction scratch (4 doubles)
  // status word in mapped host memory: a kernel whose bounded wait ran out stores 1
  int32_t* hstat = nullptr;
  int32_t* dstat = nullptr;
  double last_ms = 0.0;
  int64_t last_launches = 0;
  // per-launch timing (gpe_set_timing)
  int timing = 0;
  int capturing = 0;  // inside a stream capture: no timing events
  std::vector<cudaEvent_t> evpool;
  std::vector<int> evkind;  // kernel kind of each recorded pair
  double kms[3] = {0, 0, 0};
  int64_t kn[3] = {0, 0, 0};
  // graph replay (gpe_set_graph): a captured chunk of gsteps steps whose kernels read
  // the chunk's first step index from kdev
  int64_t gsteps = 0;
  int64_t* kdev = nullptr;
  int64_t kval = 0;
  cudaGraphExec_t gexec = nullptr;
  int64_t glaunches = 0;
  // every setter that changes what the passes read (tables, coefficients, pump, noise,
  // tiling, RNG key) bumps gen; a captured graph holds the kernel arguments of the
  // generation it was captured in and is recaptured when gen moves on
  int64_t gen = 0;
  int64_t gexec_gen = -1;
  // save chunks as graphs (one per ring slot): save_every steps between two saves, the
  // last row pass writing the save into its slot; key (steps, save buffer, gen)
  cudaGraphExec_t sgexec[4] = {nullptr, nullptr, nullptr, nullptr};
  int64_t sg_steps = 0, sg_gen = -1, sg_launches = 0;
  void* sg_buf = nullptr;
  // runs without saves: chunks of kRunChunk steps continuing the run, as one graph
  cudaGraphExec_t cgexec = nullptr;
  int64_t cg_gen = -1, cg_launches = 0;
  // energy diagnostics: transformed copy of the state, FP64 D and V samples on the device
  void* escr[2] = {nullptr, nullptr};
  double2* dsamp = nullptr;
  double2* vsamp = nullptr;
  std::string err;
};

static std::string g_create_error;
static const char* kVersion = "libgpe " "1.0" " (sm_103a; StrangSplitting backend)";

static int fail(gpe_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  else g_create_error = buf;
  return code;
}

#define CK(h, call)                                                                        \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(h, e_ == cudaErrorMemoryAllocation ? GPE_ERR_NOMEM : GPE_ERR_CUDA,      \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                        \
  } while (0)

#define LK(h, call)                                                                        \
  do {                                                                                     \
    int e_ = (call);                                                                       \
    if (e_ != 0) return fail(h, GPE_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)e_)); \
  } while (0)

static bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

// Two-component fields of at most this many points (all trajectories) take the fine line
// tiling unless a variant was set.  Measured per step, one 512^2 two-component field:
// 53.3 / 22.6 us fine against 55.3 / 26.7 us default (double-word / FP32); at 2^19 points
// and for one-component fields the default tiling is faster.
constexpr int64_t kFinePoints = int64_t(1) << 18;

// NVTX range over an API call (visible in Nsight timelines; no cost without a tool)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
static int ilog2i(int64_t v) { int r = 0; while ((1ll << r) < v) ++r; return r; }

// FP64 -> double word: hi = fl32(v), lo = fl32(v - hi)
static inline void split_dw(double v, float* hl) {
  const float hi = (float)v;
  hl[0] = hi;
  hl[1] = (float)(v - (double)hi);
}

// Upload n complex FP64 values in the handle's pass precision (double2, float2, or
// the double-word layout {re.hi, re.lo, im.hi, im.lo}).
static int upload_complex(gpe_handle* h, void** dst, const cd* src, size_t n) {
  if (!*dst) CK(h, cudaMalloc(dst, n * h->csz));
  if (h->prec == gpe::PREC_F64) {
    CK(h, cudaMemcpy(*dst, src, n * 16, cudaMemcpyHostToDevice));
  } else if (h->prec == gpe::PREC_DW) {
    std::vector<float> tmp(4 * n);
    for (size_t i = 0; i < n; ++i) { split_dw(src[i].real(), &tmp[4 * i]); split_dw(src[i].imag(), &tmp[4 * i + 2]); }
    CK(h, cudaMemcpy(*dst, tmp.data(), n * 16, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> tmp(2 * n);
    for (size_t i = 0; i < n; ++i) { tmp[2 * i] = (float)src[i].real(); tmp[2 * i + 1] = (float)src[i].imag(); }
    CK(h, cudaMemcpy(*dst, tmp.data(), n * 8, cudaMemcpyHostToDevice));
  }
  return GPE_OK;
}
// Upload n complex FP64 table entries (exp(-i dt D), exp(-i dt/2 V)) at FP64 accuracy in
// every pass precision: double2 for FP64 passes, {re.hi, re.lo, im.hi, im.lo} floats for
// the double-word and FP32 passes (16 bytes an entry either way).
// Q62 of v (|v| <= 1) as {hi, lo} with v 2^62 = hi 2^32 + lo and lo signed; a lo of -2^31
// (whose negation would overflow) moves the value by one unit, 2^-62
static void q62_split(long double v, int32_t out[2]) {
  long long q = std::llround(std::ldexp(v, 62));
  if ((int32_t)(uint32_t)(unsigned long long)q == INT32_MIN) q += 1;
  const int32_t lo = (int32_t)(uint32_t)(unsigned long long)q;
  out[0] = (int32_t)((q - (long long)lo) >> 32);
  out[1] = lo;
}
// Upload n complex FP64 entries (double2 for FP64 passes, hi/lo float pairs otherwise),
// with room for `extra` further 16-byte entries after them.
static int upload_table(gpe_handle* h, void** dst, const cd* src, size_t n, size_t extra = 0) {
  if (!*dst) CK(h, cudaMalloc(dst, (n + extra) * 16));
  if (h->prec == gpe::PREC_F64) {
    CK(h, cudaMemcpy(*dst, src, n * 16, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> tmp(4 * n);
    for (size_t i = 0; i < n; ++i) { split_dw(src[i].real(), &tmp[4 * i]); split_dw(src[i].imag(), &tmp[4 * i + 2]); }
    CK(h, cudaMemcpy(*dst, tmp.data(), n * 16, cudaMemcpyHostToDevice));
  }
  return GPE_OK;
}
// Upload n real FP64 values (double, float, or a {hi, lo} float pair).
static int upload_real(gpe_handle* h, void** dst, const double* src, size_t n) {
  if (!*dst) CK(h, cudaMalloc(dst, n * h->rsz));
  if (h->prec == gpe::PREC_F64) {
    CK(h, cudaMemcpy(*dst, src, n * 8, cudaMemcpyHostToDevice));
  } else if (h->prec == gpe::PREC_DW) {
    std::vector<float> tmp(2 * n);
    for (size_t i = 0; i < n; ++i) split_dw(src[i], &tmp[2 * i]);
    CK(h, cudaMemcpy(*dst, tmp.data(), n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; ++i) tmp[i] = (float)src[i];
    CK(h, cudaMemcpy(*dst, tmp.data(), n * 4, cudaMemcpyHostToDevice));
  }
  return GPE_OK;
}

// exp(A) for a 2x2 complex matrix: e^{tr/2} [cosh(s) I + sinh(s)/s (A - tr/2 I)],
// s^2 = ((a-d)/2)^2 + bc; sinh(s)/s by its series for small |s|.
static void expm2(const cd A[4], cd out[4]) {
  const cd a = A[0], b = A[1], c = A[2], d = A[3];
  const cd ht = 0.5 * (a + d);
  const cd s = std::sqrt(0.25 * (a - d) * (a - d) + b * c);
  const cd ch = std::cosh(s);
  cd sh;
  if (std::abs(s) < 1e-3) {
    const cd s2 = s * s;
    sh = 1.0 + s2 / 6.0 + s2 * s2 / 120.0;
  } else {
    sh = std::sinh(s) / s;
  }
  const cd e = std::exp(ht);
  out[0] = e * (ch + sh * (a - ht));
  out[3] = e * (ch + sh * (d - ht));
  out[1] = e * sh * b;
  out[2] = e * sh * c;
}

static int table_entries(const gpe_handle* h, int kind) {
  return kind == GPE_TABLE_SCALAR ? 1 : kind == GPE_TABLE_DIAG ? h->M : kind == GPE_TABLE_MATRIX ? h->M * h->M : 0;
}

// Build cis(-delta * f) * scale for samples f of the given kind; returns the kind
// actually stored (a 1x1 matrix or a 1-vector is stored as a scalar).
static int build_cis(gpe_handle* h, const double* f, int kind, double delta, double scale, std::vector<cd>& out) {
  const int64_t P = h->P;
  const int ne = table_entries(h, kind);
  const cd* fs = reinterpret_cast<const cd*>(f);
  out.resize((size_t)ne * P);
  if (kind == GPE_TABLE_MATRIX && h->M == 2) {
    for (int64_t p = 0; p < P; ++p) {
      cd A[4], E[4];
      for (int q = 0; q < 4; ++q) A[q] = cd(0.0, -delta) * fs[(size_t)q * P + p];
      expm2(A, E);
      for (int q = 0; q < 4; ++q) out[(size_t)q * P + p] = E[q] * scale;
    }
    return GPE_TABLE_MATRIX;
  }
  for (size_t i = 0; i < (size_t)ne * P; ++i) out[i] = std::exp(cd(0.0, -delta) * fs[i]) * scale;
  if (h->M == 1) return GPE_TABLE_SCALAR;
  return kind;
}

// Finiteness of n host values, split over host threads for large inputs (a field of
// 64 copies of 512^2 points is 33 M values; one thread would dominate the upload).
template <typename T> static bool all_finite_range(const T* v, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}
template <typename T> static bool all_finite_par(const T* v, size_t n) {
  const size_t kChunk = size_t(1) << 20;
  if (n < 4 * kChunk) return all_finite_range(v, n);
  unsigned nt = std::thread::hardware_concurrency();
  nt = nt == 0 ? 4 : (nt > 16 ? 16 : nt);
  std::vector<std::thread> pool;
  std::vector<char> ok(nt, 1);
  const size_t per = (n + nt - 1) / nt;
  for (unsigned k = 0; k < nt; ++k) {
    const size_t lo = k * per, hi = lo + per < n ? lo + per : n;
    if (lo >= hi) break;
    pool.emplace_back([&, k, lo, hi] { ok[k] = all_finite_range(v + lo, hi - lo); });
  }
  for (auto& th : pool) th.join();
  for (char c : ok)
    if (!c) return false;
  return true;
}
static bool all_finite(const double* v, size_t n) { return all_finite_par(v, n); }

extern "C" {

const char* gpe_version(void) { return kVersion; }

const char* gpe_last_error(const gpe_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int gpe_create(const gpe_desc* desc, gpe_handle** out) {
  if (!desc || !out) return fail(nullptr, GPE_ERR_INVALID, "null argument");
  *out = nullptr;
  if (desc->abi_version != GPE_ABI_VERSION)
    return fail(nullptr, GPE_ERR_INVALID, "abi_version %d, library has %d", desc->abi_version, GPE_ABI_VERSION);
  if (desc->ndim < 1 || desc->ndim > 3) return fail(nullptr, GPE_ERR_INVALID, "ndim must be 1, 2 or 3");
  if (desc->ncomp < 1 || desc->ncomp > 2) return fail(nullptr, GPE_ERR_UNSUPPORTED, "ncomp must be 1 or 2");
  if (desc->dtype != GPE_C128 && desc->dtype != GPE_C64) return fail(nullptr, GPE_ERR_INVALID, "bad dtype");
  if (desc->batch < 1) return fail(nullptr, GPE_ERR_INVALID, "batch must be >= 1");
  if ((desc->flags & GPE_FLAG_FP64_DW) && (desc->flags & GPE_FLAG_FP64_NATIVE))
    return fail(nullptr, GPE_ERR_INVALID, "GPE_FLAG_FP64_DW and GPE_FLAG_FP64_NATIVE exclude each other");
  if ((desc->flags & GPE_FLAG_FP64_DW) && desc->dtype != GPE_C128)
    return fail(nullptr, GPE_ERR_INVALID, "GPE_FLAG_FP64_DW applies to GPE_C128 fields only");
  if ((desc->flags & GPE_FLAG_FFT_BFP) && (desc->flags & (GPE_FLAG_FP64_DW | GPE_FLAG_FP64_NATIVE)))
    return fail(nullptr, GPE_ERR_INVALID, "GPE_FLAG_FFT_BFP, GPE_FLAG_FP64_NATIVE and GPE_FLAG_FP64_DW exclude each other");
  if ((desc->flags & (GPE_FLAG_FFT_BFP | GPE_FLAG_FP64_NATIVE)) && desc->dtype != GPE_C128)
    return fail(nullptr, GPE_ERR_INVALID, "GPE_FLAG_FFT_BFP and GPE_FLAG_FP64_NATIVE apply to GPE_C128 fields only");
  if (!(desc->dt > 0) || !std::isfinite(desc->dt)) return fail(nullptr, GPE_ERR_INVALID, "dt must be positive and finite");
  if (!std::isfinite(desc->t0)) return fail(nullptr, GPE_ERR_INVALID, "t0 must be finite");
  for (int a = 0; a < desc->ndim; ++a) {
    if (!is_pow2(desc->n[a]) || desc->n[a] < 16 || desc->n[a] > 4096)
      return fail(nullptr, GPE_ERR_UNSUPPORTED, "axis %d: n = %lld, need a power of two in [16, 4096]", a, (long long)desc->n[a]);
    if (!(desc->lengths[a] > 0) || !std::isfinite(desc->lengths[a]))
      return fail(nullptr, GPE_ERR_INVALID, "axis %d: length must be positive", a);
  }
  int dev = desc->device;
  if (dev >= 0) {
    cudaError_t se = cudaSetDevice(dev);
    if (se != cudaSuccess) return fail(nullptr, GPE_ERR_CUDA, "cudaSetDevice(%d) failed: %s", dev, cudaGetErrorString(se));
  } else if (cudaGetDevice(&dev) != cudaSuccess) {
    return fail(nullptr, GPE_ERR_CUDA, "no CUDA device");
  }
  gpe_handle* h = new gpe_handle();
  h->d = *desc;
  h->dev = dev;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && nsm > 0) h->nsm = nsm;
  h->M = desc->ncomp;
  h->dtype = desc->dtype;
  h->ndim = desc->ndim;
  h->prec = desc->dtype == GPE_C64 ? gpe::PREC_F32 : ((desc->flags & GPE_FLAG_FP64_DW) ? gpe::PREC_DW : gpe::PREC_F64);
  h->rsz = desc->dtype == GPE_C128 ? 8 : 4;
  h->csz = 2 * h->rsz;
  h->B = desc->batch;
  h->P = 1;
  h->dV = 1.0;
  for (int a = 0; a < h->ndim; ++a) {
    h->n[a] = desc->n[a];
    h->logn[a] = ilog2i(desc->n[a]);
    h->P *= desc->n[a];
    h->dV *= desc->lengths[a] / (double)desc->n[a];
  }
  h->t = desc->t0;
  auto bail = [&](int code) { gpe_destroy(h); return code; };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&h->ev0)) != cudaSuccess || (e = cudaEventCreate(&h->ev1)) != cudaSuccess) {
    fail(nullptr, GPE_ERR_CUDA, "stream/event creation failed: %s", cudaGetErrorString(e));
    return bail(GPE_ERR_CUDA);
  }
  const size_t bytes = (size_t)h->P * h->B * h->csz;
  for (int m = 0; m < h->M; ++m) {
    if ((e = cudaMalloc(&h->u[m], bytes)) != cudaSuccess) {
      fail(nullptr, GPE_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
      return bail(GPE_ERR_NOMEM);
    }
    cudaMemset(h->u[m], 0, bytes);
  }
  if ((e = cudaMalloc((void**)&h->red, 4 * sizeof(double))) != cudaSuccess) {
    fail(nullptr, GPE_ERR_NOMEM, "cudaMalloc failed: %s", cudaGetErrorString(e));
    return bail(GPE_ERR_NOMEM);
  }
  if ((e = cudaHostAlloc((void**)&h->hstat, sizeof(int32_t), cudaHostAllocMapped)) != cudaSuccess ||
      (e = cudaHostGetDevicePointer((void**)&h->dstat, h->hstat, 0)) != cudaSuccess) {
    fail(nullptr, GPE_ERR_NOMEM, "mapped status word: %s", cudaGetErrorString(e));
    return bail(GPE_ERR_NOMEM);
  }
  *h->hstat = 0;
  // twiddles w_N^k = exp(-2 pi i k / N) per axis, built in FP64 and kept at FP64 accuracy
  for (int a = 0; a < h->ndim; ++a) {
    const int64_t N = h->n[a];
    std::vector<cd> w((size_t)N);
    for (int64_t k = 0; k < N; ++k) {
      const double th = -2.0 * M_PI * (double)k / (double)N;
      w[(size_t)k] = cd(std::cos(th), std::sin(th));
    }
    int rc = upload_table(h, &h->tw[a], w.data(), (size_t)N, h->prec == gpe::PREC_F64 ? (size_t)N : 0);
    if (rc) { g_create_error = h->err; return bail(rc); }
    if (h->prec == gpe::PREC_F64) {
      // Q62 twiddles of the block floating point transforms after the FP64 ones
      std::vector<int32_t> q(4 * (size_t)N);
      for (int64_t k = 0; k < N; ++k) {
        const long double th = -2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)N;
        q62_split(std::cos(th), &q[4 * (size_t)k]);
        q62_split(std::sin(th), &q[4 * (size_t)k + 2]);
      }
      CK(h, cudaMemcpy((char*)h->tw[a] + 16 * (size_t)N, q.data(), 16 * (size_t)N, cudaMemcpyHostToDevice));
    }
  }
  cudaDeviceSynchronize();
  *out = h;
  return GPE_OK;
}

int gpe_destroy(gpe_handle* h) {
  if (!h) return GPE_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int m = 0; m < 2; ++m) {
    cudaFree(h->u[m]);
    cudaFree(h->pprof[m]);
    cudaFree(h->pcoef[m]);
    cudaFree(h->etaprof[m]);
  }
  for (int a = 0; a < 3; ++a) cudaFree(h->tw[a]);
  cudaFree(h->ktab);
  cudaFree(h->ktab_q);
  cudaFree(h->vtab);
  cudaFree(h->nlm);
  cudaFree(h->save_buf);
  if (h->pinned) cudaFreeHost(h->pinned);
  for (cudaEvent_t e : h->ring_ready) cudaEventDestroy(e);
  for (cudaEvent_t e : h->ring_done) cudaEventDestroy(e);
  if (h->cstream) cudaStreamDestroy(h->cstream);
  cudaFree(h->xi_buf);
  cudaFree(h->conv_buf);
  cudaFree(h->red);
  cudaFree(h->kdev);
  cudaFree(h->escr[0]);
  cudaFree(h->escr[1]);
  cudaFree(h->dsamp);
  cudaFree(h->vsamp);
  if (h->hstat) cudaFreeHost(h->hstat);
  for (cudaEvent_t e : h->evpool) cudaEventDestroy(e);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->ev_ext) cudaEventDestroy(h->ev_ext);
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  for (cudaGraphExec_t& g : h->sgexec)
    if (g) cudaGraphExecDestroy(g);
  if (h->cgexec) cudaGraphExecDestroy(h->cgexec);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return GPE_OK;
}

static int check_comp(gpe_handle* h, int comp) {
  if (!h) return GPE_ERR_INVALID;
  cudaSetDevice(h->dev);
  if (comp < 0 || comp >= h->M) return fail(h, GPE_ERR_INVALID, "component %d out of range [0, %d)", comp, h->M);
  return GPE_OK;
}

static int ensure(gpe_handle* h, void** buf, size_t* cap, size_t bytes);

int gpe_set_field(gpe_handle* h, int comp, const void* host) {
  NvtxRange nv("gpe_set_field");
  int rc = check_comp(h, comp);
  if (rc) return rc;
  if (!host) return fail(h, GPE_ERR_INVALID, "null field");
  const size_t n = (size_t)h->P * h->B;
  CK(h, cudaSetDevice(h->dev));
  // stage the caller's values on the device, check them there, and only then replace the
  // field: a rejected upload leaves the state as it was
  const bool f64 = h->dtype == GPE_C128;
  const size_t bytes = n * (f64 ? 16 : 8);
  rc = ensure(h, &h->conv_buf, &h->conv_cap, bytes);
  if (rc) return rc;
  CK(h, cudaMemcpyAsync(h->conv_buf, host, bytes, cudaMemcpyHostToDevice, h->stream));
  int* flag = reinterpret_cast<int*>(h->red);
  CK(h, cudaMemsetAsync(flag, 0, sizeof(int), h->stream));
  LK(h, gpe::launch_nonfinite(h->conv_buf, (int64_t)(2 * n), f64 ? 1 : 0, flag, h->stream));
  int bad = 0;
  CK(h, cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (bad) return fail(h, GPE_ERR_NONFINITE, "field %d has NaN or Inf", comp);
  if (h->prec == gpe::PREC_DW) {
    // FP64 and double-word complex numbers both take 16 bytes: split on the device
    LK(h, gpe::launch_f64_to_dw(h->conv_buf, h->u[comp], (int64_t)n, h->stream));
  } else {
    CK(h, cudaMemcpyAsync(h->u[comp], h->conv_buf, n * h->csz, cudaMemcpyDeviceToDevice, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return GPE_OK;
}

int gpe_get_field(gpe_handle* h, int comp, void* host) {
  int rc = check_comp(h, comp);
  if (rc) return rc;
  if (!host) return fail(h, GPE_ERR_INVALID, "null destination");
  const size_t n = (size_t)h->P * h->B;
  CK(h, cudaSetDevice(h->dev));
  CK(h, cudaStreamSynchronize(h->stream));
  if (h->prec == gpe::PREC_DW) {
    // rounded to FP64 on the device through a bounded staging buffer, chunk by chunk
    const size_t chunk = std::min<size_t>(n, size_t(4) << 20);  // complex numbers (64 MiB)
    rc = ensure(h, &h->conv_buf, &h->conv_cap, chunk * 16);
    if (rc) return rc;
    for (size_t o = 0; o < n; o += chunk) {
      const size_t c = std::min(chunk, n - o);
      LK(h, gpe::launch_dw_to_f64((const char*)h->u[comp] + o * 16, h->conv_buf, (int64_t)c, h->stream));
      CK(h, cudaMemcpyAsync((char*)host + o * 16, h->conv_buf, c * 16, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    return GPE_OK;
  }
  CK(h, cudaMemcpy(host, h->u[comp], n * h->csz, cudaMemcpyDeviceToHost));
  return GPE_OK;
}

// Caller-owned device buffers are usually written and read by work on the device's
// legacy default stream (PyTorch's default).  The handle's stream does not synchronise
// with it, so copies to or from such a buffer first wait for the work queued there.
static int after_legacy_stream(gpe_handle* h) {
  if (!h->ev_ext) CK(h, cudaEventCreateWithFlags(&h->ev_ext, cudaEventDisableTiming));
  CK(h, cudaEventRecord(h->ev_ext, cudaStreamLegacy));
  CK(h, cudaStreamWaitEvent(h->stream, h->ev_ext, 0));
  return GPE_OK;
}

int gpe_set_field_dev(gpe_handle* h, int comp, const void* dev) {
  int rc = check_comp(h, comp);
  if (rc) return rc;
  if (!dev) return fail(h, GPE_ERR_INVALID, "null field");
  CK(h, cudaSetDevice(h->dev));
  if ((rc = after_legacy_stream(h))) return rc;
  if (h->prec == gpe::PREC_DW) {
    LK(h, gpe::launch_f64_to_dw(dev, h->u[comp], h->P * h->B, h->stream));
  } else {
    CK(h, cudaMemcpyAsync(h->u[comp], dev, (size_t)h->P * h->B * h->csz, cudaMemcpyDeviceToDevice, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return GPE_OK;
}

int gpe_get_field_dev(gpe_handle* h, int comp, void* dev) {
  int rc = check_comp(h, comp);
  if (rc) return rc;
  if (!dev) return fail(h, GPE_ERR_INVALID, "null destination");
  CK(h, cudaSetDevice(h->dev));
  if ((rc = after_legacy_stream(h))) return rc;
  if (h->prec == gpe::PREC_DW) {
    LK(h, gpe::launch_dw_to_f64(h->u[comp], dev, h->P * h->B, h->stream));
  } else {
    CK(h, cudaMemcpyAsync(dev, h->u[comp], (size_t)h->P * h->B * h->csz, cudaMemcpyDeviceToDevice, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return GPE_OK;
}

static int check_kind(gpe_handle* h, int kind) {
  if (kind != GPE_TABLE_SCALAR && kind != GPE_TABLE_DIAG && kind != GPE_TABLE_MATRIX)
    return fail(h, GPE_ERR_INVALID, "bad table kind %d", kind);
  return GPE_OK;
}

static int store_ktable(gpe_handle* h, const std::vector<cd>& tab, int kind) {
  cudaFree(h->ktab);
  cudaFree(h->ktab_q);
  h->ktab = h->ktab_q = nullptr;
  h->kkind = GPE_TABLE_NONE;
  int rc = upload_table(h, &h->ktab, tab.data(), tab.size());
  if (rc) return rc;
  if (h->prec == gpe::PREC_F64 && !(h->d.flags & GPE_FLAG_FP64_NATIVE)) {
    // the Q62 copy the block floating point column pass applies on the integer pipes:
    // entries times P 2^-kexp, kexp the least exponent that keeps every real and imaginary
    // part within 1 (P = 2^k, so the scaling is exact)
    double mx = 0.0;
    for (const cd& v : tab) mx = std::max(mx, std::max(std::fabs(v.real()), std::fabs(v.imag())));
    mx *= (double)h->P;
    int kexp = 0;
    if (mx > 0.0) {
      std::frexp(mx, &kexp);  // mx = f 2^kexp, f in [0.5, 1)
    }
    std::vector<int32_t> q(4 * tab.size());
    const long double s = std::ldexp((long double)h->P, -kexp);
    for (size_t i = 0; i < tab.size(); ++i) {
      q62_split(s * (long double)tab[i].real(), &q[4 * i]);
      q62_split(s * (long double)tab[i].imag(), &q[4 * i + 2]);
    }
    CK(h, cudaMalloc(&h->ktab_q, q.size() * sizeof(int32_t)));
    CK(h, cudaMemcpy(h->ktab_q, q.data(), q.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    int logp = 0;
    while ((int64_t(1) << logp) < h->P) ++logp;
    h->kq_exp = kexp - logp;
  }
  h->kkind = kind;
  return GPE_OK;
}

int gpe_set_dispersion(gpe_handle* h, const double* D, int kind) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  int rc = check_kind(h, kind);
  if (rc) return rc;
  if (!D) return fail(h, GPE_ERR_INVALID, "null dispersion");
  const size_t ne = (size_t)table_entries(h, kind) * h->P;
  if (!all_finite(D, 2 * ne)) return fail(h, GPE_ERR_NONFINITE, "dispersion has NaN or Inf");
  std::vector<cd> tab;
  // exp(-i dt D) with the 1/P of the normalised inverse transform folded in (exact: P is 2^k)
  const int stored = build_cis(h, D, kind, h->d.dt, 1.0 / (double)h->P, tab);
  h->Dsamples.assign(reinterpret_cast<const cd*>(D), reinterpret_cast<const cd*>(D) + ne);
  h->dkind = kind;
  cudaFree(h->dsamp);
  h->dsamp = nullptr;
  return store_ktable(h, tab, stored);
}

int gpe_set_ktable(gpe_handle* h, const double* table, int kind) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  int rc = check_kind(h, kind);
  if (rc) return rc;
  if (!table) return fail(h, GPE_ERR_INVALID, "null table");
  const size_t ne = (size_t)table_entries(h, kind) * h->P;
  if (!all_finite(table, 2 * ne)) return fail(h, GPE_ERR_NONFINITE, "k-space table has NaN or Inf");
  std::vector<cd> tab(ne);
  const cd* src = reinterpret_cast<const cd*>(table);
  const double s = 1.0 / (double)h->P;
  for (size_t i = 0; i < ne; ++i) tab[i] = src[i] * s;
  int stored = kind;
  if (h->M == 1) stored = GPE_TABLE_SCALAR;
  h->Dsamples.clear();
  h->dkind = GPE_TABLE_NONE;
  return store_ktable(h, tab, stored);
}

static int store_vtable(gpe_handle* h, const std::vector<cd>& tab, int kind) {
  if (h->nl_matrix && kind == GPE_TABLE_DIAG)
    return fail(h, GPE_ERR_UNSUPPORTED, "a matrix nonlinearity with a diagonal potential is not supported");
  if (kind == GPE_TABLE_MATRIX && (h->nl_on[0] || h->nl_on[1]))
    return fail(h, GPE_ERR_UNSUPPORTED, "a matrix potential with a diagonal nonlinearity is undefined (SVector * SMatrix)");
  cudaFree(h->vtab);
  h->vtab = nullptr;
  h->vkind = GPE_TABLE_NONE;
  int rc = upload_table(h, &h->vtab, tab.data(), tab.size());
  if (rc) return rc;
  h->vkind = kind;
  return GPE_OK;
}

int gpe_set_potential(gpe_handle* h, const double* V, int kind) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  int rc = check_kind(h, kind);
  if (rc) return rc;
  if (!V) return fail(h, GPE_ERR_INVALID, "null potential");
  const size_t ne = (size_t)table_entries(h, kind) * h->P;
  if (!all_finite(V, 2 * ne)) return fail(h, GPE_ERR_NONFINITE, "potential has NaN or Inf");
  std::vector<cd> tab;
  const int stored = build_cis(h, V, kind, 0.5 * h->d.dt, 1.0, tab);
  h->Vsamples.assign(reinterpret_cast<const cd*>(V), reinterpret_cast<const cd*>(V) + ne);
  h->vskind = kind;
  cudaFree(h->vsamp);
  h->vsamp = nullptr;
  return store_vtable(h, tab, stored);
}

int gpe_set_vtable(gpe_handle* h, const double* table, int kind) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  int rc = check_kind(h, kind);
  if (rc) return rc;
  if (!table) return fail(h, GPE_ERR_INVALID, "null table");
  const size_t ne = (size_t)table_entries(h, kind) * h->P;
  if (!all_finite(table, 2 * ne)) return fail(h, GPE_ERR_NONFINITE, "potential table has NaN or Inf");
  std::vector<cd> tab(reinterpret_cast<const cd*>(table), reinterpret_cast<const cd*>(table) + ne);
  h->Vsamples.clear();
  h->vskind = GPE_TABLE_NONE;
  return store_vtable(h, tab, h->M == 1 ? GPE_TABLE_SCALAR : kind);
}

int gpe_set_nonlinearity(gpe_handle* h, const double* g, const double* c) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  const int M = h->M;
  double gg[2][2][2] = {}, cc[2][2] = {};
  if (g) {
    if (!all_finite(g, 2 * M * M)) return fail(h, GPE_ERR_NONFINITE, "nonlinearity g has NaN or Inf");
    for (int j = 0; j < M; ++j)
      for (int l = 0; l < M; ++l) { gg[j][l][0] = g[2 * (j * M + l)]; gg[j][l][1] = g[2 * (j * M + l) + 1]; }
  }
  if (c) {
    if (!all_finite(c, 2 * M)) return fail(h, GPE_ERR_NONFINITE, "nonlinearity c has NaN or Inf");
    for (int j = 0; j < M; ++j) { cc[j][0] = c[2 * j]; cc[j][1] = c[2 * j + 1]; }
  }
  int on[2] = {0, 0};
  for (int j = 0; j < M; ++j) {
    for (int l = 0; l < M; ++l) on[j] |= (gg[j][l][0] != 0 || gg[j][l][1] != 0);
    on[j] |= (cc[j][0] != 0 || cc[j][1] != 0);
  }
  if ((on[0] || on[1]) && h->vkind == GPE_TABLE_MATRIX)
    return fail(h, GPE_ERR_UNSUPPORTED, "a diagonal nonlinearity with a matrix potential is undefined (SVector * SMatrix)");
  h->nl_matrix = 0;
  memcpy(h->g, gg, sizeof gg);
  memcpy(h->c, cc, sizeof cc);
  h->nl_on[0] = on[0];
  h->nl_on[1] = on[1];
  return GPE_OK;
}

int gpe_set_matrix_nonlinearity(gpe_handle* h, const double* g, const double* c) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  if (h->M != 2) return fail(h, GPE_ERR_UNSUPPORTED, "the matrix nonlinearity needs two components");
  if (!g) return fail(h, GPE_ERR_INVALID, "null coefficients");
  if (!all_finite(g, 16) || (c && !all_finite(c, 8))) return fail(h, GPE_ERR_NONFINITE, "nonlinearity has NaN or Inf");
  if (h->vkind == GPE_TABLE_DIAG)
    return fail(h, GPE_ERR_UNSUPPORTED, "a matrix nonlinearity with a diagonal potential is not supported");
  double coef[24];
  for (int q = 0; q < 16; ++q) coef[q] = g[q];
  for (int q = 0; q < 8; ++q) coef[16 + q] = c ? c[q] : 0.0;
  CK(h, cudaSetDevice(h->dev));
  if (!h->nlm) CK(h, cudaMalloc(&h->nlm, sizeof coef));
  CK(h, cudaMemcpyAsync(h->nlm, coef, sizeof coef, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->nl_matrix = 1;
  h->nl_on[0] = h->nl_on[1] = 0;
  return GPE_OK;
}

int gpe_set_pump(gpe_handle* h, int comp, const double* profile, int profile_complex, const double* amp, int64_t n_amp) {
  if (h) ++h->gen;
  int rc = check_comp(h, comp);
  if (rc) return rc;
  const size_t P = (size_t)h->P;
  // check everything before touching the handle: a refused call keeps the old pump
  if (profile) {
    if (!amp || n_amp < 1) return fail(h, GPE_ERR_INVALID, "pump needs at least one amplitude");
    if (!all_finite(profile, profile_complex ? 2 * P : P)) return fail(h, GPE_ERR_NONFINITE, "pump profile has NaN or Inf");
    if (!all_finite(amp, 2 * (size_t)n_amp)) return fail(h, GPE_ERR_NONFINITE, "pump amplitude has NaN or Inf");
  }
  cudaFree(h->pprof[comp]);
  h->pprof[comp] = nullptr;
  cudaFree(h->pcoef[comp]);
  h->pcoef[comp] = nullptr;
  h->pcoef_n[comp] = 0;
  h->pprof_host[comp].clear();
  h->pump_uniform &= ~(1 << comp);
  if (!profile) return GPE_OK;
  std::vector<cd>& ph = h->pprof_host[comp];
  ph.resize(P);
  for (size_t p = 0; p < P; ++p) ph[p] = profile_complex ? cd(profile[2 * p], profile[2 * p + 1]) : cd(profile[p], 0.0);
  // a profile with one value c everywhere (a uniform drive, e.g. F = 1 of the
  // truncated-Wigner example) is folded into the coefficients: the passes then apply
  // (dt/4) a(t) c without a per-point profile load
  bool uniform = true;
  for (size_t p = 1; p < P && uniform; ++p) uniform = ph[p] == ph[0];
  h->pump_uniform = uniform ? (h->pump_uniform | (1 << comp)) : (h->pump_uniform & ~(1 << comp));
  {
    // (dt/4) a(t_h): the delta/2 = dt/4 factor of src/kernels.jl:45-46, formed in FP64
    std::vector<cd> coef((size_t)n_amp);
    const cd fold = uniform ? ph[0] : cd(1.0, 0.0);
    for (int64_t i = 0; i < n_amp; ++i) coef[(size_t)i] = 0.25 * h->d.dt * cd(amp[2 * i], amp[2 * i + 1]) * fold;
    rc = upload_complex(h, &h->pcoef[comp], coef.data(), (size_t)n_amp);
    if (rc) return rc;
    h->pcoef_n[comp] = n_amp;
  }
  // All pumped components share one profile format: complex if any profile is complex.
  int want_cplx = 0;
  for (int m = 0; m < h->M; ++m)
    for (const cd& v : h->pprof_host[m])
      if (v.imag() != 0.0) { want_cplx = 1; break; }
  h->pprof_cplx = want_cplx;
  for (int m = 0; m < h->M; ++m) {
    cudaFree(h->pprof[m]);
    h->pprof[m] = nullptr;
    if (h->pprof_host[m].empty()) continue;
    if (want_cplx) {
      rc = upload_complex(h, &h->pprof[m], h->pprof_host[m].data(), P);
    } else {
      std::vector<double> re(P);
      for (size_t p = 0; p < P; ++p) re[p] = h->pprof_host[m][p].real();
      rc = upload_real(h, &h->pprof[m], re.data(), P);
    }
    if (rc) return rc;
  }
  return GPE_OK;
}

int gpe_set_noise(gpe_handle* h, int mode, uint64_t seed, const double* eta, const double* eta_profile) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  if (mode != GPE_NOISE_OFF && mode != GPE_NOISE_PHILOX && mode != GPE_NOISE_REPLAY)
    return fail(h, GPE_ERR_INVALID, "bad noise mode %d", mode);
  // check everything before touching the handle: a refused call keeps the old noise
  if (mode != GPE_NOISE_OFF) {
    if (!eta) return fail(h, GPE_ERR_INVALID, "noise needs eta");
    if (!all_finite(eta, 2 * h->M)) return fail(h, GPE_ERR_NONFINITE, "eta has NaN or Inf");
    if (eta_profile && !all_finite(eta_profile, (size_t)h->M * h->P))
      return fail(h, GPE_ERR_NONFINITE, "eta profile has NaN or Inf");
  }
  for (int m = 0; m < 2; ++m) { cudaFree(h->etaprof[m]); h->etaprof[m] = nullptr; }
  h->noise = mode;
  h->seed = seed;
  memset(h->eta, 0, sizeof h->eta);
  if (mode == GPE_NOISE_OFF) return GPE_OK;
  for (int m = 0; m < h->M; ++m) { h->eta[m][0] = eta[2 * m]; h->eta[m][1] = eta[2 * m + 1]; }
  if (eta_profile) {
    for (int m = 0; m < h->M; ++m) {
      int rc = upload_real(h, &h->etaprof[m], eta_profile + (size_t)m * h->P, (size_t)h->P);
      if (rc) return rc;
    }
  }
  return GPE_OK;
}

// Event pair around one launch when timing is on.
struct TimedLaunch {
  gpe_handle* h;
  int kind;
  size_t idx = 0;
  TimedLaunch(gpe_handle* hh, int k) : h(hh), kind(k) {
    if (!h->timing || h->capturing) return;
    idx = h->evkind.size();
    while (h->evpool.size() < 2 * (idx + 1)) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      h->evpool.push_back(e);
    }
    h->evkind.push_back(kind);
    cudaEventRecord(h->evpool[2 * idx], h->stream);
  }
  ~TimedLaunch() {
    if (h->timing && !h->capturing) cudaEventRecord(h->evpool[2 * idx + 1], h->stream);
  }
};

// Fill the coefficient part of the pass arguments.
static int pass_variant(const gpe_handle* h) {
  if (h->variant >= 0) return h->variant;
  return h->M == 2 && h->P * h->B <= kFinePoints ? 2 : 0;
}

// The compile-time specialised half step (every pass precision) that covers this handle's families, or
// LEAN_OFF: no potential, no noise, no matrix nonlinearity, a real nonlinearity, real and
// non-uniform pump profiles, and one of the component patterns of gpe::LeanKind.
static int lean_kind(const gpe_handle* h, const PassArgs& a) {
  if (h->vkind != GPE_TABLE_NONE || h->noise != GPE_NOISE_OFF || h->nl_matrix || h->pprof_cplx)
    return gpe::LEAN_OFF;
  int gm = 0, pm = 0;
  for (int j = 0; j < h->M; ++j) {
    if (a.nl_on[j] && a.nl_imag[j]) return gpe::LEAN_OFF;
    if (a.nl_on[j]) gm |= 1 << j;
    if (h->pprof[j]) {
      if ((h->pump_uniform >> j) & 1) return gpe::LEAN_OFF;
      pm |= 1 << j;
    }
  }
  const int dm = a.dens_mask;
  if (h->M == 1 && gm == 1 && dm == 1) return pm ? gpe::LEAN_M1_GP : gpe::LEAN_M1_G;
  if (h->M == 2 && gm == 2 && dm == 2 && pm == 1) return gpe::LEAN_M2_G1P0;
  if (h->M == 2 && gm == 3 && dm == 3 && pm == 0) return gpe::LEAN_M2_GG;
  return gpe::LEAN_OFF;
}

static PassArgs base_args(gpe_handle* h) {
  PassArgs a;
  memset(&a, 0, sizeof a);
  a.n0 = (int32_t)h->n[0];
  a.n1 = (int32_t)h->n[1];
  a.n2 = (int32_t)h->n[2];
  a.P = h->P;
  a.B = h->B;
  a.nsm = h->nsm;
  a.col_tma = (h->d.flags & GPE_FLAG_NO_TMA) ? 0 : (h->d.flags & GPE_FLAG_TMA) ? 1 : 2;
  a.fx = (h->prec == gpe::PREC_F64 && !(h->d.flags & GPE_FLAG_FP64_NATIVE)) ? 1 : 0;
  a.status = h->dstat;
  for (int m = 0; m < h->M; ++m) a.u[m] = h->u[m];
  a.ktab = h->ktab;
  a.kkind = h->kkind;
  a.ktab_q = h->ktab_q;
  a.kq_exp = h->kq_exp;
  a.vtab = h->vtab;
  a.vkind = h->vkind;
  float hl[2];
  a.dens_mask = 0;
  for (int j = 0; j < h->M; ++j)
    for (int l = 0; l < h->M; ++l)
      if (h->nl_on[j] && (h->g[j][l][0] != 0.0 || h->g[j][l][1] != 0.0)) a.dens_mask |= 1 << l;
  a.g_nz = 0;
  for (int j = 0; j < 2; ++j)
    for (int l = 0; l < 2; ++l)
      for (int r = 0; r < 2; ++r)
        if (h->g[j][l][r] != 0.0) a.g_nz |= 1 << (j * 4 + l * 2 + r);
  for (int j = 0; j < 2; ++j) {
    a.nl_on[j] = h->nl_on[j];
    a.nl_imag[j] = h->c[j][1] != 0.0;
    for (int l = 0; l < 2; ++l)
      for (int r = 0; r < 2; ++r) {
        a.g[j][l][r] = h->g[j][l][r];
        a.gd[j][l][r] = 0.5 * h->d.dt * h->g[j][l][r];
        split_dw(h->g[j][l][r], hl);
        a.gf[j][l][r] = hl[0];
        a.gl[j][l][r] = hl[1];
        if (r == 1 && h->g[j][l][1] != 0.0) a.nl_imag[j] = 1;
      }
    for (int r = 0; r < 2; ++r) {
      a.c[j][r] = h->c[j][r];
      a.cd[j][r] = 0.5 * h->d.dt * h->c[j][r];
      if (h->c[j][r] != 0.0) a.c_nz |= 1 << (j * 2 + r);
      split_dw(h->c[j][r], hl);
      a.cf[j][r] = hl[0];
      a.cl[j][r] = hl[1];
    }
  }
  for (int m = 0; m < h->M; ++m) {
    a.pprof[m] = h->pprof[m];
    a.pcoef[m] = h->pcoef[m];
    a.pcoef_n[m] = h->pcoef_n[m];
    a.etaprof[m] = h->etaprof[m];
  }
  a.pprof_cplx = h->pprof_cplx;
  a.pump_uniform = h->pump_uniform;
  a.nlm = h->nl_matrix ? h->nlm : nullptr;
  a.noise = h->noise;
  a.seed_lo = (uint32_t)h->seed;
  a.seed_hi = (uint32_t)(h->seed >> 32);
  a.traj0 = h->traj0;
  // -i sqrt(dt/2) eta  (src/kernels.jl:42 with delta = dt/2)
  const double sq = std::sqrt(0.5 * h->d.dt);
  for (int m = 0; m < h->M; ++m) {
    a.nfac[m][0] = sq * h->eta[m][1];
    a.nfac[m][1] = -sq * h->eta[m][0];
    for (int r = 0; r < 2; ++r) {
      split_dw(a.nfac[m][r], hl);
      a.nfacf[m][r] = hl[0];
      a.nfacl[m][r] = hl[1];
    }
  }
  a.lean = lean_kind(h, a);
  a.dt = h->d.dt;
  split_dw(0.5 * h->d.dt, hl);
  a.dthf = hl[0];
  a.dthl = hl[1];
  a.hA = a.hB = -1;
  return a;
}

static int ensure(gpe_handle* h, void** buf, size_t* cap, size_t bytes) {
  if (*cap >= bytes) return GPE_OK;
  cudaFree(*buf);
  *buf = nullptr;
  *cap = 0;
  CK(h, cudaMalloc(buf, bytes));
  *cap = bytes;
  return GPE_OK;
}

// Enqueue nsteps steps; saves go to save_dev (layout [m][slot][b][p]) with nsaves_total
// slots per component.  Returns the number of launches in *launches.
// Saves of a long two-pass run with a host output go through a ring of kSaveRing device
// slots: after the row pass that writes save s, a copy stream moves the slot to pinned
// host memory while the next steps run; the host moves finished slots into the caller's
// buffer and stays at most kSaveRing saves ahead, and the compute stream waits for a
// slot's copy before overwriting it.  Device memory for saves stays kSaveRing slots
// however many saves the run has.
constexpr int64_t kSaveRing = 4;
static_assert(sizeof(gpe_handle::sgexec) / sizeof(cudaGraphExec_t) == kSaveRing, "one save-chunk graph per ring slot");

struct SaveRing {
  gpe_handle* h;
  int64_t comp_stride;  // saves between components in the caller's buffer
  size_t plane_bytes;
  char* out;
  int64_t drained = 0;

  int before(int64_t s) {
    if (s < kSaveRing) return GPE_OK;
    int rc = drain(s - kSaveRing + 1);
    if (rc) return rc;
    CK(h, cudaStreamWaitEvent(h->stream, h->ring_done[s % kSaveRing], 0));
    return GPE_OK;
  }
  int after(int64_t s) {
    const int64_t r = s % kSaveRing;
    CK(h, cudaEventRecord(h->ring_ready[r], h->stream));
    CK(h, cudaStreamWaitEvent(h->cstream, h->ring_ready[r], 0));
    for (int m = 0; m < h->M; ++m) {
      const size_t off = ((size_t)m * kSaveRing + r) * plane_bytes;
      CK(h, cudaMemcpyAsync((char*)h->pinned + off, (char*)h->save_buf + off, plane_bytes, cudaMemcpyDeviceToHost,
                            h->cstream));
    }
    CK(h, cudaEventRecord(h->ring_done[r], h->cstream));
    return GPE_OK;
  }
  int drain(int64_t upto) {
    for (; drained < upto; ++drained) {
      const int64_t r = drained % kSaveRing;
      CK(h, cudaEventSynchronize(h->ring_done[r]));
      for (int m = 0; m < h->M; ++m)
        memcpy(out + ((size_t)m * comp_stride + drained) * plane_bytes,
               (char*)h->pinned + ((size_t)m * kSaveRing + r) * plane_bytes, plane_bytes);
    }
    return GPE_OK;
  }
};

// Matrix nonlinearity family: the real-space half steps run in a pointwise pass of their
// own (mat_kernel) between FFT-only line passes, so the line kernels of the diagonal
// families keep their register allocation.  Per step: kinetic part, then [half A][save]
// [half B] pointwise; the first half step of the run opens it.
static int enqueue_matrix_steps(gpe_handle* h, PassArgs a, int64_t k0, int64_t nsteps, int64_t save_every,
                                void* save_dev, int64_t nsaves_total, int64_t* launches, SaveRing* ring) {
  const int64_t plane = h->P * h->B;
  auto slot_ptrs = [&](PassArgs& pa, int64_t slot) {
    for (int m = 0; m < 2; ++m) pa.save[m] = (char*)save_dev + ((size_t)m * nsaves_total + slot) * plane * h->csz;
  };
  int64_t nl = 0;
  if (!h->ktab) {
    a.nsteps = nsteps;
    a.step0 = k0;
    a.save_every = save_every;
    a.save_stride = plane;
    if (save_every > 0) slot_ptrs(a, 0);
    TimedLaunch tl(h, 2);
    LK(h, gpe::launch_mat(h->prec, a, h->stream));
    *launches = 1;
    return GPE_OK;
  }
  // FFT-only argument blocks: every real-space term off
  PassArgs f = a;
  f.vkind = gpe::TAB_NONE;
  f.nl_on[0] = f.nl_on[1] = 0;
  f.nlm = nullptr;
  f.pprof[0] = f.pprof[1] = nullptr;
  f.noise = gpe::NOISE_OFF;
  f.save[0] = f.save[1] = nullptr;
  f.hA = f.hB = -1;
  f.save_every = 0;
  const int64_t nrows = h->P / h->n[0] * h->B;
  auto row = [&](int ifft, int fft) -> int {
    PassArgs r = f;
    r.tw = h->tw[0];
    r.do_ifft = ifft;
    r.do_fft = fft;
    TimedLaunch tl(h, 0);
    LK(h, gpe::launch_row(h->prec, 2, h->logn[0], r, nrows, h->stream));
    ++nl;
    return GPE_OK;
  };
  std::vector<std::pair<PassArgs, int>> cols;
  if (h->ndim == 2) {
    PassArgs c = f;
    c.tw = h->tw[1];
    c.ld = h->n[0];
    c.ostride = 0;
    c.nouter = 1;
    c.col_fwd = c.col_inv = 1;
    cols.push_back({c, h->logn[1]});
  } else if (h->ndim == 3) {
    PassArgs y = f;
    y.tw = h->tw[1];
    y.ld = h->n[0];
    y.ostride = h->n[0] * h->n[1];
    y.nouter = h->n[2];
    y.ktab = nullptr;
    PassArgs z = f;
    z.tw = h->tw[2];
    z.ld = h->n[0] * h->n[1];
    z.ostride = h->n[0];
    z.nouter = h->n[1];
    z.col_fwd = z.col_inv = 1;
    PassArgs yf = y, yi = y;
    yf.col_fwd = 1;
    yi.col_inv = 1;
    cols.push_back({yf, h->logn[1]});
    cols.push_back({z, h->logn[2]});
    cols.push_back({yi, h->logn[1]});
  }
  auto kinetic = [&]() -> int {
    if (h->ndim == 1) {
      PassArgs l = f;
      l.tw = h->tw[0];
      l.nsteps = 1;
      l.step0 = 0;
      TimedLaunch tl(h, 2);
      LK(h, gpe::launch_line1d(h->prec, 2, h->logn[0], l, h->stream));
      ++nl;
      return GPE_OK;
    }
    int rc = row(0, 1);
    if (rc) return rc;
    for (auto& cp : cols) {
      TimedLaunch tl(h, 1);
      LK(h, gpe::launch_col(h->prec, 2, cp.second, cp.first, h->stream));
      ++nl;
    }
    return row(1, 0);
  };
  {
    PassArgs m = a;
    m.nsteps = 0;
    m.hA = -1;
    m.hB = 2 * k0;
    m.save[0] = m.save[1] = nullptr;
    TimedLaunch tl(h, 2);
    LK(h, gpe::launch_mat(h->prec, m, h->stream));
    ++nl;
  }
  for (int64_t s = 0; s < nsteps; ++s) {
    int rc = kinetic();
    if (rc) return rc;
    const bool last = (s == nsteps - 1);
    PassArgs m = a;
    m.nsteps = 0;
    m.hA = 2 * (k0 + s) + 1;
    m.hB = last ? -1 : 2 * (k0 + s + 1);
    m.save[0] = m.save[1] = nullptr;
    const bool saving = save_every > 0 && (s + 1) % save_every == 0;
    const int64_t si = saving ? (s + 1) / save_every - 1 : -1;
    if (saving) {
      if (ring) {
        rc = ring->before(si);
        if (rc) return rc;
      }
      slot_ptrs(m, ring ? si % kSaveRing : si);
    }
    {
      TimedLaunch tl(h, 2);
      LK(h, gpe::launch_mat(h->prec, m, h->stream));
    }
    ++nl;
    if (saving && ring) {
      rc = ring->after(si);
      if (rc) return rc;
    }
  }
  *launches = nl;
  return GPE_OK;
}

// entry / final: emit the run's opening row pass (the first step's leading half step and
// FFT_x) and close it with the last step's trailing half step in real space; without
// them the steps continue a run (graph-captured save chunks).  k0: first step index
// (default: the handle's step count).
static int enqueue_steps(gpe_handle* h, int64_t nsteps, int64_t save_every, void* save_dev, int64_t nsaves_total,
                         const void* xi_dev, int64_t* launches, bool relative = false, SaveRing* ring = nullptr,
                         bool entry = true, bool final_pass = true, int64_t k0_at = -1) {
  PassArgs a = base_args(h);
  if (h->nl_matrix) {
    a.xi = xi_dev;
    const int64_t k0m = relative ? 0 : h->steps;
    if (relative) a.kbase = h->kdev;
    a.xi_h0 = 2 * k0m;
    return enqueue_matrix_steps(h, a, k0m, nsteps, save_every, save_dev, nsaves_total, launches, ring);
  }
  // relative: step indices count from the value in h->kdev (graph capture)
  const int64_t k0 = relative ? 0 : (k0_at >= 0 ? k0_at : h->steps);
  if (relative) a.kbase = h->kdev;
  a.xi = xi_dev;
  a.xi_h0 = 2 * k0;  // replayed xi are indexed from this run's first half step
  const int64_t plane = h->P * h->B;
  const bool has_k = h->ktab != nullptr;
  int64_t nl = 0;
  auto slot_ptrs = [&](PassArgs& pa, int64_t slot) {
    for (int m = 0; m < h->M; ++m)
      pa.save[m] = (char*)save_dev + ((size_t)m * nsaves_total + slot) * plane * h->csz;
  };
  if (!has_k || h->ndim == 1) {
    // pointwise-only problems and 1D lines run all steps in one resident launch
    a.nsteps = nsteps;
    a.step0 = k0;
    a.save_every = save_every;
    a.save_stride = plane;
    if (save_every > 0) slot_ptrs(a, 0);
    TimedLaunch tl(h, 2);
    if (!has_k) {
      LK(h, gpe::launch_nl_only(h->prec, h->M, a, h->stream));
    } else {
      a.tw = h->tw[0];
      LK(h, gpe::launch_line1d(h->prec, h->M, h->logn[0], a, h->stream));
    }
    *launches = 1;
    return GPE_OK;
  }
  // 2D square grids whose whole field fits in shared memory: one resident launch
  if (h->ndim == 2 && h->n[0] == h->n[1] && !(h->d.flags & GPE_FLAG_NO_RESIDENT) &&
      gpe::plane_fits(h->prec, h->M, h->logn[0])) {
    a.nsteps = nsteps;
    a.step0 = k0;
    a.save_every = save_every;
    a.save_stride = plane;
    if (save_every > 0) slot_ptrs(a, 0);
    a.tw = h->tw[0];
    a.tw2 = h->tw[1];
    TimedLaunch tl(h, 2);
    LK(h, gpe::launch_plane(h->prec, h->M, h->logn[0], a, h->stream));
    *launches = 1;
    return GPE_OK;
  }
  // 2D / 3D: entry row pass, then (column pass(es), row pass) per step.  3D column
  // passes: FFT_y, then FFT_z * table * iFFT_z, then iFFT_y.
  const int64_t nrows = h->P / h->n[0] * h->B;
  if (entry) {
    PassArgs r = a;
    r.tw = h->tw[0];
    r.do_ifft = 0;
    r.do_fft = 1;
    r.hA = 2 * k0;
    r.hB = -1;
    TimedLaunch tl(h, 0);
    LK(h, gpe::launch_row(h->prec, h->M, h->logn[0], r, nrows, h->stream, pass_variant(h)));
    ++nl;
  }
  std::vector<std::pair<PassArgs, int>> cols;  // (args, log2 line length)
  if (h->ndim == 2) {
    PassArgs c = a;
    c.tw = h->tw[1];
    c.ld = h->n[0];
    c.ostride = 0;
    c.nouter = 1;
    c.col_fwd = c.col_inv = 1;
    cols.push_back({c, h->logn[1]});
  } else {
    PassArgs y = a;  // lines along y at fixed z
    y.tw = h->tw[1];
    y.ld = h->n[0];
    y.ostride = h->n[0] * h->n[1];
    y.nouter = h->n[2];
    y.ktab = nullptr;
    PassArgs z = a;  // lines along z at fixed y, carrying the k-space table
    z.tw = h->tw[2];
    z.ld = h->n[0] * h->n[1];
    z.ostride = h->n[0];
    z.nouter = h->n[1];
    z.col_fwd = z.col_inv = 1;
    PassArgs yf = y, yi = y;
    yf.col_fwd = 1;
    yi.col_inv = 1;
    cols.push_back({yf, h->logn[1]});
    cols.push_back({z, h->logn[2]});
    cols.push_back({yi, h->logn[1]});
  }
  for (int64_t s = 0; s < nsteps; ++s) {
    for (auto& cp : cols) {
      TimedLaunch tl(h, 1);
      LK(h, gpe::launch_col(h->prec, h->M, cp.second, cp.first, h->stream, pass_variant(h)));
      ++nl;
    }
    const bool last = final_pass && (s == nsteps - 1);
    PassArgs rr = a;
    rr.tw = h->tw[0];
    rr.do_ifft = 1;
    rr.hA = 2 * (k0 + s) + 1;
    rr.hB = last ? -1 : 2 * (k0 + s + 1);
    rr.do_fft = last ? 0 : 1;
    const bool saving = save_every > 0 && (s + 1) % save_every == 0;
    const int64_t si = saving ? (s + 1) / save_every - 1 : -1;
    if (saving) {
      if (ring) {
        const int rc = ring->before(si);
        if (rc) return rc;
      }
      slot_ptrs(rr, ring ? si % kSaveRing : si);
    }
    {
      TimedLaunch tl(h, 0);
      LK(h, gpe::launch_row(h->prec, h->M, h->logn[0], rr, nrows, h->stream, pass_variant(h)));
    }
    if (saving && ring) {
      const int rc = ring->after(si);
      if (rc) return rc;
    }
    ++nl;
  }
  *launches = nl;
  return GPE_OK;
}

// Capture gsteps steps (plus the step-counter advance) into a graph once.
static int capture_chunk(gpe_handle* h, cudaStream_t st, int64_t* launches) {
  h->capturing = 1;
  int64_t nl = 0;
  const int rc = enqueue_steps(h, h->gsteps, 0, nullptr, 0, nullptr, &nl, true);
  h->capturing = 0;
  if (rc) return rc;
  LK(h, gpe::launch_advance(h->kdev, h->gsteps, st));
  *launches = nl + 1;
  return GPE_OK;
}

static int ensure_graph(gpe_handle* h) {
  if (!h->kdev) CK(h, cudaMalloc((void**)&h->kdev, sizeof(int64_t)));
  if (h->gexec && h->gexec_gen == h->gen) return GPE_OK;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  cudaGraph_t g = nullptr;
  CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int64_t nl = 0;
  const int rc = capture_chunk(h, h->stream, &nl);
  const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ec != cudaSuccess) return fail(h, GPE_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
  const cudaError_t ei = cudaGraphInstantiate(&h->gexec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) return fail(h, GPE_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ei));
  h->glaunches = nl;
  h->gexec_gen = h->gen;
  return GPE_OK;
}

// Save chunks as graphs, one per ring slot: save_every steps continuing a run (no opening
// or closing pass), the last row pass writing its save into the slot and going on into
// the next step; the kernels read the chunk's first step index from kdev, which the
// chunk advances at its end.
static int ensure_save_graphs(gpe_handle* h, int64_t save_every) {
  if (!h->kdev) CK(h, cudaMalloc((void**)&h->kdev, sizeof(int64_t)));
  if (h->sgexec[0] && h->sg_steps == save_every && h->sg_gen == h->gen && h->sg_buf == h->save_buf) return GPE_OK;
  for (cudaGraphExec_t& g : h->sgexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  const size_t plane_bytes = (size_t)h->P * h->B * h->csz;
  for (int r = 0; r < kSaveRing; ++r) {
    cudaGraph_t g = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->capturing = 1;
    int64_t nl = 0;
    int rc = enqueue_steps(h, save_every, save_every, (char*)h->save_buf + r * plane_bytes, kSaveRing, nullptr, &nl,
                           true, nullptr, false, false);
    if (rc == GPE_OK && gpe::launch_advance(h->kdev, save_every, h->stream) != 0)
      rc = fail(h, GPE_ERR_CUDA, "step-counter advance failed");
    h->capturing = 0;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return rc ? rc : fail(h, GPE_ERR_CUDA, "save-chunk capture failed: %s", cudaGetErrorString(ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&h->sgexec[r], g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(h, GPE_ERR_CUDA, "save-chunk instantiate failed: %s", cudaGetErrorString(ei));
    h->sg_launches = nl + 1;
  }
  h->sg_steps = save_every;
  h->sg_gen = h->gen;
  h->sg_buf = h->save_buf;
  return GPE_OK;
}

// A run whose saves stream through the ring, one graph launch per save chunk: the
// opening row pass, chunks 0 .. nsaves-2 as graphs, then the last chunk launched directly
// with the closing pass.  The passes and their order are those of the direct launches,
// so the results are identical; the launch gaps between the passes of a chunk go.
// (the chunk graphs are ready: ensure_save_graphs)
static int run_saves_graphed(gpe_handle* h, int64_t nsteps, int64_t save_every, SaveRing& ring, int64_t* launches) {
  const int64_t nsaves = nsteps / save_every;
  int64_t nl = 0, total = 0;
  int rc = enqueue_steps(h, 0, 0, nullptr, 0, nullptr, &nl, false, nullptr, true, false);  // opening pass
  if (rc) return rc;
  total += nl;
  h->kval = h->steps;
  CK(h, cudaMemcpyAsync(h->kdev, &h->kval, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  for (int64_t si = 0; si + 1 < nsaves; ++si) {
    if ((rc = ring.before(si))) return rc;
    CK(h, cudaGraphLaunch(h->sgexec[si % kSaveRing], h->stream));
    if ((rc = ring.after(si))) return rc;
    total += h->sg_launches;
  }
  const int64_t si = nsaves - 1;
  if ((rc = ring.before(si))) return rc;
  const size_t plane_bytes = (size_t)h->P * h->B * h->csz;
  rc = enqueue_steps(h, save_every, save_every, (char*)h->save_buf + (si % kSaveRing) * plane_bytes, kSaveRing, nullptr,
                     &nl, false, nullptr, false, true, h->steps + si * save_every);
  if (rc) return rc;
  if ((rc = ring.after(si))) return rc;
  *launches = total + nl;
  return GPE_OK;
}

// Runs without saves: the opening row pass, then chunks of kRunChunk steps as one graph
// (continuing the run, step indices from kdev), then the remaining 1 .. kRunChunk steps
// launched directly with the closing pass.  Same passes in the same order as direct
// launches, so the same results; fewer launch gaps between the passes of small fields.
constexpr int64_t kRunChunk = 32;

static int ensure_chunk_graph(gpe_handle* h) {
  if (!h->kdev) CK(h, cudaMalloc((void**)&h->kdev, sizeof(int64_t)));
  if (h->cgexec && h->cg_gen != h->gen) {
    cudaGraphExecDestroy(h->cgexec);
    h->cgexec = nullptr;
  }
  if (!h->cgexec) {
    cudaGraph_t g = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->capturing = 1;
    int64_t nl = 0;
    int rc = enqueue_steps(h, kRunChunk, 0, nullptr, 0, nullptr, &nl, true, nullptr, false, false);
    if (rc == GPE_OK && gpe::launch_advance(h->kdev, kRunChunk, h->stream) != 0)
      rc = fail(h, GPE_ERR_CUDA, "step-counter advance failed");
    h->capturing = 0;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return rc ? rc : fail(h, GPE_ERR_CUDA, "chunk capture failed: %s", cudaGetErrorString(ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&h->cgexec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(h, GPE_ERR_CUDA, "chunk instantiate failed: %s", cudaGetErrorString(ei));
    h->cg_launches = nl + 1;
    h->cg_gen = h->gen;
  }
  return GPE_OK;
}

// (the chunk graph is ready: ensure_chunk_graph)
static int run_chunks_graphed(gpe_handle* h, int64_t nsteps, int64_t* launches) {
  int64_t nl = 0, total = 0;
  int rc = enqueue_steps(h, 0, 0, nullptr, 0, nullptr, &nl, false, nullptr, true, false);  // opening pass
  if (rc) return rc;
  total += nl;
  const int64_t nchunks = (nsteps - 1) / kRunChunk;
  h->kval = h->steps;
  CK(h, cudaMemcpyAsync(h->kdev, &h->kval, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  for (int64_t c = 0; c < nchunks; ++c) CK(h, cudaGraphLaunch(h->cgexec, h->stream));
  total += nchunks * h->cg_launches;
  const int64_t done = nchunks * kRunChunk;
  rc = enqueue_steps(h, nsteps - done, 0, nullptr, 0, nullptr, &nl, false, nullptr, false, true, h->steps + done);
  if (rc) return rc;
  *launches = total + nl;
  return GPE_OK;
}

static int replay_graph(gpe_handle* h, int64_t nsteps, int64_t* launches) {
  h->kval = h->steps;
  CK(h, cudaMemcpyAsync(h->kdev, &h->kval, sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  for (int64_t r = 0; r < nsteps / h->gsteps; ++r) CK(h, cudaGraphLaunch(h->gexec, h->stream));
  *launches = h->glaunches * (nsteps / h->gsteps);
  return GPE_OK;
}

// A device wait that ran out of time left 1 in the status word: report it once.
static int take_status(gpe_handle* h) {
  if (!h->hstat || !*(volatile int32_t*)h->hstat) return GPE_OK;
  *(volatile int32_t*)h->hstat = 0;
  return fail(h, GPE_ERR_TIMEOUT, "a device wait exceeded its limit (a TMA tile did not arrive); the results of this "
                                  "run are not valid");
}

static int run_common(gpe_handle* h, int64_t nsteps, int64_t save_every, void* out, bool out_is_dev, double* ts_out,
                      const void* xi_host, int64_t comp_stride = -1) {
  if (!h) return GPE_ERR_INVALID;
  NvtxRange nv("gpe_run");
  CK(h, cudaSetDevice(h->dev));
  if (nsteps < 0) return fail(h, GPE_ERR_INVALID, "nsteps must be >= 0");
  if (save_every < 0) return fail(h, GPE_ERR_INVALID, "save_every must be >= 0");
  if (save_every > 0 && nsteps % save_every != 0)
    return fail(h, GPE_ERR_INVALID, "nsteps (%lld) must be a multiple of save_every (%lld)", (long long)nsteps,
                (long long)save_every);
  const int64_t nsaves = save_every > 0 ? nsteps / save_every : 0;
  if (nsaves > 0 && !out) return fail(h, GPE_ERR_INVALID, "null save buffer");
  if (comp_stride < 0) comp_stride = nsaves;  // host output: component m, slot s at m*comp_stride + s
  if (comp_stride < nsaves) return fail(h, GPE_ERR_INVALID, "component stride %lld < %lld saves",
                                        (long long)comp_stride, (long long)nsaves);
  for (int m = 0; m < h->M; ++m)
    if (h->pprof[m] && h->pcoef_n[m] > 1 && h->pcoef_n[m] < 2 * (h->steps + nsteps) + 1)
      return fail(h, GPE_ERR_INVALID, "pump %d has %lld amplitudes, %lld steps need %lld", m, (long long)h->pcoef_n[m],
                  (long long)(h->steps + nsteps), (long long)(2 * (h->steps + nsteps) + 1));
  if (h->noise == GPE_NOISE_REPLAY && !xi_host)
    return fail(h, GPE_ERR_INVALID, "noise mode is replay: use gpe_run_replay");
  if (xi_host && h->noise != GPE_NOISE_REPLAY) return fail(h, GPE_ERR_INVALID, "gpe_run_replay needs noise mode replay");
  h->last_ms = 0.0;
  h->last_launches = 0;
  if (nsteps == 0) return GPE_OK;
  const size_t plane_bytes = (size_t)h->P * h->B * h->csz;
  if (xi_host) {
    const size_t xb = (size_t)2 * nsteps * h->M * plane_bytes;
    int rc = ensure(h, &h->xi_buf, &h->xi_cap, xb);
    if (rc) return rc;
    CK(h, cudaMemcpy(h->xi_buf, xi_host, xb, cudaMemcpyHostToDevice));
    // replayed draws arrive as FP64; a double-word state needs them split (in place:
    // both layouts take 16 bytes per complex number)
    if (h->prec == gpe::PREC_DW) LK(h, gpe::launch_f64_to_dw(h->xi_buf, h->xi_buf, (int64_t)(xb / 16), h->stream));
  }
  void* save_dev = nullptr;
  // the two-pass path writes one save per row pass, so a ring can stream them out
  const bool single_launch = !h->ktab || (!h->nl_matrix && (h->ndim == 1 || (h->ndim == 2 && h->n[0] == h->n[1] &&
                                                                            !(h->d.flags & GPE_FLAG_NO_RESIDENT) &&
                                                                            gpe::plane_fits(h->prec, h->M, h->logn[0]))));
  const bool use_ring = nsaves > kSaveRing && !out_is_dev && !single_launch;
  SaveRing ring{h, comp_stride, plane_bytes, (char*)out};
  if (nsaves > 0) {
    if (out_is_dev) {
      if (int rc = after_legacy_stream(h)) return rc;
      save_dev = out;
    } else {
      const int64_t slots = use_ring ? kSaveRing : nsaves;
      int rc = ensure(h, &h->save_buf, &h->save_cap, (size_t)h->M * slots * plane_bytes);
      if (rc) return rc;
      save_dev = h->save_buf;
    }
  }
  if (use_ring) {
    const size_t pb = (size_t)h->M * kSaveRing * plane_bytes;
    if (h->pinned_cap < pb) {
      if (h->pinned) cudaFreeHost(h->pinned);
      h->pinned = nullptr;
      h->pinned_cap = 0;
      CK(h, cudaHostAlloc(&h->pinned, pb, cudaHostAllocDefault));
      h->pinned_cap = pb;
    }
    if (!h->cstream) CK(h, cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking));
    while ((int64_t)h->ring_ready.size() < kSaveRing) {
      cudaEvent_t a, b;
      CK(h, cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
      CK(h, cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
      h->ring_ready.push_back(a);
      h->ring_done.push_back(b);
    }
  }
  h->evkind.clear();
  const bool graph = h->gsteps > 0 && save_every == 0 && !xi_host && nsteps % h->gsteps == 0;
  // save chunks / step chunks as graphs (not with per-launch timing, replayed noise or
  // the matrix family); captured before the run's start event, so capture time is not
  // counted as run time
  const bool direct_ok = !xi_host && !h->nl_matrix && !h->timing;
  const bool gsaves = !graph && use_ring && direct_ok;
  const bool gchunks = !graph && !gsaves && nsaves == 0 && nsteps > 2 * kRunChunk && direct_ok && !single_launch;
  if (graph) {
    int rc = ensure_graph(h);
    if (rc) return rc;
  }
  if (gsaves) {
    int rc = ensure_save_graphs(h, save_every);
    if (rc) return rc;
  }
  if (gchunks) {
    int rc = ensure_chunk_graph(h);
    if (rc) return rc;
  }
  CK(h, cudaEventRecord(h->ev0, h->stream));
  int64_t launches = 0;
  if (graph) {
    int rc = replay_graph(h, nsteps, &launches);
    if (rc) return rc;
  } else if (gsaves) {
    int rc = run_saves_graphed(h, nsteps, save_every, ring, &launches);
    if (rc) return rc;
  } else if (gchunks) {
    int rc = run_chunks_graphed(h, nsteps, &launches);
    if (rc) return rc;
  } else {
    int rc = enqueue_steps(h, nsteps, save_every, save_dev, use_ring ? kSaveRing : nsaves,
                           xi_host ? h->xi_buf : nullptr, &launches, false, use_ring ? &ring : nullptr);
    if (rc) return rc;
  }
  CK(h, cudaEventRecord(h->ev1, h->stream));
  CK(h, cudaEventSynchronize(h->ev1));
  if (int rc = take_status(h)) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  h->last_launches = launches;
  for (int k = 0; k < 3; ++k) { h->kms[k] = 0.0; h->kn[k] = 0; }
  for (size_t i = 0; i < h->evkind.size(); ++i) {
    float e = 0.f;
    cudaEventElapsedTime(&e, h->evpool[2 * i], h->evpool[2 * i + 1]);
    h->kms[h->evkind[i]] += e;
    h->kn[h->evkind[i]] += 1;
  }
  CK(h, cudaGetLastError());
  // times at saves: t accumulated with t += dt (src/fixed_time_stepping.jl:44,49)
  double t = h->t;
  int64_t slot = 0;
  for (int64_t s = 0; s < nsteps; ++s) {
    t += h->d.dt;
    if (save_every > 0 && (s + 1) % save_every == 0) {
      if (ts_out) ts_out[slot] = t;
      ++slot;
    }
  }
  h->t = t;
  h->steps += nsteps;
  if (use_ring) {
    const int rc = ring.drain(nsaves);
    if (rc) return rc;
  } else if (nsaves > 0 && !out_is_dev) {
    for (int m = 0; m < h->M; ++m)
      CK(h, cudaMemcpy((char*)out + (size_t)m * comp_stride * plane_bytes, (char*)save_dev + (size_t)m * nsaves * plane_bytes,
                       (size_t)nsaves * plane_bytes, cudaMemcpyDeviceToHost));
  }
  return GPE_OK;
}

int gpe_run_ex(gpe_handle* h, int64_t nsteps, int64_t save_every, const void* xi_host, void* out_host,
               int64_t comp_stride, double* ts_out) {
  return run_common(h, nsteps, save_every, out_host, false, ts_out, xi_host, comp_stride);
}

int gpe_run(gpe_handle* h, int64_t nsteps, int64_t save_every, void* out_host, double* ts_out) {
  return run_common(h, nsteps, save_every, out_host, false, ts_out, nullptr);
}

int gpe_run_dev(gpe_handle* h, int64_t nsteps, int64_t save_every, void* out_dev, double* ts_out) {
  return run_common(h, nsteps, save_every, out_dev, true, ts_out, nullptr);
}

int gpe_run_replay(gpe_handle* h, int64_t nsteps, int64_t save_every, const void* xi_host, void* out_host,
                   double* ts_out) {
  if (!h) return GPE_ERR_INVALID;
  if (!xi_host && nsteps > 0) return fail(h, GPE_ERR_INVALID, "null xi");
  return run_common(h, nsteps, save_every, out_host, false, ts_out, xi_host);
}

int gpe_set_noise_offset(gpe_handle* h, int64_t traj0) {
  if (!h) return GPE_ERR_INVALID;
  // the counter holds the global trajectory index in one 32-bit word
  if (traj0 < 0 || traj0 + h->B > (int64_t(1) << 32))
    return fail(h, GPE_ERR_INVALID, "trajectory offset %lld: offset + batch must lie in [0, 2^32]", (long long)traj0);
  if (traj0 != h->traj0) ++h->gen;  // a kernel argument: captured graphs are recaptured
  h->traj0 = traj0;
  return GPE_OK;
}

int gpe_get_state(gpe_handle* h, gpe_state* st) {
  if (!h || !st) return h ? fail(h, GPE_ERR_INVALID, "null state") : GPE_ERR_INVALID;
  st->t = h->t;
  st->steps = h->steps;
  st->seed = h->seed;
  st->noise_mode = h->noise;
  st->reserved = 0;
  return GPE_OK;
}

int gpe_set_state(gpe_handle* h, const gpe_state* st) {
  if (!h || !st) return h ? fail(h, GPE_ERR_INVALID, "null state") : GPE_ERR_INVALID;
  if (!std::isfinite(st->t) || st->steps < 0) return fail(h, GPE_ERR_INVALID, "bad state");
  h->t = st->t;
  h->steps = st->steps;
  if (st->seed != h->seed) ++h->gen;  // the key is a kernel argument; step indices are not
  h->seed = st->seed;
  return GPE_OK;
}

int gpe_norm(gpe_handle* h, double* out) {
  if (!h) return GPE_ERR_INVALID;
  NvtxRange nv("gpe_norm");
  if (!out) return fail(h, GPE_ERR_INVALID, "null output");
  PassArgs a = base_args(h);
  CK(h, cudaMemsetAsync(h->red, 0, 4 * sizeof(double), h->stream));
  LK(h, gpe::launch_norm(h->prec, h->M, a, h->red, h->stream));
  double tmp[4];
  CK(h, cudaMemcpyAsync(tmp, h->red, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  for (int m = 0; m < h->M; ++m) out[m] = tmp[m] * h->dV;
  return GPE_OK;
}

// escr[m] <- unnormalised spatial FFT of u[m] (all trajectories), with the pass kernels.
static int transform_copy(gpe_handle* h) {
  const size_t plane_bytes = (size_t)h->P * h->B * h->csz;
  for (int m = 0; m < h->M; ++m) {
    if (!h->escr[m]) CK(h, cudaMalloc(&h->escr[m], plane_bytes));
    CK(h, cudaMemcpyAsync(h->escr[m], h->u[m], plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  PassArgs f = base_args(h);
  for (int m = 0; m < h->M; ++m) f.u[m] = h->escr[m];
  f.ktab = nullptr;
  f.noise = 0;
  f.hA = f.hB = -1;
  f.col_tma = 0;  // diagnostics: plain loads, no device wait
  PassArgs r = f;
  r.tw = h->tw[0];
  r.do_fft = 1;
  LK(h, gpe::launch_row(h->prec, h->M, h->logn[0], r, h->P / h->n[0] * h->B, h->stream));
  for (int ax = 1; ax < h->ndim; ++ax) {
    PassArgs c = f;
    c.tw = h->tw[ax];
    c.col_fwd = 1;
    c.ld = ax == 1 ? h->n[0] : h->n[0] * h->n[1];
    c.ostride = (h->ndim == 3) ? (ax == 1 ? h->n[0] * h->n[1] : h->n[0]) : 0;
    c.nouter = (h->ndim == 3) ? (ax == 1 ? h->n[2] : h->n[1]) : 1;
    LK(h, gpe::launch_col(h->prec, h->M, h->logn[ax], c, h->stream));
  }
  return GPE_OK;
}

int gpe_energy(gpe_handle* h, double* out) {
  if (!h) return GPE_ERR_INVALID;
  NvtxRange nv("gpe_energy");
  if (!out) return fail(h, GPE_ERR_INVALID, "null output");
  if (h->nl_matrix) return fail(h, GPE_ERR_UNSUPPORTED, "energy is defined for the diagonal nonlinearity families only");
  CK(h, cudaSetDevice(h->dev));
  if (h->ktab && h->Dsamples.empty())
    return fail(h, GPE_ERR_UNSUPPORTED, "energy needs the dispersion samples (gpe_set_dispersion), not a finished table");
  if (h->vtab && h->Vsamples.empty())
    return fail(h, GPE_ERR_UNSUPPORTED, "energy needs the potential samples (gpe_set_potential), not a finished table");
  if (!h->Dsamples.empty() && !h->dsamp) {
    CK(h, cudaMalloc((void**)&h->dsamp, h->Dsamples.size() * sizeof(double2)));
    CK(h, cudaMemcpy(h->dsamp, h->Dsamples.data(), h->Dsamples.size() * sizeof(double2), cudaMemcpyHostToDevice));
  }
  if (!h->Vsamples.empty() && !h->vsamp) {
    CK(h, cudaMalloc((void**)&h->vsamp, h->Vsamples.size() * sizeof(double2)));
    CK(h, cudaMemcpy(h->vsamp, h->Vsamples.data(), h->Vsamples.size() * sizeof(double2), cudaMemcpyHostToDevice));
  }
  // the kinetic term needs u~: transform a copy of the state with the pass kernels
  if (h->dsamp) {
    int rc = transform_copy(h);
    if (rc) return rc;
  }
  CK(h, cudaMemsetAsync(h->red, 0, 4 * sizeof(double), h->stream));
  PassArgs a = base_args(h);
  LK(h, gpe::launch_energy_sums(h->prec, h->M, h->escr, h->u, h->P, h->B, h->dsamp, h->dkind, h->vsamp, h->vskind, a,
                                h->red, h->stream));
  double tmp[4];
  CK(h, cudaMemcpyAsync(tmp, h->red, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  out[0] = tmp[0] * h->dV / (double)h->P;
  out[1] = tmp[1] * h->dV;
  out[2] = tmp[2] * h->dV;
  return GPE_OK;
}

int gpe_set_variant(gpe_handle* h, int variant) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  if (variant < -1 || variant > 2) return fail(h, GPE_ERR_INVALID, "variant %d: expected -1, 0, 1 or 2", variant);
  if (variant == 1 && !(h->prec == gpe::PREC_F32 && h->M == 1))
    return fail(h, GPE_ERR_UNSUPPORTED, "variant 1 exists for FP32 one-component fields only");
  if (variant != h->variant) {
    h->variant = variant;
    if (h->gexec) {  // a captured chunk holds the old kernels
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
  }
  return GPE_OK;
}

int gpe_set_graph(gpe_handle* h, int64_t steps_per_graph) {
  if (!h) return GPE_ERR_INVALID;
  ++h->gen;
  if (steps_per_graph < 0) return fail(h, GPE_ERR_INVALID, "steps_per_graph must be >= 0");
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  h->gsteps = steps_per_graph;
  return GPE_OK;
}

// Enqueue without waiting: no saves, no replay.  Host bookkeeping (t, steps) advances now.
int gpe_run_async(gpe_handle* h, int64_t nsteps) {
  if (!h) return GPE_ERR_INVALID;
  NvtxRange nv("gpe_run_async");
  CK(h, cudaSetDevice(h->dev));
  if (nsteps < 0) return fail(h, GPE_ERR_INVALID, "nsteps must be >= 0");
  if (h->noise == GPE_NOISE_REPLAY) return fail(h, GPE_ERR_INVALID, "replayed noise needs gpe_run_replay");
  for (int m = 0; m < h->M; ++m)
    if (h->pprof[m] && h->pcoef_n[m] > 1 && h->pcoef_n[m] < 2 * (h->steps + nsteps) + 1)
      return fail(h, GPE_ERR_INVALID, "pump %d has too few amplitudes for %lld more steps", m, (long long)nsteps);
  if (nsteps == 0) return GPE_OK;
  int64_t launches = 0;
  if (h->gsteps > 0 && nsteps % h->gsteps == 0) {
    int rc = ensure_graph(h);
    if (rc) return rc;
    rc = replay_graph(h, nsteps, &launches);
    if (rc) return rc;
  } else {
    int rc = enqueue_steps(h, nsteps, 0, nullptr, 0, nullptr, &launches);
    if (rc) return rc;
  }
  for (int64_t s = 0; s < nsteps; ++s) h->t += h->d.dt;
  h->steps += nsteps;
  h->last_launches = launches;
  return GPE_OK;
}

int gpe_wait(gpe_handle* h) {
  if (!h) return GPE_ERR_INVALID;
  CK(h, cudaSetDevice(h->dev));
  CK(h, cudaStreamSynchronize(h->stream));
  CK(h, cudaGetLastError());
  return take_status(h);
}

// the bound of every device wait in the library (gpe::kWaitLimitNs in tma.cuh)
static constexpr int64_t kProbeWaitLimitNs = 1000000000;

int gpe_selftest_wait(int device, int arrive, int64_t limit_ns) {
  // the probe's wait must end on its own: limits above the library's own bound (1 s)
  // are refused, so no caller can make it spin for longer
  if (limit_ns < 0 || limit_ns > kProbeWaitLimitNs) return GPE_ERR_INVALID;
  if (cudaSetDevice(device < 0 ? 0 : device) != cudaSuccess) return GPE_ERR_CUDA;
  int32_t *hs = nullptr, *ds = nullptr;
  if (cudaHostAlloc((void**)&hs, sizeof(int32_t), cudaHostAllocMapped) != cudaSuccess) return GPE_ERR_NOMEM;
  int rc = GPE_OK;
  *hs = 0;
  if (cudaHostGetDevicePointer((void**)&ds, hs, 0) != cudaSuccess ||
      gpe::launch_wait_probe(arrive ? 1 : 0, (uint64_t)limit_ns, ds, 0) != 0 || cudaDeviceSynchronize() != cudaSuccess)
    rc = GPE_ERR_CUDA;
  else if (*(volatile int32_t*)hs)
    rc = GPE_ERR_TIMEOUT;
  cudaFreeHost(hs);
  return rc;
}

int gpe_set_timing(gpe_handle* h, int on) {
  if (!h) return GPE_ERR_INVALID;
  h->timing = on ? 1 : 0;
  return GPE_OK;
}

int gpe_kernel_times(const gpe_handle* h, double* ms, int64_t* n) {
  if (!h || !ms || !n) return GPE_ERR_INVALID;
  for (int k = 0; k < 3; ++k) { ms[k] = h->kms[k]; n[k] = h->kn[k]; }
  return GPE_OK;
}

int gpe_spectral_moments(gpe_handle* h, int comp, double* mean_out, double* second_out) {
  NvtxRange nv("gpe_spectral_moments");
  int rc = check_comp(h, comp);
  if (rc) return rc;
  if (!mean_out) return fail(h, GPE_ERR_INVALID, "null output");
  if (second_out && h->P > 8192) return fail(h, GPE_ERR_INVALID, "the second-moment matrix needs P <= 8192 points");
  rc = transform_copy(h);
  if (rc) return rc;
  double *nb = nullptr, *mean = nullptr, *second = nullptr;
  const size_t P = (size_t)h->P;
  if (cudaMalloc((void**)&nb, P * h->B * sizeof(double)) != cudaSuccess ||
      cudaMalloc((void**)&mean, P * sizeof(double)) != cudaSuccess ||
      (second_out && cudaMalloc((void**)&second, P * P * sizeof(double)) != cudaSuccess)) {
    cudaFree(nb);
    cudaFree(mean);
    cudaFree(second);
    return fail(h, GPE_ERR_NOMEM, "device allocation for spectral moments failed");
  }
  int lrc = gpe::launch_spectral_moments(h->prec, h->escr[comp], h->P, h->B, nb, mean, second, h->stream);
  cudaError_t e = lrc ? (cudaError_t)lrc : cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaMemcpy(mean_out, mean, P * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && second_out) e = cudaMemcpy(second_out, second, P * P * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(nb);
  cudaFree(mean);
  cudaFree(second);
  if (e != cudaSuccess) return fail(h, GPE_ERR_CUDA, "spectral moments failed: %s", cudaGetErrorString(e));
  return GPE_OK;
}

double gpe_last_run_ms(const gpe_handle* h) { return h ? h->last_ms : 0.0; }
int64_t gpe_last_run_launches(const gpe_handle* h) { return h ? h->last_launches : 0; }

// ---- ensembles: several handles (grid-size groups) advanced by one CUDA graph ----
}  // extern "C"

struct gpe_ensemble {
  std::vector<gpe_handle*> hs;
  int64_t gsteps = 0;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> joins;
  int64_t launches_per_graph = 0;
  double last_ms = 0.0;
  int64_t last_launches = 0;
  std::vector<int64_t> gens;  // the handles' setter generations the graph was captured in
  std::string err;
};

static int efail(gpe_ensemble* e, int code, const char* msg) {
  if (e) e->err = msg;
  else g_create_error = msg;
  return code;
}

extern "C" {

int gpe_ensemble_create(gpe_handle* const* handles, int n, gpe_ensemble** out) {
  if (!handles || n < 1 || !out) return efail(nullptr, GPE_ERR_INVALID, "ensemble needs at least one handle");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!handles[i]) return efail(nullptr, GPE_ERR_INVALID, "null handle in ensemble");
    if (handles[i]->dev != handles[0]->dev) return efail(nullptr, GPE_ERR_INVALID, "ensemble handles must share a device");
    if (handles[i]->noise == GPE_NOISE_REPLAY) return efail(nullptr, GPE_ERR_INVALID, "ensembles do not replay noise");
  }
  gpe_ensemble* e = new gpe_ensemble();
  e->hs.assign(handles, handles + n);
  cudaSetDevice(handles[0]->dev);
  cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  cudaEventCreate(&e->ev0);
  cudaEventCreate(&e->ev1);
  e->joins.resize((size_t)n);
  for (auto& j : e->joins) cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
  *out = e;
  return GPE_OK;
}

int gpe_ensemble_destroy(gpe_ensemble* e) {
  if (!e) return GPE_OK;
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  cudaEventDestroy(e->fork);
  cudaEventDestroy(e->ev0);
  cudaEventDestroy(e->ev1);
  for (auto j : e->joins) cudaEventDestroy(j);
  delete e;
  return GPE_OK;
}

const char* gpe_ensemble_last_error(const gpe_ensemble* e) { return e ? e->err.c_str() : g_create_error.c_str(); }

// One graph: fork from the first handle's stream to every handle's stream, each handle
// enqueues steps_per_graph steps (its resident launch or its pass chain) and advances its
// own step counter, then everything joins back.  The graph is replayed nsteps /
// steps_per_graph times.
int gpe_ensemble_run(gpe_ensemble* e, int64_t nsteps, int64_t steps_per_graph) {
  if (!e) return GPE_ERR_INVALID;
  NvtxRange nv("gpe_ensemble_run");
  if (nsteps < 0 || steps_per_graph < 1 || nsteps % steps_per_graph)
    return efail(e, GPE_ERR_INVALID, "nsteps must be a non-negative multiple of steps_per_graph >= 1");
  gpe_handle* h0 = e->hs[0];
  cudaSetDevice(h0->dev);
  for (gpe_handle* h : e->hs)
    for (int m = 0; m < h->M; ++m)
      if (h->pprof[m] && h->pcoef_n[m] > 1 && h->pcoef_n[m] < 2 * (h->steps + nsteps) + 1)
        return efail(e, GPE_ERR_INVALID, "a pump has too few amplitudes for this run");
  bool stale = e->gexec && e->gsteps != steps_per_graph;
  for (size_t i = 0; e->gexec && i < e->hs.size(); ++i) stale = stale || e->gens[i] != e->hs[i]->gen;
  if (stale) {
    cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
  }
  if (!e->gexec) {
    for (gpe_handle* h : e->hs) {
      if (!h->kdev && cudaMalloc((void**)&h->kdev, sizeof(int64_t)) != cudaSuccess)
        return efail(e, GPE_ERR_NOMEM, "cudaMalloc of a step counter failed");
      h->gsteps = steps_per_graph;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(h0->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return efail(e, GPE_ERR_CUDA, "cudaStreamBeginCapture failed");
    cudaEventRecord(e->fork, h0->stream);
    int rc = GPE_OK;
    int64_t total = 0;
    for (size_t i = 0; i < e->hs.size() && rc == GPE_OK; ++i) {
      gpe_handle* h = e->hs[i];
      if (i > 0) cudaStreamWaitEvent(h->stream, e->fork, 0);
      int64_t nl = 0;
      rc = capture_chunk(h, h->stream, &nl);
      total += nl;
      if (i > 0) {
        cudaEventRecord(e->joins[i], h->stream);
        cudaStreamWaitEvent(h0->stream, e->joins[i], 0);
      }
    }
    const cudaError_t ec = cudaStreamEndCapture(h0->stream, &g);
    if (rc != GPE_OK || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      for (gpe_handle* h : e->hs) h->gsteps = 0;
      return efail(e, rc ? rc : GPE_ERR_CUDA, rc ? "capture of a group failed" : cudaGetErrorString(ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&e->gexec, g, 0);
    cudaGraphDestroy(g);
    for (gpe_handle* h : e->hs) h->gsteps = 0;
    if (ei != cudaSuccess) return efail(e, GPE_ERR_CUDA, cudaGetErrorString(ei));
    e->gsteps = steps_per_graph;
    e->launches_per_graph = total;
    e->gens.clear();
    for (gpe_handle* h : e->hs) e->gens.push_back(h->gen);
  }
  for (gpe_handle* h : e->hs) {
    h->kval = h->steps;
    if (cudaMemcpyAsync(h->kdev, &h->kval, sizeof(int64_t), cudaMemcpyHostToDevice, h0->stream) != cudaSuccess)
      return efail(e, GPE_ERR_CUDA, "step counter upload failed");
  }
  cudaEventRecord(e->ev0, h0->stream);
  for (int64_t r = 0; r < nsteps / steps_per_graph; ++r)
    if (cudaGraphLaunch(e->gexec, h0->stream) != cudaSuccess) return efail(e, GPE_ERR_CUDA, "cudaGraphLaunch failed");
  cudaEventRecord(e->ev1, h0->stream);
  const cudaError_t es = cudaEventSynchronize(e->ev1);
  if (es != cudaSuccess) return efail(e, GPE_ERR_CUDA, cudaGetErrorString(es));
  for (gpe_handle* h : e->hs)
    if (take_status(h)) return efail(e, GPE_ERR_TIMEOUT, "a device wait exceeded its limit in a group");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e->ev0, e->ev1);
  e->last_ms = ms;
  e->last_launches = e->launches_per_graph * (nsteps / steps_per_graph);
  for (gpe_handle* h : e->hs) {
    for (int64_t s = 0; s < nsteps; ++s) h->t += h->d.dt;
    h->steps += nsteps;
  }
  return GPE_OK;
}

double gpe_ensemble_last_run_ms(const gpe_ensemble* e) { return e ? e->last_ms : 0.0; }
int64_t gpe_ensemble_last_run_launches(const gpe_ensemble* e) { return e ? e->last_launches : 0; }

}  // extern "C"
