/*
 * gpe.h -- C ABI of libgpe, the GB300 (sm_103a) StrangSplitting backend for
 * GeneralizedGrossPitaevskii.jl.
 *
 * The library advances
 *     i du = [D(-i grad) u + V(r) u + G(u) u + i F(r,t)] dt + eta dW
 * on a periodic uniform grid with the reference's Strang splitting
 * (src/strang_splitting.jl:86-90, src/kernels.jl:37-54).  It is the compute
 * backend for the reference's
 *     solve(prob, StrangSplitting(), tspan; dt, nsaves, save_start)
 * (src/fixed_time_stepping.jl:56-81): the host side (a Julia shim, or the Python
 * mirror shipped with this library) resolves dt (src/fixed_time_stepping.jl:14-24),
 * samples the user closures on the grids and passes the results here as plain
 * FP64 arrays.
 *
 * Conventions
 *  - Axis 0 is x and is the fastest varying (Julia column-major order): a field is
 *    stored as C array [batch][z][y][x] of interleaved (re, im) complex numbers.
 *    Components are separate arrays (the reference's tuple of arrays).
 *  - Field precision is GPE_C128 (FP64) or GPE_C64 (FP32).  Every table, time and
 *    coefficient crosses this ABI in FP64.
 *  - Every call returns 0 on success or a negative GPE_ERR_* code; gpe_last_error()
 *    gives a readable message.  No C++ exception crosses the ABI.
 *  - One handle owns one CUDA stream and its device buffers; a handle is not
 *    thread safe, distinct handles may be used concurrently.  Calls are synchronous
 *    unless stated otherwise.
 */
#ifndef GPE_H
#define GPE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPE_ABI_VERSION 1

/* status codes */
#define GPE_OK 0
#define GPE_ERR_INVALID (-1)     /* bad argument, shape or state */
#define GPE_ERR_UNSUPPORTED (-2) /* closure family / size this backend does not do */
#define GPE_ERR_CUDA (-3)        /* a CUDA runtime call failed */
#define GPE_ERR_NONFINITE (-4)   /* NaN/Inf found in an input or the state */
#define GPE_ERR_TIMEOUT (-5)     /* a bounded device wait expired */
#define GPE_ERR_NOMEM (-6)       /* device allocation failed */

/* field precision */
#define GPE_C128 0 /* ComplexF64 fields, FP64 arithmetic (the reference's Float64; see the flags) */
#define GPE_C64 1  /* ComplexF32 fields, FP32 arithmetic; FP64 tables, times and reductions */

/* gpe_desc.flags */
/* GPE_C128 arithmetic.  By default the pointwise steps (nonlinearity, potential, pump,
 * noise) run in FP64 and the line transforms in block floating point on the integer pipes
 * (GPE_FLAG_FFT_BFP): each line held as 64-bit integers under one exponent, rescaled after
 * every radix-8 stage so that its largest component stays below 2^58, twiddles in Q62; a
 * 2D column pass also applies the k-space table between its transforms from a Q62 copy
 * (its FP64 table scaled by a power of two).  Sums are exact and every product rounds to
 * within 2^-56 to 2^-58 of the line's largest component; measured against an FP64 oracle
 * on a 2048^2 Kerr run of 1000 steps the results land 3-11x closer than with FP64
 * floating-point transforms, and GB300 runs the polariton step 2.7x faster (a Q62 complex
 * product runs 2.7x, a 64-bit add 16x faster than the FP64 operations).
 * GPE_FLAG_FP64_NATIVE runs the line transforms in FP64 floating point too.
 * GPE_FLAG_FP64_DW: opt-in fast mode, all passes on the FP32 pipes in double-word
 * arithmetic (pairs of floats, 48-bit significands, unit roundoff 2^-48, narrower than
 * FP64's 2^-53; GB300 issues FP32 FMAs 62x faster than FP64 ones).
 * The three exclude each other and apply to GPE_C128 only; the state, the saves and every
 * result cross this ABI as FP64 in all of them. */
#define GPE_FLAG_FP64_NATIVE 1
#define GPE_FLAG_FP64_DW 16
#define GPE_FLAG_FFT_BFP 32
/* Square 2D fields small enough for one CTA's shared memory (FP32 up to 128x128 with one
 * component, 16-byte types up to 64x64) run every step of a gpe_run call in one resident
 * launch, one CTA per trajectory.  This flag forces the two-pass HBM path instead. */
#define GPE_FLAG_NO_RESIDENT 2
/* 2D column passes can stage each tile of columns into shared memory with the tensor
 * memory accelerator (cp.async.bulk.tensor), the next tile landing while the current one
 * is transformed.  By default they do so for one-component lines of at most 512 points
 * (measured faster there; two-component tiles are faster with plain per-thread loads).
 * GPE_FLAG_NO_TMA keeps plain loads everywhere; GPE_FLAG_TMA stages wherever the shape
 * and shared memory allow.  A tile that does not arrive within 1 s makes the run return
 * GPE_ERR_TIMEOUT. */
#define GPE_FLAG_NO_TMA 4
#define GPE_FLAG_TMA 8

/* table kinds: what the user closure returned per grid point */
#define GPE_TABLE_NONE 0
#define GPE_TABLE_SCALAR 1 /* one complex number per point, same for every component */
#define GPE_TABLE_DIAG 2   /* M complex numbers per point (SVector) */
#define GPE_TABLE_MATRIX 3 /* M x M complex matrix per point (SMatrix), row-major a*M+b */

/* noise modes */
#define GPE_NOISE_OFF 0
#define GPE_NOISE_PHILOX 1 /* in-kernel Philox4x32-10 + Box-Muller, E|xi|^2 = 1 */
#define GPE_NOISE_REPLAY 2 /* xi supplied by the host for every half step */

typedef struct gpe_handle gpe_handle;

typedef struct gpe_desc {
  int32_t abi_version; /* GPE_ABI_VERSION */
  int32_t ndim;        /* spatial dimensions: 1, 2 or 3 */
  int64_t n[3];        /* grid points per axis, n[0] = x; unused axes = 1 */
  double lengths[3];   /* domain size per axis (x in [0, L)) */
  int64_t batch;       /* trailing (trajectory) dims flattened, >= 1 */
  int32_t ncomp;       /* components M: 1 or 2 */
  int32_t dtype;       /* GPE_C128 or GPE_C64 */
  double dt;           /* the resolved step (src/fixed_time_stepping.jl:19-21) */
  double t0;           /* tspan[1] */
  int32_t device;      /* CUDA device ordinal; -1 = the calling thread's current device */
  int32_t flags;       /* GPE_FLAG_* bits, 0 by default */
} gpe_desc;

/* Solver state apart from the fields: enough to resume bit-identically. */
typedef struct gpe_state {
  double t;          /* time accumulated with t += dt (src/fixed_time_stepping.jl:44) */
  int64_t steps;     /* full steps taken since t0 */
  uint64_t seed;     /* Philox key */
  int32_t noise_mode;
  int32_t reserved;
} gpe_state;

/* ---- lifetime ------------------------------------------------------------ */
/* Replaces init(prob, StrangSplitting(), tspan; dt, ...) (src/strang_splitting.jl:32-67):
 * allocates the device state for the grid, batch and precision in *desc. */
int gpe_create(const gpe_desc* desc, gpe_handle** out);
int gpe_destroy(gpe_handle* h);
/* Message for the last failed call on h (or the last gpe_create failure if h is NULL). */
const char* gpe_last_error(const gpe_handle* h);
/* Version / build information string. */
const char* gpe_version(void);

/* ---- fields -------------------------------------------------------------- */
/* Upload component comp (u0[comp], src/strang_splitting.jl:48) from host memory:
 * batch*P complex numbers of the handle's precision, layout [batch][z][y][x]. */
int gpe_set_field(gpe_handle* h, int comp, const void* host);
int gpe_get_field(gpe_handle* h, int comp, void* host);
/* Same with device pointers the caller owns (e.g. a torch tensor's data_ptr()).  The
 * copy waits for the work already queued on the device's legacy default stream (where
 * PyTorch writes and reads by default); a caller that fills or reads the buffer on
 * another stream synchronises that stream first. */
int gpe_set_field_dev(gpe_handle* h, int comp, const void* dev);
int gpe_get_field_dev(gpe_handle* h, int comp, void* dev);

/* ---- linear operators ---------------------------------------------------- */
/* Dispersion samples D(k) on reciprocal_grid (src/problem.jl:135-139), FP64 complex
 * interleaved, spatial points only: kind SCALAR -> P, DIAG -> M*P ([m][p]),
 * MATRIX -> M*M*P ([a*M+b][p]).  The library forms exp(-i dt D) on the host in FP64
 * (src/misc.jl:12-20; closed-form 2x2 exponential for MATRIX). */
int gpe_set_dispersion(gpe_handle* h, const double* D, int kind);
/* The finished table exp(-i dt D(k)) instead of D (same layouts), e.g. built by the
 * caller with the reference's own get_exponential. */
int gpe_set_ktable(gpe_handle* h, const double* table, int kind);
/* Potential samples V(r) on direct_grid; the library forms exp(-i dt/2 V)
 * (src/strang_splitting.jl:54).  MATRIX potentials need a MATRIX nonlinearity or none. */
int gpe_set_potential(gpe_handle* h, const double* V, int kind);
int gpe_set_vtable(gpe_handle* h, const double* table, int kind);

/* ---- local terms --------------------------------------------------------- */
/* Diagonal nonlinearity family G_j(u) = sum_l g[j*M+l] |u_l|^2 + c[j] with complex
 * (interleaved) g (M*M) and c (M); c may be NULL.  Covers every nonlinearity of the
 * reference's tests and examples (e.g. test/kerr_propagation.jl:24,
 * examples/exciton_polariton.jl:50). */
int gpe_set_nonlinearity(gpe_handle* h, const double* g, const double* c);
/* Matrix nonlinearity family for two components (the SMatrix form of
 * src/kernels.jl:23-25,44): G_ab(u) = sum_l g[(a*2+b)*2+l] |u_l|^2 + c[a*2+b] (complex,
 * interleaved), applied as the per-point 2x2 exponential exp(-i dt/2 G) (times a scalar or
 * matrix potential table).  Replaces any diagonal nonlinearity; c may be NULL. */
int gpe_set_matrix_nonlinearity(gpe_handle* h, const double* g, const double* c);
/* Separable pump F_comp(r, t) = a(t) * p(r).  profile: P real FP64 values (or P
 * interleaved complex when profile_complex != 0); amp: n_amp complex FP64 values of
 * a(t) at the reference's pump sampling times: amp[0] = a(t0), amp[2k+1] =
 * a(t_k + dt/2), amp[2k+2] = a(t_k + dt), t_k = end time of step k accumulated with
 * t += dt (src/strang_splitting.jl:56-58,78-84, src/misc.jl:39-42).  n_amp == 1 means a
 * constant amplitude.  profile == NULL removes the pump of that component. */
int gpe_set_pump(gpe_handle* h, int comp, const double* profile, int profile_complex,
                 const double* amp, int64_t n_amp);
/* Position noise -i sqrt(dt/2) eta_m xi_m added after every real-space half step
 * (src/kernels.jl:42,49).  eta: M complex amplitudes; eta_profile: NULL or M*P real
 * factors ([m][p]).  mode GPE_NOISE_PHILOX draws xi in-kernel from (seed, half step,
 * component, point, trajectory); GPE_NOISE_REPLAY takes xi from gpe_run_replay. */
int gpe_set_noise(gpe_handle* h, int mode, uint64_t seed, const double* eta,
                  const double* eta_profile);
/* Global index of the handle's first trajectory in the Philox counter (default 0): a
 * handle with batch B' and offset b0 draws the noise of trajectories b0 .. b0 + B' - 1 of
 * an ensemble with the same seed, so an ensemble sharded over GPUs (one handle per rank,
 * each with its own contiguous slice) reproduces the single-handle run bit for bit.
 * b0 + batch must not exceed 2^32.  The reference keeps its ensemble on one device and
 * has no counterpart (its batching is the trailing dims, src/kernels.jl:27). */
int gpe_set_noise_offset(gpe_handle* h, int64_t traj0);

/* ---- stepping ------------------------------------------------------------ */
/* Advance nsteps full Strang steps (src/fixed_time_stepping.jl:38-50).  After every
 * save_every steps (0 = never) the state is stored into out_host as save slot s:
 * component m, slot s is at out_host + (m*nsaves + s) * batch*P complex numbers, with
 * nsaves = nsteps / save_every; ts_out[s] (may be NULL) receives the accumulated time.
 * out_host may be NULL when save_every == 0. */
int gpe_run(gpe_handle* h, int64_t nsteps, int64_t save_every, void* out_host,
            double* ts_out);
/* As gpe_run (xi_host NULL) or gpe_run_replay (xi_host set), with component m, slot s of
 * the saves at out_host + (m*comp_stride + s) * batch*P complex numbers, comp_stride >=
 * nsaves: a caller can leave room for the initial state beside the saves (solve's result
 * holds u0 in slot 0) and receive the run in place.  No counterpart in the reference. */
int gpe_run_ex(gpe_handle* h, int64_t nsteps, int64_t save_every, const void* xi_host, void* out_host,
               int64_t comp_stride, double* ts_out);
/* As gpe_run with out_dev a device buffer of the same layout the caller owns. */
int gpe_run_dev(gpe_handle* h, int64_t nsteps, int64_t save_every, void* out_dev,
                double* ts_out);
/* As gpe_run in GPE_NOISE_REPLAY mode: xi_host holds 2*nsteps half steps of
 * M*batch*P complex numbers (handle precision), layout [half][m][batch][p]. */
int gpe_run_replay(gpe_handle* h, int64_t nsteps, int64_t save_every, const void* xi_host,
                   void* out_host, double* ts_out);

/* ---- checkpoint / diagnostics ------------------------------------------- */
int gpe_get_state(gpe_handle* h, gpe_state* st);
int gpe_set_state(gpe_handle* h, const gpe_state* st);
/* out[m] = sum over batch and grid of |u_m|^2 dV, accumulated in FP64 on the device. */
int gpe_norm(gpe_handle* h, double* out);
/* out[0] = kinetic Re sum_k u~^H D(k) u~ dV/P (u~ the unnormalised FFT; needs the samples
 *          of gpe_set_dispersion),
 * out[1] = interaction sum_r sum_j [(1/2) sum_l Re(g_jl) |u_l|^2 + Re(c_j)] |u_j|^2 dV,
 * out[2] = potential Re sum_r u^H V(r) u dV (needs gpe_set_potential samples).
 * Summed over the batch, accumulated in FP64 on the device. */
int gpe_energy(gpe_handle* h, double* out);

/* Momentum-space statistics over the trajectories (the post-processing of the reference's
 * truncated-Wigner example, examples/truncated_wigner.jl:110-165): with n_b(k) =
 * |FFT(u_comp)_b(k)|^2 / P^2 for trajectory b (FFT unnormalised, k in FFT order),
 * mean_out[k] = (1/B) sum_b n_b(k) (P values) and, if second_out is not NULL,
 * second_out[k*P + k'] = (1/B) sum_b n_b(k) n_b(k') (P*P values, P <= 8192). */
int gpe_spectral_moments(gpe_handle* h, int comp, double* mean_out, double* second_out);

/* ---- graphs, asynchronous runs, ensembles -------------------------------- */
/* Graph mode: runs of a multiple of steps_per_graph steps (no saves, no replay) replay a
 * CUDA graph captured once from steps_per_graph steps; the kernels read the step index
 * from a device counter, so one graph serves every position.  0 turns it off. */
int gpe_set_graph(gpe_handle* h, int64_t steps_per_graph);
/* Line tiling of the two-pass passes: 0, the default tiling; 1, the alternative tiling of
 * FP32 one-component fields (8 points a thread along x, 16 along y/z instead of 16 and 8);
 * 2, the fine tiling (4 points a thread in both passes: twice the threads, for fields too
 * small to fill the GPU); -1 (the initial setting), 2 for two-component fields of at most
 * 2^18 points over all trajectories and 0 otherwise.  Tilings agree to rounding, not bit for bit.  Set it
 * before capturing graphs or ensembles that include the handle.  No counterpart in the
 * reference (the choice an autotuner makes per grid size). */
int gpe_set_variant(gpe_handle* h, int variant);
/* Enqueue nsteps steps on the handle's stream and return (no saves, no replayed noise);
 * gpe_wait blocks until they are done. */
int gpe_run_async(gpe_handle* h, int64_t nsteps);
int gpe_wait(gpe_handle* h);

/* Probe of the bounded device wait the TMA column pass relies on: one CTA waits on an
 * mbarrier with limit_ns as its limit.  arrive = 0: nothing completes the barrier, the
 * wait runs out and the call returns GPE_ERR_TIMEOUT with the context still usable;
 * arrive = 1: the barrier completes and the call returns GPE_OK.  limit_ns must lie in
 * [0, 1e9] (the library's own wait bound, 1 s); anything else is GPE_ERR_INVALID. */
int gpe_selftest_wait(int device, int arrive, int64_t limit_ns);
/* Several handles (e.g. trajectory groups on grids of different sizes) advanced together
 * by ONE captured CUDA graph: each handle's chunk of steps_per_graph steps runs on its own
 * stream inside the graph (small square grids as one resident launch, larger ones as
 * their pass chain), forked from and joined to the first handle's stream.  The handles
 * stay usable on their own; gpe_ensemble_run waits for completion.  The extension of the
 * reference's batching over trailing dims (docs/src/stochastic_simulations.md:36-48) to
 * grids of different sizes. */
typedef struct gpe_ensemble gpe_ensemble;
int gpe_ensemble_create(gpe_handle* const* handles, int n, gpe_ensemble** out);
int gpe_ensemble_run(gpe_ensemble* e, int64_t nsteps, int64_t steps_per_graph);
int gpe_ensemble_destroy(gpe_ensemble* e);
const char* gpe_ensemble_last_error(const gpe_ensemble* e);
double gpe_ensemble_last_run_ms(const gpe_ensemble* e);
int64_t gpe_ensemble_last_run_launches(const gpe_ensemble* e);

/* Per-launch timing for benchmarks: when on, gpe_run* brackets every kernel launch
 * with CUDA events on the handle's stream.  gpe_kernel_times then gives, for the last
 * run, ms[k] = summed device time and n[k] = launches of kernel kind k:
 * 0 = row pass (x lines), 1 = column pass (y lines), 2 = resident (1D lines, 2D planes,
 * pointwise-only problems). */
int gpe_set_timing(gpe_handle* h, int on);
int gpe_kernel_times(const gpe_handle* h, double* ms, int64_t* n);

/* Wall time of the device work of the last gpe_run* call, in milliseconds. */
double gpe_last_run_ms(const gpe_handle* h);
/* Number of kernels launched by the last gpe_run* call. */
int64_t gpe_last_run_launches(const gpe_handle* h);

/* ---- allocation-free entry point ---------------------------------------- */
/* No counterpart in the reference: an addition for callers that cannot allocate device
 * memory (their device memory belongs to another allocator, such as a framework's
 * caching pool or a budget fixed at start-up, or they run where cudaMalloc's implicit
 * device synchronisation is not acceptable).
 *
 * out_host[m*ntraj + b] = dV * sum over the npoints values of trajectory b of
 * |fields_dev[m]|^2, for ncomp (1 or 2) caller-owned device arrays of ntraj*npoints
 * complex numbers (GPE_C128: double2, GPE_C64: float2), reduced in FP64.  The only
 * scratch is a static device array of GPE_NOALLOC_MAX_NORMS doubles that the library
 * holds on every GPU that loads it; ncomp * ntraj above that limit (or ntraj above
 * 65535) is rejected with GPE_ERR_INVALID.  Nothing is allocated: no cudaMalloc, no
 * cudaFree, no allocating library routine.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress, with that device current), so make it
 * before any stream capture.  That address is kept for the life of the process: do not
 * call this entry point after cudaDeviceReset (or anything else that destroys and
 * recreates the device's primary context), whose new context places the array elsewhere.  The call is synchronous on the legacy default stream.
 * Every call shares the one array and overwrites the slots it uses, so calls that
 * overlap on the GPU (from several host threads or streams) race.  Errors are
 * described by gpe_noalloc_last_error() (per host thread). */
#define GPE_NOALLOC_MAX_NORMS 8192
int gpe_norms_noalloc(const void* const* fields_dev, int ncomp, int64_t npoints, int64_t ntraj,
                      int dtype, double dV, double* out_host);
const char* gpe_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* GPE_H */
