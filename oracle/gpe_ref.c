/*
 * gpe_ref.c -- CPU restatement in C (OpenMP) of the StrangSplitting stepper of
 * GeneralizedGrossPitaevskii.jl.
 *
 * TEST INFRASTRUCTURE ONLY.  Like oracle/gpe_oracle.py, this is an oracle the GPU path
 * is compared against and a CPU baseline it is timed beside; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load it.  The product never calls it.
 *
 * It restates (paths relative to the reference project):
 *   step order, pump rotation .... src/strang_splitting.jl:69-90, src/misc.jl:39-42
 *   per-point update ............. src/kernels.jl:37-54
 *   FFTs (unnormalised forward,
 *   1/P-normalised inverse) ...... src/misc.jl:53-64
 * for the coefficient families the GPU backend takes: k-space table exp(-i dt D)
 * (scalar, diagonal or 2x2 matrix per point) and real-space table exp(-i dt/2 V)
 * (scalar or diagonal), both built in FP64 by the caller (src/misc.jl:12-20); the
 * nonlinearity G_j = sum_l g_jl |u_l|^2 + c_j; separable pumps a_j(t) p_j(r) with a_j
 * sampled at the reference's times (t0, then t_k + dt/2 and t_k + dt for step k with end
 * time t_k); position noise with constant amplitudes drawn by Philox4x32-10 exactly as
 * the GPU path draws it.  1D and 2D grids, one or two components, any batch.
 *
 * Arithmetic.  fp32 = 0: everything in FP64 (the reference's ComplexF64 path).
 * fp32 = 1: the reference's ComplexF32 path as Julia evaluates it -- the fields are
 * stored in single precision and transformed by single-precision FFTs (twiddles rounded
 * to float), while every product with an FP64 table, G or pump promotes to FP64 and is
 * rounded back to single precision when stored (src/kernels.jl:44-53, src/misc.jl:16).
 *
 * The FFT is an iterative radix-2 decimation-in-time transform with a twiddle table
 * exp(-2 pi i k / N) evaluated in FP64 (its error grows like log2 N times the unit
 * roundoff, the same order as FFTW's).  2D transforms do the x lines, then the y lines in
 * chunks of adjacent columns transformed in place.  Build (no -ffast-math; no
 * contraction, so x86 and Arm give the same bits):
 *     gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared gpe_ref.c -o libgpe_ref.so -lm
 */
#define _GNU_SOURCE /* sincos */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct oref_desc {
  int32_t ndim;          /* 1 or 2 */
  int64_t n[2];          /* points per axis, n[0] = x (fastest); powers of two */
  int32_t M;             /* components: 1 or 2 */
  int64_t B;             /* trajectories */
  int32_t fp32;          /* 0: FP64 arithmetic; 1: the reference's ComplexF32 arithmetic */
  int32_t threads;       /* OpenMP threads, 0 = the runtime's default */
  const double* ktab;    /* exp(-i dt D): [entry][p] interleaved complex, or NULL */
  int32_t kkind;         /* 1 scalar, 2 diagonal (M entries), 3 matrix (M*M entries, a*M+b) */
  const double* vtab;    /* exp(-i dt/2 V): [entry][p], or NULL */
  int32_t vkind;         /* 1 scalar, 2 diagonal */
  const double* g;       /* M*M complex, G_j = sum_l g[j*M+l] |u_l|^2 + c[j]; NULL = no G */
  const double* c;       /* M complex or NULL */
  const double* pprof[2];/* pump profile of component j: P complex, or NULL */
  const double* pamp[2]; /* a_j at the sampling times: namp complex values */
  int64_t namp;
  double dt;
  /* position noise -i sqrt(dt/2) eta_j xi (src/kernels.jl:42,49) with xi drawn by
     Philox4x32-10 from (point, traj0 + trajectory, half step) as the GPU path draws it */
  int32_t noise;         /* 0 off, 1 Philox */
  int32_t draw32;        /* 1: the FP32 draw (top 24 bits of each word), evaluated in FP64 */
  uint64_t seed;
  int64_t traj0;
  const double* eta;     /* M complex noise amplitudes */
} oref_desc;

typedef struct { double re, im; } cdbl;
typedef struct { float re, im; } cflt;

static inline cdbl cd(double r, double i) { cdbl z = {r, i}; return z; }
static inline cdbl cdmul(cdbl a, cdbl b) { return cd(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cdbl cdadd(cdbl a, cdbl b) { return cd(a.re + b.re, a.im + b.im); }
static inline cdbl cdscale(cdbl a, double s) { return cd(a.re * s, a.im * s); }

static int ilog2_64(int64_t n) {
  int l = 0;
  while ((1LL << l) < n) ++l;
  return l;
}

/* ------------------------------------------------------------------ line FFTs
 * Radix-2 DIT on a contiguous line of N points: bit-reversal permutation, then log2 N
 * layers of butterflies x[j] +- w^k x[j + h].  dir = -1 forward (w = exp(-2 pi i/N)),
 * +1 inverse (conjugate twiddles), both unnormalised. */
#define DEFINE_FFT(NAME, C, R)                                                              \
  static void NAME(C* x, int64_t N, const C* tw, const int32_t* rev, int dir) {             \
    for (int64_t i = 0; i < N; ++i) {                                                       \
      const int64_t r = rev[i];                                                             \
      if (r > i) {                                                                          \
        C t = x[i];                                                                         \
        x[i] = x[r];                                                                        \
        x[r] = t;                                                                           \
      }                                                                                     \
    }                                                                                       \
    const R sg = dir < 0 ? (R)1 : (R)-1;                                                    \
    for (int64_t h = 1; h < N; h <<= 1) {                                                   \
      const C* wl = tw + (h - 1); /* w_{2h}^j, j < h, stored contiguously per layer */      \
      for (int64_t s = 0; s < N; s += 2 * h) {                                              \
        C* xa = x + s;                                                                      \
        C* xb = x + s + h;                                                                  \
        for (int64_t j = 0; j < h; ++j) {                                                   \
          const R wr = wl[j].re, wi = sg * wl[j].im;                                        \
          const R ar = xa[j].re, ai = xa[j].im, br = xb[j].re, bi = xb[j].im;               \
          const R tr = br * wr - bi * wi, ti = br * wi + bi * wr;                           \
          xa[j].re = ar + tr;                                                               \
          xa[j].im = ai + ti;                                                               \
          xb[j].re = ar - tr;                                                               \
          xb[j].im = ai - ti;                                                               \
        }                                                                                   \
      }                                                                                     \
    }                                                                                       \
  }
DEFINE_FFT(fft_line_d, cdbl, double)
DEFINE_FFT(fft_line_f, cflt, float)

/* Transform every component plane of every trajectory over the spatial axes: the x
 * lines one by one, then the y lines in chunks of XC adjacent columns transformed in
 * place, each radix-2 layer a loop over whole row segments (contiguous in x). */
#define DEFINE_FFT_PLANES(NAME, C, R, LINE)                                                  \
  static void NAME(C* u, int64_t nplanes, int ndim, const int64_t* n, const C* tw0,         \
                   const C* tw1, const int32_t* rev0, const int32_t* rev1, int dir) {       \
    const int64_t nx = n[0], ny = ndim == 2 ? n[1] : 1, P = nx * ny;                        \
    _Pragma("omp parallel for schedule(static)")                                            \
    for (int64_t l = 0; l < nplanes * ny; ++l) LINE(u + l * nx, nx, tw0, rev0, dir);        \
    if (ndim == 2) {                                                                        \
      const int64_t XC = 16; /* columns per chunk */                                        \
      const int64_t nch = nx / XC;                                                          \
      const R sg = dir < 0 ? (R)1 : (R)-1;                                                  \
      _Pragma("omp parallel for schedule(static)")                                          \
      for (int64_t w = 0; w < nplanes * nch; ++w) {                                         \
        C* pl = u + (w / nch) * P + (w % nch) * XC;                                         \
        for (int64_t i = 0; i < ny; ++i) {                                                  \
          const int64_t r = rev1[i];                                                        \
          if (r > i)                                                                        \
            for (int64_t c = 0; c < XC; ++c) {                                              \
              C t = pl[i * nx + c];                                                         \
              pl[i * nx + c] = pl[r * nx + c];                                              \
              pl[r * nx + c] = t;                                                           \
            }                                                                               \
        }                                                                                   \
        for (int64_t h = 1; h < ny; h <<= 1) {                                              \
          const C* wl = tw1 + (h - 1);                                                      \
          for (int64_t s = 0; s < ny; s += 2 * h)                                           \
            for (int64_t j = 0; j < h; ++j) {                                               \
              const R wr = wl[j].re, wi = sg * wl[j].im;                                    \
              C* xa = pl + (s + j) * nx;                                                    \
              C* xb = pl + (s + j + h) * nx;                                                \
              for (int64_t c = 0; c < XC; ++c) {                                            \
                const R ar = xa[c].re, ai = xa[c].im, br = xb[c].re, bi = xb[c].im;         \
                const R tr = br * wr - bi * wi, ti = br * wi + bi * wr;                     \
                xa[c].re = ar + tr;                                                         \
                xa[c].im = ai + ti;                                                         \
                xb[c].re = ar - tr;                                                         \
                xb[c].im = ai - ti;                                                         \
              }                                                                             \
            }                                                                               \
        }                                                                                   \
      }                                                                                     \
    }                                                                                       \
  }
DEFINE_FFT_PLANES(fft_planes_d, cdbl, double, fft_line_d)
DEFINE_FFT_PLANES(fft_planes_f, cflt, float, fft_line_f)

/* Twiddles of every radix-2 layer of a line of N points, layer h (h = 1, 2, 4, ...)
 * holding w_{2h}^j = exp(-2 pi i j / (2h)), j < h, at offset h - 1: N - 1 entries, each
 * evaluated as exp(-2 pi i (j N/(2h)) / N) in FP64. */
static cdbl* twiddles_d(int64_t N) {
  cdbl* w = (cdbl*)malloc(sizeof(cdbl) * (size_t)(N > 1 ? N - 1 : 1));
  for (int64_t h = 1; h < N; h <<= 1)
    for (int64_t j = 0; j < h; ++j) {
      const double th = -2.0 * M_PI * (double)(j * (N / (2 * h))) / (double)N;
      w[h - 1 + j] = cd(cos(th), sin(th));
    }
  return w;
}
/* index bit-reversal permutation of a line of N = 2^k points */
static int32_t* bitrev_table(int64_t N) {
  const int lg = ilog2_64(N);
  int32_t* r = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
  for (int64_t i = 0; i < N; ++i) {
    int64_t v = 0;
    for (int b = 0; b < lg; ++b) v |= ((i >> b) & 1) << (lg - 1 - b);
    r[i] = (int32_t)v;
  }
  return r;
}
static cflt* twiddles_f(const cdbl* wd, int64_t N) {
  cflt* w = (cflt*)malloc(sizeof(cflt) * (size_t)(N > 1 ? N - 1 : 1));
  for (int64_t k = 0; k < N - 1; ++k) {
    w[k].re = (float)wd[k].re;
    w[k].im = (float)wd[k].im;
  }
  return w;
}

/* ------------------------------------------------------------------ noise
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2,
 * 3", SC'11): ten rounds of two 32x32->64 multiplications with the published multipliers
 * and Weyl key increments.  Counter (point, trajectory, h mod 2^32, h >> 32), key (seed
 * mod 2^32, seed >> 32). */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1, n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
  }
}
/* Box-Muller: sqrt(-ln u1) (cos 2 pi u2, sin 2 pi u2), E|xi|^2 = 1.  FP64 draw:
 * u1 = (w0 + 1/2) 2^-32, u2 = w1 2^-32; FP32 draw: the top 24 bits of each word. */
static cdbl box_muller(uint32_t w0, uint32_t w1, int draw32) {
  double u1, u2;
  if (draw32) {
    u1 = ((double)(w0 >> 8) + 0.5) * 0x1p-24;
    u2 = (double)(w1 >> 8) * 0x1p-24;
  } else {
    u1 = ((double)w0 + 0.5) * 0x1p-32;
    u2 = (double)w1 * 0x1p-32;
  }
  const double mag = sqrt(-log(u1));
  double sn, cs;
  sincos(2.0 * M_PI * u2, &sn, &cs);
  if (draw32) return cd((double)(float)(mag * cs), (double)(float)(mag * sn)); /* an FP32 draw */
  return cd(mag * cs, mag * sn);
}
/* xi of point p (x = p mod nx) of trajectory b at half step h, components 0..M-1: two
 * components draw their own block (words 0,1 and 2,3); one component shares the block of
 * the points x and x + nx/2 of a row (words 0,1 for the lower, 2,3 for the upper). */
static void draw_xi(const oref_desc* d, int64_t p, int64_t b, int64_t h, cdbl xi[2]) {
  const int64_t nx = d->n[0];
  const int up = d->M == 1 && (p % nx) >= nx / 2;
  uint32_t c[4] = {(uint32_t)(up ? p - nx / 2 : p), (uint32_t)(b + d->traj0), (uint32_t)h, (uint32_t)((uint64_t)h >> 32)};
  philox(c, (uint32_t)d->seed, (uint32_t)(d->seed >> 32));
  if (d->M == 1) {
    xi[0] = up ? box_muller(c[2], c[3], d->draw32) : box_muller(c[0], c[1], d->draw32);
  } else {
    xi[0] = box_muller(c[0], c[1], d->draw32);
    xi[1] = box_muller(c[2], c[3], d->draw32);
  }
}

/* ------------------------------------------------------------------ half step
 * src/kernels.jl:37-54 with delta = dt/2 at one point:
 *   u <- cis(-delta G(u)) V (u + delta/2 F_now) + delta/2 F_next,
 * G evaluated on u before the pump is added (:40,44). */
static void half_point(const oref_desc* d, cdbl* v, int64_t p, int64_t b, int64_t h, int64_t P, cdbl an[2],
                       cdbl ax[2]) {
  const int M = d->M;
  const double delta = 0.5 * d->dt;
  cdbl E[2];
  int hasE[2] = {0, 0};
  if (d->g) {
    double dens[2];
    for (int l = 0; l < M; ++l) dens[l] = v[l].re * v[l].re + v[l].im * v[l].im;
    for (int j = 0; j < M; ++j) {
      cdbl G = d->c ? cd(d->c[2 * j], d->c[2 * j + 1]) : cd(0.0, 0.0);
      for (int l = 0; l < M; ++l) {
        const cdbl gl = cd(d->g[2 * (j * M + l)], d->g[2 * (j * M + l) + 1]);
        if (gl.re != 0.0 || gl.im != 0.0) G = cdadd(G, cdscale(gl, dens[l]));
      }
      /* exp(-i delta G) = exp(delta Im G) (cos(delta Re G) - i sin(delta Re G)) */
      const double mag = G.im != 0.0 ? exp(delta * G.im) : 1.0, ph = delta * G.re;
      double sn, cs;
      sincos(ph, &sn, &cs);
      E[j] = cd(mag * cs, -mag * sn);
      hasE[j] = 1;
    }
  }
  if (d->vtab) {
    for (int j = 0; j < M; ++j) {
      const int64_t e = d->vkind == 2 ? j : 0;
      const cdbl V = cd(d->vtab[2 * (e * P + p)], d->vtab[2 * (e * P + p) + 1]);
      E[j] = hasE[j] ? cdmul(E[j], V) : V;
      hasE[j] = 1;
    }
  }
  for (int j = 0; j < M; ++j) {
    cdbl w = v[j];
    const double* pr = d->pprof[j];
    cdbl prof = cd(0.0, 0.0);
    if (pr) {
      prof = cd(pr[2 * p], pr[2 * p + 1]);
      w = cdadd(w, cdscale(cdmul(an[j], prof), delta / 2));
    }
    if (hasE[j]) w = cdmul(E[j], w);
    if (pr) w = cdadd(w, cdscale(cdmul(ax[j], prof), delta / 2));
    v[j] = w;
  }
  if (d->noise) {
    /* -i sqrt(delta) eta xi, added after the linear part (src/kernels.jl:42,49) */
    cdbl xi[2];
    draw_xi(d, p, b, h, xi);
    const double sq = sqrt(delta);
    for (int j = 0; j < M; ++j) {
      const cdbl nf = cd(sq * d->eta[2 * j + 1], -sq * d->eta[2 * j]);
      v[j] = cdadd(v[j], cdmul(nf, xi[j]));
    }
  }
}

static void pump_amps(const oref_desc* d, int64_t h, cdbl an[2], cdbl ax[2]) {
  for (int j = 0; j < d->M; ++j) {
    an[j] = ax[j] = cd(0.0, 0.0);
    if (!d->pprof[j]) continue;
    const int64_t i0 = h < d->namp ? h : d->namp - 1, i1 = h + 1 < d->namp ? h + 1 : d->namp - 1;
    an[j] = cd(d->pamp[j][2 * i0], d->pamp[j][2 * i0 + 1]);
    ax[j] = cd(d->pamp[j][2 * i1], d->pamp[j][2 * i1 + 1]);
  }
}

/* ------------------------------------------------------------------ k-space product
 * src/strang_splitting.jl:69-76: ft <- exp(-i dt D(k)) ft per point (scalar, diagonal or
 * a 2x2 mat-vec), then the caller's inverse transform and 1/P. */
static void kspace_point(const oref_desc* d, cdbl* v, int64_t p, int64_t P) {
  const double* T = d->ktab;
  if (d->kkind == 3 && d->M == 2) {
    const cdbl t00 = cd(T[2 * p], T[2 * p + 1]), t01 = cd(T[2 * (P + p)], T[2 * (P + p) + 1]);
    const cdbl t10 = cd(T[2 * (2 * P + p)], T[2 * (2 * P + p) + 1]), t11 = cd(T[2 * (3 * P + p)], T[2 * (3 * P + p) + 1]);
    const cdbl y0 = cdadd(cdmul(t00, v[0]), cdmul(t01, v[1]));
    const cdbl y1 = cdadd(cdmul(t10, v[0]), cdmul(t11, v[1]));
    v[0] = y0;
    v[1] = y1;
    return;
  }
  for (int j = 0; j < d->M; ++j) {
    const int64_t e = d->kkind == 2 ? j : 0;
    v[j] = cdmul(cd(T[2 * (e * P + p)], T[2 * (e * P + p) + 1]), v[j]);
  }
}

/* Pointwise passes over every point of every trajectory; the field is FP64 (u64) or
 * single precision (u32, promoted to FP64 for the products and rounded when stored). */
static void pointwise(const oref_desc* d, cdbl* u64, cflt* u32, int64_t P, int kind, int64_t h, double scale) {
  const int M = d->M;
  const int64_t BP = d->B * P;
  cdbl an[2], ax[2];
  if (kind == 0) pump_amps(d, h, an, ax);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < BP; ++i) {
    const int64_t p = i % P;
    cdbl v[2];
    for (int j = 0; j < M; ++j) v[j] = u64 ? u64[j * BP + i] : cd(u32[j * BP + i].re, u32[j * BP + i].im);
    if (kind == 0) {
      cdbl a0[2] = {an[0], an[1]}, a1[2] = {ax[0], ax[1]};
      half_point(d, v, p, i / P, h, P, a0, a1);
    } else {
      /* the table product, then the inverse transform's 1/P: a power of two, so scaling
         before the inverse transform rounds exactly as scaling after it */
      kspace_point(d, v, p, P);
      for (int j = 0; j < M; ++j) v[j] = cdscale(v[j], scale);
    }
    for (int j = 0; j < M; ++j) {
      if (u64) {
        u64[j * BP + i] = v[j];
      } else {
        u32[j * BP + i].re = (float)v[j].re;
        u32[j * BP + i].im = (float)v[j].im;
      }
    }
  }
}

/* Advance nsteps full steps from absolute step step0 (which indexes the pump
 * amplitudes).  u: M*B*P complex FP64 values [m][b][p], in and out.  saves (may be NULL
 * when save_every == 0): slot s of component m at saves + 2*(m*nsaves + s)*B*P. */
int oref_run(const oref_desc* d, double* u, int64_t step0, int64_t nsteps, int64_t save_every, double* saves) {
  if (!d || !u || d->ndim < 1 || d->ndim > 2 || d->M < 1 || d->M > 2 || d->B < 1 || nsteps < 0) return -1;
  if (save_every < 0 || (save_every > 0 && (!saves || nsteps % save_every))) return -1;
  const int64_t nx = d->n[0], ny = d->ndim == 2 ? d->n[1] : 1, P = nx * ny;
  for (int a = 0; a < d->ndim; ++a)
    if (d->n[a] < 2 || (d->n[a] & (d->n[a] - 1))) return -1;
  if (d->ndim == 2 && nx % 16) return -1;
#ifdef _OPENMP
  if (d->threads > 0) omp_set_num_threads(d->threads);
#endif
  const int64_t BP = d->B * P, tot = d->M * BP;
  const int64_t nsaves = save_every > 0 ? nsteps / save_every : 0;
  cdbl* tw0 = twiddles_d(nx);
  cdbl* tw1 = twiddles_d(ny);
  int32_t* rv0 = bitrev_table(nx);
  int32_t* rv1 = bitrev_table(ny);
  cdbl* u64 = (cdbl*)u;
  cflt *u32 = NULL, *tf0 = NULL, *tf1 = NULL;
  if (d->fp32) {
    u32 = (cflt*)malloc(sizeof(cflt) * (size_t)tot);
    for (int64_t i = 0; i < tot; ++i) {
      u32[i].re = (float)u64[i].re;
      u32[i].im = (float)u64[i].im;
    }
    tf0 = twiddles_f(tw0, nx);
    tf1 = twiddles_f(tw1, ny);
  }
  for (int64_t k = 0; k < nsteps; ++k) {
    const int64_t h = 2 * (step0 + k);
    pointwise(d, d->fp32 ? NULL : u64, u32, P, 0, h, 0.0);
    if (d->ktab) {
      if (d->fp32) fft_planes_f(u32, d->M * d->B, d->ndim, d->n, tf0, tf1, rv0, rv1, -1);
      else fft_planes_d(u64, d->M * d->B, d->ndim, d->n, tw0, tw1, rv0, rv1, -1);
      pointwise(d, d->fp32 ? NULL : u64, u32, P, 1, h, 1.0 / (double)P);
      if (d->fp32) fft_planes_f(u32, d->M * d->B, d->ndim, d->n, tf0, tf1, rv0, rv1, +1);
      else fft_planes_d(u64, d->M * d->B, d->ndim, d->n, tw0, tw1, rv0, rv1, +1);
    }
    pointwise(d, d->fp32 ? NULL : u64, u32, P, 0, h + 1, 0.0);
    if (save_every > 0 && (k + 1) % save_every == 0) {
      const int64_t s = (k + 1) / save_every - 1;
      for (int m = 0; m < d->M; ++m) {
        double* dst = saves + 2 * (m * nsaves + s) * BP;
        for (int64_t i = 0; i < BP; ++i) {
          dst[2 * i] = d->fp32 ? (double)u32[m * BP + i].re : u64[m * BP + i].re;
          dst[2 * i + 1] = d->fp32 ? (double)u32[m * BP + i].im : u64[m * BP + i].im;
        }
      }
    }
  }
  if (d->fp32) {
    for (int64_t i = 0; i < tot; ++i) u64[i] = cd(u32[i].re, u32[i].im);
    free(u32);
    free(tf0);
    free(tf1);
  }
  free(tw0);
  free(tw1);
  free(rv0);
  free(rv1);
  return 0;
}
