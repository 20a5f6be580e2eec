/* The reference's plain case driven through the C ABI alone, as a Julia ccall shim
 * would drive it: 2D Kerr on 128x128, L = 8, u0 = exp(-(x-4)^2 - (y-4)^2), D = |k|^2/2,
 * G = -6|u|^2, solve(prob, StrangSplitting(), (0, 0.4); dt = 0.01, nsaves = 64), i.e.
 * 64 steps of the resolved dt = 0.00625 (src/fixed_time_stepping.jl:14-24), one save a
 * step.  Writes the 64th save (FP64 complex, [y][x]) and the last time to argv[1].
 *
 *     gcc -O2 -I include kerr_c0.c -L<libdir> -lgpe -lm -o kerr_c0 && ./kerr_c0 out.bin
 */
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <stdlib.h>

#include "gpe.h"

#define CHECK(h, call)                                                     \
  do {                                                                     \
    int rc_ = (call);                                                      \
    if (rc_ != GPE_OK) {                                                   \
      fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, gpe_last_error(h)); \
      return 1;                                                            \
    }                                                                      \
  } while (0)

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s out.bin [native]\n", argv[0]);
    return 2;
  }
  const int N = 128, nsaves = 64;
  const double L = 8.0, pi = 3.14159265358979323846;
  /* resolve_fixed_timestepping: dT = 0.4/64, steps per save = ceil(dT/0.01) = 1 */
  const double dT = 0.4 / nsaves;
  const long per = (long)ceil(dT / 0.01 - 1e-12);
  const double dt = dT / per;

  gpe_desc d = {0};
  d.abi_version = GPE_ABI_VERSION;
  d.ndim = 2;
  d.n[0] = N; d.n[1] = N; d.n[2] = 1;
  d.lengths[0] = L; d.lengths[1] = L; d.lengths[2] = 1.0;
  d.batch = 1;
  d.ncomp = 1;
  d.dtype = GPE_C128;
  d.dt = dt;
  d.t0 = 0.0;
  d.device = -1;
  /* block floating point line transforms by default; "native": FP64 floating point
     throughout; "dw": double-word */
  d.flags = argc > 2 && strcmp(argv[2], "dw") == 0       ? GPE_FLAG_FP64_DW
            : argc > 2 && strcmp(argv[2], "native") == 0 ? GPE_FLAG_FP64_NATIVE
                                                          : 0;
  gpe_handle* h = NULL;
  CHECK(NULL, gpe_create(&d, &h));

  const size_t P = (size_t)N * N;
  double* u0 = malloc(2 * P * sizeof(double));
  double* D = malloc(2 * P * sizeof(double));
  double* out = malloc(2 * P * nsaves * sizeof(double));
  double* ts = malloc(nsaves * sizeof(double));
  double g[2] = {-6.0, 0.0};
  if (!u0 || !D || !out || !ts) return 1;
  for (int y = 0; y < N; ++y)
    for (int x = 0; x < N; ++x) {
      const size_t p = (size_t)y * N + x;
      const double xv = x * L / N, yv = y * L / N;
      u0[2 * p] = exp(-(xv - 4) * (xv - 4) - (yv - 4) * (yv - 4));
      u0[2 * p + 1] = 0.0;
      /* reciprocal_grid: 2 pi / L * (0, 1, ..., N/2-1, -N/2, ..., -1) */
      const double kx = 2 * pi / L * (x < N / 2 ? x : x - N);
      const double ky = 2 * pi / L * (y < N / 2 ? y : y - N);
      D[2 * p] = (kx * kx + ky * ky) / 2;
      D[2 * p + 1] = 0.0;
    }
  CHECK(h, gpe_set_field(h, 0, u0));
  CHECK(h, gpe_set_dispersion(h, D, GPE_TABLE_SCALAR));
  CHECK(h, gpe_set_nonlinearity(h, g, NULL));
  CHECK(h, gpe_run(h, nsaves * per, per, out, ts));

  FILE* f = fopen(argv[1], "wb");
  if (!f) return 1;
  fwrite(out + 2 * P * (nsaves - 1), sizeof(double), 2 * P, f);
  fwrite(&ts[nsaves - 1], sizeof(double), 1, f);
  fclose(f);
  printf("kerr_c0: %s, t = %.17g\n", gpe_version(), ts[nsaves - 1]);
  CHECK(h, gpe_destroy(h));
  free(u0); free(D); free(out); free(ts);
  return 0;
}
