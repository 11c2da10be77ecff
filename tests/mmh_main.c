/* A compiled caller of the C ABI that follows the reference's driver loop
 * (mmh/main.f90:83-179) with the drop-in calls a Fortran main program makes
 * through iso_c_binding: default-real (float) arrays, u(5,n,n,n) with only
 * the density set, then per deformation iteration
 *   calcdefp(defp,tmp,tmp2,def,u,1.,1.,5); def = def + defp;
 *   relaxing(u,def,defp,1.,1.,5)
 * and finally scalar2gradient(def,grad,nn) and defp2delta(def,delta,nn).
 *
 * usage: mmh_main <n> <niter> <density.bin> <out_prefix>
 * density.bin: n^3 float32 in Fortran order (the layout of the reference's
 * 0.000den<NNNN>_<id>.bin input).  Writes <out_prefix>def.bin,
 * <out_prefix>grad.bin (n^3 x 3) and <out_prefix>delta.bin (float32), and one
 * line of diagnostics per iteration on stdout.  Exit status 0 on success. */
#include <stdio.h>
#include <stdlib.h>

#include "mmh.h"

static int write_floats(const char* prefix, const char* name, const float* a, size_t count) {
  char path[4096];
  snprintf(path, sizeof(path), "%s%s", prefix, name);
  FILE* f = fopen(path, "wb");
  if (!f) return 1;
  size_t w = fwrite(a, sizeof(float), count, f);
  fclose(f);
  return w == count ? 0 : 1;
}

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: %s <n> <niter> <density.bin> <out_prefix>\n", argv[0]);
    return 2;
  }
  const int n = atoi(argv[1]), niter = atoi(argv[2]);
  const size_t n3 = (size_t)n * n * n;
  float* rho = malloc(sizeof(float) * n3);
  float* u = calloc(5 * n3, sizeof(float));
  float* def = calloc(n3, sizeof(float));
  float* defp = calloc(n3, sizeof(float));
  float* tmp = calloc(n3, sizeof(float));
  float* tmp2 = calloc((size_t)(n + 2) * n * n, sizeof(float));
  float* grad = calloc(3 * n3, sizeof(float));
  float* delta = calloc(n3, sizeof(float));
  if (!rho || !u || !def || !defp || !tmp || !tmp2 || !grad || !delta) return 3;
  FILE* f = fopen(argv[3], "rb");
  if (!f) return 4;
  size_t got = fread(rho, sizeof(float), n3, f);
  fclose(f);
  if (got != n3) return 4;
  for (size_t t = 0; t < n3; ++t) u[5 * t] = rho[t]; /* u(1,i,j,k); u(2:5) = 0 (main.f90:57) */

  mmh_config cfg;
  mmh_config_default(&cfg, n);
  cfg.precision = MMH_FP64;
  cfg.schedule = MMH_SCHED_REF; /* the reference's algorithm */
  mmh_ctx* ctx = NULL;
  int rc = mmh_create(&ctx, &cfg);
  if (rc != MMH_OK) {
    fprintf(stderr, "mmh_create: %s\n", mmh_strerror(rc));
    return 5;
  }
  for (int it = 0; it < niter; ++it) {
    mmh_diag d;
    rc = mmh_calcdefp(ctx, defp, tmp, tmp2, def, u, 1.0f, 1.0f, 5, &d);
    if (rc != MMH_OK && rc != MMH_ERR_DIVERGED) {
      fprintf(stderr, "mmh_calcdefp: %s\n", mmh_strerror(rc));
      return 6;
    }
    for (size_t t = 0; t < n3; ++t) def[t] = def[t] + defp[t];
    rc = mmh_relaxing(ctx, u, def, defp, 1.0f, 1.0f, 5);
    if (rc != MMH_OK) {
      fprintf(stderr, "mmh_relaxing: %s\n", mmh_strerror(rc));
      return 7;
    }
    printf("iter %d r1 %.6e relaxerr %.6e cmax %.5f detmin %.5e detmax %.4f ncompress %lld nexpand %lld\n", it + 1,
           d.r1, d.relaxerr, d.cmax, d.detmin, d.detmax, (long long)d.ncompress, (long long)d.nexpand);
  }
  const int nn[3] = {n, n, n};
  rc = mmh_scalar2gradient(ctx, def, grad, nn);
  if (rc == MMH_OK) rc = mmh_defp2delta(ctx, def, delta, nn);
  if (rc != MMH_OK) {
    fprintf(stderr, "outputs: %s\n", mmh_strerror(rc));
    return 8;
  }
  mmh_destroy(ctx);
  if (write_floats(argv[4], "def.bin", def, n3) || write_floats(argv[4], "grad.bin", grad, 3 * n3) ||
      write_floats(argv[4], "delta.bin", delta, n3))
    return 9;
  free(rho); free(u); free(def); free(defp); free(tmp); free(tmp2); free(grad); free(delta);
  return 0;
}
