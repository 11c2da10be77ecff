// CPU restatement of the reference's input preparation (test infrastructure
// only): haloden.f90's particle density assignment and from1024to512.f90's
// coarsening, loop for loop, in the reference's default real (FP32) and
// real(8) where it uses them.  PARITY UNPINNED: the reference ships neither
// particle files nor outputs of these programs.
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

// Fortran MODULO for reals: A - FLOOR(A/P)*P, evaluated as the exact
// remainder and one correcting addition.
float fmodulo(float a, float p) {
  float r = std::fmod(a, p);
  if (r != 0.0f && ((r < 0.0f) != (p < 0.0f))) r += p;
  return r;
}
int imodulo(int a, int p) {
  int r = a % p;
  return r < 0 ? r + p : r;
}

}  // namespace

extern "C" {

// haloden.f90:87-180.  x: positions (3, np) in fine-cell units (the node
// offsets already added, haloden.f90:63-66); nf fine cells and ng grid cells
// per dimension.  den (ng^3, Fortran order) receives the normalised density,
// raw (ng^3, may be null) the density before normalisation, wp (np, may be
// null) the number of cells of each particle.  Returns 0, or -1 when a
// particle position lands outside the grid after the wrap (the reference
// would index out of bounds).
int orc_haloden(const float* x, long long np, int nf, int ng, float* den, float* raw, int* wp_out) {
  const long long ng3 = (long long)ng * ng * ng;
  std::vector<float> xp(3 * np);
  for (long long ip = 0; ip < np; ++ip)
    for (int a = 0; a < 3; ++a) {
      float v = fmodulo(x[3 * ip + a], (float)nf);  // haloden.f90:87-91
      xp[3 * ip + a] = v * (float)ng / (float)nf;    // haloden.f90:94
    }
  // linked lists, 1-based as in the reference (0 = end)
  std::vector<long long> hoc_g(ng3, 0), ll_p(np + 1, 0), hoc_p(np + 1, 0), ll_g(ng3 + 1, 0);
  std::vector<int> wp(np + 1, 1);
  auto cell = [&](int i, int j, int k) { return (long long)ng * ng * (k - 1) + (long long)ng * (j - 1) + i; };
  for (long long ip = 1; ip <= np; ++ip) {  // haloden.f90:98-108
    int i = (int)std::floor(xp[3 * (ip - 1)]) + 1;
    int j = (int)std::floor(xp[3 * (ip - 1) + 1]) + 1;
    int k = (int)std::floor(xp[3 * (ip - 1) + 2]) + 1;
    if (i < 1 || i > ng || j < 1 || j > ng || k < 1 || k > ng) return -1;
    long long g = cell(i, j, k);
    ll_p[ip] = hoc_g[g - 1];
    hoc_g[g - 1] = ip;
  }
  for (long long g = 1; g <= ng3; ++g)  // haloden.f90:113-124
    for (long long pp = hoc_g[g - 1]; pp != 0; pp = ll_p[pp]) hoc_p[pp] = g;
  const int h = ng / 2;
  for (int k = 1; k <= ng; ++k)  // haloden.f90:127-170
    for (int j = 1; j <= ng; ++j)
      for (int i = 1; i <= ng; ++i) {
        const long long ig = cell(i, j, k);
        if (hoc_g[ig - 1] != 0) continue;
        const float gpos[3] = {(float)i - 0.5f, (float)j - 0.5f, (float)k - 0.5f};
        float r2min = (float)(1000 * ng * ng);
        long long pp_s = 0;
        bool search = true;
        for (int r = 1; search && r <= ng; ++r) {
          for (int ks = k - r; ks <= k + r; ++ks)
            for (int js = j - r; js <= j + r; ++js)
              for (int is = i - r; is <= i + r; ++is) {
                const long long g = cell(imodulo(is - 1, ng) + 1, imodulo(js - 1, ng) + 1, imodulo(ks - 1, ng) + 1);
                for (long long pp = hoc_g[g - 1]; pp != 0; pp = ll_p[pp]) {
                  search = false;
                  float d[3];
                  for (int a = 0; a < 3; ++a) {
                    float v = xp[3 * (pp - 1) + a] - gpos[a];
                    d[a] = fmodulo(v + (float)h, (float)ng) - (float)h;
                  }
                  float r2 = d[0] * d[0] + d[1] * d[1];
                  r2 = r2 + d[2] * d[2];
                  if (r2 < r2min) {
                    r2min = r2;
                    pp_s = pp;
                  }
                }
              }
        }
        if (pp_s == 0) return -1;  // no particle at all
        ll_g[ig] = hoc_p[pp_s];
        hoc_p[pp_s] = ig;
        wp[pp_s] += 1;
      }
  std::vector<float> d(ng3, 0.0f);
  for (long long ip = 1; ip <= np; ++ip)  // haloden.f90:173-182
    for (long long g = hoc_p[ip]; g != 0; g = ll_g[g]) d[g - 1] = d[g - 1] + 1.0f / (float)wp[ip];
  double s = 0.0;
  for (long long q = 0; q < ng3; ++q) s += (double)d[q];
  const double scale = (double)((float)ng * (float)ng * (float)ng);
  for (long long q = 0; q < ng3; ++q) {  // haloden.f90:189
    den[q] = (float)((double)d[q] / s * scale);
    if (raw) raw[q] = d[q];
  }
  if (wp_out)
    for (long long ip = 0; ip < np; ++ip) wp_out[ip] = wp[ip + 1];
  return 0;
}

// from1024to512.f90:15-22, 54-66: ncoarse halvings, each cell the sum of its
// 2x2x2 block (Fortran's sum over the section, first index fastest), and the
// result scaled to mean 1 with the sum taken in real(8) (the reference sums
// in real(4), whose rounding at 10^8 cells is not reproduced).
void orc_coarsen(const float* den, int ng, int ncoarse, float* out) {
  int nf = ng;
  std::vector<float> a(den, den + (long long)ng * ng * ng);
  for (int c = 0; c < ncoarse; ++c) {
    const int h = nf / 2;
    std::vector<float> b((long long)h * h * h);
    for (int k = 0; k < h; ++k)
      for (int j = 0; j < h; ++j)
        for (int i = 0; i < h; ++i) {
          float s = 0.0f;
          for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
              for (int di = 0; di < 2; ++di)
                s = s + a[(2 * i + di) + (long long)nf * ((2 * j + dj) + (long long)nf * (2 * k + dk))];
          b[i + (long long)h * (j + (long long)h * k)] = s;
        }
    a.swap(b);
    nf = h;
  }
  const long long n3 = (long long)nf * nf * nf;
  double s = 0.0;
  for (long long q = 0; q < n3; ++q) s += (double)a[q];
  const float sf = (float)s, scale = (float)n3;
  for (long long q = 0; q < n3; ++q) out[q] = a[q] / sf * scale;
}

}  // extern "C"
