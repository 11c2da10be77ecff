// CPU restatement of the reference's input preparation and post-processing
// (test infrastructure only): haloden.f90's particle density assignment,
// from1024to512.f90's coarsening, mmh/column_density.f90 and gridfigure.f90's
// displacement interpolation and column density, loop for loop, in the reference's default real (FP32) and
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

// Exact sum of floats (128-bit fixed point, 64 fractional bits, terms
// truncated below 2^-64), rounded to double as hi + lo * 2^-64: the sum the
// GPU forms.  It restates the reference's real(4) sum(den), whose rounding
// depends on the compiler's reduction order.
static double exact_sum_f(const float* a, long long n) {
  __int128 s = 0;
  for (long long q = 0; q < n; ++q) s += (__int128)std::ldexp((double)a[q], 64);
  bool neg = s < 0;
  unsigned __int128 m = neg ? (unsigned __int128)(-s) : (unsigned __int128)s;
  double r = (double)(unsigned long long)(m >> 64) + (double)(unsigned long long)m * 5.42101086242752217e-20;
  return neg ? -r : r;
}

// den / sum(den) * ng**3 in real(4)
static std::vector<float> normalised(const float* den, int ng) {
  const long long n3 = (long long)ng * ng * ng;
  const float sf = (float)exact_sum_f(den, n3), scale = (float)(int)n3;
  std::vector<float> d(n3);
  for (long long q = 0; q < n3; ++q) d[q] = den[q] / sf * scale;
  return d;
}

// The column of (i, j) between the displaced faces kk1 and kk2 (1-based
// cells), with fractional end cells: column_density.f90:42-53.  Cells outside
// 1..ng wrap periodically (the reference reads out of bounds there).
static float column(const std::vector<float>& den, int ng, int i, int j, float kk1, float kk2) {
  auto D = [&](int k) {
    int kw = ((k - 1) % ng + ng) % ng;
    return den[(i - 1) + (long long)ng * ((j - 1) + (long long)ng * kw)];
  };
  int nk1 = (int)std::floor(kk1) + 1, nk2 = (int)std::floor(kk2) + 1;
  float r1 = (float)nk1 - kk1;
  float r2 = kk2 - (float)nk2 + 1.0f;
  float s1 = 0.0f, s2 = 0.0f;
  for (int k = nk1 + 1; k <= nk2 - 1; ++k) s1 = s1 + D(k);
  for (int k = nk2; k <= nk1; ++k) s2 = s2 + D(k);
  float t = r1 * D(nk1) + s1;
  t = t + r2 * D(nk2);
  return t - s2;
}

// mmh/column_density.f90:17-57: proj (ng^2) from den and def (ng^3).
void orc_column_density(const float* den_in, const float* def, int ng, int nplot, float* proj) {
  const std::vector<float> den = normalised(den_in, ng);
  const long long n3 = (long long)ng * ng * ng;
  std::vector<float> dz(n3);
  auto F = [&](int i, int j, int k) { return def[(i - 1) + (long long)ng * ((j - 1) + (long long)ng * (k - 1))]; };
  for (int k = 1; k <= ng; ++k)
    for (int j = 1; j <= ng; ++j)
      for (int i = 1; i <= ng; ++i) {
        int kp = k % ng + 1, jp = j % ng + 1, ip = i % ng + 1;
        float v = F(i, j, kp) + F(ip, j, kp);
        v = v + F(i, jp, kp);
        v = v + F(ip, jp, kp);
        v = v - F(i, j, k);
        v = v - F(ip, j, k);
        v = v - F(i, jp, k);
        v = v - F(ip, jp, k);
        dz[(i - 1) + (long long)ng * ((j - 1) + (long long)ng * (k - 1))] = v / 4.0f;
      }
  auto Z = [&](int i, int j, int k) { return dz[(i - 1) + (long long)ng * ((j - 1) + (long long)ng * (k - 1))]; };
  const int k1 = ng / 2, k2 = k1 + nplot - 1;
  for (int j = 1; j <= ng; ++j)
    for (int i = 1; i <= ng; ++i) {
      int jm = imodulo(j - 2, ng) + 1, im = imodulo(i - 2, ng) + 1, k1m = imodulo(k1 - 2, ng) + 1;
      float a = Z(im, jm, k1m) + Z(i, jm, k1m);
      a = a + Z(im, j, k1m);
      a = a + Z(i, j, k1m);
      float kk1 = (float)(k1 - 1) + a / 4.0f;
      float b = Z(im, jm, k2) + Z(i, jm, k2);
      b = b + Z(im, j, k2);
      b = b + Z(i, j, k2);
      float kk2 = (float)k2 + b / 4.0f;
      proj[(i - 1) + (long long)ng * (j - 1)] = column(den, ng, i, j, kk1, kk2) / (float)nplot;
    }
}

// gridfigure.f90:41-120: the displacement of the coarse def (nf^3) on the
// (0:nf)^3 node grid with the reference's halo assignment, trilinear
// interpolation to the fine cells (ratio = ng / nf), new positions, and the
// column density (nplot = 1) of den (ng^3).  proj2 (2, nf, nf) receives the
// new x, y positions of every ratio-th cell of plane ng/2, proj (ng^2) the
// column density.  A node index nf+1 (cells i = ng, read out of bounds by the
// reference) wraps to 1.
void orc_gridfigure(const float* def, int nf, const float* den_in, int ng, float* proj2, float* proj) {
  const int ratio = ng / nf, m = nf + 1;
  const std::vector<float> den = normalised(den_in, ng);
  std::vector<float> T0(3 * (long long)m * m * m, 0.0f), TD;
  auto at = [&](int c, int i, int j, int k) { return (long long)c + 3 * (i + (long long)m * (j + (long long)m * k)); };
  auto F = [&](int i, int j, int k) { return def[(i - 1) + (long long)nf * ((j - 1) + (long long)nf * (k - 1))]; };
  const float cf = (float)ratio * 1.0f / 4.0f;
  for (int k = 1; k <= nf; ++k)
    for (int j = 1; j <= nf; ++j)
      for (int i = 1; i <= nf; ++i) {
        int ip = i % nf + 1, jp = j % nf + 1, kp = k % nf + 1;
        float x = F(ip, j, k) - F(i, j, k);
        x = x + F(ip, jp, k);
        x = x - F(i, jp, k);
        x = x + F(ip, j, kp);
        x = x - F(i, j, kp);
        x = x + F(ip, jp, kp);
        x = x - F(i, jp, kp);
        float y = F(i, jp, k) - F(i, j, k);
        y = y + F(ip, jp, k);
        y = y - F(ip, j, k);
        y = y + F(i, jp, kp);
        y = y - F(i, j, kp);
        y = y + F(ip, jp, kp);
        y = y - F(ip, j, kp);
        float z = F(i, j, kp) - F(i, j, k);
        z = z + F(ip, j, kp);
        z = z - F(ip, j, k);
        z = z + F(i, jp, kp);
        z = z - F(i, jp, k);
        z = z + F(ip, jp, kp);
        z = z - F(ip, jp, k);
        T0[at(0, i, j, k)] = cf * x;
        T0[at(1, i, j, k)] = cf * y;
        T0[at(2, i, j, k)] = cf * z;
      }
  // tmp = cshift by -1 along the three node dimensions (length nf+1), then
  // the three boundary assignments of gridfigure.f90:62-64
  TD = T0;
  auto w = [&](int v) { return v < 0 ? v + m : v; };
  for (int c = 0; c < 3; ++c) {
    for (int k = 1; k <= nf; ++k)
      for (int j = 1; j <= nf; ++j) TD[at(c, 0, j, k)] = T0[at(c, w(-1), j - 1, k - 1)];
    for (int j = 0; j <= nf; ++j)
      for (int i = 1; i <= nf; ++i) TD[at(c, i, j, 0)] = T0[at(c, i - 1, w(j - 1), w(-1))];
    for (int k = 1; k <= nf; ++k)
      for (int i = 1; i <= nf; ++i) TD[at(c, i, 0, k)] = T0[at(c, i - 1, w(-1), k - 1)];
  }
  auto node = [&](int v) { return v == nf + 1 ? 1 : v; };
  auto disp = [&](int c, int i, int j, int k) {
    float ib = (float)(i % ratio) / (float)ratio, jb = (float)(j % ratio) / (float)ratio,
          kb = (float)(k % ratio) / (float)ratio;
    int ip = (int)std::floor((float)i / (float)ratio) + 1 - (int)std::floor(ib);
    int jp = (int)std::floor((float)j / (float)ratio) + 1 - (int)std::floor(jb);
    int kp = (int)std::floor((float)k / (float)ratio) + 1 - (int)std::floor(kb);
    int i0 = ip - 1, j0 = jp - 1, k0 = kp - 1, i1 = node(ip), j1 = node(jp), k1 = node(kp);
    float p111 = ib * jb * kb, p211 = (1.0f - ib) * jb * kb, p121 = ib * (1.0f - jb) * kb;
    float p112 = ib * jb * (1.0f - kb), p221 = (1.0f - ib) * (1.0f - jb) * kb, p212 = (1.0f - ib) * jb * (1.0f - kb);
    float p122 = ib * (1.0f - jb) * (1.0f - kb), p222 = (1.0f - ib) * (1.0f - jb) * (1.0f - kb);
    float d = 0.0f;
    d = d + TD[at(c, i0, j0, k0)] * p111;
    d = d + TD[at(c, i1, j0, k0)] * p211;
    d = d + TD[at(c, i0, j1, k0)] * p121;
    d = d + TD[at(c, i0, j0, k1)] * p112;
    d = d + TD[at(c, i1, j1, k0)] * p221;
    d = d + TD[at(c, i1, j0, k1)] * p212;
    d = d + TD[at(c, i0, j1, k1)] * p122;
    d = d + TD[at(c, i1, j1, k1)] * p222;
    return d;
  };
  const int k1 = ng / 2, k2 = k1;
  for (int j = 1; j <= ng; ++j)
    for (int i = 1; i <= ng; ++i) {
      int jm = imodulo(j - 2, ng) + 1, im = imodulo(i - 2, ng) + 1, k1m = imodulo(k1 - 2, ng) + 1;
      float a = disp(2, im, jm, k1m) + disp(2, i, jm, k1m);
      a = a + disp(2, im, j, k1m);
      a = a + disp(2, i, j, k1m);
      float kk1 = (float)(k1 - 1) + a / 4.0f;
      float b = disp(2, im, jm, k2) + disp(2, i, jm, k2);
      b = b + disp(2, im, j, k2);
      b = b + disp(2, i, j, k2);
      float kk2 = (float)k2 + b / 4.0f;
      proj[(i - 1) + (long long)ng * (j - 1)] = column(den, ng, i, j, kk1, kk2) / 1.0f;
    }
  for (int b = 1; b <= nf; ++b)
    for (int a = 1; a <= nf; ++a)
      for (int c = 0; c < 2; ++c) {
        int ii = ratio * a, jj = ratio * b, kk = ng / 2;
        int idx[3] = {ii, jj, kk};
        proj2[c + 2 * ((a - 1) + (long long)nf * (b - 1))] = ((float)idx[c] + 0.5f) + disp(c, ii, jj, kk);
      }
}

}  // extern "C"
