// One whole 8-colour Gauss-Seidel sweep (relax, mmh/gauss1.f90:208-499 and
// :866-991) of an FP32 grid in one pass over memory: the mixed form's
// smoother on the levels of 64^3 and up.
//
// The reference's plane schedule is the 8-colour order (plane parity, x
// parity, y parity).  Even planes see the odd planes' old values and the odd
// planes the even planes' new ones, so a sweep can advance through z as a
// wavefront: update even plane k, then odd plane k-1, which needs the new
// planes k-2 and k.  This is r1lax's own plane pyramid, run here by every
// tile column of the grid at once.  Each CTA owns a TX x TY column segment of
// planes [z0, z0+S) and keeps a ring of four planes of phi (k-2 .. k+1) and
// coefficients 1-5 of the plane being updated in shared memory; a plane's
// phi, rhs and six coefficients are read once per sweep and phi is written
// once (9 words per cell; the halos come from L2).  Two CTAs share an SM, so
// one's copies and barriers overlap the other's arithmetic.
//
// No CTA waits for another.  A tile recomputes, from the old values, the
// cells just outside it that its own cells depend on within the sweep (the
// colour-by-colour dependency cones below), and a segment recomputes the even
// plane z0+S that its last odd plane needs.  Every recomputed cell has the
// same inputs as where it is owned, so the swept field is exactly the one the
// sequential 8-colour order gives; only interior cells are written.  The
// sweep reads `src` and writes `dst` (no CTA reads a halo another has
// already overwritten).
//
// Cells are grouped in 2x2 quads (one cell of each in-plane colour), and
// shared memory holds every staged field in four colour sub-planes: cell
// (2a+io, 2b+jo) of the staged region sits at word (2*io+jo)*NQ + quad(a, b).
// A colour phase then reads consecutive words across a warp (no bank
// conflicts).  The fields each update reads only at its own cell (rhs and
// coefficient 6 of its plane, coefficients 3, 5, 6 of the planes above and
// below) come from global memory, requested one colour phase ahead.
#pragma once
#include "mmh_kernels.cuh"

namespace mmh {
namespace gsf {

// Tile of TX x TY cells (QX x QY quads).  Staged region: quads a in
// [-2, QX+2), b in [-3, QY+3) (cells x in [-4, TX+4), y in [-6, TY+6)).
constexpr int TX = 64, TY = 32, QX = TX / 2, QY = TY / 2;
constexpr int AL = 2, BL = 3;                       // staged quads left of / below the tile
constexpr int LW = QX + 2 * AL, LH = QY + 2 * BL;   // staged region in quads
constexpr int NQ = LW * LH;                         // quads per staged plane
constexpr int FP = 4 * NQ;                          // words of one staged field-plane
constexpr int NPHI = 4;                             // phi ring: planes k-2 .. k+1
constexpr int NCOEF = 5;                            // coefficients 1-5 of the plane being updated
constexpr int SMEM_WORDS = (NPHI + NCOEF) * FP;     // 111.4 KB: two CTAs per SM
constexpr int NT = 384;                             // threads per CTA (two CTAs: 768 per SM)
constexpr int NW = NT / 32;

// Quad ranges updated by each colour phase, relative to the tile.  Derived by
// following the dependencies of the interior cells of both planes back
// through the 8-colour order (a cell of colour c reads its in-plane
// neighbours of lower colour new and of higher colour old, an even plane
// reads the odd planes old and an odd plane the even planes new):
//   even plane, cells (x range; y range) relative to the tile:
//     colour 0 [-2, TX+3) x [-4, TY+5), 1 [-2, TX+3) x [-3, TY+4),
//     colour 2 [-1, TX+2) x [-2, TY+3), 3 [-1, TX+2) x [-1, TY+2);
//   odd plane: colour 0 [0, TX+1) x [-2, TY+3), 1 [0, TX+1) x [-1, TY+2),
//     colour 2 [1, TX) x [0, TY+1), 3 the interior;
// everything they read (old values) lies in x [-3, TX+4), y [-5, TY+6).
template <bool EVEN, int Q> struct Range;
template <> struct Range<true, 0> { static constexpr int a0 = -1, a1 = QX + 2, b0 = -2, b1 = QY + 3; };
template <> struct Range<true, 1> { static constexpr int a0 = -1, a1 = QX + 2, b0 = -2, b1 = QY + 2; };
template <> struct Range<true, 2> { static constexpr int a0 = -1, a1 = QX + 1, b0 = -1, b1 = QY + 2; };
template <> struct Range<true, 3> { static constexpr int a0 = -1, a1 = QX + 1, b0 = -1, b1 = QY + 1; };
template <> struct Range<false, 0> { static constexpr int a0 = 0, a1 = QX + 1, b0 = -1, b1 = QY + 2; };
template <> struct Range<false, 1> { static constexpr int a0 = 0, a1 = QX + 1, b0 = -1, b1 = QY + 1; };
template <> struct Range<false, 2> { static constexpr int a0 = 0, a1 = QX, b0 = 0, b1 = QY + 1; };
template <> struct Range<false, 3> { static constexpr int a0 = 0, a1 = QX, b0 = 0, b1 = QY; };
constexpr int NPER = ((QX + 3) * (QY + 5) + NT - 1) / NT;  // quads per thread in the largest phase

__device__ __forceinline__ constexpr int qidx(int a, int b) { return (b + BL) * LW + (a + AL); }

// cp.async of 4 bytes (staging into the colour sub-planes)
__device__ __forceinline__ void cp_async4(unsigned sdst, const float* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sdst), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Stage the cells of rows [yc0, yc1) x columns [xc0, xc1) of the staged region
// (cell coordinates relative to its corner, x = -4 + xc, y = -6 + yc) of NF
// field-planes (n^3 words apart) of plane z into dst (NF buffers FP words
// apart).  Each warp takes whole rows; lane l copies columns l, l+32, ... so
// a warp reads 128 consecutive bytes per copy and the even and odd cells of a
// row land in sub-planes 2 NQ words apart (NQ = 8 mod 16: other banks).
template <int NF, int XC0, int XC1, int YC0, int YC1>
__device__ __forceinline__ void stage(float* dst, const float* __restrict__ base, i64 n3, int n, int ti0, int tj0,
                                      int z) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned sbase = (unsigned)__cvta_generic_to_shared(dst);
  const float* zb = base + (i64)n * n * z;
  constexpr int NX = (XC1 - XC0 + 31) / 32;
#pragma unroll 1
  for (int yc = YC0 + warp; yc < YC1; yc += NW) {
    int gj = tj0 - 2 * BL + yc;
    gj += gj < 0 ? n : (gj >= n ? -n : 0);
    const float* row = zb + (i64)n * gj;
    const int jo = yc & 1, qrow = (yc >> 1) * LW;
#pragma unroll
    for (int u = 0; u < NX; ++u) {
      const int xc = XC0 + lane + 32 * u;
      if (xc < XC1) {
        int gi = ti0 - 2 * AL + xc;
        gi += gi < 0 ? n : (gi >= n ? -n : 0);
        const int w = (2 * (xc & 1) + jo) * NQ + qrow + (xc >> 1);
#pragma unroll
        for (int f = 0; f < NF; ++f) cp_async4(sbase + 4u * (unsigned)(w + f * FP), row + gi + f * n3);
      }
    }
  }
}
// the whole staged region, and the part an odd plane's coefficients need
// (its updated cells and their in-plane neighbours: x in [-1, TX+2),
// y in [-3, TY+4), i.e. quads a in [-1, QX+1), b in [-2, QY+2))
template <int NF>
__device__ __forceinline__ void stage_all(float* dst, const float* base, i64 n3, int n, int ti0, int tj0, int z) {
  stage<NF, 0, 2 * LW, 0, 2 * LH>(dst, base, n3, n, ti0, tj0, z);
}
__device__ __forceinline__ void stage_odd_coef(float* dst, const float* base, i64 n3, int n, int ti0, int tj0, int z) {
  stage<NCOEF, 2, 2 * LW - 2, 2, 2 * LH - 2>(dst, base, n3, n, ti0, tj0, z);
}

// Word offset of the neighbour (dx, dy) of a cell of colour (io, jo),
// relative to the cell's own word: its colour sub-plane and quad.
template <int IO, int JO, int DX, int DY>
__device__ __forceinline__ constexpr int nb() {
  constexpr int x = IO + DX, y = JO + DY;                 // in -1 .. 2
  constexpr int ia = x < 0 ? -1 : (x > 1 ? 1 : 0);        // quad step in x
  constexpr int jb = y < 0 ? -1 : (y > 1 ? 1 : 0);        // quad step in y
  constexpr int sio = x & 1, sjo = y & 1;
  return (2 * sio + sjo) * NQ + jb * LW + ia - (2 * IO + JO) * NQ;
}

// The cell-local fields of a thread's cells in one colour phase: rhs, f6 of
// the plane, f6, f3, f5 of the planes below (m) and above (p).
struct Local {
  float r, f6c, f6m, f6p, f3m, f5m, f3p, f5p;
};

template <bool EVEN, int Q>
__device__ __forceinline__ void load_local(Local (&o)[NPER], const float* __restrict__ rhs,
                                           const float* __restrict__ coef, i64 n3, int n, int ti0, int tj0, int k,
                                           int km, int kp) {
  typedef Range<EVEN, Q> R;
  constexpr int W = R::a1 - R::a0, CNT = W * (R::b1 - R::b0);
  constexpr int IO = Q >> 1, JO = Q & 1;
  const i64 n2 = (i64)n * n;
#pragma unroll
  for (int p = 0; p < NPER; ++p) {
    const int e = threadIdx.x + p * NT;
    if (e < CNT) {
      const int a = R::a0 + e % W, b = R::b0 + e / W;
      int gi = ti0 + 2 * a + IO, gj = tj0 + 2 * b + JO;
      gi += gi < 0 ? n : (gi >= n ? -n : 0);
      gj += gj < 0 ? n : (gj >= n ? -n : 0);
      const i64 g = (i64)n * gj + gi;
      const float* pt = coef + (g + n2 * k);
      const float* pm = coef + (g + n2 * km);
      const float* pp = coef + (g + n2 * kp);
      o[p].r = __ldg(rhs + (g + n2 * k));
      o[p].f6c = __ldg(pt + 5 * n3);
      o[p].f6m = __ldg(pm + 5 * n3);
      o[p].f6p = __ldg(pp + 5 * n3);
      o[p].f3m = __ldg(pm + 2 * n3);
      o[p].f5m = __ldg(pm + 4 * n3);
      o[p].f3p = __ldg(pp + 2 * n3);
      o[p].f5p = __ldg(pp + 4 * n3);
    }
  }
}

// Update the cells of colour Q of the plane whose phi is P (in place).
// Km/Kp: phi of the planes below/above; C: staged coefficients 1-5.
template <bool EVEN, int Q>
__device__ __forceinline__ void colour_phase(float* __restrict__ P, const float* __restrict__ Km,
                                             const float* __restrict__ Kp, const float* __restrict__ C,
                                             const Local (&cur)[NPER], float dx2) {
  typedef Range<EVEN, Q> R;
  constexpr int W = R::a1 - R::a0, CNT = W * (R::b1 - R::b0);
  constexpr int IO = Q >> 1, JO = Q & 1;
  constexpr int S0 = (2 * IO + JO) * NQ;
  constexpr int xp = nb<IO, JO, 1, 0>(), xm = nb<IO, JO, -1, 0>(), yp = nb<IO, JO, 0, 1>(), ym = nb<IO, JO, 0, -1>();
  constexpr int pp = nb<IO, JO, 1, 1>(), mp = nb<IO, JO, -1, 1>(), pm = nb<IO, JO, 1, -1>(), mm = nb<IO, JO, -1, -1>();
  const float* F1 = C;
  const float* F2 = C + FP;
  const float* F3 = C + 2 * FP;
  const float* F4 = C + 3 * FP;
  const float* F5 = C + 4 * FP;
#pragma unroll
  for (int p = 0; p < NPER; ++p) {
    const int e = threadIdx.x + p * NT;
    if (e < CNT) {
      const int c = S0 + qidx(R::a0 + e % W, R::b0 + e / W);
      Stencil<float> st;
      st.c = 0.f;  // the update does not read the cell's own value
      st.f6c = cur[p].f6c; st.f6km = cur[p].f6m; st.f6kp = cur[p].f6p;
      st.f3km = cur[p].f3m; st.f5km = cur[p].f5m; st.f3kp = cur[p].f3p; st.f5kp = cur[p].f5p;
      st.ip = P[c + xp]; st.im = P[c + xm]; st.jp = P[c + yp]; st.jm = P[c + ym];
      st.kp = Kp[c]; st.km = Km[c];
      st.ppk = P[c + pp]; st.mpk = P[c + mp]; st.pmk = P[c + pm]; st.mmk = P[c + mm];
      st.jpkp = Kp[c + yp]; st.jmkp = Kp[c + ym]; st.jpkm = Km[c + yp]; st.jmkm = Km[c + ym];
      st.ipkp = Kp[c + xp]; st.imkp = Kp[c + xm]; st.ipkm = Km[c + xp]; st.imkm = Km[c + xm];
      st.f1c = F1[c]; st.f1ip = F1[c + xp]; st.f1im = F1[c + xm];
      st.f4c = F4[c]; st.f4jp = F4[c + yp]; st.f4jm = F4[c + ym];
      st.f2jp = F2[c + yp]; st.f2jm = F2[c + ym]; st.f2ip = F2[c + xp]; st.f2im = F2[c + xm];
      st.f5jp = F5[c + yp]; st.f5jm = F5[c + ym];
      st.f3ip = F3[c + xp]; st.f3im = F3[c + xm];
      float tdiag, t1, t2;
      op_eval(st, tdiag, t1, t2);
      // the smoother of the mixed form is not bit-matched: a fast division
      P[c] = __fdividef(cur[p].r * dx2 - t1 - t2, tdiag);
    }
  }
}

// write the tile's interior of the staged plane P to plane z of dst
__device__ __forceinline__ void write_plane(const float* P, float* __restrict__ dst, int n, int ti0, int tj0, int z) {
  const i64 zoff = (i64)n * n * z;
#pragma unroll
  for (int p = 0; p < (QX * QY + NT - 1) / NT; ++p) {
    const int e = threadIdx.x + p * NT;
    if (e < QX * QY) {
      const int a = e % QX, b = e / QX;
      const int r = qidx(a, b);
      const i64 g0 = zoff + (i64)n * (tj0 + 2 * b) + (ti0 + 2 * a);
      *reinterpret_cast<float2*>(dst + g0) = make_float2(P[0 * NQ + r], P[2 * NQ + r]);
      *reinterpret_cast<float2*>(dst + g0 + n) = make_float2(P[1 * NQ + r], P[3 * NQ + r]);
    }
  }
}

}  // namespace gsf

// One 8-colour sweep of src into dst (src != dst), grid (n/TX, n/TY, n/S):
// CTA (x, y, s) owns the tile's planes [s*S, s*S+S).  n >= 64, S even, n % S == 0.
// Per step t (even plane k = z0 + 2t): stage phi of k and k+1 (into the ring
// slots of the dead planes k-4, k-3) and coefficients of k, update plane k
// (phase A), stage coefficients of k-1, update plane k-1 (phase B).  The cell-local fields of each colour phase are requested
// during the one before it.
__global__ void __launch_bounds__(gsf::NT, 2) k_gs_sweep(const float* __restrict__ src, float* __restrict__ dst,
                                                         const float* __restrict__ rhs,
                                                         const float* __restrict__ coef, int n, float dx2, int S) {
  using namespace gsf;
  extern __shared__ __align__(16) float smf[];
  float* ring = smf;            // NPHI field-planes of phi
  float* C = smf + NPHI * FP;   // coefficients 1-5 of the plane being updated
  const i64 n3 = (i64)n * n * n;
  const int ti0 = blockIdx.x * TX, tj0 = blockIdx.y * TY, z0 = blockIdx.z * S;
  auto wrapz = [n](int z) { return z < 0 ? z + n : (z >= n ? z - n : z); };
  auto slot = [&](int p) { return ring + ((p - z0 + 1) & 3) * FP; };  // p >= z0-1

  // phi of plane z0-1 (each step stages its planes k and k+1)
  stage_all<1>(slot(z0 - 1), src, n3, n, ti0, tj0, wrapz(z0 - 1));
  Local cur[NPER], nxt[NPER];
  load_local<true, 0>(nxt, rhs, coef, n3, n, ti0, tj0, z0, wrapz(z0 - 1), wrapz(z0 + 1));

  const int steps = S / 2;
#pragma unroll 1
  for (int t = 0; t <= steps; ++t) {
    const int k = z0 + 2 * t;  // even plane of this step (unwrapped)
    const int kw = wrapz(k), kmw = wrapz(k - 1), kpw = wrapz(k + 1), km2 = wrapz(k - 2);
    stage_all<1>(slot(k), src, n3, n, ti0, tj0, kw);
    stage_all<1>(slot(k + 1), src, n3, n, ti0, tj0, kpw);
    stage_all<NCOEF>(C, coef, n3, n, ti0, tj0, kw);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    // ---- phase A: even plane k ----
    {
      float* P = slot(k);
      const float* Km = slot(k - 1);
      const float* Kp = slot(k + 1);
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      load_local<true, 1>(nxt, rhs, coef, n3, n, ti0, tj0, kw, kmw, kpw);
      gsf::colour_phase<true, 0>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      load_local<true, 2>(nxt, rhs, coef, n3, n, ti0, tj0, kw, kmw, kpw);
      gsf::colour_phase<true, 1>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      load_local<true, 3>(nxt, rhs, coef, n3, n, ti0, tj0, kw, kmw, kpw);
      gsf::colour_phase<true, 2>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      if (t >= 1) load_local<false, 0>(nxt, rhs, coef, n3, n, ti0, tj0, kmw, km2, kw);
      gsf::colour_phase<true, 3>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
      if (t < steps) write_plane(P, dst, n, ti0, tj0, kw);
    }
    if (t >= 1) {
      // ---- phase B: odd plane k-1 ----
      stage_odd_coef(C, coef, n3, n, ti0, tj0, kmw);
      cp_async_commit();
      cp_async_wait_all();
      __syncthreads();
      float* P = slot(k - 1);
      const float* Km = slot(k - 2);
      const float* Kp = slot(k);
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      load_local<false, 1>(nxt, rhs, coef, n3, n, ti0, tj0, kmw, km2, kw);
      gsf::colour_phase<false, 0>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      load_local<false, 2>(nxt, rhs, coef, n3, n, ti0, tj0, kmw, km2, kw);
      gsf::colour_phase<false, 1>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      load_local<false, 3>(nxt, rhs, coef, n3, n, ti0, tj0, kmw, km2, kw);
      gsf::colour_phase<false, 2>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
#pragma unroll
      for (int p = 0; p < NPER; ++p) cur[p] = nxt[p];
      if (t < steps) load_local<true, 0>(nxt, rhs, coef, n3, n, ti0, tj0, wrapz(k + 2), kpw, wrapz(k + 3));
      gsf::colour_phase<false, 3>(P, Km, Kp, C, cur, dx2);
      __syncthreads();
      write_plane(P, dst, n, ti0, tj0, kmw);
    } else {
      // step 0 has no odd plane: request the next step's first colour
      load_local<true, 0>(nxt, rhs, coef, n3, n, ti0, tj0, wrapz(k + 2), kpw, wrapz(k + 3));
    }
    // the ring slots of k-2, k-1 (dead now) and C are restaged by the next step
    __syncthreads();
  }
}

}  // namespace mmh
