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
// planes [z0, z0+S) and keeps a ring of four planes of phi (k-2 .. k+1) and the
// coefficients of the plane being updated in shared memory; a plane's phi,
// rhs and six coefficients are read once per sweep and phi written once
// (9 words per cell; halos come from L2).
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
// shared memory holds every field in four colour sub-planes: cell (2a+io,
// 2b+jo) of the staged region sits at word (2*io+jo)*NQ + quad(a, b).  A
// colour phase then reads consecutive words across a warp (no bank
// conflicts), and each global row segment is loaded as 8-byte quad rows.
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
constexpr int NPHI = 6;                             // phi ring: planes k-2 .. k+3
constexpr int NCOEF = 5;                            // coefficients 1-5 of a plane
constexpr int SMEM_WORDS = (NPHI + 2 * NCOEF) * FP; // two coefficient buffers (even, odd plane)
constexpr int NT = 512;

// Quad ranges [a0, a1) x [b0, b1) updated by each colour phase, in quads
// relative to the tile.  Derived by following the dependencies of the
// interior cells of both planes back through the 8-colour order (a cell of
// colour c reads its in-plane neighbours of lower colour new and of higher
// colour old, an even plane reads the odd planes old and an odd plane the
// even planes new):
//   even plane, cells (x range; y range) relative to the tile:
//     colour 0 [-2, TX+3) x [-4, TY+5), 1 [-2, TX+3) x [-3, TY+4),
//     colour 2 [-1, TX+2) x [-2, TY+3), 3 [-1, TX+2) x [-1, TY+2);
//   odd plane: colour 0 [0, TX+1) x [-2, TY+3), 1 [0, TX+1) x [-1, TY+2),
//     colour 2 [1, TX) x [0, TY+1), 3 the interior;
// everything they read (old values) lies in x [-3, TX+4), y [-5, TY+6).
struct QRange { int a0, a1, b0, b1; };
__device__ __forceinline__ constexpr QRange even_range(int q) {
  return q == 0 ? QRange{-1, QX + 2, -2, QY + 3}
       : q == 1 ? QRange{-1, QX + 2, -2, QY + 2}
       : q == 2 ? QRange{-1, QX + 1, -1, QY + 2}
                : QRange{-1, QX + 1, -1, QY + 1};
}
__device__ __forceinline__ constexpr QRange odd_range(int q) {
  return q == 0 ? QRange{0, QX + 1, -1, QY + 2}
       : q == 1 ? QRange{0, QX + 1, -1, QY + 1}
       : q == 2 ? QRange{0, QX, 0, QY + 1}
                : QRange{0, QX, 0, QY};
}
// The coefficients of an odd plane are staged for its updated cells and
// their in-plane neighbours only: x in [-1, TX+2), y in [-3, TY+4).

__device__ __forceinline__ int qidx(int a, int b) { return (b + BL) * LW + (a + AL); }

// Asynchronous staging (cp.async, 4 bytes per copy): every cell of the quad
// range R of NF consecutive field-planes (n^3 words apart from `base`) of
// plane z goes straight to its colour sub-plane in dst (NF buffers FP words
// apart).  Consecutive threads copy consecutive cells of a row: the global
// reads coalesce, and the even and odd cells of a row land in sub-planes
// 2 NQ words apart (NQ = 8 mod 16: different banks).
__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int NF, int A0, int A1, int B0, int B1>
__device__ __forceinline__ void stage_async(float* dst, const float* __restrict__ base, i64 n3, int n, int ti0,
                                            int tj0, int z) {
  constexpr int WC = 2 * (A1 - A0), CNT = WC * 2 * (B1 - B0);
  const i64 zoff = (i64)n * n * z;
  for (int e = threadIdx.x; e < CNT; e += NT) {
    const int xc = e % WC, yc = e / WC;
    const int io = xc & 1, jo = yc & 1;
    const int r = qidx(A0 + (xc >> 1), B0 + (yc >> 1));
    int gi = ti0 + 2 * A0 + xc, gj = tj0 + 2 * B0 + yc;
    gi += gi < 0 ? n : (gi >= n ? -n : 0);
    gj += gj < 0 ? n : (gj >= n ? -n : 0);
    const float* g = base + zoff + (i64)n * gj + gi;
    float* d = dst + (2 * io + jo) * NQ + r;
#pragma unroll
    for (int f = 0; f < NF; ++f) cp_async4(d + f * FP, g + f * n3);
  }
}
// whole staged region / the odd plane's coefficient region
template <int NF>
__device__ __forceinline__ void stage_all(float* dst, const float* base, i64 n3, int n, int ti0, int tj0, int z) {
  stage_async<NF, -AL, QX + AL, -BL, QY + BL>(dst, base, n3, n, ti0, tj0, z);
}
__device__ __forceinline__ void stage_odd_coef(float* dst, const float* base, i64 n3, int n, int ti0, int tj0,
                                               int z) {
  stage_async<NCOEF, -1, QX + 1, -2, QY + 2>(dst, base, n3, n, ti0, tj0, z);
}

// Word offset, within a field-plane, of the neighbour (dx, dy) of a cell of
// colour (io, jo) in quad r: its colour sub-plane and quad.
template <int IO, int JO, int DX, int DY>
__device__ __forceinline__ constexpr int nb() {
  constexpr int x = IO + DX, y = JO + DY;                 // in -1 .. 2
  constexpr int ia = x < 0 ? -1 : (x > 1 ? 1 : 0);        // quad step in x
  constexpr int jb = y < 0 ? -1 : (y > 1 ? 1 : 0);        // quad step in y
  constexpr int sio = x & 1, sjo = y & 1;
  return (2 * sio + sjo) * NQ + jb * LW + ia;
}

// Update the cells of colour (IO, JO) of the plane whose phi is P (in place)
// over the quad range R.  Km/Kp: phi of the planes below/above; C: staged
// coefficients 1-5 of the plane.  Cell-local fields come from global memory.
template <int IO, int JO>
__device__ __forceinline__ void colour_phase(float* __restrict__ P, const float* __restrict__ Km,
                                             const float* __restrict__ Kp, const float* __restrict__ C,
                                             const float* __restrict__ rhs, const float* __restrict__ coef, i64 n3,
                                             int n, int ti0, int tj0, int k, int km, int kp, float dx2, QRange R) {
  const int w = R.a1 - R.a0, cnt = w * (R.b1 - R.b0);
  constexpr int S0 = (2 * IO + JO) * NQ;
  const float* F1 = C;
  const float* F2 = C + FP;
  const float* F3 = C + 2 * FP;
  const float* F4 = C + 3 * FP;
  const float* F5 = C + 4 * FP;
  const float* f3 = coef + 2 * n3;
  const float* f5 = coef + 4 * n3;
  const float* f6 = coef + 5 * n3;
  const i64 n2 = (i64)n * n;
  for (int e = threadIdx.x; e < cnt; e += NT) {
    const int a = R.a0 + e % w, b = R.b0 + e / w;
    const int r = qidx(a, b);
    int gi = ti0 + 2 * a + IO, gj = tj0 + 2 * b + JO;
    gi += gi < 0 ? n : (gi >= n ? -n : 0);
    gj += gj < 0 ? n : (gj >= n ? -n : 0);
    const i64 g = (i64)n * gj + gi;
    const i64 gt = g + n2 * k, gm = g + n2 * km, gp = g + n2 * kp;
    const float rr = __ldg(rhs + gt);
    Stencil<float> st;
    st.f6c = __ldg(f6 + gt); st.f6km = __ldg(f6 + gm); st.f6kp = __ldg(f6 + gp);
    st.f3km = __ldg(f3 + gm); st.f5km = __ldg(f5 + gm); st.f3kp = __ldg(f3 + gp); st.f5kp = __ldg(f5 + gp);
    const int c = S0 + r;
    constexpr int xp = nb<IO, JO, 1, 0>() - (2 * IO + JO) * NQ, xm = nb<IO, JO, -1, 0>() - (2 * IO + JO) * NQ;
    constexpr int yp = nb<IO, JO, 0, 1>() - (2 * IO + JO) * NQ, ym = nb<IO, JO, 0, -1>() - (2 * IO + JO) * NQ;
    constexpr int pp = nb<IO, JO, 1, 1>() - (2 * IO + JO) * NQ, mp = nb<IO, JO, -1, 1>() - (2 * IO + JO) * NQ;
    constexpr int pm = nb<IO, JO, 1, -1>() - (2 * IO + JO) * NQ, mm = nb<IO, JO, -1, -1>() - (2 * IO + JO) * NQ;
    st.c = 0.f;  // the update does not read the cell's own value
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
    P[c] = (rr * dx2 - t1 - t2) / tdiag;
  }
}

// all four in-plane colours of one plane, in the reference's order (io
// outer, jo inner), with a barrier between colours
template <bool EVEN>
__device__ __forceinline__ void plane_update(float* P, const float* Km, const float* Kp, const float* C,
                                             const float* rhs, const float* coef, i64 n3, int n, int ti0, int tj0,
                                             int k, int km, int kp, float dx2) {
  colour_phase<0, 0>(P, Km, Kp, C, rhs, coef, n3, n, ti0, tj0, k, km, kp, dx2, EVEN ? even_range(0) : odd_range(0));
  __syncthreads();
  colour_phase<0, 1>(P, Km, Kp, C, rhs, coef, n3, n, ti0, tj0, k, km, kp, dx2, EVEN ? even_range(1) : odd_range(1));
  __syncthreads();
  colour_phase<1, 0>(P, Km, Kp, C, rhs, coef, n3, n, ti0, tj0, k, km, kp, dx2, EVEN ? even_range(2) : odd_range(2));
  __syncthreads();
  colour_phase<1, 1>(P, Km, Kp, C, rhs, coef, n3, n, ti0, tj0, k, km, kp, dx2, EVEN ? even_range(3) : odd_range(3));
  __syncthreads();
}

// write the tile's interior of the staged plane P to plane z of dst
__device__ __forceinline__ void write_plane(const float* P, float* __restrict__ dst, int n, int ti0, int tj0, int z) {
  const i64 zoff = (i64)n * n * z;
  for (int e = threadIdx.x; e < QX * QY; e += NT) {
    const int a = e % QX, b = e / QX;
    const int r = qidx(a, b);
    const i64 g0 = zoff + (i64)n * (tj0 + 2 * b) + (ti0 + 2 * a);
    *reinterpret_cast<float2*>(dst + g0) = make_float2(P[0 * NQ + r], P[2 * NQ + r]);
    *reinterpret_cast<float2*>(dst + g0 + n) = make_float2(P[1 * NQ + r], P[3 * NQ + r]);
  }
}

}  // namespace gsf

// One 8-colour sweep of src into dst (src != dst), grid (n/TX, n/TY, n/S):
// CTA (x, y, s) owns the tile's planes [s*S, s*S+S).  n >= 64, S even, n % S == 0.
// Per step t (even plane k = z0 + 2t): phase A updates plane k, phase B the
// odd plane k-1; the copies for the next planes run behind the arithmetic:
//   step start : phi of k+2, k+3 and coefficients of k-1 (odd buffer) issued
//   after A    : coefficients of k+2 issued into the even buffer
//   step end   : all copies waited for.
__global__ void __launch_bounds__(gsf::NT, 1) k_gs_sweep(const float* __restrict__ src, float* __restrict__ dst,
                                                         const float* __restrict__ rhs,
                                                         const float* __restrict__ coef, int n, float dx2, int S) {
  using namespace gsf;
  extern __shared__ __align__(16) float smf[];
  float* ring = smf;                           // NPHI field-planes of phi
  float* CE = smf + NPHI * FP;                 // coefficients 1-5 of the even plane
  float* CO = CE + NCOEF * FP;                 // coefficients 1-5 of the odd plane
  const i64 n3 = (i64)n * n * n;
  const int ti0 = blockIdx.x * TX, tj0 = blockIdx.y * TY, z0 = blockIdx.z * S;
  auto wrapz = [n](int z) { return z < 0 ? z + n : (z >= n ? z - n : z); };
  auto slot = [&](int p) { return ring + ((p - z0 + 1) % NPHI) * FP; };  // p >= z0-1

  // prologue: phi of planes z0-1 .. z0+1 and coefficients 1-5 of z0
  for (int d = -1; d <= 1; ++d) stage_all<1>(slot(z0 + d), src, n3, n, ti0, tj0, wrapz(z0 + d));
  stage_all<NCOEF>(CE, coef, n3, n, ti0, tj0, z0);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();

  const int steps = S / 2;
  for (int t = 0; t <= steps; ++t) {
    const int k = z0 + 2 * t;  // even plane of this step (unwrapped)
    if (t < steps) {
      stage_all<1>(slot(k + 2), src, n3, n, ti0, tj0, wrapz(k + 2));
      stage_all<1>(slot(k + 3), src, n3, n, ti0, tj0, wrapz(k + 3));
    }
    if (t >= 1) stage_odd_coef(CO, coef, n3, n, ti0, tj0, wrapz(k - 1));
    cp_async_commit();
    // ---- phase A: even plane k ----
    plane_update<true>(slot(k), slot(k - 1), slot(k + 1), CE, rhs, coef, n3, n, ti0, tj0, wrapz(k), wrapz(k - 1),
                       wrapz(k + 1), dx2);
    if (t < steps) {
      write_plane(slot(k), dst, n, ti0, tj0, wrapz(k));
      stage_all<NCOEF>(CE, coef, n3, n, ti0, tj0, wrapz(k + 2));
    }
    cp_async_commit();
    if (t >= 1) {
      // ---- phase B: odd plane k-1 (its coefficients are the older group) ----
      cp_async_wait<1>();
      __syncthreads();
      plane_update<false>(slot(k - 1), slot(k - 2), slot(k), CO, rhs, coef, n3, n, ti0, tj0, wrapz(k - 1),
                          wrapz(k - 2), wrapz(k), dx2);
      write_plane(slot(k - 1), dst, n, ti0, tj0, wrapz(k - 1));
    }
    cp_async_wait<0>();
    __syncthreads();
  }
}

}  // namespace mmh
