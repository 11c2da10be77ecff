// Internal declarations shared by the MMH CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace mmh {

typedef long long i64;

// Count of kernel launches issued by this library (reported by bench.py).
void count_launch(int k = 1);
unsigned long long launch_count();

// Kernel timing hooks: when profiling is armed for `kind`, the launcher
// brackets each launch of that kernel with CUDA events on its stream.
enum KernelKind {
  KK_GS = 1, KK_RESIDUAL = 2, KK_RESTRICT_RESID = 3, KK_METRIC = 4, KK_SMOOTH = 5, KK_PROLONG = 6,
  KK_RESTRICT = 7, KK_LIMITER = 8, KK_RELAXING = 9, KK_SPECTRAL = 10, KK_APPLY = 11, KK_F32 = 256
};
void prof_begin(int kind, cudaStream_t s, i64 cells, int n);
void prof_end(int kind, cudaStream_t s, int n);
int prof_start(int kind);
bool prof_armed();  // timing hooks armed: launches must stay individual (no graph replay)
int prof_stop(int* launches, double* ms, long long* cells);
template <class T> inline int kk(int base) { return base | (sizeof(T) == 4 ? KK_F32 : 0); }

// Launchers, instantiated for double (mmh_kernels_f64.cu, no FMA contraction)
// and float (mmh_kernels_f32.cu).
// fast_div: one division per cell (the mixed form); false: the reference's
// operations, bit for bit
template <class T>
void launch_metric(const T* def, const T* rho, int n, T dx, T* coef, cudaStream_t s, bool fast_div = false);
void launch_residual_fma(const double* phi, const double* rhs, const double* coef, int n, double dx, float* r32,
                         unsigned long long* maxbits, cudaStream_t s);
template <class T> void launch_gs_sweeps(T* phi, const T* rhs, const T* coef, int n, T dx, int nsweeps, T* scratch, cudaStream_t s,
                                          bool zero_init = false);
// FP32 plane-kernel tile autotuning: the shape pinned for every grid (-1:
// timed per grid size and device), and the shape chosen for n (-1: none yet)
constexpr int kGsShapes = 6;
extern std::atomic<int> gs_tile_override;
// FP32 residual/operator stencil: -1 default (marching from 64^3 up), 0 one
// plane per CTA, 1 marching
extern std::atomic<int> stencil_march_pin;
int gs_tile_chosen(int n, int* tx, int* ty);
template <class T>
void launch_residual(const T* phi, const T* rhs, const T* coef, int n, T dx, T* r, float* r32,
                     unsigned long long* maxbits, cudaStream_t s);
template <class T> void launch_restrict_resid(const T* r, int n, int special, T* coarse, cudaStream_t s);
template <class T> void launch_restrict27(const T* fine, int n, T* coarse, cudaStream_t s);
template <class T> void launch_smooth27(const T* in, int n, T* out, cudaStream_t s);
template <class T> void launch_prolong_add(T* u, const T* uh, int n, cudaStream_t s);
template <class T> void launch_fxsum(const T* a, i64 count, unsigned long long* acc, int* flag, cudaStream_t s);
template <class T> void launch_det(const T* def, int n, T dx, T* det, cudaStream_t s);
template <class T> void launch_sub_mean(T* a, i64 count, const double* mean, cudaStream_t s);
template <class T> void launch_sub_dfact(T* a, const T* det, i64 count, const double* ratio, cudaStream_t s);
template <class T> void launch_fill(T* a, i64 count, T v, cudaStream_t s);
template <class T> void launch_absmax(const T* a, i64 count, unsigned long long* maxbits, cudaStream_t s);
// divergence guard: flag = relaxerr > r1*margin && r1 > floor (bits are maxbits words)
void launch_guard(const unsigned long long* r1bits, const unsigned long long* errbits, double margin, double floor_,
                  int* flag, int* guards, cudaStream_t s);
template <class T> void launch_zero_if(T* a, i64 count, const int* flag, cudaStream_t s);
template <class T> void launch_sub_mean_unless(T* a, i64 count, const double* mean, const int* flag, cudaStream_t s);
// zerosum helpers: mean = fx(acc)/count ; usum flag = (T)fx(acc) > 1e-2
void launch_fx_mean(const unsigned long long* acc, double count, double* out, cudaStream_t s);
void launch_fx_ratio(const unsigned long long* num, const unsigned long long* den, double* out, cudaStream_t s);
template <class T> void launch_usum_flag(const unsigned long long* acc, int* flag, cudaStream_t s);

// precision conversion and updates
void launch_d2f(const double* a, float* b, i64 count, cudaStream_t s);
void launch_f2d(const float* a, double* b, i64 count, cudaStream_t s);
void launch_add_f2d(double* a, const float* b, i64 count, cudaStream_t s);
void launch_add(double* a, const double* b, i64 count, cudaStream_t s);  // a = a + b
// exact FP64 solve of the 4^3 level (mixed form): M (64 x 64) from the level's
// FP64 coefficients once per metric; z = M (r - mean r) per application
void launch_coarse_inverse(const double* coef, double dx, double* M, cudaStream_t s);
void launch_coarse_apply(const float* r, const double* M, float* z, cudaStream_t s);

// limiter / spectral / relaxing (FP64)
struct LimDev;
void launch_calcdefp_rhs(double* tmp, const double* rho, int n, double dtold, bool mixed, cudaStream_t s);
void launch_limiter_pass1(double* tmp, const double* def, const double* rho, int n, double dtold, double dtaumesh,
                          LimDev* st, uint8_t* maskx, uint8_t* maskc, cudaStream_t s);
// the mixed form's pass 1: the same decisions and fluxes, FP32 screening and
// FP64 only where a decision is close; detff = the float-float metric's det
// of the same def
void launch_limiter_pass1_mixed(double* tmp, const double* def, const double* rho, const double* detff, int n,
                                double dtold, double dtaumesh, LimDev* st, uint8_t* maskx, uint8_t* maskc,
                                cudaStream_t s);
void launch_limiter_mask(double* defplim, const double* def, const double* defp, int n, double dtold, LimDev* st,
                         uint8_t* mask, cudaStream_t s);
// the same outputs, FP32 screening and FP64 only for the cells that may matter
void launch_limiter_mask_mixed(double* defplim, const double* def, const double* defp, int n, double dtold, LimDev* st,
                               uint8_t* mask, cudaStream_t s);
void launch_lim_reset(LimDev* st, cudaStream_t s);
void launch_spec_tables(double* tab, int n, cudaStream_t s);
void launch_spec_pack(const void* Xc, int n, int mode, void* Z, const LimDev* st, const double* tab, cudaStream_t s);
void launch_spec_unpack(const void* z, int n, double* out, int stride_out, int add, const LimDev* st, cudaStream_t s);
void launch_relax_stage1(const double* rho, const double* def, const double* defp, int n, double* baj, double* cc,
                         double* sd, cudaStream_t s, bool fast_div = false);
void launch_relax_flux(const double* u1, const double* defp, const double* baj, const double* cc, int n, double* sd,
                       cudaStream_t s, bool fast_div = false);
void launch_relax_dpv(const double* sd, const double* cc, int n, const double* ubase, double dt, double* out,
                      double* gface, cudaStream_t s);
// the mixed form's relaxing of the density (mmh_relax32.cu): FP32 fluxes, FP64
// update; geo (n^3 float4), uf0, uf1 (n^3 floats) are scratch
void launch_relax32(double* rho, const double* def, const double* defp, int n, double dt, float4* geo, float* uf0,
                    float* uf1, cudaStream_t s);
// u(nf,n^3) (float or double) <-> density; flag |= 1 when a component 2..nf is not zero
void launch_extract_density_f(const float* u, int nf, i64 n3, double* rho, int* flag, cudaStream_t s);
void launch_extract_density_d(const double* u, int nf, i64 n3, double* rho, int* flag, cudaStream_t s);

// flexible PCG scalars and accumulators (device)
struct PcgDev {
  unsigned long long acc[3][2];
  unsigned long long rbits, zbits, pbits, qbits;
  double rz, pq, alpha, beta;
};
template <class T>
void launch_apply(const T* p, const T* coef, int n, T dx, T* q, unsigned long long* qbits, cudaStream_t s);
template <class T>
void launch_dot(const T* a, const T* b, i64 count, const unsigned long long* abits, const unsigned long long* bbits,
                unsigned long long* acc, cudaStream_t s);
template <class T>
void launch_pcg_update(T* x, T* r, const T* p, const T* q, i64 count, const double* alpha, unsigned long long* rbits,
                       cudaStream_t s);
template <class T>
void launch_pcg_pupdate(T* p, const T* z, i64 count, const double* beta, unsigned long long* pbits, cudaStream_t s);
void launch_pcg_scalar(PcgDev* st, int stage, cudaStream_t s);
// Fast deterministic FP32 dot product (mixed form's inner solve): kDotBlocks
// block sums in `part`, result into acc in the exact dot's fixed-point form.
constexpr int kDotBlocks = 152 * 8;
void launch_dot_fast(const float* a, const float* b, i64 count, const unsigned long long* abits,
                     const unsigned long long* bbits, unsigned long long* acc, double* part, cudaStream_t s);

// the mixed form's nsmooth: three axis passes, `in` overwritten
void launch_smooth_sep(double* in, int n, double* out, cudaStream_t s);

// float-float outer loop of the mixed form (mmh_kernels_f64.cu): a double
// buffer reinterpreted as (hi, lo) float pairs, in place
void launch_ff_split(double* a, i64 count, cudaStream_t s);
// r32 = b rounded through its float-float split (the outer residual of a
// zero guess), max |r32| into maxbits
void launch_ff_rhs32(const double* b, i64 count, float* r32, unsigned long long* maxbits, cudaStream_t s);
void launch_set_u64(unsigned long long* p, unsigned long long v, cudaStream_t s);
void launch_ff_join(double* a, i64 count, cudaStream_t s);
void launch_ff_add_f(double* x, const float* e, i64 count, cudaStream_t s);
void launch_ff_sub_mean(double* x, const double* mean, i64 count, cudaStream_t s);
void launch_residual_ff(const double* phi, const double* rhs, const double* coef, int n, double dx, float* r32,
                        unsigned long long* maxbits, cudaStream_t s);
// the finest level's metric straight into float-float pairs (coef, the layout
// launch_ff_split makes) and their hi parts (coef32, FP32); det (may be null)
// receives det(A) rounded to FP64
void launch_metric_ff(const double* def, const double* rho, int n, double dx, double* coef, float* coef32,
                      double* det, cudaStream_t s);

// main.f90's iteration diagnostics: exact sums (def, def^2, defp^2, rho,
// (rho-1)^2), ord_of-encoded extrema of rho, count of rho < 0, range flag
struct StatsDev {
  unsigned long long acc[5][2];
  unsigned long long rmin, rmax, nneg;
  int flag;
  int pad;
};
void launch_state_stats(const double* def, const double* defp, const double* rho, i64 n3, StatsDev* st,
                        cudaStream_t s);

// binned power spectrum accumulators (fixed-point sums of power and |k|, mode counts)
constexpr int kPowMaxBins = 128;
struct PowDev {
  unsigned long long p[kPowMaxBins][2], k[kPowMaxBins][2], cnt[kPowMaxBins];
  int flag;
  int pad;
};
void launch_power_bins(const void* A, const void* B, int n, int nb, const double* e2, double scale, PowDev* acc,
                       cudaStream_t s);

// calcdefp adjoint pieces (mmh_adjoint.cu)
void launch_adj_pass1(double* y, const double* t, const uint8_t* maskx, const uint8_t* maskc, double dtaumesh,
                      i64 n3, cudaStream_t s);
void launch_adj_rhs(double* y, const double* rho, double dtold, i64 n3, cudaStream_t s);
void launch_adj_contract(const double* lam, const double* u, const double* cf, int n, double* out, cudaStream_t s);
void launch_box27(const double* in, int n, double* out, cudaStream_t s);
void launch_adj_mul(const double* a, const double* b, double* out, i64 n3, cudaStream_t s);
void launch_adj_sub(const double* a, const double* b, double* out, i64 n3, cudaStream_t s);
void launch_adj_metric(const double* def, const double* lam, const double* u, const double* urg, const double* y,
                       const double* rptr, int n, double* abar, cudaStream_t s);
void launch_adj_hess(const double* abar, int n, double* out, int add, cudaStream_t s);
// the final compression test's correction: abar = dJ/dC on the limited cells
// (mask) for J = sum pw * defplim; out = a + s * b
void launch_adj_limiter(const double* def, const double* defps, const double* pw, const uint8_t* mask, int n,
                        double dtold, double* abar, cudaStream_t s);
void launch_adj_axpy(const double* a, double sc, const double* b, double* out, i64 n3, cudaStream_t s);
void launch_adj_alpha(const double* baj, const double* defp, const double* cc, int n, double* alpha, cudaStream_t s);
void launch_adj_dpv(const double* sd, const double* cc, const double* alpha, const double* x, const double* rbar,
                    double scale, int n, double* xbar, double* alphabar, double* cbar, cudaStream_t s);
void launch_adj_relax_geom(const double* def, const double* defp, const double* cc, const double* alphabar,
                           const double* cbar, int n, double* abar, double* pdbar, cudaStream_t s);
void launch_adj_grad_t(const double* pdbar, int n, double* out, int add, cudaStream_t s);

}  // namespace mmh
