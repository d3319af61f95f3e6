// Launchers of the inverse-loop kernels (inverse_kernels.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "osgpu_types.h"

namespace osgpu {

// Per-element dM/dphi accumulators of one element plane (null: skipped).
struct AdjGrads {
  void* p[kMaxElements];
};

// Adam step constants, computed on the host in the reference's order:
// step = lr_frac * (hi - lo), bc1 = 1 - beta1^t, bc2 = 1 - beta2^t.
struct AdamArgs {
  double beta1, beta2, eps, bc1, bc2, step, lo, hi, clip_norm;
  int clip;
};

// Device-resident state of one Gerchberg-Saxton run.
struct GsState {
  double best_merit;
  int best_it;   // -1 before the first iteration
  int improved;  // the current iteration improved on the best merit
  int stop;      // converged or iteration cap reached: later kernels return
  int converged;
  int iterations;
  int fault;     // a staged input of this item never arrived (bounded wait ran out)
};
// One history record (layout of osgpu_gs_record).
struct GsRecordDev {
  double iteration, merit, best_merit, amplitude_mse, target_error_rms, phase_update_rms;
};

// Per-item pointers of a batched fold (fused GS path).
struct GsFoldItem {
  const double* part_merit;   // 2 frames x nb compensated pairs
  const double* part_update;  // 1 frame x nb pairs
  GsState* state;
  GsRecordDev* hist;
};
cudaError_t launch_gs_fold_merit_batch(const GsFoldItem* items, int n_items, int nb, uint64_t n,
                                       int it, cudaStream_t st);
cudaError_t launch_gs_fold_update_batch(const GsFoldItem* items, int n_items, int nb, uint64_t n,
                                        int it, int patience, double tol, int max_it,
                                        cudaStream_t st);

cudaError_t launch_gs_init(const void* init, void* phase, int f64, double lo, double hi,
                           unsigned char* open, int stop, double a, double b, double cx,
                           double cy, int nx, int ny, double dx, double dy, cudaStream_t st);
cudaError_t launch_mask_amplitude(const void* illum, const unsigned char* open, void* out,
                                  int f64, uint64_t n, cudaStream_t st);
cudaError_t launch_abs(const void* u, int c128, void* out, int f64, int square, uint64_t n,
                       cudaStream_t st);
cudaError_t launch_gs_mask(const void* phase, int f64, const void* illum,
                           const unsigned char* open, void* mask, int c128, uint64_t n,
                           const GsState* state, cudaStream_t st);
// part: reduce_scratch_bytes(2)
cudaError_t launch_gs_project(const void* u, int c128, const void* tamp, const void* tint,
                              int f64, double beta_f, void* proj, uint64_t n, double* part,
                              void* err_out, GsState* state, GsRecordDev* hist, int it,
                              cudaStream_t st);
cudaError_t launch_gs_update(const void* v, int c128, void* phase, void* best, int f64,
                             double beta_p, double lo, double hi, uint64_t n, double* part,
                             void* dphi_out, GsState* state, GsRecordDev* hist, int it,
                             int patience, double tol, int max_it, cudaStream_t st);

// Sources (see inverse_kernels.cu).
cudaError_t launch_gaussian(void* out, int c128, int nx, int ny, double dx, double dy, double cx,
                            double cy, double amp, double w2, double half_k, double inv_r,
                            double carrier, cudaStream_t st);
cudaError_t launch_plane_wave(void* out, int c128, int nx, int ny, double dx, double dy,
                              double amp, double k, double alpha, double beta, cudaStream_t st);
cudaError_t launch_fill(void* out, int c128, size_t n, double re, double im, cudaStream_t st);

cudaError_t launch_apply_intensity(const void* in, int in_c128, void* out, int out_c128,
                                   const ElementList& els, int nx, int ny, double dx, double dy,
                                   void* inten, int inten_f64, int f32, cudaStream_t st);
cudaError_t launch_adjoint_seed_plane(const void* uin, int uin_c128, const ElementList& els,
                                      const AdjGrads& grads, const void* seed, int seed_f64,
                                      double scale, int nx, int ny, double dx, double dy,
                                      void* mu_out, int mu_c128, int f32, cudaStream_t st);
// dst[k] += src[k] over n real values (f64 or f32)
cudaError_t launch_add_real(void* dst, const void* src, int f64, uint64_t n, cudaStream_t st);
// Scratch (device) needed by the reductions below for n_frames frames.
size_t reduce_scratch_bytes(int n_frames);
// out[f] = sum over win of frame f (f = 0..nf-1)
cudaError_t launch_window_sums(const void* obs, int f64, int nf, uint64_t len,
                               const unsigned char* win, double* scratch, double* out,
                               cudaStream_t st);
cudaError_t launch_window_seed(void* seed, int f64, int nf, uint64_t len,
                               const unsigned char* win, const double* coef, cudaStream_t st);
// out[f] = sum_k w[k] I_f[k]; w has the observation's real dtype
cudaError_t launch_weighted_sums(const void* obs, int f64, int nf, uint64_t len, const void* w,
                                 double* scratch, double* out, cudaStream_t st);
// seed_f[k] = coef[f] w[k]
cudaError_t launch_weighted_seed(void* seed, int f64, int nf, uint64_t len, const void* w,
                                 const double* coef, cudaStream_t st);
// out[0] = sum (selected frame - target)^2; seed (optional) per frame
cudaError_t launch_mse(const void* obs, int f64, uint64_t len, int nb, int ns, int band,
                       int scene, const double* target, void* seed, double* scratch,
                       double* out, cudaStream_t st);
// out[0] = total, out[1] = inside; seed (optional) per frame
cudaError_t launch_ee(const void* obs, int f64, int nx, int ny, double dx, double dy,
                      double radius, int nb, int ns, int band, int scene, void* seed,
                      double* scratch, double* out, cudaStream_t st);
// the selected frame of an observation summed in FP64 (Selector::frame)
cudaError_t launch_sel_frame(const void* obs, int f64, uint64_t len, int nb, int ns, int band,
                             int scene, double* out, cudaStream_t st);
// spot-RMS merit seed on every (band, scene) frame: selected ones get
// (rho^2 - rr) / denom, the others 0
cudaError_t launch_spot_seed(void* seed, int f64, int nx, int ny, double dx, double dy, int nb,
                             int ns, int band, int scene, double rr, double denom,
                             cudaStream_t st);
// detector metrics (analysis.rs): out2 = {sum I, sum I rho^2}; out = max I;
// X[k] (k <= nx/2) = DFT of the column sums (tw64: FP64 nx-point twiddles)
cudaError_t launch_psf_moments(const void* img, int f64, int nx, int ny, double dx, double dy,
                               double* scratch, double* out2, cudaStream_t st);
// encircled-energy curve: perm = pixel order by radius, group_end = last
// index of each tied-radius group; v (n doubles) and tot (ceil(n/1024)) are
// scratch; frac[g] = cumulative power at group g / total (total_out, host;
// frac untouched when total <= 0).  Synchronises st.
cudaError_t launch_ee_curve(const void* img, int f64, const unsigned* perm, uint64_t n,
                            const unsigned* group_end, uint64_t ng, double* v, double* tot,
                            double* frac, double* total_out, cudaStream_t st);
cudaError_t launch_psf_max(const void* img, int f64, uint64_t n, double* scratch, double* out,
                           cudaStream_t st);
cudaError_t launch_row_mtf(const void* img, int f64, int nx, int ny, const void* tw64,
                           double* colsum, double2* X, cudaStream_t st);
cudaError_t launch_power(const void* u, int c128, uint64_t n, double* scratch, double* out,
                         cudaStream_t st);
cudaError_t launch_adam(double* x, float* x32, const void* g, int g_f64, double* m, double* v,
                        uint64_t n, const AdamArgs& p, double* scratch, double* norm2,
                        cudaStream_t st);

}  // namespace osgpu
