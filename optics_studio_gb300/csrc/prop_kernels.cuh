// Kernel argument blocks and host launchers for the propagation passes.
#pragma once
#include <cuda_runtime.h>
#include "osgpu_types.h"

namespace osgpu {

// Everything the three propagation passes need for one propagation.
// Pointers are device pointers.  `T` is the arithmetic type (float/double);
// complex buffers are float2/double2 (input/output may be complex128 while
// the engine computes in f32: see in_c128/out_c128).
// Kernel variants of the f32 register-FFT passes.  Every variant of a pass
// computes the same transform; the schedule names one per pass (0: the
// built-in default).  Environment overrides OSGPU_SCHED_A / _B / _C (variant
// names below) take precedence; an ineligible choice falls back to the default.
enum { SA_DEFAULT = 0, SA_BULK, SA_TILE4, SA_TILE2, SA_G1, SA_G2, SA_G4, SA_TSTORE, SA_N };
enum { SB_DEFAULT = 0, SB_PAIR, SB_G1, SB_G2, SB_G4, SB_N };
enum { SC_DEFAULT = 0, SC_TMA, SC_PIPE, SC_TILE2, SC_TILE4, SC_G1, SC_G2, SC_G4, SC_N };
struct Schedule {
  int a, b, c;
};
// Variant names (index = enum value) of pass 0 (A), 1 (B), 2 (C).
const char* sched_name(int pass, int v);
int sched_count(int pass);

struct PropArgs {
  Schedule sched;  // host-side choice of pass variants (not read by kernels)
  int nx, ny;
  double dx, dy;
  AxisPlan ax, ay;
  const void* in;      // field in, row-major ny x nx
  int in_c128;
  void* out;           // field out, row-major ny x nx
  int out_c128;
  float* out_intensity;  // optional |u|^2 (f32) of the output, row-major
  double* out_intensity64;
  void* work;          // Px x ny spectrum scratch (column-major)
  const void* tw_mx;   // m-point twiddles (x)
  const void* tw_Px;   // P-point twiddles (x), used when r > 1
  const void* tw_my;
  const void* tw_Py;
  ElementList els;
  // transfer function
  int engine;
  int h_mode;          // 0 exact per-bin FP64, 1 f32 split tables
  double lam, lam_n, z, kz;   // kz = (2 pi / lam_n) * z  (ASM) or (2 pi/lam)*z (Fresnel)
  double cfr;          // Fresnel: (pi * lam) * z
  int band_limited;
  double lim_x, lim_y;
  double scale;        // 1 / (Px * Py)
  int conj_h;          // 1: use conj(H) (adjoint of a kernel-spectrum engine)
  // per-axis tables produced by the prep kernel
  const double* fxv;   // fftfreq(Px, dx)
  const double* fyv;   // fftfreq(Py, dy)
  const float2* Ex;    // f32 split: per-column factor (includes e^{i kz} and scale)
  const float2* Ey;    // per-row factor
  const float* ca_hi;  // -kz a/4 (double-float)
  const float* ca_lo;
  const float* sa;     // a = (lam_n fx)^2
  const float* b_hi;   // b = (lam_n fy)^2 (double-float)
  const float* b_lo;
  const int* kmax;     // per column: largest unmasked |k_y| (-1: column masked)
  const void* rowtab;  // f32 split: per row {Ey.x, Ey.y, b_hi, b_lo} packed (float4)
  float Kf;            // kz as f32 (for the small residual term)
  // kernel spectra
  const void* kspec;   // ENG_KSPEC: column-major Px x Py spectrum (type of engine);
                       // ENG_KEVEN: f32 quarter table K[kx (Py/2 + 1) + ky], kx <= Px/2,
                       // ky <= Py/2, of a spectrum even in both axes (scale folded in)
  const void* hx;      // ENG_KSEP: per-column spectrum factor (includes prefactor, scale)
  const void* hy;      // ENG_KSEP: per-row spectrum factor
  int* status;         // bit 0: non-finite input sample, bit 1: non-finite output
  // adjoint seed (pass A): each input sample is multiplied by the real weight
  // seed[k] * seed_scale (seed is float, or double when seed_f64)
  const void* seed;
  int seed_f64;
  double seed_scale;
  // adjoint element plane (pass C epilogue, see adjoint_plane in
  // elements.cuh): els is the element chain the plane crosses (pass A then
  // applies no elements), adj_uin the forward field that entered the chain,
  // adj_grad the per-element dM/dphi accumulators (null: skipped)
  int adj;
  const void* adj_uin;
  int adj_uin_c128;
  void* adj_grad[kMaxElements];
  // f32 engine: the element chain of els precomputed as one complex
  // transmission per sample (row-major ny x nx, launch_transmission); pass A
  // multiplies by it instead of evaluating the chain
  const float2* trans;
};

// Fraunhofer arguments (no padding; two passes).
struct FraunArgs {
  int nx, ny;
  double dx, dy;
  AxisPlan ax, ay;
  const void* in;
  int in_c128;
  void* out;
  int out_c128;
  float* out_intensity;
  void* work;
  const void* tw_mx;
  const void* tw_my;
  ElementList els;
  double lam, z, k;
  double xs, ys, f_s, g_s;
  double dxo, dyo;
  double cxc, cyc;     // (n-1)/2
  double quad_re, quad_im;  // e^{ikz}/(i lam z)
  int adjoint;         // 1: exact adjoint of the forward operator
  int* status;
  // f32 engine: the separable phase factors as per-axis tables (FP64 values
  // rounded to f32, launch_fraunhofer fills them): pre = tpx[ix] tpy[iy],
  // post = tqx[mx] tqy[my] for the source bin (mx, my); null for FP64
  float2 *tpx, *tpy, *tqx, *tqy;
};

template <typename T> cudaError_t launch_asm_prep(const PropArgs& a, void* tables, cudaStream_t st);
template <typename T> cudaError_t launch_passA(const PropArgs& a, cudaStream_t st);
template <typename T> cudaError_t launch_passB(const PropArgs& a, cudaStream_t st);
template <typename T> cudaError_t launch_passC(const PropArgs& a, cudaStream_t st);
template <typename T> cudaError_t launch_fraunhofer(const FraunArgs& a, cudaStream_t st);
// Plain 2D DFT (see prop_kernels.cu) and the conjugating copy of an inverse.
template <typename T>
cudaError_t launch_fft2(const PropArgs& a, void* spec, void* out, int out_c128, int conj,
                        cudaStream_t st);
template <typename T>
cudaError_t launch_conj_copy(const void* src, int c128, void* dst, size_t n, cudaStream_t st);

cudaError_t launch_twiddles(void* dst, int n, int is_double, cudaStream_t st);
// f32 tables of register-FFT lengths (reg_fft_size): fills the stage-ordered
// copy at tw + m from the m-point table at tw (the allocation holds 2 m float2).
cudaError_t launch_stage_twiddles(void* tw, int m, cudaStream_t st);
// Separable Fresnel-convolution kernel spectrum: fills hx (Px) and hy (Py).
template <typename T>
cudaError_t launch_fresnel_ksep(const PropArgs& a, void* hx, void* hy, void* tmp, cudaStream_t st);
// Rayleigh-Sommerfeld kernel spectrum, column-major Px x Py, built in f64
// and stored as T.
template <typename T>
cudaError_t launch_rs_kspec(const PropArgs& a, void* kspec, void* tmp64, cudaStream_t st);
// Quarter table (ENG_KEVEN) of the spectrum of the 2n-periodic even extension
// of a kernel quadrant hq (hny x hnx complex128, hq[y][x] = h(y, x); its
// first row and column are halved in place): `a` carries the zero-padding
// axis plans make_axis(hnx, 2 hnx), make_axis(hny, 2 hny), their FP64
// twiddle tables and scale = 1 / (Px Py); tmp64 holds Px hny + Px Py double2.
cudaError_t launch_even_kspec(const PropArgs& a, void* hq, int hnx, int hny, void* kq,
                              void* tmp64, cudaStream_t st);

// Standalone element application (Element::apply chain, no propagation).
template <typename T>
cudaError_t launch_apply_elements(const void* in, int in_c128, void* out, int out_c128,
                                  const ElementList& els, int nx, int ny, double dx, double dy,
                                  int* status, cudaStream_t st);

// f32 fast element tables (psi == 0 elements): bytes of scratch needed and
// the build; fills e.span / tabx / taby / bilx / bily / latf.
size_t element_tables_bytes(const DevElement& e, int nx, int ny);
// complex128 <-> complex64 conversion of n samples (host-buffer batch: on the
// copy streams, so the passes read and write complex64)
cudaError_t launch_c128_to_c64(const void* src, void* dst, size_t n, cudaStream_t st);
cudaError_t launch_c64_to_c128(const void* src, void* dst, size_t n, cudaStream_t st);
// t[iy nx + ix] = the f32 transmission of the chain L (fast tables) at each
// sample: apply_elements_fast applied to 1.
cudaError_t launch_transmission(const ElementList& L, int nx, int ny, float2* t, cudaStream_t st);
cudaError_t launch_element_tables(DevElement& e, int nx, int ny, double dx, double dy,
                                  void* scratch, cudaStream_t st);

// Register-FFT f32 passes (prop_fast.cu) for power-of-two sub-FFT lengths
// in [256, 4096]; the generic launchers route to them.
bool reg_fft_size(int m);
cudaError_t launch_passA_reg(const PropArgs& a, cudaStream_t st);
cudaError_t launch_passB_reg(const PropArgs& a, cudaStream_t st);
cudaError_t launch_passC_reg(const PropArgs& a, cudaStream_t st);

// Kernel launches issued by the library since load.
unsigned long long launch_count();

size_t smem_passA_bytes(const AxisPlan& ax, int is_double, int rows);
size_t smem_passB_bytes(const AxisPlan& ay, int is_double);
int rows_per_cta(const AxisPlan& ax, int is_double);
// Whether the three passes of a propagation on these axis plans fit the
// per-block shared memory `max_smem` (every entry point checks this before
// its first launch).
bool prop_smem_fits(const AxisPlan& ax, const AxisPlan& ay, int is_double, size_t max_smem);

// The message osgpu_last_error returns on this thread (printf format).
void set_last_error(const char* fmt, ...);
// Forget the cached device addresses of the allocation-free entry point's
// static scratch (their contexts may have been reset).
void noalloc_forget_scratch();

}  // namespace osgpu
