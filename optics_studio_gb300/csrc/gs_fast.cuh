// Fused f32 Gerchberg-Saxton kernels of the Fraunhofer engine (gs_fast.cu).
#pragma once
#include <cuda_runtime.h>

#include "inverse_kernels.cuh"

namespace osgpu {

// Device-side view of one GS item on an M x M grid.
struct GsFastItem {
  float2* W;                  // spectrum scratch, column-major M x M
  float* phase;               // current phase
  float* best;                // best phase (the caller's phase buffer)
  const float* amask;         // illumination amplitude, zero outside the carrier aperture
  const float* tamp_t;        // target amplitude, column-major
  const float* tint_t;        // merit target intensity, column-major (null: T^2)
  const float2* prx;          // pre = prx[ix] pry[iy]
  const float2* pry;
  const float2* qx;           // D = qx[ix] qy[iy]
  const float2* qy;
  float c;                    // |D|
  float* terr;                // optional: |U| - T of the last iteration (column-major)
  float* perr;                // optional: phase update of the last iteration
  GsState* state;
  double* part_col;           // 2 frames x gs_fast_blocks(M) pairs
  double* part_row;           // 1 frame x gs_fast_row_blocks(M) pairs
  float* out_intensity;       // intensity_only pass: |U|^2 (row-major)
};

struct GsFastArgs {
  int M;
  const void* tw;  // M-point f32 twiddle table
  float beta_f, beta_p, lo, hi;
  int wrap;        // hi - lo >= 2 pi (encode_bounds wraps instead of clamping)
  int intensity_only;  // column pass: forward transform and |U|^2 only
  // every item's W lies at w_base + i w_stride bytes (one allocation; the row
  // kernel's tensor map of the spectra); null: the row kernel gathers directly
  const void* w_base;
  unsigned long long w_stride;
};

bool gs_fast_size(int m);
int gs_fast_blocks(int m);      // CTAs per item of the column kernel
int gs_fast_row_blocks(int m);  // CTAs per item of the row kernel
cudaError_t launch_gs_cols(const GsFastItem* items, int n_items, const GsFastArgs& a,
                           cudaStream_t st);
// iterate = 0: first forward rows from the initial phase only
cudaError_t launch_gs_rows(const GsFastItem* items, int n_items, const GsFastArgs& a,
                           int iterate, cudaStream_t st);
cudaError_t launch_transpose_real(const float* in, float* out, int M, cudaStream_t st);

}  // namespace osgpu
