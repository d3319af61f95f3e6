// Fused f32 Gerchberg-Saxton iteration for the Fraunhofer engine (square
// power-of-two grids, M in [256, 4096]), batched over items.
//
// Forward operator (reference fraunhofer.rs:364-443, z > 0, no source
// offset): U = D o FFT2(pre o u), pre(ix, iy) = prx[ix] pry[iy] and
// D(ix, iy) = qx[ix] qy[iy] with |D| = c = dx dy / (lam z) everywhere.  Its
// adjoint is conj(pre) o FFT2^H(conj(D) o U).  The target-plane projection
// U' = U a / |U| (gs.rs:533-545) followed by conj(D) is therefore
// c a F / |F| in the raw transform domain F = FFT2(pre o u), so one column
// pass does the forward column FFT, the projection and its reductions, and
// the inverse column FFT; one row pass does the inverse row FFT, conj(pre),
// the DOE-plane update (gs.rs:557-566) and, for the next iteration, the
// mask, pre and the forward row FFT.  The spectrum W is column-major
// (W[kx * M + ky]).  Every kernel returns at once for an item whose state
// says stop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "fft_reg.cuh"
#include "gs_fast.cuh"
#include "inverse_kernels.cuh"
#include "tma.cuh"

namespace osgpu {

extern unsigned long long& launch_counter();

namespace {

using namespace regfft;

constexpr float kPiF = 3.14159265358979f;
constexpr float kTauF = 6.28318530717959f;

// r mod 2 pi in [0, 2 pi): one conditional step covers the common range
// (|r| < 4 pi), fmodf the rest.
__device__ __forceinline__ float rem_tau(float r) {
  if (r < 0.f) r += kTauF;
  else if (r >= kTauF) r -= kTauF;
  if (r < 0.f || r >= kTauF) {
    r = fmodf(r, kTauF);
    if (r < 0.f) r += kTauF;
  }
  return r;
}

__device__ __forceinline__ float wrap_pi_f(float v) { return rem_tau(v + kPiF) - kPiF; }

__device__ __forceinline__ float encode_f(float p, const GsFastArgs& a) {
  if (a.wrap) return a.lo + rem_tau(p - a.lo);
  return p < a.lo ? a.lo : (p > a.hi ? a.hi : p);
}

// Sum of one float per thread over the CTA into part[(f * gridDim.x + blockIdx.x) * 2]
// (compensation slot 0), the layout of the GS fold kernels.
__device__ __forceinline__ void cta_sum(float x, double* part, int f, double* red, int blk,
                                        int nblk) {
  double v = (double)x;
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += red[i];
    const size_t o = ((size_t)f * nblk + blk) * 2;
    part[o] = s;
    part[o + 1] = 0.0;
  }
}

// e^{-i pi q / 16}, q = 0..15 (cos and -sin of pi q / 16)
__device__ __constant__ float2 kW32[16] = {
    {1.000000000e+00f, -0.000000000e+00f}, {9.807852804e-01f, -1.950903220e-01f},
    {9.238795325e-01f, -3.826834324e-01f}, {8.314696123e-01f, -5.555702330e-01f},
    {7.071067812e-01f, -7.071067812e-01f}, {5.555702330e-01f, -8.314696123e-01f},
    {3.826834324e-01f, -9.238795325e-01f}, {1.950903220e-01f, -9.807852804e-01f},
    {0.000000000e+00f, -1.000000000e+00f}, {-1.950903220e-01f, -9.807852804e-01f},
    {-3.826834324e-01f, -9.238795325e-01f}, {-5.555702330e-01f, -8.314696123e-01f},
    {-7.071067812e-01f, -7.071067812e-01f}, {-8.314696123e-01f, -5.555702330e-01f},
    {-9.238795325e-01f, -3.826834324e-01f}, {-9.807852804e-01f, -1.950903220e-01f}};

template <int M, int G>
struct GsLay {
  static constexpr int T = M / 16;
  static constexpr int THREADS = G * T;
  static constexpr int MINB = THREADS >= 512 ? 1 : 2;  // 128 registers per thread
  // exchange-buffer stride: the transform's padded size plus 4 entries, so
  // that buffers 0..3 start 0, 8, 16 and 24 banks apart (the paired-lane
  // tile gather / scatter of the row kernel reads two buffers per lane pair)
  static constexpr int SB = Plan<M>::SMEM + 4;
  static constexpr size_t SMEM =
      ((size_t)TwLay<M>::SIZE + (size_t)G * SB) * sizeof(float2) + 32 * sizeof(double);
};

template <int M, int G>
__global__ void __launch_bounds__(GsLay<M, G>::THREADS, GsLay<M, G>::MINB)
    k_gs_cols(const GsFastItem* __restrict__ items, GsFastArgs a, int n_items) {
  constexpr int T = M / 16;
  constexpr int NB = M / G;  // CTAs' worth of columns per item
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* bufs = tws + TwLay<M>::SIZE;
  double* red = reinterpret_cast<double*>(bufs + G * GsLay<M, G>::SB);
  const int g = threadIdx.x / T, tid = threadIdx.x - g * T;
  const int BAR_ID = (T % 32 == 0) ? 1 + g : 1;
  const int BAR_N = (T % 32 == 0) ? T : GsLay<M, G>::THREADS;
  float2* buf = bufs + g * GsLay<M, G>::SB;
  {  // stage-ordered table stored behind the M-point table
    const float2* twm = reinterpret_cast<const float2*>(a.tw);
    for (int i = threadIdx.x; i < TwLay<M>::SIZE; i += blockDim.x) tws[i] = __ldg(twm + M + i);
  }
  // persistent: the CTA walks (item, column block) units, the twiddles loaded once
  for (int u = blockIdx.x; u < NB * n_items; u += gridDim.x) {
  const GsFastItem& it = items[u / NB];
  const int blk = u - (u / NB) * NB;
  if (a.intensity_only ? !it.out_intensity : it.state->stop) continue;
  const int kx = blk * G + g;
  float2* col = it.W + (size_t)kx * M;
  float2 v[16];
  float tq[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = col[tid + T * q];
  if (!a.intensity_only) {
#pragma unroll
    for (int q = 0; q < 16; ++q) tq[q] = __ldg(it.tamp_t + (size_t)kx * M + tid + T * q);
  }
  __syncthreads();
  fft1s<M, false>(v, buf, tws, tid, BAR_ID, BAR_N);
  const float c = it.c, bf = a.beta_f;
  if (a.intensity_only) {  // |U|^2 = c^2 |F|^2 of the forward pass, row-major
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float m2q = v[q].x * v[q].x + v[q].y * v[q].y;
      it.out_intensity[(size_t)(tid + T * q) * M + kx] = c * c * m2q;
    }
    continue;
  }
  float e2 = 0.f, m2 = 0.f;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int ky = tid + T * q;
    const size_t kt = (size_t)kx * M + ky;  // column-major target index
    const float2 f = v[q];
    const float m = sqrtf(f.x * f.x + f.y * f.y);
    const float amp = c * m;
    const float t = tq[q];
    const float ti = it.tint_t ? __ldg(it.tint_t + kt) : t * t;
    const float err = amp - t;
    const float inten = amp * amp;
    e2 = fmaf(err, err, e2);
    m2 = fmaf(inten - ti, inten - ti, m2);
    if (it.terr) it.terr[kt] = err;  // column-major, coalesced; transposed after the loop
    const float aa = (1.f - bf) * amp + bf * t;
    float2 gq;
    if (m > 0.f) {
      const float s = c * aa / m;
      gq = make_float2(f.x * s, f.y * s);
    } else {  // projection (a, 0) through conj(D)
      const float2 d = cmul(__ldg(it.qx + kx), __ldg(it.qy + ky));
      gq = make_float2(d.x * aa, -d.y * aa);
    }
    v[q] = gq;
  }
  fft1s<M, true>(v, buf, tws, tid, BAR_ID, BAR_N);
#pragma unroll
  for (int q = 0; q < 16; ++q) col[tid + T * q] = v[q];
  cta_sum(e2, it.part_col, 0, red, blk, NB);
  cta_sum(m2, it.part_col, 1, red, blk, NB);
  }
}

// One row unit of the fused GS row pass after its inputs are in place (v:
// the group's spectrum row when iterating, ph / am: its phase and amplitude
// samples tid + T q): inverse row FFT, conj(pre), the DOE-plane update, the
// next mask and pre, forward row FFT, the spectrum tile written back.
template <int M, int G>
__device__ __forceinline__ void gs_row_unit(const GsFastItem& it, const GsFastArgs& a,
                                            int iterate, int iy0, int g, int tid,
                                            float2 (&v)[16], float (&ph)[16],
                                            const float (&am)[16], float2* buf, float2* bufs,
                                            const float2* tws, double* red, int blk) {
  constexpr int T = M / 16;
  constexpr int NB = M / G;
  constexpr bool kTile = (G == 4) && (T % 32 == 0);
  const int BAR_ID = (T % 32 == 0) ? 1 + g : 1;
  const int BAR_N = (T % 32 == 0) ? T : GsLay<M, G>::THREADS;
  const int iy = iy0 + g;
  const float2 py = __ldg(it.pry + iy);
  float* __restrict__ prow = it.phase + (size_t)iy * M;
  float d2 = 0.f;
  if (iterate) {
    fft1s<M, true>(v, buf, tws, tid, BAR_ID, BAR_N);
  }
  const bool keep = iterate && it.state->improved;
  // pre-phase of column ix = tid + T q: prx[ix] = e^{i pi (M - 1) ix / M}
  // = prx[tid] e^{-i pi q / 16} (T even), so one load per thread and the
  // 32nd roots of unity replace sixteen loads behind the stores below
  const float2 p0 = __ldg(it.prx + tid);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int ix = tid + T * q;
    const size_t k = (size_t)iy * M + ix;
    const float2 pre = cmul(cmul(p0, kW32[q]), py);
    float p = ph[q];
    if (iterate) {
      const float2 w = cmulc(v[q], pre);  // conj(pre) v
      const float dphi = wrap_pi_f(atan2f(w.y, w.x) - p);
      if (keep) it.best[k] = p;
      p = encode_f(p + a.beta_p * dphi, a);
      prow[ix] = p;
      d2 = fmaf(dphi, dphi, d2);
      if (it.perr) it.perr[k] = dphi;
    }
    // open ? illum e^{i p} : 0, with the aperture folded into the amplitude
    float s, cs;
    __sincosf(wrap_pi_f(p), &s, &cs);  // argument in [-pi, pi)
    v[q] = cmul(make_float2(am[q] * cs, am[q] * s), pre);
  }
  fft1s<M, false>(v, buf, tws, tid, BAR_ID, BAR_N);
  if (kTile) {
    group_sync(BAR_ID, BAR_N);  // the transform's last reads of buf are done
#pragma unroll
    for (int q = 0; q < 16; ++q) buf[tid + T * q] = v[q];
    __syncthreads();
    constexpr int SB = GsLay<M, G>::SB;
    for (int h = threadIdx.x; h < 2 * M; h += blockDim.x) {  // whole sectors per lane pair
      const int p = h >> 1, hf = h & 1;
      const float2 r0 = bufs[2 * hf * SB + p], r1 = bufs[(2 * hf + 1) * SB + p];
      reinterpret_cast<float4*>(it.W + (size_t)p * M + iy0)[hf] = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 16; ++q) it.W[(size_t)(tid + T * q) * M + iy] = v[q];
  }
  if (iterate) cta_sum(d2, it.part_row, 0, red, blk, NB);
  (void)NB;
}

template <int M, int G>
__global__ void __launch_bounds__(GsLay<M, G>::THREADS, GsLay<M, G>::MINB)
    k_gs_rows(const GsFastItem* __restrict__ items, GsFastArgs a, int iterate, int n_items) {
  constexpr int T = M / 16;
  constexpr int NB = M / G;  // CTAs' worth of rows per item
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* bufs = tws + TwLay<M>::SIZE;
  double* red = reinterpret_cast<double*>(bufs + G * GsLay<M, G>::SB);
  const int g = threadIdx.x / T, tid = threadIdx.x - g * T;
  float2* buf = bufs + g * GsLay<M, G>::SB;
  {  // stage-ordered table stored behind the M-point table
    const float2* twm = reinterpret_cast<const float2*>(a.tw);
    for (int i = threadIdx.x; i < TwLay<M>::SIZE; i += blockDim.x) tws[i] = __ldg(twm + M + i);
  }
  // persistent: the CTA walks (item, row block) units, the twiddles loaded once
  for (int u = blockIdx.x; u < NB * n_items; u += gridDim.x) {
  const GsFastItem& it = items[u / NB];
  const int blk = u - (u / NB) * NB;
  if (iterate && it.state->stop) continue;
  const int iy0 = blk * G, iy = iy0 + g;
  const float* prow = it.phase + (size_t)iy * M;
  // 4-row tiles: the spectrum moves through the groups' exchange buffers in
  // 32-byte runs W[kx * M + iy0 .. iy0 + 3] (one sector per request)
  constexpr bool kTile = (G == 4) && (T % 32 == 0);
  float2 v[16];
  float ph[16], am[16];
  if (iterate) {
    if (kTile) {
      // the two lanes of a pair read the two 16-byte halves of one 32-byte run
      constexpr int SB = GsLay<M, G>::SB;
      for (int h = threadIdx.x; h < 2 * M; h += blockDim.x) {
        const int p = h >> 1, hf = h & 1;
        const float4 a0 = reinterpret_cast<const float4*>(it.W + (size_t)p * M + iy0)[hf];
        bufs[2 * hf * SB + p] = make_float2(a0.x, a0.y);
        bufs[(2 * hf + 1) * SB + p] = make_float2(a0.z, a0.w);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = it.W[(size_t)(tid + T * q) * M + iy];
    }
  }
  // per-sample inputs issued before the transform (no store precedes them)
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    ph[q] = prow[tid + T * q];
    am[q] = __ldg(it.amask + (size_t)iy * M + tid + T * q);
  }
  __syncthreads();
  if (iterate && kTile) {
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = buf[tid + T * q];
  }
  gs_row_unit<M, G>(it, a, iterate, iy0, g, tid, v, ph, am, buf, bufs, tws, red, blk);
  __syncthreads();  // the next unit's tile gather rewrites the exchange buffers
  }
}

// The row pass with its inputs staged by the tensor-memory accelerator: the
// same persistent walk over (item, 4-row block) units as k_gs_rows (G = 4),
// but the next unit's inputs arrive in shared memory while the current one
// is transformed -- its 4-row tile of the column-major spectrum (M / 256
// three-dimensional box copies, iy 4 x kx 256 x item 1, of the spectra viewed
// as [item][kx][ky]) and its 4 phase and 4 amplitude rows (two contiguous
// bulk copies), completing one mbarrier.  Every wait is bounded (status bit
// of the item's state on timeout: the CTA leaves as a whole).
template <int M>
__global__ void __launch_bounds__(GsLay<M, 4>::THREADS, 1)
    k_gs_rows_tma(const GsFastItem* __restrict__ items, GsFastArgs a, int iterate, int n_items,
                  const __grid_constant__ CUtensorMap wmap) {
  constexpr int G = 4;
  constexpr int T = M / 16;
  constexpr int NB = M / G;
  constexpr int SB = GsLay<M, G>::SB;
  extern __shared__ __align__(128) unsigned char smem_gs_tma[];
  float4* stw = reinterpret_cast<float4*>(smem_gs_tma);            // [kx][4 rows]: 2 float4 per kx
  float* stp = reinterpret_cast<float*>(stw + 2 * M);           // 4 phase rows
  float* sta = stp + 4 * M;                                     // 4 amplitude rows
  float2* tws = reinterpret_cast<float2*>(sta + 4 * M);
  float2* bufs = tws + TwLay<M>::SIZE;
  double* red = reinterpret_cast<double*>(bufs + G * SB);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(red + 32);
  const int g = threadIdx.x / T, tid = threadIdx.x - g * T;
  float2* buf = bufs + g * SB;
  const unsigned rows_bytes = 4u * M * 4u;
  const unsigned bytes = (iterate ? (unsigned)M * 32u : 0u) + 2u * rows_bytes;
  if (threadIdx.x == 0) {
    tma::prefetch_map(&wmap);
    tma::mbar_init(bar, 1);
  }
  {  // stage-ordered table stored behind the M-point table
    const float2* twm = reinterpret_cast<const float2*>(a.tw);
    for (int i = threadIdx.x; i < TwLay<M>::SIZE; i += blockDim.x) tws[i] = __ldg(twm + M + i);
  }
  __syncthreads();  // the barrier is initialised
  auto issue = [&](int u) {  // thread 0: the inputs of unit u
    const int item = u / NB, iy0 = (u - item * NB) * G;
    const GsFastItem& it = items[item];
    tma::mbar_expect_tx(bar, bytes);
    if (iterate)
#pragma unroll 1
      for (int b = 0; b < M / 256; ++b) tma::load_3d(stw + 2 * 256 * b, &wmap, iy0, 256 * b, item, bar);
    tma::load_bulk(stp, it.phase + (size_t)iy0 * M, rows_bytes, bar);
    tma::load_bulk(sta, it.amask + (size_t)iy0 * M, rows_bytes, bar);
  };
  unsigned phase = 0;
  int u = blockIdx.x;
  if (u < NB * n_items && threadIdx.x == 0) issue(u);
  for (; u < NB * n_items; u += gridDim.x) {
    const GsFastItem& it = items[u / NB];
    const int blk = u - (u / NB) * NB;
    const int iy0 = blk * G;
    const bool arrived = tma::mbar_wait(bar, phase);
    if (!__syncthreads_and(arrived)) {
      if (threadIdx.x == 0) {
        it.state->fault = 1;  // reported by the host after the loop
        it.state->stop = 1;
        tma::mbar_wait(bar, phase);  // a late copy lands before the CTA's memory is reused
      }
      return;
    }
    phase ^= 1u;
    float2 v[16];
    float ph[16], am[16];
    if (iterate) {
      for (int h = threadIdx.x; h < 2 * M; h += blockDim.x) {
        const int p = h >> 1, hf = h & 1;
        const float4 a0 = stw[2 * p + hf];
        bufs[2 * hf * SB + p] = make_float2(a0.x, a0.y);
        bufs[(2 * hf + 1) * SB + p] = make_float2(a0.z, a0.w);
      }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      ph[q] = stp[g * M + tid + T * q];
      am[q] = sta[g * M + tid + T * q];
    }
    __syncthreads();  // the staging buffers are consumed: the next unit's inputs
    const int nu = u + gridDim.x;
    if (nu < NB * n_items && threadIdx.x == 0) issue(nu);
    const bool stopped = iterate && it.state->stop;
    if (!stopped) {
      if (iterate) {
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] = buf[tid + T * q];
      }
      gs_row_unit<M, G>(it, a, iterate, iy0, g, tid, v, ph, am, buf, bufs, tws, red, blk);
    }
    __syncthreads();  // the next unit's tile rewrites the exchange buffers
  }
}

// Column-major copy of a real M x M array (32 x 32 tiles through shared memory).
__global__ void k_transpose_real(const float* __restrict__ in, float* __restrict__ out, int M) {
  __shared__ float tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y)
    tile[j][threadIdx.x] = in[(size_t)(by + j) * M + bx + threadIdx.x];
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y)
    out[(size_t)(bx + j) * M + by + threadIdx.x] = tile[threadIdx.x][j];
}

constexpr int kG = 2;   // columns per CTA
constexpr int kGR = 4;  // rows per CTA: 4 adjacent rows share the 32-byte sectors
                        // of the column-major spectrum they gather and scatter

template <int M>
cudaError_t launch_cols(const GsFastItem* items, int n_items, const GsFastArgs& a,
                        cudaStream_t st) {
  using L = GsLay<M, kG>;
  cudaError_t e = cudaFuncSetAttribute(k_gs_cols<M, kG>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::SMEM);
  if (e != cudaSuccess) return e;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gs_cols<M, kG>, L::THREADS, L::SMEM);
  const int units = (M / kG) * n_items;
  const int grid = std::max(1, std::min(units, std::max(1, per_sm) * std::max(1, sms)));
  ++launch_counter();
  k_gs_cols<M, kG><<<grid, L::THREADS, L::SMEM, st>>>(items, a, n_items);
  return cudaGetLastError();
}

template <int M>
size_t gs_rows_tma_smem() {
  return (size_t)M * 32 + 2 * (size_t)4 * M * 4 + GsLay<M, 4>::SMEM + 16;
}

template <int M>
cudaError_t launch_rows(const GsFastItem* items, int n_items, const GsFastArgs& a, int iterate,
                        cudaStream_t st) {
  constexpr int G = (M / 16 * kGR <= 512) ? kGR : 512 / (M / 16);
  if constexpr (G == 4 && (M / 16) % 32 == 0) {
    const char* te = getenv("OSGPU_GS_TMA");
    if ((!te || atoi(te) != 0) && a.w_base && a.w_stride % 16 == 0 &&
        gs_rows_tma_smem<M>() <= 232448) {
      const unsigned long long dims[3] = {(unsigned long long)M, (unsigned long long)M,
                                          (unsigned long long)n_items};
      const unsigned long long strides[2] = {(unsigned long long)M * 8ull, a.w_stride};
      const unsigned box[3] = {4u, 256u, 1u};
      CUtensorMap map;
      if (encode_map_3d_c64(&map, a.w_base, dims, strides, box)) {
        const size_t smem = gs_rows_tma_smem<M>();
        cudaError_t e = cudaFuncSetAttribute(
            k_gs_rows_tma<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int units = (M / 4) * n_items;
        const int grid = std::max(1, std::min(units, std::max(1, sms)));
        ++launch_counter();
        k_gs_rows_tma<M><<<grid, GsLay<M, 4>::THREADS, smem, st>>>(items, a, iterate, n_items,
                                                                  map);
        return cudaGetLastError();
      }
    }
  }
  using L = GsLay<M, G>;
  cudaError_t e = cudaFuncSetAttribute(k_gs_rows<M, G>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::SMEM);
  if (e != cudaSuccess) return e;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gs_rows<M, G>, L::THREADS, L::SMEM);
  const int units = (M / G) * n_items;
  const int grid = std::max(1, std::min(units, std::max(1, per_sm) * std::max(1, sms)));
  ++launch_counter();
  k_gs_rows<M, G><<<grid, L::THREADS, L::SMEM, st>>>(items, a, iterate, n_items);
  return cudaGetLastError();
}

}  // namespace

bool gs_fast_size(int m) { return m == 256 || m == 512 || m == 1024 || m == 2048 || m == 4096; }

int gs_fast_blocks(int m) { return m / kG; }

int gs_fast_row_blocks(int m) {
  const int g = (m / 16 * kGR <= 512) ? kGR : 512 / (m / 16);
  return m / g;
}

#define OSGPU_GS_DISPATCH(m, fn, ...)          \
  switch (m) {                                 \
    case 256: return fn<256>(__VA_ARGS__);     \
    case 512: return fn<512>(__VA_ARGS__);     \
    case 1024: return fn<1024>(__VA_ARGS__);   \
    case 2048: return fn<2048>(__VA_ARGS__);   \
    case 4096: return fn<4096>(__VA_ARGS__);   \
    default: return cudaErrorInvalidValue;     \
  }

cudaError_t launch_gs_cols(const GsFastItem* items, int n_items, const GsFastArgs& a,
                           cudaStream_t st) {
  OSGPU_GS_DISPATCH(a.M, launch_cols, items, n_items, a, st)
}

cudaError_t launch_gs_rows(const GsFastItem* items, int n_items, const GsFastArgs& a,
                           int iterate, cudaStream_t st) {
  OSGPU_GS_DISPATCH(a.M, launch_rows, items, n_items, a, iterate, st)
}

cudaError_t launch_transpose_real(const float* in, float* out, int M, cudaStream_t st) {
  ++launch_counter();
  k_transpose_real<<<dim3(M / 32, M / 32), dim3(32, 8), 0, st>>>(in, out, M);
  return cudaGetLastError();
}

}  // namespace osgpu
