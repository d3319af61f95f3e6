// f32 propagation passes built on the register FFT (fft_reg.cuh), for
// power-of-two sub-FFT lengths m in [256, 4096].  Same data layout and the
// same pruned decomposition as the generic passes in prop_kernels.cu:
//   pass A: rows   x_s[j] = u[j] W_P^{s j}  -> FFT_m -> W[(r q + s) ny + iy]
//   pass B: column kx: for t < r: c W_P^{t j} -> FFT_m -> x H -> IFFT_m
//           -> x W_P^{-t j}, summed; rewritten in place
//   pass C: rows   sum_s W_P^{-s j} IFFT_m(W[(r q + s) ny + iy])
// Pass B runs one CTA per column pair (kx, Px - kx): the transfer functions
// of the engines it serves are even in fx and fy, so one shared table of
// H(kx, |k_y|) for |k_y| <= Py/2 serves all 4 quadrant bins of both columns.
#include "fft_reg.cuh"
#include "prop_kernels.cuh"
#include "elements.cuh"

namespace osgpu {

extern unsigned long long& launch_counter();

namespace {

using namespace regfft;

__device__ __forceinline__ float2 ld_in(const void* p, int c128, size_t i) {
  if (c128) {
    const double2 v = reinterpret_cast<const double2*>(p)[i];
    return make_float2((float)v.x, (float)v.y);
  }
  return __ldg(reinterpret_cast<const float2*>(p) + i);
}

// f32 split transfer function at (column data, row ky) — same arithmetic as
// the generic pass B (prop_kernels.cu, k_passB h_mode 1).
__device__ __forceinline__ float2 h_asm_split(const PropArgs& a, float2 exc, float cah, float cal,
                                              float sac, int kmc, int ky, int akk) {
  if (akk > kmc) return make_float2(0.f, 0.f);
  const float bh = a.b_hi[ky], blo = a.b_lo[ky];
  const float s = sac + bh;
  const float q = sqrtf(fmaxf(1.f - s, 0.f));
  const float opq = 1.f + q;
  const float tau = a.Kf * (s * s * s) * (3.f + q) / (8.f * opq * opq * opq);
  const float pr = cah * bh;
  const float er = fmaf(cah, bh, -pr);
  const float corr = er + (cah * blo + cal * bh);
  const float nq = rintf(pr * 0.159154943091895336f);
  float rr = fmaf(-nq, 6.28125f, pr);
  rr = fmaf(-nq, 1.93530717958647692e-3f, rr);
  const float th = rr + (corr - tau);
  float sn, cs;
  __sincosf(th, &sn, &cs);
  const float2 ey = a.Ey[ky];
  const float hr = exc.x * ey.x - exc.y * ey.y;
  const float hi = exc.x * ey.y + exc.y * ey.x;
  return make_float2(hr * cs - hi * sn, hr * sn + hi * cs);
}

// ---------------------------------------------------------------- pass B

template <int M>
__global__ void __launch_bounds__(2 * (M / 16), (M <= 2048 ? 2 : 1)) k_passB_reg(PropArgs a, int use_table) {
  constexpr int T = M / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  const int half = threadIdx.x / T;  // which column of the pair
  const int tid = threadIdx.x - half * T;
  float2* s0 = sm + (size_t)half * 2 * Plan<M>::SMEM;
  float2* s1 = s0 + Plan<M>::SMEM;
  float2* htab = sm + 4 * Plan<M>::SMEM;
  const int Px = a.ax.P, Py = a.ay.P, ry = a.ay.r, ny = a.ny;
  const int p = blockIdx.x;
  int kx = p;
  bool active = true;
  if (half == 1) {
    // columns 0 and Px/2 have no partner: the second half recomputes column
    // p and does not store (every thread must reach the FFT barriers)
    const bool single = (p == 0) || (2 * p == Px);
    kx = single ? p : Px - p;
    active = !single;
  }
  const float2* twm = reinterpret_cast<const float2*>(a.tw_my);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Py);
  float2* W = reinterpret_cast<float2*>(a.work) + (size_t)kx * ny;

  // Column data of kx0 = p (shared by the pair: |fx| is equal).
  const bool asm_split = (a.engine == ENG_ASM && a.h_mode == 1);
  const bool fres = (a.engine == ENG_FRESNEL_TF && a.h_mode == 1);
  float2 exc = make_float2(0.f, 0.f);
  float cah = 0.f, cal = 0.f, sac = 0.f;
  int kmc = -1;
  if (asm_split || fres) exc = a.Ex[p];
  if (asm_split) {
    cah = a.ca_hi[p];
    cal = a.ca_lo[p];
    sac = a.sa[p];
    kmc = a.kmax[p];
  }
  const int hh = Py / 2;
  if (use_table) {
    for (int k = threadIdx.x; k <= hh; k += blockDim.x) {
      float2 h;
      if (asm_split) {
        h = h_asm_split(a, exc, cah, cal, sac, kmc, k, k);
      } else {  // Fresnel TF: Ex[kx] Ey[ky]
        const float2 ey = a.Ey[k];
        h = make_float2(exc.x * ey.x - exc.y * ey.y, exc.x * ey.y + exc.y * ey.x);
      }
      htab[k] = h;
    }
  }
  __syncthreads();

  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
  for (int t = 0; t < ry; ++t) {
    // W_P^{t j} for j = tid + T q  (t j < ry M = Py, no reduction needed):
    // W_P^{t tid} (per thread) times W_P^{t T q} (uniform across the CTA)
    const float2 wb = __ldg(&twP[t * tid]);
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      float2 x = make_float2(0.f, 0.f);
      if (j < ny) {
        x = W[j];
        if (t > 0) x = cmul(x, cmul(wb, __ldg(&twP[t * T * q])));
      }
      v[q] = x;
    }
    fft<M, false>(v, s0, s1, twm, tid);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int ky = ry * (tid + T * q) + t;
      const int kk = (ky <= (Py - 1) / 2) ? ky : ky - Py;
      const int akk = kk < 0 ? -kk : kk;
      float2 h;
      if (use_table) {
        h = htab[akk];
      } else if (a.engine == ENG_KSPEC) {
        h = __ldg(reinterpret_cast<const float2*>(a.kspec) + (size_t)kx * Py + ky);
        if (a.conj_h) h.y = -h.y;
      } else if (a.engine == ENG_KSEP) {
        h = cmul(__ldg(reinterpret_cast<const float2*>(a.hx) + kx),
                 __ldg(reinterpret_cast<const float2*>(a.hy) + ky));
        if (a.conj_h) h.y = -h.y;
      } else {  // ENG_IDENTITY
        h = make_float2((float)a.scale, 0.f);
      }
      v[q] = cmul(v[q], h);
    }
    fft<M, true>(v, s0, s1, twm, tid);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      float2 y = v[q];
      if (t > 0 && j < ny) y = cmulc(y, cmul(wb, __ldg(&twP[t * T * q])));
      acc[q] = cadd(acc[q], y);
    }
  }
  if (active) {
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      if (j < ny) W[j] = acc[q];
    }
  }
}

// ---------------------------------------------------------------- pass A

template <int M>
__global__ void __launch_bounds__(256, 2) k_passA_reg(PropArgs a, int rows) {
  constexpr int T = M / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  const int r = threadIdx.x / T;
  const int tid = threadIdx.x - r * T;
  float2* s0 = sm + (size_t)r * 2 * Plan<M>::SMEM;
  float2* s1 = s0 + Plan<M>::SMEM;
  const int nx = a.nx, ny = a.ny, rx = a.ax.r, Px = a.ax.P;
  const int iy = blockIdx.x * rows + r;
  const bool live = iy < ny;
  const float2* twm = reinterpret_cast<const float2*>(a.tw_mx);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Px);
  float2* W = reinterpret_cast<float2*>(a.work);
  float2 xin[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = tid + T * q;
    float2 x = make_float2(0.f, 0.f);
    if (live && j < nx) {
      x = ld_in(a.in, a.in_c128, (size_t)iy * nx + j);
      if (a.status && (!isfinite(x.x) || !isfinite(x.y))) atomicOr(a.status, 1);
      if (a.els.count) {
        if (a.els.fast) {
          x = apply_elements_fast(a.els, j, iy, x);
        } else {
          double re = x.x, im = x.y;
          apply_elements_exact(a.els, j, iy, nx, ny, a.dx, a.dy, re, im);
          x = make_float2((float)re, (float)im);
        }
      }
    }
    xin[q] = x;
  }
  for (int s = 0; s < rx; ++s) {
    const float2 wb = __ldg(&twP[s * tid]);  // s j < rx M = Px
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      v[q] = (s > 0 && j < nx) ? cmul(xin[q], cmul(wb, __ldg(&twP[s * T * q]))) : xin[q];
    }
    fft<M, false>(v, s0, s1, twm, tid);
    if (live) {
#pragma unroll
      for (int q = 0; q < 16; ++q) W[(size_t)(rx * (tid + T * q) + s) * ny + iy] = v[q];
    }
  }
}

// ---------------------------------------------------------------- pass C

template <int M>
__global__ void __launch_bounds__(256, 2) k_passC_reg(PropArgs a, int rows) {
  constexpr int T = M / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  const int r = threadIdx.x / T;
  const int tid = threadIdx.x - r * T;
  float2* s0 = sm + (size_t)r * 2 * Plan<M>::SMEM;
  float2* s1 = s0 + Plan<M>::SMEM;
  const int nx = a.nx, ny = a.ny, rx = a.ax.r, Px = a.ax.P;
  const int iy = blockIdx.x * rows + r;
  const bool live = iy < ny;
  const float2* twm = reinterpret_cast<const float2*>(a.tw_mx);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Px);
  const float2* W = reinterpret_cast<const float2*>(a.work);
  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
  for (int s = 0; s < rx; ++s) {
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q)
      v[q] = live ? W[(size_t)(rx * (tid + T * q) + s) * ny + iy] : make_float2(0.f, 0.f);
    fft<M, true>(v, s0, s1, twm, tid);
    const float2 wb = __ldg(&twP[s * tid]);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      float2 y = v[q];
      if (s > 0 && j < nx) y = cmulc(y, cmul(wb, __ldg(&twP[s * T * q])));
      acc[q] = cadd(acc[q], y);
    }
  }
  if (!live) return;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = tid + T * q;
    if (j >= nx) continue;
    const float2 v = acc[q];
    const size_t o = (size_t)iy * nx + j;
    if (a.status && (!isfinite(v.x) || !isfinite(v.y))) atomicOr(a.status, 2);
    if (a.out) {
      if (a.out_c128) reinterpret_cast<double2*>(a.out)[o] = make_double2(v.x, v.y);
      else reinterpret_cast<float2*>(a.out)[o] = v;
    }
    if (a.out_intensity) a.out_intensity[o] = v.x * v.x + v.y * v.y;
    if (a.out_intensity64) a.out_intensity64[o] = (double)v.x * v.x + (double)v.y * v.y;
  }
}

template <int M>
size_t smem_B() { return (4 * (size_t)Plan<M>::SMEM) * sizeof(float2); }

template <int M>
cudaError_t launch_B(const PropArgs& a, cudaStream_t st) {
  const bool even = (a.engine == ENG_ASM || a.engine == ENG_FRESNEL_TF) && a.h_mode == 1;
  const int use_table = even ? 1 : 0;
  const size_t smem = smem_B<M>() + (use_table ? (size_t)(a.ay.P / 2 + 1) * sizeof(float2) : 0);
  cudaError_t e = cudaFuncSetAttribute(k_passB_reg<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const int pairs = a.ax.P / 2 + 1;
  ++launch_counter();
  k_passB_reg<M><<<pairs, 2 * (M / 16), smem, st>>>(a, use_table);
  return cudaGetLastError();
}

template <int M>
cudaError_t launch_A(const PropArgs& a, cudaStream_t st) {
  const int rows = 256 / (M / 16) > 0 ? 256 / (M / 16) : 1;
  const size_t smem = (size_t)rows * 2 * Plan<M>::SMEM * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(k_passA_reg<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  k_passA_reg<M><<<(a.ny + rows - 1) / rows, rows * (M / 16), smem, st>>>(a, rows);
  return cudaGetLastError();
}

template <int M>
cudaError_t launch_C(const PropArgs& a, cudaStream_t st) {
  const int rows = 256 / (M / 16) > 0 ? 256 / (M / 16) : 1;
  const size_t smem = (size_t)rows * 2 * Plan<M>::SMEM * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(k_passC_reg<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  k_passC_reg<M><<<(a.ny + rows - 1) / rows, rows * (M / 16), smem, st>>>(a, rows);
  return cudaGetLastError();
}

}  // namespace

bool reg_fft_size(int m) {
  return m == 256 || m == 512 || m == 1024 || m == 2048 || m == 4096;
}

#define OSGPU_DISPATCH(m, fn, ...)                    \
  switch (m) {                                        \
    case 256: return fn<256>(__VA_ARGS__);            \
    case 512: return fn<512>(__VA_ARGS__);            \
    case 1024: return fn<1024>(__VA_ARGS__);          \
    case 2048: return fn<2048>(__VA_ARGS__);          \
    case 4096: return fn<4096>(__VA_ARGS__);          \
    default: return cudaErrorInvalidValue;            \
  }

cudaError_t launch_passA_reg(const PropArgs& a, cudaStream_t st) { OSGPU_DISPATCH(a.ax.m, launch_A, a, st) }
cudaError_t launch_passB_reg(const PropArgs& a, cudaStream_t st) { OSGPU_DISPATCH(a.ay.m, launch_B, a, st) }
cudaError_t launch_passC_reg(const PropArgs& a, cudaStream_t st) { OSGPU_DISPATCH(a.ax.m, launch_C, a, st) }

}  // namespace osgpu
