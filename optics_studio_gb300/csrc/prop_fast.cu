// f32 propagation passes built on the register FFT (fft_reg.cuh), for
// power-of-two sub-FFT lengths m in [256, 4096].  Same data layout and the
// same pruned decomposition as the generic passes in prop_kernels.cu:
//   pass A: rows   x_s[j] = u[j] W_P^{s j}  -> FFT_m -> W[(r q + s) ny + iy]
//   pass B: column kx: for t < r: c W_P^{t j} -> FFT_m -> x H -> IFFT_m
//           -> x W_P^{-t j}, summed; rewritten in place
//   pass C: rows   sum_s W_P^{-s j} IFFT_m(W[(r q + s) ny + iy])
// Pass B runs one CTA per spectral column kx: the transfer functions of the
// engines it serves are even in fy, so one shared-memory table of
// H(kx, |k_y|) for |k_y| <= Py/2 serves both halves of the column.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "fft_reg.cuh"
#include "prop_kernels.cuh"
#include "elements.cuh"
#include "tma.cuh"

#include <cudaTypedefs.h>
#include <cstdint>

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
  // denominator in [8, 64]: the fast division is within 2 ulp
  const float tau = __fdividef(a.Kf * (s * s * s) * (3.f + q), 8.f * opq * opq * opq);
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

// ------------------------------------------------------------ layout
//
// One CTA per row (passes A, C) or per spectral column (pass B), G thread
// groups of T = M/16 threads.  The r sub-transforms of the pruned
// decomposition are spread over the groups (group g takes s = g, g + G, ...;
// every group runs the same number of iterations so the barriers inside the
// FFT match).  Shared memory holds the M-point twiddle table, the staged row
// or column, one exchange buffer per group, and the pruning twiddles
// W_P^{s j} = W_P^{s tid} W_P^{s T q} as two small tables.  Passes B and C
// reduce the groups' partial sums through the exchange buffers.

template <int M, int G>
struct Lay {
  static constexpr int T = M / 16;
  static constexpr int THREADS = G * T;
  static constexpr int MINB = THREADS >= 512 ? 1 : 512 / THREADS;
};

// The f32 twiddle tables of register-FFT lengths carry the stage-ordered
// copy (TwLay<M>) right behind the M-point table (launch_stage_twiddles).
template <int M>
__device__ __forceinline__ void copy_stage_twiddles(float2* tws, const float2* __restrict__ twm,
                                                    int t0, int nt) {
  for (int i = t0; i < TwLay<M>::SIZE; i += nt) tws[i] = __ldg(twm + M + i);
}

template <int M>
__global__ void k_stage_twiddles(float2* tw) {
  load_stage_twiddles<M>(tw + M, tw, blockIdx.x * blockDim.x + threadIdx.x,
                         gridDim.x * blockDim.x);
}

// Programmatic dependent launch (sm_90+).  The three f32 passes of a
// propagation are launched with programmatic stream serialization: each
// block signals at its start that the next pass may be scheduled (so the
// next pass's blocks fill the SMs its last wave leaves idle), and each pass
// runs its prologue that needs nothing from the pass before it (twiddle and
// pruning tables; in pass B the H table, built from the per-axis tables of
// the prep kernel, which every pass-A block has waited for) before
// griddepcontrol.wait, which returns once the previous pass has completed
// and its memory is visible.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename K, typename... Args>
cudaError_t launch_pdl(K kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = getenv("OSGPU_NO_PDL") ? 0 : 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

__device__ __forceinline__ void load_ptw(float2* tb, float2* tq, const float2* __restrict__ twP, int r,
                                         int T) {
  for (int i = threadIdx.x; i < r * T; i += blockDim.x) {
    const int s = i / T, t = i - s * T;
    tb[i] = twP[s * t];
  }
  for (int i = threadIdx.x; i < r * 16; i += blockDim.x) {
    const int s = i >> 4, q = i & 15;
    tq[i] = twP[s * T * q];
  }
}

// h_asm_split with the row data (Ey, b_hi, b_lo) already loaded.
__device__ __forceinline__ float2 h_asm_split_row(const PropArgs& a, float2 exc, float cah,
                                                  float cal, float sac, int kmc, int akk,
                                                  float2 ey, float bh, float blo) {
  if (akk > kmc) return make_float2(0.f, 0.f);
  const float s = sac + bh;
  const float q = sqrtf(fmaxf(1.f - s, 0.f));
  const float opq = 1.f + q;
  // denominator in [8, 64]: the fast division is within 2 ulp
  const float tau = __fdividef(a.Kf * (s * s * s) * (3.f + q), 8.f * opq * opq * opq);
  const float pr = cah * bh;
  const float er = fmaf(cah, bh, -pr);
  const float corr = er + (cah * blo + cal * bh);
  const float nq = rintf(pr * 0.159154943091895336f);
  float rr = fmaf(-nq, 6.28125f, pr);
  rr = fmaf(-nq, 1.93530717958647692e-3f, rr);
  const float th = rr + (corr - tau);
  float sn, cs;
  __sincosf(th, &sn, &cs);
  const float hr = exc.x * ey.x - exc.y * ey.y;
  const float hi = exc.x * ey.y + exc.y * ey.x;
  return make_float2(hr * cs - hi * sn, hr * sn + hi * cs);
}

// H(kx, |k_y|) for |k_y| <= Py/2 of an even transfer function (ASM split
// phase or Fresnel TF) into the shared table htab[rr * U + u], |k_y| = ry u + rr
// (row rr = residue class of |k_y| mod ry, so the pass-B reads are unit
// stride), by threads t0, t0 + nt, ...
template <int M>
__device__ __forceinline__ void build_htab(const PropArgs& a, int kx, float2* htab, int t0,
                                           int nt) {
  constexpr int U = M / 2 + 1;
  const int Py = a.ay.P, ry = a.ay.r;
  const int hh = Py / 2;
  if (a.engine == ENG_KEVEN) {  // quarter table of a kernel-spectrum plan
    const float2* kq = reinterpret_cast<const float2*>(a.kspec) + (size_t)kx * (hh + 1);
    for (int idx = t0; idx < ry * U; idx += nt) {
      const int rr = idx / U, u = idx - rr * U;
      const int ak = ry * u + rr;
      if (ak > hh) continue;
      float2 h = __ldg(kq + ak);
      if (a.conj_h) h.y = -h.y;
      htab[idx] = h;
    }
    return;
  }
  const bool asm_split = (a.engine == ENG_ASM);
  const float2 exc = a.Ex[kx];
  float cah = 0.f, cal = 0.f, sac = 0.f;
  int kmc = -1;
  if (asm_split) {
    cah = a.ca_hi[kx];
    cal = a.ca_lo[kx];
    sac = a.sa[kx];
    kmc = a.kmax[kx];
  }
  const float4* rt = reinterpret_cast<const float4*>(a.rowtab);
  constexpr int UNR = 4;
  for (int base = t0; base < ry * U; base += UNR * nt) {
    float4 rv[UNR];
    int ak[UNR];
#pragma unroll
    for (int k = 0; k < UNR; ++k) {  // issue the loads first
      const int idx = base + k * nt;
      const int rr = idx / U, u = idx - rr * U;
      ak[k] = ry * u + rr;
      rv[k] = (idx < ry * U && ak[k] <= hh) ? __ldg(rt + ak[k]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < UNR; ++k) {
      const int idx = base + k * nt;
      if (idx >= ry * U || ak[k] > hh) continue;
      const float2 ey = make_float2(rv[k].x, rv[k].y);
      float2 h;
      if (asm_split) {
        h = h_asm_split_row(a, exc, cah, cal, sac, kmc, ak[k], ey, rv[k].z, rv[k].w);
      } else {
        h = make_float2(exc.x * ey.x - exc.y * ey.y, exc.x * ey.y + exc.y * ey.x);
      }
      htab[idx] = h;
    }
  }
}

// ---------------------------------------------------------------- pass B

template <int M, int G>
__global__ void __launch_bounds__(Lay<M, G>::THREADS, Lay<M, G>::MINB)
    k_passB_v3(PropArgs a, int use_table) {
  constexpr int T = M / 16;
  constexpr int U = M / 2 + 1;
  constexpr int SB = Plan<M>::SMEM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Py = a.ay.P, ry = a.ay.r, ny = a.ny;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* col = tws + M;
  float2* bufs = col + M;
  float2* tb = bufs + G * SB;
  float2* tq = tb + ry * T;
  float2* htab = tq + ry * 16;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  // per-group barrier when a group is whole warps, else one CTA-wide barrier
  const int BAR_ID = (T % 32 == 0) ? 1 + g : 1;
  const int BAR_N = (T % 32 == 0) ? T : Lay<M, G>::THREADS;
  const int kx = blockIdx.x;
  float2* buf = bufs + g * SB;
  float2* W = reinterpret_cast<float2*>(a.work) + (size_t)kx * ny;
  const float2* twm = reinterpret_cast<const float2*>(a.tw_my);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Py);

  constexpr int NT = Lay<M, G>::THREADS;
#pragma unroll
  for (int k = 0; k < M / NT; ++k) {
    const int i = threadIdx.x + k * NT;
    col[i] = (i < ny) ? W[i] : make_float2(0.f, 0.f);
  }
  copy_stage_twiddles<M>(tws, twm, threadIdx.x, NT);
  load_ptw(tb, tq, twP, ry, T);
  if (use_table) build_htab<M>(a, kx, htab, threadIdx.x, NT);
  __syncthreads();

  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
  const int iters = (ry + G - 1) / G;
  for (int it = 0; it < iters; ++it) {
    const int t = g + G * it;
    const bool valid = t < ry;
    const int tt = valid ? t : 0;
    const float2 wb = tb[tt * T + tid];
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 x = valid ? col[tid + T * q] : make_float2(0.f, 0.f);
      if (tt > 0) x = cmul(x, cmul(wb, tq[tt * 16 + q]));
      v[q] = x;
    }
    fft1s<M, false>(v, buf, tws, tid, BAR_ID, BAR_N);
    // Table index of bin ky = ry (tid + T q) + tt: with Py = ry M, ky is in the
    // non-negative half (ky <= (Py - 1) / 2) exactly when q < 8; otherwise
    // |k_y| = Py - ky lies in residue class (ry - tt) mod ry (0 when tt = 0).
    const int hb_lo = tt * U + tid;
    const int hb_hi = (tt == 0) ? M - tid : (ry - tt) * U + M - 1 - tid;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int pp = tid + T * q;
      const int ky = ry * pp + tt;
      float2 h;
      if (use_table) {
        h = (q < 8) ? htab[hb_lo + T * q] : htab[hb_hi - T * q];
      } else if (a.engine == ENG_KSPEC) {
        h = __ldg(reinterpret_cast<const float2*>(a.kspec) + (size_t)kx * Py + ky);
        if (a.conj_h) h.y = -h.y;
      } else if (a.engine == ENG_KEVEN) {
        const int kxq = min(kx, a.ax.P - kx), kyq = min(ky, Py - ky);
        h = __ldg(reinterpret_cast<const float2*>(a.kspec) + (size_t)kxq * (Py / 2 + 1) + kyq);
        if (a.conj_h) h.y = -h.y;
      } else if (a.engine == ENG_KSEP) {
        h = cmul(__ldg(reinterpret_cast<const float2*>(a.hx) + kx),
                 __ldg(reinterpret_cast<const float2*>(a.hy) + ky));
        if (a.conj_h) h.y = -h.y;
      } else if (a.engine == ENG_ASM) {  // table did not fit: per bin
        const int kk = (ky <= (Py - 1) / 2) ? ky : ky - Py;
        h = h_asm_split(a, a.Ex[kx], a.ca_hi[kx], a.ca_lo[kx], a.sa[kx], a.kmax[kx], ky,
                        kk < 0 ? -kk : kk);
      } else if (a.engine == ENG_FRESNEL_TF) {
        const float2 ex = a.Ex[kx], ey = a.Ey[ky];
        h = make_float2(ex.x * ey.x - ex.y * ey.y, ex.x * ey.y + ex.y * ey.x);
      } else {
        h = make_float2((float)a.scale, 0.f);
      }
      v[q] = cmul(v[q], h);
    }
    fft1s<M, true>(v, buf, tws, tid, BAR_ID, BAR_N);
    if (valid) {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float2 y = v[q];
        if (tt > 0) y = cmulc(y, cmul(wb, tq[tt * 16 + q]));
        acc[q] = cadd(acc[q], y);
      }
    }
  }
  // reduce the G partial columns through the exchange buffers
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 16; ++q) buf[tid + T * q] = acc[q];
  __syncthreads();
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    float2 sum = bufs[j];
#pragma unroll
    for (int gg = 1; gg < G; ++gg) sum = cadd(sum, bufs[gg * SB + j]);
    W[j] = sum;
  }
}

// Pass B for an even transfer function with a shared-memory table, one CTA
// per mirror pair of columns (kx, Px - kx): H depends on fx only through
// fx^2 and fftfreq(Px - kx) = -fftfreq(kx) exactly, so the two columns have
// bit-identical tables and per-column factors.  The CTA builds the table
// once; group 0 then runs all ry sub-transforms of column kx and group 1
// those of column Px - kx (the self-mirrored columns 0 and Px/2 leave group 1
// idle), reading its column from global memory for each sub-transform and
// accumulating in registers.
template <int M>
__global__ void __launch_bounds__(Lay<M, 2>::THREADS, Lay<M, 2>::MINB)
    k_passB_pair(PropArgs a) {
  constexpr int T = M / 16;
  constexpr int U = M / 2 + 1;
  constexpr int SB = Plan<M>::SMEM;
  constexpr int NT = Lay<M, 2>::THREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Px = a.ax.P, ry = a.ay.r, ny = a.ny;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* bufs = tws + TwLay<M>::SIZE;
  float2* tb = bufs + 2 * SB;
  float2* tq = tb + ry * T;
  float2* htab = tq + ry * 16;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  const int BAR_ID = (T % 32 == 0) ? 1 + g : 1;
  const int BAR_N = (T % 32 == 0) ? T : NT;
  const int c = blockIdx.x;                        // 0 .. Px/2
  const bool mirrored = (c == 0 || 2 * c == Px);   // column equals its mirror
  const bool active = (g == 0) || !mirrored;
  const int kx = (g == 0) ? c : (mirrored ? c : Px - c);
  float2* buf = bufs + g * SB;
  const float2* twm = reinterpret_cast<const float2*>(a.tw_my);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Py);
  pdl_trigger();
  copy_stage_twiddles<M>(tws, twm, threadIdx.x, NT);
  load_ptw(tb, tq, twP, ry, T);
  build_htab<M>(a, c, htab, threadIdx.x, NT);
  pdl_wait();  // pass A's spectrum is complete
  __syncthreads();
  if (!active && T % 32 == 0) return;  // per-group barriers only from here on
  float2* col = reinterpret_cast<float2*>(a.work) + (size_t)kx * ny;
  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
  for (int t = 0; t < ry; ++t) {
    const float2 wb = tb[t * T + tid];
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      float2 x = (active && j < ny) ? col[j] : make_float2(0.f, 0.f);
      if (t > 0) x = cmul(x, cmul(wb, tq[t * 16 + q]));
      v[q] = x;
    }
    fft1s<M, false, true>(v, buf, tws, tid, BAR_ID, BAR_N);
    const int hb_lo = t * U + tid;
    const int hb_hi = (t == 0) ? M - tid : (ry - t) * U + M - 1 - tid;
#pragma unroll
    for (int q = 0; q < 16; ++q)
      v[q] = cmul(v[q], (q < 8) ? htab[hb_lo + T * q] : htab[hb_hi - T * q]);
    fft1s<M, true, true>(v, buf, tws, tid, BAR_ID, BAR_N);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 y = v[q];
      if (t > 0) y = cmulc(y, cmul(wb, tq[t * 16 + q]));
      acc[q] = cadd(acc[q], y);
    }
  }
  // every read of the column precedes this group's last barrier
  if (active) {
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      if (j < ny) col[j] = acc[q];
    }
  }
}

// ---------------------------------------------------------------- pass A

template <int M, int G>
__global__ void __launch_bounds__(Lay<M, G>::THREADS, Lay<M, G>::MINB) k_passA_v3(PropArgs a) {
  constexpr int T = M / 16;
  constexpr int SB = Plan<M>::SMEM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = a.nx, ny = a.ny, rx = a.ax.r;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* xin = tws + M;
  float2* bufs = xin + M;
  float2* tb = bufs + G * SB;
  float2* tq = tb + rx * T;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  // per-group barrier when a group is whole warps, else one CTA-wide barrier
  const int BAR_ID = (T % 32 == 0) ? 1 + g : 1;
  const int BAR_N = (T % 32 == 0) ? T : Lay<M, G>::THREADS;
  const int iy = blockIdx.x;
  float2* buf = bufs + g * SB;
  const float2* twm = reinterpret_cast<const float2*>(a.tw_mx);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Px);
  float2* W = reinterpret_cast<float2*>(a.work);
  constexpr int NT = Lay<M, G>::THREADS;
  constexpr int KS = M / NT;  // input samples per thread
  // all input loads first (no store or atomic between them), then one status
  // check, then the per-sample stage
  float2 xs[KS];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < KS; ++k) {
    const int j = threadIdx.x + k * NT;
    xs[k] = (j < nx) ? ld_in(a.in, a.in_c128, (size_t)iy * nx + j) : make_float2(0.f, 0.f);
  }
#pragma unroll
  for (int k = 0; k < KS; ++k) bad = bad || !isfinite(xs[k].x) || !isfinite(xs[k].y);
  if (a.status && bad) atomicOr(a.status, 1);
#pragma unroll
  for (int k = 0; k < KS; ++k) {
    const int j = threadIdx.x + k * NT;
    float2 x = xs[k];
    if (j < nx) {
      if (a.seed) {
        const size_t kk = (size_t)iy * nx + j;
        const double w = a.seed_f64 ? reinterpret_cast<const double*>(a.seed)[kk]
                                    : (double)reinterpret_cast<const float*>(a.seed)[kk];
        const float ws = (float)(w * a.seed_scale);
        x = make_float2(ws * x.x, ws * x.y);
      } else if (a.els.count && !a.adj) {
        if (a.els.fast) {
          x = apply_elements_fast(a.els, j, iy, x);
        } else {
          double re = x.x, im = x.y;
          apply_elements_exact(a.els, j, iy, nx, ny, a.dx, a.dy, re, im);
          x = make_float2((float)re, (float)im);
        }
      }
    }
    xin[j] = x;
  }
  copy_stage_twiddles<M>(tws, twm, threadIdx.x, NT);
  load_ptw(tb, tq, twP, rx, T);
  __syncthreads();
  const int iters = (rx + G - 1) / G;
  for (int it = 0; it < iters; ++it) {
    const int s = g + G * it;
    const bool valid = s < rx;
    const int ss = valid ? s : 0;
    const float2 wb = tb[ss * T + tid];
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 x = xin[tid + T * q];
      if (ss > 0) x = cmul(x, cmul(wb, tq[ss * 16 + q]));
      v[q] = x;
    }
    fft1s<M, false>(v, buf, tws, tid, BAR_ID, BAR_N);
    if (valid) {
#pragma unroll
      for (int q = 0; q < 16; ++q) W[(size_t)(rx * (tid + T * q) + s) * ny + iy] = v[q];
    }
  }
}

// ---------------------------------------------------------------- pass C

template <int M, int G, bool ADJ>
__global__ void __launch_bounds__(Lay<M, G>::THREADS, Lay<M, G>::MINB) k_passC_v3(PropArgs a) {
  constexpr int T = M / 16;
  constexpr int SB = Plan<M>::SMEM;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = a.nx, ny = a.ny, rx = a.ax.r;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* bufs = tws + M;
  float2* tb = bufs + G * SB;
  float2* tq = tb + rx * T;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  // per-group barrier when a group is whole warps, else one CTA-wide barrier
  const int BAR_ID = (T % 32 == 0) ? 1 + g : 1;
  const int BAR_N = (T % 32 == 0) ? T : Lay<M, G>::THREADS;
  const int iy = blockIdx.x;
  float2* buf = bufs + g * SB;
  const float2* twm = reinterpret_cast<const float2*>(a.tw_mx);
  const float2* twP = reinterpret_cast<const float2*>(a.tw_Px);
  const float2* W = reinterpret_cast<const float2*>(a.work);
  constexpr int NT = Lay<M, G>::THREADS;
  pdl_trigger();
  copy_stage_twiddles<M>(tws, twm, threadIdx.x, NT);
  load_ptw(tb, tq, twP, rx, T);
  pdl_wait();  // pass B's spectrum is complete
  const int iters = (rx + G - 1) / G;
  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
  __syncthreads();
  for (int it = 0; it < iters; ++it) {
    const int s = g + G * it;
    const bool valid = s < rx;
    const int ss = valid ? s : 0;
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q)
      v[q] = valid ? W[(size_t)(rx * (tid + T * q) + s) * ny + iy] : make_float2(0.f, 0.f);
    fft1s<M, true>(v, buf, tws, tid, BAR_ID, BAR_N);
    if (valid) {
      const float2 wb = tb[ss * T + tid];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float2 y = v[q];
        if (ss > 0) y = cmulc(y, cmul(wb, tq[ss * 16 + q]));
        acc[q] = cadd(acc[q], y);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 16; ++q) buf[tid + T * q] = acc[q];
  __syncthreads();
  for (int j = threadIdx.x; j < nx; j += blockDim.x) {
    float2 v = bufs[j];
#pragma unroll
    for (int gg = 1; gg < G; ++gg) v = cadd(v, bufs[gg * SB + j]);
    const size_t o = (size_t)iy * nx + j;
    if (ADJ) {  // adjoint element plane (a.adj)
      const float2 u = ld_in(a.adj_uin, a.adj_uin_c128, o);
      adjoint_plane<float>(a.els, a.adj_grad, j, iy, nx, ny, a.dx, a.dy, o, u.x, u.y, v.x, v.y);
    }
    if (a.status && (!isfinite(v.x) || !isfinite(v.y))) atomicOr(a.status, 2);
    if (a.out) {
      if (a.out_c128) reinterpret_cast<double2*>(a.out)[o] = make_double2(v.x, v.y);
      else reinterpret_cast<float2*>(a.out)[o] = v;
    }
    if (a.out_intensity) a.out_intensity[o] = v.x * v.x + v.y * v.y;
    if (a.out_intensity64) a.out_intensity64[o] = (double)v.x * v.x + (double)v.y * v.y;
  }
}

// ---------------------------------------------------- row tiles (pass A)
//
// The spectrum is column-major (W[kx * ny + iy]), so one row of it is a
// strided scatter with 8 bytes per 32-byte sector.  This variant gives a CTA
// R adjacent rows (one group of T threads per row, every sub-transform of
// its row in turn) and stores each sub-transform's R-row tile through shared
// memory in runs W[kx * ny + iy0 .. iy0 + R - 1] of 8 R bytes (R = 4: one
// full sector per request).  Needs ny % R == 0 and R T <= 512 threads.

// Per-sample input stage shared by the pass-A kernels.
__device__ __forceinline__ float2 pass_a_sample(const PropArgs& a, int j, int iy, float2 x) {
  if (a.seed) {
    const size_t kk = (size_t)iy * a.nx + j;
    const double w = a.seed_f64 ? reinterpret_cast<const double*>(a.seed)[kk]
                                : (double)reinterpret_cast<const float*>(a.seed)[kk];
    const float ws = (float)(w * a.seed_scale);
    return make_float2(ws * x.x, ws * x.y);
  }
  if (a.els.count && !a.adj) {
    if (a.els.fast) return apply_elements_fast(a.els, j, iy, x);
    double re = x.x, im = x.y;
    apply_elements_exact(a.els, j, iy, a.nx, a.ny, a.dx, a.dy, re, im);
    return make_float2((float)re, (float)im);
  }
  return x;
}

// Exchange-buffer stride of the row-tile kernel: the FFT's padded size plus
// 4 entries, so that buffers 0..3 start 0, 8, 16 and 24 banks apart and the
// paired-lane spectrum stores read them without bank conflicts.
template <int M>
__host__ __device__ constexpr int tile_stride() {
  return Plan<M>::SMEM + 4;
}

// The R input rows iy0 .. iy0 + R - 1 of a row-tile kernel (R T threads),
// each sample through the per-sample stage, into xin[r * M + j] (zero past
// nx).  Loads are batched, then one status check (returns true when a
// sample is not finite).
template <int M, int R>
__device__ __forceinline__ bool pass_a_tile_inputs(const PropArgs& a, float2* xin, int iy0) {
  constexpr int NT = R * (M / 16);
  const int nx = a.nx;
  constexpr int KS = R * M / NT;  // 16 samples per thread
  static_assert(KS <= 32, "sample mask is 32 bits");
  bool bad = false;
  {
    float2 xs[KS];
    int jx[KS], jy[KS];
    unsigned inb = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      const int e = threadIdx.x + k * NT;
      const int r = e / M, j = e - r * M;
      jx[k] = j;
      jy[k] = iy0 + r;
      if (j < nx) inb |= 1u << k;
      xs[k] = (j < nx) ? ld_in(a.in, a.in_c128, (size_t)(iy0 + r) * nx + j)
                       : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < KS; ++k) bad = bad || !isfinite(xs[k].x) || !isfinite(xs[k].y);
    // per-sample stage, each kind for all KS samples at once (loads in flight together)
    if (a.trans && !a.seed && !a.adj) {  // precomputed chain transmission
      float2 tr[KS];
#pragma unroll
      for (int k = 0; k < KS; ++k)
        tr[k] = (inb >> k & 1u) ? __ldg(a.trans + (size_t)jy[k] * nx + jx[k])
                                : make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < KS; ++k)
        if (inb >> k & 1u) xs[k] = cmul(xs[k], tr[k]);
    } else if (a.seed) {
#pragma unroll
      for (int k = 0; k < KS; ++k)
        if (inb >> k & 1u) xs[k] = pass_a_sample(a, jx[k], jy[k], xs[k]);
    } else if (a.els.count && !a.adj) {
      if (a.els.fast) {
        // two halves of KS / 2 samples (bounded register pressure)
        constexpr int KH = KS / 2;
        float2 xh[KH];
        int hx[KH], hy[KH];
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
#pragma unroll
          for (int k = 0; k < KH; ++k) {
            xh[k] = xs[hh * KH + k];
            hx[k] = jx[hh * KH + k];
            hy[k] = jy[hh * KH + k];
          }
          apply_elements_fast_k<KH>(a.els, hx, hy, (inb >> (hh * KH)) & ((1u << KH) - 1u), xh);
#pragma unroll
          for (int k = 0; k < KH; ++k) xs[hh * KH + k] = xh[k];
        }
      } else {
#pragma unroll
        for (int k = 0; k < KS; ++k)
          if (inb >> k & 1u) xs[k] = pass_a_sample(a, jx[k], jy[k], xs[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < KS; ++k) xin[threadIdx.x + k * NT] = xs[k];
  }
  return bad;
}

template <int M, int R>
__global__ void __launch_bounds__(R * (M / 16), R == 4 ? 1 : 2) k_passA_tile(PropArgs a) {
  constexpr int T = M / 16;
  constexpr int SBT = tile_stride<M>();
  constexpr int NT = R * T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ny = a.ny, rx = a.ax.r;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* xin = tws + TwLay<M>::SIZE;  // R rows of M
  float2* bufs = xin + R * M;
  float2* tb = bufs + R * SBT;
  float2* tq = tb + rx * T;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  const int iy0 = blockIdx.x * R;
  float2* buf = bufs + g * SBT;
  float2* W = reinterpret_cast<float2*>(a.work);
  pdl_trigger();
  copy_stage_twiddles<M>(tws, reinterpret_cast<const float2*>(a.tw_mx), threadIdx.x, NT);
  load_ptw(tb, tq, reinterpret_cast<const float2*>(a.tw_Px), rx, T);
  const bool bad = pass_a_tile_inputs<M, R>(a, xin, iy0);
  if (a.status && bad) atomicOr(a.status, 1);
  pdl_wait();  // the kernel before this one has completed (its workspace is ours to write)
  __syncthreads();
  const float2* xr = xin + g * M;
  for (int s = 0; s < rx; ++s) {
    const float2 wb = tb[s * T + tid];
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 x = xr[tid + T * q];
      if (s > 0) x = cmul(x, cmul(wb, tq[s * 16 + q]));
      v[q] = x;
    }
    fft1s<M, false>(v, buf, tws, tid, 1 + g, T);
    group_sync(1 + g, T);  // the transform's last reads of buf are done
#pragma unroll
    for (int q = 0; q < 16; ++q) buf[tid + T * q] = v[q];
    __syncthreads();
    // 16 bytes (two rows) per lane; with R = 4 the two lanes of a pair write
    // the two halves of one 32-byte run, so a warp store covers whole sectors
    constexpr int HV = R / 2;
    for (int h = threadIdx.x; h < HV * M; h += NT) {
      const int p = h / HV, hf = h - p * HV;
      float4* dst = reinterpret_cast<float4*>(W + (size_t)(rx * p + s) * ny + iy0) + hf;
      const float2 r0 = bufs[2 * hf * SBT + p], r1 = bufs[(2 * hf + 1) * SBT + p];
      *dst = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
    __syncthreads();
  }
}

// Pass A on 4-row tiles whose sub-transform tiles leave through TMA tensor
// stores: the CTA assembles tile s in shared memory in the spectrum's own
// order (p-major, the 4 rows of one kx adjacent: 32 bytes) and one thread
// stores it as M/256 boxes (iy 4 x s 1 x p 256) of the 3-D view
// (iy, s, p) -> W[(rx p + s) ny + iy].  The stores run in the async proxy
// while the CTA transforms the next sub-transform; the staging buffer is
// reused only after the previous tile's stores have read it.
template <int M>
__global__ void __launch_bounds__(4 * (M / 16), 1)
    k_passA_tstore(PropArgs a, const __grid_constant__ CUtensorMap wmap) {
  constexpr int R = 4;
  constexpr int T = M / 16;
  constexpr int SBT = tile_stride<M>();
  constexpr int NT = R * T;
  extern __shared__ __align__(128) unsigned char smem_atst[];
  const int rx = a.ax.r;
  float2* stage = reinterpret_cast<float2*>(smem_atst);  // M x R, p-major
  float2* tws = stage + R * M;
  float2* xin = tws + TwLay<M>::SIZE;  // R rows of M
  float2* bufs = xin + R * M;
  float2* tb = bufs + R * SBT;
  float2* tq = tb + rx * T;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  const int iy0 = blockIdx.x * R;
  float2* buf = bufs + g * SBT;
  if (threadIdx.x == 0) tma::prefetch_map(&wmap);
  pdl_trigger();
  copy_stage_twiddles<M>(tws, reinterpret_cast<const float2*>(a.tw_mx), threadIdx.x, NT);
  load_ptw(tb, tq, reinterpret_cast<const float2*>(a.tw_Px), rx, T);
  const bool bad = pass_a_tile_inputs<M, R>(a, xin, iy0);
  if (a.status && bad) atomicOr(a.status, 1);
  pdl_wait();  // the kernel before this one has completed (its workspace is ours to write)
  __syncthreads();
  const float2* xr = xin + g * M;
  for (int s = 0; s < rx; ++s) {
    const float2 wb = tb[s * T + tid];
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 x = xr[tid + T * q];
      if (s > 0) x = cmul(x, cmul(wb, tq[s * 16 + q]));
      v[q] = x;
    }
    fft1s<M, false>(v, buf, tws, tid, 1 + g, T);
    group_sync(1 + g, T);  // the transform's last reads of buf are done
#pragma unroll
    for (int q = 0; q < 16; ++q) buf[tid + T * q] = v[q];
    if (threadIdx.x == 0) tma::bulk_wait_read();  // the previous tile has left the stage
    __syncthreads();
    // stage[4 p + r] = row r's bin p: 16 bytes (two rows) per lane, dense
    for (int h = threadIdx.x; h < 2 * M; h += NT) {
      const int p = h >> 1, hf = h & 1;
      const float2 r0 = bufs[2 * hf * SBT + p], r1 = bufs[(2 * hf + 1) * SBT + p];
      reinterpret_cast<float4*>(stage)[h] = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
    tma::fence_async_shared();  // this thread's stage writes, before the stores read them
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll 1
      for (int b = 0; b < M / 256; ++b) tma::store_3d(&wmap, stage + b * 256 * R, iy0, s, 256 * b);
      tma::bulk_commit();
    }
  }
  if (threadIdx.x == 0) tma::bulk_wait_all();  // the last tile is written before the CTA leaves
}

// Pass A, persistent, with the next tile's rows prefetched by bulk async
// copies: for a complex64 input with a precomputed chain transmission, the
// CTA (4 groups, one row each) walks 4-row tiles; the tile's 4 input rows
// and 4 transmission rows (each a contiguous 4 nx-sample run) arrive in
// shared memory through two untiled bulk copies (cp.async.bulk, one mbarrier
// each).  The transmission run is consumed first (x t formed in place), so
// the next tile's transmission is requested at once; the input run is free
// after the last sub-transform has read it, and the next tile's input is
// requested there, so both copies overlap the current tile's transforms.
// The sub-transform tiles leave as in k_passA_tile (32-byte runs of the
// column-major spectrum).  Every wait is bounded (status bit 8 on timeout).
template <int M>
__global__ void __launch_bounds__(4 * (M / 16), 1) k_passA_bulk(PropArgs a) {
  constexpr int R = 4;
  constexpr int T = M / 16;
  constexpr int SBT = tile_stride<M>();
  constexpr int NT = R * T;
  extern __shared__ __align__(128) unsigned char smem_abulk[];
  const int nx = a.nx, ny = a.ny, rx = a.ax.r;
  const int n_tiles = ny / R;
  const unsigned run_bytes = (unsigned)(R * nx) * 8u;
  float2* xin = reinterpret_cast<float2*>(smem_abulk);  // R rows of nx (input, then x t)
  float2* trs = xin + R * M;                          // R rows of nx (transmission)
  float2* tws = trs + R * M;
  float2* bufs = tws + TwLay<M>::SIZE;
  float2* tb = bufs + R * SBT;
  float2* tq = tb + rx * T;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(tq + rx * 16);  // [in, trans]
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  float2* buf = bufs + g * SBT;
  float2* W = reinterpret_cast<float2*>(a.work);
  const float2* gin = reinterpret_cast<const float2*>(a.in);
  if (threadIdx.x == 0) {
    tma::mbar_init(bar, 1);
    tma::mbar_init(bar + 1, 1);
  }
  pdl_trigger();
  copy_stage_twiddles<M>(tws, reinterpret_cast<const float2*>(a.tw_mx), threadIdx.x, NT);
  load_ptw(tb, tq, reinterpret_cast<const float2*>(a.tw_Px), rx, T);
  __syncthreads();  // barriers initialised
  // The transmission comes from the auxiliary stream, joined before this
  // launch, so its first run is requested at once; the input may be the
  // output of the kernel just before this one, so it waits for that kernel.
  int tile = blockIdx.x;
  if (tile < n_tiles && threadIdx.x == 0) {
    tma::mbar_expect_tx(bar + 1, run_bytes);
    tma::load_bulk(trs, a.trans + (size_t)tile * R * nx, run_bytes, bar + 1);
  }
  pdl_wait();  // the kernel before this one has completed and its memory is visible
  if (tile < n_tiles && threadIdx.x == 0) {
    tma::mbar_expect_tx(bar, run_bytes);
    tma::load_bulk(xin, gin + (size_t)tile * R * nx, run_bytes, bar);
  }
  unsigned ph_in = 0, ph_tr = 0;
  bool bad = false;
  for (; tile < n_tiles; tile += gridDim.x) {
    const bool arrived = tma::mbar_wait(bar + 1, ph_tr) && tma::mbar_wait(bar, ph_in);
    if (!__syncthreads_and(arrived)) {
      if (threadIdx.x == 0) {
        if (a.status) atomicOr(a.status, 8);
        tma::mbar_wait(bar + 1, ph_tr);
        tma::mbar_wait(bar, ph_in);
      }
      return;
    }
    ph_in ^= 1u;
    ph_tr ^= 1u;
    // x t in place (R nx staged samples, 16 per thread when nx == M)
    for (int e = threadIdx.x; e < R * nx; e += NT) {
      const float2 x = xin[e];
      bad = bad || !isfinite(x.x) || !isfinite(x.y);
      xin[e] = cmul(x, trs[e]);
    }
    __syncthreads();  // the transmission run is consumed
    const int nxt = tile + gridDim.x;
    if (nxt < n_tiles && threadIdx.x == 0) {
      tma::mbar_expect_tx(bar + 1, run_bytes);
      tma::load_bulk(trs, a.trans + (size_t)nxt * R * nx, run_bytes, bar + 1);
    }
    const int iy0 = tile * R;
    const float2* xr = xin + g * nx;
    for (int s = 0; s < rx; ++s) {
      const float2 wb = tb[s * T + tid];
      float2 v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int j = tid + T * q;
        float2 x = (j < nx) ? xr[j] : make_float2(0.f, 0.f);
        if (s > 0) x = cmul(x, cmul(wb, tq[s * 16 + q]));
        v[q] = x;
      }
      fft1s<M, false>(v, buf, tws, tid, 1 + g, T);
      group_sync(1 + g, T);  // the transform's last reads of buf are done
#pragma unroll
      for (int q = 0; q < 16; ++q) buf[tid + T * q] = v[q];
      __syncthreads();
      if (s == rx - 1 && nxt < n_tiles && threadIdx.x == 0) {
        // every group has read its row for the last time: the next input run
        tma::mbar_expect_tx(bar, run_bytes);
        tma::load_bulk(xin, gin + (size_t)nxt * R * nx, run_bytes, bar);
      }
      constexpr int HV = R / 2;
      for (int h = threadIdx.x; h < HV * M; h += NT) {
        const int p = h / HV, hf = h - p * HV;
        float4* dst = reinterpret_cast<float4*>(W + (size_t)(rx * p + s) * ny + iy0) + hf;
        const float2 r0 = bufs[2 * hf * SBT + p], r1 = bufs[(2 * hf + 1) * SBT + p];
        *dst = make_float4(r0.x, r0.y, r1.x, r1.y);
      }
      __syncthreads();
    }
  }
  if (a.status && bad) atomicOr(a.status, 1);
}

// Pass C on R-row tiles: the CTA stages each sub-transform's R-row tile of
// the column-major spectrum through shared memory, read in runs
// W[kx * ny + iy0 .. iy0 + R - 1] of 8 R bytes (with R = 4 the two lanes of a
// pair read the two halves of one 32-byte sector), then group g transforms
// row iy0 + g and accumulates it in registers; the epilogue writes the
// group's row directly (samples tid + T q).  Needs ny % R == 0.
template <int M, int R, bool ADJ>
__global__ void __launch_bounds__(R * (M / 16), R == 4 ? 1 : 2) k_passC_tile(PropArgs a) {
  constexpr int T = M / 16;
  constexpr int SBT = tile_stride<M>();
  constexpr int NT = R * T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = a.nx, ny = a.ny, rx = a.ax.r;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* bufs = tws + TwLay<M>::SIZE;
  float2* tb = bufs + R * SBT;
  float2* tq = tb + rx * T;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  const int iy0 = blockIdx.x * R;
  float2* buf = bufs + g * SBT;
  const float2* W = reinterpret_cast<const float2*>(a.work);
  pdl_trigger();
  copy_stage_twiddles<M>(tws, reinterpret_cast<const float2*>(a.tw_mx), threadIdx.x, NT);
  load_ptw(tb, tq, reinterpret_cast<const float2*>(a.tw_Px), rx, T);
  pdl_wait();  // pass B's spectrum is complete
  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
  constexpr int HV = R / 2;
  for (int s = 0; s < rx; ++s) {
    // the tile of sub-transform s into row buffers (natural order, padded index)
#pragma unroll 4
    for (int h = threadIdx.x; h < HV * M; h += NT) {
      const int p = h / HV, hf = h - p * HV;
      const float4 v =
          __ldg(reinterpret_cast<const float4*>(W + (size_t)(rx * p + s) * ny + iy0) + hf);
      const int pp = p + (p >> 4);
      bufs[2 * hf * SBT + pp] = make_float2(v.x, v.y);
      bufs[(2 * hf + 1) * SBT + pp] = make_float2(v.z, v.w);
    }
    __syncthreads();
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = tid + T * q;
      v[q] = buf[j + (j >> 4)];
    }
    fft1s<M, true, true>(v, buf, tws, tid, 1 + g, T);
    const float2 wb = tb[s * T + tid];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 y = v[q];
      if (s > 0) y = cmulc(y, cmul(wb, tq[s * 16 + q]));
      acc[q] = cadd(acc[q], y);
    }
    __syncthreads();  // every group is done with its buffer before the next tile
  }
  const int iy = iy0 + g;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = tid + T * q;
    if (j >= nx) continue;
    float2 v = acc[q];
    const size_t o = (size_t)iy * nx + j;
    if (ADJ) {  // adjoint element plane (a.adj)
      const float2 u = ld_in(a.adj_uin, a.adj_uin_c128, o);
      adjoint_plane<float>(a.els, a.adj_grad, j, iy, nx, ny, a.dx, a.dy, o, u.x, u.y, v.x, v.y);
    }
    if (a.status && (!isfinite(v.x) || !isfinite(v.y))) atomicOr(a.status, 2);
    if (a.out) {
      if (a.out_c128) reinterpret_cast<double2*>(a.out)[o] = make_double2(v.x, v.y);
      else reinterpret_cast<float2*>(a.out)[o] = v;
    }
    if (a.out_intensity) a.out_intensity[o] = v.x * v.x + v.y * v.y;
    if (a.out_intensity64) a.out_intensity64[o] = (double)v.x * v.x + (double)v.y * v.y;
  }
}

// Pass C, persistent and software-pipelined: a CTA of two row groups walks
// its 2-row tiles; the next sub-transform's tile (2 rows x M columns, 16 bytes
// per column) is copied into a shared staging buffer with cp.async while the
// groups transform the current one, so the strided spectrum reads overlap
// the FFTs.  Needs ny % 2 == 0.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// The adjoint epilogue's inputs of output row iy (forward field, element
// transmission, gradient accumulator) requested into L2 at the start of the
// row's tile, one prefetch per 128-byte line, so that pass_c_store finds
// them there after the row's sub-transforms.
template <int M, bool ADJ>
__device__ __forceinline__ void pass_c_prefetch(const PropArgs& a, int iy, int tid) {
  if (!ADJ || !a.trans || a.els.count != 1) return;
  constexpr int T = M / 16;
  const int nx = a.nx;
  const int ue = a.adj_uin_c128 ? 8 : 16;  // samples per 128-byte line of the field
  const float* grad = reinterpret_cast<const float*>(a.adj_grad[0]);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = tid + T * q;
    if (j >= nx) continue;
    const size_t o = (size_t)iy * nx + j;
    if (j % ue == 0) {
      const char* pu = static_cast<const char*>(a.adj_uin) + o * (a.adj_uin_c128 ? 16 : 8);
      asm volatile("prefetch.global.L2 [%0];" ::"l"(pu));
    }
    if (j % 16 == 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.trans + o));
    if (grad && j % 32 == 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(grad + o));
  }
}

// Pass C epilogue of one output row held by a group (samples tid + T q):
// the adjoint element plane, the finiteness status, the field and the
// optional intensities.
template <int M, bool ADJ>
__device__ __forceinline__ void pass_c_store(const PropArgs& a, const float2 (&acc)[16], int iy,
                                             int tid) {
  constexpr int T = M / 16;
  const int nx = a.nx, ny = a.ny;
  if (ADJ && a.trans && a.els.count == 1) {
    // one element with its precomputed transmission t: v = t u,
    // grad += -2 Im(conj(mu) v), mu <- conj(t) mu (adjoint_plane's steps).
    // The loads of 8 samples go out together, ahead of their stores (a
    // store may alias a later load, so the compiler keeps them in order).
    float* grad = reinterpret_cast<float*>(a.adj_grad[0]);
    constexpr int CH = 8;
#pragma unroll
    for (int c0 = 0; c0 < 16; c0 += CH) {
      float2 u[CH], t[CH];
      float gv[CH];
#pragma unroll
      for (int k = 0; k < CH; ++k) {
        const int j = tid + T * (c0 + k);
        const size_t o = (size_t)iy * nx + j;
        u[k] = t[k] = make_float2(0.f, 0.f);
        gv[k] = 0.f;
        if (j < nx) {
          u[k] = ld_in(a.adj_uin, a.adj_uin_c128, o);
          t[k] = __ldg(a.trans + o);
          if (grad) gv[k] = grad[o];
        }
      }
#pragma unroll
      for (int k = 0; k < CH; ++k) {
        const int j = tid + T * (c0 + k);
        if (j >= nx) continue;
        const size_t o = (size_t)iy * nx + j;
        float2 v = acc[c0 + k];
        const float vr = u[k].x * t[k].x - u[k].y * t[k].y;
        const float vi = u[k].x * t[k].y + u[k].y * t[k].x;
        if (grad) grad[o] = gv[k] + -2.f * (v.x * vi + (-v.y) * vr);
        const float nr = v.x * t[k].x - v.y * (-t[k].y), ni = v.x * (-t[k].y) + v.y * t[k].x;
        v = make_float2(nr, ni);
        if (a.status && (!isfinite(v.x) || !isfinite(v.y))) atomicOr(a.status, 2);
        if (a.out) {
          if (a.out_c128) reinterpret_cast<double2*>(a.out)[o] = make_double2(v.x, v.y);
          else reinterpret_cast<float2*>(a.out)[o] = v;
        }
        if (a.out_intensity) a.out_intensity[o] = v.x * v.x + v.y * v.y;
        if (a.out_intensity64) a.out_intensity64[o] = (double)v.x * v.x + (double)v.y * v.y;
      }
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = tid + T * q;
    if (j >= nx) continue;
    float2 v = acc[q];
    const size_t o = (size_t)iy * nx + j;
    if (ADJ) {  // adjoint element plane (a.adj), general chain
      const float2 u = ld_in(a.adj_uin, a.adj_uin_c128, o);
      adjoint_plane<float>(a.els, a.adj_grad, j, iy, nx, ny, a.dx, a.dy, o, u.x, u.y, v.x, v.y);
    }
    if (a.status && (!isfinite(v.x) || !isfinite(v.y))) atomicOr(a.status, 2);
    if (a.out) {
      if (a.out_c128) reinterpret_cast<double2*>(a.out)[o] = make_double2(v.x, v.y);
      else reinterpret_cast<float2*>(a.out)[o] = v;
    }
    if (a.out_intensity) a.out_intensity[o] = v.x * v.x + v.y * v.y;
    if (a.out_intensity64) a.out_intensity64[o] = (double)v.x * v.x + (double)v.y * v.y;
  }
}

template <int M, bool ADJ>
__global__ void __launch_bounds__(2 * (M / 16), 2) k_passC_pipe(PropArgs a) {
  constexpr int T = M / 16;
  constexpr int SBT = tile_stride<M>();
  constexpr int NT = 2 * T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ny = a.ny, rx = a.ax.r;
  const int n_tiles = ny / 2;
  float2* tws = reinterpret_cast<float2*>(smem_raw);
  float2* bufs = tws + TwLay<M>::SIZE;
  float4* stage = reinterpret_cast<float4*>(bufs + 2 * SBT);  // column p: (row 0, row 1)
  float2* tb = reinterpret_cast<float2*>(stage + M);
  float2* tq = tb + rx * T;
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  float2* buf = bufs + g * SBT;
  const float2* W = reinterpret_cast<const float2*>(a.work);
  pdl_trigger();
  copy_stage_twiddles<M>(tws, reinterpret_cast<const float2*>(a.tw_mx), threadIdx.x, NT);
  load_ptw(tb, tq, reinterpret_cast<const float2*>(a.tw_Px), rx, T);
  pdl_wait();  // pass B's spectrum is complete
  auto issue = [&](int tile, int s) {
    const float2* src = W + (size_t)s * ny + 2 * tile;
    for (int p = threadIdx.x; p < M; p += NT) cp_async16(stage + p, src + (size_t)rx * p * ny);
    cp_async_commit();
  };
  int tile = blockIdx.x;
  if (tile < n_tiles) issue(tile, 0);
  for (; tile < n_tiles; tile += gridDim.x) {
    pass_c_prefetch<M, ADJ>(a, 2 * tile + g, tid);
    float2 acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
    for (int s = 0; s < rx; ++s) {
      cp_async_wait_all();
      __syncthreads();  // the tile of sub-transform s is in the staging buffer
      float2 v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const float4 t = stage[tid + T * q];
        v[q] = g ? make_float2(t.z, t.w) : make_float2(t.x, t.y);
      }
      __syncthreads();  // every group holds its row: the buffer takes the next tile
      int ns = s + 1, nt = tile;
      if (ns == rx) {
        ns = 0;
        nt = tile + gridDim.x;
      }
      if (nt < n_tiles) issue(nt, ns);
      // twiddles by products (TWREC): fewer shared-memory loads, so the pass
      // leaves more of the LSU to the other lane's co-resident pass-B CTAs
      fft1s<M, true, true>(v, buf, tws, tid, 1 + g, T);
      const float2 wb = tb[s * T + tid];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float2 y = v[q];
        if (s > 0) y = cmulc(y, cmul(wb, tq[s * 16 + q]));
        acc[q] = cadd(acc[q], y);
      }
    }
    pass_c_store<M, ADJ>(a, acc, 2 * tile + g, tid);
  }
  cp_async_wait_all();  // no copy outlives the CTA
}

// Pass C with TMA-staged tiles: the same persistent 2-row-tile walk as
// k_passC_pipe, but each sub-transform's tile (2 rows x M spectral columns,
// column-major spectrum) arrives through the tensor-memory accelerator: one
// thread issues M / 256 three-dimensional box copies (iy: 2, s: 1, p: 256 of
// the spectrum viewed as [p][s][iy]) into the staging buffer, completing an
// mbarrier with the tile's bytes, while the groups transform the previous
// tile.  The strided gather costs no load instructions, registers or LSU
// issue slots in the threads.  Every wait is bounded: a tile that does not
// arrive sets status bit 8 and the CTA leaves.
template <int M, bool ADJ>
__global__ void __launch_bounds__(2 * (M / 16), 2)
    k_passC_tma(PropArgs a, const __grid_constant__ CUtensorMap wmap) {
  constexpr int T = M / 16;
  constexpr int SBT = tile_stride<M>();
  constexpr int NT = 2 * T;
  constexpr unsigned TILE_BYTES = (unsigned)M * 16u;
  extern __shared__ __align__(128) unsigned char smem_ctma[];
  const int ny = a.ny, rx = a.ax.r;
  const int n_tiles = ny / 2;
  float4* stage = reinterpret_cast<float4*>(smem_ctma);  // column p: (row 0, row 1); 128-B aligned
  float2* tws = reinterpret_cast<float2*>(stage + M);
  float2* bufs = tws + TwLay<M>::SIZE;
  float2* tb = bufs + 2 * SBT;
  float2* tq = tb + rx * T;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(tq + rx * 16);
  const int g = threadIdx.x / T;
  const int tid = threadIdx.x - g * T;
  float2* buf = bufs + g * SBT;
  if (threadIdx.x == 0) {
    tma::prefetch_map(&wmap);
    tma::mbar_init(bar, 1);
  }
  pdl_trigger();
  copy_stage_twiddles<M>(tws, reinterpret_cast<const float2*>(a.tw_mx), threadIdx.x, NT);
  load_ptw(tb, tq, reinterpret_cast<const float2*>(a.tw_Px), rx, T);
  pdl_wait();  // pass B's spectrum is complete
  __syncthreads();  // the barrier is initialised
  auto issue = [&](int tile, int s) {  // thread 0 only
    tma::mbar_expect_tx(bar, TILE_BYTES);
#pragma unroll 1
    for (int b = 0; b < M / 256; ++b)
      tma::load_3d(stage + 256 * b, &wmap, 2 * tile, s, 256 * b, bar);
  };
  unsigned phase = 0;
  int tile = blockIdx.x;
  if (tile < n_tiles && threadIdx.x == 0) issue(tile, 0);
  for (; tile < n_tiles; tile += gridDim.x) {
    pass_c_prefetch<M, ADJ>(a, 2 * tile + g, tid);
    float2 acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.f, 0.f);
    for (int s = 0; s < rx; ++s) {
      const bool arrived = tma::mbar_wait(bar, phase);
      if (!__syncthreads_and(arrived)) {  // the whole CTA leaves together
        if (threadIdx.x == 0) {
          if (a.status) atomicOr(a.status, 8);
          tma::mbar_wait(bar, phase);  // a late copy lands before the CTA's memory is reused
        }
        return;
      }
      phase ^= 1u;
      float2 v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const float4 t = stage[tid + T * q];
        v[q] = g ? make_float2(t.z, t.w) : make_float2(t.x, t.y);
      }
      __syncthreads();  // every group holds its row: the buffer takes the next tile
      int ns = s + 1, nt = tile;
      if (ns == rx) {
        ns = 0;
        nt = tile + gridDim.x;
      }
      if (nt < n_tiles && threadIdx.x == 0) issue(nt, ns);
      // twiddles by products (TWREC): fewer shared-memory loads, so the pass
      // leaves more of the LSU to the other lane's co-resident pass-B CTAs
      fft1s<M, true, true>(v, buf, tws, tid, 1 + g, T);
      const float2 wb = tb[s * T + tid];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float2 y = v[q];
        if (s > 0) y = cmulc(y, cmul(wb, tq[s * 16 + q]));
        acc[q] = cadd(acc[q], y);
      }
    }
    pass_c_store<M, ADJ>(a, acc, 2 * tile + g, tid);
  }
}

template <int M>
constexpr bool r4_ok() {
  return M >= 512 && M <= 2048;
}

template <int M, int R>
size_t smem_tile(int r) {
  constexpr int T = M / 16;
  return ((size_t)TwLay<M>::SIZE + R * (size_t)tile_stride<M>() + (size_t)r * (T + 16) +
          R * (size_t)M) * sizeof(float2);
}

template <int M, int R>
cudaError_t launch_A_tile(const PropArgs& a, cudaStream_t st) {
  const size_t smem = smem_tile<M, R>(a.ax.r);
  cudaError_t e = cudaFuncSetAttribute(k_passA_tile<M, R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  return launch_pdl(k_passA_tile<M, R>, dim3(a.ny / R), dim3(R * (M / 16)), smem, st, a);
}

constexpr size_t kMaxSmemB = 232448;

template <int M, int G>
size_t smem_v3(int kind, int r, int table) {
  constexpr int T = M / 16;
  size_t n = (size_t)M + (size_t)G * Plan<M>::SMEM + (size_t)r * (T + 16);
  if (kind != 2) n += M;  // staged row (A) or column (B)
  if (kind == 1 && table) n += (size_t)r * (M / 2 + 1);
  return n * sizeof(float2);
}

template <int M, int G>
cudaError_t launchB_mg(const PropArgs& a, int use_table, cudaStream_t st) {
  const size_t smem = smem_v3<M, G>(1, a.ay.r, use_table);
  cudaError_t e = cudaFuncSetAttribute(k_passB_v3<M, G>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  k_passB_v3<M, G><<<a.ax.P, Lay<M, G>::THREADS, smem, st>>>(a, use_table);
  return cudaGetLastError();
}

template <int M, int G>
cudaError_t launchA_mg(const PropArgs& a, cudaStream_t st) {
  const size_t smem = smem_v3<M, G>(0, a.ax.r, 0);
  cudaError_t e = cudaFuncSetAttribute(k_passA_v3<M, G>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  k_passA_v3<M, G><<<a.ny, Lay<M, G>::THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int M, int G, bool ADJ>
cudaError_t launchC_mga(const PropArgs& a, cudaStream_t st) {
  const size_t smem = smem_v3<M, G>(2, a.ax.r, 0);
  cudaError_t e = cudaFuncSetAttribute(k_passC_v3<M, G, ADJ>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  return launch_pdl(k_passC_v3<M, G, ADJ>, dim3(a.ny), dim3(Lay<M, G>::THREADS), smem, st, a);
}

template <int M, int G>
cudaError_t launchC_mg(const PropArgs& a, cudaStream_t st) {
  return a.adj ? launchC_mga<M, G, true>(a, st) : launchC_mga<M, G, false>(a, st);
}

// Largest group count <= want (and <= r) whose shared memory fits, with
// 32..512 threads per CTA (one warp at least; at most 512 so that the
// 128-register budget of the FFT holds).
template <int M>
int pick_groups(int kind, int r, int table, int want) {
  constexpr int T = M / 16;
  int g = want;
  while (g > r && g > 1) g >>= 1;
  while (g > 1 && g * T > 512) g >>= 1;
  if (g * T < 32) g = 32 / T;
  while (g > 1 && g * T > 32) {
    const size_t b = g == 4 ? smem_v3<M, 4>(kind, r, table)
                            : smem_v3<M, 2>(kind, r, table);
    if (b <= kMaxSmemB) break;
    g >>= 1;
  }
  return g;
}

template <int M>
size_t smem_pair(int r) {
  constexpr int T = M / 16;
  return ((size_t)TwLay<M>::SIZE + 2 * (size_t)Plan<M>::SMEM + (size_t)r * (T + 16) +
          (size_t)r * (M / 2 + 1)) * sizeof(float2);
}

const char* const kNamesA[SA_N] = {"default", "bulk", "tile4", "tile2", "g1", "g2", "g4",
                                    "tstore"};
const char* const kNamesB[SB_N] = {"default", "pair", "g1", "g2", "g4"};
const char* const kNamesC[SC_N] = {"default", "tma", "pipe", "tile2", "tile4", "g1", "g2", "g4"};

// Variant forced by the environment (OSGPU_SCHED_A/_B/_C = name), else 0.
int env_variant(const char* var, const char* const* names, int n) {
  const char* e = getenv(var);
  if (!e) return 0;
  for (int v = 1; v < n; ++v)
    if (!strcmp(e, names[v])) return v;
  return 0;
}

template <int M>
bool B_even(const PropArgs& a) {
  return ((a.engine == ENG_ASM || a.engine == ENG_FRESNEL_TF) && a.h_mode == 1) ||
         a.engine == ENG_KEVEN;
}

template <int M>
int B_table(const PropArgs& a) {
  return B_even<M>(a) && smem_v3<M, 1>(1, a.ay.r, 1) <= kMaxSmemB ? 1 : 0;
}

template <int M>
bool B_ok(int v, const PropArgs& a) {
  if (v == SB_PAIR)
    return B_even<M>(a) && (a.ax.P % 2) == 0 && smem_pair<M>(a.ay.r) <= kMaxSmemB;
  const int want = v == SB_G1 ? 1 : v == SB_G2 ? 2 : 4;
  return pick_groups<M>(1, a.ay.r, B_table<M>(a), want) == want;
}

// Default: one CTA per mirror pair of columns for even transfer functions
// (one H table for two columns), else the generic column kernel.
template <int M>
int B_default(const PropArgs& a) {
  if (B_ok<M>(SB_PAIR, a)) return SB_PAIR;
  const int g = pick_groups<M>(1, a.ay.r, B_table<M>(a), 2);
  return g == 4 ? SB_G4 : g == 2 ? SB_G2 : SB_G1;
}

template <int M>
cudaError_t launch_B(const PropArgs& a, cudaStream_t st) {
  int v = env_variant("OSGPU_SCHED_B", kNamesB, SB_N);
  if (!v || !B_ok<M>(v, a)) v = a.sched.b;
  if (!v || !B_ok<M>(v, a)) v = B_default<M>(a);
  if (v == SB_PAIR) {
    const size_t smem = smem_pair<M>(a.ay.r);
    cudaError_t e = cudaFuncSetAttribute(k_passB_pair<M>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ++launch_counter();
    return launch_pdl(k_passB_pair<M>, dim3(a.ax.P / 2 + 1), dim3(Lay<M, 2>::THREADS), smem, st,
                      a);
  }
  const int table = B_table<M>(a);
  if (v == SB_G4) return launchB_mg<M, 4>(a, table, st);
  if (v == SB_G2) return launchB_mg<M, 2>(a, table, st);
  return launchB_mg<M, 1>(a, table, st);
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

template <int M>
size_t smem_abulk(int r) {
  constexpr int T = M / 16;
  return (8 * (size_t)M + (size_t)TwLay<M>::SIZE + 4 * (size_t)tile_stride<M>() +
          (size_t)r * (T + 16)) * sizeof(float2) + 16;
}

template <int M>
cudaError_t launch_A_bulk(const PropArgs& a, cudaStream_t st) {
  const size_t smem = smem_abulk<M>(a.ax.r);
  cudaError_t e = cudaFuncSetAttribute(k_passA_bulk<M>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = std::min(a.ny / 4, sm_count());
  ++launch_counter();
  return launch_pdl(k_passA_bulk<M>, dim3(grid), dim3(4 * (M / 16)), smem, st, a);
}

template <int M>
size_t smem_atstore(int r) {
  return smem_tile<M, 4>(r) + 4 * (size_t)M * sizeof(float2);
}

// cudaErrorNotSupported when the tensor map cannot be encoded (the caller
// then takes the 4-row tile kernel).
template <int M>
cudaError_t launch_A_tstore(const PropArgs& a, cudaStream_t st) {
  const unsigned long long dims[3] = {(unsigned long long)a.ny, (unsigned long long)a.ax.r,
                                      (unsigned long long)M};
  const unsigned long long strides[2] = {(unsigned long long)a.ny * 8ull,
                                         (unsigned long long)a.ax.r * a.ny * 8ull};
  const unsigned box[3] = {4u, 1u, 256u};
  CUtensorMap map;
  if (!encode_map_3d_c64(&map, a.work, dims, strides, box)) return cudaErrorNotSupported;
  const size_t smem = smem_atstore<M>(a.ax.r);
  cudaError_t e = cudaFuncSetAttribute(k_passA_tstore<M>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  return launch_pdl(k_passA_tstore<M>, dim3(a.ny / 4), dim3(4 * (M / 16)), smem, st, a, map);
}

template <int M>
bool A_ok(int v, const PropArgs& a) {
  if (v == SA_TSTORE)
    return r4_ok<M>() && a.ny % 4 == 0 && reinterpret_cast<uintptr_t>(a.work) % 16 == 0 &&
           smem_atstore<M>(a.ax.r) <= kMaxSmemB;
  if (v == SA_BULK || v == SA_TILE4 || v == SA_TILE2) {
    if constexpr (!r4_ok<M>()) return false;
    if (v == SA_BULK)
      return a.trans && !a.seed && !a.adj && !a.in_c128 && a.ny % 4 == 0 &&
             reinterpret_cast<uintptr_t>(a.in) % 16 == 0 &&
             reinterpret_cast<uintptr_t>(a.trans) % 16 == 0 && smem_abulk<M>(a.ax.r) <= kMaxSmemB;
    if (v == SA_TILE4) return a.ny % 4 == 0 && smem_tile<M, 4>(a.ax.r) <= kMaxSmemB;
    return a.ny % 2 == 0 && smem_tile<M, 2>(a.ax.r) <= kMaxSmemB;
  }
  const int want = v == SA_G1 ? 1 : v == SA_G2 ? 2 : 4;
  return pick_groups<M>(0, a.ax.r, 0, want) == want;
}

// Default: 4-row tiles (measured best inside the two-lane batch, where the
// persistent bulk kernel would hold every SM), else 2-row tiles, else the
// generic row kernel with up to 2 sub-transform groups.
template <int M>
int A_default(const PropArgs& a) {
  if (A_ok<M>(SA_TILE4, a)) return SA_TILE4;
  if (A_ok<M>(SA_TILE2, a)) return SA_TILE2;
  const int g = pick_groups<M>(0, a.ax.r, 0, 2);
  return g == 4 ? SA_G4 : g == 2 ? SA_G2 : SA_G1;
}

template <int M>
cudaError_t launch_A(const PropArgs& a, cudaStream_t st) {
  int v = env_variant("OSGPU_SCHED_A", kNamesA, SA_N);
  if (!v || !A_ok<M>(v, a)) v = a.sched.a;
  if (!v || !A_ok<M>(v, a)) v = A_default<M>(a);
  if constexpr (r4_ok<M>()) {
    if (v == SA_TSTORE) {
      const cudaError_t e = launch_A_tstore<M>(a, st);
      if (e != cudaErrorNotSupported) return e;
      v = SA_TILE4;
    }
    if (v == SA_BULK) return launch_A_bulk<M>(a, st);
    if (v == SA_TILE4) return launch_A_tile<M, 4>(a, st);
    if (v == SA_TILE2) return launch_A_tile<M, 2>(a, st);
  }
  if (v == SA_G4) return launchA_mg<M, 4>(a, st);
  if (v == SA_G2) return launchA_mg<M, 2>(a, st);
  return launchA_mg<M, 1>(a, st);
}

template <int M, int R, bool ADJ>
size_t smem_ctile(int r) {
  constexpr int T = M / 16;
  return ((size_t)TwLay<M>::SIZE + R * (size_t)tile_stride<M>() + (size_t)r * (T + 16)) *
         sizeof(float2);
}

template <int M, int R, bool ADJ>
cudaError_t launch_C_tile(const PropArgs& a, cudaStream_t st) {
  const size_t smem = smem_ctile<M, R, ADJ>(a.ax.r);
  cudaError_t e = cudaFuncSetAttribute(k_passC_tile<M, R, ADJ>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  ++launch_counter();
  return launch_pdl(k_passC_tile<M, R, ADJ>, dim3(a.ny / R), dim3(R * (M / 16)), smem, st, a);
}

template <int M>
size_t smem_cpipe(int r) {
  constexpr int T = M / 16;
  return ((size_t)TwLay<M>::SIZE + 2 * (size_t)tile_stride<M>() + 2 * (size_t)M +
          (size_t)r * (T + 16)) * sizeof(float2);
}

template <int M, bool ADJ>
cudaError_t launch_C_pipe(const PropArgs& a, cudaStream_t st) {
  const size_t smem = smem_cpipe<M>(a.ax.r);
  cudaError_t e = cudaFuncSetAttribute(k_passC_pipe<M, ADJ>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int tiles = a.ny / 2;
  const int grid = std::min(tiles, 2 * sm_count());
  ++launch_counter();
  return launch_pdl(k_passC_pipe<M, ADJ>, dim3(grid), dim3(2 * (M / 16)), smem, st, a);
}

template <int M>
size_t smem_ctma(int r) {
  constexpr int T = M / 16;
  return (2 * (size_t)M + (size_t)TwLay<M>::SIZE + 2 * (size_t)tile_stride<M>() +
          (size_t)r * (T + 16)) * sizeof(float2) + 16;
}

// Pass C through TMA when the tensor map of the spectrum can be encoded;
// cudaErrorNotSupported tells the caller to take the cp.async kernel.
template <int M, bool ADJ>
cudaError_t launch_C_tma(const PropArgs& a, cudaStream_t st) {
  const unsigned long long dims[3] = {(unsigned long long)a.ny, (unsigned long long)a.ax.r,
                                      (unsigned long long)M};
  const unsigned long long strides[2] = {(unsigned long long)a.ny * 8ull,
                                         (unsigned long long)a.ax.r * a.ny * 8ull};
  const unsigned box[3] = {2u, 1u, 256u};
  CUtensorMap map;
  if (!encode_map_3d_c64(&map, a.work, dims, strides, box)) return cudaErrorNotSupported;
  const size_t smem = smem_ctma<M>(a.ax.r);
  cudaError_t e = cudaFuncSetAttribute(k_passC_tma<M, ADJ>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = std::min(a.ny / 2, 2 * sm_count());
  ++launch_counter();
  return launch_pdl(k_passC_tma<M, ADJ>, dim3(grid), dim3(2 * (M / 16)), smem, st, a, map);
}

template <int M>
bool C_ok(int v, const PropArgs& a) {
  if (v == SC_TMA || v == SC_PIPE || v == SC_TILE2 || v == SC_TILE4) {
    if constexpr (!r4_ok<M>()) return false;
    if (v == SC_TMA)
      return a.ny % 2 == 0 && reinterpret_cast<uintptr_t>(a.work) % 16 == 0 &&
             smem_ctma<M>(a.ax.r) <= kMaxSmemB;
    if (v == SC_PIPE) return a.ny % 2 == 0 && smem_cpipe<M>(a.ax.r) <= kMaxSmemB;
    if (v == SC_TILE4) return a.ny % 4 == 0 && smem_ctile<M, 4, false>(a.ax.r) <= kMaxSmemB;
    return a.ny % 2 == 0 && smem_ctile<M, 2, false>(a.ax.r) <= kMaxSmemB;
  }
  const int want = v == SC_G1 ? 1 : v == SC_G2 ? 2 : 4;
  return pick_groups<M>(2, a.ax.r, 0, want) == want;
}

// Default: the persistent TMA-staged kernel (0.095 -> 0.075 ms per 2048^2
// band against the cp.async pipeline), else the cp.async pipeline, else the
// generic row kernel.
template <int M>
int C_default(const PropArgs& a) {
  if (C_ok<M>(SC_TMA, a)) return SC_TMA;
  if (C_ok<M>(SC_PIPE, a)) return SC_PIPE;
  const int g = pick_groups<M>(2, a.ax.r, 0, 2);
  return g == 4 ? SC_G4 : g == 2 ? SC_G2 : SC_G1;
}

template <int M>
cudaError_t launch_C(const PropArgs& a, cudaStream_t st) {
  int v = env_variant("OSGPU_SCHED_C", kNamesC, SC_N);
  if (!v || !C_ok<M>(v, a)) v = a.sched.c;
  if (!v || !C_ok<M>(v, a)) v = C_default<M>(a);
  if constexpr (r4_ok<M>()) {
    if (v == SC_TMA) {
      const cudaError_t e = a.adj ? launch_C_tma<M, true>(a, st) : launch_C_tma<M, false>(a, st);
      if (e != cudaErrorNotSupported) return e;
      v = SC_PIPE;  // the driver could not encode the tensor map
    }
    if (v == SC_PIPE && C_ok<M>(SC_PIPE, a))
      return a.adj ? launch_C_pipe<M, true>(a, st) : launch_C_pipe<M, false>(a, st);
    if (v == SC_TILE4)
      return a.adj ? launch_C_tile<M, 4, true>(a, st) : launch_C_tile<M, 4, false>(a, st);
    if (v == SC_TILE2)
      return a.adj ? launch_C_tile<M, 2, true>(a, st) : launch_C_tile<M, 2, false>(a, st);
  }
  if (v == SC_G4) return launchC_mg<M, 4>(a, st);
  if (v == SC_G2) return launchC_mg<M, 2>(a, st);
  return launchC_mg<M, 1>(a, st);
}

}  // namespace

template <int M>
cudaError_t launch_stage(void* tw, cudaStream_t st) {
  ++launch_counter();
  k_stage_twiddles<M><<<(TwLay<M>::SIZE + 255) / 256, 256, 0, st>>>(reinterpret_cast<float2*>(tw));
  return cudaGetLastError();
}

bool encode_map_3d_c64(CUtensorMap* map, const void* base, const unsigned long long dims[3],
                       const unsigned long long strides[2], const unsigned box[3]) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  if (!fn) return false;
  const cuuint64_t gdim[3] = {dims[0], dims[1], dims[2]};
  const cuuint64_t gstr[2] = {strides[0], strides[1]};
  const cuuint32_t bdim[3] = {box[0], box[1], box[2]};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_INT64, 3, const_cast<void*>(base), gdim, gstr, bdim, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

const char* sched_name(int pass, int v) {
  if (pass == 0 && v >= 0 && v < SA_N) return kNamesA[v];
  if (pass == 1 && v >= 0 && v < SB_N) return kNamesB[v];
  if (pass == 2 && v >= 0 && v < SC_N) return kNamesC[v];
  return "?";
}

int sched_count(int pass) {
  if (pass == 0) return (int)SA_N;
  return pass == 1 ? (int)SB_N : (int)SC_N;
}

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

cudaError_t launch_stage_twiddles(void* tw, int m, cudaStream_t st) {
  OSGPU_DISPATCH(m, launch_stage, tw, st)
}

cudaError_t launch_passA_reg(const PropArgs& a, cudaStream_t st) { OSGPU_DISPATCH(a.ax.m, launch_A, a, st) }
cudaError_t launch_passB_reg(const PropArgs& a, cudaStream_t st) { OSGPU_DISPATCH(a.ay.m, launch_B, a, st) }
cudaError_t launch_passC_reg(const PropArgs& a, cudaStream_t st) { OSGPU_DISPATCH(a.ax.m, launch_C, a, st) }

}  // namespace osgpu
