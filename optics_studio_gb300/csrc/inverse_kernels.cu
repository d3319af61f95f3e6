// Device kernels of the inverse loops (optics-inverse observe.rs, merit.rs,
// adjoint.rs, fd.rs): element planes outside a propagation, intensity
// frames, FP64-compensated merit and power reductions, the merit seeds
// dM/dI, and the Adam parameter update.
//
// Reductions are deterministic: each block folds a grid-stride slice into a
// Neumaier-compensated FP64 pair, the pairs of all blocks land in a partial
// buffer, and one block folds the partials in a fixed order.
#include <cuda_runtime.h>

#include "elements.cuh"
#include "inverse_kernels.cuh"
#include "prop_kernels.cuh"

namespace osgpu {

extern unsigned long long& launch_counter();

namespace {

constexpr int kRedThreads = 256;

// Compensated FP64 accumulator (Neumaier).
struct Acc {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ void add(const Acc& o) {
    add(o.s);
    c += o.c;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

// Per-thread partial of a sum of f32 products for the f32 engine's
// reductions, kept as an unevaluated pair hi + lo of f32 values: each product
// is split exactly (TwoProduct by FMA) and added to hi by TwoSum (Knuth), the
// rounding errors collecting in lo (the Dot2 scheme of Ogita, Rump and
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005).
// The partial is as accurate as an FP64 sum of the exact products (relative
// error ~n 2^-48 for n terms) while every operation runs on the FP32 pipe;
// the pairs are then folded by the compensated FP64 Acc.  Explicit _rn
// intrinsics keep the compiler from contracting the error terms.
struct AccF {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);  // a b - p exactly
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // hi + p - s
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
  }
  // another partial: hi by TwoSum, the rounding error and both lo into lo
  __device__ __forceinline__ void add(float ohi, float olo) {
    const float s = __fadd_rn(hi, ohi);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(ohi, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, olo));
  }
};

__device__ __forceinline__ Acc shfl_down(const Acc& a, int d) {
  Acc b;
  b.s = __shfl_down_sync(0xffffffffu, a.s, d);
  b.c = __shfl_down_sync(0xffffffffu, a.c, d);
  return b;
}

// Block fold of one Acc per thread; the result is valid in thread 0.
__device__ Acc block_fold(Acc a) {
  __shared__ double ss[kRedThreads / 32], sc[kRedThreads / 32];
  for (int d = 16; d > 0; d >>= 1) a.add(shfl_down(a, d));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    ss[w] = a.s;
    sc[w] = a.c;
  }
  __syncthreads();
  Acc r;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRedThreads / 32; ++i) {
      Acc o;
      o.s = ss[i];
      o.c = sc[i];
      r.add(o);
    }
  }
  __syncthreads();
  return r;
}

// Block fold of one AccF per thread: the warp's partials combine on the
// FP32 pipe (AccF::add, five shuffle levels), then each warp's pair enters
// the compensated FP64 fold once.  The result is valid in thread 0.
__device__ Acc block_fold_f32(AccF t) {
  for (int d = 16; d > 0; d >>= 1) {
    const float ohi = __shfl_down_sync(0xffffffffu, t.hi, d);
    const float olo = __shfl_down_sync(0xffffffffu, t.lo, d);
    t.add(ohi, olo);
  }
  Acc a;
  if ((threadIdx.x & 31) == 0) {
    a.add((double)t.hi);
    a.add((double)t.lo);
  }
  __shared__ double ss[kRedThreads / 32], sc[kRedThreads / 32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    ss[w] = a.s;
    sc[w] = a.c;
  }
  __syncthreads();
  Acc r;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kRedThreads / 32; ++i) {
      Acc o;
      o.s = ss[i];
      o.c = sc[i];
      r.add(o);
    }
  }
  __syncthreads();
  return r;
}

template <typename R>
__device__ __forceinline__ double ldr(const void* p, size_t i) {
  return (double)reinterpret_cast<const R*>(p)[i];
}

__device__ __forceinline__ double ld_real(const void* p, int f64, size_t i) {
  return f64 ? ldr<double>(p, i) : ldr<float>(p, i);
}

__device__ __forceinline__ void st_real(void* p, int f64, size_t i, double v) {
  if (f64) reinterpret_cast<double*>(p)[i] = v;
  else reinterpret_cast<float*>(p)[i] = (float)v;
}

template <typename T>
__device__ __forceinline__ void ld_cx(const void* p, int c128, size_t i, T& re, T& im) {
  if (c128) {
    const double2 v = reinterpret_cast<const double2*>(p)[i];
    re = (T)v.x;
    im = (T)v.y;
  } else {
    const float2 v = reinterpret_cast<const float2*>(p)[i];
    re = (T)v.x;
    im = (T)v.y;
  }
}

template <typename T>
__device__ __forceinline__ void st_cx(void* p, int c128, size_t i, T re, T im) {
  if (c128) reinterpret_cast<double2*>(p)[i] = make_double2((double)re, (double)im);
  else reinterpret_cast<float2*>(p)[i] = make_float2((float)re, (float)im);
}

template <typename T>
__device__ __forceinline__ void apply_chain(const ElementList& L, int ix, int iy, int nx, int ny,
                                            double dx, double dy, T& re, T& im) {
  if (L.count == 0) return;
  if (sizeof(T) == 4 && L.fast) {
    float2 v = make_float2((float)re, (float)im);
    v = apply_elements_fast(L, ix, iy, v);
    re = (T)v.x;
    im = (T)v.y;
    return;
  }
  double r = (double)re, i = (double)im;
  apply_elements_exact(L, ix, iy, nx, ny, dx, dy, r, i);
  re = (T)r;
  im = (T)i;
}

// Elements then |u|^2 (render of a design whose last steps are elements).
template <typename T>
__global__ void k_apply_intensity(const void* in, int in_c128, void* out, int out_c128,
                                  ElementList els, int nx, int ny, double dx, double dy,
                                  void* inten, int inten_f64) {
  const size_t n = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    T re, im;
    ld_cx<T>(in, in_c128, k, re, im);
    apply_chain<T>(els, ix, iy, nx, ny, dx, dy, re, im);
    if (out) st_cx<T>(out, out_c128, k, re, im);
    if (inten) {
      if (inten_f64) reinterpret_cast<double*>(inten)[k] = (double)re * re + (double)im * im;
      else reinterpret_cast<float*>(inten)[k] = re * re + im * im;
    }
  }
}

// Detector seed plus the element plane in front of it, outside any
// propagation: u_det = chain(u_in), mu = w u_det (w = seed * scale), then
// the adjoint plane of the chain (reference adjoint.rs:198-227).
template <typename T>
__global__ void k_adjoint_seed_plane(const void* uin, int uin_c128, ElementList els,
                                     AdjGrads grads, const void* seed, int seed_f64,
                                     double scale, int nx, int ny, double dx, double dy,
                                     void* mu_out, int mu_c128) {
  const size_t n = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    T ur, ui;
    ld_cx<T>(uin, uin_c128, k, ur, ui);
    T dr = ur, di = ui;
    apply_chain<T>(els, ix, iy, nx, ny, dx, dy, dr, di);
    const T w = (T)(ld_real(seed, seed_f64, k) * scale);
    T mr = w * dr, mi = w * di;
    adjoint_plane<T>(els, grads.p, ix, iy, nx, ny, dx, dy, k, ur, ui, mr, mi);
    if (mu_out) st_cx<T>(mu_out, mu_c128, k, mr, mi);
  }
}

// Per-frame partial sums: part[(f * nb + b) * 2 + {0,1}] = (s, c).
__device__ __forceinline__ void write_part(double* part, int f, const Acc& a) {
  if (threadIdx.x == 0) {
    const size_t o = ((size_t)f * gridDim.x + blockIdx.x) * 2;
    part[o] = a.s;
    part[o + 1] = a.c;
  }
}

// sum over the window mask of each frame's intensity.
__global__ void k_window_sums(const void* obs, int f64, uint64_t len, const unsigned char* win,
                              double* part) {
  const int f = blockIdx.y;
  const size_t base = (size_t)f * len;
  Acc a;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x)
    if (win[k]) a.add(ld_real(obs, f64, base + k));
  write_part(part, f, block_fold(a));
}

// seed_f[k] = win[k] ? coef[f] : 0
__global__ void k_window_seed(void* seed, int f64, uint64_t len, const unsigned char* win,
                              const double* coef) {
  const int f = blockIdx.y;
  const double c = coef[f];
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x)
    st_real(seed, f64, (size_t)f * len + k, win[k] ? c : 0.0);
}

// sum of w[k] I_f[k] over each frame (w in the observation's real dtype).
__global__ void k_weighted_sums(const void* obs, int f64, uint64_t len, const void* w,
                                double* part) {
  const int f = blockIdx.y;
  const size_t base = (size_t)f * len;
  Acc a;
  // RU grid-stride steps per pass, all loads of a pass issued before its sums
  // (the terms are added in the plain grid-stride order)
  constexpr int RU = 4;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (!f64) {  // f32 frames and weights: FP32-pipe partials (AccF), FP64 fold
    const float* wf = static_cast<const float*>(w);
    const float* of = static_cast<const float*>(obs) + base;
    AccF t;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len; k += RU * stride) {
      float wv[RU], ov[RU];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const size_t kk = k + u * stride;
        wv[u] = kk < len ? wf[kk] : 0.f;
        ov[u] = kk < len ? of[kk] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < RU; ++u)
        if (wv[u] != 0.f) t.add_prod(wv[u], ov[u]);
    }
    write_part(part, f, block_fold_f32(t));
    return;
  } else {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len; k += RU * stride) {
      double wv[RU], ov[RU];
#pragma unroll
      for (int u = 0; u < RU; ++u) {
        const size_t kk = k + u * stride;
        wv[u] = kk < len ? ld_real(w, f64, kk) : 0.0;
        ov[u] = kk < len ? ld_real(obs, f64, base + kk) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < RU; ++u)
        if (wv[u] != 0.0) a.add(wv[u] * ov[u]);
    }
  }
  write_part(part, f, block_fold(a));
}

// seed_f[k] = coef[f] w[k].  For f32 seeds the FP64 coefficient is split into
// two f32 parts (c = ch + cl to ~2^-48) and the product formed on the FP32
// pipe, ch w + cl w, then rounded once to f32.
__global__ void k_weighted_seed(void* seed, int f64, uint64_t len, const void* w,
                                const double* coef) {
  const int f = blockIdx.y;
  const double c = coef[f];
  if (!f64) {
    const float ch = (float)c, cl = (float)(c - (double)ch);
    const float* wf = static_cast<const float*>(w);
    float* sf = static_cast<float*>(seed) + (size_t)f * len;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
         k += (size_t)gridDim.x * blockDim.x) {
      const float wk = wf[k];
      sf[k] = __fmaf_rn(cl, wk, __fmul_rn(ch, wk));
    }
    return;
  }
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x)
    st_real(seed, f64, (size_t)f * len + k, c * ld_real(w, f64, k));
}

// Sum of the selected frames at sample k (reference merit.rs:44-81: bands
// outer, scenes inner, from 0).
__device__ __forceinline__ double selected_sum(const void* obs, int f64, uint64_t len, int nb,
                                               int ns, int band, int scene, size_t k) {
  double acc = 0.0;
  for (int b = 0; b < nb; ++b) {
    if (band >= 0 && b != band) continue;
    for (int s = 0; s < ns; ++s) {
      if (scene >= 0 && s != scene) continue;
      acc += ld_real(obs, f64, ((size_t)b * ns + s) * len + k);
    }
  }
  return acc;
}

// MSE: sum_k (frame[k] - target[k])^2.
__global__ void k_mse_sum(const void* obs, int f64, uint64_t len, int nb, int ns, int band,
                          int scene, const double* target, double* part) {
  Acc a;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x) {
    const double d = selected_sum(obs, f64, len, nb, ns, band, scene, k) - target[k];
    a.add(d * d);
  }
  write_part(part, 0, block_fold(a));
}

// MSE seed (merit.rs:141-163): 2 (I_f[k] - target[k]) / len on selected frames.
__global__ void k_mse_seed(const void* obs, int f64, void* seed, uint64_t len, int nb, int ns,
                           int band, int scene, const double* target) {
  const int f = blockIdx.y;
  const int b = f / ns, s = f - b * ns;
  const bool sel = (band < 0 || b == band) && (scene < 0 || s == scene);
  const double n = (double)len;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x) {
    const size_t i = (size_t)f * len + k;
    st_real(seed, f64, i, sel ? 2.0 * (ld_real(obs, f64, i) - target[k]) / n : 0.0);
  }
}

// Encircled-energy mask (merit.rs:175-189): centred coordinates in FP64.
__device__ __forceinline__ bool ee_inside(size_t k, int nx, int ny, double dx, double dy,
                                          double radius) {
  const int ix = (int)(k % nx), iy = (int)(k / nx);
  const double y = ((double)iy - ((double)ny - 1.0) / 2.0) * dy;
  const double x = ((double)ix - ((double)nx - 1.0) / 2.0) * dx;
  return x * x + y * y <= radius * radius;
}

// EE: part frame 0 = total, frame 1 = inside.
__global__ void k_ee_sums(const void* obs, int f64, int nx, int ny, double dx, double dy,
                          double radius, int nb, int ns, int band, int scene, double* part) {
  const uint64_t len = (uint64_t)nx * ny;
  Acc tot, ins;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x) {
    const double v = selected_sum(obs, f64, len, nb, ns, band, scene, k);
    tot.add(v);
    if (ee_inside(k, nx, ny, dx, dy, radius)) ins.add(v);
  }
  write_part(part, 0, block_fold(tot));
  write_part(part, 1, block_fold(ins));
}

// EE seed (merit.rs:214-244): -((m_k total - inside) / total^2) on selected frames.
__global__ void k_ee_seed(void* seed, int f64, int nx, int ny, double dx, double dy,
                          double radius, int ns, int band, int scene, const double* sums) {
  const uint64_t len = (uint64_t)nx * ny;
  const int f = blockIdx.y;
  const int b = f / ns, s = f - b * ns;
  const bool sel = (band < 0 || b == band) && (scene < 0 || s == scene);
  const double total = sums[0], inside = sums[1];
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x) {
    double g = 0.0;
    if (sel) g = -(((ee_inside(k, nx, ny, dx, dy, radius) ? total : 0.0) - inside) /
                   (total * total));
    st_real(seed, f64, (size_t)f * len + k, g);
  }
}

// The selected frame (Selector::frame, merit.rs:47-80) materialised in FP64:
// out[k] = sum over the selected (band, scene) frames, band-major, from 0.0.
__global__ void k_sel_frame(const void* obs, int f64, uint64_t len, int nb, int ns, int band,
                            int scene, double* out) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x)
    out[k] = selected_sum(obs, f64, len, nb, ns, band, scene, k);
}

// Spot RMS seed (merit.rs:285-320): (rho_k^2 - R^2) / (2 R sum I) on the
// selected frames, 0 elsewhere; rr = R^2, denom = 2 R sum I.
__global__ void k_spot_seed(void* seed, int f64, int nx, int ny, double dx, double dy, int ns,
                            int band, int scene, double rr, double denom) {
  const uint64_t len = (uint64_t)nx * ny;
  const int f = blockIdx.y;
  const int b = f / ns, s = f - b * ns;
  const bool sel = (band < 0 || b == band) && (scene < 0 || s == scene);
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x) {
    double g = 0.0;
    if (sel) {
      const int ix = (int)(k % nx), iy = (int)(k / nx);
      const double y = ((double)iy - ((double)ny - 1.0) / 2.0) * dy;
      const double x = ((double)ix - ((double)nx - 1.0) / 2.0) * dx;
      g = ((x * x + y * y) - rr) / denom;
    }
    st_real(seed, f64, (size_t)f * len + k, g);
  }
}

// Field power sum |u|^2.
__global__ void k_power(const void* u, int c128, uint64_t n, double* part) {
  Acc a;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double re, im;
    ld_cx<double>(u, c128, k, re, im);
    a.add(re * re + im * im);
  }
  write_part(part, 0, block_fold(a));
}

// Sum of squares of a real vector.
__global__ void k_sumsq(const void* g, int f64, uint64_t n, double* part) {
  Acc a;
  if (!f64) {  // f32 vector: FP32-pipe partials (AccF), FP64 fold
    const float* gf = static_cast<const float*>(g);
    constexpr int RU = 4;  // loads of RU grid-stride steps in flight together
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    AccF t;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += RU * stride) {
      float v[RU];
#pragma unroll
      for (int u = 0; u < RU; ++u) v[u] = k + u * stride < n ? gf[k + u * stride] : 0.f;
#pragma unroll
      for (int u = 0; u < RU; ++u) t.add_prod(v[u], v[u]);
    }
    write_part(part, 0, block_fold_f32(t));
    return;
  } else {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x) {
      const double v = ld_real(g, f64, k);
      a.add(v * v);
    }
  }
  write_part(part, 0, block_fold(a));
}

// Final fold of nb partial pairs per frame: out[f] = compensated sum (one
// block per frame).
__global__ void k_fold_parts(const double* part, int nb, int nf, double* out) {
  for (int f = blockIdx.x; f < nf; f += gridDim.x) {
    Acc a;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      Acc o;
      o.s = part[((size_t)f * nb + b) * 2];
      o.c = part[((size_t)f * nb + b) * 2 + 1];
      a.add(o);
    }
    a = block_fold(a);
    if (threadIdx.x == 0) out[f] = a.value();
  }
}

// Adam update (reference fd.rs:217-235): optional global-norm clip scale from
// norm2 = sum g^2 (device), bias-corrected moments, x -= step m^/(sqrt(v^)+eps)
// when the denominator is positive, then clamp into [lo, hi].
__global__ void k_adam(double* x, float* x32, const void* g, int g_f64, double* m, double* v,
                       uint64_t n, AdamArgs p, const double* norm2) {
  double scale = 1.0;
  if (p.clip) {
    const double norm = sqrt(*norm2);
    if (norm > p.clip_norm && norm > 0.0) scale = p.clip_norm / norm;
  }
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    // reference operation order, no contraction
    const double gi = __dmul_rn(ld_real(g, g_f64, i), scale);
    const double mi = __dadd_rn(__dmul_rn(p.beta1, m[i]), __dmul_rn(1.0 - p.beta1, gi));
    const double vi =
        __dadd_rn(__dmul_rn(p.beta2, v[i]), __dmul_rn(__dmul_rn(1.0 - p.beta2, gi), gi));
    m[i] = mi;
    v[i] = vi;
    const double mh = __ddiv_rn(mi, p.bc1);
    const double vh = __ddiv_rn(vi, p.bc2);
    const double denom = __dadd_rn(__dsqrt_rn(vh), p.eps);
    double xi = x[i];
    if (denom > 0.0) xi = __dsub_rn(xi, __ddiv_rn(__dmul_rn(p.step, mh), denom));
    if (xi < p.lo) xi = p.lo;  // f64::clamp (NaN stays NaN)
    if (xi > p.hi) xi = p.hi;
    x[i] = xi;
    if (x32) x32[i] = (float)xi;
  }
}

// ------------------------------------------------------------ GS loop
// (reference gs.rs:425-597).  Per iteration: k_gs_mask -> forward half ->
// k_gs_project -> k_gs_fold_merit -> back half -> k_gs_update ->
// k_gs_fold_update.  The loop state lives on the device (GsState); every
// kernel returns at once when state->stop is set, so the host can queue
// iterations ahead of the convergence decision.

constexpr double kTau = 6.283185307179586;  // 2 pi as f64 (gs.rs:105)
constexpr double kPi = 3.141592653589793;

__device__ __forceinline__ double rem_euclid(double a, double m) {
  const double r = fmod(a, m);
  return r < 0.0 ? r + fabs(m) : r;
}

// gs.rs:108-110
__device__ __forceinline__ double wrap_pi(double v) {
  return __dsub_rn(rem_euclid(__dadd_rn(v, kPi), kTau), kPi);
}

// gs.rs:115-121
__device__ __forceinline__ double encode_bounds(double phi, double lo, double hi) {
  if (__dsub_rn(hi, lo) >= kTau) return __dadd_rn(lo, rem_euclid(__dsub_rn(phi, lo), kTau));
  return phi < lo ? lo : (phi > hi ? hi : phi);
}

// mask = open ? illum e^{i phase} : 0   (gs.rs:482-491, Complex::from_polar)
__global__ void k_gs_mask(const void* phase, int f64, const void* illum,
                          const unsigned char* open, void* mask, int c128, uint64_t n,
                          const GsState* state) {
  if (state && state->stop) return;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    if (open[k]) {
      const double r = ld_real(illum, f64, k), th = ld_real(phase, f64, k);
      double s, c;
      sincos(th, &s, &c);
      re = r * c;
      im = r * s;
    }
    st_cx<double>(mask, c128, k, re, im);
  }
}

// Target-plane error, merit terms and projection (gs.rs:494-545):
// part frame 0 = sum (|u| - T)^2, frame 1 = sum (|u|^2 - Tint)^2.
__global__ void k_gs_project(const void* u, int c128, const void* tamp, const void* tint,
                             int f64, double beta_f, void* proj, uint64_t n, double* part,
                             void* err_out, const GsState* state) {
  if (state && state->stop) return;
  Acc e2, m2;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double re, im;
    ld_cx<double>(u, c128, k, re, im);
    const double amp = hypot(re, im);
    const double t = ld_real(tamp, f64, k);
    const double inten = __dmul_rn(amp, amp);
    const double err = amp - t;
    const double ti = tint ? ld_real(tint, f64, k) : __dmul_rn(t, t);
    const double dm = inten - ti;
    e2.add(__dmul_rn(err, err));
    m2.add(__dmul_rn(dm, dm));
    if (err_out) st_real(err_out, f64, k, err);
    const double a = __dadd_rn(__dmul_rn(1.0 - beta_f, amp), __dmul_rn(beta_f, t));
    double pr, pi;
    if (amp > 0.0) {
      const double sc = a / amp;
      pr = re * sc;
      pi = im * sc;
    } else {
      pr = a;
      pi = 0.0;
    }
    st_cx<double>(proj, c128, k, pr, pi);
  }
  write_part(part, 0, block_fold(e2));
  write_part(part, 1, block_fold(m2));
}

// Merit, best-so-far and the history record of iteration `it` (gs.rs:496-531).
__device__ void gs_fold_merit(const double* part, int nb, uint64_t n, int it, GsState* state,
                              GsRecordDev* hist) {
  if (state->stop) return;
  double sums[2];
  for (int f = 0; f < 2; ++f) {
    Acc a;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      Acc o;
      o.s = part[((size_t)f * nb + b) * 2];
      o.c = part[((size_t)f * nb + b) * 2 + 1];
      a.add(o);
    }
    a = block_fold(a);
    sums[f] = a.value();
  }
  if (threadIdx.x == 0) {
    const double amp_mse = sums[0] / (double)n;
    const double merit = sums[1] / (double)n;  // MseToTarget::evaluate (merit.rs:128-146)
    const bool improved = state->best_it < 0 || merit < state->best_merit;
    if (improved) {
      state->best_merit = merit;
      state->best_it = it;
    }
    state->improved = improved ? 1 : 0;
    GsRecordDev& h = hist[it];
    h.iteration = (double)it;
    h.merit = merit;
    h.best_merit = state->best_merit;
    h.amplitude_mse = amp_mse;
    h.target_error_rms = sqrt(amp_mse);
    h.phase_update_rms = 0.0;
  }
}

__global__ void k_gs_fold_merit(const double* part, int nb, uint64_t n, int it, GsState* state,
                                GsRecordDev* hist) {
  gs_fold_merit(part, nb, n, it, state, hist);
}

// One block per item of a batch.
__global__ void k_gs_fold_merit_batch(const GsFoldItem* items, int nb, uint64_t n, int it) {
  const GsFoldItem& f = items[blockIdx.x];
  gs_fold_merit(f.part_merit, nb, n, it, f.state, f.hist);
}

// DOE-plane update (gs.rs:557-566); the phase of an improving iteration is
// kept as the best phase first.  part frame 0 = sum dphi^2.
__global__ void k_gs_update(const void* v, int c128, void* phase, void* best, int f64,
                            double beta_p, double lo, double hi, uint64_t n, double* part,
                            void* dphi_out, const GsState* state) {
  if (state->stop) return;
  const bool keep = state->improved != 0;
  Acc d2;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double re, im;
    ld_cx<double>(v, c128, k, re, im);
    const double p = ld_real(phase, f64, k);
    if (keep) st_real(best, f64, k, p);
    const double dphi = wrap_pi(__dsub_rn(atan2(im, re), p));
    st_real(phase, f64, k, encode_bounds(__dadd_rn(p, __dmul_rn(beta_p, dphi)), lo, hi));
    if (dphi_out) st_real(dphi_out, f64, k, dphi);
    d2.add(dphi * dphi);
  }
  write_part(part, 0, block_fold(d2));
}

// Phase-update RMS and the patience stop (gs.rs:567-578).
__device__ void gs_fold_update(const double* part, int nb, uint64_t n, int it, int patience,
                               double tol, int max_it, GsState* state, GsRecordDev* hist) {
  if (state->stop) return;
  Acc a;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    Acc o;
    o.s = part[(size_t)b * 2];
    o.c = part[(size_t)b * 2 + 1];
    a.add(o);
  }
  a = block_fold(a);
  if (threadIdx.x == 0) {
    hist[it].phase_update_rms = sqrt(a.value()) / sqrt((double)n);
    state->iterations = it + 1;
    if (it + 1 > patience) {
      const double earlier = hist[it - patience].best_merit;
      const double scale = fmax(fabs(earlier), 1e-30);
      if ((earlier - state->best_merit) / scale < tol) {
        state->converged = 1;
        state->stop = 1;
      }
    }
    if (it + 1 >= max_it) state->stop = 1;
  }
}

__global__ void k_gs_fold_update(const double* part, int nb, uint64_t n, int it, int patience,
                                 double tol, int max_it, GsState* state, GsRecordDev* hist) {
  gs_fold_update(part, nb, n, it, patience, tol, max_it, state, hist);
}

__global__ void k_gs_fold_update_batch(const GsFoldItem* items, int nb, uint64_t n, int it,
                                       int patience, double tol, int max_it) {
  const GsFoldItem& f = items[blockIdx.x];
  gs_fold_update(f.part_update, nb, n, it, patience, tol, max_it, f.state, f.hist);
}

// |u| (illumination amplitude) and |u|^2 (best intensity).
__global__ void k_abs(const void* u, int c128, void* out, int f64, int square, uint64_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    double re, im;
    ld_cx<double>(u, c128, k, re, im);
    const double a = hypot(re, im);
    st_real(out, f64, k, square ? a * a : a);
  }
}

// Illumination amplitude with the carrier aperture folded in (zero outside).
__global__ void k_mask_amplitude(const void* illum, const unsigned char* open, void* out, int f64,
                                 uint64_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    st_real(out, f64, k, open[k] ? ld_real(illum, f64, k) : 0.0);
}

// Initial phase encoded into the bounds, and the carrier aperture mask
// (gs.rs:429-435, 446-475).
__global__ void k_gs_init(const void* init, void* phase, int f64, double lo, double hi,
                          unsigned char* open, int stop, double a, double b, double cx,
                          double cy, int nx, int ny, double dx, double dy) {
  const uint64_t n = (uint64_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    st_real(phase, f64, k, encode_bounds(ld_real(init, f64, k), lo, hi));
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    const double x = coord_d(ix, nx, dx), y = coord_d(iy, ny, dy);
    open[k] = stop_contains(stop, a, b, __dsub_rn(x, cx), __dsub_rn(y, cy)) ? 1 : 0;
  }
}

// ------------------------------------------------------------ sources
// (reference sources.rs:259-296, field.rs:315-386): per sample in FP64,
// scalars of the beam formed on the host in the reference's order.
__global__ void k_gaussian(void* out, int c128, int nx, int ny, double dx, double dy, double cx,
                           double cy, double amp, double w2, double half_k, double inv_r,
                           double carrier) {
  const size_t n = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    const double x = __dsub_rn(coord_d(ix, nx, dx), cx);
    const double y = __dsub_rn(coord_d(iy, ny, dy), cy);
    const double rho2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    const double env = __dmul_rn(amp, exp(__ddiv_rn(-rho2, w2)));
    const double ph = __dadd_rn(carrier, __dmul_rn(__dmul_rn(half_k, rho2), inv_r));
    double s, c;
    sincos(ph, &s, &c);
    st_cx<double>(out, c128, k, __dmul_rn(env, c), __dmul_rn(env, s));
  }
}

__global__ void k_plane_wave(void* out, int c128, int nx, int ny, double dx, double dy,
                             double amp, double k_, double alpha, double beta) {
  const size_t n = (size_t)nx * ny;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    const double x = coord_d(ix, nx, dx), y = coord_d(iy, ny, dy);
    const double ph = __dmul_rn(k_, __dadd_rn(__dmul_rn(alpha, x), __dmul_rn(beta, y)));
    double s, c;
    sincos(ph, &s, &c);
    st_cx<double>(out, c128, k, __dmul_rn(amp, c), __dmul_rn(amp, s));
  }
}

// dst[k] += src[k] (real arrays of one dtype)
__global__ void k_add_real(void* dst, const void* src, int f64, uint64_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    if (f64) reinterpret_cast<double*>(dst)[k] += reinterpret_cast<const double*>(src)[k];
    else reinterpret_cast<float*>(dst)[k] += reinterpret_cast<const float*>(src)[k];
  }
}

__global__ void k_fill(void* out, int c128, size_t n, double re, double im) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    st_cx<double>(out, c128, k, re, im);
}

int red_blocks(uint64_t n) {
  const uint64_t b = (n + kRedThreads - 1) / kRedThreads;
  return (int)(b < 1216 ? (b ? b : 1) : 1216);  // <= 8 per SM on 152 SMs
}

// Blocks for a reduction whose per-thread partials run on the FP32 pipe
// (AccF, folded by block_fold_f32): about 64 terms per thread (with 4 steps'
// loads in flight per thread, enough to cover the memory latency), so that
// the per-block fold (barriers and a short serial FP64 tail in thread 0;
// the GPU's FP64 rate is a small fraction of its FP32 rate) is amortised.
int red_blocks_f32(uint64_t n) {
  const uint64_t b = (n + 64 * kRedThreads - 1) / (64 * kRedThreads);
  return (int)(b < 1216 ? (b ? b : 1) : 1216);  // the partials' scratch holds 1216 per frame
}

}  // namespace

#define OSGPU_LAUNCH ++launch_counter()

cudaError_t launch_apply_intensity(const void* in, int in_c128, void* out, int out_c128,
                                   const ElementList& els, int nx, int ny, double dx, double dy,
                                   void* inten, int inten_f64, int f32, cudaStream_t st) {
  const uint64_t n = (uint64_t)nx * ny;
  OSGPU_LAUNCH;
  if (f32)
    k_apply_intensity<float><<<red_blocks(n), kRedThreads, 0, st>>>(in, in_c128, out, out_c128,
                                                                   els, nx, ny, dx, dy, inten,
                                                                   inten_f64);
  else
    k_apply_intensity<double><<<red_blocks(n), kRedThreads, 0, st>>>(in, in_c128, out, out_c128,
                                                                    els, nx, ny, dx, dy, inten,
                                                                    inten_f64);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_seed_plane(const void* uin, int uin_c128, const ElementList& els,
                                      const AdjGrads& grads, const void* seed, int seed_f64,
                                      double scale, int nx, int ny, double dx, double dy,
                                      void* mu_out, int mu_c128, int f32, cudaStream_t st) {
  const uint64_t n = (uint64_t)nx * ny;
  OSGPU_LAUNCH;
  if (f32)
    k_adjoint_seed_plane<float><<<red_blocks(n), kRedThreads, 0, st>>>(
        uin, uin_c128, els, grads, seed, seed_f64, scale, nx, ny, dx, dy, mu_out, mu_c128);
  else
    k_adjoint_seed_plane<double><<<red_blocks(n), kRedThreads, 0, st>>>(
        uin, uin_c128, els, grads, seed, seed_f64, scale, nx, ny, dx, dy, mu_out, mu_c128);
  return cudaGetLastError();
}

cudaError_t launch_add_real(void* dst, const void* src, int f64, uint64_t n, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_add_real<<<red_blocks(n), kRedThreads, 0, st>>>(dst, src, f64, n);
  return cudaGetLastError();
}

size_t reduce_scratch_bytes(int n_frames) {
  return (size_t)n_frames * 1216 * 2 * sizeof(double) + (size_t)(n_frames + 2) * sizeof(double);
}

cudaError_t launch_window_sums(const void* obs, int f64, int nf, uint64_t len,
                               const unsigned char* win, double* scratch, double* out,
                               cudaStream_t st) {
  const int nb = red_blocks(len);
  OSGPU_LAUNCH;
  k_window_sums<<<dim3(nb, nf), kRedThreads, 0, st>>>(obs, f64, len, win, scratch);
  OSGPU_LAUNCH;
  k_fold_parts<<<nf, kRedThreads, 0, st>>>(scratch, nb, nf, out);
  return cudaGetLastError();
}

cudaError_t launch_window_seed(void* seed, int f64, int nf, uint64_t len,
                               const unsigned char* win, const double* coef, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_window_seed<<<dim3(red_blocks(len), nf), kRedThreads, 0, st>>>(seed, f64, len, win, coef);
  return cudaGetLastError();
}

cudaError_t launch_weighted_sums(const void* obs, int f64, int nf, uint64_t len, const void* w,
                                 double* scratch, double* out, cudaStream_t st) {
  const int nb = f64 ? red_blocks(len) : red_blocks_f32(len);
  OSGPU_LAUNCH;
  k_weighted_sums<<<dim3(nb, nf), kRedThreads, 0, st>>>(obs, f64, len, w, scratch);
  OSGPU_LAUNCH;
  k_fold_parts<<<nf, kRedThreads, 0, st>>>(scratch, nb, nf, out);
  return cudaGetLastError();
}

cudaError_t launch_weighted_seed(void* seed, int f64, int nf, uint64_t len, const void* w,
                                 const double* coef, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_weighted_seed<<<dim3(red_blocks(len), nf), kRedThreads, 0, st>>>(seed, f64, len, w, coef);
  return cudaGetLastError();
}

cudaError_t launch_mse(const void* obs, int f64, uint64_t len, int nb, int ns, int band,
                       int scene, const double* target, void* seed, double* scratch,
                       double* out, cudaStream_t st) {
  const int blocks = red_blocks(len);
  OSGPU_LAUNCH;
  k_mse_sum<<<blocks, kRedThreads, 0, st>>>(obs, f64, len, nb, ns, band, scene, target, scratch);
  OSGPU_LAUNCH;
  k_fold_parts<<<1, kRedThreads, 0, st>>>(scratch, blocks, 1, out);
  if (seed) {
    OSGPU_LAUNCH;
    k_mse_seed<<<dim3(blocks, nb * ns), kRedThreads, 0, st>>>(obs, f64, seed, len, nb, ns, band,
                                                              scene, target);
  }
  return cudaGetLastError();
}

cudaError_t launch_ee(const void* obs, int f64, int nx, int ny, double dx, double dy,
                      double radius, int nb, int ns, int band, int scene, void* seed,
                      double* scratch, double* out, cudaStream_t st) {
  const uint64_t len = (uint64_t)nx * ny;
  const int blocks = red_blocks(len);
  OSGPU_LAUNCH;
  k_ee_sums<<<blocks, kRedThreads, 0, st>>>(obs, f64, nx, ny, dx, dy, radius, nb, ns, band,
                                            scene, scratch);
  OSGPU_LAUNCH;
  k_fold_parts<<<2, kRedThreads, 0, st>>>(scratch, blocks, 2, out);
  if (seed) {
    OSGPU_LAUNCH;
    k_ee_seed<<<dim3(blocks, nb * ns), kRedThreads, 0, st>>>(seed, f64, nx, ny, dx, dy, radius,
                                                             ns, band, scene, out);
  }
  return cudaGetLastError();
}

cudaError_t launch_sel_frame(const void* obs, int f64, uint64_t len, int nb, int ns, int band,
                             int scene, double* out, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_sel_frame<<<red_blocks(len), kRedThreads, 0, st>>>(obs, f64, len, nb, ns, band, scene, out);
  return cudaGetLastError();
}

cudaError_t launch_spot_seed(void* seed, int f64, int nx, int ny, double dx, double dy, int nb,
                             int ns, int band, int scene, double rr, double denom,
                             cudaStream_t st) {
  OSGPU_LAUNCH;
  k_spot_seed<<<dim3(red_blocks((uint64_t)nx * ny), nb * ns), kRedThreads, 0, st>>>(
      seed, f64, nx, ny, dx, dy, ns, band, scene, rr, denom);
  return cudaGetLastError();
}

// ------------------------------------------------- detector metrics
// (reference src/analysis.rs)

// part frame 0 = sum I, frame 1 = sum I (x^2 + y^2) at the centred pixel
// coordinates of field.rs:490-495 (spot_rms_radius, analysis.rs:111-124).
__global__ void k_psf_moments(const void* img, int f64, int nx, int ny, double dx, double dy,
                              double* part) {
  const uint64_t len = (uint64_t)nx * ny;
  Acc sw, swr2;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(k % nx), iy = (int)(k / nx);
    const double x = ((double)ix - ((double)nx - 1.0) / 2.0) * dx;
    const double y = ((double)iy - ((double)ny - 1.0) / 2.0) * dy;
    const double i = ld_real(img, f64, k);
    sw.add(i);
    swr2.add(i * (x * x + y * y));
  }
  write_part(part, 0, block_fold(sw));
  write_part(part, 1, block_fold(swr2));
}

// Per-block maximum of a real grid (analysis.rs:167, fold from 0.0).
__global__ void k_psf_max(const void* img, int f64, uint64_t len, double* part) {
  __shared__ double sm[kRedThreads / 32];
  double m = 0.0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < len;
       k += (size_t)gridDim.x * blockDim.x)
    m = fmax(m, ld_real(img, f64, k));
  for (int d = 16; d > 0; d >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, d));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kRedThreads / 32; ++w) m = fmax(m, sm[w]);
    part[blockIdx.x] = m;
  }
}

__global__ void k_fold_max(const double* part, int nb, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double m = 0.0;
    for (int b = 0; b < nb; ++b) m = fmax(m, part[b]);
    *out = m;
  }
}

// Column sums s[ix] = sum_y I[y][ix] (compensated): row 0 of the 2D DFT of I
// is the 1D DFT of s (the MTF along +fx, analysis.rs:136-150).
__global__ void k_col_sums(const void* img, int f64, int nx, int ny, double* s) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= nx) return;
  Acc a;
  for (int iy = 0; iy < ny; ++iy) a.add(ld_real(img, f64, (size_t)iy * nx + ix));
  s[ix] = a.value();
}

// X[k] = sum_x s[x] W_nx^{k x}, k <= nx / 2, one block per bin, twiddles
// from the FP64 table tw[e] = W_nx^e.
__global__ void k_row_dft(const double* s, int nx, const double2* tw, double2* X) {
  const int k = blockIdx.x;
  Acc re, im;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    const double2 w = tw[(int)(((long long)k * x) % nx)];
    re.add(s[x] * w.x);
    im.add(s[x] * w.y);
  }
  re = block_fold(re);
  im = block_fold(im);
  if (threadIdx.x == 0) X[k] = make_double2(re.value(), im.value());
}

// Encircled-energy walk (analysis.rs:81-108): v[k] = I[perm[k]] in radius
// order, inclusive prefix sums in FP64 (block scans of 1024, then the block
// totals, then the offsets), fraction at the end of each tied-radius group.
constexpr int kScan = 1024;

__device__ __forceinline__ double warp_incl_scan(double v) {
  const int l = threadIdx.x & 31;
  for (int d = 1; d < 32; d <<= 1) {
    const double o = __shfl_up_sync(0xffffffffu, v, d);
    if (l >= d) v += o;
  }
  return v;
}

// Inclusive scan of one 1024-element block in place; block total to tot[b].
__device__ void block_incl_scan(double* data, uint64_t n, double* tot) {
  __shared__ double ws[kScan / 32];
  const uint64_t i = (uint64_t)blockIdx.x * kScan + threadIdx.x;
  double v = i < n ? data[i] : 0.0;
  v = warp_incl_scan(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 31) ws[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = ws[l];
    t = warp_incl_scan(t);
    ws[l] = t;
  }
  __syncthreads();
  if (w > 0) v += ws[w - 1];
  if (i < n) data[i] = v;
  if (threadIdx.x == kScan - 1 && tot) tot[blockIdx.x] = v;
}

__global__ void k_ee_gather_scan(const void* img, int f64, const unsigned* perm, uint64_t n,
                                 double* v, double* tot) {
  const uint64_t i = (uint64_t)blockIdx.x * kScan + threadIdx.x;
  if (i < n) v[i] = ld_real(img, f64, perm[i]);
  __syncthreads();
  block_incl_scan(v, n, tot);
}

// exclusive prefix of the block totals, serial per 1024-chunk inside one block
__global__ void k_scan_totals(double* tot, int nb) {
  __shared__ double carry;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  for (int base = 0; base < nb; base += kScan) {
    const int i = base + threadIdx.x;
    double v = i < nb ? tot[i] : 0.0;
    v = warp_incl_scan(v);
    __shared__ double ws[kScan / 32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 31) ws[w] = v;
    __syncthreads();
    if (w == 0) ws[l] = warp_incl_scan(ws[l]);
    __syncthreads();
    if (w > 0) v += ws[w - 1];
    const double c = carry;
    if (i < nb) tot[i] = c + v;  // inclusive prefix including the earlier chunks
    __syncthreads();
    if (threadIdx.x == kScan - 1) carry = c + v;
    __syncthreads();
  }
}

__global__ void k_ee_fraction(const double* v, const double* tot_incl, uint64_t n,
                              const unsigned* group_end, uint64_t ng, double total,
                              double* frac) {
  const uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (g >= ng) return;
  const uint64_t k = group_end[g];
  const uint64_t b = k / kScan;
  const double acc = v[k] + (b > 0 ? tot_incl[b - 1] : 0.0);
  frac[g] = acc / total;
}

cudaError_t launch_ee_curve(const void* img, int f64, const unsigned* perm, uint64_t n,
                            const unsigned* group_end, uint64_t ng, double* v, double* tot,
                            double* frac, double* total_out, cudaStream_t st) {
  const unsigned nb = (unsigned)((n + kScan - 1) / kScan);
  OSGPU_LAUNCH;
  k_ee_gather_scan<<<nb, kScan, 0, st>>>(img, f64, perm, n, v, tot);
  OSGPU_LAUNCH;
  k_scan_totals<<<1, kScan, 0, st>>>(tot, (int)nb);
  cudaError_t e = cudaMemcpyAsync(total_out, tot + nb - 1, sizeof(double),
                                  cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (!(*total_out > 0.0)) return cudaSuccess;
  OSGPU_LAUNCH;
  k_ee_fraction<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(v, tot, n, group_end, ng,
                                                               *total_out, frac);
  return cudaGetLastError();
}

cudaError_t launch_psf_moments(const void* img, int f64, int nx, int ny, double dx, double dy,
                               double* scratch, double* out2, cudaStream_t st) {
  const uint64_t n = (uint64_t)nx * ny;
  const int blocks = red_blocks(n);
  OSGPU_LAUNCH;
  k_psf_moments<<<blocks, kRedThreads, 0, st>>>(img, f64, nx, ny, dx, dy, scratch);
  OSGPU_LAUNCH;
  k_fold_parts<<<2, kRedThreads, 0, st>>>(scratch, blocks, 2, out2);
  return cudaGetLastError();
}

cudaError_t launch_psf_max(const void* img, int f64, uint64_t n, double* scratch, double* out,
                           cudaStream_t st) {
  const int blocks = red_blocks(n);
  OSGPU_LAUNCH;
  k_psf_max<<<blocks, kRedThreads, 0, st>>>(img, f64, n, scratch);
  OSGPU_LAUNCH;
  k_fold_max<<<1, 32, 0, st>>>(scratch, blocks, out);
  return cudaGetLastError();
}

cudaError_t launch_row_mtf(const void* img, int f64, int nx, int ny, const void* tw64,
                           double* colsum, double2* X, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_col_sums<<<(nx + 127) / 128, 128, 0, st>>>(img, f64, nx, ny, colsum);
  OSGPU_LAUNCH;
  k_row_dft<<<nx / 2 + 1, kRedThreads, 0, st>>>(colsum, nx, reinterpret_cast<const double2*>(tw64),
                                                X);
  return cudaGetLastError();
}

cudaError_t launch_power(const void* u, int c128, uint64_t n, double* scratch, double* out,
                         cudaStream_t st) {
  const int blocks = red_blocks(n);
  OSGPU_LAUNCH;
  k_power<<<blocks, kRedThreads, 0, st>>>(u, c128, n, scratch);
  OSGPU_LAUNCH;
  k_fold_parts<<<1, kRedThreads, 0, st>>>(scratch, blocks, 1, out);
  return cudaGetLastError();
}

cudaError_t launch_adam(double* x, float* x32, const void* g, int g_f64, double* m, double* v,
                        uint64_t n, const AdamArgs& p, double* scratch, double* norm2,
                        cudaStream_t st) {
  const int blocks = red_blocks(n);
  if (p.clip) {
    const int sb = g_f64 ? blocks : red_blocks_f32(n);
    OSGPU_LAUNCH;
    k_sumsq<<<sb, kRedThreads, 0, st>>>(g, g_f64, n, scratch);
    OSGPU_LAUNCH;
    k_fold_parts<<<1, kRedThreads, 0, st>>>(scratch, sb, 1, norm2);
  }
  OSGPU_LAUNCH;
  k_adam<<<blocks, kRedThreads, 0, st>>>(x, x32, g, g_f64, m, v, n, p, norm2);
  return cudaGetLastError();
}

cudaError_t launch_gs_init(const void* init, void* phase, int f64, double lo, double hi,
                           unsigned char* open, int stop, double a, double b, double cx,
                           double cy, int nx, int ny, double dx, double dy, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_gs_init<<<red_blocks((uint64_t)nx * ny), kRedThreads, 0, st>>>(init, phase, f64, lo, hi, open,
                                                                   stop, a, b, cx, cy, nx, ny, dx,
                                                                   dy);
  return cudaGetLastError();
}

cudaError_t launch_mask_amplitude(const void* illum, const unsigned char* open, void* out,
                                  int f64, uint64_t n, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_mask_amplitude<<<red_blocks(n), kRedThreads, 0, st>>>(illum, open, out, f64, n);
  return cudaGetLastError();
}

cudaError_t launch_abs(const void* u, int c128, void* out, int f64, int square, uint64_t n,
                       cudaStream_t st) {
  OSGPU_LAUNCH;
  k_abs<<<red_blocks(n), kRedThreads, 0, st>>>(u, c128, out, f64, square, n);
  return cudaGetLastError();
}

cudaError_t launch_gs_mask(const void* phase, int f64, const void* illum,
                           const unsigned char* open, void* mask, int c128, uint64_t n,
                           const GsState* state, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_gs_mask<<<red_blocks(n), kRedThreads, 0, st>>>(phase, f64, illum, open, mask, c128, n, state);
  return cudaGetLastError();
}

cudaError_t launch_gs_project(const void* u, int c128, const void* tamp, const void* tint,
                              int f64, double beta_f, void* proj, uint64_t n, double* part,
                              void* err_out, GsState* state, GsRecordDev* hist, int it,
                              cudaStream_t st) {
  const int nb = red_blocks(n);
  OSGPU_LAUNCH;
  k_gs_project<<<nb, kRedThreads, 0, st>>>(u, c128, tamp, tint, f64, beta_f, proj, n, part,
                                           err_out, state);
  OSGPU_LAUNCH;
  k_gs_fold_merit<<<1, kRedThreads, 0, st>>>(part, nb, n, it, state, hist);
  return cudaGetLastError();
}

cudaError_t launch_gs_update(const void* v, int c128, void* phase, void* best, int f64,
                             double beta_p, double lo, double hi, uint64_t n, double* part,
                             void* dphi_out, GsState* state, GsRecordDev* hist, int it,
                             int patience, double tol, int max_it, cudaStream_t st) {
  const int nb = red_blocks(n);
  OSGPU_LAUNCH;
  k_gs_update<<<nb, kRedThreads, 0, st>>>(v, c128, phase, best, f64, beta_p, lo, hi, n, part,
                                          dphi_out, state);
  OSGPU_LAUNCH;
  k_gs_fold_update<<<1, kRedThreads, 0, st>>>(part, nb, n, it, patience, tol, max_it, state,
                                              hist);
  return cudaGetLastError();
}

cudaError_t launch_gs_fold_merit_batch(const GsFoldItem* items, int n_items, int nb, uint64_t n,
                                       int it, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_gs_fold_merit_batch<<<n_items, kRedThreads, 0, st>>>(items, nb, n, it);
  return cudaGetLastError();
}

cudaError_t launch_gs_fold_update_batch(const GsFoldItem* items, int n_items, int nb, uint64_t n,
                                        int it, int patience, double tol, int max_it,
                                        cudaStream_t st) {
  OSGPU_LAUNCH;
  k_gs_fold_update_batch<<<n_items, kRedThreads, 0, st>>>(items, nb, n, it, patience, tol,
                                                          max_it);
  return cudaGetLastError();
}

cudaError_t launch_gaussian(void* out, int c128, int nx, int ny, double dx, double dy, double cx,
                            double cy, double amp, double w2, double half_k, double inv_r,
                            double carrier, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_gaussian<<<red_blocks((uint64_t)nx * ny), kRedThreads, 0, st>>>(out, c128, nx, ny, dx, dy, cx,
                                                                    cy, amp, w2, half_k, inv_r,
                                                                    carrier);
  return cudaGetLastError();
}

cudaError_t launch_plane_wave(void* out, int c128, int nx, int ny, double dx, double dy,
                              double amp, double k, double alpha, double beta, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_plane_wave<<<red_blocks((uint64_t)nx * ny), kRedThreads, 0, st>>>(out, c128, nx, ny, dx, dy,
                                                                      amp, k, alpha, beta);
  return cudaGetLastError();
}

cudaError_t launch_fill(void* out, int c128, size_t n, double re, double im, cudaStream_t st) {
  OSGPU_LAUNCH;
  k_fill<<<red_blocks(n), kRedThreads, 0, st>>>(out, c128, n, re, im);
  return cudaGetLastError();
}

}  // namespace osgpu
