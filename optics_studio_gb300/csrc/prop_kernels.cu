// Propagation passes for sm_103a: table prep, pass A (row FFTs + element
// fusion), pass B (column FFT -> transfer function -> inverse column FFT),
// pass C (inverse row FFTs + crop), plus kernel-spectrum builds and the
// two-pass Fraunhofer transform.
//
// Pruned padded transform along one axis (support n, padded P = r*m):
//   X[r q + s] = DFT_m( x[j] W_P^{s j} )[q]          (j < n, zero to m)
//   y[j]       = sum_s W_P^{-s j} IDFT_m( Y[r q + s] )[j]   (j < n)
// The centred embed offset of the reference cancels against the centred
// crop (a circular shift of the input by o followed by a shift of the
// output by -o leaves a circular convolution unchanged), so the support
// starts at index 0 here.
#include <algorithm>
#include <cstdio>
#include "prop_kernels.cuh"
#include "fft_smem.cuh"
#include "elements.cuh"

namespace osgpu {

constexpr int kThreads = 256;
constexpr size_t kSmemBudgetRows = 100 * 1024;

static unsigned long long g_launches = 0;
unsigned long long launch_count() { return g_launches; }
unsigned long long& launch_counter() { return g_launches; }
#define COUNT_LAUNCH() (++g_launches)

__device__ __forceinline__ bool nonfinite2(double a, double b) { return !isfinite(a) || !isfinite(b); }

// ---------------------------------------------------------------- helpers

template <typename T>
__device__ __forceinline__ cx<T> load_in(const void* p, int in_c128, size_t idx) {
  if (in_c128) {
    double2 v = reinterpret_cast<const double2*>(p)[idx];
    return mkc<cx<T>>((T)v.x, (T)v.y);
  }
  float2 v = reinterpret_cast<const float2*>(p)[idx];
  return mkc<cx<T>>((T)v.x, (T)v.y);
}

template <typename T>
__device__ __forceinline__ void store_out(void* p, int out_c128, size_t idx, cx<T> v) {
  if (out_c128) {
    double2 w; w.x = (double)v.x; w.y = (double)v.y;
    reinterpret_cast<double2*>(p)[idx] = w;
  } else {
    float2 w; w.x = (float)v.x; w.y = (float)v.y;
    reinterpret_cast<float2*>(p)[idx] = w;
  }
}

template <typename T>
__device__ __forceinline__ cx<T> apply_elements(const ElementList& L, int ix, int iy, int nx,
                                                int ny, double dx, double dy, cx<T> v) {
  if (sizeof(T) == 4 && L.fast) {
    float2 w = make_float2((float)v.x, (float)v.y);
    w = apply_elements_fast(L, ix, iy, w);
    return mkc<cx<T>>((T)w.x, (T)w.y);
  }
  double re = (double)v.x, im = (double)v.y;
  apply_elements_exact(L, ix, iy, nx, ny, dx, dy, re, im);
  return mkc<cx<T>>((T)re, (T)im);
}

// Per-sample input stage of pass A: adjoint seed weight, else the fused
// forward elements.
template <typename T>
__device__ __forceinline__ cx<T> pass_a_input(const PropArgs& a, int ix, int iy, size_t k,
                                              cx<T> v) {
  if (a.seed) {
    const double w = a.seed_f64 ? reinterpret_cast<const double*>(a.seed)[k]
                                : (double)reinterpret_cast<const float*>(a.seed)[k];
    const T ws = (T)(w * a.seed_scale);
    return mkc<cx<T>>(ws * v.x, ws * v.y);
  }
  if (a.els.count && !a.adj) return apply_elements<T>(a.els, ix, iy, a.nx, a.ny, a.dx, a.dy, v);
  return v;
}

// Per-sample output stage of pass C for an adjoint element plane.
template <typename T>
__device__ __forceinline__ cx<T> pass_c_adjoint(const PropArgs& a, int ix, int iy, size_t o,
                                                cx<T> v) {
  const cx<T> u = load_in<T>(a.adj_uin, a.adj_uin_c128, o);
  T mr = v.x, mi = v.y;
  adjoint_plane<T>(a.els, a.adj_grad, ix, iy, a.nx, a.ny, a.dx, a.dy, o, (T)u.x, (T)u.y, mr, mi);
  return mkc<cx<T>>(mr, mi);
}

// Transmitting-set predicate of one element with psi == 0 (frame
// coordinates are then exactly (xr, yr)); same FP64 expressions as
// apply_elements_exact.
__device__ bool el_inside_psi0(const DevElement& e, double xr, double yr) {
  switch (e.kind) {
    case EL_ELLIPSE: {
      double a2 = __dmul_rn(e.a, e.a), b2 = __dmul_rn(e.b, e.b);
      double lhs = __dadd_rn(__dmul_rn(__dmul_rn(b2, xr), xr), __dmul_rn(__dmul_rn(a2, yr), yr));
      return !(lhs > __dmul_rn(a2, b2));
    }
    case EL_RECT:
      return !(fabs(xr) > e.a || fabs(yr) > e.b);
    default:
      return stop_contains(e.stop, e.a, e.b, xr, yr);
  }
}

// Per-row spans, per-axis factors and bilinear lookups for one element.
// Along a row the predicate depends on |fl(x - cx)| monotonically, so the
// transmitting set is an interval around the column nearest cx; it is
// found by binary search with the exact predicate.
__global__ void k_element_tables(DevElement e, int nx, int ny, double dx, double dy, int2* span,
                                 float2* tabx, float2* taby, int4* bilx, int4* bily) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (span && i < ny) {
    const double yr = __dsub_rn(coord_d(i, ny, dy), e.cy);
    auto xr_of = [&](int ix) { return __dsub_rn(coord_d(ix, nx, dx), e.cx); };
    auto inside = [&](int ix) { return el_inside_psi0(e, xr_of(ix), yr); };
    int ic = (int)rint(e.cx / dx + ((double)nx - 1.0) / 2.0);
    ic = max(0, min(nx - 1, ic));
    for (int d = -2; d <= 2; ++d) {
      const int j = ic + d;
      if (j >= 0 && j < nx && fabs(xr_of(j)) < fabs(xr_of(ic))) ic = j;
    }
    int2 sp = make_int2(1, 0);
    if (inside(ic)) {
      int lo, hi;
      if (inside(0)) {
        lo = 0;
      } else {
        int a = 0, b = ic;
        while (b - a > 1) {
          const int mid = (a + b) / 2;
          if (inside(mid)) b = mid; else a = mid;
        }
        lo = b;
      }
      if (inside(nx - 1)) {
        hi = nx - 1;
      } else {
        int a = ic, b = nx - 1;
        while (b - a > 1) {
          const int mid = (a + b) / 2;
          if (inside(mid)) a = mid; else b = mid;
        }
        hi = a;
      }
      sp = make_int2(lo, hi);
    }
    span[i] = sp;
  }
  if (i < nx) {
    const double xr = __dsub_rn(coord_d(i, nx, dx), e.cx);
    if (tabx && e.kind == EL_LENS) {
      double s, c;
      sincos(__ddiv_rn(__dmul_rn(-e.k, __dmul_rn(xr, xr)), __dmul_rn(2.0, e.f)), &s, &c);
      tabx[i] = make_float2((float)c, (float)s);
    }
    if (tabx && e.kind == EL_GRATING) {
      const double u = __dmul_rn(xr, e.inv_period);
      double s, c;
      sincos(__dmul_rn(e.depth, __dsub_rn(u, floor(u))), &s, &c);
      tabx[i] = make_float2((float)c, (float)s);
    }
    if (bilx) {
      const double g = __dadd_rn(__ddiv_rn(xr, e.ldx), ((double)e.lnx - 1.0) / 2.0);
      const bool ok = !(g < 0.0 || g > (double)e.lnx - 1.0);
      int i0 = 0, i1 = 0;
      float t = 0.f;
      if (ok) {
        i0 = (int)floor(g);
        i1 = min(i0 + 1, e.lnx - 1);
        t = (float)__dsub_rn(g, (double)i0);
      }
      bilx[i] = make_int4(i0, i1, __float_as_int(t), ok ? 1 : 0);
    }
  }
  if (i < ny) {
    const double yr = __dsub_rn(coord_d(i, ny, dy), e.cy);
    if (taby && e.kind == EL_LENS) {
      double s, c;
      sincos(__ddiv_rn(__dmul_rn(-e.k, __dmul_rn(yr, yr)), __dmul_rn(2.0, e.f)), &s, &c);
      taby[i] = make_float2((float)c, (float)s);
    }
    if (bily) {
      const double g = __dadd_rn(__ddiv_rn(yr, e.ldy), ((double)e.lny - 1.0) / 2.0);
      const bool ok = !(g < 0.0 || g > (double)e.lny - 1.0);
      int j0 = 0, j1 = 0;
      float t = 0.f;
      if (ok) {
        j0 = (int)floor(g);
        j1 = min(j0 + 1, e.lny - 1);
        t = (float)__dsub_rn(g, (double)j0);
      }
      bily[i] = make_int4(j0, j1, __float_as_int(t), ok ? 1 : 0);
    }
  }
}

__global__ void k_cast_f64_f32(const double* src, float* dst, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

// Grid-screen transmission e^{i depth v}: the phase formed and reduced mod
// 2 pi in FP64 (a thick element's phase reaches hundreds of radians), the
// reduced angle's sine and cosine in f32.
__global__ void k_screen_table(const double* v64, const float* v32, double depth, float2* out,
                               size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double phi = __dmul_rn(depth, v64 ? v64[i] : (double)v32[i]);
  const double r = phi - 6.283185307179586 * rint(phi * 0.15915494309189535);
  float s, c;
  sincosf((float)r, &s, &c);
  out[i] = make_float2(c, s);
}

__global__ void k_transmission(ElementList L, int nx, int ny, float2* t) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nx * ny) return;
  const int ix = (int)(i % nx), iy = (int)(i / nx);
  t[i] = apply_elements_fast(L, ix, iy, make_float2(1.f, 0.f));
}

// Four consecutive samples of a row per thread (nx % 4 == 0): the chain is
// evaluated element by element for the four, so their table and lattice loads
// are in flight together, and the result leaves as two 16-byte stores.
__global__ void k_transmission4(ElementList L, int nx, int ny, float2* t) {
  const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int nq = nx / 4;
  if (q >= (size_t)nq * ny) return;
  const int iy = (int)(q / nq), ix0 = 4 * (int)(q % nq);
  int ix[4], iyv[4];
  float2 v[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    ix[k] = ix0 + k;
    iyv[k] = iy;
    v[k] = make_float2(1.f, 0.f);
  }
  apply_elements_fast_k<4>(L, ix, iyv, 0xfu, v);
  float4* o = reinterpret_cast<float4*>(t + (size_t)iy * nx + ix0);
  o[0] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
  o[1] = make_float4(v[2].x, v[2].y, v[3].x, v[3].y);
}

cudaError_t launch_transmission(const ElementList& L, int nx, int ny, float2* t, cudaStream_t st) {
  const size_t n = (size_t)nx * ny;
  COUNT_LAUNCH();
  if (nx % 4 == 0) {
    const size_t nq = n / 4;
    k_transmission4<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(L, nx, ny, t);
  } else {
    k_transmission<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(L, nx, ny, t);
  }
  return cudaGetLastError();
}

__global__ void k_c128_to_c64(const double2* src, float4* dst, size_t n2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const double2 a = src[2 * i], b = src[2 * i + 1];  // two samples
  dst[i] = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
}

__global__ void k_c64_to_c128(const float4* src, double2* dst, size_t n2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n2) return;
  const float4 v = src[i];
  dst[2 * i] = make_double2(v.x, v.y);
  dst[2 * i + 1] = make_double2(v.z, v.w);
}

__global__ void k_c128_to_c64_1(const double2* src, float2* dst, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}

__global__ void k_c64_to_c128_1(const float2* src, double2* dst, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = make_double2(src[i].x, src[i].y);
}

cudaError_t launch_c128_to_c64(const void* src, void* dst, size_t n, cudaStream_t st) {
  COUNT_LAUNCH();
  if (n % 2 == 0) {
    const size_t n2 = n / 2;
    k_c128_to_c64<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const double2*>(src), reinterpret_cast<float4*>(dst), n2);
  } else {
    k_c128_to_c64_1<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const double2*>(src), reinterpret_cast<float2*>(dst), n);
  }
  return cudaGetLastError();
}

cudaError_t launch_c64_to_c128(const void* src, void* dst, size_t n, cudaStream_t st) {
  COUNT_LAUNCH();
  if (n % 2 == 0) {
    const size_t n2 = n / 2;
    k_c64_to_c128<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const float4*>(src), reinterpret_cast<double2*>(dst), n2);
  } else {
    k_c64_to_c128_1<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const float2*>(src), reinterpret_cast<double2*>(dst), n);
  }
  return cudaGetLastError();
}

size_t element_tables_bytes(const DevElement& e, int nx, int ny) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t b = al((size_t)ny * sizeof(int2));
  if (e.kind == EL_LENS || e.kind == EL_GRATING) b += al((size_t)nx * sizeof(float2));
  if (e.kind == EL_LENS) b += al((size_t)ny * sizeof(float2));
  if (e.kind == EL_PHASE)
    b += al((size_t)nx * sizeof(int4)) + al((size_t)ny * sizeof(int4)) +
         al((size_t)e.lnx * e.lny * sizeof(float));
  if (e.kind == EL_SCREEN) b += al((size_t)e.lnx * e.lny * sizeof(float2));
  return b;
}

cudaError_t launch_element_tables(DevElement& e, int nx, int ny, double dx, double dy,
                                  void* scratch, cudaStream_t st) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* p = reinterpret_cast<char*>(scratch);
  const bool has_span = (e.kind == EL_ELLIPSE || e.kind == EL_RECT || e.stop != STOP_FIELD);
  int2* span = reinterpret_cast<int2*>(p);
  p += al((size_t)ny * sizeof(int2));
  float2 *tx = nullptr, *ty = nullptr;
  int4 *bx = nullptr, *by = nullptr;
  float* lf = nullptr;
  if (e.kind == EL_LENS || e.kind == EL_GRATING) {
    tx = reinterpret_cast<float2*>(p);
    p += al((size_t)nx * sizeof(float2));
  }
  if (e.kind == EL_LENS) {
    ty = reinterpret_cast<float2*>(p);
    p += al((size_t)ny * sizeof(float2));
  }
  if (e.kind == EL_PHASE) {
    bx = reinterpret_cast<int4*>(p);
    p += al((size_t)nx * sizeof(int4));
    by = reinterpret_cast<int4*>(p);
    p += al((size_t)ny * sizeof(int4));
  }
  if (e.kind == EL_SCREEN) {
    float2* t = reinterpret_cast<float2*>(p);
    p += al((size_t)e.lnx * e.lny * sizeof(float2));
    const size_t n = (size_t)e.lnx * e.lny;
    COUNT_LAUNCH();
    k_screen_table<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(e.lat, e.latf, e.depth, t, n);
    e.scr = t;
  }
  if (e.kind == EL_PHASE) {
    if (e.latf) {
      lf = const_cast<float*>(e.latf);  // f32 copy kept with the lattice handle
    } else {
      lf = reinterpret_cast<float*>(p);
      const size_t n = (size_t)e.lnx * e.lny;
      COUNT_LAUNCH();
      k_cast_f64_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(e.lat, lf, n);
    }
  }
  const int n = max(nx, ny);
  COUNT_LAUNCH();
  k_element_tables<<<(n + 127) / 128, 128, 0, st>>>(e, nx, ny, dx, dy, has_span ? span : nullptr,
                                                    tx, ty, bx, by);
  e.span = has_span ? span : nullptr;
  e.tabx = tx;
  e.taby = ty;
  e.bilx = bx;
  e.bily = by;
  e.latf = lf;
  return cudaGetLastError();
}

// ----------------------------------------------------------------- tables

__global__ void k_twiddles(void* dst, int n, int is_double) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  // W_n^k = e^{-2 pi i k / n}; sincospi on the exact ratio 2k/n.
  double s, c;
  sincospi(2.0 * (double)k / (double)n, &s, &c);
  if (is_double) {
    reinterpret_cast<double2*>(dst)[k] = make_double2(c, -s);
  } else {
    reinterpret_cast<float2*>(dst)[k] = make_float2((float)c, (float)-s);
  }
}

cudaError_t launch_twiddles(void* dst, int n, int is_double, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  COUNT_LAUNCH();
  k_twiddles<<<(n + 255) / 256, 256, 0, st>>>(dst, n, is_double);
  return cudaGetLastError();
}

// Per-axis tables for the transfer function.  fxv/fyv always; the f32
// split tables when h_mode == 1:
//   ASM: phi = K sqrt(1-s), s = a + b, a = (lam_n fx)^2, b = (lam_n fy)^2
//        = K + [-K a/2 - K a^2/8] + [-K b/2 - K b^2/8] + [-K a b/4] - K tau(s)
//        with tau(s) = s^3 (3+q) / (8 (1+q)^3), q = sqrt(1-s).
//   The bracketed separable terms and e^{iK} are evaluated in FP64 into Ex/Ey;
//   the cross term -K a b/4 runs in double-float; tau in f32.
//   kmax[kx] is the largest |k_y| whose bin the reference keeps (evanescent
//   and band-limit tests evaluated in FP64 exactly as asm.rs:505-522).
//   Fresnel TF: Ex = e^{i (kz - c fx^2)} * scale, Ey = e^{-i c fy^2}.
__global__ void k_axis_prep(PropArgs a, double* fxv, double* fyv, float2* Ex, float2* Ey,
                            float* ca_hi, float* ca_lo, float* sa, float* b_hi, float* b_lo,
                            int* kmax, float4* rowtab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int Px = a.ax.P, Py = a.ay.P;
  const double K = a.kz;
  if (i < Px) {
    const double fx = fftfreq_d(i, Px, a.dx);
    fxv[i] = fx;
    if (a.h_mode == 1) {
      if (a.engine == ENG_ASM) {
        const double al = a.lam_n * fx;
        const double aa = al * al;
        const double phx = K - K * aa * 0.5 - K * aa * aa * 0.125;
        double s, c;
        sincos(phx, &s, &c);
        Ex[i] = make_float2((float)(c * a.scale), (float)(s * a.scale));
        const double ca = -K * aa * 0.25;
        const float h = (float)ca;
        ca_hi[i] = h;
        ca_lo[i] = (float)(ca - (double)h);
        sa[i] = (float)aa;
        // kmax: exact reference predicate, monotone in |k_y|.
        int km = -1;
        if (!(a.band_limited && fabs(fx) > a.lim_x)) {
          const double axx = __dmul_rn(a.lam_n, fx);
          const double t1 = __dsub_rn(1.0, __dmul_rn(axx, axx));
          auto ok = [&](int kk) {
            double fy = __ddiv_rn((double)kk, __dmul_rn((double)Py, a.dy));
            if (a.band_limited && fabs(fy) > a.lim_y) return false;
            double ayy = __dmul_rn(a.lam_n, fy);
            return !(__dsub_rn(t1, __dmul_rn(ayy, ayy)) < 0.0);
          };
          if (ok(0)) {
            int lo = 0, hi = Py / 2;
            if (ok(hi)) {
              lo = hi;
            } else {
              while (hi - lo > 1) {
                int mid = (lo + hi) / 2;
                if (ok(mid)) lo = mid; else hi = mid;
              }
            }
            km = lo;
          }
        }
        kmax[i] = km;
      } else if (a.engine == ENG_FRESNEL_TF) {
        const double ph = a.kz - a.cfr * (fx * fx);
        double s, c;
        sincos(ph, &s, &c);
        Ex[i] = make_float2((float)(c * a.scale), (float)(s * a.scale));
      }
    }
  }
  if (i < Py) {
    const double fy = fftfreq_d(i, Py, a.dy);
    fyv[i] = fy;
    if (a.h_mode == 1) {
      if (a.engine == ENG_ASM) {
        const double bl = a.lam_n * fy;
        const double bb = bl * bl;
        const double phy = -K * bb * 0.5 - K * bb * bb * 0.125;
        double s, c;
        sincos(phy, &s, &c);
        Ey[i] = make_float2((float)c, (float)s);
        const float h = (float)bb;
        b_hi[i] = h;
        b_lo[i] = (float)(bb - (double)h);
        if (rowtab) rowtab[i] = make_float4((float)c, (float)s, h, (float)(bb - (double)h));
      } else if (a.engine == ENG_FRESNEL_TF) {
        const double ph = -a.cfr * (fy * fy);
        double s, c;
        sincos(ph, &s, &c);
        Ey[i] = make_float2((float)c, (float)s);
        if (rowtab) rowtab[i] = make_float4((float)c, (float)s, 0.f, 0.f);
      }
    }
  }
}

template <typename T>
cudaError_t launch_asm_prep(const PropArgs& a, void* tables, cudaStream_t st) {
  (void)tables;
  const int n = max(a.ax.P, a.ay.P);
  COUNT_LAUNCH();
  k_axis_prep<<<(n + 127) / 128, 128, 0, st>>>(
      a, const_cast<double*>(a.fxv), const_cast<double*>(a.fyv), const_cast<float2*>(a.Ex),
      const_cast<float2*>(a.Ey), const_cast<float*>(a.ca_hi), const_cast<float*>(a.ca_lo),
      const_cast<float*>(a.sa), const_cast<float*>(a.b_hi), const_cast<float*>(a.b_lo),
      const_cast<int*>(a.kmax), reinterpret_cast<float4*>(const_cast<void*>(a.rowtab)));
  return cudaGetLastError();
}

// ---------------------------------------------------------------- pass A

size_t smem_passA_bytes(const AxisPlan& ax, int is_double, int rows) {
  const size_t es = is_double ? 16 : 8;
  const size_t ld = (size_t)ax.m + 1;
  return (2 * ld + (ax.r > 1 ? (size_t)ax.n : 0)) * rows * es;
}

bool prop_smem_fits(const AxisPlan& ax, const AxisPlan& ay, int is_double, size_t max_smem) {
  const size_t es = is_double ? 16 : 8;
  return smem_passA_bytes(ax, is_double, 1) <= max_smem &&
         smem_passB_bytes(ay, is_double) <= max_smem &&
         (2 * ((size_t)ax.m + 1) + (size_t)ax.n) * es <= max_smem;  // pass C, one row
}

int rows_per_cta(const AxisPlan& ax, int is_double) {
  int rows = 16;
  while (rows > 1 && smem_passA_bytes(ax, is_double, rows) > kSmemBudgetRows) rows /= 2;
  return rows;
}

// Row forward transforms of the n input rows (elements fused), written to
// the column-major spectrum scratch W[kx * ny + iy].
template <typename T>
__global__ void __launch_bounds__(kThreads) k_passA(PropArgs a, int rows) {
  using V = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = a.ax.m, r = a.ax.r, nx = a.nx, ny = a.ny;
  const int ld = m + 1;
  V* bufA = reinterpret_cast<V*>(smem_raw);
  V* bufB = bufA + (size_t)rows * ld;
  V* xin = bufB + (size_t)rows * ld;  // staged input rows when r > 1
  const int row0 = blockIdx.x * rows;
  const V* twm = reinterpret_cast<const V*>(a.tw_mx);
  const V* twP = reinterpret_cast<const V*>(a.tw_Px);
  V* W = reinterpret_cast<V*>(a.work);
  const V zero = mkc<V>((T)0, (T)0);

  if (r > 1) {
    for (int e = threadIdx.x; e < rows * nx; e += blockDim.x) {
      const int i = e / nx, j = e - i * nx, iy = row0 + i;
      V v = zero;
      if (iy < ny) {
        v = load_in<T>(a.in, a.in_c128, (size_t)iy * nx + j);
        if (a.status && nonfinite2((double)v.x, (double)v.y)) atomicOr(a.status, 1);
        v = pass_a_input<T>(a, j, iy, (size_t)iy * nx + j, v);
      }
      xin[(size_t)i * nx + j] = v;
    }
    __syncthreads();
  }
  for (int s = 0; s < r; ++s) {
    for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
      const int i = e / m, j = e - i * m, iy = row0 + i;
      V v = zero;
      if (iy < ny && j < nx) {
        if (r > 1) {
          v = xin[(size_t)i * nx + j];
          if (s > 0) v = cmul(v, twP[s * j]);
        } else {
          v = load_in<T>(a.in, a.in_c128, (size_t)iy * nx + j);
          if (a.status && nonfinite2((double)v.x, (double)v.y)) atomicOr(a.status, 1);
          v = pass_a_input<T>(a, j, iy, (size_t)iy * nx + j, v);
        }
      }
      bufA[(size_t)i * ld + j] = v;
    }
    __syncthreads();
    V* res = stockham<T, false>(bufA, bufB, m, rows, ld, a.ax, twm);
    for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
      const int i = e % rows, q = e / rows, iy = row0 + i;
      if (iy < ny) W[(size_t)(r * q + s) * ny + iy] = res[(size_t)i * ld + q];
    }
    __syncthreads();
  }
}

template <typename T>
cudaError_t launch_passA(const PropArgs& a, cudaStream_t st) {
  if (sizeof(T) == 4 && reg_fft_size(a.ax.m)) return launch_passA_reg(a, st);
  const int is_d = sizeof(T) == 8;
  const int rows = rows_per_cta(a.ax, is_d);
  const size_t smem = smem_passA_bytes(a.ax, is_d, rows);
  cudaError_t e = cudaFuncSetAttribute(k_passA<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((a.ny + rows - 1) / rows);
  COUNT_LAUNCH();
  k_passA<T><<<grid, kThreads, smem, st>>>(a, rows);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- pass B

size_t smem_passB_bytes(const AxisPlan& ay, int is_double) {
  const size_t es = is_double ? 16 : 8;
  return (2 * (size_t)ay.m + 2 * (size_t)ay.n) * es;
}

template <typename T>
__device__ __forceinline__ cx<T> transfer_exact(const PropArgs& a, double fx, double fy) {
  using V = cx<T>;
  double ph;
  if (a.engine == ENG_ASM) {
    if (a.band_limited && (fabs(fx) > a.lim_x || fabs(fy) > a.lim_y)) return mkc<V>((T)0, (T)0);
    const double axx = __dmul_rn(a.lam_n, fx), ayy = __dmul_rn(a.lam_n, fy);
    const double sv = __dsub_rn(__dsub_rn(1.0, __dmul_rn(axx, axx)), __dmul_rn(ayy, ayy));
    if (sv < 0.0) return mkc<V>((T)0, (T)0);
    ph = __dmul_rn(a.kz, __dsqrt_rn(sv));
  } else {  // ENG_FRESNEL_TF
    ph = __dsub_rn(a.kz, __dmul_rn(a.cfr, __dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy))));
  }
  double s, c;
  sincos(ph, &s, &c);
  return mkc<V>((T)(c * a.scale), (T)(s * a.scale));
}

// One CTA per spectral column kx: pruned forward column FFT, transfer
// function, pruned inverse column FFT; the column is rewritten in place.
// fwd_only: forward transform only, result (all Py bins) written to `dst`.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_passB(PropArgs a, int fwd_only, void* dst) {
  using V = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int my = a.ay.m, ry = a.ay.r, Py = a.ay.P, ny = a.ny;
  const int kx = blockIdx.x;
  V* buf0 = reinterpret_cast<V*>(smem_raw);
  V* buf1 = buf0 + my;
  V* col = buf1 + my;
  V* acc = col + ny;
  const V* twm = reinterpret_cast<const V*>(a.tw_my);
  const V* twP = reinterpret_cast<const V*>(a.tw_Py);
  V* W = reinterpret_cast<V*>(a.work) + (size_t)kx * ny;
  const V zero = mkc<V>((T)0, (T)0);

  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    col[j] = W[j];
    acc[j] = zero;
  }
  // Per-column transfer-function data.
  double fx = 0.0;
  float2 exc = make_float2(0.f, 0.f);
  float cah = 0.f, cal = 0.f, sac = 0.f;
  int kmc = -1;
  if (!fwd_only) {
    if (a.h_mode == 0 && (a.engine == ENG_ASM || a.engine == ENG_FRESNEL_TF)) fx = a.fxv[kx];
    if (a.h_mode == 1 && (a.engine == ENG_ASM || a.engine == ENG_FRESNEL_TF)) {
      exc = a.Ex[kx];
      if (a.engine == ENG_ASM) {
        cah = a.ca_hi[kx];
        cal = a.ca_lo[kx];
        sac = a.sa[kx];
        kmc = a.kmax[kx];
      }
    }
  }
  __syncthreads();
  for (int t = 0; t < ry; ++t) {
    for (int j = threadIdx.x; j < my; j += blockDim.x) {
      V v = zero;
      if (j < ny) {
        v = col[j];
        if (t > 0) v = cmul(v, twP[t * j]);
      }
      buf0[j] = v;
    }
    __syncthreads();
    V* res = stockham<T, false>(buf0, buf1, my, 1, my, a.ay, twm);
    if (fwd_only) {
      V* D = reinterpret_cast<V*>(dst) + (size_t)kx * Py;
      for (int p = threadIdx.x; p < my; p += blockDim.x) D[ry * p + t] = cscale(res[p], (T)a.scale);
      __syncthreads();
      continue;
    }
    for (int p = threadIdx.x; p < my; p += blockDim.x) {
      const int ky = ry * p + t;
      V h;
      if (a.engine == ENG_KSPEC) {
        h = reinterpret_cast<const V*>(a.kspec)[(size_t)kx * Py + ky];
        if (a.conj_h) h.y = -h.y;
      } else if (a.engine == ENG_KEVEN) {
        const int kxq = min(kx, a.ax.P - kx), kyq = min(ky, Py - ky);
        const float2 k = reinterpret_cast<const float2*>(a.kspec)[(size_t)kxq * (Py / 2 + 1) + kyq];
        h = mkc<V>((T)k.x, (T)(a.conj_h ? -k.y : k.y));
      } else if (a.engine == ENG_KSEP) {
        h = cmul(reinterpret_cast<const V*>(a.hx)[kx], reinterpret_cast<const V*>(a.hy)[ky]);
        if (a.conj_h) h.y = -h.y;
      } else if (a.engine == ENG_IDENTITY) {
        h = mkc<V>((T)a.scale, (T)0);
      } else if (a.h_mode == 0) {
        h = transfer_exact<T>(a, fx, a.fyv[ky]);
      } else if (a.engine == ENG_FRESNEL_TF) {
        const float2 ey = a.Ey[ky];
        h = mkc<V>((T)(exc.x * ey.x - exc.y * ey.y), (T)(exc.x * ey.y + exc.y * ey.x));
      } else {
        const int kk = (ky <= (Py - 1) / 2) ? ky : ky - Py;
        if (abs(kk) > kmc) {
          h = zero;
        } else {
          const float bh = a.b_hi[ky], blo = a.b_lo[ky];
          const float s = sac + bh;
          const float q = sqrtf(fmaxf(1.f - s, 0.f));
          const float opq = 1.f + q;
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
          h = mkc<V>((T)(hr * cs - hi * sn), (T)(hr * sn + hi * cs));
        }
      }
      res[p] = cmul(res[p], h);
    }
    __syncthreads();
    V* other = (res == buf0) ? buf1 : buf0;
    V* res2 = stockham<T, true>(res, other, my, 1, my, a.ay, twm);
    for (int j = threadIdx.x; j < ny; j += blockDim.x) {
      V v = res2[j];
      if (t > 0) v = cmulc(v, twP[t * j]);
      acc[j] = cadd(acc[j], v);
    }
    __syncthreads();
  }
  if (!fwd_only) {
    for (int j = threadIdx.x; j < ny; j += blockDim.x) W[j] = acc[j];
  }
}

template <typename T>
static cudaError_t launch_passB_impl(const PropArgs& a, int fwd_only, void* dst, cudaStream_t st) {
  const int is_d = sizeof(T) == 8;
  const size_t smem = smem_passB_bytes(a.ay, is_d);
  cudaError_t e = cudaFuncSetAttribute(k_passB<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_passB<T><<<a.ax.P, kThreads, smem, st>>>(a, fwd_only, dst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_passB(const PropArgs& a, cudaStream_t st) {
  const bool tf = (a.engine == ENG_ASM || a.engine == ENG_FRESNEL_TF);
  if (sizeof(T) == 4 && reg_fft_size(a.ay.m) && (!tf || a.h_mode == 1))
    return launch_passB_reg(a, st);
  return launch_passB_impl<T>(a, 0, nullptr, st);
}

// ---------------------------------------------------------------- pass C

// Inverse row transforms + crop: out[iy][j] = sum_s W_Px^{-s j} IDFT_m(Z_s)[j].
template <typename T>
__global__ void __launch_bounds__(kThreads) k_passC(PropArgs a, int rows) {
  using V = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = a.ax.m, r = a.ax.r, nx = a.nx, ny = a.ny;
  const int ld = m + 1;
  V* bufA = reinterpret_cast<V*>(smem_raw);
  V* bufB = bufA + (size_t)rows * ld;
  V* acc = bufB + (size_t)rows * ld;
  const int row0 = blockIdx.x * rows;
  const V* twm = reinterpret_cast<const V*>(a.tw_mx);
  const V* twP = reinterpret_cast<const V*>(a.tw_Px);
  const V* W = reinterpret_cast<const V*>(a.work);

  for (int s = 0; s < r; ++s) {
    for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
      const int i = e % rows, q = e / rows, iy = row0 + i;
      bufA[(size_t)i * ld + q] =
          (iy < ny) ? W[(size_t)(r * q + s) * ny + iy] : mkc<V>((T)0, (T)0);
    }
    __syncthreads();
    V* res = stockham<T, true>(bufA, bufB, m, rows, ld, a.ax, twm);
    for (int e = threadIdx.x; e < rows * nx; e += blockDim.x) {
      const int i = e / nx, j = e - i * nx;
      V v = res[(size_t)i * ld + j];
      if (s > 0) v = cmulc(v, twP[s * j]);
      if (r > 1) {
        if (s == 0) acc[(size_t)i * nx + j] = v;
        else acc[(size_t)i * nx + j] = cadd(acc[(size_t)i * nx + j], v);
      } else {
        acc[(size_t)i * nx + j] = v;
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < rows * nx; e += blockDim.x) {
    const int i = e / nx, j = e - i * nx, iy = row0 + i;
    if (iy >= ny) continue;
    V v = acc[(size_t)i * nx + j];
    const size_t o = (size_t)iy * nx + j;
    if (a.adj) v = pass_c_adjoint<T>(a, j, iy, o, v);
    if (a.status && nonfinite2((double)v.x, (double)v.y)) atomicOr(a.status, 2);
    if (a.out) store_out<T>(a.out, a.out_c128, o, v);
    if (a.out_intensity) a.out_intensity[o] = (float)((double)v.x * v.x + (double)v.y * v.y);
    if (a.out_intensity64) a.out_intensity64[o] = (double)v.x * v.x + (double)v.y * v.y;
  }
}

static size_t smem_passC_bytes(const AxisPlan& ax, int is_double, int rows) {
  const size_t es = is_double ? 16 : 8;
  return (2 * ((size_t)ax.m + 1) + (size_t)ax.n) * rows * es;
}

template <typename T>
cudaError_t launch_passC(const PropArgs& a, cudaStream_t st) {
  if (sizeof(T) == 4 && reg_fft_size(a.ax.m)) return launch_passC_reg(a, st);
  const int is_d = sizeof(T) == 8;
  int rows = 16;
  while (rows > 1 && smem_passC_bytes(a.ax, is_d, rows) > kSmemBudgetRows) rows /= 2;
  const size_t smem = smem_passC_bytes(a.ax, is_d, rows);
  cudaError_t e = cudaFuncSetAttribute(k_passC<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_passC<T><<<(a.ny + rows - 1) / rows, kThreads, smem, st>>>(a, rows);
  return cudaGetLastError();
}

// ------------------------------------------------------ kernel spectra

// DFT-order coordinate (reference fresnel.rs:322-328).
__device__ __forceinline__ double dft_coord(int i, int n, double d) {
  return (i <= n / 2) ? __dmul_rn((double)i, d) : __dmul_rn(__dsub_rn((double)i, (double)n), d);
}

// Direct length-n DFT of one row (used for the two 1-D chirp spectra of the
// separable Fresnel kernel; O(n^2) once per (lambda, z, grid)).
// chirp[j] = e^{i A x_j^2} at the DFT-order coordinates (computed once, not
// per output bin)
__global__ void k_chirp_vals(int n, double d, double A, double2* chirp) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double x = dft_coord(j, n, d);
  double s, c;
  sincos(__dmul_rn(A, __dmul_rn(x, x)), &s, &c);
  chirp[j] = make_double2(c, s);
}

// One block of kChirpThreads per output bin k: thread t sums the terms
// j = t, t + kChirpThreads, ... with the twiddle index (j k) mod n advanced
// by a conditional subtraction (no division in the loop), then the block
// adds the partial sums (FP64 throughout).
constexpr int kChirpThreads = 128;

__global__ void __launch_bounds__(kChirpThreads)
    k_chirp_dft(int n, const double2* __restrict__ chirp, const double2* __restrict__ tw,
                double2* out, double pre_re, double pre_im) {
  const int k = blockIdx.x, t = threadIdx.x;
  int idx = (int)(((long long)t * k) % n);
  const int step = (int)(((long long)kChirpThreads * k) % n);
  double sr = 0.0, si = 0.0;
  for (int j = t; j < n; j += kChirpThreads) {
    const double2 cs = __ldg(chirp + j);
    const double2 w = __ldg(tw + idx);
    sr += cs.x * w.x - cs.y * w.y;
    si += cs.x * w.y + cs.y * w.x;
    idx += step;
    if (idx >= n) idx -= n;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  __shared__ double2 part[kChirpThreads / 32];
  if ((t & 31) == 0) part[t >> 5] = make_double2(sr, si);
  __syncthreads();
  if (t == 0) {
    sr = part[0].x;
    si = part[0].y;
    for (int w = 1; w < kChirpThreads / 32; ++w) {
      sr += part[w].x;
      si += part[w].y;
    }
    out[k] = make_double2(sr * pre_re - si * pre_im, sr * pre_im + si * pre_re);
  }
}

template <typename T>
__global__ void k_cast_c128(const double2* src, void* dst, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = src[i];
  if (sizeof(T) == 8) reinterpret_cast<double2*>(dst)[i] = v;
  else reinterpret_cast<float2*>(dst)[i] = make_float2((float)v.x, (float)v.y);
}

// hx[kx] = pref * scale * DFT(e^{i A x^2}), hy[ky] = DFT(e^{i A y^2}),
// A = pi / (lam z); the product is the 2-D spectrum of the sampled kernel
// h = pref e^{i pi (x^2+y^2)/(lam z)} (reference fresnel.rs:312-338).
template <typename T>
cudaError_t launch_fresnel_ksep(const PropArgs& a, void* hx, void* hy, void* tmp, cudaStream_t st) {
  // tmp: (Px + Py) double2 twiddles, results and chirp samples each
  const int Px = a.ax.P, Py = a.ay.P;
  double2* twx = reinterpret_cast<double2*>(tmp);
  double2* twy = twx + Px;
  double2* ox = twy + Py;
  double2* oy = ox + Px;
  double2* cx = oy + Py;
  double2* cy = cx + Px;
  cudaError_t e = launch_twiddles(twx, Px, 1, st);
  if (e != cudaSuccess) return e;
  e = launch_twiddles(twy, Py, 1, st);
  if (e != cudaSuccess) return e;
  const double A = M_PI / (a.lam * a.z);
  // pref = e^{ikz}/(i lam z) * dx dy, folded with the 1/(Px Py) scale.
  const double k = 2.0 * M_PI / a.lam;
  const double kz = k * a.z;
  const double lz = a.lam * a.z;
  // e^{ikz} / (i lz) = (cos + i sin) * (-i / lz) = (sin / lz) - i (cos / lz)
  const double pr = sin(kz) / lz * (a.dx * a.dy) * a.scale;
  const double pi_ = -cos(kz) / lz * (a.dx * a.dy) * a.scale;
  COUNT_LAUNCH();
  k_chirp_vals<<<(Px + 127) / 128, 128, 0, st>>>(Px, a.dx, A, cx);
  COUNT_LAUNCH();
  k_chirp_vals<<<(Py + 127) / 128, 128, 0, st>>>(Py, a.dy, A, cy);
  COUNT_LAUNCH();
  k_chirp_dft<<<Px, kChirpThreads, 0, st>>>(Px, cx, twx, ox, pr, pi_);
  COUNT_LAUNCH();
  k_chirp_dft<<<Py, kChirpThreads, 0, st>>>(Py, cy, twy, oy, 1.0, 0.0);
  COUNT_LAUNCH();
  k_cast_c128<T><<<(Px + 255) / 256, 256, 0, st>>>(ox, hx, Px);
  COUNT_LAUNCH();
  k_cast_c128<T><<<(Py + 255) / 256, 256, 0, st>>>(oy, hy, Py);
  return cudaGetLastError();
}

// RS-I kernel samples in DFT order, dx dy folded in (reference
// rayleigh_sommerfeld.rs:228-235, 277-301).
// (2-D grid: x over a row, blockIdx.y the row.)
__global__ void k_rs_kernel(int Px, int Py, double dx, double dy, double lam, double z,
                            double2* h) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y;
  if (ix >= Px) return;
  const size_t idx = (size_t)iy * Px + ix;
  const double x = dft_coord(ix, Px, dx), y = dft_coord(iy, Py, dy);
  const double k = __ddiv_rn(2.0 * M_PI, lam);
  const double sg = z > 0.0 ? 1.0 : -1.0;
  const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
  const double amp = __ddiv_rn(fabs(z), __dmul_rn(__dmul_rn(2.0 * M_PI, r), r));
  const double ob_re = __ddiv_rn(1.0, r), ob_im = -sg * k;
  double s, c;
  sincos(__dmul_rn(__dmul_rn(sg, k), r), &s, &c);
  // amp * obliquity * e^{i s k r} * (dx dy)
  const double pr = amp * ob_re, pi_ = amp * ob_im;
  const double w = __dmul_rn(dx, dy);
  h[idx] = make_double2((pr * c - pi_ * s) * w, (pr * s + pi_ * c) * w);
}

// f32 engine: the same kernel samples with r and the phase s k r in FP64,
// the phase reduced to [-pi, pi] by a two-constant Cody-Waite step
// (2 pi = hi + lo, each product by FMA), and the amplitude, obliquity and
// e^{i phase} in f32.  r = sqrt(s) from the f32 square root r0 of s and one
// Newton step in FP64, r = r0 + (s - r0^2) / (2 r0): r0^2 is exact in FP64
// (24-bit operands) and the step takes the relative error from 2^-24 to
// about 2^-49, so the phase k r (~1e5 rad) keeps ~1e-9 rad with a few FP64
// operations instead of an FP64 square root.
__global__ void k_rs_kernel_f32(int Px, int Py, double dx, double dy, double sk, double z,
                                float2* h) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y;
  if (ix >= Px) return;
  const size_t idx = (size_t)iy * Px + ix;
  const double x = dft_coord(ix, Px, dx), y = dft_coord(iy, Py, dy);
  const double sq = fma(x, x, fma(y, y, z * z));
  const float r0 = sqrtf((float)sq);
  const double e = fma(-(double)r0, (double)r0, sq);
  const double r = fma(e, (double)(0.5f / r0), (double)r0);
  const double ph = __dmul_rn(sk, r);
  const double q = rint(__dmul_rn(ph, 0.15915494309189533577));
  const double red = fma(-q, 2.4492935982947064e-16, fma(-q, 6.283185307179586232, ph));
  float s, c;
  sincosf((float)red, &s, &c);
  const float rf = (float)r;
  const float amp = (float)fabs(z) / (6.2831853071795865f * rf * rf);
  const float pr = amp / rf, pi_ = -amp * (float)sk;
  const float w = (float)(dx * dy);
  h[idx] = make_float2((pr * c - pi_ * s) * w, (pr * s + pi_ * c) * w);
}

template <typename T>
cudaError_t launch_rs_kspec(const PropArgs& a, void* kspec, void* tmp64, cudaStream_t st) {
  // FP64: tmp64 holds h (Px*Py double2), then the column-major work (Px*Py
  // double2), then twiddles (Px + Py double2); `a` carries full-support axis
  // plans.  f32: h and the work as float2 in the same space, and the f32
  // twiddle tables of Px and Py come with `a` (tw_mx, tw_my).
  const int Px = a.ax.P, Py = a.ay.P;
  const size_t n = (size_t)Px * Py;
  if (sizeof(T) == 4) {
    if (!a.tw_mx || !a.tw_my) return cudaErrorInvalidValue;
    float2* hf = reinterpret_cast<float2*>(tmp64);
    const double sg = a.z > 0.0 ? 1.0 : -1.0;
    COUNT_LAUNCH();
    k_rs_kernel_f32<<<dim3((Px + 255) / 256, Py), 256, 0, st>>>(
        Px, Py, a.dx, a.dy, sg * (2.0 * M_PI / a.lam), a.z, hf);
    PropArgs b = a;
    b.nx = Px;
    b.ny = Py;
    b.in = hf;
    b.in_c128 = 0;
    b.work = hf + n;
    b.tw_Px = a.tw_mx;
    b.tw_Py = a.tw_my;
    b.els.count = 0;
    b.trans = nullptr;
    b.seed = nullptr;
    b.adj = 0;
    b.out_intensity = nullptr;
    b.out_intensity64 = nullptr;
    b.engine = ENG_IDENTITY;
    b.sched = Schedule{0, 0, 0};
    cudaError_t e = launch_passA<float>(b, st);
    if (e != cudaSuccess) return e;
    return launch_passB_impl<float>(b, 1, kspec, st);
  }
  double2* h = reinterpret_cast<double2*>(tmp64);
  double2* work = h + (size_t)Px * Py;
  double2* twx = work + (size_t)Px * Py;
  double2* twy = twx + Px;
  cudaError_t e = launch_twiddles(twx, Px, 1, st);
  if (e != cudaSuccess) return e;
  e = launch_twiddles(twy, Py, 1, st);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_rs_kernel<<<dim3((Px + 255) / 256, Py), 256, 0, st>>>(Px, Py, a.dx, a.dy, a.lam, a.z, h);
  PropArgs b = a;
  b.nx = Px;
  b.ny = Py;
  b.in = h;
  b.in_c128 = 1;
  b.work = work;
  b.tw_mx = twx;
  b.tw_Px = twx;
  b.tw_my = twy;
  b.tw_Py = twy;
  b.els.count = 0;
  b.engine = ENG_IDENTITY;
  e = launch_passA<double>(b, st);
  if (e != cudaSuccess) return e;
  double2* spec = reinterpret_cast<double2*>(h);  // reuse h as the f64 spectrum
  e = launch_passB_impl<double>(b, 1, spec, st);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_cast_c128<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(spec, kspec, n);
  return cudaGetLastError();
}

// ------------------------------------------------- kernel-spectrum plans
//
// A propagation out = crop_n(IFFT_P(H FFT_P(pad_n(u)))) only reaches kernel
// offsets |d| < n of h = IFFT_P(H), so it equals the circular convolution of
// period 2n with h restricted to those offsets.  For a transfer function
// even in each axis (ASM: fx^2, fy^2 and |fx|, |fy| band limits), h is even
// too: the quadrant h(y, x), 0 <= x, y < n, is the propagation of a unit
// sample at the origin, and the spectrum of its 2n-periodic even extension
// (zero at offset n, which no output reaches) is
//   K(ky, kx) = sum over the four sign pairs of A(+-ky, +-kx),
//   A = FFT_2n(pad_n(c_y c_x h)),  c_0 = 1/2, c_d = 1 otherwise,
// (the halved first row and column are the offsets shared by two
// reflections), so the pruned zero-padded passes give it directly.  K is
// even; the quarter kx <= n, ky <= n is kept.

// hq[y][x] *= (y == 0 ? 1/2 : 1) (x == 0 ? 1/2 : 1)
__global__ void k_halve_axes(double2* hq, int hnx, int hny) {
  const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (idx >= (size_t)hnx * hny) return;
  const int x = (int)(idx % hnx), y = (int)(idx / hnx);
  const double w = (x == 0 ? 0.5 : 1.0) * (y == 0 ? 0.5 : 1.0);
  if (w != 1.0) hq[idx] = make_double2(hq[idx].x * w, hq[idx].y * w);
}

// kq[kx (Py/2 + 1) + ky] = sum of the column-major spectrum A at (+-kx, +-ky).
__global__ void k_quarter_fold(const double2* A, int Px, int Py, float2* kq) {
  const int hx = Px / 2 + 1, hy = Py / 2 + 1;
  const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (idx >= (size_t)hx * hy) return;
  const int kx = (int)(idx / hy), ky = (int)(idx % hy);
  const int mx = kx == 0 ? 0 : Px - kx, my = ky == 0 ? 0 : Py - ky;
  const double2 a = A[(size_t)kx * Py + ky], b = A[(size_t)mx * Py + ky];
  const double2 c = A[(size_t)kx * Py + my], d = A[(size_t)mx * Py + my];
  kq[idx] = make_float2((float)((a.x + b.x) + (c.x + d.x)), (float)((a.y + b.y) + (c.y + d.y)));
}

cudaError_t launch_even_kspec(const PropArgs& a, void* hq, int hnx, int hny, void* kq,
                              void* tmp64, cudaStream_t st) {
  const int Px = a.ax.P, Py = a.ay.P;
  if (Px != 2 * hnx || Py != 2 * hny || a.ax.n != hnx || a.ay.n != hny) return cudaErrorInvalidValue;
  double2* h = reinterpret_cast<double2*>(hq);
  double2* work = reinterpret_cast<double2*>(tmp64);
  double2* spec = work + (size_t)Px * hny;
  const size_t n = (size_t)hnx * hny;
  COUNT_LAUNCH();
  k_halve_axes<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(h, hnx, hny);
  PropArgs b = a;
  b.nx = hnx;
  b.ny = hny;
  b.in = h;
  b.in_c128 = 1;
  b.work = work;
  b.els.count = 0;
  b.seed = nullptr;
  b.adj = 0;
  b.status = nullptr;
  b.engine = ENG_IDENTITY;
  cudaError_t e = launch_passA<double>(b, st);
  if (e != cudaSuccess) return e;
  e = launch_passB_impl<double>(b, 1, spec, st);
  if (e != cudaSuccess) return e;
  const size_t nq = (size_t)(Px / 2 + 1) * (Py / 2 + 1);
  COUNT_LAUNCH();
  k_quarter_fold<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(spec, Px, Py,
                                                               reinterpret_cast<float2*>(kq));
  return cudaGetLastError();
}

// ------------------------------------------------------------ plain 2D DFT

// Input stage of an inverse transform: dst = conj(src) in the engine's type.
template <typename T>
__global__ void k_conj_copy(const void* src, int c128, cx<T>* dst, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  cx<T> v = load_in<T>(src, c128, i);
  v.y = -v.y;
  dst[i] = v;
}

// Column-major spectrum S[kx * ny + ky] -> row-major out[ky * nx + kx]
// (conjugated for an inverse), 32 x 32 tiles through shared memory.
template <typename T>
__global__ void k_fft2_finish(const cx<T>* S, int nx, int ny, void* out, int out_c128, int conj) {
  __shared__ cx<T> tile[32][33];
  const int kx0 = blockIdx.x * 32, ky0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int kx = kx0 + j, ky = ky0 + threadIdx.x;
    if (kx < nx && ky < ny) tile[j][threadIdx.x] = S[(size_t)kx * ny + ky];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int ky = ky0 + j, kx = kx0 + threadIdx.x;
    if (kx < nx && ky < ny) {
      cx<T> v = tile[threadIdx.x][j];
      if (conj) v.y = -v.y;
      store_out<T>(out, out_c128, (size_t)ky * nx + kx, v);
    }
  }
}

// fft::transform2 (reference propagation/fft.rs:40-108) on the device: row
// transforms (pass A with P = n), forward-only column transforms (pass B,
// scaled by a.scale), then the transpose to row-major.  `a` carries the
// full-support axis plans, twiddles, engine ENG_IDENTITY and the input;
// `spec` is an nx * ny scratch of the engine's type.
template <typename T>
cudaError_t launch_fft2(const PropArgs& a, void* spec, void* out, int out_c128, int conj,
                        cudaStream_t st) {
  cudaError_t e = launch_passA<T>(a, st);
  if (e != cudaSuccess) return e;
  e = launch_passB_impl<T>(a, 1, spec, st);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_fft2_finish<T><<<dim3((a.nx + 31) / 32, (a.ny + 31) / 32), dim3(32, 8), 0, st>>>(
      reinterpret_cast<const cx<T>*>(spec), a.nx, a.ny, out, out_c128, conj);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_conj_copy(const void* src, int c128, void* dst, size_t n, cudaStream_t st) {
  COUNT_LAUNCH();
  k_conj_copy<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, c128,
                                                                reinterpret_cast<cx<T>*>(dst), n);
  return cudaGetLastError();
}

template cudaError_t launch_fft2<float>(const PropArgs&, void*, void*, int, int, cudaStream_t);
template cudaError_t launch_fft2<double>(const PropArgs&, void*, void*, int, int, cudaStream_t);
template cudaError_t launch_conj_copy<float>(const void*, int, void*, size_t, cudaStream_t);
template cudaError_t launch_conj_copy<double>(const void*, int, void*, size_t, cudaStream_t);

// ------------------------------------------------------------ Fraunhofer

// Pass FA: offset-DFT pre-phase and off-axis ramp (reference
// fraunhofer.rs:396-412), then forward row FFTs into column-major scratch.
// Adjoint mode: input is the far-field grid; rows carry conj(post * chirp *
// quad) dx dy (and the mirror), followed by inverse row FFTs.
template <typename T>
__device__ __forceinline__ void fraun_pre(const FraunArgs& a, int ix, int iy, double& re,
                                          double& im) {
  const double cy = a.cyc, cx = a.cxc;
  const double eta = __dmul_rn(__dsub_rn((double)iy, cy), a.dy);
  const double xi = __dmul_rn(__dsub_rn((double)ix, cx), a.dx);
  const double py = __ddiv_rn(__dmul_rn(__dmul_rn(2.0 * M_PI, cy), (double)iy), (double)a.ny);
  const double ry = __dmul_rn(__dmul_rn(2.0 * M_PI, a.g_s), eta);
  const double px = __dmul_rn(2.0 * M_PI, __dadd_rn(__ddiv_rn(__dmul_rn(cx, (double)ix), (double)a.nx),
                                                    __dmul_rn(a.f_s, xi)));
  double s1, c1, s2, c2, s3, c3;
  sincos(py, &s1, &c1);
  sincos(ry, &s2, &c2);
  sincos(px, &s3, &c3);
  // pre = pre_y * ramp_y * pre_x
  double ar = c1 * c2 - s1 * s2, ai = c1 * s2 + s1 * c2;
  double br = ar * c3 - ai * s3, bi = ar * s3 + ai * c3;
  if (a.adjoint) bi = -bi;
  const double r2 = re * br - im * bi, i2 = re * bi + im * br;
  re = r2;
  im = i2;
}

// Output factor quad * chirp * post * (dx dy) for output sample (ix, iy)
// with source bin (mx, my) (reference fraunhofer.rs:421-438).
__device__ __forceinline__ void fraun_post(const FraunArgs& a, int ix, int iy, int mx, int my,
                                           double& fr, double& fi) {
  const double cy = a.cyc, cx = a.cxc;
  const double dyp = __dsub_rn(__dmul_rn(__dsub_rn((double)iy, cy), a.dyo), a.ys);
  const double dxp = __dsub_rn(__dmul_rn(__dsub_rn((double)ix, cx), a.dxo), a.xs);
  const double py = __ddiv_rn(__dmul_rn(__dmul_rn(2.0 * M_PI, cy), __dsub_rn((double)my, cy)), (double)a.ny);
  const double px = __ddiv_rn(__dmul_rn(__dmul_rn(2.0 * M_PI, cx), __dsub_rn((double)mx, cx)), (double)a.nx);
  const double ch = __ddiv_rn(__dmul_rn(M_PI, __dadd_rn(__dmul_rn(dxp, dxp), __dmul_rn(dyp, dyp))),
                              __dmul_rn(a.lam, a.z));
  double s1, c1, s2, c2, s3, c3;
  sincos(py, &s1, &c1);
  sincos(px, &s2, &c2);
  sincos(ch, &s3, &c3);
  // quad * chirp
  double qr = a.quad_re * c3 - a.quad_im * s3, qi = a.quad_re * s3 + a.quad_im * c3;
  // * post_y * post_x
  double pr = c1 * c2 - s1 * s2, pi_ = c1 * s2 + s1 * c2;
  double tr = qr * pr - qi * pi_, ti = qr * pi_ + qi * pr;
  const double w = __dmul_rn(a.dx, a.dy);
  fr = tr * w;
  fi = ti * w;
}

// The f32 engine's per-axis tables of the pre and post factors (FP64, the
// reference's formulas, rounded once to f32):
//   tpx[ix] = e^{i px(ix)},  tpy[iy] = e^{i py(iy)} e^{i ry(iy)}          (fraun_pre)
//   tqx[mx] = quad (dx dy) e^{i pi dxp(ix)^2 / (lam z)} e^{i px'(mx)},
//   tqy[my] = e^{i pi dyp(iy)^2 / (lam z)} e^{i py'(my)}                 (fraun_post)
// with (ix, iy) the output sample of the bin (mx, my) (the mirror map for
// z < 0, its own inverse): the chirp e^{i pi (dxp^2 + dyp^2) / (lam z)}
// factors into its two axes.
__global__ void k_fraun_tables(FraunArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double cx = a.cxc, cy = a.cyc;
  const double sgn = a.z > 0.0 ? 1.0 : -1.0;
  const double lz = __dmul_rn(a.lam, a.z);
  if (i < a.nx) {
    const double xi = __dmul_rn(__dsub_rn((double)i, cx), a.dx);
    const double px = __dmul_rn(2.0 * M_PI, __dadd_rn(__ddiv_rn(__dmul_rn(cx, (double)i), (double)a.nx),
                                                      __dmul_rn(a.f_s, xi)));
    double s, c;
    sincos(px, &s, &c);
    a.tpx[i] = make_float2((float)c, (float)s);
    const int ix = (int)rint(sgn * ((double)i - cx) + cx);  // output sample of bin mx = i
    const double dxp = __dsub_rn(__dmul_rn(__dsub_rn((double)ix, cx), a.dxo), a.xs);
    const double ch = __ddiv_rn(__dmul_rn(M_PI, __dmul_rn(dxp, dxp)), lz);
    const double pp = __ddiv_rn(__dmul_rn(__dmul_rn(2.0 * M_PI, cx), __dsub_rn((double)i, cx)), (double)a.nx);
    double s1, c1, s2, c2;
    sincos(ch, &s1, &c1);
    sincos(pp, &s2, &c2);
    const double qr = a.quad_re * c1 - a.quad_im * s1, qi = a.quad_re * s1 + a.quad_im * c1;
    const double w = __dmul_rn(a.dx, a.dy);
    a.tqx[i] = make_float2((float)((qr * c2 - qi * s2) * w), (float)((qr * s2 + qi * c2) * w));
  }
  if (i < a.ny) {
    const double eta = __dmul_rn(__dsub_rn((double)i, cy), a.dy);
    const double py = __ddiv_rn(__dmul_rn(__dmul_rn(2.0 * M_PI, cy), (double)i), (double)a.ny);
    const double ry = __dmul_rn(__dmul_rn(2.0 * M_PI, a.g_s), eta);
    double s1, c1, s2, c2;
    sincos(py, &s1, &c1);
    sincos(ry, &s2, &c2);
    a.tpy[i] = make_float2((float)(c1 * c2 - s1 * s2), (float)(c1 * s2 + s1 * c2));
    const int iy = (int)rint(sgn * ((double)i - cy) + cy);
    const double dyp = __dsub_rn(__dmul_rn(__dsub_rn((double)iy, cy), a.dyo), a.ys);
    const double ch = __ddiv_rn(__dmul_rn(M_PI, __dmul_rn(dyp, dyp)), lz);
    const double pp = __ddiv_rn(__dmul_rn(__dmul_rn(2.0 * M_PI, cy), __dsub_rn((double)i, cy)), (double)a.ny);
    double s3, c3, s4, c4;
    sincos(ch, &s3, &c3);
    sincos(pp, &s4, &c4);
    a.tqy[i] = make_float2((float)(c3 * c4 - s3 * s4), (float)(c3 * s4 + s3 * c4));
  }
}

__device__ __forceinline__ float2 fcmul(float2 p, float2 q) {
  return make_float2(p.x * q.x - p.y * q.y, p.x * q.y + p.y * q.x);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_fraunA(FraunArgs a, int rows) {
  using V = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = a.ax.m, nx = a.nx, ny = a.ny;
  const int ld = m + 1;
  V* bufA = reinterpret_cast<V*>(smem_raw);
  V* bufB = bufA + (size_t)rows * ld;
  const int row0 = blockIdx.x * rows;
  const V* twm = reinterpret_cast<const V*>(a.tw_mx);
  V* W = reinterpret_cast<V*>(a.work);
  const double sgn = a.z > 0.0 ? 1.0 : -1.0;
  for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
    const int i = e / m, j = e - i * m, iy = row0 + i;
    double re = 0.0, im = 0.0;
    int pos = j;
    if (iy < ny) {
      V v = load_in<T>(a.in, a.in_c128, (size_t)iy * nx + j);
      re = (double)v.x;
      im = (double)v.y;
      if (a.status && nonfinite2(re, im)) atomicOr(a.status, 1);
      if (!a.adjoint) {
        if (a.els.count) apply_elements_exact(a.els, j, iy, nx, ny, a.dx, a.dy, re, im);
        if constexpr (sizeof(T) == 4) {
          const float2 f = fcmul(a.tpy[iy], a.tpx[j]);
          const float xr = (float)re, xi = (float)im;
          re = xr * f.x - xi * f.y;
          im = xr * f.y + xi * f.x;
        } else {
          fraun_pre<T>(a, j, iy, re, im);
        }
      } else {
        // adjoint: far-field sample (ix = j, iy) came from DFT bin (mx, my);
        // multiply conj(factor) and place it at its bin index mx.
        const int mx = (int)rint(sgn * ((double)j - a.cxc) + a.cxc);
        const int my = (int)rint(sgn * ((double)iy - a.cyc) + a.cyc);
        double fr, fi;
        if constexpr (sizeof(T) == 4) {
          const float2 f = fcmul(a.tqx[mx], a.tqy[my]);
          fr = f.x;
          fi = f.y;
        } else {
          fraun_post(a, j, iy, mx, my, fr, fi);
        }
        const double r2 = re * fr + im * fi, i2 = im * fr - re * fi;  // * conj(f)
        re = r2;
        im = i2;
        pos = mx;
      }
    }
    bufA[(size_t)i * ld + pos] = mkc<V>((T)re, (T)im);
  }
  __syncthreads();
  V* res = a.adjoint ? stockham<T, true>(bufA, bufB, m, rows, ld, a.ax, twm)
                     : stockham<T, false>(bufA, bufB, m, rows, ld, a.ax, twm);
  // adjoint: the DFT index of this row is the source bin mx(ix); scatter so
  // that W[mx][my] holds the row.  Forward: identity placement.
  for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
    const int i = e % rows, q = e / rows, iy = row0 + i;
    if (iy >= ny) continue;
    int dst_row = iy;
    if (a.adjoint) dst_row = (int)rint(sgn * ((double)iy - a.cyc) + a.cyc);
    W[(size_t)q * ny + dst_row] = res[(size_t)i * ld + q];
  }
}

// Pass FB: forward column FFT over y, then the output factor and mirror
// (forward), or inverse column FFT and conj(pre) (adjoint).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_fraunB(FraunArgs a) {
  using V = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int my = a.ay.m, ny = a.ny, nx = a.nx;
  const int kx = blockIdx.x;
  V* buf0 = reinterpret_cast<V*>(smem_raw);
  V* buf1 = buf0 + my;
  const V* twm = reinterpret_cast<const V*>(a.tw_my);
  const V* W = reinterpret_cast<const V*>(a.work) + (size_t)kx * ny;
  for (int j = threadIdx.x; j < my; j += blockDim.x) buf0[j] = W[j];
  __syncthreads();
  V* res = a.adjoint ? stockham<T, true>(buf0, buf1, my, 1, my, a.ay, twm)
                     : stockham<T, false>(buf0, buf1, my, 1, my, a.ay, twm);
  const double sgn = a.z > 0.0 ? 1.0 : -1.0;
  for (int p = threadIdx.x; p < my; p += blockDim.x) {
    V v = res[p];
    double re = (double)v.x, im = (double)v.y;
    int ox, oy;
    if (!a.adjoint) {
      // bin (mx = kx, my = p) lands on output (ix, iy) with mx = sgn (ix - c) + c
      const int ix = (int)rint(sgn * ((double)kx - a.cxc) + a.cxc);
      const int iy = (int)rint(sgn * ((double)p - a.cyc) + a.cyc);
      double fr, fi;
      if constexpr (sizeof(T) == 4) {
        const float2 f = fcmul(a.tqx[kx], a.tqy[p]);
        fr = f.x;
        fi = f.y;
      } else {
        fraun_post(a, ix, iy, kx, p, fr, fi);
      }
      const double r2 = fr * re - fi * im, i2 = fr * im + fi * re;
      re = r2;
      im = i2;
      ox = ix;
      oy = iy;
    } else {
      // spatial sample (ix = kx, iy = p): multiply conj(pre)
      if constexpr (sizeof(T) == 4) {
        const float2 f = fcmul(a.tpy[p], a.tpx[kx]);
        const float xr = (float)re, xi = (float)im;
        re = xr * f.x + xi * f.y;
        im = xi * f.x - xr * f.y;
      } else {
        fraun_pre<T>(a, kx, p, re, im);
      }
      ox = kx;
      oy = p;
    }
    const size_t o = (size_t)oy * nx + ox;
    const V w = mkc<V>((T)re, (T)im);
    if (a.status && nonfinite2(re, im)) atomicOr(a.status, 2);
    if (a.out) store_out<T>(a.out, a.out_c128, o, w);
    if (a.out_intensity) a.out_intensity[o] = (float)(re * re + im * im);
  }
}

template <typename T>
cudaError_t launch_fraunhofer(const FraunArgs& a, cudaStream_t st) {
  const int is_d = sizeof(T) == 8;
  const size_t es = is_d ? 16 : 8;
  if (!is_d) {
    if (!a.tpx || !a.tpy || !a.tqx || !a.tqy) return cudaErrorInvalidValue;
    const int nt = std::max(a.nx, a.ny);
    COUNT_LAUNCH();
    k_fraun_tables<<<(nt + 127) / 128, 128, 0, st>>>(a);
    cudaError_t e0 = cudaGetLastError();
    if (e0 != cudaSuccess) return e0;
  }
  int rows = 16;
  while (rows > 1 && 2 * ((size_t)a.ax.m + 1) * rows * es > kSmemBudgetRows) rows /= 2;
  size_t smem = 2 * ((size_t)a.ax.m + 1) * rows * es;
  cudaError_t e = cudaFuncSetAttribute(k_fraunA<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_fraunA<T><<<(a.ny + rows - 1) / rows, kThreads, smem, st>>>(a, rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  smem = 2 * (size_t)a.ay.m * es;
  e = cudaFuncSetAttribute(k_fraunB<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  COUNT_LAUNCH();
  k_fraunB<T><<<a.nx, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------ element kernel

template <typename T>
__global__ void k_apply_elements(const void* in, int in_c128, void* out, int out_c128,
                                 ElementList els, int nx, int ny, double dx, double dy,
                                 int* status) {
  const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (idx >= (size_t)nx * ny) return;
  const int ix = (int)(idx % nx), iy = (int)(idx / nx);
  cx<T> v = load_in<T>(in, in_c128, idx);
  v = apply_elements<T>(els, ix, iy, nx, ny, dx, dy, v);
  if (status && nonfinite2((double)v.x, (double)v.y)) atomicOr(status, 2);
  store_out<T>(out, out_c128, idx, v);
}

template <typename T>
cudaError_t launch_apply_elements(const void* in, int in_c128, void* out, int out_c128,
                                  const ElementList& els, int nx, int ny, double dx, double dy,
                                  int* status, cudaStream_t st) {
  const size_t n = (size_t)nx * ny;
  COUNT_LAUNCH();
  k_apply_elements<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, in_c128, out, out_c128,
                                                                    els, nx, ny, dx, dy, status);
  return cudaGetLastError();
}

// -------------------------------------------------------- instantiations

template cudaError_t launch_apply_elements<float>(const void*, int, void*, int, const ElementList&,
                                                  int, int, double, double, int*, cudaStream_t);
template cudaError_t launch_apply_elements<double>(const void*, int, void*, int, const ElementList&,
                                                   int, int, double, double, int*, cudaStream_t);

template cudaError_t launch_asm_prep<float>(const PropArgs&, void*, cudaStream_t);
template cudaError_t launch_asm_prep<double>(const PropArgs&, void*, cudaStream_t);
template cudaError_t launch_passA<float>(const PropArgs&, cudaStream_t);
template cudaError_t launch_passA<double>(const PropArgs&, cudaStream_t);
template cudaError_t launch_passB<float>(const PropArgs&, cudaStream_t);
template cudaError_t launch_passB<double>(const PropArgs&, cudaStream_t);
template cudaError_t launch_passC<float>(const PropArgs&, cudaStream_t);
template cudaError_t launch_passC<double>(const PropArgs&, cudaStream_t);
template cudaError_t launch_fraunhofer<float>(const FraunArgs&, cudaStream_t);
template cudaError_t launch_fraunhofer<double>(const FraunArgs&, cudaStream_t);
template cudaError_t launch_fresnel_ksep<float>(const PropArgs&, void*, void*, void*, cudaStream_t);
template cudaError_t launch_fresnel_ksep<double>(const PropArgs&, void*, void*, void*, cudaStream_t);
template cudaError_t launch_rs_kspec<float>(const PropArgs&, void*, void*, cudaStream_t);
template cudaError_t launch_rs_kspec<double>(const PropArgs&, void*, void*, cudaStream_t);

}  // namespace osgpu
