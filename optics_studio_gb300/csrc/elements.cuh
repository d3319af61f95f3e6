// Element transmissions evaluated on the device (shared by the generic
// and the register-FFT passes).
#pragma once
#include <cuda_runtime.h>
#include "osgpu_types.h"

namespace osgpu {

// fftfreq value k/(n d) with negative wrap (reference propagation/fft.rs:115-126).
static __device__ __forceinline__ double fftfreq_d(int k, int n, double d) {
  double kk = (k <= (n - 1) / 2) ? (double)k : (double)k - (double)n;
  return __ddiv_rn(kk, __dmul_rn((double)n, d));
}

// Origin-centred coordinate (i - (n-1)/2) d (reference field.rs:216-221).
static __device__ __forceinline__ double coord_d(int i, int n, double d) {
  return __dmul_rn(__dsub_rn((double)i, ((double)n - 1.0) / 2.0), d);
}

// Element-frame rotation (reference element.rs:557-560), no FMA contraction.
static __device__ __forceinline__ void to_frame(double x, double y, double c, double s, double& fx,
                                         double& fy) {
  fx = __dadd_rn(__dmul_rn(c, x), __dmul_rn(s, y));
  fy = __dadd_rn(__dmul_rn(-s, x), __dmul_rn(c, y));
}

// ClearAperture::contains (reference element.rs:476-488).
static __device__ __forceinline__ bool stop_contains(int kind, double a, double b, double x, double y) {
  switch (kind) {
    case STOP_CIRCLE:
      return __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)) <= __dmul_rn(a, a);
    case STOP_ELLIPSE: {
      double a2 = __dmul_rn(a, a), b2 = __dmul_rn(b, b);
      return __dadd_rn(__dmul_rn(__dmul_rn(b2, x), x), __dmul_rn(__dmul_rn(a2, y), y)) <=
             __dmul_rn(a2, b2);
    }
    case STOP_RECT:
      return fabs(x) <= a && fabs(y) <= b;
    default:
      return true;
  }
}

// SampledPhase::at, bilinear, zero outside the span (reference element.rs:1189-1207).
static __device__ double lattice_at(const DevElement& e, double x, double y) {
  double gx = __dadd_rn(__ddiv_rn(x, e.ldx), ((double)e.lnx - 1.0) / 2.0);
  double gy = __dadd_rn(__ddiv_rn(y, e.ldy), ((double)e.lny - 1.0) / 2.0);
  double lx = (double)e.lnx - 1.0, ly = (double)e.lny - 1.0;
  if (gx < 0.0 || gx > lx || gy < 0.0 || gy > ly) return 0.0;
  int i0 = (int)floor(gx), j0 = (int)floor(gy);
  int i1 = min(i0 + 1, e.lnx - 1), j1 = min(j0 + 1, e.lny - 1);
  double tx = __dsub_rn(gx, (double)i0), ty = __dsub_rn(gy, (double)j0);
  const double* v = e.lat;
  double v00 = v[(size_t)j0 * e.lnx + i0], v10 = v[(size_t)j0 * e.lnx + i1];
  double v01 = v[(size_t)j1 * e.lnx + i0], v11 = v[(size_t)j1 * e.lnx + i1];
  double A = __dadd_rn(v00, __dmul_rn(__dsub_rn(v10, v00), tx));
  double B = __dadd_rn(v01, __dmul_rn(__dsub_rn(v11, v01), tx));
  return __dadd_rn(A, __dmul_rn(__dsub_rn(B, A), ty));
}

static __device__ __forceinline__ void cmul_phase(double& re, double& im, double phi) {
  double s, c;
  sincos(phi, &s, &c);
  double r2 = re * c - im * s;
  double i2 = re * s + im * c;
  re = r2;
  im = i2;
}

// FP64 evaluation of one element at the origin-centred coordinate (x, y),
// in the reference's operation order (element.rs:754-790, 900-929,
// 1115-1154, 1443-1484, 1668-1703): (re, im) <- t(x, y) (re, im).
static __device__ __forceinline__ void apply_one_exact(const DevElement& e, int ix, int iy,
                                                       double x, double y, double& re,
                                                       double& im) {
  const double xr = __dsub_rn(x, e.cx), yr = __dsub_rn(y, e.cy);
  double fx, fy;
  to_frame(xr, yr, e.cpsi, e.spsi, fx, fy);
  switch (e.kind) {
    case EL_ELLIPSE: {
      double a2 = __dmul_rn(e.a, e.a), b2 = __dmul_rn(e.b, e.b);
      double lhs = __dadd_rn(__dmul_rn(__dmul_rn(b2, fx), fx), __dmul_rn(__dmul_rn(a2, fy), fy));
      if (lhs > __dmul_rn(a2, b2)) { re = 0.0; im = 0.0; }
      break;
    }
    case EL_RECT:
      if (fabs(fx) > e.a || fabs(fy) > e.b) { re = 0.0; im = 0.0; }
      break;
    case EL_LENS: {
      if (!stop_contains(e.stop, e.a, e.b, fx, fy)) { re = 0.0; im = 0.0; break; }
      double r2 = __dadd_rn(__dmul_rn(xr, xr), __dmul_rn(yr, yr));
      double phase = __ddiv_rn(__dmul_rn(-e.k, r2), __dmul_rn(2.0, e.f));
      cmul_phase(re, im, phase);
      break;
    }
    case EL_PHASE: {
      if (!stop_contains(e.stop, e.a, e.b, fx, fy)) { re = 0.0; im = 0.0; break; }
      cmul_phase(re, im, lattice_at(e, fx, fy));
      break;
    }
    case EL_SCREEN: {  // exp(i (depth * v)), the reference's (k * dn * z) order
      if (!stop_contains(e.stop, e.a, e.b, fx, fy)) { re = 0.0; im = 0.0; break; }
      cmul_phase(re, im, __dmul_rn(e.depth, e.lat[(size_t)iy * e.lnx + ix]));
      break;
    }
    case EL_GRATING: {
      if (!stop_contains(e.stop, e.a, e.b, fx, fy)) { re = 0.0; im = 0.0; break; }
      double u = __dmul_rn(fx, e.inv_period);
      double phi = __dmul_rn(e.depth, __dsub_rn(u, floor(u)));
      cmul_phase(re, im, phi);
      break;
    }
    default:
      break;
  }
}

// Per-sample FP64 evaluation of every element of L at sample (ix, iy), in
// list order.
static __device__ void apply_elements_exact(const ElementList& L, int ix, int iy, int nx, int ny,
                                     double dx, double dy, double& re, double& im) {
  const double x = coord_d(ix, nx, dx);
  const double y = coord_d(iy, ny, dy);
  for (int q = 0; q < L.count; ++q) apply_one_exact(L.el[q], ix, iy, x, y, re, im);
}

// f32 fast path for one element (psi == 0, tables built in FP64 by
// k_element_tables): table lookups plus one sincosf for a phase lattice.
// The decisions (stops, lattice span) are the reference's exact FP64
// decisions, precomputed per row / column.  Returns false when the sample
// is outside the element's transmitting set (the result is then zero).
static __device__ __forceinline__ bool apply_one_fast(const DevElement& e, int ix, int iy,
                                                      float2& v) {
  // the tables are read-only for the kernel's lifetime: non-coherent loads
  if (e.span) {
    const int2 sp = __ldg(e.span + iy);
    if (ix < sp.x || ix > sp.y) {
      v = make_float2(0.f, 0.f);
      return false;
    }
  }
  switch (e.kind) {
    case EL_LENS: {
      const float2 a = __ldg(e.tabx + ix), b = __ldg(e.taby + iy);
      const float2 t = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
      v = make_float2(v.x * t.x - v.y * t.y, v.x * t.y + v.y * t.x);
      break;
    }
    case EL_GRATING: {
      const float2 t = __ldg(e.tabx + ix);
      v = make_float2(v.x * t.x - v.y * t.y, v.x * t.y + v.y * t.x);
      break;
    }
    case EL_PHASE: {
      const int4 bx = __ldg(e.bilx + ix), by = __ldg(e.bily + iy);
      float phi = 0.f;
      if (bx.w && by.w) {
        const float tx = __int_as_float(bx.z), ty = __int_as_float(by.z);
        const float* r0 = e.latf + (size_t)by.x * e.lnx;
        const float v00 = __ldg(r0 + bx.x);
        if (bx.z == 0 && by.z == 0) {
          phi = v00;  // sample on a lattice node: the bilinear form reduces to v00
        } else {
          const float* r1 = e.latf + (size_t)by.y * e.lnx;
          const float v10 = __ldg(r0 + bx.y), v01 = __ldg(r1 + bx.x), v11 = __ldg(r1 + bx.y);
          const float A = v00 + (v10 - v00) * tx;
          const float B = v01 + (v11 - v01) * tx;
          phi = A + (B - A) * ty;
        }
      }
      // reduce by 2 pi (two-part Cody-Waite constant) into [-pi, pi], then the
      // hardware sine / cosine, accurate to ~5e-7 absolute on that range
      const float nq = rintf(phi * 0.159154943091895336f);
      float rr = fmaf(-nq, 6.28125f, phi);
      rr = fmaf(-nq, 1.93530717958647692e-3f, rr);
      float sn, cs;
      __sincosf(rr, &sn, &cs);
      v = make_float2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
      break;
    }
    case EL_SCREEN: {  // transmission table built with the phase in FP64
      const float2 t = __ldg(e.scr + (size_t)iy * e.lnx + ix);
      v = make_float2(v.x * t.x - v.y * t.y, v.x * t.y + v.y * t.x);
      break;
    }
    default:
      break;
  }
  return true;
}

static __device__ __forceinline__ float2 apply_elements_fast(const ElementList& L, int ix, int iy,
                                                             float2 v) {
  for (int q = 0; q < L.count; ++q)
    if (!apply_one_fast(L.el[q], ix, iy, v)) return make_float2(0.f, 0.f);
  return v;
}

// The same transmissions for K samples of one thread at (ix[k], iy[k]),
// element by element, so that the table and lattice loads of all K samples
// are in flight together (the per-sample form above chains them sample after
// sample).  Samples whose bit in `live` is clear are left untouched and read
// no table (zero padding); a sample outside an element's transmitting set
// becomes zero, as in apply_one_fast.  K <= 32.
template <int K>
static __device__ __forceinline__ void apply_elements_fast_k(const ElementList& L,
                                                             const int (&ix)[K],
                                                             const int (&iy)[K], unsigned live,
                                                             float2 (&v)[K]) {
  const unsigned inb = live;
  for (int q = 0; q < L.count; ++q) {
    const DevElement& e = L.el[q];
    unsigned pass = inb;
    if (e.span) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int2 sp = (inb >> k & 1u) ? __ldg(e.span + iy[k]) : make_int2(0, -1);
        if (ix[k] < sp.x || ix[k] > sp.y) pass &= ~(1u << k);
      }
    }
    switch (e.kind) {
      case EL_LENS:
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (!(inb >> k & 1u)) continue;
          const float2 a = __ldg(e.tabx + ix[k]), b = __ldg(e.taby + iy[k]);
          const float2 t = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
          v[k] = make_float2(v[k].x * t.x - v[k].y * t.y, v[k].x * t.y + v[k].y * t.x);
        }
        break;
      case EL_GRATING:
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (!(inb >> k & 1u)) continue;
          const float2 t = __ldg(e.tabx + ix[k]);
          v[k] = make_float2(v[k].x * t.x - v[k].y * t.y, v[k].x * t.y + v[k].y * t.x);
        }
        break;
      case EL_PHASE: {
        float phi[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
          phi[k] = 0.f;
          if (!(inb >> k & 1u)) continue;
          const int4 bx = __ldg(e.bilx + ix[k]), by = __ldg(e.bily + iy[k]);
          if (!(bx.w && by.w)) continue;
          const float* r0 = e.latf + (size_t)by.x * e.lnx;
          const float v00 = __ldg(r0 + bx.x);
          if (bx.z == 0 && by.z == 0) {
            phi[k] = v00;
          } else {
            const float tx = __int_as_float(bx.z), ty = __int_as_float(by.z);
            const float* r1 = e.latf + (size_t)by.y * e.lnx;
            const float v10 = __ldg(r0 + bx.y), v01 = __ldg(r1 + bx.x), v11 = __ldg(r1 + bx.y);
            const float A = v00 + (v10 - v00) * tx;
            const float B = v01 + (v11 - v01) * tx;
            phi[k] = A + (B - A) * ty;
          }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (!(inb >> k & 1u)) continue;
          const float nq = rintf(phi[k] * 0.159154943091895336f);
          float rr = fmaf(-nq, 6.28125f, phi[k]);
          rr = fmaf(-nq, 1.93530717958647692e-3f, rr);
          float sn, cs;
          __sincosf(rr, &sn, &cs);
          v[k] = make_float2(v[k].x * cs - v[k].y * sn, v[k].x * sn + v[k].y * cs);
        }
        break;
      }
      case EL_SCREEN:
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if (!(inb >> k & 1u)) continue;
          const float2 t = __ldg(e.scr + (size_t)iy[k] * e.lnx + ix[k]);
          v[k] = make_float2(v[k].x * t.x - v[k].y * t.y, v[k].x * t.y + v[k].y * t.x);
        }
        break;
      default:
        break;
    }
    live &= pass;
  }
#pragma unroll
  for (int k = 0; k < K; ++k)
    if ((inb >> k & 1u) && !(live >> k & 1u)) v[k] = make_float2(0.f, 0.f);
}

// Adjoint element plane at sample (ix, iy) (reference adjoint.rs:205-227,
// element by element in reverse): the chain L acted on the forward field
// u (the field entering the plane); mu is the adjoint field arriving from
// the detector side.  For the last element first: grad[q] += -2 Im(conj(mu)
// v_q) with v_q the forward field right after element q, then mu <-
// conj(t_q) mu with t_q = element q applied to 1.  grad[q] is a double* for
// the FP64 engine and a float* for the f32 engine (arithmetic in T); null
// entries are skipped.  Elements are evaluated in FP64 (exact) unless the
// list carries f32 tables (`fast`).
template <typename T>
static __device__ __forceinline__ void adjoint_plane(const ElementList& L, void* const* grad,
                                                     int ix, int iy, int nx, int ny, double dx,
                                                     double dy, size_t o, T ur, T ui, T& mr,
                                                     T& mi) {
  T vr[kMaxElements], vi[kMaxElements], tr[kMaxElements], ti[kMaxElements];
  if (sizeof(T) == 4 && L.fast) {
    float2 w = make_float2((float)ur, (float)ui);
#pragma unroll
    for (int q = 0; q < kMaxElements; ++q) {
      if (q < L.count) {
        float2 t = make_float2(1.f, 0.f);
        apply_one_fast(L.el[q], ix, iy, t);
        apply_one_fast(L.el[q], ix, iy, w);
        tr[q] = (T)t.x; ti[q] = (T)t.y;
        vr[q] = (T)w.x; vi[q] = (T)w.y;
      }
    }
  } else {
    const double x = coord_d(ix, nx, dx), y = coord_d(iy, ny, dy);
    double wr = (double)ur, wi = (double)ui;
#pragma unroll
    for (int q = 0; q < kMaxElements; ++q) {
      if (q < L.count) {
        double a = 1.0, b = 0.0;
        apply_one_exact(L.el[q], ix, iy, x, y, a, b);
        apply_one_exact(L.el[q], ix, iy, x, y, wr, wi);
        tr[q] = (T)a; ti[q] = (T)b;
        vr[q] = (T)wr; vi[q] = (T)wi;
      }
    }
  }
#pragma unroll
  for (int q = kMaxElements - 1; q >= 0; --q) {
    if (q < L.count) {
      if (grad[q]) {
        // Im(conj(mu) v) = mu.re v.im + (-mu.im) v.re
        const T im = mr * vi[q] + (-mi) * vr[q];
        reinterpret_cast<T*>(grad[q])[o] += (T)-2 * im;
      }
      // mu * conj(t)
      const T nr = mr * tr[q] - mi * (-ti[q]);
      const T ni = mr * (-ti[q]) + mi * tr[q];
      mr = nr;
      mi = ni;
    }
  }
}

}  // namespace osgpu
