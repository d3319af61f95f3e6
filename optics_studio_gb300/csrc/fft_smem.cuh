// Shared-memory mixed-radix Stockham FFT for sm_103a.
//
// A CTA transforms `rows` rows of length m held in shared memory (row
// stride `ld` complex elements), ping-ponging between two buffers, one
// __syncthreads per stage.  Stage s with radix R and accumulated span Ns:
//   for every butterfly j in [0, m/R):
//     k = j mod Ns
//     v[q] = src[j + q*m/R] * W_{Ns R}^{q k}      (q = 0..R-1)
//     v    = DFT_R(v)
//     dst[(j - k) R + k + q Ns] = v[q]
// which leaves the result in natural order (self-sorting Stockham form).
// W_N = e^{-2 pi i / N} forward, its conjugate for the inverse; the
// twiddle W_{Ns R}^{q k} is read from one table tw[t] = W_m^t at
// t = q k m/(Ns R).  Radices 2, 3, 4, 5, 8 run in registers; any other
// prime factor uses a direct O(R^2) butterfly.
#pragma once
#include <cuda_runtime.h>
#include "osgpu_types.h"

namespace osgpu {

template <typename T> struct CxT;
template <> struct CxT<float> { using type = float2; };
template <> struct CxT<double> { using type = double2; };
template <typename T> using cx = typename CxT<T>::type;

template <typename V> __device__ __forceinline__ V mkc(decltype(V::x) a, decltype(V::x) b) {
  V r; r.x = a; r.y = b; return r;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return mkc<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return mkc<V>(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  return mkc<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename V> __device__ __forceinline__ V cmulc(V a, V b) {  // a * conj(b)
  return mkc<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename V> __device__ __forceinline__ V cscale(V a, decltype(V::x) s) { return mkc<V>(a.x * s, a.y * s); }
template <typename V> __device__ __forceinline__ V cconj(V a) { return mkc<V>(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <typename V, bool INV> __device__ __forceinline__ V rot90(V a) {
  return INV ? mkc<V>(-a.y, a.x) : mkc<V>(a.y, -a.x);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft2(cx<T>* v) {
  cx<T> a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4(cx<T>* v) {
  cx<T> a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
  cx<T> a2 = cadd(v[1], v[3]), a3 = rot90<cx<T>, INV>(csub(v[1], v[3]));
  v[0] = cadd(a0, a2);
  v[2] = csub(a0, a2);
  v[1] = cadd(a1, a3);
  v[3] = csub(a1, a3);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(cx<T>* v) {
  using V = cx<T>;
  const T h = (T)0.70710678118654752440;
  V e[4] = {v[0], v[2], v[4], v[6]};
  V o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T, INV>(e);
  dft4<T, INV>(o);
  // o1 *= W8, o2 *= W8^2, o3 *= W8^3 (W8 = e^{-i pi/4} forward)
  V o1 = o[1], o3 = o[3];
  if (!INV) {
    o[1] = mkc<V>(h * (o1.x + o1.y), h * (o1.y - o1.x));
    o[3] = mkc<V>(h * (o3.y - o3.x), -h * (o3.x + o3.y));
  } else {
    o[1] = mkc<V>(h * (o1.x - o1.y), h * (o1.x + o1.y));
    o[3] = mkc<V>(-h * (o3.x + o3.y), h * (o3.x - o3.y));
  }
  o[2] = rot90<V, INV>(o[2]);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = cadd(e[q], o[q]);
    v[q + 4] = csub(e[q], o[q]);
  }
}

template <typename T, bool INV>
__device__ __forceinline__ void dft3(cx<T>* v) {
  using V = cx<T>;
  const T s = (T)0.86602540378443864676;
  V t = cadd(v[1], v[2]);
  V u = csub(v[1], v[2]);
  V y0 = cadd(v[0], t);
  V m = mkc<V>(v[0].x - (T)0.5 * t.x, v[0].y - (T)0.5 * t.y);
  // forward: y1 = m - i s u, y2 = m + i s u
  V isu = mkc<V>(-s * u.y, s * u.x);  // i s u
  v[0] = y0;
  if (!INV) { v[1] = csub(m, isu); v[2] = cadd(m, isu); }
  else      { v[1] = cadd(m, isu); v[2] = csub(m, isu); }
}

template <typename T, bool INV>
__device__ __forceinline__ void dft5(cx<T>* v) {
  using V = cx<T>;
  const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
  const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
  V t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  V u1 = csub(v[1], v[4]), u2 = csub(v[2], v[3]);
  V y0 = cadd(v[0], cadd(t1, t2));
  V m1 = mkc<V>(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  V m2 = mkc<V>(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  // p1 = s1 u1 + s2 u2, p2 = s2 u1 - s1 u2; forward y1 = m1 - i p1, y4 = m1 + i p1,
  // y2 = m2 - i p2, y3 = m2 + i p2
  V p1 = mkc<V>(s1 * u1.x + s2 * u2.x, s1 * u1.y + s2 * u2.y);
  V p2 = mkc<V>(s2 * u1.x - s1 * u2.x, s2 * u1.y - s1 * u2.y);
  V ip1 = mkc<V>(-p1.y, p1.x), ip2 = mkc<V>(-p2.y, p2.x);
  v[0] = y0;
  if (!INV) { v[1] = csub(m1, ip1); v[4] = cadd(m1, ip1); v[2] = csub(m2, ip2); v[3] = cadd(m2, ip2); }
  else      { v[1] = cadd(m1, ip1); v[4] = csub(m1, ip1); v[2] = cadd(m2, ip2); v[3] = csub(m2, ip2); }
}

template <typename T, bool INV>
__device__ __forceinline__ cx<T> twid(const cx<T>* __restrict__ tw, int t) {
  cx<T> w = tw[t];
  if (INV) w.y = -w.y;
  return w;
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void bfly_reg(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst, int j,
                                         int nb, int k, int Ns, int tstride,
                                         const cx<T>* __restrict__ tw) {
  cx<T> v[R];
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = src[j + q * nb];
  if (Ns > 1) {
#pragma unroll
    for (int q = 1; q < R; ++q) v[q] = cmul(v[q], twid<T, INV>(tw, q * k * tstride));
  }
  if (R == 2) dft2<T, INV>(v);
  if (R == 3) dft3<T, INV>(v);
  if (R == 4) dft4<T, INV>(v);
  if (R == 5) dft5<T, INV>(v);
  if (R == 8) dft8<T, INV>(v);
  const int base = (j - k) * R + k;
#pragma unroll
  for (int q = 0; q < R; ++q) dst[base + q * Ns] = v[q];
}

// Direct butterfly for an arbitrary prime factor R (O(R^2), no register array).
template <typename T, bool INV>
__device__ void bfly_generic(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst, int j, int nb,
                             int k, int Ns, int tstride, int R, int m,
                             const cx<T>* __restrict__ tw) {
  const int base = (j - k) * R + k;
  const int wstep = m / R;  // tw[e * m/R] = W_R^e
  for (int p = 0; p < R; ++p) {
    cx<T> acc = mkc<cx<T>>((T)0, (T)0);
    for (int q = 0; q < R; ++q) {
      cx<T> x = src[j + q * nb];
      if (Ns > 1 && q > 0) x = cmul(x, twid<T, INV>(tw, q * k * tstride));
      int e = (q * p) % R;
      acc = cadd(acc, cmul(x, twid<T, INV>(tw, e * wstep)));
    }
    dst[base + p * Ns] = acc;
  }
}

// Transforms `rows` rows (stride ld) from buffer a, using b as the partner
// buffer.  Returns the buffer holding the result.  All threads of the CTA
// must call it; it ends with a __syncthreads.
template <typename T, bool INV>
__device__ cx<T>* stockham(cx<T>* a, cx<T>* b, int m, int rows, int ld, const AxisPlan& ax,
                           const cx<T>* __restrict__ tw) {
  int Ns = 1;
  for (int s = 0; s < ax.nst; ++s) {
    const int R = ax.radix[s];
    const int nb = m / R;
    const int total = nb * rows;
    const int tstride = m / (Ns * R);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int row = t / nb;
      const int j = t - row * nb;
      const int k = j % Ns;
      const cx<T>* src = a + (size_t)row * ld;
      cx<T>* dst = b + (size_t)row * ld;
      switch (R) {
        case 2: bfly_reg<T, INV, 2>(src, dst, j, nb, k, Ns, tstride, tw); break;
        case 3: bfly_reg<T, INV, 3>(src, dst, j, nb, k, Ns, tstride, tw); break;
        case 4: bfly_reg<T, INV, 4>(src, dst, j, nb, k, Ns, tstride, tw); break;
        case 5: bfly_reg<T, INV, 5>(src, dst, j, nb, k, Ns, tstride, tw); break;
        case 8: bfly_reg<T, INV, 8>(src, dst, j, nb, k, Ns, tstride, tw); break;
        default: bfly_generic<T, INV>(src, dst, j, nb, k, Ns, tstride, R, m, tw); break;
      }
    }
    __syncthreads();
    cx<T>* tmp = a; a = b; b = tmp;
    Ns *= R;
  }
  return a;
}

}  // namespace osgpu
