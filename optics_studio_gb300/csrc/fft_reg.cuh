// Register-resident Stockham FFT for power-of-two lengths M in [256, 4096],
// f32 complex.  T = M/16 threads cooperate on one transform; every thread
// owns one radix-16 butterfly per stage and holds 16 points in registers:
//   on entry  v[q] = x[tid + T q]      on exit  v[q] = X[tid + T q]
// (same layout both ways, so a forward and an inverse transform chain
// without reshuffling).  Stages: floor(log16 M) radix-16 stages plus a final
// radix-2/4/8 stage when log2 M is not a multiple of 4.  Between stages the
// data goes through shared memory once (padded index i + i/16 to keep the
// transposed stage-0 store conflict free): 2 exchanges for M = 512..4096.
//
// Stage (Ns = product of earlier radices, radix R, butterfly j, k = j mod Ns):
//   v[q] = src[j + q M/R] * W_{Ns R}^{q k};  v = DFT_R(v);
//   dst[(j - k) R + k + q Ns] = v[q]
// Twiddles come from a stage-ordered copy of the table e^{-2 pi i t / M}
// (conjugated for the inverse), TwLay below.
#pragma once
#include <cuda_runtime.h>

namespace osgpu {
namespace regfft {

#ifndef OSGPU_NO_F32X2
// Complex add / subtract as one packed f32x2 instruction (sm_100+): each lane
// rounds like the scalar add, so results are bit-identical; it halves the
// issue slots of the butterflies' additions (OSGPU_NO_F32X2 builds the
// scalar form for comparison).
__device__ __forceinline__ unsigned long long pk2(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 upk2(unsigned long long r) {
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(r));
  return d;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
  return upk2(d);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
  return upk2(d);
}
#else
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <bool INV> __device__ __forceinline__ float2 rot(float2 a) {  // * (-i) fwd, * (+i) inv
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV> __device__ __forceinline__ float2 twiddle(float2 a, float2 w) {
  return INV ? cmulc(a, w) : cmul(a, w);
}

template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  float2 b0 = cadd(a0, a2), b1 = csub(a0, a2);
  float2 b2 = cadd(a1, a3), d = csub(a1, a3);
  a0 = cadd(b0, b2);
  a2 = csub(b0, b2);
  // b1 +- rot(d), rot(d) = -i d (fwd) or +i d (inv), componentwise
  if (INV) {
    a1 = make_float2(b1.x - d.y, b1.y + d.x);
    a3 = make_float2(b1.x + d.y, b1.y - d.x);
  } else {
    a1 = make_float2(b1.x + d.y, b1.y - d.x);
    a3 = make_float2(b1.x - d.y, b1.y + d.x);
  }
}

// multiply by W8^1 = e^{-i pi/4} (fwd) or its conjugate (inv)
template <bool INV> __device__ __forceinline__ float2 w8_1(float2 a) {
  const float h = 0.70710678118654752f;
  return INV ? make_float2(h * (a.x - a.y), h * (a.x + a.y))
             : make_float2(h * (a.x + a.y), h * (a.y - a.x));
}
// multiply by W8^3 (fwd) or conjugate (inv)
template <bool INV> __device__ __forceinline__ float2 w8_3(float2 a) {
  const float h = 0.70710678118654752f;
  return INV ? make_float2(-h * (a.x + a.y), h * (a.x - a.y))
             : make_float2(h * (a.y - a.x), -h * (a.x + a.y));
}

template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
  // v[0..7] -> DFT_8 in natural order
  dft4<INV>(v[0], v[2], v[4], v[6]);
  dft4<INV>(v[1], v[3], v[5], v[7]);
  // evens E0..E3 at v0,v2,v4,v6 ; odds O0..O3 at v1,v3,v5,v7
  float2 o1 = w8_1<INV>(v[3]);
  float2 o2 = rot<INV>(v[5]);
  float2 o3 = w8_3<INV>(v[7]);
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}

// In-place DFT_16 of v[0..15] (natural order in and out): 16 = 4 x 4,
// n = 4 n1 + n2, k = k1 + 4 k2.
template <bool INV>
__device__ __forceinline__ void dft16(float2* v) {
  const float c1 = 0.92387953251128676f, s1 = 0.38268343236508977f;
  const float h = 0.70710678118654752f;
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4<INV>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
  // slot n2 + 4 k1 holds Y[n2][k1]; twiddle W16^{n2 k1}
  // W16^1 = (c1, -s1), W16^2 = (h, -h), W16^3 = (s1, -c1), W16^4 = -i,
  // W16^6 = (-h, -h), W16^9 = (-c1, s1)... (conjugates for the inverse)
  const float sg = INV ? -1.f : 1.f;
  v[5] = cmul(v[5], make_float2(c1, -sg * s1));   // n2=1,k1=1 : W^1
  v[9] = cmul(v[9], make_float2(h, -sg * h));     // n2=1,k1=2 : W^2
  v[13] = cmul(v[13], make_float2(s1, -sg * c1)); // n2=1,k1=3 : W^3
  v[6] = cmul(v[6], make_float2(h, -sg * h));     // n2=2,k1=1 : W^2
  v[10] = rot<INV>(v[10]);                        // n2=2,k1=2 : W^4
  v[14] = cmul(v[14], make_float2(-h, -sg * h));  // n2=2,k1=3 : W^6
  v[7] = cmul(v[7], make_float2(s1, -sg * c1));   // n2=3,k1=1 : W^3
  v[11] = cmul(v[11], make_float2(-h, -sg * h));  // n2=3,k1=2 : W^6
  v[15] = cmul(v[15], make_float2(-c1, sg * s1)); // n2=3,k1=3 : W^9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  // slot k2 + 4 k1 holds X[k1 + 4 k2]: transpose the 4x4 index (register renaming)
  float2 t;
  t = v[1]; v[1] = v[4]; v[4] = t;
  t = v[2]; v[2] = v[8]; v[8] = t;
  t = v[3]; v[3] = v[12]; v[12] = t;
  t = v[6]; v[6] = v[9]; v[9] = t;
  t = v[7]; v[7] = v[13]; v[13] = t;
  t = v[11]; v[11] = v[14]; v[14] = t;
}

constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x / 2); }

// Twiddle powers w^q, q = 1..15, from w^1 and w^4 read from the table
// (products of at most three table values, so within a few f32 ulps of the
// table's own values): 2 shared-memory reads instead of 15.
__device__ __forceinline__ void tw_powers16(float2 w1, float2 w4, float2 (&w)[16]) {
  w[1] = w1;
  w[2] = cmul(w1, w1);
  w[3] = cmul(w[2], w1);
  w[4] = w4;
  w[5] = cmul(w4, w1);
  w[6] = cmul(w4, w[2]);
  w[7] = cmul(w4, w[3]);
  w[8] = cmul(w4, w4);
  w[9] = cmul(w[8], w1);
  w[10] = cmul(w[8], w[2]);
  w[11] = cmul(w[8], w[3]);
  w[12] = cmul(w[8], w4);
  w[13] = cmul(w[12], w1);
  w[14] = cmul(w[12], w[2]);
  w[15] = cmul(w[12], w[3]);
}

template <int M> struct Plan {
  static constexpr int T = M / 16;
  static constexpr int E = ilog2(M);
  static constexpr int N16 = E / 4;          // radix-16 stages
  static constexpr int RF = 1 << (E % 4);    // final radix (1: none)
  static constexpr int SMEM = M + M / 16;    // padded elements per buffer
};

// Twiddle table in stage order, laid out so that the lanes of a warp read
// consecutive entries (no shared-memory bank conflicts):
//   middle radix-16 stage st (span Ns = 16^(st+1), butterfly k = tid mod Ns):
//     entry mid_off(st) + (q-1) Ns + k = W_{16 Ns}^{q k},   q = 1..15
//   last stage (radix LR = RF, or 16 when log2 M is a multiple of 4; span LS = M/LR,
//   butterfly j < LS):
//     entry LAST + (q-1) LS + j = W_M^{q j},                q = 1..LR-1
// Every entry is a copy of one entry of the M-point table W_M^e, so the
// values are those of a plain table lookup.  SIZE <= M.
template <int M> struct TwLay {
  using P = Plan<M>;
  static constexpr int MID = (P::RF == 1) ? P::N16 - 2 : P::N16 - 1;  // middle radix-16 stages
  static constexpr int LR = (P::RF == 1) ? 16 : P::RF;
  static constexpr int LS = M / LR;
  __host__ __device__ static constexpr int span(int st) { return st < 0 ? 1 : 16 * span(st - 1); }
  __host__ __device__ static constexpr int mid_off(int st) { return st <= 0 ? 0 : mid_off(st - 1) + 15 * span(st - 1); }
  static constexpr int LAST = mid_off(MID);
  static constexpr int SIZE = LAST + (LR - 1) * LS;
};

// Fill the stage-ordered table from the M-point table twm[e] = W_M^e
// (threads t0, t0 + nt, ...).
template <int M>
__device__ __forceinline__ void load_stage_twiddles(float2* tws, const float2* __restrict__ twm,
                                                    int t0, int nt) {
  using L = TwLay<M>;
  for (int i = t0; i < L::SIZE; i += nt) {
    int e;
    if (i >= L::LAST) {
      const int r = i - L::LAST;
      const int q = r / L::LS + 1;
      e = q * (r - (q - 1) * L::LS);
    } else {
      int off = 0, ns = 16;
      while (i >= off + 15 * ns) {
        off += 15 * ns;
        ns *= 16;
      }
      const int r = i - off;
      const int q = r / ns + 1;
      e = q * (r - (q - 1) * ns) * (M / (16 * ns));
    }
    tws[i] = __ldg(twm + e);
  }
}

// Named barrier `id` (1..15; id 0 is __syncthreads) over `nthreads`
// threads, which must be whole warps: callers whose groups are narrower than
// a warp pass one shared id and the CTA's thread count.
__device__ __forceinline__ void group_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// One transform of length M by the T = M/16 threads with local index tid.
// TWREC: the middle stage's twiddles w^q from w^1 and w^4 and a final
// radix-8 stage's from w^1 (cmul products, fewer shared-memory reads; passes
// B and C use it, where shared-memory wavefronts are the tighter resource).
// buf: one padded shared buffer of Plan<M>::SMEM float2 owned by this
// transform (padded index i + i/16 keeps the transposed stores conflict
// free); tws: the stage-ordered twiddle table of TwLay<M> in shared memory.
// Every padded index is a per-thread base plus a compile-time offset (T, Ns
// and M/RF are multiples of 16, so pad(b + 16 c) = pad(b) + 17 c).  The
// barrier (bar_id, bar_count) covers the threads of this transform, so the
// groups of a CTA proceed independently.
template <int M, bool INV, bool TWREC = false>
__device__ __forceinline__ void fft1s(float2 (&v)[16], float2* buf, const float2* tws, int tid,
                                      int bar_id, int bar_count) {
  using P = Plan<M>;
  using L = TwLay<M>;
  constexpr int T = P::T;
  constexpr int TP = T + T / 16;  // pad(x + T) - pad(x)
  static_assert(T % 16 == 0, "register FFT needs M >= 256");
  dft16<INV>(v);
  group_sync(bar_id, bar_count);  // earlier readers of buf are done
  {
    float2* b0 = buf + 17 * tid;  // pad(16 tid + q) = 17 tid + q
#pragma unroll
    for (int q = 0; q < 16; ++q) b0[q] = v[q];
  }
  group_sync(bar_id, bar_count);
  const float2* bl = buf + (tid + (tid >> 4));  // pad(tid + T q) = pad(tid) + TP q
#pragma unroll
  for (int st = 0; st < L::MID; ++st) {
    const int Ns = L::span(st);
    const int k = tid & (Ns - 1);
    const float2* tk = tws + L::mid_off(st) + k;
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = bl[TP * q];
    group_sync(bar_id, bar_count);
    if constexpr (TWREC) {
      float2 w[16];
      tw_powers16(tk[0], tk[3 * Ns], w);
#pragma unroll
      for (int q = 1; q < 16; ++q) v[q] = twiddle<INV>(v[q], w[q]);
    } else {
#pragma unroll
      for (int q = 1; q < 16; ++q) v[q] = twiddle<INV>(v[q], tk[(q - 1) * Ns]);
    }
    dft16<INV>(v);
    const int base = (tid - k) * 16 + k;
    float2* bs = buf + (base + (base >> 4));
    const int NP = Ns + Ns / 16;
#pragma unroll
    for (int q = 0; q < 16; ++q) bs[NP * q] = v[q];
    group_sync(bar_id, bar_count);
  }
  const float2* tl = tws + L::LAST + tid;
  if (P::RF == 1) {
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = bl[TP * q];
#pragma unroll
    for (int q = 1; q < 16; ++q) v[q] = twiddle<INV>(v[q], tl[(q - 1) * T]);
    dft16<INV>(v);
  } else {
    // last stage radix RF, span M/RF; butterflies j = tid + T i, i < 16/RF
    constexpr int RF = P::RF;
    constexpr int NB = 16 / RF;
    constexpr int NSF = M / RF;
    constexpr int FP = NSF + NSF / 16;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      const float2* bj = bl + TP * i;  // pad(j)
      float2 u[RF];
#pragma unroll
      for (int q = 0; q < RF; ++q) u[q] = bj[FP * q];
      if (TWREC && RF == 8) {  // w^2..w^7 from w^1: one table read instead of seven
        const float2 w1 = tl[T * i];
        const float2 w2 = cmul(w1, w1), w3 = cmul(w2, w1), w4 = cmul(w2, w2);
        u[1] = twiddle<INV>(u[1], w1);
        u[2] = twiddle<INV>(u[2], w2);
        u[3] = twiddle<INV>(u[3], w3);
        u[4] = twiddle<INV>(u[4], w4);
        u[5] = twiddle<INV>(u[5], cmul(w4, w1));
        u[6] = twiddle<INV>(u[6], cmul(w4, w2));
        u[7] = twiddle<INV>(u[7], cmul(w4, w3));
      } else
#pragma unroll
      for (int q = 1; q < RF; ++q) u[q] = twiddle<INV>(u[q], tl[(q - 1) * NSF + T * i]);
      if (RF == 2) dft2<INV>(u[0], u[1]);
      if (RF == 4) dft4<INV>(u[0], u[1], u[2], u[3]);
      if (RF == 8) dft8<INV>(u);
      // output index j + q NSF = tid + T (i + q NB)
#pragma unroll
      for (int q = 0; q < RF; ++q) v[i + q * NB] = u[q];
    }
  }
}

}  // namespace regfft
}  // namespace osgpu
