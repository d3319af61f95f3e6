// Plain structs shared by the host planner and the sm_103a kernels.
//
// Layouts in HBM:
//   field      row-major ny x nx complex (index iy*nx + ix), interleaved
//              {re, im}; complex128 for the f64 engine, complex64 for f32.
//   spectrum   "column-major" scratch Px x ny: element (kx, iy) at
//              kx*ld + iy, so a spectral column is contiguous (pass B reads
//              and writes it with unit stride).
#pragma once
#include <cstdint>
#include <vector_types.h>

namespace osgpu {

constexpr int kMaxStages = 20;
constexpr int kMaxElements = 8;

// One axis of a padded transform: support n (field samples), padded
// length P = r*m, sub-FFT length m (m | P, m >= n), Stockham radices of m.
struct AxisPlan {
  int n;
  int P;
  int m;
  int r;
  int nst;
  int radix[kMaxStages];
};

enum EngineKind : int {
  ENG_ASM = 0,          // exact angular spectrum (on-the-fly H)
  ENG_FRESNEL_TF = 1,   // Fresnel transfer function (on-the-fly H)
  ENG_KSPEC = 2,        // precomputed kernel spectrum (Fresnel conv, RS)
  ENG_KSEP = 3,         // separable kernel spectrum Hx[kx]*Hy[ky] (Fresnel conv)
  ENG_IDENTITY = 4,     // spectrum untouched (used to build 2D FFTs)
  ENG_KEVEN = 5,        // even kernel spectrum, quarter table (kernel-spectrum plans, f32)
};

enum ElementKind : int {
  EL_ELLIPSE = 1,   // EllipticalAperture (element predicate b2 x^2 + a2 y^2 > a2 b2)
  EL_RECT = 2,      // RectangularAperture
  EL_LENS = 3,      // ThinLens with a clear-aperture stop
  EL_PHASE = 4,     // PhaseMask::sampled (bilinear lattice) with a stop
  EL_GRATING = 5,   // BlazedGrating with a stop
  EL_SCREEN = 6,    // phase screen sampled on the field grid, with a stop
};

enum StopKind : int { STOP_FIELD = 0, STOP_CIRCLE = 1, STOP_ELLIPSE = 2, STOP_RECT = 3 };

// Device-side element: everything in FP64 plus optional f32 fast tables.
struct DevElement {
  int kind;
  int stop;        // stop of lens / mask / grating
  double a, b;     // semi-axes, half-widths or stop half-extents (m)
  double psi, cpsi, spsi;
  double cx, cy;
  double k;        // 2 pi / lambda (lens)
  double f;        // focal length at this band (lens)
  double inv_period, depth;  // grating
  const double* lat;         // sampled phase lattice (device, row-major lny x lnx)
  int lnx, lny;
  double ldx, ldy;
  // f32 fast tables (psi == 0 elements; built by launch_element_tables).
  const int2* span;          // per row inclusive [lo, hi] of the transmitting set (lo > hi: none)
  const float2* tabx;        // per column factor (lens x part, grating)
  const float2* taby;        // per row factor (lens y part)
  const float* latf;         // f32 copy of the phase lattice (caller-owned f32 screen values)
  const float2* scr;         // screen: per-sample transmission e^{i depth v} (f32 engine)
  const int4* bilx;          // per column bilinear lookup (i0, i1, bits of tx, inside)
  const int4* bily;          // per row bilinear lookup (j0, j1, bits of ty, inside)
};

struct ElementList {
  int count;
  int fast;  // 1: every element carries f32 fast tables (f32 engine only)
  DevElement el[kMaxElements];
};

}  // namespace osgpu
