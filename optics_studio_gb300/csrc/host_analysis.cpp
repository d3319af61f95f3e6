// Host-side analysis: see host_analysis.h.  Compiled with -ffp-contract=off.
#include "host_analysis.h"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace osgpu {

static const double PI = 3.14159265358979323846;

uint64_t padded_len(uint64_t n, double padding) {
  if (padding <= 1.0) return n;
  return (uint64_t)std::ceil((double)n * padding);
}

double axis_band_limit(double lam, double z, double grid_width, bool band_limited, double medium) {
  const double lam_n = lam / medium;
  if (band_limited) {
    const double t = 2.0 * z / grid_width;
    return 1.0 / (lam_n * std::sqrt(t * t + 1.0));
  }
  return 1.0 / lam_n;
}

// asm.rs:307-368
static double asm_step_along(uint64_t n_pad, double d, double f_other, double lim_other,
                             double lim_self, double lam_n, double kz, bool band_limited) {
  const double df = 1.0 / ((double)n_pad * d);
  const double nyq = (double)(n_pad / 2) * df;
  const double inv = 1.0 / lam_n;
  const double f_circle = std::sqrt(std::fmax(inv * inv - f_other * f_other, 0.0));
  double f_edge = std::fmin(f_circle, nyq);
  if (band_limited) {
    if (std::fabs(f_other) > lim_other) return 0.0;
    f_edge = std::fmin(f_edge, lim_self);
  }
  const double hi = std::fmax(std::floor(f_edge / df), 0.0) * df;
  const double lo = std::fmax(hi - df, 0.0);
  auto root = [&](double f) {
    return std::sqrt(std::fmax(1.0 - lam_n * lam_n * (f * f + f_other * f_other), 0.0));
  };
  return kz * std::fabs(root(hi) - root(lo));
}

void asm_analyze(const osgpu_grid& g, double z, const osgpu_asm_config& cfg, double padding,
                 osgpu_asm_report& r) {
  const uint64_t nx_pad = padded_len(g.nx, padding), ny_pad = padded_len(g.ny, padding);
  const bool bl = cfg.band_limited != 0;
  const double lim_x = axis_band_limit(g.lambda, z, (double)nx_pad * g.dx, bl, cfg.medium);
  const double lim_y = axis_band_limit(g.lambda, z, (double)ny_pad * g.dy, bl, cfg.medium);
  const double lam_n = g.lambda / cfg.medium;
  const double kz = (2.0 * PI / lam_n) * std::fabs(z);
  double sx = asm_step_along(nx_pad, g.dx, 0.0, lim_y, lim_x, lam_n, kz, bl);
  double sy = asm_step_along(ny_pad, g.dy, 0.0, lim_x, lim_y, lam_n, kz, bl);
  if (bl) {
    sx = std::fmax(sx, asm_step_along(nx_pad, g.dx, lim_y, lim_y, lim_x, lam_n, kz, bl));
    sy = std::fmax(sy, asm_step_along(ny_pad, g.dy, lim_x, lim_x, lim_y, lam_n, kz, bl));
  }
  r.lambda = g.lambda;
  r.medium = cfg.medium;
  r.z = z;
  r.nx = g.nx;
  r.ny = g.ny;
  r.dx = g.dx;
  r.dy = g.dy;
  r.requested_padding = cfg.padding;
  r.used_padding = padding;
  r.nx_pad = nx_pad;
  r.ny_pad = ny_pad;
  r.band_limit_fx = lim_x;
  r.band_limit_fy = lim_y;
  r.max_phase_step_x = sx;
  r.max_phase_step_y = sy;
  r.nyquist_ok = (sx < PI && sy < PI) ? 1 : 0;
}

int asm_resolve(const osgpu_grid& g, double z, const osgpu_asm_config& cfg, osgpu_asm_report& r) {
  std::memset(&r, 0, sizeof(r));
  if (!std::isfinite(z)) return OSGPU_E_INVALID_DISTANCE;
  if (!std::isfinite(g.lambda) || g.lambda <= 0.0) return OSGPU_E_INVALID_WAVELENGTH;
  if (!std::isfinite(cfg.medium) || cfg.medium <= 0.0) return OSGPU_E_INVALID_MEDIUM;
  if (g.nx == 0 || g.ny == 0) return OSGPU_E_EMPTY_GRID;
  if (z == 0.0) return -1;
  asm_analyze(g, z, cfg, cfg.padding, r);
  if (cfg.strict && !r.nyquist_ok) {
    double padding = cfg.padding;
    while (!r.nyquist_ok && padding < cfg.max_padding) {
      padding = std::fmin(padding * 2.0, cfg.max_padding);
      asm_analyze(g, z, cfg, padding, r);
    }
    if (!r.nyquist_ok) return OSGPU_E_ALIASING_RISK;
  }
  return OSGPU_OK;
}

// fresnel.rs:267-298
static double fr_worst_axis_step(uint64_t n_pad, double d, double lam, double z) {
  const double df = 1.0 / ((double)n_pad * d);
  const double f_nyq = (double)(n_pad / 2) * df;
  const double hi = std::fmax(std::floor(f_nyq / df), 0.0) * df;
  const double lo = std::fmax(hi - df, 0.0);
  return PI * lam * std::fabs(z) * (hi * hi - lo * lo);
}
static double fr_worst_paraxial_error(double dx, double dy, double lam, double z) {
  const double fx = 1.0 / (2.0 * dx), fy = 1.0 / (2.0 * dy);
  const double s = (lam * fx) * (lam * fx) + (lam * fy) * (lam * fy);
  const double k = 2.0 * PI / lam;
  return k * std::fabs(z) * (1.0 - 0.5 * s - std::sqrt(std::fmax(1.0 - s, 0.0)));
}
static double fr_worst_kernel_axis_step(uint64_t n_pad, double d, double lam, double z) {
  const double hi = (double)(n_pad / 2) * d;
  const double lo = hi - d;
  return PI * (hi * hi - lo * lo) / (lam * std::fabs(z));
}

void fresnel_analyze(const osgpu_grid& g, double z, const osgpu_fresnel_config& cfg,
                     double padding, osgpu_fresnel_report& r) {
  const uint64_t nx_pad = padded_len(g.nx, padding), ny_pad = padded_len(g.ny, padding);
  r.lambda = g.lambda;
  r.z = z;
  r.nx = g.nx;
  r.ny = g.ny;
  r.dx = g.dx;
  r.dy = g.dy;
  r.requested_padding = cfg.padding;
  r.used_padding = padding;
  r.nx_pad = nx_pad;
  r.ny_pad = ny_pad;
  r.max_phase_step_x = fr_worst_axis_step(nx_pad, g.dx, g.lambda, z);
  r.max_phase_step_y = fr_worst_axis_step(ny_pad, g.dy, g.lambda, z);
  r.nyquist_ok = (r.max_phase_step_x < PI && r.max_phase_step_y < PI) ? 1 : 0;
  r.max_kernel_step_x = fr_worst_kernel_axis_step(nx_pad, g.dx, g.lambda, z);
  r.max_kernel_step_y = fr_worst_kernel_axis_step(ny_pad, g.dy, g.lambda, z);
  r.kernel_nyquist_ok = (r.max_kernel_step_x < PI && r.max_kernel_step_y < PI) ? 1 : 0;
  r.max_phase_error_vs_asm = fr_worst_paraxial_error(g.dx, g.dy, g.lambda, z);
  r.paraxial_ok = r.max_phase_error_vs_asm < 0.01 ? 1 : 0;
}

static int fresnel_validate(const osgpu_grid& g, double z) {
  if (!std::isfinite(z)) return OSGPU_E_INVALID_DISTANCE;
  if (!std::isfinite(g.lambda) || g.lambda <= 0.0) return OSGPU_E_INVALID_WAVELENGTH;
  if (g.nx == 0 || g.ny == 0) return OSGPU_E_EMPTY_GRID;
  return OSGPU_OK;
}

int fresnel_resolve_tf(const osgpu_grid& g, double z, const osgpu_fresnel_config& cfg,
                       osgpu_fresnel_report& r) {
  std::memset(&r, 0, sizeof(r));
  int st = fresnel_validate(g, z);
  if (st) return st;
  if (z == 0.0) return -1;
  fresnel_analyze(g, z, cfg, cfg.padding, r);
  if (cfg.strict && !r.nyquist_ok) {
    double padding = cfg.padding;
    while (!r.nyquist_ok && padding < cfg.max_padding) {
      padding = std::fmin(padding * 2.0, cfg.max_padding);
      fresnel_analyze(g, z, cfg, padding, r);
    }
    if (!r.nyquist_ok) return OSGPU_E_ALIASING_RISK;
  }
  return OSGPU_OK;
}

int fresnel_resolve_conv(const osgpu_grid& g, double z, const osgpu_fresnel_config& cfg,
                         osgpu_fresnel_report& r) {
  std::memset(&r, 0, sizeof(r));
  int st = fresnel_validate(g, z);
  if (st) return st;
  if (z == 0.0) return -1;
  fresnel_analyze(g, z, cfg, cfg.padding, r);
  if (cfg.strict && !r.kernel_nyquist_ok) return OSGPU_E_ALIASING_RISK;
  return OSGPU_OK;
}

void fraunhofer_report(const osgpu_grid& g, double z, const osgpu_fraunhofer_config& cfg,
                       osgpu_fraunhofer_report& r) {
  const double az = std::fabs(z);
  const double xs = cfg.has_source_pos ? cfg.source_x : 0.0;
  const double ys = cfg.has_source_pos ? cfg.source_y : 0.0;
  const double hx = ((double)g.nx - 1.0) / 2.0 * g.dx;
  const double hy = ((double)g.ny - 1.0) / 2.0 * g.dy;
  double rx, ry;
  bool from_ap = false;
  if (cfg.has_aperture_extent && std::isfinite(cfg.aperture_extent) && cfg.aperture_extent > 0.0) {
    rx = ry = cfg.aperture_extent;
    from_ap = true;
  } else {
    rx = hx + std::fabs(xs);
    ry = hy + std::fabs(ys);
  }
  const double n_f_x = rx * rx / (g.lambda * az);
  const double n_f_y = ry * ry / (g.lambda * az);
  const double n_f = std::fmax(n_f_x, n_f_y);
  r.lambda = g.lambda;
  r.z = z;
  r.nx = g.nx;
  r.ny = g.ny;
  r.dx = g.dx;
  r.dy = g.dy;
  r.dx_out = g.lambda * az / ((double)g.nx * g.dx);
  r.dy_out = g.lambda * az / ((double)g.ny * g.dy);
  r.n_f_x = n_f_x;
  r.n_f_y = n_f_y;
  r.source_x = xs;
  r.source_y = ys;
  r.extent_used = std::fmax(rx, ry);
  r.extent_is_aperture = from_ap ? 1 : 0;
  r.quad_phase_error_rad = PI * n_f;
  r.max_n_f = cfg.max_n_f;
  r.regime_ok = (n_f <= cfg.max_n_f) ? 1 : 0;
}

int fraunhofer_resolve(const osgpu_grid& g, double z, const osgpu_fraunhofer_config& cfg,
                       osgpu_fraunhofer_report& r) {
  std::memset(&r, 0, sizeof(r));
  if (!std::isfinite(z) || z == 0.0) return OSGPU_E_INVALID_DISTANCE;
  if (!std::isfinite(g.lambda) || g.lambda <= 0.0) return OSGPU_E_INVALID_WAVELENGTH;
  if (g.nx == 0 || g.ny == 0) return OSGPU_E_EMPTY_GRID;
  fraunhofer_report(g, z, cfg, r);
  if (cfg.strict && !r.regime_ok) return OSGPU_E_REGIME_VIOLATION;
  return OSGPU_OK;
}

// rayleigh_sommerfeld.rs:240-270
static double rs_worst_kernel_axis_step(uint64_t n_pad, double d, double lam, double z) {
  const double k = 2.0 * PI / lam;
  const double x_hi = (double)(n_pad / 2) * d;
  const double x_lo = x_hi - d;
  const double r_hi = std::sqrt(x_hi * x_hi + z * z);
  const double r_lo = std::sqrt(x_lo * x_lo + z * z);
  return k * (r_hi - r_lo) + k * d / (1.0 + k * k * z * z);
}

void rs_analyze(const osgpu_grid& g, double z, double padding, osgpu_rs_report& r) {
  const uint64_t nx_pad = padded_len(g.nx, padding), ny_pad = padded_len(g.ny, padding);
  r.lambda = g.lambda;
  r.z = z;
  r.nx = g.nx;
  r.ny = g.ny;
  r.dx = g.dx;
  r.dy = g.dy;
  r.padding = padding;
  r.nx_pad = nx_pad;
  r.ny_pad = ny_pad;
  r.max_kernel_step_x = rs_worst_kernel_axis_step(nx_pad, g.dx, g.lambda, z);
  r.max_kernel_step_y = rs_worst_kernel_axis_step(ny_pad, g.dy, g.lambda, z);
  r.kernel_nyquist_ok = (r.max_kernel_step_x < PI && r.max_kernel_step_y < PI) ? 1 : 0;
  const double k = 2.0 * PI / g.lambda;
  const double x = (double)(nx_pad / 2) * g.dx;
  const double y = (double)(ny_pad / 2) * g.dy;
  const double az = std::fabs(z);
  const double rr = std::sqrt(x * x + y * y + az * az);
  r.max_phase_error_vs_fresnel = std::fmax(k * (rr - az - (x * x + y * y) / (2.0 * az)), 0.0);
  r.paraxial_ok = r.max_phase_error_vs_fresnel < 0.01 ? 1 : 0;
}

int rs_resolve(const osgpu_grid& g, double z, const osgpu_rs_config& cfg, osgpu_rs_report& r) {
  std::memset(&r, 0, sizeof(r));
  if (!std::isfinite(z) || z == 0.0) return OSGPU_E_INVALID_DISTANCE;
  if (!std::isfinite(g.lambda) || g.lambda <= 0.0) return OSGPU_E_INVALID_WAVELENGTH;
  if (g.nx == 0 || g.ny == 0) return OSGPU_E_EMPTY_GRID;
  rs_analyze(g, z, cfg.padding, r);
  if (cfg.strict && !r.kernel_nyquist_ok) return OSGPU_E_ALIASING_RISK;
  return OSGPU_OK;
}

AxisPlan make_axis(int n, int P) {
  AxisPlan a;
  std::memset(&a, 0, sizeof(a));
  a.n = n;
  a.P = P;
  int m = P;
  for (int d = (n > 0 ? n : 1); d <= P; ++d) {
    if (P % d == 0) {
      m = d;
      break;
    }
  }
  a.m = m;
  a.r = P / m;
  int rem = m, ns = 0;
  while (rem % 8 == 0 && ns < kMaxStages) { a.radix[ns++] = 8; rem /= 8; }
  if (rem % 4 == 0 && ns < kMaxStages) { a.radix[ns++] = 4; rem /= 4; }
  if (rem % 2 == 0 && ns < kMaxStages) { a.radix[ns++] = 2; rem /= 2; }
  while (rem % 3 == 0 && ns < kMaxStages) { a.radix[ns++] = 3; rem /= 3; }
  while (rem % 5 == 0 && ns < kMaxStages) { a.radix[ns++] = 5; rem /= 5; }
  for (int p = 7; rem > 1 && ns < kMaxStages; p += 2) {
    if ((long long)p * p > rem) { a.radix[ns++] = rem; rem = 1; break; }
    while (rem % p == 0 && ns < kMaxStages) { a.radix[ns++] = p; rem /= p; }
  }
  a.nst = ns;
  if (rem != 1) a.nst = -1;  // more than kMaxStages factors: unsupported
  return a;
}

static double wrap_angle(double r) {
  const double tau = 2.0 * PI;
  double w = std::fmod(r, tau);
  if (w < 0.0) w += tau;
  return w;
}

static int validate_footprint(double hx, double hy, double cx, double cy) {
  if (!std::isfinite(hx) || hx <= 0.0 || !std::isfinite(hy) || hy <= 0.0 || !std::isfinite(cx) ||
      !std::isfinite(cy))
    return OSGPU_E_INVALID_APERTURE;
  return OSGPU_OK;
}

static void rotated_box(double hx, double hy, double psi, double& bx, double& by) {
  const double c = std::fabs(std::cos(psi)), s = std::fabs(std::sin(psi));
  bx = hx * c + hy * s;
  by = hx * s + hy * c;
}

int element_check(const osgpu_element& e, const osgpu_grid& g, double lambda, DevElement& d,
                  char* msg, size_t msglen) {
  std::memset(&d, 0, sizeof(d));
  if (!std::isfinite(e.orientation))
    return OSGPU_E_INVALID_ORIENTATION;
  const double psi = wrap_angle(e.orientation);
  d.psi = psi;
  d.cpsi = std::cos(psi);
  d.spsi = std::sin(psi);
  d.cx = e.center_x;
  d.cy = e.center_y;
  d.a = e.a;
  d.b = e.b;
  d.stop = e.stop;
  const double gx = ((double)g.nx - 1.0) / 2.0 * g.dx;
  const double gy = ((double)g.ny - 1.0) / 2.0 * g.dy;
  auto outside = [&](double fx, double fy) {
    if (std::fabs(e.center_x) + fx > gx || std::fabs(e.center_y) + fy > gy) {
      if (msg)
        std::snprintf(msg, msglen,
                      "aperture half-extents (%g m x %g m) at (%g, %g) m exceed the field grid "
                      "half-extents (%g m x %g m)",
                      fx, fy, e.center_x, e.center_y, gx, gy);
      return true;
    }
    return false;
  };
  // ClearAperture::validate (construction time, element.rs:415-432).
  auto stop_validate = [&]() -> int {
    if (e.stop == OSGPU_STOP_FIELD) {
      if (!std::isfinite(e.center_x) || !std::isfinite(e.center_y)) return OSGPU_E_INVALID_AXIS;
      return OSGPU_OK;
    }
    if (e.stop < 0 || e.stop > OSGPU_STOP_RECT) return OSGPU_E_BAD_ARGUMENT;
    return validate_footprint(e.a, e.b, e.center_x, e.center_y);
  };
  // Footprint-vs-grid check of apply (element.rs:498-505 footprint_at).
  auto stop_outside = [&]() -> int {
    if (e.stop == OSGPU_STOP_FIELD) return OSGPU_OK;
    double fx = e.a, fy = e.b;
    if (e.stop != OSGPU_STOP_CIRCLE) rotated_box(e.a, e.b, psi, fx, fy);
    return outside(fx, fy) ? OSGPU_E_OUTSIDE_FIELD : OSGPU_OK;
  };
  auto stop_check = [&]() -> int {
    int st = stop_validate();
    return st ? st : stop_outside();
  };
  switch (e.kind) {
    case OSGPU_EL_ELLIPTICAL_APERTURE: {
      d.kind = EL_ELLIPSE;
      int st = validate_footprint(e.a, e.b, e.center_x, e.center_y);
      if (st) return st;
      double bx = e.a, by = e.b;
      if (e.a != e.b) rotated_box(e.a, e.b, psi, bx, by);
      if (outside(bx, by)) return OSGPU_E_OUTSIDE_FIELD;
      return OSGPU_OK;
    }
    case OSGPU_EL_RECTANGULAR_APERTURE: {
      d.kind = EL_RECT;
      int st = validate_footprint(e.a, e.b, e.center_x, e.center_y);
      if (st) return st;
      double bx, by;
      rotated_box(e.a, e.b, psi, bx, by);
      if (outside(bx, by)) return OSGPU_E_OUTSIDE_FIELD;
      return OSGPU_OK;
    }
    case OSGPU_EL_THIN_LENS: {
      d.kind = EL_LENS;
      int st = stop_validate();
      if (st) return st;
      if (!std::isfinite(e.focal) || e.focal == 0.0) return OSGPU_E_INVALID_FOCAL;
      st = stop_outside();
      if (st) return st;
      d.k = 2.0 * PI / lambda;
      d.f = e.focal;
      return OSGPU_OK;
    }
    case OSGPU_EL_PHASE_MASK_SAMPLED: {
      d.kind = EL_PHASE;
      if (e.lnx == 0 || e.lny == 0 || e.lattice == nullptr) return OSGPU_E_INVALID_GRID;
      if (!std::isfinite(e.ldx) || e.ldx <= 0.0 || !std::isfinite(e.ldy) || e.ldy <= 0.0)
        return OSGPU_E_INVALID_GRID_PITCH;
      // A host lattice is scanned here, as PhaseMask::sampled does; a device
      // lattice (lattice_on_device) was scanned when it was created and is
      // never dereferenced on the host.
      if (!e.lattice_on_device) {
        const double* lat = reinterpret_cast<const double*>(e.lattice);
        const uint64_t n = e.lnx * e.lny;
        for (uint64_t k = 0; k < n; ++k)
          if (!std::isfinite(lat[k])) return OSGPU_E_INVALID_PHASE;
      }
      int st = stop_check();
      if (st) return st;
      d.lnx = (int)e.lnx;
      d.lny = (int)e.lny;
      d.ldx = e.ldx;
      d.ldy = e.ldy;
      return OSGPU_OK;
    }
    case OSGPU_EL_GRID_SCREEN: {
      d.kind = EL_SCREEN;
      if (e.lattice == nullptr || e.lnx != g.nx || e.lny != g.ny) return OSGPU_E_INVALID_GRID;
      if (!std::isfinite(e.depth)) return OSGPU_E_INVALID_PHASE;
      if (!e.lattice_on_device) {  // host values: all finite (0 outside the stop)
        const double* v = reinterpret_cast<const double*>(e.lattice);
        const uint64_t n = e.lnx * e.lny;
        for (uint64_t k = 0; k < n; ++k)
          if (!std::isfinite(v[k])) return OSGPU_E_INVALID_PHASE;
      }
      int st = stop_check();
      if (st) return st;
      d.lnx = (int)e.lnx;
      d.lny = (int)e.lny;
      d.depth = e.depth;
      return OSGPU_OK;
    }
    case OSGPU_EL_BLAZED_GRATING: {
      d.kind = EL_GRATING;
      if (!std::isfinite(e.period) || e.period <= 0.0 || !std::isfinite(e.depth))
        return OSGPU_E_INVALID_GRATING;
      int st = stop_check();
      if (st) return st;
      d.inv_period = 1.0 / e.period;
      d.depth = e.depth;
      return OSGPU_OK;
    }
    default:
      return OSGPU_E_BAD_ARGUMENT;
  }
}

int asm_f32_split_ok(const osgpu_grid& g, double z, double medium, uint64_t Px, uint64_t Py,
                     bool band_limited, double lim_x, double lim_y) {
  const double lam_n = g.lambda / medium;
  double fxm = (double)(Px / 2) / ((double)Px * g.dx);
  double fym = (double)(Py / 2) / ((double)Py * g.dy);
  if (band_limited) {
    fxm = std::fmin(fxm, lim_x);
    fym = std::fmin(fym, lim_y);
  }
  const double a = (lam_n * fxm) * (lam_n * fxm);
  const double b = (lam_n * fym) * (lam_n * fym);
  double s = std::fmin(a + b, 1.0);
  const double K = (2.0 * PI / lam_n) * std::fabs(z);
  const double q = std::sqrt(1.0 - s);
  const double tau = s * s * s * (3.0 + q) / (8.0 * (1.0 + q) * (1.0 + q) * (1.0 + q));
  const double cross = K * a * b / 4.0;
  return (K * tau <= 3.0 && cross <= 1.0e4 && s < 0.5) ? 1 : 0;
}

}  // namespace osgpu
