/*
 * osgpu.h -- C ABI of the GB300 (sm_103a) propagation library.
 *
 * This is the drop-in boundary for the optics-studio hot path: every entry
 * point is what the Rust FFI crate behind optics-core / optics-inverse
 * binds.  Plain C: status-int returns, plain pointers and sizes, no
 * exceptions cross the boundary.  Field samples are interleaved {re, im}
 * doubles in the reference's row-major layout (index iy*nx + ix), i.e.
 * `Vec<Complex64>::as_ptr()` of `optics_core::field::Field` viewed as
 * `const double*` (reference src/field.rs:99-105).
 *
 * Threading: calls are serialised internally on one stream per device.
 * Status codes map 1:1 onto the reference's error variants (see the
 * OSGPU_E_* list); on failure osgpu_last_error() holds a message.
 */
#ifndef OSGPU_H
#define OSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  OSGPU_OK = 0,
  /* PropagationError / FresnelError / FraunhoferError / RayleighSommerfeldError
   * (src/propagation/asm.rs:219-250, fresnel.rs:225-254, fraunhofer.rs:259-282,
   * rayleigh_sommerfeld.rs:197-223) */
  OSGPU_E_INVALID_DISTANCE = 1,
  OSGPU_E_INVALID_WAVELENGTH = 2,
  OSGPU_E_INVALID_MEDIUM = 3,
  OSGPU_E_EMPTY_GRID = 4,
  OSGPU_E_NON_FINITE_SAMPLE = 5,
  OSGPU_E_ALIASING_RISK = 6,
  OSGPU_E_REGIME_VIOLATION = 7,
  /* OpticsError (src/element.rs:62-230) */
  OSGPU_E_INVALID_APERTURE = 20,
  OSGPU_E_OUTSIDE_FIELD = 21,
  OSGPU_E_INVALID_AXIS = 22,
  OSGPU_E_INVALID_FOCAL = 23,
  OSGPU_E_INVALID_ORIENTATION = 24,
  OSGPU_E_INVALID_PHASE = 25,
  OSGPU_E_INVALID_GRID = 26,
  OSGPU_E_INVALID_GRID_PITCH = 27,
  OSGPU_E_INVALID_GRATING = 28,
  OSGPU_E_INVALID_SAG = 29, /* raised by bindings that evaluate a sag (RefractiveSurface) */
  OSGPU_E_INVALID_THICKNESS = 30, /* ThickLens central thickness (bindings, element.rs:207) */
  OSGPU_E_INVALID_SURFACE = 31,   /* surface profile parameters or conic domain (element.rs:177) */
  /* InverseError (crates/optics-inverse/src/error.rs:11-85) */
  OSGPU_E_WRONG_DIMENSION = 40,
  OSGPU_E_NOT_FINITE = 41,
  OSGPU_E_OUT_OF_BOUNDS = 42,
  OSGPU_E_RENDER = 43,
  OSGPU_E_ADJOINT = 44,
  /* library conditions with no reference counterpart */
  OSGPU_E_UNSUPPORTED = 100, /* size beyond the kernels' shared-memory plan */
  OSGPU_E_CUDA = 101,
  OSGPU_E_BAD_ARGUMENT = 102,
  OSGPU_E_NO_DEVICE = 103,
  OSGPU_E_OUT_OF_MEMORY = 104
};

/* Arithmetic of a propagation.  F64 is the plain path (parity <= 1e-12 with
 * the f64 reference); F32 computes the FFTs and multiplies in complex64 with
 * FP64-derived phase tables. */
enum { OSGPU_F64 = 0, OSGPU_F32 = 1 };

/* Device buffer element type for the *_device entry points. */
enum { OSGPU_C128 = 0, OSGPU_C64 = 1 };

/* Grid of one BandField: Field dims/pitch + BandField wavelength
 * (src/field.rs:99-105, 287-290). */
typedef struct {
  uint64_t nx, ny;
  double dx, dy;
  double lambda;
} osgpu_grid;

/* ------------------------------------------------------------ ASM engine */
/* AsmConfig (src/propagation/asm.rs:101-137). */
typedef struct {
  double padding;
  int32_t band_limited;
  int32_t strict;
  double max_padding;
  double medium;
} osgpu_asm_config;

/* SamplingReport (src/propagation/asm.rs:145-179). */
typedef struct {
  double lambda, medium, z;
  uint64_t nx, ny;
  double dx, dy;
  double requested_padding, used_padding;
  uint64_t nx_pad, ny_pad;
  double band_limit_fx, band_limit_fy;
  double max_phase_step_x, max_phase_step_y;
  int32_t nyquist_ok;
} osgpu_asm_report;

/* asm::sampling_report (asm.rs:418-420): diagnostics at cfg->padding. */
int osgpu_asm_sampling_report(const osgpu_grid* g, double z, const osgpu_asm_config* cfg,
                              osgpu_asm_report* out);

/* asm::propagate (asm.rs:438-538).  in/out: host complex128, nx*ny samples
 * (may alias).  `report` (optional) receives the report the propagation ran
 * on (also filled on OSGPU_E_ALIASING_RISK).  z == 0 copies in to out. */
int osgpu_asm_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                        const osgpu_asm_config* cfg, int32_t precision,
                        osgpu_asm_report* report);

/* Device-resident form: d_in/d_out are device buffers of `dtype`
 * (OSGPU_C128 -> f64 engine, OSGPU_C64 -> f32 engine), `stream` a
 * cudaStream_t (NULL: the library stream).  Asynchronous; the NonFinite
 * check is folded into the first pass and reported by osgpu_sync_status. */
int osgpu_asm_propagate_device(const void* d_in, void* d_out, int32_t dtype,
                               const osgpu_grid* g, double z, const osgpu_asm_config* cfg,
                               void* stream, osgpu_asm_report* report);

/* -------------------------------------------------------- Fresnel engine */
/* FresnelConfig (src/propagation/fresnel.rs:99-123). */
typedef struct {
  double padding;
  int32_t strict;
  double max_padding;
} osgpu_fresnel_config;

/* FresnelSamplingReport (fresnel.rs:130-170). */
typedef struct {
  double lambda, z;
  uint64_t nx, ny;
  double dx, dy;
  double requested_padding, used_padding;
  uint64_t nx_pad, ny_pad;
  double max_phase_step_x, max_phase_step_y;
  int32_t nyquist_ok;
  double max_kernel_step_x, max_kernel_step_y;
  int32_t kernel_nyquist_ok;
  double max_phase_error_vs_asm;
  int32_t paraxial_ok;
} osgpu_fresnel_report;

int osgpu_fresnel_sampling_report(const osgpu_grid* g, double z, const osgpu_fresnel_config* cfg,
                                  osgpu_fresnel_report* out);
/* fresnel::propagate (transfer-function form, fresnel.rs:430-509). */
int osgpu_fresnel_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                            const osgpu_fresnel_config* cfg, int32_t precision,
                            osgpu_fresnel_report* report);
/* fresnel::propagate_convolution (fresnel.rs:531-590). */
int osgpu_fresnel_propagate_convolution(const double* in, double* out, const osgpu_grid* g,
                                        double z, const osgpu_fresnel_config* cfg,
                                        int32_t precision, osgpu_fresnel_report* report);

/* ----------------------------------------------------- Fraunhofer engine */
/* FraunhoferConfig (src/propagation/fraunhofer.rs:118-171).  has_* select
 * the Option<_> fields. */
typedef struct {
  int32_t strict;
  double max_n_f;
  int32_t has_source_pos;
  double source_x, source_y;
  int32_t has_aperture_extent;
  double aperture_extent;
} osgpu_fraunhofer_config;

/* FraunhoferReport (fraunhofer.rs:177-213). */
typedef struct {
  double lambda, z;
  uint64_t nx, ny;
  double dx, dy;
  double dx_out, dy_out;
  double n_f_x, n_f_y;
  double source_x, source_y;
  double extent_used;
  int32_t extent_is_aperture;
  double quad_phase_error_rad;
  double max_n_f;
  int32_t regime_ok;
} osgpu_fraunhofer_report;

int osgpu_fraunhofer_regime_report(const osgpu_grid* g, double z,
                                   const osgpu_fraunhofer_config* cfg,
                                   osgpu_fraunhofer_report* out);
/* fraunhofer::propagate (fraunhofer.rs:364-443).  The output lives on the
 * far-field grid: same dims, pitch (report->dx_out, report->dy_out). */
int osgpu_fraunhofer_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                               const osgpu_fraunhofer_config* cfg, int32_t precision,
                               osgpu_fraunhofer_report* report);

/* ------------------------------------------- Rayleigh-Sommerfeld engine */
/* RayleighSommerfeldConfig (rayleigh_sommerfeld.rs:95-116). */
typedef struct {
  double padding;
  int32_t strict;
} osgpu_rs_config;

/* RayleighSommerfeldSamplingReport (rayleigh_sommerfeld.rs:123-160). */
typedef struct {
  double lambda, z;
  uint64_t nx, ny;
  double dx, dy;
  double padding;
  uint64_t nx_pad, ny_pad;
  double max_kernel_step_x, max_kernel_step_y;
  int32_t kernel_nyquist_ok;
  double max_phase_error_vs_fresnel;
  int32_t paraxial_ok;
} osgpu_rs_report;

int osgpu_rs_sampling_report(const osgpu_grid* g, double z, const osgpu_rs_config* cfg,
                             osgpu_rs_report* out);
/* rayleigh_sommerfeld::propagate (rayleigh_sommerfeld.rs:384-442). */
int osgpu_rs_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                       const osgpu_rs_config* cfg, int32_t precision, osgpu_rs_report* report);

/* --------------------------------------------------------------- fft */
/* fft::fft2 / fft::ifft2 (propagation/fft.rs:40-108): 2D DFT of a row-major
 * ny x nx complex grid in the NumPy convention (forward unnormalised with
 * kernel e^{-2 pi i k n / N}, inverse scaled by 1/(nx ny), unshifted bins),
 * any sizes the shared-memory plan holds.  Host complex128 buffers (may
 * alias); precision OSGPU_F64, or OSGPU_F32 (computed in f32). */
int osgpu_fft2(const double* in, double* out, uint64_t nx, uint64_t ny, int32_t inverse,
               int32_t precision);
/* Device variant: complex128 (f64 engine) or complex64 (f32 engine) buffers
 * (may not alias), asynchronous on `stream` (NULL: the library stream). */
int osgpu_fft2_device(const void* d_in, void* d_out, int32_t dtype, uint64_t nx, uint64_t ny,
                      int32_t inverse, void* stream);

/* --------------------------------------------------------------- sources */
/* Source fields written on the device (complex128 or complex64 per dtype),
 * per sample in FP64: sources::gaussian, the q-form beam at distance z from
 * its waist (sources.rs:259-296; invalid beam or plane: OSGPU_E_BAD_ARGUMENT),
 * BandField::plane_wave (field.rs:360-386) and BandField::uniform
 * (field.rs:315-330).  Asynchronous on `stream` (NULL: the library stream). */
int osgpu_source_gaussian_device(void* d_out, int32_t dtype, const osgpu_grid* g, double w0,
                                 double amplitude, double center_x, double center_y, double z,
                                 void* stream);
int osgpu_source_plane_wave_device(void* d_out, int32_t dtype, const osgpu_grid* g,
                                   double theta_x, double theta_y, double amplitude,
                                   void* stream);
int osgpu_source_uniform_device(void* d_out, int32_t dtype, const osgpu_grid* g,
                                double amplitude, double phase, void* stream);

/* --------------------------------------------------------------- elements */
enum {
  OSGPU_EL_ELLIPTICAL_APERTURE = 1, /* element.rs:635-790 */
  OSGPU_EL_RECTANGULAR_APERTURE = 2, /* element.rs:817-929 */
  OSGPU_EL_THIN_LENS = 3,            /* element.rs:965-1154 */
  OSGPU_EL_PHASE_MASK_SAMPLED = 4,   /* element.rs:1321-1484 */
  OSGPU_EL_BLAZED_GRATING = 5,       /* element.rs:1519-1703 */
  /* Phase screen sampled on the field grid: transmission stop(x', y') *
   * exp(i * depth * v[iy][ix]) with v the lattice (lnx = nx, lny = ny, one
   * value per field sample, finite everywhere; ldx/ldy unused) and the stop
   * evaluated in the element frame (orientation, center).  The binding of the
   * elements whose phase the caller evaluates per sample at the exact
   * element-frame coordinates: analytic PhaseMask::new (v = profile, depth =
   * 1), RefractiveSurface (v = surface_z, depth = k (n1 - n2), element.rs:
   * 2043-2123), ThickLens (v = thickness, element.rs:2272-2330) and Wedge
   * (v = thickness, depth = k (n - 1), element.rs:2470-2540). */
  OSGPU_EL_GRID_SCREEN = 6
};
/* ClearAperture (element.rs:384-408) */
enum { OSGPU_STOP_FIELD = 0, OSGPU_STOP_CIRCLE = 1, OSGPU_STOP_ELLIPSE = 2, OSGPU_STOP_RECT = 3 };

/* One thin element at a plane.  Host-side closures of the reference
 * (ThinLens f(lambda), analytic PhaseMask) are evaluated by the caller:
 * `focal` is f(band lambda); an analytic PhaseMask is passed as its lattice
 * sampled on the field grid. */
typedef struct {
  int32_t kind;
  int32_t stop;          /* clear aperture of lens / mask / grating */
  double a, b;           /* semi-axes (ellipse), half-widths (rect) or stop extents */
  double orientation;    /* radians (wrapped into [0, 2pi) as Angle::new) */
  double center_x, center_y;
  double focal;          /* thin lens: f(lambda) */
  double period, depth;  /* blazed grating */
  const void* lattice;   /* sampled phase (double), row-major lny x lnx */
  uint64_t lnx, lny;
  double ldx, ldy;
  int32_t lattice_on_device; /* 0: `lattice` is host memory (scanned for non-finite
                                values as PhaseMask::sampled does, then uploaded);
                                1: device memory, used in place (the caller owns the
                                finiteness guarantee);
                                2: device memory holding float (f32 engine only,
                                orientation 0), used in place */
} osgpu_element;

/* Device copy of a sampled phase lattice, created once (PhaseMask::sampled,
 * element.rs:1321-1368: the lattice is scanned for non-finite values here,
 * OSGPU_E_INVALID_PHASE).  `*handle` is a device pointer to the f64 lattice
 * usable as osgpu_element.lattice with lattice_on_device = 1; the library
 * also keeps an f32 copy for the f32 engine.  Destroy when no call uses it. */
int osgpu_lattice_create(const double* host, uint64_t lnx, uint64_t lny, void** handle);
int osgpu_lattice_destroy(void* handle);

/* Element::apply of each element in order (pointwise transmission). */
int osgpu_apply_elements(const double* in, double* out, const osgpu_grid* g,
                         const osgpu_element* els, int32_t n_els, int32_t precision);

/* --------------------------------------------------------------- beamline */
/* One Beamline step (src/beamline.rs:52-99): elements applied at the plane,
 * then a propagation of z_after through `medium` (skipped when 0). */
typedef struct {
  const osgpu_element* elements;
  int32_t n_elements;
  double z_after;
  double medium;
} osgpu_step;

/* Beamline::trace with the ASM engine closure (observe.rs:195-210 form:
 * AsmConfig with the step's medium).  Each plane costs one fused pass set:
 * elements are applied inside the first FFT pass.  `reports` (optional)
 * receives one report per step (zeroed for z_after == 0). */
int osgpu_beamline_trace(const double* in, double* out, const osgpu_grid* g,
                         const osgpu_step* steps, int32_t n_steps, const osgpu_asm_config* cfg,
                         int32_t precision, osgpu_asm_report* reports);

/* Batched, device-resident Beamline::trace with the ASM engine: one item per
 * band (or independent propagation).  d_in/d_out are device fields of
 * `dtype` (may alias); items may differ in grid size, wavelength, distances
 * and elements.  Asynchronous on `stream` (NULL: the library stream); a
 * non-finite input is reported by osgpu_sync_status.  `reports` (optional)
 * receives n_items * reports_stride reports, item-major. */
typedef struct {
  const void* d_in;
  void* d_out;
  osgpu_grid grid;
  const osgpu_step* steps;
  int32_t n_steps;
} osgpu_trace_item;

int osgpu_beamline_trace_batch_device(const osgpu_trace_item* items, int32_t n_items,
                                      const osgpu_asm_config* cfg, int32_t dtype, void* stream,
                                      osgpu_asm_report* reports, int32_t reports_stride);

/* Beamline::trace of many bands from HOST buffers (complex128, the Rust
 * layout), e.g. every band of Renderer::render_frame (observe.rs:195-210):
 * the host->device copy of band i+1 and the device->host copy of band i-1
 * run on their own streams while band i is traced (two device slots each
 * way).  Page-locked host buffers overlap fully; pageable ones are staged
 * by the CUDA runtime.  Synchronous: outputs are on the host when it returns; a
 * non-finite input sample anywhere returns OSGPU_E_NON_FINITE_SAMPLE. */
typedef struct {
  const double* in;
  double* out;
  osgpu_grid grid;
  const osgpu_step* steps;
  int32_t n_steps;
} osgpu_host_trace_item;

int osgpu_beamline_trace_batch(const osgpu_host_trace_item* items, int32_t n_items,
                               const osgpu_asm_config* cfg, int32_t precision,
                               osgpu_asm_report* reports, int32_t reports_stride);

/* A batched trace captured once into a CUDA graph and replayed: creation
 * runs the batch once on the library stream (so every twiddle table and
 * kernel attribute exists), then captures it; each launch replays the same
 * kernels and stream-ordered workspace on `stream` (NULL: the library
 * stream).  The items' device buffers are baked into the graph and must
 * stay valid; host-memory phase lattices are not capturable (use
 * lattice_on_device).  Batched frames of a renderer are the use: the same
 * wavelengths, designs and buffers every frame. */
typedef struct osgpu_graph osgpu_graph;
int osgpu_beamline_trace_batch_graph(const osgpu_trace_item* items, int32_t n_items,
                                     const osgpu_asm_config* cfg, int32_t dtype,
                                     osgpu_graph** out);
int osgpu_graph_launch(osgpu_graph* graph, void* stream);
int osgpu_graph_destroy(osgpu_graph* graph);

/* ---------------------------------------------------------- inverse loops */
/* One frame (band x scene) of a render or adjoint batch: the design traced on
 * the frame's source field with the ASM engine (optics-inverse observe.rs:
 * 195-210; the carrier's Design is passed as Beamline steps).  Device
 * buffers use the call's dtype: complex fields of `dtype`, real arrays of
 * double (OSGPU_C128) or float (OSGPU_C64). */
typedef struct {
  osgpu_grid grid;
  const void* d_source;     /* source field (device) */
  const osgpu_step* steps;  /* design: elements at each plane, then z_after */
  int32_t n_steps;
  void* d_intensity;        /* render: |u|^2 at the detector (NULL: not written) */
  const void* d_dmdi;       /* push_back: seed dM/dI of this frame (real) */
  double dmdi_scale;        /* push_back: seed multiplier (1 for a plain seed) */
  void* const* d_grad;      /* push_back: one dM/dphi accumulator (real, nx*ny) per
                               element of the design in step order; NULL entries are
                               skipped, NULL: none.  Frames may share accumulators
                               (grid_gradient's sum over frames). */
} osgpu_frame;

/* Forward planes kept between a render and the adjoint sweep (the
 * checkpoints of push_back's tape): one device allocation reused and grown
 * across renders.  budget_bytes > 0 caps it; a render whose planes exceed
 * the cap records nothing and push_back recomputes the forward planes per
 * frame, as the reference's push_back does (adjoint.rs:158-190). */
typedef struct osgpu_tape osgpu_tape;
int osgpu_tape_create(uint64_t budget_bytes, osgpu_tape** out);
int osgpu_tape_destroy(osgpu_tape* tape);
uint64_t osgpu_tape_bytes(const osgpu_tape* tape);

/* Renderer::render intensity channel (observe.rs:213-314, one frame per
 * (band, scene)): forward trace of every frame, |u|^2 of the detector field
 * into d_intensity; with a tape, the output field of every propagation is
 * recorded for osgpu_push_back_batch_device.  Asynchronous on `stream`
 * (NULL: the library stream). */
int osgpu_render_batch_device(const osgpu_frame* frames, int32_t n_frames,
                              const osgpu_asm_config* cfg, int32_t dtype, void* stream,
                              osgpu_tape* tape, osgpu_asm_report* reports,
                              int32_t reports_stride);

/* adjoint::push_back per frame (adjoint.rs:140-246), accumulated into the
 * frames' d_grad (adjoint::grid_gradient's sum, adjoint.rs:268-340):
 * w = (dmdi * dmdi_scale) U at the detector, then in reverse order the
 * adjoint propagation A(-z) (asm_adjoint, adjoint.rs:90-92) and at each
 * element grad += -2 Im(conj(mu) V_after), mu <- conj(t) mu.  The seed
 * multiply runs inside the first FFT pass of the first adjoint propagation
 * and each element plane inside the last pass of the propagation before it.
 * With a valid tape from the render of the same frames the forward planes
 * are read from it; otherwise they are recomputed.  Asynchronous. */
int osgpu_push_back_batch_device(const osgpu_frame* frames, int32_t n_frames,
                                 const osgpu_asm_config* cfg, int32_t dtype, void* stream,
                                 const osgpu_tape* tape);

/* sum |u|^2 of a device field in FP64 (compensated); synchronous. */
int osgpu_field_power_device(const void* d_field, int32_t dtype, uint64_t n, void* stream,
                             double* out);

/* Merits over device observations (real_dtype OSGPU_F64 / OSGPU_F32; frames
 * band-major, scenes inner).  `value` receives the merit (synchronous);
 * d_seed (optional, same layout as d_obs) receives dM/dI.  Sums run in FP64
 * with compensation.
 * Spot-window efficiency (no reference counterpart: the merit of the spot-
 * array inverse design): M = -sum_f sum_{k in windows} I_f[k] / p_in[f],
 * p_in host array of n_frames input powers, d_windows a 0/1 byte mask. */
int osgpu_merit_spot_efficiency_device(const void* d_obs, int32_t real_dtype, int32_t n_frames,
                                       uint64_t frame_len, const uint8_t* d_windows,
                                       const double* p_in, void* d_seed, void* stream,
                                       double* value);
/* Weighted spot-array efficiency (no reference counterpart: the merit of the
 * inverse-design workload with a Gaussian spot-array target):
 * M = -sum_f sum_k w[k] I_f[k] / p_in[f], with d_weights a device array of
 * frame_len real weights in the observation's real dtype (e.g. a sum of
 * Gaussian spots of peak 1) and p_in the positive input power of each frame.
 * The seed is dM/dI_f[k] = -w[k] / p_in[f]. */
int osgpu_merit_weighted_efficiency_device(const void* d_obs, int32_t real_dtype,
                                           int32_t n_frames, uint64_t frame_len,
                                           const void* d_weights, const double* p_in,
                                           void* d_seed, void* stream, double* value);
/* MseToTarget (merit.rs:112-164); band/scene -1 selects all (Selector). */
int osgpu_merit_mse_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                           int32_t n_scenes, uint64_t frame_len, const double* d_target,
                           int32_t band, int32_t scene, void* d_seed, void* stream,
                           double* value);
/* EncircledEnergyMerit (merit.rs:167-245); a seed request with a
 * non-positive total returns OSGPU_E_ADJOINT (obs_gradient is None). */
int osgpu_merit_encircled_energy_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                                        int32_t n_scenes, uint64_t nx, uint64_t ny, double dx,
                                        double dy, double radius, int32_t band, int32_t scene,
                                        void* d_seed, void* stream, double* value);
/* SpotRmsMerit (merit.rs:248-321): sqrt(sum I rho^2 / sum I) of the selected
 * frame (0 when sum I <= 0); the seed (rho^2 - R^2) / (2 R sum I) goes to the
 * selected frames and 0 to the others.  A seed request with sum I <= 0 or
 * R <= 0 returns OSGPU_E_ADJOINT (obs_gradient is None). */
int osgpu_merit_spot_rms_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                                int32_t n_scenes, uint64_t nx, uint64_t ny, double dx, double dy,
                                int32_t band, int32_t scene, void* d_seed, void* stream,
                                double* value);
/* StrehlMerit (merit.rs:323-352): -((max I / sum I) / (max R / sum R)) of the
 * selected frame against d_reference (FP64, nx ny samples, the frame's
 * grid); 0 when either sum is <= 0.  No obs gradient. */
int osgpu_merit_strehl_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                              int32_t n_scenes, uint64_t nx, uint64_t ny,
                              const double* d_reference, int32_t band, int32_t scene,
                              void* stream, double* value);
/* MtfMerit (merit.rs:354-400): -|DFT_x(I)[m]| / sum I of the selected frame
 * (summed over rows) at the bin m = freq nx dx.  freq < 0, 2 freq dx >= 1
 * or m more than 1e-9 from an integer returns OSGPU_E_RENDER.  No obs
 * gradient. */
int osgpu_merit_mtf_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                           int32_t n_scenes, uint64_t nx, uint64_t ny, double dx, double freq,
                           int32_t band, int32_t scene, void* stream, double* value);

/* Adam update of fd.rs:186-257 (AdamConfig, fd.rs:63-110): optional global
 * gradient-norm clip, bias-corrected moments, x -= lr_frac (hi - lo) m^ /
 * (sqrt(v^) + eps), clamp into [lo, hi].  t >= 1 is the step number.  d_x32
 * (optional) receives a float copy of x (the f32 engine's lattice).
 * Asynchronous. */
typedef struct {
  double lr_frac, beta1, beta2, eps;
  double clip_norm; /* used when clip != 0 */
  int32_t clip;
} osgpu_adam_config;
int osgpu_adam_step_device(double* d_x, float* d_x32, const void* d_g, int32_t g_real_dtype,
                           double* d_m, double* d_v, uint64_t n, const osgpu_adam_config* cfg,
                           int32_t t, double lo, double hi, void* stream);

/* ------------------------------------------------------ Gerchberg-Saxton */
/* gs::run (optics-inverse gs.rs:347-597) on the device, batched over items.
 * Engines: OSGPU_GS_ASM_RELAY is the reference's relay (input -> ASM z/2 ->
 * DOE -> ASM z/2 -> target, back-propagation ASM -z/2, illumination
 * |ASM(input, z/2)|); OSGPU_GS_FRAUNHOFER puts the DOE at the input plane
 * (illumination |input|), propagates with fraunhofer::propagate (source_pos
 * None) and back with its exact adjoint (no reference counterpart).  The
 * merit of the stopping test is MseToTarget over the target-plane intensity
 * (merit.rs:112-146); the loop state, best-so-far phase and history stay on
 * the device.  Synchronous: results and history are on the host when the
 * call returns. */
enum { OSGPU_GS_CLASSIC = 0, OSGPU_GS_DVR = 1, OSGPU_GS_FPR = 2 }; /* GsVariant (gs.rs:125-179) */
enum { OSGPU_GS_ASM_RELAY = 0, OSGPU_GS_FRAUNHOFER = 1 };

/* GsConfig (gs.rs:197-221) plus the carrier slot bounds and the engine. */
typedef struct {
  int32_t max_iterations;
  int32_t patience;
  double merit_tolerance;
  int32_t variant;  /* OSGPU_GS_* */
  double beta;      /* Dvr / Fpr beta */
  double lo, hi;    /* carrier slot bounds (encode_bounds, gs.rs:115-121) */
  int32_t engine;   /* OSGPU_GS_ASM_RELAY / OSGPU_GS_FRAUNHOFER */
} osgpu_gs_config;

/* GsRecord (gs.rs:252-266). */
typedef struct {
  uint64_t iteration;
  double merit, best_merit, amplitude_mse, target_error_rms, phase_update_rms;
} osgpu_gs_record;

/* Scalars of GsSolution (gs.rs:268-306). */
typedef struct {
  double merit;
  uint64_t best_iteration;
  double amplitude_mse;
  int32_t converged;
  uint64_t iterations;
} osgpu_gs_result;

/* One GS problem.  Real arrays are double (OSGPU_C128) or float (OSGPU_C64). */
typedef struct {
  osgpu_grid grid;                 /* input / DOE grid and wavelength */
  double z;                        /* ASM relay: z_total; Fraunhofer: DOE -> target */
  int32_t aperture;                /* carrier aperture (OSGPU_STOP_*), centred at center_x/y */
  double aperture_a, aperture_b, center_x, center_y;
  const void* d_input;             /* complex input field */
  const void* d_target_amplitude;  /* T (target-plane layout) */
  const void* d_target_intensity;  /* MseToTarget target; NULL: T^2 */
  void* d_phase;                   /* in: initial phase (GsInit::Given); out: best phase */
  void* d_last_phase;              /* optional: phase after the last update */
  void* d_best_intensity;          /* optional: target intensity of the best iteration */
  void* d_target_error;            /* optional: |U_t| - T of the last iteration */
  void* d_phase_error;             /* optional: wrapped phase update of the last iteration */
  void* d_illumination;            /* optional: illumination amplitude at the DOE */
  osgpu_gs_record* history;        /* optional host array of max_iterations records */
  osgpu_gs_result result;          /* out */
} osgpu_gs_item;

int osgpu_gs_run_batch_device(osgpu_gs_item* items, int32_t n_items, const osgpu_gs_config* cfg,
                              const osgpu_asm_config* asm_cfg,
                              const osgpu_fraunhofer_config* fraunhofer_cfg, int32_t dtype,
                              void* stream);

/* ------------------------------------------------------- allocation-free */
/* ASM propagation that allocates no device memory, on any call.  No
 * counterpart in the reference: it exists for callers that must not have a
 * library allocate, such as applications whose device memory is owned by
 * another allocator that reserved it up front, latency-critical loops that
 * cannot absorb cudaMalloc's synchronisation, and plugins hosted by a
 * process that forbids a library from allocating.
 * d_in/d_out: caller-owned device complex64 fields (f32 engine); stream: a
 * cudaStream_t (NULL: the default stream).  All other scratch (spectrum
 * buffer, transfer-function and twiddle tables) comes from one static
 * device array of 32 MiB that every GPU loading the library holds until
 * exit; sizes needing more, or more shared memory than a block has, return
 * OSGPU_E_UNSUPPORTED before any GPU work (a 1024 x 1024 field at padding 2
 * fits, 2048 x 2048 padded to 4096 does not).  The first call on a device
 * looks up the array's address (cudaGetSymbolAddress, with that device
 * current): make it before any stream capture.  After a cudaDeviceReset,
 * call osgpu_shutdown() before the next call so the address is looked up
 * again.  Calls share the array, so calls whose GPU work overlaps race:
 * serialise them on one stream.  Input finiteness is not checked. */
int osgpu_asm_propagate_noalloc(const void* d_in, void* d_out, const osgpu_grid* g, double z,
                                const osgpu_asm_config* cfg, void* stream,
                                osgpu_asm_report* report);

/* ------------------------------------------------------------- autotuning */
/* The counterpart of the reference's FftPlanner (src/propagation/fft.rs:41,53,
 * built on every call there): a measured schedule of the f32 register-FFT
 * passes per geometry.  Each pass has interchangeable kernel variants
 * (pass A: bulk, tstore, tile4, tile2, g1, g2, g4; pass B: pair, g1, g2, g4;
 * pass C: tma, pipe, tile2, tile4, g1, g2, g4 -- row tiles, persistent
 * TMA/bulk-copy kernels, TMA tensor stores, sub-transform groups per CTA) that
 * compute the same transform.
 * osgpu_autotune_asm times a synthetic batch of the geometry (one element
 * plane, `lanes` 1: one item, 2: four items on the device batch's two lanes)
 * under each variant of pass A, then B, then C, starting from the built-in
 * defaults, and keeps the fastest; later f32 propagations of that geometry
 * (m, r per axis, nx, ny, lanes) use it.  With osgpu_autotune_config(1) the
 * device batch tunes every new geometry itself before its first run (not
 * while its stream is being captured).  Off by default: the built-in
 * defaults are used.  The environment variables OSGPU_SCHED_A / _B / _C
 * (variant names) override both. */
typedef struct {
  uint32_t mx, rx, my, ry, nx, ny, lanes;
  char pass_a[8], pass_b[8], pass_c[8];
  double ms_default; /* synthetic batch under the built-in defaults */
  double ms_best;    /* under the chosen schedule */
} osgpu_schedule_info;

int osgpu_autotune_config(int32_t enable);
int osgpu_autotune_asm(const osgpu_grid* g, double z, const osgpu_asm_config* cfg, int32_t lanes,
                       osgpu_schedule_info* out);
int osgpu_autotune_list(osgpu_schedule_info* out, int32_t max_out, int32_t* n_out);
int osgpu_autotune_clear(void);

/* --------------------------------------------------------------- profiling */
/* Per-kernel-class CUDA-event timing on the launching stream.  Between
 * osgpu_profile_begin and osgpu_profile_end every pass launch is bracketed by
 * events; _end synchronises and returns, per class, the launch count, total
 * device time and the algorithmic bytes those launches move (reads of the
 * inputs they must read + writes of their outputs).  While profiling, the
 * per-item table builds that normally overlap on an auxiliary stream run on
 * the launching stream, so every class's events time its own kernels. */
typedef struct {
  char name[32];
  uint64_t launches;
  double total_ms;
  double bytes;
} osgpu_kernel_stat;

int osgpu_profile_begin(void);
int osgpu_profile_end(osgpu_kernel_stat* out, int32_t max_out, int32_t* n_out);

/* ------------------------------------------------------- detector metrics */
/* src/analysis.rs on a device intensity grid (real, row-major ny x nx:
 * double for OSGPU_F64, float for OSGPU_F32; grid pitch dx, dy; lambda
 * unused), sums FP64-compensated, results on the host.
 *   spot_rms: sqrt(sum I rho^2 / sum I) (m), rho at the centred pixel
 *             coordinates (analysis.rs:111-124; 0 for a zero grid).
 *   mtf:      |F{I}(fx, 0)| / max(|F{I}(0, 0)|, MIN_POSITIVE), capped at 1,
 *             for fx = k / (nx dx), k = 0..nx/2: freqs and values hold
 *             nx/2 + 1 entries (analysis.rs:136-150).
 *   strehl:   (max I_m / P_m) / (max I_r / P_r), P = sum I dx dy; 0 when a
 *             power is not positive (analysis.rs:159-168).
 *   encircled_energy: the cumulative power fraction at the end of each group
 *             of equal pixel radius, radii ascending (analysis.rs:81-108);
 *             *n_out = number of points (0 for a zero grid); radii and
 *             fraction must hold cap >= *n_out entries (nx * ny always
 *             suffices).  The radius order, a function of the geometry only,
 *             is sorted on the host once per geometry; the walk itself is a
 *             gather and an FP64 prefix sum on the device.
 * marechal_strehl (a closed form of a scalar) and the curve's interpolation
 * stay in the caller's code. */
int osgpu_psf_spot_rms_device(const void* d_int, int32_t real_dtype, const osgpu_grid* g,
                              void* stream, double* out_m);
int osgpu_psf_mtf_device(const void* d_int, int32_t real_dtype, const osgpu_grid* g,
                         void* stream, double* freqs, double* values);
int osgpu_psf_encircled_energy_device(const void* d_int, int32_t real_dtype,
                                      const osgpu_grid* g, void* stream, double* radii,
                                      double* fraction, uint64_t cap, uint64_t* n_out);
int osgpu_psf_strehl_device(const void* d_meas, const osgpu_grid* g_meas, const void* d_ref,
                            const osgpu_grid* g_ref, int32_t real_dtype, void* stream,
                            double* out);

/* ------------------------------------------------- kernel-spectrum plans */
/* No counterpart in the reference (its ASM recomputes H on every call,
 * src/propagation/asm.rs:505-522).  An f32 ASM propagation whose padded grid
 * exceeds twice the field only reaches kernel offsets |d| < n, so it equals a
 * circular convolution of period 2n with the kernel h = IFFT_P(H) restricted
 * to those offsets.  With plans enabled, the first f32 ASM propagation of a
 * given (grid, pitch, wavelength, medium, |z|, padding, band limits) builds
 * that kernel's spectrum once (an FP64 propagation of a unit sample, then a
 * 2n x 2n FP64 transform, rounded to an f32 quarter table of (nx+1)(ny+1)
 * entries) and every later one, forward (+z) or adjoint (-z, the conjugate
 * table), runs at 2n instead of the padded size.  Applies to power-of-two
 * sides 256..4096 on streams that are not being captured; other calls take
 * the padded path.  Tables are evicted least recently used beyond max_bytes
 * (eviction synchronises the device).  Off by default. */
typedef struct {
  uint64_t plans;   /* tables held */
  uint64_t bytes;   /* device bytes held */
  uint64_t hits;    /* propagations that used a held table */
  uint64_t builds;  /* tables built */
} osgpu_plan_stats;

int osgpu_plan_cache_config(int32_t enable, uint64_t max_bytes);
int osgpu_plan_cache_clear(void);
int osgpu_plan_cache_stats(osgpu_plan_stats* out);

/* ---------------------------------------------------------------- runtime */
int osgpu_init(int32_t device);
/* Waits for all queued work and releases the library's cached device memory
 * (kernel-spectrum plans, the encircled-energy order, the pooled scratch).
 * Streams, twiddle tables, lattices, field handles and captured graphs stay
 * valid; later calls rebuild what they need (the plan-cache setting is
 * kept). */
int osgpu_shutdown(void);
/* Copies the last error message (NUL-terminated, truncated to len). */
int osgpu_last_error(char* buf, size_t len);
/* Waits for the library stream; returns a pending device-side status
 * (e.g. OSGPU_E_NON_FINITE_SAMPLE from an asynchronous call). */
int osgpu_sync_status(void);
const char* osgpu_version(void);
/* Number of kernel launches issued by the library since load. */
uint64_t osgpu_launch_count(void);

/* ------------------------------------------------- device-resident fields
 * For callers without a device allocator of their own (the Rust binding): a
 * handle owns the nx x ny samples of one field on the device, stored as
 * complex128 (OSGPU_C128) or complex64 (OSGPU_C64), so that a beamline's
 * planes stay on the device between the *_device calls.  Host buffers are
 * interleaved complex128 (the reference's Vec<Complex64>, field.rs:100);
 * a complex64 handle converts on the device.  Upload and download are
 * synchronous: they return when the copy is complete. */
typedef struct osgpu_field_s* osgpu_field;
/* A zero-filled field. */
int osgpu_field_create(uint64_t nx, uint64_t ny, int32_t dtype, osgpu_field* out);
int osgpu_field_upload(osgpu_field f, const double* host_c128, void* stream);
int osgpu_field_download(osgpu_field f, double* host_c128, void* stream);
/* The device buffer (d_in / d_out of the *_device entry points) and shape;
 * any output pointer may be NULL. */
int osgpu_field_info(osgpu_field f, void** d_samples, uint64_t* nx, uint64_t* ny,
                     int32_t* dtype);
/* Frees the samples after the work queued on them (NULL: no-op). */
int osgpu_field_destroy(osgpu_field f);

#ifdef __cplusplus
}
#endif
#endif /* OSGPU_H */
