// Host-side sampling / regime analysis, validation and planning.
//
// The analysis functions restate the reference's closed-form host scalars
// operation for operation (compiled with -ffp-contract=off so no multiply-add
// is fused), so the padded grid they choose and the reports they return are
// identical to the Rust ones.
#pragma once
#include <cstdint>
#include "../../include/osgpu.h"
#include "osgpu_types.h"

namespace osgpu {

uint64_t padded_len(uint64_t n, double padding);

// asm.rs:258-265
double axis_band_limit(double lam, double z, double grid_width, bool band_limited, double medium);
// asm.rs:373-412
void asm_analyze(const osgpu_grid& g, double z, const osgpu_asm_config& cfg, double padding,
                 osgpu_asm_report& r);
// asm.rs:438-479 (validation without the sample scan, densification ladder).
// Returns OSGPU_OK, an error, or -1 for the z == 0 identity.
int asm_resolve(const osgpu_grid& g, double z, const osgpu_asm_config& cfg, osgpu_asm_report& r);

// fresnel.rs:342-373
void fresnel_analyze(const osgpu_grid& g, double z, const osgpu_fresnel_config& cfg,
                     double padding, osgpu_fresnel_report& r);
int fresnel_resolve_tf(const osgpu_grid& g, double z, const osgpu_fresnel_config& cfg,
                       osgpu_fresnel_report& r);
int fresnel_resolve_conv(const osgpu_grid& g, double z, const osgpu_fresnel_config& cfg,
                         osgpu_fresnel_report& r);

// fraunhofer.rs:284-347
void fraunhofer_report(const osgpu_grid& g, double z, const osgpu_fraunhofer_config& cfg,
                       osgpu_fraunhofer_report& r);
int fraunhofer_resolve(const osgpu_grid& g, double z, const osgpu_fraunhofer_config& cfg,
                       osgpu_fraunhofer_report& r);

// rayleigh_sommerfeld.rs:304-362
void rs_analyze(const osgpu_grid& g, double z, double padding, osgpu_rs_report& r);
int rs_resolve(const osgpu_grid& g, double z, const osgpu_rs_config& cfg, osgpu_rs_report& r);

// Sub-FFT plan for one axis: m = smallest divisor of P with m >= n.
AxisPlan make_axis(int n, int P);

// Element validation (constructor + apply-time checks of element.rs) and
// conversion to the device form (lattice pointer filled by the caller).
int element_check(const osgpu_element& e, const osgpu_grid& g, double lambda, DevElement& out,
                  char* msg, size_t msglen);

// f32 transfer-function mode: 1 when the split-phase tables meet the error
// budget for this geometry, else 0 (per-bin FP64 phase).
int asm_f32_split_ok(const osgpu_grid& g, double z, double medium, uint64_t Px, uint64_t Py,
                     bool band_limited, double lim_x, double lim_y);

}  // namespace osgpu
