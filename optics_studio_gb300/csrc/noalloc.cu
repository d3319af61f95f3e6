// Allocation-free ASM propagation (osgpu_asm_propagate_noalloc).
//
// Some callers cannot let a library allocate device memory: applications
// whose device memory is owned by another allocator that reserved it up
// front (a framework's caching pool, a real-time pipeline), where an extra
// cudaMalloc can fail or fragment memory at an unpredictable moment;
// latency-critical loops that cannot absorb the implicit synchronisation of
// cudaMalloc/cudaFree; and plugins hosted by a process whose rules forbid a
// library from allocating on its own.  This entry point serves them: the
// caller passes the input and output buffers, and every other byte the
// propagation needs (the column-major spectrum buffer, the per-axis
// transfer-function tables and the twiddle tables) is carved from one
// file-scope device array of kScratchBytes.  It calls no cudaMalloc,
// cudaFree or allocating library routine, on the first call or any other.
//
// Properties a caller must know:
//  * Every GPU that loads the library holds the array (kScratchBytes) until
//    the process exits.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress, with that device current, and caches it; make
//    that first call before any stream capture.  Later calls do no set-up.
//    A cudaDeviceReset invalidates the cached address: call osgpu_shutdown()
//    after a reset (it forgets the addresses), and the next call looks the
//    array up again.
//  * All calls share the array, which keeps the last call's contents.  Each
//    call rewrites every scratch entry it reads before reading it (twiddle
//    tables, per-axis tables, the full spectrum buffer), so nothing has to
//    start at zero.  Calls whose GPU work overlaps (different streams, or
//    different host threads on one device) race on the array: serialise
//    them on one stream.
//  * Sizes whose scratch exceeds kScratchBytes (32 MiB: for example a
//    1024 x 1024 field at the default padding of 2, which needs 17 MB, fits;
//    a 2048 x 2048 field padded to 4096 x 4096 does not), or whose passes
//    exceed the per-block shared memory, are rejected with
//    OSGPU_E_UNSUPPORTED before any GPU work; osgpu_last_error says which.
//  * Input samples are not checked for finiteness (the caller owns that).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/osgpu.h"
#include "host_analysis.h"
#include "prop_kernels.cuh"

using namespace osgpu;

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;  // 32 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// Device address of the scratch array on `dev` (which is current).  In host
// code the name g_noalloc_scratch is only a host-side stand-in for the
// array, so kernels get the address looked up here.
cudaError_t scratch_address(int dev, void** out) {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

const double PI = 3.14159265358979323846;

}  // namespace

void osgpu::noalloc_forget_scratch() {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  for (void*& p : g_scratch_addr) p = nullptr;
}

extern "C" int osgpu_asm_propagate_noalloc(const void* d_in, void* d_out, const osgpu_grid* g,
                                           double z, const osgpu_asm_config* cfg, void* stream,
                                           osgpu_asm_report* report) {
  if (!g || !cfg || !d_in || !d_out) {
    set_last_error("noalloc ASM: null grid, config or field pointer");
    return OSGPU_E_BAD_ARGUMENT;
  }
  osgpu_asm_report r;
  int rc = asm_resolve(*g, z, *cfg, r);
  if (report) *report = r;
  if (rc > 0) {
    set_last_error("noalloc ASM: invalid propagation arguments or sampling (status %d)", rc);
    return rc;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const size_t nfield = g->nx * g->ny;
  if (rc == -1) {  // z == 0: identity
    if (d_out == d_in) return OSGPU_OK;
    const cudaError_t ce =
        cudaMemcpyAsync(d_out, d_in, nfield * sizeof(float2), cudaMemcpyDeviceToDevice, st);
    if (ce != cudaSuccess) {
      set_last_error("noalloc ASM: identity copy: %s", cudaGetErrorString(ce));
      return OSGPU_E_CUDA;
    }
    return OSGPU_OK;
  }
  const int nx = (int)g->nx, ny = (int)g->ny;
  const size_t Px = r.nx_pad, Py = r.ny_pad;
  PropArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nx = nx;
  a.ny = ny;
  a.dx = g->dx;
  a.dy = g->dy;
  a.ax = make_axis(nx, (int)Px);
  a.ay = make_axis(ny, (int)Py);
  const size_t kSmem = 232448;  // sm_103a opt-in shared memory per block
  if (a.ax.nst < 0 || a.ay.nst < 0 || !prop_smem_fits(a.ax, a.ay, 0, kSmem)) {
    set_last_error("noalloc ASM: grid %dx%d padded to %zux%zu exceeds the shared-memory plan",
                   nx, ny, Px, Py);
    return OSGPU_E_UNSUPPORTED;
  }
  // Scratch layout (all complex64 / f32 except the f64 frequency axes).
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    const size_t o = off;
    off += al(bytes);
    return o;
  };
  // m-point tables carry their stage-ordered copy behind them (2 m entries)
  const size_t o_twmx = carve((size_t)a.ax.m * 16), o_twPx = carve(Px * 8);
  const size_t o_twmy = carve((size_t)a.ay.m * 16), o_twPy = carve(Py * 8);
  const size_t o_work = carve(Px * (size_t)ny * 8);
  const size_t o_fxv = carve(Px * 8), o_fyv = carve(Py * 8);
  const size_t o_Ex = carve(Px * 8), o_Ey = carve(Py * 8);
  const size_t o_cah = carve(Px * 4), o_cal = carve(Px * 4), o_sa = carve(Px * 4);
  const size_t o_bh = carve(Py * 4), o_bl = carve(Py * 4), o_km = carve(Px * 4);
  const size_t o_rt = carve(Py * 16);
  if (off > kScratchBytes) {
    set_last_error("noalloc ASM: scratch of %zu bytes exceeds the static %zu MiB", off,
                   kScratchBytes >> 20);
    return OSGPU_E_UNSUPPORTED;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_last_error("noalloc ASM: no usable current CUDA device");
    return OSGPU_E_NO_DEVICE;
  }
  void* sp = nullptr;
  cudaError_t e = scratch_address(dev, &sp);
  if (e != cudaSuccess) {
    set_last_error("noalloc ASM: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    return OSGPU_E_CUDA;
  }
  char* base = reinterpret_cast<char*>(sp);
  a.tw_mx = base + o_twmx;
  a.tw_Px = base + o_twPx;
  a.tw_my = base + o_twmy;
  a.tw_Py = base + o_twPy;
  if ((e = launch_twiddles(base + o_twmx, a.ax.m, 0, st)) != cudaSuccess ||
      (e = launch_twiddles(base + o_twPx, (int)Px, 0, st)) != cudaSuccess ||
      (e = launch_twiddles(base + o_twmy, a.ay.m, 0, st)) != cudaSuccess ||
      (e = launch_twiddles(base + o_twPy, (int)Py, 0, st)) != cudaSuccess ||
      (reg_fft_size(a.ax.m) && (e = launch_stage_twiddles(base + o_twmx, a.ax.m, st)) != cudaSuccess) ||
      (reg_fft_size(a.ay.m) && (e = launch_stage_twiddles(base + o_twmy, a.ay.m, st)) != cudaSuccess)) {
    set_last_error("noalloc ASM: twiddle tables: %s", cudaGetErrorString(e));
    return OSGPU_E_CUDA;
  }
  a.in = d_in;
  a.in_c128 = 0;
  a.out = d_out;
  a.out_c128 = 0;
  a.work = base + o_work;
  a.engine = ENG_ASM;
  a.lam = g->lambda;
  a.z = z;
  a.scale = 1.0 / ((double)Px * (double)Py);
  const double lam_n = g->lambda / cfg->medium;
  a.lam_n = lam_n;
  a.kz = (2.0 * PI / lam_n) * z;
  a.band_limited = cfg->band_limited;
  a.lim_x = r.band_limit_fx;
  a.lim_y = r.band_limit_fy;
  a.h_mode = asm_f32_split_ok(*g, z, cfg->medium, Px, Py, cfg->band_limited != 0,
                              r.band_limit_fx, r.band_limit_fy);
  a.Kf = (float)a.kz;
  a.fxv = reinterpret_cast<const double*>(base + o_fxv);
  a.fyv = reinterpret_cast<const double*>(base + o_fyv);
  a.Ex = reinterpret_cast<const float2*>(base + o_Ex);
  a.Ey = reinterpret_cast<const float2*>(base + o_Ey);
  a.ca_hi = reinterpret_cast<const float*>(base + o_cah);
  a.ca_lo = reinterpret_cast<const float*>(base + o_cal);
  a.sa = reinterpret_cast<const float*>(base + o_sa);
  a.b_hi = reinterpret_cast<const float*>(base + o_bh);
  a.b_lo = reinterpret_cast<const float*>(base + o_bl);
  a.kmax = reinterpret_cast<const int*>(base + o_km);
  a.rowtab = base + o_rt;
  a.status = nullptr;
  if ((e = launch_asm_prep<float>(a, nullptr, st)) != cudaSuccess ||
      (e = launch_passA<float>(a, st)) != cudaSuccess ||
      (e = launch_passB<float>(a, st)) != cudaSuccess ||
      (e = launch_passC<float>(a, st)) != cudaSuccess) {
    set_last_error("noalloc ASM: pass launch: %s", cudaGetErrorString(e));
    return OSGPU_E_CUDA;
  }
  return OSGPU_OK;
}
