// C ABI (include/osgpu.h) over the sm_103a propagation kernels.
//
// Host control flow per call: reference-identical validation and sampling
// analysis (host_analysis.cpp) -> device plan (axis plans, twiddle tables,
// workspace) -> kernels on the library stream.  The sample finiteness scan
// that the reference runs on the CPU before propagating
// (src/propagation/asm.rs:458) is folded into the first pass on the GPU;
// only on an error path that the reference would rank after it does the
// host scan the input itself.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <array>
#include <map>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include "../../include/osgpu.h"
#include "host_analysis.h"
#include "gs_fast.cuh"
#include "inverse_kernels.cuh"
#include "prop_kernels.cuh"

using namespace osgpu;

namespace {

const double PI = 3.14159265358979323846;
const size_t kMaxSmem = 232448;  // sm_103a opt-in shared memory per block

thread_local char t_err[1024] = "";

void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
}

// Per-kernel-class event timing (osgpu_profile_begin/end).
struct ProfRec {
  int cls;
  cudaEvent_t a, b;
  double bytes;
};
enum { PC_PREP = 0, PC_ELEMENTS, PC_APPLY, PC_PASS_A, PC_PASS_B, PC_PASS_C, PC_KSPEC, PC_FRAUN,
       PC_GS, PC_GS_COLS, PC_GS_ROWS, PC_FFT2, PC_PLAN, PC_N };
const char* kProfNames[PC_N] = {"prep_tables", "element_tables", "element_apply",
                                "pass_a_rows", "pass_b_columns", "pass_c_rows",
                                "kernel_spectrum", "fraunhofer", "gs_planes", "gs_columns",
                                "gs_rows", "fft2", "plan_build"};

// Kernel-spectrum plan of an f32 ASM propagation whose padded grid exceeds
// twice the field (prop_kernels.cu, launch_even_kspec): keyed by everything
// that determines H and the padding; |z| (the plan of -z is the conjugate).
struct KPlan {
  uint64_t nx, ny, Px, Py;
  double dx, dy, lam, medium, zabs, lim_x, lim_y;
  int band_limited;
  void* kq = nullptr;  // f32 quarter table, (nx + 1) x (ny + 1)
  size_t bytes = 0;
  uint64_t last_use = 0;
};

struct Context {
  std::recursive_mutex mu;
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_in = nullptr, copy_out = nullptr;  // host-buffer batch pipeline
  cudaStream_t aux = nullptr;  // element tables of the next batch item
  cudaStream_t lane2 = nullptr, aux2 = nullptr;  // second lane of the device batch
  int* d_status = nullptr;
  std::map<std::pair<int, int>, void*> tw;  // (n, is_double) -> twiddle table
  bool profiling = false;
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> event_pool;
  std::map<const void*, float*> lattices;  // osgpu_lattice_create handle -> f32 copy
  // encircled-energy walk order of the last detector geometry (radius sort on the host)
  struct EeOrder {
    uint64_t nx = 0, ny = 0;
    double dx = 0.0, dy = 0.0;
    std::vector<double> radii;  // one per tied-radius group, ascending
    void* d = nullptr;          // device: perm (n u32) then group ends (ng u32)
    uint64_t ng = 0;
  } ee;
  // kernel-spectrum plans (osgpu_plan_cache_config); off by default
  bool plans_on = false;
  size_t plan_cap = 0, plan_bytes = 0;
  uint64_t plan_tick = 0, plan_hits = 0, plan_builds = 0;
  std::vector<KPlan> plans;
  // measured schedules of the f32 register-FFT passes (osgpu_autotune_*),
  // keyed by (m_x, r_x, m_y, r_y, nx, ny, lanes); off by default
  struct Tuned {
    Schedule s;
    double ms_default, ms_best;
  };
  bool autotune = false;
  bool tuning = false;    // a tuning run is in progress (its batches do not tune)
  bool force_on = false;  // the tuner's forced schedule
  Schedule force = {0, 0, 0};
  int lane_mode = 1;      // lanes of the batch being run
  std::map<std::array<int, 7>, Tuned> tuned;
  uint64_t tunes = 0;
  // pinned copies of the fused GS loop state (two chunks) and their events,
  // kept between calls: a pinned allocation and free per call (the free
  // synchronises the device) cost more than the loop's own host work
  GsState* gs_pin = nullptr;
  size_t gs_pin_bytes = 0;
  cudaEvent_t gs_ev[2] = {nullptr, nullptr};
};

Context& ctx() {
  static Context c;
  return c;
}

int cuda_fail(cudaError_t e, const char* where) {
  set_err("%s: %s", where, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? OSGPU_E_OUT_OF_MEMORY : OSGPU_E_CUDA;
}

#define CK(call)                                        \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

int ensure_init(Context& c) {
  if (c.device >= 0) return OSGPU_OK;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    set_err("no CUDA device visible");
    return OSGPU_E_NO_DEVICE;
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaSetDevice(dev));
  CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  CK(cudaMalloc(&c.d_status, sizeof(int)));
  CK(cudaMemset(c.d_status, 0, sizeof(int)));
  cudaMemPool_t pool;
  CK(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t thr = UINT64_MAX;
  CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  c.device = dev;
  return OSGPU_OK;
}

// Stream-ordered device buffer (pool allocator; freed at scope exit).
struct DBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), s(o.s) { o.p = nullptr; }
  ~DBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  cudaError_t alloc(size_t bytes, cudaStream_t st) {
    s = st;
    return cudaMallocAsync(&p, bytes ? bytes : 16, st);
  }
};

cudaEvent_t pool_event(Context& c) {
  if (!c.event_pool.empty()) {
    cudaEvent_t e = c.event_pool.back();
    c.event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets one launch group with events when profiling.
struct ProfScope {
  Context& c;
  cudaStream_t st;
  int cls;
  double bytes;
  cudaEvent_t a = nullptr;
  ProfScope(Context& c_, cudaStream_t st_, int cls_, double bytes_)
      : c(c_), st(st_), cls(cls_), bytes(bytes_) {
    if (c.profiling) {
      a = pool_event(c);
      cudaEventRecord(a, st);
    }
  }
  ~ProfScope() {
    if (c.profiling && a) {
      cudaEvent_t b = pool_event(c);
      cudaEventRecord(b, st);
      c.prof.push_back(ProfRec{cls, a, b, bytes});
    }
  }
};

// Twiddle tables are cached per (n, precision) and shared by every stream:
// the first build is synchronised so later users on any stream see it.
int get_tw(Context& c, int n, int is_d, const void** out) {
  auto key = std::make_pair(n, is_d);
  auto it = c.tw.find(key);
  if (it != c.tw.end()) {
    *out = it->second;
    return OSGPU_OK;
  }
  void* p = nullptr;
  const bool staged = !is_d && reg_fft_size(n);  // + stage-ordered copy behind it
  CK(cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * (is_d ? 16 : 8) * (staged ? 2 : 1)));
  CK(launch_twiddles(p, n, is_d, c.stream));
  if (staged) CK(launch_stage_twiddles(p, n, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  c.tw[key] = p;
  *out = p;
  return OSGPU_OK;
}

// Device element list + uploaded lattices and fast tables (kept alive for
// the call; freed stream-ordered).
struct Elements {
  ElementList list;
  std::vector<DBuf> lattices;
  DBuf tables;
  DBuf prop_tables;  // per-axis tables of the propagation after this step (prebuild_tables)
  DBuf trans;        // f32: transmission of the element chain in front of that propagation
};

// Element tables (and per-axis propagation tables and chain transmissions)
// of the next batch item / frame are built on the auxiliary stream while the
// previous one runs on the compute stream.  fork() makes the auxiliary
// stream follow the compute stream's work so far; ready() makes the compute
// stream wait for the tables built so far (the one in finish() also joins the
// auxiliary stream back, as graph capture requires).  An item's buffers are
// allocated and freed on the auxiliary stream, so the pool reuses them in
// stream order: take() hands them over for the item's passes, end() marks
// the passes queued, and begin() of the item after next frees them once that
// item has completed on the compute stream (two generations in flight keep
// the tables of item i + 1 building while item i runs).  The destructor
// covers early returns: it waits for everything queued so far.
struct AuxTables {
  cudaStream_t st = nullptr, ax = nullptr;
  cudaEvent_t ev = nullptr, e0 = nullptr, e1 = nullptr;
  std::vector<Elements> cur, gen0, gen1;
  bool joined = false;
  // `second`: the auxiliary stream of the device batch's second lane
  int fork(Context& c, cudaStream_t compute, bool second = false);
  int ready() {
    CK(cudaEventRecord(ev, ax));
    CK(cudaStreamWaitEvent(st, ev, 0));
    return OSGPU_OK;
  }
  int begin() {
    if (!e0) return OSGPU_OK;
    CK(cudaStreamWaitEvent(ax, e0, 0));
    gen0.clear();
    cudaEventDestroy(e0);
    e0 = nullptr;
    return OSGPU_OK;
  }
  std::vector<Elements>& take(std::vector<Elements>& E) {
    cur = std::move(E);
    return cur;
  }
  int end() {
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(cudaEventRecord(e, st));
    if (e0) {  // begin() was skipped: keep the order of the frees
      CK(cudaStreamWaitEvent(ax, e0, 0));
      gen0.clear();
      cudaEventDestroy(e0);
    }
    gen0 = std::move(gen1);
    e0 = e1;
    gen1 = std::move(cur);
    e1 = e;
    cur.clear();
    return OSGPU_OK;
  }
  int finish() {
    int rc;
    if ((rc = begin())) return rc;
    if (e1) {
      CK(cudaStreamWaitEvent(ax, e1, 0));
      gen1.clear();
      cudaEventDestroy(e1);
      e1 = nullptr;
    }
    if ((rc = ready())) return rc;
    joined = true;
    return OSGPU_OK;
  }
  ~AuxTables() {
    if (ev && ax && !joined) {  // early return: free only after what was queued on st
      cudaEventRecord(ev, st);
      cudaStreamWaitEvent(ax, ev, 0);
    }
    cur.clear();
    gen0.clear();
    gen1.clear();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (ev) cudaEventDestroy(ev);
  }
};

int AuxTables::fork(Context& c, cudaStream_t compute, bool second) {
  cudaStream_t& own = second ? c.aux2 : c.aux;
  if (!own) CK(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
  st = compute;
  // While profiling, the table builds run on the compute stream: events on
  // an overlapped auxiliary stream would time its waits for free SMs, not
  // the kernels.
  ax = c.profiling ? compute : own;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(cudaEventRecord(ev, st));
  CK(cudaStreamWaitEvent(ax, ev, 0));
  return OSGPU_OK;
}

// Two lanes for a batch of independent items: the caller's stream and a
// second stream forked from it (joined back by join()), each with its own
// auxiliary stream for the per-item tables.  Item i runs on lane i % n, so one
// item's passes fill the SMs another's leave idle at the ends of their
// grids.  One lane for a single item, while profiling (per-kernel events) or
// with OSGPU_LANES=1.
struct Lanes {
  int n = 1;
  cudaStream_t ls[2] = {nullptr, nullptr};
  AuxTables aux[2];
  bool forked = false;
  static int want(const Context& c, int n_items) {
    const char* e = getenv("OSGPU_LANES");
    return (n_items > 1 && !c.profiling && !(e && atoi(e) == 1)) ? 2 : 1;
  }
  int fork(Context& c, cudaStream_t st, int lanes) {
    n = lanes;
    ls[0] = st;
    if (n == 2) {
      if (!c.lane2) CK(cudaStreamCreateWithFlags(&c.lane2, cudaStreamNonBlocking));
      ls[1] = c.lane2;
      cudaEvent_t fk = nullptr;
      CK(cudaEventCreateWithFlags(&fk, cudaEventDisableTiming));
      CK(cudaEventRecord(fk, st));
      CK(cudaStreamWaitEvent(ls[1], fk, 0));
      cudaEventDestroy(fk);
      forked = true;
    }
    int rc;
    for (int l = 0; l < n; ++l)
      if ((rc = aux[l].fork(c, ls[l], l == 1))) return rc;
    return OSGPU_OK;
  }
  int finish() {
    int rc;
    for (int l = n - 1; l >= 0; --l)
      if ((rc = aux[l].finish())) return rc;
    return OSGPU_OK;
  }
  // the second lane's work joins the caller's stream (also on error paths)
  void join() {
    if (!forked) return;
    cudaEvent_t jn = nullptr;
    if (cudaEventCreateWithFlags(&jn, cudaEventDisableTiming) == cudaSuccess) {
      cudaEventRecord(jn, ls[1]);
      cudaStreamWaitEvent(ls[0], jn, 0);
      cudaEventDestroy(jn);
    }
    forked = false;
  }
  ~Lanes() { join(); }
};

int build_elements(Context& c, const osgpu_element* els, int n, const osgpu_grid& g,
                   Elements& E, cudaStream_t st) {
  std::memset(&E.list, 0, sizeof(E.list));
  if (n < 0 || (n > 0 && els == nullptr)) {
    set_err("bad element list");
    return OSGPU_E_BAD_ARGUMENT;
  }
  if (n > kMaxElements) {
    set_err("at most %d elements per plane", kMaxElements);
    return OSGPU_E_UNSUPPORTED;
  }
  for (int i = 0; i < n; ++i) {
    DevElement d;
    char msg[512] = "";
    int est = element_check(els[i], g, g.lambda, d, msg, sizeof(msg));
    if (est) {
      set_err("element %d: %s (status %d)", i, msg, est);
      return est;
    }
    const bool lat_el = els[i].kind == OSGPU_EL_PHASE_MASK_SAMPLED ||
                        els[i].kind == OSGPU_EL_GRID_SCREEN;
    if (lat_el && els[i].lattice_on_device == 2) {
      d.lat = nullptr;  // f32 engine only (checked in prepare_trace)
      d.latf = reinterpret_cast<const float*>(els[i].lattice);
    } else if (lat_el && els[i].lattice_on_device) {
      d.lat = reinterpret_cast<const double*>(els[i].lattice);
    } else if (lat_el) {
      const size_t bytes = (size_t)els[i].lnx * els[i].lny * sizeof(double);
      DBuf b;
      CK(b.alloc(bytes, st));
      CK(cudaMemcpyAsync(b.p, els[i].lattice, bytes, cudaMemcpyHostToDevice, st));
      d.lat = reinterpret_cast<const double*>(b.p);
      E.lattices.push_back(std::move(b));
    }
    E.list.el[E.list.count++] = d;
  }
  return OSGPU_OK;
}

// f32 engine: build the FP64-derived fast tables of every element of `L`
// for grid `g`; L.fast = 1 when all elements qualify (orientation 0).
int build_fast_tables(Context& c, ElementList& L, const osgpu_grid& g, DBuf& keep,
                      cudaStream_t st) {
  L.fast = 0;
  if (L.count == 0) return OSGPU_OK;
  size_t bytes = 0;
  for (int q = 0; q < L.count; ++q) {
    if (L.el[q].psi != 0.0) {
      if ((L.el[q].kind == EL_PHASE || L.el[q].kind == EL_SCREEN) && !L.el[q].lat) {
        set_err("an f32 device lattice needs orientation 0");
        return OSGPU_E_UNSUPPORTED;
      }
      return OSGPU_OK;
    }
    bytes += element_tables_bytes(L.el[q], (int)g.nx, (int)g.ny);
  }
  CK(keep.alloc(bytes, st));
  ProfScope ps(c, st, PC_ELEMENTS, 0.0);
  char* p = reinterpret_cast<char*>(keep.p);
  for (int q = 0; q < L.count; ++q) {
    DevElement& e = L.el[q];
    const bool lat_el = (e.kind == EL_PHASE || e.kind == EL_SCREEN);
    if (!(lat_el && e.latf && !e.lat)) {  // not a caller-owned f32 lattice
      auto hit = c.lattices.find(e.lat);
      e.latf = (lat_el && hit != c.lattices.end()) ? hit->second : nullptr;
    }
    CK(launch_element_tables(e, (int)g.nx, (int)g.ny, g.dx, g.dy, p, st));
    p += element_tables_bytes(e, (int)g.nx, (int)g.ny);
  }
  L.fast = 1;
  return OSGPU_OK;
}

// Algorithmic bytes of the lattice reads of one plane's elements.
double element_bytes(const ElementList& L, int f32) {
  double b = 0;
  for (int q = 0; q < L.count; ++q)
    if (L.el[q].kind == EL_PHASE || L.el[q].kind == EL_SCREEN)
      b += (double)L.el[q].lnx * L.el[q].lny * (f32 ? 4 : 8);
  return b;
}

bool host_all_finite(const double* p, size_t n_doubles) {
  for (size_t i = 0; i < n_doubles; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

struct PropJob {
  int engine;
  osgpu_grid g;
  double z;
  uint64_t Px, Py;
  double medium;
  int band_limited;
  double lim_x, lim_y;
  ElementList els;
  const void* d_in;
  int in_c128;
  void* d_out;
  int out_c128;
  float* d_int;
  double* d_int64;
  int conj_h;
  // adjoint hooks (PropArgs::seed*, adj*)
  const void* seed;
  int seed_f64;
  double seed_scale;
  int adj;
  const void* adj_uin;
  int adj_uin_c128;
  void* adj_grad[kMaxElements];
  const void* kspec_ext;  // ENG_KEVEN: the plan's quarter table
  const void* tables_pre;  // ASM / Fresnel TF: per-axis tables already built (prebuild_tables)
  const float2* trans;     // f32: precomputed transmission of els (prepare_trace)
};

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <typename T>
int run_prop(Context& c, const PropJob& j, cudaStream_t st);

// Per-axis transfer-function tables of an ASM / Fresnel TF propagation
// (k_axis_prep): byte offsets within one allocation.
struct TfLayout {
  size_t fxv, fyv, Ex, Ey, cah, cal, sa, bh, bl, km, rt, total;
};

TfLayout tf_layout(size_t Px, size_t Py) {
  TfLayout L;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off += align256(bytes);
    return o;
  };
  L.fxv = carve(Px * 8);
  L.fyv = carve(Py * 8);
  L.Ex = carve(Px * 8);
  L.Ey = carve(Py * 8);
  L.cah = carve(Px * 4);
  L.cal = carve(Px * 4);
  L.sa = carve(Px * 4);
  L.bh = carve(Py * 4);
  L.bl = carve(Py * 4);
  L.km = carve(Px * 4);
  L.rt = carve(Py * 16);
  L.total = off;
  return L;
}

void tf_bind(PropArgs& a, char* tb, const TfLayout& L) {
  a.fxv = reinterpret_cast<const double*>(tb + L.fxv);
  a.fyv = reinterpret_cast<const double*>(tb + L.fyv);
  a.Ex = reinterpret_cast<const float2*>(tb + L.Ex);
  a.Ey = reinterpret_cast<const float2*>(tb + L.Ey);
  a.ca_hi = reinterpret_cast<const float*>(tb + L.cah);
  a.ca_lo = reinterpret_cast<const float*>(tb + L.cal);
  a.sa = reinterpret_cast<const float*>(tb + L.sa);
  a.b_hi = reinterpret_cast<const float*>(tb + L.bh);
  a.b_lo = reinterpret_cast<const float*>(tb + L.bl);
  a.kmax = reinterpret_cast<const int*>(tb + L.km);
  a.rowtab = tb + L.rt;
}

// Scalars of the transfer function shared by k_axis_prep and pass B.
void tf_scalars(PropArgs& a, const PropJob& j, int is_d) {
  if (j.engine == ENG_ASM) {
    const double lam_n = j.g.lambda / j.medium;
    a.lam_n = lam_n;
    a.kz = (2.0 * PI / lam_n) * j.z;
    a.band_limited = j.band_limited;
    a.lim_x = j.lim_x;
    a.lim_y = j.lim_y;
    a.h_mode = is_d ? 0
                    : asm_f32_split_ok(j.g, j.z, j.medium, j.Px, j.Py, j.band_limited != 0,
                                       j.lim_x, j.lim_y);
  } else {
    a.kz = (2.0 * PI / j.g.lambda) * j.z;
    a.cfr = PI * j.g.lambda * j.z;
    a.h_mode = is_d ? 0 : 1;
  }
  a.Kf = (float)a.kz;
}

// Builds the per-axis tables of propagation j on stream st into `keep`
// (prepare_trace: on the auxiliary stream, ahead of the item's passes).
// Leaves `keep` empty when the job has no such tables or will take a
// kernel-spectrum plan.
int prebuild_tables(Context& c, const PropJob& j, int is_d, DBuf& keep, cudaStream_t st) {
  if (j.engine != ENG_ASM && j.engine != ENG_FRESNEL_TF) return OSGPU_OK;
  if (!is_d && c.plans_on && j.engine == ENG_ASM &&
      (j.Px > 2 * j.g.nx || j.Py > 2 * j.g.ny))
    return OSGPU_OK;
  PropArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nx = (int)j.g.nx;
  a.ny = (int)j.g.ny;
  a.dx = j.g.dx;
  a.dy = j.g.dy;
  a.ax = make_axis(a.nx, (int)j.Px);
  a.ay = make_axis(a.ny, (int)j.Py);
  if (a.ax.nst < 0 || a.ay.nst < 0) return OSGPU_OK;  // run_prop reports it
  a.engine = j.engine;
  a.lam = j.g.lambda;
  a.z = j.z;
  a.scale = 1.0 / ((double)j.Px * (double)j.Py);
  tf_scalars(a, j, is_d);
  const TfLayout L = tf_layout(j.Px, j.Py);
  CK(keep.alloc(L.total, st));
  tf_bind(a, reinterpret_cast<char*>(keep.p), L);
  ProfScope ps(c, st, PC_PREP, 0.0);
  CK(is_d ? launch_asm_prep<double>(a, nullptr, st) : launch_asm_prep<float>(a, nullptr, st));
  return OSGPU_OK;
}

__global__ void k_unit_sample(double2* p) { *p = make_double2(1.0, 0.0); }

}  // namespace
namespace osgpu {
unsigned long long& launch_counter();
}
namespace {

// Quarter table of the kernel-spectrum plan for the f32 ASM job j, built on
// first use: the FP64 propagation of a unit sample at the origin gives the
// kernel quadrant h(y, x) on the field grid, whose even 2n-periodic extension
// is transformed (launch_even_kspec).  *kq stays null when no plan applies:
// plans off, padding at most 2n, a grid outside the register-FFT lengths,
// a stream being captured, or a table larger than the cache.
int plan_lookup(Context& c, const PropJob& j, cudaStream_t st, const void** kq) {
  *kq = nullptr;
  if (!c.plans_on || j.engine != ENG_ASM) return OSGPU_OK;
  const uint64_t nx = j.g.nx, ny = j.g.ny;
  if (j.Px <= 2 * nx && j.Py <= 2 * ny) return OSGPU_OK;
  if (!reg_fft_size((int)nx) || !reg_fft_size((int)ny)) return OSGPU_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
    return OSGPU_OK;
  const double zabs = std::fabs(j.z);
  for (KPlan& p : c.plans) {
    if (p.nx == nx && p.ny == ny && p.Px == j.Px && p.Py == j.Py && p.dx == j.g.dx &&
        p.dy == j.g.dy && p.lam == j.g.lambda && p.medium == j.medium && p.zabs == zabs &&
        p.band_limited == j.band_limited && p.lim_x == j.lim_x && p.lim_y == j.lim_y) {
      p.last_use = ++c.plan_tick;
      ++c.plan_hits;
      *kq = p.kq;
      return OSGPU_OK;
    }
  }
  const size_t qbytes = (size_t)(nx + 1) * (ny + 1) * sizeof(float2);
  if (qbytes > c.plan_cap) return OSGPU_OK;
  if (c.plan_bytes + qbytes > c.plan_cap) {
    CK(cudaDeviceSynchronize());  // evicted tables may still be read by queued work
    while (c.plan_bytes + qbytes > c.plan_cap && !c.plans.empty()) {
      auto lru = std::min_element(c.plans.begin(), c.plans.end(),
                                  [](const KPlan& a, const KPlan& b) { return a.last_use < b.last_use; });
      cudaFree(lru->kq);
      c.plan_bytes -= lru->bytes;
      c.plans.erase(lru);
    }
  }
  KPlan p;
  p.nx = nx; p.ny = ny; p.Px = j.Px; p.Py = j.Py;
  p.dx = j.g.dx; p.dy = j.g.dy; p.lam = j.g.lambda; p.medium = j.medium; p.zabs = zabs;
  p.lim_x = j.lim_x; p.lim_y = j.lim_y; p.band_limited = j.band_limited;
  p.bytes = qbytes;
  CK(cudaMalloc(&p.kq, qbytes));
  int rc = OSGPU_OK;
  const bool prof = c.profiling;
  {
    ProfScope ps(c, st, PC_PLAN, 0.0);
    c.profiling = false;  // the build's own passes are not counted as propagation passes
    const size_t n = (size_t)nx * ny;
    DBuf tmp;
    cudaError_t e = tmp.alloc(2 * n * sizeof(double2), st);
    double2* delta = reinterpret_cast<double2*>(tmp.p);
    double2* hq = delta + n;
    if (e == cudaSuccess) e = cudaMemsetAsync(delta, 0, n * sizeof(double2), st);
    if (e == cudaSuccess) {
      k_unit_sample<<<1, 1, 0, st>>>(delta);
      ++launch_counter();
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "plan build");
    } else {
      PropJob jd;
      std::memset(&jd, 0, sizeof(jd));
      jd.engine = ENG_ASM;
      jd.g = j.g;
      jd.z = zabs;
      jd.Px = j.Px;
      jd.Py = j.Py;
      jd.medium = j.medium;
      jd.band_limited = j.band_limited;
      jd.lim_x = j.lim_x;
      jd.lim_y = j.lim_y;
      jd.d_in = delta;
      jd.in_c128 = 1;
      jd.d_out = hq;
      jd.out_c128 = 1;
      // the kernel quadrant from the f32 engine on the padded path (its
      // rounding, ~3e-7 of the kernel, stays far inside the f32 bound of the
      // propagations that use the table); the fold below runs in FP64
      c.plans_on = false;
      rc = run_prop<float>(c, jd, st);
      c.plans_on = true;
    }
    if (rc == OSGPU_OK) {
      PropArgs b;
      std::memset(&b, 0, sizeof(b));
      const int Qx = (int)(2 * nx), Qy = (int)(2 * ny);
      b.dx = j.g.dx;
      b.dy = j.g.dy;
      b.ax = make_axis((int)nx, Qx);
      b.ay = make_axis((int)ny, Qy);
      b.scale = 1.0 / ((double)Qx * (double)Qy);
      if (b.ax.nst < 0 || b.ay.nst < 0 || smem_passA_bytes(b.ax, 1, 1) > kMaxSmem ||
          smem_passB_bytes(b.ay, 1) > kMaxSmem) {
        set_err("kernel-spectrum plan of %dx%d exceeds the shared-memory plan", Qx, Qy);
        rc = OSGPU_E_UNSUPPORTED;
      } else if ((rc = get_tw(c, b.ax.m, 1, &b.tw_mx)) == OSGPU_OK &&
                 (rc = get_tw(c, b.ay.m, 1, &b.tw_my)) == OSGPU_OK &&
                 (rc = get_tw(c, Qx, 1, &b.tw_Px)) == OSGPU_OK &&
                 (rc = get_tw(c, Qy, 1, &b.tw_Py)) == OSGPU_OK) {
        DBuf tmp2;
        cudaError_t e = tmp2.alloc(((size_t)Qx * ny + (size_t)Qx * Qy) * sizeof(double2), st);
        if (e == cudaSuccess) e = launch_even_kspec(b, hq, (int)nx, (int)ny, p.kq, tmp2.p, st);
        if (e != cudaSuccess) rc = cuda_fail(e, "plan build");
      }
    }
    c.profiling = prof;
  }
  if (rc != OSGPU_OK) {
    cudaStreamSynchronize(st);
    cudaFree(p.kq);
    return rc;
  }
  p.last_use = ++c.plan_tick;
  ++c.plan_builds;
  c.plan_bytes += qbytes;
  c.plans.push_back(p);
  *kq = p.kq;
  return OSGPU_OK;
}

template <typename T>
int run_prop(Context& c, const PropJob& j0, cudaStream_t st) {
  const int is_d = sizeof(T) == 8;
  const size_t es = is_d ? 16 : 8;
  PropJob jp;
  const PropJob* jj = &j0;
  if (!is_d) {  // f32 ASM with padding above 2n: the kernel-spectrum plan at 2n
    const void* kq = nullptr;
    const int prc = plan_lookup(c, j0, st, &kq);
    if (prc) return prc;
    if (kq) {
      jp = j0;
      jp.engine = ENG_KEVEN;
      jp.Px = 2 * j0.g.nx;
      jp.Py = 2 * j0.g.ny;
      jp.kspec_ext = kq;
      jp.conj_h = j0.z < 0.0;
      jj = &jp;
    }
  }
  const PropJob& j = *jj;
  PropArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nx = (int)j.g.nx;
  a.ny = (int)j.g.ny;
  a.dx = j.g.dx;
  a.dy = j.g.dy;
  a.ax = make_axis(a.nx, (int)j.Px);
  a.ay = make_axis(a.ny, (int)j.Py);
  if (a.ax.nst < 0 || a.ay.nst < 0) {
    set_err("padded length has too many prime factors");
    return OSGPU_E_UNSUPPORTED;
  }
  if (!prop_smem_fits(a.ax, a.ay, is_d, kMaxSmem)) {
    set_err("grid %dx%d (sub-FFT %d x %d) exceeds the shared-memory plan of this library",
            a.nx, a.ny, a.ax.m, a.ay.m);
    return OSGPU_E_UNSUPPORTED;
  }
  a.in = j.d_in;
  a.in_c128 = j.in_c128;
  a.out = j.d_out;
  a.out_c128 = j.out_c128;
  a.out_intensity = j.d_int;
  a.out_intensity64 = j.d_int64;
  a.els = j.els;
  a.engine = j.engine;
  a.status = c.d_status;
  a.lam = j.g.lambda;
  a.z = j.z;
  a.scale = 1.0 / ((double)j.Px * (double)j.Py);
  a.conj_h = j.conj_h;
  a.seed = j.seed;
  a.seed_f64 = j.seed_f64;
  a.seed_scale = j.seed_scale;
  a.adj = j.adj;
  a.adj_uin = j.adj_uin;
  a.adj_uin_c128 = j.adj_uin_c128;
  for (int q = 0; q < kMaxElements; ++q) a.adj_grad[q] = j.adj_grad[q];
  a.trans = is_d ? nullptr : j.trans;
  if (!is_d) {  // schedule of the f32 passes: the tuner's forced one, else a measured one
    if (c.force_on) {
      a.sched = c.force;
    } else if (!c.tuned.empty()) {
      const auto it = c.tuned.find({a.ax.m, a.ax.r, a.ay.m, a.ay.r, a.nx, a.ny, c.lane_mode});
      if (it != c.tuned.end()) a.sched = it->second.s;
    }
  }
  int rc;
  if ((rc = get_tw(c, a.ax.m, is_d, &a.tw_mx))) return rc;
  if ((rc = get_tw(c, a.ay.m, is_d, &a.tw_my))) return rc;
  a.tw_Px = a.tw_mx;
  a.tw_Py = a.tw_my;
  if (a.ax.r > 1 && (rc = get_tw(c, (int)j.Px, is_d, &a.tw_Px))) return rc;
  if (a.ay.r > 1 && (rc = get_tw(c, (int)j.Py, is_d, &a.tw_Py))) return rc;

  const size_t Px = j.Px, Py = j.Py, ny = j.g.ny;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off += align256(bytes);
    return o;
  };
  const size_t o_work = carve(Px * ny * es);
  size_t o_tf = 0, o_hx = 0, o_hy = 0, o_tmp = 0, o_ks = 0;
  const bool tf = (j.engine == ENG_ASM || j.engine == ENG_FRESNEL_TF);
  const TfLayout L = tf_layout(Px, Py);
  if (tf) {
    if (!j.tables_pre) o_tf = carve(L.total);
  } else if (j.engine == ENG_KSEP) {
    o_hx = carve(Px * es);
    o_hy = carve(Py * es);
    o_tmp = carve(3 * (Px + Py) * 16);
  } else if (j.engine == ENG_KSPEC) {
    o_ks = carve(Px * Py * es);
    o_tmp = carve((2 * Px * Py + Px + Py) * 16);
  }
  DBuf ws;
  CK(ws.alloc(off, st));
  char* base = reinterpret_cast<char*>(ws.p);
  a.work = base + o_work;
  if (tf) {
    tf_bind(a, j.tables_pre ? reinterpret_cast<char*>(const_cast<void*>(j.tables_pre))
                            : base + o_tf, L);
    tf_scalars(a, j, is_d);
    if (!j.tables_pre) {
      ProfScope ps(c, st, PC_PREP, 0.0);
      CK(launch_asm_prep<T>(a, nullptr, st));
    }
  } else if (j.engine == ENG_KSEP) {
    a.hx = base + o_hx;
    a.hy = base + o_hy;
    ProfScope ps(c, st, PC_KSPEC, 0.0);
    CK(launch_fresnel_ksep<T>(a, base + o_hx, base + o_hy, base + o_tmp, st));
  } else if (j.engine == ENG_KEVEN) {
    a.kspec = j.kspec_ext;
  } else if (j.engine == ENG_KSPEC) {
    PropArgs b = a;
    b.ax = make_axis((int)Px, (int)Px);
    b.ay = make_axis((int)Py, (int)Py);
    if (b.ax.nst < 0 || b.ay.nst < 0 || smem_passA_bytes(b.ax, 1, 1) > kMaxSmem ||
        smem_passB_bytes(b.ay, 1) > kMaxSmem) {
      set_err("kernel-spectrum build of %zux%zu exceeds the shared-memory plan", Px, Py);
      return OSGPU_E_UNSUPPORTED;
    }
    if (!is_d) {  // the f32 build transforms with the f32 passes and tables
      if ((rc = get_tw(c, (int)Px, 0, &b.tw_mx))) return rc;
      if ((rc = get_tw(c, (int)Py, 0, &b.tw_my))) return rc;
    }
    ProfScope ps(c, st, PC_KSPEC, 0.0);
    CK(launch_rs_kspec<T>(b, base + o_ks, base + o_tmp, st));
    a.kspec = base + o_ks;
  }
  // every engine's spectrum data must be in place before pass B reads it
  if ((tf && (!a.fxv || !a.rowtab)) || (j.engine == ENG_KSEP && (!a.hx || !a.hy)) ||
      ((j.engine == ENG_KSPEC || j.engine == ENG_KEVEN) && !a.kspec)) {
    set_err("internal: transfer-function data of engine %d missing", j.engine);
    return OSGPU_E_UNSUPPORTED;
  }
  const double nin = (double)j.g.nx * j.g.ny, nsp = (double)Px * ny;
  const double el_bytes = element_bytes(j.els, !is_d);
  double adj_bytes = 0.0;  // pass C adjoint plane: forward field read + gradient RMW
  if (j.adj) {
    adj_bytes = nin * (j.adj_uin_c128 ? 16 : 8) + el_bytes;
    for (int q = 0; q < j.els.count; ++q)
      if (j.adj_grad[q]) adj_bytes += 2.0 * nin * (is_d ? 8 : 4);
  }
  {
    const double seed_bytes = j.seed ? nin * (j.seed_f64 ? 8 : 4) : 0.0;
    ProfScope ps(c, st, PC_PASS_A,
                 nin * (j.in_c128 ? 16 : 8) + nsp * es + (j.adj ? 0.0 : el_bytes) + seed_bytes);
    CK(launch_passA<T>(a, st));
  }
  {
    ProfScope ps(c, st, PC_PASS_B,
                 2 * nsp * es + (j.engine == ENG_KSPEC ? (double)Px * Py * es : 0.0) +
                     (j.engine == ENG_KEVEN ? (double)(Px / 2 + 1) * (Py / 2 + 1) * 8 : 0.0));
    CK(launch_passB<T>(a, st));
  }
  {
    const double ob = (j.d_out ? (j.out_c128 ? 16 : 8) : 0) + (j.d_int ? 4 : 0) +
                      (j.d_int64 ? 8 : 0);
    ProfScope ps(c, st, PC_PASS_C, nsp * es + nin * ob + adj_bytes);
    CK(launch_passC<T>(a, st));
  }
  return OSGPU_OK;
}

// fft::transform2 of an nx x ny grid: forward (unnormalised) or inverse
// (1/(nx ny)) through conj(fft2(conj x)) / N.
template <typename T>
int run_fft2(Context& c, const void* d_in, int in_c128, void* d_out, int out_c128, int nx, int ny,
             int inverse, cudaStream_t st) {
  const int is_d = sizeof(T) == 8;
  const size_t es = is_d ? 16 : 8;
  PropArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nx = nx;
  a.ny = ny;
  a.ax = make_axis(nx, nx);
  a.ay = make_axis(ny, ny);
  if (a.ax.nst < 0 || a.ay.nst < 0 || smem_passA_bytes(a.ax, is_d, 1) > kMaxSmem ||
      smem_passB_bytes(a.ay, is_d) > kMaxSmem) {
    set_err("fft2 of %dx%d exceeds the shared-memory plan of this library", nx, ny);
    return OSGPU_E_UNSUPPORTED;
  }
  int rc;
  if ((rc = get_tw(c, nx, is_d, &a.tw_mx))) return rc;
  if ((rc = get_tw(c, ny, is_d, &a.tw_my))) return rc;
  a.tw_Px = a.tw_mx;
  a.tw_Py = a.tw_my;
  const size_t n = (size_t)nx * ny;
  DBuf ws;
  CK(ws.alloc(align256(n * es) * (inverse ? 3 : 2), st));
  char* base = reinterpret_cast<char*>(ws.p);
  a.work = base;
  void* spec = base + align256(n * es);
  a.in = d_in;
  a.in_c128 = in_c128;
  if (inverse) {  // conj(x) in the engine's type
    void* tmp = base + 2 * align256(n * es);
    CK(launch_conj_copy<T>(d_in, in_c128, tmp, n, st));
    a.in = tmp;
    a.in_c128 = is_d;
  }
  a.engine = ENG_IDENTITY;
  a.scale = inverse ? 1.0 / ((double)nx * (double)ny) : 1.0;
  a.status = nullptr;  // transform2 does not validate samples
  ProfScope ps(c, st, PC_FFT2, (double)n * (2 * es + 4 * es));
  CK(launch_fft2<T>(a, spec, d_out, out_c128, inverse, st));
  return OSGPU_OK;
}

int run_prop_dispatch(Context& c, const PropJob& j, int f32, cudaStream_t st) {
  return f32 ? run_prop<float>(c, j, st) : run_prop<double>(c, j, st);
}

// Upload host complex128 input, run `fn(d_in, d_out)`, download output, map
// the device status.
template <typename F>
int host_call(Context& c, const double* in, double* out, size_t n, F&& fn) {
  cudaStream_t st = c.stream;
  DBuf din, dout;
  CK(din.alloc(n * 16, st));
  CK(dout.alloc(n * 16, st));
  CK(cudaMemcpyAsync(din.p, in, n * 16, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(c.d_status, 0, sizeof(int), st));
  int rc = fn(din.p, dout.p);
  if (rc) {
    cudaStreamSynchronize(st);
    return rc;
  }
  CK(cudaMemcpyAsync(out, dout.p, n * 16, cudaMemcpyDeviceToHost, st));
  int status = 0;
  CK(cudaMemcpyAsync(&status, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (status) {
    // reported here: clear it, so a later osgpu_sync_status does not see it again
    CK(cudaMemset(c.d_status, 0, sizeof(int)));
    set_err("field contains non-finite samples");
    return OSGPU_E_NON_FINITE_SAMPLE;
  }
  return OSGPU_OK;
}

int check_grid(const osgpu_grid* g) {
  if (!g) {
    set_err("null grid");
    return OSGPU_E_BAD_ARGUMENT;
  }
  return OSGPU_OK;
}

int check_precision(int32_t p) {
  if (p != OSGPU_F64 && p != OSGPU_F32) {
    set_err("precision must be OSGPU_F64 or OSGPU_F32");
    return OSGPU_E_BAD_ARGUMENT;
  }
  return OSGPU_OK;
}

// Identity / error-path helper: scan host input first, as the reference does.
int identity_copy(const double* in, double* out, size_t n) {
  if (!host_all_finite(in, 2 * n)) {
    set_err("field contains non-finite samples");
    return OSGPU_E_NON_FINITE_SAMPLE;
  }
  if (out != in) std::memmove(out, in, n * 16);
  return OSGPU_OK;
}

int scan_then(const double* in, size_t n, int code) {
  if (in && !host_all_finite(in, 2 * n)) {
    set_err("field contains non-finite samples");
    return OSGPU_E_NON_FINITE_SAMPLE;
  }
  return code;
}

template <typename T>
int run_fraun(Context& c, const osgpu_grid& g, double z, const osgpu_fraunhofer_report& r,
              const ElementList& els, const void* d_in, int in_c128, void* d_out, int out_c128,
              float* d_int, int adjoint, cudaStream_t st) {
  const int is_d = sizeof(T) == 8;
  const size_t es = is_d ? 16 : 8;
  FraunArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nx = (int)g.nx;
  a.ny = (int)g.ny;
  a.dx = g.dx;
  a.dy = g.dy;
  a.ax = make_axis(a.nx, a.nx);
  a.ay = make_axis(a.ny, a.ny);
  if (a.ax.nst < 0 || a.ay.nst < 0 || 2 * ((size_t)a.ax.m + 1) * es > kMaxSmem ||
      2 * (size_t)a.ay.m * es > kMaxSmem) {
    set_err("Fraunhofer grid %dx%d exceeds the shared-memory plan", a.nx, a.ny);
    return OSGPU_E_UNSUPPORTED;
  }
  int rc;
  if ((rc = get_tw(c, a.ax.m, is_d, &a.tw_mx))) return rc;
  if ((rc = get_tw(c, a.ay.m, is_d, &a.tw_my))) return rc;
  DBuf ws;
  const size_t work_bytes = ((size_t)a.nx * a.ny * es + 255) & ~(size_t)255;
  const size_t tab_bytes = is_d ? 0 : 2 * ((size_t)a.nx + a.ny) * sizeof(float2);
  CK(ws.alloc(work_bytes + tab_bytes, st));
  a.work = ws.p;
  if (!is_d) {  // the f32 engine's per-axis phase tables behind the spectrum
    float2* t = reinterpret_cast<float2*>(static_cast<char*>(ws.p) + work_bytes);
    a.tpx = t;
    a.tqx = t + a.nx;
    a.tpy = t + 2 * a.nx;
    a.tqy = t + 2 * a.nx + a.ny;
  }
  a.in = d_in;
  a.in_c128 = in_c128;
  a.out = d_out;
  a.out_c128 = out_c128;
  a.out_intensity = d_int;
  a.els = els;
  a.lam = g.lambda;
  a.z = z;
  a.k = 2.0 * PI / g.lambda;
  a.xs = r.source_x;
  a.ys = r.source_y;
  a.f_s = r.source_x / (g.lambda * z);
  a.g_s = r.source_y / (g.lambda * z);
  a.dxo = r.dx_out;
  a.dyo = r.dy_out;
  a.cxc = ((double)g.nx - 1.0) / 2.0;
  a.cyc = ((double)g.ny - 1.0) / 2.0;
  // quad = e^{ikz} / (i lam z), num_complex division order (fraunhofer.rs:420)
  const double kz = a.k * z;
  const double cre = std::cos(kz), cim = std::sin(kz);
  const double dre = 0.0 * z, dim = g.lambda * z;
  const double ns = dre * dre + dim * dim;
  a.quad_re = (cre * dre + cim * dim) / ns;
  a.quad_im = (cim * dre - cre * dim) / ns;
  a.adjoint = adjoint;
  a.status = c.d_status;
  ProfScope ps(c, st, PC_FRAUN, (double)a.nx * a.ny * (es + 2 * es + es));
  CK(launch_fraunhofer<T>(a, st));
  return OSGPU_OK;
}

void fill_asm_job(PropJob& j, const osgpu_grid& g, double z, const osgpu_asm_report& r,
                  const osgpu_asm_config& cfg) {
  std::memset(&j, 0, sizeof(j));
  j.engine = ENG_ASM;
  j.g = g;
  j.z = z;
  j.Px = r.nx_pad;
  j.Py = r.ny_pad;
  j.medium = cfg.medium;
  j.band_limited = cfg.band_limited;
  j.lim_x = r.band_limit_fx;
  j.lim_y = r.band_limit_fy;
}

// ------------------------------------------------------------ inverse loops

// The element chain in front of each propagation of a design (elements of
// the steps since the previous propagation), and the trailing chain after
// the last one.  flat[q] is the element's index in step order (the order
// of osgpu_frame.d_grad).
struct Chain {
  int prop_step = -1;  // step whose z_after follows the chain (-1: trailing chain)
  ElementList list;
  int flat[kMaxElements];
};

int make_chains(const osgpu_step* steps, int n_steps, const std::vector<Elements>& E, int f32,
                std::vector<Chain>& out) {
  out.clear();
  Chain cur;
  std::memset(&cur.list, 0, sizeof(cur.list));
  bool fast = true;
  int flat = 0;
  for (int s = 0; s < n_steps; ++s) {
    for (int q = 0; q < E[s].list.count; ++q) {
      if (cur.list.count == kMaxElements) {
        set_err("more than %d elements between two propagations", kMaxElements);
        return OSGPU_E_UNSUPPORTED;
      }
      cur.flat[cur.list.count] = flat++;
      cur.list.el[cur.list.count++] = E[s].list.el[q];
      fast = fast && E[s].list.fast;
    }
    if (steps[s].z_after != 0.0) {
      cur.prop_step = s;
      cur.list.fast = f32 && fast;
      out.push_back(cur);
      std::memset(&cur.list, 0, sizeof(cur.list));
      fast = true;
    }
  }
  cur.prop_step = -1;
  cur.list.fast = f32 && fast;
  out.push_back(cur);
  return OSGPU_OK;
}

int check_frames(const osgpu_frame* frames, int n, int dtype) {
  if ((n > 0 && !frames) || n < 0 || (dtype != OSGPU_C128 && dtype != OSGPU_C64)) {
    set_err("bad frame list or dtype");
    return OSGPU_E_BAD_ARGUMENT;
  }
  for (int f = 0; f < n; ++f) {
    const osgpu_frame& fr = frames[f];
    if (!fr.d_source || fr.n_steps < 0 || (fr.n_steps > 0 && !fr.steps)) {
      set_err("frame %d: bad source or steps", f);
      return OSGPU_E_BAD_ARGUMENT;
    }
    if (fr.grid.nx == 0 || fr.grid.ny == 0) {
      set_err("frame %d: empty grid", f);
      return OSGPU_E_EMPTY_GRID;
    }
  }
  return OSGPU_OK;
}

int count_props(const osgpu_frame& fr) {
  int k = 0;
  for (int s = 0; s < fr.n_steps; ++s)
    if (fr.steps[s].z_after != 0.0) ++k;
  return k;
}

}  // namespace

// An instantiated capture of a batched trace (osgpu_beamline_trace_batch_graph).
struct osgpu_graph {
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;
};

// Forward planes recorded by osgpu_render_batch_device: for every frame,
// the output field of each propagation, in one device allocation that is
// kept and grown across calls.
struct osgpu_tape {
  uint64_t budget = 0;  // 0: unlimited
  void* buf = nullptr;
  size_t cap = 0;
  int valid = 0;
  int dtype = -1;
  std::vector<size_t> off;     // per frame: byte offset of its first plane
  std::vector<int> planes;     // per frame: number of planes
  std::vector<uint64_t> nfld;  // per frame: samples per plane
};

namespace {

// Forward trace of one frame: propagations write into `plane(k)` (k-th
// propagation); the detector intensity goes to fr.d_intensity.
template <typename PlaneFn>
int forward_frame(Context& c, const osgpu_frame& fr, const std::vector<Elements>& E,
                  const std::vector<osgpu_asm_report>& R, const std::vector<Chain>& ch,
                  const osgpu_asm_config& cfg, int f32, int c128, PlaneFn plane,
                  bool want_last_field, cudaStream_t st) {
  const osgpu_grid& g = fr.grid;
  const void* src = fr.d_source;
  const int K = (int)ch.size() - 1;  // propagations
  const Chain& tail = ch[K];
  int rc;
  for (int k = 0; k < K; ++k) {
    const int s = ch[k].prop_step;
    osgpu_asm_config sc = cfg;
    sc.medium = fr.steps[s].medium;
    PropJob j;
    fill_asm_job(j, g, fr.steps[s].z_after, R[s], sc);
    j.tables_pre = E[s].prop_tables.p;
    j.trans = reinterpret_cast<const float2*>(E[s].trans.p);
    j.els = ch[k].list;
    j.d_in = src;
    j.in_c128 = c128;
    const bool last = (k == K - 1);
    void* out = plane(k);
    j.d_out = (last && tail.list.count == 0 && !want_last_field) ? nullptr : out;
    j.out_c128 = c128;
    if (last && tail.list.count == 0 && fr.d_intensity) {
      if (c128) j.d_int64 = reinterpret_cast<double*>(fr.d_intensity);
      else j.d_int = reinterpret_cast<float*>(fr.d_intensity);
    }
    if ((rc = run_prop_dispatch(c, j, f32, st))) return rc;
    src = out;
  }
  if ((K == 0 || tail.list.count > 0) && fr.d_intensity) {
    ProfScope ps(c, st, PC_APPLY, (double)g.nx * g.ny * ((c128 ? 16 : 8) + (c128 ? 8 : 4)));
    CK(launch_apply_intensity(src, c128, nullptr, c128, tail.list, (int)g.nx, (int)g.ny, g.dx,
                              g.dy, fr.d_intensity, c128, f32, st));
  }
  return OSGPU_OK;
}

// Fused f32 Fraunhofer GS (gs_fast.cu) over all items of a batch: every
// item is M x M, z > 0, no source offset.
int gs_fused(Context& c, osgpu_gs_item* items, int n_items, const osgpu_gs_config& cfg,
             const osgpu_fraunhofer_config& fcfg, double beta_f, double beta_p, int M,
             cudaStream_t st) {
  const size_t n = (size_t)M * M;
  const int nb = gs_fast_blocks(M), nbr = gs_fast_row_blocks(M);
  const int max_it = cfg.max_iterations;
  int rc;
  const void* tw = nullptr;
  if ((rc = get_tw(c, M, 0, &tw))) return rc;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  // per-item layout in one allocation
  const size_t o_W = 0, o_ph = o_W + al(n * 8), o_il = o_ph + al(n * 4), o_op = o_il + al(n * 4),
               o_ta = o_op + al(n), o_ti = o_ta + al(n * 4), o_tab = o_ti + al(n * 4),
               o_am = o_tab + al((size_t)4 * M * 8), o_pc = o_am + al(n * 4),
               o_pr = o_pc + al((size_t)4 * nb * 8),
               o_hi = o_pr + al((size_t)2 * nb * 8), o_te = o_hi + al(sizeof(GsRecordDev) * max_it),
               per = o_te + al(n * 4);  // o_te: |U| - T column-major, transposed at the end
  DBuf mem, dstates, ditems, dfolds;
  CK(mem.alloc(per * n_items, st));
  CK(dstates.alloc(sizeof(GsState) * n_items, st));
  CK(ditems.alloc(sizeof(GsFastItem) * n_items, st));
  CK(dfolds.alloc(sizeof(GsFoldItem) * n_items, st));
  char* base = reinterpret_cast<char*>(mem.p);
  GsState* S = reinterpret_cast<GsState*>(dstates.p);
  std::vector<GsState> hs(n_items);
  for (auto& h : hs) {
    std::memset(&h, 0, sizeof(h));
    h.best_it = -1;
  }
  CK(cudaMemcpyAsync(S, hs.data(), sizeof(GsState) * n_items, cudaMemcpyHostToDevice, st));
  std::vector<GsFastItem> fi(n_items);
  std::vector<GsFoldItem> fo(n_items);
  std::vector<float2> tabs((size_t)4 * M * n_items);
  for (int i = 0; i < n_items; ++i) {
    osgpu_gs_item& it = items[i];
    const osgpu_grid& g = it.grid;
    char* b = base + per * i;
    osgpu_fraunhofer_report fr;
    if ((rc = fraunhofer_resolve(g, it.z, fcfg, fr)) > 0) {
      set_err("GS item %d: Fraunhofer regime check failed (status %d)", i, rc);
      return rc;
    }
    // separable pre / post factors in FP64 (fraunhofer.rs:396-438, no source offset)
    const double cxc = ((double)M - 1.0) / 2.0, lz = g.lambda * it.z;
    const double kz = (2.0 * PI / g.lambda) * it.z;
    const double qre = std::sin(kz) / lz, qim = -std::cos(kz) / lz;  // e^{ikz} / (i lam z)
    const double w = g.dx * g.dy;
    float2* T4 = tabs.data() + (size_t)4 * M * i;
    for (int j = 0; j < M; ++j) {
      const double pre = 2.0 * PI * cxc * (double)j / (double)M;
      T4[j] = make_float2((float)std::cos(pre), (float)std::sin(pre));          // prx
      T4[M + j] = T4[j];                                                          // pry
      const double dxp = ((double)j - cxc) * fr.dx_out, dyp = ((double)j - cxc) * fr.dy_out;
      const double post = 2.0 * PI * cxc * ((double)j - cxc) / (double)M;
      const double ax = PI * dxp * dxp / lz + post, ay = PI * dyp * dyp / lz + post;
      const double cx_ = std::cos(ax), sx_ = std::sin(ax);
      T4[2 * M + j] = make_float2((float)((qre * cx_ - qim * sx_) * w),
                                  (float)((qre * sx_ + qim * cx_) * w));          // qx
      T4[3 * M + j] = make_float2((float)std::cos(ay), (float)std::sin(ay));      // qy
    }
    GsFastItem& f = fi[i];
    std::memset(&f, 0, sizeof(f));
    f.W = reinterpret_cast<float2*>(b + o_W);
    f.phase = reinterpret_cast<float*>(b + o_ph);
    f.best = reinterpret_cast<float*>(it.d_phase);
    f.amask = reinterpret_cast<const float*>(b + o_am);
    f.tamp_t = reinterpret_cast<const float*>(b + o_ta);
    f.tint_t = it.d_target_intensity ? reinterpret_cast<const float*>(b + o_ti) : nullptr;
    f.prx = reinterpret_cast<const float2*>(b + o_tab);
    f.pry = f.prx + M;
    f.qx = f.prx + 2 * M;
    f.qy = f.prx + 3 * M;
    f.c = (float)(w / lz);
    f.terr = it.d_target_error ? reinterpret_cast<float*>(b + o_te) : nullptr;
    f.perr = reinterpret_cast<float*>(it.d_phase_error);
    f.state = S + i;
    f.part_col = reinterpret_cast<double*>(b + o_pc);
    f.part_row = reinterpret_cast<double*>(b + o_pr);
    fo[i].part_merit = f.part_col;
    fo[i].part_update = f.part_row;
    fo[i].state = S + i;
    fo[i].hist = reinterpret_cast<GsRecordDev*>(b + o_hi);
    CK(cudaMemcpyAsync(b + o_tab, T4, sizeof(float2) * 4 * M, cudaMemcpyHostToDevice, st));
    CK(launch_gs_init(it.d_phase, f.phase, 0, cfg.lo, cfg.hi,
                      reinterpret_cast<unsigned char*>(b + o_op), it.aperture,
                      it.aperture_a, it.aperture_b, it.center_x, it.center_y, M, M, g.dx, g.dy,
                      st));
    CK(launch_abs(it.d_input, 0, b + o_il, 0, 0, n, st));
    CK(launch_mask_amplitude(b + o_il, reinterpret_cast<const unsigned char*>(b + o_op),
                             b + o_am, 0, n, st));
    CK(launch_transpose_real(reinterpret_cast<const float*>(it.d_target_amplitude),
                             reinterpret_cast<float*>(b + o_ta), M, st));
    if (it.d_target_intensity)
      CK(launch_transpose_real(reinterpret_cast<const float*>(it.d_target_intensity),
                               reinterpret_cast<float*>(b + o_ti), M, st));
  }
  CK(cudaMemcpyAsync(ditems.p, fi.data(), sizeof(GsFastItem) * n_items, cudaMemcpyHostToDevice,
                     st));
  CK(cudaMemcpyAsync(dfolds.p, fo.data(), sizeof(GsFoldItem) * n_items, cudaMemcpyHostToDevice,
                     st));
  CK(cudaStreamSynchronize(st));  // host tables and descriptors are copied
  const GsFastItem* DI = reinterpret_cast<const GsFastItem*>(ditems.p);
  const GsFoldItem* DF = reinterpret_cast<const GsFoldItem*>(dfolds.p);
  GsFastArgs a;
  a.M = M;
  a.tw = tw;
  a.beta_f = (float)beta_f;
  a.beta_p = (float)beta_p;
  a.lo = (float)cfg.lo;
  a.hi = (float)cfg.hi;
  a.wrap = (cfg.hi - cfg.lo >= 2.0 * PI) ? 1 : 0;
  a.intensity_only = 0;
  a.w_base = base + o_W;
  a.w_stride = per;
  const double bytes_cols = (double)n * (2 * 8 + 4) * n_items;
  const double bytes_rows = (double)n * (2 * 8 + 4 + 4 + 4 + 1) * n_items;
  {
    ProfScope ps(c, st, PC_GS_ROWS, bytes_rows);
    CK(launch_gs_rows(DI, n_items, a, 0, st));
  }
  // The loop state is copied to pinned host memory after every chunk of
  // iterations, and the host looks at the copy of the chunk before the one
  // just queued, so the GPU always has a chunk of work ahead of the check
  // (one extra chunk after every item has stopped: its kernels return at
  // once for stopped items).
  constexpr int kChunk = 8;
  const size_t pin_need = sizeof(GsState) * 2 * n_items;
  if (c.gs_pin_bytes < pin_need) {  // grows only; the previous call's copies have completed
    if (c.gs_pin) CK(cudaFreeHost(c.gs_pin));
    c.gs_pin = nullptr;
    c.gs_pin_bytes = 0;
    CK(cudaMallocHost(&c.gs_pin, pin_need));
    c.gs_pin_bytes = pin_need;
  }
  for (cudaEvent_t& e : c.gs_ev)
    if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  GsState* pin = c.gs_pin;
  int pending = -1;
  for (int k = 0; k < max_it; ++k) {
    if (k > 0 && k % kChunk == 0) {
      const int b = (k / kChunk) & 1;
      CK(cudaMemcpyAsync(pin + (size_t)b * n_items, S, sizeof(GsState) * n_items,
                         cudaMemcpyDeviceToHost, st));
      CK(cudaEventRecord(c.gs_ev[b], st));
      if (pending >= 0) {
        CK(cudaEventSynchronize(c.gs_ev[pending]));
        bool all = true;
        for (int i = 0; i < n_items; ++i) all = all && pin[(size_t)pending * n_items + i].stop;
        if (all) break;
      }
      pending = b;
    }
    {
      ProfScope ps(c, st, PC_GS_COLS, bytes_cols);
      CK(launch_gs_cols(DI, n_items, a, st));
    }
    CK(launch_gs_fold_merit_batch(DF, n_items, nb, n, k, st));
    {
      ProfScope ps(c, st, PC_GS_ROWS, bytes_rows);
      CK(launch_gs_rows(DI, n_items, a, 1, st));
    }
    CK(launch_gs_fold_update_batch(DF, n_items, nbr, n, k, cfg.patience, cfg.merit_tolerance,
                                   max_it, st));
  }
  CK(cudaMemcpyAsync(hs.data(), S, sizeof(GsState) * n_items, cudaMemcpyDeviceToHost, st));
  std::vector<GsRecordDev> hh((size_t)max_it * n_items);
  for (int i = 0; i < n_items; ++i)
    CK(cudaMemcpyAsync(hh.data() + (size_t)max_it * i, fo[i].hist, sizeof(GsRecordDev) * max_it,
                       cudaMemcpyDeviceToHost, st));
  bool want_int = false;
  for (int i = 0; i < n_items; ++i) {
    osgpu_gs_item& it = items[i];
    char* b = base + per * i;
    if (it.d_last_phase)
      CK(cudaMemcpyAsync(it.d_last_phase, b + o_ph, n * 4, cudaMemcpyDeviceToDevice, st));
    if (it.d_target_error)
      CK(launch_transpose_real(reinterpret_cast<const float*>(b + o_te),
                               reinterpret_cast<float*>(it.d_target_error), M, st));
    if (it.d_illumination)
      CK(cudaMemcpyAsync(it.d_illumination, b + o_il, n * 4, cudaMemcpyDeviceToDevice, st));
    want_int = want_int || it.d_best_intensity;
  }
  if (want_int) {  // the best iteration's forward pass, recomputed by the fused kernels
    for (int i = 0; i < n_items; ++i) {
      CK(cudaMemcpyAsync(fi[i].phase, items[i].d_phase, n * 4, cudaMemcpyDeviceToDevice, st));
      fi[i].out_intensity = reinterpret_cast<float*>(items[i].d_best_intensity);
    }
    CK(cudaMemcpyAsync(ditems.p, fi.data(), sizeof(GsFastItem) * n_items,
                       cudaMemcpyHostToDevice, st));
    GsFastArgs af = a;
    af.intensity_only = 1;
    {
      ProfScope ps(c, st, PC_GS_ROWS, bytes_rows);
      CK(launch_gs_rows(DI, n_items, af, 0, st));
    }
    {
      ProfScope ps(c, st, PC_GS_COLS, bytes_cols);
      CK(launch_gs_cols(DI, n_items, af, st));
    }
  }
  CK(cudaStreamSynchronize(st));
  {  // a row pass whose staged inputs never arrived marked its items
    std::vector<GsState> hf(n_items);
    CK(cudaMemcpy(hf.data(), S, sizeof(GsState) * n_items, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n_items; ++i)
      if (hf[i].fault) {
        set_err("GS item %d: a staged row-pass input did not arrive (bounded wait ran out)", i);
        return OSGPU_E_CUDA;
      }
  }
  for (int i = 0; i < n_items; ++i) {
    osgpu_gs_item& it = items[i];
    const GsState& h = hs[i];
    const GsRecordDev* H = hh.data() + (size_t)max_it * i;
    if (h.best_it < 0) {
      set_err("gs loop ran zero iterations");
      return OSGPU_E_RENDER;
    }
    it.result.merit = h.best_merit;
    it.result.best_iteration = (uint64_t)h.best_it;
    it.result.amplitude_mse = H[h.best_it].amplitude_mse;
    it.result.converged = h.converged;
    it.result.iterations = (uint64_t)h.iterations;
    if (it.history)
      for (int k = 0; k < h.iterations; ++k) {
        osgpu_gs_record& r = it.history[k];
        r.iteration = (uint64_t)k;
        r.merit = H[k].merit;
        r.best_merit = H[k].best_merit;
        r.amplitude_mse = H[k].amplitude_mse;
        r.target_error_rms = H[k].target_error_rms;
        r.phase_update_rms = H[k].phase_update_rms;
      }
  }
  return OSGPU_OK;
}

int tune_geometry(Context& c, const osgpu_grid& g, double z, const osgpu_asm_config& cfg,
                  int lanes, cudaStream_t st);

}  // namespace

void osgpu::set_last_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
}

// ====================================================================== ABI

extern "C" {

int osgpu_init(int32_t device) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if (c.device >= 0) return OSGPU_OK;
  if (device >= 0) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  }
  return ensure_init(c);
}

struct osgpu_field_s {
  void* p;
  uint64_t nx, ny;
  int32_t dtype;
};

int osgpu_field_create(uint64_t nx, uint64_t ny, int32_t dtype, osgpu_field* out) {
  if (!out) return OSGPU_E_BAD_ARGUMENT;
  *out = nullptr;
  if (nx == 0 || ny == 0 || (dtype != OSGPU_C128 && dtype != OSGPU_C64) ||
      nx > (uint64_t)INT32_MAX || ny > (uint64_t)INT32_MAX ||
      nx * ny > ((uint64_t)1 << 40)) {  // 16 TiB of complex128: beyond any device
    set_err("field handle: bad shape or dtype");
    return OSGPU_E_BAD_ARGUMENT;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  const size_t bytes = (size_t)(nx * ny) * (dtype == OSGPU_C128 ? 16 : 8);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaSuccess) e = cudaMemset(p, 0, bytes);
  if (e != cudaSuccess) {
    if (p) cudaFree(p);
    return cuda_fail(e, "field handle allocation");
  }
  osgpu_field f = new (std::nothrow) osgpu_field_s{p, nx, ny, dtype};
  if (!f) {
    cudaFree(p);
    return OSGPU_E_OUT_OF_MEMORY;
  }
  *out = f;
  return OSGPU_OK;
}

int osgpu_field_upload(osgpu_field f, const double* host_c128, void* stream) {
  if (!f || !host_c128) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const size_t n = (size_t)(f->nx * f->ny);
  if (f->dtype == OSGPU_C128) {
    CK(cudaMemcpyAsync(f->p, host_c128, n * 16, cudaMemcpyHostToDevice, st));
  } else {
    DBuf tmp;
    CK(tmp.alloc(n * 16, st));
    CK(cudaMemcpyAsync(tmp.p, host_c128, n * 16, cudaMemcpyHostToDevice, st));
    CK(launch_c128_to_c64(tmp.p, f->p, n, st));
  }
  CK(cudaStreamSynchronize(st));
  return OSGPU_OK;
}

int osgpu_field_download(osgpu_field f, double* host_c128, void* stream) {
  if (!f || !host_c128) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const size_t n = (size_t)(f->nx * f->ny);
  if (f->dtype == OSGPU_C128) {
    CK(cudaMemcpyAsync(host_c128, f->p, n * 16, cudaMemcpyDeviceToHost, st));
  } else {
    DBuf tmp;
    CK(tmp.alloc(n * 16, st));
    CK(launch_c64_to_c128(f->p, tmp.p, n, st));
    CK(cudaMemcpyAsync(host_c128, tmp.p, n * 16, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  return OSGPU_OK;
}

int osgpu_field_info(osgpu_field f, void** d_samples, uint64_t* nx, uint64_t* ny,
                     int32_t* dtype) {
  if (!f) return OSGPU_E_BAD_ARGUMENT;
  if (d_samples) *d_samples = f->p;
  if (nx) *nx = f->nx;
  if (ny) *ny = f->ny;
  if (dtype) *dtype = f->dtype;
  return OSGPU_OK;
}

int osgpu_field_destroy(osgpu_field f) {
  if (!f) return OSGPU_OK;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  const cudaError_t e = cudaFree(f->p);  // waits for the work queued on the samples
  delete f;
  return e == cudaSuccess ? OSGPU_OK : cuda_fail(e, "field handle free");
}

int osgpu_shutdown(void) {
  noalloc_forget_scratch();  // looked up again by the next allocation-free call
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if (c.device < 0) return OSGPU_OK;  // nothing else was initialised
  CK(cudaDeviceSynchronize());  // no queued work reads what is freed below
  // twiddle tables stay: captured graphs (osgpu_beamline_trace_batch_graph)
  // hold their addresses; plans and the encircled-energy order are never
  // used under capture
  for (KPlan& p : c.plans) cudaFree(p.kq);
  c.plans.clear();
  c.plan_bytes = 0;
  if (c.ee.d) cudaFree(c.ee.d);
  c.ee = Context::EeOrder();
  if (c.gs_pin) cudaFreeHost(c.gs_pin);
  c.gs_pin = nullptr;
  c.gs_pin_bytes = 0;
  for (cudaEvent_t& e : c.gs_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  cudaMemPool_t pool;
  CK(cudaDeviceGetDefaultMemPool(&pool, c.device));
  CK(cudaMemPoolTrimTo(pool, 0));  // scratch returned by the stream-ordered frees
  return OSGPU_OK;
}

int osgpu_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return OSGPU_E_BAD_ARGUMENT;
  std::snprintf(buf, len, "%s", t_err);
  return OSGPU_OK;
}

const char* osgpu_version(void) { return "osgpu 0.1 (sm_103a)"; }

uint64_t osgpu_launch_count(void) { return (uint64_t)launch_count(); }

int osgpu_sync_status(void) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc = ensure_init(c);
  if (rc) return rc;
  int status = 0;
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(&status, c.d_status, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemset(c.d_status, 0, sizeof(int)));
  if (status) {
    set_err("field contains non-finite samples");
    return OSGPU_E_NON_FINITE_SAMPLE;
  }
  return OSGPU_OK;
}

// ------------------------------------------------------------------ ASM

int osgpu_asm_sampling_report(const osgpu_grid* g, double z, const osgpu_asm_config* cfg,
                              osgpu_asm_report* out) {
  if (!g || !cfg || !out) return OSGPU_E_BAD_ARGUMENT;
  asm_analyze(*g, z, *cfg, cfg->padding, *out);
  return OSGPU_OK;
}

int osgpu_asm_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                        const osgpu_asm_config* cfg, int32_t precision,
                        osgpu_asm_report* report) {
  int rc;
  if ((rc = check_grid(g)) || (rc = check_precision(precision))) return rc;
  if (!cfg || !in || !out) return OSGPU_E_BAD_ARGUMENT;
  osgpu_asm_report r;
  rc = asm_resolve(*g, z, *cfg, r);
  if (report) *report = r;
  const size_t n = g->nx * g->ny;
  if (rc == -1) return identity_copy(in, out, n);
  if (rc == OSGPU_E_ALIASING_RISK) {
    set_err("sampling criteria not met (ASM transfer function undersampled)");
    return scan_then(in, n, rc);
  }
  if (rc) {
    set_err("invalid ASM propagation arguments (status %d)", rc);
    return rc;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  return host_call(c, in, out, n, [&](const void* din, void* dout) {
    PropJob j;
    fill_asm_job(j, *g, z, r, *cfg);
    j.d_in = din;
    j.in_c128 = 1;
    j.d_out = dout;
    j.out_c128 = 1;
    return run_prop_dispatch(c, j, precision == OSGPU_F32, c.stream);
  });
}

int osgpu_fft2(const double* in, double* out, uint64_t nx, uint64_t ny, int32_t inverse,
               int32_t precision) {
  int rc;
  if ((rc = check_precision(precision))) return rc;
  if (!in || !out) return OSGPU_E_BAD_ARGUMENT;
  if (nx == 0 || ny == 0) return OSGPU_OK;  // nothing to transform (fft.rs:41-44)
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  const size_t n = nx * ny;
  DBuf din, dout;
  CK(din.alloc(n * 16, c.stream));
  CK(dout.alloc(n * 16, c.stream));
  CK(cudaMemcpyAsync(din.p, in, n * 16, cudaMemcpyHostToDevice, c.stream));
  rc = precision == OSGPU_F32
           ? run_fft2<float>(c, din.p, 1, dout.p, 1, (int)nx, (int)ny, inverse, c.stream)
           : run_fft2<double>(c, din.p, 1, dout.p, 1, (int)nx, (int)ny, inverse, c.stream);
  if (rc) {
    cudaStreamSynchronize(c.stream);
    return rc;
  }
  CK(cudaMemcpyAsync(out, dout.p, n * 16, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return OSGPU_OK;
}

int osgpu_fft2_device(const void* d_in, void* d_out, int32_t dtype, uint64_t nx, uint64_t ny,
                      int32_t inverse, void* stream) {
  if (!d_in || !d_out || (dtype != OSGPU_C128 && dtype != OSGPU_C64)) return OSGPU_E_BAD_ARGUMENT;
  if (nx == 0 || ny == 0) return OSGPU_OK;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int c128 = dtype == OSGPU_C128;
  return c128 ? run_fft2<double>(c, d_in, 1, d_out, 1, (int)nx, (int)ny, inverse, st)
              : run_fft2<float>(c, d_in, 0, d_out, 0, (int)nx, (int)ny, inverse, st);
}

int osgpu_asm_propagate_device(const void* d_in, void* d_out, int32_t dtype,
                               const osgpu_grid* g, double z, const osgpu_asm_config* cfg,
                               void* stream, osgpu_asm_report* report) {
  int rc;
  if ((rc = check_grid(g))) return rc;
  if (!cfg || !d_in || !d_out || (dtype != OSGPU_C128 && dtype != OSGPU_C64))
    return OSGPU_E_BAD_ARGUMENT;
  osgpu_asm_report r;
  rc = asm_resolve(*g, z, *cfg, r);
  if (report) *report = r;
  if (rc > 0) return rc;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int e0 = ensure_init(c);
  if (e0) return e0;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const size_t es = dtype == OSGPU_C128 ? 16 : 8;
  if (rc == -1) {
    if (d_out != d_in) CK(cudaMemcpyAsync(d_out, d_in, g->nx * g->ny * es, cudaMemcpyDeviceToDevice, st));
    return OSGPU_OK;
  }
  PropJob j;
  fill_asm_job(j, *g, z, r, *cfg);
  j.d_in = d_in;
  j.in_c128 = dtype == OSGPU_C128;
  j.d_out = d_out;
  j.out_c128 = dtype == OSGPU_C128;
  return run_prop_dispatch(c, j, dtype == OSGPU_C64, st);
}

// -------------------------------------------------------------- Fresnel

int osgpu_fresnel_sampling_report(const osgpu_grid* g, double z, const osgpu_fresnel_config* cfg,
                                  osgpu_fresnel_report* out) {
  if (!g || !cfg || !out) return OSGPU_E_BAD_ARGUMENT;
  fresnel_analyze(*g, z, *cfg, cfg->padding, *out);
  return OSGPU_OK;
}

static int fresnel_common(const double* in, double* out, const osgpu_grid* g, double z,
                          const osgpu_fresnel_config* cfg, int32_t precision,
                          osgpu_fresnel_report* report, int conv) {
  int rc;
  if ((rc = check_grid(g)) || (rc = check_precision(precision))) return rc;
  if (!cfg || !in || !out) return OSGPU_E_BAD_ARGUMENT;
  osgpu_fresnel_report r;
  rc = conv ? fresnel_resolve_conv(*g, z, *cfg, r) : fresnel_resolve_tf(*g, z, *cfg, r);
  if (report) *report = r;
  const size_t n = g->nx * g->ny;
  if (rc == -1) return identity_copy(in, out, n);
  if (rc == OSGPU_E_ALIASING_RISK) {
    set_err("sampling criteria not met (Fresnel %s)", conv ? "kernel" : "transfer function");
    return scan_then(in, n, rc);
  }
  if (rc) {
    set_err("invalid Fresnel propagation arguments (status %d)", rc);
    return rc;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  return host_call(c, in, out, n, [&](const void* din, void* dout) {
    PropJob j;
    std::memset(&j, 0, sizeof(j));
    j.engine = conv ? ENG_KSEP : ENG_FRESNEL_TF;
    j.g = *g;
    j.z = z;
    j.Px = r.nx_pad;
    j.Py = r.ny_pad;
    j.medium = 1.0;
    j.d_in = din;
    j.in_c128 = 1;
    j.d_out = dout;
    j.out_c128 = 1;
    return run_prop_dispatch(c, j, precision == OSGPU_F32, c.stream);
  });
}

int osgpu_fresnel_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                            const osgpu_fresnel_config* cfg, int32_t precision,
                            osgpu_fresnel_report* report) {
  return fresnel_common(in, out, g, z, cfg, precision, report, 0);
}

int osgpu_fresnel_propagate_convolution(const double* in, double* out, const osgpu_grid* g,
                                        double z, const osgpu_fresnel_config* cfg,
                                        int32_t precision, osgpu_fresnel_report* report) {
  return fresnel_common(in, out, g, z, cfg, precision, report, 1);
}

// ----------------------------------------------------------- Fraunhofer

int osgpu_fraunhofer_regime_report(const osgpu_grid* g, double z,
                                   const osgpu_fraunhofer_config* cfg,
                                   osgpu_fraunhofer_report* out) {
  if (!g || !cfg || !out) return OSGPU_E_BAD_ARGUMENT;
  fraunhofer_report(*g, z, *cfg, *out);
  return OSGPU_OK;
}

int osgpu_fraunhofer_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                               const osgpu_fraunhofer_config* cfg, int32_t precision,
                               osgpu_fraunhofer_report* report) {
  int rc;
  if ((rc = check_grid(g)) || (rc = check_precision(precision))) return rc;
  if (!cfg || !in || !out) return OSGPU_E_BAD_ARGUMENT;
  osgpu_fraunhofer_report r;
  rc = fraunhofer_resolve(*g, z, *cfg, r);
  if (report) *report = r;
  const size_t n = g->nx * g->ny;
  if (rc == OSGPU_E_REGIME_VIOLATION) {
    set_err("far-field regime criteria not met");
    return scan_then(in, n, rc);
  }
  if (rc) {
    set_err("invalid Fraunhofer propagation arguments (status %d)", rc);
    return rc;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  return host_call(c, in, out, n, [&](const void* din, void* dout) {
    ElementList none;
    std::memset(&none, 0, sizeof(none));
    return precision == OSGPU_F32
               ? run_fraun<float>(c, *g, z, r, none, din, 1, dout, 1, nullptr, 0, c.stream)
               : run_fraun<double>(c, *g, z, r, none, din, 1, dout, 1, nullptr, 0, c.stream);
  });
}

// ----------------------------------------------------- Rayleigh-Sommerfeld

int osgpu_rs_sampling_report(const osgpu_grid* g, double z, const osgpu_rs_config* cfg,
                             osgpu_rs_report* out) {
  if (!g || !cfg || !out) return OSGPU_E_BAD_ARGUMENT;
  rs_analyze(*g, z, cfg->padding, *out);
  return OSGPU_OK;
}

int osgpu_rs_propagate(const double* in, double* out, const osgpu_grid* g, double z,
                       const osgpu_rs_config* cfg, int32_t precision, osgpu_rs_report* report) {
  int rc;
  if ((rc = check_grid(g)) || (rc = check_precision(precision))) return rc;
  if (!cfg || !in || !out) return OSGPU_E_BAD_ARGUMENT;
  osgpu_rs_report r;
  rc = rs_resolve(*g, z, *cfg, r);
  if (report) *report = r;
  const size_t n = g->nx * g->ny;
  if (rc == OSGPU_E_ALIASING_RISK) {
    set_err("sampling criteria not met (RS kernel undersampled)");
    return scan_then(in, n, rc);
  }
  if (rc) {
    set_err("invalid RS propagation arguments (status %d)", rc);
    return rc;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  return host_call(c, in, out, n, [&](const void* din, void* dout) {
    PropJob j;
    std::memset(&j, 0, sizeof(j));
    j.engine = ENG_KSPEC;
    j.g = *g;
    j.z = z;
    j.Px = r.nx_pad;
    j.Py = r.ny_pad;
    j.medium = 1.0;
    j.d_in = din;
    j.in_c128 = 1;
    j.d_out = dout;
    j.out_c128 = 1;
    return run_prop_dispatch(c, j, precision == OSGPU_F32, c.stream);
  });
}

// ------------------------------------------------------------- elements

int osgpu_apply_elements(const double* in, double* out, const osgpu_grid* g,
                         const osgpu_element* els, int32_t n_els, int32_t precision) {
  int rc;
  if ((rc = check_grid(g)) || (rc = check_precision(precision))) return rc;
  if (!in || !out) return OSGPU_E_BAD_ARGUMENT;
  if (g->nx == 0 || g->ny == 0) return OSGPU_E_EMPTY_GRID;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  Elements E;
  if ((rc = build_elements(c, els, n_els, *g, E, c.stream))) return rc;
  if (precision == OSGPU_F32 && (rc = build_fast_tables(c, E.list, *g, E.tables, c.stream)))
    return rc;
  const size_t n = g->nx * g->ny;
  return host_call(c, in, out, n, [&](const void* din, void* dout) {
    ProfScope ps(c, c.stream, PC_APPLY, (double)n * 32);
    cudaError_t e = precision == OSGPU_F32
                        ? launch_apply_elements<float>(din, 1, dout, 1, E.list, (int)g->nx,
                                                       (int)g->ny, g->dx, g->dy, nullptr, c.stream)
                        : launch_apply_elements<double>(din, 1, dout, 1, E.list, (int)g->nx,
                                                        (int)g->ny, g->dx, g->dy, nullptr,
                                                        c.stream);
    return e == cudaSuccess ? OSGPU_OK : cuda_fail(e, "apply_elements");
  });
}

int osgpu_lattice_create(const double* host, uint64_t lnx, uint64_t lny, void** handle) {
  if (!host || !handle) return OSGPU_E_BAD_ARGUMENT;
  if (lnx == 0 || lny == 0) return OSGPU_E_INVALID_GRID;
  const size_t n = lnx * lny;
  for (size_t k = 0; k < n; ++k)
    if (!std::isfinite(host[k])) {
      set_err("lattice value %zu is not finite", k);
      return OSGPU_E_INVALID_PHASE;
    }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc = ensure_init(c);
  if (rc) return rc;
  void* d64 = nullptr;
  float* d32 = nullptr;
  CK(cudaMalloc(&d64, n * sizeof(double)));
  CK(cudaMalloc(reinterpret_cast<void**>(&d32), n * sizeof(float)));
  std::vector<float> h32(n);
  for (size_t k = 0; k < n; ++k) h32[k] = (float)host[k];
  CK(cudaMemcpy(d64, host, n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d32, h32.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  c.lattices[d64] = d32;
  *handle = d64;
  return OSGPU_OK;
}

int osgpu_lattice_destroy(void* handle) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  auto it = c.lattices.find(handle);
  if (it == c.lattices.end()) return OSGPU_E_BAD_ARGUMENT;
  CK(cudaDeviceSynchronize());
  cudaFree(it->second);
  cudaFree(handle);
  c.lattices.erase(it);
  return OSGPU_OK;
}

// ------------------------------------------------------------- beamline

}  // extern "C"

namespace {

// Validates every step of one beamline in trace order (beamline.rs:109-127):
// element errors, then the engine's; the first failure wins.  Builds the
// device element lists (and the f32 fast tables) and the per-step reports.
int prepare_trace(Context& c, const double* host_in, size_t n, const osgpu_grid& g,
                  const osgpu_step* steps, int n_steps, const osgpu_asm_config& cfg, int f32,
                  std::vector<Elements>& E, std::vector<osgpu_asm_report>& R, cudaStream_t st) {
  E.clear();
  E.resize(n_steps > 0 ? n_steps : 0);
  R.assign(n_steps > 0 ? n_steps : 0, osgpu_asm_report());
  int first_prop = -1;
  for (int s = 0; s < n_steps; ++s) {
    int rc = build_elements(c, steps[s].elements, steps[s].n_elements, g, E[s], st);
    if (rc) {
      if (first_prop >= 0 && first_prop < s) rc = scan_then(host_in, n, rc);
      return rc;
    }
    if (!f32)
      for (int q = 0; q < E[s].list.count; ++q)
        if ((E[s].list.el[q].kind == EL_PHASE || E[s].list.el[q].kind == EL_SCREEN) &&
            !E[s].list.el[q].lat) {
          set_err("step %d: an f32 device lattice needs the f32 engine", s);
          return OSGPU_E_BAD_ARGUMENT;
        }
    if (f32 && (rc = build_fast_tables(c, E[s].list, g, E[s].tables, st))) return rc;
    std::memset(&R[s], 0, sizeof(R[s]));
    if (steps[s].z_after != 0.0) {
      osgpu_asm_config sc = cfg;
      sc.medium = steps[s].medium;
      rc = asm_resolve(g, steps[s].z_after, sc, R[s]);
      if (rc > 0) {
        if (rc == OSGPU_E_ALIASING_RISK || (first_prop >= 0 && first_prop < s))
          rc = scan_then(host_in, n, rc);
        set_err("beamline step %d: propagation failed (status %d)", s, rc);
        return rc;
      }
      if (first_prop < 0) first_prop = s;
      PropJob pj;
      fill_asm_job(pj, g, steps[s].z_after, R[s], sc);
      if ((rc = prebuild_tables(c, pj, !f32, E[s].prop_tables, st))) return rc;
    }
  }
  // f32: the element chain in front of each propagation as one transmission
  // per sample (built here, on the preparing stream; pass A multiplies by it)
  if (f32) {
    ElementList pend;
    std::memset(&pend, 0, sizeof(pend));
    bool ok = true;
    for (int s = 0; s < n_steps; ++s) {
      for (int q = 0; q < E[s].list.count; ++q) {
        if (pend.count == kMaxElements) {  // run_trace applies these on their own
          ok = false;
          pend.count = 0;
        }
        pend.el[pend.count++] = E[s].list.el[q];
        ok = ok && E[s].list.fast;
      }
      if (steps[s].z_after != 0.0) {
        if (ok && pend.count > 0) {
          pend.fast = 1;
          const size_t ns = (size_t)g.nx * g.ny;
          CK(E[s].trans.alloc(ns * sizeof(float2), st));
          ProfScope ps(c, st, PC_ELEMENTS, 0.0);
          CK(launch_transmission(pend, (int)g.nx, (int)g.ny,
                                 reinterpret_cast<float2*>(E[s].trans.p), st));
        }
        pend.count = 0;
        ok = true;
      }
    }
  }
  return OSGPU_OK;
}

// Runs one prepared beamline on the device: elements of consecutive planes
// are merged and fused into the first pass of the propagation that follows
// them; trailing elements run as one element kernel.
int run_trace(Context& c, const void* d_in, int in_c128, void* d_out, int out_c128,
              const osgpu_grid& g, const osgpu_step* steps, int n_steps, std::vector<Elements>& E,
              const std::vector<osgpu_asm_report>& R, const osgpu_asm_config& cfg, int f32,
              cudaStream_t st) {
  const size_t n = g.nx * g.ny;
  const size_t es = f32 ? 8 : 16;
  DBuf work;
  CK(work.alloc(n * es, st));
  int last_prop = -1;
  for (int s = 0; s < n_steps; ++s)
    if (steps[s].z_after != 0.0) last_prop = s;
  bool tail_elements = false;
  for (int s = last_prop + 1; s < n_steps; ++s)
    if (E[s].list.count) tail_elements = true;

  auto apply = [&](const void* src, int src_c, void* dst, int dst_c, const ElementList& L) {
    ProfScope ps(c, st, PC_APPLY, (double)n * ((src_c ? 16 : 8) + (dst_c ? 16 : 8)));
    cudaError_t e =
        f32 ? launch_apply_elements<float>(src, src_c, dst, dst_c, L, (int)g.nx, (int)g.ny, g.dx,
                                           g.dy, c.d_status, st)
            : launch_apply_elements<double>(src, src_c, dst, dst_c, L, (int)g.nx, (int)g.ny,
                                            g.dx, g.dy, c.d_status, st);
    return e == cudaSuccess ? OSGPU_OK : cuda_fail(e, "apply_elements");
  };

  const void* src = d_in;
  int src_c = in_c128;
  ElementList pending;
  std::memset(&pending, 0, sizeof(pending));
  bool pending_fast = true;
  int rc;
  for (int s = 0; s < n_steps; ++s) {
    for (int q = 0; q < E[s].list.count; ++q) {
      if (pending.count == kMaxElements) {
        pending.fast = f32 && pending_fast;
        if ((rc = apply(src, src_c, work.p, !f32, pending))) return rc;
        src = work.p;
        src_c = !f32;
        pending.count = 0;
        pending_fast = true;
      }
      pending.el[pending.count++] = E[s].list.el[q];
      pending_fast = pending_fast && E[s].list.fast;
    }
    if (steps[s].z_after != 0.0) {
      osgpu_asm_config sc = cfg;
      sc.medium = steps[s].medium;
      PropJob j;
      fill_asm_job(j, g, steps[s].z_after, R[s], sc);
      j.tables_pre = E[s].prop_tables.p;
      j.trans = reinterpret_cast<const float2*>(E[s].trans.p);
      pending.fast = f32 && pending_fast;
      j.els = pending;
      j.d_in = src;
      j.in_c128 = src_c;
      const bool final_write = (s == last_prop && !tail_elements);
      j.d_out = final_write ? d_out : work.p;
      j.out_c128 = final_write ? out_c128 : !f32;
      if ((rc = run_prop_dispatch(c, j, f32, st))) return rc;
      src = j.d_out;
      src_c = j.out_c128;
      pending.count = 0;
      pending_fast = true;
    }
  }
  if (pending.count > 0 || src != d_out) {
    pending.fast = f32 && pending_fast;
    if ((rc = apply(src, src_c, d_out, out_c128, pending))) return rc;
  }
  return OSGPU_OK;
}

}  // namespace

extern "C" {

int osgpu_beamline_trace(const double* in, double* out, const osgpu_grid* g,
                         const osgpu_step* steps, int32_t n_steps, const osgpu_asm_config* cfg,
                         int32_t precision, osgpu_asm_report* reports) {
  int rc;
  if ((rc = check_grid(g)) || (rc = check_precision(precision))) return rc;
  if (!cfg || !in || !out || n_steps < 0 || (n_steps > 0 && !steps)) return OSGPU_E_BAD_ARGUMENT;
  if (g->nx == 0 || g->ny == 0) return OSGPU_E_EMPTY_GRID;
  const size_t n = g->nx * g->ny;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  const int f32 = precision == OSGPU_F32;
  std::vector<Elements> E;
  std::vector<osgpu_asm_report> R;
  rc = prepare_trace(c, in, n, *g, steps, n_steps, *cfg, f32, E, R, c.stream);
  if (reports)
    for (int s = 0; s < n_steps && s < (int)R.size(); ++s) reports[s] = R[s];
  if (rc) {
    cudaStreamSynchronize(c.stream);
    return rc;
  }
  return host_call(c, in, out, n, [&](const void* din, void* dout) {
    return run_trace(c, din, 1, dout, 1, *g, steps, n_steps, E, R, *cfg, f32, c.stream);
  });
}

int osgpu_beamline_trace_batch(const osgpu_host_trace_item* items, int32_t n_items,
                               const osgpu_asm_config* cfg, int32_t precision,
                               osgpu_asm_report* reports, int32_t reports_stride) {
  int rc;
  if ((rc = check_precision(precision))) return rc;
  if (!cfg || n_items < 0 || (n_items > 0 && !items)) return OSGPU_E_BAD_ARGUMENT;
  size_t max_n = 0;
  for (int i = 0; i < n_items; ++i) {
    const osgpu_host_trace_item& it = items[i];
    if (!it.in || !it.out || it.n_steps < 0 || (it.n_steps > 0 && !it.steps))
      return OSGPU_E_BAD_ARGUMENT;
    if (it.grid.nx == 0 || it.grid.ny == 0) return OSGPU_E_EMPTY_GRID;
    max_n = std::max(max_n, (size_t)(it.grid.nx * it.grid.ny));
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  if (!c.copy_in) {
    CK(cudaStreamCreateWithFlags(&c.copy_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c.copy_out, cudaStreamNonBlocking));
  }
  const int f32 = precision == OSGPU_F32;
  const cudaStream_t cs = c.stream, si = c.copy_in, so = c.copy_out;
  // Items alternate over the compute lanes (Lanes); each lane has two device
  // slots each way, and the copy streams run ahead of the compute lanes.  The
  // slots hold the caller's complex128 samples; the f32 engine converts on
  // its first pass's loads and its last pass's stores (the same roundings as
  // a separate conversion, without its extra pass over the field)
  const int n_lanes = Lanes::want(c, n_items);
  const int S = 2 * n_lanes;  // slot of item i: i % S, lane: i % n_lanes
  DBuf din[4], dout[4];
  for (int k = 0; k < S; ++k) {
    CK(din[k].alloc(max_n * 16, cs));
    CK(dout[k].alloc(max_n * 16, cs));
  }
  CK(cudaMemsetAsync(c.d_status, 0, sizeof(int), cs));
  CK(cudaStreamSynchronize(cs));  // slots allocated before the copy streams use them
  // element tables of item i on the lane's auxiliary stream, overlapped with item i - lanes
  Lanes lanes;
  if ((rc = lanes.fork(c, cs, n_lanes))) return rc;
  cudaEvent_t ev_in[4], ev_comp[4], ev_out[4];
  for (int k = 0; k < S; ++k) {
    CK(cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_comp[k], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_out[k], cudaEventDisableTiming));
  }
  auto release = [&]() {
    cudaStreamSynchronize(si);
    for (int l = 0; l < lanes.n; ++l) {
      cudaStreamSynchronize(lanes.aux[l].ax);
      cudaStreamSynchronize(lanes.ls[l]);
    }
    cudaStreamSynchronize(so);
    for (int k = 0; k < S; ++k) {
      cudaEventDestroy(ev_in[k]);
      cudaEventDestroy(ev_comp[k]);
      cudaEventDestroy(ev_out[k]);
    }
  };
  for (int i = 0; i < n_items; ++i) {
    const osgpu_host_trace_item& it = items[i];
    const int k = i % S;
    const int l = i % lanes.n;
    AuxTables& aux = lanes.aux[l];
    const cudaStream_t ls = lanes.ls[l];
    const size_t bytes = (size_t)(it.grid.nx * it.grid.ny) * 16;
    if ((rc = aux.begin())) {
      release();
      return rc;
    }
    std::vector<Elements> E;
    std::vector<osgpu_asm_report> R;
    rc = prepare_trace(c, it.in, bytes / 16, it.grid, it.steps, it.n_steps, *cfg, f32, E, R,
                       aux.ax);
    if (reports && reports_stride > 0)
      for (int s = 0; s < it.n_steps && s < reports_stride && s < (int)R.size(); ++s)
        reports[(size_t)i * reports_stride + s] = R[s];
    if (rc) {
      set_err("item %d: %s", i, t_err);
      release();
      return rc;
    }
    if ((rc = aux.ready())) {
      release();
      return rc;
    }
    std::vector<Elements>& Ei = aux.take(E);
    cudaError_t e = cudaSuccess;
    if (i >= S) e = cudaStreamWaitEvent(si, ev_comp[k], 0);  // slot k read by item i - S
    if (e == cudaSuccess) e = cudaMemcpyAsync(din[k].p, it.in, bytes, cudaMemcpyHostToDevice, si);
    if (e == cudaSuccess) e = cudaEventRecord(ev_in[k], si);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ls, ev_in[k], 0);
    if (e == cudaSuccess && i >= S) e = cudaStreamWaitEvent(ls, ev_out[k], 0);  // out slot drained
    if (e != cudaSuccess) {
      release();
      return cuda_fail(e, "batch copy in");
    }
    if ((rc = run_trace(c, din[k].p, 1, dout[k].p, 1, it.grid, it.steps, it.n_steps, Ei, R,
                        *cfg, f32, ls))) {
      release();
      return rc;
    }
    e = cudaEventRecord(ev_comp[k], ls);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(so, ev_comp[k], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(it.out, dout[k].p, bytes, cudaMemcpyDeviceToHost, so);
    if (e == cudaSuccess) e = cudaEventRecord(ev_out[k], so);
    if (e == cudaSuccess && (rc = aux.end())) {
      release();
      return rc;
    }
    if (e != cudaSuccess) {
      release();
      return cuda_fail(e, "batch copy out");
    }
  }
  if ((rc = lanes.finish())) {
    release();
    return rc;
  }
  lanes.join();
  int status = 0;
  cudaError_t e = cudaStreamSynchronize(so);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, cs);
  release();
  if (e != cudaSuccess) return cuda_fail(e, "batch sync");
  if (status & 1) {
    // reported here: clear it, so a later osgpu_sync_status does not see it again
    CK(cudaMemset(c.d_status, 0, sizeof(int)));
    set_err("a field of the batch contains non-finite samples");
    return OSGPU_E_NON_FINITE_SAMPLE;
  }
  return OSGPU_OK;
}

int osgpu_beamline_trace_batch_device(const osgpu_trace_item* items, int32_t n_items,
                                      const osgpu_asm_config* cfg, int32_t dtype, void* stream,
                                      osgpu_asm_report* reports, int32_t reports_stride) {
  if (!items || n_items < 0 || !cfg || (dtype != OSGPU_C128 && dtype != OSGPU_C64))
    return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f32 = dtype == OSGPU_C64;
  const int c128 = dtype == OSGPU_C128;
  for (int i = 0; i < n_items; ++i) {
    const osgpu_trace_item& it = items[i];
    if (!it.d_in || !it.d_out || it.n_steps < 0 || (it.n_steps > 0 && !it.steps))
      return OSGPU_E_BAD_ARGUMENT;
    if (it.grid.nx == 0 || it.grid.ny == 0) return OSGPU_E_EMPTY_GRID;
  }
  // Items are independent: they alternate over two lanes (Lanes).  The
  // schedule key keeps the lane count of the unprofiled run, so a profiled
  // pass times the kernels that run otherwise.
  const char* lenv = getenv("OSGPU_LANES");
  const int lanes_key = (n_items > 1 && !(lenv && atoi(lenv) == 1)) ? 2 : 1;
  if (c.autotune && !c.tuning) {
    // measure the pass schedule of every geometry not seen yet (not while the
    // stream is being captured: tuning synchronises)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cap));
    if (cap == cudaStreamCaptureStatusNone && f32)
      for (int i = 0; i < n_items; ++i)
        for (int s = 0; s < items[i].n_steps; ++s) {
          if (items[i].steps[s].z_after == 0.0) continue;
          osgpu_asm_config sc = *cfg;
          sc.medium = items[i].steps[s].medium;
          if ((rc = tune_geometry(c, items[i].grid, items[i].steps[s].z_after, sc, lanes_key,
                                  st)))
            return rc;
        }
  }
  struct LaneMode {  // the schedule key of this batch's propagations
    Context& c;
    int old;
    LaneMode(Context& c_, int l) : c(c_), old(c_.lane_mode) { c.lane_mode = l; }
    ~LaneMode() { c.lane_mode = old; }
  } lane_mode(c, lanes_key);
  Lanes lanes;
  if ((rc = lanes.fork(c, st, Lanes::want(c, n_items)))) return rc;
  for (int i = 0; i < n_items; ++i) {
    const osgpu_trace_item& it = items[i];
    AuxTables& ax = lanes.aux[i % lanes.n];
    if ((rc = ax.begin())) return rc;
    std::vector<Elements> E;
    std::vector<osgpu_asm_report> R;
    rc = prepare_trace(c, nullptr, 0, it.grid, it.steps, it.n_steps, *cfg, f32, E, R, ax.ax);
    if (reports && reports_stride > 0)
      for (int s = 0; s < it.n_steps && s < reports_stride && s < (int)R.size(); ++s)
        reports[(size_t)i * reports_stride + s] = R[s];
    if (rc) {
      set_err("batch item %d: %s", i, t_err);
      return rc;
    }
    if ((rc = ax.ready())) return rc;
    std::vector<Elements>& Ei = ax.take(E);
    if ((rc = run_trace(c, it.d_in, c128, it.d_out, c128, it.grid, it.steps, it.n_steps, Ei, R,
                        *cfg, f32, lanes.ls[i % lanes.n])))
      return rc;
    if ((rc = ax.end())) return rc;
  }
  rc = lanes.finish();
  lanes.join();
  return rc;
}

}  // extern "C"

namespace {

// Measured pass schedule of one f32 ASM geometry (the counterpart of the
// reference's per-call FftPlanner, fft.rs:41,53, run once per geometry): a
// synthetic batch of that geometry (`lanes` = 1: one item; 2: four items on
// the two lanes, as a batch runs them) with one element plane, so the chain
// transmission exists as in a beamline, is timed with CUDA events under each
// candidate variant of pass A, then B, then C (coordinate descent from the
// built-in defaults; a candidate must beat the current choice by 2 %).
// Every variant computes the same transform; only the kernel differs.
int tune_geometry(Context& c, const osgpu_grid& g, double z, const osgpu_asm_config& cfg,
                  int lanes, cudaStream_t st) {
  osgpu_asm_report r;
  int rc = asm_resolve(g, z, cfg, r);
  if (rc == -1) return OSGPU_OK;  // z == 0: nothing to propagate
  if (rc > 0) return OSGPU_OK;    // the real call reports the error
  const AxisPlan ax = make_axis((int)g.nx, (int)r.nx_pad), ay = make_axis((int)g.ny, (int)r.ny_pad);
  if (ax.nst < 0 || ay.nst < 0 || !reg_fft_size(ax.m) || !reg_fft_size(ay.m)) return OSGPU_OK;
  const std::array<int, 7> key = {ax.m, ax.r, ay.m, ay.r, (int)g.nx, (int)g.ny, lanes};
  if (c.tuned.count(key)) return OSGPU_OK;
  const int n_items = lanes == 2 ? 4 : 1;
  const size_t n = g.nx * g.ny;
  DBuf fin, fout;
  CK(fin.alloc(n * 8, st));
  CK(fout.alloc(n * 8 * n_items, st));
  CK(cudaMemsetAsync(fin.p, 0, n * 8, st));
  osgpu_element ap;
  std::memset(&ap, 0, sizeof(ap));
  ap.kind = OSGPU_EL_RECTANGULAR_APERTURE;
  ap.stop = OSGPU_STOP_FIELD;
  ap.a = ((double)g.nx - 1.0) / 2.0 * g.dx;
  ap.b = ((double)g.ny - 1.0) / 2.0 * g.dy;
  const osgpu_step step = {&ap, 1, z, cfg.medium};
  std::vector<osgpu_trace_item> items(n_items);
  for (int i = 0; i < n_items; ++i)
    items[i] = osgpu_trace_item{fin.p, static_cast<char*>(fout.p) + i * n * 8, g, &step, 1};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  struct Guard {
    Context& c;
    cudaEvent_t a, b;
    bool plans_on;
    ~Guard() {
      c.tuning = false;
      c.force_on = false;
      c.plans_on = plans_on;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } guard{c, e0, e1, c.plans_on};
  c.tuning = true;
  // the synthetic batch runs the padded passes of the key's geometry (with
  // kernel-spectrum plans on, its propagations would run another geometry)
  c.plans_on = false;
  auto measure = [&](const Schedule& s, double* ms) -> int {
    c.force_on = true;
    c.force = s;
    int rc2 = osgpu_beamline_trace_batch_device(items.data(), n_items, &cfg, OSGPU_C64, st,
                                                nullptr, 0);  // warm-up
    if (rc2) return rc2;
    CK(cudaEventRecord(e0, st));
    for (int rep = 0; rep < 3; ++rep)
      if ((rc2 = osgpu_beamline_trace_batch_device(items.data(), n_items, &cfg, OSGPU_C64, st,
                                                   nullptr, 0)))
        return rc2;
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / 3.0;
    return OSGPU_OK;
  };
  Schedule best = {0, 0, 0};
  double t_best = 0.0;
  if ((rc = measure(best, &t_best))) return rc;
  const double t_default = t_best;
  for (int pass = 0; pass < 3; ++pass)
    for (int v = 1; v < sched_count(pass); ++v) {
      Schedule cand = best;
      (pass == 0 ? cand.a : pass == 1 ? cand.b : cand.c) = v;
      double t = 0.0;
      if ((rc = measure(cand, &t))) return rc;
      if (t < 0.98 * t_best) {
        best = cand;
        t_best = t;
      }
    }
  c.tuned[key] = Context::Tuned{best, t_default, t_best};
  ++c.tunes;
  return OSGPU_OK;
}

void fill_info(osgpu_schedule_info& o, const std::array<int, 7>& k, const Context::Tuned& t) {
  std::memset(&o, 0, sizeof(o));
  o.mx = k[0];
  o.rx = k[1];
  o.my = k[2];
  o.ry = k[3];
  o.nx = k[4];
  o.ny = k[5];
  o.lanes = k[6];
  std::snprintf(o.pass_a, sizeof(o.pass_a), "%s", sched_name(0, t.s.a));
  std::snprintf(o.pass_b, sizeof(o.pass_b), "%s", sched_name(1, t.s.b));
  std::snprintf(o.pass_c, sizeof(o.pass_c), "%s", sched_name(2, t.s.c));
  o.ms_default = t.ms_default;
  o.ms_best = t.ms_best;
}

}  // namespace

extern "C" {

int osgpu_autotune_config(int32_t enable) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  c.autotune = enable != 0;
  return OSGPU_OK;
}

int osgpu_autotune_asm(const osgpu_grid* g, double z, const osgpu_asm_config* cfg, int32_t lanes,
                       osgpu_schedule_info* out) {
  if (!g || !cfg || (lanes != 1 && lanes != 2)) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  if ((rc = tune_geometry(c, *g, z, *cfg, lanes, c.stream))) return rc;
  osgpu_asm_report r;
  if (asm_resolve(*g, z, *cfg, r) != 0) return OSGPU_E_BAD_ARGUMENT;
  const AxisPlan ax = make_axis((int)g->nx, (int)r.nx_pad);
  const AxisPlan ay = make_axis((int)g->ny, (int)r.ny_pad);
  const auto it = c.tuned.find({ax.m, ax.r, ay.m, ay.r, (int)g->nx, (int)g->ny, lanes});
  if (it == c.tuned.end()) {
    set_err("geometry has no f32 register-FFT schedule to tune");
    return OSGPU_E_UNSUPPORTED;
  }
  if (out) fill_info(*out, it->first, it->second);
  return OSGPU_OK;
}

int osgpu_autotune_list(osgpu_schedule_info* out, int32_t max_out, int32_t* n_out) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int n = 0;
  for (const auto& kv : c.tuned) {
    if (out && n < max_out) fill_info(out[n], kv.first, kv.second);
    ++n;
  }
  if (n_out) *n_out = n;
  return OSGPU_OK;
}

int osgpu_autotune_clear(void) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  c.tuned.clear();
  return OSGPU_OK;
}

// ------------------------------------------------------------ graphs

int osgpu_beamline_trace_batch_graph(const osgpu_trace_item* items, int32_t n_items,
                                     const osgpu_asm_config* cfg, int32_t dtype,
                                     osgpu_graph** out) {
  if (!out) return OSGPU_E_BAD_ARGUMENT;
  *out = nullptr;
  for (int i = 0; i < n_items && items; ++i)
    for (int s = 0; s < items[i].n_steps; ++s)
      for (int q = 0; q < items[i].steps[s].n_elements; ++q) {
        const osgpu_element& e = items[i].steps[s].elements[q];
        if ((e.kind == OSGPU_EL_PHASE_MASK_SAMPLED || e.kind == OSGPU_EL_GRID_SCREEN) &&
            !e.lattice_on_device) {
          set_err("item %d: a host-memory lattice cannot be captured", i);
          return OSGPU_E_BAD_ARGUMENT;
        }
      }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  // warm-up run: twiddle tables and kernel attributes are created outside capture
  if ((rc = osgpu_beamline_trace_batch_device(items, n_items, cfg, dtype, c.stream, nullptr, 0)))
    return rc;
  CK(cudaStreamSynchronize(c.stream));
  cudaStream_t cs = nullptr;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  const bool prof = c.profiling;
  c.profiling = false;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess)
    rc = osgpu_beamline_trace_batch_device(items, n_items, cfg, dtype, cs, nullptr, 0);
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
  c.profiling = prof;
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  osgpu_graph* g = new osgpu_graph();
  g->exec = exec;
  g->kernels = 0;
  *out = g;
  return OSGPU_OK;
}

int osgpu_graph_launch(osgpu_graph* graph, void* stream) {
  if (!graph || !graph->exec) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  CK(cudaGraphLaunch(graph->exec, st));
  return OSGPU_OK;
}

int osgpu_graph_destroy(osgpu_graph* graph) {
  if (!graph) return OSGPU_OK;
  if (graph->exec) cudaGraphExecDestroy(graph->exec);
  delete graph;
  return OSGPU_OK;
}

// ------------------------------------------------------------ inverse loops

int osgpu_tape_create(uint64_t budget_bytes, osgpu_tape** out) {
  if (!out) return OSGPU_E_BAD_ARGUMENT;
  *out = new osgpu_tape();
  (*out)->budget = budget_bytes;
  return OSGPU_OK;
}

int osgpu_tape_destroy(osgpu_tape* t) {
  if (!t) return OSGPU_OK;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if (t->buf) cudaFree(t->buf);
  delete t;
  return OSGPU_OK;
}

uint64_t osgpu_tape_bytes(const osgpu_tape* t) { return t ? (uint64_t)t->cap : 0; }

int osgpu_render_batch_device(const osgpu_frame* frames, int32_t n_frames,
                              const osgpu_asm_config* cfg, int32_t dtype, void* stream,
                              osgpu_tape* tape, osgpu_asm_report* reports,
                              int32_t reports_stride) {
  int rc;
  if (!cfg) return OSGPU_E_BAD_ARGUMENT;
  if ((rc = check_frames(frames, n_frames, dtype))) return rc;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f32 = dtype == OSGPU_C64, c128 = dtype == OSGPU_C128;
  const size_t es = c128 ? 16 : 8;
  bool record = false;
  if (tape) {
    tape->valid = 0;
    size_t need = 0;
    tape->off.assign(n_frames, 0);
    tape->planes.assign(n_frames, 0);
    tape->nfld.assign(n_frames, 0);
    for (int f = 0; f < n_frames; ++f) {
      tape->off[f] = need;
      tape->planes[f] = count_props(frames[f]);
      tape->nfld[f] = frames[f].grid.nx * frames[f].grid.ny;
      need += (size_t)tape->planes[f] * ((tape->nfld[f] * es + 255) & ~(size_t)255);
    }
    if (tape->budget == 0 || need <= tape->budget) {
      if (need > tape->cap) {
        CK(cudaStreamSynchronize(st));
        if (tape->buf) CK(cudaFree(tape->buf));
        tape->buf = nullptr;
        tape->cap = 0;
        CK(cudaMalloc(&tape->buf, need ? need : 256));
        tape->cap = need;
      }
      record = true;
    }
  }
  Lanes lanes;  // frames write their own planes and intensities: independent
  if ((rc = lanes.fork(c, st, Lanes::want(c, n_frames)))) return rc;
  for (int f = 0; f < n_frames; ++f) {
    const osgpu_frame& fr = frames[f];
    AuxTables& aux = lanes.aux[f % lanes.n];
    const cudaStream_t lst = lanes.ls[f % lanes.n];
    if ((rc = aux.begin())) return rc;
    std::vector<Elements> E0;
    std::vector<osgpu_asm_report> R;
    std::vector<Chain> ch;
    rc = prepare_trace(c, nullptr, 0, fr.grid, fr.steps, fr.n_steps, *cfg, f32, E0, R, aux.ax);
    if (reports && reports_stride > 0)
      for (int s = 0; s < fr.n_steps && s < reports_stride && s < (int)R.size(); ++s)
        reports[(size_t)f * reports_stride + s] = R[s];
    if (rc) {
      set_err("frame %d: %s", f, t_err);
      return rc;
    }
    if ((rc = aux.ready())) return rc;
    std::vector<Elements>& E = aux.take(E0);
    if ((rc = make_chains(fr.steps, fr.n_steps, E, f32, ch))) return rc;
    const size_t pl = (fr.grid.nx * fr.grid.ny * es + 255) & ~(size_t)255;
    DBuf work;
    if (!record) CK(work.alloc(pl, lst));
    char* base = record ? reinterpret_cast<char*>(tape->buf) + tape->off[f] : nullptr;
    auto plane = [&](int k) -> void* {
      return record ? static_cast<void*>(base + (size_t)k * pl) : work.p;
    };
    if ((rc = forward_frame(c, fr, E, R, ch, *cfg, f32, c128, plane, record, lst))) return rc;
    if ((rc = aux.end())) return rc;
  }
  if (record) {
    tape->valid = 1;
    tape->dtype = dtype;
  }
  rc = lanes.finish();
  lanes.join();
  return rc;
}

int osgpu_push_back_batch_device(const osgpu_frame* frames, int32_t n_frames,
                                 const osgpu_asm_config* cfg, int32_t dtype, void* stream,
                                 const osgpu_tape* tape) {
  int rc;
  if (!cfg) return OSGPU_E_BAD_ARGUMENT;
  if ((rc = check_frames(frames, n_frames, dtype))) return rc;
  const bool use_tape = tape && tape->valid;
  if (use_tape) {
    if (tape->dtype != dtype || (int)tape->planes.size() != n_frames) {
      set_err("tape was recorded for another frame list or dtype");
      return OSGPU_E_BAD_ARGUMENT;
    }
    for (int f = 0; f < n_frames; ++f)
      if (tape->planes[f] != count_props(frames[f]) ||
          tape->nfld[f] != frames[f].grid.nx * frames[f].grid.ny) {
        set_err("frame %d does not match the tape", f);
        return OSGPU_E_BAD_ARGUMENT;
      }
  }
  for (int f = 0; f < n_frames; ++f)
    if (!frames[f].d_dmdi) {
      set_err("frame %d: no seed dM/dI", f);
      return OSGPU_E_BAD_ARGUMENT;
    }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f32 = dtype == OSGPU_C64, c128 = dtype == OSGPU_C128;
  const size_t es = c128 ? 16 : 8;
  const size_t rs = c128 ? 8 : 4;  // bytes per gradient value
  Lanes lanes;
  if ((rc = lanes.fork(c, st, Lanes::want(c, n_frames)))) return rc;
  // Frames accumulate into shared gradient arrays (grid_gradient's sum), so
  // the second lane accumulates into zeroed scratch copies of them, added to
  // the caller's arrays once both lanes are done.
  std::map<void*, size_t> gsize;  // caller's gradient array -> values
  std::map<void*, DBuf> gscr;  // caller's array -> lane-2 scratch
  auto lane_grad = [&](void* p, size_t n) -> int {
    if (!p || gscr.count(p)) return OSGPU_OK;
    DBuf& b = gscr[p];
    CK(b.alloc(n * rs, lanes.ls[1]));
    CK(cudaMemsetAsync(b.p, 0, n * rs, lanes.ls[1]));
    gsize[p] = n;
    return OSGPU_OK;
  };
  for (int f = 0; f < n_frames; ++f) {
    const osgpu_frame& fr = frames[f];
    const osgpu_grid& g = fr.grid;
    const int lane = f % lanes.n;
    AuxTables& aux = lanes.aux[lane];
    st = lanes.ls[lane];
    if ((rc = aux.begin())) return rc;
    std::vector<Elements> E0;
    std::vector<osgpu_asm_report> R;
    std::vector<Chain> ch;
    if ((rc = prepare_trace(c, nullptr, 0, g, fr.steps, fr.n_steps, *cfg, f32, E0, R, aux.ax))) {
      set_err("frame %d: %s", f, t_err);
      return rc;
    }
    if ((rc = aux.ready())) return rc;
    std::vector<Elements>& E = aux.take(E0);
    if ((rc = make_chains(fr.steps, fr.n_steps, E, f32, ch))) return rc;
    const int K = (int)ch.size() - 1;
    const size_t pl = (g.nx * g.ny * es + 255) & ~(size_t)255;
    // forward planes: from the tape, or recomputed (reference push_back)
    DBuf planes;
    char* base;
    if (use_tape) {
      base = reinterpret_cast<char*>(tape->buf) + tape->off[f];
    } else {
      CK(planes.alloc(pl * (K > 0 ? K : 1), st));
      base = reinterpret_cast<char*>(planes.p);
      osgpu_frame fw = fr;
      fw.d_intensity = nullptr;
      auto plane = [&](int k) -> void* { return base + (size_t)k * pl; };
      if ((rc = forward_frame(c, fw, E, R, ch, *cfg, f32, c128, plane, true, st))) return rc;
    }
    auto uin = [&](int k) -> const void* {
      return k == 0 ? fr.d_source : static_cast<const void*>(base + (size_t)(k - 1) * pl);
    };
    if (lane == 1)
      for (const Chain& cn : ch)
        for (int q = 0; q < cn.list.count; ++q)
          if (fr.d_grad && (rc = lane_grad(fr.d_grad[cn.flat[q]], g.nx * g.ny))) return rc;
    auto grads = [&](const Chain& cn, void** out) {
      for (int q = 0; q < kMaxElements; ++q) {
        void* p = (q < cn.list.count && fr.d_grad) ? fr.d_grad[cn.flat[q]] : nullptr;
        out[q] = (p && lane == 1) ? gscr[p].p : p;
      }
    };
    const int seed_f64 = c128;
    DBuf mu;
    CK(mu.alloc(pl, st));
    const Chain& tail = ch[K];
    bool seeded = false;
    if (K == 0 || tail.list.count > 0) {
      AdjGrads ag;
      grads(tail, ag.p);
      ProfScope ps(c, st, PC_APPLY, (double)g.nx * g.ny * (2.0 * es + (c128 ? 8 : 4)));
      CK(launch_adjoint_seed_plane(uin(K), c128, tail.list, ag, fr.d_dmdi, seed_f64,
                                   fr.dmdi_scale, (int)g.nx, (int)g.ny, g.dx, g.dy,
                                   K > 0 ? mu.p : nullptr, c128, f32, st));
      seeded = true;
    }
    for (int k = K - 1; k >= 0; --k) {
      const Chain& cn = ch[k];
      if (k == 0 && cn.list.count == 0) break;  // nothing left to differentiate
      const int s = cn.prop_step;
      osgpu_asm_config sc = *cfg;
      sc.medium = fr.steps[s].medium;
      osgpu_asm_report ra;
      const double z = -fr.steps[s].z_after;  // asm_adjoint: A(z)^dagger = A(-z)
      if ((rc = asm_resolve(g, z, sc, ra)) > 0) {
        set_err("frame %d step %d: adjoint propagation failed (status %d)", f, s, rc);
        return rc;
      }
      PropJob j;
      fill_asm_job(j, g, z, ra, sc);
      if (!seeded) {
        j.d_in = uin(K);
        j.seed = fr.d_dmdi;
        j.seed_f64 = seed_f64;
        j.seed_scale = fr.dmdi_scale;
        seeded = true;
      } else {
        j.d_in = mu.p;
      }
      j.in_c128 = c128;
      j.els = cn.list;
      j.trans = reinterpret_cast<const float2*>(E[s].trans.p);
      j.adj = cn.list.count > 0;
      j.adj_uin = uin(k);
      j.adj_uin_c128 = c128;
      grads(cn, j.adj_grad);
      j.d_out = k > 0 ? mu.p : nullptr;
      j.out_c128 = c128;
      if ((rc = run_prop_dispatch(c, j, f32, st))) return rc;
    }
    if ((rc = aux.end())) return rc;
  }
  st = lanes.ls[0];
  if ((rc = lanes.finish())) return rc;
  lanes.join();
  for (auto& kv : gscr) {  // the second lane's sums into the caller's arrays
    CK(launch_add_real(kv.first, kv.second.p, c128, gsize[kv.first], st));
    kv.second.s = st;  // freed after the add, in the caller's stream order
  }
  return OSGPU_OK;
}

namespace {
int merit_sync(cudaStream_t st, const DBuf& buf, double* host, int n) {
  CK(cudaMemcpyAsync(host, buf.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return OSGPU_OK;
}
}  // namespace

int osgpu_field_power_device(const void* d_field, int32_t dtype, uint64_t n, void* stream,
                             double* out) {
  if (!d_field || !out || (dtype != OSGPU_C128 && dtype != OSGPU_C64))
    return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  DBuf scr;
  CK(scr.alloc(reduce_scratch_bytes(1), st));
  double* part = reinterpret_cast<double*>(scr.p);
  double* res = part + (reduce_scratch_bytes(1) / sizeof(double) - 3);
  CK(launch_power(d_field, dtype == OSGPU_C128, n, part, res, st));
  CK(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return OSGPU_OK;
}

namespace {
int psf_check(const void* d, int32_t real_dtype, const osgpu_grid* g) {
  if (!d || !g || (real_dtype != OSGPU_F64 && real_dtype != OSGPU_F32)) {
    set_err("bad detector grid arguments");
    return OSGPU_E_BAD_ARGUMENT;
  }
  if (g->nx == 0 || g->ny == 0) {
    set_err("empty detector grid");
    return OSGPU_E_EMPTY_GRID;
  }
  if (!(g->dx > 0.0) || !(g->dy > 0.0) || !std::isfinite(g->dx) || !std::isfinite(g->dy)) {
    set_err("detector pitch must be positive and finite");
    return OSGPU_E_BAD_ARGUMENT;
  }
  return OSGPU_OK;
}
}  // namespace

int osgpu_psf_spot_rms_device(const void* d_int, int32_t real_dtype, const osgpu_grid* g,
                              void* stream, double* out_m) {
  int rc;
  if ((rc = psf_check(d_int, real_dtype, g))) return rc;
  if (!out_m) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  DBuf scr;
  const size_t sb = reduce_scratch_bytes(2);
  CK(scr.alloc(sb, st));
  double* part = reinterpret_cast<double*>(scr.p);
  double* res = part + (sb / sizeof(double) - 4);
  CK(launch_psf_moments(d_int, real_dtype == OSGPU_F64, (int)g->nx, (int)g->ny, g->dx, g->dy,
                        part, res, st));
  double h[2];
  CK(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *out_m = h[0] > 0.0 ? std::sqrt(h[1] / h[0]) : 0.0;  // analysis.rs:124
  return OSGPU_OK;
}

int osgpu_psf_encircled_energy_device(const void* d_int, int32_t real_dtype,
                                      const osgpu_grid* g, void* stream, double* radii,
                                      double* fraction, uint64_t cap, uint64_t* n_out) {
  int rc;
  if ((rc = psf_check(d_int, real_dtype, g))) return rc;
  if (!n_out || (cap > 0 && (!radii || !fraction))) return OSGPU_E_BAD_ARGUMENT;
  const uint64_t n = g->nx * g->ny;
  if (n >= 0xffffffffull) {
    set_err("detector grid too large for the encircled-energy walk");
    return OSGPU_E_UNSUPPORTED;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  Context::EeOrder& E = c.ee;
  if (!(E.d && E.nx == g->nx && E.ny == g->ny && E.dx == g->dx && E.dy == g->dy)) {
    // pixel radii at the centred coordinates (field.rs:490-495), stable sort by
    // radius, one group per run of equal radii (analysis.rs:84-106)
    std::vector<std::pair<double, unsigned>> px(n);
    for (uint64_t iy = 0; iy < g->ny; ++iy) {
      const double y = ((double)iy - ((double)g->ny - 1.0) / 2.0) * g->dy;
      for (uint64_t ix = 0; ix < g->nx; ++ix) {
        const double x = ((double)ix - ((double)g->nx - 1.0) / 2.0) * g->dx;
        px[iy * g->nx + ix] = {std::sqrt(x * x + y * y), (unsigned)(iy * g->nx + ix)};
      }
    }
    std::stable_sort(px.begin(), px.end(),
                     [](const std::pair<double, unsigned>& a, const std::pair<double, unsigned>& b) {
                       return a.first < b.first;
                     });
    std::vector<unsigned> host(n);
    std::vector<unsigned> ends;
    std::vector<double> radii_g;
    for (uint64_t k = 0; k < n; ++k) {
      host[k] = px[k].second;
      if (k + 1 == n || px[k + 1].first != px[k].first) {
        ends.push_back((unsigned)k);
        radii_g.push_back(px[k].first);
      }
    }
    if (E.d) {
      CK(cudaDeviceSynchronize());
      cudaFree(E.d);
      E.d = nullptr;
    }
    CK(cudaMalloc(&E.d, (n + ends.size()) * sizeof(unsigned)));
    CK(cudaMemcpy(E.d, host.data(), n * sizeof(unsigned), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(static_cast<unsigned*>(E.d) + n, ends.data(), ends.size() * sizeof(unsigned),
                  cudaMemcpyHostToDevice));
    E.nx = g->nx;
    E.ny = g->ny;
    E.dx = g->dx;
    E.dy = g->dy;
    E.ng = ends.size();
    E.radii = std::move(radii_g);
  }
  const uint64_t nb = (n + 1023) / 1024;
  DBuf scr;
  CK(scr.alloc((n + nb + E.ng) * sizeof(double), st));
  double* v = reinterpret_cast<double*>(scr.p);
  double* tot = v + n;
  double* frac = tot + nb;
  const unsigned* perm = static_cast<const unsigned*>(E.d);
  double total = 0.0;
  CK(launch_ee_curve(d_int, real_dtype == OSGPU_F64, perm, n, perm + n, E.ng, v, tot, frac,
                     &total, st));
  if (!(total > 0.0)) {  // analysis.rs:95: an empty curve
    *n_out = 0;
    return OSGPU_OK;
  }
  *n_out = E.ng;
  if (cap < E.ng) {
    set_err("curve has %llu points, buffers hold %llu", (unsigned long long)E.ng,
            (unsigned long long)cap);
    return OSGPU_E_BAD_ARGUMENT;
  }
  CK(cudaMemcpyAsync(fraction, frac, E.ng * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::copy(E.radii.begin(), E.radii.end(), radii);
  return OSGPU_OK;
}

int osgpu_psf_mtf_device(const void* d_int, int32_t real_dtype, const osgpu_grid* g,
                         void* stream, double* freqs, double* values) {
  int rc;
  if ((rc = psf_check(d_int, real_dtype, g))) return rc;
  if (!freqs || !values) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int nx = (int)g->nx, half = nx / 2;
  const void* tw = nullptr;
  if ((rc = get_tw(c, nx, 1, &tw))) return rc;
  DBuf scr;
  CK(scr.alloc((size_t)nx * sizeof(double) + (size_t)(half + 1) * sizeof(double2), st));
  double* colsum = reinterpret_cast<double*>(scr.p);
  double2* X = reinterpret_cast<double2*>(colsum + nx);
  CK(launch_row_mtf(d_int, real_dtype == OSGPU_F64, nx, (int)g->ny, tw, colsum, X, st));
  std::vector<double2> hx(half + 1);
  CK(cudaMemcpyAsync(hx.data(), X, hx.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  // analysis.rs:141-150: |X[k]| / max(|X[0]|, MIN_POSITIVE), capped at 1
  const double dc = std::max(std::hypot(hx[0].x, hx[0].y), 2.2250738585072014e-308);
  for (int k = 0; k <= half; ++k) {
    freqs[k] = (double)k / ((double)nx * g->dx);
    values[k] = std::min(std::hypot(hx[k].x, hx[k].y) / dc, 1.0);
  }
  return OSGPU_OK;
}

int osgpu_psf_strehl_device(const void* d_meas, const osgpu_grid* g_meas, const void* d_ref,
                            const osgpu_grid* g_ref, int32_t real_dtype, void* stream,
                            double* out) {
  int rc;
  if ((rc = psf_check(d_meas, real_dtype, g_meas)) || (rc = psf_check(d_ref, real_dtype, g_ref)))
    return rc;
  if (!out) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  // per grid: moment partials (2 frames), then the max partials (1216), results at the tail
  const size_t sb = reduce_scratch_bytes(3);
  DBuf scr;
  CK(scr.alloc(2 * sb, st));
  double h[2][3];
  for (int q = 0; q < 2; ++q) {
    const void* d = q ? d_ref : d_meas;
    const osgpu_grid* g = q ? g_ref : g_meas;
    double* part = reinterpret_cast<double*>(static_cast<char*>(scr.p) + q * sb);
    double* res = part + (sb / sizeof(double) - 4);
    const int f64 = real_dtype == OSGPU_F64;
    CK(launch_psf_moments(d, f64, (int)g->nx, (int)g->ny, g->dx, g->dy, part, res, st));
    CK(launch_psf_max(d, f64, g->nx * g->ny, part + 2 * 1216 * 2, res + 2, st));
    CK(cudaMemcpyAsync(h[q], res, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  // analysis.rs:159-168: (peak_m / P_m) / (peak_r / P_r), P = sum I dx dy
  const double pm = h[0][0] * g_meas->dx * g_meas->dy, pr = h[1][0] * g_ref->dx * g_ref->dy;
  *out = (pm <= 0.0 || pr <= 0.0) ? 0.0 : (h[0][2] / pm) / (h[1][2] / pr);
  return OSGPU_OK;
}

int osgpu_merit_spot_efficiency_device(const void* d_obs, int32_t real_dtype, int32_t n_frames,
                                       uint64_t frame_len, const uint8_t* d_windows,
                                       const double* p_in, void* d_seed, void* stream,
                                       double* value) {
  if (!d_obs || !d_windows || !p_in || n_frames <= 0 || frame_len == 0 ||
      (real_dtype != OSGPU_F64 && real_dtype != OSGPU_F32))
    return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f64 = real_dtype == OSGPU_F64;
  const size_t sb = reduce_scratch_bytes(n_frames);
  DBuf scr, res;
  CK(scr.alloc(sb, st));
  CK(res.alloc(sizeof(double) * 2 * n_frames, st));
  double* sums = reinterpret_cast<double*>(res.p);
  CK(launch_window_sums(d_obs, f64, n_frames, frame_len, d_windows,
                        reinterpret_cast<double*>(scr.p), sums, st));
  if (d_seed) {
    std::vector<double> coef(n_frames);
    for (int f = 0; f < n_frames; ++f) coef[f] = -1.0 / p_in[f];
    CK(cudaMemcpyAsync(sums + n_frames, coef.data(), sizeof(double) * n_frames,
                       cudaMemcpyHostToDevice, st));
    CK(launch_window_seed(d_seed, f64, n_frames, frame_len, d_windows, sums + n_frames, st));
  }
  std::vector<double> h(n_frames);
  if ((rc = merit_sync(st, res, h.data(), n_frames))) return rc;
  if (value) {
    double tot = 0.0;
    for (int f = 0; f < n_frames; ++f) tot += h[f] / p_in[f];
    *value = -tot;
  }
  return OSGPU_OK;
}

int osgpu_merit_weighted_efficiency_device(const void* d_obs, int32_t real_dtype,
                                           int32_t n_frames, uint64_t frame_len,
                                           const void* d_weights, const double* p_in,
                                           void* d_seed, void* stream, double* value) {
  if (!d_obs || !d_weights || !p_in || n_frames <= 0 || frame_len == 0 ||
      (real_dtype != OSGPU_F64 && real_dtype != OSGPU_F32))
    return OSGPU_E_BAD_ARGUMENT;
  for (int f = 0; f < n_frames; ++f)
    if (!(p_in[f] > 0.0) || !std::isfinite(p_in[f])) {
      set_err("frame %d: input power must be positive and finite", f);
      return OSGPU_E_BAD_ARGUMENT;
    }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f64 = real_dtype == OSGPU_F64;
  const size_t sb = reduce_scratch_bytes(n_frames);
  DBuf scr, res;
  CK(scr.alloc(sb, st));
  CK(res.alloc(sizeof(double) * 2 * n_frames, st));
  double* sums = reinterpret_cast<double*>(res.p);
  CK(launch_weighted_sums(d_obs, f64, n_frames, frame_len, d_weights,
                          reinterpret_cast<double*>(scr.p), sums, st));
  if (d_seed) {
    std::vector<double> coef(n_frames);
    for (int f = 0; f < n_frames; ++f) coef[f] = -1.0 / p_in[f];
    CK(cudaMemcpyAsync(sums + n_frames, coef.data(), sizeof(double) * n_frames,
                       cudaMemcpyHostToDevice, st));
    CK(launch_weighted_seed(d_seed, f64, n_frames, frame_len, d_weights, sums + n_frames, st));
  }
  std::vector<double> h(n_frames);
  if ((rc = merit_sync(st, res, h.data(), n_frames))) return rc;
  if (value) {
    double tot = 0.0;
    for (int f = 0; f < n_frames; ++f) tot += h[f] / p_in[f];
    *value = -tot;
  }
  return OSGPU_OK;
}

int osgpu_merit_mse_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                           int32_t n_scenes, uint64_t frame_len, const double* d_target,
                           int32_t band, int32_t scene, void* d_seed, void* stream,
                           double* value) {
  if (!d_obs || !d_target || n_bands <= 0 || n_scenes <= 0 || frame_len == 0 ||
      band >= n_bands || scene >= n_scenes ||
      (real_dtype != OSGPU_F64 && real_dtype != OSGPU_F32))
    return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  DBuf scr, res;
  CK(scr.alloc(reduce_scratch_bytes(1), st));
  CK(res.alloc(sizeof(double), st));
  CK(launch_mse(d_obs, real_dtype == OSGPU_F64, frame_len, n_bands, n_scenes, band, scene,
                d_target, d_seed, reinterpret_cast<double*>(scr.p),
                reinterpret_cast<double*>(res.p), st));
  double h = 0.0;
  if ((rc = merit_sync(st, res, &h, 1))) return rc;
  if (value) *value = h / (double)frame_len;
  return OSGPU_OK;
}

int osgpu_merit_encircled_energy_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                                        int32_t n_scenes, uint64_t nx, uint64_t ny, double dx,
                                        double dy, double radius, int32_t band, int32_t scene,
                                        void* d_seed, void* stream, double* value) {
  if (!d_obs || n_bands <= 0 || n_scenes <= 0 || nx == 0 || ny == 0 || band >= n_bands ||
      scene >= n_scenes || (real_dtype != OSGPU_F64 && real_dtype != OSGPU_F32))
    return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  DBuf scr, res;
  CK(scr.alloc(reduce_scratch_bytes(2), st));
  CK(res.alloc(2 * sizeof(double), st));
  double* sums = reinterpret_cast<double*>(res.p);
  CK(launch_ee(d_obs, real_dtype == OSGPU_F64, (int)nx, (int)ny, dx, dy, radius, n_bands,
               n_scenes, band, scene, nullptr, reinterpret_cast<double*>(scr.p), sums, st));
  double h[2];
  if ((rc = merit_sync(st, res, h, 2))) return rc;
  if (value) *value = (h[0] <= 0.0) ? 0.0 : -h[1] / h[0];
  if (d_seed) {
    if (h[0] <= 0.0) {  // obs_gradient is None (merit.rs:222-224)
      set_err("encircled energy: total intensity is not positive, no obs gradient");
      return OSGPU_E_ADJOINT;
    }
    CK(launch_ee(d_obs, real_dtype == OSGPU_F64, (int)nx, (int)ny, dx, dy, radius, n_bands,
                 n_scenes, band, scene, d_seed, reinterpret_cast<double*>(scr.p), sums, st));
  }
  return OSGPU_OK;
}

namespace {
int merit_args(const void* d_obs, int32_t real_dtype, int32_t nb, int32_t ns, uint64_t nx,
               uint64_t ny, int32_t band, int32_t scene) {
  if (!d_obs || nb <= 0 || ns <= 0 || nx == 0 || ny == 0 || band >= nb || scene >= ns ||
      (real_dtype != OSGPU_F64 && real_dtype != OSGPU_F32) || nx > INT32_MAX || ny > INT32_MAX)
    return OSGPU_E_BAD_ARGUMENT;
  return OSGPU_OK;
}

// The frame a merit reads (Selector::frame, merit.rs:47-80): the
// observation's own frame when the selector picks exactly one, else the FP64
// sum of the selected frames, materialised in `buf`.
int merit_frame(const void* d_obs, int f64, int nb, int ns, uint64_t len, int band, int scene,
                DBuf& buf, cudaStream_t st, const void** img, int* img_f64) {
  if ((band >= 0 || nb == 1) && (scene >= 0 || ns == 1)) {
    const size_t f = (size_t)(band >= 0 ? band : 0) * ns + (scene >= 0 ? scene : 0);
    *img = static_cast<const char*>(d_obs) + f * len * (f64 ? sizeof(double) : sizeof(float));
    *img_f64 = f64;
    return OSGPU_OK;
  }
  CK(buf.alloc(len * sizeof(double), st));
  CK(launch_sel_frame(d_obs, f64, len, nb, ns, band, scene, reinterpret_cast<double*>(buf.p),
                      st));
  *img = buf.p;
  *img_f64 = 1;
  return OSGPU_OK;
}
}  // namespace

int osgpu_merit_spot_rms_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                                int32_t n_scenes, uint64_t nx, uint64_t ny, double dx, double dy,
                                int32_t band, int32_t scene, void* d_seed, void* stream,
                                double* value) {
  int rc;
  if ((rc = merit_args(d_obs, real_dtype, n_bands, n_scenes, nx, ny, band, scene))) return rc;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f64 = real_dtype == OSGPU_F64;
  DBuf frame, scr;
  const void* img;
  int img_f64;
  if ((rc = merit_frame(d_obs, f64, n_bands, n_scenes, nx * ny, band, scene, frame, st, &img,
                        &img_f64)))
    return rc;
  const size_t sb = reduce_scratch_bytes(2);
  CK(scr.alloc(sb, st));
  double* part = reinterpret_cast<double*>(scr.p);
  double* res = part + (sb / sizeof(double) - 4);
  CK(launch_psf_moments(img, img_f64, (int)nx, (int)ny, dx, dy, part, res, st));
  double h[2];
  CK(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const double sw = h[0];
  if (value) *value = sw <= 0.0 ? 0.0 : std::sqrt(h[1] / sw);
  if (d_seed) {
    const double rr = h[1] / sw, root = std::sqrt(rr);
    if (sw <= 0.0 || root <= 0.0) {  // obs_gradient is None (merit.rs:291-299)
      set_err("spot rms: total intensity or radius is not positive, no obs gradient");
      return OSGPU_E_ADJOINT;
    }
    CK(launch_spot_seed(d_seed, f64, (int)nx, (int)ny, dx, dy, n_bands, n_scenes, band, scene,
                        rr, 2.0 * root * sw, st));
  }
  return OSGPU_OK;
}

int osgpu_merit_strehl_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                              int32_t n_scenes, uint64_t nx, uint64_t ny,
                              const double* d_reference, int32_t band, int32_t scene,
                              void* stream, double* value) {
  int rc;
  if ((rc = merit_args(d_obs, real_dtype, n_bands, n_scenes, nx, ny, band, scene))) return rc;
  if (!d_reference || !value) return OSGPU_E_BAD_ARGUMENT;
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f64 = real_dtype == OSGPU_F64;
  DBuf frame, scr;
  const void* img;
  int img_f64;
  if ((rc = merit_frame(d_obs, f64, n_bands, n_scenes, nx * ny, band, scene, frame, st, &img,
                        &img_f64)))
    return rc;
  // per grid: moment partials (2 frames), then the max partials, results at the tail
  const size_t sb = reduce_scratch_bytes(3);
  CK(scr.alloc(2 * sb, st));
  double h[2][3];
  for (int q = 0; q < 2; ++q) {
    double* part = reinterpret_cast<double*>(static_cast<char*>(scr.p) + q * sb);
    double* res = part + (sb / sizeof(double) - 4);
    const void* d = q ? static_cast<const void*>(d_reference) : img;
    const int df = q ? 1 : img_f64;
    CK(launch_psf_moments(d, df, (int)nx, (int)ny, 1.0, 1.0, part, res, st));
    CK(launch_psf_max(d, df, nx * ny, part + 2 * 1216 * 2, res + 2, st));
    CK(cudaMemcpyAsync(h[q], res, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  const double pm = h[0][0], pr = h[1][0];
  *value = (pm <= 0.0 || pr <= 0.0) ? 0.0 : -((h[0][2] / pm) / (h[1][2] / pr));
  return OSGPU_OK;
}

int osgpu_merit_mtf_device(const void* d_obs, int32_t real_dtype, int32_t n_bands,
                           int32_t n_scenes, uint64_t nx, uint64_t ny, double dx, double freq,
                           int32_t band, int32_t scene, void* stream, double* value) {
  int rc;
  if ((rc = merit_args(d_obs, real_dtype, n_bands, n_scenes, nx, ny, band, scene))) return rc;
  if (!value) return OSGPU_E_BAD_ARGUMENT;
  if (freq < 0.0 || 2.0 * freq * dx >= 1.0) {
    set_err("MTF frequency beyond Nyquist");
    return OSGPU_E_RENDER;
  }
  // the bin, with the saturating float-to-integer cast of the reference
  // (a NaN frequency lands on bin 0)
  const double kf = freq * (double)nx * dx;
  const double kr = std::round(kf);
  const long long m = std::isnan(kr) ? 0 : (long long)kr;
  if (std::fabs(kf - (double)m) > 1e-9) {
    set_err("MTF frequency must land on a DFT bin (f = m / (nx dx))");
    return OSGPU_E_RENDER;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f64 = real_dtype == OSGPU_F64;
  DBuf frame, scr;
  const void* img;
  int img_f64;
  if ((rc = merit_frame(d_obs, f64, n_bands, n_scenes, nx * ny, band, scene, frame, st, &img,
                        &img_f64)))
    return rc;
  const int half = (int)(nx / 2);
  if (m > half) return OSGPU_E_RENDER;  // excluded by the Nyquist test above
  const void* tw = nullptr;
  if ((rc = get_tw(c, (int)nx, 1, &tw))) return rc;
  CK(scr.alloc(nx * sizeof(double) + (size_t)(half + 1) * sizeof(double2), st));
  double* colsum = reinterpret_cast<double*>(scr.p);
  double2* X = reinterpret_cast<double2*>(colsum + nx);
  CK(launch_row_mtf(img, img_f64, (int)nx, (int)ny, tw, colsum, X, st));
  double2 h[2];
  CK(cudaMemcpyAsync(&h[0], X, sizeof(double2), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&h[1], X + m, sizeof(double2), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const double dc = h[0].x;  // the frame sum
  *value = dc <= 0.0 ? 0.0 : -(std::hypot(h[1].x, h[1].y) / dc);
  return OSGPU_OK;
}

int osgpu_adam_step_device(double* d_x, float* d_x32, const void* d_g, int32_t g_real_dtype,
                           double* d_m, double* d_v, uint64_t n, const osgpu_adam_config* cfg,
                           int32_t t, double lo, double hi, void* stream) {
  if (!d_x || !d_g || !d_m || !d_v || !cfg || t < 1 ||
      (g_real_dtype != OSGPU_F64 && g_real_dtype != OSGPU_F32))
    return OSGPU_E_BAD_ARGUMENT;
  // AdamConfig::validate (fd.rs:95-121)
  if (!std::isfinite(cfg->lr_frac) || !(cfg->lr_frac > 0.0) ||
      !std::isfinite(cfg->beta1) || !(cfg->beta1 >= 0.0 && cfg->beta1 < 1.0) ||
      !std::isfinite(cfg->beta2) || !(cfg->beta2 >= 0.0 && cfg->beta2 < 1.0) ||
      !std::isfinite(cfg->eps) || cfg->eps < 0.0 ||
      (cfg->clip && (!std::isfinite(cfg->clip_norm) || !(cfg->clip_norm > 0.0)))) {
    set_err("invalid Adam config");
    return OSGPU_E_RENDER;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  AdamArgs p;
  p.beta1 = cfg->beta1;
  p.beta2 = cfg->beta2;
  p.eps = cfg->eps;
  p.bc1 = 1.0 - std::pow(cfg->beta1, (double)t);
  p.bc2 = 1.0 - std::pow(cfg->beta2, (double)t);
  p.step = cfg->lr_frac * (hi - lo);
  p.lo = lo;
  p.hi = hi;
  p.clip = cfg->clip;
  p.clip_norm = cfg->clip_norm;
  DBuf scr;
  CK(scr.alloc(reduce_scratch_bytes(1), st));
  double* part = reinterpret_cast<double*>(scr.p);
  double* norm2 = part + (reduce_scratch_bytes(1) / sizeof(double) - 3);
  CK(launch_adam(d_x, d_x32, d_g, g_real_dtype == OSGPU_F64, d_m, d_v, n, p, part, norm2, st));
  return OSGPU_OK;
}

// ------------------------------------------------------------ sources

namespace {
int source_prologue(void* d_out, int32_t dtype, const osgpu_grid* g, Context*& cp,
                    cudaStream_t& st, void* stream) {
  if (!d_out || !g || (dtype != OSGPU_C128 && dtype != OSGPU_C64)) return OSGPU_E_BAD_ARGUMENT;
  if (g->nx == 0 || g->ny == 0) return OSGPU_E_EMPTY_GRID;
  if (!(std::isfinite(g->lambda) && g->lambda > 0.0)) return OSGPU_E_INVALID_WAVELENGTH;
  Context& c = ctx();
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cp = &c;
  st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  return OSGPU_OK;
}
}  // namespace

int osgpu_source_gaussian_device(void* d_out, int32_t dtype, const osgpu_grid* g, double w0,
                                 double amplitude, double center_x, double center_y, double z,
                                 void* stream) {
  Context* c = nullptr;
  cudaStream_t st;
  int rc;
  if ((rc = source_prologue(d_out, dtype, g, c, st, stream))) return rc;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  if (!(std::isfinite(w0) && w0 > 0.0 && std::isfinite(amplitude) && std::isfinite(center_x) &&
        std::isfinite(center_y))) {
    set_err("invalid beam");
    return OSGPU_E_BAD_ARGUMENT;
  }
  if (!std::isfinite(z)) {
    set_err("invalid plane z");
    return OSGPU_E_BAD_ARGUMENT;
  }
  // q-form beam at distance z from the waist (sources.rs:259-296)
  const double lam = g->lambda;
  const double z_r = PI * w0 * w0 / lam;
  const double w_z = w0 * std::sqrt(1.0 + (z / z_r) * (z / z_r));
  const double k = 2.0 * PI / lam;
  const double inv_r = z / (z * z + z_r * z_r);
  const double carrier = k * z - std::atan(z / z_r);
  const double amp = amplitude * w0 / w_z;
  CK(launch_gaussian(d_out, dtype == OSGPU_C128, (int)g->nx, (int)g->ny, g->dx, g->dy, center_x,
                     center_y, amp, w_z * w_z, 0.5 * k, inv_r, carrier, st));
  return OSGPU_OK;
}

int osgpu_source_plane_wave_device(void* d_out, int32_t dtype, const osgpu_grid* g,
                                   double theta_x, double theta_y, double amplitude,
                                   void* stream) {
  Context* c = nullptr;
  cudaStream_t st;
  int rc;
  if ((rc = source_prologue(d_out, dtype, g, c, st, stream))) return rc;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  // BandField::plane_wave (field.rs:360-386)
  const double k = 2.0 * PI / g->lambda;
  CK(launch_plane_wave(d_out, dtype == OSGPU_C128, (int)g->nx, (int)g->ny, g->dx, g->dy,
                       amplitude, k, std::sin(theta_x), std::sin(theta_y), st));
  return OSGPU_OK;
}

int osgpu_source_uniform_device(void* d_out, int32_t dtype, const osgpu_grid* g,
                                double amplitude, double phase, void* stream) {
  Context* c = nullptr;
  cudaStream_t st;
  int rc;
  if ((rc = source_prologue(d_out, dtype, g, c, st, stream))) return rc;
  std::lock_guard<std::recursive_mutex> lk(c->mu);
  // BandField::uniform (field.rs:315-330): A e^{i phase}
  CK(launch_fill(d_out, dtype == OSGPU_C128, (size_t)(g->nx * g->ny),
                 amplitude * std::cos(phase), amplitude * std::sin(phase), st));
  return OSGPU_OK;
}

// ------------------------------------------------------------ Gerchberg-Saxton

int osgpu_gs_run_batch_device(osgpu_gs_item* items, int32_t n_items, const osgpu_gs_config* cfg,
                              const osgpu_asm_config* asm_cfg,
                              const osgpu_fraunhofer_config* fraunhofer_cfg, int32_t dtype,
                              void* stream) {
  if (!items || n_items < 0 || !cfg || (dtype != OSGPU_C128 && dtype != OSGPU_C64) ||
      (cfg->engine != OSGPU_GS_ASM_RELAY && cfg->engine != OSGPU_GS_FRAUNHOFER) ||
      (cfg->engine == OSGPU_GS_ASM_RELAY && !asm_cfg) ||
      (cfg->engine == OSGPU_GS_FRAUNHOFER && !fraunhofer_cfg)) {
    set_err("bad GS arguments");
    return OSGPU_E_BAD_ARGUMENT;
  }
  // GsVariant::validate (gs.rs:165-178)
  double beta_f = 1.0, beta_p = 1.0;
  if (cfg->variant == OSGPU_GS_DVR) {
    if (!(std::isfinite(cfg->beta) && cfg->beta > 0.0 && cfg->beta < 2.0)) {
      set_err("Dvr beta must be in (0, 2), got %g", cfg->beta);
      return OSGPU_E_RENDER;
    }
    beta_p = cfg->beta;
  } else if (cfg->variant == OSGPU_GS_FPR) {
    if (!(std::isfinite(cfg->beta) && cfg->beta > 0.0 && cfg->beta <= 1.0)) {
      set_err("Fpr beta must be in (0, 1], got %g", cfg->beta);
      return OSGPU_E_RENDER;
    }
    beta_f = cfg->beta;
  } else if (cfg->variant != OSGPU_GS_CLASSIC) {
    return OSGPU_E_BAD_ARGUMENT;
  }
  if (cfg->max_iterations <= 0) {
    set_err("gs max_iterations must be > 0");
    return OSGPU_E_RENDER;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc;
  if ((rc = ensure_init(c))) return rc;
  cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  const int f32 = dtype == OSGPU_C64, c128 = dtype == OSGPU_C128, rf64 = c128;
  const size_t es = c128 ? 16 : 8, rs = c128 ? 8 : 4;
  const int max_it = cfg->max_iterations;
  // fused f32 Fraunhofer path: every item M x M (power of two), z > 0, no source offset
  if (f32 && cfg->engine == OSGPU_GS_FRAUNHOFER && !fraunhofer_cfg->has_source_pos &&
      n_items > 0 && !std::getenv("OSGPU_GS_GENERIC")) {
    const int M = (int)items[0].grid.nx;
    bool ok = gs_fast_size(M);
    for (int i = 0; i < n_items && ok; ++i) {
      const osgpu_gs_item& it = items[i];
      ok = it.grid.nx == (uint64_t)M && it.grid.ny == (uint64_t)M && it.d_input &&
           it.d_target_amplitude && it.d_phase && std::isfinite(it.z) && it.z > 0.0;
    }
    if (ok) return gs_fused(c, items, n_items, *cfg, *fraunhofer_cfg, beta_f, beta_p, M, st);
  }
  for (int i = 0; i < n_items; ++i) {
    osgpu_gs_item& it = items[i];
    const osgpu_grid& g = it.grid;
    const uint64_t n = g.nx * g.ny;
    if (!it.d_input || !it.d_target_amplitude || !it.d_phase || n == 0) {
      set_err("GS item %d: missing buffers or empty grid", i);
      return OSGPU_E_BAD_ARGUMENT;
    }
    if (!(std::isfinite(it.z) && it.z > 0.0)) {
      set_err("z must be positive and finite, got %g", it.z);
      return OSGPU_E_RENDER;
    }
    // engine set-up (host analysis once per item)
    osgpu_asm_report rf, rb;
    osgpu_fraunhofer_report fr;
    const double half = it.z / 2.0;
    if (cfg->engine == OSGPU_GS_ASM_RELAY) {
      if ((rc = asm_resolve(g, half, *asm_cfg, rf)) > 0 ||
          (rc = asm_resolve(g, -half, *asm_cfg, rb)) > 0) {
        set_err("GS item %d: ASM half-transform failed (status %d)", i, rc);
        return rc;
      }
    } else if ((rc = fraunhofer_resolve(g, it.z, *fraunhofer_cfg, fr)) > 0) {
      set_err("GS item %d: Fraunhofer regime check failed (status %d)", i, rc);
      return rc;
    }
    ElementList none;
    std::memset(&none, 0, sizeof(none));
    auto prop = [&](const void* in, void* out, int back) -> int {
      if (cfg->engine == OSGPU_GS_FRAUNHOFER) {
        return f32 ? run_fraun<float>(c, g, it.z, fr, none, in, c128, out, c128, nullptr, back, st)
                   : run_fraun<double>(c, g, it.z, fr, none, in, c128, out, c128, nullptr, back,
                                       st);
      }
      PropJob j;
      fill_asm_job(j, g, back ? -half : half, back ? rb : rf, *asm_cfg);
      j.d_in = in;
      j.in_c128 = c128;
      j.d_out = out;
      j.out_c128 = c128;
      return run_prop_dispatch(c, j, f32, st);
    };
    DBuf cur, open, illum, mask, ubuf, vbuf, part, dstate, hist;
    CK(cur.alloc(n * rs, st));
    CK(open.alloc(n, st));
    CK(illum.alloc(n * rs, st));
    CK(mask.alloc(n * es, st));
    CK(ubuf.alloc(n * es, st));
    CK(vbuf.alloc(n * es, st));
    CK(part.alloc(reduce_scratch_bytes(2), st));
    CK(dstate.alloc(sizeof(GsState), st));
    CK(hist.alloc(sizeof(GsRecordDev) * max_it, st));
    GsState h0;
    std::memset(&h0, 0, sizeof(h0));
    h0.best_it = -1;
    CK(cudaMemcpyAsync(dstate.p, &h0, sizeof(h0), cudaMemcpyHostToDevice, st));
    GsState* S = reinterpret_cast<GsState*>(dstate.p);
    GsRecordDev* H = reinterpret_cast<GsRecordDev*>(hist.p);
    double* P = reinterpret_cast<double*>(part.p);
    unsigned char* O = reinterpret_cast<unsigned char*>(open.p);
    CK(launch_gs_init(it.d_phase, cur.p, rf64, cfg->lo, cfg->hi, O, it.aperture, it.aperture_a,
                      it.aperture_b, it.center_x, it.center_y, (int)g.nx, (int)g.ny, g.dx, g.dy,
                      st));
    if (cfg->engine == OSGPU_GS_ASM_RELAY) {  // gs.rs:436-444
      if ((rc = prop(it.d_input, ubuf.p, 0))) return rc;
      CK(launch_abs(ubuf.p, c128, illum.p, rf64, 0, n, st));
    } else {
      CK(launch_abs(it.d_input, c128, illum.p, rf64, 0, n, st));
    }
    constexpr int kChunk = 8;  // iterations queued between looks at the stop flag
    for (int k = 0; k < max_it; ++k) {
      if (k > 0 && k % kChunk == 0) {
        int stop = 0;
        CK(cudaMemcpyAsync(&stop, &S->stop, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (stop) break;
      }
      {
        ProfScope ps(c, st, PC_GS, (double)n * (rs + 1 + rs + es));
        CK(launch_gs_mask(cur.p, rf64, illum.p, O, mask.p, c128, n, S, st));
      }
      if ((rc = prop(mask.p, ubuf.p, 0))) return rc;
      {
        ProfScope ps(c, st, PC_GS, (double)n * (es + rs * (it.d_target_intensity ? 2 : 1) + es));
        CK(launch_gs_project(ubuf.p, c128, it.d_target_amplitude, it.d_target_intensity, rf64,
                             beta_f, vbuf.p, n, P, it.d_target_error, S, H, k, st));
      }
      if ((rc = prop(vbuf.p, ubuf.p, 1))) return rc;
      {
        ProfScope ps(c, st, PC_GS, (double)n * (es + 2 * rs));
        CK(launch_gs_update(ubuf.p, c128, cur.p, it.d_phase, rf64, beta_p, cfg->lo, cfg->hi, n,
                            P, it.d_phase_error, S, H, k, cfg->patience, cfg->merit_tolerance,
                            max_it, st));
      }
    }
    GsState hs;
    CK(cudaMemcpyAsync(&hs, S, sizeof(hs), cudaMemcpyDeviceToHost, st));
    std::vector<GsRecordDev> hh(max_it);
    CK(cudaMemcpyAsync(hh.data(), H, sizeof(GsRecordDev) * max_it, cudaMemcpyDeviceToHost, st));
    if (it.d_best_intensity) {  // the best iteration's forward pass, recomputed
      CK(launch_gs_mask(it.d_phase, rf64, illum.p, O, mask.p, c128, n, nullptr, st));
      if ((rc = prop(mask.p, ubuf.p, 0))) return rc;
      CK(launch_abs(ubuf.p, c128, it.d_best_intensity, rf64, 1, n, st));
    }
    if (it.d_last_phase)
      CK(cudaMemcpyAsync(it.d_last_phase, cur.p, n * rs, cudaMemcpyDeviceToDevice, st));
    if (it.d_illumination)
      CK(cudaMemcpyAsync(it.d_illumination, illum.p, n * rs, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    if (hs.best_it < 0) {
      set_err("gs loop ran zero iterations");
      return OSGPU_E_RENDER;
    }
    it.result.merit = hs.best_merit;
    it.result.best_iteration = (uint64_t)hs.best_it;
    it.result.amplitude_mse = hh[hs.best_it].amplitude_mse;
    it.result.converged = hs.converged;
    it.result.iterations = (uint64_t)hs.iterations;
    if (it.history)
      for (int k = 0; k < hs.iterations; ++k) {
        osgpu_gs_record& r = it.history[k];
        r.iteration = (uint64_t)k;
        r.merit = hh[k].merit;
        r.best_merit = hh[k].best_merit;
        r.amplitude_mse = hh[k].amplitude_mse;
        r.target_error_rms = hh[k].target_error_rms;
        r.phase_update_rms = hh[k].phase_update_rms;
      }
  }
  return OSGPU_OK;
}

// ------------------------------------------------------------ profiling

int osgpu_plan_cache_config(int32_t enable, uint64_t max_bytes) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc = ensure_init(c);
  if (rc) return rc;
  c.plans_on = enable != 0;
  c.plan_cap = (size_t)max_bytes;
  if (c.plan_bytes > c.plan_cap) {
    CK(cudaDeviceSynchronize());
    while (c.plan_bytes > c.plan_cap && !c.plans.empty()) {
      auto lru = std::min_element(c.plans.begin(), c.plans.end(),
                                  [](const KPlan& a, const KPlan& b) { return a.last_use < b.last_use; });
      cudaFree(lru->kq);
      c.plan_bytes -= lru->bytes;
      c.plans.erase(lru);
    }
  }
  return OSGPU_OK;
}

int osgpu_plan_cache_clear(void) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc = ensure_init(c);
  if (rc) return rc;
  CK(cudaDeviceSynchronize());
  for (KPlan& p : c.plans) cudaFree(p.kq);
  c.plans.clear();
  c.plan_bytes = 0;
  c.plan_hits = c.plan_builds = 0;
  return OSGPU_OK;
}

int osgpu_plan_cache_stats(osgpu_plan_stats* out) {
  if (!out) {
    set_err("null stats pointer");
    return OSGPU_E_BAD_ARGUMENT;
  }
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  out->plans = c.plans.size();
  out->bytes = c.plan_bytes;
  out->hits = c.plan_hits;
  out->builds = c.plan_builds;
  return OSGPU_OK;
}

int osgpu_profile_begin(void) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc = ensure_init(c);
  if (rc) return rc;
  for (auto& r : c.prof) {
    c.event_pool.push_back(r.a);
    c.event_pool.push_back(r.b);
  }
  c.prof.clear();
  c.profiling = true;
  return OSGPU_OK;
}

int osgpu_profile_end(osgpu_kernel_stat* out, int32_t max_out, int32_t* n_out) {
  Context& c = ctx();
  std::lock_guard<std::recursive_mutex> lk(c.mu);
  int rc = ensure_init(c);
  if (rc) return rc;
  c.profiling = false;
  CK(cudaDeviceSynchronize());
  osgpu_kernel_stat agg[PC_N];
  std::memset(agg, 0, sizeof(agg));
  for (auto& r : c.prof) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    agg[r.cls].launches += 1;
    agg[r.cls].total_ms += ms;
    agg[r.cls].bytes += r.bytes;
    c.event_pool.push_back(r.a);
    c.event_pool.push_back(r.b);
  }
  c.prof.clear();
  int k = 0;
  for (int q = 0; q < PC_N; ++q) {
    if (!agg[q].launches) continue;
    if (out && k < max_out) {
      out[k] = agg[q];
      std::snprintf(out[k].name, sizeof(out[k].name), "%s", kProfNames[q]);
    }
    ++k;
  }
  if (n_out) *n_out = k;
  return OSGPU_OK;
}

}  // extern "C"
