// sif's C API for the exodus path over the GPU engine, and the additive
// device-resident entry points (include/sif_gb300.h).
//
// The structs are the reference's and live in host memory; each call copies
// what it needs to the GPU and its results back, and checks its arguments as
// the reference does, with the same statuses (include/sif/core/macros.h:
// 690-707) and an error message for sif_error_message().
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <condition_variable>
#include <map>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include <unistd.h>

#include "../../include/sif_gb300.h"
#include "checkpoint.cuh"
#include "engine.cuh"

namespace sifg {

void noalloc_forget();  // noalloc.cu

namespace {
std::mutex g_mu;
std::unique_ptr<Engine> g_engine;
bool g_init = false;
int g_log_level = SIF_LOG_LEVEL_INFO;
int g_status = SIF_OK;
std::string g_message;
std::vector<RungStat> g_stats;
sifg_timings_t g_timings{};
int g_window = 8;

void log_msg(int level, const char* tag, const std::string& msg) {
  if (level < g_log_level) return;
  static const char* names[] = {"TRACE", "DEBUG", "INFO", "WARNING", "ERROR"};
  fprintf(stderr, "[%s] %s: %s\n", names[level < 5 ? level : 4], tag, msg.c_str());
}

std::string fmt(const char* f, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, f);
  vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}
}  // namespace

static std::mutex g_err_mu;  // set_error may be called from several batch workers

void set_error(int status, const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_status = status;
  g_message = msg;
  log_msg(SIF_LOG_LEVEL_ERROR, "gb300", msg);
}

static int fail(int status, const std::string& msg) {
  set_error(status, msg);
  return status;
}

// Maps a CUDA failure to a status; a missing or lost device is an error the
// caller sees, never a silent fallback.
static int cuda_fail(const CudaError& e) {
  return fail(e.code == cudaErrorMemoryAllocation ? SIF_ERR_ALLOC : SIF_ERR_INVALID,
              fmt("CUDA: %s (%s)", cudaGetErrorString(e.code), e.where));
}

static Engine* engine() {
  if (!g_init || !g_engine) {
    set_error(SIF_ERR_UNINITIALISED, "sif_system_init() has not been called");
    return nullptr;
  }
  SIFG_CUDA(cudaSetDevice(g_engine->device()));
  return g_engine.get();
}

// --- device scratch for the C API's copies -------------------------------

struct ApiBufs {
  DevBuf px, py, pz, grid, grid64, mx, my, mz, offs, orig, bad, wide, mesh_sums;
  DevBuf pw, mw, mcw, wtotal;  // a weighted field's weights; a weighted mesh's columns, total
};
static ApiBufs& bufs() {
  static ApiBufs b;
  return b;
}

// sif__field_check_in_box (src/structures/field.c:889-935): every coordinate
// in [0, L), or within 4 float epsilons of L of a face (folded later). The
// reference compares in double against -tol and L + tol; a float v passes
// those exactly when it passes the float bounds lo and hi found on the host
// (the nearest floats inside them), so the kernel compares floats only.
template <class R>
__global__ void box_check_kernel(const R* __restrict__ x, const R* __restrict__ y,
                                 const R* __restrict__ z, uint64_t n, R lo, R hi,
                                 unsigned long long* __restrict__ out) {
  unsigned long long bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const R v[3] = {x[i], y[i], z[i]};
    bool ok = true;
    for (int a = 0; a < 3; a++) ok = ok && v[a] >= lo && v[a] <= hi;  // false for NaN
    bad += ok ? 0u : 1u;
  }
  for (int d = 16; d > 0; d >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, d);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(out, bad);
}

// The bounds: in the float form the nearest floats inside [-tol, L + tol];
// in the FP64 form the double bounds themselves (tol of 4 DBL_EPSILON, the
// SIF_USE_DOUBLE build's SIF__REAL_EPSILON).
static void box_bounds(float box, float* lo, float* hi) {
  const double tol = (double)box * 4.0 * (double)FLT_EPSILON;
  *lo = (float)(-tol);
  *hi = (float)((double)box + tol);
  if ((double)*lo < -tol) *lo = std::nextafter(*lo, 0.0f);
  if ((double)*hi > (double)box + tol) *hi = std::nextafter(*hi, 0.0f);
}
static void box_bounds(double box, double* lo, double* hi) {
  const double tol = box * 4.0 * DBL_EPSILON;
  *lo = -tol;
  *hi = box + tol;
}

template <class R>
static int check_in_box(const R* dx, const R* dy, const R* dz, uint64_t n, R box,
                        const char* name, cudaStream_t st, DevBuf& flag) {
  unsigned long long* d = (unsigned long long*)flag.ensure(16);
  SIFG_CUDA(cudaMemsetAsync(d, 0, 16, st));
  R lo, hi;
  box_bounds(box, &lo, &hi);
  box_check_kernel<R><<<grid_for(n, 256), 256, 0, st>>>(dx, dy, dz, n, lo, hi, d);
  SIFG_LAUNCH_CHECK();
  unsigned long long h[2];
  SIFG_CUDA(cudaMemcpyAsync(h, d, 16, cudaMemcpyDeviceToHost, st));
  SIFG_CUDA(cudaStreamSynchronize(st));
  if (h[0])
    return fail(SIF_ERR_RANGE,
                fmt("%s: %llu of %llu particles outside the box [0, %g)", name, h[0],
                    (unsigned long long)n, (double)box));
  return SIF_OK;
}

static int check_field(const sif_field_t* field, const char* tag) {
  if (!field) return fail(SIF_ERR_INVALID, fmt("%s: field: NULL", tag));
  if (field->n_particles == 0) return fail(SIF_ERR_INVALID, fmt("%s: field: no particles", tag));
  if (!field->x || !field->y || !field->z)
    return fail(SIF_ERR_INVALID, fmt("%s: field: no positions", tag));
  if (field->units != SIF_COORDINATES_CARTESIAN)
    return fail(SIF_ERR_INVALID, fmt("%s: field: sky coordinates (expected Cartesian)", tag));
  return SIF_OK;
}

__global__ void widen_kernel(const uint32_t* __restrict__ in, uint64_t* __restrict__ out, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

__global__ void narrow_kernel(const uint64_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)in[i];
}

static void widen(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t st) {
  widen_kernel<<<grid_for(n, 256), 256, 0, st>>>(in, out, n);
  SIFG_LAUNCH_CHECK();
}

static void narrow(const uint64_t* in, uint32_t* out, uint64_t n, cudaStream_t st) {
  narrow_kernel<<<grid_for(n, 256), 256, 0, st>>>(in, out, n);
  SIFG_LAUNCH_CHECK();
}

// The bytes the C API's calls copied between the structs' host arrays and
// the device, since the library was loaded (sifg_copy_bytes).
static uint64_t g_h2d_bytes = 0, g_d2h_bytes = 0;

static void copy_up(void* d, const void* h, size_t b, cudaStream_t st) {
  SIFG_CUDA(cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, st));
  g_h2d_bytes += b;
}

static void copy_down(void* h, const void* d, size_t b, cudaStream_t st) {
  SIFG_CUDA(cudaMemcpyAsync(h, d, b, cudaMemcpyDeviceToHost, st));
  g_d2h_bytes += b;
}

// Host array h (b bytes) on the device for a call that only reads it: its
// mirror where that stands, else copied up on st (into its mirror, or into
// the API's scratch when mirrors are off).
static const void* array_in(const void* h, size_t b, DevBuf& scratch, cudaStream_t st) {
  bool holds = false;
  void* d = mirror_acquire(h, b, b, scratch, &holds);
  if (!holds) copy_up(d, h, b, st);
  mirror_commit(h);
  return d;
}

// The field's positions on the device, axis by axis.
static void positions_in(const sif_field_t* f, cudaStream_t st, const float* d[3]) {
  const size_t b = f->n_particles * sizeof(float);
  d[0] = (const float*)array_in(f->x, b, bufs().px, st);
  d[1] = (const float*)array_in(f->y, b, bufs().py, st);
  d[2] = (const float*)array_in(f->z, b, bufs().pz, st);
}

// A catalogue of c's voids; with footprint, its footprint columns too
// (sif_catalogue_reserve_footprint, src/structures/catalogue.c), from c's.
static sif_catalogue_t* make_catalogue(const HostCatalogue& c, bool footprint = false) {
  const uint64_t n = c.cx.size();
  sif_catalogue_t* cat = (sif_catalogue_t*)calloc(1, sizeof(sif_catalogue_t));
  if (!cat) return nullptr;
  const uint64_t cap = n ? n : 1;
  cat->_block = (float*)host_block_get(4 * cap * sizeof(float));
  if (!cat->_block) {
    free(cat);
    return nullptr;
  }
  if (footprint) {
    cat->_footprint_block = (float*)malloc(2 * cap * sizeof(float));
    if (!cat->_footprint_block) {
      host_block_put(cat->_block);
      free(cat);
      return nullptr;
    }
    cat->footprint = cat->_footprint_block;
    cat->footprint_shell = cat->_footprint_block + cap;
    if (n) {
      memcpy(cat->footprint, c.foot.data(), n * 4);
      memcpy(cat->footprint_shell, c.shell.data(), n * 4);
    }
  }
  cat->cx = cat->_block;
  cat->cy = cat->_block + cap;
  cat->cz = cat->_block + 2 * cap;
  cat->radii = cat->_block + 3 * cap;
  if (n) {
    memcpy(cat->cx, c.cx.data(), n * 4);
    memcpy(cat->cy, c.cy.data(), n * 4);
    memcpy(cat->cz, c.cz.data(), n * 4);
    memcpy(cat->radii, c.r.data(), n * 4);
  }
  cat->units = SIF_COORDINATES_CARTESIAN;
  cat->n_voids = n;
  cat->capacity = cap;
  return cat;
}

// The last run's timeline (sifg_last_trace).
static std::vector<sifg_trace_event_t> g_trace;

static void append_trace(KernelTimer& k, int32_t kind, cudaEvent_t origin) {
  for (size_t i = 0; i < k.stops.size() && i < k.starts.size(); i++) {
    SIFG_CUDA(cudaEventSynchronize(k.stops[i]));
    float a = 0.f, b = 0.f;
    SIFG_CUDA(cudaEventElapsedTime(&a, origin, k.starts[i]));
    SIFG_CUDA(cudaEventElapsedTime(&b, origin, k.stops[i]));
    g_trace.push_back(sifg_trace_event_t{kind, a, b});
  }
}

static void record_trace(RunTimings& t) {
  g_trace.clear();
  if (!t.origin) return;
  SIFG_CUDA(cudaEventSynchronize(t.origin));
  append_trace(t.cic, SIFG_TRACE_CIC, t.origin);
  append_trace(t.mesh, SIFG_TRACE_MESH, t.origin);
  append_trace(t.smoothing, SIFG_TRACE_SMOOTHING, t.origin);
  append_trace(t.filter, SIFG_TRACE_FILTER, t.origin);
  append_trace(t.rung, SIFG_TRACE_RUNG, t.origin);
  append_trace(t.witness, SIFG_TRACE_WITNESS, t.origin);
  append_trace(t.growth, SIFG_TRACE_GROWTH, t.origin);
  append_trace(t.commit, SIFG_TRACE_COMMIT, t.origin);
  append_trace(t.cic_stage, SIFG_TRACE_CIC_STAGE, t.origin);
}

// The last run's events, kept until its timings or its timeline are asked
// for: reading them (a synchronize and an elapsed time per event) between
// runs would leave the GPU idle meanwhile.
static RunTimings g_last_run;
static bool g_last_pending = false;

static void resolve_timings() {
  if (!g_last_pending) return;
  g_last_pending = false;
  RunTimings& t = g_last_run;
  record_trace(t);
  g_timings.growth_ms = t.growth.total_ms();
  g_timings.growth_launches = t.growth.launches();
  g_timings.filter_ms = t.filter.total_ms();
  g_timings.filter_launches = t.filter.launches();
  g_timings.cic_ms = t.cic.total_ms();
  g_timings.cic_launches = t.cic.launches();
  g_timings.mesh_ms = t.mesh.total_ms();
  g_timings.mesh_launches = t.mesh.launches();
  g_timings.witness_ms = t.witness.total_ms();
  g_timings.witness_launches = t.witness.launches();
  g_timings.commit_ms = t.commit.total_ms();
  g_timings.commit_launches = t.commit.launches();
  g_timings.cic_stage_ms = t.cic_stage.total_ms();
  t.reset();
}

// A stage timed and read at once (a single-stage call) supersedes a run's
// timings that were not read.
static void drop_pending_timings() {
  if (!g_last_pending) return;
  g_last_pending = false;
  g_last_run.reset();
  g_trace.clear();
}

static void record_timings(RunTimings& t) {
  drop_pending_timings();
  g_timings = sifg_timings_t{};
  g_timings.wall_ms = t.wall_ms;
  g_timings.growth_particles = t.growth_particles;
  g_timings.growth_cells = t.growth_cells;
  g_last_run.swap_events(t);
  g_last_pending = true;
}

// The API lock, for entry points outside this file that hold it for a whole
// call (every entry point here does).
std::mutex& api_mutex() { return g_mu; }

// The library's stream and device; false (with the error set) before
// sif_system_init(). The caller holds api_mutex().
bool api_stream(cudaStream_t* st, int* device) {
  if (!g_init || !g_engine) {
    set_error(SIF_ERR_UNINITIALISED, "sif_system_init() has not been called");
    return false;
  }
  *st = g_engine->stream();
  *device = g_engine->device();
  return true;
}

}  // namespace sifg

using namespace sifg;

#define API_GUARD_BEGIN try {
#define API_GUARD_END(ret)                                                              \
  }                                                                                     \
  catch (const CudaError& e) {                                                          \
    cuda_fail(e);                                                                       \
    return ret;                                                                         \
  }                                                                                     \
  catch (const std::bad_alloc&) {                                                       \
    fail(SIF_ERR_ALLOC, "out of host memory");                                          \
    return ret;                                                                         \
  }

extern "C" {

// ---------------------------------------------------------------------------
// System
// ---------------------------------------------------------------------------

int sif_system_init(sif_config_t* config) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (config) g_log_level = config->log_level;
  if (g_init) return SIF_OK;
  API_GUARD_BEGIN
  int n_dev = 0;
  const cudaError_t e = cudaGetDeviceCount(&n_dev);
  if (e != cudaSuccess || n_dev == 0)
    return fail(SIF_ERR_UNSUPPORTED,
                fmt("no CUDA device (%s): this library runs the exodus path on a GPU only",
                    e != cudaSuccess ? cudaGetErrorString(e) : "none found"));
  g_engine.reset(new Engine(0));
  g_engine->host_threads =
      (config && config->omp_config && config->omp_config->n_threads) ? (int)config->omp_config->n_threads
                                                                      : omp_get_max_threads();
  if (const char* v = getenv("SIFG_HOST_MIRRORS")) mirror_enable(atoi(v) != 0);
  g_init = true;
  g_status = SIF_OK;
  g_message.clear();
  return SIF_OK;
  API_GUARD_END(SIF_ERR_INVALID)
}

void sif_system_finalise(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  noalloc_forget();
  drop_pending_timings();
  event_pool_clear();
  mirror_clear();  // device memory goes with the engine; the switch stays
  g_engine.reset();
  host_pool_trim();
  g_init = false;
  g_log_level = SIF_LOG_LEVEL_INFO;
}

const char* sif_error_message(void) { return g_message.c_str(); }
int sif_error_status(void) { return g_status; }

// ---------------------------------------------------------------------------
// Field, grid, catalogue (host structs; src/structures/field.c, grid.c:64-108,
// catalogue.c)
// ---------------------------------------------------------------------------

sif_field_t* sif_field_alloc(uint64_t n_particles) {
  sif_field_t* f = (sif_field_t*)calloc(1, sizeof(sif_field_t));
  if (!f) {
    fail(SIF_ERR_ALLOC, "field: cannot allocate");
    return nullptr;
  }
  f->n_particles = n_particles;
  f->units = SIF_COORDINATES_CARTESIAN;
  return f;
}

void sif_field_free(sif_field_t* f) {
  if (!f) return;
  host_block_put(f->_position_block);
  free(f->_velocity_block);
  host_block_put(f->weights);
  free(f->original_indices);
  free(f);
}

int sif_field_assign_positions(sif_field_t* f, const sif_real* x, const sif_real* y,
                               const sif_real* z) {
  if (!f || !x || !y || !z) return fail(SIF_ERR_INVALID, "field: NULL argument");
  const uint64_t n = f->n_particles;
  if (!f->_position_block) {
    f->_position_block = (float*)host_block_get(3 * (n ? n : 1) * sizeof(float));
    if (!f->_position_block) return fail(SIF_ERR_ALLOC, "field: cannot allocate positions");
    f->x = f->_position_block;
    f->y = f->_position_block + n;
    f->z = f->_position_block + 2 * n;
  }
  // The three columns in slices over the host's threads (one thread's
  // memcpy moves a gigabyte-sized field at a tenth of what the memory gives).
  const float* src[3] = {x, y, z};
  float* dst[3] = {f->x, f->y, f->z};
  const int64_t slices = n >= (1u << 22) ? 64 : 1;
#pragma omp parallel for schedule(static) if (slices > 1)
  for (int64_t k = 0; k < 3 * slices; k++) {
    const uint64_t a = n * (uint64_t)(k % slices) / slices, b = n * (uint64_t)(k % slices + 1) / slices;
    memcpy(dst[k / slices] + a, src[k / slices] + a, (b - a) * sizeof(float));
  }
  mirror_forget(f->x);
  mirror_forget(f->y);
  mirror_forget(f->z);
  free(f->original_indices);
  f->original_indices = nullptr;
  f->state_flags = 0;
  return SIF_OK;
}

// sif_field_reserve_weights / sif_field_assign_weights (src/structures/
// field.c:171-182, 292-321): the weight column, in the field's order (this
// library never reorders a field, so the caller's order is the field's).
int sif_field_reserve_weights(sif_field_t* f) {
  if (!f) return fail(SIF_ERR_INVALID, "field: NULL");
  if (f->n_particles == 0) return fail(SIF_ERR_INVALID, "field: no particles");
  if (f->weights) return SIF_OK;
  f->weights = (float*)host_block_get(f->n_particles * sizeof(float));
  return f->weights ? SIF_OK : fail(SIF_ERR_ALLOC, "field: cannot allocate weights");
}

int sif_field_assign_weights(sif_field_t* f, const sif_real* weights) {
  if (!f) return fail(SIF_ERR_INVALID, "field: NULL");
  if (f->n_particles == 0) return fail(SIF_ERR_INVALID, "field: no particles");
  if (!weights) return fail(SIF_ERR_INVALID, "weights: NULL");
  const int st = sif_field_reserve_weights(f);
  if (st != SIF_OK) return st;
  memcpy(f->weights, weights, f->n_particles * sizeof(float));
  mirror_forget(f->weights);
  return SIF_OK;
}

sif_grid_t* sif_grid_alloc(uint32_t n_cells, sif_real box_length) {
  if (n_cells == 0) {
    fail(SIF_ERR_INVALID, "n_cells: 0 (expected > 0)");
    return nullptr;
  }
  if (!(box_length > 0.0f)) {
    fail(SIF_ERR_INVALID, fmt("box_length: %g (expected > 0)", (double)box_length));
    return nullptr;
  }
  sif_grid_t* g = (sif_grid_t*)calloc(1, sizeof(sif_grid_t));
  if (!g) {
    fail(SIF_ERR_ALLOC, "grid: cannot allocate");
    return nullptr;
  }
  g->n_cells = n_cells;
  g->total_cells = (uint64_t)n_cells * n_cells * n_cells;
  g->box_length = box_length;
  g->cell_length = box_length / (float)n_cells;
  g->p2_mask = ((n_cells & (n_cells - 1)) == 0) ? (n_cells - 1) : 0;
  g->p2_shift = g->p2_mask ? (uint32_t)__builtin_ctz(n_cells) : 0;
  g->content = SIF_GRID_EMPTY;
  g->assignment = SIF_ASSIGNMENT_UNKNOWN;
  g->values = (float*)host_block_get(g->total_cells * sizeof(float));
  if (g->values) memset(g->values, 0, g->total_cells * sizeof(float));
  if (!g->values) {
    free(g);
    fail(SIF_ERR_ALLOC, fmt("grid: cannot allocate %u^3 cells", n_cells));
    return nullptr;
  }
  return g;
}

void sif_grid_free(sif_grid_t* g) {
  if (!g) return;
  host_block_put(g->values);
  free(g);
}

void sif_catalogue_free(sif_catalogue_t* c) {
  if (!c) return;
  host_block_put(c->_block);
  free(c->_footprint_block);
  free(c);
}

// sif_grid_assign with SIF_ASSIGNMENT_CIC (src/structures/grid.c:1042-1175).
int sif_grid_assign_cic(sif_grid_t* grid, const sif_field_t* field) {
  if (!grid || !grid->values) return fail(SIF_ERR_INVALID, grid ? "grid: no cell values" : "grid: NULL");
  if (grid->n_cells < 4)
    return fail(SIF_ERR_INVALID,
                fmt("n_cells: %u (expected at least 4 to assign onto)", grid->n_cells));
  int st = check_field(field, "grid");
  if (st != SIF_OK) return st;
  std::lock_guard<std::mutex> lk(g_mu);
  API_GUARD_BEGIN
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  cudaStream_t s = e->stream();
  const float* dp[3];
  positions_in(field, s, dp);
  st = check_in_box(dp[0], dp[1], dp[2], field->n_particles, grid->box_length, "field", s, bufs().bad);
  if (st != SIF_OK) return st;
  const size_t gb = grid->total_cells * sizeof(float);
  bool holds = false;
  float* dg = (float*)mirror_acquire(grid->values, gb, gb, bufs().grid, &holds);
  // Weighted (grid.c:635-639): the weights go up beside the positions.
  const float* dw = nullptr;
  if (field->weights)
    dw = (const float*)array_in(field->weights, field->n_particles * sizeof(float), bufs().pw, s);
  e->scratch.ensure(cic_scratch_bytes(field->n_particles, grid->n_cells, dw != nullptr));
  cic_deposit(dp[0], dp[1], dp[2], field->n_particles, grid->n_cells, grid->box_length, dg,
              e->scratch.ptr, s, nullptr, nullptr, nullptr, nullptr, dw);
  copy_down(grid->values, dg, gb, s);
  SIFG_CUDA(cudaStreamSynchronize(s));
  mirror_commit(grid->values);
  grid->content = SIF_GRID_DENSITY;
  grid->assignment = SIF_ASSIGNMENT_CIC;
  grid->interlaced = 0;
  return SIF_OK;
  API_GUARD_END(SIF_ERR_INVALID)
}

// src/structures/grid.c:1177-1244.
int sif_grid_to_density_contrast(sif_grid_t* grid) {
  if (!grid || !grid->values) return fail(SIF_ERR_INVALID, grid ? "grid: no cell values" : "grid: NULL");
  if (grid->content == SIF_GRID_DENSITY_CONTRAST)
    return fail(SIF_ERR_INVALID,
                "grid: already a density contrast (converting again would divide by a mean of about 0)");
  std::lock_guard<std::mutex> lk(g_mu);
  API_GUARD_BEGIN
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  cudaStream_t s = e->stream();
  const size_t b = grid->total_cells * sizeof(float);
  bool holds = false;
  float* dg = (float*)mirror_acquire(grid->values, b, b, bufs().grid, &holds);
  if (!holds) copy_up(dg, grid->values, b, s);
  double* scratch = (double*)e->scratch.ensure(density_contrast_scratch_bytes());
  density_contrast(dg, grid->total_cells, scratch, s);
  const double mean = read_mean(scratch, s);
  if (!(mean > 0.0))
    return fail(SIF_ERR_RANGE, fmt("grid: mean density %g (expected > 0)", mean));
  copy_down(grid->values, dg, b, s);
  SIFG_CUDA(cudaStreamSynchronize(s));
  mirror_commit(grid->values);
  grid->content = SIF_GRID_DENSITY_CONTRAST;
  return SIF_OK;
  API_GUARD_END(SIF_ERR_INVALID)
}

// sif_chain_mesh_alloc / _consume (src/structures/chain_mesh.c:49-215).
static sif_chain_mesh_t* mesh_alloc(uint32_t n_cells, sif_real box, sif_field_t* field,
                                    sif_option opt, bool consume) {
  if (check_field(field, "mesh") != SIF_OK) return nullptr;
  if (n_cells == 0) {
    fail(SIF_ERR_INVALID, "n_cells: 0 (expected > 0)");
    return nullptr;
  }
  if (n_cells > kMaxMeshSide) {
    fail(SIF_ERR_RANGE, fmt("n_cells: %u (the GPU mesh holds at most %u^3 cells)", n_cells,
                            kMaxMeshSide));
    return nullptr;
  }
  if (!(box > 0.0f)) {
    fail(SIF_ERR_INVALID, fmt("box_length: %g (expected > 0)", (double)box));
    return nullptr;
  }
  if (field->vx) {
    fail(SIF_ERR_UNSUPPORTED, "mesh: velocity-carrying fields are not supported on the GPU");
    return nullptr;
  }
  const uint64_t n = field->n_particles;
  if (n >= 0xffffffffull) {
    fail(SIF_ERR_RANGE, "mesh: 2^32 particles or more");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  API_GUARD_BEGIN
  Engine* e = engine();
  if (!e) return nullptr;
  cudaStream_t s = e->stream();
  const float* dp[3];
  positions_in(field, s, dp);
  if (check_in_box(dp[0], dp[1], dp[2], n, box, "field", s, bufs().bad) != SIF_OK) return nullptr;
  const uint64_t cells = (uint64_t)n_cells * n_cells * n_cells;
  const bool keep_idx = !(opt & SIF_MESH_DROP_INDICES);
  const bool weighted = field->weights != nullptr;
  // The struct and its host arrays first: the device buffers the build
  // writes are their mirrors.
  sif_chain_mesh_t* mesh = (sif_chain_mesh_t*)calloc(1, sizeof(sif_chain_mesh_t));
  if (!mesh) {
    fail(SIF_ERR_ALLOC, "mesh: cannot allocate");
    return nullptr;
  }
  struct Unwind {  // frees the half-built mesh on every early return
    sif_chain_mesh_t* m;
    ~Unwind() { sif_chain_mesh_free(m); }
  } unwind{mesh};
  mesh->n_cells = n_cells;
  mesh->total_cells = cells;
  mesh->box_length = box;
  mesh->cell_length = box / (float)n_cells;
  mesh->n_particles = n;
  mesh->total_weight = (double)n;
  mesh->_position_block = (float*)host_block_get(3 * (n ? n : 1) * sizeof(float));
  mesh->cell_offsets = (uint64_t*)host_block_get((cells + 1) * sizeof(uint64_t));
  if (keep_idx) mesh->original_indices = (uint64_t*)host_block_get(n * sizeof(uint64_t));
  if (weighted) {
    mesh->weights = (float*)host_block_get(n * sizeof(float));
    mesh->cell_weights = (float*)host_block_get(cells * sizeof(float));
  }
  if (!mesh->_position_block || !mesh->cell_offsets || (keep_idx && !mesh->original_indices) ||
      (weighted && (!mesh->weights || !mesh->cell_weights))) {
    fail(SIF_ERR_ALLOC, "mesh: cannot allocate host arrays");
    return nullptr;
  }
  mesh->x = mesh->_position_block;
  mesh->y = mesh->_position_block + n;
  mesh->z = mesh->_position_block + 2 * n;

  DeviceMesh m;
  m.n_cells = n_cells;
  m.box_length = box;
  m.cell_length = mesh->cell_length;
  bool holds = false;
  m.x = (float*)mirror_acquire(mesh->x, n * 4, n * 4, bufs().mx, &holds);
  m.y = (float*)mirror_acquire(mesh->y, n * 4, n * 4, bufs().my, &holds);
  m.z = (float*)mirror_acquire(mesh->z, n * 4, n * 4, bufs().mz, &holds);
  // The device keeps 32-bit offsets; the struct's are 64-bit.
  m.offsets = (uint32_t*)mirror_acquire(mesh->cell_offsets, (cells + 1) * 8, (cells + 1) * 4,
                                        bufs().offs, &holds);
  // A weighted mesh takes its weights through the source indices, kept on
  // the device whether or not the caller keeps them.
  m.orig = (keep_idx || weighted) ? (uint32_t*)bufs().orig.ensure(n * 4) : nullptr;
  e->scratch.ensure(std::max(mesh_scratch_bytes(n, n_cells),
                             weighted ? mesh_weights_scratch_bytes(n_cells) : (size_t)0));
  mesh_build(dp[0], dp[1], dp[2], n, m, e->scratch.ptr, s, nullptr);
  if (weighted) {
    // chain_mesh.c:800-801, 624-672: the weights in mesh order, each cell's
    // sum, the total.
    const float* fw = (const float*)array_in(field->weights, n * 4, bufs().pw, s);
    m.w = (float*)mirror_acquire(mesh->weights, n * 4, n * 4, bufs().mw, &holds);
    m.cell_w = (float*)mirror_acquire(mesh->cell_weights, cells * 4, cells * 4, bufs().mcw, &holds);
    double* d_total = (double*)bufs().wtotal.ensure(sizeof(double));
    mesh_weights(fw, m, e->scratch.ptr, d_total, s);
    copy_down(mesh->weights, m.w, n * 4, s);
    copy_down(mesh->cell_weights, m.cell_w, cells * 4, s);
    SIFG_CUDA(cudaMemcpyAsync(&mesh->total_weight, d_total, 8, cudaMemcpyDeviceToHost, s));
  }
  copy_down(mesh->x, m.x, n * 4, s);
  copy_down(mesh->y, m.y, n * 4, s);
  copy_down(mesh->z, m.z, n * 4, s);
  // The 64-bit offsets and indices of the reference's struct, widened on the
  // device and copied straight into the struct's arrays.
  uint64_t* wide = (uint64_t*)bufs().wide.ensure((keep_idx ? std::max<uint64_t>(n, cells + 1) : cells + 1) * 8);
  widen(m.offsets, wide, cells + 1, s);
  copy_down(mesh->cell_offsets, wide, (cells + 1) * 8, s);
  if (keep_idx) {
    SIFG_CUDA(cudaStreamSynchronize(s));
    widen(m.orig, wide, n, s);
    copy_down(mesh->original_indices, wide, n * 8, s);
  }
  SIFG_CUDA(cudaStreamSynchronize(s));
  for (const void* h : {(const void*)mesh->x, (const void*)mesh->y, (const void*)mesh->z,
                        (const void*)mesh->cell_offsets})
    mirror_commit(h);
  if (weighted) {
    mirror_commit(mesh->weights);
    mirror_commit(mesh->cell_weights);
  }
  unwind.m = nullptr;
  if (consume) {
    host_block_put(field->_position_block);
    field->_position_block = nullptr;
    field->x = field->y = field->z = nullptr;
    field->n_particles = 0;
  }
  return mesh;
  API_GUARD_END(nullptr)
}

sif_chain_mesh_t* sif_chain_mesh_alloc(uint32_t n_cells, sif_real box_length,
                                       const sif_field_t* field, sif_option opt) {
  return mesh_alloc(n_cells, box_length, const_cast<sif_field_t*>(field), opt, false);
}

sif_chain_mesh_t* sif_chain_mesh_alloc_consume(uint32_t n_cells, sif_real box_length,
                                               sif_field_t* field, sif_option opt) {
  return mesh_alloc(n_cells, box_length, field, opt, true);
}

void sif_chain_mesh_free(sif_chain_mesh_t* m) {
  if (!m) return;
  host_block_put(m->_position_block);
  free(m->_velocity_block);
  host_block_put(m->weights);
  host_block_put(m->cell_weights);
  host_block_put(m->original_indices);
  host_block_put(m->cell_offsets);
  free(m);
}

// ---------------------------------------------------------------------------
// Variants (src/finder/exodus_finder.c:1199-1254)
// ---------------------------------------------------------------------------

static const struct {
  const char* name;
  float overlap;
  uint32_t options;
} kVariants[SIF__EXODUS_N_VARIANTS] = {
    {"excursion-set", 0.0f, SIF_FINDER_SEEDS_CELLS},
    {"excursion-peak", 1.0f, SIF_FINDER_SEEDS_MINIMA | SIF_FINDER_EXTEND_REACH | SIF_FINDER_DISPLACE},
    {"lagrangian-overlap", 0.0f, SIF_FINDER_SEEDS_CELLS | SIF_FINDER_LAGRANGIAN_OVERLAP},
};

int sif_finder_exodus_preset(sif_exodus_variant_t variant, sif_real* overlap, sif_option* opt) {
  if ((unsigned)variant >= (unsigned)SIF__EXODUS_N_VARIANTS)
    return fail(SIF_ERR_INVALID, fmt("variant: %d (expected 0 to %d)", (int)variant,
                                     SIF__EXODUS_N_VARIANTS - 1));
  if (overlap) *overlap = kVariants[variant].overlap;
  if (opt) *opt = kVariants[variant].options;
  return SIF_OK;
}

const char* sif_finder_exodus_variant_name(sif_exodus_variant_t variant) {
  return (unsigned)variant < (unsigned)SIF__EXODUS_N_VARIANTS ? kVariants[variant].name : nullptr;
}

int sif_finder_exodus_variant_from_name(const char* name, sif_exodus_variant_t* variant) {
  for (int v = 0; name && v < SIF__EXODUS_N_VARIANTS; v++) {
    if (strcmp(name, kVariants[v].name) == 0) {
      if (variant) *variant = (sif_exodus_variant_t)v;
      return SIF_OK;
    }
  }
  return fail(SIF_ERR_INVALID,
              fmt("variant: \"%s\" (expected excursion-set, excursion-peak or lagrangian-overlap)",
                  name ? name : "(null)"));
}

// ---------------------------------------------------------------------------
// The finder
// ---------------------------------------------------------------------------

}  // extern "C"

// sif__finder_check_args, src/finder/utils.c:33-57.
template <class R>
static int check_args(const R* radii, uint32_t n_radii, R threshold, R f) {
  if (!radii || n_radii == 0) return fail(SIF_ERR_INVALID, "radii: none given");
  for (uint32_t i = 0; i < n_radii; i++)
    if (!(radii[i] > 0.0f) || !std::isfinite(radii[i]))
      return fail(SIF_ERR_INVALID,
                  fmt("radii[%u] = %g: not a positive radius", i, (double)radii[i]));
  if (!(threshold > -1.0f && threshold < 0.0f))
    return fail(SIF_ERR_INVALID,
                fmt("threshold %g: not a density contrast in (-1, 0)", (double)threshold));
  if (!(f >= 0.0f && f <= 1.0f))
    return fail(SIF_ERR_INVALID, fmt("overlap_fraction %g: not in [0, 1]", (double)f));
  return SIF_OK;
}

// The prior voids sif__exodus_check_extras accepts (src/finder/exodus_finder.c:
// 1163-1197): radii positive and finite, centres inside [0, box).
template <class R>
static int check_prior(const R* cx, const R* cy, const R* cz, const R* r, uint64_t n, R box) {
  for (uint64_t i = 0; i < n; i++) {
    if (!(r[i] > R(0)) || !std::isfinite(r[i]))
      return fail(SIF_ERR_INVALID, fmt("prior: void %llu: radius %g (expected positive and finite)",
                                       (unsigned long long)i, (double)r[i]));
    const R c[3] = {cx[i], cy[i], cz[i]};
    for (int k = 0; k < 3; k++)
      if (!(c[k] >= R(0) && c[k] < box))
        return fail(SIF_ERR_INVALID,
                    fmt("prior: void %llu: centre (%g, %g, %g) outside the box [0, %g)",
                        (unsigned long long)i, (double)c[0], (double)c[1], (double)c[2],
                        (double)box));
  }
  return SIF_OK;
}

static uint32_t g_halt_after = 0;  // sifg_set_halt_after

// A run's checkpoint and where it stands (checkpoint_t and run_start,
// checkpoint_rung, checkpoint_finish of exodus_finder.c:1384-1574).
struct RunCheckpoint {
  bool active = false;    // written after every rung
  bool on_disk = false;   // written or resumed by this run
  bool progress = false;  // the one on disk holds a finished rung
  bool keep = false;      // left in place on success
  std::string path;
  sif_finder_exodus_checkpoint_t header{};
  std::vector<float> sorted;    // the ladder, largest first
  std::vector<float> voids[4];  // where the run starts: prior or resumed voids
  uint32_t first_rung = 0;
  std::vector<float> host[4];   // a rung's catalogue, copied back to write

  // random_mesh and offset: a survey's randoms and what it was moved into
  // the box by (NULL for none), for the header; the prior voids are moved by
  // it (prior_in_box, exodus_finder.c:1404-1423).
  int start(const sif_grid_t* grid, const sif_chain_mesh_t* mesh, const float* radii,
            uint32_t n_radii, float threshold, float f, sif_option opt,
            const sif_finder_exodus_extras_t* extras,
            const sif_chain_mesh_t* random_mesh = nullptr, const float* offset = nullptr) {
    const sif_catalogue_t* prior = extras ? extras->prior : nullptr;
    const char* named = extras ? extras->checkpoint : nullptr;
    keep = extras && extras->keep_checkpoint;
    auto take_prior = [&]() {
      const uint64_t np = prior ? prior->n_voids : 0;
      const float* cols[4] = {np ? prior->cx : nullptr, np ? prior->cy : nullptr,
                              np ? prior->cz : nullptr, np ? prior->radii : nullptr};
      for (int k = 0; k < 4; k++) voids[k].assign(cols[k], cols[k] + np);
      for (int k = 0; offset && k < 3; k++)
        for (float& v : voids[k]) v = v + offset[k];
    };
    if (opt & SIF_FINDER_NO_CHECKPOINT) {
      take_prior();
      return SIF_OK;
    }
    sorted.assign(radii, radii + n_radii);
    std::sort(sorted.begin(), sorted.end(), [](float a, float b) { return a > b; });
    sif_finder_exodus_checkpoint_t& h = header;
    h = sif_finder_exodus_checkpoint_t{};
    h.is_survey = random_mesh != nullptr;
    h.is_weighted = mesh->weights != nullptr;
    h.options = opt & (SIF_FINDER_SEARCH_2_00 | SIF_FINDER_KEEP_CIC_WINDOW | SIF_FINDER_SEEDS_MINIMA |
                       SIF_FINDER_REFINE_HILL | SIF_FINDER_EXTEND_REACH | SIF_FINDER_DISPLACE |
                       SIF_FINDER_ALIASING_WINDOW | SIF_FINDER_LAGRANGIAN_OVERLAP);
    h.n_radii = n_radii;
    h.grid_n_cells = grid->n_cells;
    // The window order of the grid's assignment (CIC for an unknown one) and
    // the interlacing bit (sif__fft_grid_window_order, src/math/fft.c).
    const uint32_t order = (grid->assignment >= SIF_ASSIGNMENT_NGP && grid->assignment <= SIF_ASSIGNMENT_PCS)
                               ? (uint32_t)grid->assignment
                               : (uint32_t)SIF_ASSIGNMENT_CIC;
    h.assignment = (order & 0xffu) | ((grid->interlaced ? 1u : 0u) << 8);
    h.box_length = (double)grid->box_length;
    h.threshold = (double)threshold;
    h.overlap_fraction = (double)f;
    h.n_particles = mesh->n_particles;
    h.total_weight = mesh->total_weight;
    if (random_mesh) {
      h.random_n_particles = random_mesh->n_particles;
      h.random_total_weight = random_mesh->total_weight;
      for (int k = 0; offset && k < 3; k++) h.offset[k] = (double)offset[k];
    }
    if (prior && prior->n_voids) {
      h.n_prior = prior->n_voids;
      h.prior_crc32 = catalogue_crc(prior->cx, prior->cy, prior->cz, prior->radii, prior->n_voids);
    }
    path = named ? std::string(named) : checkpoint_default_name();
    std::string msg;
    if (named && access(named, F_OK) == 0) {
      sif_finder_exodus_checkpoint_t got;
      std::vector<float> got_radii;
      int st = checkpoint_load(path, got, got_radii, voids, &msg);
      if (st == SIF_OK) st = checkpoint_match(path, h, sorted.data(), got, got_radii.data(), &msg);
      if (st != SIF_OK) {
        for (auto& v : voids) v.clear();
        return fail(st, "checkpoint: " + msg);
      }
      first_rung = got.next_rung;
      header.n_mismatched = got.n_mismatched;
      active = on_disk = progress = true;
      log_msg(SIF_LOG_LEVEL_INFO, "finder.exodus",
              fmt("checkpoint: %s: resuming with %u of %u rungs done, %llu voids", named,
                  got.next_rung, n_radii, (unsigned long long)got.n_voids));
      return SIF_OK;
    }
    take_prior();
    const int st = checkpoint_write(path, h, sorted.data(), voids[0].data(), voids[1].data(),
                                    voids[2].data(), voids[3].data(), voids[0].size(),
                                    named ? nullptr : "running without a checkpoint", &msg);
    if (st == SIF_OK) {
      active = on_disk = true;
      log_msg(SIF_LOG_LEVEL_INFO, "finder.exodus", "checkpoint: " + path);
      return SIF_OK;
    }
    // Only a checkpoint the caller asked for by name is worth failing over.
    if (named) return fail(st, "checkpoint: " + msg);
    log_msg(SIF_LOG_LEVEL_WARNING, "finder.exodus", "checkpoint: " + msg);
    return SIF_OK;
  }

  // After a rung: the catalogue so far, copied back, and the rungs it covers;
  // a failure leaves the previous checkpoint. Then the halt hook.
  int rung(uint32_t done, const float* cx, const float* cy, const float* cz, const float* r,
           uint32_t nv, uint64_t mismatched, cudaStream_t st) {
    const float* cols[4] = {cx, cy, cz, r};
    for (int k = 0; k < 4; k++) {
      host[k].resize(nv);
      if (nv)
        SIFG_CUDA(cudaMemcpyAsync(host[k].data(), cols[k], nv * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    SIFG_CUDA(cudaStreamSynchronize(st));
    header.next_rung = done;
    header.n_mismatched += mismatched;
    std::string msg;
    if (checkpoint_write(path, header, sorted.data(), host[0].data(), host[1].data(), host[2].data(),
                         host[3].data(), nv, "checkpoint not updated, the previous one stands",
                         &msg) == SIF_OK)
      progress = true;
    else
      log_msg(SIF_LOG_LEVEL_WARNING, "finder.exodus", "checkpoint: " + msg);
    if (g_halt_after && g_halt_after == done) {
      set_error(SIF_ERR_INVALID, fmt("halted after rung %u of %u (test hook)", done, header.n_radii));
      return SIF_ERR_INVALID;
    }
    return SIF_OK;
  }

  // A finished run removes its checkpoint unless kept; one that failed keeps
  // it if it holds a finished rung.
  void finish(int status) {
    if (!on_disk) return;
    if (status != SIF_OK && progress) {
      log_msg(SIF_LOG_LEVEL_INFO, "finder.exodus",
              "checkpoint: " + path + ": kept, resume the run from it");
      return;
    }
    if (status == SIF_OK && keep) return;
    if (unlink(path.c_str()) != 0)
      log_msg(SIF_LOG_LEVEL_WARNING, "finder.exodus",
              "checkpoint: " + path + ": cannot remove: " + strerror(errno));
  }
};

extern "C" {

void sifg_set_halt_after(uint32_t n_rungs) { g_halt_after = n_rungs; }

// sif_finder_exodus_checkpoint_read (src/finder/exodus_checkpoint.c:451-488):
// the voids as saved; a survey's moved back to the caller's frame by the
// offset the run recorded.
sif_catalogue_t* sif_finder_exodus_checkpoint_read(const char* filepath,
                                                   sif_finder_exodus_checkpoint_t* header) {
  if (!filepath) {
    fail(SIF_ERR_INVALID, "filepath: NULL");
    return nullptr;
  }
  sif_finder_exodus_checkpoint_t h;
  std::vector<float> radii, cols[4];
  std::string msg;
  const int st = checkpoint_load(filepath, h, radii, cols, &msg);
  if (st != SIF_OK) {
    fail(st, "checkpoint: " + msg);
    return nullptr;
  }
  HostCatalogue c;
  c.cx = std::move(cols[0]);
  c.cy = std::move(cols[1]);
  c.cz = std::move(cols[2]);
  c.r = std::move(cols[3]);
  if (h.is_survey && (h.offset[0] != 0.0 || h.offset[1] != 0.0 || h.offset[2] != 0.0)) {
    const float back[3] = {(float)-h.offset[0], (float)-h.offset[1], (float)-h.offset[2]};
    std::vector<float>* cc[3] = {&c.cx, &c.cy, &c.cz};
    for (int k = 0; k < 3; k++)
      for (float& v : *cc[k]) v = v + back[k];
  }
  sif_catalogue_t* cat = make_catalogue(c);
  if (!cat) {
    fail(SIF_ERR_ALLOC, "catalogue: cannot allocate");
    return nullptr;
  }
  if (header) *header = h;
  return cat;
}

sif_catalogue_t* sif_finder_exodus(sif_grid_t* grid, const sif_chain_mesh_t* mesh,
                                   const sif_real* radii, uint32_t n_radii, sif_real threshold,
                                   sif_exodus_variant_t variant,
                                   const sif_finder_exodus_extras_t* extras) {
  sif_real f;
  sif_option opt;
  if (sif_finder_exodus_preset(variant, &f, &opt) != SIF_OK) return nullptr;
  return sif_finder_exodus_raw(grid, mesh, radii, n_radii, threshold, f, opt, extras);
}

// sif_finder_exodus_raw, src/finder/exodus_finder.c:1272-1345.
sif_catalogue_t* sif_finder_exodus_raw(sif_grid_t* grid, const sif_chain_mesh_t* mesh,
                                       const sif_real* radii, uint32_t n_radii,
                                       sif_real threshold, sif_real f, sif_option opt,
                                       const sif_finder_exodus_extras_t* extras) {
  if (!grid || !grid->values || !mesh) {
    fail(SIF_ERR_INVALID, !grid ? "grid: NULL" : (!grid->values ? "grid: no values" : "mesh: NULL"));
    return nullptr;
  }
  if (check_args(radii, n_radii, threshold, f) != SIF_OK) return nullptr;
  if (grid->content == SIF_GRID_DENSITY)
    log_msg(SIF_LOG_LEVEL_WARNING, "finder.exodus",
            "this grid holds a density, not a density contrast; call "
            "sif_grid_to_density_contrast first");
  if (!mesh->x || mesh->n_particles == 0) {
    fail(SIF_ERR_INVALID, "mesh: no particles");
    return nullptr;
  }
  if (mesh->box_length != grid->box_length) {
    fail(SIF_ERR_INVALID, fmt("mesh: box of %g, grid: box of %g (must match)",
                              (double)mesh->box_length, (double)grid->box_length));
    return nullptr;
  }
  // sif__exodus_check_weights (exodus_finder.c:1076-1106), before the run
  // starts or writes a checkpoint: by the bits, a negative zero passing.
  if (mesh->weights) {
    if (!mesh->cell_weights) {
      fail(SIF_ERR_INVALID, "mesh: weights but no per-cell weight table");
      return nullptr;
    }
    uint64_t neg = 0, bad = 0;
    const uint64_t nw = mesh->n_particles;
#pragma omp parallel for schedule(static) reduction(+ : neg, bad)
    for (uint64_t i = 0; i < nw; i++) {
      uint32_t b;
      memcpy(&b, mesh->weights + i, 4);
      const bool nonfinite = ((b >> 23) & 0xffu) == 0xffu;
      bad += nonfinite;
      neg += !nonfinite && (b >> 31) && (b << 1);
    }
    if (neg || bad) {
      fail(SIF_ERR_INVALID, fmt("mesh: weights must be finite and non-negative (%llu negative, "
                                "%llu not finite, of %llu)",
                                (unsigned long long)neg, (unsigned long long)bad,
                                (unsigned long long)nw));
      return nullptr;
    }
    if (!(mesh->total_weight > 0.0)) {
      fail(SIF_ERR_INVALID, "mesh: weights sum to zero (no mean density)");
      return nullptr;
    }
  }
  if (mesh->n_cells == 0 || mesh->n_cells > kMaxMeshSide) {
    fail(SIF_ERR_RANGE, fmt("mesh: %u cells a side (the GPU mesh holds 1 to %u)", mesh->n_cells,
                            kMaxMeshSide));
    return nullptr;
  }
  // sif__exodus_check_extras, src/finder/exodus_finder.c:1145-1200: a prior
  // catalogue the finder can place, and no checkpoint path beside the
  // option that turns checkpoints off.
  const sif_catalogue_t* prior = extras ? extras->prior : nullptr;
  if (extras) {
    if (extras->checkpoint && (opt & SIF_FINDER_NO_CHECKPOINT)) {
      fail(SIF_ERR_INVALID, fmt("checkpoint: %s, with SIF_FINDER_NO_CHECKPOINT set", extras->checkpoint));
      return nullptr;
    }
    // save_memory changes where the reference keeps the grid's transform, and
    // nothing of the run; the GPU run keeps its own in device memory.
    if (prior) {
      if (prior->units != SIF_COORDINATES_CARTESIAN) {
        fail(SIF_ERR_INVALID, "prior: centres on the sky (expected Cartesian coordinates)");
        return nullptr;
      }
      if (check_prior(prior->cx, prior->cy, prior->cz, prior->radii, prior->n_voids,
                      grid->box_length) != SIF_OK)
        return nullptr;
    }
  }
  if (mesh->n_particles >= 0xffffffffull) {
    fail(SIF_ERR_RANGE, "mesh: 2^32 particles or more");
    return nullptr;
  }
  // Where the run starts (run_start, exodus_finder.c:1437-1540): a
  // checkpoint the caller named and that exists is resumed -- its header must
  // describe this run -- else the run starts from the prior voids and writes
  // its first checkpoint now, unless SIF_FINDER_NO_CHECKPOINT.
  RunCheckpoint ck;
  if (ck.start(grid, mesh, radii, n_radii, threshold, f, opt, extras) != SIF_OK) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  API_GUARD_BEGIN
  Engine* e = engine();
  if (!e) return nullptr;
  cudaStream_t s = e->stream();
  const uint64_t n = mesh->n_particles;
  const uint64_t mcells = mesh->total_cells;
  const size_t gb = grid->total_cells * sizeof(float);
  const float* dg = (const float*)array_in(grid->values, gb, bufs().grid, s);
  DeviceMesh m;
  m.n_cells = mesh->n_cells;
  m.box_length = mesh->box_length;
  m.cell_length = mesh->cell_length;
  m.n_particles = n;
  // The mesh goes up on the copy stream while the first rungs are smoothed;
  // the run waits for it before its first sphere growth.
  cudaStream_t cs = e->copy_stream();
  SIFG_CUDA(cudaEventRecord(e->ev_copy_start(), s));
  SIFG_CUDA(cudaStreamWaitEvent(cs, e->ev_copy_start(), 0));
  bool holds = false;
  m.offsets = (uint32_t*)mirror_acquire(mesh->cell_offsets, (mcells + 1) * 8, (mcells + 1) * 4,
                                        bufs().offs, &holds);
  if (!holds) {
    uint64_t* wide = (uint64_t*)bufs().wide.ensure((mcells + 1) * 8);
    copy_up(wide, mesh->cell_offsets, (mcells + 1) * 8, cs);
    narrow(wide, m.offsets, mcells + 1, cs);
  }
  mirror_commit(mesh->cell_offsets);
  m.x = (float*)array_in(mesh->x, n * 4, bufs().mx, cs);
  m.y = (float*)array_in(mesh->y, n * 4, bufs().my, cs);
  m.z = (float*)array_in(mesh->z, n * 4, bufs().mz, cs);
  if (mesh->weights) {
    m.w = (float*)array_in(mesh->weights, n * 4, bufs().mw, cs);
    m.cell_w = (float*)array_in(mesh->cell_weights, mcells * 4, bufs().mcw, cs);
    m.total_weight = mesh->total_weight;
  }
  SIFG_CUDA(cudaEventRecord(e->ev_mesh_ready(), cs));
  // Whatever the run's outcome, the copies out of the caller's mesh end
  // before this call returns.
  struct CopyDrain {
    cudaStream_t s;
    ~CopyDrain() { cudaStreamSynchronize(s); }
  } drain{cs};

  RunParams p;
  p.grid_n = grid->n_cells;
  p.box = grid->box_length;
  p.threshold = threshold;
  p.overlap = f;
  p.options = opt;
  p.radii.assign(radii, radii + n_radii);
  p.window = g_window;
  p.mesh_ready = e->ev_mesh_ready();
  p.weights_checked = true;  // above, on the host copy
  if (!ck.voids[0].empty()) {
    p.prior_cx = ck.voids[0].data();
    p.prior_cy = ck.voids[1].data();
    p.prior_cz = ck.voids[2].data();
    p.prior_r = ck.voids[3].data();
    p.n_prior = ck.voids[0].size();
  }
  p.first_rung = ck.first_rung;
  if (ck.active)
    p.after_rung = [&](uint32_t done, const float* cx, const float* cy, const float* cz,
                       const float* r, uint32_t nv, uint64_t mismatched) {
      return ck.rung(done, cx, cy, cz, r, nv, mismatched, s);
    };
  float* consume = nullptr;
  if (opt & SIF_FINDER_CONSUME_GRID) consume = (float*)bufs().px.ensure(gb);
  p.consume_out = consume;
  HostCatalogue cat;
  RunTimings tm;
  g_stats.clear();
  const int st = e->exodus(dg, m, p, cat, &g_stats, &tm);
  record_timings(tm);
  ck.finish(st);
  if (st != SIF_OK) return nullptr;
  // The grid handed back: untouched, which restores it exactly; under
  // SIF_FINDER_CONSUME_GRID it holds the last rung's smoothing, as the
  // reference leaves it (exodus_finder.c:2426-2453).
  if (consume) {
    mirror_forget(grid->values);
    copy_down(grid->values, consume, gb, s);
    SIFG_CUDA(cudaStreamSynchronize(s));
  }
  g_d2h_bytes += 4 * sizeof(float) * (uint64_t)cat.cx.size();  // the catalogue's columns
  sif_catalogue_t* out = make_catalogue(cat);
  if (!out) fail(SIF_ERR_ALLOC, "catalogue: cannot allocate");
  return out;
  API_GUARD_END(nullptr)
}

// sif__exodus_check_weights (exodus_finder.c:1076-1106) on a mesh's host
// column: by the bits, a negative zero passing.
static int host_weights_ok(const sif_chain_mesh_t* mesh, const char* which) {
  if (!mesh->weights) return SIF_OK;
  if (!mesh->cell_weights)
    return fail(SIF_ERR_INVALID, fmt("%s: weights but no per-cell weight table", which));
  uint64_t neg = 0, bad = 0;
  const uint64_t nw = mesh->n_particles;
#pragma omp parallel for schedule(static) reduction(+ : neg, bad)
  for (uint64_t i = 0; i < nw; i++) {
    uint32_t b;
    memcpy(&b, mesh->weights + i, 4);
    const bool nonfinite = ((b >> 23) & 0xffu) == 0xffu;
    bad += nonfinite;
    neg += !nonfinite && (b >> 31) && (b << 1);
  }
  if (neg || bad)
    return fail(SIF_ERR_INVALID,
                fmt("%s: weights must be finite and non-negative (%llu negative, %llu not finite, "
                    "of %llu)",
                    which, (unsigned long long)neg, (unsigned long long)bad,
                    (unsigned long long)nw));
  return SIF_OK;
}

static float search_factor_of(sif_option opt) {
  static const float factors[4] = {1.5f, 1.25f, 1.75f, 2.0f};
  return factors[(opt >> 12) & 3u];
}

// sif_finder_exodus_survey_raw, src/finder/exodus_survey.c:401-545: the
// finder on a survey -- any geometry, described by its randoms -- inside a
// box padded so that nothing wraps (see the margin below). The grids are the
// CIC densities of data and randoms as sif_grid_assign_cic leaves them; each
// rung scans the smoothed data over alpha times the smoothed randoms and
// grows each radius against the randoms; the catalogue comes back in the
// caller's frame (less `offset`), with its footprint columns.
sif_catalogue_t* sif_finder_exodus_survey_raw(sif_grid_t* data_grid, sif_grid_t* random_grid,
                                              const sif_chain_mesh_t* data_mesh,
                                              const sif_chain_mesh_t* random_mesh,
                                              const sif_real offset[3], const sif_real* radii,
                                              uint32_t n_radii, sif_real threshold,
                                              sif_real f, sif_option opt,
                                              const sif_finder_exodus_extras_t* extras) {
  const char* missing = !data_grid                              ? "data grid: NULL"
                        : !data_grid->values                    ? "data grid: no values"
                        : !random_grid                          ? "random grid: NULL"
                        : !random_grid->values                  ? "random grid: no values"
                        : !data_mesh                            ? "data mesh: NULL"
                        : !random_mesh                          ? "random mesh: NULL"
                        : !data_mesh->x || !data_mesh->n_particles ? "data mesh: no particles"
                        : !random_mesh->x || !random_mesh->n_particles
                            ? "random mesh: no particles"
                            : nullptr;
  if (missing) {
    fail(SIF_ERR_INVALID, missing);
    return nullptr;
  }
  if (check_args(radii, n_radii, threshold, f) != SIF_OK) return nullptr;
  // sif__exodus_check_seeds (exodus_finder.c:1114-1137): cell seeds on their
  // nodes only, in a survey.
  const sif_option refine = opt & (3u << 19);
  const char* box_only = (opt & SIF_FINDER_SEEDS_MINIMA)   ? "SIF_FINDER_SEEDS_MINIMA"
                         : refine == (1u << 19)             ? "SIF_FINDER_REFINE_GAUSSIAN"
                         : refine == (2u << 19)             ? "SIF_FINDER_REFINE_TRACERS"
                         : refine                           ? "SIF_FINDER_REFINE_HILL"
                         : (opt & SIF_FINDER_EXTEND_REACH) ? "SIF_FINDER_EXTEND_REACH"
                         : (opt & SIF_FINDER_DISPLACE)     ? "SIF_FINDER_DISPLACE"
                                                            : nullptr;
  if (box_only) {
    fail(SIF_ERR_INVALID,
         fmt("options: %s: a survey (expected SIF_FINDER_SEEDS_CELLS on their nodes, for now)",
             box_only));
    return nullptr;
  }
  for (int k = 0; offset && k < 3; k++)
    if (!std::isfinite(offset[k])) {
      fail(SIF_ERR_INVALID, fmt("offset[%d]: %g, expected finite", k, (double)offset[k]));
      return nullptr;
    }
  // The contrast is formed against the randoms: a grid already turned into
  // one against the box mean is the wrong input.
  if (data_grid->content == SIF_GRID_DENSITY_CONTRAST ||
      random_grid->content == SIF_GRID_DENSITY_CONTRAST) {
    fail(SIF_ERR_INVALID,
         fmt("%s grid: holds a density contrast; a survey takes the CIC densities as assign_cic "
             "leaves them",
             data_grid->content == SIF_GRID_DENSITY_CONTRAST ? "data" : "random"));
    return nullptr;
  }
  if (data_grid->n_cells != random_grid->n_cells || data_grid->box_length != random_grid->box_length) {
    fail(SIF_ERR_INVALID, fmt("data grid: %u cells over %g, random grid: %u over %g (must match)",
                              data_grid->n_cells, (double)data_grid->box_length,
                              random_grid->n_cells, (double)random_grid->box_length));
    return nullptr;
  }
  if (data_mesh->box_length != data_grid->box_length ||
      random_mesh->box_length != data_grid->box_length) {
    fail(SIF_ERR_INVALID, fmt("meshes: boxes of %g (data) and %g (randoms), grids: %g (must match)",
                              (double)data_mesh->box_length, (double)random_mesh->box_length,
                              (double)data_grid->box_length));
    return nullptr;
  }
  if (host_weights_ok(data_mesh, "data mesh") != SIF_OK ||
      host_weights_ok(random_mesh, "random mesh") != SIF_OK)
    return nullptr;
  if (!(data_mesh->total_weight > 0.0) || !(random_mesh->total_weight > 0.0)) {
    fail(SIF_ERR_INVALID, fmt("%s mesh: total weight is zero",
                              data_mesh->total_weight > 0.0 ? "random" : "data"));
    return nullptr;
  }
  for (const sif_chain_mesh_t* m : {data_mesh, random_mesh})
    if (m->n_cells == 0 || m->n_cells > kMaxMeshSide || m->n_particles >= 0xffffffffull) {
      fail(SIF_ERR_RANGE, fmt("mesh: %u cells a side and %llu tracers (the GPU mesh holds 1 to %u "
                              "cells a side, fewer than 2^32 tracers)",
                              m->n_cells, (unsigned long long)m->n_particles, kMaxMeshSide));
      return nullptr;
    }
  const sif_catalogue_t* prior = extras ? extras->prior : nullptr;
  if (extras) {
    if (extras->checkpoint && (opt & SIF_FINDER_NO_CHECKPOINT)) {
      fail(SIF_ERR_INVALID, fmt("checkpoint: %s, with SIF_FINDER_NO_CHECKPOINT set", extras->checkpoint));
      return nullptr;
    }
    // sif__exodus_check_extras (1145-1200): the prior voids placed in the
    // box once moved by the offset.
    if (prior && prior->n_voids) {
      if (prior->units != SIF_COORDINATES_CARTESIAN) {
        fail(SIF_ERR_INVALID, "prior: centres on the sky (expected Cartesian coordinates)");
        return nullptr;
      }
      std::vector<float> moved[3];
      for (int k = 0; k < 3; k++) {
        const float* c = k == 0 ? prior->cx : (k == 1 ? prior->cy : prior->cz);
        moved[k].assign(c, c + prior->n_voids);
        for (float& v : moved[k]) v = v + (offset ? offset[k] : 0.0f);
      }
      if (check_prior(moved[0].data(), moved[1].data(), moved[2].data(), prior->radii,
                      prior->n_voids, data_grid->box_length) != SIF_OK)
        return nullptr;
    }
  }
  RunCheckpoint ck;
  if (ck.start(data_grid, data_mesh, radii, n_radii, threshold, f, opt, extras, random_mesh,
               offset) != SIF_OK)
    return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  API_GUARD_BEGIN
  Engine* e = engine();
  if (!e) return nullptr;
  cudaStream_t s = e->stream();
  const size_t gb = data_grid->total_cells * sizeof(float);
  const float* dg = (const float*)array_in(data_grid->values, gb, bufs().grid, s);
  thread_local DevBuf rgrid_scratch;
  const float* rg = (const float*)array_in(random_grid->values, gb, rgrid_scratch, s);
  // The meshes, each with its 32-bit offsets on the device.
  thread_local ApiBufs rbufs;  // the randoms' columns, beside the data's
  auto mesh_in = [&](const sif_chain_mesh_t* mesh, ApiBufs& b) {
    DeviceMesh m;
    const uint64_t n = mesh->n_particles, mc = mesh->total_cells;
    m.n_cells = mesh->n_cells;
    m.box_length = mesh->box_length;
    m.cell_length = mesh->cell_length;
    m.n_particles = n;
    bool holds = false;
    m.offsets = (uint32_t*)mirror_acquire(mesh->cell_offsets, (mc + 1) * 8, (mc + 1) * 4, b.offs,
                                          &holds);
    if (!holds) {
      uint64_t* wide = (uint64_t*)b.wide.ensure((mc + 1) * 8);
      copy_up(wide, mesh->cell_offsets, (mc + 1) * 8, s);
      narrow(wide, m.offsets, mc + 1, s);
    }
    mirror_commit(mesh->cell_offsets);
    m.x = (float*)array_in(mesh->x, n * 4, b.mx, s);
    m.y = (float*)array_in(mesh->y, n * 4, b.my, s);
    m.z = (float*)array_in(mesh->z, n * 4, b.mz, s);
    m.total_weight = mesh->total_weight;
    if (mesh->weights) {
      m.w = (float*)array_in(mesh->weights, n * 4, b.mw, s);
      m.cell_w = (float*)array_in(mesh->cell_weights, mc * 4, b.mcw, s);
    }
    return m;
  };
  DeviceMesh dm = mesh_in(data_mesh, bufs());
  DeviceMesh rm = mesh_in(random_mesh, rbufs);
  // survey_check_margin (exodus_survey.c:350-372): every tracer at least the
  // margin from every face, so that nothing downstream -- the transforms,
  // the mesh walks, the overlap tests, all periodic -- sees the wrap.
  {
    float r_max = radii[0], r_min = radii[0];
    for (uint32_t i = 1; i < n_radii; i++) {
      r_max = std::max(r_max, radii[i]);
      r_min = std::min(r_min, radii[i]);
    }
    const float cell = data_grid->cell_length;
    const float r_search = r_max + std::fmax((search_factor_of(opt) - 1.0f) * r_max, 3.0f * cell);
    const float mesh_cell = std::fmax(data_mesh->cell_length, random_mesh->cell_length);
    const float margin = std::fmax(r_search, 0.5f * (r_search + mesh_cell)) + cell;
    const std::string hint =
        cell > r_min ? fmt("; survey_box allows for grid cells up to the smallest radius, %g, and "
                           "these are %g",
                           (double)r_min, (double)cell)
                     : std::string(", as survey_box sizes it");
    const struct {
      const DeviceMesh* m;
      const char* what;
    } sets[2] = {{&rm, "randoms"}, {&dm, "data"}};
    for (const auto& set : sets) {
      float lo[3], hi[3];
      extent(set.m->x, set.m->y, set.m->z, set.m->n_particles, lo, hi, s);
      const float L = set.m->box_length;
      for (int k = 0; k < 3; k++)
        if (lo[k] < margin || hi[k] > L - margin) {
          fail(SIF_ERR_INVALID,
               fmt("%s: span [%g, %g] on axis %d of a box of %g, %g from its face (needs %g of "
                   "padding on every side%s)",
                   set.what, (double)lo[k], (double)hi[k], k, (double)L,
                   (double)std::min(lo[k], L - hi[k]), (double)margin, hint.c_str()));
          return nullptr;
        }
    }
  }
  RunParams p;
  p.grid_n = data_grid->n_cells;
  p.box = data_grid->box_length;
  p.threshold = threshold;
  p.overlap = f;
  p.options = opt;
  p.radii.assign(radii, radii + n_radii);
  p.window = g_window;
  p.weights_checked = true;  // above, on the host columns
  p.random_mesh = &rm;
  p.random_density = rg;
  // exodus_finder.c:1649-1653: how much data weight a unit of random weight
  // stands for.
  p.survey_alpha = (float)(data_mesh->total_weight / random_mesh->total_weight);
  if (!ck.voids[0].empty()) {
    p.prior_cx = ck.voids[0].data();
    p.prior_cy = ck.voids[1].data();
    p.prior_cz = ck.voids[2].data();
    p.prior_r = ck.voids[3].data();
    p.n_prior = ck.voids[0].size();
  }
  p.first_rung = ck.first_rung;
  if (ck.active)
    p.after_rung = [&](uint32_t done, const float* cx, const float* cy, const float* cz,
                       const float* r, uint32_t nv, uint64_t mismatched) {
      return ck.rung(done, cx, cy, cz, r, nv, mismatched, s);
    };
  HostCatalogue cat;
  RunTimings tm;
  g_stats.clear();
  const int st = e->exodus(dg, dm, p, cat, &g_stats, &tm);
  record_timings(tm);
  ck.finish(st);
  if (st != SIF_OK) return nullptr;
  // Back to the caller's frame (sif_catalogue_translate by -offset); the
  // prior voids, the caller's own, as given.
  if (offset) {
    const float back[3] = {-offset[0], -offset[1], -offset[2]};
    std::vector<float>* cc[3] = {&cat.cx, &cat.cy, &cat.cz};
    for (int k = 0; k < 3; k++)
      for (float& v : *cc[k]) v = v + back[k];
    const uint64_t np = prior ? prior->n_voids : 0;
    if (np && cat.cx.size() >= np) {
      std::copy(prior->cx, prior->cx + np, cat.cx.begin());
      std::copy(prior->cy, prior->cy + np, cat.cy.begin());
      std::copy(prior->cz, prior->cz + np, cat.cz.begin());
    }
  }
  g_d2h_bytes += 6 * sizeof(float) * (uint64_t)cat.cx.size();
  sif_catalogue_t* out = make_catalogue(cat, true);
  if (!out) fail(SIF_ERR_ALLOC, "catalogue: cannot allocate");
  return out;
  API_GUARD_END(nullptr)
}

sif_catalogue_t* sif_finder_exodus_survey(sif_grid_t* data_grid, sif_grid_t* random_grid,
                                          const sif_chain_mesh_t* data_mesh,
                                          const sif_chain_mesh_t* random_mesh,
                                          const sif_real offset[3], const sif_real* radii,
                                          uint32_t n_radii, sif_real threshold,
                                          sif_exodus_variant_t variant,
                                          const sif_finder_exodus_extras_t* extras) {
  sif_real f;
  sif_option opt;
  if (sif_finder_exodus_preset(variant, &f, &opt) != SIF_OK) return nullptr;
  return sif_finder_exodus_survey_raw(data_grid, random_grid, data_mesh, random_mesh, offset,
                                      radii, n_radii, threshold, f, opt, extras);
}

// sif_finder_exodus_survey_box, src/finder/exodus_survey.c:590-703: the box
// a survey is searched in -- its extent (data and randoms) plus, on every
// side, the margin survey_raw checks for at the largest grid cell the
// ladder's smallest radius allows, times 1.01 -- and the offset that centres
// the survey in it.
int sif_finder_exodus_survey_box(const sif_field_t* data, const sif_field_t* randoms,
                                 const sif_real* radii, uint32_t n_radii, sif_option opt,
                                 sif_real offset[3], sif_real* box_length) {
  const char* names[2] = {"data", "randoms"};
  const sif_field_t* given[2] = {data, randoms};
  for (int i = 0; i < 2; i++) {
    const sif_field_t* fl = given[i];
    if (!fl || !fl->x || !fl->y || !fl->z || fl->n_particles == 0)
      return fail(SIF_ERR_INVALID, fmt("%s: %s", names[i],
                                       !fl ? "NULL" : (fl->n_particles == 0 ? "no particles"
                                                                            : "no positions")));
    if (fl->units != SIF_COORDINATES_CARTESIAN)
      return fail(SIF_ERR_INVALID,
                  fmt("%s: sky coordinates (expected Cartesian; convert them first)", names[i]));
  }
  if (!radii || n_radii == 0 || !offset || !box_length)
    return fail(SIF_ERR_INVALID, !radii || n_radii == 0 ? "radii: none given"
                                                        : "offset, box_length: NULL");
  for (uint32_t i = 0; i < n_radii; i++)
    if (!(radii[i] > 0.0f) || !std::isfinite(radii[i]))
      return fail(SIF_ERR_INVALID, fmt("radii[%u] = %g: not a positive radius", i, (double)radii[i]));
  // survey_field_extent (595-628): the bounding box grown by a field, a
  // coordinate that is not finite counted and refused.
  auto grow = [&](const sif_field_t* fl, const char* what, float lo[3], float hi[3]) {
    float x0 = lo[0], y0 = lo[1], z0 = lo[2], x1 = hi[0], y1 = hi[1], z1 = hi[2];
    uint64_t bad = 0;
    const uint64_t n = fl->n_particles;
#pragma omp parallel for schedule(static) reduction(min : x0, y0, z0) reduction(max : x1, y1, z1) \
    reduction(+ : bad)
    for (uint64_t p = 0; p < n; p++) {
      const float x = fl->x[p], y = fl->y[p], z = fl->z[p];
      bad += !(std::isfinite(x) && std::isfinite(y) && std::isfinite(z));
      x0 = std::fmin(x0, x);
      y0 = std::fmin(y0, y);
      z0 = std::fmin(z0, z);
      x1 = std::fmax(x1, x);
      y1 = std::fmax(y1, y);
      z1 = std::fmax(z1, z);
    }
    if (bad)
      return fail(SIF_ERR_INVALID, fmt("%s: %llu of %llu with a coordinate that is not finite", what,
                                       (unsigned long long)bad, (unsigned long long)n));
    lo[0] = x0, lo[1] = y0, lo[2] = z0;
    hi[0] = x1, hi[1] = y1, hi[2] = z1;
    return SIF_OK;
  };
  float lo[3] = {randoms->x[0], randoms->y[0], randoms->z[0]};
  float hi[3] = {lo[0], lo[1], lo[2]};
  if (grow(randoms, "randoms", lo, hi) != SIF_OK) return SIF_ERR_INVALID;
  const float r_lo[3] = {lo[0], lo[1], lo[2]}, r_hi[3] = {hi[0], hi[1], hi[2]};
  if (grow(data, "data", lo, hi) != SIF_OK) return SIF_ERR_INVALID;
  float beyond = 0.0f;
  for (int k = 0; k < 3; k++) beyond = std::fmax(beyond, std::fmax(r_lo[k] - lo[k], hi[k] - r_hi[k]));
  if (beyond > 0.0f)
    log_msg(SIF_LOG_LEVEL_WARNING, "finder.exodus",
            fmt("the data reach %g past the randoms' bounding box; the box is sized around both, "
                "but tracers outside the randoms are outside the footprint",
                (double)beyond));
  float extent_max = 0.0f;
  for (int k = 0; k < 3; k++) extent_max = std::fmax(extent_max, hi[k] - lo[k]);
  float r_min = radii[0], r_max = radii[0];
  for (uint32_t i = 1; i < n_radii; i++) {
    r_min = std::fmin(r_min, radii[i]);
    r_max = std::fmax(r_max, radii[i]);
  }
  const float fs = search_factor_of(opt);
  const float cell = r_min;
  const float margin = r_max + std::fmax((fs - 1.0f) * r_max, 3.0f * cell) + cell;
  const float L = extent_max + 2.0f * 1.01f * margin;  // SURVEY_BOX_SLACK, 573
  for (int k = 0; k < 3; k++) offset[k] = 0.5f * L - 0.5f * (lo[k] + hi[k]);
  *box_length = L;
  return SIF_OK;
}

// sif_finder_grid_cells_from_size, src/finder/exodus_finder.c:2494-2560.
uint32_t sif_finder_grid_cells_from_size(uint64_t n_particles, sif_real box_length,
                                         sif_real cell_size, sif_finder_units_t units,
                                         sif_real volume) {
  if (!(box_length > 0.0f) || !std::isfinite(box_length) || !(cell_size > 0.0f) ||
      !std::isfinite(cell_size)) {
    fail(SIF_ERR_INVALID, "grid cells: box and cell size must be positive and finite");
    return 0;
  }
  double cell = (double)cell_size;
  if (units == SIF_FINDER_UNITS_MPS) {
    if (n_particles == 0 || !(volume >= 0.0f)) {
      fail(SIF_ERR_INVALID, "grid cells: no tracers to take a mean separation from");
      return 0;
    }
    const double vol = volume > 0.0f ? (double)volume
                                     : (double)box_length * box_length * box_length;
    cell *= std::cbrt(vol / (double)n_particles);
  }
  const double ratio = (double)box_length / cell;
  const double nearest = std::round(ratio);
  const double n = std::fabs(ratio - nearest) <= 1e-5 * nearest ? nearest : std::ceil(ratio);
  if (!(n >= 1.0) || n > 4294967295.0) {
    fail(SIF_ERR_RANGE, "grid cells: count does not fit in 32 bits");
    return 0;
  }
  return (uint32_t)n;
}

// ---------------------------------------------------------------------------
// Part 2: device-resident entry points
// ---------------------------------------------------------------------------

}  // extern "C"

// ---------------------------------------------------------------------------
// Device entry points, one template per stage for the float form and the
// FP64 form (the reference's SIF_USE_DOUBLE build).
// ---------------------------------------------------------------------------

template <class R>
static int cic_device(const R* x, const R* y, const R* z, uint64_t n, uint32_t n_grid, R box,
                      R* grid, const R* w = nullptr) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  if (n_grid < 4) return fail(SIF_ERR_INVALID, "n_grid: expected at least 4");
  cudaStream_t s = e->stream();
  const int st = check_in_box(x, y, z, n, box, "field", s, e->io.flag);
  if (st != SIF_OK) return st;
  RunTimings tm;
  if constexpr (sizeof(R) == 4) {
    e->scratch.ensure(cic_scratch_bytes(n, n_grid, w != nullptr));
    cic_deposit(x, y, z, n, n_grid, box, grid, e->scratch.ptr, s, &tm.cic, nullptr, nullptr,
                nullptr, w);
  } else {
    e->scratch.ensure(cic_f64_scratch_bytes(n_grid));
    cic_deposit_f64(x, y, z, n, n_grid, box, grid, e->scratch.ptr, s, &tm.cic, w);
  }
  SIFG_CUDA(cudaStreamSynchronize(s));
  drop_pending_timings();
  g_timings.cic_ms = tm.cic.total_ms();
  g_timings.cic_launches = tm.cic.launches();
  return SIF_OK;
}

template <class R>
static int contrast_device(R* grid, uint64_t total_cells, double* mean_out) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  cudaStream_t s = e->stream();
  double* scratch = (double*)e->scratch.ensure(density_contrast_scratch_bytes());
  density_contrast(grid, total_cells, scratch, s);
  const double mean = read_mean(scratch, s);
  if (mean_out) *mean_out = mean;
  if (!(mean > 0.0)) return fail(SIF_ERR_RANGE, fmt("grid: mean density %g (expected > 0)", mean));
  SIFG_CUDA(cudaStreamSynchronize(s));
  return SIF_OK;
}

template <class R>
static int mesh_device(const R* x, const R* y, const R* z, uint64_t n, uint32_t n_cells, R box,
                       R* mx, R* my, R* mz, uint32_t* offsets, uint32_t* orig) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  if (n_cells == 0 || !(box > 0.0f)) return fail(SIF_ERR_INVALID, "mesh: bad geometry");
  if (n_cells > kMaxMeshSide)
    return fail(SIF_ERR_RANGE, fmt("mesh: %u cells a side (at most %u)", n_cells, kMaxMeshSide));
  cudaStream_t s = e->stream();
  const int st = check_in_box(x, y, z, n, box, "field", s, e->io.flag);
  if (st != SIF_OK) return st;
  DeviceMeshT<R> m;
  m.n_cells = n_cells;
  m.box_length = box;
  m.cell_length = box / (R)n_cells;
  m.x = mx;
  m.y = my;
  m.z = mz;
  m.offsets = offsets;
  m.orig = orig;
  e->scratch.ensure(mesh_scratch_bytes(n, n_cells) * sizeof(R) / sizeof(float));
  RunTimings tm;
  mesh_build(x, y, z, n, m, e->scratch.ptr, s, &tm.mesh);
  SIFG_CUDA(cudaStreamSynchronize(s));
  drop_pending_timings();
  g_timings.mesh_ms = tm.mesh.total_ms();
  g_timings.mesh_launches = tm.mesh.launches();
  return SIF_OK;
}

template <class R>
static int smooth_device(const R* delta, uint32_t n_grid, R box, R r, int filter,
                         int window_mode, R* out) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  cudaStream_t s = e->stream();
  SmootherT<R>& sm = e->smoother_for<R>();
  sm.setup(n_grid, box, window_mode, s);
  sm.forward(delta);
  RunTimings tm;
  sm.smooth(filter, r, R(0), out, &tm.filter);
  SIFG_CUDA(cudaStreamSynchronize(s));
  drop_pending_timings();
  g_timings.filter_ms = tm.filter.total_ms();
  g_timings.filter_launches = tm.filter.launches();
  return SIF_OK;
}

template <class R>
static int contrast_vjp_device(const R* x, const R* y, const R* z, uint64_t n, uint32_t n_grid,
                               R box, const R* g, R* gx, R* gy, R* gz) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  if (n_grid < 4 || n == 0) return fail(SIF_ERR_INVALID, "vjp: bad grid or no particles");
  cudaStream_t s = e->stream();
  cic_contrast_vjp(x, y, z, n, n_grid, box, g, gx, gy, gz, s);
  SIFG_CUDA(cudaStreamSynchronize(s));
  return SIF_OK;
}

template <class R>
static int run_device(Engine* e, const R* delta, uint32_t n_grid, R box, DeviceMeshT<R>& m,
                      const R* radii, uint32_t n_radii, R threshold, R overlap, uint32_t opt,
                      const R* inject, R* cx, R* cy, R* cz, R* r, uint64_t capacity,
                      uint64_t* n_voids, RunTimings& tm, cudaEvent_t mesh_ready = nullptr,
                      std::vector<RungStat>* stats = &g_stats,
                      const double* contrast_mean = nullptr, const R* prior = nullptr,
                      uint64_t n_prior = 0) {
  if (check_args(radii, n_radii, threshold, overlap) != SIF_OK) return kErrInvalid;
  RunParamsT<R> p;
  p.grid_n = n_grid;
  p.box = box;
  p.threshold = threshold;
  p.overlap = overlap;
  p.options = opt;
  p.radii.assign(radii, radii + n_radii);
  p.window = g_window;
  p.inject = inject;
  p.inject_on_device = true;
  p.mesh_ready = mesh_ready;
  p.contrast_mean = contrast_mean;
  if (n_prior) {
    p.prior_cx = prior;
    p.prior_cy = prior + n_prior;
    p.prior_cz = prior + 2 * n_prior;
    p.prior_r = prior + 3 * n_prior;
    p.n_prior = n_prior;
  }
  // Kept per thread between runs (cleared, capacity kept): fresh vectors would
  // take their page faults on every run.
  thread_local HostCatalogueT<R> cat;
  cat.cx.clear();
  cat.cy.clear();
  cat.cz.clear();
  cat.r.clear();
  if (stats) stats->clear();
  const int st = e->exodus(delta, m, p, cat, stats, &tm);
  if (st != SIF_OK) return st;
  const uint64_t nv = cat.cx.size();
  if (n_voids) *n_voids = nv;
  const uint64_t w = nv < capacity ? nv : capacity;
  if (w) {
    memcpy(cx, cat.cx.data(), w * sizeof(R));
    memcpy(cy, cat.cy.data(), w * sizeof(R));
    memcpy(cz, cat.cz.data(), w * sizeof(R));
    memcpy(r, cat.r.data(), w * sizeof(R));
  }
  return SIF_OK;
}

// A weighted device mesh's columns from the field's weights and the mesh's
// source indices (chain_mesh.c:624-672, 800-801); *total_out (host) gets the
// total weight.
template <class R>
static int mesh_weights_device(const R* field_w, const uint32_t* orig, uint64_t n,
                               const uint32_t* offsets, uint32_t n_cells, R* w_out, R* cell_w_out,
                               double* total_out) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  if (!field_w || !orig || !offsets || !w_out || !cell_w_out || !total_out)
    return fail(SIF_ERR_INVALID, "mesh weights: NULL argument");
  if (n_cells == 0 || n_cells > kMaxMeshSide)
    return fail(SIF_ERR_RANGE, fmt("mesh: %u cells a side (the GPU mesh holds 1 to %u)", n_cells,
                                   kMaxMeshSide));
  cudaStream_t s = e->stream();
  DeviceMeshT<R> m;
  m.n_cells = n_cells;
  m.n_particles = n;
  m.orig = const_cast<uint32_t*>(orig);
  m.offsets = const_cast<uint32_t*>(offsets);
  m.w = w_out;
  m.cell_w = cell_w_out;
  e->scratch.ensure(mesh_weights_scratch_bytes(n_cells) + 64);
  double* d_total = (double*)((char*)e->scratch.ptr + mesh_weights_scratch_bytes(n_cells));
  mesh_weights(field_w, m, e->scratch.ptr, d_total, s);
  SIFG_CUDA(cudaMemcpyAsync(total_out, d_total, sizeof(double), cudaMemcpyDeviceToHost, s));
  SIFG_CUDA(cudaStreamSynchronize(s));
  return SIF_OK;
}

template <class R>
static int exodus_device(const R* delta, uint32_t n_grid, R box, const R* mx, const R* my,
                         const R* mz, const uint32_t* offsets, uint64_t n_particles,
                         uint32_t mesh_cells, const R* radii, uint32_t n_radii, R threshold,
                         R overlap, uint32_t opt, const R* inject, const R* prior,
                         uint64_t n_prior, R* cx, R* cy, R* cz, R* r, uint64_t capacity,
                         uint64_t* n_voids, const R* mw = nullptr, const R* mcw = nullptr,
                         double total_weight = 0.0) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  if (n_prior && !prior) return fail(SIF_ERR_INVALID, "prior: NULL with voids to start from");
  if (mesh_cells == 0 || mesh_cells > kMaxMeshSide)
    return fail(SIF_ERR_RANGE, fmt("mesh: %u cells a side (the GPU mesh holds 1 to %u)", mesh_cells,
                                   kMaxMeshSide));
  if (n_prior) {
    const int st = check_prior(prior, prior + n_prior, prior + 2 * n_prior, prior + 3 * n_prior,
                               n_prior, box);
    if (st != SIF_OK) return st;
  }
  DeviceMeshT<R> m;
  m.n_cells = mesh_cells;
  m.box_length = box;
  m.cell_length = box / (R)mesh_cells;
  m.n_particles = n_particles;
  m.x = const_cast<R*>(mx);
  m.y = const_cast<R*>(my);
  m.z = const_cast<R*>(mz);
  m.offsets = const_cast<uint32_t*>(offsets);
  m.w = const_cast<R*>(mw);
  m.cell_w = const_cast<R*>(mcw);
  m.total_weight = total_weight;
  RunTimings tm;
  const int st = run_device(e, delta, n_grid, box, m, radii, n_radii, threshold, overlap, opt,
                            inject, cx, cy, cz, r, capacity, n_voids, tm, nullptr, &g_stats,
                            nullptr, n_prior ? prior : nullptr, n_prior);
  record_timings(tm);
  return st;
}

static int survey_device(const float* dd, const float* rd, uint32_t n_grid, float box,
                         const sifg_device_mesh_t* data, const sifg_device_mesh_t* randoms,
                         const float* radii, uint32_t n_radii, float threshold, float overlap,
                         uint32_t opt, const float* inject, const float* prior, uint64_t n_prior,
                         float* cx, float* cy, float* cz, float* r, float* foot, float* shell,
                         uint64_t capacity, uint64_t* n_voids) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  if (!dd || !rd || !data || !randoms) return fail(SIF_ERR_INVALID, "survey: NULL argument");
  if (check_args(radii, n_radii, threshold, overlap) != SIF_OK) return SIF_ERR_INVALID;
  if (n_prior && !prior) return fail(SIF_ERR_INVALID, "prior: NULL with voids to start from");
  DeviceMesh m[2];
  const sifg_device_mesh_t* src[2] = {data, randoms};
  for (int k = 0; k < 2; k++) {
    const sifg_device_mesh_t* d = src[k];
    if (d->n_cells == 0 || d->n_cells > kMaxMeshSide || d->n_particles == 0 ||
        d->n_particles >= 0xffffffffull || !d->x || !d->y || !d->z || !d->offsets ||
        (!d->w) != (!d->cell_w) || !(d->total_weight > 0.0))
      return fail(SIF_ERR_INVALID, fmt("%s mesh: bad description", k ? "random" : "data"));
    m[k].n_cells = d->n_cells;
    m[k].box_length = box;
    m[k].cell_length = box / (float)d->n_cells;
    m[k].n_particles = d->n_particles;
    m[k].x = const_cast<float*>(d->x);
    m[k].y = const_cast<float*>(d->y);
    m[k].z = const_cast<float*>(d->z);
    m[k].offsets = const_cast<uint32_t*>(d->offsets);
    m[k].w = const_cast<float*>(d->w);
    m[k].cell_w = const_cast<float*>(d->cell_w);
    m[k].total_weight = d->total_weight;
  }
  RunParams p;
  p.grid_n = n_grid;
  p.box = box;
  p.threshold = threshold;
  p.overlap = overlap;
  p.options = opt;
  p.radii.assign(radii, radii + n_radii);
  p.window = g_window;
  p.inject = inject;
  p.inject_on_device = true;
  p.random_mesh = &m[1];
  p.random_density = rd;
  p.survey_alpha = (float)(data->total_weight / randoms->total_weight);
  if (n_prior) {
    p.prior_cx = prior;
    p.prior_cy = prior + n_prior;
    p.prior_cz = prior + 2 * n_prior;
    p.prior_r = prior + 3 * n_prior;
    p.n_prior = n_prior;
  }
  thread_local HostCatalogue cat;
  for (auto* v : {&cat.cx, &cat.cy, &cat.cz, &cat.r, &cat.foot, &cat.shell}) v->clear();
  g_stats.clear();
  RunTimings tm;
  const int st = e->exodus(dd, m[0], p, cat, &g_stats, &tm);
  record_timings(tm);
  if (st != SIF_OK) return st;
  const uint64_t nv = cat.cx.size();
  if (n_voids) *n_voids = nv;
  const uint64_t w = nv < capacity ? nv : capacity;
  float* dst[6] = {cx, cy, cz, r, foot, shell};
  const std::vector<float>* col[6] = {&cat.cx, &cat.cy, &cat.cz, &cat.r, &cat.foot, &cat.shell};
  for (int k = 0; k < 6 && w; k++)
    if (dst[k]) memcpy(dst[k], col[k]->data(), w * sizeof(float));
  return SIF_OK;
}

// The whole box path on one engine, with the engine's own buffers: the
// device entry point's body, and one job of a batch. stats NULL: no
// per-rung record (a batch worker).
template <class R>
static int box_run(Engine* e, const R* x, const R* y, const R* z, uint64_t n, uint32_t n_grid,
                   R box, uint32_t mesh_cells, const R* radii, uint32_t n_radii, R threshold,
                   R overlap, uint32_t opt, R* cx, R* cy, R* cz, R* r, uint64_t capacity,
                   uint64_t* n_voids, RunTimings& tm, std::vector<RungStat>* stats) {
  if (n_grid < 4 || mesh_cells == 0) return fail(SIF_ERR_INVALID, "grid or mesh: bad size");
  if (mesh_cells > kMaxMeshSide)
    return fail(SIF_ERR_RANGE, fmt("mesh: %u cells a side (at most %u)", mesh_cells, kMaxMeshSide));
  BoxBufs& io = e->io;
  cudaStream_t s = e->stream();
  const uint64_t cells = (uint64_t)n_grid * n_grid * n_grid;
  const uint64_t mcells = (uint64_t)mesh_cells * mesh_cells * mesh_cells;
  R* dg = (R*)io.grid.ensure(cells * sizeof(R));
  // The box check (sif__field_check_in_box) is counted on the device and read
  // when the run ends, not waited for: every stage indexes safely whatever
  // the positions, and a run over positions outside the box returns the
  // range error and no catalogue.
  if (tm.timed) tm.mark_origin(s);
  unsigned long long* outside = (unsigned long long*)io.flag.ensure(16);
  SIFG_CUDA(cudaMemsetAsync(outside, 0, 16, s));
  R bounds[2];
  box_bounds(box, &bounds[0], &bounds[1]);
  // The mesh is built on the copy stream with its own scratch, beside the
  // deposit proper (bound by shared-memory atomics, not by HBM: it starts
  // once the deposit's tile sort has streamed the particles) and the first
  // smoothings; the run waits for it before its first sphere growth. (Queued
  // after the forward transform instead, it took as much time from the first
  // rungs' smoothing as it gave the transform.)
  cudaStream_t cs = e->copy_stream();
  struct CopyDrain {
    cudaStream_t s;
    ~CopyDrain() { cudaStreamSynchronize(s); }
  } drain{cs};
  io.mesh_scratch.ensure(mesh_scratch_bytes(n, mesh_cells) * sizeof(R) / sizeof(float));
  if constexpr (sizeof(R) == 4) {
    e->scratch.ensure(cic_scratch_bytes(n, n_grid));
    cic_deposit(x, y, z, n, n_grid, box, dg, e->scratch.ptr, s, tm.timed ? &tm.cic : nullptr,
                bounds, outside, e->ev_copy_start(), nullptr, tm.timed ? &tm.cic_stage : nullptr);
  } else {
    box_check_kernel<R><<<grid_for(n, 256), 256, 0, s>>>(x, y, z, n, bounds[0], bounds[1], outside);
    SIFG_LAUNCH_CHECK();
    SIFG_CUDA(cudaEventRecord(e->ev_copy_start(), s));
    e->scratch.ensure(cic_f64_scratch_bytes(n_grid));
    cic_deposit_f64(x, y, z, n, n_grid, box, dg, e->scratch.ptr, s, tm.timed ? &tm.cic : nullptr);
  }
  SIFG_CUDA(cudaStreamWaitEvent(cs, e->ev_copy_start(), 0));
  DeviceMeshT<R> m;
  m.n_cells = mesh_cells;
  m.box_length = box;
  m.cell_length = box / (R)mesh_cells;
  if constexpr (sizeof(R) == 4) {
    m.xyzw = (float4*)io.mx.ensure(n * sizeof(float4));
  } else {
    m.x = (R*)io.mx.ensure(n * sizeof(R));
    m.y = (R*)io.my.ensure(n * sizeof(R));
    m.z = (R*)io.mz.ensure(n * sizeof(R));
  }
  m.offsets = (uint32_t*)io.offs.ensure((mcells + 1) * 4);
  m.orig = nullptr;
  uint32_t* sums = (uint32_t*)io.mesh_sums.ensure(
      (size_t)scan_sums_needed((uint32_t)(mcells + 1)) * sizeof(uint32_t));
  // Only the sphere growth reads this mesh: its cells need not be in the
  // canonical order (a radius does not depend on the order within a cell).
  mesh_build(x, y, z, n, m, io.mesh_scratch.ptr, cs, tm.timed ? &tm.mesh : nullptr, sums, false);
  SIFG_CUDA(cudaEventRecord(e->ev_mesh_ready(), cs));
  // The mean only: the contrast is taken by the run's forward transform as it
  // reads the density (the grid is used for nothing else).
  double* cscratch = (double*)io.mean.ensure(density_contrast_scratch_bytes() + 64);
  density_contrast(dg, cells, cscratch, s, true);
  int st = run_device(e, dg, n_grid, box, m, radii, n_radii, threshold, overlap, opt,
                      (const R*)nullptr, cx, cy, cz, r, capacity, n_voids, tm, e->ev_mesh_ready(),
                      stats, contrast_mean(cscratch));
  unsigned long long h_outside = 0;
  SIFG_CUDA(cudaMemcpyAsync(&h_outside, outside, sizeof(h_outside), cudaMemcpyDeviceToHost, s));
  SIFG_CUDA(cudaStreamSynchronize(s));
  if (h_outside) {
    *n_voids = 0;
    return fail(SIF_ERR_RANGE, fmt("field: %llu of %llu particles outside the box [0, %g)",
                                   h_outside, (unsigned long long)n, (double)box));
  }
  return st;
}

template <class R>
static int box_device(const R* x, const R* y, const R* z, uint64_t n, uint32_t n_grid, R box,
                      uint32_t mesh_cells, const R* radii, uint32_t n_radii, R threshold,
                      R overlap, uint32_t opt, R* cx, R* cy, R* cz, R* r, uint64_t capacity,
                      uint64_t* n_voids) {
  Engine* e = engine();
  if (!e) return SIF_ERR_UNINITIALISED;
  const auto t0 = std::chrono::steady_clock::now();
  RunTimings tm;
  const int st = box_run(e, x, y, z, n, n_grid, box, mesh_cells, radii, n_radii, threshold,
                         overlap, opt, cx, cy, cz, r, capacity, n_voids, tm, &g_stats);
  tm.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  record_timings(tm);
  return st;
}

// ---------------------------------------------------------------------------
// The batched form: many independent boxes, each the whole box path, run by a
// pool of engines (each its own streams, buffers and host thread) that take
// the boxes largest first. Every box's catalogue is what sifg_box_device
// gives for it alone: boxes share nothing but the GPU. How many engines run at
// once is the one tuned parameter (sifg_box_batch_autotune).
// ---------------------------------------------------------------------------

static std::vector<std::unique_ptr<Engine>> g_pool;
static std::map<std::pair<int, int>, uint32_t> g_tuned;  // (log2 particles, log2 jobs) -> engines

static std::pair<int, int> batch_key(const sifg_box_job_t* jobs, uint32_t n_jobs) {
  uint64_t total = 0;
  for (uint32_t k = 0; k < n_jobs; k++) total += jobs[k].n_particles;
  return {(int)std::log2((double)std::max<uint64_t>(total, 1)),
          (int)std::log2((double)std::max<uint32_t>(n_jobs, 1))};
}

// One job on one engine.
static void batch_job(Engine* e, sifg_box_job_t& j) {
  const auto t0 = std::chrono::steady_clock::now();
  j.n_voids = 0;
  try {
    uint32_t mc = j.mesh_cells;
    if (mc == 0) {
      float rmax = 0.0f;
      for (uint32_t i = 0; i < j.n_radii; i++) rmax = std::max(rmax, j.radii[i]);
      mc = sif_finder_suggest_mesh_cells(j.n_particles, j.box, rmax, 0.0f);
    }
    RunTimings tm;
    tm.timed = false;
    j.status = box_run<float>(e, j.x, j.y, j.z, j.n_particles, j.n_grid, j.box, mc, j.radii,
                              j.n_radii, j.threshold, j.overlap, j.options, j.cx, j.cy, j.cz,
                              j.r, j.capacity, &j.n_voids, tm, nullptr);
  } catch (const CudaError& err) {
    j.status = cuda_fail(err);
  } catch (const std::bad_alloc&) {
    j.status = fail(SIF_ERR_ALLOC, "batch: out of host memory");
  }
  j.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// The batch's host threads, one per engine, kept between calls (a thread's
// scan scratch lives as long as it does). A call hands each worker the same
// job list and a shared cursor, and waits until every worker is done.
struct BatchPool {
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<std::thread> threads;
  uint64_t generation = 0;
  uint32_t active = 0;  // workers taking part in the current call
  uint32_t busy = 0;    // of them, still working
  sifg_box_job_t* jobs = nullptr;
  const std::vector<uint32_t>* order = nullptr;
  std::atomic<uint32_t> next{0};
  bool stop = false;

  void worker(uint32_t id) {
    uint64_t seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stop || generation != seen; });
      if (stop) return;
      seen = generation;
      const bool mine = id < active;
      lk.unlock();
      if (mine) {
        Engine* e = g_pool[id].get();
        cudaSetDevice(e->device());
        for (;;) {
          const uint32_t k = next.fetch_add(1);
          if (k >= order->size()) break;
          batch_job(e, jobs[(*order)[k]]);
        }
        lk.lock();
        if (--busy == 0) cv_done.notify_all();
      }
    }
  }

  void run(uint32_t n_engines, sifg_box_job_t* j, const std::vector<uint32_t>* o) {
    while (threads.size() < n_engines) {
      const uint32_t id = (uint32_t)threads.size();
      threads.emplace_back(&BatchPool::worker, this, id);
    }
    std::unique_lock<std::mutex> lk(mu);
    jobs = j;
    order = o;
    next = 0;
    active = busy = n_engines;
    generation++;
    cv_work.notify_all();
    cv_done.wait(lk, [&] { return busy == 0; });
  }

  ~BatchPool() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    for (auto& t : threads) t.join();
  }
};

static BatchPool& batch_pool() {
  static BatchPool p;
  return p;
}

static int run_batch(sifg_box_job_t* jobs, uint32_t n_jobs, uint32_t n_engines) {
  Engine* main = engine();
  if (!main) return SIF_ERR_UNINITIALISED;
  if (!jobs && n_jobs) return fail(SIF_ERR_INVALID, "batch: NULL jobs");
  if (n_jobs == 0) return SIF_OK;
  n_engines = std::max(1u, std::min(n_engines, n_jobs));
  while (g_pool.size() < n_engines) g_pool.emplace_back(new Engine(main->device()));
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  for (uint32_t k = 0; k < n_engines; k++) g_pool[k]->host_threads = (int)std::max(1u, hw / n_engines);
  std::vector<uint32_t> order(n_jobs);
  for (uint32_t k = 0; k < n_jobs; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    return jobs[a].n_particles > jobs[b].n_particles;
  });
  batch_pool().run(n_engines, jobs, &order);
  cudaSetDevice(main->device());
  for (uint32_t k = 0; k < n_jobs; k++)
    if (jobs[k].status != SIF_OK) return jobs[k].status;
  return SIF_OK;
}

// Times the batch at 1, 2, 3, 4, 6 and 8 engines (capped by the job count) and
// keeps the fastest for batches of this size. Each count runs twice and the
// second run is timed: an engine's first boxes of a size make its transform
// plans, a cost that later batches do not pay.
static int autotune_batch(sifg_box_job_t* jobs, uint32_t n_jobs, uint32_t* best_out) {
  uint32_t best = 1;
  double best_ms = 1e300;
  for (uint32_t k : {1u, 2u, 3u, 4u, 6u, 8u}) {
    if (k > n_jobs && k > 1) break;
    int st = run_batch(jobs, n_jobs, k);
    if (st != SIF_OK) return st;
    const auto t0 = std::chrono::steady_clock::now();
    st = run_batch(jobs, n_jobs, k);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st != SIF_OK) return st;
    if (ms < best_ms) {
      best_ms = ms;
      best = k;
    }
  }
  g_tuned[batch_key(jobs, n_jobs)] = best;
  if (best_out) *best_out = best;
  return SIF_OK;
}

extern "C" {

#define SIFG_LOCKED(call)               \
  std::lock_guard<std::mutex> lk(g_mu); \
  API_GUARD_BEGIN                       \
  return call;                          \
  API_GUARD_END(SIF_ERR_INVALID)

int sifg_cic_device(const float* x, const float* y, const float* z, uint64_t n, uint32_t n_grid,
                    float box, float* grid) {
  SIFG_LOCKED(cic_device(x, y, z, n, n_grid, box, grid))
}
int sifg_cic_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                        uint32_t n_grid, double box, double* grid) {
  SIFG_LOCKED(cic_device(x, y, z, n, n_grid, box, grid))
}
int sifg_contrast_device(float* grid, uint64_t total_cells, double* mean_out) {
  SIFG_LOCKED(contrast_device(grid, total_cells, mean_out))
}
int sifg_contrast_device_f64(double* grid, uint64_t total_cells, double* mean_out) {
  SIFG_LOCKED(contrast_device(grid, total_cells, mean_out))
}
int sifg_mesh_device(const float* x, const float* y, const float* z, uint64_t n,
                     uint32_t n_cells, float box, float* mx, float* my, float* mz,
                     uint32_t* offsets, uint32_t* orig) {
  SIFG_LOCKED(mesh_device(x, y, z, n, n_cells, box, mx, my, mz, offsets, orig))
}
int sifg_mesh_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                         uint32_t n_cells, double box, double* mx, double* my, double* mz,
                         uint32_t* offsets, uint32_t* orig) {
  SIFG_LOCKED(mesh_device(x, y, z, n, n_cells, box, mx, my, mz, offsets, orig))
}
int sifg_smooth_device(const float* delta, uint32_t n_grid, float box, float r, int filter,
                       int window_mode, float* out) {
  SIFG_LOCKED(smooth_device(delta, n_grid, box, r, filter, window_mode, out))
}
int sifg_smooth_device_f64(const double* delta, uint32_t n_grid, double box, double r,
                           int filter, int window_mode, double* out) {
  SIFG_LOCKED(smooth_device(delta, n_grid, box, r, filter, window_mode, out))
}
int sifg_contrast_vjp_device(const float* x, const float* y, const float* z, uint64_t n,
                             uint32_t n_grid, float box, const float* g, float* gx, float* gy,
                             float* gz) {
  SIFG_LOCKED(contrast_vjp_device(x, y, z, n, n_grid, box, g, gx, gy, gz))
}
int sifg_contrast_vjp_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                                 uint32_t n_grid, double box, const double* g, double* gx,
                                 double* gy, double* gz) {
  SIFG_LOCKED(contrast_vjp_device(x, y, z, n, n_grid, box, g, gx, gy, gz))
}
int sifg_exodus_device(const float* delta, uint32_t n_grid, float box, const float* mx,
                       const float* my, const float* mz, const uint32_t* offsets,
                       uint64_t n_particles, uint32_t mesh_cells, const float* radii,
                       uint32_t n_radii, float threshold, float overlap, uint32_t opt,
                       const float* inject, const float* prior, uint64_t n_prior, float* cx,
                       float* cy, float* cz, float* r, uint64_t capacity, uint64_t* n_voids) {
  SIFG_LOCKED(exodus_device(delta, n_grid, box, mx, my, mz, offsets, n_particles, mesh_cells,
                            radii, n_radii, threshold, overlap, opt, inject, prior, n_prior, cx,
                            cy, cz, r, capacity, n_voids))
}
int sifg_cic_weighted_device(const float* x, const float* y, const float* z, const float* w,
                             uint64_t n, uint32_t n_grid, float box, float* grid) {
  if (!w) return fail(SIF_ERR_INVALID, "weights: NULL");
  SIFG_LOCKED(cic_device(x, y, z, n, n_grid, box, grid, w))
}
int sifg_cic_weighted_device_f64(const double* x, const double* y, const double* z,
                                 const double* w, uint64_t n, uint32_t n_grid, double box,
                                 double* grid) {
  if (!w) return fail(SIF_ERR_INVALID, "weights: NULL");
  SIFG_LOCKED(cic_device(x, y, z, n, n_grid, box, grid, w))
}
int sifg_mesh_weights_device(const float* field_w, const uint32_t* orig, uint64_t n,
                             const uint32_t* offsets, uint32_t n_cells, float* w, float* cell_w,
                             double* total_weight) {
  SIFG_LOCKED(mesh_weights_device(field_w, orig, n, offsets, n_cells, w, cell_w, total_weight))
}
int sifg_mesh_weights_device_f64(const double* field_w, const uint32_t* orig, uint64_t n,
                                 const uint32_t* offsets, uint32_t n_cells, double* w,
                                 double* cell_w, double* total_weight) {
  SIFG_LOCKED(mesh_weights_device(field_w, orig, n, offsets, n_cells, w, cell_w, total_weight))
}
int sifg_exodus_weighted_device(const float* delta, uint32_t n_grid, float box, const float* mx,
                                const float* my, const float* mz, const uint32_t* offsets,
                                const float* w, const float* cell_w, double total_weight,
                                uint64_t n_particles, uint32_t mesh_cells, const float* radii,
                                uint32_t n_radii, float threshold, float overlap, uint32_t opt,
                                const float* inject, const float* prior, uint64_t n_prior,
                                float* cx, float* cy, float* cz, float* r, uint64_t capacity,
                                uint64_t* n_voids) {
  if (!w || !cell_w) return fail(SIF_ERR_INVALID, "mesh weights: NULL");
  SIFG_LOCKED(exodus_device(delta, n_grid, box, mx, my, mz, offsets, n_particles, mesh_cells,
                            radii, n_radii, threshold, overlap, opt, inject, prior, n_prior, cx,
                            cy, cz, r, capacity, n_voids, w, cell_w, total_weight))
}
int sifg_exodus_weighted_device_f64(const double* delta, uint32_t n_grid, double box,
                                    const double* mx, const double* my, const double* mz,
                                    const uint32_t* offsets, const double* w,
                                    const double* cell_w, double total_weight,
                                    uint64_t n_particles, uint32_t mesh_cells,
                                    const double* radii, uint32_t n_radii, double threshold,
                                    double overlap, uint32_t opt, const double* inject,
                                    const double* prior, uint64_t n_prior, double* cx,
                                    double* cy, double* cz, double* r, uint64_t capacity,
                                    uint64_t* n_voids) {
  if (!w || !cell_w) return fail(SIF_ERR_INVALID, "mesh weights: NULL");
  SIFG_LOCKED(exodus_device(delta, n_grid, box, mx, my, mz, offsets, n_particles, mesh_cells,
                            radii, n_radii, threshold, overlap, opt, inject, prior, n_prior, cx,
                            cy, cz, r, capacity, n_voids, w, cell_w, total_weight))
}
int sifg_exodus_survey_device(const float* data_density, const float* random_density,
                              uint32_t n_grid, float box, const sifg_device_mesh_t* data,
                              const sifg_device_mesh_t* randoms, const float* radii,
                              uint32_t n_radii, float threshold, float overlap, uint32_t opt,
                              const float* inject, const float* prior, uint64_t n_prior,
                              float* cx, float* cy, float* cz, float* r, float* footprint,
                              float* footprint_shell, uint64_t capacity, uint64_t* n_voids) {
  SIFG_LOCKED(survey_device(data_density, random_density, n_grid, box, data, randoms, radii,
                            n_radii, threshold, overlap, opt, inject, prior, n_prior, cx, cy, cz,
                            r, footprint, footprint_shell, capacity, n_voids))
}
int sifg_exodus_device_f64(const double* delta, uint32_t n_grid, double box, const double* mx,
                           const double* my, const double* mz, const uint32_t* offsets,
                           uint64_t n_particles, uint32_t mesh_cells, const double* radii,
                           uint32_t n_radii, double threshold, double overlap, uint32_t opt,
                           const double* inject, const double* prior, uint64_t n_prior,
                           double* cx, double* cy, double* cz, double* r, uint64_t capacity,
                           uint64_t* n_voids) {
  SIFG_LOCKED(exodus_device(delta, n_grid, box, mx, my, mz, offsets, n_particles, mesh_cells,
                            radii, n_radii, threshold, overlap, opt, inject, prior, n_prior, cx,
                            cy, cz, r, capacity, n_voids))
}
int sifg_box_device(const float* x, const float* y, const float* z, uint64_t n, uint32_t n_grid,
                    float box, uint32_t mesh_cells, const float* radii, uint32_t n_radii,
                    float threshold, float overlap, uint32_t opt, float* cx, float* cy,
                    float* cz, float* r, uint64_t capacity, uint64_t* n_voids) {
  SIFG_LOCKED(box_device(x, y, z, n, n_grid, box, mesh_cells, radii, n_radii, threshold, overlap,
                         opt, cx, cy, cz, r, capacity, n_voids))
}
int sifg_box_batch_device(sifg_box_job_t* jobs, uint32_t n_jobs, uint32_t n_engines,
                          uint32_t* n_engines_used) {
  std::lock_guard<std::mutex> lk(g_mu);
  API_GUARD_BEGIN
  if (n_engines == 0) {
    auto it = g_tuned.find(batch_key(jobs, n_jobs));
    if (it != g_tuned.end()) {
      n_engines = it->second;
    } else {
      const int st = autotune_batch(jobs, n_jobs, &n_engines);
      if (st != SIF_OK) return st;
    }
  }
  if (n_engines_used) *n_engines_used = std::max(1u, std::min(n_engines, std::max(n_jobs, 1u)));
  return run_batch(jobs, n_jobs, n_engines);
  API_GUARD_END(SIF_ERR_INVALID)
}

int sifg_box_batch_autotune(sifg_box_job_t* jobs, uint32_t n_jobs, uint32_t* n_engines) {
  SIFG_LOCKED(autotune_batch(jobs, n_jobs, n_engines))
}

int sifg_box_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                        uint32_t n_grid, double box, uint32_t mesh_cells, const double* radii,
                        uint32_t n_radii, double threshold, double overlap, uint32_t opt,
                        double* cx, double* cy, double* cz, double* r, uint64_t capacity,
                        uint64_t* n_voids) {
  SIFG_LOCKED(box_device(x, y, z, n, n_grid, box, mesh_cells, radii, n_radii, threshold, overlap,
                         opt, cx, cy, cz, r, capacity, n_voids))
}

uint32_t sifg_last_rung_stats(sifg_rung_stat_t* out, uint32_t max_rungs) {
  const uint32_t n = (uint32_t)g_stats.size();
  for (uint32_t i = 0; i < n && i < max_rungs; i++) {
    const RungStat& s = g_stats[i];
    out[i] = sifg_rung_stat_t{s.radius, s.r_search, s.n_candidates, s.n_survivors, s.n_accepted,
                              s.rounds, s.n_rescale_fail, s.n_overflow, s.rung_ms,
                              s.count_wait_ms, s.sort_ms, s.commit_ms, s.growth_particles,
                              s.growth_cells, s.cand_wait_ms, s.from_list, s.n_witness,
                              s.n_displaced};
  }
  return n;
}

void sifg_last_timings(sifg_timings_t* out) {
  std::lock_guard<std::mutex> lk(g_mu);
  try {
    resolve_timings();
  } catch (const CudaError&) {
    g_last_run.reset();
  }
  if (out) *out = g_timings;
}

uint32_t sifg_last_trace(sifg_trace_event_t* out, uint32_t capacity) {
  std::lock_guard<std::mutex> lk(g_mu);
  try {
    resolve_timings();
  } catch (const CudaError&) {
    g_last_run.reset();
  }
  const uint32_t n = (uint32_t)g_trace.size();
  if (out)
    for (uint32_t i = 0; i < n && i < capacity; i++) out[i] = g_trace[i];
  return n;
}

uint64_t sifg_launch_count(void) { return g_kernel_launches.load(); }

uint64_t sifg_stream(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  try {
    Engine* e = engine();
    return e ? (uint64_t)(uintptr_t)e->stream() : 0;
  } catch (const CudaError& err) {
    cuda_fail(err);
    return 0;
  }
}

void sifg_set_growth_mode(int mode) { set_growth_mode(mode < 0 || mode > 2 ? 0 : mode); }
void sifg_set_shell_list(int entries) { set_shell_list(entries < 0 ? -1 : entries); }
void sifg_set_commit_mode(int mode) { set_commit_mode(mode == 1 ? 1 : 0); }
void sifg_set_scan_mode(int mode) { set_scan_mode(mode == 1 ? 1 : 0); }

void sifg_set_witness(int on) { set_witness(on); }

void sifg_set_factor_tables(int on) { set_factor_tables(on); }

void sifg_set_host_mirrors(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  mirror_enable(on != 0);
}

int sifg_host_mirrors(void) { return mirror_enabled() ? 1 : 0; }

void sifg_host_modified(const void* ptr) {
  std::lock_guard<std::mutex> lk(g_mu);
  mirror_forget(ptr);
}

void sifg_copy_bytes(uint64_t* h2d, uint64_t* d2h) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (h2d) *h2d = g_h2d_bytes;
  if (d2h) *d2h = g_d2h_bytes;
}

void sifg_set_window(int bins) { g_window = bins < 1 ? 1 : (bins > 64 ? 64 : bins); }

void sifg_candidate_ranks(const float* delta, uint32_t m, uint32_t* rank) {
  candidate_ranks(delta, m, rank, 0);
}

}  // extern "C"
