// The per-rung finder stages (finder.cu): candidate scan, pre-filter,
// sphere growth, the commit rounds, mask painting and the void index.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace sifg {

// Cell classes of the rescaling template (src/finder/exodus_rescale.c:156-160).
constexpr uint8_t kCellCore = 1;
constexpr uint8_t kCellStraddle = 2;
constexpr uint8_t kCellEdge = 3;
constexpr uint8_t kCellShell = 4;

// Rescaling outcomes (src/finder/exodus_internal.h:167-176), plus the one
// the GPU adds: a resolve window larger than its largest scratch.
enum : uint8_t {
  kRescaleOk = 0,
  kRescaleEmpty,
  kRescaleBeyondSearch,
  kRescaleBelowRung,
  kRescaleDegenerate,
  kRescaleOverflow,
};

// Commit states.
enum : uint8_t { kUndecided = 0, kAccepted = 1, kRejected = 2 };

constexpr uint32_t kVoidCells = 32;  // VOID_CLL_CELLS, src/finder/exodus_finder.c:219

struct MeshView {
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* offsets;
  int32_t n;
  float box;
  float inv_l;  // 1.0f / cell_length
};

struct TemplateView {
  const int32_t* dx;
  const int32_t* dy;
  const int32_t* dz;
  const uint8_t* type;
  const float* min_d2;
  const float* max_d2;
  uint32_t count;
};

// Everything a rung's kernels share, computed on the host in the reference's
// float expressions (src/finder/exodus_finder.c:1629-1632, 1771-1817, 1848-1851;
// src/finder/exodus_rescale.c:681-720, 894-908).
struct RungConsts {
  float radius, r_search, rmin;
  float rs2, rc2, inv_w, bin_w, K2, expected, threshold;
  uint32_t nb;
  int32_t proxy_pole;
  float scale, f;  // overlap scale (Lagrangian) and fraction
  float cell;      // grid cell length
  uint32_t grid_n;
  float box;
  float gbox;  // (float)grid_n * cell, the box paint_sphere measures in
  uint32_t window;
};

// Accepted voids in a 32^3 periodic cell index, as compressed rows.
struct VoidView {
  const float* cx;
  const float* cy;
  const float* cz;
  const float* r;
  const uint32_t* start;  // kVoidCells^3 + 1
  const uint32_t* ids;
  float inv_cell;  // (float)32 / box
  float max_r;
  uint32_t n;
};

// Survivors of the pre-filter, hashed on a coarse grid for the commit's
// neighbour queries.
struct SurvivorGrid {
  const uint32_t* start;  // ng^3 + 1
  const uint32_t* ids;
  int32_t ng;
  float inv_cell;  // ng / box
};

struct Survivors {
  const uint32_t* cand;  // candidate index of each survivor
  const uint32_t* flat;  // its node, as a flat grid index
  float* cx;
  float* cy;
  float* cz;
  float* r;         // rescaled radius, or -1
  uint8_t* reason;  // rescale outcome
  const uint32_t* count;  // device-side survivor count
};

// --- host wrappers (finder.cu) ---

// Candidate scan (src/finder/utils.c:130-213): cells with delta <= threshold
// whose mask bit is clear, in flat order. The count pass leaves per-block
// offsets in `block_counts` (scan_blocks(n) + 1 entries) and the total in
// *d_count; the write pass fills the candidates.
uint32_t scan_blocks(uint64_t n_cells);
void scan_count_pass(const float* field, const uint32_t* mask, uint64_t n_cells, float threshold,
                     uint32_t* block_counts, uint32_t* d_count, cudaStream_t st);
void scan_write_pass(const float* field, const uint32_t* mask, uint64_t n_cells, float threshold,
                     const uint32_t* block_counts, float* cand_delta, uint32_t* cand_flat,
                     cudaStream_t st);

// Pre-filter at the rung radius (prefilter_cells, exodus_finder.c:871-944)
// and compaction of the survivors, candidate order kept.
void prefilter(const uint32_t* cand_flat, uint32_t m, const uint32_t* mask, VoidView voids,
               RungConsts rc, uint8_t* alive, uint32_t* block_counts, uint32_t* surv_cand,
               uint32_t* surv_flat, float* scx, float* scy, float* scz, uint32_t* d_surv_count,
               cudaStream_t st);

// Sphere growth of every survivor. gbuf: a global overflow scratch of
// grid * gcap floats.
unsigned growth_grid();
// traffic (may be NULL): two counters the kernel adds to -- particles read
// and template cells visited.
void grow(MeshView mesh, TemplateView tpl, RungConsts rc, Survivors s, uint32_t max_survivors,
          float* gbuf, uint32_t gcap, unsigned long long* traffic, cudaStream_t st,
          KernelTimer* timer);

// The survivor hash for the commit.
void build_survivor_grid(const float* scx, const float* scy, const float* scz,
                         const uint32_t* d_count, uint32_t max_survivors, int32_t ng, float box,
                         uint32_t* start, uint32_t* ids, uint32_t* cell_of, cudaStream_t st);

// Survivors whose rescaling failed start rejected, the rest undecided;
// counters[4] counts the failures, counters[5] the resolve overflows.
void commit_init(Survivors s, uint8_t* state, uint32_t* counters, uint32_t max_survivors,
                 cudaStream_t st);

// One commit round: sweep, readiness, acceptance. counters[0] accepted so
// far (appended to acc), counters[1] left undecided, counters[2] the
// accepted count when the round began, counters[3] the largest accepted
// radius (float bits).
void commit_round(Survivors s, const uint32_t* rank, SurvivorGrid g, VoidView voids,
                  const uint32_t* mask, RungConsts rc, const uint8_t* state_in, uint8_t* state_out,
                  uint32_t* acc, uint32_t* counters, uint32_t max_survivors, cudaStream_t st);
void paint_new(Survivors s, const uint32_t* acc, const uint32_t* counters, uint32_t* mask,
               RungConsts rc, uint32_t max_survivors, cudaStream_t st);

// Appends the rung's accepted voids to the catalogue in candidate-rank order.
void append_accepted(Survivors s, const uint32_t* rank, const uint32_t* acc,
                     const uint32_t* counters, uint32_t m_candidates, uint32_t* rank_slots,
                     float* cat_x, float* cat_y, float* cat_z, float* cat_r, uint32_t n_voids,
                     uint32_t max_survivors, cudaStream_t st);

// Rebuilds the void index over the first n voids.
void build_void_index(const float* cx, const float* cy, const float* cz, uint32_t n, float box,
                      uint32_t* start, uint32_t* ids, uint32_t* cell_of, cudaStream_t st);

}  // namespace sifg
