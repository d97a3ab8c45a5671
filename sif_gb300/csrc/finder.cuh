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
  kRescalePending,  // left by the warp-per-survivor growth for the per-CTA one
  kRescaleWitness,  // refused by the collision witness before any growth
  kRescaleNoRandoms,  // a survey: no random weight inside r_search (RESCALE_NO_RANDOMS)
};

// Commit states.
enum : uint8_t { kUndecided = 0, kAccepted = 1, kRejected = 2 };

constexpr uint32_t kVoidCells = 32;  // VOID_CLL_CELLS, src/finder/exodus_finder.c:219

template <class R>
struct MeshViewT {
  const R* x;
  const R* y;
  const R* z;
  const uint32_t* offsets;
  int32_t n;
  R box;
  R inv_l;  // 1 / cell_length
  const float4* xyzw;  // the float form's 16-byte position records, or NULL (x, y, z)
  // A weighted mesh: weights in mesh order and per-cell sums (NULL when
  // unweighted), and the fixed point every sum of them is taken in -- a
  // weight w counts llrint(w * wscale) units of winv -- so that the sums are
  // exact and do not depend on the order the GPU adds in.
  const R* w = nullptr;
  const R* cell_w = nullptr;
  R wscale = 0;
  double winv = 0;
};

template <class R>
struct TemplateViewT {
  const int32_t* dx;
  const int32_t* dy;
  const int32_t* dz;
  const uint8_t* type;
  const R* min_d2;
  const R* max_d2;
  uint32_t count;
};

// Everything a rung's kernels share, computed on the host in the reference's
// sif_real expressions (src/finder/exodus_finder.c:1629-1632, 1771-1817,
// 1848-1851; src/finder/exodus_rescale.c:681-720, 894-908).
template <class R>
struct RungConstsT {
  R radius, r_search, rmin;
  R rs2, rc2, inv_w, bin_w, K2, expected, threshold;
  uint32_t nb;
  int32_t proxy_pole;
  R scale, f;  // overlap scale (Lagrangian) and fraction
  R cell;      // grid cell length
  uint32_t grid_n;
  R box;
  R gbox;  // grid_n * cell, the box paint_sphere measures in
  uint32_t window;
};

// Accepted voids in a 32^3 periodic cell index, as compressed rows.
template <class R>
struct VoidViewT {
  const R* cx;
  const R* cy;
  const R* cz;
  const R* r;
  const uint32_t* start;  // kVoidCells^3 + 1
  const uint32_t* ids;
  R inv_cell;  // 32 / box
  R max_r;
  uint32_t n;
};

// A survivor's centre and rescaled radius, as the commit's neighbour walk
// reads them: one load a neighbour.
template <class R>
struct SurvPackT {
  R x, y, z, r;
};

// Survivors of the pre-filter, hashed on a coarse grid for the commit's
// neighbour queries.
template <class R>
struct SurvivorGridT {
  const uint32_t* start;  // ng^3 + 1
  const uint32_t* ids;
  int32_t ng;
  R inv_cell;  // ng / box
  const SurvPackT<R>* pack;  // each slot's survivor's centre and radius, in the grid's order
  const uint32_t* hrank;     // and its rank (survivor_grid_ranks, once the order is known)
};

template <class R>
struct SurvivorsT {
  const uint32_t* cand;  // candidate index of each survivor
  const uint32_t* flat;  // its node, as a flat grid index
  R* cx;
  R* cy;
  R* cz;
  R* r;             // rescaled radius, or -1
  uint8_t* reason;  // rescale outcome
  const uint32_t* count;  // device-side survivor count
  // Under SIF_FINDER_REFINE_GAUSSIAN: each survivor's centre's distance off
  // its node (|offset| * cell), or -1 on the node; NULL: all on their nodes.
  const R* off = nullptr;
};

// A candidate's centre off its node (sif_offset_t, src/finder/utils.h:
// 164-172), in cells, and len = |offset| * cell as masked_overlap takes it
// (exodus_finder.c:440-452); len -1 for a candidate on its node.
template <class R>
struct CandOffT {
  R dx, dy, dz, len;
};

using MeshView = MeshViewT<float>;
using TemplateView = TemplateViewT<float>;
using RungConsts = RungConstsT<float>;
using VoidView = VoidViewT<float>;
using SurvivorGrid = SurvivorGridT<float>;
using Survivors = SurvivorsT<float>;

// --- host wrappers (finder.cu), instantiated for float and double ---

// Candidate scan (src/finder/utils.c:130-213): cells with delta <= threshold
// whose mask bit is clear, in flat order; with `minima` only those that are
// local minima of the field (SIF_FINDER_SEEDS_MINIMA, utils.c:406-552).
// The count pass leaves per-block offsets in `block_counts`
// (scan_blocks(n) + 1 entries) and the total in *d_count; the write pass
// fills the candidates. grid_n: the grid's side.
uint32_t scan_blocks(uint64_t n_cells);
template <class R>
void scan_count_pass(const R* field, const uint32_t* mask, uint64_t n_cells, R threshold,
                     uint32_t* block_counts, uint32_t* d_count, cudaStream_t st, uint32_t grid_n,
                     bool minima);
template <class R>
void scan_write_pass(const R* field, const uint32_t* mask, uint64_t n_cells, R threshold,
                     const uint32_t* block_counts, R* cand_delta, uint32_t* cand_flat,
                     cudaStream_t st, uint32_t grid_n, bool minima);
// The same candidates from one pass over the field: each block's go to its
// own region (scan_region_slots(n) slots in all) with the count and offsets
// as scan_count_pass leaves them; scan_compact then gathers them in order.
uint64_t scan_region_slots(uint64_t n_cells);
template <class R>
void scan_fused_pass(const R* field, const uint32_t* mask, uint64_t n_cells, R threshold,
                     uint32_t* block_counts, uint32_t* d_count, R* region_delta,
                     uint32_t* region_flat, cudaStream_t st, uint32_t grid_n, bool minima);
template <class R>
void scan_compact(const uint32_t* block_counts, uint64_t n_cells, const R* region_delta,
                  const uint32_t* region_flat, R* cand_delta, uint32_t* cand_flat,
                  cudaStream_t st);

// The candidates (cells mode) from the below-threshold list a smoothing made
// (blocks of `block` cells, counts per block, block b's entries at the start
// of its region of delta and flat): the listed cells whose mask bit is
// clear, in flat order. The count pass leaves the per-block offsets in
// block_counts (nb + 1 entries) and the total in *d_count, as
// scan_count_pass does; the write pass fills the candidates.
void below_count_pass(const uint32_t* counts, const uint32_t* flat, uint32_t nb, uint32_t block,
                      const uint32_t* mask, uint32_t* block_counts, uint32_t* d_count,
                      cudaStream_t st);
void below_write_pass(const uint32_t* counts, const float* delta, const uint32_t* flat,
                      uint32_t nb, uint32_t block, const uint32_t* mask,
                      const uint32_t* block_offsets, float* cand_delta, uint32_t* cand_flat,
                      cudaStream_t st);

// Pre-filter at the rung radius (prefilter_cells, exodus_finder.c:871-944)
// and compaction of the survivors, candidate order kept; with keep_all
// (displacement) every candidate survives.
// coff: the candidates' offsets (SIF_FINDER_REFINE_GAUSSIAN), or NULL when
// every candidate sits on its node; soff then receives each survivor's
// offset length (or is NULL).
template <class R>
void prefilter(const uint32_t* cand_flat, uint32_t m, const uint32_t* mask, VoidViewT<R> voids,
               RungConstsT<R> rc, uint8_t* alive, uint32_t* block_counts, uint32_t* surv_cand,
               uint32_t* surv_flat, R* scx, R* scy, R* scz, uint32_t* d_surv_count,
               cudaStream_t st, bool keep_all = false, const CandOffT<R>* coff = nullptr,
               R* soff = nullptr);

// SIF_FINDER_REFINE_GAUSSIAN's placing (sif__finder_scan_refined, src/finder/
// utils.c:406-552): the m candidates (cdelta, cflat: the cells at or below
// thr on the top-hat fa, unmasked, flat order) placed on the refinement's
// field fb -- depth from fb, minima moved by a Newton step -- and, under
// minima_only, reduced to the minima. On return cdelta and cflat point at
// the placed list (the tmp buffers or the originals, swapped as needed),
// coff at its offsets (o_tmp or o_out); keep holds m + 1 entries; h_count is
// pinned host memory. Returns the candidates left (a host sync under
// minima_only).
template <class R>
uint32_t refine_candidates(const R* fa, const R* fb, const uint32_t* mask, R thr, uint32_t n,
                           R cell, uint32_t m, bool minima_only, R*& cdelta, uint32_t*& cflat,
                           R* d_tmp, uint32_t* f_tmp, CandOffT<R>* o_tmp, CandOffT<R>*& coff,
                           CandOffT<R>* o_out, uint32_t* keep, uint32_t* h_count,
                           cudaStream_t st);

// The collision witness (collision_radius, src/finder/exodus_finder.c:
// 780-845, and sif__exodus_witness, src/finder/exodus_rescale.c:1074-1167):
// a survivor whose crossing is certain to lie past the radius at which it
// collides with a void of `voids` (the catalogue as the rung begins) is
// refused before any growth, as the reference refuses it -- the commit would
// refuse it at any radius it could return. Writes every survivor's outcome:
// kRescaleWitness (radius -1) or kRescaleOk (to be grown). traffic as grow's;
// work: a device counter (zeroed here) from which the warps take survivors.
template <class R>
void witness(MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> s,
             VoidViewT<R> voids, uint32_t max_survivors, unsigned long long* traffic,
             cudaStream_t st, KernelTimer* timer, uint32_t* work);

// 1 (default): the witness runs; 0: every survivor is grown. The catalogue
// does not depend on it (tests run both).
void set_witness(int on);

// Sphere growth of every survivor, or (only != kAllSurvivors) of those whose
// rescale outcome is `only`; with only == kAllSurvivors, survivors the
// witness refused are left as they are. gbuf: a global overflow scratch of
// grid * gcap values.
constexpr uint8_t kAllSurvivors = 0xff;
unsigned growth_grid();
// traffic (may be NULL): two counters the kernel adds to -- particles read
// and template cells visited. work: two device counters (zeroed here) from
// which the warps or CTAs take survivors.
template <class R>
void grow(MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> s,
          uint32_t max_survivors, R* gbuf, uint32_t gcap, unsigned long long* traffic,
          cudaStream_t st, KernelTimer* timer, uint8_t only, uint32_t* work,
          uint32_t* pend = nullptr);
// The weighted sphere growth (sif__exodus_find_radius_weighted,
// exodus_rescale.c:642-1037 with the weighted flag): mesh.w set. A CTA per
// survivor; gbuf and gwbuf (gcap entries per CTA each) hold the windows too
// wide for shared memory.
template <class R>
void grow_weighted(MeshViewT<R> mesh, TemplateViewT<R> tpl, RungConstsT<R> rc, SurvivorsT<R> s,
                   uint32_t max_survivors, R* gbuf, long long* gwbuf, uint32_t gcap,
                   unsigned long long* traffic, cudaStream_t st, KernelTimer* timer,
                   uint8_t only, uint32_t* work);
// A survey's sphere growth (sif__exodus_find_radius_survey, src/finder/
// exodus_rescale.c:2154-2317): the largest data distance at which the data
// weight inside is at most K times the random weight, data on dm with
// template dt, randoms on rm with rt (each mesh's weights, or 1 a tracer,
// in its own fixed point: wscale and winv set either way). Every survivor.
template <class R>
void grow_survey(MeshViewT<R> dm, TemplateViewT<R> dt, MeshViewT<R> rm, TemplateViewT<R> rt,
                 RungConstsT<R> rc, R K, SurvivorsT<R> s, uint32_t max_survivors, R* gbuf,
                 long long* gwbuf, uint32_t gcap, unsigned long long* traffic, cudaStream_t st,
                 KernelTimer* timer, uint32_t* work);
// The survey's footprint and field (survey.cu; src/finder/exodus_survey.c).
// The nodes nearest the randoms (n^3 bits, (n^3 + 31) / 32 words of occ),
// and how many: survey_mark returns the marked count (synchronises st).
template <class R>
uint64_t survey_mark(const R* x, const R* y, const R* z, uint64_t n_randoms, uint32_t n, R box,
                     uint32_t* occ, unsigned long long* d_count, cudaStream_t st);
// The closing over 2k + 1 nodes (dilate then erode along each axis; tmp of
// the same size as occ), the result back in occ.
void survey_close(uint32_t* occ, uint32_t* tmp, uint32_t n, int32_t k, cudaStream_t st);
// The closing's k for n_randoms over `marked` nodes (exodus_survey.c:181-188).
int32_t survey_closing_k(uint64_t n_randoms, uint64_t marked);
// The scanned field over the smoothed data: data / (alpha randoms) - 1 on
// observed nodes with randoms, SIF__FINDER_UNOBSERVED elsewhere.
template <class R>
void survey_contrast(R* data, const R* randoms, const uint32_t* occ, R alpha, uint64_t cells,
                     cudaStream_t st);
// Each void's observed fractions of its sphere and of the shell to twice its
// radius (survey_void_footprint, exodus_survey.c:240-296).
template <class R>
void survey_footprint(const R* cx, const R* cy, const R* cz, const R* r, uint32_t n_voids,
                      const uint32_t* occ, uint32_t n, R box, R* inside, R* shell,
                      cudaStream_t st);
// The bounding box of n positions (lo[3], hi[3] on the host; synchronises).
template <class R>
void extent(const R* x, const R* y, const R* z, uint64_t n, R lo[3], R hi[3], cudaStream_t st);
// Counts a weighted mesh's negative (below zero; a negative zero is not)
// and non-finite weights into counts[0], counts[1] (device, zeroed here).
template <class R>
void check_weights(const R* w, uint64_t n, unsigned long long* counts, cudaStream_t st);
// The fixed-point scale of a weighted mesh's sums (MeshViewT::wscale and
// winv): 2^s with s chosen so that `bound` (the most weight any one sum can
// reach) stays below 2^58 units.
void weight_fixed_point(double bound, double* wscale, double* winv);

// Which growth kernel runs: 0 by the survivor count (a CTA per survivor for
// few, a warp per survivor for many), 1 always a CTA, 2 always a warp. The
// radii are the same either way (tests run both).
void set_growth_mode(int mode);
// The warp growth kernel's shell list: -1 sized per rung from the shell's
// expected count (none for large spheres), 0 none, n > 0 that many entries
// (rounded up to 32, at most 512) on every rung. The radii are the same.
void set_shell_list(int entries);

// The survivor hash for the commit (after the growth: pack holds the radii).
template <class R>
void build_survivor_grid(const R* scx, const R* scy, const R* scz, const R* sr,
                         const uint32_t* d_count, uint32_t max_survivors, int32_t ng, R box,
                         uint32_t* start, uint32_t* ids, uint32_t* cell_of, SurvPackT<R>* pack,
                         cudaStream_t st);
// hrank[k] = rank of the survivor in slot k of the hash (rank: the candidates').
template <class R>
void survivor_grid_ranks(SurvivorsT<R> s, const uint32_t* rank, const uint32_t* ids,
                         uint32_t* hrank, uint32_t max_survivors, cudaStream_t st);

// Survivors whose rescaling failed, or whose sphere at the rescaled radius
// overlaps a void of the catalogue as the rung began (voids), start
// rejected, the rest undecided; counters[4] counts the failures,
// counters[5] the resolve overflows, counters[8] the witness's refusals
// (among the failures).
template <class R>
void commit_init(SurvivorsT<R> s, VoidViewT<R> voids, RungConstsT<R> rc, uint8_t* state,
                 uint32_t* counters, uint32_t max_survivors, cudaStream_t st);

// The commit's counters: [0] accepted so far (appended to acc); the largest
// accepted radius as the bits of a float in [3], of a double in [6..7]; [4]
// rescaling failures, [5] resolve overflows, [8] witness refusals, [9]
// acceptances at more than twice the rung's radius; then two rings of kRoundRing
// slots indexed by round % kRoundRing: the accepted count when the round
// began (written by the previous round's paint), and the survivors the round
// left undecided (zeroed by the host before each batch of rounds).
constexpr uint32_t kCommitWork = 15;  // counters[]: the round's pass's next survivor
constexpr uint32_t kRoundRing = 64;
constexpr uint32_t kRoundBegin = 16;
constexpr uint32_t kRoundUndecided = kRoundBegin + kRoundRing;
constexpr uint32_t kCommitCounters = kRoundUndecided + kRoundRing;

// One commit round: sweep, readiness, acceptance.
template <class R>
void commit_round(SurvivorsT<R> s, const uint32_t* rank, SurvivorGridT<R> g, VoidViewT<R> voids,
                  const uint32_t* mask, RungConstsT<R> rc, const uint8_t* state_in,
                  uint8_t* state_out, uint32_t* acc, uint32_t* counters, uint32_t round,
                  uint32_t max_survivors, cudaStream_t st);
// The rounds from `round0` on in one cooperative launch, until a round leaves
// no survivor undecided or max_rounds (at most kRoundRing) have run; round k
// reads states from sa (k even) or sb and writes the other. bar: four
// words, reset by the call; bar[3] ends up holding the rounds run and
// bar[2] is set if a grid barrier timed out. Returns false, launching
// nothing, where the device cannot run it (or set_commit_mode(1) asked for
// a kernel launch per round): the caller then runs commit_round and
// paint_new per round. max_survivors bounds the survivors: the launch takes
// a block per kCommitT of them, at most one per SM.
template <class R>
bool commit_rounds(SurvivorsT<R> s, const uint32_t* rank, SurvivorGridT<R> g, VoidViewT<R> voids,
                   uint32_t* mask, RungConstsT<R> rc, uint8_t* sa, uint8_t* sb, uint32_t* acc,
                   uint32_t* counters, uint32_t round0, uint32_t max_rounds, unsigned* bar,
                   uint32_t max_survivors, cudaStream_t st);
// 0 (default): the commit's rounds in one cooperative launch where the device
// allows it; 1: a launch per round. The catalogue does not depend on it.
void set_commit_mode(int mode);

// Paints n_voids given voids (a prior catalogue) into the mask at scale * r
// (rc: scale, cell, gbox, grid_n), as the commit paints the ones it accepts.
template <class R>
void paint_voids(const R* cx, const R* cy, const R* cz, const R* r, uint32_t n_voids,
                 uint32_t* mask, RungConstsT<R> rc, cudaStream_t st);
// Paints the voids round `round` accepted and records where the next round's
// acceptances begin.
template <class R>
void paint_new(SurvivorsT<R> s, const uint32_t* acc, uint32_t* counters, uint32_t round,
               uint32_t* mask, RungConstsT<R> rc, uint32_t max_survivors, cudaStream_t st);

// Appends the rung's accepted voids to the catalogue in candidate-rank order.
template <class R>
void append_accepted(SurvivorsT<R> s, const uint32_t* rank, const uint32_t* acc,
                     const uint32_t* counters, uint32_t m_candidates, uint32_t* rank_slots,
                     R* cat_x, R* cat_y, R* cat_z, R* cat_r, uint32_t n_voids,
                     uint32_t max_survivors, cudaStream_t st);

// Displacement (SIF_FINDER_DISPLACE, exodus_finder.c:696-756, 946-1078,
// 2239-2275): every survivor (every candidate: no pre-filter) in rank order
// by one CTA, against a linked void index rebuilt from the compressed one
// (vstart, vids over the first state[0] voids of the catalogue): refused by
// its mask bit, the poles and the exact overlap at the rung radius, or by a
// colliding void at least its size; else the smaller voids it collides with
// are displaced (radius negated, sphere cleared, intersecting spheres painted
// back) and it is appended. state: [0] the catalogue's voids (in and out),
// [1] accepted, [2] displaced, [3] a list overflowed (cap entries each for
// conflicts and paints), [4..5] the largest radius (in and out), [6]
// acceptances at more than twice the rung's radius.
template <class R>
void displace_commit(SurvivorsT<R> s, const uint32_t* rank, uint32_t m, uint32_t* order,
                     const uint32_t* vstart, uint32_t* vids, int32_t* head, int32_t* next,
                     R* cat_x, R* cat_y, R* cat_z, R* cat_r, R box, uint32_t* mask,
                     RungConstsT<R> rc, uint32_t* state, uint32_t* conflicts, uint32_t* paints,
                     uint32_t cap, cudaStream_t st);
// The displaced voids (radius <= 0) dropped, order kept; state[0] updated.
template <class R>
void compact_voids(R* cx, R* cy, R* cz, R* r, uint32_t* state, cudaStream_t st);

// Rebuilds the void index over the first n voids.
template <class R>
void build_void_index(const R* cx, const R* cy, const R* cz, uint32_t n, R box, uint32_t* start,
                      uint32_t* ids, uint32_t* cell_of, cudaStream_t st);

}  // namespace sifg
