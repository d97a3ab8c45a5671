/*
 * CPU restatement of sif's exodus void-finder path. TEST INFRASTRUCTURE ONLY:
 * the checker the GPU library is compared against, and the CPU baseline
 * bench.py times ("port"). Never linked by the product.
 *
 * Each function cites the reference file:line it restates. Single precision
 * throughout the finder, in the reference's operation order, built with
 * -ffp-contract=off so that no multiply-add is fused: bit for bit what the
 * reference computes in a strict IEEE build (-fno-fast-math, no contraction).
 */
#ifndef SIF_ORACLE_EXODUS_H
#define SIF_ORACLE_EXODUS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A chain mesh: particles grouped by cell, cells in flat (x-major) order,
 * each cell's particles in source order (src/structures/chain_mesh.c:420-542).
 */
typedef struct {
  const float* x;
  const float* y;
  const float* z;
  const uint64_t* offsets; /* total_cells + 1 */
  uint64_t n_particles;
  uint32_t n_cells;
  float box_length;
  float cell_length;
  /* A weighted mesh (sif_chain_mesh_t::weights, cell_weights, total_weight,
   * include/sif/structures/chain_mesh.h:60-89): per-particle weights in mesh
   * order, their per-cell sums and their total; w NULL when unweighted. */
  const float* w;
  const float* cell_w;
  double total_weight;
} orc_mesh_t;

/* The mesh's weight columns (chain_mesh.c:624-672, 800-801): the field's
 * weights in mesh order through the source-index map, each cell's sum in
 * double rounded to float, and the total over 64 fixed blocks of cells. */
void orc_mesh_weights(const float* field_w, const uint64_t* orig, uint64_t n,
  const uint64_t* offsets, uint32_t n_cells, float* out_w, float* out_cell_w,
  double* total);

/* Builds a mesh into caller storage (n entries per column, n_cells^3 + 1
 * offsets, optional source-index map). 0, or -2 for invalid input. */
int orc_chain_mesh(const float* x, const float* y, const float* z, uint64_t n,
  uint32_t n_cells, float box, float* ox, float* oy, float* oz,
  uint64_t* offsets, uint64_t* orig);

/* CIC density per unit volume in double, every corner weight in double. */
void orc_cic_f64(const float* x, const float* y, const float* z, uint64_t n,
  uint32_t grid_n, float box, double* out);

/* The reference's float CIC (src/structures/grid.c:455-746): density per
 * unit volume, its slab and chunk order, so its bits. */
void orc_cic_float(const float* x, const float* y, const float* z, uint64_t n,
  uint32_t grid_n, float box, float* out);
/* Both with per-particle weights (NULL: every weight 1), grid.c:635-639. */
void orc_cic_float_w(const float* x, const float* y, const float* z, const float* w,
  uint64_t n, uint32_t grid_n, float box, float* out);
void orc_cic_f64_w(const float* x, const float* y, const float* z, const float* w,
  uint64_t n, uint32_t grid_n, float box, double* out);

/* The density contrast of an FP64 density in double: 0, or -3 if the mean
 * is not positive. */
int orc_density_contrast_f64(double* v, uint64_t n);

/* sif_grid_to_density_contrast in place: 0, or -3 if the mean is not
 * positive. */
int orc_density_contrast(float* v, uint64_t n);

/* The smoothing: a density-contrast grid transformed once, then filtered per
 * radius. mode 0 computes the reference's formulas in exact double (the FP64
 * oracle field); mode 1 follows the reference's float filter table and float
 * spectrum rounding. filter: 1 top-hat, 2 Gaussian. */
typedef struct orc_spectrum orc_spectrum_t;
orc_spectrum_t* orc_spectrum_new(const float* delta, uint32_t n, float box,
  int window_mode /* 0 none, 1 full CIC, 2 aliasing-aware CIC */, int mode);
/* The FP64 spectrum (mode 0) of a double contrast: the whole chain in double. */
orc_spectrum_t* orc_spectrum_new_f64(const double* delta, uint32_t n, float box,
  int window_mode);
void orc_spectrum_smooth(orc_spectrum_t* s, int filter, float r, float sigma,
  float* out_f, double* out_d);
void orc_spectrum_free(orc_spectrum_t* s);

/* Candidate records and the reference's 3-way quicksort permutation of them
 * (include/sif/utils/sort.h:56-98 over sif_candidate_t, src/finder/utils.h:122-131). */
typedef struct {
  float delta;
  uint32_t refined;
  uint64_t flat;
} orc_candidate_t;
void orc_sort_candidates(orc_candidate_t* c, uint64_t n);

/* The rescaling template (src/finder/exodus_rescale.c:175-283). */
typedef struct {
  int32_t* dx;
  int32_t* dy;
  int32_t* dz;
  uint8_t* type;
  float* min_d2;
  float* max_d2;
  uint32_t count;
} orc_template_t;
int orc_template_build(orc_template_t* t, uint32_t mesh_n, float cell_length,
  float rmin, float r_search);
void orc_template_free(orc_template_t* t);

/* Reasons, src/finder/exodus_internal.h:167-176. */
enum {
  ORC_RESCALE_OK = 0,
  ORC_RESCALE_EMPTY,
  ORC_RESCALE_BEYOND_SEARCH,
  ORC_RESCALE_BELOW_RUNG,
  ORC_RESCALE_DEGENERATE,
  ORC_RESCALE_ALLOC
};

/* sif__exodus_find_radius (src/finder/exodus_rescale.c:642-1027), unweighted.
 * `window` bins are resolved per pass; span_sum/span_count accumulate as the
 * reference's scratch does. Returns the radius, or -1 with *reason set. */
float orc_find_radius(const orc_mesh_t* m, const orc_template_t* tpl, float cx,
  float cy, float cz, float r_search, float threshold, float vol_factor,
  float rmin, uint32_t window, uint8_t* reason, uint64_t* span_sum,
  uint64_t* span_count);

/* sif__exodus_find_radius_weighted (exodus_rescale.c:642-1037 with the
 * weighted flag): the mesh's weights in every sum, double accumulators in the
 * reference's order, mass_factor in the density tests. */
float orc_find_radius_weighted(const orc_mesh_t* m, const orc_template_t* tpl, float cx,
  float cy, float cz, float r_search, float threshold, float vol_factor,
  float mass_factor, float rmin, uint32_t window, uint8_t* reason, uint64_t* span_sum,
  uint64_t* span_count);

/* Double-precision brute force over every particle (the definition the
 * reference's tests/test_finders.c:419-459 checks against). */
double orc_brute_force_radius(const float* x, const float* y, const float* z,
  uint64_t n, float box, double cx, double cy, double cz, double rung,
  double r_search, double threshold);

/* Per-rung counts, as src/finder/utils.h sif_finder_radius_stats_t. */
typedef struct {
  uint64_t n_candidates;
  uint64_t rejected_masked;
  uint64_t rejected_proxy;
  uint64_t rejected_overlap;
  uint64_t rejected_rescale;
  uint64_t rejected_proxy_recheck;
  uint64_t rejected_exact;
  uint64_t rejected_witness;
  uint64_t accepted;
  uint64_t n_rescaled;
} orc_rung_stats_t;

typedef struct {
  uint32_t grid_n;
  float box_length;
  float threshold;
  float overlap_fraction;
  uint32_t options;   /* sif option bits; only the excursion-set ones */
  int n_threads;      /* the team, which also sets the batch floor */
  int window;         /* 0: the reference's adaptive window; >0: fixed */
  int smoothing_mode; /* as orc_spectrum_new when no fields are injected */
  /* NULL, or fields of grid_n^3 taken in the order the run's transforms
   * return them: per rung (largest first) the top-hat and, under
   * SIF_FINDER_REFINE_GAUSSIAN for a rung with candidates, the top-hat times
   * the Gaussian the minima are found on. */
  const float* inject;
  /* Voids to start from (sif_finder_exodus_extras_t::prior): accepted before
   * the first rung and returned first. NULL when n_prior is 0. */
  const float* prior_cx;
  const float* prior_cy;
  const float* prior_cz;
  const float* prior_r;
  uint64_t n_prior;
  /* A survey (sif_finder_exodus_survey_raw, src/finder/exodus_survey.c:
   * 401-545): the randoms' mesh and their CIC density grid (grid_n^3), NULL
   * for a periodic box. `delta` is then the data's CIC density, not a
   * contrast; each rung scans the smoothed data over alpha times the smoothed
   * randoms and grows every radius against the randoms; injected fields come
   * two a rung, the data's top-hat, then the randoms'. Only cell seeds on
   * their nodes; the catalogue gets its footprint columns. */
  const orc_mesh_t* random_mesh;
  const float* random_grid;
} orc_exodus_params_t;

typedef struct {
  float* cx;
  float* cy;
  float* cz;
  float* r;
  uint64_t n_voids;
  /* A survey run's observed fractions of each sphere and of the shell out to
   * twice its radius (sif_catalogue_t::footprint, footprint_shell); NULL for
   * a box. */
  float* footprint;
  float* footprint_shell;
} orc_catalogue_t;

/* The observed nodes of a survey's grid (sif__exodus_survey_occupancy,
 * src/finder/exodus_survey.c:159-201) into occ, (n^3 + 63) / 64 words; the
 * closing's k into *k_out. Returns the observed node count. */
uint64_t orc_survey_occupancy(const orc_mesh_t* random_mesh, uint32_t n, float box,
  uint64_t* occ, int32_t* k_out);

/* sif__exodus_find_radius_survey (src/finder/exodus_rescale.c:2154-2317). */
float orc_find_radius_survey(const orc_mesh_t* data_mesh, const orc_template_t* data_tpl,
  const orc_mesh_t* random_mesh, const orc_template_t* random_tpl, float cx, float cy,
  float cz, float r_search, float K, float rmin, uint32_t window, uint8_t* reason,
  uint64_t* span_sum, uint64_t* span_count);

/* sif_finder_exodus_raw on a periodic box (src/finder/exodus_finder.c:1272,
 * 1585-2492), for SIF_FINDER_SEEDS_CELLS on their nodes. `delta` is the
 * density contrast, left untouched; `radii` in any order. stats, if not
 * NULL, holds n_radii entries, sorted order. 0, or a negative sif status. */
int orc_exodus(const float* delta, const orc_mesh_t* mesh, const float* radii,
  uint32_t n_radii, const orc_exodus_params_t* p, orc_catalogue_t* out,
  orc_rung_stats_t* stats);
void orc_catalogue_free(orc_catalogue_t* c);

#ifdef __cplusplus
}
#endif

#endif
