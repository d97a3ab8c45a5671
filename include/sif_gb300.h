/*
 * sif_gb300.h -- the C ABI of the GB300 exodus library (libsif_gb300.so).
 *
 * Part 1 is sif's own C API for the exodus path: the same symbol names, the
 * same struct layouts and the same status conventions as the reference's
 * headers (single-precision build, sif_real = float), so that pysif, the
 * sif-exodus CLI and C callers link against this library unchanged. Each
 * declaration names the reference declaration it replaces. The work runs on
 * one GPU; the structs stay in host memory, and every call copies what it
 * needs to the device and its result back.
 *
 * Part 2 is additive: entry points that take device pointers, for callers
 * that keep particles and grids resident in GPU memory, plus the stage-level
 * calls the parity tests use. They have no counterpart in the reference.
 */
#ifndef SIF_GB300_H
#define SIF_GB300_H

#include <math.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* Part 1: sif's API                                                       */
/* ---------------------------------------------------------------------- */

/* include/sif/core/macros.h:42, 468-506 */
typedef uint32_t sif_option;
typedef float sif_real;

/* include/sif/core/macros.h:690-707 */
#define SIF_OK                0
#define SIF_ERR_ALLOC         (-1)
#define SIF_ERR_INVALID       (-2)
#define SIF_ERR_RANGE         (-3)
#define SIF_ERR_IO            (-4)
#define SIF_ERR_UNSUPPORTED   (-5)
#define SIF_ERR_UNINITIALISED (-6)

/* include/sif/core/macros.h:73-292 (the finder and mesh options) */
#define SIF_FINDER_ALIASING_WINDOW    (1u << 8)
#define SIF_FINDER_SEEDS_CELLS        (0u << 9)
#define SIF_FINDER_SEEDS_MINIMA       (1u << 9)
#define SIF_FINDER_NO_CHECKPOINT      (1u << 11)
#define SIF_FINDER_SEARCH_1_50        (0u << 12)
#define SIF_FINDER_SEARCH_1_25        (1u << 12)
#define SIF_FINDER_SEARCH_1_75        (2u << 12)
#define SIF_FINDER_SEARCH_2_00        (3u << 12)
#define SIF_FINDER_KEEP_CIC_WINDOW    (1u << 14)
#define SIF_FINDER_CONSUME_GRID       (1u << 15)
#define SIF_MESH_DROP_INDICES         (1u << 16)
#define SIF_MESH_NO_CANONICAL         (1u << 17)
#define SIF_FINDER_LAGRANGIAN_OVERLAP (1u << 18)
#define SIF_FINDER_REFINE_NONE        (0u << 19)
#define SIF_FINDER_REFINE_GAUSSIAN    (1u << 19)
#define SIF_FINDER_REFINE_TRACERS     (2u << 19)
#define SIF_FINDER_REFINE_HILL        (3u << 19)
#define SIF_FINDER_EXTEND_REACH       (1u << 21)
#define SIF_FINDER_DISPLACE           (1u << 22)

/* include/sif/core/macros.h:772-777 */
#define SIF_LOG_LEVEL_TRACE   0
#define SIF_LOG_LEVEL_DEBUG   1
#define SIF_LOG_LEVEL_INFO    2
#define SIF_LOG_LEVEL_WARNING 3
#define SIF_LOG_LEVEL_ERROR   4
#define SIF_LOG_LEVEL_NONE    5

/* include/sif/core/system.h:44-100 */
typedef struct {
  bool skip_tuning;
} sif_fft_config_t;
typedef struct {
  uint32_t n_threads;
} sif_omp_config_t;
typedef struct {
  const char* key;
  const char* value;
} sif_setting_t;
typedef struct {
  sif_fft_config_t* fft_config;
  sif_omp_config_t* omp_config;
  uint8_t log_level;
  const sif_setting_t* settings;
  size_t n_settings;
} sif_config_t;

/* include/sif/structures/field.h:90-133 */
typedef enum { SIF_COORDINATES_CARTESIAN = 0, SIF_COORDINATES_SKY } sif_coordinates_t;
typedef struct {
  sif_real* _position_block;
  sif_real* _velocity_block;
  sif_real* x;
  sif_real* y;
  sif_real* z;
  sif_real* vx;
  sif_real* vy;
  sif_real* vz;
  sif_real* weights;
  uint64_t* original_indices;
  sif_real min_p[3];
  sif_real max_p[3];
  sif_real centre[3];
  sif_real half_span;
  uint32_t state_flags;
  uint64_t n_particles;
  sif_coordinates_t units;
} sif_field_t;

/* include/sif/structures/grid.h:32-128 */
typedef enum {
  SIF_GRID_EMPTY = 0,
  SIF_GRID_DENSITY,
  SIF_GRID_DENSITY_CONTRAST
} sif_grid_content_t;
typedef enum {
  SIF_ASSIGNMENT_UNKNOWN = 0,
  SIF_ASSIGNMENT_NGP = 1,
  SIF_ASSIGNMENT_CIC = 2,
  SIF_ASSIGNMENT_TSC = 3,
  SIF_ASSIGNMENT_PCS = 4
} sif_assignment_t;
typedef struct {
  sif_real* values;
  sif_grid_content_t content;
  sif_assignment_t assignment;
  uint32_t interlaced;
  uint32_t n_cells;
  uint64_t total_cells;
  sif_real box_length;
  sif_real cell_length;
  uint32_t p2_mask;
  uint32_t p2_shift;
} sif_grid_t;

/* include/sif/structures/chain_mesh.h:40-108 */
typedef struct {
  uint32_t n_cells;
  uint64_t total_cells;
  sif_real box_length;
  sif_real cell_length;
  sif_real* _position_block;
  sif_real* _velocity_block;
  sif_real* x;
  sif_real* y;
  sif_real* z;
  sif_real* vx;
  sif_real* vy;
  sif_real* vz;
  sif_real* weights;
  double total_weight;
  sif_real* cell_weights;
  uint64_t* original_indices;
  uint64_t n_particles;
  uint64_t* cell_offsets;
} sif_chain_mesh_t;

/* include/sif/structures/catalogue.h:38-93 */
typedef struct {
  sif_real* _block;
  sif_real* cx;
  sif_real* cy;
  sif_real* cz;
  sif_real* radii;
  sif_real* _footprint_block;
  sif_real* footprint;
  sif_real* footprint_shell;
  sif_coordinates_t units;
  void* _meta;
  uint32_t _n_meta;
  uint64_t n_voids;
  uint64_t capacity;
} sif_catalogue_t;

/* include/sif/finder/exodus_finder.h:40-106 */
typedef struct {
  const char* checkpoint;
  const sif_catalogue_t* prior;
  int keep_checkpoint;
  int save_memory;
} sif_finder_exodus_extras_t;

/* include/sif/finder/exodus_finder.h:409-507: the exodus checkpoint's fixed
 * 192-byte header. The file is this header, then the ladder largest first
 * (n_radii sif_real), then the voids as four columns of n_voids sif_real
 * (every x, then every y, z, radius), in host byte order. */
#define SIF_FINDER_CHECKPOINT_MAGIC "XCKP"
#define SIF_FINDER_CHECKPOINT_VERSION 3
typedef struct {
  char magic[4];
  uint32_t version;
  uint32_t byte_order; /* 0x01020304 as written */
  uint32_t is_double;
  uint32_t is_survey;
  uint32_t is_weighted;
  uint32_t options;    /* the options that change the catalogue */
  uint32_t n_radii;
  uint32_t next_rung;  /* rungs done */
  uint32_t grid_n_cells;
  double box_length;
  double threshold;
  double overlap_fraction;
  uint64_t n_particles;
  double total_weight;
  uint64_t random_n_particles;
  double random_total_weight;
  double offset[3];
  uint64_t n_prior;
  uint32_t prior_crc32;
  uint32_t crc32;
  uint64_t n_voids;
  uint64_t n_mismatched;
  uint32_t assignment;
  char reserved[36];
} sif_finder_exodus_checkpoint_t;

/* include/sif/finder/exodus_finder.h:124-133 */
typedef enum {
  SIF_EXODUS_EXCURSION_SET = 0,
  SIF_EXODUS_EXCURSION_PEAK,
  SIF_EXODUS_LAGRANGIAN_OVERLAP,
  SIF__EXODUS_N_VARIANTS
} sif_exodus_variant_t;

/* include/sif/finder/exodus_finder.h:689-695 */
typedef enum { SIF_FINDER_UNITS_PHYSICAL = 0, SIF_FINDER_UNITS_MPS } sif_finder_units_t;

/* include/sif/core/system.h:118 -- selects the GPU (CUDA_VISIBLE_DEVICES /
 * device 0) and sizes the host team that replays the candidate order. */
int sif_system_init(sif_config_t* config);
/* include/sif/core/system.h:127 */
void sif_system_finalise(void);
/* include/sif/utils/logger.h:330 */
const char* sif_error_message(void);
/* include/sif/utils/logger.h:346 */
int sif_error_status(void);

/* include/sif/structures/field.h:146, 165, 202 */
sif_field_t* sif_field_alloc(uint64_t n_particles);
void sif_field_free(sif_field_t* field);
int sif_field_assign_positions(sif_field_t* field, const sif_real* x, const sif_real* y,
                               const sif_real* z);
/* include/sif/structures/field.h:188, 231: the weight column (uninitialised,
 * or copied from the caller's array in the field's particle order). A
 * weighted field deposits its weights (sif_grid_assign_cic) and gives a
 * weighted mesh (weights in mesh order, cell_weights, total_weight), which
 * the finder measures against the mean weight density. */
int sif_field_reserve_weights(sif_field_t* field);
int sif_field_assign_weights(sif_field_t* field, const sif_real* weights);

/* include/sif/structures/grid.h:140, 147, 212, 233 */
sif_grid_t* sif_grid_alloc(uint32_t n_cells, sif_real box_length);
void sif_grid_free(sif_grid_t* grid);
int sif_grid_assign_cic(sif_grid_t* grid, const sif_field_t* field);
int sif_grid_to_density_contrast(sif_grid_t* grid);

/* include/sif/structures/chain_mesh.h:141, 175, 182 */
sif_chain_mesh_t* sif_chain_mesh_alloc(uint32_t n_cells, sif_real box_length,
                                       const sif_field_t* field, sif_option opt);
sif_chain_mesh_t* sif_chain_mesh_alloc_consume(uint32_t n_cells, sif_real box_length,
                                               sif_field_t* field, sif_option opt);
void sif_chain_mesh_free(sif_chain_mesh_t* mesh);

/* include/sif/structures/catalogue.h:116 */
void sif_catalogue_free(sif_catalogue_t* catalogue);

/* include/sif/finder/exodus_finder.h:547: a checkpoint's voids (and its
 * header, when asked), read and checked as a resume reads it. */
sif_catalogue_t* sif_finder_exodus_checkpoint_read(const char* filepath,
                                                   sif_finder_exodus_checkpoint_t* header);

/* include/sif/finder/exodus_finder.h:147, 155, 163 */
int sif_finder_exodus_preset(sif_exodus_variant_t variant, sif_real* overlap_fraction,
                             sif_option* opt);
const char* sif_finder_exodus_variant_name(sif_exodus_variant_t variant);
int sif_finder_exodus_variant_from_name(const char* name, sif_exodus_variant_t* variant);

/* include/sif/finder/exodus_finder.h:177-180 */
sif_catalogue_t* sif_finder_exodus(sif_grid_t* grid, const sif_chain_mesh_t* mesh,
                                   const sif_real* radii, uint32_t n_radii, sif_real threshold,
                                   sif_exodus_variant_t variant,
                                   const sif_finder_exodus_extras_t* extras);
/* include/sif/finder/exodus_finder.h:290-293 */
sif_catalogue_t* sif_finder_exodus_raw(sif_grid_t* grid, const sif_chain_mesh_t* mesh,
                                       const sif_real* radii, uint32_t n_radii,
                                       sif_real threshold, sif_real overlap_fraction,
                                       sif_option opt, const sif_finder_exodus_extras_t* extras);

/* include/sif/finder/exodus_finder.h:296-310, 312-413: the finder on a
 * survey -- any geometry, described by a random catalogue -- inside a box
 * padded so that nothing wraps (every tracer at least max(r_search,
 * (r_search + mesh cell) / 2) + a grid cell from every face; r_search the
 * largest rung's reach), sif_finder_exodus_survey_box sizing it. The grids
 * hold the CIC densities of data and randoms (sif_grid_assign_cic, not
 * converted to a contrast), on the same n_cells and box; each mesh may
 * carry weights. Each rung scans the smoothed data over alpha times the
 * smoothed randoms on the observed nodes (those the randoms reach, their
 * chance holes closed; alpha the data's total weight over the randoms') and
 * grows each radius against the randoms. `offset` is what the survey was
 * moved into the box by (NULL: not moved); the voids come back less it, with
 * the footprint columns (the observed fraction of each sphere and of its
 * shell to twice the radius). Cell seeds on their nodes only: the
 * excursion-peak preset and SIF_FINDER_SEEDS_MINIMA, REFINE_*, EXTEND_REACH
 * and DISPLACE fail with SIF_ERR_INVALID. */
sif_catalogue_t* sif_finder_exodus_survey(sif_grid_t* data_grid, sif_grid_t* random_grid,
                                          const sif_chain_mesh_t* data_mesh,
                                          const sif_chain_mesh_t* random_mesh,
                                          const sif_real offset[3], const sif_real* radii,
                                          uint32_t n_radii, sif_real threshold,
                                          sif_exodus_variant_t variant,
                                          const sif_finder_exodus_extras_t* extras);
sif_catalogue_t* sif_finder_exodus_survey_raw(sif_grid_t* data_grid, sif_grid_t* random_grid,
                                              const sif_chain_mesh_t* data_mesh,
                                              const sif_chain_mesh_t* random_mesh,
                                              const sif_real offset[3], const sif_real* radii,
                                              uint32_t n_radii, sif_real threshold,
                                              sif_real overlap_fraction, sif_option options,
                                              const sif_finder_exodus_extras_t* extras);
/* include/sif/finder/exodus_finder.h:551-606: the box a survey is searched
 * in (its data and randoms' extent, plus the margin above at the largest grid
 * cell the smallest radius allows, 1% over) and the offset that centres the
 * survey in it. */
int sif_finder_exodus_survey_box(const sif_field_t* data, const sif_field_t* randoms,
                                 const sif_real* radii, uint32_t n_radii, sif_option opt,
                                 sif_real offset[3], sif_real* box_length);

/* include/sif/finder/exodus_finder.h:721-723 */
uint32_t sif_finder_grid_cells_from_size(uint64_t n_particles, sif_real box_length,
                                         sif_real cell_size, sif_finder_units_t units,
                                         sif_real volume);

/* include/sif/finder/exodus_finder.h:595-683: a static inline function
 * there, so it is one here too. The mesh resolution the finder runs fastest
 * at: about SIF_FINDER_MESH_PARTICLES_PER_CELL tracers per cell at the
 * tracers' density over the whole box, no coarser than the widest search
 * sphere's stencil allows (the traversal wraps a cell index once), between 8
 * and SIF_FINDER_MESH_MAX_CELLS cells per side. The catalogue does not depend
 * on it. 0 for arguments it cannot size a mesh from. */
#define SIF_FINDER_MESH_PARTICLES_PER_CELL 30.0
#define SIF_FINDER_MESH_MAX_CELLS 1024u
static inline uint32_t sif_finder_suggest_mesh_cells(uint64_t n_particles, sif_real box_length,
                                                     sif_real max_radius, sif_real volume) {
  if (n_particles == 0 || !(box_length > 0.0f) || !isfinite(box_length) || !(volume >= 0.0f) ||
      !isfinite(volume))
    return 0;
  const double L = (double)box_length;
  /* Tracers the whole box would hold at their density. */
  const double whole = volume > 0.0f ? (double)n_particles * (L * L * L) / (double)volume
                                     : (double)n_particles;
  double cells = cbrt(whole / SIF_FINDER_MESH_PARTICLES_PER_CELL);
  if (max_radius > 0.0f) {
    const double reach = 2.0 * (double)max_radius;
    if (reach >= L) return 0;
    const double at_least = L / (L - reach) + 1.0;
    if (cells < at_least) cells = at_least;
  }
  if (cells < 8.0) cells = 8.0;
  if (cells > (double)SIF_FINDER_MESH_MAX_CELLS) cells = (double)SIF_FINDER_MESH_MAX_CELLS;
  return (uint32_t)cells;
}

/* ---------------------------------------------------------------------- */
/* Part 2: device-resident entry points (no counterpart in the reference)  */
/* ---------------------------------------------------------------------- */

/* Per-rung counts of the last sifg_exodus_device / sifg_box_device run. */
typedef struct {
  float radius;
  float r_search;
  uint64_t n_candidates;
  uint64_t n_survivors;
  uint64_t n_accepted;
  uint64_t rounds;
  uint64_t n_rescale_fail;
  uint64_t n_overflow;
  /* Host wall time of the rung's phases, milliseconds: the whole rung, the
   * wait for the candidate count, the candidate sort, the commit rounds. */
  double rung_ms;
  double count_wait_ms;
  double sort_ms;
  double commit_ms;
  /* Particles read and template cells visited by the rung's sphere growth. */
  uint64_t growth_particles;
  uint64_t growth_cells;
  /* Host wait for the candidates' depths before the sort, milliseconds. */
  double cand_wait_ms;
  uint64_t from_list;      /* 1: the candidates came from the smoothing's below-threshold list */
  uint64_t n_witness;      /* survivors the collision witness refused before any growth */
  uint64_t n_displaced;    /* voids the rung's acceptances displaced (SIF_FINDER_DISPLACE) */
} sifg_rung_stat_t;

/* Kernel timings of the last run, CUDA events on the launching stream. */
typedef struct {
  double wall_ms;
  double growth_ms;
  int growth_launches;
  double filter_ms;
  int filter_launches;
  double cic_ms;
  int cic_launches;
  double mesh_ms;
  int mesh_launches;
  /* What the sphere growth and the collision witness gathered: particle
   * positions read (12 bytes each) and template cells visited (16 bytes
   * each). */
  uint64_t growth_particles;
  uint64_t growth_cells;
  /* The collision witness, run ahead of each rung's growth. */
  double witness_ms;
  int witness_launches;
  double commit_ms; /* the commit's rounds, kernel time on the run's stream */
  int commit_launches;
  /* The box path's whole deposit: the tile sort, the deposit kernel (cic_ms)
   * and the faces' fix-up. */
  double cic_stage_ms;
} sifg_timings_t;

/* One span of the last run's timeline: a tracked launch (or stage) with its
 * start and end in milliseconds after the run's first event, CUDA events on
 * the stream it ran on. */
typedef enum {
  SIFG_TRACE_GROWTH = 0,    /* a sphere-growth launch (run's stream) */
  SIFG_TRACE_FILTER = 1,    /* the filter pass of a smoothing (smoothing stream) */
  SIFG_TRACE_CIC = 2,       /* the deposit kernel */
  SIFG_TRACE_MESH = 3,      /* the chain mesh build (copy stream in the box path) */
  SIFG_TRACE_WITNESS = 4,   /* a collision-witness launch */
  SIFG_TRACE_COMMIT = 5,    /* a commit launch (its rounds) */
  SIFG_TRACE_SMOOTHING = 6, /* a rung's whole smoothing (smoothing stream) */
  SIFG_TRACE_RUNG = 7,      /* a rung on the run's stream, from its field's arrival */
  SIFG_TRACE_CIC_STAGE = 8  /* the box path's whole deposit (tile sort, deposit, faces) */
} sifg_trace_kind_t;
typedef struct {
  int32_t kind; /* sifg_trace_kind_t */
  float start_ms;
  float end_ms;
} sifg_trace_event_t;

/* The CIC density (per unit volume, float) of n device-resident particles
 * on an n_grid^3 device grid. */
int sifg_cic_device(const float* x, const float* y, const float* z, uint64_t n, uint32_t n_grid,
                    float box, float* grid);
/* Density to density contrast in place; *mean_out (may be NULL) receives
 * the mean density. */
int sifg_contrast_device(float* grid, uint64_t total_cells, double* mean_out);
/* A chain mesh of device particles into device arrays: positions (n each),
 * offsets (n_cells^3 + 1, uint32), source indices (n, uint32; may be NULL). */
int sifg_mesh_device(const float* x, const float* y, const float* z, uint64_t n,
                     uint32_t n_cells, float box, float* mx, float* my, float* mz,
                     uint32_t* offsets, uint32_t* orig);
/* The density contrast on the device smoothed at radius r (filter 1
 * top-hat, 2 Gaussian; window_mode 0 none, 1 CIC, 2 aliasing-aware) into a
 * device grid. */
int sifg_smooth_device(const float* delta, uint32_t n_grid, float box, float r, int filter,
                       int window_mode, float* out);
/* The exodus finder on a device density contrast and a device mesh. radii in
 * host memory. inject: NULL, or device grids that replace the smoothing, in
 * the order the run's transforms return them: per rung (largest radius
 * first) its top-hat and, under SIF_FINDER_REFINE_GAUSSIAN for a rung with
 * candidates, the top-hat times the Gaussian of 0.15 of the rung the minima
 * are found on (2 * n_radii grids cover any run). prior: NULL, or n_prior voids to start
 * from in host memory, as four columns one after another (cx, cy, cz, r),
 * checked and used as sif_finder_exodus_extras_t::prior is. The catalogue is
 * written to the host arrays (capacity entries each); *n_voids receives the
 * count (which may exceed capacity: then only capacity are written). */
int sifg_exodus_device(const float* delta, uint32_t n_grid, float box, const float* mx,
                       const float* my, const float* mz, const uint32_t* offsets,
                       uint64_t n_particles, uint32_t mesh_cells, const float* radii,
                       uint32_t n_radii, float threshold, float overlap, uint32_t opt,
                       const float* inject, const float* prior, uint64_t n_prior, float* cx,
                       float* cy, float* cz, float* r, uint64_t capacity, uint64_t* n_voids);
/* The whole box path on device particles: CIC, contrast, mesh, exodus. */
int sifg_box_device(const float* x, const float* y, const float* z, uint64_t n, uint32_t n_grid,
                    float box, uint32_t mesh_cells, const float* radii, uint32_t n_radii,
                    float threshold, float overlap, uint32_t opt, float* cx, float* cy,
                    float* cz, float* r, uint64_t capacity, uint64_t* n_voids);
/* The FP64 form: the calls above with every value in double, computing what
 * the reference's SIF_USE_DOUBLE build computes (sif_real = double; its
 * catalogue, on the same smoothed fields, bit for bit). The deposit sums each
 * particle's weights as multiples of 2^-40 (exact, order-independent). These
 * have no counterpart in the reference's float build, whose ABI they do not
 * change; they are the form the float path is measured against. */
int sifg_cic_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                        uint32_t n_grid, double box, double* grid);
int sifg_contrast_device_f64(double* grid, uint64_t total_cells, double* mean_out);
int sifg_mesh_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                         uint32_t n_cells, double box, double* mx, double* my, double* mz,
                         uint32_t* offsets, uint32_t* orig);
int sifg_smooth_device_f64(const double* delta, uint32_t n_grid, double box, double r,
                           int filter, int window_mode, double* out);
int sifg_exodus_device_f64(const double* delta, uint32_t n_grid, double box, const double* mx,
                           const double* my, const double* mz, const uint32_t* offsets,
                           uint64_t n_particles, uint32_t mesh_cells, const double* radii,
                           uint32_t n_radii, double threshold, double overlap, uint32_t opt,
                           const double* inject, const double* prior, uint64_t n_prior,
                           double* cx, double* cy, double* cz, double* r, uint64_t capacity,
                           uint64_t* n_voids);
int sifg_box_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                        uint32_t n_grid, double box, uint32_t mesh_cells, const double* radii,
                        uint32_t n_radii, double threshold, double overlap, uint32_t opt,
                        double* cx, double* cy, double* cz, double* r, uint64_t capacity,
                        uint64_t* n_voids);
/* Weighted meshes on the device (the reference's sif_field_assign_weights
 * path, for device data; float and FP64 forms). sifg_cic_weighted_device: the
 * CIC density of weighted particles (w: one weight each, device).
 * sifg_mesh_weights_device: a mesh's weight columns from the field's
 * weights (source order) and the mesh's offsets and source indices (from
 * sifg_mesh_device with orig): w (mesh order), cell_w (n_cells^3 per-cell
 * sums), *total_weight (host). sifg_exodus_weighted_device: sifg_exodus_device
 * on a weighted mesh (its w, cell_w and total_weight added after offsets):
 * the weights must be finite and non-negative (SIF_ERR_INVALID otherwise),
 * the density tests measure against the mean weight density. */
int sifg_cic_weighted_device(const float* x, const float* y, const float* z, const float* w,
                             uint64_t n, uint32_t n_grid, float box, float* grid);
int sifg_cic_weighted_device_f64(const double* x, const double* y, const double* z,
                                 const double* w, uint64_t n, uint32_t n_grid, double box,
                                 double* grid);
int sifg_mesh_weights_device(const float* field_w, const uint32_t* orig, uint64_t n,
                             const uint32_t* offsets, uint32_t n_cells, float* w, float* cell_w,
                             double* total_weight);
int sifg_mesh_weights_device_f64(const double* field_w, const uint32_t* orig, uint64_t n,
                                 const uint32_t* offsets, uint32_t n_cells, double* w,
                                 double* cell_w, double* total_weight);
int sifg_exodus_weighted_device(const float* delta, uint32_t n_grid, float box, const float* mx,
                                const float* my, const float* mz, const uint32_t* offsets,
                                const float* w, const float* cell_w, double total_weight,
                                uint64_t n_particles, uint32_t mesh_cells, const float* radii,
                                uint32_t n_radii, float threshold, float overlap, uint32_t opt,
                                const float* inject, const float* prior, uint64_t n_prior,
                                float* cx, float* cy, float* cz, float* r, uint64_t capacity,
                                uint64_t* n_voids);
int sifg_exodus_weighted_device_f64(const double* delta, uint32_t n_grid, double box,
                                    const double* mx, const double* my, const double* mz,
                                    const uint32_t* offsets, const double* w,
                                    const double* cell_w, double total_weight,
                                    uint64_t n_particles, uint32_t mesh_cells,
                                    const double* radii, uint32_t n_radii, double threshold,
                                    double overlap, uint32_t opt, const double* inject,
                                    const double* prior, uint64_t n_prior, double* cx,
                                    double* cy, double* cz, double* r, uint64_t capacity,
                                    uint64_t* n_voids);
/* A chain mesh on the device, for the survey entry point: positions in mesh
 * order, n_cells^3 + 1 offsets, and optionally its weight columns (w in mesh
 * order and cell_w per cell, both or neither) with their total; total_weight
 * is the tracer count for a mesh without weights. */
typedef struct {
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* offsets;
  const float* w;
  const float* cell_w;
  double total_weight;
  uint64_t n_particles;
  uint32_t n_cells;
} sifg_device_mesh_t;
/* The survey finder on device arrays (sif_finder_exodus_survey_raw's run,
 * src/finder/exodus_survey.c:401-545, without its margin check and offset):
 * the data's and the randoms' CIC densities (n_grid^3 each) and meshes in the
 * box's frame, the voids (prior ones in the same frame, prior[4 * n_prior]
 * as cx.., cy.., cz.., r..) and their footprint columns written to the host
 * arrays cx .. footprint_shell (capacity entries each; *n_voids is the
 * count). inject: NULL, or 2 n_radii device fields in the order the run's
 * transforms return them (per rung, largest first, the data's top-hat then
 * the randoms'), replacing the smoothing. */
int sifg_exodus_survey_device(const float* data_density, const float* random_density,
                              uint32_t n_grid, float box, const sifg_device_mesh_t* data,
                              const sifg_device_mesh_t* randoms, const float* radii,
                              uint32_t n_radii, float threshold, float overlap, uint32_t opt,
                              const float* inject, const float* prior, uint64_t n_prior,
                              float* cx, float* cy, float* cz, float* r, float* footprint,
                              float* footprint_shell, uint64_t capacity, uint64_t* n_voids);
/* The adjoint of the CIC density contrast (sifg_cic_device followed by
 * sifg_contrast_device) with respect to the positions: given g = dL/d(delta)
 * on the n_grid^3 device grid, writes dL/dx, dL/dy, dL/dz of every particle
 * (device arrays of n). The smoothing is self-adjoint, so the gradient of a
 * loss on a smoothed field is this call on the smoothed incoming gradient.
 * No counterpart in the reference (which has no gradients); it backs the
 * torch.autograd.Function in sif_gb300.autograd. */
int sifg_contrast_vjp_device(const float* x, const float* y, const float* z, uint64_t n,
                             uint32_t n_grid, float box, const float* g, float* gx, float* gy,
                             float* gz);
int sifg_contrast_vjp_device_f64(const double* x, const double* y, const double* z, uint64_t n,
                                 uint32_t n_grid, double box, const double* g, double* gx,
                                 double* gy, double* gz);
/* The batched form: independent boxes (particles on the device), each
 * run through the whole box path as sifg_box_device would run it alone --
 * same catalogue bit for bit -- by a pool of n_engines engines working
 * concurrently (each its own streams and buffers), largest box first.
 * n_engines 0: the count sifg_box_batch_autotune found for batches of this
 * size (tuned on the spot the first time). Each job's status and n_voids are
 * written; the call returns the first failing job's status, or SIF_OK. No
 * counterpart in the reference, which runs one box per call. */
typedef struct {
  const float* x; /* device, n_particles each */
  const float* y;
  const float* z;
  uint64_t n_particles;
  uint32_t n_grid;
  float box;
  uint32_t mesh_cells; /* 0: sif_finder_suggest_mesh_cells(n_particles, box, max radius, 0) */
  const float* radii;  /* host */
  uint32_t n_radii;
  float threshold;
  float overlap;
  uint32_t options;
  float* cx; /* host, capacity each */
  float* cy;
  float* cz;
  float* r;
  uint64_t capacity;
  uint64_t n_voids; /* out */
  int status;       /* out */
  double wall_ms;   /* out: host wall time of this box's run */
} sifg_box_job_t;
int sifg_box_batch_device(sifg_box_job_t* jobs, uint32_t n_jobs, uint32_t n_engines,
                          uint32_t* n_engines_used);
/* Times the batch at 1, 2, 3, 4, 6 and 8 engines (each count run twice, the second
 * run timed), keeps the fastest for batches of this size (total particles and
 * job count, to a factor of two) and returns it in *n_engines. The catalogues
 * do not depend on the choice. */
int sifg_box_batch_autotune(sifg_box_job_t* jobs, uint32_t n_jobs, uint32_t* n_engines);
/* Statistics and timings of the last run (up to max_rungs entries). A run
 * keeps its timing events; the first of sifg_last_timings and
 * sifg_last_trace after it reads them (waiting for the run's last event),
 * so that runs back to back pay nothing for timings nobody reads. */
uint32_t sifg_last_rung_stats(sifg_rung_stat_t* out, uint32_t max_rungs);
void sifg_last_timings(sifg_timings_t* out);
/* The last run's timeline: copies up to `capacity` spans (in the order
 * recorded, kind by kind) and returns how many there are. */
uint32_t sifg_last_trace(sifg_trace_event_t* out, uint32_t capacity);
/* Kernels of this library launched so far in the process (cuFFT's own are
 * not counted). */
uint64_t sifg_launch_count(void);
/* The CUDA stream every call above runs on (a cudaStream_t), for callers
 * that time or order work against it; 0 before sif_system_init(). */
uint64_t sifg_stream(void);
/* The resolve window (bins per pass) the sphere growth uses; default 8. */
void sifg_set_window(int bins);
/* Which sphere-growth kernel runs: 0 (default) by the survivor count, 1 a
 * CTA per survivor, 2 a warp per survivor. The radii do not depend on it. */
void sifg_set_growth_mode(int mode);
/* The warp-per-survivor growth keeps the distances its windows can collect
 * in a list in shared memory, so that a window need not read the particles
 * again: -1 (default) a list sized per rung from the shell's expected
 * particle count (none for the large spheres of the early rungs), 0 no list,
 * n > 0 a list of n entries (rounded up to 32, at most 512) on every rung.
 * The radii do not depend on it. */
void sifg_set_shell_list(int entries);
/* How the commit's rounds run: 0 (default) all in one cooperative launch
 * where the device allows it, 1 a kernel launch per round. The catalogue
 * does not depend on it. */
void sifg_set_commit_mode(int mode);
/* How a rung's candidates are found under the cell seeds: 0 (default) from
 * the list of cells at or below the threshold that the smoothing writes as
 * it goes, where it can (the float form at a 512^3 grid), less the masked
 * cells; 1 a scan of the whole field. The catalogue does not depend on it. */
void sifg_set_scan_mode(int mode);
/* The float form's own inverse transform at a 512^3 grid: 1 (default) the
 * filter pass reads each smoothing's filter factors from a table built on its
 * first use (257^3 floats, 68 MB, up to 24 kept); 0 it evaluates them as it
 * applies them. The smoothed fields are the same bits either way. */
void sifg_set_factor_tables(int on);
/* Device mirrors of the structs' host arrays. Each C API call copies its
 * inputs up from the structs' host arrays and its results down into them, so
 * a pipeline (sif_grid_assign_cic, sif_grid_to_density_contrast,
 * sif_chain_mesh_alloc, sif_finder_exodus) copies the positions up twice and
 * the grid and the mesh up again right after copying them down. With mirrors
 * on (1; or SIFG_HOST_MIRRORS=1 in the environment at sif_system_init), the
 * device copy a call made of an array inside one of the library's own
 * blocks (a field's positions and weights, a grid's values, a chain mesh's
 * columns) is kept, and later calls that read the array use it instead of
 * copying it again. A caller that writes such an array through the struct's
 * pointer must then call sifg_host_modified with the array (or any address
 * inside the block it lies in; NULL forgets every mirror) before the next
 * call reads it. As a net for writes not declared, each mirror samples 1024
 * evenly spaced words of its array when the two sides last agreed, and a call
 * that finds any of them changed copies the array again; a write that misses
 * every sampled word reads stale data. The library's own writes
 * (sif_field_assign_positions, sif_field_assign_weights) and freed structs
 * forget their mirrors themselves. 0 (default) copies every input on every
 * call, as the reference's arrays behave. Mirrors hold at most 96 GB of
 * device memory; an array past that is copied as without them. */
void sifg_set_host_mirrors(int on);
int sifg_host_mirrors(void);
void sifg_host_modified(const void* ptr);
/* The bytes the C API's calls have copied up from and down into the structs'
 * host arrays (and the catalogues' columns) since the library was loaded. */
void sifg_copy_bytes(uint64_t* h2d, uint64_t* d2h);
/* A test hook, as the reference's sif__exodus_halt_after_set
 * (src/finder/exodus_checkpoint.h): the finder runs that follow stop after
 * n_rungs rungs of their ladder, checkpoint written, and fail as a job killed
 * there would; 0 lets them finish. */
void sifg_set_halt_after(uint32_t n_rungs);
/* The collision witness (exodus_finder.c:780-845, exodus_rescale.c:
 * 1074-1167): 1 survivors whose sphere is certain to collide with a void of
 * an earlier rung at any radius they could return are refused before growth,
 * as the reference refuses them; 0 (default) every survivor is grown and the
 * commit refuses them. The catalogue does not depend on it. On the GPU the
 * proof costs more than the growth it saves (at 512^3: 2.1 ms a step to
 * refuse 1.5% of the survivors, 1.1 ms a step more in all). */
void sifg_set_witness(int on);
/* The chain-mesh build of sifg_mesh_device, for callers that cannot let the
 * library allocate device memory: a process whose framework reserves the
 * GPU's memory in its own pool, a latency-bound pipeline that cannot afford
 * cudaFree's device-wide wait, a host that enforces its own memory budget.
 * It has no counterpart in the reference. Its scratch is a static device
 * array of the library (about 17 MB, held on every GPU that loads the
 * library until the process exits), which limits it to 1,048,576 particles
 * and 64^3 = 262,144 mesh cells; larger inputs fail with SIF_ERR_RANGE. It
 * calls no cudaMalloc, cudaFree or allocating library routine. The first call
 * on a device after sif_system_init() looks up the array's device address.
 * Every call synchronises the library's stream before it returns (it reads
 * the box check's count back), so it must not be made while a stream capture
 * is in progress. Every call shares the one array, so calls that overlap on
 * the GPU would race; the library holds its API lock for the whole call and
 * runs it on its one stream, so calls from several host threads run one after
 * another. A caller that resets the device calls sif_system_finalise() and
 * sif_system_init() again before the next call. */
int sifg_mesh_device_noalloc(const float* x, const float* y, const float* z, uint64_t n,
                             uint32_t n_cells, float box, float* mx, float* my, float* mz,
                             uint32_t* offsets, uint32_t* orig);
/* The replay of the reference's candidate order on host data, for tests:
 * rank[k] = sorted position of delta[k]. */
void sifg_candidate_ranks(const float* delta, uint32_t m, uint32_t* rank);

#ifdef __cplusplus
}
#endif

#endif /* SIF_GB300_H */
