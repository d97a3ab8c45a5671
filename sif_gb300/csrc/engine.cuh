// The exodus run on one GPU (engine.cu): the rung loop around the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <vector>

#include "finder.cuh"
#include "kernels.cuh"
#include "smooth.cuh"

namespace sifg {

// A run's parameters, in the precision of its form (sif_real of the float
// build, or of the SIF_USE_DOUBLE build).
template <class R>
struct RunParamsT {
  uint32_t grid_n = 0;
  R box = 0;
  R threshold = R(-0.8f);
  R overlap = 0;
  uint32_t options = 0;
  std::vector<R> radii;  // any order
  int window = 8;        // bins resolved per pass
  // Fields that replace the smoothing, in the order the run's transforms
  // return them (largest rung first): each rung's top-hat and, under
  // SIF_FINDER_REFINE_GAUSSIAN for a rung with candidates, the refinement's
  // field; grid_n^3 values each, host or device memory as inject_on_device
  // says.
  const R* inject = nullptr;
  bool inject_on_device = false;
  // Where the last rung's field goes under SIF_FINDER_CONSUME_GRID (device).
  R* consume_out = nullptr;
  // When set, the grid handed to the run is the density itself and this the
  // device-side mean: the forward transform takes the contrast as it reads.
  const double* contrast_mean = nullptr;
  // Recorded once the mesh is on the device, if it is still being copied
  // when the run starts: the first sphere growth waits for it.
  cudaEvent_t mesh_ready = nullptr;
  // A weighted mesh's weights already checked (finite, non-negative) by the
  // caller; else the run checks them on the device before it starts.
  bool weights_checked = false;
  // Voids to start from (sif_finder_exodus_extras_t::prior), host memory:
  // accepted before the first rung and returned first (exodus_finder.c:
  // 1614-1622, 656-683).
  const R* prior_cx = nullptr;
  const R* prior_cy = nullptr;
  const R* prior_cz = nullptr;
  const R* prior_r = nullptr;
  uint64_t n_prior = 0;
  // A resumed run: the rungs before this one (largest first) are done, and
  // their voids are the prior ones. The ladder stays whole: the reach and
  // the extended reach's levels come from it.
  uint32_t first_rung = 0;
  // Called after each rung with the rungs done, the catalogue on the device
  // (its n_voids voids) and the rung's acceptances at more than twice its
  // radius, e.g. to write a checkpoint; a status other than SIF_OK ends the
  // run with that status.
  std::function<int(uint32_t, const R*, const R*, const R*, const R*, uint32_t, uint64_t)>
      after_rung;
  // A survey (sif_finder_exodus_survey_raw, src/finder/exodus_survey.c:
  // 401-545; the survey branches of exodus_finder.c): the randoms' mesh and
  // their CIC density grid on the device, NULL for a periodic box. The run's
  // grid is then the data's CIC density (no contrast); each rung scans the
  // smoothed data over survey_alpha times the smoothed randoms on the
  // observed nodes, and grows every radius against the randoms; injected
  // fields come two a rung, the data's top-hat then the randoms'. The
  // catalogue gets its footprint columns. Cell seeds on their nodes only.
  const DeviceMeshT<R>* random_mesh = nullptr;
  const R* random_density = nullptr;
  R survey_alpha = 0;  // the data's total weight over the randoms'
};
using RunParams = RunParamsT<float>;

struct RungStat {
  float radius = 0.f, r_search = 0.f;
  uint64_t n_candidates = 0, n_survivors = 0, n_accepted = 0, rounds = 0;
  uint64_t n_rescale_fail = 0, n_overflow = 0;
  double rung_ms = 0, count_wait_ms = 0, sort_ms = 0, commit_ms = 0;  // host wall time
  double cand_wait_ms = 0;  // waiting for the candidates' depths before the sort
  uint64_t from_list = 0;   // 1: candidates from the smoothing's below-threshold list
  uint64_t growth_particles = 0, growth_cells = 0;  // gathered by the rung's sphere growth
  uint64_t n_witness = 0;  // survivors the collision witness refused before growth
  uint64_t n_displaced = 0;  // voids displaced by the rung's acceptances (SIF_FINDER_DISPLACE)
  uint64_t n_mismatched = 0;  // acceptances at more than twice the rung's radius
};

struct RunTimings {
  KernelTimer growth, filter, cic, mesh, witness, commit;
  KernelTimer smoothing, rung;  // the timeline's stage spans
  KernelTimer cic_stage;        // the whole deposit: tile sort, deposit, faces
  cudaEvent_t origin = nullptr;  // the run's first event: the timeline's zero
  // False: nothing is timed and no event is made (a batch job: event creation
  // from several host threads at once serialises them).
  bool timed = true;
  double wall_ms = 0.0;
  uint64_t growth_particles = 0, growth_cells = 0;  // gathered by the sphere growth
  void mark_origin(cudaStream_t st) {
    if (origin) return;
    if (cudaEventCreate(&origin) != cudaSuccess || cudaEventRecord(origin, st) != cudaSuccess) {
      if (origin) cudaEventDestroy(origin);
      origin = nullptr;
    }
  }
  void reset() {
    growth_particles = growth_cells = 0;
    growth.reset();
    witness.reset();
    commit.reset();
    filter.reset();
    cic.reset();
    mesh.reset();
    smoothing.reset();
    rung.reset();
    cic_stage.reset();
    if (origin) cudaEventDestroy(origin);
    origin = nullptr;
    wall_ms = 0.0;
  }
  // Exchanges every timer's events and the origin with o's (the plain
  // counts are not exchanged).
  void swap_events(RunTimings& o) {
    for (auto [a, b] : {std::pair<KernelTimer*, KernelTimer*>{&growth, &o.growth},
                        {&filter, &o.filter}, {&cic, &o.cic}, {&mesh, &o.mesh},
                        {&witness, &o.witness}, {&commit, &o.commit},
                        {&smoothing, &o.smoothing}, {&rung, &o.rung},
                        {&cic_stage, &o.cic_stage}})
      a->swap(*b);
    std::swap(origin, o.origin);
  }
  RunTimings() = default;
  RunTimings(const RunTimings&) = delete;
  RunTimings& operator=(const RunTimings&) = delete;
  ~RunTimings() {
    if (origin) cudaEventDestroy(origin);
  }
};

template <class R>
struct HostCatalogueT {
  std::vector<R> cx, cy, cz, r;
  // A survey's observed fractions of each sphere and of its shell to twice
  // the radius (sif_catalogue_t::footprint, footprint_shell); empty for a box.
  std::vector<R> foot, shell;
};
using HostCatalogue = HostCatalogueT<float>;

// Device buffers of one engine's box path (grid, mesh, flags).
struct BoxBufs {
  DevBuf grid, mx, my, mz, offs, mesh_sums, flag, mean;
  DevBuf mesh_scratch;  // the mesh build's own, so that it runs beside the deposit
};

class Engine {
 public:
  explicit Engine(int device);
  ~Engine();

  cudaStream_t stream() const { return st_; }
  // A stream for uploads that overlap the run, and two events for them.
  cudaStream_t copy_stream() const { return st_copy_; }
  cudaEvent_t ev_copy_start() const { return ev_copy_start_; }
  cudaEvent_t ev_mesh_ready() const { return ev_mesh_ready_; }
  int device() const { return device_; }

  // The finder on a density contrast on the device and a device mesh.
  // Returns a sif status; the catalogue is appended to `out`.
  template <class R>
  int exodus(const R* d_delta, const DeviceMeshT<R>& mesh, const RunParamsT<R>& p,
             HostCatalogueT<R>& out, std::vector<RungStat>* stats, RunTimings* timings);

  DevBuf scratch;  // shared scratch for CIC / mesh builds
  BoxBufs io;      // the box path's buffers
  Smoother smoother;        // the float form's
  SmootherT<double> smoother64;  // the FP64 form's
  // A survey's randoms, smoothed beside the data (their own spectrum).
  Smoother rsmoother;
  SmootherT<double> rsmoother64;
  template <class R>
  SmootherT<R>& smoother_for();
  template <class R>
  SmootherT<R>& rsmoother_for();
  int host_threads = 0;

 private:
  int device_;
  cudaStream_t st_ = 0;
  DevBuf field_[2], mask_, cand_delta_, cand_flat_, blocks_, rank_, rank_slots_, alive_;
  DevBuf surv_cand_, surv_flat_, scx_, scy_, scz_, sr_, sreason_, state_a_, state_b_, acc_;
  DevBuf commit_bar_;  // the cooperative commit's grid barrier and its report
  DevBuf counters_, dcount_, sgrid_start_, sgrid_ids_, sgrid_cellof_, sgrid_pack_, sgrid_rank_;
  DevBuf pend_;  // the sphere growth's warp-kernel leftovers
  DevBuf cat_x_, cat_y_, cat_z_, cat_r_, vstart_, vids_, vcell_;
  DevBuf vhead_, vnext_, dlist_;  // displacement: the linked void index, its lists
  DevBuf work_;  // the sphere growth's and the witness's survivor queues
  DevBuf gwbuf_, wcheck_;  // a weighted mesh: the wide windows' weights, the weight check
  // SIF_FINDER_REFINE_GAUSSIAN: the refinement's fields, the placed
  // candidates and their offsets, the minima's keep flags, the survivors'
  // offset lengths.
  DevBuf gfield_[2], cand_delta2_, cand_flat2_, cand_off_, cand_off2_, keep_, soff_;
  DevBuf tpl_, gbuf_, traffic_, region_delta_, region_flat_;
  // A survey: the randoms' smoothed fields, the footprint (and the closing's
  // other mask, the marked count), the randoms' template, the voids' observed
  // fractions.
  DevBuf rfield_[2], occ_, occ_tmp_, occ_count_, rtpl_, foot_, shell_;
  static constexpr uint32_t kExtMaxLevels = 32;  // EXT_MAX_LEVELS, exodus_finder.c:244
  DevBuf ext_tpl_[kExtMaxLevels];  // the extended reach's templates, one per level
  DevBuf below_counts_[2], below_delta_[2], below_flat_[2];  // the smoothing's below-threshold lists
  std::vector<uint8_t> h_tpl_;  // the packed template, staged for its upload
  void* h_delta_ = nullptr;  // candidate depths, float or double
  uint32_t* h_flat_ = nullptr;
  uint32_t* h_rank_ = nullptr;
  uint32_t* h_counters_ = nullptr;
  size_t h_cap_ = 0;
  cudaEvent_t ev_cand_ = nullptr;
  // The smoothing runs on its own, lower-priority stream into two field
  // buffers: rung i+1's transform overlaps rung i's growth and commit.
  cudaStream_t st_fft_ = 0, st_copy_ = 0;
  cudaEvent_t ev_copy_start_ = nullptr, ev_mesh_ready_ = nullptr;
  cudaEvent_t ev_start_ = nullptr, ev_smoothed_[2] = {nullptr, nullptr},
              ev_scanned_[2] = {nullptr, nullptr};
  void ensure_host(size_t m);
};

// The reference's candidate order (include/sif/utils/sort.h:56-145 over
// src/finder/utils.c:24): rank[k] is the position of candidate k, given in
// flat order, once sorted by depth with the three-way quicksort.
// 0 (default): under the cell seeds, where the smoothing lists the cells at
// or below the threshold as it writes them, the candidates are that list
// less the masked cells; 1: a scan of the whole field every rung. The
// catalogue does not depend on it.
void set_scan_mode(int mode);

template <class K>
void candidate_ranks(const K* delta, uint32_t m, uint32_t* rank, int threads);

// Template of the rescaling (src/finder/exodus_rescale.c:175-283).
template <class R>
struct HostTemplateT {
  std::vector<int32_t> dx, dy, dz;
  std::vector<uint8_t> type;
  std::vector<R> min_d2, max_d2;
};
template <class R>
int build_template(HostTemplateT<R>& t, uint32_t mesh_n, R cell_length, R rmin, R r_search);

template <>
inline SmootherT<float>& Engine::smoother_for<float>() { return smoother; }
template <>
inline SmootherT<double>& Engine::smoother_for<double>() { return smoother64; }
template <>
inline SmootherT<float>& Engine::rsmoother_for<float>() { return rsmoother; }
template <>
inline SmootherT<double>& Engine::rsmoother_for<double>() { return rsmoother64; }

}  // namespace sifg
