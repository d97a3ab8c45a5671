// The smoothing stage (smooth.cu).
#pragma once

#include <cufft.h>

#include <memory>
#include <vector>

#include "kernels.cuh"

namespace sifg {

constexpr int kFilterNone = 0;
constexpr int kFilterTopHat = 1;
constexpr int kFilterGaussian = 2;

// Where a smoothing can list the cells it writes at or below a threshold, in
// flat order, by blocks of kBelowBlock cells: block b's entries at the start
// of its region [b * kBelowBlock, (b + 1) * kBelowBlock) of delta and flat,
// their number in counts[b]. counts NULL: no list.
constexpr uint32_t kBelowBlock = 8192;
struct BelowList {
  float thr = 0.f;
  uint32_t* counts = nullptr;  // cells / kBelowBlock
  float* delta = nullptr;      // cells slots
  uint32_t* flat = nullptr;    // cells slots
  // The field itself written too; false where the list is all its reader
  // needs (a run's candidates, under the cell seeds).
  bool field = true;
};

// Window modes: 0 none (SIF_FINDER_KEEP_CIC_WINDOW), 1 full CIC deconvolution,
// 2 aliasing-aware (SIF_FINDER_ALIASING_WINDOW). R is the form's precision:
// float (cuFFT R2C/C2R) or double (D2Z/Z2D).
template <class R>
struct SmootherT {
  uint32_t n = 0;
  R box = 0;
  int window_mode = 1;
  cudaStream_t stream = 0;
  cufftHandle plan_r2c = 0, plan_c2r = 0;  // the plans for n (unset on the own path at 512)
  DevBuf spectrum, work, lut, win;
  // The plans' work area, one for all of them: they run on `stream`, one at a
  // time. A plan made with its own area would allocate it, and destroying
  // it free it, a device-wide wait that stalls every other engine.
  DevBuf area;
  // Plans by grid size, kept between runs: at most kPlanCache sizes, oldest
  // out; a batch of boxes of many sizes keeps them all.
  static constexpr int kPlanCache = 64;
  struct Plans {
    uint32_t n;
    cufftHandle r2c, c2r;
    size_t work = 0;           // bytes of work area the two need
    void* twiddles = nullptr;  // the float form's own inverse at n = 512: its tables (no plans)
  };
  size_t plan_work = 0;  // the current plans' need
  const void* twiddles = nullptr;
  std::vector<Plans> plans;
  // The own inverse's filter factors at n = 512, one table per smoothing
  // (filter, radius, sigma, window, box): 257^3 floats (68 MB), the factor of
  // mode (|kx|, |ky|, kz) as the filter pass applies it. Built once, kept
  // (least recently used out past kFactorTables): a run's rungs smooth at the
  // same radii every time.
  struct FactorTable {
    int filter = 0, window_mode = 0;
    R r = 0, sigma = 0, box = 0;
    uint64_t used = 0;
    DevBuf buf;
  };
  static constexpr int kFactorTables = 24;
  std::vector<std::unique_ptr<FactorTable>> factor_tables;
  uint64_t factor_clock = 0;
  const float* factor_table(int filter, R r, R sigma);

  void setup(uint32_t n, R box, int window_mode, cudaStream_t st);
  // grid: n^3 values on the device; with mean set, the density, whose
  // contrast v * (1 / mean) - 1 is transformed (taken as the transform reads
  // it where it can, else in place first).
  void forward(const R* grid, const double* mean = nullptr);
  // Writes the grid smoothed at r (and, with sigma > 0, a Gaussian of sigma
  // on top) into out (n^3 values), asynchronously on the stream.
  // below (float form): the cells at or below below->thr listed as the
  // transform writes them, where lists_below() -- else the caller scans.
  void smooth(int filter, R r, R sigma, R* out, KernelTimer* timer,
              const BelowList* below = nullptr);
  bool lists_below() const { return sizeof(R) == 4 && twiddles != nullptr; }
  void restore(R* out);
  void release();
  ~SmootherT();
};
using Smoother = SmootherT<float>;

// 1 (default): the own inverse at 512 reads per-smoothing factor tables; 0:
// it evaluates the factors as it applies them. The same bits either way.
void set_factor_tables(int on);

}  // namespace sifg
