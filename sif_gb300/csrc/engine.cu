// The exodus run on one GPU: the rung loop of sif__exodus_run
// (src/finder/exodus_finder.c:1585-2492) for a periodic box, unweighted,
// seeds (every cell, or the local minima) on their nodes.
//
// Per rung, on one stream:
//   smooth (filter + C2R)  ->  candidate count  ->  [host: M]  ->  candidate
//   write  ->  copy to the host  ->  pre-filter  ->  sphere growth of every
//   survivor  ->  commit rounds  ->  append in rank order  ->  void index.
// While the GPU runs the pre-filter and the sphere growth, the host replays
// the reference's quicksort over the candidates (the depth order, ties
// included, is part of what the reference's catalogue is) and uploads each
// candidate's rank; the commit rounds are the first kernels that need it.
//
// The commit is the reference's sequential greedy pass, decided in rounds:
// a survivor is decided once every survivor ranked before it that could
// interact with it has been. Its tests -- node masked, pole masked at the
// rescaled radius, exact overlap -- are the reference's, against every void
// accepted before it; a failed test stays failed as the catalogue grows, so
// a survivor that fails against the current state is rejected at once.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "engine.cuh"

namespace sifg {

// SIF_PI, include/sif/core/macros.h:542.
template <class R>
static constexpr R kPi = (R)3.14159265358979323846;
static constexpr uint32_t kOptSeedsMinima = 1u << 9;
static constexpr uint32_t kOptKeepWindow = 1u << 14;
static constexpr uint32_t kOptAliasing = 1u << 8;
static constexpr uint32_t kOptLagrangian = 1u << 18;
static constexpr uint32_t kOptRefineMask = 3u << 19;
static constexpr uint32_t kOptRefineGaussian = 1u << 19;
static constexpr uint32_t kOptExtendReach = 1u << 21;
static constexpr uint32_t kOptDisplace = 1u << 22;
static constexpr uint32_t kGrowCap = 1u << 15;  // overflow window, floats per CTA

Engine::Engine(int device) : device_(device) {
  SIFG_CUDA(cudaSetDevice(device));
  int lo_prio = 0, hi_prio = 0;  // numerically, lo_prio >= hi_prio
  SIFG_CUDA(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
  // The run's stream first; then the smoothing, which the early rungs wait on;
  // the chain-mesh build last: it is needed only at the first sphere growth
  // and takes what bandwidth the smoothing leaves.
  const int mid_prio = hi_prio < lo_prio ? hi_prio + 1 : lo_prio;
  SIFG_CUDA(cudaStreamCreateWithPriority(&st_, cudaStreamNonBlocking, hi_prio));
  SIFG_CUDA(cudaStreamCreateWithPriority(&st_fft_, cudaStreamNonBlocking, mid_prio));
  SIFG_CUDA(cudaStreamCreateWithPriority(&st_copy_, cudaStreamNonBlocking, lo_prio));
  SIFG_CUDA(cudaEventCreateWithFlags(&ev_copy_start_, cudaEventDisableTiming));
  SIFG_CUDA(cudaEventCreateWithFlags(&ev_mesh_ready_, cudaEventDisableTiming));
  SIFG_CUDA(cudaEventCreateWithFlags(&ev_cand_, cudaEventDisableTiming));
  SIFG_CUDA(cudaEventCreateWithFlags(&ev_start_, cudaEventDisableTiming));
  for (int k = 0; k < 2; k++) {
    SIFG_CUDA(cudaEventCreateWithFlags(&ev_smoothed_[k], cudaEventDisableTiming));
    SIFG_CUDA(cudaEventCreateWithFlags(&ev_scanned_[k], cudaEventDisableTiming));
  }
  SIFG_CUDA(cudaMallocHost(&h_counters_, 2 * kCommitCounters * sizeof(uint32_t)));
}

Engine::~Engine() {
  cudaFreeHost(h_delta_);
  cudaFreeHost(h_flat_);
  cudaFreeHost(h_rank_);
  cudaFreeHost(h_counters_);
  if (ev_cand_) cudaEventDestroy(ev_cand_);
  for (cudaEvent_t ev : {ev_start_, ev_smoothed_[0], ev_smoothed_[1], ev_scanned_[0], ev_scanned_[1],
                         ev_copy_start_, ev_mesh_ready_})
    if (ev) cudaEventDestroy(ev);
  if (st_fft_) cudaStreamDestroy(st_fft_);
  if (st_copy_) cudaStreamDestroy(st_copy_);
  if (st_) cudaStreamDestroy(st_);
}

void Engine::ensure_host(size_t m) {
  if (m <= h_cap_) return;
  cudaFreeHost(h_delta_);
  cudaFreeHost(h_flat_);
  cudaFreeHost(h_rank_);
  const size_t cap = m + m / 4 + 1024;
  SIFG_CUDA(cudaMallocHost(&h_delta_, cap * sizeof(double)));
  SIFG_CUDA(cudaMallocHost(&h_flat_, cap * sizeof(uint32_t)));
  SIFG_CUDA(cudaMallocHost(&h_rank_, cap * sizeof(uint32_t)));
  h_cap_ = cap;
}

// ---------------------------------------------------------------------------
// The candidate order
// ---------------------------------------------------------------------------

namespace {

template <class K>
struct Rec {
  K d;
  uint32_t i;
};

// One three-way partition as the reference performs it: the pivot is the
// middle element's key; scanning from the left, a smaller key is exchanged to
// the low end, a larger one with the high end (and examined again), an equal
// one is passed over.
template <class K>
inline void partition3(Rec<K>* a, int64_t lo, int64_t hi, int64_t* lt_out, int64_t* gt_out) {
  const K pivot = a[lo + (hi - lo) / 2].d;
  int64_t lt = lo, i = lo, gt = hi;
  while (i <= gt) {
    const K v = a[i].d;
    if (v < pivot) {
      std::swap(a[lt], a[i]);
      lt++;
      i++;
    } else if (pivot < v) {
      std::swap(a[i], a[gt]);
      gt--;
    } else {
      i++;
    }
  }
  *lt_out = lt;
  *gt_out = gt;
}

template <class K>
void qsort_serial(Rec<K>* a, int64_t lo, int64_t hi) {
  std::vector<std::pair<int64_t, int64_t>> stack;
  stack.emplace_back(lo, hi);
  while (!stack.empty()) {
    const auto [l, h] = stack.back();
    stack.pop_back();
    if (l >= h) continue;
    int64_t lt, gt;
    partition3(a, l, h, &lt, &gt);
    stack.emplace_back(l, lt - 1);
    stack.emplace_back(gt + 1, h);
  }
}

// The two sides of a partition are disjoint, so sorting them in any order, on
// any threads, leaves the serial sort's permutation: tasks are spawned down
// to about a thousand elements, well below the reference's task cutoff
// (SIF_QUICKSORT_TASK_CUTOFF, include/sif/utils/sort.h:104), which only
// bounds its task overhead. (On 16 Grace cores, 100k candidates: 1.05 ms at
// 1024, 1.22 at 4096, 1.55 at 256, 1.71 at 16384.)
constexpr int64_t kTaskCutoff = 1024;

template <class K>
void qsort_tasks(Rec<K>* a, int64_t lo, int64_t hi) {
  if (hi - lo < kTaskCutoff) {
    qsort_serial(a, lo, hi);
    return;
  }
  int64_t lt, gt;
  partition3(a, lo, hi, &lt, &gt);
#pragma omp task untied
  qsort_tasks(a, lo, lt - 1);
  qsort_tasks(a, gt + 1, hi);
}

}  // namespace

// One Dijkstra partition of a[lo..hi] on t threads, with the same result as
// partition3. The sequential scan consumes the segment from two ends: from
// the left while it meets smaller or equal keys, and, after each larger key,
// from the right until it meets one that is not larger. So with K keys not
// larger than the pivot, the left end consumes positions [0, s) -- s = K, or
// K + 1 when position K holds a larger key -- and the right end the rest,
// last to first; the j-th larger key from the left is followed by the right
// end's run up to its j-th not-larger key. Every key's place follows from
// counts in the two streams:
//   smaller keys go to the front in the order examined, larger keys to the
//   back in reverse order examined, and equal keys fill the middle as a queue
//   that each later smaller key rotates by one (its exchange with the low
//   end moves the first equal key to the back).
// Returns false (nothing moved) when more than kMaxEqualQueue keys equal the
// pivot: the caller then partitions sequentially.
constexpr int64_t kParallelPartition = 32768;
constexpr int64_t kMaxEqualQueue = 2048;

template <class K>
bool partition3_parallel(Rec<K>* a, int64_t lo, int64_t hi, int t, int64_t* lt_out,
                         int64_t* gt_out) {
  const int64_t n = hi - lo + 1;
  Rec<K>* seg = a + lo;
  const K pivot = a[lo + (hi - lo) / 2].d;
  auto cls = [&](int64_t p) -> int { return seg[p].d < pivot ? 0 : (pivot < seg[p].d ? 2 : 1); };
  // Counts of smaller (L), equal (E) and larger (G) keys.
  std::vector<int64_t> cnt(3 * (size_t)t, 0);
  auto chunk = [&](int64_t len, int c) { return len * c / t; };
#pragma omp parallel for num_threads(t) schedule(static, 1)
  for (int c = 0; c < t; c++) {
    int64_t k3[3] = {0, 0, 0};  // counted in registers: the array is shared by every thread
    for (int64_t p = chunk(n, c); p < chunk(n, c + 1); p++) k3[cls(p)]++;
    for (int k = 0; k < 3; k++) cnt[3 * c + k] = k3[k];
  }
  int64_t nl = 0, ne = 0;
  for (int c = 0; c < t; c++) {
    nl += cnt[3 * c];
    ne += cnt[3 * c + 1];
  }
  if (ne > kMaxEqualQueue) return false;
  const int64_t k_ng = nl + ne;
  const int64_t s = k_ng + ((k_ng < n && cls(k_ng) == 2) ? 1 : 0);
  const int64_t nr = n - s;  // the right stream: r = 0..nr-1 is position n-1-r
  // Per-chunk counts over each stream (L, G, not-G), then exclusive prefixes.
  std::vector<int64_t> lc(3 * (size_t)(t + 1), 0), rc(3 * (size_t)(t + 1), 0);
#pragma omp parallel for num_threads(t) schedule(static, 1)
  for (int c = 0; c < t; c++) {
    int64_t l = 0, g = 0, ng = 0;
    for (int64_t p = chunk(s, c); p < chunk(s, c + 1); p++) {
      const int k = cls(p);
      l += k == 0;
      g += k == 2;
      ng += k != 2;
    }
    lc[3 * (c + 1)] = l;
    lc[3 * (c + 1) + 1] = g;
    lc[3 * (c + 1) + 2] = ng;
    l = g = ng = 0;
    for (int64_t r = chunk(nr, c); r < chunk(nr, c + 1); r++) {
      const int k = cls(n - 1 - r);
      l += k == 0;
      g += k == 2;
      ng += k != 2;
    }
    rc[3 * (c + 1)] = l;
    rc[3 * (c + 1) + 1] = g;
    rc[3 * (c + 1) + 2] = ng;
  }
  for (int c = 1; c <= t; c++)
    for (int k = 0; k < 3; k++) {
      lc[3 * c + k] += lc[3 * (c - 1) + k];
      rc[3 * c + k] += rc[3 * (c - 1) + k];
    }
  // The j-th larger key of the left stream (1-based): the smaller and the
  // not-larger keys before it (pa, pb). The right stream's j-th not-larger
  // key: the smaller keys up to and including it (ra) and its index (rb).
  // Scratch kept by the calling thread between calls (fresh multi-megabyte
  // vectors cost a page fault per page on every partition), reached from
  // the team through plain pointers: a thread_local named inside the
  // parallel regions would be each worker's own.
  thread_local std::vector<int64_t> scratch;
  thread_local std::vector<Rec<K>> out_buf;
  if (scratch.size() < 4 * ((size_t)n + 2)) scratch.resize(4 * ((size_t)n + 2));
  if (out_buf.size() < (size_t)n) out_buf.resize(n);
  int64_t* const pa = scratch.data();
  int64_t* const pb = pa + (n + 2);
  int64_t* const ra = pb + (n + 2);
  int64_t* const rb = ra + (n + 2);
  Rec<K>* const out = out_buf.data();
#pragma omp parallel for num_threads(t) schedule(static, 1)
  for (int c = 0; c < t; c++) {
    int64_t l = lc[3 * c], g = lc[3 * c + 1], ng = lc[3 * c + 2];
    for (int64_t p = chunk(s, c); p < chunk(s, c + 1); p++) {
      const int k = cls(p);
      if (k == 2) {
        pa[g + 1] = l;
        pb[g + 1] = ng;
      }
      l += k == 0;
      g += k == 2;
      ng += k != 2;
    }
    l = rc[3 * c];
    g = rc[3 * c + 1];
    ng = rc[3 * c + 2];
    for (int64_t r = chunk(nr, c); r < chunk(nr, c + 1); r++) {
      const int k = cls(n - 1 - r);
      if (k != 2) {
        ra[ng + 1] = l + (k == 0);
        rb[ng + 1] = r;
      }
      l += k == 0;
      g += k == 2;
      ng += k != 2;
    }
  }
  // Destinations; the equal keys with their place among the not-larger keys
  // in the order examined.
  std::vector<std::vector<std::pair<int64_t, Rec<K>>>> eq(t);
#pragma omp parallel for num_threads(t) schedule(static, 1)
  for (int c = 0; c < t; c++) {
    int64_t l = lc[3 * c], g = lc[3 * c + 1], ng = lc[3 * c + 2];
    for (int64_t p = chunk(s, c); p < chunk(s, c + 1); p++) {
      const int k = cls(p);
      if (k == 0)
        out[l + (g ? ra[g] : 0)] = seg[p];
      else if (k == 2)
        out[n - 1 - (g + (g ? rb[g] + 1 - g : 0))] = seg[p];
      else
        eq[c].emplace_back(ng + g, seg[p]);
      l += k == 0;
      g += k == 2;
      ng += k != 2;
    }
    l = rc[3 * c];
    g = rc[3 * c + 1];
    ng = rc[3 * c + 2];
    for (int64_t r = chunk(nr, c); r < chunk(nr, c + 1); r++) {
      const int64_t p = n - 1 - r;
      const int k = cls(p);
      const int64_t j = ng + 1;
      if (k == 2)
        out[n - 1 - (j + g)] = seg[p];
      else if (k == 0)
        out[pa[j] + l] = seg[p];
      else
        eq[c].emplace_back(pb[j] + (j - 1), seg[p]);
      l += k == 0;
      g += k == 2;
      ng += k != 2;
    }
  }
  // The equal keys: in the order examined, each joins the back of the queue;
  // each smaller key examined between two of them moves the front to the back.
  std::vector<std::pair<int64_t, Rec<K>>> e;
  for (auto& v : eq) e.insert(e.end(), v.begin(), v.end());
  std::sort(e.begin(), e.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
  std::vector<Rec<K>> q;
  q.reserve(e.size());
  size_t head = 0;
  for (size_t i = 0; i < e.size(); i++) {
    q.insert(q.begin() + (ptrdiff_t)head, e[i].second);  // the back of the queue
    head = (head + 1) % q.size();
    const int64_t next_t = i + 1 < e.size() ? e[i + 1].first : k_ng;
    const int64_t smaller = next_t - e[i].first - 1;  // not-larger keys between: all smaller
    head = (size_t)((head + (uint64_t)smaller) % q.size());
  }
  for (size_t i = 0; i < q.size(); i++) out[nl + (int64_t)i] = q[(head + i) % q.size()];
#pragma omp parallel for num_threads(t) schedule(static)
  for (int64_t p = 0; p < n; p++) seg[p] = out[p];
  *lt_out = lo + nl;
  *gt_out = lo + nl + ne - 1;
  return true;
}

template <class K>
void candidate_ranks(const K* delta, uint32_t m, uint32_t* rank, int threads) {
  thread_local std::vector<Rec<K>> keep;  // kept between calls, as the partition's scratch
  if (keep.size() < m) keep.resize(m);
  Rec<K>* const a = keep.data();  // the tasks reach it through this pointer
  const int t = threads > 0 ? threads : omp_get_max_threads();
  // The records and, after the sort, the ranks: independent per entry.
  const bool wide = m > 2 * (uint32_t)kTaskCutoff && t > 1;
#pragma omp parallel for num_threads(t) schedule(static) if (wide)
  for (int64_t k = 0; k < (int64_t)m; k++) a[k] = Rec<K>{delta[k], (uint32_t)k};
  if (m > 2 * (uint32_t)kTaskCutoff && t > 1) {
    // The large segments partitioned one at a time on every thread, the
    // rest as tasks; disjoint segments, so the permutation is the serial one.
    std::vector<std::pair<int64_t, int64_t>> big{{0, (int64_t)m - 1}}, small;
    while (!big.empty()) {
      const auto [l, h] = big.back();
      big.pop_back();
      if (h - l + 1 < kParallelPartition) {
        small.emplace_back(l, h);
        continue;
      }
      int64_t lt, gt;
      if (!partition3_parallel(a, l, h, t, &lt, &gt)) partition3(a, l, h, &lt, &gt);
      big.emplace_back(l, lt - 1);
      big.emplace_back(gt + 1, h);
    }
#pragma omp parallel num_threads(t)
#pragma omp single nowait
    for (const auto& [l, h] : small) {
#pragma omp task firstprivate(l, h)
      qsort_tasks(a, l, h);
    }
  } else if (m > 1) {
    qsort_serial(a, 0, (int64_t)m - 1);
  }
#pragma omp parallel for num_threads(t) schedule(static) if (wide)
  for (int64_t k = 0; k < (int64_t)m; k++) rank[a[k].i] = (uint32_t)k;
}

template void candidate_ranks<float>(const float*, uint32_t, uint32_t*, int);
template void candidate_ranks<double>(const double*, uint32_t, uint32_t*, int);

// ---------------------------------------------------------------------------
// The template
// ---------------------------------------------------------------------------

template <class R>
int build_template(HostTemplateT<R>& t, uint32_t mesh_n, R cell_length, R rmin, R r_search) {
  t = HostTemplateT<R>();
  const int32_t cr = (int32_t)(r_search / cell_length) + 1;
  if (cr >= (int32_t)mesh_n) return kErrRange;
  const R rs2 = r_search * r_search;
  const R rc2 = rmin * rmin;
  for (int32_t dx = -cr; dx <= cr; dx++)
    for (int32_t dy = -cr; dy <= cr; dy++)
      for (int32_t dz = -cr; dz <= cr; dz++) {
        const R mnx = dx == 0 ? 0.0f : (std::fabs((R)dx) - 1.0f) * cell_length;
        const R mny = dy == 0 ? 0.0f : (std::fabs((R)dy) - 1.0f) * cell_length;
        const R mnz = dz == 0 ? 0.0f : (std::fabs((R)dz) - 1.0f) * cell_length;
        const R mn = mnx * mnx + mny * mny + mnz * mnz;
        if (mn > rs2) continue;
        const R mxx = (std::fabs((R)dx) + 1.0f) * cell_length;
        const R mxy = (std::fabs((R)dy) + 1.0f) * cell_length;
        const R mxz = (std::fabs((R)dz) + 1.0f) * cell_length;
        const R mx = mxx * mxx + mxy * mxy + mxz * mxz;
        t.dx.push_back(dx);
        t.dy.push_back(dy);
        t.dz.push_back(dz);
        t.min_d2.push_back(mn);
        t.max_d2.push_back(mx);
        uint8_t type;
        if (mx <= rc2)
          type = kCellCore;
        else if (mn > rc2)
          type = mx <= rs2 ? kCellShell : kCellEdge;
        else
          type = kCellStraddle;
        t.type.push_back(type);
      }
  return kOk;
}

template int build_template<float>(HostTemplateT<float>&, uint32_t, float, float, float);
template int build_template<double>(HostTemplateT<double>&, uint32_t, double, double, double);

// ---------------------------------------------------------------------------
// The run
// ---------------------------------------------------------------------------

static int g_scan_mode = 0;
void set_scan_mode(int mode) { g_scan_mode = mode; }

template <class T>
static T* grow_to(DevBuf& b, size_t n) {
  return (T*)b.ensure(n * sizeof(T));
}

template <class R>
int Engine::exodus(const R* d_delta, const DeviceMeshT<R>& mesh, const RunParamsT<R>& p,
                   HostCatalogueT<R>& out, std::vector<RungStat>* stats, RunTimings* tm) {
  SmootherT<R>& smoother = smoother_for<R>();
  const auto t_start = std::chrono::steady_clock::now();
  if (tm && !tm->timed) tm = nullptr;
  if (tm) tm->mark_origin(st_);
  // The run appends one entry to stats per rung it runs (from first_rung).
  const size_t stats0 = stats ? stats->size() : 0;
  const uint32_t N = p.grid_n;
  const uint64_t cells = (uint64_t)N * N * N;
  const R box = p.box;
  const R cell = box / (R)N;
  const R threshold = p.threshold, f = p.overlap;
  const uint32_t opt = p.options;
  // SIF_FINDER_REFINE_GAUSSIAN (exodus_finder.c:1362-1380, 1740-1760;
  // utils.c:406-552): the minima found on the top-hat times a Gaussian of
  // 0.15 of the rung, placed between the nodes by a Newton step, and every
  // candidate ordered on that field. The tracer and hill refinements are
  // not run here.
  const bool gaussian = (opt & kOptRefineMask) == kOptRefineGaussian;
  if ((opt & kOptRefineMask) && !gaussian) {
    set_error(kErrUnsupported,
              "options: SIF_FINDER_REFINE_TRACERS and SIF_FINDER_REFINE_HILL are not supported by "
              "the GPU finder");
    return kErrUnsupported;
  }
  // SIF_FINDER_DISPLACE: no pre-filter, no witness against the rung's
  // starting catalogue (voids can leave it), and the commit one survivor at a
  // time in rank order (displace_commit).
  const bool displace = (opt & kOptDisplace) != 0;
  const bool extend = (opt & kOptExtendReach) != 0;
  // A survey (exodus_finder.c:1114-1137): cell seeds on their nodes only.
  const bool survey = p.random_mesh != nullptr;
  if (survey && (gaussian || displace || extend || (opt & kOptSeedsMinima) || !p.random_density)) {
    set_error(kErrInvalid, "options: a survey (expected SIF_FINDER_SEEDS_CELLS on their nodes)");
    return kErrInvalid;
  }
  if (cells >= (1ull << 32)) {
    set_error(kErrRange, "grid: more than 2^32 cells");
    return kErrRange;
  }
  // A weighted mesh (exodus_finder.c:1316-1319, 1076-1106): its weights
  // finite and non-negative, their total positive, before anything runs.
  const bool weighted = mesh.w != nullptr;
  if (weighted) {
    if (!mesh.cell_w) {
      set_error(kErrInvalid, "mesh: weights but no per-cell weight table");
      return kErrInvalid;
    }
    unsigned long long h_wc[2] = {0, 0};
    if (!p.weights_checked) {
      unsigned long long* wc = (unsigned long long*)grow_to<uint64_t>(wcheck_, 2);
      if (p.mesh_ready) SIFG_CUDA(cudaStreamWaitEvent(st_, p.mesh_ready, 0));
      check_weights(mesh.w, mesh.n_particles, wc, st_);
      SIFG_CUDA(cudaMemcpyAsync(h_wc, wc, sizeof(h_wc), cudaMemcpyDeviceToHost, st_));
      SIFG_CUDA(cudaStreamSynchronize(st_));
    }
    if (h_wc[0] || h_wc[1]) {
      set_error(kErrInvalid, "mesh: weights must be finite and non-negative (" +
                                 std::to_string(h_wc[0]) + " negative, " +
                                 std::to_string(h_wc[1]) + " not finite, of " +
                                 std::to_string(mesh.n_particles) + ")");
      return kErrInvalid;
    }
    if (!(mesh.total_weight > 0.0)) {
      set_error(kErrInvalid, "mesh: weights sum to zero (no mean density)");
      return kErrInvalid;
    }
  }
  const R scale = (opt & kOptLagrangian) ? (R)std::cbrt(1.0 + (double)threshold) : 1.0f;
  static const R factors[4] = {1.5f, 1.25f, 1.75f, 2.0f};
  const R search_factor = factors[(opt >> 12) & 3u];
  const int window_mode = (opt & kOptKeepWindow) ? 0 : ((opt & kOptAliasing) ? 2 : 1);
  // SIF_FINDER_SEEDS_MINIMA without refinement changes the candidates alone:
  // the local minima of the rung's field among them (exodus_finder.c:287-292).
  const bool minima = (opt & kOptSeedsMinima) != 0;

  std::vector<R> radii = p.radii;
  std::sort(radii.begin(), radii.end(), [](R a, R b) { return a > b; });

  R* fields[2] = {grow_to<R>(field_[0], cells), grow_to<R>(field_[1], cells)};
  // The refinement's own fields (the top-hat times the Gaussian), alongside.
  R* gfields[2] = {nullptr, nullptr};
  if (gaussian)
    for (int k = 0; k < 2; k++) gfields[k] = grow_to<R>(gfield_[k], cells);
  // Injected fields are consumed in the order the run's transforms return
  // them: per rung the top-hat and, refined, for a rung with candidates, the
  // refinement's field (the reference runs that transform only then).
  uint64_t inj_k = 0;
  uint32_t* mask = grow_to<uint32_t>(mask_, (cells + 31) / 32);
  SIFG_CUDA(cudaMemsetAsync(mask, 0, ((cells + 31) / 32) * sizeof(uint32_t), st_));
  // A survey's footprint, before any field is scanned
  // (sif__exodus_survey_occupancy, exodus_survey.c:159-201): the nodes the
  // randoms are nearest to, closed over the window that expects enough of
  // them; and the randoms' two fields.
  R* rfields[2] = {nullptr, nullptr};
  uint32_t* occ = nullptr;
  bool mesh_waited = false;
  if (survey) {
    for (int k = 0; k < 2; k++) rfields[k] = grow_to<R>(rfield_[k], cells);
    const uint64_t words = (cells + 31) / 32;
    occ = grow_to<uint32_t>(occ_, words);
    if (p.mesh_ready) {
      SIFG_CUDA(cudaStreamWaitEvent(st_, p.mesh_ready, 0));
      mesh_waited = true;
    }
    const DeviceMeshT<R>& rmesh = *p.random_mesh;
    const uint64_t marked =
        survey_mark(rmesh.x, rmesh.y, rmesh.z, rmesh.n_particles, N, box, occ,
                    (unsigned long long*)grow_to<uint64_t>(occ_count_, 1), st_);
    if (marked)
      survey_close(occ, grow_to<uint32_t>(occ_tmp_, words), N,
                   survey_closing_k(rmesh.n_particles, marked), st_);
  }
  SmootherT<R>& rsmoother = rsmoother_for<R>();
  // The smoothing stream starts after everything queued on the run's stream
  // (the density contrast among it); rung ri's field is fields[ri % 2].
  SIFG_CUDA(cudaEventRecord(ev_start_, st_));
  SIFG_CUDA(cudaStreamWaitEvent(st_fft_, ev_start_, 0));
  for (int k = 0; k < 2; k++) SIFG_CUDA(cudaEventRecord(ev_scanned_[k], st_));
  // Under the cell seeds, where the smoothing can list the cells at or below
  // the threshold as it writes them (the float form's own transform), the
  // scan is a mask filter over that list; two lists alternate with the fields.
  BelowList below[2];
  bool listed = false;
  auto smooth_rung = [&](uint32_t ri) {
    SIFG_CUDA(cudaStreamWaitEvent(st_fft_, ev_scanned_[ri % 2], 0));
    if (tm) tm->smoothing.begin(st_fft_);
    // With the list, the field's only other reader is SIF_FINDER_CONSUME_GRID
    // (the last rung's): the other rungs' fields are not written.
    if (listed) below[ri % 2].field = p.consume_out && ri + 1 == radii.size();
    smoother.smooth(kFilterTopHat, radii[ri], 0.0f, fields[ri % 2], tm ? &tm->filter : nullptr,
                    listed ? &below[ri % 2] : nullptr);
    // RUNG_MINIMA_SIGMA (exodus_finder.c:1362-1365) of the rung on top of
    // the top-hat, for every rung: a rung without candidates never reads it.
    if (gaussian)
      smoother.smooth(kFilterTopHat, radii[ri], R(0.15f) * radii[ri], gfields[ri % 2],
                      tm ? &tm->filter : nullptr);
    // A survey's rung (exodus_finder.c:1729-1737): the randoms smoothed the
    // same way, and the field scanned is the data against them.
    if (survey) {
      rsmoother.smooth(kFilterTopHat, radii[ri], 0.0f, rfields[ri % 2], nullptr);
      survey_contrast(fields[ri % 2], (const R*)rfields[ri % 2], occ, p.survey_alpha, cells, st_fft_);
    }
    if (tm) tm->smoothing.end(st_fft_);
    SIFG_CUDA(cudaEventRecord(ev_smoothed_[ri % 2], st_fft_));
  };
  // On every way out, nothing of the run is left in flight on the smoothing
  // stream.
  struct FftDrain {
    cudaStream_t s;
    ~FftDrain() { cudaStreamSynchronize(s); }
  } drain{st_fft_};
  const uint32_t nb_below = (uint32_t)((cells + kBelowBlock - 1) / kBelowBlock);
  if (!p.inject) {
    smoother.setup(N, box, window_mode, st_fft_);
    listed = g_scan_mode == 0 && sizeof(R) == 4 && !minima && !gaussian && !survey &&
             smoother.lists_below() && cells % kBelowBlock == 0;
    if (survey) {
      rsmoother.setup(N, box, window_mode, st_fft_);
      rsmoother.forward(p.random_density, nullptr);
    }
    if (listed)
      for (int k = 0; k < 2; k++) {
        below[k].thr = (float)threshold;
        below[k].counts = grow_to<uint32_t>(below_counts_[k], nb_below);
        below[k].delta = grow_to<float>(below_delta_[k], cells);
        below[k].flat = grow_to<uint32_t>(below_flat_[k], cells);
      }
    smoother.forward(d_delta, p.contrast_mean);
    if (p.first_rung < radii.size()) smooth_rung(p.first_rung);
  }

  // Loop invariants, exodus_finder.c:1629-1632.
  const R box_volume = box * box * box;
  const R mean_density = (R)mesh.n_particles / box_volume;
  const R vol_factor = (4.0f / 3.0f) * kPi<R> * mean_density;
  // What the density tests measure against (1634-1642): on a weighted mesh
  // the mean weight density, rounded and divided as the count is; the
  // histogram is still sized by the tracer count.
  const R mass_factor =
      weighted ? (4.0f / 3.0f) * kPi<R> * ((R)mesh.total_weight / box_volume) : vol_factor;

  uint32_t n_voids = 0;
  // The catalogue's buffers keep their size from run to run (a cudaFree
  // waits for the whole device, which would stall every other engine of a
  // batch); they grow, keeping the voids so far, only when a run needs more.
  auto ensure_cat = [&](size_t want) {
    const size_t have = cat_x_.bytes / sizeof(R);
    if (want <= have && cat_r_.ptr && vids_.bytes >= want * sizeof(uint32_t) &&
        vcell_.bytes >= want * sizeof(uint32_t))
      return;
    size_t cap = std::max<size_t>(want + want / 2, 1 << 16);
    DevBuf* bufs[4] = {&cat_x_, &cat_y_, &cat_z_, &cat_r_};
    for (DevBuf* b : bufs) {
      if (b->ptr && b->bytes >= cap * sizeof(R)) continue;
      void* fresh = nullptr;
      SIFG_CUDA(cudaMalloc(&fresh, cap * sizeof(R)));
      if (n_voids && b->ptr)
        SIFG_CUDA(cudaMemcpyAsync(fresh, b->ptr, n_voids * sizeof(R), cudaMemcpyDeviceToDevice, st_));
      SIFG_CUDA(cudaStreamSynchronize(st_));
      b->release();
      b->ptr = fresh;
      b->bytes = cap * sizeof(R);
    }
    vids_.ensure(cap * sizeof(uint32_t));
    vcell_.ensure(cap * sizeof(uint32_t));
  };
  ensure_cat(1 << 16);
  const uint32_t vcells = kVoidCells * kVoidCells * kVoidCells;
  uint32_t* vstart = grow_to<uint32_t>(vstart_, vcells + 1);
  build_void_index(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), 0, box, vstart,
                   vids_.as<uint32_t>(), vcell_.as<uint32_t>(), st_);
  R max_r = 0.0f;
  if (p.n_prior) {
    // The prior voids, as though earlier rungs had accepted them: the
    // catalogue, the overlap mask at scale * r, the void index and the
    // largest radius (accept_void, exodus_finder.c:656-683).
    if (p.n_prior >= (1ull << 31)) {
      set_error(kErrRange, "prior: 2^31 voids or more");
      return kErrRange;
    }
    const uint32_t np = (uint32_t)p.n_prior;
    ensure_cat(np);
    const R* cols[4] = {p.prior_cx, p.prior_cy, p.prior_cz, p.prior_r};
    DevBuf* dst[4] = {&cat_x_, &cat_y_, &cat_z_, &cat_r_};
    for (int k = 0; k < 4; k++)
      SIFG_CUDA(cudaMemcpyAsync(dst[k]->ptr, cols[k], np * sizeof(R), cudaMemcpyHostToDevice, st_));
    for (uint32_t v = 0; v < np; v++)
      if (p.prior_r[v] > max_r) max_r = p.prior_r[v];
    RungConstsT<R> pc{};
    pc.scale = scale;
    pc.cell = cell;
    pc.gbox = (R)N * cell;
    pc.grid_n = N;
    paint_voids(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), cat_r_.as<R>(), np, mask, pc, st_);
    n_voids = np;
    build_void_index(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), n_voids, box, vstart,
                     vids_.as<uint32_t>(), vcell_.as<uint32_t>(), st_);
  }
  R* gbuf = grow_to<R>(gbuf_, (size_t)growth_grid() * kGrowCap);
  uint32_t* dcount = grow_to<uint32_t>(dcount_, 16);
  // The growth and witness kernels' work counters (the survivors' queue).
  uint32_t* work = grow_to<uint32_t>(work_, 4);
  // Gathered particles and visited cells of each rung's sphere growth.
  const size_t n_rungs = radii.size();
  unsigned long long* traffic = (unsigned long long*)grow_to<uint64_t>(traffic_, 2 * n_rungs + 2);
  SIFG_CUDA(cudaMemsetAsync(traffic, 0, (2 * n_rungs + 2) * sizeof(uint64_t), st_));
  uint32_t* counters = grow_to<uint32_t>(counters_, kCommitCounters);
  const uint32_t nb_scan = scan_blocks(cells);
  uint32_t* blocks = grow_to<uint32_t>(
      blocks_, (size_t)std::max<uint64_t>(std::max<uint64_t>(nb_scan, nb_below) + 1, 1024));

  MeshViewT<R> mv{mesh.x,          mesh.y,          mesh.z,
                  mesh.offsets,    (int32_t)mesh.n_cells, mesh.box_length,
                  1.0f / mesh.cell_length, mesh.xyzw};
  long long* gwbuf = nullptr;
  if (weighted) {
    // The fixed point of the weight sums: no sum exceeds the total weight
    // times the times a search's template can meet one cell (its side over
    // the mesh's, cubed; the top rung's reach is the widest).
    const R r_top = radii.front();
    const R reach = r_top + std::fmax((search_factor - 1.0f) * r_top, 3.0f * cell);
    const double side = 2.0 * ((double)(int64_t)(reach / mesh.cell_length) + 2.0) + 1.0;
    const double rep = std::pow(std::ceil(side / (double)mesh.n_cells), 3.0);
    double ws = 0, wi = 0;
    weight_fixed_point(mesh.total_weight * rep, &ws, &wi);
    mv.w = mesh.w;
    mv.cell_w = mesh.cell_w;
    mv.wscale = (R)ws;
    mv.winv = wi;
    gwbuf = grow_to<long long>(gwbuf_, (size_t)growth_grid() * kGrowCap);
  }
  // A survey weighs on both meshes: a mesh without weights counts each
  // tracer 1 (a unit of 1); the randoms' weights in a fixed point of their own.
  MeshViewT<R> rmv{};
  R survey_K = 0;
  if (survey) {
    if (!weighted) {
      mv.wscale = (R)1;
      mv.winv = 1.0;
    }
    const DeviceMeshT<R>& rm = *p.random_mesh;
    rmv = MeshViewT<R>{rm.x, rm.y, rm.z, rm.offsets, (int32_t)rm.n_cells, rm.box_length,
                       1.0f / rm.cell_length, rm.xyzw};
    rmv.wscale = (R)1;
    rmv.winv = 1.0;
    if (rm.w) {
      const R r_top = radii.front();
      const R reach = r_top + std::fmax((search_factor - 1.0f) * r_top, 3.0f * cell);
      const double side = 2.0 * ((double)(int64_t)(reach / rm.cell_length) + 2.0) + 1.0;
      const double rep = std::pow(std::ceil(side / (double)rm.n_cells), 3.0);
      double ws = 0, wi = 0;
      weight_fixed_point(rm.total_weight * rep, &ws, &wi);
      rmv.w = rm.w;
      rmv.cell_w = rm.cell_w;
      rmv.wscale = (R)ws;
      rmv.winv = wi;
    }
    // exodus_finder.c:1649-1653.
    survey_K = (1.0f + threshold) * p.survey_alpha;
    gwbuf = grow_to<long long>(gwbuf_, (size_t)growth_grid() * kGrowCap);
  }

  // The sphere growth's constants for a search shell [rmin, r_search]
  // (exodus_rescale.c:681-720, 894-908), on top of the rung's own.
  auto shell_consts = [&](RungConstsT<R> rc, R rmin, R r_search) {
    rc.r_search = r_search;
    rc.rmin = rmin;
    rc.rs2 = r_search * r_search;
    rc.rc2 = rmin * rmin;
    const R span = rc.rs2 - rc.rc2;
    uint32_t nb = 2048u;
    const R expected_shell = vol_factor * (r_search * r_search * r_search - rmin * rmin * rmin);
    const R want = expected_shell / 16.0f;
    if (!(want >= 64.0f))
      nb = 64u;
    else if (want < 2048.0f)
      nb = (uint32_t)want;
    rc.nb = nb;
    rc.inv_w = (R)nb / span;
    rc.bin_w = span / (R)nb;
    const R K = (threshold + 1.0f) * mass_factor;
    rc.K2 = K * K;
    rc.expected = mass_factor * r_search * r_search * r_search;
    rc.threshold = threshold;
    rc.window = (uint32_t)std::max(1, p.window);
    return rc;
  };
  // A template in one upload into `buf`: min and max d^2, the three offsets,
  // the classes, packed in that order (each part aligned for its type).
  auto upload_template = [&](const HostTemplateT<R>& ht, DevBuf& buf) {
    const uint32_t tcount = (uint32_t)ht.type.size();
    const size_t t_real = ((size_t)tcount * sizeof(R) + 15) & ~(size_t)15;
    const size_t t_int = ((size_t)tcount * sizeof(int32_t) + 15) & ~(size_t)15;
    const size_t t_bytes = 2 * t_real + 3 * t_int + tcount;
    if (h_tpl_.size() < t_bytes) h_tpl_.resize(t_bytes);
    uint8_t* hp = h_tpl_.data();
    std::memcpy(hp, ht.min_d2.data(), tcount * sizeof(R));
    std::memcpy(hp + t_real, ht.max_d2.data(), tcount * sizeof(R));
    std::memcpy(hp + 2 * t_real, ht.dx.data(), tcount * sizeof(int32_t));
    std::memcpy(hp + 2 * t_real + t_int, ht.dy.data(), tcount * sizeof(int32_t));
    std::memcpy(hp + 2 * t_real + 2 * t_int, ht.dz.data(), tcount * sizeof(int32_t));
    std::memcpy(hp + 2 * t_real + 3 * t_int, ht.type.data(), tcount);
    uint8_t* dp = grow_to<uint8_t>(buf, t_bytes);
    // Pageable source: the copy is staged before the call returns, so the
    // staging vector is free for the next template at once.
    SIFG_CUDA(cudaMemcpyAsync(dp, hp, t_bytes, cudaMemcpyHostToDevice, st_));
    return TemplateViewT<R>{(const int32_t*)(dp + 2 * t_real),
                            (const int32_t*)(dp + 2 * t_real + t_int),
                            (const int32_t*)(dp + 2 * t_real + 2 * t_int),
                            dp + 2 * t_real + 3 * t_int,
                            (const R*)dp,
                            (const R*)(dp + t_real),
                            tcount};
  };

  // SIF_FINDER_EXTEND_REACH (exodus_finder.c:1664-1702, 242-244, 1342-1353):
  // a crossing past a rung's reach is measured again at the levels of an
  // extended reach, from the top rung's reach down by EXT_GROWTH to below the
  // bottom rung; level k measures [ext_rmin[k], ext_reach[k]]. The levels are
  // the same for every rung and built once.
  const R kExtGrowth = 1.5f, kExtSlack = 1.2f;
  uint32_t n_ext = 0;
  R ext_reach[kExtMaxLevels], ext_rmin[kExtMaxLevels];
  TemplateViewT<R> ext_tv[kExtMaxLevels];
  if (extend && !radii.empty()) {
    const R r_top = radii.front();
    const R r_ext = r_top + std::fmax((search_factor - 1.0f) * r_top, 3.0f * cell);
    const R r_low = radii.back();
    while (n_ext < kExtMaxLevels &&
           (n_ext == 0 || r_ext / std::pow(kExtGrowth, (R)(n_ext - 1)) > r_low))
      n_ext++;
    for (uint32_t k = 0; k < n_ext; k++)
      ext_reach[k] = r_ext / std::pow(kExtGrowth, (R)(n_ext - 1 - k));
    for (uint32_t k = 0; k < n_ext; k++) {
      ext_rmin[k] = (k ? ext_reach[k - 1] : ext_reach[0] / kExtGrowth) / kExtSlack;
      HostTemplateT<R> ht;
      if (build_template(ht, mesh.n_cells, mesh.cell_length, ext_rmin[k], ext_reach[k]) != kOk) {
        set_error(kErrRange, "extended reach of " + std::to_string(ext_reach[k]) +
                                 " wider than the mesh; use a finer mesh or smaller radii");
        return kErrRange;
      }
      ext_tv[k] = upload_template(ht, ext_tpl_[k]);
    }
  }

  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t0) {
    return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  };
  // Called at each rung's end (after the commit's voids are in the catalogue).
  auto rung_done = [&](uint32_t done, uint64_t mismatched) -> int {
    if (!p.after_rung) return kOk;
    return p.after_rung(done, cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), cat_r_.as<R>(),
                        n_voids, mismatched);
  };
  for (uint32_t ri = p.first_rung; ri < radii.size(); ri++) {
    const auto t_rung = clk::now();
    RungStat rs;
    const R radius = radii[ri];
    rs.radius = radius;

    // 1. The rung's field; the next rung's smoothing queued behind this
    //    rung's last read of the buffer it overwrites.
    R* field = fields[ri % 2];
    const cudaMemcpyKind inj_kind =
        p.inject_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (p.inject) {
      SIFG_CUDA(cudaMemcpyAsync(field, p.inject + inj_k++ * cells, cells * sizeof(R), inj_kind, st_));
      if (survey) {
        R* rf = rfields[ri % 2];
        SIFG_CUDA(cudaMemcpyAsync(rf, p.inject + inj_k++ * cells, cells * sizeof(R), inj_kind, st_));
        survey_contrast(field, (const R*)rf, occ, p.survey_alpha, cells, st_);
      }
    } else {
      if (ri + 1 < radii.size()) smooth_rung(ri + 1);
      SIFG_CUDA(cudaStreamWaitEvent(st_, ev_smoothed_[ri % 2], 0));
    }
    if (tm) tm->rung.begin(st_);

    // 2. Candidates, in flat order.
    R* region_delta = nullptr;
    uint32_t* region_flat = nullptr;
    const BelowList& bl = below[ri % 2];
    rs.from_list = listed ? 1u : 0u;
    if (listed) {
      below_count_pass(bl.counts, bl.flat, nb_below, kBelowBlock, mask, blocks, dcount, st_);
    } else {
      const uint64_t slots = scan_region_slots(cells);
      region_delta = grow_to<R>(region_delta_, slots);
      region_flat = grow_to<uint32_t>(region_flat_, slots);
      // Refined, the candidates are every cell at or below the threshold
      // (the minima are found on the refinement's field, below).
      scan_fused_pass(field, mask, cells, threshold, blocks, dcount, region_delta, region_flat, st_,
                      N, minima && !gaussian);
      // The field's last reader: the next rung but one may smooth into it
      // (refined, the placing reads it again: recorded after that).
      if (!gaussian) SIFG_CUDA(cudaEventRecord(ev_scanned_[ri % 2], st_));
    }
    SIFG_CUDA(cudaMemcpyAsync(h_counters_, dcount, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
    const auto t_wait = clk::now();
    SIFG_CUDA(cudaStreamSynchronize(st_));
    rs.count_wait_ms = ms_since(t_wait);
    uint32_t m = h_counters_[0];
    rs.n_candidates = m;
    R* cdelta = nullptr;
    uint32_t* cflat = nullptr;
    const CandOffT<R>* coff = nullptr;
    if (gaussian) {
      if (m > 0) {
        // The cells to place, then the refinement's field: the next injected
        // one, or the smoothing's.
        cdelta = grow_to<R>(cand_delta_, m);
        cflat = grow_to<uint32_t>(cand_flat_, m);
        scan_compact(blocks, cells, region_delta, region_flat, cdelta, cflat, st_);
        R* gf = gfields[ri % 2];
        if (p.inject)
          SIFG_CUDA(cudaMemcpyAsync(gf, p.inject + inj_k++ * cells, cells * sizeof(R), inj_kind, st_));
        CandOffT<R>* ocoff = nullptr;
        m = refine_candidates(field, gf, mask, threshold, N, cell, m, minima, cdelta, cflat,
                              grow_to<R>(cand_delta2_, m), grow_to<uint32_t>(cand_flat2_, m),
                              grow_to<CandOffT<R>>(cand_off2_, m), ocoff,
                              grow_to<CandOffT<R>>(cand_off_, m), grow_to<uint32_t>(keep_, m + 1),
                              h_counters_ + 1, st_);
        coff = ocoff;
      }
      // Both fields' last reader was the placing.
      SIFG_CUDA(cudaEventRecord(ev_scanned_[ri % 2], st_));
      rs.n_candidates = m;
    }

    // The reach and the rescaling's constants (exodus_finder.c:1771-1817,
    // exodus_rescale.c:681-720, 894-908).
    const R rmin = 1.0f * radius;
    R r_search = radius + std::fmax((search_factor - 1.0f) * radius, 3.0f * cell);
    if (ri > 0 && radii[ri - 1] > r_search) r_search = radii[ri - 1];
    rs.r_search = r_search;
    if (m == 0) {
      // The list's last reader was its count pass.
      if (listed) SIFG_CUDA(cudaEventRecord(ev_scanned_[ri % 2], st_));
      if (tm) tm->rung.end(st_);
      rs.rung_ms = ms_since(t_rung);
      if (stats) stats->push_back(rs);
      if (const int hs = rung_done(ri + 1, 0); hs != kOk) return hs;
      continue;
    }

    if (gaussian) {
      // placed above
    } else if (listed) {
      cdelta = grow_to<R>(cand_delta_, m);
      cflat = grow_to<uint32_t>(cand_flat_, m);
      if constexpr (sizeof(R) == 4)
        below_write_pass(bl.counts, bl.delta, bl.flat, nb_below, kBelowBlock, mask, blocks, cdelta,
                         cflat, st_);
      // The list's last reader: the next rung but one may smooth into it.
      SIFG_CUDA(cudaEventRecord(ev_scanned_[ri % 2], st_));
    } else {
      cdelta = grow_to<R>(cand_delta_, m);
      cflat = grow_to<uint32_t>(cand_flat_, m);
      scan_compact(blocks, cells, region_delta, region_flat, cdelta, cflat, st_);
    }
    ensure_host(m);
    SIFG_CUDA(cudaMemcpyAsync(h_delta_, cdelta, m * sizeof(R), cudaMemcpyDeviceToHost, st_));
    SIFG_CUDA(cudaEventRecord(ev_cand_, st_));

    RungConstsT<R> rc0{};
    rc0.radius = radius;
    rc0.proxy_pole = (int32_t)(scale * radius * (1.0f - f) / cell) - 1;
    rc0.scale = scale;
    rc0.f = f;
    rc0.cell = cell;
    rc0.grid_n = N;
    rc0.box = box;
    rc0.gbox = (R)N * cell;
    const RungConstsT<R> rc = shell_consts(rc0, rmin, r_search);
    const R span = rc.rs2 - rc.rc2;

    HostTemplateT<R> ht;
    if (build_template(ht, mesh.n_cells, mesh.cell_length, rmin, r_search) != kOk) {
      set_error(kErrRange, "search sphere of " + std::to_string(r_search) +
                               " wider than the mesh; use a finer mesh or smaller radii");
      return kErrRange;
    }
    const TemplateViewT<R> tv = upload_template(ht, tpl_);
    // The randoms' mesh is free to use cells of its own, so it gets its own
    // template (exodus_finder.c:1834-1845).
    TemplateViewT<R> rtv{};
    if (survey) {
      HostTemplateT<R> rht;
      if (build_template(rht, p.random_mesh->n_cells, p.random_mesh->cell_length, rmin, r_search) !=
          kOk) {
        set_error(kErrRange, "search sphere of " + std::to_string(r_search) +
                                 " wider than the random mesh; use a finer mesh or smaller radii");
        return kErrRange;
      }
      rtv = upload_template(rht, rtpl_);
    }
    // The first level of the extended reach this rung enters: the lowest
    // EXT_SLACK past its own reach, or the top if none is
    // (exodus_finder.c:1826-1832).
    uint32_t ext0 = n_ext;
    for (uint32_t k = 0; k < n_ext && ext0 == n_ext; k++)
      if (ext_reach[k] >= kExtSlack * r_search) ext0 = k;
    if (ext0 == n_ext && n_ext > 0 && ext_reach[n_ext - 1] > r_search) ext0 = n_ext - 1;

    // 3. Pre-filter at the rung, against the catalogue as the rung begins.
    VoidViewT<R> vv{cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), cat_r_.as<R>(),
                vstart, vids_.as<uint32_t>(), (R)kVoidCells / box, max_r, n_voids};
    uint8_t* alive = grow_to<uint8_t>(alive_, m);
    uint32_t* scand = grow_to<uint32_t>(surv_cand_, m);
    uint32_t* sflat = grow_to<uint32_t>(surv_flat_, m);
    R* scx = grow_to<R>(scx_, m);
    R* scy = grow_to<R>(scy_, m);
    R* scz = grow_to<R>(scz_, m);
    R* sr = grow_to<R>(sr_, m);
    uint8_t* sreason = grow_to<uint8_t>(sreason_, m);
    uint32_t* blocks2 = grow_to<uint32_t>(rank_slots_, (size_t)m + 2048);
    R* soff = coff ? grow_to<R>(soff_, m) : nullptr;
    prefilter(cflat, m, mask, vv, rc, alive, blocks2, scand, sflat, scx, scy, scz, dcount + 1, st_,
              displace, coff, soff);
    SurvivorsT<R> sv{scand, sflat, scx, scy, scz, sr, sreason, dcount + 1, soff};

    // 4. Sphere growth of every survivor.
    if (!(span > 0.0f)) {
      // RESCALE_DEGENERATE for every candidate: no annulus.
      std::vector<R> neg(m, -1.0f);
      SIFG_CUDA(cudaMemcpyAsync(sr, neg.data(), m * sizeof(R), cudaMemcpyHostToDevice, st_));
      SIFG_CUDA(cudaMemsetAsync(sreason, kRescaleDegenerate, m, st_));
    } else {
      if (p.mesh_ready && !mesh_waited) {
        SIFG_CUDA(cudaStreamWaitEvent(st_, p.mesh_ready, 0));
        mesh_waited = true;
      }
      // The collision witness against the catalogue as the rung begins
      // (exodus_finder.c:2019-2030), then the growth of the rest. Under
      // displacement every survivor is grown: a void refusing it now may be
      // displaced before its turn.
      // No witness on a weighted mesh either (1865-1868).
      if (displace || weighted || survey)
        SIFG_CUDA(cudaMemsetAsync(sreason, kRescaleOk, m, st_));
      else
        witness(mv, tv, rc, sv, vv, m, traffic + 2 * ri, st_, tm ? &tm->witness : nullptr, work);
      if (survey)
        grow_survey(mv, tv, rmv, rtv, rc, survey_K, sv, m, gbuf, gwbuf, kGrowCap, traffic + 2 * ri,
                    st_, tm ? &tm->growth : nullptr, work);
      else if (weighted)
        grow_weighted(mv, tv, rc, sv, m, gbuf, gwbuf, kGrowCap, traffic + 2 * ri, st_,
                      tm ? &tm->growth : nullptr, kAllSurvivors, work);
      else
        grow(mv, tv, rc, sv, m, gbuf, kGrowCap, traffic + 2 * ri, st_, tm ? &tm->growth : nullptr,
             kAllSurvivors, work, grow_to<uint32_t>(pend_, m));
      // Each level of the extended reach, for the survivors whose crossing
      // still lies past the reach (exodus_finder.c:2060-2072).
      for (uint32_t e = ext0; e < n_ext; e++) {
        const RungConstsT<R> ec = shell_consts(rc, ext_rmin[e], ext_reach[e]);
        if (weighted)
          grow_weighted(mv, ext_tv[e], ec, sv, m, gbuf, gwbuf, kGrowCap, traffic + 2 * ri, st_,
                        tm ? &tm->growth : nullptr, kRescaleBeyondSearch, work);
        else
          grow(mv, ext_tv[e], ec, sv, m, gbuf, kGrowCap, traffic + 2 * ri, st_,
               tm ? &tm->growth : nullptr, kRescaleBeyondSearch, work, grow_to<uint32_t>(pend_, m));
      }
    }

    // The commit's preparation, which needs the radii but not the order:
    // queued now, so that it runs while the host sorts.
    SurvivorGridT<R> sg{};
    uint8_t* sa = nullptr;
    uint8_t* sb = nullptr;
    uint32_t* acc = nullptr;
    if (!displace) {
      // Radii reach the top level's reach where the rung enters the extended one.
      const R r_max = ext0 < n_ext ? std::max(r_search, ext_reach[n_ext - 1]) : r_search;
      const R reach = 2.0f * scale * r_max + 2.0f * cell;
      int32_t ng = (int32_t)std::floor(box / reach);
      if (ng < 3) ng = 1;
      if (ng > 256) ng = 256;
      const uint32_t sg_cells = (uint32_t)(ng * ng * ng);
      uint32_t* sg_start = grow_to<uint32_t>(sgrid_start_, sg_cells + 1);
      uint32_t* sg_ids = grow_to<uint32_t>(sgrid_ids_, m);
      uint32_t* sg_cell = grow_to<uint32_t>(sgrid_cellof_, m);
      SurvPackT<R>* sg_pack = grow_to<SurvPackT<R>>(sgrid_pack_, m);
      build_survivor_grid(scx, scy, scz, (const R*)sr, dcount + 1, m, ng, box, sg_start, sg_ids,
                          sg_cell, sg_pack, st_);
      sg = SurvivorGridT<R>{sg_start, sg_ids, ng, (R)ng / box, sg_pack,
                            grow_to<uint32_t>(sgrid_rank_, m)};
      sa = grow_to<uint8_t>(state_a_, m);
      sb = grow_to<uint8_t>(state_b_, m);
      acc = grow_to<uint32_t>(acc_, m);
      SIFG_CUDA(cudaMemsetAsync(counters, 0, kCommitCounters * sizeof(uint32_t), st_));
      commit_init(sv, vv, rc, sa, counters, m, st_);
    }

    // 5. The order, on the host while the GPU grows spheres.
    const auto t_wait_cand = clk::now();
    SIFG_CUDA(cudaEventSynchronize(ev_cand_));
    rs.cand_wait_ms = ms_since(t_wait_cand);
    const auto t_sort = clk::now();
    candidate_ranks((const R*)h_delta_, m, h_rank_, host_threads);
    rs.sort_ms = ms_since(t_sort);
    uint32_t* rank = grow_to<uint32_t>(rank_, m);
    SIFG_CUDA(cudaMemcpyAsync(rank, h_rank_, m * sizeof(uint32_t), cudaMemcpyHostToDevice, st_));
    if (!displace) survivor_grid_ranks(sv, rank, sg.ids, (uint32_t*)sg.hrank, m, st_);

    // 6. The commit, in rounds; under displacement one survivor at a time.
    const auto t_commit = clk::now();
    if (displace) {
      ensure_cat(n_voids + m);
      // The compressed index again: growing the catalogue may have moved its
      // buffers. The chains are built from it.
      build_void_index(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), n_voids, box, vstart,
                       vids_.as<uint32_t>(), vcell_.as<uint32_t>(), st_);
      uint32_t* order = grow_to<uint32_t>(acc_, m);
      int32_t* head = grow_to<int32_t>(vhead_, kVoidCells * kVoidCells * kVoidCells);
      int32_t* next = grow_to<int32_t>(vnext_, (size_t)n_voids + m + 1);
      const uint32_t cap = n_voids + m + 1;
      uint32_t* conflicts = grow_to<uint32_t>(dlist_, 2 * (size_t)cap);
      uint32_t hstate[8] = {n_voids, 0, 0, 0, 0, 0, 0, 0};
      std::memcpy(&hstate[4], &max_r, sizeof(R));
      uint32_t* dstate = counters;
      SIFG_CUDA(cudaMemcpyAsync(dstate, hstate, sizeof hstate, cudaMemcpyHostToDevice, st_));
      displace_commit(sv, rank, m, order, vstart, vids_.as<uint32_t>(), head, next, cat_x_.as<R>(),
                      cat_y_.as<R>(), cat_z_.as<R>(), cat_r_.as<R>(), box, mask, rc, dstate,
                      conflicts, conflicts + cap, cap, st_);
      SIFG_CUDA(cudaMemcpyAsync(h_counters_, dstate, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
      SIFG_CUDA(cudaStreamSynchronize(st_));
      if (h_counters_[3]) {
        set_error(kErrInvalid, "displacement: a conflict list outgrew its scratch");
        return kErrInvalid;
      }
      const uint32_t n_acc = h_counters_[1], n_removed = h_counters_[2];
      rs.n_mismatched = h_counters_[6];
      std::memcpy(&max_r, &h_counters_[4], sizeof(R));
      if (n_removed) {
        compact_voids(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), cat_r_.as<R>(), dstate, st_);
        SIFG_CUDA(cudaMemcpyAsync(h_counters_, dstate, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
        SIFG_CUDA(cudaStreamSynchronize(st_));
      }
      n_voids = h_counters_[0];
      build_void_index(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), n_voids, box, vstart,
                       vids_.as<uint32_t>(), vcell_.as<uint32_t>(), st_);
      if (tm) tm->rung.end(st_);
      rs.commit_ms = ms_since(t_commit);
      rs.n_survivors = m;
      rs.n_accepted = n_acc;
      rs.n_displaced = n_removed;
      rs.rung_ms = ms_since(t_rung);
      if (stats) stats->push_back(rs);
      if (const int hs = rung_done(ri + 1, rs.n_mismatched); hs != kOk) return hs;
      continue;
    }
    // The rounds run in one cooperative launch, to the round that leaves no
    // survivor undecided (or a ring's worth, then another launch); where
    // the device cannot, a few rounds are issued at a time between reads of
    // the undecided count (a round after the last one decides nothing and
    // paints nothing).
    uint64_t rounds = 0;
    uint32_t* h_count = h_counters_ + kCommitCounters;
    uint32_t* h_bar = h_count + 1;  // the cooperative launch's report: bar[2] error, bar[3] rounds
    unsigned* bar = grow_to<unsigned>(commit_bar_, 4);
    for (uint32_t batch = 3;; batch = 4) {
      if (tm) tm->commit.begin(st_);
      SIFG_CUDA(cudaMemsetAsync(counters + kRoundUndecided, 0, kRoundRing * sizeof(uint32_t), st_));
      const bool one_launch = commit_rounds(sv, rank, sg, vv, mask, rc, sa, sb, acc, counters,
                                            (uint32_t)rounds, kRoundRing, bar, m, st_);
      if (one_launch) {
        SIFG_CUDA(cudaMemcpyAsync(h_bar, bar, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, st_));
      } else {
        for (uint32_t b = 0; b < batch; b++) {
          commit_round(sv, rank, sg, vv, mask, rc, sa, sb, acc, counters, (uint32_t)rounds, m, st_);
          paint_new(sv, acc, counters, (uint32_t)rounds, mask, rc, m, st_);
          std::swap(sa, sb);
          rounds++;
        }
      }
      if (tm) tm->commit.end(st_);
      SIFG_CUDA(cudaMemcpyAsync(h_counters_, counters, kCommitCounters * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, st_));
      SIFG_CUDA(cudaMemcpyAsync(h_count, dcount + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
      SIFG_CUDA(cudaStreamSynchronize(st_));
      if (one_launch) {
        if (h_bar[2] || h_bar[3] == 0) {
          set_error(kErrInvalid, "commit: a grid barrier of the cooperative commit timed out");
          return kErrInvalid;
        }
        if (h_bar[3] & 1u) std::swap(sa, sb);
        rounds += h_bar[3];
      }
      if (h_counters_[kRoundUndecided + (rounds - 1) % kRoundRing] == 0) break;
      if (rounds > (uint64_t)m + 8) {
        set_error(kErrInvalid, "commit: no progress");
        return kErrInvalid;
      }
    }
    rs.commit_ms = ms_since(t_commit);
    const uint32_t n_acc = h_counters_[0];
    rs.n_survivors = h_count[0];
    rs.n_accepted = n_acc;
    rs.rounds = rounds;
    rs.n_rescale_fail = h_counters_[4];
    rs.n_overflow = h_counters_[5];
    rs.n_witness = h_counters_[8];
    rs.n_mismatched = h_counters_[9];
    if (n_acc) {
      R rmax;
      std::memcpy(&rmax, sizeof(R) == 4 ? (void*)&h_counters_[3] : (void*)&h_counters_[6], sizeof(R));
      if (rmax > max_r) max_r = rmax;
      ensure_cat(n_voids + n_acc);
      append_accepted(sv, rank, acc, counters, m, blocks2, cat_x_.as<R>(), cat_y_.as<R>(),
                      cat_z_.as<R>(), cat_r_.as<R>(), n_voids, m, st_);
      n_voids += n_acc;
      build_void_index(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), n_voids, box,
                       vstart, vids_.as<uint32_t>(), vcell_.as<uint32_t>(), st_);
    }
    if (tm) tm->rung.end(st_);
    rs.rung_ms = ms_since(t_rung);
    if (stats) stats->push_back(rs);
    if (const int hs = rung_done(ri + 1, rs.n_mismatched); hs != kOk) return hs;
  }

  if (p.consume_out) {
    const R* last = fields[(radii.size() + 1) % 2];
    SIFG_CUDA(cudaMemcpyAsync(p.consume_out, last, cells * sizeof(R), cudaMemcpyDeviceToDevice, st_));
  }
  const size_t base = out.cx.size();
  out.cx.resize(base + n_voids);
  out.cy.resize(base + n_voids);
  out.cz.resize(base + n_voids);
  out.r.resize(base + n_voids);
  // A survey's footprints, once the catalogue is final
  // (sif__exodus_survey_footprint, exodus_survey.c:299-311).
  if (survey) {
    out.foot.resize(base + n_voids);
    out.shell.resize(base + n_voids);
    if (n_voids) {
      R* foot = grow_to<R>(foot_, n_voids);
      R* shell = grow_to<R>(shell_, n_voids);
      survey_footprint(cat_x_.as<R>(), cat_y_.as<R>(), cat_z_.as<R>(), cat_r_.as<R>(), n_voids, occ,
                       N, box, foot, shell, st_);
      SIFG_CUDA(cudaMemcpyAsync(out.foot.data() + base, foot, n_voids * sizeof(R),
                                cudaMemcpyDeviceToHost, st_));
      SIFG_CUDA(cudaMemcpyAsync(out.shell.data() + base, shell, n_voids * sizeof(R),
                                cudaMemcpyDeviceToHost, st_));
    }
  }
  if (n_voids) {
    SIFG_CUDA(cudaMemcpyAsync(out.cx.data() + base, cat_x_.ptr, n_voids * sizeof(R), cudaMemcpyDeviceToHost, st_));
    SIFG_CUDA(cudaMemcpyAsync(out.cy.data() + base, cat_y_.ptr, n_voids * sizeof(R), cudaMemcpyDeviceToHost, st_));
    SIFG_CUDA(cudaMemcpyAsync(out.cz.data() + base, cat_z_.ptr, n_voids * sizeof(R), cudaMemcpyDeviceToHost, st_));
    SIFG_CUDA(cudaMemcpyAsync(out.r.data() + base, cat_r_.ptr, n_voids * sizeof(R), cudaMemcpyDeviceToHost, st_));
  }
  std::vector<uint64_t> h_traffic(2 * n_rungs + 2, 0);
  SIFG_CUDA(cudaMemcpyAsync(h_traffic.data(), traffic, h_traffic.size() * sizeof(uint64_t),
                            cudaMemcpyDeviceToHost, st_));
  SIFG_CUDA(cudaStreamSynchronize(st_));
  for (size_t ri = 0; ri < n_rungs; ri++) {
    if (tm) {
      tm->growth_particles += h_traffic[2 * ri];
      tm->growth_cells += h_traffic[2 * ri + 1];
    }
    // Rung ri's entry: the rungs before first_rung (a resumed run) have none.
    const size_t k = stats0 + (ri - p.first_rung);
    if (stats && ri >= p.first_rung && k < stats->size()) {
      (*stats)[k].growth_particles = h_traffic[2 * ri];
      (*stats)[k].growth_cells = h_traffic[2 * ri + 1];
    }
  }
  if (tm)
    tm->wall_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start)
                       .count();
  return kOk;
}

template int Engine::exodus<float>(const float*, const DeviceMeshT<float>&, const RunParamsT<float>&,
                                  HostCatalogueT<float>&, std::vector<RungStat>*, RunTimings*);
template int Engine::exodus<double>(const double*, const DeviceMeshT<double>&,
                                   const RunParamsT<double>&, HostCatalogueT<double>&,
                                   std::vector<RungStat>*, RunTimings*);

}  // namespace sifg
