// Exodus checkpoints (the XCKP v3 file of include/sif/finder/exodus_finder.h:
// 409-535, written and read by src/finder/exodus_checkpoint.c): host code
// for sif's C API over the GPU run.
//
// What a run carries from one rung to the next is its catalogue: the overlap
// mask, the void index and the largest radius are rebuilt from the voids as
// they are accepted, and every rung smooths from the grid's own transform.
// So the file is the run's parameters (to refuse a resume of another run),
// the ladder, and the voids so far; a resumed run accepts those voids before
// the next rung, as it accepts a prior catalogue, and goes on from there.
//
// Layout, in host byte order: the 192-byte header, the ladder largest first
// (n_radii floats), then the voids as four columns of n_voids floats (every
// x, then y, z, radius). The header's CRC-32 (the IEEE 802.3 reflected
// polynomial 0xEDB88320, initial value and final complement all ones, as
// zlib computes it) covers the header with that field zero, then the ladder
// and the four columns in file order.
#include <errno.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sif_gb300.h"
#include "checkpoint.cuh"

namespace sifg {

static_assert(sizeof(sif_finder_exodus_checkpoint_t) == 192, "the header is 192 bytes");

constexpr uint32_t kByteOrderMark = 0x01020304u;

// The CRC-32 table of the reflected polynomial, built on first use.
static uint32_t g_crc_table[256];
static std::once_flag g_crc_once;

static void crc_table_build() {
  for (uint32_t n = 0; n < 256; n++) {
    uint32_t c = n;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
    g_crc_table[n] = c;
  }
}

uint32_t crc32_update(uint32_t crc, const void* data, size_t n) {
  std::call_once(g_crc_once, crc_table_build);
  const uint8_t* p = (const uint8_t*)data;
  for (size_t i = 0; i < n; i++) crc = g_crc_table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
  return crc;
}

uint32_t catalogue_crc(const float* cx, const float* cy, const float* cz, const float* r,
                       uint64_t n) {
  const size_t bytes = (size_t)n * sizeof(float);
  uint32_t c = kCrcInit;
  c = crc32_update(c, cx, bytes);
  c = crc32_update(c, cy, bytes);
  c = crc32_update(c, cz, bytes);
  c = crc32_update(c, r, bytes);
  return crc32_final(c);
}

static uint32_t file_crc(const sif_finder_exodus_checkpoint_t& header, const float* radii,
                         const float* cx, const float* cy, const float* cz, const float* r) {
  sif_finder_exodus_checkpoint_t h = header;
  h.crc32 = 0;
  const size_t bytes = (size_t)h.n_voids * sizeof(float);
  uint32_t c = kCrcInit;
  c = crc32_update(c, &h, sizeof h);
  c = crc32_update(c, radii, (size_t)h.n_radii * sizeof(float));
  c = crc32_update(c, cx, bytes);
  c = crc32_update(c, cy, bytes);
  c = crc32_update(c, cz, bytes);
  c = crc32_update(c, r, bytes);
  return crc32_final(c);
}

// splitmix64 of a seed from the clock, the process and the kernel's entropy:
// a name no earlier run used, even for two runs started together.
static uint64_t unique_id() {
  struct timespec ts;
  clock_gettime(CLOCK_REALTIME, &ts);
  uint64_t seed = ((uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec) ^
                  ((uint64_t)getpid() << 32);
  if (FILE* u = fopen("/dev/urandom", "rb")) {
    uint64_t noise = 0;
    if (fread(&noise, sizeof noise, 1, u) == 1) seed ^= noise;
    fclose(u);
  }
  uint64_t z = seed + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

std::string checkpoint_default_name() {
  char name[64];
  snprintf(name, sizeof name, "exodus-%016llx.ckpt", (unsigned long long)unique_id());
  return name;
}

int checkpoint_write(const std::string& path, sif_finder_exodus_checkpoint_t& header,
                     const float* radii, const float* cx, const float* cy, const float* cz,
                     const float* r, uint64_t n_voids, const char* consequence,
                     std::string* message) {
  std::memcpy(header.magic, SIF_FINDER_CHECKPOINT_MAGIC, 4);
  header.version = SIF_FINDER_CHECKPOINT_VERSION;
  header.byte_order = kByteOrderMark;
  header.is_double = 0;
  header.n_voids = n_voids;
  std::memset(header.reserved, 0, sizeof header.reserved);
  header.crc32 = file_crc(header, radii, cx, cy, cz, r);
  auto failed = [&](const std::string& what, int err) {
    *message = path + ": " + what + (err ? std::string(": ") + strerror(err) : std::string()) +
               (consequence ? std::string(" (") + consequence + ")" : std::string());
    return SIF_ERR_IO;
  };
  const std::string tmp = path + ".tmp." + std::to_string((long)getpid());
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return failed("cannot create " + tmp, errno);
  const size_t col = (size_t)n_voids;
  bool ok = fwrite(&header, sizeof header, 1, f) == 1 &&
            fwrite(radii, sizeof(float), header.n_radii, f) == header.n_radii &&
            fwrite(cx, sizeof(float), col, f) == col && fwrite(cy, sizeof(float), col, f) == col &&
            fwrite(cz, sizeof(float), col, f) == col && fwrite(r, sizeof(float), col, f) == col;
  int err = ok ? 0 : errno;
  // The bytes on the disk before the rename: otherwise a node that dies just
  // after could leave the name on a file of zeros.
  if (ok && (fflush(f) != 0 || fsync(fileno(f)) != 0)) {
    ok = false;
    err = errno;
  }
  if (fclose(f) != 0 && ok) {
    ok = false;
    err = errno;
  }
  if (!ok) {
    unlink(tmp.c_str());
    return failed("cannot write " + tmp, err);
  }
  if (rename(tmp.c_str(), path.c_str()) != 0) {
    err = errno;
    unlink(tmp.c_str());
    return failed("cannot replace", err);
  }
  return SIF_OK;
}

// sif__finder_checkpoint_upgrade (include/sif/finder/exodus_finder.h:
// 509-531): a version 1 header is CIC, not interlaced; up to version 2
// refinement was bit 10 and only Gaussian, and the minima implied it, the
// extended reach and displacement.
static void upgrade(sif_finder_exodus_checkpoint_t& h) {
  if (h.version < 2) h.assignment = 2;  // SIF_ASSIGNMENT_CIC
  if (h.version < 3) {
    const uint32_t old_refine = 1u << 10;
    if (h.options & old_refine) h.options |= SIF_FINDER_REFINE_GAUSSIAN;
    if (h.options & SIF_FINDER_SEEDS_MINIMA)
      h.options |= SIF_FINDER_REFINE_GAUSSIAN | SIF_FINDER_EXTEND_REACH | SIF_FINDER_DISPLACE;
    h.options &= ~old_refine;
  }
}

int checkpoint_load(const std::string& path, sif_finder_exodus_checkpoint_t& header,
                    std::vector<float>& radii, std::vector<float> cols[4], std::string* message) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    *message = path + ": " + strerror(errno);
    return SIF_ERR_IO;
  }
  struct stat st;
  if (fstat(fileno(f), &st) != 0) {
    *message = path + ": " + strerror(errno);
    fclose(f);
    return SIF_ERR_IO;
  }
  const uint64_t bytes = (uint64_t)st.st_size;
  auto bad = [&](const std::string& what) {
    *message = path + ": " + what;
    fclose(f);
    return SIF_ERR_IO;
  };
  sif_finder_exodus_checkpoint_t h;
  if (fread(&h, sizeof h, 1, f) != 1)
    return bad(std::to_string(bytes) + " bytes, shorter than a checkpoint header (192)");
  if (std::memcmp(h.magic, SIF_FINDER_CHECKPOINT_MAGIC, 4) != 0)
    return bad("not an exodus checkpoint (no XCKP at byte 0)");
  if (h.byte_order != kByteOrderMark) return bad("written on a machine of the other byte order");
  if (h.version == 0 || h.version > SIF_FINDER_CHECKPOINT_VERSION)
    return bad("version " + std::to_string(h.version) + " (expected 1 to 3)");
  if (h.is_double) return bad("FP64 values, this build is FP32");
  if (h.n_radii == 0 || h.next_rung > h.n_radii || h.n_prior > h.n_voids)
    return bad("header: inconsistent counts");
  // Sized against the file before anything is allocated from the header.
  const uint64_t expect = sizeof h + ((uint64_t)h.n_radii + 4ull * h.n_voids) * sizeof(float);
  if (h.n_voids > UINT64_MAX / 64u || bytes != expect)
    return bad(std::to_string(bytes) + " bytes, header says " + std::to_string(expect));
  radii.resize(h.n_radii);
  for (int k = 0; k < 4; k++) cols[k].resize(h.n_voids);
  if (fread(radii.data(), sizeof(float), h.n_radii, f) != h.n_radii) return bad("short read");
  for (int k = 0; k < 4; k++)
    if (fread(cols[k].data(), sizeof(float), h.n_voids, f) != h.n_voids) return bad("short read");
  fclose(f);
  const uint32_t got = file_crc(h, radii.data(), cols[0].data(), cols[1].data(), cols[2].data(),
                                cols[3].data());
  if (got != h.crc32) {
    char b[96];
    snprintf(b, sizeof b, "corrupt: checksum %08x (expected %08x)", got, h.crc32);
    *message = path + ": " + b;
    return SIF_ERR_IO;
  }
  upgrade(h);
  header = h;
  return SIF_OK;
}

// sif__exodus_checkpoint_match (src/finder/exodus_checkpoint.c:330-451): the
// first parameter that differs, or SIF_OK.
int checkpoint_match(const std::string& path, const sif_finder_exodus_checkpoint_t& want,
                     const float* want_radii, const sif_finder_exodus_checkpoint_t& got,
                     const float* got_radii, std::string* message) {
  char b[384];
  auto mismatch = [&](const char* what) {
    *message = path + ": not this run: " + what;
    return SIF_ERR_INVALID;
  };
  if (got.is_survey != want.is_survey)
    return mismatch(got.is_survey ? "saved from a survey (this run is a box)"
                                  : "saved from a box (this run is a survey)");
  if (got.is_weighted != want.is_weighted) return mismatch("tracer weighting differs");
  if (got.n_radii != want.n_radii) {
    snprintf(b, sizeof b, "ladder of %u radii (expected %u)", got.n_radii, want.n_radii);
    return mismatch(b);
  }
  for (uint32_t i = 0; i < want.n_radii; i++)
    if (got_radii[i] != want_radii[i]) {
      snprintf(b, sizeof b, "radius %u of the ladder, largest first: %g (expected %g)", i,
               (double)got_radii[i], (double)want_radii[i]);
      return mismatch(b);
    }
  if (got.threshold != want.threshold) {
    snprintf(b, sizeof b, "threshold %g (expected %g)", got.threshold, want.threshold);
    return mismatch(b);
  }
  if (got.overlap_fraction != want.overlap_fraction) {
    snprintf(b, sizeof b, "overlap fraction %g (expected %g)", got.overlap_fraction,
             want.overlap_fraction);
    return mismatch(b);
  }
  const struct {
    uint32_t bits;
    const char* what;
  } fields[] = {{SIF_FINDER_SEARCH_2_00, "search factor"},
                {SIF_FINDER_KEEP_CIC_WINDOW, "CIC window"},
                {SIF_FINDER_SEEDS_MINIMA | SIF_FINDER_REFINE_HILL, "centres"},
                {SIF_FINDER_EXTEND_REACH, "reach"},
                {SIF_FINDER_DISPLACE, "displacement"},
                {SIF_FINDER_LAGRANGIAN_OVERLAP, "overlap radii"}};
  for (const auto& fl : fields)
    if ((got.options ^ want.options) & fl.bits) return mismatch(fl.what);
  if (got.grid_n_cells != want.grid_n_cells || got.box_length != want.box_length) {
    snprintf(b, sizeof b, "grid of %u cells over %g (expected %u over %g)", got.grid_n_cells,
             got.box_length, want.grid_n_cells, want.box_length);
    return mismatch(b);
  }
  if ((got.options ^ want.options) & SIF_FINDER_ALIASING_WINDOW)
    return mismatch("window deconvolution");
  if (got.assignment != want.assignment) return mismatch("grid assignment scheme");
  // A total weight is a parallel sum whose last bits follow the thread count.
  const double tw = std::fabs(got.total_weight - want.total_weight);
  if (got.n_particles != want.n_particles ||
      tw > 1e-9 * std::fmax(std::fabs(got.total_weight), std::fabs(want.total_weight))) {
    snprintf(b, sizeof b, "%llu tracers of total weight %.17g (expected %llu of %.17g)",
             (unsigned long long)got.n_particles, got.total_weight,
             (unsigned long long)want.n_particles, want.total_weight);
    return mismatch(b);
  }
  if (want.is_survey) {
    const double rw = std::fabs(got.random_total_weight - want.random_total_weight);
    if (got.random_n_particles != want.random_n_particles ||
        rw > 1e-9 * std::fmax(std::fabs(got.random_total_weight),
                              std::fabs(want.random_total_weight))) {
      snprintf(b, sizeof b, "%llu randoms of total weight %.17g (expected %llu of %.17g)",
               (unsigned long long)got.random_n_particles, got.random_total_weight,
               (unsigned long long)want.random_n_particles, want.random_total_weight);
      return mismatch(b);
    }
    for (int k = 0; k < 3; k++)
      if (got.offset[k] != want.offset[k]) {
        snprintf(b, sizeof b, "offset[%d] %g (expected %g)", k, got.offset[k], want.offset[k]);
        return mismatch(b);
      }
  }
  if (got.n_prior != want.n_prior || got.prior_crc32 != want.prior_crc32) {
    snprintf(b, sizeof b, "started from %llu prior voids, checksum %08x (this run's: %llu, %08x)",
             (unsigned long long)got.n_prior, got.prior_crc32, (unsigned long long)want.n_prior,
             want.prior_crc32);
    return mismatch(b);
  }
  return SIF_OK;
}

}  // namespace sifg
