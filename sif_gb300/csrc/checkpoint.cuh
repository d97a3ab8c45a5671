// Exodus checkpoints (checkpoint.cu): the XCKP v3 file, host side.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/sif_gb300.h"

namespace sifg {

constexpr uint32_t kCrcInit = 0xFFFFFFFFu;
uint32_t crc32_update(uint32_t crc, const void* data, size_t n);
inline uint32_t crc32_final(uint32_t crc) { return crc ^ 0xFFFFFFFFu; }
// CRC-32 of a catalogue's four columns, chained in order.
uint32_t catalogue_crc(const float* cx, const float* cy, const float* cz, const float* r,
                       uint64_t n);

// `exodus-<16 hex digits>.ckpt`, a name no earlier run has used.
std::string checkpoint_default_name();

// Writes atomically: to `<path>.tmp.<pid>`, flushed to the disk, renamed over
// path. The format fields, the void count and the checksum are filled in.
// SIF_OK, or SIF_ERR_IO with *message (and `consequence`, when given,
// appended: the failure is then a warning, not an error).
int checkpoint_write(const std::string& path, sif_finder_exodus_checkpoint_t& header,
                     const float* radii, const float* cx, const float* cy, const float* cz,
                     const float* r, uint64_t n_voids, const char* consequence,
                     std::string* message);

// Reads a whole file: the header (upgraded to this version's option bits),
// the ladder and the four columns. SIF_OK or SIF_ERR_IO with *message.
int checkpoint_load(const std::string& path, sif_finder_exodus_checkpoint_t& header,
                    std::vector<float>& radii, std::vector<float> cols[4], std::string* message);

// Whether a file's header describes the run about to resume it: SIF_OK, or
// SIF_ERR_INVALID with the first difference in *message.
int checkpoint_match(const std::string& path, const sif_finder_exodus_checkpoint_t& want,
                     const float* want_radii, const sif_finder_exodus_checkpoint_t& got,
                     const float* got_radii, std::string* message);

}  // namespace sifg
