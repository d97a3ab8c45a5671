// Shared definitions of the GB300 exodus library: error plumbing, the
// strict single-precision helpers the bit-exact kernels are written with, and
// small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <string>

namespace sifg {

// Kernels this library has launched (every launch site checks itself with
// SIFG_LAUNCH_CHECK, which counts it); read by sifg_launch_count().
extern std::atomic<uint64_t> g_kernel_launches;

// sif's status codes (include/sif/core/macros.h:690-707).
constexpr int kOk = 0;
constexpr int kErrAlloc = -1;
constexpr int kErrInvalid = -2;
constexpr int kErrRange = -3;
constexpr int kErrUnsupported = -5;
constexpr int kErrUninitialised = -6;

// Records a status and message for sif_error_status()/sif_error_message().
void set_error(int status, const std::string& msg);

struct CudaError {
  cudaError_t code;
  const char* where;
};

#define SIFG_CUDA(call)                                                      \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) throw ::sifg::CudaError{e_, #call};               \
  } while (0)

#define SIFG_LAUNCH_CHECK()                                                  \
  do {                                                                       \
    ::sifg::g_kernel_launches.fetch_add(1, std::memory_order_relaxed);       \
    SIFG_CUDA(cudaGetLastError());                                           \
  } while (0)

inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap = 152u * 32u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}

// ---------------------------------------------------------------------------
// Strict IEEE arithmetic in the type the path computes in (float, or double
// for the FP64 form). The reference computes its distances, bins and density
// tests in sif_real with one rounding per operation; the _rn intrinsics are
// never contracted into fused multiply-adds, so these give the same bits as
// the strict CPU build of either precision.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double fsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double fdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double fsqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float ffloor(float a) { return floorf(a); }
__device__ __forceinline__ double ffloor(double a) { return floor(a); }
__device__ __forceinline__ float fabs_(float a) { return fabsf(a); }
__device__ __forceinline__ double fabs_(double a) { return fabs(a); }
__device__ __forceinline__ int32_t to_int_rz(float a) { return __float2int_rz(a); }
__device__ __forceinline__ int32_t to_int_rz(double a) { return __double2int_rz(a); }

// Conversions of counts, rounded to nearest as a C cast rounds them.
template <class R> __device__ __forceinline__ R from_u32(uint32_t v);
template <> __device__ __forceinline__ float from_u32<float>(uint32_t v) { return __uint2float_rn(v); }
template <> __device__ __forceinline__ double from_u32<double>(uint32_t v) { return (double)v; }
template <class R> __device__ __forceinline__ R from_u64(unsigned long long v);
template <> __device__ __forceinline__ float from_u64<float>(unsigned long long v) { return __ull2float_rn(v); }
template <> __device__ __forceinline__ double from_u64<double>(unsigned long long v) { return __ull2double_rn(v); }
template <class R> __device__ __forceinline__ R real_inf();
template <> __device__ __forceinline__ float real_inf<float>() { return __int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double real_inf<double>() { return __longlong_as_double(0x7ff0000000000000ll); }

// dist2 of src/finder/exodus_rescale.c:349-355: ((dx*dx + dy*dy) + dz*dz).
template <class R>
__device__ __forceinline__ R dist2(R px, R py, R pz, R cx, R cy, R cz) {
  const R dx = fsub(px, cx), dy = fsub(py, cy), dz = fsub(pz, cz);
  return fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
}

// bin_of of src/finder/exodus_rescale.c:360-369: truncation toward zero.
template <class R>
__device__ __forceinline__ uint32_t bin_of(R d2, R rc2, R inv_w, uint32_t nb) {
  const int32_t b = to_int_rz(fmul(fsub(d2, rc2), inv_w));
  if (b < 0) return 0;
  if ((uint32_t)b >= nb) return nb - 1;
  return (uint32_t)b;
}

// sif__box_fold, src/structures/field_internal.h:58-64.
template <class R>
__host__ __device__ __forceinline__ R box_fold(R v, R box) {
  if (v >= box)
    v -= box;
  else if (v < 0.0f)
    v += box;
  return v >= box ? R(0) : v;
}

__device__ __forceinline__ uint32_t wrap_pbc(int32_t v, uint32_t n) {
  int32_t w = v % (int32_t)n;
  return (uint32_t)(w < 0 ? w + (int32_t)n : w);
}

__device__ __forceinline__ bool mask_get(const uint32_t* m, uint64_t i) {
  return (__ldg(m + (i >> 5)) >> (i & 31)) & 1u;
}

// The mask is also read with plain loads by kernels that run after writers
// in the same stream; __ldg is only used where the mask is read-only for the
// whole kernel.
// Read past L1: the mask is written (atomicOr) while kernels that read it
// run, by other SMs within one cooperative launch.
__device__ __forceinline__ bool mask_get_rw(const uint32_t* m, uint64_t i) {
  return (__ldcg(m + (i >> 5)) >> (i & 31)) & 1u;
}

}  // namespace sifg
