// The per-rung smoothing: cuFFT R2C of the density contrast once, then per
// radius one fused filter kernel and a cuFFT C2R -- or, for the float form on
// a 512^3 grid, three passes of its own that fuse the filter into the first
// (below).
//
// Replaces sif__fft_grid_forward, fft_build_filter_lut,
// sif__fft_apply_filter_smoothed and sif__fft_grid_backward
// (src/math/fft.c:790-818, 521-568, 703-788, 820-888) and the window setup of
// sif__finder_deconvolve_window (src/finder/utils.c:75-110,
// src/math/fft.c:958-1046). cuFFT stands in for FFTW's planes and pencils.
//
// The filter kernel multiplies each mode by W(k R) (top-hat
// 3(sin x - x cos x)/x^3, or Gaussian exp(-x^2/2)), by the CIC window
// correction 1/sinc^2 per axis (or the aliasing-aware W/S), and by the C2R's
// 1/N^3, reading the spectrum once and writing the transform's input once.
// The radial factor comes from a table indexed by the integer |k|^2, built in
// double by a small kernel, as the reference tabulates it (the own inverse at
// 512 evaluates the same formulas in float as it applies them). The unfiltered
// pass (the grid handed back at the end of a run) applies no window, as the
// reference's SIF__FILTER_NONE copies the spectrum untouched.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "smooth.cuh"

namespace sifg {

#define SIFG_CUFFT(call)                                                        \
  do {                                                                          \
    cufftResult r_ = (call);                                                    \
    if (r_ != CUFFT_SUCCESS) throw ::sifg::CudaError{cudaErrorUnknown, #call};  \
  } while (0)

__device__ __forceinline__ float filter_factor(uint32_t ix, uint32_t iy, uint32_t iz, uint32_t n,
                                               const float* __restrict__ lut,
                                               const float* __restrict__ win, float norm) {
  const uint32_t h = n >> 1;
  const int32_t kx = ix > h ? (int32_t)ix - (int32_t)n : (int32_t)ix;
  const int32_t ky = iy > h ? (int32_t)iy - (int32_t)n : (int32_t)iy;
  const uint32_t k2 = (uint32_t)(kx * kx + ky * ky) + iz * iz;
  float s = __ldg(lut + k2) * norm;
  if (win) s = s * __ldg(win + ix) * __ldg(win + iy) * __ldg(win + iz);
  return s;
}

// Two modes per 16-byte load and store (an odd grid's last mode on its own),
// four loads in flight per thread before any is used: the kernel is bound by
// the latency of its loads. Index is 32-bit whenever the count allows.
template <class Index>
__device__ __forceinline__ float4 filter_pair(float4 v, Index j, uint32_t n, uint32_t zd,
                                              const float* __restrict__ lut,
                                              const float* __restrict__ win, float norm) {
  const Index i = 2 * j;
  const Index row = i / zd;
  const uint32_t iz = (uint32_t)(i - row * zd);
  const uint32_t iy = (uint32_t)(row % n), ix = (uint32_t)(row / n);
  const float s0 = filter_factor(ix, iy, iz, n, lut, win, norm);
  float s1;
  if (iz + 1 < zd) {
    s1 = filter_factor(ix, iy, iz + 1, n, lut, win, norm);
  } else {
    const uint32_t iy1 = iy + 1 == n ? 0u : iy + 1;
    s1 = filter_factor(iy1 == 0 ? ix + 1 : ix, iy1, 0, n, lut, win, norm);
  }
  return make_float4(v.x * s0, v.y * s0, v.z * s1, v.w * s1);
}

constexpr int kFilterUnroll = 4;

template <class Index>
__global__ void __launch_bounds__(256) filter_kernel(const float4* __restrict__ spec,
                                                     float4* __restrict__ out, uint32_t n,
                                                     const float* __restrict__ lut,
                                                     const float* __restrict__ win, float norm) {
  const uint32_t zd = n / 2 + 1;
  const Index pairs = (Index)n * n * zd / 2;
  const Index stride = (Index)gridDim.x * blockDim.x;
  for (Index j0 = (Index)blockIdx.x * blockDim.x + threadIdx.x; j0 < pairs;
       j0 += kFilterUnroll * stride) {
    float4 v[kFilterUnroll];
#pragma unroll
    for (int u = 0; u < kFilterUnroll; u++) {
      const Index j = j0 + u * stride;
      if (j < pairs) v[u] = __ldg(spec + j);
    }
#pragma unroll
    for (int u = 0; u < kFilterUnroll; u++) {
      const Index j = j0 + u * stride;
      if (j < pairs) out[j] = filter_pair(v[u], j, n, zd, lut, win, norm);
    }
  }
  const Index total = (Index)n * n * zd;
  if ((total & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const float s = filter_factor(n - 1, n - 1, zd - 1, n, lut, win, norm);
    const float2 v = ((const float2*)spec)[total - 1];
    ((float2*)out)[total - 1] = make_float2(v.x * s, v.y * s);
  }
}

// The FP64 form's filter: one mode per 16-byte load, four in flight.
__global__ void __launch_bounds__(256) filter_kernel_f64(const double2* __restrict__ spec,
                                                         double2* __restrict__ out, uint32_t n,
                                                         const double* __restrict__ lut,
                                                         const double* __restrict__ win,
                                                         double norm) {
  const uint32_t zd = n / 2 + 1, h = n >> 1;
  const uint64_t total = (uint64_t)n * n * zd;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < total;
       i0 += kFilterUnroll * stride) {
    double2 v[kFilterUnroll];
#pragma unroll
    for (int u = 0; u < kFilterUnroll; u++)
      if (i0 + u * stride < total) v[u] = __ldg(spec + i0 + u * stride);
#pragma unroll
    for (int u = 0; u < kFilterUnroll; u++) {
      const uint64_t i = i0 + u * stride;
      if (i >= total) continue;
      const uint64_t row = i / zd;
      const uint32_t iz = (uint32_t)(i - row * zd);
      const uint32_t iy = (uint32_t)(row % n), ix = (uint32_t)(row / n);
      const int32_t kx = ix > h ? (int32_t)ix - (int32_t)n : (int32_t)ix;
      const int32_t ky = iy > h ? (int32_t)iy - (int32_t)n : (int32_t)iy;
      const uint32_t k2 = (uint32_t)(kx * kx + ky * ky) + iz * iz;
      double s = __ldg(lut + k2) * norm;
      if (win) s = s * __ldg(win + ix) * __ldg(win + iy) * __ldg(win + iz);
      out[i] = make_double2(v[u].x * s, v[u].y * s);
    }
  }
}

// ---------------------------------------------------------------------------
// The float form's inverse transform at n = 512, in three passes of its own
// in place of the filter kernel and cuFFT's C2R:
//   (1) filter + inverse FFT along kx (spectrum -> work),
//   (2) inverse FFT along ky (work, in place),
//   (3) C2R along kz (work -> the real grid).
// A 512-point transform belongs to one warp, 16 values per lane: a 16-point
// DFT in registers over the lane's stride-32 values, a twiddle, an exchange
// through shared memory, a second 16-point DFT and a radix-2 step between
// lane pairs by shuffles (512 = 16 x 32, 32 = 16 x 2). Passes (1) and (2)
// give a CTA 16 neighbouring kz columns of one line (128 contiguous bytes
// per row of the line); pass (3) gives each 257-mode kz row to a half-warp
// as a 256-point complex transform of the packed even and odd samples.
// Twiddles come from tables computed in double; the three passes read and
// write the transform's data once each.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul_i(float2 a) { return make_float2(-a.y, a.x); }  // a * i

// Asynchronous global -> shared copies (LDGSTS): a CTA's whole tile is in
// flight at once, with no registers held for it.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// e^{+2 pi i k/32}, k < 16, rounded to float.
__constant__ float2 kW32[16] = {
    {1.0f, 0.0f},
    {0.9807852506637573f, 0.19509032368659973f},
    {0.9238795042037964f, 0.3826834261417389f},
    {0.8314695954322815f, 0.5555702447891235f},
    {0.7071067690849304f, 0.7071067690849304f},
    {0.5555702447891235f, 0.8314695954322815f},
    {0.3826834261417389f, 0.9238795042037964f},
    {0.19509032368659973f, 0.9807852506637573f},
    {0.0f, 1.0f},
    {-0.19509032368659973f, 0.9807852506637573f},
    {-0.3826834261417389f, 0.9238795042037964f},
    {-0.5555702447891235f, 0.8314695954322815f},
    {-0.7071067690849304f, 0.7071067690849304f},
    {-0.8314695954322815f, 0.5555702447891235f},
    {-0.9238795042037964f, 0.3826834261417389f},
    {-0.9807852506637573f, 0.19509032368659973f},
};

// Inverse (e^{+2 pi i jk/R}) DFTs of 4, 8 and 16 points, in place, natural order.
__device__ __forceinline__ void dft_inv(float2 (&v)[4]) {
  const float2 c0 = cadd(v[0], v[2]), c2 = csub(v[0], v[2]);
  const float2 c1 = cadd(v[1], v[3]), d = cmul_i(csub(v[1], v[3]));
  v[0] = cadd(c0, c1);
  v[2] = csub(c0, c1);
  v[1] = cadd(c2, d);
  v[3] = csub(c2, d);
}
__device__ __forceinline__ void dft_inv(float2 (&v)[8]) {
  const float h = 0.70710678118654752440f;  // cos(pi/4)
  float2 a[4], b[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    a[j] = cadd(v[j], v[j + 4]);
    b[j] = csub(v[j], v[j + 4]);
  }
  // b[j] *= w^j, w = e^{+i pi/4}
  b[1] = make_float2(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y));
  b[2] = cmul_i(b[2]);
  b[3] = make_float2(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));
  dft_inv(a);
  dft_inv(b);
#pragma unroll
  for (int m = 0; m < 4; m++) {
    v[2 * m] = a[m];
    v[2 * m + 1] = b[m];
  }
}
__device__ __forceinline__ void dft_inv(float2 (&v)[16]) {
  float2 e[8], o[8];
#pragma unroll
  for (int m = 0; m < 8; m++) {
    e[m] = v[2 * m];
    o[m] = v[2 * m + 1];
  }
  dft_inv(e);
  dft_inv(o);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    float2 t;
    if (k == 0)
      t = o[0];
    else if (k == 4)
      t = cmul_i(o[4]);
    else
      t = cmul(o[k], kW32[2 * k]);
    v[k] = cadd(e[k], t);
    v[k + 8] = csub(e[k], t);
  }
}

// A column of 512 in shared memory: element i at col_slot(i), columns
// kColStride slots apart (odd). The stage-to-stage exchange uses rows of
// kColSpan slots. With these, every shared access of the transform, and the
// 16-column row loads and stores, is free of bank conflicts.
__host__ __device__ constexpr int col_slot(int i) { return i + (i >> 4) + 8 * (i >> 8); }
constexpr int kColCols = 16;
constexpr int kColWarps = 8;  // each warp transforms kColCols / kColWarps columns
constexpr int kColSpan = 34;
constexpr int kColStride = 551;
static_assert(kColStride > col_slot(511) && kColStride >= 16 * kColSpan && (kColStride & 1),
              "column layout");

// Twiddle tables of the n = 512 transform, one device block:
//   [0, 512):    W512^(j k), at k * 32 + j (j < 32, k < 16), the column pass
//   [512, 768):  W256^(j k), at k * 16 + j (j, k < 16), the row pass
//   [768, 1024): W512^k, k < 256, the row pass's even/odd packing
constexpr int kTw512 = 1024;

// The filter of one kx column at (ky, kz): mode kx is scaled by
// lut[k^2] * norm * win[kx] * win[ky] * win[kz] (win optional), the factor
// and the order of its products as the per-mode filter kernel has them.
// The radial factor of the filter pass, evaluated where it is applied: a
// table by |k|^2 (as the other grids use) is a gather whose lanes fall in as
// many cache lines, and it doubled the pass's time. These are the table's
// formulas (fft_build_filter_lut, src/math/fft.c:521-568) in float: the
// top-hat 3 (sin x - x cos x) / x^3 by its Taylor series below x = 2, where
// the formula cancels, and through sin and cos above; the Gaussian
// exp(-x^2 / 2); the extra Gaussian of sigma on top of either. Above x = 2
// the phase x = f |k| carries its rounding error as a second float (f's low
// part, the square root's residual, the product's error by fma): a float x
// alone is off by up to x ulp, as much as 4e-6 in the factor at x = 70. sin
// and cos of that pair come from a reduction by pi/2 (Cody and Waite: pi/2 in
// three parts, the first two of 12 significant bits so that n times them is
// exact, the pair's low part added to the remainder) and Taylor series on
// [-pi/4, pi/4] (to x^9 and x^10: the first term left out is below 2e-10);
// within 1.5 ulp. The factor is then within about 4 ulp of the table's
// double value (2e-7 rms relative over the modes above x = 2).
struct RadialFilter {
  int kind;         // kFilterTopHat, kFilterGaussian, else 1
  float x2;         // x^2 per unit |k|^2: f^2, f = R 2 pi / L
  float g2;         // the extra Gaussian's exponent per unit |k|^2: (sigma 2 pi / L)^2 / 2; 0 for none
  float f, f_lo;    // f as a float and its remainder
};

// sin and cos of x + x_lo (|x_lo| below an ulp of x, 0 < x < 4096 pi / 2).
__device__ __forceinline__ void sincos_pair(float x, float x_lo, float& s, float& c) {
  constexpr float kP1 = 1.57080078125f;             // pi/2 to 12 bits
  constexpr float kP2 = -4.4535845518112183e-06f;   // the remainder to 12 bits
  constexpr float kP3 = (float)(1.57079632679489661923 - 1.57080078125 + 4.4535845518112183e-06);
  const float n = rintf(x * (float)(2.0 / 3.14159265358979323846));
  float r = fmaf(-n, kP1, x);  // exact: n kP1 has 24 bits and lies within a factor 2 of x
  r = fmaf(-n, kP2, r);
  r = fmaf(-n, kP3, r) + x_lo;
  const float r2 = r * r;
  float ps = (float)(1.0 / 362880.0);
  ps = fmaf(ps, r2, (float)(-1.0 / 5040.0));
  ps = fmaf(ps, r2, (float)(1.0 / 120.0));
  ps = fmaf(ps, r2, (float)(-1.0 / 6.0));
  const float sr = fmaf(ps * r2, r, r);
  float pc = (float)(-1.0 / 3628800.0);
  pc = fmaf(pc, r2, (float)(1.0 / 40320.0));
  pc = fmaf(pc, r2, (float)(-1.0 / 720.0));
  pc = fmaf(pc, r2, (float)(1.0 / 24.0));
  pc = fmaf(pc, r2, -0.5f);
  const float cr = fmaf(pc, r2, 1.0f);
  // x = n pi/2 + r: quadrant q of n turns (sin r, cos r) by q quarter turns.
  const int q = (int)n & 3;
  s = (q & 1) ? cr : sr;
  c = (q & 1) ? sr : cr;
  if (q & 2) s = -s;
  if ((q + 1) & 2) c = -c;
}

// The series sum_{n >= 1} (-1)^(n+1) 6n x^(2n-2) / (2n+1)! of the top-hat,
// through n = 8: the first term left out is below 3e-11 for x < 2.
__device__ __forceinline__ float tophat_series(float x2) {
  float p = (float)(-48.0 / 355687428096000.0);
  p = fmaf(p, x2, (float)(42.0 / 1307674368000.0));
  p = fmaf(p, x2, (float)(-36.0 / 6227020800.0));
  p = fmaf(p, x2, (float)(30.0 / 39916800.0));
  p = fmaf(p, x2, (float)(-24.0 / 362880.0));
  p = fmaf(p, x2, (float)(18.0 / 5040.0));
  p = fmaf(p, x2, (float)(-12.0 / 120.0));
  return fmaf(p, x2, 1.0f);
}

__device__ __forceinline__ float radial_factor(uint32_t k2, const RadialFilter& rf) {
  if (k2 == 0) return 1.0f;
  const float kk = (float)k2;  // exact: k2 <= 3 * 256^2
  float v = 1.0f;
  if (rf.kind == kFilterTopHat) {
    const float x2 = rf.x2 * kk;
    if (x2 < 4.0f) {
      v = tophat_series(x2);
    } else {
      // |k| as k + k_lo: a reciprocal square root, and the residual's
      // first-order correction (exact to well below an ulp whatever the
      // reciprocal's own error).
      const float y = rsqrtf(kk);
      const float k = kk * y;
      const float k_lo = fmaf(-k, k, kk) * (0.5f * y);
      const float x = rf.f * k;
      const float x_lo = fmaf(rf.f, k, -x) + fmaf(rf.f, k_lo, rf.f_lo * k);
      float s, c;
      sincos_pair(x, x_lo, s, c);
      v = 3.0f * fmaf(-x, c, s) * __frcp_rn(x2 * x);
    }
  } else if (rf.kind == kFilterGaussian) {
    v = expf(-0.5f * (rf.x2 * kk));
  }
  if (rf.g2 > 0.0f) v *= expf(-(rf.g2 * kk));
  return v;
}

constexpr RadialFilter kNoFilter{-1, 0.0f, 0.0f, 0.0f, 0.0f};  // a pass that applies no filter

struct ColumnFilter {
  bool on;
  RadialFilter rf;
  const float* win;
  float norm, wy, wz;
  uint32_t q;  // ky'^2 + kz^2
  const float* tab;  // the column's factors by |kx| (257), or NULL: evaluate them
};

// The factor table of a smoothing at n = 512: entry ((|ky| * 257 + kz) * 257
// + |kx|) holds the factor the filter pass applies to mode (kx, ky, kz) --
// radial_factor(k^2) * norm, then the window's three factors, in the order
// and with the values ifft512_column computes them, so the table changes no
// bit of the transform.
constexpr uint32_t kFactorSide = 257;
__global__ void factor_table_kernel(float* __restrict__ tab, RadialFilter rf,
                                    const float* __restrict__ win, float norm) {
  constexpr uint64_t total = (uint64_t)kFactorSide * kFactorSide * kFactorSide;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t kx = (uint32_t)(i % kFactorSide);
    const uint32_t kz = (uint32_t)((i / kFactorSide) % kFactorSide);
    const uint32_t ky = (uint32_t)(i / ((uint64_t)kFactorSide * kFactorSide));
    float v = radial_factor(kx * kx + (ky * ky + kz * kz), rf) * norm;
    if (win) v = v * __ldg(win + kx) * __ldg(win + ky) * __ldg(win + kz);
    tab[i] = v;
  }
}

// One warp's inverse DFT of the 512 values in `col`, in place; with a filter
// (f.on) each value is first scaled by its filter factor.
// With `forward` the forward DFT instead (e^{-2 pi i jk/512}), as the
// conjugate of the inverse DFT of the conjugate.
__device__ __forceinline__ void ifft512_column(float2* col, const float2* __restrict__ tw,
                                               unsigned lane, const ColumnFilter& f,
                                               bool forward) {
  float2 v[16];
#pragma unroll
  for (int r = 0; r < 16; r++) {
    v[r] = col[col_slot((int)lane + 32 * r)];
    if (forward) v[r].y = -v[r].y;
  }
  if (f.on) {
    // The factor is even in kx (the window table is built from |k|): a lane
    // finds it for its kx < 256 and takes kx > 256 from the lane holding
    // 512 - kx, half the evaluations. Lane 0 holds both kx = 32 r and
    // 512 - 32 r itself, and alone finds kx = 256.
    float lo[8];
    float nyq = 0.f;
    if (f.tab) {
#pragma unroll
      for (int r = 0; r < 8; r++) lo[r] = __ldg(f.tab + lane + 32u * r);
      if (lane == 0) nyq = __ldg(f.tab + 256);
    } else {
#pragma unroll
      for (int r = 0; r < 8; r++) {
        const uint32_t kx = lane + 32u * r;
        lo[r] = radial_factor(kx * kx + f.q, f.rf) * f.norm;
        if (f.win) lo[r] = lo[r] * __ldg(f.win + kx) * f.wy * f.wz;
      }
      if (lane == 0) {
        nyq = radial_factor(256u * 256u + f.q, f.rf) * f.norm;
        if (f.win) nyq = nyq * __ldg(f.win + 256) * f.wy * f.wz;
      }
    }
    const unsigned partner = (32u - lane) & 31u;
#pragma unroll
    for (int r = 0; r < 16; r++) {
      float s;
      if (r < 8) {
        s = lo[r];
      } else {
        s = __shfl_sync(0xffffffffu, lo[15 - r], partner);
        if (lane == 0) s = r == 8 ? nyq : lo[(16 - r) & 7];
      }
      v[r] = make_float2(v[r].x * s, v[r].y * s);
    }
  }
  dft_inv(v);
#pragma unroll
  for (int k = 1; k < 16; k++) v[k] = cmul(v[k], __ldg(tw + k * 32 + lane));
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; k++) col[kColSpan * k + lane] = v[k];
  __syncwarp();
  const unsigned k1 = lane >> 1, q = lane & 1u;
#pragma unroll
  for (int m = 0; m < 16; m++) v[m] = col[kColSpan * k1 + q + 2 * m];
  dft_inv(v);  // E_q[k], k < 16
  // The radix-2 step between the pair: X[k1 + 16 k] = E_0[k] + W32^k E_1[k],
  // X[k1 + 16 (k + 16)] = E_0[k] - W32^k E_1[k]. Lane q = 0 finishes k < 8,
  // lane q = 1 k >= 8; each sends the half of its E it does not keep, and
  // W32^(8 + i) = i W32^i leaves one twiddle per register for both lanes.
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const float2 send = q ? v[i] : v[8 + i];
    const float2 got = make_float2(__shfl_xor_sync(0xffffffffu, send.x, 1),
                                   __shfl_xor_sync(0xffffffffu, send.y, 1));
    const float2 a = q ? got : v[i];          // E_0[8 q + i]
    const float2 b = q ? cmul_i(v[8 + i]) : got;  // E_1[8 q + i] (times i for q = 1)
    const float2 t = i == 0 ? b : cmul(b, kW32[i]);
    v[i] = cadd(a, t);
    v[8 + i] = csub(a, t);
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int x = (int)k1 + 16 * (8 * (int)q + i);
    col[col_slot(x)] = forward ? make_float2(v[i].x, -v[i].y) : v[i];
    col[col_slot(x + 256)] = forward ? make_float2(v[8 + i].x, -v[8 + i].y) : v[8 + i];
  }
  __syncwarp();
}

// The work buffer between the passes holds the half spectrum in tiles of 16
// kz columns by 512: tile (x, kb) holds kz = 16 kb .. 16 kb + 15 for every
// ky, at ((x * kKzBlocks + kb) * 512 + ky) * 16 + kz % 16. Pass (2) reads
// and writes each tile as one contiguous 64 KB block, pass (3) reads each
// row's modes as 16-row, 2 KB blocks. kz past 256 are never written or read.
constexpr uint32_t kKzBlocks = 17;
constexpr size_t kTileWorkElems = (size_t)512 * kKzBlocks * 512 * 16;

// Where passes (1) and (2) find their columns: line `blockIdx.y`, kz block
// `blockIdx.x`; element a of the block's column c at
// line * line + kb * kblock + a * elem + c.
struct ColumnLayout {
  uint32_t line, kblock, elem;
};

// Passes (1) and (2): the inverse FFT along one axis of 16 neighbouring kz
// columns of one line. The tile arrives by asynchronous copies; pass (1)
// (rf.kind >= 0) reads the spectrum (line = ky, kx along the column), scales each
// mode by its filter factor as the transform first reads it, and writes the
// tiles; pass (2) (line = x, ky along the column) works on the tiles in
// place. Columns past kz = 256 (in the last CTA of a line) are neither read,
// transformed nor written.
__global__ void __launch_bounds__(32 * kColWarps, 3)
    colfft512_kernel(const float2* src, float2* dst, ColumnLayout in, ColumnLayout out,
                     RadialFilter rf, const float* __restrict__ win, float norm,
                     const float2* __restrict__ tw, bool forward,
                     const float* __restrict__ ftab = nullptr) {
  extern __shared__ float2 cols[];  // kColCols columns of kColStride slots
  constexpr uint32_t zd = 257;
  constexpr uint32_t kRowStep = 32 * kColWarps / kColCols;  // rows a pass of the CTA covers
  const uint32_t kb = blockIdx.x, kz0 = kb * kColCols, line = blockIdx.y;
  const uint32_t c = threadIdx.x % kColCols, row0 = threadIdx.x / kColCols;
  const bool live = kz0 + c < zd;
  if (live) {
    const float2* p = src + (size_t)line * in.line + (size_t)kb * in.kblock + c +
                      (size_t)row0 * in.elem;
    const size_t step = (size_t)kRowStep * in.elem;
#pragma unroll 8
    for (uint32_t i = 0; i < 512 / kRowStep; i++, p += step)
      cp_async8(cols + c * kColStride + col_slot((int)(row0 + kRowStep * i)), p);
  }
  cp_async_wait_all();
  __syncthreads();
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
#pragma unroll 1
  for (uint32_t w = warp; w < kColCols && kz0 + w < zd; w += kColWarps) {
    ColumnFilter f{};
    if (rf.kind >= 0) {
      const uint32_t kz = kz0 + w;
      const int32_t ks = line > 256 ? (int32_t)line - 512 : (int32_t)line;
      const uint32_t aky = (uint32_t)(ks < 0 ? -ks : ks);
      f = ColumnFilter{true, rf, win, norm, win ? __ldg(win + line) : 1.f,
                       win ? __ldg(win + kz) : 1.f, (uint32_t)(ks * ks) + kz * kz,
                       ftab ? ftab + ((size_t)aky * kFactorSide + kz) * kFactorSide : nullptr};
    }
    ifft512_column(cols + w * kColStride, tw, lane, f, forward);
  }
  __syncthreads();
  if (live) {
    float2* p = dst + (size_t)line * out.line + (size_t)kb * out.kblock + c +
                (size_t)row0 * out.elem;
    const size_t step = (size_t)kRowStep * out.elem;
#pragma unroll 8
    for (uint32_t i = 0; i < 512 / kRowStep; i++, p += step)
      *p = cols[c * kColStride + col_slot((int)(row0 + kRowStep * i))];
  }
}

// Pass (3): 16 rows of 257 modes per CTA, a half-warp per row. With Z the
// row's modes (the imaginary parts of Z[0] and Z[256] taken as zero, as a
// C2R does), c[k] = Fe[k] + i Fo[k] for k < 256, Fe = Z[k] + conj Z[256-k],
// Fo = (Z[k] - conj Z[256-k]) W512^k, and its 256-point inverse DFT y gives
// the real samples x[2m] = Re y[m], x[2m+1] = Im y[m]. The CTA's 16 rows
// (x, y0 .. y0 + 15) come from the tiles in 16 contiguous 2 KB blocks (kz <
// 256, by 16-byte asynchronous copies) and one mode each for kz = 256; a row
// has kRowSlots slots in shared memory (even, for the 16-byte copies); the
// stage exchange swizzles slots (k1, j) -> 16 k1 + (j ^ k1) within the row.
//
// With `below` set the pass also lists, in flat order, the cells it writes
// whose value is at most below.thr: the CTA's 8192 cells are one contiguous
// flat range, and their entries go to the start of the CTA's own region of
// 8192 slots, their number to below.counts[CTA] (the candidate scan's
// threshold test, from the values in hand).
constexpr int kRowsPerCta = 16;
constexpr uint32_t kRowSlots = 258;
static_assert(kRowsPerCta * 512 == kBelowBlock, "a CTA's cells are one below-list block");
__global__ void __launch_bounds__(16 * kRowsPerCta, 4)
    c2r512_rows_kernel(const float2* __restrict__ work, float* __restrict__ out,
                       const float2* __restrict__ tw, BelowList below) {
  __shared__ __align__(16) float2 buf[kRowsPerCta * kRowSlots];
  const uint32_t x = blockIdx.x / (512 / kRowsPerCta);
  const uint32_t y0 = (blockIdx.x % (512 / kRowsPerCta)) * kRowsPerCta;
  const float2* tiles = work + ((size_t)x * kKzBlocks * 512 + y0) * 16;  // kz block 0
  constexpr size_t kBlock = (size_t)512 * 16;                            // one kz block further
  for (uint32_t f = threadIdx.x; f < 16 * kRowsPerCta * 8; f += blockDim.x) {
    const uint32_t kb = f / (kRowsPerCta * 8), e = f % (kRowsPerCta * 8);
    const uint32_t r = e / 8, jj = e % 8;
    cp_async16(buf + r * kRowSlots + 16 * kb + 2 * jj,
               reinterpret_cast<const float4*>(tiles + kb * kBlock) + e);
  }
  if (threadIdx.x < kRowsPerCta)
    cp_async8(buf + threadIdx.x * kRowSlots + 256, tiles + 16 * kBlock + threadIdx.x * 16);
  cp_async_wait_all();
  __syncthreads();
  const unsigned j = threadIdx.x & 15u;
  float2* row = buf + (threadIdx.x >> 4) * kRowSlots;
  const float2* twb = tw + 512;
  const float2* wpre = tw + 768;
  float2 v[16];
#pragma unroll
  for (int r = 0; r < 16; r++) {
    const unsigned k = j + 16u * r;
    float2 z = row[k], zc = row[256 - k];
    if (r == 0 && j == 0) z.y = zc.y = 0.f;
    zc.y = -zc.y;
    const float2 fe = cadd(z, zc), fo = cmul(csub(z, zc), __ldg(wpre + k));
    v[r] = make_float2(fe.x - fo.y, fe.y + fo.x);
  }
  dft_inv(v);
#pragma unroll
  for (int k = 1; k < 16; k++) v[k] = cmul(v[k], __ldg(twb + k * 16 + j));
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; k++) row[16 * k + (j ^ k)] = v[k];
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 16; m++) v[m] = row[16 * j + (m ^ j)];
  dft_inv(v);
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; k++) row[j + 16 * k] = v[k];
  __syncthreads();
  float2* dst = reinterpret_cast<float2*>(out + ((size_t)x * 512 + y0) * 512);
  if (!below.counts) {
    for (uint32_t f = threadIdx.x; f < kRowsPerCta * 256; f += blockDim.x)
      dst[f] = buf[(f >> 8) * kRowSlots + (f & 255u)];
    return;
  }
  // Each warp takes 512 consecutive pairs (two rows), 32 at a time: it writes
  // them out and keeps its lanes' threshold bits (two per pair) in `bits`;
  // the warps' totals place each warp's entries, and a second walk over the
  // pairs with set bits writes the entries in flat order.
  constexpr uint32_t kWarps = 16 * kRowsPerCta / 32;
  constexpr uint32_t kWarpPairs = kRowsPerCta * 256 / kWarps;
  static_assert(kWarpPairs == 32 * 16, "16 pairs a lane, two bits each in one word");
  __shared__ uint32_t ws[kWarps];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t base = warp * kWarpPairs;
  uint32_t bits = 0;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const uint32_t f = base + 32u * i + lane;
    const float2 v = buf[(f >> 8) * kRowSlots + (f & 255u)];
    if (below.field) dst[f] = v;
    bits |= ((v.x <= below.thr ? 1u : 0u) | (v.y <= below.thr ? 2u : 0u)) << (2 * i);
  }
  const uint32_t n_warp = __reduce_add_sync(0xffffffffu, (unsigned)__popc(bits));
  if (lane == 0) ws[warp] = n_warp;
  __syncthreads();
  uint32_t pos = 0, total = 0;
#pragma unroll
  for (uint32_t w = 0; w < kWarps; w++) {
    pos += w < warp ? ws[w] : 0u;
    total += ws[w];
  }
  if (threadIdx.x == 0) below.counts[blockIdx.x] = total;
  if (n_warp == 0) return;
  const uint32_t cell0 = (x * 512 + y0) * 512;
  const size_t region = (size_t)blockIdx.x * (kRowsPerCta * 512);
  const uint32_t lower = (1u << lane) - 1u;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const uint32_t b = (bits >> (2 * i)) & 3u;
    const uint32_t mx = __ballot_sync(0xffffffffu, b & 1u), my = __ballot_sync(0xffffffffu, b & 2u);
    if ((mx | my) == 0u) continue;
    if (b) {
      const uint32_t f = base + 32u * i + lane;
      const float2 v = buf[(f >> 8) * kRowSlots + (f & 255u)];
      uint32_t p = pos + __popc(mx & lower) + __popc(my & lower);
      if (b & 1u) {
        below.delta[region + p] = v.x;
        below.flat[region + p] = cell0 + 2 * f;
        p++;
      }
      if (b & 2u) {
        below.delta[region + p] = v.y;
        below.flat[region + p] = cell0 + 2 * f + 1;
      }
    }
    pos += __popc(mx) + __popc(my);
  }
}

// The forward transform's first pass, the R2C along z: 16 rows of 512 reals
// per CTA (one contiguous 32 KB block), a half-warp per row. The row read
// as 256 complex values c[m] = x[2m] + i x[2m+1] is transformed forward (the
// conjugate of the inverse of the conjugate); then, with C[-k] taken mod 256,
// E[k] = (C[k] + conj C[-k]) / 2, O[k] = (C[k] - conj C[-k]) / 2i and
// X[k] = E[k] + W512^-k O[k] for k < 256, X[256] = E[0] - O[0]. The 257 modes
// go to the tiles (16 rows by 16 kz, 2 KB blocks).
__global__ void __launch_bounds__(16 * kRowsPerCta, 4)
    r2c512_rows_kernel(const float* __restrict__ grid, float2* __restrict__ work,
                       const float2* __restrict__ tw, const double* __restrict__ mean) {
  __shared__ __align__(16) float2 buf[kRowsPerCta * kRowSlots];
  const uint32_t x = blockIdx.x / (512 / kRowsPerCta);
  const uint32_t y0 = (blockIdx.x % (512 / kRowsPerCta)) * kRowsPerCta;
  const float4* src = reinterpret_cast<const float4*>(grid + ((size_t)x * 512 + y0) * 512);
  for (uint32_t f = threadIdx.x; f < kRowsPerCta * 128; f += blockDim.x)
    cp_async16(buf + (f >> 7) * kRowSlots + 2 * (f & 127u), src + f);
  // With the mean, the rows are the density: its contrast, as the contrast
  // kernel computes it (inv rounded from the double 1 / mean), the double
  // division done once for the CTA while its copies land.
  __shared__ float inv_s;
  if (mean && threadIdx.x == 0) inv_s = (float)(1.0 / __ldg(mean));
  cp_async_wait_all();
  __syncthreads();
  const unsigned j = threadIdx.x & 15u;
  float2* row = buf + (threadIdx.x >> 4) * kRowSlots;
  const float2* twb = tw + 512;
  const float2* wpre = tw + 768;
  float2 v[16];
  const float inv = mean ? inv_s : 0.f;
#pragma unroll
  for (int r = 0; r < 16; r++) {
    v[r] = row[j + 16u * r];
    if (mean) v[r] = make_float2(__fsub_rn(__fmul_rn(v[r].x, inv), 1.0f),
                                 __fsub_rn(__fmul_rn(v[r].y, inv), 1.0f));
    v[r].y = -v[r].y;
  }
  dft_inv(v);
#pragma unroll
  for (int k = 1; k < 16; k++) v[k] = cmul(v[k], __ldg(twb + k * 16 + j));
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; k++) row[16 * k + (j ^ k)] = v[k];
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 16; m++) v[m] = row[16 * j + (m ^ j)];
  dft_inv(v);
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; k++) row[j + 16 * k] = make_float2(v[k].x, -v[k].y);  // C
  __syncwarp();
  float2 out[16];
  float2 nyq = make_float2(0.f, 0.f);
#pragma unroll
  for (int r = 0; r < 16; r++) {
    const unsigned k = j + 16u * r;
    const float2 c = row[k], m = row[(256u - k) & 255u];
    const float2 e = make_float2(0.5f * (c.x + m.x), 0.5f * (c.y - m.y));  // (C + conj C[-k]) / 2
    const float2 d = make_float2(c.x - m.x, c.y + m.y);                    // C - conj C[-k]
    const float2 o = make_float2(0.5f * d.y, -0.5f * d.x);                 // d / 2i
    const float2 w = __ldg(wpre + k);
    out[r] = cadd(e, cmul(o, make_float2(w.x, -w.y)));
    if (r == 0 && j == 0) nyq = make_float2(e.x - o.x, e.y - o.y);
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 16; r++) row[j + 16u * r] = out[r];
  if (j == 0) row[256] = nyq;
  __syncthreads();
  float2* tiles = work + ((size_t)x * kKzBlocks * 512 + y0) * 16;
  constexpr size_t kBlock = (size_t)512 * 16;
  for (uint32_t f = threadIdx.x; f < 16 * kRowsPerCta * 8; f += blockDim.x) {
    const uint32_t kb = f / (kRowsPerCta * 8), e = f % (kRowsPerCta * 8);
    const uint32_t r = e / 8, jj = e % 8;
    reinterpret_cast<float4*>(tiles + kb * kBlock)[e] =
        *reinterpret_cast<const float4*>(buf + r * kRowSlots + 16 * kb + 2 * jj);
  }
  if (threadIdx.x < kRowsPerCta)
    tiles[16 * kBlock + threadIdx.x * 16] = buf[threadIdx.x * kRowSlots + 256];
}

static bool own_inverse(uint32_t n) { return n == 512; }

// fft_build_filter_lut, src/math/fft.c:521-568: the radial factor by integer
// |k|^2, computed in double.
template <class R>
__global__ void lut_kernel(R* __restrict__ lut, uint32_t max_k2, int filter, double factor,
                           double gfactor) {
  for (uint32_t k2 = blockIdx.x * blockDim.x + threadIdx.x; k2 <= max_k2;
       k2 += gridDim.x * blockDim.x) {
    double v;
    if (k2 == 0) {
      v = 1.0;
    } else if (filter == kFilterTopHat) {
      const double kr = factor * sqrt((double)k2);
      v = kr > 1e-4 ? 3.0 * (sin(kr) - kr * cos(kr)) / (kr * kr * kr) : 1.0;
    } else if (filter == kFilterGaussian) {
      v = exp(-0.5 * factor * factor * (double)k2);
    } else {
      v = 1.0;
    }
    if (gfactor > 0.0 && k2 > 0) v *= exp(-0.5 * gfactor * gfactor * (double)k2);
    lut[k2] = (R)v;
  }
}

template <class R>
SmootherT<R>::~SmootherT() {
  release();
}

template <class R>
static void destroy_plans(typename SmootherT<R>::Plans& p) {
  if (p.r2c) cufftDestroy(p.r2c);
  if (p.c2r) cufftDestroy(p.c2r);
  if (p.twiddles) cudaFree(p.twiddles);
}

// A plan without a work area of its own (the smoother's shared one is set
// before it runs); `need` grows to the area it asks for.
static cufftHandle make_plan(uint32_t n, cufftType type, size_t* need) {
  cufftHandle h = 0;
  SIFG_CUFFT(cufftCreate(&h));
  size_t ws = 0;
  const cufftResult a = cufftSetAutoAllocation(h, 0);
  const cufftResult m = a == CUFFT_SUCCESS ? cufftMakePlan3d(h, (int)n, (int)n, (int)n, type, &ws) : a;
  if (m != CUFFT_SUCCESS) {
    cufftDestroy(h);
    throw CudaError{cudaErrorUnknown, "cufftMakePlan3d"};
  }
  if (ws > *need) *need = ws;
  return h;
}

template <class R>
void SmootherT<R>::release() {
  for (auto& p : plans) destroy_plans<R>(p);
  plans.clear();
  plan_r2c = plan_c2r = 0;
  plan_work = 0;
  twiddles = nullptr;
  factor_tables.clear();
  n = 0;
}

template <class R>
void SmootherT<R>::setup(uint32_t n_, R box_, int window_mode_, cudaStream_t st) {
  constexpr bool dbl = sizeof(R) == 8;
  bool rebind = false;
  if (n_ != n) {
    auto it = std::find_if(plans.begin(), plans.end(), [&](const Plans& p) { return p.n == n_; });
    if (it == plans.end()) {
      if ((int)plans.size() >= kPlanCache) {
        destroy_plans<R>(plans.front());
        plans.erase(plans.begin());
      }
      Plans p{n_, 0, 0};
      if (!dbl && own_inverse(n_)) {
        // The tables of the three-pass inverse, computed in double.
        std::vector<float2> tw(kTw512);
        auto root = [](double num, double den) {
          const double a = 2.0 * M_PI * num / den;
          return make_float2((float)std::cos(a), (float)std::sin(a));
        };
        for (int k = 0; k < 16; k++)
          for (int j = 0; j < 32; j++) tw[k * 32 + j] = root((double)(j * k), 512.0);
        for (int k = 0; k < 16; k++)
          for (int j = 0; j < 16; j++) tw[512 + k * 16 + j] = root((double)(j * k), 256.0);
        for (int k = 0; k < 256; k++) tw[768 + k] = root((double)k, 512.0);
        SIFG_CUDA(cudaMalloc(&p.twiddles, kTw512 * sizeof(float2)));
        // On the smoothing stream, which every use of the tables follows (a
        // plain cudaMemcpy runs on the legacy stream, which the library's
        // non-blocking streams do not wait for), and finished before the
        // staging vector goes.
        SIFG_CUDA(cudaMemcpyAsync(p.twiddles, tw.data(), kTw512 * sizeof(float2),
                                  cudaMemcpyHostToDevice, st));
        SIFG_CUDA(cudaStreamSynchronize(st));
      } else {
        p.r2c = make_plan(n_, dbl ? CUFFT_D2Z : CUFFT_R2C, &p.work);
        p.c2r = make_plan(n_, dbl ? CUFFT_Z2D : CUFFT_C2R, &p.work);
      }
      plans.push_back(p);
      it = plans.end() - 1;
    }
    n = n_;
    plan_r2c = it->r2c;
    plan_c2r = it->c2r;
    plan_work = it->work;
    twiddles = it->twiddles;
    rebind = true;  // a cached plan may be bound to another stream and area
  }
  if (plan_work > area.bytes) {
    area.ensure(plan_work);
    rebind = true;
  }
  if (rebind || st != stream) {
    for (cufftHandle h : {plan_r2c, plan_c2r}) {
      if (!h) continue;
      SIFG_CUFFT(cufftSetStream(h, st));
      if (plan_work) SIFG_CUFFT(cufftSetWorkArea(h, area.ptr));
    }
    stream = st;
  }
  box = box_;
  window_mode = window_mode_;
  const uint64_t modes = (uint64_t)n * n * (n / 2 + 1);
  spectrum.ensure(twiddles ? kTileWorkElems * sizeof(float2) : modes * 2 * sizeof(R));
  work.ensure(twiddles ? kTileWorkElems * sizeof(float2) : modes * 2 * sizeof(R));
  const uint32_t h = n >> 1;
  const uint32_t max_k2 = 3 * h * h;
  lut.ensure(((size_t)max_k2 + 1) * sizeof(R));
  win.ensure((size_t)n * sizeof(R));
  if (window_mode) {
    // fft_build_window_axis, src/math/fft.c:958-975, CIC (order 2): 1/W full,
    // W/S aliasing-aware, W = sinc^2(pi k / N), S = 1 - 2 sin^2/3.
    std::vector<R> w(n);
    for (uint32_t i = 0; i < n; i++) {
      const int32_t k = i > h ? (int32_t)n - (int32_t)i : (int32_t)i;  // |k|: an even table
      const double x = M_PI * (double)k / (double)n;
      const double s = (x < 1e-9 && x > -1e-9) ? 1.0 : std::sin(x) / x;
      const double W = s * s;
      w[i] = (R)(window_mode == 2 ? W / (1.0 - 2.0 * std::sin(x) * std::sin(x) / 3.0) : 1.0 / W);
    }
    SIFG_CUDA(cudaMemcpyAsync(win.ptr, w.data(), n * sizeof(R), cudaMemcpyHostToDevice, st));
    SIFG_CUDA(cudaStreamSynchronize(st));
  }
}

static void launch_forward512(const SmootherT<float>& s, const float* grid, const double* mean);

template <>
void SmootherT<float>::forward(const float* grid, const double* mean) {
  if (twiddles) {
    launch_forward512(*this, grid, mean);
    return;
  }
  if (mean) apply_contrast(const_cast<float*>(grid), (uint64_t)n * n * n, mean, stream);
  SIFG_CUFFT(cufftExecR2C(plan_r2c, (cufftReal*)grid, (cufftComplex*)spectrum.ptr));
}
template <>
void SmootherT<double>::forward(const double* grid, const double* mean) {
  if (mean) apply_contrast(const_cast<double*>(grid), (uint64_t)n * n * n, mean, stream);
  SIFG_CUFFT(cufftExecD2Z(plan_r2c, (cufftDoubleReal*)grid, (cufftDoubleComplex*)spectrum.ptr));
}

static void launch_filter(const SmootherT<float>& s, int filter, float norm) {
  const uint64_t modes = (uint64_t)s.n * s.n * (s.n / 2 + 1);
  const float* w = (s.window_mode && filter != kFilterNone) ? s.win.as<float>() : nullptr;
  const unsigned grd = grid_for(modes / 2 + 1, 256, 152u * 8u);
  if (modes < (1ull << 32))
    filter_kernel<uint32_t><<<grd, 256, 0, s.stream>>>(s.spectrum.as<float4>(), s.work.as<float4>(),
                                                       s.n, s.lut.as<float>(), w, norm);
  else
    filter_kernel<uint64_t><<<grd, 256, 0, s.stream>>>(s.spectrum.as<float4>(), s.work.as<float4>(),
                                                       s.n, s.lut.as<float>(), w, norm);
}

// The three passes of the n = 512 inverse transform, on the smoother's stream.
// Tiles ((u * kKzBlocks + kb) * N + v) * 16 + kz % 16 read as columns along v
// with line u, or along u with line v. The forward leaves the spectrum as
// tiles of line ky along kx; the inverse's pass (1) writes the work buffer as
// tiles of line x along ky (read along x by nothing, along ky by pass (2)).
constexpr ColumnLayout kTilesByLine{kKzBlocks * 512 * kColCols, 512 * kColCols, kColCols};
constexpr ColumnLayout kTilesByRow{kColCols, 512 * kColCols, kKzBlocks * 512 * kColCols};

static void set_column_smem() {
  thread_local bool attr = false;  // set once per thread
  if (!attr) {
    SIFG_CUDA(cudaFuncSetAttribute(colfft512_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(kColCols * kColStride * sizeof(float2))));
    attr = true;
  }
}

// The float form's forward transform at n = 512: the R2C along z into the
// work tiles, the forward ky FFT in place, the forward kx FFT into the
// spectrum's tiles.
static void launch_forward512(const SmootherT<float>& s, const float* grid, const double* mean) {
  constexpr uint32_t N = 512;
  set_column_smem();
  const size_t smem = (size_t)kColCols * kColStride * sizeof(float2);
  const float2* tw = (const float2*)s.twiddles;
  r2c512_rows_kernel<<<N * N / kRowsPerCta, 16 * kRowsPerCta, 0, s.stream>>>(
      grid, s.work.as<float2>(), tw, mean);
  SIFG_LAUNCH_CHECK();
  colfft512_kernel<<<dim3(kKzBlocks, N), 32 * kColWarps, smem, s.stream>>>(
      s.work.as<float2>(), s.work.as<float2>(), kTilesByLine, kTilesByLine, kNoFilter, nullptr, 1.f,
      tw, true);
  SIFG_LAUNCH_CHECK();
  colfft512_kernel<<<dim3(kKzBlocks, N), 32 * kColWarps, smem, s.stream>>>(
      s.work.as<float2>(), s.spectrum.as<float2>(), kTilesByRow, kTilesByLine, kNoFilter, nullptr,
      1.f, tw, true);
  SIFG_LAUNCH_CHECK();
}

// The timer, begun by the caller, ends after pass (1): the filter's kernel.
// ftab: the smoothing's factor table, or NULL (the factors evaluated).
static void launch_inverse512(const SmootherT<float>& s, int filter, const RadialFilter& rf,
                              float norm, float* out, KernelTimer* timer, const BelowList& below,
                              const float* ftab) {
  constexpr uint32_t N = 512;
  const float* w = (s.window_mode && filter != kFilterNone) ? s.win.as<float>() : nullptr;
  const size_t smem = (size_t)kColCols * kColStride * sizeof(float2);
  set_column_smem();
  const float2* tw = (const float2*)s.twiddles;
  const dim3 grid(kKzBlocks, N);
  colfft512_kernel<<<grid, 32 * kColWarps, smem, s.stream>>>(
      s.spectrum.as<float2>(), s.work.as<float2>(), kTilesByLine, kTilesByRow, rf, w,
      norm, tw, false, ftab);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(s.stream);
  colfft512_kernel<<<grid, 32 * kColWarps, smem, s.stream>>>(
      s.work.as<float2>(), s.work.as<float2>(), kTilesByLine, kTilesByLine, kNoFilter, nullptr, 1.f,
      tw, false);
  SIFG_LAUNCH_CHECK();
  c2r512_rows_kernel<<<N * N / kRowsPerCta, 16 * kRowsPerCta, 0, s.stream>>>(s.work.as<float2>(),
                                                                           out, tw, below);
  SIFG_LAUNCH_CHECK();
}
static void launch_inverse512(const SmootherT<double>&, int, const RadialFilter&, double, double*,
                              KernelTimer*, const BelowList&, const float*) {}

static int g_factor_tables = 1;
void set_factor_tables(int on) { g_factor_tables = on; }

static RadialFilter radial_filter_of(int filter, double factor, double gfactor) {
  const float f = (float)factor;
  return RadialFilter{filter == kFilterTopHat || filter == kFilterGaussian ? filter : kFilterNone,
                      (float)(factor * factor), (float)(0.5 * gfactor * gfactor), f,
                      (float)(factor - (double)f)};
}

template <class R>
const float* SmootherT<R>::factor_table(int filter, R r, R sigma) {
  if constexpr (sizeof(R) != 4) {
    return nullptr;
  } else {
    if (!g_factor_tables || !twiddles || filter == kFilterNone) return nullptr;
    factor_clock++;
    for (auto& t : factor_tables)
      if (t->filter == filter && t->r == r && t->sigma == sigma && t->box == box &&
          t->window_mode == window_mode) {
        t->used = factor_clock;
        return t->buf.template as<float>();
      }
    std::unique_ptr<FactorTable> t;
    if ((int)factor_tables.size() >= kFactorTables) {
      auto lru = std::min_element(factor_tables.begin(), factor_tables.end(),
                                  [](const auto& a, const auto& b) { return a->used < b->used; });
      t = std::move(*lru);
      factor_tables.erase(lru);
    } else {
      t.reset(new FactorTable);
    }
    t->filter = filter;
    t->r = r;
    t->sigma = sigma;
    t->box = box;
    t->window_mode = window_mode;
    t->used = factor_clock;
    float* tab = (float*)t->buf.ensure((size_t)kFactorSide * kFactorSide * kFactorSide * sizeof(float));
    const double factor = (double)r * 2.0 * M_PI / (double)box;
    const double gfactor = sigma > R(0) ? (double)sigma * 2.0 * M_PI / (double)box : 0.0;
    const float norm = (float)(1.0 / ((double)n * n * n));
    factor_table_kernel<<<152u * 8u, 256, 0, stream>>>(tab, radial_filter_of(filter, factor, gfactor),
                                                       window_mode ? win.template as<float>() : nullptr,
                                                       norm);
    SIFG_LAUNCH_CHECK();
    factor_tables.push_back(std::move(t));
    return factor_tables.back()->buf.template as<float>();
  }
}

static void launch_filter(const SmootherT<double>& s, int filter, double norm) {
  const uint64_t modes = (uint64_t)s.n * s.n * (s.n / 2 + 1);
  const double* w = (s.window_mode && filter != kFilterNone) ? s.win.as<double>() : nullptr;
  filter_kernel_f64<<<grid_for(modes, 256, 152u * 8u), 256, 0, s.stream>>>(
      s.spectrum.as<double2>(), s.work.as<double2>(), s.n, s.lut.as<double>(), w, norm);
}

template <class R>
void SmootherT<R>::smooth(int filter, R r, R sigma, R* out, KernelTimer* timer,
                          const BelowList* below) {
  const uint32_t h = n >> 1;
  const uint32_t max_k2 = 3 * h * h;
  const double factor = (double)r * 2.0 * M_PI / (double)box;
  const double gfactor = sigma > R(0) ? (double)sigma * 2.0 * M_PI / (double)box : 0.0;
  const R norm = (R)(1.0 / ((double)n * n * n));
  if (twiddles) {
    // The own inverse reads the smoothing's factor table (built on first use)
    // or evaluates the radial factor as it applies it.
    const RadialFilter rf = radial_filter_of(filter, factor, gfactor);
    const float* ftab = factor_table(filter, r, sigma);
    if (timer) timer->begin(stream);
    launch_inverse512(*this, filter, rf, norm, out, timer, below ? *below : BelowList{}, ftab);
    return;
  }
  lut_kernel<R><<<grid_for((uint64_t)max_k2 + 1, 256), 256, 0, stream>>>(lut.as<R>(), max_k2, filter,
                                                                         factor, gfactor);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->begin(stream);
  launch_filter(*this, filter, norm);
  SIFG_LAUNCH_CHECK();
  if (timer) timer->end(stream);
  if (sizeof(R) == 8)
    SIFG_CUFFT(cufftExecZ2D(plan_c2r, (cufftDoubleComplex*)work.ptr, (cufftDoubleReal*)out));
  else
    SIFG_CUFFT(cufftExecC2R(plan_c2r, (cufftComplex*)work.ptr, (cufftReal*)out));
}

template <class R>
void SmootherT<R>::restore(R* out) {
  smooth(kFilterNone, R(0), R(0), out, nullptr);
}

template struct SmootherT<float>;
template struct SmootherT<double>;

}  // namespace sifg
