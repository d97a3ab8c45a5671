// The per-rung smoothing: cuFFT R2C of the density contrast once, then per
// radius one fused filter kernel and a cuFFT C2R.
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
// double by a small kernel, as the reference tabulates it. The unfiltered
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
void SmootherT<R>::release() {
  for (const Plans& p : plans) {
    cufftDestroy(p.r2c);
    cufftDestroy(p.c2r);
  }
  plans.clear();
  plan_r2c = plan_c2r = 0;
  n = 0;
}

template <class R>
void SmootherT<R>::setup(uint32_t n_, R box_, int window_mode_, cudaStream_t st) {
  constexpr bool dbl = sizeof(R) == 8;
  bool rebind = false;
  if (n_ != n || !plan_r2c) {
    auto it = std::find_if(plans.begin(), plans.end(), [&](const Plans& p) { return p.n == n_; });
    if (it == plans.end()) {
      if ((int)plans.size() >= kPlanCache) {
        cufftDestroy(plans.front().r2c);
        cufftDestroy(plans.front().c2r);
        plans.erase(plans.begin());
      }
      Plans p{n_, 0, 0};
      SIFG_CUFFT(cufftPlan3d(&p.r2c, (int)n_, (int)n_, (int)n_, dbl ? CUFFT_D2Z : CUFFT_R2C));
      SIFG_CUFFT(cufftPlan3d(&p.c2r, (int)n_, (int)n_, (int)n_, dbl ? CUFFT_Z2D : CUFFT_C2R));
      plans.push_back(p);
      it = plans.end() - 1;
    }
    n = n_;
    plan_r2c = it->r2c;
    plan_c2r = it->c2r;
    rebind = true;  // a cached plan may be bound to another stream
  }
  if (rebind || st != stream) {
    SIFG_CUFFT(cufftSetStream(plan_r2c, st));
    SIFG_CUFFT(cufftSetStream(plan_c2r, st));
    stream = st;
  }
  box = box_;
  window_mode = window_mode_;
  const uint64_t modes = (uint64_t)n * n * (n / 2 + 1);
  spectrum.ensure(modes * 2 * sizeof(R));
  work.ensure(modes * 2 * sizeof(R));
  const uint32_t h = n >> 1;
  const uint32_t max_k2 = 3 * h * h;
  lut.ensure(((size_t)max_k2 + 1) * sizeof(R));
  win.ensure((size_t)n * sizeof(R));
  if (window_mode) {
    // fft_build_window_axis, src/math/fft.c:958-975, CIC (order 2): 1/W full,
    // W/S aliasing-aware, W = sinc^2(pi k / N), S = 1 - 2 sin^2/3.
    std::vector<R> w(n);
    for (uint32_t i = 0; i < n; i++) {
      const int32_t k = i > h ? (int32_t)i - (int32_t)n : (int32_t)i;
      const double x = M_PI * (double)k / (double)n;
      const double s = (x < 1e-9 && x > -1e-9) ? 1.0 : std::sin(x) / x;
      const double W = s * s;
      w[i] = (R)(window_mode == 2 ? W / (1.0 - 2.0 * std::sin(x) * std::sin(x) / 3.0) : 1.0 / W);
    }
    SIFG_CUDA(cudaMemcpyAsync(win.ptr, w.data(), n * sizeof(R), cudaMemcpyHostToDevice, st));
    SIFG_CUDA(cudaStreamSynchronize(st));
  }
}

template <>
void SmootherT<float>::forward(const float* grid) {
  SIFG_CUFFT(cufftExecR2C(plan_r2c, (cufftReal*)grid, (cufftComplex*)spectrum.ptr));
}
template <>
void SmootherT<double>::forward(const double* grid) {
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

static void launch_filter(const SmootherT<double>& s, int filter, double norm) {
  const uint64_t modes = (uint64_t)s.n * s.n * (s.n / 2 + 1);
  const double* w = (s.window_mode && filter != kFilterNone) ? s.win.as<double>() : nullptr;
  filter_kernel_f64<<<grid_for(modes, 256, 152u * 8u), 256, 0, s.stream>>>(
      s.spectrum.as<double2>(), s.work.as<double2>(), s.n, s.lut.as<double>(), w, norm);
}

template <class R>
void SmootherT<R>::smooth(int filter, R r, R sigma, R* out, KernelTimer* timer) {
  const uint32_t h = n >> 1;
  const uint32_t max_k2 = 3 * h * h;
  const double factor = (double)r * 2.0 * M_PI / (double)box;
  const double gfactor = sigma > R(0) ? (double)sigma * 2.0 * M_PI / (double)box : 0.0;
  lut_kernel<R><<<grid_for((uint64_t)max_k2 + 1, 256), 256, 0, stream>>>(lut.as<R>(), max_k2, filter,
                                                                         factor, gfactor);
  SIFG_LAUNCH_CHECK();
  const R norm = (R)(1.0 / ((double)n * n * n));
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
