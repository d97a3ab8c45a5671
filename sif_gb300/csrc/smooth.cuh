// The smoothing stage (smooth.cu).
#pragma once

#include <cufft.h>

#include <vector>

#include "kernels.cuh"

namespace sifg {

constexpr int kFilterNone = 0;
constexpr int kFilterTopHat = 1;
constexpr int kFilterGaussian = 2;

// Window modes: 0 none (SIF_FINDER_KEEP_CIC_WINDOW), 1 full CIC deconvolution,
// 2 aliasing-aware (SIF_FINDER_ALIASING_WINDOW).
struct Smoother {
  uint32_t n = 0;
  float box = 0.f;
  int window_mode = 1;
  cudaStream_t stream = 0;
  cufftHandle plan_r2c = 0, plan_c2r = 0;
  DevBuf spectrum, work, lut, win;

  void setup(uint32_t n, float box, int window_mode, cudaStream_t st);
  void forward(const float* grid);  // grid: n^3 floats on the device
  // Writes the grid smoothed at r (and, with sigma > 0, a Gaussian of sigma
  // on top) into out (n^3 floats), asynchronously on the stream.
  void smooth(int filter, float r, float sigma, float* out, KernelTimer* timer);
  void restore(float* out);
  void release();
  ~Smoother();
};

}  // namespace sifg
