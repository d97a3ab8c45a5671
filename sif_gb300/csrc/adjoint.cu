// The adjoint of the CIC density contrast with respect to the particle
// positions: given g = dL/d(delta) on the grid, dL/dx_p for every particle.
//
// delta_c = rho_c / rho_mean - 1 with rho_c = (1/V_cell) sum_p w_c(x_p) (the
// deposit of grid.c:585-650); the mean density is N_p / V whatever the
// positions (the deposit conserves each particle's unit mass), so
//   dL/dx_p = (1 / (rho_mean V_cell)) * (N / L) *
//             sum over the 8 corners of (+-1 along x) * wy * wz * g_corner,
// and likewise along y and z: a CIC gather of g with one weight replaced by
// its derivative. The base cell and fractions are the deposit's own (the same
// cell coordinate, so the two are each other's transpose exactly); the
// derivative at a cell face, where the weight has a kink, is the one from the
// cell the particle is assigned to.
//
// The smoothing that usually sits between delta and the loss is
// self-adjoint (a real, even filter between an R2C and a C2R), so its
// adjoint is the smoothing of the incoming gradient, done by the caller.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.cuh"

namespace sifg {

// The deposit's cell coordinate of one axis: base cell c0, its upper
// neighbour c1 (periodic) and the fraction t, in the form's precision.
__device__ __forceinline__ void adj_axis(float v, uint32_t n, float box, float idx_hi,
                                         float idx_lo, uint32_t& c0, uint32_t& c1, float& t) {
  // As the float deposit: u = fold(v) * n / box kept exact as hi + lo.
  const float x = box_fold(v, box);
  const float hi = fmul(x, idx_hi);
  const float lo = fadd(__fmaf_rn(x, idx_hi, -hi), fmul(x, idx_lo));
  float r = floorf(hi);
  float f = fadd(fsub(hi, r), lo);
  if (f < 0.0f) {
    r -= 1.0f;
    f = fadd(f, 1.0f);
  } else if (f >= 1.0f) {
    r += 1.0f;
    f = fsub(f, 1.0f);
  }
  int32_t c = (int32_t)r;
  if (c < 0) c += (int32_t)n;
  if (c >= (int32_t)n) c -= (int32_t)n;
  c0 = (uint32_t)c;
  c1 = c0 + 1 == n ? 0u : c0 + 1;
  t = f;
}

__device__ __forceinline__ void adj_axis(double v, uint32_t n, double box, double idx, double,
                                         uint32_t& c0, uint32_t& c1, double& t) {
  const double u = fmul(box_fold(v, box), idx);
  const uint32_t raw = (uint32_t)u;
  c0 = raw >= n ? 0u : raw;
  c1 = c0 + 1 == n ? 0u : c0 + 1;
  t = fsub(u, (double)raw);
}

template <class R>
__global__ void cic_vjp_kernel(const R* __restrict__ x, const R* __restrict__ y,
                               const R* __restrict__ z, uint64_t np, uint32_t n, R box, R idx_hi,
                               R idx_lo, const R* __restrict__ g, R scale, R* __restrict__ gx,
                               R* __restrict__ gy, R* __restrict__ gz) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    uint32_t xs[2], ys[2], zs[2];
    R tx, ty, tz;
    adj_axis(x[p], n, box, idx_hi, idx_lo, xs[0], xs[1], tx);
    adj_axis(y[p], n, box, idx_hi, idx_lo, ys[0], ys[1], ty);
    adj_axis(z[p], n, box, idx_hi, idx_lo, zs[0], zs[1], tz);
    const R wx[2] = {R(1) - tx, tx}, wy[2] = {R(1) - ty, ty}, wz[2] = {R(1) - tz, tz};
    R ax = 0, ay = 0, az = 0;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int b = 0; b < 2; b++)
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const R v = __ldg(g + ((uint64_t)xs[a] * n + ys[b]) * n + zs[c]);
          const R sa = a ? R(1) : R(-1), sb = b ? R(1) : R(-1), sc = c ? R(1) : R(-1);
          ax += sa * wy[b] * wz[c] * v;
          ay += wx[a] * sb * wz[c] * v;
          az += wx[a] * wy[b] * sc * v;
        }
    gx[p] = ax * scale;
    gy[p] = ay * scale;
    gz[p] = az * scale;
  }
}

template <class R>
void cic_contrast_vjp(const R* x, const R* y, const R* z, uint64_t np, uint32_t n, R box,
                      const R* g, R* gx, R* gy, R* gz, cudaStream_t st) {
  // scale = (N / L) / (rho_mean V_cell), rho_mean = N_p / L^3, V_cell = (L/N)^3:
  // = (N / L) * N^3 / N_p.
  const double nd = (double)n;
  const R scale = (R)((nd / (double)box) * nd * nd * nd / (double)np);
  R idx_hi, idx_lo = 0;
  const double idx = nd / (double)box;
  idx_hi = (R)idx;
  if (sizeof(R) == 4) idx_lo = (R)(idx - (double)idx_hi);
  cic_vjp_kernel<R><<<grid_for(np, 256), 256, 0, st>>>(x, y, z, np, n, box, idx_hi, idx_lo, g,
                                                       scale, gx, gy, gz);
  SIFG_LAUNCH_CHECK();
}

template void cic_contrast_vjp<float>(const float*, const float*, const float*, uint64_t,
                                      uint32_t, float, const float*, float*, float*, float*,
                                      cudaStream_t);
template void cic_contrast_vjp<double>(const double*, const double*, const double*, uint64_t,
                                       uint32_t, double, const double*, double*, double*, double*,
                                       cudaStream_t);

}  // namespace sifg
