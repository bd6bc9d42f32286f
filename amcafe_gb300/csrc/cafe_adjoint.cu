// Differentiable part of the CA step with hand-written adjoints (no
// counterpart in the reference).
//
// Temperature: the Rosenthal point source moving along +x over a half space,
//   T = T0 + q / R exp(-v (R + xi) / (2 alpha)),  q = eta P / (2 pi k),
// xi = x - (x_start + v t), R = |(xi, y - y_src, z - z_src)| clamped below at
// half a voxel, t = step dt: the field the CA steps under the deck keyword
// "rosenthal" (csrc/cafe_device.cuh, cafe_rosenthal_T) for a track along +x
// of an unrotated laser frame. Parameters theta = (P, eta, v, a, n).
//
// Melt-pool shape at one step from the soft melt indicator
// m = 1 / (1 + exp(-(T - T_liq) / tau_T)) over the cells: with the m-weighted
// moments, length = sqrt(12 var_x), width = sqrt(12 var_y) and depth =
// sqrt(3 E[d^2]), d the depth below the source plane (the extents of a box
// of uniform weight).
//
// Growth: G = sum over the growth log (cell c, step s, growth time tau) of
// a (T_liq - T(c, s))^n tau, the time-integrated octahedron growth
// v = a dT^n of VoxelsCA.C:405, 511-516 with the capture and nucleation
// events (hence the growth times) held fixed.
//
// Each kernel evaluates the values and, given output cotangents, the
// vector-Jacobian product with respect to theta in one pass over the cells (or
// log entries), accumulating per-block partial sums in FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/cafe_gpu.h"

void cafe_internal_set_error(const char *msg);

namespace {

struct AdjTheta {
  double P, eta, v, a, n;
};

// T and dT/d(P, eta, v) at a point, time t
__device__ __forceinline__ void adj_temp(const cafe_adjoint_setup &S, const AdjTheta &th, double x, double y, double z,
                                         double t, double &T, double dT[3]) {
  const double pi = 3.14159265358979323846;
  double xi = x - (S.x_start + th.v * t);
  double dy = y - S.y_src, dz = z - S.z_src;
  double R = sqrt(xi * xi + dy * dy + dz * dz);
  const bool clamped = R < 0.5 * S.dx;  // R fixed at half a voxel: no dependence on v through R
  if (clamped) R = 0.5 * S.dx;
  double q = th.eta * th.P / (2 * pi * S.k);
  double E = exp(-th.v * (R + xi) / (2 * S.alpha));
  double U = q / R * E;  // T - T0
  T = S.T0 + U;
  dT[0] = U / th.P;
  dT[1] = U / th.eta;
  if (clamped)
    dT[2] = U * (-(R + xi) / (2 * S.alpha) + th.v * t / (2 * S.alpha));
  else
    dT[2] = U * (-(R + xi) / (2 * S.alpha) + th.v * t * (1 + xi / R) / (2 * S.alpha) + xi * t / (R * R));
}

// Per-block partial sums of n values (n <= 16, 256 threads) in a fixed order:
// warp shuffles, then warp 0 adds the warps' sums in warp order and writes
// the block's partials to part[blockIdx.x * n + j]; k_adj_total adds the
// blocks' partials in block order. The sums are thus the same at every call
// (no atomics), which keeps finite differences of the outputs clean.
__device__ __forceinline__ void block_sum(double *v, int n, double *part) {
  __shared__ double ws[8][16];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < n; ++j) {
    double x = v[j];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) ws[w][j] = x;
  }
  __syncthreads();
  if (threadIdx.x < n) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += ws[q][threadIdx.x];
    part[(long long)blockIdx.x * n + threadIdx.x] = t;
  }
}

__global__ void k_adj_total(const double *part, int nblocks, int n, double *out) {
  if (threadIdx.x < n) {
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t += part[(long long)b * n + threadIdx.x];
    out[threadIdx.x] = t;
  }
}

// sums[0..5] = {S m, S m x, S m x^2, S m y, S m y^2, S m d^2}; with w (cotangents
// of the six sums) also grad[0..2] += sum w . d(m-moments)/d(P, eta, v)
__global__ void k_adj_pool(cafe_adjoint_setup S, AdjTheta th, int with_grad, const double *w, double *acc) {
  const long long N = (long long)S.nx * S.ny * S.nz;
  const double t = S.step_final * S.dt;
  double loc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double w6[6] = {0, 0, 0, 0, 0, 0};
  if (with_grad)
    for (int j = 0; j < 6; ++j) w6[j] = w[j];
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
    long long k = c / ((long long)S.nx * S.ny), r = c - k * (long long)S.nx * S.ny;
    long long j = r / S.nx, i = r - j * S.nx;
    double x = (i + .5) * S.dx, y = (j + .5) * S.dx, z = (k + .5) * S.dx;
    if (z > S.z_src) continue;  // above the source plane: no melt
    double T, dT[3];
    adj_temp(S, th, x, y, z, t, T, dT);
    double u = (T - S.Tl) / S.tau_T;
    double m = 1.0 / (1.0 + exp(-u));
    double d = S.z_src - z;
    double f[6] = {1.0, x, x * x, y, y * y, d * d};
    for (int q = 0; q < 6; ++q) loc[q] += m * f[q];
    if (with_grad) {
      double wf = 0.0;
      for (int q = 0; q < 6; ++q) wf += w6[q] * f[q];
      double dm = m * (1.0 - m) / S.tau_T * wf;
      loc[6] += dm * dT[0];
      loc[7] += dm * dT[1];
      loc[8] += dm * dT[2];
    }
  }
  block_sum(loc, 9, acc);
}

// acc[0] += sum a dT^n tau; acc[1..5] += cot * d/d(P, eta, v, a, n)
__global__ void k_adj_growth(cafe_adjoint_setup S, AdjTheta th, const int32_t *cells, const int32_t *steps,
                             const double *tau, long long n, double cot, double *acc) {
  double loc[6] = {0, 0, 0, 0, 0, 0};
  const long long nxy = (long long)S.nx * S.ny;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    double ta = tau[e];  // negative after negative-time events (VoxelsCA.C:511-516)
    if (!(ta != 0.0) || isinf(ta)) continue;
    long long c = cells[e];
    long long k = c / nxy, r = c - k * nxy;
    long long j = r / S.nx, i = r - j * S.nx;
    double x = (i + .5) * S.dx, y = (j + .5) * S.dx, z = (k + .5) * S.dx;
    double T, dT[3];
    adj_temp(S, th, x, y, z, steps[e] * S.dt, T, dT);
    double D = S.Tl - T;
    if (!(D > 0.0)) continue;
    double pw = pow(D, th.n);
    double g = th.a * pw * ta;
    loc[0] += g;
    double dgdT = -th.a * th.n * pow(D, th.n - 1.0) * ta;
    loc[1] += cot * dgdT * dT[0];
    loc[2] += cot * dgdT * dT[1];
    loc[3] += cot * dgdT * dT[2];
    loc[4] += cot * pw * ta;
    loc[5] += cot * g * log(D);
  }
  block_sum(loc, 6, acc);
}

int adj_fail(int rc, const char *msg) {
  cafe_internal_set_error(msg);
  return rc;
}

}  // namespace

extern "C" {

int cafe_adjoint_pool(const cafe_adjoint_setup *S, const double theta[5], const double *cot, double out[3],
                      double grad[5], void *stream) {
  if (!S || !theta || !out) return adj_fail(CAFE_E_ARG, "cafe_adjoint_pool: null argument");
  if (!(S->tau_T > 0) || S->nx <= 0 || S->ny <= 0 || S->nz <= 0 || !(S->dx > 0))
    return adj_fail(CAFE_E_ARG, "cafe_adjoint_pool: bad setup");
  cudaStream_t st = (cudaStream_t)stream;
  AdjTheta th = {theta[0], theta[1], theta[2], theta[3], theta[4]};
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nb = nsm * 8;
  double *d = nullptr;  // [16] totals and cotangents, then [nb][9] block partials
  if (cudaMalloc((void **)&d, (16 + (size_t)nb * 9) * sizeof(double)) != cudaSuccess)
    return adj_fail(CAFE_E_CUDA, "cafe_adjoint_pool: cudaMalloc failed");
  double *part = d + 16;
  double h[16] = {0};
  int rc = CAFE_OK;
  // forward sums
  if (cudaMemsetAsync(d, 0, 16 * sizeof(double), st) != cudaSuccess) rc = CAFE_E_CUDA;
  if (!rc) {
    k_adj_pool<<<nb, 256, 0, st>>>(*S, th, 0, d + 9, part);
    k_adj_total<<<1, 32, 0, st>>>(part, nb, 9, d);
    if (cudaMemcpyAsync(h, d, 9 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = CAFE_E_CUDA;
  }
  double S0 = h[0], mx = h[1] / S0, my = h[3] / S0;
  double vx = h[2] / S0 - mx * mx, vy = h[4] / S0 - my * my, ed = h[5] / S0;
  if (!rc) {
    if (!(S0 > 0) || !(vx > 0) || !(vy > 0) || !(ed > 0)) rc = adj_fail(CAFE_E_ARG, "cafe_adjoint_pool: no melt");
  }
  if (!rc) {
    out[0] = std::sqrt(12 * vx);
    out[1] = std::sqrt(12 * vy);
    out[2] = std::sqrt(3 * ed);
    if (cot && grad) {
      // cotangents of the six sums (chain rule through the moments)
      double cL = cot[0], cW = cot[1], cD = cot[2];
      double gvx = cL * 6 / out[0], gvy = cW * 6 / out[1], ged = cD * 1.5 / out[2];
      // vx = S2/S0 - (S1/S0)^2, vy likewise, ed = S5/S0
      double w[6];
      w[1] = gvx * (-2 * mx / S0);
      w[2] = gvx / S0;
      w[3] = gvy * (-2 * my / S0);
      w[4] = gvy / S0;
      w[5] = ged / S0;
      w[0] = gvx * (-h[2] / (S0 * S0) + 2 * mx * h[1] / (S0 * S0)) + gvy * (-h[4] / (S0 * S0) + 2 * my * h[3] / (S0 * S0)) +
             ged * (-h[5] / (S0 * S0));
      if (cudaMemsetAsync(d, 0, 9 * sizeof(double), st) != cudaSuccess ||
          cudaMemcpyAsync(d + 9, w, 6 * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = CAFE_E_CUDA;
      if (!rc) {
        k_adj_pool<<<nb, 256, 0, st>>>(*S, th, 1, d + 9, part);
        k_adj_total<<<1, 32, 0, st>>>(part, nb, 9, d);
        if (cudaMemcpyAsync(h, d, 9 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          rc = CAFE_E_CUDA;
      }
      if (!rc) {
        grad[0] = h[6];
        grad[1] = h[7];
        grad[2] = h[8];
        grad[3] = 0.0;
        grad[4] = 0.0;
      }
    }
  }
  cudaFree(d);
  if (rc == CAFE_E_CUDA) return adj_fail(rc, "cafe_adjoint_pool: CUDA error");
  return rc;
}

int cafe_adjoint_growth(const cafe_adjoint_setup *S, const double theta[5], const int32_t *cells,
                        const int32_t *steps, const double *tau, long long n, double cot, double *out,
                        double grad[5], void *stream) {
  if (!S || !theta || !out || (n > 0 && (!cells || !steps || !tau)))
    return adj_fail(CAFE_E_ARG, "cafe_adjoint_growth: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  AdjTheta th = {theta[0], theta[1], theta[2], theta[3], theta[4]};
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nb = nsm * 8;
  double *d = nullptr;  // [8] totals, then [nb][6] block partials
  if (cudaMalloc((void **)&d, (8 + (size_t)nb * 6) * sizeof(double)) != cudaSuccess)
    return adj_fail(CAFE_E_CUDA, "cafe_adjoint_growth: cudaMalloc failed");
  double h[8] = {0};
  int rc = CAFE_OK;
  if (cudaMemsetAsync(d, 0, 8 * sizeof(double), st) != cudaSuccess) rc = CAFE_E_CUDA;
  if (!rc && n > 0) {
    k_adj_growth<<<nb, 256, 0, st>>>(*S, th, cells, steps, tau, n, cot, d + 8);
    k_adj_total<<<1, 32, 0, st>>>(d + 8, nb, 6, d);
  }
  if (!rc && (cudaGetLastError() != cudaSuccess ||
              cudaMemcpyAsync(h, d, 6 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess))
    rc = CAFE_E_CUDA;
  cudaFree(d);
  if (rc) return adj_fail(rc, "cafe_adjoint_growth: CUDA error");
  *out = h[0];
  if (grad)
    for (int q = 0; q < 5; ++q) grad[q] = h[1 + q];
  return CAFE_OK;
}

}  // extern "C"
