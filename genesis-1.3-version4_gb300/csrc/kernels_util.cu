// Layout conversions between the reference's host records and the device
// structure-of-arrays storage.
//   particles: host AoS [n][6] doubles (gamma, theta, x, y, px, py) <-> device SoA;
//              in the mixed form gamma is stored as the FP32 offset from gammaref,
//              x, y, px, py as FP32 and theta as a Q32.32 fixed-point turn count
//   fields:    host double2 <-> device float2 in the mixed form
#include <cuda_runtime.h>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

__global__ void k_aos_to_soa_d(const double *__restrict__ aos, double *g, double *th, double *x,
                               double *y, double *px, double *py, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double *r = aos + 6 * i;
    g[i] = r[0];
    th[i] = r[1];
    x[i] = r[2];
    y[i] = r[3];
    px[i] = r[4];
    py[i] = r[5];
  }
}
// theta in radians -> Q32.32 turn count (the mixed form's phase accumulator)
__device__ __forceinline__ long long to_turns(double th) {
  return __double2ll_rn(th * (4294967296.0 / 6.283185307179586476925286766559));
}
__device__ __forceinline__ double from_turns(long long t) {
  return (double)t * (6.283185307179586476925286766559 / 4294967296.0);
}

__global__ void k_aos_to_soa_f(const double *__restrict__ aos, double gref, float *g, long long *th,
                               float *x, float *y, float *px, float *py, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double *r = aos + 6 * i;
    g[i] = (float)(r[0] - gref);
    th[i] = to_turns(r[1]);
    x[i] = (float)r[2];
    y[i] = (float)r[3];
    px[i] = (float)r[4];
    py[i] = (float)r[5];
  }
}
__global__ void k_soa_to_aos_d(const double *g, const double *th, const double *x, const double *y,
                               const double *px, const double *py, double *__restrict__ aos, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double *r = aos + 6 * i;
    r[0] = g[i];
    r[1] = th[i];
    r[2] = x[i];
    r[3] = y[i];
    r[4] = px[i];
    r[5] = py[i];
  }
}
__global__ void k_soa_to_aos_f(const float *g, double gref, const long long *th, const float *x,
                               const float *y, const float *px, const float *py,
                               double *__restrict__ aos, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double *r = aos + 6 * i;
    r[0] = gref + (double)g[i];
    r[1] = from_turns(th[i]);
    r[2] = x[i];
    r[3] = y[i];
    r[4] = px[i];
    r[5] = py[i];
  }
}
__global__ void k_d2f(const double2 *in, float2 *out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_f2d(const float2 *in, double2 *out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 v = in[i];
    out[i] = make_double2(v.x, v.y);
  }
}

unsigned grid_for(size_t n) {
  size_t b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace

void launch_aos_to_soa(void *stream, const double *aos, void *const *soa, int mixed, double gref,
                       size_t n) {
  cudaStream_t s = (cudaStream_t)stream;
  if (mixed)
    k_aos_to_soa_f<<<grid_for(n), 256, 0, s>>>(aos, gref, (float *)soa[0], (long long *)soa[1],
                                               (float *)soa[2], (float *)soa[3], (float *)soa[4],
                                               (float *)soa[5], n);
  else
    k_aos_to_soa_d<<<grid_for(n), 256, 0, s>>>(aos, (double *)soa[0], (double *)soa[1],
                                               (double *)soa[2], (double *)soa[3],
                                               (double *)soa[4], (double *)soa[5], n);
}

void launch_soa_to_aos(void *stream, const void *const *soa, double *aos, int mixed, double gref,
                       size_t n) {
  cudaStream_t s = (cudaStream_t)stream;
  if (mixed)
    k_soa_to_aos_f<<<grid_for(n), 256, 0, s>>>((const float *)soa[0], gref, (const long long *)soa[1],
                                               (const float *)soa[2], (const float *)soa[3],
                                               (const float *)soa[4], (const float *)soa[5], aos, n);
  else
    k_soa_to_aos_d<<<grid_for(n), 256, 0, s>>>((const double *)soa[0], (const double *)soa[1],
                                               (const double *)soa[2], (const double *)soa[3],
                                               (const double *)soa[4], (const double *)soa[5], aos, n);
}

void launch_convert_field(void *stream, const void *in, void *out, size_t n, int to_float) {
  cudaStream_t s = (cudaStream_t)stream;
  if (to_float)
    k_d2f<<<grid_for(n), 256, 0, s>>>((const double2 *)in, (float2 *)out, n);
  else
    k_f2d<<<grid_for(n), 256, 0, s>>>((const float2 *)in, (double2 *)out, n);
}

}  // namespace g4
