// Layout conversions between the reference's host records and the device
// structure-of-arrays storage.
//   particles: host AoS [n][6] doubles (gamma, theta, x, y, px, py) <-> device SoA;
//              in the mixed form gamma is stored as the FP32 offset from gammaref,
//              x, y, px, py as FP32 and theta as a Q32.32 fixed-point turn count
//   fields:    host double2 <-> device float2 in the mixed form
#include <cuda_runtime.h>

#include <cstdint>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

// A record of six doubles is 48 bytes: with the array 16-byte aligned it is read or
// written as three double2 (V), else as six doubles.
template <bool V>
__device__ __forceinline__ void get_rec(const double *r, double *v) {
  if (V) {
    const double2 a = reinterpret_cast<const double2 *>(r)[0], b = reinterpret_cast<const double2 *>(r)[1],
                  c = reinterpret_cast<const double2 *>(r)[2];
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y, v[4] = c.x, v[5] = c.y;
  } else {
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = r[k];
  }
}
template <bool V>
__device__ __forceinline__ void put_rec(double *r, const double *v) {
  if (V) {
    reinterpret_cast<double2 *>(r)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(r)[1] = make_double2(v[2], v[3]);
    reinterpret_cast<double2 *>(r)[2] = make_double2(v[4], v[5]);
  } else {
#pragma unroll
    for (int k = 0; k < 6; k++) r[k] = v[k];
  }
}

template <bool V>
__global__ void k_aos_to_soa_d(const double *__restrict__ aos, double *g, double *th, double *x,
                               double *y, double *px, double *py, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v[6];
    get_rec<V>(aos + 6 * i, v);
    g[i] = v[0];
    th[i] = v[1];
    x[i] = v[2];
    y[i] = v[3];
    px[i] = v[4];
    py[i] = v[5];
  }
}
// theta in radians -> Q32.32 turn count (the mixed form's phase accumulator)
__device__ __forceinline__ long long to_turns(double th) {
  return __double2ll_rn(th * (4294967296.0 / 6.283185307179586476925286766559));
}
__device__ __forceinline__ double from_turns(long long t) {
  return (double)t * (6.283185307179586476925286766559 / 4294967296.0);
}

template <bool V>
__global__ void k_aos_to_soa_f(const double *__restrict__ aos, double gref, float *g, long long *th,
                               float *x, float *y, float *px, float *py, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v[6];
    get_rec<V>(aos + 6 * i, v);
    g[i] = (float)(v[0] - gref);
    th[i] = to_turns(v[1]);
    x[i] = (float)v[2];
    y[i] = (float)v[3];
    px[i] = (float)v[4];
    py[i] = (float)v[5];
  }
}
template <bool V>
__global__ void k_soa_to_aos_d(const double *g, const double *th, const double *x, const double *y,
                               const double *px, const double *py, double *__restrict__ aos, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v[6] = {g[i], th[i], x[i], y[i], px[i], py[i]};
    put_rec<V>(aos + 6 * i, v);
  }
}
template <bool V>
__global__ void k_soa_to_aos_f(const float *g, double gref, const long long *th, const float *x,
                               const float *y, const float *px, const float *py,
                               double *__restrict__ aos, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v[6] = {gref + (double)g[i], from_turns(th[i]), x[i], y[i], px[i], py[i]};
    put_rec<V>(aos + 6 * i, v);
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
  const bool v = ((uintptr_t)aos & 15) == 0;
  if (mixed) {
    auto k = v ? k_aos_to_soa_f<true> : k_aos_to_soa_f<false>;
    k<<<grid_for(n), 256, 0, s>>>(aos, gref, (float *)soa[0], (long long *)soa[1], (float *)soa[2],
                                  (float *)soa[3], (float *)soa[4], (float *)soa[5], n);
  } else {
    auto k = v ? k_aos_to_soa_d<true> : k_aos_to_soa_d<false>;
    k<<<grid_for(n), 256, 0, s>>>(aos, (double *)soa[0], (double *)soa[1], (double *)soa[2], (double *)soa[3],
                                  (double *)soa[4], (double *)soa[5], n);
  }
}

void launch_soa_to_aos(void *stream, const void *const *soa, double *aos, int mixed, double gref,
                       size_t n) {
  cudaStream_t s = (cudaStream_t)stream;
  const bool v = ((uintptr_t)aos & 15) == 0;
  if (mixed) {
    auto k = v ? k_soa_to_aos_f<true> : k_soa_to_aos_f<false>;
    k<<<grid_for(n), 256, 0, s>>>((const float *)soa[0], gref, (const long long *)soa[1], (const float *)soa[2],
                                  (const float *)soa[3], (const float *)soa[4], (const float *)soa[5], aos, n);
  } else {
    auto k = v ? k_soa_to_aos_d<true> : k_soa_to_aos_d<false>;
    k<<<grid_for(n), 256, 0, s>>>((const double *)soa[0], (const double *)soa[1], (const double *)soa[2],
                                  (const double *)soa[3], (const double *)soa[4], (const double *)soa[5], aos, n);
  }
}

void launch_convert_field(void *stream, const void *in, void *out, size_t n, int to_float) {
  cudaStream_t s = (cudaStream_t)stream;
  if (to_float)
    k_d2f<<<grid_for(n), 256, 0, s>>>((const double2 *)in, (float2 *)out, n);
  else
    k_f2d<<<grid_for(n), 256, 0, s>>>((const float2 *)in, (double2 *)out, n);
}

}  // namespace g4

// ---- FP64 instruction rate of the device (the roofline of the plain form) ----------

namespace {

// Eight independent chains of FP64 fused multiply-adds per thread: the FP64 pipe, not
// the dependent latency, bounds the rate. x -> a x + b with |a| < 1 stays bounded.
__global__ void k_dfma_chains(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = 1e-3 * (threadIdx.x + 1) + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int g4gpu_measure_fp64_rate(int device, double *instr_per_s) {
  if (!instr_per_s) return G4GPU_ERR_ARG;
  *instr_per_s = 0;
  if (cudaSetDevice(device) != cudaSuccess) return G4GPU_ERR_CUDA;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return G4GPU_ERR_CUDA;
  const int threads = 256, blocks = nsm * 8, iters = 4096;
  double *out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return G4GPU_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0;
  for (int rep = 0; rep < 4; rep++) {  // the first launch warms up; the best of the others
    cudaEventRecord(e0);
    k_dfma_chains<<<blocks, threads>>>(out, iters, 0.9999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0 || ms < best)) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || best <= 0) return G4GPU_ERR_CUDA;
  *instr_per_s = (double)blocks * threads * 8.0 * iters / (best * 1e-3);
  return G4GPU_OK;
}
