// Per-slice features and corrections of the learned coarse-step closure.
//
// Features of one slice (kClosureNin floats, unnormalised):
//   0-5    Re, Im of the bunching <exp(i h theta)>, h = 1, 2, 3
//   6, 7   <gamma> - gamma0, rms of gamma
//   8      log(1 + |u_axis|^2 / u0^2), u_axis the field on the grid centre
//   9, 10  cos and sin of arg(u_axis)
//   11-26  log(1 + |c_mn|^2 / c0^2), c_mn the projections of the field slice on the
//          Gauss-Hermite modes HG_mn, m, n = 0..3 (basis tables from the host)
//   27     current / 1 kA
//   28-31  zero
// Corrections of one slice (kClosureNout floats): phase shift of every particle,
// energy shift of every particle, relative amplitude and phase of the field slice.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

constexpr float kTwoPiF = 6.283185307f;
constexpr float kRadPerUnit = 6.283185307f / 4294967296.0f;

template <int BS>
__device__ __forceinline__ float bsumf(float v, float *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float r = 0.f;
  if (threadIdx.x == 0)
    for (int i = 0; i < BS / 32; i++) r += sh[i];
  return r;
}

// particle phase (radians, reduced) for either storage of theta
__device__ __forceinline__ float phase_h(const void *theta, size_t i, int mixed, int h) {
  if (mixed) {
    long long t = reinterpret_cast<const long long *>(theta)[i];
    return (float)(int)((unsigned)t * (unsigned)h) * kRadPerUnit;
  }
  double th = reinterpret_cast<const double *>(theta)[i] * (double)h;
  return (float)(th - 6.283185307179586 * rint(th * 0.15915494309189535));
}
__device__ __forceinline__ float gamma_of(const void *g, size_t i, int mixed, double gref) {
  return mixed ? reinterpret_cast<const float *>(g)[i]
               : (float)(reinterpret_cast<const double *>(g)[i] - gref);
}
__device__ __forceinline__ float2 field_at(const void *f, size_t i, int mixed) {
  if (mixed) return reinterpret_cast<const float2 *>(f)[i];
  double2 v = reinterpret_cast<const double2 *>(f)[i];
  return make_float2((float)v.x, (float)v.y);
}

template <int BS>
__global__ void __launch_bounds__(BS) k_features(const void *theta, const void *gam, const double *current,
                                                 const void *field, const float *basis, int mixed,
                                                 double gref, int ns, int np, int ng, int first, float u0,
                                                 float c0, float *out) {
  constexpr int NW = BS / 32;
  extern __shared__ __align__(16) float fsm[];
  float *hb = fsm;                                         // [4][ng] 1-D Gauss-Hermite factors
  float2 *rp = reinterpret_cast<float2 *>(fsm + 4 * ng);  // [4][ng] row projections (16 ng bytes on)
  __shared__ float red[NW][8];
  __shared__ float2 cm[16];
  const int is = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < 4 * ng; t += BS) hb[t] = basis[t];
  // particles: bunching b1..b3, mean and second moment of gamma
  const size_t base = (size_t)is * np;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int ip = threadIdx.x; ip < np; ip += BS) {
#pragma unroll
    for (int h = 1; h <= 3; h++) {
      float s, c;
      __sincosf(phase_h(theta, base + ip, mixed, h), &s, &c);
      acc[2 * (h - 1)] += c;
      acc[2 * (h - 1) + 1] += s;
    }
    float g = gamma_of(gam, base + ip, mixed, gref);
    acc[6] += g;
    acc[7] += g * g;
  }
#pragma unroll
  for (int q = 0; q < 8; q++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
    if (lane == 0) red[warp][q] = acc[q];
  }
  __syncthreads();  // hb and the particle sums
  // field slice: HG_mn projections c_mn = sum_iy h_n(iy) sum_ix h_m(ix) u(ix, iy); each
  // warp forms the four row projections of its rows
  const size_t ncell = (size_t)ng * ng;
  const size_t fb = (size_t)((is + first) % ns) * ncell;
  for (int iy = warp; iy < ng; iy += NW) {
    float2 r[4] = {};
    for (int ix = lane; ix < ng; ix += 32) {
      const float2 u = field_at(field, fb + (size_t)iy * ng + ix, mixed);
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const float b = hb[m * ng + ix];
        r[m].x += b * u.x;
        r[m].y += b * u.y;
      }
    }
#pragma unroll
    for (int m = 0; m < 4; m++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        r[m].x += __shfl_down_sync(0xffffffffu, r[m].x, o);
        r[m].y += __shfl_down_sync(0xffffffffu, r[m].y, o);
      }
      if (lane == 0) rp[m * ng + iy] = r[m];
    }
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    const int m = threadIdx.x / 4, n = threadIdx.x % 4;
    float2 c = make_float2(0.f, 0.f);
    for (int iy = 0; iy < ng; iy++) {
      const float b = hb[n * ng + iy];
      const float2 v = rp[m * ng + iy];
      c.x += b * v.x;
      c.y += b * v.y;
    }
    cm[threadIdx.x] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float res[8];
    for (int q = 0; q < 8; q++) {
      float v = 0.f;
      for (int w = 0; w < NW; w++) v += red[w][q];
      res[q] = v;
    }
    float *o = out + (size_t)is * kClosureNin;
    float inv = 1.f / (float)np;
    for (int q = 0; q < 6; q++) o[q] = res[q] * inv;
    float mg = res[6] * inv;
    o[6] = mg;
    o[7] = sqrtf(fmaxf(res[7] * inv - mg * mg, 0.f));
    float2 ua = field_at(field, fb + (size_t)(ng / 2) * ng + ng / 2, mixed);
    float a2 = ua.x * ua.x + ua.y * ua.y;
    o[8] = log1pf(a2 / (u0 * u0));
    float am = sqrtf(a2);
    o[9] = am > 0 ? ua.x / am : 1.f;
    o[10] = am > 0 ? ua.y / am : 0.f;
    for (int q = 0; q < 16; q++) o[11 + q] = log1pf((cm[q].x * cm[q].x + cm[q].y * cm[q].y) / (c0 * c0));
    o[27] = (float)(current[is] * 1e-3);
    for (int q = 28; q < kClosureNin; q++) o[q] = 0.f;
  }
}

// applies corr[is][0..3] to the particles and the field slice of slice is
__global__ void k_apply(void *theta, void *gam, void *field, const float *corr, int mixed, int ns, int np,
                        int ng, int first) {
  int is = blockIdx.y;
  const float *c = corr + (size_t)is * kClosureNout;
  float dth = c[0], dg = c[1], da = c[2], dphi = c[3];
  size_t base = (size_t)is * np;
  for (int ip = blockIdx.x * blockDim.x + threadIdx.x; ip < np; ip += gridDim.x * blockDim.x) {
    if (mixed) {
      long long *t = reinterpret_cast<long long *>(theta);
      float turns = dth * (1.0f / kTwoPiF);
      float k = floorf(turns);
      unsigned fu = (unsigned)((turns - k) * 4294967296.0f);
      t[base + ip] += ((long long)(int)k << 32) + (long long)fu;
      reinterpret_cast<float *>(gam)[base + ip] += dg;
    } else {
      reinterpret_cast<double *>(theta)[base + ip] += (double)dth;
      reinterpret_cast<double *>(gam)[base + ip] += (double)dg;
    }
  }
  size_t ncell = (size_t)ng * ng;
  size_t fb = (size_t)((is + first) % ns) * ncell;
  float s, co;
  __sincosf(dphi, &s, &co);
  float fr = (1.f + da) * co, fi = (1.f + da) * s;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncell; i += (size_t)gridDim.x * blockDim.x) {
    if (mixed) {
      float2 *f = reinterpret_cast<float2 *>(field) + fb;
      float2 u = f[i];
      f[i] = make_float2(u.x * fr - u.y * fi, u.x * fi + u.y * fr);
    } else {
      double2 *f = reinterpret_cast<double2 *>(field) + fb;
      double2 u = f[i];
      f[i] = make_double2(u.x * fr - u.y * fi, u.x * fi + u.y * fr);
    }
  }
}

// Training targets of one slice: what the fine solve did beyond the coarse one over
// the same interval, in the form of the corrections: mean phase and energy
// difference of the particles, and the complex ratio r = <u_c, u_f> / <u_c, u_c>
// of the field slices as relative amplitude |r| - 1 and phase arg r.
template <int BS>
__global__ void __launch_bounds__(BS) k_targets(const void *th_c, const void *g_c, const void *f_c,
                                                const void *th_f, const void *g_f, const void *f_f, int mixed,
                                                int ns, int np, int ng, int first_c, int first_f, float *out) {
  __shared__ float sh[BS / 32];
  int is = blockIdx.x;
  size_t base = (size_t)is * np;
  float a0 = 0.f, a1 = 0.f;
  for (int ip = threadIdx.x; ip < np; ip += BS) {
    size_t i = base + ip;
    float dth, dg;
    if (mixed) {
      long long d = reinterpret_cast<const long long *>(th_f)[i] - reinterpret_cast<const long long *>(th_c)[i];
      dth = (float)((double)d * (6.283185307179586 / 4294967296.0));
      dg = reinterpret_cast<const float *>(g_f)[i] - reinterpret_cast<const float *>(g_c)[i];
    } else {
      dth = (float)(reinterpret_cast<const double *>(th_f)[i] - reinterpret_cast<const double *>(th_c)[i]);
      dg = (float)(reinterpret_cast<const double *>(g_f)[i] - reinterpret_cast<const double *>(g_c)[i]);
    }
    a0 += dth;
    a1 += dg;
  }
  size_t ncell = (size_t)ng * ng;
  size_t bc = (size_t)((is + first_c) % ns) * ncell, bf = (size_t)((is + first_f) % ns) * ncell;
  float nr = 0.f, ni = 0.f, dd = 0.f;
  for (size_t i = threadIdx.x; i < ncell; i += BS) {
    float2 c = field_at(f_c, bc + i, mixed), f = field_at(f_f, bf + i, mixed);
    nr += c.x * f.x + c.y * f.y;
    ni += c.x * f.y - c.y * f.x;
    dd += c.x * c.x + c.y * c.y;
  }
  float s0 = bsumf<BS>(a0, sh), s1 = bsumf<BS>(a1, sh);
  float rr = bsumf<BS>(nr, sh), ri = bsumf<BS>(ni, sh), d2 = bsumf<BS>(dd, sh);
  if (threadIdx.x == 0) {
    float *o = out + (size_t)is * kClosureNout;
    o[0] = s0 / (float)np;
    o[1] = s1 / (float)np;
    if (d2 > 0.f) {
      float xr = rr / d2, xi = ri / d2;
      o[2] = sqrtf(xr * xr + xi * xi) - 1.f;
      o[3] = atan2f(xi, xr);
    } else {
      o[2] = 0.f;
      o[3] = 0.f;
    }
  }
}

// y = (x - mean) / std, into a row-padded BF16 matrix [rows][ld]
__global__ void k_normalize(const float *x, const float *mean, const float *stdv, void *yb, int rows, int n,
                            int ld) {
  size_t total = (size_t)rows * ld;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(i % ld);
    float v = 0.f;
    if (c < n) {
      size_t r = i / ld;
      v = (x[r * n + c] - mean[c]) / stdv[c];
    }
    reinterpret_cast<__nv_bfloat16 *>(yb)[i] = __float2bfloat16(v);
  }
}

// out[r][c] = y[r][c] * scale[c] + shift[c] for the first n of ld columns
__global__ void k_denormalize(const float *y, const float *scale, const float *shift, float *out, int rows,
                              int n, int ld) {
  size_t total = (size_t)rows * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(i % n);
    size_t r = i / n;
    out[i] = y[r * ld + c] * scale[c] + shift[c];
  }
}

}  // namespace

void closure_features(void *stream, const void *theta, const void *gam, const double *current,
                      const void *field, const float *basis, int mixed, double gref, int ns, int np, int ng,
                      int first, float u0, float c0, float *out) {
  // shared memory: the 1-D factors [4][ng] floats, then the row projections [4][ng]
  // float2 (at 16 ng bytes, aligned for float2)
  const size_t smem = (size_t)4 * ng * sizeof(float) + (size_t)4 * ng * sizeof(float2);
  if (smem > 48u * 1024u)
    cudaFuncSetAttribute(k_features<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_features<256><<<ns, 256, smem, (cudaStream_t)stream>>>(theta, gam, current, field, basis, mixed, gref, ns, np,
                                                           ng, first, u0, c0, out);
}

void closure_apply(void *stream, void *theta, void *gam, void *field, const float *corr, int mixed, int ns,
                   int np, int ng, int first) {
  dim3 grid(8, ns);
  k_apply<<<grid, 256, 0, (cudaStream_t)stream>>>(theta, gam, field, corr, mixed, ns, np, ng, first);
}

void closure_targets(void *stream, const void *th_c, const void *g_c, const void *f_c, const void *th_f,
                     const void *g_f, const void *f_f, int mixed, int ns, int np, int ng, int first_c,
                     int first_f, float *out) {
  k_targets<256><<<ns, 256, 0, (cudaStream_t)stream>>>(th_c, g_c, f_c, th_f, g_f, f_f, mixed, ns, np, ng,
                                                       first_c, first_f, out);
}

void closure_normalize(void *stream, const float *x, const float *mean, const float *stdv, void *yb, int rows,
                       int n, int ld) {
  size_t t = (size_t)rows * ld;
  unsigned b = (unsigned)((t + 255) / 256 > 4096 ? 4096 : (t + 255) / 256);
  k_normalize<<<b, 256, 0, (cudaStream_t)stream>>>(x, mean, stdv, yb, rows, n, ld);
}

void closure_denormalize(void *stream, const float *y, const float *scale, const float *shift, float *out,
                         int rows, int n, int ld) {
  size_t t = (size_t)rows * n;
  unsigned b = (unsigned)((t + 255) / 256 > 4096 ? 4096 : (t + 255) / 256);
  k_denormalize<<<b, 256, 0, (cudaStream_t)stream>>>(y, scale, shift, out, rows, n, ld);
}

}  // namespace g4
