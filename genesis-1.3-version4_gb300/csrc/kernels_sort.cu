// One4one sorting of a window on the device: Beam::sort for one rank
// (src/Core/Beam.cpp:81-94) with Sorting::globalSort and Sorting::localSort
// (src/Util/Sorting.cpp:55-145, 198-474, run with doshift off as the reference does).
//
// A particle at phase theta in slice i sits at s = slen i + theta (slen = 2 pi sample).
// Outside the window (s < 0 or s > slen nslice) it leaves the run (the single rank has no
// neighbour to send it to); else it moves floor(theta / slen) slices, its phase reduced
// by that many slice lengths. Every slice then holds its staying particles, in their
// previous order, followed by the arrivals; the reference's removal by swapping with
// the last element orders them differently, which changes only the summation order of
// later per-slice sums. The arrivals take their slots by atomic increments, so their
// order behind the staying particles varies from run to run (and with it the
// summation order); when a slice overflows its capacity, which arrivals are lost
// varies too. The set of particles in a slice without overflow does not.
//
// Three kernels, one CTA per slice: (1) count each slice's staying particles and every
// slice's arrivals; (2) compact the staying particles in order into the scratch arrays
// (a CTA-wide scan of the stay flags) and place the arrivals behind them (an atomic slot
// per destination); (3) set the slices' counts and currents (np ce / slicelength,
// Beam.cpp:87-89). Particles beyond a slice's capacity are counted, not written.
// Compiled with --fmad=false: theta - slen atar rounds as the reference's does.
#include <cuda_runtime.h>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

constexpr int kSortThreads = 256;

struct SortArgs {
  void *src[6];  // gamma, theta, x, y, px, py of the window
  void *dst[6];  // scratch arrays of the same layout
  int *count;    // particles per slice, updated
  double *current;
  int *stay, *arr, *fill, *over;  // [ns] each, then the overflow counter
  int ns, cap;
  double slen, invslen, keepmax, slicelength;  // FP64 form
  long long unit;                              // Q32.32 turns of one slice (FP32 form: integer sample)
};

// FP64 form: theta in radians. Returns the destination slice (the slice itself when the
// particle stays) and the reduced phase, or -1 when the particle leaves the window.
// Sorting.cpp:373-374, 391-406 (fillPushVectors) and 90-100 (localSort).
struct PlainSort {
  static __device__ __forceinline__ constexpr int size(int) { return 8; }
  static __device__ __forceinline__ int dest(const SortArgs &a, int is, const void *th_arr, size_t o, double &thd,
                                             long long &) {
    const double theta = reinterpret_cast<const double *>(th_arr)[o];
    const double s = a.slen * (double)is + theta;
    if (s < 0 || s > a.keepmax) return -1;
    const int atar = (int)floor(theta * a.invslen);
    thd = theta;
    if (atar == 0) return is;
    const int d = is + atar;
    // the reference indexes out of its slices there (a particle on the window's end
    // within rounding): the particle leaves
    if (d < 0 || d >= a.ns) return -1;
    thd = theta - a.slen * atar;
    return d;
  }
  static __device__ __forceinline__ void put_theta(void *th_arr, size_t o, double thd, long long) {
    reinterpret_cast<double *>(th_arr)[o] = thd;
  }
};

// FP32 form: theta as a Q32.32 turn count, exact integer arithmetic (integer sample)
struct MixedSort {
  static __device__ __forceinline__ constexpr int size(int k) { return k == 1 ? 8 : 4; }
  static __device__ __forceinline__ int dest(const SortArgs &a, int is, const void *th_arr, size_t o, double &,
                                             long long &thq) {
    const long long th = reinterpret_cast<const long long *>(th_arr)[o];
    const long long s = a.unit * (long long)is + th;
    if (s < 0 || s > a.unit * (long long)a.ns) return -1;
    const long long atar = th >= 0 ? th / a.unit : -((-th + a.unit - 1) / a.unit);
    thq = th;
    if (atar == 0) return is;
    const long long d = is + atar;
    if (d < 0 || d >= a.ns) return -1;
    thq = th - atar * a.unit;
    return (int)d;
  }
  static __device__ __forceinline__ void put_theta(void *th_arr, size_t o, double, long long thq) {
    reinterpret_cast<long long *>(th_arr)[o] = thq;
  }
};

template <class F>
__device__ __forceinline__ void copy_particle(const SortArgs &a, size_t from, size_t to) {
#pragma unroll
  for (int k = 0; k < 6; k++) {
    if (k == 1) continue;  // theta is written by the caller
    if (F::size(k) == 8)
      reinterpret_cast<double *>(a.dst[k])[to] = reinterpret_cast<const double *>(a.src[k])[from];
    else
      reinterpret_cast<float *>(a.dst[k])[to] = reinterpret_cast<const float *>(a.src[k])[from];
  }
}

template <class F>
__global__ void __launch_bounds__(kSortThreads) k_sort_count(SortArgs a) {
  __shared__ int red[kSortThreads / 32];
  const int is = blockIdx.x, n = min(a.count[is], a.cap);
  int stays = 0;
  for (int ip = threadIdx.x; ip < n; ip += blockDim.x) {
    double thd;
    long long thq;
    const int d = F::dest(a, is, a.src[1], (size_t)is * a.cap + ip, thd, thq);
    if (d == is)
      stays++;
    else if (d >= 0)
      atomicAdd(&a.arr[d], 1);
  }
  for (int o = 16; o > 0; o >>= 1) stays += __shfl_xor_sync(0xffffffffu, stays, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = stays;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    a.stay[is] = t;
  }
}

template <class F>
__global__ void __launch_bounds__(kSortThreads) k_sort_place(SortArgs a) {
  __shared__ int woff[kSortThreads / 32];
  __shared__ int base;
  const int is = blockIdx.x, n = min(a.count[is], a.cap), lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  // rounds of blockDim particles: a stable scan of the stay flags within the round
  for (int r0 = 0; r0 < n; r0 += blockDim.x) {
    const int ip = r0 + threadIdx.x;
    int d = -1;
    double thd = 0;
    long long thq = 0;
    const size_t from = (size_t)is * a.cap + ip;
    if (ip < n) d = F::dest(a, is, a.src[1], from, thd, thq);
    const bool st = d == is;
    const unsigned m = __ballot_sync(0xffffffffu, st);
    if (lane == 0) woff[w] = __popc(m);
    __syncthreads();
    int before = base, total = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      if (k < w) before += woff[k];
      total += woff[k];
    }
    if (st) {
      const size_t to = (size_t)is * a.cap + before + __popc(m & ((1u << lane) - 1u));
      copy_particle<F>(a, from, to);
      F::put_theta(a.dst[1], to, thd, thq);
    } else if (d >= 0) {
      const int slot = a.stay[d] + atomicAdd(&a.fill[d], 1);
      if (slot < a.cap) {
        const size_t to = (size_t)d * a.cap + slot;
        copy_particle<F>(a, from, to);
        F::put_theta(a.dst[1], to, thd, thq);
      } else {
        atomicAdd(a.over, 1);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
}

__global__ void k_sort_finish(SortArgs a) {
  const int is = blockIdx.x * blockDim.x + threadIdx.x;
  if (is >= a.ns) return;
  const int n = min(a.stay[is] + a.arr[is], a.cap);
  a.count[is] = n;
  // Beam::sort, Beam.cpp:87-89
  a.current[is] = static_cast<double>(n) * kCe / a.slicelength;
}

}  // namespace

// scratch: 6 arrays of ns * cap elements (the beam's layout) and 3 ns + 1 ints
void launch_sort(void *stream, int mixed, const DeviceBeam &b, void *const *scratch, int *iscratch, int ns, int cap,
                 double lambda0, double sample) {
  cudaStream_t s = (cudaStream_t)stream;
  SortArgs a{};
  void *src[6] = {b.gamma, b.theta, b.x, b.y, b.px, b.py};
  for (int k = 0; k < 6; k++) {
    a.src[k] = src[k];
    a.dst[k] = scratch[k];
  }
  a.count = b.count;
  a.current = b.current;
  a.stay = iscratch;
  a.arr = iscratch + ns;
  a.fill = iscratch + 2 * ns;
  a.over = iscratch + 3 * ns;
  a.ns = ns;
  a.cap = cap;
  // Beam::initSorting, Beam.cpp:73-78: slen = 2 pi slicelength / reflength
  const double slicelength = lambda0 * sample;
  a.slicelength = slicelength;
  a.slen = 4 * asin(1.) * slicelength / lambda0;
  a.invslen = 1. / a.slen;
  a.keepmax = a.slen * (unsigned long)ns;
  a.unit = (long long)llrint(sample) << 32;
  cudaMemsetAsync(iscratch + ns, 0, (2 * (size_t)ns + 1) * sizeof(int), s);
  if (mixed) {
    k_sort_count<MixedSort><<<ns, kSortThreads, 0, s>>>(a);
    k_sort_place<MixedSort><<<ns, kSortThreads, 0, s>>>(a);
  } else {
    k_sort_count<PlainSort><<<ns, kSortThreads, 0, s>>>(a);
    k_sort_place<PlainSort><<<ns, kSortThreads, 0, s>>>(a);
  }
  k_sort_finish<<<(ns + 255) / 256, 256, 0, s>>>(a);
}

}  // namespace g4
