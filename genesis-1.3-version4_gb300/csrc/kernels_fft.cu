// FFT field solver of the undulator step (FieldSolverFFT, src/Core/FieldSolverFFT.cpp:64-114):
//   unfiltered:  u <- IFFT( FFT(u) * exp(K2 dz) ) / n^2 + 2 src
//   filtered:    u <- IFFT( FFT(u) * exp(K2 dz) + 2 FFT(src) * sigmoid ) / n^2
// with FFTW's sign convention (forward e^{-2 pi i jk/n}, backward e^{+...},
// unnormalised) and K2 = -i (dx^2 + dy^2) dk^2 / (2 xks) on the reference's
// shifted frequency map (FieldSolverFFT.cpp:131-145).
//
// The 2-D transform of each ngrid x ngrid slice is done as three passes over
// global memory, each in shared memory:
//   rows:    forward FFT of every row (and of the source rows when filtered)
//   columns: forward FFT of every column, the k-space propagator (and filtered
//            source), inverse FFT of every column
//   rows:    inverse FFT of every row, 1/n^2, + 2 src when unfiltered
// Every 1-D transform is a Stockham autosort mixed-radix FFT over the prime
// factors of ngrid (any ngrid: a prime factor p costs O(p) per point), with the
// n-th roots of unity in shared memory. Templated on the precision: double2 for
// the plain form, float2 for the mixed form.
#include <cuda_runtime.h>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

template <typename T2>
struct Real;
template <>
struct Real<double2> {
  typedef double T;
};
template <>
struct Real<float2> {
  typedef float T;
};

template <typename T2>
__device__ __forceinline__ T2 mk(typename Real<T2>::T x, typename Real<T2>::T y) {
  T2 r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename T2>
__device__ __forceinline__ T2 cm(T2 a, T2 b) {
  return mk<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One 1-D Stockham FFT of length n over `lines` lines stored with line stride
// `ls` in shared memory; the result ends in A (ping-pong through B). Roots W[m] =
// exp(-2 pi i m / n); the inverse uses conj(W). Each thread computes whole outputs
// of a stage: with radix r, sub-transform length ns and output index
// o = (j / ns) ns r + tt ns + k (k = j mod ns), the output is
//   sum_q in[j + q n/r] W^{q (k n/(ns r) + tt n/r) mod n},
// i.e. the twiddled radix-r butterfly in one pass, O(r) per output for any r.
template <typename T2>
__device__ void fft_lines(T2 *A, T2 *B, int ls, int lines, const FFTPlan &pl, const T2 *W,
                          bool inverse) {
  const int n = pl.n;
  int ns = 1;
  T2 *in = A, *out = B;
  for (int s = 0; s < pl.nstage; s++) {
    const int r = pl.radix[s];
    const int nb = n / r;
    const int nsr = ns * r;
    for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
      int line = t / n, o = t - line * n;
      int q1 = o / nsr, rem = o - q1 * nsr;
      int tt = rem / ns, k = rem - tt * ns;
      int j = q1 * ns + k;
      int e = k * (n / nsr) + tt * nb;  // < n
      const T2 *src = in + line * ls + j;
      T2 acc = src[0];
      int m = 0;
      for (int q = 1; q < r; q++) {
        m += e;
        if (m >= n) m -= n;
        T2 w = W[m];
        if (inverse) w.y = -w.y;
        T2 p = cm(src[q * nb], w);
        acc.x += p.x;
        acc.y += p.y;
      }
      out[line * ls + o] = acc;
    }
    __syncthreads();
    ns = nsr;
    T2 *tmp = in;
    in = out;
    out = tmp;
  }
  if (in != A) {
    for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
      int line = t / n, e = t - line * n;
      A[line * ls + e] = in[line * ls + e];
    }
    __syncthreads();
  }
}

// Row pass. mode 0: forward FFT of the rows of the field (and, with src_rows_out,
// of the source rows into that buffer); mode 1: inverse FFT of the rows, times
// `scale`, plus 2 src when `src` is given.
template <typename T2>
__global__ void k_fft_rows(T2 *__restrict__ field, const T2 *__restrict__ src,
                           T2 *__restrict__ src_rows_out, const T2 *__restrict__ roots,
                           FFTPlan pl, int ns, int first, int mode, double scale, int rows_per_cta) {
  extern __shared__ unsigned char smem_raw[];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *A = W + n;
  T2 *B = A + rows_per_cta * n;
  int ii = blockIdx.y;
  int i = (ii + first) % ns;
  size_t ncell = (size_t)n * n;
  int r0 = blockIdx.x * rows_per_cta;
  int lines = min(rows_per_cta, n - r0);
  for (int t = threadIdx.x; t < n; t += blockDim.x) W[t] = roots[t];
  for (int pass = 0; pass < ((mode == 0 && src_rows_out) ? 2 : 1); pass++) {
    T2 *base = pass == 0 ? field + (size_t)i * ncell : nullptr;
    const T2 *sbase = pass == 1 ? src + (size_t)ii * ncell : nullptr;
    for (int t = threadIdx.x; t < lines * n; t += blockDim.x)
      A[t] = pass == 0 ? base[(size_t)r0 * n + t] : sbase[(size_t)r0 * n + t];
    __syncthreads();
    fft_lines(A, B, n, lines, pl, W, mode == 1);
    if (mode == 0) {
      T2 *dst = pass == 0 ? base : src_rows_out + (size_t)ii * ncell;
      for (int t = threadIdx.x; t < lines * n; t += blockDim.x) dst[(size_t)r0 * n + t] = A[t];
    } else {
      typedef typename Real<T2>::T R;
      const T2 *s = src ? src + (size_t)ii * ncell + (size_t)r0 * n : nullptr;
      for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
        T2 v = A[t];
        T2 o = mk<T2>(v.x * (R)scale, v.y * (R)scale);
        if (s) {
          T2 sv = s[t];
          o.x += (R)2. * sv.x;
          o.y += (R)2. * sv.y;
        }
        base[(size_t)r0 * n + t] = o;
      }
    }
    __syncthreads();
  }
}

// Column pass: forward FFT of the columns, the propagator exp(K2 dz) (and the
// filtered source 2 FFT(src) sigmoid), inverse FFT of the columns.
// k2[ii] is Im(K2) and sig[ii] the sigmoid on the FFT index ii = ky n + kx.
template <typename T2>
__global__ void k_fft_cols(T2 *__restrict__ field, const T2 *__restrict__ srcf,
                           const T2 *__restrict__ roots, const typename Real<T2>::T *__restrict__ k2,
                           const typename Real<T2>::T *__restrict__ sig, double delz, FFTPlan pl,
                           int ns, int first, int cols_per_cta) {
  typedef typename Real<T2>::T R;
  extern __shared__ unsigned char smem_raw[];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *A = W + n;
  T2 *B = A + cols_per_cta * n;
  T2 *SA = B + cols_per_cta * n;  // filtered source columns (only with srcf)
  int ii = blockIdx.y;
  int i = (ii + first) % ns;
  size_t ncell = (size_t)n * n;
  int c0 = blockIdx.x * cols_per_cta;
  int lines = min(cols_per_cta, n - c0);
  T2 *u = field + (size_t)i * ncell;
  const T2 *sf = srcf ? srcf + (size_t)ii * ncell : nullptr;
  for (int t = threadIdx.x; t < n; t += blockDim.x) W[t] = roots[t];
  // transposed load: line c holds column c0 + c
  for (int t = threadIdx.x; t < n * cols_per_cta; t += blockDim.x) {
    int row = t / cols_per_cta, c = t - row * cols_per_cta;
    if (c < lines) {
      A[c * n + row] = u[(size_t)row * n + c0 + c];
      if (sf) SA[c * n + row] = sf[(size_t)row * n + c0 + c];
    }
  }
  __syncthreads();
  fft_lines(A, B, n, lines, pl, W, false);
  if (sf) fft_lines(SA, B, n, lines, pl, W, false);
  for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
    int c = t / n, ky = t - c * n;
    size_t kk = (size_t)ky * n + c0 + c;
    R ang = k2[kk] * (R)delz;
    R sn, cs;
    sincos(ang, &sn, &cs);
    T2 v = cm(A[t], mk<T2>(cs, sn));
    if (sf) {
      R g = (R)2. * sig[kk];
      v.x += g * SA[t].x;
      v.y += g * SA[t].y;
    }
    A[t] = v;
  }
  __syncthreads();
  fft_lines(A, B, n, lines, pl, W, true);
  for (int t = threadIdx.x; t < n * cols_per_cta; t += blockDim.x) {
    int row = t / cols_per_cta, c = t - row * cols_per_cta;
    if (c < lines) u[(size_t)row * n + c0 + c] = A[c * n + row];
  }
}

// lines per CTA so that the column pass (roots + 3 line buffers) fits in 227 KB
int fft_lines_per_cta(int n, int es) {
  int lines = 16;
  while (lines > 1 && (size_t)(n + 3 * lines * n) * es > 227u * 1024u) lines--;
  return lines;
}

template <typename T2>
void launch_fft(void *stream, void *field, const void *src, void *work, const void *roots,
                const void *k2, const void *sig, int filtered, double delz, const FFTPlan &pl,
                int ns, int first) {
  cudaStream_t s = (cudaStream_t)stream;
  const int n = pl.n;
  size_t es = sizeof(T2);
  const int lines = fft_lines_per_cta(n, (int)es);
  size_t smem_rows = (size_t)(n + 2 * lines * n) * es;
  size_t smem_cols = (size_t)(n + 3 * lines * n) * es;
  static unsigned long long configured = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured & (1ull << dev))) {
    cudaFuncSetAttribute(k_fft_rows<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_fft_cols<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    configured |= 1ull << dev;
  }
  dim3 grid((n + lines - 1) / lines, ns);
  T2 *f = (T2 *)field;
  const T2 *sr = (const T2 *)src;
  T2 *sfw = filtered ? (T2 *)work : nullptr;
  k_fft_rows<T2><<<grid, 256, smem_rows, s>>>(f, sr, sfw, (const T2 *)roots, pl, ns, first, 0, 1.0, lines);
  typedef typename Real<T2>::T R;
  k_fft_cols<T2><<<grid, 256, smem_cols, s>>>(f, sfw, (const T2 *)roots, (const R *)k2, (const R *)sig,
                                             delz, pl, ns, first, lines);
  k_fft_rows<T2><<<grid, 256, smem_rows, s>>>(f, filtered ? nullptr : sr, nullptr, (const T2 *)roots, pl,
                                             ns, first, 1, 1.0 / ((double)n * n), lines);
}

}  // namespace

int fft_max_ngrid(int mixed) {
  // one line per CTA at least: roots + 3 lines of ngrid complex values
  int es = mixed ? (int)sizeof(float2) : (int)sizeof(double2);
  return (int)(227u * 1024u / (4u * (unsigned)es));
}

void launch_fft_solve(void *stream, int mixed, void *field, const void *src, void *work,
                      const void *roots, const void *k2, const void *sig, int filtered, double delz,
                      const FFTPlan &pl, int ns, int first) {
  if (mixed)
    launch_fft<float2>(stream, field, src, work, roots, k2, sig, filtered, delz, pl, ns, first);
  else
    launch_fft<double2>(stream, field, src, work, roots, k2, sig, filtered, delz, pl, ns, first);
}

}  // namespace g4
