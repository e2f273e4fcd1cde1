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
// Every 1-D transform is a Stockham autosort mixed-radix FFT over the factors of
// ngrid (radices 2, 3, 4, 5, 7, 8, 9, 11, 13, 15, 16, 17 as register butterflies;
// any other prime factor p as an O(p)-per-point stage), with the n-th roots of
// unity in shared memory. Templated on the precision: double2 for
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

// One radix-R Stockham stage over `lines` lines (line stride `ls`) from `in` to
// `out`, one butterfly per thread at a time, held in registers. With ns the product
// of the earlier radices and nb = n / R, butterfly j (k = j mod ns) reads
// in[j + q nb], q < R, multiplies input q by the twiddle W^{q k n/(ns R)}, takes the
// R-point DFT, and writes output t to out[(j - k) R + t ns + k]:
//   out[...] = sum_q in[j + q nb] W^{q (k n/(ns R) + t n/R)},
// the stage of the transform with roots W[m] = exp(-2 pi i m / n) (conj(W) when
// inverse). The R-point DFT's roots exp(-2 pi i m / R) are the table's W[m n / R],
// read once per stage into registers.
template <typename T2>
__device__ __forceinline__ T2 add(T2 a, T2 b) {
  return mk<T2>(a.x + b.x, a.y + b.y);
}
template <typename T2>
__device__ __forceinline__ T2 sub(T2 a, T2 b) {
  return mk<T2>(a.x - b.x, a.y - b.y);
}

// In-place R-point DFT y_t = sum_q x_q w^{q t}, w = exp(-+ 2 pi i / R), of x[0..R)
// with the roots w^m = wr[m S] (R S = R0; the conjugate is taken when INV).
// Odd prime R: the pairs (t, R - t) share the sums over x_m + x_{R-m} (real cosine
// weights) and x_m - x_{R-m} (real sine weights), so that each output costs R - 1
// real multiply-adds per component. Composite R = P M: M-point DFTs of the P
// interleaved subsequences joined by twiddles and P-point DFTs (decimation in
// time; for P = 2 the radix-2 split).
__host__ __device__ constexpr int small_factor(int r) {
  for (int p = 2; p * p <= r; p++)
    if (r % p == 0) return p;
  return r;
}

template <int R, int S, bool INV, typename T2, int R0>
__device__ __forceinline__ void dft(T2 *x, const T2 (&wr)[R0]) {
  typedef typename Real<T2>::T Rt;
  if constexpr (R == 1) {
    return;
  } else if constexpr (R == 2) {
    T2 a = x[0], b = x[1];
    x[0] = add(a, b);
    x[1] = sub(a, b);
  } else if constexpr (R == 4) {
    // w = -i forward, +i inverse: exact
    T2 t0 = add(x[0], x[2]), t1 = sub(x[0], x[2]), t2 = add(x[1], x[3]), t3 = sub(x[1], x[3]);
    T2 jt3 = INV ? mk<T2>(-t3.y, t3.x) : mk<T2>(t3.y, -t3.x);  // w t3
    x[0] = add(t0, t2);
    x[2] = sub(t0, t2);
    x[1] = add(t1, jt3);
    x[3] = sub(t1, jt3);
  } else if constexpr (small_factor(R) != R) {
    // R = P M: the P interleaved subsequences x[P i + s] of length M, their M-point
    // DFTs, the twiddles w^{s k}, and P-point DFTs across them (decimation in time):
    //   y_{k + t M} = sum_s w^{s k} w_P^{s t} DFT_M(x_s)_k
    constexpr int P = small_factor(R), M = R / P;
    T2 sub[P][M];
#pragma unroll
    for (int sidx = 0; sidx < P; sidx++)
#pragma unroll
      for (int i = 0; i < M; i++) sub[sidx][i] = x[P * i + sidx];
#pragma unroll
    for (int sidx = 0; sidx < P; sidx++) dft<M, P * S, INV>(sub[sidx], wr);
#pragma unroll
    for (int k = 0; k < M; k++) {
      T2 y[P];
#pragma unroll
      for (int sidx = 0; sidx < P; sidx++) {
        if (sidx == 0 || k == 0) {
          y[sidx] = sub[sidx][k];
        } else {
          T2 w = wr[sidx * k * S];
          if (INV) w.y = -w.y;
          y[sidx] = cm(sub[sidx][k], w);
        }
      }
      dft<P, M * S, INV>(y, wr);
#pragma unroll
      for (int t = 0; t < P; t++) x[k + t * M] = y[t];
    }
  } else {
    constexpr int H = (R - 1) / 2;
    T2 a[H + 1], b[H + 1];
    T2 y0 = x[0];
#pragma unroll
    for (int m = 1; m <= H; m++) {
      a[m] = add(x[m], x[R - m]);
      b[m] = sub(x[m], x[R - m]);
      y0 = add(y0, a[m]);
    }
#pragma unroll
    for (int t = 1; t <= H; t++) {
      T2 A = x[0];
      Rt bx = 0, by = 0;
#pragma unroll
      for (int m = 1; m <= H; m++) {
        const int id = (m * t) % R;
        // w^{id} = cos(2 pi id / R) -+ i sin(2 pi id / R); wr holds the forward roots
        const Rt c = wr[id * S].x, sn = -wr[id * S].y;
        A.x += c * a[m].x;
        A.y += c * a[m].y;
        bx += sn * b[m].x;
        by += sn * b[m].y;
      }
      // forward: y_t = A - i B, y_{R-t} = A + i B; inverse: the other way round
      if (!INV) {
        x[t] = mk<T2>(A.x + by, A.y - bx);
        x[R - t] = mk<T2>(A.x - by, A.y + bx);
      } else {
        x[t] = mk<T2>(A.x - by, A.y + bx);
        x[R - t] = mk<T2>(A.x + by, A.y - bx);
      }
    }
    x[0] = y0;
  }
}

template <int R, bool INV, typename T2>
__device__ void stage_r(const T2 *in, T2 *out, int ls, int lines, int n, int ns, const T2 *W) {
  const int nb = n / R;
  const int tws = n / (ns * R);
  T2 wr[R];
#pragma unroll
  for (int m = 0; m < R; m++) wr[m] = W[m * nb];
  const int total = lines * nb;
  // butterfly b = line nb + j, k = j mod ns, advanced by the CTA's stride without
  // divisions (ns divides nb, so j wrapping past nb leaves k unchanged)
  const int T = blockDim.x;
  int line = threadIdx.x / nb, j = threadIdx.x - line * nb, k = j % ns;
  const int dl = T / nb, dj = T - dl * nb, dk = dj % ns;
  for (int b = threadIdx.x; b < total; b += T) {
    const T2 *src = in + line * ls + j;
    T2 x[R];
#pragma unroll
    for (int q = 0; q < R; q++) x[q] = src[q * nb];
    if (ns > 1) {
      const int e1 = k * tws;
      int e = 0;
#pragma unroll
      for (int q = 1; q < R; q++) {
        e += e1;  // q k tws < n
        T2 w = W[e];
        if (INV) w.y = -w.y;
        x[q] = cm(x[q], w);
      }
    }
    dft<R, 1, INV>(x, wr);
    T2 *dst = out + line * ls + (j - k) * R + k;
#pragma unroll
    for (int t = 0; t < R; t++) dst[t * ns] = x[t];
    line += dl;
    j += dj;
    k += dk;
    if (k >= ns) k -= ns;
    if (j >= nb) {
      j -= nb;
      line++;
    }
  }
}

// Stage of any radix r: each output is the O(r) sum over its butterfly's inputs
// with the twiddled root read from the table (radices without a register DFT).
template <typename T2>
__device__ void stage_any(const T2 *in, T2 *out, int ls, int lines, int n, int ns, int r, const T2 *W,
                          bool inverse) {
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
}

template <bool INV, typename T2>
__device__ __forceinline__ void stage(const T2 *in, T2 *out, int ls, int lines, int n, int ns, int r,
                                      const T2 *W) {
  switch (r) {
    case 2: stage_r<2, INV>(in, out, ls, lines, n, ns, W); break;
    case 3: stage_r<3, INV>(in, out, ls, lines, n, ns, W); break;
    case 4: stage_r<4, INV>(in, out, ls, lines, n, ns, W); break;
    case 5: stage_r<5, INV>(in, out, ls, lines, n, ns, W); break;
    case 7: stage_r<7, INV>(in, out, ls, lines, n, ns, W); break;
    case 8: stage_r<8, INV>(in, out, ls, lines, n, ns, W); break;
    case 9: stage_r<9, INV>(in, out, ls, lines, n, ns, W); break;
    case 11: stage_r<11, INV>(in, out, ls, lines, n, ns, W); break;
    case 13: stage_r<13, INV>(in, out, ls, lines, n, ns, W); break;
    case 15: stage_r<15, INV>(in, out, ls, lines, n, ns, W); break;
    case 16: stage_r<16, INV>(in, out, ls, lines, n, ns, W); break;
    case 17: stage_r<17, INV>(in, out, ls, lines, n, ns, W); break;
    default: stage_any(in, out, ls, lines, n, ns, r, W, INV); break;
  }
}

// One 1-D Stockham FFT of length n over `lines` lines stored with line stride `ls`
// in shared memory, the stages of the plan's radices in turn; the result ends in A
// (ping-pong through B). Roots W[m] = exp(-2 pi i m / n); the inverse uses conj(W).
template <typename T2>
__device__ void fft_lines(T2 *A, T2 *B, int ls, int lines, const FFTPlan &pl, const T2 *W,
                          bool inverse) {
  const int n = pl.n;
  int ns = 1;
  T2 *in = A, *out = B;
  for (int s = 0; s < pl.nstage; s++) {
    const int r = pl.radix[s];
    if (inverse)
      stage<true>(in, out, ls, lines, n, ns, r, W);
    else
      stage<false>(in, out, ls, lines, n, ns, r, W);
    __syncthreads();
    ns *= r;
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

// Asynchronous copy of one complex element from global to shared memory
// (cp.async: 8 bytes for float2, 16 for double2; both addresses are aligned to the
// element's size), so that a CTA has all its loads in flight at once.
template <typename T2>
__device__ __forceinline__ void cp_elem(T2 *dst, const T2 *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T2) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// waits until at most N of this thread's committed groups are pending
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Row pass over `rows_per_cta` rows of one slice. mode 0: forward FFT of the rows of
// the field (and, with src_rows_out, of the source rows into that buffer); mode 1:
// inverse FFT of the rows, times `scale`, plus 2 src when `src` is given. The field
// rows go to A and the second input (the source rows) to C by asynchronous copies
// issued together; the transform of A starts as soon as A has landed.
// Two CTAs per SM in FP32 (at most 128 registers a thread).
template <typename T2>
__global__ void __launch_bounds__(256, sizeof(T2) == 8 ? 2 : 1)
    k_fft_rows(T2 *__restrict__ field, const T2 *__restrict__ src, T2 *__restrict__ src_rows_out,
               const T2 *__restrict__ roots, FFTPlan pl, int ns, int first, int mode, double scale,
               int rows_per_cta) {
  typedef typename Real<T2>::T R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *A = W + n;
  T2 *B = A + rows_per_cta * n;
  T2 *C = B + rows_per_cta * n;
  const int ii = blockIdx.y;
  const int i = (ii + first) % ns;
  const size_t ncell = (size_t)n * n;
  const int r0 = blockIdx.x * rows_per_cta;
  const int lines = min(rows_per_cta, n - r0);
  const int cnt = lines * n;
  T2 *base = field + (size_t)i * ncell + (size_t)r0 * n;
  const T2 *sb = src ? src + (size_t)ii * ncell + (size_t)r0 * n : nullptr;
  for (int t = threadIdx.x; t < n; t += blockDim.x) cp_elem(W + t, roots + t);
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) cp_elem(A + t, base + t);
  cp_commit();
  if (sb)
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) cp_elem(C + t, sb + t);
  cp_commit();
  cp_wait<1>();
  __syncthreads();
  fft_lines(A, B, n, lines, pl, W, mode == 1);
  if (mode == 0) {
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) base[t] = A[t];
    if (src_rows_out) {
      cp_wait<0>();
      __syncthreads();
      fft_lines(C, B, n, lines, pl, W, false);
      T2 *dst = src_rows_out + (size_t)ii * ncell + (size_t)r0 * n;
      for (int t = threadIdx.x; t < cnt; t += blockDim.x) dst[t] = C[t];
    }
  } else {
    cp_wait<0>();
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      T2 v = A[t];
      T2 o = mk<T2>(v.x * (R)scale, v.y * (R)scale);
      if (sb) {
        T2 sv = C[t];
        o.x += (R)2. * sv.x;
        o.y += (R)2. * sv.y;
      }
      base[t] = o;
    }
  }
}

// sin and cos of the propagator's phase: FP64 library sincos for the plain form;
// in FP32 the phase is first reduced to [-pi, pi] (the FP32 phase itself carries
// an error of ~6e-8 of its size) and the fast hardware approximation taken
__device__ __forceinline__ void phase_sincos(double a, double *sn, double *cs) { sincos(a, sn, cs); }
__device__ __forceinline__ void phase_sincos(float a, float *sn, float *cs) {
  const float two_pi = 6.283185307179586f;
  a -= two_pi * rintf(a * (1.0f / two_pi));
  __sincosf(a, sn, cs);
}

// Column pass over `cols_per_cta` columns of one slice: forward FFT of the columns,
// the propagator exp(K2 dz) (and the filtered source 2 FFT(src) sigmoid), inverse
// FFT of the columns. k2t and sigt hold Im(K2) and the sigmoid transposed,
// k2t[kx n + ky] for the FFT index (ky, kx), so that the reads of a column are
// contiguous.
template <typename T2>
__global__ void __launch_bounds__(256, sizeof(T2) == 8 ? 2 : 1)
    k_fft_cols(T2 *__restrict__ field, const T2 *__restrict__ srcf, const T2 *__restrict__ roots,
               const typename Real<T2>::T *__restrict__ k2t, const typename Real<T2>::T *__restrict__ sigt,
               double delz, FFTPlan pl, int ns, int first, int cols_per_cta) {
  typedef typename Real<T2>::T R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *A = W + n;
  T2 *B = A + cols_per_cta * n;
  T2 *SA = B + cols_per_cta * n;  // filtered source columns (only with srcf)
  const int ii = blockIdx.y;
  const int i = (ii + first) % ns;
  const size_t ncell = (size_t)n * n;
  const int c0 = blockIdx.x * cols_per_cta;
  const int lines = min(cols_per_cta, n - c0);
  T2 *u = field + (size_t)i * ncell;
  const T2 *sf = srcf ? srcf + (size_t)ii * ncell : nullptr;
  for (int t = threadIdx.x; t < n; t += blockDim.x) cp_elem(W + t, roots + t);
  // transposed load: line c holds column c0 + c
  for (int t = threadIdx.x; t < n * cols_per_cta; t += blockDim.x) {
    const int row = t / cols_per_cta, c = t - row * cols_per_cta;
    if (c < lines) cp_elem(A + c * n + row, u + (size_t)row * n + c0 + c);
  }
  cp_commit();
  if (sf)
    for (int t = threadIdx.x; t < n * cols_per_cta; t += blockDim.x) {
      const int row = t / cols_per_cta, c = t - row * cols_per_cta;
      if (c < lines) cp_elem(SA + c * n + row, sf + (size_t)row * n + c0 + c);
    }
  cp_commit();
  cp_wait<1>();
  __syncthreads();
  fft_lines(A, B, n, lines, pl, W, false);
  if (sf) {
    cp_wait<0>();
    __syncthreads();
    fft_lines(SA, B, n, lines, pl, W, false);
  }
  const R dz = (R)delz;
  const R *kt = k2t + (size_t)c0 * n;
  const R *st = sigt ? sigt + (size_t)c0 * n : nullptr;
  for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
    R sn, cs;
    phase_sincos(kt[t] * dz, &sn, &cs);
    T2 v = cm(A[t], mk<T2>(cs, sn));
    if (sf) {
      R g = (R)2. * st[t];
      v.x += g * SA[t].x;
      v.y += g * SA[t].y;
    }
    A[t] = v;
  }
  __syncthreads();
  fft_lines(A, B, n, lines, pl, W, true);
  for (int t = threadIdx.x; t < n * cols_per_cta; t += blockDim.x) {
    const int row = t / cols_per_cta, c = t - row * cols_per_cta;
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
  // roots and three line buffers (the third holds the second input)
  size_t smem_rows = (size_t)(n + 3 * lines * n) * es;
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
