// FFT field solver of the undulator step (FieldSolverFFT, src/Core/FieldSolverFFT.cpp:64-114):
//   unfiltered:  u <- IFFT( FFT(u) * exp(K2 dz) ) / n^2 + 2 src
//   filtered:    u <- IFFT( FFT(u) * exp(K2 dz) + 2 FFT(src) * sigmoid ) / n^2
// with FFTW's sign convention (forward e^{-2 pi i jk/n}, backward e^{+...},
// unnormalised) and K2 = -i (dx^2 + dy^2) dk^2 / (2 xks) on the reference's
// shifted frequency map (FieldSolverFFT.cpp:131-145).
//
// The 2-D transform of each ngrid x ngrid slice is done as three passes over
// global memory, each on tiles of whole lines in shared memory:
//   rows:    forward FFT of every row (and, filtered, of the source rows)
//   columns: forward FFT of every column, the k-space propagator (and filtered
//            source), inverse FFT of every column
//   rows:    inverse FFT of every row, 1/n^2, + 2 src when unfiltered
// The passes are persistent CTAs whose next tile's loads, issued at once as
// asynchronous copies, are in flight while the current tile is transformed.
// Every 1-D transform is a Stockham autosort mixed-radix FFT over the factors of
// ngrid: radices 2, 3, 4, 5, 7, 8, 9, 11, 13, 15, 16, 17 as butterflies held in
// registers (one butterfly per thread, their roots compile-time constants), any
// other prime factor p as an O(p)-per-point stage. The stage twiddles come from a table laid out per stage so
// that a warp reads consecutive entries. Templated on the precision: double2 for
// the plain form, float2 for the mixed form, whose complex arithmetic uses the
// paired FP32 instructions (both lanes of a float2 in one instruction).
#include <cuda_runtime.h>

#include <atomic>

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

// Complex arithmetic: add, sub; axpy(c, a, y) = y + c a (c real); cm(a, w) = a w;
// addi(a, b) = a + i b; subi(a, b) = a - i b.
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 axpy(float c, float2 a, float2 y) { return __ffma2_rn(make_float2(c, c), a, y); }
__device__ __forceinline__ float2 cm(float2 a, float2 w) {
  return __ffma2_rn(make_float2(-a.y, a.y), make_float2(w.y, w.x), __fmul2_rn(make_float2(a.x, a.x), w));
}
__device__ __forceinline__ float2 addi(float2 a, float2 b) {
  return __ffma2_rn(make_float2(b.y, b.x), make_float2(-1.f, 1.f), a);
}
__device__ __forceinline__ float2 subi(float2 a, float2 b) {
  return __ffma2_rn(make_float2(b.y, b.x), make_float2(1.f, -1.f), a);
}

__device__ __forceinline__ double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 axpy(double c, double2 a, double2 y) {
  return make_double2(y.x + c * a.x, y.y + c * a.y);
}
__device__ __forceinline__ double2 cm(double2 a, double2 w) {
  return make_double2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
__device__ __forceinline__ double2 addi(double2 a, double2 b) { return make_double2(a.x - b.y, a.y + b.x); }
__device__ __forceinline__ double2 subi(double2 a, double2 b) { return make_double2(a.x + b.y, a.y - b.x); }

__host__ __device__ constexpr int small_factor(int r) {
  for (int p = 2; p * p <= r; p++)
    if (r % p == 0) return p;
  return r;
}

// cos and sin of 2 pi m / R at compile time: the angle is reduced to a quadrant
// offset a in [0, pi/2) exactly in rationals (4 m = quadrant R + rem), and cos a,
// sin a are summed from their Taylor series (24 terms: below 1e-17 there).
struct Root {
  double c, s;
};
__host__ __device__ constexpr Root root_of(int m, int R) {
  const double half_pi = 1.57079632679489661923;
  const int q4 = (4 * m) / R % 4, rem = (4 * m) % R;
  const double a = half_pi * (double)rem / (double)R;
  double sn = a, cs = 1, ts = a, tc = 1;
  for (int k = 1; k < 24; k++) {
    ts *= -a * a / (double)((2 * k) * (2 * k + 1));
    tc *= -a * a / (double)((2 * k - 1) * (2 * k));
    sn += ts;
    cs += tc;
  }
  switch (q4) {
    case 0: return Root{cs, sn};
    case 1: return Root{-sn, cs};
    case 2: return Root{-cs, -sn};
    default: return Root{sn, -cs};
  }
}
// the forward roots w^m = exp(-2 pi i m / R)
template <int R>
struct Roots {
  double c[R], s[R];
  __host__ __device__ constexpr Roots() : c(), s() {
    for (int m = 0; m < R; m++) {
      const Root r = root_of(m, R);
      c[m] = r.c;
      s[m] = -r.s;
    }
  }
};

// R-point DFT y_t = sum_q x_q w^{q t} of x[0..R), w = exp(-2 pi i / R) forward and
// exp(+2 pi i / R) inverse (sgn = +1 forward, -1 inverse: the sine of every root
// is scaled by sgn; the roots themselves are compile-time constants). OUT 0: y
// replaces x; 1: y_t is written to dst[t ds] as it is formed; 2: likewise through
// the epilogue (scale, + 2 src at the same offset).
// Odd prime R: with a_m = x_m + x_{R-m} and b_m = x_m - x_{R-m},
//   y_t = A_t + i B_t,  y_{R-t} = A_t - i B_t,
//   A_t = x_0 + sum_m a_m Re(w^{m t}),  B_t = sum_m b_m Im(w^{m t}),
// so that each output costs R - 1 real multiply-adds per component.
// Composite R = P M: the M-point DFTs of the P interleaved subsequences x[P i + s],
// the twiddles w^{s k}, and P-point DFTs across them (decimation in time):
//   y_{k + t M} = sum_s w^{s k} w_P^{s t} DFT_M(x_s)_k.
#define G4_PUT(t, v)                       \
  do {                                     \
    if constexpr (OUT == 0)                \
      x[t] = (v);                          \
    else if constexpr (OUT == 1)           \
      dst[(t) * ds] = (v);                 \
    else                                   \
      epi.put(dst + (t) * ds, (t) * ds, (v)); \
  } while (0)
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

// What the last stage of a row pass writes to global memory: scale y (+ 2 src).
template <typename T2>
struct Epilogue {
  typename Real<T2>::T scale;
  const T2 *src;  // the source at the same place as the output, or null
  __device__ __forceinline__ void put(T2 *g, int off, T2 v) const {
    v = axpy(scale, v, mk<T2>(0, 0));
    if (src) v = axpy((typename Real<T2>::T)2, src[off], v);
    *g = v;
  }
};
template <int R, int OUT, typename T2>
__device__ __forceinline__ void dft(T2 *x, T2 *dst, int ds, typename Real<T2>::T sgn,
                                    const Epilogue<T2> &epi = Epilogue<T2>{}) {
  typedef typename Real<T2>::T Rt;
  constexpr Roots<R> w{};
  if constexpr (R == 1) {
    G4_PUT(0, x[0]);
  } else if constexpr (R == 2) {
    const T2 a = x[0], b = x[1];
    G4_PUT(0, add(a, b));
    G4_PUT(1, sub(a, b));
  } else if constexpr (R == 4) {
    // w = -i sgn: exact
    const T2 t0 = add(x[0], x[2]), t1 = sub(x[0], x[2]), t2 = add(x[1], x[3]);
    const T2 t3 = axpy(sgn, sub(x[1], x[3]), mk<T2>(0, 0));
    G4_PUT(0, add(t0, t2));
    G4_PUT(2, sub(t0, t2));
    G4_PUT(1, subi(t1, t3));
    G4_PUT(3, addi(t1, t3));
  } else if constexpr (small_factor(R) != R) {
    constexpr int P = small_factor(R), M = R / P;
    T2 part[P][M];
#pragma unroll
    for (int s = 0; s < P; s++)
#pragma unroll
      for (int i = 0; i < M; i++) part[s][i] = x[P * i + s];
#pragma unroll
    for (int s = 0; s < P; s++) dft<M, 0>(part[s], (T2 *)nullptr, 0, sgn);
#pragma unroll
    for (int k = 0; k < M; k++) {
      T2 y[P];
#pragma unroll
      for (int s = 0; s < P; s++)
        y[s] = (s == 0 || k == 0) ? part[s][k] : cm(part[s][k], mk<T2>((Rt)w.c[s * k], sgn * (Rt)w.s[s * k]));
      if constexpr (OUT == 0) {
        dft<P, 0>(y, (T2 *)nullptr, 0, sgn);
#pragma unroll
        for (int t = 0; t < P; t++) x[k + t * M] = y[t];
      } else {
        Epilogue<T2> e2 = epi;
        if (OUT == 2 && e2.src) e2.src += k * ds;
        dft<P, OUT>(y, dst + k * ds, M * ds, sgn, e2);
      }
    }
  } else {
    constexpr int H = (R - 1) / 2;
    T2 a[H + 1], b[H + 1];
    const T2 x0 = x[0];
    T2 y0 = x0;
#pragma unroll
    for (int m = 1; m <= H; m++) {
      a[m] = add(x[m], x[R - m]);
      b[m] = axpy(sgn, sub(x[m], x[R - m]), mk<T2>(0, 0));
      y0 = add(y0, a[m]);
    }
    G4_PUT(0, y0);
#pragma unroll
    for (int t = 1; t <= H; t++) {
      T2 A = x0, B = mk<T2>(0, 0);
#pragma unroll
      for (int m = 1; m <= H; m++) {
        const int id = (m * t) % R;
        A = axpy((Rt)w.c[id], a[m], A);
        B = axpy((Rt)w.s[id], b[m], B);
      }
      G4_PUT(t, addi(A, B));
      G4_PUT(R - t, subi(A, B));
    }
  }
}
#undef G4_PUT

// x / d for x d < 2^32 with m = ceil(2^32 / d) (exact there); d = 1 passes x through
__device__ __forceinline__ int fdiv(int x, int d, unsigned m) {
  return d == 1 ? x : (int)__umulhi((unsigned)x, m);
}

// One radix-R Stockham stage in place over lines of A, one butterfly per thread:
// every thread loads its butterfly into registers (stage_load), the CTA
// synchronises, and every thread writes its outputs (stage_store). With ns the
// product of the earlier radices and nb = n / R, butterfly j (k = j mod ns) of a
// line reads in[j + q nb], q < R, multiplies input q by the twiddle
// exp(-+2 pi i q k / (ns R)), takes the R-point DFT, and writes output t to
// out[(j - k) R + t ns + k]:
//   out[...] = sum_q in[j + q nb] W^{q (k n/(ns R) + t n/R)},  W = exp(-+2 pi i / n).
// The twiddles are tw[(q - 1) ns + k] (forward; conjugated when inverse). The
// butterfly lives in one register array of the largest radix for every stage, so
// that the stages' code paths share the registers held across the barrier.
constexpr int MAX_RADIX = 17;
template <int R, typename T2>
__device__ __forceinline__ void stage_load(T2 *x, const T2 *src, int nb, int ns, int k, const T2 *tw,
                                           typename Real<T2>::T sgn) {
#pragma unroll
  for (int q = 0; q < R; q++) x[q] = src[q * nb];
  if (ns > 1) {
#pragma unroll
    for (int q = 1; q < R; q++) {
      const T2 w = tw[(q - 1) * ns + k];
      x[q] = cm(x[q], mk<T2>(w.x, sgn * w.y));
    }
  }
}

// Stage of any radix r in place: output o of a line is the O(r) sum over its
// butterfly's inputs with the twiddled root read from the table; a thread forms at
// most STAGE_ANY_OUT outputs (lines n <= STAGE_ANY_OUT blockDim.x) in registers
// before the CTA synchronises and they are written.
constexpr int STAGE_ANY_OUT = 8;
template <typename T2>
__device__ __forceinline__ void any_load(T2 *acc, const T2 *A, int ls, int lines, int n, int ns, int r,
                                         const T2 *W, bool inverse) {
  const int nb = n / r, nsr = ns * r;
#pragma unroll
  for (int u = 0; u < STAGE_ANY_OUT; u++) {
    const int t = threadIdx.x + u * blockDim.x;
    if (t < lines * n) {
      const int line = t / n, o = t - line * n;
      const int q1 = o / nsr, rem = o - q1 * nsr;
      const int tt = rem / ns, k = rem - tt * ns;
      const int e = k * (n / nsr) + tt * nb;  // < n
      const T2 *src = A + line * ls + q1 * ns + k;
      T2 v = src[0];
      int m = 0;
      for (int q = 1; q < r; q++) {
        m += e;
        if (m >= n) m -= n;
        T2 w = W[m];
        if (inverse) w.y = -w.y;
        v = add(v, cm(src[q * nb], w));
      }
      acc[u] = v;
    }
  }
}
template <typename T2>
__device__ __forceinline__ void any_store(const T2 *acc, T2 *A, int ls, int lines, int n, T2 *gout,
                                          const Epilogue<T2> &epi) {
#pragma unroll
  for (int u = 0; u < STAGE_ANY_OUT; u++) {
    const int t = threadIdx.x + u * blockDim.x;
    if (t < lines * n) {
      const int line = t / n, pos = line * ls + (t - line * n);
      if (gout)
        epi.put(gout + pos, pos, acc[u]);
      else
        A[pos] = acc[u];
    }
  }
}

// Radices with a register butterfly (the others take the generic stage).
__host__ __device__ constexpr bool register_radix(int r) {
  return r == 2 || r == 3 || r == 4 || r == 5 || r == 7 || r == 8 || r == 9 || r == 11 || r == 13 || r == 15 ||
         r == 16 || r == 17;
}

// One 1-D Stockham FFT of length n, in place over `lines` lines of A stored with
// line stride `ls`, the stages of the plan's radices in turn, forward or inverse
// (the direction is a run-time argument, so that a kernel with several transforms
// holds one copy of the code). W: the n roots exp(-2 pi i m / n), followed by the
// stage twiddle table (stage s's at W + n + plan.tw_off[s]).
template <typename T2>
__device__ __forceinline__ void fft_lines(T2 *A, int ls, int lines, const FFTPlan &pl, const T2 *W, bool inverse,
                                          T2 *gout = nullptr, const Epilogue<T2> &epi = Epilogue<T2>{},
                                          bool wait_epi_copy = false) {
  typedef typename Real<T2>::T Rt;
  const Rt sgn = inverse ? (Rt)-1 : (Rt)1;
  int ns = 1;
  for (int s = 0; s < pl.nstage; s++) {
    // the last stage of a pass with a global output writes it there (line stride ls)
    const bool to_global = gout && s == pl.nstage - 1;
    const int r = pl.radix[s], nb = pl.nb[s];
    const T2 *tw = W + pl.n + pl.tw_off[s];
    const bool act = (int)threadIdx.x < lines * nb;
    const int line = fdiv(threadIdx.x, nb, pl.mnb[s]), j = threadIdx.x - line * nb;
    const int k = j - fdiv(j, ns, pl.mns[s]) * ns;
    const T2 *src = A + line * ls + j;
    T2 *dst = A + line * ls + (j - k) * r + k;
    T2 x[MAX_RADIX];
    switch (r) {
#define G4_LOAD(R) \
  case R:          \
    if (act) stage_load<R>(x, src, nb, ns, k, tw, sgn); \
    break;
      G4_LOAD(2) G4_LOAD(3) G4_LOAD(4) G4_LOAD(5) G4_LOAD(7) G4_LOAD(8) G4_LOAD(9) G4_LOAD(11) G4_LOAD(13)
      G4_LOAD(15) G4_LOAD(16) G4_LOAD(17)
#undef G4_LOAD
      default: any_load(x, A, ls, lines, pl.n, ns, r, W, inverse); break;
    }
    // the epilogue's source, copied asynchronously by the caller, must have landed
    // before the barrier ahead of the last stage's stores (all but the most recent
    // copy group of this thread)
    if (to_global && wait_epi_copy) cp_wait<1>();
    __syncthreads();
    const int o = line * ls + (j - k) * r + k;
    Epilogue<T2> e = epi;
    if (e.src) e.src += o;
    switch (r) {
#define G4_STORE(R)                                      \
  case R:                                                \
    if (act) {                                           \
      if (to_global)                                     \
        dft<R, 2>(x, gout + o, ns, sgn, e);              \
      else                                               \
        dft<R, 1>(x, dst, ns, sgn);                      \
    }                                                    \
    break;
      G4_STORE(2) G4_STORE(3) G4_STORE(4) G4_STORE(5) G4_STORE(7) G4_STORE(8) G4_STORE(9) G4_STORE(11)
      G4_STORE(13) G4_STORE(15) G4_STORE(16) G4_STORE(17)
#undef G4_STORE
      default: any_store(x, A, ls, lines, pl.n, to_global ? gout : (T2 *)nullptr, epi); break;
    }
    if (!to_global) __syncthreads();
    ns *= r;
  }
}

// CTAs per SM the passes' launch bounds provide for (the register budget of a
// thread is 64K / (256 x CTAs): 80 registers in FP32, 128 in FP64).
constexpr int FFT_CTAS_FP32 = 3, FFT_CTAS_FP64 = 2;

// Both passes are persistent: tile = ii nblk + blk runs over the window's slices ii
// and each slice's blocks of L lines; CTA b takes tiles b, b + gridDim.x, ... and
// prefetches its next tile by asynchronous copies into the second of two tile
// buffers while it transforms the current one in place.

// Row pass over tiles of L rows. MODE 0: forward FFT of the rows of `in` into `out`
// (the same place of slice (ii + first) mod ns of each); MODE 1: inverse FFT of
// the rows of `in`, times `scale`, plus 2 src (slice ii) when src is given, into
// `out`, with the source rows in a third tile buffer and one CTA per SM fewer.
// in == out transforms in place.
template <typename T2, int MODE>
__global__ void __launch_bounds__(256, (sizeof(T2) == 8 ? FFT_CTAS_FP32 : FFT_CTAS_FP64) - MODE)
    k_fft_rows(const T2 *in, T2 *out, const T2 *__restrict__ src, const T2 *__restrict__ roots, FFTPlan pl,
               int ns, int first, double scale, int L) {
  typedef typename Real<T2>::T R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *Abuf = W + 2 * n;      // two tile buffers
  T2 *S = Abuf + 2 * L * n;  // MODE 1: the tile's source rows
  const int nblk = (n + L - 1) / L, ntiles = ns * nblk;
  const size_t ncell = (size_t)n * n;
  for (int t = threadIdx.x; t < 2 * n - 1; t += blockDim.x) cp_elem(W + t, roots + t);
  int tile = blockIdx.x;
  if (tile < ntiles) {
    const int ii = tile / nblk, r0 = (tile - ii * nblk) * L, cnt = min(L, n - r0) * n;
    const T2 *g = in + (size_t)((ii + first) % ns) * ncell + (size_t)r0 * n;
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) cp_elem(Abuf + t, g + t);
  }
  cp_commit();
  for (int it = 0; tile < ntiles; tile += gridDim.x, it++) {
    T2 *A = Abuf + (it & 1) * L * n;
    const int ii = tile / nblk, r0 = (tile - ii * nblk) * L, lines = min(L, n - r0), cnt = lines * n;
    const T2 *sb = (MODE == 1 && src) ? src + (size_t)ii * ncell + (size_t)r0 * n : nullptr;
    // the source rows of the epilogue: copied while the rows are transformed
    if (sb)
      for (int t = threadIdx.x; t < cnt; t += blockDim.x) cp_elem(S + t, sb + t);
    cp_commit();
    const int nx = tile + gridDim.x;
    if (nx < ntiles) {
      const int jj = nx / nblk, q0 = (nx - jj * nblk) * L, qc = min(L, n - q0) * n;
      const T2 *g = in + (size_t)((jj + first) % ns) * ncell + (size_t)q0 * n;
      T2 *dst = Abuf + ((it + 1) & 1) * L * n;
      for (int t = threadIdx.x; t < qc; t += blockDim.x) cp_elem(dst + t, g + t);
    }
    cp_commit();
    cp_wait<2>();  // this tile's rows (committed one iteration earlier)
    __syncthreads();
    // the last stage writes the rows to global memory, scaled and with 2 src (MODE 1)
    T2 *o = out + (size_t)((ii + first) % ns) * ncell + (size_t)r0 * n;
    fft_lines(A, n, lines, pl, W, MODE == 1, o, Epilogue<T2>{(R)scale, sb ? S : nullptr}, sb != nullptr);
    __syncthreads();  // A is free for the copies of the next iteration
  }
  cp_wait<0>();
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

// Transposed load of columns c0 .. c0 + lines - 1 of slice `g` (rows of n) into
// lines of `dst` (line c = column c0 + c): thread t takes column t mod 16 of rows
// t / 16, t / 16 + blockDim / 16, ... (lines <= 16)
template <typename T2>
__device__ __forceinline__ void load_cols(T2 *dst, const T2 *g, int n, int c0, int lines) {
  const int tc = threadIdx.x & 15;
  if (tc < lines)
    for (int row = threadIdx.x >> 4; row < n; row += blockDim.x >> 4)
      cp_elem(dst + tc * n + row, g + (size_t)row * n + c0 + tc);
}

// Column pass over tiles of L (<= 16) columns: forward FFT of the columns, the
// propagator exp(K2 dz) (and the filtered source 2 FFT(src) sigmoid), inverse FFT
// of the columns, written back in place. The propagator's phase at the FFT index
// (ky, kx) is (dx^2 + dy^2) k2dz, k2dz = -dk^2 dz / (2 xks), with dx = ix - (n-1)/2
// and ix = (kx + n - (n+1)/2) mod n (the reference's shifted frequency map), and
// likewise dy; sigt holds the sigmoid transposed, sigt[kx n + ky], so that the
// reads of a column are contiguous; srcf (filtered) holds the row-transformed
// source of slice ii, staged in a third tile buffer.
template <typename T2>
__global__ void __launch_bounds__(256, sizeof(T2) == 8 ? FFT_CTAS_FP32 : FFT_CTAS_FP64)
    k_fft_cols(T2 *__restrict__ field, const T2 *__restrict__ srcf, const T2 *__restrict__ roots, double k2dz,
               const typename Real<T2>::T *__restrict__ sigt, FFTPlan pl, int ns, int first, int L) {
  typedef typename Real<T2>::T R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *Abuf = W + 2 * n;
  T2 *SA = Abuf + 2 * L * n;  // filtered source columns (only with srcf)
  const int nblk = (n + L - 1) / L, ntiles = ns * nblk;
  const size_t ncell = (size_t)n * n;
  const R kdz = (R)k2dz, half = (R)(0.5 * (n - 1));
  const int off = n - (n + 1) / 2;
  // element t of a tile: column t / n, ky = t mod n, advanced by the CTA's stride
  const int c_init = fdiv(threadIdx.x, n, pl.mn), ky_init = threadIdx.x - c_init * n;
  const int dc = fdiv(blockDim.x, n, pl.mn), dky = blockDim.x - dc * n;
  for (int t = threadIdx.x; t < 2 * n - 1; t += blockDim.x) cp_elem(W + t, roots + t);
  int tile = blockIdx.x;
  if (tile < ntiles) {
    const int ii = tile / nblk, c0 = (tile - ii * nblk) * L;
    load_cols(Abuf, field + (size_t)((ii + first) % ns) * ncell, n, c0, min(L, n - c0));
  }
  cp_commit();
  for (int it = 0; tile < ntiles; tile += gridDim.x, it++) {
    T2 *A = Abuf + (it & 1) * L * n;
    const int ii = tile / nblk, c0 = (tile - ii * nblk) * L, lines = min(L, n - c0);
    T2 *u = field + (size_t)((ii + first) % ns) * ncell;
    if (srcf) load_cols(SA, srcf + (size_t)ii * ncell, n, c0, lines);
    cp_commit();
    const int nx = tile + gridDim.x;
    if (nx < ntiles) {
      const int jj = nx / nblk, q0 = (nx - jj * nblk) * L;
      load_cols(Abuf + ((it + 1) & 1) * L * n, field + (size_t)((jj + first) % ns) * ncell, n, q0,
                min(L, n - q0));
    }
    cp_commit();
    cp_wait<2>();
    __syncthreads();
    // the transforms in one loop, so that the kernel holds one copy of their code:
    // forward on the field's columns, (filtered) forward on the source's, then the
    // propagator and the inverse on the field's
    const int njob = srcf ? 3 : 2;
    for (int job = 0; job < njob; job++) {
      const bool inverse = job == njob - 1;
      if (job == 1 && srcf) {
        cp_wait<1>();
        __syncthreads();
      }
      if (inverse) {
        const R *st = sigt + (size_t)c0 * n;
        int c = c_init, ky = ky_init;
        for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
          int ix = c0 + c + off, iy = ky + off;
          ix -= ix >= n ? n : 0;
          iy -= iy >= n ? n : 0;
          const R dx = (R)ix - half, dy = (R)iy - half;
          R sn, cs;
          phase_sincos((dx * dx + dy * dy) * kdz, &sn, &cs);
          T2 v = cm(A[t], mk<T2>(cs, sn));
          if (srcf) v = axpy((R)2 * st[t], SA[t], v);
          A[t] = v;
          c += dc;
          ky += dky;
          if (ky >= n) {
            ky -= n;
            c++;
          }
        }
        __syncthreads();
      }
      fft_lines(job == 1 && srcf ? SA : A, n, lines, pl, W, inverse);
    }
    const int tc = threadIdx.x & 15;
    if (tc < lines)
      for (int row = threadIdx.x >> 4; row < n; row += blockDim.x >> 4)
        u[(size_t)row * n + c0 + tc] = A[tc * n + row];
    __syncthreads();
  }
  cp_wait<0>();
}

// Far-field moments of the field diagnostics (DiagField with FFTW,
// Diagnostic.cpp:786-847): a column pass over the row-transformed field `work`
// (k_fft_rows<T,0> into it first) that takes the forward FFT of the columns and the
// power-weighted moments of the tile's elements on the shifted frequency map (dx, dy
// as in k_fft_cols' propagator). One partial per tile, deterministic:
// part[(ii nblk + blk) 5 + k] = sum |F|^2, dx |F|^2, dx^2 |F|^2, dy |F|^2, dy^2 |F|^2.
template <typename T2>
__global__ void __launch_bounds__(256, sizeof(T2) == 8 ? FFT_CTAS_FP32 : FFT_CTAS_FP64)
    k_fft_cols_moments(const T2 *__restrict__ work, const T2 *__restrict__ roots, FFTPlan pl, int ns, int first,
                       int L, double *__restrict__ part) {
  typedef typename Real<T2>::T R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[8][5];
  T2 *W = reinterpret_cast<T2 *>(smem_raw);
  const int n = pl.n;
  T2 *Abuf = W + 2 * n;
  const int nblk = (n + L - 1) / L, ntiles = ns * nblk;
  const size_t ncell = (size_t)n * n;
  const R half = (R)(0.5 * (n - 1));
  const int off = n - (n + 1) / 2;
  const int c_init = fdiv(threadIdx.x, n, pl.mn), ky_init = threadIdx.x - c_init * n;
  const int dc = fdiv(blockDim.x, n, pl.mn), dky = blockDim.x - dc * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < 2 * n - 1; t += blockDim.x) cp_elem(W + t, roots + t);
  int tile = blockIdx.x;
  if (tile < ntiles) {
    const int ii = tile / nblk, c0 = (tile - ii * nblk) * L;
    load_cols(Abuf, work + (size_t)((ii + first) % ns) * ncell, n, c0, min(L, n - c0));
  }
  cp_commit();
  for (int it = 0; tile < ntiles; tile += gridDim.x, it++) {
    T2 *A = Abuf + (it & 1) * L * n;
    const int ii = tile / nblk, blk = tile - ii * nblk, c0 = blk * L, lines = min(L, n - c0);
    const int nx = tile + gridDim.x;
    if (nx < ntiles) {
      const int jj = nx / nblk, q0 = (nx - jj * nblk) * L;
      load_cols(Abuf + ((it + 1) & 1) * L * n, work + (size_t)((jj + first) % ns) * ncell, n, q0,
                min(L, n - q0));
    }
    cp_commit();
    cp_wait<1>();
    __syncthreads();
    fft_lines(A, n, lines, pl, W, false);
    R m[5] = {0, 0, 0, 0, 0};
    int c = c_init, ky = ky_init;
    for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
      int ix = c0 + c + off, iy = ky + off;
      ix -= ix >= n ? n : 0;
      iy -= iy >= n ? n : 0;
      const R dx = (R)ix - half, dy = (R)iy - half;
      const T2 v = A[t];
      const R w = v.x * v.x + v.y * v.y;
      m[0] += w;
      m[1] += dx * w;
      m[2] += dx * dx * w;
      m[3] += dy * w;
      m[4] += dy * dy * w;
      c += dc;
      ky += dky;
      if (ky >= n) {
        ky -= n;
        c++;
      }
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
      R v = m[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][k] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
      double r = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += red[w][threadIdx.x];
      part[((size_t)ii * nblk + blk) * 5 + threadIdx.x] = r;
    }
    __syncthreads();
  }
  cp_wait<0>();
}

constexpr int FFT_THREADS = 256;

// Shared memory of a pass with `bufs` tile buffers of L lines and the roots and
// twiddles (2 n elements).
size_t fft_smem(int n, int L, int bufs, size_t es) { return (size_t)(2 * n + bufs * L * n) * es; }

// CTAs of a pass resident on one SM: the register bound of its launch bounds,
// fewer where the shared memory does not allow them.
int fft_ctas_per_sm(int regs_bound, size_t smem) {
  const size_t sm_bytes = 228u * 1024u;
  int k = regs_bound;
  while (k > 1 && (size_t)k * (smem + 1024) > sm_bytes) k--;
  return k;
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v > 0 ? v : 152;
  }
  return cached[dev];
}

template <typename T2>
void launch_fft(void *stream, void *field, const void *src, void *work, const void *roots, double k2c,
                const void *sig, int filtered, double delz, const FFTPlan &pl, int ns, int first) {
  cudaStream_t s = (cudaStream_t)stream;
  const int n = pl.n;
  const int es = (int)sizeof(T2);
  static std::atomic<unsigned long long> configured{0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured.load() & (1ull << dev))) {
    cudaFuncSetAttribute(k_fft_rows<T2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_fft_rows<T2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaFuncSetAttribute(k_fft_cols<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    configured.fetch_or(1ull << dev);
  }
  const int nsm = sm_count();
  const int rows_ctas = es == 8 ? FFT_CTAS_FP32 : FFT_CTAS_FP64, cols_ctas = rows_ctas;
  auto grid = [&](int L, size_t smem, int regs_bound) {
    const long long tiles = (long long)ns * ((n + L - 1) / L);
    const long long cap = (long long)nsm * fft_ctas_per_sm(regs_bound, smem);
    return (unsigned)(tiles < cap ? tiles : cap);
  };
  T2 *f = (T2 *)field;
  const T2 *sr = (const T2 *)src;
  T2 *sfw = filtered ? (T2 *)work : nullptr;
  const T2 *rt = (const T2 *)roots;
  typedef typename Real<T2>::T R;
  // forward rows of the field (and, filtered, of the source into the work array)
  const int Lr = fft_lines_per_cta(pl, es, 2, 32, rows_ctas);
  const size_t mr = fft_smem(n, Lr, 2, (size_t)es);
  const unsigned gr = grid(Lr, mr, rows_ctas);
  k_fft_rows<T2, 0><<<gr, FFT_THREADS, mr, s>>>(f, f, nullptr, rt, pl, ns, first, 1.0, Lr);
  if (sfw) k_fft_rows<T2, 0><<<gr, FFT_THREADS, mr, s>>>(sr, sfw, nullptr, rt, pl, ns, 0, 1.0, Lr);
  // columns
  const int bc = sfw ? 3 : 2;
  const int Lc = fft_lines_per_cta(pl, es, bc, 16, cols_ctas);
  const size_t mc = fft_smem(n, Lc, bc, (size_t)es);
  k_fft_cols<T2><<<grid(Lc, mc, cols_ctas), FFT_THREADS, mc, s>>>(f, sfw, rt, k2c * delz, (const R *)sig, pl,
                                                                 ns, first, Lc);
  // inverse rows, 1/n^2, + 2 src when unfiltered (the source rows in a third tile
  // buffer, at one CTA per SM fewer)
  const T2 *s1 = filtered ? nullptr : sr;
  const int c1 = rows_ctas - 1;
  const int L1 = fft_lines_per_cta(pl, es, s1 ? 3 : 2, 32, c1);
  const size_t m1 = fft_smem(n, L1, s1 ? 3 : 2, (size_t)es);
  k_fft_rows<T2, 1><<<grid(L1, m1, c1), FFT_THREADS, m1, s>>>(f, f, s1, rt, pl, ns, first, 1.0 / ((double)n * n),
                                                              L1);
}

template <typename T2>
void launch_fft_diag_t(void *stream, const void *field, void *work, const void *roots, const FFTPlan &pl, int ns,
                       int first, double *part, int L) {
  cudaStream_t s = (cudaStream_t)stream;
  const int n = pl.n;
  const int es = (int)sizeof(T2);
  static std::atomic<unsigned long long> configured{0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured.load() & (1ull << dev))) {
    cudaFuncSetAttribute(k_fft_rows<T2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    // (the kernel's static reduction array counts against the 227 KB too)
    cudaFuncSetAttribute(k_fft_cols_moments<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 226 * 1024);
    configured.fetch_or(1ull << dev);
  }
  const int ctas = es == 8 ? FFT_CTAS_FP32 : FFT_CTAS_FP64;
  const long long nsm = sm_count();
  auto grid = [&](int lines, size_t smem) {
    const long long tiles = (long long)ns * ((n + lines - 1) / lines);
    const long long cap = nsm * fft_ctas_per_sm(ctas, smem);
    return (unsigned)(tiles < cap ? tiles : cap);
  };
  const int Lr = fft_lines_per_cta(pl, es, 2, 32, ctas);
  const size_t mr = fft_smem(n, Lr, 2, (size_t)es);
  k_fft_rows<T2, 0><<<grid(Lr, mr), FFT_THREADS, mr, s>>>((const T2 *)field, (T2 *)work, nullptr, (const T2 *)roots,
                                                          pl, ns, first, 1.0, Lr);
  const size_t mc = fft_smem(n, L, 2, (size_t)es);
  k_fft_cols_moments<T2><<<grid(L, mc), FFT_THREADS, mc, s>>>((const T2 *)work, (const T2 *)roots, pl, ns, first, L,
                                                              part);
}

}  // namespace

// Lines per CTA of a pass with `bufs` tile buffers: the largest L <= maxL such that
// every register stage has a butterfly per thread for all L lines (L n / R <= T),
// the generic stages at most 8 outputs per thread (L n <= 8 T), and the shared
// memory of `per_sm` CTAs fits an SM (or one CTA's, in 227 KB, where not even
// L = 1 fits that).
int fft_lines_per_cta(const FFTPlan &pl, int es, int bufs, int maxL, int per_sm) {
  const int n = pl.n;
  int L = maxL;
  for (int s = 0; s < pl.nstage; s++) {
    const int r = pl.radix[s];
    const int lim = register_radix(r) ? FFT_THREADS / (n / r) : STAGE_ANY_OUT * FFT_THREADS / n;
    if (lim < L) L = lim;
  }
  if (L < 1) L = 1;
  (void)es;
  const size_t cap = 228u * 1024u / per_sm - 1024;
  while (L > 1 && fft_smem(n, L, bufs, es) > cap) L--;
  return L;
}

int fft_max_ngrid(int mixed) {
  // a register stage of one line with n / R <= 256 butterflies, the generic stages
  // of one line with at most 8 outputs per thread (n <= 2048), and one line in
  // each of three tile buffers plus the roots and twiddles in 227 KB
  int es = mixed ? (int)sizeof(float2) : (int)sizeof(double2);
  int m = (int)(227u * 1024u / (5u * (unsigned)es));
  return m < STAGE_ANY_OUT * FFT_THREADS ? m : STAGE_ANY_OUT * FFT_THREADS;
}

// Whether every stage of the plan can take its lines (n / R butterflies of a
// register stage per thread, n outputs of a generic stage at most 8 per thread).
int fft_plan_fits(const FFTPlan &pl) {
  for (int s = 0; s < pl.nstage; s++) {
    const int r = pl.radix[s];
    if (register_radix(r) ? pl.n / r > FFT_THREADS : pl.n > STAGE_ANY_OUT * FFT_THREADS) return 0;
  }
  return 1;
}

int fft_diag_lines(const FFTPlan &pl, int mixed) {
  const int es = mixed ? (int)sizeof(float2) : (int)sizeof(double2);
  return fft_lines_per_cta(pl, es, 2, 16, mixed ? FFT_CTAS_FP32 : FFT_CTAS_FP64);
}

void launch_fft_diag(void *stream, int mixed, const void *field, void *work, const void *roots, const FFTPlan &pl,
                     int ns, int first, double *part) {
  const int L = fft_diag_lines(pl, mixed);
  if (mixed)
    launch_fft_diag_t<float2>(stream, field, work, roots, pl, ns, first, part, L);
  else
    launch_fft_diag_t<double2>(stream, field, work, roots, pl, ns, first, part, L);
}

void launch_fft_solve(void *stream, int mixed, void *field, const void *src, void *work, const void *roots,
                      double k2c, const void *sig, int filtered, double delz, const FFTPlan &pl, int ns,
                      int first) {
  if (mixed)
    launch_fft<float2>(stream, field, src, work, roots, k2c, sig, filtered, delz, pl, ns, first);
  else
    launch_fft<double2>(stream, field, src, work, roots, k2c, sig, filtered, delz, pl, ns, first);
}

}  // namespace g4
