// Tiled two-pass ADI step (FieldSolverADI::ADI, src/Core/FieldSolverADI.cpp:60-122)
// for fields of the mixed form that do not fit one CTA's shared memory (ngrid above
// 168). Included by kernels_mixed.cu after it defines its complex-arithmetic policy P
// (the header takes the arithmetic as a parameter so that the passes state the
// algorithm once):
//   V          value type in registers and shared memory
//   G          element type of the global field arrays
//   R          real type
//   ld, st     global load / store of one element
//   zero, sub, mul
//   lap(hp, hn, prev, u, next)   Dirichlet second difference
//   rhs(s, u, l, cs)             (s + u) + (i cs) l, as the form's other kernels form it
//
// X pass: one CTA per (slice, band of R rows). It loads the band with one halo row
// on each side and the band's source rows (coalesced: contiguous rows), forms the
// first right-hand side r1 = (src + u) + i cs Dy u, solves along the rows, then forms
// the second right-hand side r2 = (src + w) + i cs Dx w along the rows it now holds
// complete, and writes r2.
// Y pass: one CTA per (slice, band of columns); solves along the columns of r2 and
// writes the field.
// The solves are the Thomas recurrences split into segments (see thomas_seg): the
// first segment's forward and the last segment's backward pass are the reference's
// sweeps; the others start W elements early, with W from the host such that the
// truncated start is below the form's rounding. With W = 0 each line is solved by one
// thread exactly as in the reference.
// Traffic per cell and half-step pair: the field read once and written once, the
// source read once, the intermediate written and read once.
#pragma once

namespace g4 {
namespace tiled {

template <class P>
struct CoefP {
  const typename P::G *c, *cbet, *cwet;
};

// In-place stencil r = (src + v) + i cs lap(v) along nline lines of ng elements
// (element k of line l at L0[l * lstride + k * estride]; its source at
// src0[l * slstride + k * sestride]), nseg threads per line. The Dirichlet flags come
// from the element's index in the grid, gk0 + k of gn; the neighbours just outside a
// line are read only where the grid has them (the tile holds them there). Values
// across segment boundaries are read before the barrier that precedes any write.
template <class P>
__device__ __forceinline__ void stencil_seg(typename P::V *L0, int nline, int lstride, int estride, int n,
                                            int nseg, const typename P::V *src0, int slstride, int sestride,
                                            typename P::R cs, int gk0, int gn) {
  using V = typename P::V;
  const int tid = threadIdx.x;
  const int line = tid % nline, seg = tid / nline;
  const int len = (n + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, n);
  const bool act = seg < nseg && b < e;
  V *L = L0 + (size_t)line * lstride;
  const V *sv = src0 + (size_t)line * slstride;
  V above = P::zero(), below = P::zero();
  if (act) {
    if (gk0 + b > 0) above = L[(b - 1) * estride];
    if (gk0 + e - 1 < gn - 1) below = L[e * estride];
  }
  __syncthreads();
  if (act) {
    V prev = above, cur = L[b * estride];
    for (int k = b; k < e; k++) {
      const bool hp = gk0 + k > 0, hn = gk0 + k < gn - 1;
      V nx = (k + 1 < e) ? L[(k + 1) * estride] : below;
      V r = P::rhs(sv[k * sestride], cur, P::lap(hp, hn, prev, cur, nx), cs);
      prev = cur;
      cur = nx;
      L[k * estride] = r;
    }
  }
  __syncthreads();
}

// Tridiagonal solve (I - c D) x = r of nline lines of n elements in place (element k
// of line l at S[l * lstride + k * estride]), nseg threads per line, warm-up W (0:
// one thread per line, the exact sweeps). Forward d_k = (r_k - c_k d_{k-1}) cbet_k
// (d_0 = r_0 cbet_0), backward x_k = d_k - cwet_{k+1} x_{k+1} (x_{n-1} = d_{n-1}).
template <class P>
__device__ __forceinline__ void thomas_seg(typename P::V *S, int nline, int lstride, int estride, int n, int nseg,
                                           int W, CoefP<P> cf) {
  using V = typename P::V;
  if (W <= 0) nseg = 1;
  const int tid = threadIdx.x;
  const int line = tid % nline, seg = tid / nline;
  const int len = (n + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, n);
  const bool act = seg < nseg && b < e;
  V *L = S + (size_t)line * lstride;
  V d = P::zero();
  if (act)
    for (int k = max(0, b - W); k < b; k++) {
      V r = L[k * estride];
      d = (k == 0) ? P::mul(r, P::ld(cf.cbet)) : P::mul(P::sub(r, P::mul(P::ld(cf.c + k), d)), P::ld(cf.cbet + k));
    }
  __syncthreads();
  if (act)
    for (int k = b; k < e; k++) {
      V r = L[k * estride];
      d = (k == 0) ? P::mul(r, P::ld(cf.cbet)) : P::mul(P::sub(r, P::mul(P::ld(cf.c + k), d)), P::ld(cf.cbet + k));
      L[k * estride] = d;
    }
  __syncthreads();
  const int k1 = min(n - 1, e - 1 + W);
  V x = P::zero();
  if (act && k1 >= e) {
    x = L[k1 * estride];
    for (int k = k1 - 1; k >= e; k--) x = P::sub(L[k * estride], P::mul(P::ld(cf.cwet + k + 1), x));
  }
  __syncthreads();
  if (act)
    for (int k = e - 1; k >= b; k--) {
      V v = L[k * estride];
      if (k < n - 1) v = P::sub(v, P::mul(P::ld(cf.cwet + k + 1), x));
      x = v;
      L[k * estride] = x;
    }
  __syncthreads();
}

// X pass; dynamic shared memory (2 R + 2) ngrid elements. grid (ceil(ng / R), ns).
template <class P, int BS>
__global__ void __launch_bounds__(BS) k_adi_xt(const typename P::G *__restrict__ field,
                                               const typename P::G *__restrict__ src, typename P::G *__restrict__ tmp,
                                               CoefP<P> cf, typename P::R cstep, int ns, int ng, int first, int R,
                                               int W) {
  using V = typename P::V;
  extern __shared__ __align__(16) unsigned char tiled_smem[];
  V *T = reinterpret_cast<V *>(tiled_smem);  // rows r0-1 .. r0+nr, ng each
  V *Sb = T + (size_t)(R + 2) * ng;           // source rows r0 .. r0+nr-1
  const int ii = blockIdx.y, r0 = blockIdx.x * R;
  const int nr = min(R, ng - r0);
  const size_t ncell = (size_t)ng * ng;
  const int i = (ii + first) % ns;
  const typename P::G *u = field + (size_t)i * ncell;
  const typename P::G *s = src ? src + (size_t)ii * ncell : nullptr;
  typename P::G *w = tmp + (size_t)i * ncell;
  const long long base = (long long)(r0 - 1) * ng;
  for (int e = threadIdx.x; e < (nr + 2) * ng; e += BS) {
    const int g = r0 - 1 + e / ng;
    T[e] = (g >= 0 && g < ng) ? P::ld(u + base + e) : P::zero();
  }
  for (int e = threadIdx.x; e < nr * ng; e += BS) Sb[e] = s ? P::ld(s + (size_t)r0 * ng + e) : P::zero();
  __syncthreads();
  // r1 on rows 1..nr of the tile: lines are the columns, elements the rows
  stencil_seg<P>(T + ng, ng, 1, ng, nr, max(1, min(BS / ng, 8)), Sb, 1, ng, cstep, r0, ng);
  // solve along the rows
  const int nseg = max(1, min(BS / nr, 32));
  thomas_seg<P>(T + ng, nr, ng, 1, ng, nseg, W, cf);
  // r2 along the rows
  stencil_seg<P>(T + ng, nr, ng, 1, ng, nseg, Sb, ng, 1, cstep, 0, ng);
  for (int e = threadIdx.x; e < nr * ng; e += BS) P::st(w + (size_t)r0 * ng + e, T[ng + e]);
}

// Y pass; dynamic shared memory ngrid * Cw elements. grid (ceil(ng / Cw), ns).
template <class P, int BS>
__global__ void __launch_bounds__(BS) k_adi_yt(typename P::G *__restrict__ field,
                                               const typename P::G *__restrict__ tmp, CoefP<P> cf, int ns, int ng,
                                               int first, int Cw, int W) {
  using V = typename P::V;
  extern __shared__ __align__(16) unsigned char tiled_smem[];
  V *T = reinterpret_cast<V *>(tiled_smem);  // [ng][Cw]
  const int ii = blockIdx.y, c0 = blockIdx.x * Cw;
  const int nc = min(Cw, ng - c0);
  const size_t ncell = (size_t)ng * ng;
  const int i = (ii + first) % ns;
  const typename P::G *w = tmp + (size_t)i * ncell;
  typename P::G *u = field + (size_t)i * ncell;
  for (int e = threadIdx.x; e < ng * nc; e += BS) {
    const int row = e / nc, j = e % nc;
    T[row * Cw + j] = P::ld(w + (size_t)row * ng + c0 + j);
  }
  __syncthreads();
  thomas_seg<P>(T, nc, 1, Cw, ng, max(1, min(BS / nc, 32)), W, cf);
  for (int e = threadIdx.x; e < ng * nc; e += BS) {
    const int row = e / nc, j = e % nc;
    P::st(u + (size_t)row * ng + c0 + j, T[row * Cw + j]);
  }
}

// Band sizes: the largest R (rows, X pass) and Cw (columns, Y pass) whose tiles fit
// the shared-memory budget of two CTAs per SM, clamped to [1, 32] and [8, 64].
inline int band_rows(int ng, size_t elem) {
  const size_t budget = 110u * 1024u;
  long long r = ((long long)(budget / (elem * (size_t)ng)) - 2) / 2;
  if (r > 32) r = 32;
  if (r < 1) r = 1;
  return (int)r;
}
inline int band_cols(int ng, size_t elem) {
  const size_t budget = 110u * 1024u;
  long long c = (long long)(budget / (elem * (size_t)ng));
  if (c > 64) c = 64;
  if (c < 8) c = 8;
  return (int)c;
}

}  // namespace tiled
}  // namespace g4
