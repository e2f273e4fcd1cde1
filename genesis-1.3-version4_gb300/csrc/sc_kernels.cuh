// Space charge (&efield) of the undulator step, EFieldSolver.cpp: the long-range
// energy loss of every slice (longRange, EFieldSolver.cpp:56-118) and the
// short-range longitudinal field of every particle (shortRange with analyseBeam,
// constructLaplaceOperator and tridiag, EFieldSolver.cpp:120-272). BeamSolver::advance
// (BeamSolver.cpp:43-61) evaluates both after the first transverse half step of every
// slice (Beam::track, Beam.cpp:97-112) and adds ez + eloss to the energy equation.
//
// Included by kernels_plain.cu (FP64, the reference's arithmetic, F = PlainSC) and by
// kernels_mixed.cu (FP32, F = MixedSC). A form F supplies
//   R, R2            real and complex types of the arithmetic;
//   Th               stored phase type (FP64 radians or Q32.32 turns);
//   Step             the push's per-step constants;
//   gamma(s, g)      gamma of a stored energy coordinate;
//   half(s, g, x, y, px, py)  the first transverse half step (TrackBeam::track);
//   kPlain           true for the reference's summation of the slice moments;
//   eil(th, l)       e^{-i l theta} of a stored phase.
//
// Two kernels per step (one CTA per slice each), between which the push's first
// transverse half step has run for every slice:
//   k_sc_moments  the first transverse half step of the slice's particles (the push
//                 then runs the rest of the step), the slice's centroid, transverse
//                 size (Beam::getSize) and extreme radius; the last CTA to finish
//                 replays the reference's slice-by-slice growth of the radial grid
//                 (rmax, kept across steps) and records the extent every slice used;
//   k_sc_field    the slice's long-range loss from every slice's size and current,
//                 then its short-range field: the radial-mode source deposited in
//                 shared memory, one tridiagonal solve per mode, gathered back per
//                 particle into ez.
// Buffer `st` holds, per slice, [0,ns) xcen, [ns,2ns) ycen, [2ns,3ns) size,
// [3ns,4ns) rbound, [4ns,5ns) the grid extent rmax of the slice, [5ns,6ns) eloss, then
// (FP32 form) as floats the size and scl * current / size of every slice.
#pragma once

#include <atomic>

namespace g4 {
namespace {

constexpr int kScThreads = 256;
constexpr int kScScanChunk = 2048;

template <typename T>
__device__ __forceinline__ T sc_warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T sc_warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// CTA-wide sums of N doubles; every thread receives the totals
template <int N>
__device__ __forceinline__ void sc_block_sum(double (&v)[N], double (*red)[kScThreads / 32]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; k++) v[k] = sc_warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) red[k][w] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; k++) {
    double s = 0;
    for (int i = 0; i < nw; i++) s += red[k][i];
    v[k] = s;
  }
}

// Per particle: radial bin and azimuth z = e^{i phi} (EFieldSolver.cpp:166-173). A bin
// index outside the grid, which the reference leaves undefined (a particle on the
// centroid of a slice with a zero grid extent), is clamped into it.
template <class F>
__device__ __forceinline__ void sc_particle(typename F::R x, typename F::R y, typename F::R xc,
                                            typename F::R yc, typename F::R dr, int ng, int &idx,
                                            typename F::R2 &z) {
  using R = typename F::R;
  const R tx = x - xc, ty = y - yc;
  const R radi = sqrt(tx * tx + ty * ty);
  z.x = tx / radi;
  z.y = ty / radi;
  const R q = floor(radi / dr);
  idx = q >= 0 ? (q < (R)(ng - 1) ? (int)q : ng - 1) : 0;
}

// z^-m as std::pow(z, -m) forms it for |z| = 1: repeated products of z (m < 0) or
// of its conjugate, the reciprocal of z (m > 0); 1 exactly for m = 0
template <class F>
__device__ __forceinline__ typename F::R2 sc_zpow_neg(typename F::R2 z, int m) {
  using R2 = typename F::R2;
  R2 base = m > 0 ? R2{z.x, -z.y} : z;
  R2 r{1, 0};
  for (int n = m > 0 ? m : -m; n > 0; n--) r = R2{r.x * base.x - r.y * base.y, r.x * base.y + r.y * base.x};
  return r;
}

// Mode k of the slice's expansion, k = (l - 1)(2 nphi + 1) + (m + nphi): the walk over
// a pass's modes evaluates e^{-i l theta} once per l and steps z^-m by the conjugate of
// z (the reciprocal of the unit z) from z^nphi, taking 1 exactly at m = 0
template <class F>
struct ScModeWalk {
  using R2 = typename F::R2;
  R2 zc, ztop, zm, el;
  typename F::Th th;
  int m, l, nphi;
  __device__ __forceinline__ ScModeWalk(R2 z, typename F::Th th_, int k0, int nphi_) : th(th_), nphi(nphi_) {
    const int nm = 2 * nphi + 1;
    l = k0 / nm + 1;
    m = k0 % nm - nphi;
    zc = R2{z.x, -z.y};
    ztop = sc_zpow_neg<F>(z, -nphi);
    zm = sc_zpow_neg<F>(z, m);
    el = F::eil(th, l);
  }
  // z^-m e^{-i l theta}
  __device__ __forceinline__ R2 value() const {
    return R2{zm.x * el.x - zm.y * el.y, zm.x * el.y + zm.y * el.x};
  }
  __device__ __forceinline__ void next() {
    if (++m > nphi) {
      m = -nphi;
      el = F::eil(th, ++l);
      zm = ztop;
    } else {
      zm = m == 0 ? R2{1, 0} : R2{zm.x * zc.x - zm.y * zc.y, zm.x * zc.y + zm.y * zc.x};
    }
  }
};

// The radial Laplace operator of mode (m, l) and its tridiagonal solve, in place on
// the mode's source cs[ng] (constructLaplaceOperator and tridiag,
// EFieldSolver.cpp:175-190, 238-249, 274-292); gm[ng] is scratch. One thread per mode.
template <class F>
__device__ void sc_solve(typename F::R2 *cs, typename F::R *gm, int ng, int m, int l, typename F::R dr,
                         typename F::R pi, typename F::R coef, typename F::R econst) {
  using R = typename F::R;
  using R2 = typename F::R2;
  const R rl = (R)l, rm = (R)m;
  R bet = 0, cupp_prev = 0;
  R2 prev{0, 0};
  for (int i = 0; i < ng; i++) {
    const R vol = i == 0 ? pi * dr * dr : pi * dr * dr * (R)(2 * i + 1);
    const R ldig = 2 * pi * (R)i;
    const R ldig1 = i + 1 < ng ? 2 * pi * (R)(i + 1) : (R)0;
    const R rlog = i == 0 ? (R)0.5 : log((R)(i + 1) / (R)i);
    R lmid = -ldig - ldig1 - 2 * pi * rm * rm * rlog;
    if (i == ng - 1) lmid -= 2 * pi * (R)ng;
    const R q = econst / rl / vol;
    const R2 s0 = cs[i];
    const R2 s{-s0.y * q, s0.x * q};  // times i econst / l / vol
    const R clow = coef * ldig / rl / rl / vol;
    const R cmid = 1 + coef * lmid / rl / rl / vol;
    const R cupp = coef * ldig1 / rl / rl / vol;
    if (i == 0) {
      bet = cmid;
      prev = R2{s.x / bet, s.y / bet};
    } else {
      const R g = cupp_prev / bet;
      gm[i] = g;
      bet = cmid - clow * g;
      prev = R2{(s.x - clow * prev.x) / bet, (s.y - clow * prev.y) / bet};
    }
    cs[i] = prev;
    cupp_prev = cupp;
  }
  for (int i = ng - 2; i >= 0; i--) {
    const R2 a = cs[i], b = cs[i + 1];
    const R g = gm[i + 1];
    cs[i] = R2{a.x - g * b.x, a.y - g * b.y};
  }
}

template <class F>
struct ScBeam {
  typename F::R *g, *x, *y, *px, *py;
  const typename F::Th *theta;
  const double *current;
  const int *count;  // particles per slice (one4one windows), null: np in every slice
};

// The first transverse half step and the slice moments, then (last CTA) the radial
// grid extent of every slice. state[0]: rmax carried from slice to slice and from step
// to step; count: CTAs done.
template <class F>
__global__ void __launch_bounds__(kScThreads) k_sc_moments(ScBeam<F> b, typename F::Step step, double *st,
                                                           double *state, unsigned *count, ScConst c) {
  using R = typename F::R;
  __shared__ double red[4][kScThreads / 32];
  __shared__ double rb[kScScanChunk];
  __shared__ int last;
  const int is = blockIdx.x, tid = threadIdx.x, lane = tid & 31, ns = c.ns;
  const int np = b.count ? min(b.count[is], c.np) : c.np;  // the slice's particles
  const size_t o0 = (size_t)is * c.np;
  const R *xs = b.x + o0, *ys = b.y + o0;

  // pass 1: the half step (Beam.cpp:103, TrackBeam.cpp:17-64), and the sums of x, y
  // (and, in the reference's form, of x^2, y^2), Beam.cpp:42-67; four particles per
  // thread and round, their loads issued together
  constexpr int U = 4;
  double s[4] = {0, 0, 0, 0};
  R sx = 0, sy = 0;
  for (int i0 = tid; i0 < np; i0 += U * blockDim.x) {
    R g[U], x[U], y[U], px[U], py[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int i = i0 + u * blockDim.x;
      if (i < np) {
        g[u] = b.g[o0 + i];
        x[u] = b.x[o0 + i];
        y[u] = b.y[o0 + i];
        px[u] = b.px[o0 + i];
        py[u] = b.py[o0 + i];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int i = i0 + u * blockDim.x;
      if (i < np) {
        F::half(step, F::gamma(step, g[u]), x[u], y[u], px[u], py[u]);
        b.x[o0 + i] = x[u];
        b.y[o0 + i] = y[u];
        b.px[o0 + i] = px[u];
        b.py[o0 + i] = py[u];
        if constexpr (F::kPlain) {
          s[0] += x[u];
          s[1] += x[u] * x[u];
          s[2] += y[u];
          s[3] += y[u] * y[u];
        } else {
          sx += x[u];
          sy += y[u];
        }
      }
    }
  }
  if constexpr (F::kPlain) {
    sc_block_sum<4>(s, red);
  } else {
    double t[2] = {sx, sy};
    sc_block_sum<2>(t, red);
    s[0] = t[0];
    s[2] = t[1];
  }
  const double n = (double)np;
  const double xcen = s[0] / n, ycen = s[2] / n;

  // pass 2: the extreme radius about the centroid (EFieldSolver::analyseBeam,
  // EFieldSolver.cpp:138-157); the mixed form takes its variances here, about the
  // centroid, where FP32 does not cancel
  const R xc = (R)xcen, yc = (R)ycen;
  R r2max = 0, vx = 0, vy = 0;
  for (int i = tid; i < np; i += blockDim.x) {
    R tx = xs[i] - xc, ty = ys[i] - yc;
    R rad2 = tx * tx + ty * ty;
    if (rad2 > r2max) r2max = rad2;
    if constexpr (!F::kPlain) {
      vx += tx * tx;
      vy += ty * ty;
    }
  }
  r2max = sc_warp_max(r2max);
  double v2[2] = {(double)vx, (double)vy};
  if constexpr (!F::kPlain) sc_block_sum<2>(v2, red);
  __shared__ R wmax[kScThreads / 32];
  if (lane == 0) wmax[tid >> 5] = r2max;
  __syncthreads();
  if (tid == 0) {
    R m = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = wmax[i] > m ? wmax[i] : m;
    double size;
    if (b.current[is] <= 0 || np == 0) {
      size = 1;  // Beam::getSize of a slice without current or particles
    } else if constexpr (F::kPlain) {
      double x1 = s[0] / n, x2 = s[1] / n, y1 = s[2] / n, y2 = s[3] / n;
      size = sqrt(fabs(x2 - x1 * x1)) * sqrt(fabs(y2 - y1 * y1));
    } else {
      size = sqrt(v2[0] / n) * sqrt(v2[1] / n);
    }
    st[is] = xcen;
    st[ns + is] = ycen;
    st[2 * ns + is] = size;
    st[3 * ns + is] = sqrt((double)m);
    if constexpr (!F::kPlain) {
      // the long-range kernel's per-slice factors in FP32 (EFieldSolver.cpp:89-93, 113)
      const double fs = size <= 0 ? 1. : size;
      float *sf = reinterpret_cast<float *>(st + 6 * (size_t)ns);
      sf[is] = (float)fs;
      sf[ns + is] = (float)(c.lr_scl * b.current[is] / fs);
    }
    __threadfence();
    last = atomicAdd(count, 1u) == (unsigned)ns - 1;
  }
  __syncthreads();
  if (!last) return;

  // The last CTA: the grid extent grows to 1.5 rbound whenever a slice's rbound
  // exceeds it (EFieldSolver.cpp:159-163), slice after slice. Warp 0 resolves 32
  // slices at a time: a ballot finds the first slice beyond the current extent, which
  // sets the next one; at most 32 rounds per group.
  if (c.shortrange) {
    double r = state[0];
    for (int c0 = 0; c0 < ns; c0 += kScScanChunk) {
      const int nc = min(kScScanChunk, ns - c0);
      for (int i = tid; i < nc; i += blockDim.x) rb[i] = __ldcg(st + 3 * ns + c0 + i);
      __syncthreads();
      if (tid < 32) {
        for (int g0 = 0; g0 < nc; g0 += 32) {
          const int j = g0 + lane;
          const double bj = j < nc ? rb[j] : -1.0;
          double mine = r;
          int pos = -1;
          for (int round = 0; round < 32; round++) {
            const unsigned m = __ballot_sync(0xffffffffu, lane > pos && bj > r);
            if (!m) break;
            const int t = __ffs(m) - 1;
            const double rnew = __shfl_sync(0xffffffffu, bj, t) * 1.5;
            if (lane > pos && lane < t) mine = r;
            if (lane == t) mine = rnew;
            r = rnew;
            pos = t;
          }
          if (lane > pos) mine = r;
          if (j < nc) st[4 * ns + c0 + j] = mine;
        }
      }
      __syncthreads();
    }
    if (tid == 0) state[0] = r;
  }
  if (tid == 0) *count = 0;
}

// Long-range loss and short-range field of one slice. ez: [ns][np] (may be null when
// the short-range part is off); smem: modes_per_pass * ng * (R2 + R).
template <class F>
__global__ void __launch_bounds__(kScThreads) k_sc_field(ScBeam<F> b, double *st, typename F::R *ez, ScConst c) {
  using R = typename F::R;
  using R2 = typename F::R2;
  __shared__ double red[4][kScThreads / 32];
  extern __shared__ __align__(16) unsigned char sc_smem[];
  const int is = blockIdx.x, tid = threadIdx.x, ns = c.ns, ng = c.ng;
  const int np = b.count ? min(b.count[is], c.np) : c.np;  // the slice's particles

  // EFieldSolver::longRange, EFieldSolver.cpp:77-117
  if (c.longrange) {
    double e[1] = {0};
    if constexpr (F::kPlain) {
      for (int j = tid; j < ns; j += blockDim.x) {
        double fs = st[2 * ns + j];
        if (fs <= 0) fs = 1;
        const double sgn = (j > is) ? -1. : ((j < is) ? 1. : 0.);
        double ds = (double)(j - is) * c.slicelength * c.gamma_lr;
        double coef = 1 - sqrt(ds * ds / (ds * ds + fs));
        e[0] += sgn * coef * c.lr_scl * b.current[j] / fs;
      }
    }
    if constexpr (!F::kPlain) {
      // 1 - sqrt(a / (a + f)) = (f / (a + f)) / (1 + sqrt(a / (a + f))), without the
      // cancellation of the left side in FP32; w = scl current / size of the slice
      const float *sf = reinterpret_cast<const float *>(st + 6 * (size_t)ns), *wf = sf + ns;
      const float dsl = (float)(c.slicelength * c.gamma_lr);
      float acc = 0.f;
      for (int j = tid; j < ns; j += blockDim.x) {
        const float ds = (float)(j - is) * dsl, a = ds * ds, ff = sf[j], den = a + ff;
        const float coef = (ff / den) / (1.f + sqrtf(a / den));
        const float sgn = (j > is) ? -1.f : ((j < is) ? 1.f : 0.f);
        acc += sgn * coef * wf[j];
      }
      e[0] = acc;
    }
    sc_block_sum<1>(e, red);
    if (tid == 0) st[5 * ns + is] = -e[0] / kEev;
  }
  if (!c.shortrange || np < 1) return;

  // EFieldSolver::shortRange, EFieldSolver.cpp:197-272
  const int nz = c.nz, nphi = c.nphi, M = (2 * nphi + 1) * nz, mp = c.modes_per_pass;
  R2 *csrc = reinterpret_cast<R2 *>(sc_smem);
  R *gam = reinterpret_cast<R *>(csrc + (size_t)mp * ng);
  const R xc = (R)st[is], yc = (R)st[ns + is];
  const R dr = (R)(st[4 * ns + is] / (double)(ng - 1));
  const R pi = (R)3.14159265358979323846;
  const R coef = (R)c.coef;
  const R econst = (R)(kVacimp / kEev * b.current[is] / c.ks / (double)np);
  const typename F::R *xs = b.x + (size_t)is * c.np, *ys = b.y + (size_t)is * c.np;
  const typename F::Th *ths = b.theta + (size_t)is * c.np;
  R *ezs = ez + (size_t)is * c.np;

  for (int k0 = 0; k0 < M; k0 += mp) {
    const int k1 = min(M, k0 + mp), nk = k1 - k0;
    for (int i = tid; i < nk * ng; i += blockDim.x) csrc[i] = R2{0, 0};
    __syncthreads();
    // source: sum over the slice's particles of z^-m e^{-i l theta} in the radial bin,
    // z = e^{i phi} the particle's azimuth (EFieldSolver.cpp:228-236)
    // Aligned groups of 2, 4 or 8 lanes whose particles fall in the same radial bin
    // (a beamlet of the quiet loading always does) sum their terms by shuffles, and
    // one lane adds the sum; every lane of the CTA takes part in the shuffles.
    for (int base = 0; base < np; base += blockDim.x) {
      const int ip = base + tid;
      const bool valid = ip < np;
      const int ipc = valid ? ip : np - 1;
      int idx;
      R2 z;
      sc_particle<F>(xs[ipc], ys[ipc], xc, yc, dr, ng, idx, z);
      const unsigned full = 0xffffffffu;
      const int key = valid ? idx : -1 - (int)(threadIdx.x & 31);  // lanes without a particle match no one
      const int key1 = __shfl_xor_sync(full, key, 1), key2 = __shfl_xor_sync(full, key, 2),
                key4 = __shfl_xor_sync(full, key, 4);
      const bool g1 = key == key1;
      const int g1p = __shfl_xor_sync(full, (int)g1, 2);
      const bool g2 = g1 && g1p && key == key2;
      const int g2p = __shfl_xor_sync(full, (int)g2, 4);
      const bool g4 = g2 && g2p && key == key4;
      const int gsize = g4 ? 8 : (g2 ? 4 : (g1 ? 2 : 1));
      const bool leader = valid && ((threadIdx.x & 31) & (gsize - 1)) == 0;
      ScModeWalk<F> w(z, ths[ipc], k0, nphi);
      R2 *a = csrc + idx;
      for (int k = k0; k < k1; k++, w.next(), a += ng) {
        R2 d = w.value();
        R tx = __shfl_xor_sync(full, d.x, 1), ty = __shfl_xor_sync(full, d.y, 1);
        if (g1) d = R2{d.x + tx, d.y + ty};
        tx = __shfl_xor_sync(full, d.x, 2);
        ty = __shfl_xor_sync(full, d.y, 2);
        if (g2) d = R2{d.x + tx, d.y + ty};
        tx = __shfl_xor_sync(full, d.x, 4);
        ty = __shfl_xor_sync(full, d.y, 4);
        if (g4) d = R2{d.x + tx, d.y + ty};
        if (leader) {
          atomicAdd(&a->x, d.x);
          atomicAdd(&a->y, d.y);
        }
      }
    }
    __syncthreads();
    for (int t = tid; t < nk; t += blockDim.x) {
      const int k = k0 + t, m = k % (2 * nphi + 1) - nphi, l = k / (2 * nphi + 1) + 1;
      sc_solve<F>(csrc + (size_t)t * ng, gam + (size_t)t * ng, ng, m, l, dr, pi, coef, econst);
    }
    __syncthreads();
    // ez += 2 Re(z^m e^{i l theta} celm[idx]) (EFieldSolver.cpp:250-255): the mode
    // factor is the conjugate of the deposited one
    for (int ip = tid; ip < np; ip += blockDim.x) {
      int idx;
      R2 z;
      sc_particle<F>(xs[ip], ys[ip], xc, yc, dr, ng, idx, z);
      ScModeWalk<F> w(z, ths[ip], k0, nphi);
      R acc = k0 == 0 ? (R)0 : ezs[ip];
      const R2 *a = csrc + idx;
      for (int k = k0; k < k1; k++, w.next(), a += ng) {
        const R2 d = w.value(), ce = *a;
        acc += 2 * (d.x * ce.x + d.y * ce.y);
      }
      ezs[ip] = acc;
    }
    __syncthreads();
  }
}

// The two launches of a step's space charge, part 0 or 1 (ez: [ns][np] R, used when
// the short-range part runs)
template <class F>
void sc_launch(const Launch &L, const ScConst &c, const typename F::Step &step, ScBeam<F> sb,
               const ScBuffers &buf, int part) {
  static std::atomic<unsigned long long> configured{0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured.load() & (1ull << dev))) {
    cudaFuncSetAttribute(k_sc_field<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_max_smem());
    configured.fetch_or(1ull << dev);
  }
  cudaStream_t s = (cudaStream_t)L.stream;
  if (part == 0) {
    k_sc_moments<F><<<c.ns, kScThreads, 0, s>>>(sb, step, buf.st, buf.state, buf.count, c);
    return;
  }
  const size_t smem = c.shortrange ? (size_t)c.modes_per_pass * sc_bytes_per_mode(c.ng, !F::kPlain) : 0;
  k_sc_field<F><<<c.ns, kScThreads, smem, s>>>(sb, buf.st, (typename F::R *)buf.ez, c);
}

}  // namespace
}  // namespace g4
