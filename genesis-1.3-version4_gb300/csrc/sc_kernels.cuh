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
//   kPlain           true for the reference's summation of the slice moments;
//   eil(th, l)       e^{-i l theta} of a stored phase;
//   eil_step(e, e1, th, l)  e^{-i l theta} given e = e^{-i (l-1) theta} and e1 = e^{-i theta}
//                    (the FP64 form multiplies, the Q32.32 phase forms l theta exactly).
//
// Two kernels per step (one CTA per slice each):
//   k_sc_moments  the slice's centroid, transverse size (Beam::getSize) and extreme
//                 radius; the last CTA to finish then replays the reference's
//                 slice-by-slice growth of the radial grid (rmax, kept across steps)
//                 and records the extent every slice used;
//   k_sc_field    the slice's long-range loss from every slice's size and current,
//                 then its short-range field: the radial-mode source deposited in
//                 shared memory, one tridiagonal solve per mode, gathered back per
//                 particle into ez.
// Buffer `st` holds, per slice, [0,ns) xcen, [ns,2ns) ycen, [2ns,3ns) size,
// [3ns,4ns) rbound, [4ns,5ns) the grid extent rmax of the slice, [5ns,6ns) eloss.
#pragma once

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

// Per particle: radial bin, azimuth z = e^{i phi} and e^{-i theta}
// (EFieldSolver.cpp:166-173). A bin index outside the grid, which the reference
// leaves undefined (a particle on the centroid of a slice with a zero grid extent),
// is clamped into it.
template <class F>
__device__ __forceinline__ void sc_particle(typename F::R x, typename F::R y, typename F::Th th,
                                            typename F::R xc, typename F::R yc, typename F::R dr, int ng,
                                            int &idx, typename F::R2 &z, typename F::R2 &e1) {
  using R = typename F::R;
  const R tx = x - xc, ty = y - yc;
  const R radi = sqrt(tx * tx + ty * ty);
  z.x = tx / radi;
  z.y = ty / radi;
  const R q = floor(radi / dr);
  idx = q >= 0 ? (q < (R)(ng - 1) ? (int)q : ng - 1) : 0;
  e1 = F::eil(th, 1);
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

// Mode k of the slice's expansion, k = (m + nphi) nz + (l - 1): the walk over a pass's
// modes keeps z^-m and e^{-i l theta} and steps l, then m
template <class F>
struct ScModeWalk {
  using R2 = typename F::R2;
  R2 z, e1, zm, el;
  typename F::Th th;
  int m, l, nz;
  __device__ __forceinline__ ScModeWalk(R2 z_, R2 e1_, typename F::Th th_, int k0, int nz_, int nphi)
      : z(z_), e1(e1_), th(th_), nz(nz_) {
    m = k0 / nz - nphi;
    l = k0 % nz + 1;
    zm = sc_zpow_neg<F>(z, m);
    el = e1;
    for (int j = 2; j <= l; j++) el = F::eil_step(el, e1, th, j);
  }
  // z^-m e^{-i l theta}
  __device__ __forceinline__ R2 value() const {
    return R2{zm.x * el.x - zm.y * el.y, zm.x * el.y + zm.y * el.x};
  }
  __device__ __forceinline__ void next() {
    if (++l > nz) {
      l = 1;
      zm = sc_zpow_neg<F>(z, ++m);
      el = e1;
    } else {
      el = F::eil_step(el, e1, th, l);
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
  const typename F::R *x, *y;
  const typename F::Th *theta;
  const double *current;
};

// Per slice moments, then (last CTA) the radial grid extent of every slice.
// state[0]: rmax carried from slice to slice and from step to step; count: CTAs done.
template <class F>
__global__ void __launch_bounds__(kScThreads) k_sc_moments(ScBeam<F> b, double *st, double *state,
                                                           unsigned *count, int ns, int np, int shortrange) {
  using R = typename F::R;
  __shared__ double red[4][kScThreads / 32];
  __shared__ double rb[kScScanChunk];
  __shared__ int last;
  const int is = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
  const R *xs = b.x + (size_t)is * np, *ys = b.y + (size_t)is * np;

  // pass 1: sums of x, y (and, in the reference's form, of x^2, y^2), Beam.cpp:42-67
  double s[4] = {0, 0, 0, 0};
  if constexpr (F::kPlain) {
    for (int i = tid; i < np; i += blockDim.x) {
      double x = xs[i], y = ys[i];
      s[0] += x;
      s[1] += x * x;
      s[2] += y;
      s[3] += y * y;
    }
    sc_block_sum<4>(s, red);
  } else {
    float sx = 0.f, sy = 0.f;
    for (int i = tid; i < np; i += blockDim.x) {
      sx += xs[i];
      sy += ys[i];
    }
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
    if (b.current[is] <= 0) {
      size = 1;  // Beam::getSize of a slice without current
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
    __threadfence();
    last = atomicAdd(count, 1u) == (unsigned)ns - 1;
  }
  __syncthreads();
  if (!last) return;

  // The last CTA: the grid extent grows to 1.5 rbound whenever a slice's rbound
  // exceeds it (EFieldSolver.cpp:159-163), slice after slice. Warp 0 resolves 32
  // slices at a time: a ballot finds the first slice beyond the current extent, which
  // sets the next one; at most 32 rounds per group.
  if (shortrange) {
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
  const int is = blockIdx.x, tid = threadIdx.x, ns = c.ns, np = c.np, ng = c.ng;

  // EFieldSolver::longRange, EFieldSolver.cpp:77-117
  if (c.longrange) {
    double e[1] = {0};
    for (int j = tid; j < ns; j += blockDim.x) {
      double fs = st[2 * ns + j];
      if (fs <= 0) fs = 1;
      const double sgn = (j > is) ? -1. : ((j < is) ? 1. : 0.);
      if constexpr (F::kPlain) {
        double ds = (double)(j - is) * c.slicelength * c.gamma_lr;
        double coef = 1 - sqrt(ds * ds / (ds * ds + fs));
        e[0] += sgn * coef * c.lr_scl * b.current[j] / fs;
      } else {
        // 1 - sqrt(a / (a + f)) = (f / (a + f)) / (1 + sqrt(a / (a + f))), without the
        // cancellation of the left side in FP32
        float ds = (float)(j - is) * (float)(c.slicelength * c.gamma_lr);
        float a = ds * ds, ff = (float)fs, q = a / (a + ff);
        float coef = (ff / (a + ff)) / (1.f + sqrtf(q));
        e[0] += (double)(sgn * coef * (float)(c.lr_scl * b.current[j] / fs));
      }
    }
    sc_block_sum<1>(e, red);
    if (tid == 0) st[5 * ns + is] = -e[0] / kEev;
  }
  if (!c.shortrange) return;

  // EFieldSolver::shortRange, EFieldSolver.cpp:197-272
  const int nz = c.nz, nphi = c.nphi, M = (2 * nphi + 1) * nz, mp = c.modes_per_pass;
  R2 *csrc = reinterpret_cast<R2 *>(sc_smem);
  R *gam = reinterpret_cast<R *>(csrc + (size_t)mp * ng);
  const R xc = (R)st[is], yc = (R)st[ns + is];
  const R dr = (R)(st[4 * ns + is] / (double)(ng - 1));
  const R pi = (R)3.14159265358979323846;
  const R coef = (R)c.coef;
  const R econst = (R)(kVacimp / kEev * b.current[is] / c.ks / (double)np);
  const typename F::R *xs = b.x + (size_t)is * np, *ys = b.y + (size_t)is * np;
  const typename F::Th *ths = b.theta + (size_t)is * np;
  R *ezs = ez + (size_t)is * np;

  for (int k0 = 0; k0 < M; k0 += mp) {
    const int k1 = min(M, k0 + mp), nk = k1 - k0;
    for (int i = tid; i < nk * ng; i += blockDim.x) csrc[i] = R2{0, 0};
    __syncthreads();
    // source: sum over the slice's particles of z^-m e^{-i l theta} in the radial bin,
    // z = e^{i phi} the particle's azimuth (EFieldSolver.cpp:228-236)
    for (int ip = tid; ip < np; ip += blockDim.x) {
      int idx;
      R2 z, e1;
      sc_particle<F>(xs[ip], ys[ip], ths[ip], xc, yc, dr, ng, idx, z, e1);
      ScModeWalk<F> w(z, e1, ths[ip], k0, nz, nphi);
      for (int k = k0; k < k1; k++, w.next()) {
        const R2 d = w.value();
        R2 *a = csrc + (size_t)(k - k0) * ng + idx;
        atomicAdd(&a->x, d.x);
        atomicAdd(&a->y, d.y);
      }
    }
    __syncthreads();
    for (int t = tid; t < nk; t += blockDim.x) {
      const int k = k0 + t, m = k / nz - nphi, l = k % nz + 1;
      sc_solve<F>(csrc + (size_t)t * ng, gam + (size_t)t * ng, ng, m, l, dr, pi, coef, econst);
    }
    __syncthreads();
    // ez += 2 Re(z^m e^{i l theta} celm[idx]) (EFieldSolver.cpp:250-255): the mode
    // factor is the conjugate of the deposited one
    for (int ip = tid; ip < np; ip += blockDim.x) {
      int idx;
      R2 z, e1;
      sc_particle<F>(xs[ip], ys[ip], ths[ip], xc, yc, dr, ng, idx, z, e1);
      ScModeWalk<F> w(z, e1, ths[ip], k0, nz, nphi);
      R acc = k0 == 0 ? (R)0 : ezs[ip];
      for (int k = k0; k < k1; k++, w.next()) {
        const R2 d = w.value();
        const R2 ce = csrc[(size_t)(k - k0) * ng + idx];
        acc += 2 * (d.x * ce.x + d.y * ce.y);
      }
      ezs[ip] = acc;
    }
    __syncthreads();
  }
}

// The two launches of a step's space charge (ez: [ns][np] R, used when the
// short-range part runs)
template <class F>
void sc_launch(const Launch &L, const ScConst &c, ScBeam<F> sb, const ScBuffers &buf) {
  static unsigned long long configured = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured & (1ull << dev))) {
    cudaFuncSetAttribute(k_sc_field<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc_max_smem());
    configured |= 1ull << dev;
  }
  cudaStream_t s = (cudaStream_t)L.stream;
  k_sc_moments<F><<<c.ns, kScThreads, 0, s>>>(sb, buf.st, buf.state, buf.count, c.ns, c.np, c.shortrange);
  const size_t smem = c.shortrange ? (size_t)c.modes_per_pass * sc_bytes_per_mode(c.ng, !F::kPlain) : 0;
  k_sc_field<F><<<c.ns, kScThreads, smem, s>>>(sb, buf.st, (typename F::R *)buf.ez, c);
}

}  // namespace
}  // namespace g4
