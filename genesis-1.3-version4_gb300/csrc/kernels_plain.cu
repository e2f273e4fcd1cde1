// FP64 kernels of the undulator step with the reference's arithmetic.
//
// This translation unit is compiled with --fmad=false so that every product and
// sum rounds separately, as the reference's x86-64 build does; together with the
// IEEE-rounded division and square root of CUDA, only the transcendental
// functions (sin, cos, sinh, cosh of the CUDA math library) differ in the last
// bits from the reference. Operation order follows the cited reference lines.
//
// Layout: particles are structure-of-arrays, slice-major (index is*np + ip);
// fields are [nslice][ngrid*ngrid] double2, storage order with the ring start
// `first`; the deposited source is [nslice][ngrid*ngrid] double2 indexed by
// beam slice.
#include <cuda_runtime.h>

#include "g4gpu_internal.h"
#include "philox.cuh"

namespace g4 {
namespace {

struct C2 {
  double x, y;
};
__device__ __forceinline__ C2 ld(const double2 *p) {
  double2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ void st(double2 *p, C2 v) { *p = make_double2(v.x, v.y); }
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ C2 csub(C2 a, C2 b) { return {a.x - b.x, a.y - b.y}; }
// The std::complex<double> product (ac - bd, ad + bc), with each component's first
// product fused into its sum: one rounding fewer per component than GCC's evaluation
// (a last-bit difference), and two FP64 instructions instead of three
__device__ __forceinline__ C2 cmul_fma(C2 a, C2 b) { return {fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x)}; }
// a + i b l for real b. The ADI's cstep and off-diagonal coefficients c[k] are purely
// imaginary (FieldSolverADI.cpp:139, 161-165: real part exactly 0), so the reference's
// complex product i b l is exactly (-b l.y, b l.x); here it is fused into the sum (a
// last-bit difference, two FP64 instructions instead of four).
__device__ __forceinline__ C2 add_imul(C2 a, double b, C2 l) { return {fma(-b, l.y, a.x), fma(b, l.x, a.y)}; }
// d - w n for complex w, both products fused into the difference (four FP64
// instructions instead of six)
__device__ __forceinline__ C2 sub_cmul(C2 d, C2 w, C2 n) {
  return {fma(-w.x, n.x, fma(w.y, n.y, d.x)), fma(-w.x, n.y, fma(-w.y, n.x, d.y))};
}
// real * complex
__device__ __forceinline__ C2 rmul(double s, C2 a) { return {s * a.x, s * a.y}; }
// complex * real
__device__ __forceinline__ C2 mulr(C2 a, double s) { return {a.x * s, a.y * s}; }

// TrackBeam::applyDrift / applyFQuad / applyDQuad (TrackBeam.cpp:84-116). The
// divisions by gammaz are multiplications by igz = 1 / gammaz (the products differ
// from the quotients in the last bit).
__device__ __forceinline__ void plane_step(int kind, double q, double off, double delz, double &x,
                                           double &p, double gammaz, double igz) {
  if (kind == 0) {
    x = fma(p * delz, igz, x);
  } else if (kind == 1) {
    double foc = sqrt(q * igz);
    double omg = foc * delz;
    double a1 = cos(omg);
    double a2 = sin(omg) / foc;
    double a3 = -a2 * foc * foc;
    double xtmp = x - off;
    x = a1 * xtmp + a2 * p * igz + off;
    p = a3 * xtmp * gammaz + a1 * p;
  } else {
    double foc = sqrt(-q * igz);
    double omg = foc * delz;
    double a1 = cosh(omg);
    double a2 = sinh(omg) / foc;
    double a3 = a2 * foc * foc;
    double xtmp = x - off;
    x = a1 * xtmp + a2 * p * igz + off;
    p = a3 * xtmp * gammaz + a1 * p;
  }
}

// TrackBeam::track over half a step (TrackBeam.cpp:66-76); `last` applies the
// corrector kick first (TrackBeam.cpp:37-38, 118-128).
__device__ __forceinline__ void transverse(const StepConst &sc, bool last, double g, double &x,
                                           double &y, double &px, double &py) {
  if (last && sc.corr) {
    px += sc.cxk;
    py += sc.cyk;
  } else if (!last && sc.chic) {
    // TrackBeam::applyChicane (TrackBeam.cpp:224-240): the chicane's transfer minus the
    // drift over its length, which the two half steps then add back
    const double gz = sqrt(g * g - 1 - px * px - py * py);
    double tmp = x;
    x = sc.cm[0] * tmp + sc.cm[1] * px / gz;
    px = sc.cm[2] * tmp * gz + sc.cm[3] * px;
    tmp = y;
    y = sc.cm[4] * tmp + sc.cm[5] * py / gz;
    py = sc.cm[6] * tmp * gz + sc.cm[7] * py;
  }
  const double delz = sc.half_delz;
  // 1 / gammaz by one reciprocal square root, gammaz (the quadrupoles' only) as
  // gammaz^2 / gammaz; both within an ulp or two of the reference's sqrt and quotients
  const double gz2 = fma(-py, py, fma(-px, px, fma(g, g, -1.) - sc.aw_t2));
  const double igz = rsqrt(gz2);
  const double gammaz = gz2 * igz;
  plane_step(sc.kindx, sc.qx, sc.xoff, delz, x, px, gammaz, igz);
  plane_step(sc.kindy, sc.qy, sc.yoff, delz, y, py, gammaz, igz);
}

// Field::getLLGridpoint (Field.cpp:160-174). Returns the lower-left cell and the
// weights. A particle within rounding of the upper edge can land on index
// ngrid-1, where the reference's right/upper neighbour carries weight exactly 0;
// the neighbour index is then clamped so that no access leaves the grid.
struct Cell {
  int i00, i10, i01, i11;
  double wx, wy;  // the lower-left weights, 1 - ux and 1 - uy
  double ux, uy;  // the cell coordinates' fractions: the upper/right neighbours' weights
};
// The reference divides x + gridmax by the spacing; the push forms the cell coordinate
// as fma(x, 1 / dgrid, gridmax / dgrid) with host-computed factors (the weights then
// differ in the last bit, and a particle within rounding of a cell boundary may take the
// neighbouring cell, where the bilinear weights give the same value).
// |v| < gm for gm > 0 as an integer comparison of the magnitudes' bit patterns: the
// same verdict as -gm < v < gm for every v (NaN fails both), without the FP64 pipe.
__device__ __forceinline__ bool inside(double v, double gm) {
  return (unsigned long long)(__double_as_longlong(v) & 0x7fffffffffffffffLL) <
         (unsigned long long)__double_as_longlong(gm);
}
// floor(t) and the fraction t - floor(t), both exact, for 0 <= t < 2^31, from the bit
// pattern on the integer pipe (no FP64 rounding, conversion or subtraction): the
// significand's bits below the binary point, shifted up to a normalised significand,
// are the fraction.
__device__ __forceinline__ int floor_frac(double t, double &frac) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(t);
  const int e = (int)(b >> 52) - 1023;
  if (e < 0) {  // t < 1
    frac = t;
    return 0;
  }
  const int sh = 52 - e;  // bits below the binary point
  const unsigned long long m = (b & ((1ULL << 52) - 1)) | (1ULL << 52);
  const unsigned long long fb = m & ((1ULL << sh) - 1);
  const int ip = (int)(m >> sh);
  if (fb == 0) {
    frac = 0.;
    return ip;
  }
  const int lz = __clzll((long long)fb);  // fb < 2^52: lz >= 12; its leading one at bit 63 - lz
  const unsigned long long mant = (fb << (lz - 11)) & ((1ULL << 52) - 1);
  frac = __longlong_as_double((long long)(((unsigned long long)(1023 + 63 - lz - sh) << 52) | mant));
  return ip;
}
__device__ __forceinline__ bool ll_gridpoint(double gm, double idg, double gmi, int ng, double x, double y,
                                             Cell &c) {
  if (inside(x, gm) && inside(y, gm)) {
    // x > -gm, so the coordinate is positive
    const int ix = floor_frac(fma(x, idg, gmi), c.ux), iy = floor_frac(fma(y, idg, gmi), c.uy);
    c.wx = 1. - c.ux;
    c.wy = 1. - c.uy;
    int ix1 = ix + 1 < ng ? ix + 1 : ix;
    int iy1 = iy + 1 < ng ? iy + 1 : iy;
    c.i00 = ix + iy * ng;
    c.i10 = ix1 + iy * ng;
    c.i01 = ix + iy1 * ng;
    c.i11 = ix1 + iy1 * ng;
    return true;
  }
  return false;
}

// |v| < 2^-k for the exponent field ek = 1023 - k: a comparison of the high word's
// magnitude bits (integer pipe; NaN and infinities fail)
__device__ __forceinline__ bool below_pow2(double v, int ek) {
  return (__double2hiint(v) & 0x7fffffff) < (ek << 20);
}
// 1 / x given r, the reciprocal of a nearby value: two Newton steps, each squaring
// the relative error e = 1 - x r, when |e| < 2^-17 (then the error is below 1e-20
// before rounding), else the division. The RK4 stages of a step change gamma by far
// less than that, so each stage's 1 / gamma follows from the previous one.
__device__ __forceinline__ double recip_near(double x, double r) {
  double e = fma(-x, r, 1.);
  if (!below_pow2(e, 1023 - 17)) return 1. / x;
  r = fma(r, e, r);
  e = fma(-x, r, 1.);
  return fma(r, e, r);
}

// 1 / sqrt(a) as the correctly rounded quotient of 1 by the correctly rounded square
// root (BeamSolver::ODE's btpar0 = sqrt(...), 1 / btpar0), without the square root and
// the division when a = 1 - d, |d| < 2^-14 (btpar0 is 1 - O(1 / gamma^2)):
//  - s0 = 1 - d/2 - d^2/8 - d^3/16 (Taylor series of sqrt(1 - d); the omitted terms
//    are below 2^-60) is within an ulp of sqrt(a). Tuckerman's rounding test picks
//    RN(sqrt(a)) among s0 and its neighbours: with u = next(s0) - s0, sqrt(a) lies above
//    s0 + u/2 iff a > s0 next(s0), the sign of fma(s0, next(s0), -a) (exact: a and
//    s0 next(s0) are multiples of a spacing above u^2 / 4), and the same below.
//  - q0 = 1 + e + e^2 + e^3 for e = 1 - s (exact) is within an ulp of 1 / s. The residual
//    1 - s q0 is exact, and q0 is RN(1 / s) iff it is smaller in magnitude than s g / 2,
//    g the spacing of the doubles on its side of q0 (2^-52 in [1, 2), 2^-53 below 1);
//    1 / s is never a midpoint, as s is a double.
// Both tests run on the integer pipe but the three residuals. Bit-identical to
// 1. / sqrt(a) (checked against IEEE sqrt and division on 1.5e8 arguments either side
// of 1); outside the range, sqrt and the division.
__device__ __forceinline__ double recip_sqrt_near1(double a) {
  const double d = 1. - a;
  if (!below_pow2(d, 1023 - 14)) return 1. / sqrt(a);
  double s = fma(d, fma(d, fma(d, -1. / 16., -1. / 8.), -0.5), 1.);
  const long long sb = __double_as_longlong(s);
  const double su = __longlong_as_double(sb + 1), sd = __longlong_as_double(sb - 1);
  if (__double2hiint(fma(s, su, -a)) < 0) s = su;
  else if (__double2hiint(fma(s, sd, -a)) >= 0) s = sd;
  const double e = 1. - s;
  double q = 1. + fma(fma(e, e, e), e, e);
  const long long qb = __double_as_longlong(q), rb = __double_as_longlong(fma(-s, q, 1.));
  const bool up = rb > 0;  // 1 / s > q
  const bool wide = up ? qb >= 0x3FF0000000000000LL : qb > 0x3FF0000000000000LL;
  const long long hb = __double_as_longlong(s) - ((wide ? 53LL : 54LL) << 52);  // s g / 2
  if ((rb & 0x7fffffffffffffffLL) > hb) q = __longlong_as_double(qb + (up ? 1 : -1));
  return q;
}

// BeamSolver::ODE (BeamSolver.cpp:144-163) for NF fields, given cs[i] = (cos, sin) of
// rharm_i * tthet and itg = 1 / tgam. Two of the reference's four divisions become
// products with the reciprocals 1 / tgam and 1 / btpar0 (the latter rounded as the
// reference's sqrt and quotient round it, by recip_sqrt_near1, so that xks (1 - 1/btpar0),
// which xks ~ 1e11 amplifies, is the reference's value; a last-bit change of 1 / tgam changes btper0 / tgam^2 ~ 1e-8
// far below the last bit of btpar0); ztemp1 = -2 / xks comes with the step constants.
// ACC: how the stage's derivative f enters the RK4 accumulators k2: 0 k2 = f (the first
// two stages, where the reference adds f to zero), 1 k2 = -k2 / 2 + f and 2 k2 = 2 k2 + f
// (the third and fourth, where the reference scales k2 by -0.5 or 2 first): each one
// fma, exact as the reference's product (a scaling by a power of two) and rounded sum.
template <int NF, int ACC>
__device__ __forceinline__ void ode(const StepConst &sc, const C2 *rpart, const C2 *cs, double btpar, double ez,
                                    double itg, double &k2gg, double &k2pp) {
  // sum of rpart_i conj(cs_i), products fused into the sums
  C2 ctmp = {fma(rpart[0].x, cs[0].x, rpart[0].y * cs[0].y), fma(rpart[0].y, cs[0].x, -rpart[0].x * cs[0].y)};
#pragma unroll
  for (int i = 1; i < NF; i++) {
    if (i >= sc.nfld) break;
    ctmp.x = fma(rpart[i].x, cs[i].x, fma(rpart[i].y, cs[i].y, ctmp.x));
    ctmp.y = fma(rpart[i].y, cs[i].x, fma(-rpart[i].x, cs[i].y, ctmp.y));
  }
  double btper0 = fma(sc.ztemp1, ctmp.x, btpar);
  const double ib = recip_sqrt_near1(fma(-btper0, itg * itg, 1.));
  const double fpp = fma(sc.xks, 1. - ib, sc.xku), fgg = fma(ctmp.y * ib, itg, -ez);
  if (ACC == 0) {
    k2pp = fpp;
    k2gg = fgg;
  } else {
    const double scale = ACC == 1 ? -0.5 : 2.0;
    k2pp = fma(scale, k2pp, fpp);
    k2gg = fma(scale, k2gg, fgg);
  }
}

// e^{i eps} by its Taylor series, for |eps| < 1/4: the first omitted terms are
// eps^14 / 14! (cosine) and eps^13 / 13! (sine), below 1e-19 at 1/4.
// the RK4 weights' divisions by 6 as products with 1 / 6 (a last-bit difference)
constexpr double kSixth = 1. / 6.;
__device__ __forceinline__ C2 expi_small(double e) {
  const double z = e * e;
  double c = fma(z, 1. / 479001600., -1. / 3628800.);
  c = fma(z, c, 1. / 40320.);
  c = fma(z, c, -1. / 720.);
  c = fma(z, c, 1. / 24.);
  c = fma(z, c, -0.5);
  c = fma(z, c, 1.);
  double sn = fma(z, -1. / 39916800., 1. / 362880.);
  sn = fma(z, sn, -1. / 5040.);
  sn = fma(z, sn, 1. / 120.);
  sn = fma(z, sn, -1. / 6.);
  sn = fma(z, sn, 1.);
  return {c, sn * e};
}
// The same for |eps| < 1/16, the usual case (the remainder is the phase slip of the
// particle's energy and angle offsets over a stage, ~1e-2 rad at 3 sigma of the
// benchmark beam): the first omitted terms, eps^10 / 10! and eps^11 / 11!, are below
// 2.6e-19. Ten FP64 instructions instead of thirteen.
__device__ __forceinline__ C2 expi_tiny(double e) {
  const double z = e * e;
  double c = fma(z, 1. / 40320., -1. / 720.);
  c = fma(z, c, 1. / 24.);
  c = fma(z, c, -0.5);
  c = fma(z, c, 1.);
  double sn = fma(z, 1. / 362880., -1. / 5040.);
  sn = fma(z, sn, 1. / 120.);
  sn = fma(z, sn, -1. / 6.);
  sn = fma(z, sn, 1.);
  return {c, sn * e};
}

// (cos, sin) of h theta for a phase theta = theta0 + dth near theta0 + dnom: the
// particle's e^{i h theta0} rotated by e^{i h dnom} (brot: their product, formed once
// per particle and harmonic) and by e^{i h (dth - dnom)}; sincos of h theta where the
// remainder is not small.
__device__ __forceinline__ C2 rotated(C2 brot, double h, double theta, double dth, double dnom) {
  const double e = h * (dth - dnom);
  if (below_pow2(e, 1023 - 4)) return cmul_fma(brot, expi_tiny(e));
  if (below_pow2(e, 1023 - 2)) return cmul_fma(brot, expi_small(e));
  double sn, c;
  sincos(h * theta, &sn, &c);
  return {c, sn};
}

// cs = e^{i h theta_p} rotated on to e^{i h theta} for a phase theta a small step dth =
// theta - theta_p past theta_p (RK4 stage 3 after stage 2, the deposition after stage 4:
// the stages' phase velocities differ by a few parts in 1e5 of a radian per step): for
// d = h dth below 2^-12, (1 - z/2 + z^2/24, d - d z/6) with z = d^2 (the first omitted terms
// are below 2^-72 / 720 and 2^-60 / 120); else `rotated` from the step's start.
__device__ __forceinline__ C2 rotated_on(C2 cs, double dth, C2 brot, double h, double theta, double theta0,
                                         double dnom) {
  const double d = h * dth;
  if (below_pow2(d, 1023 - 12)) {
    const double z = d * d;
    return cmul_fma(cs, C2{fma(z, fma(z, 1. / 24., -0.5), 1.), fma(d * z, -1. / 6., d)});
  }
  return rotated(brot, h, theta, theta - theta0, dnom);
}

// Deposition of one particle into the source of every field
// (FieldSolverADI.cpp:19-51; FieldSolverFFT.cpp:19-51 is identical).
// cs: (cos, sin) of rharm_k * theta of every field, or null (computed here).
// The source scale of field k for a slice of current cur and npd particles
// (FieldSolverADI.cpp:21-22), in the reference's operation order.
__device__ __forceinline__ double deposit_scale(const StepConst &sc, const FieldStep &fs, double cur, double npd) {
  double scl = fs.fc * kVacimp * cur * fs.xks * sc.delz;
  scl /= 4 * kEev * npd * fs.dgrid * fs.dgrid;
  return scl;
}

// scls: every field's deposit_scale for this slice, or null (computed here). ig: 1 / g,
// or 0 (divided here).
template <int NF>
__device__ __forceinline__ void deposit_particle(const StepConst &sc, double2 *const *src,
                                                 size_t slice_off, int ng, double cur,
                                                 double npd, double g, double th, double x,
                                                 double y, const C2 *cs = nullptr, const double *scls = nullptr,
                                                 double ig = 0.) {
#pragma unroll
  for (int k = 0; k < NF; k++) {
    if (k >= sc.nfld) break;
    const FieldStep &fs = sc.f[k];
    if (!fs.dep_on) continue;
    Cell c;
    if (!ll_gridpoint(fs.gridmax, fs.idgrid, fs.gm_idg, ng, x, y, c)) continue;
    const double scl = scls ? scls[k] : deposit_scale(sc, fs, cur, npd);
    double dx = x - sc.ax, dy = y - sc.ay;
    double faw2 = fma(2., fma(sc.grady, dy, sc.gradx * dx), fma(sc.ky * dy, dy, fma(sc.kx * dx, dx, 1.)));
    double part = ig != 0. ? sqrt(faw2) * scl * ig : sqrt(faw2) * scl / g;
    double s, co;
    if (cs) {
      co = cs[k].x;
      s = cs[k].y;
    } else {
      sincos(fs.rharm * th, &s, &co);
    }
    C2 cpart = mulr(C2{s, co}, part);
    double2 *d = src[k] + slice_off;
    double w = c.wx * c.wy;
    atomicAdd(&d[c.i00].x, w * cpart.x);
    atomicAdd(&d[c.i00].y, w * cpart.y);
    w = c.ux * c.wy;
    atomicAdd(&d[c.i10].x, w * cpart.x);
    atomicAdd(&d[c.i10].y, w * cpart.y);
    w = c.wx * c.uy;
    atomicAdd(&d[c.i01].x, w * cpart.x);
    atomicAdd(&d[c.i01].y, w * cpart.y);
    w = c.ux * c.uy;
    atomicAdd(&d[c.i11].x, w * cpart.x);
    atomicAdd(&d[c.i11].y, w * cpart.y);
  }
}

struct Ptrs {
  double *gamma, *theta, *x, *y, *px, *py;
  const double *current;
  const double2 *field[G4GPU_MAX_FIELDS];
  double2 *src[G4GPU_MAX_FIELDS];
  // space charge: the short-range field per particle and the long-range loss per
  // slice (null: zero), and which part of the step a launch runs (0 all, 1 the first
  // transverse half step, 2 the rest)
  const double *ez, *eloss;
  int mode;
  // wakes: the loss of every slice (eV/m, Collective::apply), null without them
  const double *wake;
  // particles per slice (one4one windows), null: np in every slice
  const int *count;
  // incoherent radiation: the stream of the step (ctr null: off)
  IsrStream isr;
  // the cached e^{i rharm theta} of every field ([nfield][pstride]) and its validity flag
  // (DeviceBeam::phasor), null: none
  double2 *phasor;
  const int *phasor_ok;
  size_t pstride;
};

// particles of slice is: np, or the slice's own count
__device__ __forceinline__ int slice_np(const Ptrs &p, int is, int np) {
  return p.count ? min(p.count[is], np) : np;
}

// Beam::track (Beam.cpp:296-311): half transverse step, BeamSolver::advance with
// the bilinear field gather and RK4 (BeamSolver.cpp:48-141), half transverse step
// with the corrector; then, with `deposit`, the source deposition of the
// following Field::track. One thread per particle; blockIdx.y is the slice.
template <int NF>
__global__ void __launch_bounds__(512) k_push(StepConst sc, Ptrs p, int ns, int np, int ng,
                                              int deposit) {
  int is = blockIdx.y;
  int ip = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = slice_np(p, is, np);
  // the slice's source scales, one thread per field (the block is one slice)
  __shared__ double scls[NF];
  if (deposit && threadIdx.x < NF && (int)threadIdx.x < sc.nfld)
    scls[threadIdx.x] = deposit_scale(sc, sc.f[threadIdx.x], p.current[is], (double)n);
  __syncthreads();
  if (ip >= n) return;
  size_t o = (size_t)is * np + ip;
  double g = p.gamma[o], th = p.theta[o], x = p.x[o], y = p.y[o], px = p.px[o], py = p.py[o];
  size_t ncell = (size_t)ng * ng;

  if (p.mode != 2) transverse(sc, false, g, x, y, px, py);
  if (p.mode == 1) {
    p.x[o] = x;
    p.y[o] = y;
    p.px[o] = px;
    p.py[o] = py;
    return;
  }
  // BeamSolver.cpp:50, 61: ez = the particle's short-range field + the slice's loss
  const double ez = (p.ez ? p.ez[o] : 0.) + (p.eloss ? p.eloss[is] : 0.);

  // BeamSolver::advance, BeamSolver.cpp:53-80
  double gamma = g, theta = th + sc.autophase;
  double dx = x - sc.ax, dy = y - sc.ay;
  const double awloc = fma(sc.grady, dy, fma(sc.gradx, dx, fma(0.5, fma(sc.ky * dy, dy, sc.kx * dx * dx), 1.)));
  const double btpar = fma(sc.aw2 * awloc, awloc, fma(py, py, fma(px, px, 1.)));
  C2 rpart[NF];
#pragma unroll
  for (int k = 0; k < NF; k++) {
    if (k >= sc.nfld) break;
    const FieldStep &fs = sc.f[k];
    int islice = (is + fs.first) % ns;
    const double2 *f = p.field[k] + (size_t)islice * ncell;
    Cell c;
    if (ll_gridpoint(fs.gridmax, fs.idgrid, fs.gm_idg, ng, x, y, c)) {
      // bilinear weights formed once, the four terms fused into their sum
      const double w00 = c.wx * c.wy, w10 = c.ux * c.wy, w01 = c.wx * c.uy, w11 = c.ux * c.uy;
      const C2 f00 = ld(f + c.i00), f10 = ld(f + c.i10), f01 = ld(f + c.i01), f11 = ld(f + c.i11);
      C2 cpart;
      cpart.x = fma(f11.x, w11, fma(f01.x, w01, fma(f10.x, w10, f00.x * w00)));
      cpart.y = fma(f11.y, w11, fma(f01.y, w01, fma(f10.y, w10, f00.y * w00)));
      rpart[k] = rmul(fs.rtmp * awloc, C2{cpart.x, -cpart.y});
    } else {
      rpart[k] = C2{0, 0};
    }
  }

  // e^{i h theta} of every field at the start, and rotated towards the stages: one
  // sincos per harmonic and particle instead of one per stage, or none where the last
  // push left it (the phasor of the stored phase, turned by the step's phase offset)
  const double theta0 = theta;
  const bool cached = p.phasor && *p.phasor_ok;
  C2 bhalf[NF], bfull[NF], cs[NF];
#pragma unroll
  for (int k = 0; k < NF; k++) {
    if (k >= sc.nfld) break;
    if (cached) {
      const C2 c = ld(p.phasor + k * p.pstride + o);
      cs[k] = sc.autophase != 0. ? cmul_fma(c, C2{sc.f[k].rot_auto[0], sc.f[k].rot_auto[1]}) : c;
    } else {
      double sn, c;
      sincos(sc.f[k].rharm * theta0, &sn, &c);
      cs[k] = C2{c, sn};
    }
    bhalf[k] = cmul_fma(cs[k], C2{sc.f[k].rot_half[0], sc.f[k].rot_half[1]});
    bfull[k] = cmul_fma(cs[k], C2{sc.f[k].rot_full[0], sc.f[k].rot_full[1]});
  }
  auto stage = [&](const C2 *b, double dnom) {
#pragma unroll
    for (int k = 0; k < NF; k++) {
      if (k >= sc.nfld) break;
      cs[k] = rotated(b[k], sc.f[k].rharm, theta, theta - theta0, dnom);
    }
  };

  // BeamSolver::RungeKutta, BeamSolver.cpp:89-141
  double k2gg, k2pp, k3gg, k3pp;
  double itg = 1. / gamma;  // 1 / gamma of the stage, each stage's from the previous one
  ode<NF, 0>(sc, rpart, cs, btpar, ez, itg, k2gg, k2pp);
  double stpz = sc.half_delz;
  gamma = fma(stpz, k2gg, gamma);
  theta = fma(stpz, k2pp, theta);
  k3gg = k2gg;
  k3pp = k2pp;
  stage(bhalf, sc.dnom_half);
  itg = recip_near(gamma, itg);
  ode<NF, 0>(sc, rpart, cs, btpar, ez, itg, k2gg, k2pp);
  gamma = fma(stpz, k2gg - k3gg, gamma);
  const double theta1 = theta;
  theta = fma(stpz, k2pp - k3pp, theta);
  k3gg *= kSixth;
  k3pp *= kSixth;
#pragma unroll
  for (int k = 0; k < NF; k++) {
    if (k >= sc.nfld) break;
    cs[k] = rotated_on(cs[k], theta - theta1, bhalf[k], sc.f[k].rharm, theta, theta0, sc.dnom_half);
  }
  itg = recip_near(gamma, itg);
  ode<NF, 1>(sc, rpart, cs, btpar, ez, itg, k2gg, k2pp);  // k2 = -k2 / 2 + f
  stpz = sc.delz;
  gamma = fma(stpz, k2gg, gamma);
  theta = fma(stpz, k2pp, theta);
  k3gg -= k2gg;
  k3pp -= k2pp;
  stage(bfull, sc.dnom_full);
  itg = recip_near(gamma, itg);
  ode<NF, 2>(sc, rpart, cs, btpar, ez, itg, k2gg, k2pp);  // k2 = 2 k2 + f
  const double theta3 = theta;
  gamma = fma(stpz, fma(k2gg, kSixth, k3gg), gamma);
  theta = fma(stpz, fma(k2pp, kSixth, k3pp), theta);

  // Incoherent::apply (Incoherent.cpp:66-77): one draw per beamlet of nbins particles
  if (p.isr.ctr) {
    const double u = isr_uniform(p.isr.seed, *p.isr.ctr, is, ip / p.isr.nbins);
    gamma += -sc.isr_avg + sc.isr_sig * (2 * u - 1);
  }
  // Collective::apply (Collective.cpp:119-128), before the second half step
  if (p.wake) gamma += p.wake[is] * sc.delz / kEev;
  // TrackBeam::applyR56 (TrackBeam.cpp:260-277)
  if (sc.chic) theta += sc.r56 * (gamma - sc.gammaref);

  transverse(sc, true, gamma, x, y, px, py);

  p.gamma[o] = gamma;
  p.theta[o] = theta;
  p.x[o] = x;
  p.y[o] = y;
  p.px[o] = px;
  p.py[o] = py;

  if (deposit || p.phasor) {
    // the deposition's phases, rotated on from stage 4's, kept for the next push
#pragma unroll
    for (int k = 0; k < NF; k++) {
      if (k >= sc.nfld) break;
      cs[k] = rotated_on(cs[k], theta - theta3, bfull[k], sc.f[k].rharm, theta, theta0, sc.dnom_full);
      if (p.phasor) st(p.phasor + k * p.pstride + o, cs[k]);
    }
  }
  if (deposit) {
    deposit_particle<NF>(sc, p.src, (size_t)is * ncell, ng, p.current[is], (double)n, gamma,
                         theta, x, y, cs, scls, recip_near(gamma, itg));
  }
}

// Deposition alone, for a Field::track without a preceding push.
template <int NF>
__global__ void __launch_bounds__(256) k_deposit(StepConst sc, Ptrs p, int ns, int np, int ng) {
  int is = blockIdx.y;
  int ip = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = slice_np(p, is, np);
  if (ip >= n) return;
  size_t o = (size_t)is * np + ip;
  size_t ncell = (size_t)ng * ng;
  deposit_particle<NF>(sc, p.src, (size_t)is * ncell, ng, p.current[is], (double)n, p.gamma[o],
                       p.theta[o], p.x[o], p.y[o]);
}

// ADI coefficient set: c[ng], cbet[ng], cwet[ng] (FieldSolverADI.cpp:125-182)
struct Coef {
  const double2 *c, *cbet, *cwet;
};

// Right-hand side term cstep * (second difference) with the reference's operand
// order (FieldSolverADI.cpp:64-86): (next - 2 u) + prev, one-sided at the edges.
// next - 2 u as one fma: 2 u is exact, so the single rounding of the fma is the
// reference's rounding of the difference (bit-identical, one FP64 instruction fewer)
__device__ __forceinline__ C2 sub2(C2 next, C2 u) { return {fma(-2.0, u.x, next.x), fma(-2.0, u.y, next.y)}; }
__device__ __forceinline__ C2 lap(bool has_prev, bool has_next, C2 prev, C2 u, C2 next) {
  if (!has_prev) return sub2(next, u);
  if (!has_next) return sub2(prev, u);
  return cadd(sub2(next, u), prev);
}

// First ADI half step: implicit along x (tridagx, FieldSolverADI.cpp:63-75, 94-104).
// One thread per (slice, row); writes the intermediate field to tmp.
__global__ void __launch_bounds__(128) k_adi_x(const double2 *__restrict__ field,
                                               const double2 *__restrict__ src,
                                               double2 *__restrict__ tmp, Coef cf, double cstep,
                                               int ns, int ng, int first) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ns * ng) return;
  int ii = (int)(t / ng), iy = (int)(t % ng);
  size_t ncell = (size_t)ng * ng;
  int i = (ii + first) % ns;
  const double2 *u = field + (size_t)i * ncell + (size_t)iy * ng;
  // a null source means no deposition this step (outside the undulator or an even
  // harmonic): the reference then solves with a zero source (FieldSolverADI.cpp:14-16)
  const double2 *s = src ? src + (size_t)ii * ncell + (size_t)iy * ng : nullptr;
  double2 *w = tmp + (size_t)i * ncell + (size_t)iy * ng;
  bool hp = iy > 0, hn = iy < ng - 1;
  C2 prev = {0, 0};
  for (int k = 0; k < ng; k++) {
    C2 uc = ld(u + k);
    C2 un = hn ? ld(u + k + ng) : C2{0, 0};
    C2 us = hp ? ld(u + k - ng) : C2{0, 0};
    C2 sv = s ? ld(s + k) : C2{0, 0};
    C2 r = add_imul(cadd(sv, uc), cstep, lap(hp, hn, us, uc, un));
    // r - c[k] u_{k-1} with c[k] = (0, -mlow[k]); c[0] = 0
    C2 v = (k == 0) ? cmul_fma(r, ld(cf.cbet)) : cmul_fma(add_imul(r, -cf.c[k].y, prev), ld(cf.cbet + k));
    st(w + k, v);
    prev = v;
  }
  C2 next = prev;
  for (int k = ng - 2; k >= 0; k--) {
    C2 v = sub_cmul(ld(w + k), ld(cf.cwet + k + 1), next);
    st(w + k, v);
    next = v;
  }
}

// Second ADI half step: implicit along y (tridagy, FieldSolverADI.cpp:77-89, 106-122).
// One thread per (slice, column); reads tmp, writes the field.
__global__ void __launch_bounds__(128) k_adi_y(double2 *__restrict__ field,
                                               const double2 *__restrict__ src,
                                               const double2 *__restrict__ tmp, Coef cf,
                                               double cstep, int ns, int ng, int first) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ns * ng) return;
  int ii = (int)(t / ng), ix = (int)(t % ng);
  size_t ncell = (size_t)ng * ng;
  int i = (ii + first) % ns;
  double2 *u = field + (size_t)i * ncell + ix;
  const double2 *s = src ? src + (size_t)ii * ncell + ix : nullptr;
  const double2 *w = tmp + (size_t)i * ncell + ix;
  bool hp = ix > 0, hn = ix < ng - 1;
  C2 prev = {0, 0};
  for (int k = 0; k < ng; k++) {
    size_t o = (size_t)k * ng;
    C2 wc = ld(w + o);
    C2 wn = hn ? ld(w + o + 1) : C2{0, 0};
    C2 wp = hp ? ld(w + o - 1) : C2{0, 0};
    C2 sv = s ? ld(s + o) : C2{0, 0};
    C2 r = add_imul(cadd(sv, wc), cstep, lap(hp, hn, wp, wc, wn));
    C2 v = (k == 0) ? cmul_fma(r, ld(cf.cbet)) : cmul_fma(add_imul(r, -cf.c[k].y, prev), ld(cf.cbet + k));
    st(u + o, v);
    prev = v;
  }
  C2 next = prev;
  for (int k = ng - 2; k >= 0; k--) {
    size_t o = (size_t)k * ng;
    C2 v = sub_cmul(ld(u + o), ld(cf.cwet + k + 1), next);
    st(u + o, v);
    next = v;
  }
}

// ---- diagnostics: per-slice FP64 sums, finished on the host -----------------
template <int BS>
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < BS / 32; i++) r += sh[i];
  return r;
}
template <int BS, bool MAX>
__device__ __forceinline__ double block_ext(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_down_sync(0xffffffffu, v, o);
    v = MAX ? fmax(v, w) : fmin(v, w);
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = sh[0];
  if (threadIdx.x == 0)
    for (int i = 1; i < BS / 32; i++) r = MAX ? fmax(r, sh[i]) : fmin(r, sh[i]);
  return r;
}

// DiagBeam::getValues sums (Diagnostic.cpp:415-456): one block per slice.
template <int BS>
__global__ void __launch_bounds__(BS) k_diag_beam(Ptrs p, int np, int nharm, double *out) {
  __shared__ double sh[BS / 32];
  int is = blockIdx.x;
  size_t base = (size_t)is * np;
  const int n = slice_np(p, is, np);
  double s[kBeamSums] = {0};
  double mn[5] = {1e5, 1e5, 1e5, 1e5, 1e7}, mx[5] = {-1e5, -1e5, -1e5, -1e5, 1};
  double br[G4GPU_MAX_HARM], bi[G4GPU_MAX_HARM];
  for (int h = 0; h < G4GPU_MAX_HARM; h++) br[h] = bi[h] = 0;
  for (int ip = threadIdx.x; ip < n; ip += BS) {
    double x = p.x[base + ip], y = p.y[base + ip], g = p.gamma[base + ip];
    double px = p.px[base + ip], py = p.py[base + ip], th = p.theta[base + ip];
    s[0] += g; s[1] += g * g; s[2] += x; s[3] += x * x; s[4] += y; s[5] += y * y;
    s[6] += px; s[7] += px * px; s[8] += py; s[9] += py * py; s[10] += x * px; s[11] += y * py;
    mn[0] = fmin(mn[0], x); mx[0] = fmax(mx[0], x);
    mn[1] = fmin(mn[1], px); mx[1] = fmax(mx[1], px);
    mn[2] = fmin(mn[2], y); mx[2] = fmax(mx[2], y);
    mn[3] = fmin(mn[3], py); mx[3] = fmax(mx[3], py);
    mn[4] = fmin(mn[4], g); mx[4] = fmax(mx[4], g);
    for (int h = 0; h < nharm && h < G4GPU_MAX_HARM; h++) {
      double sn, cs;
      sincos((h + 1) * th, &sn, &cs);
      br[h] += cs;
      bi[h] += sn;
    }
  }
  int w = beam_diag_width(nharm);
  double *o = out + (size_t)is * w;
  for (int k = 0; k < kBeamSums; k++) {
    double r = block_sum<BS>(s[k], sh);
    if (threadIdx.x == 0) o[k] = r;
  }
  for (int k = 0; k < 5; k++) {
    double a = block_ext<BS, false>(mn[k], sh);
    if (threadIdx.x == 0) o[kBeamSums + 2 * k] = a;
    double b = block_ext<BS, true>(mx[k], sh);
    if (threadIdx.x == 0) o[kBeamSums + 2 * k + 1] = b;
  }
  for (int h = 0; h < nharm && h < G4GPU_MAX_HARM; h++) {
    double a = block_sum<BS>(br[h], sh);
    double b = block_sum<BS>(bi[h], sh);
    if (threadIdx.x == 0) {
      o[kBeamSums + kBeamMinMax + 2 * h] = a;
      o[kBeamSums + kBeamMinMax + 2 * h + 1] = b;
    }
  }
}

// DiagField::getValues sums (Diagnostic.cpp:754-776): one block per storage slot.
template <int BS>
__global__ void __launch_bounds__(BS) k_diag_field(const double2 *field, int ng, double *out) {
  __shared__ double sh[BS / 32];
  int is0 = blockIdx.x;
  size_t ncell = (size_t)ng * ng;
  const double2 *f = field + (size_t)is0 * ncell;
  double shift = -0.5 * (double)(ng - 1);
  double s[7] = {0};
  for (size_t i = threadIdx.x; i < ncell; i += BS) {
    int iy = (int)(i / ng), ix = (int)(i % ng);
    double dx = (double)ix + shift, dy = (double)iy + shift;
    double2 v = f[i];
    double wei = v.x * v.x + v.y * v.y;
    s[0] += wei; s[1] += dx * wei; s[2] += dx * dx * wei; s[3] += dy * wei; s[4] += dy * dy * wei;
    s[5] += v.x; s[6] += v.y;
  }
  double *o = out + (size_t)is0 * (kFieldSums + 2);
  for (int k = 0; k < 7; k++) {
    double r = block_sum<BS>(s[k], sh);
    if (threadIdx.x == 0) o[k] = r;
  }
  if (threadIdx.x == 0) {
    double2 v = f[(size_t)(ng / 2) * ng + ng / 2];
    o[7] = v.x;
    o[8] = v.y;
  }
}

Ptrs make_ptrs(const DeviceBeam &b, void *const *field, void *const *src, int nfld) {
  Ptrs p{};
  p.gamma = (double *)b.gamma;
  p.theta = (double *)b.theta;
  p.x = (double *)b.x;
  p.y = (double *)b.y;
  p.px = (double *)b.px;
  p.py = (double *)b.py;
  p.current = b.current;
  p.count = b.count;
  p.phasor = (double2 *)b.phasor;
  p.phasor_ok = b.phasor_ok;
  for (int k = 0; k < nfld && k < G4GPU_MAX_FIELDS; k++) {
    p.field[k] = field ? (const double2 *)field[k] : nullptr;
    p.src[k] = src ? (double2 *)src[k] : nullptr;
  }
  return p;
}

// FP64 space charge in the reference's arithmetic
struct PlainSC {
  using R = double;
  using R2 = double2;
  using Th = double;
  using Step = StepConst;
  static constexpr bool kPlain = true;
  static __device__ __forceinline__ double gamma(const StepConst &, double g) { return g; }
  static __device__ __forceinline__ void half(const StepConst &s, double g, double &x, double &y, double &px,
                                              double &py) {
    transverse(s, false, g, x, y, px, py);
  }
  static __device__ __forceinline__ double2 eil(double th, int l) {
    double s, c;
    sincos((double)l * th, &s, &c);
    return make_double2(c, -s);
  }
};

}  // namespace
}  // namespace g4

#include "sc_kernels.cuh"

namespace g4 {

namespace {

// Collective::update for one rank (Collective.cpp:144-161): the window's current
// interpolated to the fine grid, in electrons per fine slice, and its derivative
__global__ void k_wake_profile(const double *cur, int ncur, int ns_hr, double ds, double dscur, double *curh,
                               double *dcur) {
  const int is = blockIdx.x * blockDim.x + threadIdx.x;
  if (is >= ns_hr) return;
  const double s = ds * (double)is;
  unsigned idx = (unsigned)(int)floor(s / dscur);
  if (idx > (unsigned)ncur) idx = (unsigned)ncur;  // s < ncur dscur: never taken
  const double c0 = idx < (unsigned)ncur ? cur[idx] : 0., c1 = idx + 1 < (unsigned)ncur ? cur[idx + 1] : 0.;
  const double wei = 1 - (s - idx * dscur) / dscur;
  double v = wei * c0 + (1 - wei) * c1;
  v *= ds / kCe;
  curh[is] = v;
  dcur[is] = -(c1 - c0) * ds / kCe / dscur;
}

// Collective.cpp:167-179: the wake of slice ic from the fine points ahead of each of
// its `sample` fine points, averaged; loss = external + wake (eV/m), lossf = loss / eev
// in FP32 for the mixed push. One CTA per slice.
__global__ void __launch_bounds__(256) k_wake_slices(const double *curh, const double *dcur, const double *res,
                                                     const double *geo, const double *rou, const double *ext,
                                                     int ns_hr, int sample, double *loss, float *lossf) {
  __shared__ double red[256 / 32];
  const int ic = blockIdx.x, tid = threadIdx.x;
  double w = 0;
  for (int j = 0; j < sample; j++) {
    const int is = ic * sample + j;
    for (int i = tid; i < ns_hr - is; i += blockDim.x) {
      w += curh[is + i] * (res[i] + rou[i]);
      w += dcur[is + i] * geo[i];
    }
  }
  for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  if ((tid & 31) == 0) red[tid >> 5] = w;
  __syncthreads();
  if (tid == 0) {
    double t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    const double l = ext[ic] + t / (double)sample;
    loss[ic] = l;
    lossf[ic] = (float)(l / kEev);
  }
}

}  // namespace

void launch_wake_update(const Launch &L, const double *cur, int nslice, int ns_hr, double ds, const double *ext,
                        const double *res, const double *geo, const double *rou, double *scratch, double *loss,
                        float *lossf) {
  cudaStream_t s = (cudaStream_t)L.stream;
  const double dscur = ds * (unsigned)ns_hr / nslice;
  int sample = (int)(dscur / ds);
  if (sample < 1) sample = 1;
  k_wake_profile<<<(ns_hr + 255) / 256, 256, 0, s>>>(cur, nslice, ns_hr, ds, dscur, scratch, scratch + ns_hr);
  k_wake_slices<<<nslice, 256, 0, s>>>(scratch, scratch + ns_hr, res, geo, rou, ext, ns_hr, sample, loss, lossf);
}

size_t sc_bytes_per_mode(int ng, int mixed) {
  return (size_t)ng * (mixed ? sizeof(float2) + sizeof(float) : sizeof(double2) + sizeof(double));
}
size_t sc_max_smem() { return 220 * 1024; }

void launch_sc_plain(const Launch &L, const ScConst &c, const StepConst &step, const DeviceBeam &b,
                     const ScBuffers &buf, int part) {
  ScBeam<PlainSC> sb{(double *)b.gamma, (double *)b.x,           (double *)b.y, (double *)b.px,
                     (double *)b.py,    (const double *)b.theta, b.current,    b.count};
  sc_launch<PlainSC>(L, c, step, sb, buf, part);
}

void launch_push_plain(const Launch &L, const StepConst &sc, const DeviceBeam &b,
                       void *const *field, void *const *src, int ns, int np, int ngrid,
                       int deposit, int block) {
  launch_push_plain_sc(L, sc, b, field, src, ns, np, ngrid, deposit, block, 0, nullptr, nullptr, nullptr,
                       IsrStream{});
}

namespace {
__global__ void k_isr_advance(unsigned long long *ctr) { *ctr += 1; }
}  // namespace

void launch_isr_advance(void *stream, unsigned long long *ctr) {
  k_isr_advance<<<1, 1, 0, (cudaStream_t)stream>>>(ctr);
}

void launch_push_plain_sc(const Launch &L, const StepConst &sc, const DeviceBeam &b, void *const *field,
                          void *const *src, int ns, int np, int ngrid, int deposit, int block, int mode,
                          const void *ez, const double *eloss, const void *wake, const IsrStream &isr) {
  Ptrs p = make_ptrs(b, field, src, sc.nfld);
  if (isr.ctr && (sc.isr_avg != 0 || sc.isr_sig != 0) && mode != 1) p.isr = isr;
  p.mode = mode;
  p.ez = (const double *)ez;
  p.eloss = eloss;
  p.wake = (const double *)wake;
  if (mode == 1) deposit = 0;
  p.pstride = (size_t)ns * np;
  // a launch that only moves the particles transversely leaves theta and the cache as
  // they are
  if (mode == 1) p.phasor = nullptr;
  dim3 grid((np + block - 1) / block, ns);
  cudaStream_t s = (cudaStream_t)L.stream;
  switch (sc.nfld) {
    case 1: k_push<1><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
    case 2: k_push<2><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
    case 3: k_push<3><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
    default: k_push<G4GPU_MAX_FIELDS><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
  }
  // every particle's phasor now matches its phase (bytes of 1: a nonzero flag)
  if (p.phasor) cudaMemsetAsync((void *)p.phasor_ok, 1, sizeof(int), s);
}

void launch_deposit_plain(const Launch &L, const StepConst &sc, const DeviceBeam &b,
                          void *const *src, int ns, int np, int ngrid) {
  Ptrs p = make_ptrs(b, nullptr, src, sc.nfld);
  dim3 grid((np + 255) / 256, ns);
  cudaStream_t s = (cudaStream_t)L.stream;
  switch (sc.nfld) {
    case 1: k_deposit<1><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
    case 2: k_deposit<2><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
    case 3: k_deposit<3><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
    default: k_deposit<G4GPU_MAX_FIELDS><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
  }
}

void launch_adi_plain(const Launch &L, const StepConst &sc, int k, int phase, void *field,
                      const void *src, void *tmp, const void *coef, int ns, int ngrid) {
  const double2 *cb = (const double2 *)coef;
  cudaStream_t s = (cudaStream_t)L.stream;
  // One thread per grid line over all slices. The FP64 ADI is bound by the FP64 rate
  // (about 76 FP64 operations per cell and step; GB300 runs FP64 at 1/64 of the FP32
  // rate), not by memory: these kernels keep every line's sweep as the reference's single
  // sequential pass. The tiled passes of adi_tiled.cuh, which split lines into segments
  // with redundant warm-up work, were measured slower for this form.
  Coef cf{cb, cb + ngrid, cb + 2 * ngrid};
  long long n = (long long)ns * ngrid;
  unsigned blocks = (unsigned)((n + 127) / 128);
  if (phase == 0)
    k_adi_x<<<blocks, 128, 0, s>>>((const double2 *)field, (const double2 *)src, (double2 *)tmp,
                                   cf, sc.f[k].cstep, ns, ngrid, sc.f[k].first);
  else
    k_adi_y<<<blocks, 128, 0, s>>>((double2 *)field, (const double2 *)src, (const double2 *)tmp,
                                   cf, sc.f[k].cstep, ns, ngrid, sc.f[k].first);
}

void launch_diag_beam_plain(const Launch &L, const DeviceBeam &b, int ns, int np, int nharm,
                            double *out) {
  Ptrs p = make_ptrs(b, nullptr, nullptr, 0);
  k_diag_beam<256><<<ns, 256, 0, (cudaStream_t)L.stream>>>(p, np, nharm, out);
}

void launch_diag_field_plain(const Launch &L, const void *field, int ns, int ngrid,
                             double *out) {
  k_diag_field<256><<<ns, 256, 0, (cudaStream_t)L.stream>>>((const double2 *)field, ngrid, out);
}

}  // namespace g4
