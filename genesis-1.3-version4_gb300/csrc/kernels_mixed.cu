// Mixed-precision kernels of the undulator step: FP32 field, ADI solve,
// deposition and transverse optics; FP64 accumulated ponderomotive phase.
//
// Storage: the accumulated phase theta is a 64-bit fixed-point count of turns
// (Q32.32: integer turns in the high word, 2^-32 turn = 1.5e-9 rad in the low word);
// gamma is the FP32 offset from gammaref (|offset| is a few units, so FP32 resolves
// it to ~1e-7); x, y, px, py FP32; fields float2.
//
// Why fixed point and not FP64 for the phase: GB300 executes FP64 at 1/64 of the
// FP32 rate, and the seven FP64 operations per particle of an FP64 phase (add the
// step increment, reduce modulo 2 pi, convert) kept the FP64 pipe 55 % busy and
// bounded the push. The 64-bit integer accumulates without any rounding, reduces
// modulo 2 pi by taking the low word, and gives exact harmonics (h * low word mod
// 2^32); its 1.5e-9 rad resolution is far below the ~5e-7 rad FP32 error of one
// step's increment, so it loses nothing an FP64 phase would keep. Host copies
// convert to and from the reference's FP64 theta.
//
// Numerics that differ in form (not in value) from the reference's FP64 code:
//  * the RK4 stages and the deposition work on FP32 offsets from the reduced phase;
//  * 1 - 1/beta_par is evaluated as -eps / (s (1 + s)), s = sqrt(1 - eps), which
//    has no cancellation in FP32 (eps ~ 1e-8);
//  * RK4 is written in its classic form, algebraically identical to the reference's
//    "pushp" sequence (BeamSolver.cpp:89-141).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <atomic>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "g4gpu_internal.h"
#include "philox.cuh"

// Scratch of g4gpu_adi_advance_noalloc: 32 MiB, shared by every call on a device and
// held by every device that loads this module until the process exits. Host code
// uses the name only to look up the device address (cudaGetSymbolAddress).
static __device__ __align__(256) unsigned char g4_noalloc_scratch[32u << 20];

namespace g4 {

constexpr double kTwoPiHost = 6.283185307179586476925286766559;

StepConstF to_float(const StepConst &s, int npart) {
  StepConstF f{};
  f.aw_t = (float)s.aw_t;
  f.qx = (float)s.qx;
  f.qy = (float)s.qy;
  f.xoff = (float)s.xoff;
  f.yoff = (float)s.yoff;
  f.cxk = (float)s.cxk;
  f.cyk = (float)s.cyk;
  f.kindx = s.kindx;
  f.kindy = s.kindy;
  f.corr = s.corr;
  f.nfld = s.nfld;
  f.aw = (float)s.aw;
  f.ax = (float)s.ax;
  f.ay = (float)s.ay;
  f.kx = (float)s.kx;
  f.ky = (float)s.ky;
  f.gradx = (float)s.gradx;
  f.grady = (float)s.grady;
  f.xks = (float)s.xks;
  f.xku = (float)s.xku;
  f.delz = (float)s.delz;
  f.ztemp1 = (float)(-2. / s.xks);
  f.autophase = s.autophase;
  f.autophase_q = (long long)llrint(s.autophase * (4294967296.0 / kTwoPiHost));
  f.gammaref = s.gammaref;
  f.chic = s.chic;
  for (int i = 0; i < 8; i++) f.cm[i] = (float)s.cm[i];
  f.r56 = (float)s.r56;
  f.isr_avg = (float)s.isr_avg;
  f.isr_sig = (float)s.isr_sig;
  for (int k = 0; k < G4GPU_MAX_FIELDS; k++) {
    const FieldStep &a = s.f[k];
    FieldStepF &b = f.f[k];
    b.rtmp = (float)a.rtmp;
    b.rharm = (float)a.rharm;
    b.gridmax = (float)a.gridmax;
    b.dgrid = (float)a.dgrid;
    b.cstep = (float)a.cstep;
    b.dep_scl = a.dgrid > 0 ? (float)(a.fc * kVacimp * a.xks * s.delz /
                                      (4 * kEev * (double)npart * a.dgrid * a.dgrid))
                            : 0.f;
    b.dep_on = a.dep_on;
    b.coef = a.coef;
    b.first = a.first;
    b.harm = (int)a.rharm;
    b.tw = a.tw;
  }
  return f;
}

namespace {

constexpr float kTwoPiF = 6.283185307f;
// radians per unit of the low word of the fixed-point phase
constexpr float kRadPerUnit = 6.283185307f / 4294967296.0f;

// phase in [-pi, pi) of a Q32.32 turn count, optionally times a harmonic number
__device__ __forceinline__ float phase_of(long long t, unsigned h = 1u) {
  return (float)(int)((unsigned)t * h) * kRadPerUnit;
}
// adds an FP32 angle increment (radians) to a Q32.32 turn count without rounding
// the accumulator: the integer turns and the 32-bit fraction are added separately
__device__ __forceinline__ long long add_phase(long long t, float dth) {
  float turns = dth * (1.0f / 6.283185307f);
  float k = floorf(turns);
  float f = turns - k;  // exact, in [0, 1)
  unsigned fu = (unsigned)(f * 4294967296.0f);
  return t + ((long long)(int)k << 32) + (long long)fu;
}
constexpr float kInvTwoPiF = 0.159154943f;

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// r - c d for a coefficient c = (0, cy) with zero real part: the ADI's off-diagonal
// coefficients c[k] = (0, -mlow[k]) and cstep are purely imaginary
// (FieldSolverADI.cpp:139, 161-165), so c d = (-cy d.y, cy d.x): two FMAs instead of
// a complex product and a difference
__device__ __forceinline__ float2 sub_imulf(float2 r, float cy, float2 d) {
  return make_float2(fmaf(cy, d.y, r.x), fmaf(-cy, d.x, r.y));
}
// v - w x for complex w, both products fused into the difference
__device__ __forceinline__ float2 sub_cmulf(float2 v, float2 w, float2 x) {
  return make_float2(fmaf(-w.x, x.x, fmaf(w.y, x.y, v.x)), fmaf(-w.x, x.y, fmaf(-w.y, x.x, v.y)));
}
// reduces an FP32 angle of moderate size (|a| < ~1e3) to [-pi, pi]
__device__ __forceinline__ float wrapf(float a) { return fmaf(-kTwoPiF, rintf(a * kInvTwoPiF), a); }

__device__ __forceinline__ void plane_step_f(int kind, float q, float off, float delz, float &x,
                                             float &p, float gz) {
  if (kind == 0) {
    x += p * delz / gz;
  } else if (kind == 1) {
    float foc = sqrtf(q / gz), omg = foc * delz, s, c;
    sincosf(omg, &s, &c);
    float a2 = s / foc, a3 = -a2 * foc * foc, xt = x - off;
    x = c * xt + a2 * p / gz + off;
    p = a3 * xt * gz + c * p;
  } else {
    float foc = sqrtf(-q / gz), omg = foc * delz;
    float a1 = coshf(omg), a2 = sinhf(omg) / foc, a3 = a2 * foc * foc, xt = x - off;
    x = a1 * xt + a2 * p / gz + off;
    p = a3 * xt * gz + a1 * p;
  }
}

// TrackBeam::track over half a step in FP32; g is the full Lorentz factor.
__device__ __forceinline__ void transverse_f(const StepConstF &sc, bool last, float g, float &x,
                                             float &y, float &px, float &py) {
  if (last && sc.corr) {
    px += sc.cxk;
    py += sc.cyk;
  } else if (!last && sc.chic) {
    // TrackBeam::applyChicane (TrackBeam.cpp:224-240)
    const float gz = g * sqrtf(1.f - (1.f + px * px + py * py) / (g * g));
    float tmp = x;
    x = sc.cm[0] * tmp + sc.cm[1] * px / gz;
    px = sc.cm[2] * tmp * gz + sc.cm[3] * px;
    tmp = y;
    y = sc.cm[4] * tmp + sc.cm[5] * py / gz;
    py = sc.cm[6] * tmp * gz + sc.cm[7] * py;
  }
  float a = 1.f + sc.aw_t * sc.aw_t + px * px + py * py;
  float gz = g * sqrtf(1.f - a / (g * g));
  float dz = 0.5f * sc.delz;
  plane_step_f(sc.kindx, sc.qx, sc.xoff, dz, x, px, gz);
  plane_step_f(sc.kindy, sc.qy, sc.yoff, dz, y, py, gz);
}

struct CellF {
  int i00, i10, i01, i11;
  float wx, wy;
};
__device__ __forceinline__ bool ll_gridpoint_f(float gm, float dg, int ng, float x, float y, CellF &c) {
  if ((x > -gm) && (x < gm) && (y > -gm) && (y < gm)) {
    float wx = (x + gm) / dg, wy = (y + gm) / dg;
    float fx = floorf(wx), fy = floorf(wy);
    int ix = min((int)fx, ng - 1), iy = min((int)fy, ng - 1);
    c.wx = 1.f + fx - wx;
    c.wy = 1.f + fy - wy;
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

// e^{-i h a} for the harmonics of one ODE evaluation, a in [-pi, pi] + small
template <int NF>
__device__ __forceinline__ void ode_f(const StepConstF &sc, const float2 *rpart, float btpar, float ez,
                                      float g, float a, float &dgam, float &dth) {
  float2 ctmp = make_float2(0.f, 0.f);
#pragma unroll
  for (int i = 0; i < NF; i++) {
    if (i >= sc.nfld) break;
    float s, c;
    __sincosf(wrapf(sc.f[i].rharm * a), &s, &c);
    ctmp.x += rpart[i].x * c + rpart[i].y * s;
    ctmp.y += rpart[i].y * c - rpart[i].x * s;
  }
  float btper0 = btpar + sc.ztemp1 * ctmp.x;
  float eps = btper0 / (g * g);
  float s = sqrtf(1.f - eps);
  dth = -sc.xks * eps / (s * (1.f + s)) + sc.xku;
  dgam = ctmp.y / (s * g) - ez;
}

struct PtrsF {
  float *dg, *x, *y, *px, *py;
  long long *theta;  // Q32.32 turns
  const double *current;
  const float2 *field[G4GPU_MAX_FIELDS];
  float2 *src[G4GPU_MAX_FIELDS];
  // space charge: the short-range field per particle and the long-range loss per
  // slice (null: zero), and which part of the step a push launch runs (0 all, 1 the
  // first transverse half step, 2 the rest)
  const float *ez;
  const double *eloss;
  int mode;
  // wakes: the loss of every slice over eev (1/m, Collective::apply), null without them
  const float *wake;
  // particles per slice (one4one windows), null: np in every slice
  const int *count;
  // incoherent radiation: the stream of the step (ctr null: off)
  IsrStream isr;
};

// the field storage slot (is + first) % ns of beam slice is, for is and first in
// [0, ns): a compare instead of an integer division per thread
__device__ __forceinline__ int ring_slot(int is, int first, int ns) {
  const int t = is + first;
  return t >= ns ? t - ns : t;
}

// particles of slice is: np, or the slice's own count
__device__ __forceinline__ int slice_np_f(const PtrsF &p, int is, int np) {
  return p.count ? min(p.count[is], np) : np;
}
// the current the deposition scales with: dep_scl holds 1 / npart, and the reference
// divides by the slice's own particle count (FieldSolverADI.cpp:27)
__device__ __forceinline__ float slice_cur_f(const PtrsF &p, int is, int np) {
  const float cur = (float)p.current[is];
  if (!p.count) return cur;
  const int n = min(p.count[is], np);
  return n > 0 ? cur * ((float)np / (float)n) : 0.f;
}

// Deposition into the global source grids (FieldSolverADI.cpp:11-52) by a whole
// warp. The particles of a beamlet (nbins consecutive particles of the quiet
// loading) keep bit-identical x and y in FP32 for many steps, so they share the
// cell and the bilinear weights: aligned groups of 2, 4 or 8 lanes with identical
// positions first sum their complex amplitudes by shuffles, and one lane of the
// group adds weight x sum to the four cells. Every shuffle is executed by all 32
// lanes before any predicate uses its result; lanes without a particle (`valid`
// false) take part in the shuffles and contribute nothing.
template <int NF>
__device__ __forceinline__ void deposit_f(const StepConstF &sc, const PtrsF &p, size_t off, int ng,
                                          float cur, float g, long long th, float x, float y, bool valid) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const float x1 = __shfl_xor_sync(full, x, 1), y1 = __shfl_xor_sync(full, y, 1);
  const float x2 = __shfl_xor_sync(full, x, 2), y2 = __shfl_xor_sync(full, y, 2);
  const float x4 = __shfl_xor_sync(full, x, 4), y4 = __shfl_xor_sync(full, y, 4);
  const int v1 = __shfl_xor_sync(full, (int)valid, 1);
  const bool e1 = valid && v1 && x == x1 && y == y1;
  const int e1p = __shfl_xor_sync(full, (int)e1, 2);
  const bool e2 = e1 && e1p && x == x2 && y == y2;
  const int e2p = __shfl_xor_sync(full, (int)e2, 4);
  const bool e4 = e2 && e2p && x == x4 && y == y4;
  const int gsize = e4 ? 8 : (e2 ? 4 : (e1 ? 2 : 1));
  const bool leader = valid && (lane & (gsize - 1)) == 0;
  float dx = x - sc.ax, dy = y - sc.ay;
  float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
  float base = valid ? sqrtf(faw2) / g : 0.f;
#pragma unroll
  for (int k = 0; k < NF; k++) {
    if (k >= sc.nfld) break;
    const FieldStepF &fs = sc.f[k];
    if (!fs.dep_on) continue;
    CellF c;
    const bool on = valid && ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x, y, c);
    float2 cp = make_float2(0.f, 0.f);
    if (on) {
      float part = base * fs.dep_scl * cur;
      float s, co;
      __sincosf(phase_of(th, (unsigned)fs.harm), &s, &co);
      cp = make_float2(s * part, co * part);
    }
    float tx = __shfl_xor_sync(full, cp.x, 1), ty = __shfl_xor_sync(full, cp.y, 1);
    if (e1) cp = make_float2(cp.x + tx, cp.y + ty);
    tx = __shfl_xor_sync(full, cp.x, 2);
    ty = __shfl_xor_sync(full, cp.y, 2);
    if (e2) cp = make_float2(cp.x + tx, cp.y + ty);
    tx = __shfl_xor_sync(full, cp.x, 4);
    ty = __shfl_xor_sync(full, cp.y, 4);
    if (e4) cp = make_float2(cp.x + tx, cp.y + ty);
    if (on && leader) {
      float2 *d = p.src[k] + off;
      float w = c.wx * c.wy;
      atomicAdd(d + c.i00, make_float2(w * cp.x, w * cp.y));
      w = (1.f - c.wx) * c.wy;
      atomicAdd(d + c.i10, make_float2(w * cp.x, w * cp.y));
      w = c.wx * (1.f - c.wy);
      atomicAdd(d + c.i01, make_float2(w * cp.x, w * cp.y));
      w = (1.f - c.wx) * (1.f - c.wy);
      atomicAdd(d + c.i11, make_float2(w * cp.x, w * cp.y));
    }
  }
}

// Beam::track of one particle of slice `is` after its first transverse half step
// (Beam.cpp:97-112): the field gather of BeamSolver::advance (BeamSolver.cpp:48-86)
// from fslice[k], the storage slice of field k this beam slice sees, RK4 of the
// energy offset and phase, incoherent radiation, wakes, R56, the second transverse
// half step. th already holds the autophase shift.
template <int NF>
__device__ __forceinline__ void push_rest_f(const StepConstF &sc, const PtrsF &p, const float2 *const *fslice,
                                            int is, int ip, int ng, float ez, float &dg, long long &th, float &x,
                                            float &y, float &px, float &py) {
  const float g0 = (float)sc.gammaref;
  // the step works on FP32 offsets from the reduced phase
  float a0 = phase_of(th);

  float ddx = x - sc.ax, ddy = y - sc.ay;
  float awloc = 1.f + 0.5f * (sc.kx * ddx * ddx + sc.ky * ddy * ddy) + sc.gradx * ddx + sc.grady * ddy;
  float btpar = 1.f + px * px + py * py + sc.aw * sc.aw * awloc * awloc;
  float2 rpart[NF];
#pragma unroll
  for (int k = 0; k < NF; k++) {
    if (k >= sc.nfld) break;
    const FieldStepF &fs = sc.f[k];
    const float2 *f = fslice[k];
    CellF c;
    if (ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x, y, c)) {
      float2 v00 = f[c.i00], v10 = f[c.i10], v01 = f[c.i01], v11 = f[c.i11];
      float w00 = c.wx * c.wy, w10 = (1.f - c.wx) * c.wy, w01 = c.wx * (1.f - c.wy),
            w11 = (1.f - c.wx) * (1.f - c.wy);
      float cr = v00.x * w00 + v10.x * w10 + v01.x * w01 + v11.x * w11;
      float ci = v00.y * w00 + v10.y * w10 + v01.y * w01 + v11.y * w11;
      float r = fs.rtmp * awloc;
      rpart[k] = make_float2(r * cr, -r * ci);
    } else {
      rpart[k] = make_float2(0.f, 0.f);
    }
  }

  // classic RK4 on (gamma offset, phase offset)
  const float h = sc.delz, h2 = 0.5f * sc.delz;
  float k1g, k1t, k2g, k2t, k3g, k3t, k4g, k4t;
  ode_f<NF>(sc, rpart, btpar, ez, g0 + dg, a0, k1g, k1t);
  ode_f<NF>(sc, rpart, btpar, ez, g0 + (dg + h2 * k1g), a0 + h2 * k1t, k2g, k2t);
  ode_f<NF>(sc, rpart, btpar, ez, g0 + (dg + h2 * k2g), a0 + h2 * k2t, k3g, k3t);
  ode_f<NF>(sc, rpart, btpar, ez, g0 + (dg + h * k3g), a0 + h * k3t, k4g, k4t);
  const float h6 = sc.delz * (1.f / 6.f);
  float dgam = h6 * (k1g + 2.f * k2g + 2.f * k3g + k4g);
  float dth = h6 * (k1t + 2.f * k2t + 2.f * k3t + k4t);
  dg += dgam;
  // Incoherent::apply (Incoherent.cpp:66-77): one draw per beamlet of nbins particles
  if (p.isr.ctr) {
    const float u = (float)isr_uniform(p.isr.seed, *p.isr.ctr, is, ip / p.isr.nbins);
    dg += -sc.isr_avg + sc.isr_sig * (2.f * u - 1.f);
  }
  // Collective::apply (Collective.cpp:119-128), before the second half step
  if (p.wake) dg += p.wake[is] * sc.delz;
  th = add_phase(th, dth);
  // TrackBeam::applyR56 (TrackBeam.cpp:260-277): gamma - gamma0 is the stored offset
  if (sc.chic) th = add_phase(th, sc.r56 * dg);
  transverse_f(sc, true, g0 + dg, x, y, px, py);
}

template <int NF>
__global__ void __launch_bounds__(512) k_push_f(StepConstF sc, PtrsF p, int ns, int np, int ng,
                                                int deposit) {
  int is = blockIdx.y;
  int ip = blockIdx.x * blockDim.x + threadIdx.x;
  // lanes past the slice's particles stay for the deposition's warp shuffles
  const bool valid = ip < slice_np_f(p, is, np);
  if (!valid && !deposit) return;
  size_t o = (size_t)is * np + (valid ? ip : 0);
  const float g0 = (float)sc.gammaref;
  float dg = p.dg[o], x = p.x[o], y = p.y[o], px = p.px[o], py = p.py[o];
  long long th = p.theta[o] + sc.autophase_q;
  size_t ncell = (size_t)ng * ng;

  if (p.mode != 2) transverse_f(sc, false, g0 + dg, x, y, px, py);
  if (p.mode == 1) {
    if (valid) {
      p.x[o] = x;
      p.y[o] = y;
      p.px[o] = px;
      p.py[o] = py;
    }
    return;
  }
  // BeamSolver.cpp:50, 61: ez = the particle's short-range field + the slice's loss
  const float ez = (p.ez ? p.ez[o] : 0.f) + (p.eloss ? (float)p.eloss[is] : 0.f);
  const float2 *fslice[NF];
#pragma unroll
  for (int k = 0; k < NF; k++) fslice[k] = k < sc.nfld ? p.field[k] + (size_t)ring_slot(is, sc.f[k].first, ns) * ncell
                                                       : nullptr;
  push_rest_f<NF>(sc, p, fslice, is, ip, ng, ez, dg, th, x, y, px, py);
  const float g = g0 + dg;

  if (valid) {
    p.dg[o] = dg;
    p.theta[o] = th;
    p.x[o] = x;
    p.y[o] = y;
    p.px[o] = px;
    p.py[o] = py;
  }
  if (deposit) deposit_f<NF>(sc, p, (size_t)is * ncell, ng, slice_cur_f(p, is, np), g, th, x, y, valid);
}

template <int NF>
__global__ void __launch_bounds__(256) k_deposit_f(StepConstF sc, PtrsF p, int ns, int np, int ng) {
  int is = blockIdx.y;
  int ip = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = ip < slice_np_f(p, is, np);
  size_t o = (size_t)is * np + (valid ? ip : 0);
  deposit_f<NF>(sc, p, (size_t)is * (size_t)ng * ng, ng, slice_cur_f(p, is, np),
                (float)sc.gammaref + p.dg[o], p.theta[o], p.x[o], p.y[o], valid);
}

struct CoefF {
  const float2 *c, *cbet, *cwet;
};
__device__ __forceinline__ float2 lapf(bool hp, bool hn, float2 pv, float2 u, float2 nx) {
  float2 r;
  if (!hp) {
    r.x = nx.x - 2.f * u.x;
    r.y = nx.y - 2.f * u.y;
  } else if (!hn) {
    r.x = pv.x - 2.f * u.x;
    r.y = pv.y - 2.f * u.y;
  } else {
    r.x = nx.x - 2.f * u.x + pv.x;
    r.y = nx.y - 2.f * u.y + pv.y;
  }
  return r;
}

// ADI implicit in x (FieldSolverADI.cpp:63-75, 94-104), FP32; thread per (slice, row)
__global__ void __launch_bounds__(128) k_adi_x_f(const float2 *__restrict__ field,
                                                 const float2 *__restrict__ src,
                                                 float2 *__restrict__ tmp, CoefF cf, float cstep,
                                                 int ns, int ng, int first) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ns * ng) return;
  int ii = (int)(t / ng), iy = (int)(t % ng);
  size_t ncell = (size_t)ng * ng;
  int i = (ii + first) % ns;
  const float2 *u = field + (size_t)i * ncell + (size_t)iy * ng;
  const float2 *s = src ? src + (size_t)ii * ncell + (size_t)iy * ng : nullptr;
  float2 *w = tmp + (size_t)i * ncell + (size_t)iy * ng;
  bool hp = iy > 0, hn = iy < ng - 1;
  float2 prev = make_float2(0.f, 0.f);
  for (int k = 0; k < ng; k++) {
    float2 uc = u[k];
    float2 un = hn ? u[k + ng] : make_float2(0.f, 0.f);
    float2 us = hp ? u[k - ng] : make_float2(0.f, 0.f);
    float2 l = lapf(hp, hn, us, uc, un);
    float2 sv = s ? s[k] : make_float2(0.f, 0.f);
    float2 r = make_float2(sv.x + uc.x - cstep * l.y, sv.y + uc.y + cstep * l.x);
    float2 v;
    if (k == 0) {
      v = cmulf(r, cf.cbet[0]);
    } else {
      v = cmulf(sub_imulf(r, cf.c[k].y, prev), cf.cbet[k]);
    }
    w[k] = v;
    prev = v;
  }
  float2 next = prev;
  for (int k = ng - 2; k >= 0; k--) {
    float2 v = sub_cmulf(w[k], cf.cwet[k + 1], next);
    w[k] = v;
    next = v;
  }
}

// ADI implicit in y (FieldSolverADI.cpp:77-89, 106-122), FP32; thread per (slice, column)
__global__ void __launch_bounds__(128) k_adi_y_f(float2 *__restrict__ field,
                                                 const float2 *__restrict__ src,
                                                 const float2 *__restrict__ tmp, CoefF cf,
                                                 float cstep, int ns, int ng, int first) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ns * ng) return;
  int ii = (int)(t / ng), ix = (int)(t % ng);
  size_t ncell = (size_t)ng * ng;
  int i = (ii + first) % ns;
  float2 *u = field + (size_t)i * ncell + ix;
  const float2 *s = src ? src + (size_t)ii * ncell + ix : nullptr;
  const float2 *w = tmp + (size_t)i * ncell + ix;
  bool hp = ix > 0, hn = ix < ng - 1;
  float2 prev = make_float2(0.f, 0.f);
  for (int k = 0; k < ng; k++) {
    size_t o = (size_t)k * ng;
    float2 wc = w[o];
    float2 wn = hn ? w[o + 1] : make_float2(0.f, 0.f);
    float2 wp = hp ? w[o - 1] : make_float2(0.f, 0.f);
    float2 l = lapf(hp, hn, wp, wc, wn);
    float2 sv = s ? s[o] : make_float2(0.f, 0.f);
    float2 r = make_float2(sv.x + wc.x - cstep * l.y, sv.y + wc.y + cstep * l.x);
    float2 v;
    if (k == 0) {
      v = cmulf(r, cf.cbet[0]);
    } else {
      v = cmulf(sub_imulf(r, cf.c[k].y, prev), cf.cbet[k]);
    }
    u[o] = v;
    prev = v;
  }
  float2 next = prev;
  for (int k = ng - 2; k >= 0; k--) {
    size_t o = (size_t)k * ng;
    float2 v = sub_cmulf(u[o], cf.cwet[k + 1], next);
    u[o] = v;
    next = v;
  }
}

// ---- fused field step: deposition + ADI of one slice in shared memory --------
//
// One CTA per (field, slice). The slice's FP32 field (ngrid^2 float2, 182 KB at
// ngrid 151) lives in shared memory for the whole solve, so the field is read and
// written once and the source never touches global memory:
//   S = u                                   bulk load
//   S = (I + c Dy) S = S1                    column pass (column segments)
//   S = S1 + src                             deposition
//   S = Thomas_x(S)                          row sweeps, two-ended  -> u'
//   S = 2 u' - S1                            = (I + c Dx) u' + src, because
//                                              (I - c Dx) u' = S1 + src; S1 recomputed
//                                              from u, still unmodified in global memory
//   S = Thomas_y(S)                          column sweeps          -> u''
//   u = S                                   bulk store
// This is the reference's ADI (FieldSolverADI.cpp:60-122) with its source
// (FieldSolverADI.cpp:19-51) added after, instead of before, the stencil term, and
// the second right-hand side formed from the first instead of from a second
// deposition.
constexpr int kFusedMaxThreads = 1024;


// c * (i * lap): cstep is purely imaginary
__device__ __forceinline__ float2 stencil(float cs, float2 u, float2 l) {
  return make_float2(u.x - cs * l.y, u.y + cs * l.x);
}

// Tridiagonal solve of one line of S (stride between elements) by two threads,
// eliminating from both ends at once ("burn at both ends"). The matrix
// (I - c D), D the Dirichlet second difference, is the one of tridagx / tridagy
// (FieldSolverADI.cpp:94-122, coefficients :125-182): symmetric Toeplitz, hence
// persymmetric, so the upward elimination uses the same cbet / cwet tables as the
// downward one, indexed from the far end. Thread `up` == 0 eliminates rows 0..m-1,
// thread 1 rows n-1..m+1; they exchange their last values (lanes 2l and 2l+1 of a
// warp), both solve row m, and back-substitute outward. Half the dependent chain of
// a one-thread sweep; the same solution up to FP32 rounding.
// a: off-diagonal, bm: diagonal, invden: 1 / (bm - a cwet_m - a cwet_{n-1-m}).
__device__ __forceinline__ void thomas2(float2 *S, int stride, int ng, int up, const float2 *CB,
                                        const float2 *CW, float2 a, float2 invden, unsigned mask) {
  const int m = ng / 2;
  // elimination: thread 0 over rows 0..m-1, thread 1 over rows n-1..m+1
  const int len = up ? ng - 1 - m : m;
  const int step = up ? -stride : stride;
  float2 *L = up ? S + (ng - 1) * stride : S;
  float2 d = make_float2(0.f, 0.f);
  float2 rn = L[0];
  for (int t = 0; t < len; t++) {
    float2 r = rn;
    if (t + 1 < len) rn = L[(t + 1) * step];
    d = cmulf(sub_imulf(r, a.y, d), CB[t]);
    L[t * step] = d;
  }
  // meet at row m
  float2 d_other;
  d_other.x = __shfl_xor_sync(mask, d.x, 1);
  d_other.y = __shfl_xor_sync(mask, d.y, 1);
  float2 dsum = make_float2(d.x + d_other.x, d.y + d_other.y);
  float2 rm = S[m * stride];
  float2 xm = cmulf(sub_imulf(rm, a.y, dsum), invden);
  // back substitution outward from m
  float2 x = xm;
  for (int t = len - 1; t >= 0; t--) {
    x = sub_cmulf(L[t * step], CW[t + 1], x);
    L[t * step] = x;
  }
  if (!up) S[m * stride] = xm;
}

// Tridiagonal solve (I - c D) x = r (FieldSolverADI.cpp:94-122: the Thomas recurrences
// with the cbet / cwet tables) of the ng lines of S, nseg threads per line: thread
// tid takes line tid % ng and the segment tid / ng of consecutive elements (element
// k of line l at S[l * lstride + k * estride]). The recurrences forget their start
// by a factor alpha per element (the host's segment_warmup), so each segment starts
// W elements before its first element from zero (forward) and W elements after its
// last one from d (backward): the carries then agree with the full sweep to within
// alpha^W <= 2^-32. Each warm-up runs on values its neighbour has not yet overwritten
// (a barrier separates it from the in-place pass). The first segment's forward pass
// and the last segment's backward pass are the exact sweeps. Every thread of the
// block must call it. With SUMS (a column solve: lstride 1, estride ng), the final pass
// also sums the record terms of k_diag_field_f over the thread's solved elements into
// fsum[kFieldSums] (power, its first and second moments in x and y, the field's sum):
// the slice's diagnostics without another pass over it.
template <bool SUMS = false>
__device__ __forceinline__ void thomas_seg(float2 *S, int lstride, int estride, int ng, int nseg, int W,
                                           const float2 *Cc, const float2 *CB, const float2 *CW,
                                           float *fsum = nullptr) {
  const int tid = threadIdx.x;
  const int line = tid % ng, seg = tid / ng;
  const int len = (ng + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, ng);
  const bool act = seg < nseg && b < e;
  float2 *L = S + (size_t)line * lstride;
  // forward: d_k = (r_k - c_k d_{k-1}) cbet_k
  float2 d = make_float2(0.f, 0.f);
  if (act)
    for (int k = max(0, b - W); k < b; k++) {
      float2 r = L[k * estride];
      d = cmulf(sub_imulf(r, Cc[k].y, d), CB[k]);
    }
  __syncthreads();
  if (act)
    for (int k = b; k < e; k++) {
      float2 r = L[k * estride];
      d = cmulf(sub_imulf(r, Cc[k].y, d), CB[k]);
      L[k * estride] = d;
    }
  __syncthreads();
  // backward: x_k = d_k - cwet_{k+1} x_{k+1}, x_{ng-1} = d_{ng-1}
  const int k1 = min(ng - 1, e - 1 + W);
  float2 x = make_float2(0.f, 0.f);
  if (act && k1 >= e) {
    x = L[k1 * estride];
    for (int k = k1 - 1; k >= e; k--) {
      x = sub_cmulf(L[k * estride], CW[k + 1], x);
    }
  }
  __syncthreads();
  const float shift = -0.5f * (float)(ng - 1);
  float sw = 0.f, swy = 0.f, swyy = 0.f, sre = 0.f, sim = 0.f;
  if (act)
    for (int k = e - 1; k >= b; k--) {
      float2 v = L[k * estride];
      if (k < ng - 1) {
        v = sub_cmulf(v, CW[k + 1], x);
      }
      x = v;
      L[k * estride] = x;
      if (SUMS) {
        const float dy = (float)k + shift, wei = x.x * x.x + x.y * x.y;
        sw += wei;
        swy += dy * wei;
        swyy += dy * dy * wei;
        sre += x.x;
        sim += x.y;
      }
    }
  if (SUMS) {
    const float dx = act ? (float)line + shift : 0.f;
    fsum[0] = sw;
    fsum[1] = dx * sw;
    fsum[2] = dx * dx * sw;
    fsum[3] = swy;
    fsum[4] = swyy;
    fsum[5] = sre;
    fsum[6] = sim;
  }
  __syncthreads();
}

// (I + c D) along a line of S with stride, in place, with a rolling register window
// and the next-but-one element fetched ahead
__device__ __forceinline__ void stencil_line(float2 *S, int stride, int ng, float cs) {
  float2 prev = make_float2(0.f, 0.f), cur = S[0], next = S[stride], nn = S[2 * stride];
  for (int k = 0; k < ng; k++) {
    float2 nx = (k + 1 < ng) ? next : make_float2(0.f, 0.f);
    float2 l = lapf(k > 0, k < ng - 1, prev, cur, nx);
    float2 out = stencil(cs, cur, l);
    prev = cur;
    cur = next;
    next = nn;
    if (k + 3 < ng) nn = S[(k + 3) * stride];
    S[k * stride] = out;
  }
}

// (I + c Dy) on every column of S in place, each column split into nseg segments of
// consecutive rows, one thread each (thread tid: column tid % ng, segment tid / ng),
// so that the column pass has nseg times the threads and 1/nseg the dependent chain
// of one thread per column. The rows just outside each segment are read before
// anything is written; every thread of the block must call it. The outputs are the
// same operations on the same operands as stencil_line's.
__device__ __forceinline__ void stencil_cols_seg(float2 *S, int ng, float cs, int nseg) {
  const int tid = threadIdx.x;
  const int col = tid % ng, seg = tid / ng;
  const int len = (ng + nseg - 1) / nseg;
  const int r0 = seg * len, r1 = min(r0 + len, ng);
  const bool act = seg < nseg && r0 < r1;
  float2 above = make_float2(0.f, 0.f), below = make_float2(0.f, 0.f);
  if (act) {
    if (r0 > 0) above = S[(r0 - 1) * ng + col];
    if (r1 < ng) below = S[r1 * ng + col];
  }
  __syncthreads();
  if (act) {
    float2 prev = above, cur = S[r0 * ng + col];
    float2 next = (r0 + 1 < r1) ? S[(r0 + 1) * ng + col] : below;
    for (int r = r0; r < r1; r++) {
      float2 nx = next;
      if (r + 2 < r1)
        next = S[(r + 2) * ng + col];
      else if (r + 2 == r1)
        next = below;
      float2 l = lapf(r > 0, r < ng - 1, prev, cur, nx);
      float2 out = stencil(cs, cur, l);
      prev = cur;
      cur = nx;
      S[r * ng + col] = out;
    }
  }
}

// The second right-hand side, S = 2 u' - S1 with S1 = (I + c Dy) u recomputed from
// the slice still unmodified in global memory (read through L2, where the slice
// load left it) instead of stored: the same column segments and the same operations
// as stencil_cols_seg, so S1 is bitwise the value the first half step used.
__device__ __forceinline__ void r2_cols_seg(float2 *S, const float2 *__restrict__ u, int ng, float cs,
                                            int nseg) {
  const int tid = threadIdx.x;
  const int col = tid % ng, seg = tid / ng;
  const int len = (ng + nseg - 1) / nseg;
  const int r0 = seg * len, r1 = min(r0 + len, ng);
  if (seg >= nseg || r0 >= r1) return;
  float2 prev = r0 > 0 ? u[(r0 - 1) * ng + col] : make_float2(0.f, 0.f);
  float2 cur = u[r0 * ng + col];
  float2 next = r0 + 1 < ng ? u[(r0 + 1) * ng + col] : make_float2(0.f, 0.f);
  for (int r = r0; r < r1; r++) {
    float2 nx = next;
    if (r + 2 < ng) next = u[(r + 2) * ng + col];
    float2 l = lapf(r > 0, r < ng - 1, prev, cur, nx);
    float2 s1 = stencil(cs, cur, l);
    prev = cur;
    cur = nx;
    float2 v = S[r * ng + col];
    S[r * ng + col] = make_float2(2.f * v.x - s1.x, 2.f * v.y - s1.y);
  }
}

// Adds the source contribution of the 32 particles held by the lanes of a warp (one
// each; lanes past the end carry x = 1e30, off the grid) to S with shared-memory
// atomics. Lanes whose particles share the lower-left cell (quiet loading stores
// the nbins mirrored beamlet members, which share x and y, in adjacent lanes) first
// sum their four weighted contributions with a segmented shuffle reduction over
// runs of equal cells; only the first lane of each run issues the atomics. This cuts
// the atomics (and their same-address conflicts) by the run length and keeps the
// result exact up to FP32 summation order. Every lane of the warp must call it.
__device__ __forceinline__ void deposit_lanes(const StepConstF &sc, const FieldStepF &fs, float scl, float2 *S,
                                              int ng, float x, float y, long long th, float dgam) {
  const unsigned lane = threadIdx.x & 31u;
  CellF c;
  bool on = ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x, y, c);
  float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (on) {
    float g = (float)sc.gammaref + dgam;
    float dx = x - sc.ax, dy = y - sc.ay;
    float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
    float part = sqrtf(faw2) * scl / g;
    float sn, co;
    __sincosf(phase_of(th, (unsigned)fs.harm), &sn, &co);
    float cpx = sn * part, cpy = co * part;
    float w00 = c.wx * c.wy, w10 = (1.f - c.wx) * c.wy, w01 = c.wx * (1.f - c.wy),
          w11 = (1.f - c.wx) * (1.f - c.wy);
    v[0] = w00 * cpx; v[1] = w00 * cpy; v[2] = w10 * cpx; v[3] = w10 * cpy;
    v[4] = w01 * cpx; v[5] = w01 * cpy; v[6] = w11 * cpx; v[7] = w11 * cpy;
  }
  // runs of equal lower-left cells among adjacent lanes (off-grid lanes carry
  // zeros and key -1; they issue no atomics)
  int key = on ? c.i00 : -1;
  bool run_head;
  // both shuffles run on every lane (a short-circuit && would leave some lanes out
  // of a full-mask shuffle)
  const int key1 = __shfl_xor_sync(0xffffffffu, key, 1);
  const int key2 = __shfl_xor_sync(0xffffffffu, key, 2);
  bool quads = __all_sync(0xffffffffu, (key == key1) & (key == key2));
  if (quads) {
    // every aligned group of four lanes shares one cell (quiet loading with nbins = 4)
#pragma unroll
    for (int q = 0; q < 8; q++) {
      v[q] += __shfl_xor_sync(0xffffffffu, v[q], 1);
      v[q] += __shfl_xor_sync(0xffffffffu, v[q], 2);
    }
    run_head = (lane & 3u) == 0u;
  } else {
    int knext = __shfl_down_sync(0xffffffffu, key, 1);
    int kprev = __shfl_up_sync(0xffffffffu, key, 1);
    bool run_end = (lane == 31u) || (knext != key);
    run_head = (lane == 0u) || (kprev != key);
    unsigned ends = __ballot_sync(0xffffffffu, run_end);
    int seg_end = __ffs(ends & (0xffffffffu << lane)) - 1;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float o = __shfl_down_sync(0xffffffffu, v[q], off);
        if ((int)lane + off <= seg_end) v[q] += o;
      }
    }
  }
  if (on && run_head) {
    atomicAdd(&S[c.i00].x, v[0]);
    atomicAdd(&S[c.i00].y, v[1]);
    atomicAdd(&S[c.i10].x, v[2]);
    atomicAdd(&S[c.i10].y, v[3]);
    atomicAdd(&S[c.i01].x, v[4]);
    atomicAdd(&S[c.i01].y, v[5]);
    atomicAdd(&S[c.i11].x, v[6]);
    atomicAdd(&S[c.i11].y, v[7]);
  }
}

// Adds the deposited source of beam slice `is` to S, the particles read from global
// memory (used when no staging buffer fits beside the slice).
__device__ __forceinline__ void deposit_smem(const StepConstF &sc, const FieldStepF &fs,
                                             const PtrsF &p, float2 *S, int is, int np, int ng) {
  const float scl = fs.dep_scl * slice_cur_f(p, is, np);
  const size_t base = (size_t)is * np;
  const int n = slice_np_f(p, is, np);
  const unsigned lane = threadIdx.x & 31u;
  const int warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  constexpr int U = 4;  // particles per lane per round: their loads are issued together
  for (int w0 = warp * 32 * U; w0 < n; w0 += nwarp * 32 * U) {
    float xs[U], ys[U], gs[U];
    long long ths[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      int ip = w0 + u * 32 + (int)lane;
      bool in = ip < n;
      xs[u] = in ? p.x[base + ip] : 1e30f;
      ys[u] = in ? p.y[base + ip] : 1e30f;
      ths[u] = in ? p.theta[base + ip] : 0;
      gs[u] = in ? p.dg[base + ip] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < U; u++) deposit_lanes(sc, fs, scl, S, ng, xs[u], ys[u], ths[u], gs[u]);
  }
}

// The contribution of one particle to the four cells around it (no aggregation).
__device__ __forceinline__ void deposit_one(const StepConstF &sc, const FieldStepF &fs, float scl, float2 *S,
                                            int ng, float x, float y, long long th, float dgam) {
  CellF c;
  if (!ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x, y, c)) return;
  float dx = x - sc.ax, dy = y - sc.ay;
  float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
  float part = sqrtf(faw2) * scl / ((float)sc.gammaref + dgam);
  float sn, co;
  __sincosf(phase_of(th, (unsigned)fs.harm), &sn, &co);
  float cpx = sn * part, cpy = co * part;
  float w00 = c.wx * c.wy, w10 = (1.f - c.wx) * c.wy, w01 = c.wx * (1.f - c.wy), w11 = (1.f - c.wx) * (1.f - c.wy);
  atomicAdd(&S[c.i00].x, w00 * cpx);
  atomicAdd(&S[c.i00].y, w00 * cpy);
  atomicAdd(&S[c.i10].x, w10 * cpx);
  atomicAdd(&S[c.i10].y, w10 * cpy);
  atomicAdd(&S[c.i01].x, w01 * cpx);
  atomicAdd(&S[c.i01].y, w01 * cpy);
  atomicAdd(&S[c.i11].x, w11 * cpx);
  atomicAdd(&S[c.i11].y, w11 * cpy);
}

// The summed contribution of n particles that share x and y (one cell, one set of
// weights, one undulator factor), n = 2 or 4.
template <int N>
__device__ __forceinline__ void deposit_group(const StepConstF &sc, const FieldStepF &fs, float scl, float2 *S,
                                              int ng, float x, float y, const long long *th, const float *dgam) {
  CellF c;
  if (!ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x, y, c)) return;
  float dx = x - sc.ax, dy = y - sc.ay;
  float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
  float a = sqrtf(faw2) * scl;
  float cpx = 0.f, cpy = 0.f;
#pragma unroll
  for (int m = 0; m < N; m++) {
    float part = a / ((float)sc.gammaref + dgam[m]);
    float sn, co;
    __sincosf(phase_of(th[m], (unsigned)fs.harm), &sn, &co);
    cpx += sn * part;
    cpy += co * part;
  }
  float w00 = c.wx * c.wy, w10 = (1.f - c.wx) * c.wy, w01 = c.wx * (1.f - c.wy), w11 = (1.f - c.wx) * (1.f - c.wy);
  atomicAdd(&S[c.i00].x, w00 * cpx);
  atomicAdd(&S[c.i00].y, w00 * cpy);
  atomicAdd(&S[c.i10].x, w10 * cpx);
  atomicAdd(&S[c.i10].y, w10 * cpy);
  atomicAdd(&S[c.i01].x, w01 * cpx);
  atomicAdd(&S[c.i01].y, w01 * cpy);
  atomicAdd(&S[c.i11].x, w11 * cpx);
  atomicAdd(&S[c.i11].y, w11 * cpy);
}

// Four particles that lie in one cell without sharing x and y exactly: a beamlet's
// mirrored members once their energies, and with them their transverse steps, differ in
// the last bits. Each particle's own weights and phasor are summed in registers, then
// one set of eight atomics (exact up to FP32 summation order). Returns false, having
// deposited nothing, unless all four lie inside the grid in the same cell.
__device__ __forceinline__ bool deposit_cell4(const StepConstF &sc, const FieldStepF &fs, float scl, float2 *S,
                                              int ng, const float *x, const float *y, const long long *th,
                                              const float *dgam) {
  CellF c;
  if (!ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x[0], y[0], c)) return false;
#pragma unroll
  for (int m = 1; m < 4; m++) {
    CellF cm;
    if (!ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x[m], y[m], cm) || cm.i00 != c.i00) return false;
  }
  float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int m = 0; m < 4; m++) {
    CellF cm;
    ll_gridpoint_f(fs.gridmax, fs.dgrid, ng, x[m], y[m], cm);
    const float dx = x[m] - sc.ax, dy = y[m] - sc.ay;
    const float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
    const float part = sqrtf(faw2) * scl / ((float)sc.gammaref + dgam[m]);
    float sn, co;
    __sincosf(phase_of(th[m], (unsigned)fs.harm), &sn, &co);
    const float cpx = sn * part, cpy = co * part;
    const float w00 = cm.wx * cm.wy, w10 = (1.f - cm.wx) * cm.wy, w01 = cm.wx * (1.f - cm.wy),
                w11 = (1.f - cm.wx) * (1.f - cm.wy);
    v[0] += w00 * cpx; v[1] += w00 * cpy; v[2] += w10 * cpx; v[3] += w10 * cpy;
    v[4] += w01 * cpx; v[5] += w01 * cpy; v[6] += w11 * cpx; v[7] += w11 * cpy;
  }
  atomicAdd(&S[c.i00].x, v[0]);
  atomicAdd(&S[c.i00].y, v[1]);
  atomicAdd(&S[c.i10].x, v[2]);
  atomicAdd(&S[c.i10].y, v[3]);
  atomicAdd(&S[c.i01].x, v[4]);
  atomicAdd(&S[c.i01].y, v[5]);
  atomicAdd(&S[c.i11].x, v[6]);
  atomicAdd(&S[c.i11].y, v[7]);
  return true;
}

// Adds the deposited source of beam slice `is` to S with one thread per four
// consecutive particles. Quiet loading stores the nbins mirrored members of a
// beamlet consecutively (nbins a multiple of 4 gives aligned groups of four sharing
// x and y; nbins = 2, pairs): a group that shares x and y is deposited once with the
// sum of its members' phasors, a group in one cell with the sum of its members' weighted
// phasors, pairs that share x and y like the first, anything else particle by particle.
// No warp-level exchange is needed, and the loads are 16-byte vectors. Needs
// npart % 4 == 0.
__device__ __forceinline__ void deposit_quads(const StepConstF &sc, const FieldStepF &fs, const PtrsF &p,
                                              float2 *S, int is, int np, int ng) {
  const float scl = fs.dep_scl * (float)p.current[is];
  const size_t base = (size_t)is * np;
  const float4 *X = reinterpret_cast<const float4 *>(p.x + base);
  const float4 *Y = reinterpret_cast<const float4 *>(p.y + base);
  const float4 *G = reinterpret_cast<const float4 *>(p.dg + base);
  const longlong2 *T = reinterpret_cast<const longlong2 *>(p.theta + base);
  for (int q = threadIdx.x; q < (np >> 2); q += blockDim.x) {
    const float4 x = X[q], y = Y[q], g = G[q];
    const longlong2 t01 = T[2 * q], t23 = T[2 * q + 1];
    const long long th[4] = {t01.x, t01.y, t23.x, t23.y};
    const float dg[4] = {g.x, g.y, g.z, g.w};
    const bool p01 = x.x == x.y && y.x == y.y, p23 = x.z == x.w && y.z == y.w;
    const float xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
    if (p01 && p23 && x.x == x.z && y.x == y.z) {
      deposit_group<4>(sc, fs, scl, S, ng, x.x, y.x, th, dg);
    } else if (!deposit_cell4(sc, fs, scl, S, ng, xs, ys, th, dg)) {
      if (p01) {
        deposit_group<2>(sc, fs, scl, S, ng, x.x, y.x, th, dg);
      } else {
        deposit_one(sc, fs, scl, S, ng, x.x, y.x, th[0], dg[0]);
        deposit_one(sc, fs, scl, S, ng, x.y, y.y, th[1], dg[1]);
      }
      if (p23) {
        deposit_group<2>(sc, fs, scl, S, ng, x.z, y.z, th + 2, dg + 2);
      } else {
        deposit_one(sc, fs, scl, S, ng, x.z, y.z, th[2], dg[2]);
        deposit_one(sc, fs, scl, S, ng, x.w, y.w, th[3], dg[3]);
      }
    }
  }
}


// One source sub-step of a coarse step (g4gpu_set_field_substeps): the deposition of
// beam slice `is` (FieldSolverADI.cpp:19-51) added to its field storage slot
// (is + first) % ns as the Crank-Nicolson step adds a source without diffraction, u +=
// 2 src, with float atomics in global memory. Every particle's phase, x and y are
// interpolated at `frac` of the coarse push, between the start (tp, xp, yp: copies
// taken before the push) and the end (the beam's arrays): exact for the free drift
// of the phase and the straight transverse path over a few periods. `scale` is 2 / c
// for a coarse step of c periods (the step constants hold the whole step's dz). One
// thread per four consecutive particles, grouped as deposit_quads groups them; needs
// npart % 4 == 0 and full slices.
__global__ void __launch_bounds__(128) k_source_f(StepConstF sc, PtrsF p, const long long *__restrict__ tp,
                                                  const float *__restrict__ xp, const float *__restrict__ yp,
                                                  float frac, float scale, float2 *field, int ns, int np,
                                                  int ng) {
  const int is = blockIdx.y;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (np >> 2)) return;
  const FieldStepF &fs = sc.f[0];
  const float scl = scale * fs.dep_scl * (float)p.current[is];
  float2 *S = field + (size_t)ring_slot(is, fs.first, ns) * ng * ng;
  const size_t base = (size_t)is * np;
  const float4 x1 = reinterpret_cast<const float4 *>(p.x + base)[q];
  const float4 y1 = reinterpret_cast<const float4 *>(p.y + base)[q];
  const float4 x0 = reinterpret_cast<const float4 *>(xp + base)[q];
  const float4 y0 = reinterpret_cast<const float4 *>(yp + base)[q];
  const float4 g = reinterpret_cast<const float4 *>(p.dg + base)[q];
  const longlong2 *T1 = reinterpret_cast<const longlong2 *>(p.theta + base);
  const longlong2 *T0 = reinterpret_cast<const longlong2 *>(tp + base);
  const longlong2 a01 = T1[2 * q], a23 = T1[2 * q + 1], b01 = T0[2 * q], b23 = T0[2 * q + 1];
  // the phase advance over the coarse push is a few turns: (float)(t1 - t0) keeps it to
  // ~1e-7 of itself, ~1e-6 rad
  const long long t1[4] = {a01.x, a01.y, a23.x, a23.y}, t0[4] = {b01.x, b01.y, b23.x, b23.y};
  long long th[4];
#pragma unroll
  for (int m = 0; m < 4; m++) th[m] = t0[m] + (long long)llrintf((float)(t1[m] - t0[m]) * frac);
  const float x[4] = {fmaf(frac, x1.x - x0.x, x0.x), fmaf(frac, x1.y - x0.y, x0.y), fmaf(frac, x1.z - x0.z, x0.z),
                      fmaf(frac, x1.w - x0.w, x0.w)};
  const float y[4] = {fmaf(frac, y1.x - y0.x, y0.x), fmaf(frac, y1.y - y0.y, y0.y), fmaf(frac, y1.z - y0.z, y0.z),
                      fmaf(frac, y1.w - y0.w, y0.w)};
  const float dg[4] = {g.x, g.y, g.z, g.w};
  const bool p01 = x[0] == x[1] && y[0] == y[1], p23 = x[2] == x[3] && y[2] == y[3];
  if (p01 && p23 && x[0] == x[2] && y[0] == y[2]) {
    deposit_group<4>(sc, fs, scl, S, ng, x[0], y[0], th, dg);
    return;
  }
  if (deposit_cell4(sc, fs, scl, S, ng, x, y, th, dg)) return;
  if (p01) {
    deposit_group<2>(sc, fs, scl, S, ng, x[0], y[0], th, dg);
  } else {
    deposit_one(sc, fs, scl, S, ng, x[0], y[0], th[0], dg[0]);
    deposit_one(sc, fs, scl, S, ng, x[1], y[1], th[1], dg[1]);
  }
  if (p23) {
    deposit_group<2>(sc, fs, scl, S, ng, x[2], y[2], th + 2, dg + 2);
  } else {
    deposit_one(sc, fs, scl, S, ng, x[2], y[2], th[2], dg[2]);
    deposit_one(sc, fs, scl, S, ng, x[3], y[3], th[3], dg[3]);
  }
}

// Bounded wait on an mbarrier phase; returns false (and raises the device error
// flag) if the phase does not complete within the iteration limit.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int *err) {
  for (long long it = 0; it < (1LL << 22); it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  if (err) atomicExch(err, 2);
  return false;
}

// Copies `count` float2 from global g to shared s with one TMA bulk copy for the
// 16-byte aligned middle and plain loads for an 8-byte head / tail. The shared
// copy is laid out so that s and g agree modulo 16 bytes (see the caller).
__device__ __forceinline__ void bulk_load_issue(float2 *s, const float2 *g, int count, uint32_t bar) {
  uintptr_t ga = reinterpret_cast<uintptr_t>(g);
  int head = (ga & 15) ? 1 : 0;
  int body = (count - head) & ~1;
  int tail = count - head - body;
  if (threadIdx.x == 0) {
    uint32_t bytes = (uint32_t)body * 8u;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    if (bytes) {
      uint32_t dst = (uint32_t)__cvta_generic_to_shared(s + head);
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(dst), "l"(g + head), "r"(bytes), "r"(bar)
          : "memory");
    }
  }
  if (head && threadIdx.x == 32) s[0] = g[0];
  if (tail && threadIdx.x == 64) s[count - 1] = g[count - 1];
}
// The CTA's verdict on a bounded wait for a bulk copy: false for every thread if the
// phase timed out for any of them (so that all threads leave together and none is
// left at a later barrier). A copy that timed out gets one more bounded wait before
// the CTA leaves, so that it is not still writing shared memory that the SM hands to
// another CTA.
__device__ __forceinline__ bool bulk_wait_uniform(uint32_t bar, uint32_t parity, int *err) {
  const bool ok = __syncthreads_and(mbar_wait(bar, parity, err)) != 0;
  if (!ok) {
    mbar_wait(bar, parity, nullptr);
    __syncthreads();
  }
  return ok;
}
// Waits for bulk_load_issue's copy (bounded) and makes it visible to the CTA.
__device__ __forceinline__ bool bulk_load_wait(uint32_t bar, int *err) { return bulk_wait_uniform(bar, 0, err); }
__device__ __forceinline__ bool bulk_load(float2 *s, const float2 *g, int count, uint32_t bar, int *err) {
  bulk_load_issue(s, g, count, bar);
  return bulk_load_wait(bar, err);
}

__device__ __forceinline__ void bulk_store(float2 *g, const float2 *s, int count) {
  uintptr_t ga = reinterpret_cast<uintptr_t>(g);
  int head = (ga & 15) ? 1 : 0;
  int body = (count - head) & ~1;
  int tail = count - head - body;
  // make the generic-proxy writes to s visible to the bulk copy engine
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0 && body) {
    uint32_t src = (uint32_t)__cvta_generic_to_shared(s + head);
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(g + head), "r"(src),
                 "r"((uint32_t)body * 8u)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  }
  if (head && threadIdx.x == 32) g[0] = s[0];
  if (tail && threadIdx.x == 64) g[count - 1] = s[count - 1];
}

// ---- diagnostics of a step recorded by the fused field kernel -----------------
//
// With the slice and its particles on chip, the fused kernel forms the per-slice sums
// of k_diag_beam_f (first field only) and k_diag_field_f into the run's diagnostic
// record, in the layouts of those kernels. A thread takes np / blockDim particles
// (or ngrid^2 / blockDim cells), few enough for FP32 partial sums; the CTA folds the
// partials in FP64.
constexpr int kFusedDiagHarm = 2;  // bunching harmonics the fused kernel records
constexpr int kFusedDiagValues = kBeamSums + 2 * kFusedDiagHarm + 10;

// The NS sums and NX min/max pairs of the CTA: within a warp in FP32 (the lanes'
// partials are FP32; FP64 adds run at 1/64 of the FP32 rate here and would dominate
// the kernel), then folded over the warps in FP64 through `sh` (warps x (NS + 2 NX)
// doubles); thread k < NS + 2 NX gets value k in *out.
template <int NS, int NX>
__device__ __forceinline__ void cta_reduce(const float *s, const float *mn, const float *mx, double *sh,
                                           double *out) {
  constexpr int NV = NS + 2 * NX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NS; k++) {
    float v = s[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp * NV + k] = v;
  }
#pragma unroll
  for (int k = 0; k < NX; k++) {
    float a = mn[k], b = mx[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = fminf(a, __shfl_down_sync(0xffffffffu, a, o));
      b = fmaxf(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    if (lane == 0) {
      sh[warp * NV + NS + 2 * k] = a;
      sh[warp * NV + NS + 2 * k + 1] = b;
    }
  }
  __syncthreads();
  const int k = threadIdx.x;
  if (k < NV) {
    double r = sh[k];
    for (int w = 1; w < nw; w++) {
      const double v = sh[w * NV + k];
      if (k < NS)
        r += v;
      else
        r = ((k - NS) & 1) ? fmax(r, v) : fmin(r, v);
    }
    out[k] = r;
  }
  __syncthreads();
}

// Beam sums of slice `is` into o[beam_diag_width(nharm)] (k_diag_beam_f's record).
__device__ __forceinline__ void slice_beam_sums(const PtrsF &p, double gref, int is, int np, int nharm,
                                                double *sh, double *res, double *o) {
  constexpr int NSUM = kBeamSums + 2 * kFusedDiagHarm;
  const size_t base = (size_t)is * np;
  const int cnt = slice_np_f(p, is, np);
  float c[NSUM];
#pragma unroll
  for (int k = 0; k < NSUM; k++) c[k] = 0.f;
  float mn[5], mx[5];  // x, px, y, py, dg
#pragma unroll
  for (int k = 0; k < 5; k++) {
    mn[k] = INFINITY;
    mx[k] = -INFINITY;
  }
  // unrolled so that the loads of several particles are in flight together
#pragma unroll 8
  for (int ip = threadIdx.x; ip < cnt; ip += blockDim.x) {
    const float x = p.x[base + ip], y = p.y[base + ip], dg = p.dg[base + ip];
    const float px = p.px[base + ip], py = p.py[base + ip];
    const long long th = p.theta[base + ip];
    c[0] += dg; c[1] += dg * dg; c[2] += x; c[3] += x * x; c[4] += y; c[5] += y * y;
    c[6] += px; c[7] += px * px; c[8] += py; c[9] += py * py; c[10] += x * px; c[11] += y * py;
    mn[0] = fminf(mn[0], x); mx[0] = fmaxf(mx[0], x);
    mn[1] = fminf(mn[1], px); mx[1] = fmaxf(mx[1], px);
    mn[2] = fminf(mn[2], y); mx[2] = fmaxf(mx[2], y);
    mn[3] = fminf(mn[3], py); mx[3] = fmaxf(mx[3], py);
    mn[4] = fminf(mn[4], dg); mx[4] = fmaxf(mx[4], dg);
#pragma unroll
    for (int h = 0; h < kFusedDiagHarm; h++) {
      if (h < nharm) {
        float sn, cs;
        sincosf(phase_of(th, (unsigned)(h + 1)), &sn, &cs);
        c[kBeamSums + 2 * h] += cs;
        c[kBeamSums + 2 * h + 1] += sn;
      }
    }
  }
  cta_reduce<NSUM, 5>(c, mn, mx, sh, res);
  const int k = threadIdx.x;
  const double n = (double)cnt;
  if (k == 0) o[0] = n * gref + res[0];
  if (k == 1) o[1] = n * gref * gref + 2.0 * gref * res[0] + res[1];
  if (k >= 2 && k < kBeamSums) o[k] = res[k];
  if (k >= kBeamSums && k < kBeamSums + 2 * nharm) o[kBeamMinMax + k] = res[k];
  if (k < 10) o[kBeamSums + k] = (k >= 8 ? gref : 0.0) + res[NSUM + k];
}

// The field record o[kFieldSums + 2] of the slice S from every thread's partial sums c
// (slice_field_sums, or the column sweep of thomas_seg<true>) and the on-axis value.
__device__ __forceinline__ void finish_field_sums(const float2 *S, int ng, const float *c, double *sh, double *res,
                                                  double *o) {
  cta_reduce<kFieldSums, 0>(c, nullptr, nullptr, sh, res);
  if (threadIdx.x < kFieldSums) o[threadIdx.x] = res[threadIdx.x];
  if (threadIdx.x == 0) {
    const float2 v = S[(ng / 2) * ng + ng / 2];
    o[7] = v.x;
    o[8] = v.y;
  }
}

// Field sums of the slice S (ng x ng, in shared memory) into o[kFieldSums + 2]
// (k_diag_field_f's record).
__device__ __forceinline__ void slice_field_sums(const float2 *S, int ng, double *sh, double *res, double *o) {
  const int ncell = ng * ng;
  const float shift = -0.5f * (float)(ng - 1);
  float c[kFieldSums];
#pragma unroll
  for (int k = 0; k < kFieldSums; k++) c[k] = 0.f;
  int row = threadIdx.x / ng, col = threadIdx.x - row * ng;
  const int drow = blockDim.x / ng, dcol = blockDim.x - drow * ng;
  for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
    const float dx = (float)col + shift, dy = (float)row + shift;
    const float2 v = S[i];
    const float wei = v.x * v.x + v.y * v.y;
    c[0] += wei; c[1] += dx * wei; c[2] += dx * dx * wei; c[3] += dy * wei; c[4] += dy * dy * wei;
    c[5] += v.x; c[6] += v.y;
    row += drow;
    col += dcol;
    if (col >= ng) {
      col -= ng;
      row++;
    }
  }
  finish_field_sums(S, ng, c, sh, res, o);
}

__global__ void __launch_bounds__(kFusedMaxThreads, 1)
    k_field_fused_f(StepConstF sc, int k, PtrsF p, float2 *__restrict__ field,
                    const float2 *__restrict__ coef, int ns, int np, int ng, int deposit, int *err,
                    double *dbeam, double *dfield, int nharm, double gref) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ncell = ng * ng;
  const FieldStepF &fs = sc.f[k];
  int is = blockIdx.x;
  int i = (is + fs.first) % ns;
  float2 *u = field + (size_t)i * ncell;
  // layout: [mbarrier 16 B][solve constants 16 B][coefficients 3 ng][pad][S: ncell],
  // S congruent to u mod 16 (the bulk copies need equal alignment on both sides)
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
  float2 *K = reinterpret_cast<float2 *>(smem_raw + 8);  // K[0] = 1 / den of the meeting row
  float2 *C = reinterpret_cast<float2 *>(smem_raw + 16);
  float2 *CB = C + ng, *CW = CB + ng;
  size_t soff = (16 + 3 * (size_t)ng * 8 + 15) & ~(size_t)15;
  soff += reinterpret_cast<uintptr_t>(u) & 15;
  float2 *S = reinterpret_cast<float2 *>(smem_raw + soff);
  uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int t = threadIdx.x; t < 3 * ng; t += blockDim.x) C[t] = coef[t];
  __syncthreads();
  // constants of the two-ended solve: a (off-diagonal) = c[1], diagonal = 1 / cbet[0]
  const float2 a = C[1];
  if (threadIdx.x == 0) {
    int m = ng / 2;
    float2 bm = make_float2(CB[0].x, -CB[0].y);
    float n0 = CB[0].x * CB[0].x + CB[0].y * CB[0].y;
    bm.x /= n0;
    bm.y /= n0;
    float2 t1 = cmulf(a, CW[m]), t2 = cmulf(a, CW[ng - 1 - m]);
    float2 den = make_float2(bm.x - t1.x - t2.x, bm.y - t1.y - t2.y);
    float nd = den.x * den.x + den.y * den.y;
    K[0] = make_float2(den.x / nd, -den.y / nd);
  }
  // diagnostic scratch after the slice: warps x kFusedDiagValues doubles, then the
  // folded values
  double *dsh = reinterpret_cast<double *>(smem_raw + ((soff + (size_t)ncell * 8 + 15) & ~(size_t)15));
  double *dres = dsh + (blockDim.x >> 5) * kFusedDiagValues;
  bulk_load_issue(S, u, ncell, bar_s);
  // the beam record of this slice while the field is in flight
  if (dbeam) slice_beam_sums(p, gref, is, np, nharm, dsh, dres, dbeam + (size_t)is * beam_diag_width(nharm));
  if (!bulk_load_wait(bar_s, err)) return;
  const float cs = fs.cstep;
  const int tid = threadIdx.x;
  const int nseg = max(1, min((int)blockDim.x / ng, 8));
  stencil_cols_seg(S, ng, cs, nseg);  // S1 = (I + c Dy) u
  __syncthreads();
  if (deposit) {  // S = S1 + src
    // full slices of a multiple of 4 particles take the 16-byte vector loads
    if ((np & 3) == 0 && !p.count)
      deposit_quads(sc, fs, p, S, is, np, ng);
    else
      deposit_smem(sc, fs, p, S, is, np, ng);
    __syncthreads();
  }
  const float2 invden = K[0];
  const int line = tid >> 1, up = tid & 1;
  // segmented solves when the recurrences forget fast enough (tw > 0) and a line gets
  // at least two threads; else the two-ended solve: lanes 2l and 2l+1 on line l, the
  // mask covering the lanes of the warp with a line
  const bool segmented = fs.tw > 0 && nseg >= 2;
  const unsigned mask = __ballot_sync(0xffffffffu, line < ng);
  if (segmented)
    thomas_seg(S, ng, 1, ng, nseg, fs.tw, C, CB, CW);  // rows: u'
  else if (line < ng)
    thomas2(S + line * ng, 1, ng, up, CB, CW, a, invden, mask);
  __syncthreads();
  // (I + c Dx) u' + src = 2 u' - S1, because (I - c Dx) u' = S1 + src: the second
  // right-hand side needs neither a second deposition nor a stored S1
  r2_cols_seg(S, u, ng, cs, nseg);
  __syncthreads();
  // the field record's sums are formed by the segmented column sweep itself
  float fsum[kFieldSums];
  if (segmented && dfield)
    thomas_seg<true>(S, 1, ng, ng, nseg, fs.tw, C, CB, CW, fsum);  // columns
  else if (segmented)
    thomas_seg(S, 1, ng, ng, nseg, fs.tw, C, CB, CW);  // columns
  else if (line < ng)
    thomas2(S + line, ng, ng, up, CB, CW, a, invden, mask);
  __syncthreads();
  bulk_store(u, S, ncell);
  // the field record of storage slice i (from S alongside the store where the sweep
  // did not form its sums)
  if (dfield) {
    if (segmented)
      finish_field_sums(S, ng, fsum, dsh, dres, dfield + (size_t)i * (kFieldSums + 2));
    else
      slice_field_sums(S, ng, dsh, dres, dfield + (size_t)i * (kFieldSums + 2));
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// ---- the whole step of one slice in one CTA: push, deposition and ADI -----------
//
// One CTA per slice of a one-field window (mixed form, slice in shared memory, no
// space charge). Beam slice `is` sees only field storage slot (is + first) % ns in its
// push, and that slot's solve uses only beam slice `is` (BeamSolver.cpp:66,
// FieldSolverADI.cpp:11-55), so the slice's whole step runs on chip:
//   S = u                                   bulk load of the field slice
//   S = (I + c Dy) S = S1                    column pass
//   push every particle of the slice        gathering from u, still unmodified in
//                                           global memory (and in L2 from the load),
//                                           storing it and depositing it at once:
//                                           S = S1 + src
//   row sweeps, 2 u' - S1, column sweeps, bulk store, as k_field_fused_f.
// Against the push kernel followed by k_field_fused_f, the particles are read and
// written once and never read again for the deposition, the push's field gather
// and the second right-hand side hit L2, and one launch replaces two. Each lane
// takes U particles per round (their loads issued together); the 32 lanes of a warp
// hold consecutive particles, so deposit_lanes sums the beamlets that share a cell.
template <int U, int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
    k_step_fused_f(StepConstF sc, PtrsF p, float2 *__restrict__ field, const float2 *__restrict__ coef,
                   int ns, int np, int ng, int deposit, int *err, double *dbeam, double *dfield, int nharm,
                   double gref) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ncell = ng * ng;
  const FieldStepF &fs = sc.f[0];
  const int is = blockIdx.x;
  const int i = (is + fs.first) % ns;
  float2 *u = field + (size_t)i * ncell;
  // shared layout as k_field_fused_f's
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
  float2 *K = reinterpret_cast<float2 *>(smem_raw + 8);
  float2 *C = reinterpret_cast<float2 *>(smem_raw + 16);
  float2 *CB = C + ng, *CW = CB + ng;
  size_t soff = (16 + 3 * (size_t)ng * 8 + 15) & ~(size_t)15;
  soff += reinterpret_cast<uintptr_t>(u) & 15;
  float2 *S = reinterpret_cast<float2 *>(smem_raw + soff);
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int t = threadIdx.x; t < 3 * ng; t += blockDim.x) C[t] = coef[t];
  __syncthreads();
  const float2 a = C[1];
  if (threadIdx.x == 0) {
    const int m = ng / 2;
    float2 bm = make_float2(CB[0].x, -CB[0].y);
    const float n0 = CB[0].x * CB[0].x + CB[0].y * CB[0].y;
    bm.x /= n0;
    bm.y /= n0;
    const float2 t1 = cmulf(a, CW[m]), t2 = cmulf(a, CW[ng - 1 - m]);
    const float2 den = make_float2(bm.x - t1.x - t2.x, bm.y - t1.y - t2.y);
    const float nd = den.x * den.x + den.y * den.y;
    K[0] = make_float2(den.x / nd, -den.y / nd);
  }
  double *dsh = reinterpret_cast<double *>(smem_raw + ((soff + (size_t)ncell * 8 + 15) & ~(size_t)15));
  double *dres = dsh + (blockDim.x >> 5) * kFusedDiagValues;
  bulk_load_issue(S, u, ncell, bar_s);
  if (!bulk_load_wait(bar_s, err)) return;
  const float cs = fs.cstep;
  const int tid = threadIdx.x;
  const int nseg = max(1, min((int)blockDim.x / ng, 8));
  stencil_cols_seg(S, ng, cs, nseg);  // S1 = (I + c Dy) u
  __syncthreads();

  // push and deposit: S = S1 + src
  {
    const int n = slice_np_f(p, is, np);
    const float scl = fs.dep_scl * slice_cur_f(p, is, np);
    const float2 *fslice[1] = {u};
    const size_t base = (size_t)is * np;
    const int lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    const float g0 = (float)sc.gammaref;
    const float ez = p.eloss ? (float)p.eloss[is] : 0.f;
    for (int w0 = warp * 32 * U; w0 < n; w0 += nwarp * 32 * U) {
      float dg[U], x[U], y[U], px[U], py[U];
      long long th[U];
#pragma unroll
      for (int v = 0; v < U; v++) {
        const int ip = w0 + v * 32 + lane;
        const bool in = ip < n;
        const size_t o = base + (in ? ip : 0);
        dg[v] = p.dg[o];
        x[v] = p.x[o];
        y[v] = p.y[o];
        px[v] = p.px[o];
        py[v] = p.py[o];
        th[v] = p.theta[o];
      }
#pragma unroll
      for (int v = 0; v < U; v++) {
        const int ip = w0 + v * 32 + lane;
        const bool in = ip < n;
        if (in) {
          th[v] += sc.autophase_q;
          transverse_f(sc, false, g0 + dg[v], x[v], y[v], px[v], py[v]);
          push_rest_f<1>(sc, p, fslice, is, ip, ng, ez, dg[v], th[v], x[v], y[v], px[v], py[v]);
          const size_t o = base + ip;
          p.dg[o] = dg[v];
          p.theta[o] = th[v];
          p.x[o] = x[v];
          p.y[o] = y[v];
          p.px[o] = px[v];
          p.py[o] = py[v];
        }
        if (deposit)
          deposit_lanes(sc, fs, scl, S, ng, in ? x[v] : 1e30f, in ? y[v] : 1e30f, th[v], dg[v]);
      }
    }
  }
  __syncthreads();
  // the beam record of this slice, from the pushed particles (read back from L2)
  if (dbeam) slice_beam_sums(p, gref, is, np, nharm, dsh, dres, dbeam + (size_t)is * beam_diag_width(nharm));
  const float2 invden = K[0];
  const int line = tid >> 1, up = tid & 1;
  const bool segmented = fs.tw > 0 && nseg >= 2;
  const unsigned mask = __ballot_sync(0xffffffffu, line < ng);
  if (segmented)
    thomas_seg(S, ng, 1, ng, nseg, fs.tw, C, CB, CW);  // rows: u'
  else if (line < ng)
    thomas2(S + line * ng, 1, ng, up, CB, CW, a, invden, mask);
  __syncthreads();
  r2_cols_seg(S, u, ng, cs, nseg);  // 2 u' - S1
  __syncthreads();
  float fsum[kFieldSums];
  if (segmented && dfield)
    thomas_seg<true>(S, 1, ng, ng, nseg, fs.tw, C, CB, CW, fsum);  // columns, with the record's sums
  else if (segmented)
    thomas_seg(S, 1, ng, ng, nseg, fs.tw, C, CB, CW);  // columns
  else if (line < ng)
    thomas2(S + line, ng, ng, up, CB, CW, a, invden, mask);
  __syncthreads();
  bulk_store(u, S, ncell);
  if (dfield) {
    if (segmented)
      finish_field_sums(S, ng, fsum, dsh, dres, dfield + (size_t)i * (kFieldSums + 2));
    else
      slice_field_sums(S, ng, dsh, dres, dfield + (size_t)i * (kFieldSums + 2));
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

template <int BS>
__device__ __forceinline__ double bsum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < BS / 32; i++) r += sh[i];
  return r;
}
template <int BS, bool MAX>
__device__ __forceinline__ double bext(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_down_sync(0xffffffffu, v, o);
    v = MAX ? fmax(v, w) : fmin(v, w);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = sh[0];
  if (threadIdx.x == 0)
    for (int i = 1; i < BS / 32; i++) r = MAX ? fmax(r, sh[i]) : fmin(r, sh[i]);
  return r;
}

// DiagBeam sums with FP64 accumulation (Diagnostic.cpp:415-456); one block per slice
// Compensated (Kahan) FP32 sum: a thread's partial sum of a slice quantity keeps
// ~FP32 relative accuracy however many terms it takes, so it can be folded into the
// FP64 slice total once (GB300's FP64 rate is 1/64 of FP32; per-term FP64 adds would
// bound the diagnostics).
struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// All NS sums and NX min/max pairs of a block in one pass: every warp reduces its
// lanes' values with shuffles, lane 0 stores them, and after one barrier thread k
// combines value k over the warps (sums in FP64). Thread 0..NS-1 return their sum in
// *sum, threads NS..NS+2NX-1 their minimum or maximum in *ext. The lanes' compensated
// sums enter as FP32 pairs (s, -c): no FP64 arithmetic before lane 0's store.
template <int BS, int NS, int NX>
__device__ __forceinline__ void block_reduce_all(const KahanF *s, const float *mn, const float *mx, double *sh,
                                                 double *out) {
  constexpr int NW = BS / 32, NV = NS + 2 * NX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // within a warp as an unevaluated pair of FP32 numbers (hi + lo: the lane's Kahan
  // sum and its negated compensation), added level by level with the exact rounding
  // error of hi's sum (Knuth's TwoSum) carried into lo: FP32 shuffles and adds instead
  // of FP64 ones, which run at 1/64 of the FP32 rate, to about 44 bits
#pragma unroll
  for (int k = 0; k < NS; k++) {
    float hi = s[k].s;
    float lo = -s[k].c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
      const float t = hi + oh, bp = t - hi;
      const float e = (hi - (t - bp)) + (oh - bp);
      hi = t;
      lo = lo + ol + e;
    }
    if (lane == 0) sh[warp * NV + k] = (double)hi + (double)lo;
  }
#pragma unroll
  for (int k = 0; k < NX; k++) {
    float a = mn[k], b = mx[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = fminf(a, __shfl_down_sync(0xffffffffu, a, o));
      b = fmaxf(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    if (lane == 0) {
      sh[warp * NV + NS + 2 * k] = a;
      sh[warp * NV + NS + 2 * k + 1] = b;
    }
  }
  __syncthreads();
  const int k = threadIdx.x;
  if (k < NV) {
    double r = sh[k];
    for (int w = 1; w < NW; w++) {
      const double v = sh[w * NV + k];
      if (k < NS)
        r += v;
      else
        r = ((k - NS) & 1) ? fmax(r, v) : fmin(r, v);
    }
    out[k] = r;
  }
}

// Per-slice beam sums of the mixed form (layout of k_diag_beam in the FP64 form):
// the coordinates are FP32 and gamma is the FP32 offset from gammaref, so every
// particle's terms are formed in FP32; each thread sums its particles' terms with
// compensated FP32 sums, folded into FP64 once, and the slice totals are FP64 sums
// over the threads (the per-slice reductions, bunching and energy included, stay
// FP64; GB300 runs FP64 at 1/64 of the FP32 rate, so per-particle FP64 arithmetic
// would bound the kernel). The energy moments are
// taken about gammaref: sum g = N gref + sum dg and sum g^2 = N gref^2 + 2 gref sum dg
// + sum dg^2, without the cancellation of squaring g itself. NH: compile-time bound on
// the number of harmonics (the arrays stay in registers).
template <int BS, int NH>
__global__ void __launch_bounds__(BS) k_diag_beam_f(PtrsF p, double gref, int np, int nharm, double *out) {
  constexpr int NSUM = kBeamSums + 2 * NH;
  __shared__ double sh[(BS / 32) * (NSUM + 10)];
  __shared__ double res[NSUM + 10];
  const int is = blockIdx.x;
  const size_t base = (size_t)is * np;
  const int cnt = slice_np_f(p, is, np);
  const int nh = min(nharm, NH);
  // dg, dg^2, x, x^2, y, y^2, px, px^2, py, py^2, x px, y py, then (Re, Im) b_h
  KahanF c[NSUM];
  float mn[5], mx[5];  // x, px, y, py, dg
#pragma unroll
  for (int k = 0; k < 5; k++) {
    mn[k] = INFINITY;
    mx[k] = -INFINITY;
  }
#pragma unroll 4
  for (int ip = threadIdx.x; ip < cnt; ip += BS) {
    const float x = p.x[base + ip], y = p.y[base + ip], dg = p.dg[base + ip];
    const float px = p.px[base + ip], py = p.py[base + ip];
    const long long th = p.theta[base + ip];
    c[0].add(dg); c[1].add(dg * dg); c[2].add(x); c[3].add(x * x); c[4].add(y); c[5].add(y * y);
    c[6].add(px); c[7].add(px * px); c[8].add(py); c[9].add(py * py); c[10].add(x * px); c[11].add(y * py);
    mn[0] = fminf(mn[0], x); mx[0] = fmaxf(mx[0], x);
    mn[1] = fminf(mn[1], px); mx[1] = fmaxf(mx[1], px);
    mn[2] = fminf(mn[2], y); mx[2] = fmaxf(mx[2], y);
    mn[3] = fminf(mn[3], py); mx[3] = fmaxf(mx[3], py);
    mn[4] = fminf(mn[4], dg); mx[4] = fmaxf(mx[4], dg);
#pragma unroll
    for (int h = 0; h < NH; h++) {
      if (h < nh) {
        float sn, cs;
        sincosf(phase_of(th, (unsigned)(h + 1)), &sn, &cs);  // exact harmonic of the phase
        c[kBeamSums + 2 * h].add(cs);
        c[kBeamSums + 2 * h + 1].add(sn);
      }
    }
  }
  block_reduce_all<BS, NSUM, 5>(c, mn, mx, sh, res);
  __syncthreads();
  const int w = beam_diag_width(nharm);
  double *o = out + (size_t)is * w;
  const int k = threadIdx.x;
  const double n = (double)cnt;
  if (k == 0) o[0] = n * gref + res[0];
  if (k == 1) o[1] = n * gref * gref + 2.0 * gref * res[0] + res[1];
  if (k >= 2 && k < kBeamSums) o[k] = res[k];
  if (k >= kBeamSums && k < kBeamSums + 2 * nh) o[kBeamMinMax + k] = res[k];  // bunching after min/max
  if (k < 10) o[kBeamSums + k] = (k >= 8 ? gref : 0.0) + res[NSUM + k];
}

// Per-slice field sums of the mixed form (layout of k_diag_field): a flat walk over
// the cells (row and column carried along, no division per cell), each thread's
// terms summed with compensated FP32 sums and folded into the FP64 slice totals once.
template <int BS>
__global__ void __launch_bounds__(BS) k_diag_field_f(const float2 *field, int ng, double *out) {
  __shared__ double sh[(BS / 32) * kFieldSums];
  __shared__ double res[kFieldSums];
  const int is0 = blockIdx.x;
  const int ncell = ng * ng;
  const float2 *f = field + (size_t)is0 * ncell;
  const float shift = -0.5f * (float)(ng - 1);
  KahanF c[kFieldSums];
  int row = threadIdx.x / ng, col = threadIdx.x % ng;
#pragma unroll 4
  for (int i = threadIdx.x; i < ncell; i += BS) {
    const float dx = (float)col + shift, dy = (float)row + shift;
    const float2 v = f[i];
    const float wei = v.x * v.x + v.y * v.y;
    c[0].add(wei); c[1].add(dx * wei); c[2].add(dx * dx * wei); c[3].add(dy * wei); c[4].add(dy * dy * wei);
    c[5].add(v.x); c[6].add(v.y);
    col += BS;  // the next cell of this thread, BS further on
    while (col >= ng) {
      col -= ng;
      row++;
    }
  }
  block_reduce_all<BS, kFieldSums, 0>(c, nullptr, nullptr, sh, res);
  __syncthreads();
  double *o = out + (size_t)is0 * (kFieldSums + 2);
  if (threadIdx.x < kFieldSums) o[threadIdx.x] = res[threadIdx.x];
  if (threadIdx.x == 0) {
    float2 v = f[(size_t)(ng / 2) * ng + ng / 2];
    o[7] = v.x;
    o[8] = v.y;
  }
}

PtrsF make_ptrs_f(const DeviceBeam &b, void *const *field, void *const *src, int nfld) {
  PtrsF p{};
  p.dg = (float *)b.gamma;
  p.theta = (long long *)b.theta;
  p.x = (float *)b.x;
  p.y = (float *)b.y;
  p.px = (float *)b.px;
  p.py = (float *)b.py;
  p.current = b.current;
  p.count = b.count;
  for (int k = 0; k < nfld && k < G4GPU_MAX_FIELDS; k++) {
    p.field[k] = field ? (const float2 *)field[k] : nullptr;
    p.src[k] = src ? (float2 *)src[k] : nullptr;
  }
  return p;
}

// ---- fused field step on a cluster of CTAs (2, 3 or 4 per slice) ---------------
//
// The slice's rows are split between the CL CTAs of a thread-block cluster: CTA q
// holds the band of rows [q h, min((q + 1) h, ng)), h = ceil(ng / CL). A band is a
// fraction of the slice (92 KB at ngrid 151 for a pair, 131 KB at ngrid 255 for four),
// so grids too large for one CTA still take the one-pass step with the field read and
// written once, and a pair's two CTAs share an SM, one CTA's bulk copies, barriers and
// latency overlapping the other's arithmetic. The phases are those of k_field_fused_f,
// with what crosses a band boundary done as follows:
//  * the column stencils take the rows just outside a CTA's band from the slice in
//    global memory, which stays unmodified until the final stores;
//  * the deposition: every CTA reads every particle of the slice and deposits the
//    contributions to its own rows (deposit_pair);
//  * the column solves' segments next to a boundary take their warm-up values from
//    the neighbouring CTA's shared memory (distributed shared memory), read between
//    cluster barriers that order them against that CTA's in-place writes. A warm-up
//    spans W <= 21 rows, so only the adjacent bands are read, and the host requires
//    the last band to hold at least W rows.
// Every thread of every CTA passes every cluster barrier (no early exit), and the
// last distributed-shared-memory access precedes the last cluster barrier.
namespace cg = cooperative_groups;

// CTA size: a pair shares an SM (two CTAs of 512 threads); larger clusters take one
// CTA of 1024 threads per SM
template <int CL>
constexpr int band_threads() {
  return CL == 2 ? 512 : 1024;
}

template <int CL>
__device__ __forceinline__ void band_rows(int ng, int q, int &r0, int &nrow) {
  const int h = (ng + CL - 1) / CL;
  r0 = q * h;
  nrow = min(h, ng - r0);
}

// thomas_seg for nline lines of n elements (the rows of a band)
__device__ __forceinline__ void thomas_lines(float2 *S, int nline, int lstride, int estride, int n, int nseg, int W,
                                             const float2 *Cc, const float2 *CB, const float2 *CW) {
  const int tid = threadIdx.x;
  const int line = tid % nline, seg = tid / nline;
  const int len = (n + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, n);
  const bool act = seg < nseg && b < e;
  float2 *L = S + (size_t)line * lstride;
  float2 d = make_float2(0.f, 0.f);
  if (act)
    for (int k = max(0, b - W); k < b; k++) {
      float2 r = L[k * estride];
      d = cmulf(sub_imulf(r, Cc[k].y, d), CB[k]);
    }
  __syncthreads();
  if (act)
    for (int k = b; k < e; k++) {
      float2 r = L[k * estride];
      d = cmulf(sub_imulf(r, Cc[k].y, d), CB[k]);
      L[k * estride] = d;
    }
  __syncthreads();
  const int k1 = min(n - 1, e - 1 + W);
  float2 x = make_float2(0.f, 0.f);
  if (act && k1 >= e) {
    x = L[k1 * estride];
    for (int k = k1 - 1; k >= e; k--) {
      x = sub_cmulf(L[k * estride], CW[k + 1], x);
    }
  }
  __syncthreads();
  if (act)
    for (int k = e - 1; k >= b; k--) {
      float2 v = L[k * estride];
      if (k < n - 1) {
        v = sub_cmulf(v, CW[k + 1], x);
      }
      x = v;
      L[k * estride] = x;
    }
  __syncthreads();
}

// S1 = (I + c Dy) u on the band's rows [r0, r0 + nrow) in place (band row k at
// S[k * ng + col]), column segments as stencil_cols_seg; the rows just outside the
// band are read from u in global memory.
__device__ __forceinline__ void stencil_cols_band(float2 *S, const float2 *__restrict__ u, int ng, int r0, int nrow,
                                                  float cs, int nseg) {
  const int tid = threadIdx.x;
  const int col = tid % ng, seg = tid / ng;
  const int len = (nrow + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, nrow);
  const bool act = seg < nseg && b < e;
  float2 above = make_float2(0.f, 0.f), below = make_float2(0.f, 0.f);
  if (act) {
    const int ga = r0 + b - 1, gb = r0 + e;
    if (ga >= 0) above = b > 0 ? S[(b - 1) * ng + col] : u[(size_t)ga * ng + col];
    if (gb < ng) below = e < nrow ? S[e * ng + col] : u[(size_t)gb * ng + col];
  }
  __syncthreads();
  if (act) {
    float2 prev = above, cur = S[b * ng + col];
    float2 next = (b + 1 < e) ? S[(b + 1) * ng + col] : below;
    for (int k = b; k < e; k++) {
      float2 nx = next;
      if (k + 2 < e)
        next = S[(k + 2) * ng + col];
      else if (k + 2 == e)
        next = below;
      const int g = r0 + k;
      float2 out = stencil(cs, cur, lapf(g > 0, g < ng - 1, prev, cur, nx));
      prev = cur;
      cur = nx;
      S[k * ng + col] = out;
    }
  }
}

// S = 2 u' - S1 on the band's rows, S1 recomputed from u in global memory (r2_cols_seg)
__device__ __forceinline__ void r2_cols_band(float2 *S, const float2 *__restrict__ u, int ng, int r0, int nrow,
                                             float cs, int nseg) {
  const int tid = threadIdx.x;
  const int col = tid % ng, seg = tid / ng;
  const int len = (nrow + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, nrow);
  if (seg >= nseg || b >= e) return;
  const int g0 = r0 + b;
  float2 prev = g0 > 0 ? u[(size_t)(g0 - 1) * ng + col] : make_float2(0.f, 0.f);
  float2 cur = u[(size_t)g0 * ng + col];
  float2 next = g0 + 1 < ng ? u[(size_t)(g0 + 1) * ng + col] : make_float2(0.f, 0.f);
  for (int k = b; k < e; k++) {
    const int g = r0 + k;
    float2 nx = next;
    if (g + 2 < ng) next = u[(size_t)(g + 2) * ng + col];
    float2 s1 = stencil(cs, cur, lapf(g > 0, g < ng - 1, prev, cur, nx));
    prev = cur;
    cur = nx;
    float2 v = S[k * ng + col];
    S[k * ng + col] = make_float2(2.f * v.x - s1.x, 2.f * v.y - s1.y);
  }
}

// Column solve of a cluster (thomas_seg along the columns, rows split between the
// CTAs): band row k of this CTA is global row r0 + k; the warm-ups of the segments
// next to a boundary read the band above (Pa, nrow_above rows) or below (Pb) in the
// neighbouring CTA's shared memory (distributed shared memory).
__device__ __forceinline__ void thomas_cols_band(cg::cluster_group &cl, float2 *S, const float2 *Pa,
                                                 const float2 *Pb, int ng, int r0, int nrow, int nrow_above,
                                                 int nseg, int W, const float2 *Cc, const float2 *CB,
                                                 const float2 *CW) {
  const int tid = threadIdx.x;
  const int col = tid % ng, seg = tid / ng;
  const int len = (nrow + nseg - 1) / nseg;
  const int b = seg * len, e = min(b + len, nrow);
  const bool act = seg < nseg && b < e;
  // band row k, k < 0 or k >= nrow meaning the rows of the band above or below (k
  // stays within W rows of the band, and only the first band has none above, the
  // last none below: their sweeps start and end at the grid's edge)
  auto at = [&](int k) -> float2 {
    if (k >= 0 && k < nrow) return S[k * ng + col];
    return k < 0 ? Pa[(nrow_above + k) * ng + col] : Pb[(k - nrow) * ng + col];
  };
  float2 d = make_float2(0.f, 0.f);
  if (act)
    for (int k = max(-r0, b - W); k < b; k++) {
      const int g = r0 + k;
      float2 r = at(k);
      d = cmulf(sub_imulf(r, Cc[g].y, d), CB[g]);
    }
  cl.sync();
  if (act)
    for (int k = b; k < e; k++) {
      const int g = r0 + k;
      float2 r = S[k * ng + col];
      d = cmulf(sub_imulf(r, Cc[g].y, d), CB[g]);
      S[k * ng + col] = d;
    }
  cl.sync();
  const int k1 = min(ng - 1 - r0, e - 1 + W);
  float2 x = make_float2(0.f, 0.f);
  if (act && k1 >= e) {
    x = at(k1);
    for (int k = k1 - 1; k >= e; k--) {
      x = sub_cmulf(at(k), CW[r0 + k + 1], x);
    }
  }
  cl.sync();
  if (act)
    for (int k = e - 1; k >= b; k--) {
      const int g = r0 + k;
      float2 v = S[k * ng + col];
      if (g < ng - 1) {
        v = sub_cmulf(v, CW[g + 1], x);
      }
      x = v;
      S[k * ng + col] = x;
    }
  __syncthreads();
}

// Cell and weights of a particle (ll_gridpoint_f) with the row and column kept.
struct CellRC {
  int ix, iy, ix1, iy1;
  float wx, wy;
};
__device__ __forceinline__ bool cell_rc(float gm, float dg, int ng, float x, float y, CellRC &c) {
  if ((x > -gm) && (x < gm) && (y > -gm) && (y < gm)) {
    float wx = (x + gm) / dg, wy = (y + gm) / dg;
    float fx = floorf(wx), fy = floorf(wy);
    c.ix = min((int)fx, ng - 1);
    c.iy = min((int)fy, ng - 1);
    c.wx = 1.f + fx - wx;
    c.wy = 1.f + fy - wy;
    c.ix1 = c.ix + 1 < ng ? c.ix + 1 : c.ix;
    c.iy1 = c.iy + 1 < ng ? c.iy + 1 : c.iy;
    return true;
  }
  return false;
}

// The contribution to cell (ix, iy) if row iy is one of this CTA's rows [r0, r0 + nrow)
// (its band S): every CTA of a cluster deposits into its own shared memory only.
__device__ __forceinline__ void pair_add(float2 *S, int r0, int nrow, int ng, int ix, int iy, float w, float cpx,
                                         float cpy) {
  if (iy < r0 || iy >= r0 + nrow) return;
  float2 *t = S + (size_t)(iy - r0) * ng + ix;
  atomicAdd(&t->x, w * cpx);
  atomicAdd(&t->y, w * cpy);
}
__device__ __forceinline__ void pair_group(const StepConstF &sc, const FieldStepF &fs, float scl, float2 *S,
                                           int r0, int nrow, int ng, float x, float y, const long long *th,
                                           const float *dgam, int n) {
  CellRC c;
  if (!cell_rc(fs.gridmax, fs.dgrid, ng, x, y, c)) return;
  if (c.iy1 < r0 || c.iy >= r0 + nrow) return;  // the particle's rows are another band's
  float dx = x - sc.ax, dy = y - sc.ay;
  float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
  float a = sqrtf(faw2) * scl;
  float cpx = 0.f, cpy = 0.f;
  for (int m = 0; m < n; m++) {
    float part = a / ((float)sc.gammaref + dgam[m]);
    float sn, co;
    __sincosf(phase_of(th[m], (unsigned)fs.harm), &sn, &co);
    cpx += sn * part;
    cpy += co * part;
  }
  pair_add(S, r0, nrow, ng, c.ix, c.iy, c.wx * c.wy, cpx, cpy);
  pair_add(S, r0, nrow, ng, c.ix1, c.iy, (1.f - c.wx) * c.wy, cpx, cpy);
  pair_add(S, r0, nrow, ng, c.ix, c.iy1, c.wx * (1.f - c.wy), cpx, cpy);
  pair_add(S, r0, nrow, ng, c.ix1, c.iy1, (1.f - c.wx) * (1.f - c.wy), cpx, cpy);
}
// Four particles in one cell that do not share x and y exactly (deposit_cell4's case),
// into the rows [r0, r0 + nrow) of a band: each particle's weighted phasor summed in
// registers, then one atomic pair per corner in the band. Returns false, having
// deposited nothing, unless all four lie inside the grid in the same cell.
__device__ __forceinline__ bool pair_cell4(const StepConstF &sc, const FieldStepF &fs, float scl, float2 *S,
                                           int r0, int nrow, int ng, const float *x, const float *y,
                                           const long long *th, const float *dgam) {
  CellRC c;
  if (!cell_rc(fs.gridmax, fs.dgrid, ng, x[0], y[0], c)) return false;
#pragma unroll
  for (int m = 1; m < 4; m++) {
    CellRC cm;
    if (!cell_rc(fs.gridmax, fs.dgrid, ng, x[m], y[m], cm) || cm.ix != c.ix || cm.iy != c.iy) return false;
  }
  if (c.iy1 < r0 || c.iy >= r0 + nrow) return true;  // the four particles' rows are another band's
  float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int m = 0; m < 4; m++) {
    CellRC cm;
    cell_rc(fs.gridmax, fs.dgrid, ng, x[m], y[m], cm);
    const float dx = x[m] - sc.ax, dy = y[m] - sc.ay;
    const float faw2 = 1.f + sc.kx * dx * dx + sc.ky * dy * dy + 2.f * (sc.gradx * dx + sc.grady * dy);
    const float part = sqrtf(faw2) * scl / ((float)sc.gammaref + dgam[m]);
    float sn, co;
    __sincosf(phase_of(th[m], (unsigned)fs.harm), &sn, &co);
    const float cpx = sn * part, cpy = co * part;
    const float w00 = cm.wx * cm.wy, w10 = (1.f - cm.wx) * cm.wy, w01 = cm.wx * (1.f - cm.wy),
                w11 = (1.f - cm.wx) * (1.f - cm.wy);
    v[0] += w00 * cpx; v[1] += w00 * cpy; v[2] += w10 * cpx; v[3] += w10 * cpy;
    v[4] += w01 * cpx; v[5] += w01 * cpy; v[6] += w11 * cpx; v[7] += w11 * cpy;
  }
  pair_add(S, r0, nrow, ng, c.ix, c.iy, 1.f, v[0], v[1]);
  pair_add(S, r0, nrow, ng, c.ix1, c.iy, 1.f, v[2], v[3]);
  pair_add(S, r0, nrow, ng, c.ix, c.iy1, 1.f, v[4], v[5]);
  pair_add(S, r0, nrow, ng, c.ix1, c.iy1, 1.f, v[6], v[7]);
  return true;
}
// A cluster's deposition: each CTA reads every particle of the slice and deposits the
// contributions to its own rows into its own band, with shared-memory atomics only. A
// particle whose footprint straddles two bands is deposited by both, each into its
// rows. (Splitting the particles between the CTAs of a pair instead sends half of
// every CTA's contributions to the peer as distributed-shared-memory atomics, which
// took 2.8 times as long as the single CTA's whole deposition.)
__device__ __forceinline__ void deposit_pair(const StepConstF &sc, const FieldStepF &fs, const PtrsF &p, float2 *S,
                                             int r0, int nrow, int is, int np, int ng) {
  const float scl = fs.dep_scl * slice_cur_f(p, is, np);
  const size_t base = (size_t)is * np;
  if ((np & 3) == 0 && !p.count) {
    const int nq = np >> 2;
    const float4 *X = reinterpret_cast<const float4 *>(p.x + base);
    const float4 *Y = reinterpret_cast<const float4 *>(p.y + base);
    const float4 *G = reinterpret_cast<const float4 *>(p.dg + base);
    const longlong2 *TH = reinterpret_cast<const longlong2 *>(p.theta + base);
    for (int g = threadIdx.x; g < nq; g += blockDim.x) {
      const float4 x = X[g], y = Y[g], gg = G[g];
      const longlong2 t01 = TH[2 * g], t23 = TH[2 * g + 1];
      const long long th[4] = {t01.x, t01.y, t23.x, t23.y};
      const float dg[4] = {gg.x, gg.y, gg.z, gg.w};
      const bool p01 = x.x == x.y && y.x == y.y, p23 = x.z == x.w && y.z == y.w;
      const float xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
      if (p01 && p23 && x.x == x.z && y.x == y.z) {
        pair_group(sc, fs, scl, S, r0, nrow, ng, x.x, y.x, th, dg, 4);
      } else if (!pair_cell4(sc, fs, scl, S, r0, nrow, ng, xs, ys, th, dg)) {
        if (p01) {
          pair_group(sc, fs, scl, S, r0, nrow, ng, x.x, y.x, th, dg, 2);
        } else {
          pair_group(sc, fs, scl, S, r0, nrow, ng, x.x, y.x, th, dg, 1);
          pair_group(sc, fs, scl, S, r0, nrow, ng, x.y, y.y, th + 1, dg + 1, 1);
        }
        if (p23) {
          pair_group(sc, fs, scl, S, r0, nrow, ng, x.z, y.z, th + 2, dg + 2, 2);
        } else {
          pair_group(sc, fs, scl, S, r0, nrow, ng, x.z, y.z, th + 2, dg + 2, 1);
          pair_group(sc, fs, scl, S, r0, nrow, ng, x.w, y.w, th + 3, dg + 3, 1);
        }
      }
    }
  } else {
    const int n = slice_np_f(p, is, np);
    for (int ip = threadIdx.x; ip < n; ip += blockDim.x) {
      const long long th = p.theta[base + ip];
      const float dg = p.dg[base + ip];
      pair_group(sc, fs, scl, S, r0, nrow, ng, p.x[base + ip], p.y[base + ip], &th, &dg, 1);
    }
  }
}

// shared memory of one CTA of a cluster of CL: mbarrier, coefficients, slack, its band
size_t band_smem_bytes(int ng, int CL) {
  return ((16 + 3 * (size_t)ng * 8 + 15) & ~(size_t)15) + 8 + (size_t)((ng + CL - 1) / CL) * ng * 8;
}

template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(band_threads<CL>(), CL == 2 ? 2 : 1)
    k_field_band_f(StepConstF sc, int k, PtrsF p, float2 *__restrict__ field, const float2 *__restrict__ coef,
                   int ns, int np, int ng, int deposit, int *err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cl = cg::this_cluster();
  const int q = (int)cl.block_rank();
  const int ncell = ng * ng;
  const FieldStepF &fs = sc.f[k];
  const int is = blockIdx.x / CL;
  const int i = (is + fs.first) % ns;
  float2 *u = field + (size_t)i * ncell;
  int r0, nrow, r0a, nrowa, r0b, nrowb;
  band_rows<CL>(ng, q, r0, nrow);
  band_rows<CL>(ng, q > 0 ? q - 1 : q, r0a, nrowa);
  band_rows<CL>(ng, q < CL - 1 ? q + 1 : q, r0b, nrowb);
  float2 *ub = u + (size_t)r0 * ng;  // this CTA's band in global memory
  // layout as k_field_fused_f: [mbarrier][8 B][coefficients 3 ng][pad][band], the band
  // congruent to its global rows mod 16; a neighbour's band at its own offset
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
  float2 *C = reinterpret_cast<float2 *>(smem_raw + 16);
  float2 *CB = C + ng, *CW = CB + ng;
  const size_t soff = (16 + 3 * (size_t)ng * 8 + 15) & ~(size_t)15;
  float2 *S = reinterpret_cast<float2 *>(smem_raw + soff + (reinterpret_cast<uintptr_t>(ub) & 15));
  auto band_of = [&](int r0n, int rank) -> float2 * {
    float2 *local = reinterpret_cast<float2 *>(
        smem_raw + soff + (reinterpret_cast<uintptr_t>(u + (size_t)r0n * ng) & 15));
    return cl.map_shared_rank(local, rank);
  };
  // the bands above and below (a CTA's own band stands in at the grid's edges, where
  // the column solve reads no neighbour)
  const float2 *Pa = band_of(r0a, q > 0 ? q - 1 : q);
  const float2 *Pb = band_of(r0b, q < CL - 1 ? q + 1 : q);
  uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int t = threadIdx.x; t < 3 * ng; t += blockDim.x) C[t] = coef[t];
  __syncthreads();
  // a wait that runs out raises the flag and the step goes on: leaving early would
  // strand the peer at a cluster barrier
  bulk_load(S, ub, nrow * ng, bar_s, err);
  const float cs = fs.cstep;
  const int nseg = max(1, min((int)blockDim.x / ng, 8));
  stencil_cols_band(S, u, ng, r0, nrow, cs, nseg);  // S1 on this band
  __syncthreads();  // the band holds S1 before any deposit
  if (deposit) deposit_pair(sc, fs, p, S, r0, nrow, is, np, ng);
  cl.sync();  // every band is complete before the solves read across the cluster
  thomas_lines(S, nrow, ng, 1, ng, max(1, min((int)blockDim.x / nrow, 32)), fs.tw, C, CB, CW);  // rows
  r2_cols_band(S, u, ng, r0, nrow, cs, nseg);
  __syncthreads();
  thomas_cols_band(cl, S, Pa, Pb, ng, r0, nrow, nrowa, nseg, fs.tw, C, CB, CW);  // columns
  bulk_store(ub, S, nrow * ng);
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// ---- ADI step without device allocation (g4gpu_adi_advance_noalloc) -------------
//
// Layout of the file-scope scratch array (g4_noalloc_scratch below):
//   [0, 4)              device error flag, cleared by every call
//   [256, 256 + 24 ng)  ADI coefficients c, cbet, cwet as float2, written by every call
//   [8192, ...)         one S1 slot per CTA: (I + c Dy) u of the slice in hand, 256-byte
//                       aligned slots of (ngrid^2 + 2) float2 rounded up
constexpr size_t kNoallocScratchBytes = 32u << 20;
constexpr size_t kNoallocCoefOffset = 256;
constexpr size_t kNoallocSlotOffset = 8192;

// bulk_load with the mbarrier phase parity given (a CTA that loads several slices
// waits on phases 0, 1, 0, ...); also orders this CTA's earlier generic-proxy
// accesses of s before the bulk copy overwrites it
__device__ __forceinline__ bool bulk_load_parity(float2 *s, const float2 *g, int count, uint32_t bar,
                                                 uint32_t parity, int *err) {
  uintptr_t ga = reinterpret_cast<uintptr_t>(g);
  int head = (ga & 15) ? 1 : 0;
  int body = (count - head) & ~1;
  int tail = count - head - body;
  if (threadIdx.x == 0) {
    uint32_t bytes = (uint32_t)body * 8u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    if (bytes) {
      uint32_t dst = (uint32_t)__cvta_generic_to_shared(s + head);
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(dst), "l"(g + head), "r"(bytes), "r"(bar)
          : "memory");
    }
  }
  if (head && threadIdx.x == 32) s[0] = g[0];
  if (tail && threadIdx.x == 64) s[count - 1] = g[count - 1];
  return bulk_wait_uniform(bar, parity, err);
}

// The ADI half steps of k_field_fused_f with the source read from a caller's array
// instead of deposited from particles, and with a fixed number of CTAs that take
// slices is = blockIdx.x, blockIdx.x + gridDim.x, ... so that the S1 scratch is one
// slot per CTA rather than one per slice. Field storage slot (is + first) % ns is
// advanced with source slice is (the ring order of FieldSolverADI::advance,
// FieldSolverADI.cpp:9-58).
__global__ void __launch_bounds__(kFusedMaxThreads, 1)
    k_adi_noalloc_f(float2 *__restrict__ field, const float2 *__restrict__ source,
                    unsigned char *__restrict__ scratch, float cs, int ns, int ng, int first,
                    size_t slot_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int *err = reinterpret_cast<int *>(scratch);
  const float2 *coef = reinterpret_cast<const float2 *>(scratch + kNoallocCoefOffset);
  float2 *slot =
      reinterpret_cast<float2 *>(scratch + kNoallocSlotOffset + (size_t)blockIdx.x * slot_bytes);
  const int ncell = ng * ng;
  const int tid = threadIdx.x;
  // shared layout as in k_field_fused_f; S moves by 8 bytes per slice to stay
  // congruent to the slice's address mod 16
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
  float2 *K = reinterpret_cast<float2 *>(smem_raw + 8);
  float2 *C = reinterpret_cast<float2 *>(smem_raw + 16);
  float2 *CB = C + ng, *CW = CB + ng;
  const size_t soff = (16 + 3 * (size_t)ng * 8 + 15) & ~(size_t)15;
  uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int t = tid; t < 3 * ng; t += blockDim.x) C[t] = coef[t];
  __syncthreads();
  const float2 a = C[1];
  if (tid == 0) {
    int m = ng / 2;
    float2 bm = make_float2(CB[0].x, -CB[0].y);
    float n0 = CB[0].x * CB[0].x + CB[0].y * CB[0].y;
    bm.x /= n0;
    bm.y /= n0;
    float2 t1 = cmulf(a, CW[m]), t2 = cmulf(a, CW[ng - 1 - m]);
    float2 den = make_float2(bm.x - t1.x - t2.x, bm.y - t1.y - t2.y);
    float nd = den.x * den.x + den.y * den.y;
    K[0] = make_float2(den.x / nd, -den.y / nd);
  }
  __syncthreads();
  const float2 invden = K[0];
  const int line = tid >> 1, up = tid & 1;
  const unsigned mask = __ballot_sync(0xffffffffu, line < ng);
  uint32_t parity = 0;
  for (int is = blockIdx.x; is < ns; is += gridDim.x, parity ^= 1u) {
    const int i = (is + first) % ns;
    float2 *u = field + (size_t)i * ncell;
    const uintptr_t mis = reinterpret_cast<uintptr_t>(u) & 15;  // 0 or 8
    float2 *S = reinterpret_cast<float2 *>(smem_raw + soff + mis);
    float2 *s1 = slot + (mis ? 1 : 0);
    if (!bulk_load_parity(S, u, ncell, bar_s, parity, err)) return;
    if (tid < ng) stencil_line(S + tid, ng, ng, cs);  // S1 = (I + c Dy) u
    // the previous slice's generic reads of the slot precede its overwrite
    if (tid == 0) asm volatile("fence.proxy.async.global;" ::: "memory");
    bulk_store(s1, S, ncell);
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (source) {
      const float2 *src = source + (size_t)is * ncell;
      for (int t = tid; t < ncell; t += blockDim.x) {
        float2 v = S[t], w = src[t];
        S[t] = make_float2(v.x + w.x, v.y + w.y);
      }
      __syncthreads();
    }
    if (line < ng) thomas2(S + line * ng, 1, ng, up, CB, CW, a, invden, mask);  // rows: u'
    if (tid == 0) {
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
      asm volatile("fence.proxy.async.global;" ::: "memory");
    }
    __syncthreads();
    for (int t = tid; t < ncell; t += blockDim.x) {  // (I + c Dx) u' + src = 2 u' - S1
      float2 v = S[t], w = s1[t];
      S[t] = make_float2(2.f * v.x - w.x, 2.f * v.y - w.y);
    }
    __syncthreads();
    if (line < ng) thomas2(S + line, ng, ng, up, CB, CW, a, invden, mask);  // columns
    __syncthreads();
    bulk_store(u, S, ncell);
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();  // the next slice's load may overwrite S
  }
}

// complex arithmetic of the mixed form for the tiled ADI (adi_tiled.cuh), as in
// k_adi_x_f / k_adi_y_f
struct MixedOps {
  using V = float2;
  using G = float2;
  using R = float;
  static __device__ __forceinline__ V ld(const G *p) { return *p; }
  static __device__ __forceinline__ void st(G *p, V v) { *p = v; }
  static __device__ __forceinline__ V zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ V sub(V a, V b) { return make_float2(a.x - b.x, a.y - b.y); }
  static __device__ __forceinline__ V mul(V a, V b) { return cmulf(a, b); }
  static __device__ __forceinline__ V lap(bool hp, bool hn, V p, V u, V n) { return lapf(hp, hn, p, u, n); }
  static __device__ __forceinline__ V rhs(V s, V u, V l, R cs) {
    return make_float2(s.x + u.x - cs * l.y, s.y + u.y + cs * l.x);
  }
};

// FP32 space charge: e^{-i l theta} from the Q32.32 phase, whose l-th multiple is exact
struct MixedSC {
  using R = float;
  using R2 = float2;
  using Th = long long;
  using Step = StepConstF;
  static constexpr bool kPlain = false;
  static __device__ __forceinline__ float gamma(const StepConstF &s, float dg) { return (float)s.gammaref + dg; }
  static __device__ __forceinline__ void half(const StepConstF &s, float g, float &x, float &y, float &px,
                                              float &py) {
    transverse_f(s, false, g, x, y, px, py);
  }
  static __device__ __forceinline__ float2 eil(long long th, int l) {
    float s, c;
    __sincosf(phase_of(th, (unsigned)l), &s, &c);
    return make_float2(c, -s);
  }
};

}  // namespace
}  // namespace g4

#include "adi_tiled.cuh"
#include "sc_kernels.cuh"

namespace g4 {

void launch_sc_mixed(const Launch &L, const ScConst &c, const StepConstF &step, const DeviceBeam &b,
                     const ScBuffers &buf, int part) {
  ScBeam<MixedSC> sb{(float *)b.gamma, (float *)b.x,              (float *)b.y, (float *)b.px,
                     (float *)b.py,    (const long long *)b.theta, b.current,    b.count};
  sc_launch<MixedSC>(L, c, step, sb, buf, part);
}

void launch_push_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b,
                       void *const *field, void *const *src, int ns, int np, int ngrid,
                       int deposit, int block) {
  launch_push_mixed_sc(L, sc, b, field, src, ns, np, ngrid, deposit, block, 0, nullptr, nullptr, nullptr,
                       IsrStream{});
}

void launch_push_mixed_sc(const Launch &L, const StepConstF &sc, const DeviceBeam &b, void *const *field,
                          void *const *src, int ns, int np, int ngrid, int deposit, int block, int mode,
                          const void *ez, const double *eloss, const void *wake, const IsrStream &isr) {
  PtrsF p = make_ptrs_f(b, field, src, sc.nfld);
  if (isr.ctr && (sc.isr_avg != 0 || sc.isr_sig != 0) && mode != 1) p.isr = isr;
  p.mode = mode;
  p.ez = (const float *)ez;
  p.eloss = eloss;
  p.wake = (const float *)wake;
  if (mode == 1) deposit = 0;
  dim3 grid((np + block - 1) / block, ns);
  cudaStream_t s = (cudaStream_t)L.stream;
  switch (sc.nfld) {
    case 1: k_push_f<1><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
    case 2: k_push_f<2><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
    case 3: k_push_f<3><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
    default: k_push_f<G4GPU_MAX_FIELDS><<<grid, block, 0, s>>>(sc, p, ns, np, ngrid, deposit); break;
  }
}

void launch_deposit_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b,
                          void *const *src, int ns, int np, int ngrid) {
  PtrsF p = make_ptrs_f(b, nullptr, src, sc.nfld);
  dim3 grid((np + 255) / 256, ns);
  cudaStream_t s = (cudaStream_t)L.stream;
  switch (sc.nfld) {
    case 1: k_deposit_f<1><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
    case 2: k_deposit_f<2><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
    case 3: k_deposit_f<3><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
    default: k_deposit_f<G4GPU_MAX_FIELDS><<<grid, 256, 0, s>>>(sc, p, ns, np, ngrid); break;
  }
}

void launch_adi_mixed(const Launch &L, const StepConstF &sc, int k, int phase, void *field,
                      const void *src, void *tmp, const void *coef, int ns, int ngrid) {
  const float2 *cb = (const float2 *)coef;
  cudaStream_t s = (cudaStream_t)L.stream;
  // tiled passes (adi_tiled.cuh) when their tiles fit a CTA's shared memory
  const int R = tiled::band_rows(ngrid, sizeof(float2)), Cw = tiled::band_cols(ngrid, sizeof(float2));
  const size_t smx = (size_t)(2 * R + 2) * ngrid * sizeof(float2), smy = (size_t)ngrid * Cw * sizeof(float2);
  if (smx <= 227u * 1024u && smy <= 227u * 1024u) {
    static std::atomic<unsigned long long> configured{0};  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !(configured.load() & (1ull << dev))) {
      cudaFuncSetAttribute(tiled::k_adi_xt<MixedOps, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      cudaFuncSetAttribute(tiled::k_adi_yt<MixedOps, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      configured.fetch_or(1ull << dev);
    }
    tiled::CoefP<MixedOps> cf{cb, cb + ngrid, cb + 2 * ngrid};
    const int W = sc.f[k].tw;
    if (phase == 0)
      tiled::k_adi_xt<MixedOps, 256><<<dim3((ngrid + R - 1) / R, ns), 256, smx, s>>>(
          (const float2 *)field, (const float2 *)src, (float2 *)tmp, cf, sc.f[k].cstep, ns, ngrid,
          sc.f[k].first, R, W);
    else
      tiled::k_adi_yt<MixedOps, 256><<<dim3((ngrid + Cw - 1) / Cw, ns), 256, smy, s>>>(
          (float2 *)field, (const float2 *)tmp, cf, ns, ngrid, sc.f[k].first, Cw, W);
    return;
  }
  CoefF cf{cb, cb + ngrid, cb + 2 * ngrid};
  long long n = (long long)ns * ngrid;
  unsigned blocks = (unsigned)((n + 127) / 128);
  if (phase == 0)
    k_adi_x_f<<<blocks, 128, 0, s>>>((const float2 *)field, (const float2 *)src, (float2 *)tmp, cf,
                                     sc.f[k].cstep, ns, ngrid, sc.f[k].first);
  else
    k_adi_y_f<<<blocks, 128, 0, s>>>((float2 *)field, (const float2 *)src, (const float2 *)tmp, cf,
                                     sc.f[k].cstep, ns, ngrid, sc.f[k].first);
}

void launch_diag_beam_mixed(const Launch &L, const DeviceBeam &b, double gammaref, int ns, int np,
                            int nharm, double *out) {
  PtrsF p = make_ptrs_f(b, nullptr, nullptr, 0);
  cudaStream_t s = (cudaStream_t)L.stream;
  if (nharm <= 1)
    k_diag_beam_f<256, 1><<<ns, 256, 0, s>>>(p, gammaref, np, nharm, out);
  else if (nharm <= 3)
    k_diag_beam_f<256, 3><<<ns, 256, 0, s>>>(p, gammaref, np, nharm, out);
  else if (nharm <= 5)
    k_diag_beam_f<256, 5><<<ns, 256, 0, s>>>(p, gammaref, np, nharm, out);
  else
    k_diag_beam_f<256, G4GPU_MAX_HARM><<<ns, 256, 0, s>>>(p, gammaref, np, nharm, out);
}

void launch_diag_field_mixed(const Launch &L, const void *field, int ns, int ngrid, double *out) {
  k_diag_field_f<256><<<ns, 256, 0, (cudaStream_t)L.stream>>>((const float2 *)field, ngrid, out);
}

// shared memory of the fused kernel: mbarrier, coefficients, alignment slack, slice
size_t fused_smem_bytes(int ng) {
  return ((16 + 3 * (size_t)ng * 8 + 15) & ~(size_t)15) + 8 + (size_t)ng * ng * 8;
}
// ... and with the diagnostic scratch of `threads` threads
size_t fused_diag_smem_bytes(int ng, int threads) {
  return ((fused_smem_bytes(ng) + 15) & ~(size_t)15) + (size_t)(threads / 32 + 1) * kFusedDiagValues * 8;
}
int fused_threads(int ngrid, int threads) {
  if (threads < 2 * ngrid) threads = (2 * ngrid + 31) / 32 * 32;
  if (threads > kFusedMaxThreads) threads = kFusedMaxThreads;
  return threads;
}
bool fused_diag_fits(int ngrid, int threads, int nharm) {
  return nharm <= kFusedDiagHarm && fused_diag_smem_bytes(ngrid, fused_threads(ngrid, threads)) <= 227u * 1024u;
}

int fused_max_ngrid() {
  int ng = 3;
  while (fused_smem_bytes(ng + 1) <= 227u * 1024u) ng++;
  return ng;
}

void launch_field_fused_mixed(const Launch &L, const StepConstF &sc, int k, const DeviceBeam &b,
                              void *field, const void *coef, int ns, int np, int ngrid, int deposit,
                              int threads, double *dbeam, double *dfield, int nharm, double gref) {
  static std::atomic<unsigned long long> configured{0};  // one bit per device
  threads = fused_threads(ngrid, threads);
  size_t smem = (dbeam || dfield) ? fused_diag_smem_bytes(ngrid, threads) : fused_smem_bytes(ngrid);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured.load() & (1ull << dev))) {
    cudaFuncSetAttribute(k_field_fused_f, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    configured.fetch_or(1ull << dev);
  }
  PtrsF p = make_ptrs_f(b, nullptr, nullptr, 0);
  k_field_fused_f<<<ns, threads, smem, (cudaStream_t)L.stream>>>(
      sc, k, p, (float2 *)field, (const float2 *)coef, ns, np, ngrid, deposit, L.err, dbeam, dfield, nharm, gref);
}

void launch_source_substep_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b, const void *tp,
                                 const void *xp, const void *yp, float frac, float scale, void *field, int ns,
                                 int np, int ngrid) {
  PtrsF p = make_ptrs_f(b, nullptr, nullptr, 0);
  dim3 grid((np / 4 + 127) / 128, ns);
  k_source_f<<<grid, 128, 0, (cudaStream_t)L.stream>>>(sc, p, (const long long *)tp, (const float *)xp,
                                                        (const float *)yp, frac, scale, (float2 *)field, ns, np,
                                                        ngrid);
}

// k_step_fused_f's particles per lane and round (their loads in flight together) by
// CTA size: the register cap of 1024 threads (64) holds one particle's push, that of
// 768 threads (85) two, of 512 threads (128) four.
template <int U, int MAXT>
void launch_step_variant(cudaStream_t st, int threads, size_t smem, const StepConstF &sc, const PtrsF &p,
                         float2 *field, const float2 *coef, int ns, int np, int ng, int deposit, int *err,
                         double *dbeam, double *dfield, int nharm, double gref) {
  static std::atomic<unsigned long long> configured{0};  // one bit per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured.load() & (1ull << dev))) {
    cudaFuncSetAttribute(k_step_fused_f<U, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    configured.fetch_or(1ull << dev);
  }
  k_step_fused_f<U, MAXT><<<ns, threads, smem, st>>>(sc, p, field, coef, ns, np, ng, deposit, err, dbeam, dfield,
                                                       nharm, gref);
}

bool step_fused_ok(int nfield, int ngrid, int threads, bool dbeam, bool dfield, int nharm) {
  if (nfield != 1 || ngrid > fused_max_ngrid()) return false;
  if ((dbeam || dfield) && !fused_diag_fits(ngrid, threads, nharm)) return false;
  return true;
}

void launch_step_fused_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b, void *field,
                             const void *coef, int ns, int np, int ngrid, int deposit, int threads,
                             const void *wake, const IsrStream &isr, double *dbeam, double *dfield, int nharm,
                             double gref) {
  threads = fused_threads(ngrid, threads);
  const size_t smem = (dbeam || dfield) ? fused_diag_smem_bytes(ngrid, threads) : fused_smem_bytes(ngrid);
  void *const fld[1] = {field};
  PtrsF p = make_ptrs_f(b, fld, nullptr, 1);
  if (isr.ctr && (sc.isr_avg != 0 || sc.isr_sig != 0)) p.isr = isr;
  p.mode = 0;
  p.wake = (const float *)wake;
  cudaStream_t st = (cudaStream_t)L.stream;
  float2 *f = (float2 *)field;
  const float2 *cf = (const float2 *)coef;
  if (threads <= 512)
    launch_step_variant<4, 512>(st, threads, smem, sc, p, f, cf, ns, np, ngrid, deposit, L.err, dbeam, dfield,
                                nharm, gref);
  else if (threads <= 768)
    launch_step_variant<2, 768>(st, threads, smem, sc, p, f, cf, ns, np, ngrid, deposit, L.err, dbeam, dfield,
                                nharm, gref);
  else
    launch_step_variant<1, kFusedMaxThreads>(st, threads, smem, sc, p, f, cf, ns, np, ngrid, deposit, L.err,
                                             dbeam, dfield, nharm, gref);
}

int band_cluster(int ngrid, int W) {
  for (int cl = 2; cl <= kMaxBandCluster; cl++) {
    const int h = (ngrid + cl - 1) / cl, last = ngrid - (cl - 1) * h;
    if (band_smem_bytes(ngrid, cl) <= 227u * 1024u && last >= max(W, 2)) return cl;
  }
  return 0;
}

template <int CL>
static void launch_band(const Launch &L, const StepConstF &sc, int k, const PtrsF &p, void *field, const void *coef,
                        int ns, int np, int ngrid, int deposit) {
  static std::atomic<unsigned long long> configured{0};  // one bit per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(configured.load() & (1ull << dev))) {
    cudaFuncSetAttribute(k_field_band_f<CL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    configured.fetch_or(1ull << dev);
  }
  k_field_band_f<CL><<<CL * ns, band_threads<CL>(), band_smem_bytes(ngrid, CL), (cudaStream_t)L.stream>>>(
      sc, k, p, (float2 *)field, (const float2 *)coef, ns, np, ngrid, deposit, L.err);
}

void launch_field_band_mixed(const Launch &L, const StepConstF &sc, int k, const DeviceBeam &b, void *field,
                             const void *coef, int ns, int np, int ngrid, int deposit, int cl) {
  PtrsF p = make_ptrs_f(b, nullptr, nullptr, 0);
  if (cl == 2)
    launch_band<2>(L, sc, k, p, field, coef, ns, np, ngrid, deposit);
  else if (cl == 3)
    launch_band<3>(L, sc, k, p, field, coef, ns, np, ngrid, deposit);
  else
    launch_band<4>(L, sc, k, p, field, coef, ns, np, ngrid, deposit);
}

namespace {
// Per-device set-up of the no-allocation path: the device address of the scratch
// array, the kernel's shared-memory limit and the SM count, done by the first call
// on each device.
struct NoallocDevice {
  bool ready = false;
  unsigned char *scratch = nullptr;
  int nsm = 0;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];
}  // namespace

size_t noalloc_scratch_bytes() { return kNoallocScratchBytes; }

int adi_noalloc_mixed(int device, void *stream, void *field, const void *source, const float *coef,
                      float cstep, int ns, int ngrid, int first, std::string *msg) {
  if (device < 0 || device >= 64) {
    *msg = "device index outside [0, 64)";
    return G4GPU_ERR_ARG;
  }
  unsigned char *scratch;
  int nsm;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocDevice &d = g_noalloc_dev[device];
    if (!d.ready) {
      // host code names g4_noalloc_scratch only to look up its device address
      cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&d.scratch), g4_noalloc_scratch);
      if (e != cudaSuccess) {
        *msg = std::string("cudaGetSymbolAddress of the scratch array: ") + cudaGetErrorString(e);
        return G4GPU_ERR_CUDA;
      }
      e = cudaFuncSetAttribute(k_adi_noalloc_f, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, device);
      if (e != cudaSuccess) {
        *msg = std::string("set-up of the no-allocation kernel: ") + cudaGetErrorString(e);
        return G4GPU_ERR_CUDA;
      }
      d.ready = true;
    }
    scratch = d.scratch;
    nsm = d.nsm;
  }
  const size_t ncell = (size_t)ngrid * ngrid;
  const size_t slot_bytes = ((ncell + 2) * sizeof(float2) + 255) & ~(size_t)255;
  const size_t nslot = (kNoallocScratchBytes - kNoallocSlotOffset) / slot_bytes;
  if (nslot < 1 || 3 * (size_t)ngrid * sizeof(float2) > kNoallocSlotOffset - kNoallocCoefOffset) {
    *msg = "ngrid too large for the scratch array";
    return G4GPU_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the coefficients come from pageable host memory: the copy is staged before the
  // call returns, so the caller's buffer may go away afterwards
  cudaError_t e = cudaMemcpyAsync(scratch + kNoallocCoefOffset, coef, 3 * (size_t)ngrid * sizeof(float2),
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, sizeof(int), s);
  if (e != cudaSuccess) {
    *msg = std::string("scratch set-up copy: ") + cudaGetErrorString(e);
    return G4GPU_ERR_CUDA;
  }
  int grid = ns;
  if ((size_t)grid > nslot) grid = (int)nslot;
  if (nsm > 0 && grid > nsm) grid = nsm;
  int threads = 512;
  if (threads < 2 * ngrid) threads = (2 * ngrid + 31) / 32 * 32;
  if (threads > kFusedMaxThreads) threads = kFusedMaxThreads;
  k_adi_noalloc_f<<<grid, threads, fused_smem_bytes(ngrid), s>>>(
      (float2 *)field, (const float2 *)source, scratch, cstep, ns, ngrid, first, slot_bytes);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    *msg = std::string("k_adi_noalloc_f launch: ") + cudaGetErrorString(e);
    return G4GPU_ERR_CUDA;
  }
  int flag = 0;
  e = cudaMemcpyAsync(&flag, scratch, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *msg = std::string("k_adi_noalloc_f: ") + cudaGetErrorString(e);
    return G4GPU_ERR_CUDA;
  }
  if (flag != 0) {
    *msg = "device error flag raised (code " + std::to_string(flag) + ")";
    return G4GPU_ERR_DEVICE;
  }
  return G4GPU_OK;
}

}  // namespace g4
