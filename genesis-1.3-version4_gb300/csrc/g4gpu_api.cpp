// Host implementation of the C ABI in include/g4gpu.h: handle lifetime, device
// memory, per-step constants, the step sequence and the slippage bookkeeping.
//
// The step sequence replaces the body of the reference's step loop
// (src/Core/Gencore.cpp:102-147) for one time window held in GPU memory:
//   push      Beam::track                      -> one fused kernel (+ deposition)
//   field     Field::track of every field       -> deposition + ADI (or FFT) kernels
//   slippage  Control::applySlippage            -> ring-start bookkeeping on the host
//                                                  and a clear of the entering slice
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <utility>
#include <vector>

#include "g4gpu.h"
#include "g4gpu_ctx.h"
#include "g4gpu_internal.h"

using g4::StepConst;

namespace g4 {
// kernels_util.cu
void launch_aos_to_soa(void *stream, const double *aos, void *const *soa, int mixed, double gref,
                       size_t n);
void launch_soa_to_aos(void *stream, const void *const *soa, double *aos, int mixed, double gref,
                       size_t n);
void launch_convert_field(void *stream, const void *in, void *out, size_t n, int to_float);
}

namespace {

std::mutex g_err_mu;
std::string g_create_err;

int fail(g4gpu_handle h, int code, const std::string &msg) {
  if (h) {
    h->err = msg;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
  }
  return code;
}

int cuda_fail(g4gpu_handle h, cudaError_t e, const char *what) {
  return fail(h, e == cudaErrorMemoryAllocation ? G4GPU_ERR_NOMEM : G4GPU_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define G4_CUDA(h, call)                            \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

cudaEvent_t take_event(g4gpu_handle h) {
  if (!h->pool.empty()) {
    cudaEvent_t e = h->pool.back();
    h->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// Brackets one kernel launch for accounting.
struct Timed {
  g4gpu_handle h;
  int cls;
  cudaEvent_t a = nullptr, b = nullptr;
  Timed(g4gpu_handle h_, int cls_, int kernels = 1) : h(h_), cls(cls_) {
    h->launches[cls] += kernels;
    if (h->prof && !h->capturing) {
      a = take_event(h);
      b = take_event(h);
      cudaEventRecord(a, h->stream);
    }
  }
  ~Timed() {
    if (h->prof && a) {
      cudaEventRecord(b, h->stream);
      h->pending.push_back({cls, a, b});
    }
  }
};

void collect_events(g4gpu_handle h) {
  if (h->pending.empty()) return;
  cudaStreamSynchronize(h->stream);
  for (auto &p : h->pending) {
    float t = 0;
    cudaEventElapsedTime(&t, p.a, p.b);
    h->ms[p.cls] += t;
    h->pool.push_back(p.a);
    h->pool.push_back(p.b);
  }
  h->pending.clear();
}

int check_device_flag(g4gpu_handle h) {
  int v = 0;
  G4_CUDA(h, cudaMemcpyAsync(&v, h->derr, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  if (v != 0) {
    char buf[128];
    snprintf(buf, sizeof(buf), "device error flag raised (code %d)", v);
    return fail(h, G4GPU_ERR_DEVICE, buf);
  }
  return G4GPU_OK;
}

int alloc(g4gpu_handle h, void **p, size_t n) {
  cudaError_t e = cudaMalloc(p, n);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc");
  h->bytes += n;
  return G4GPU_OK;
}

// ADI coefficients of FieldSolverADI::init (src/Core/FieldSolverADI.cpp:125-182),
// computed with std::complex<double> exactly as the reference does.
void adi_coefficients(double delz, double dgrid, double xks, int ngrid, std::vector<std::complex<double>> &c,
                      std::vector<std::complex<double>> &cbet, std::vector<std::complex<double>> &cwet,
                      double *cstep_im) {
  typedef std::complex<double> cd;
  double rtmp = 0.25 * delz / (xks * dgrid * dgrid);
  *cstep_im = rtmp;
  std::vector<double> mupp(ngrid), mmid(ngrid), mlow(ngrid);
  std::vector<cd> w1(ngrid), w2(ngrid);
  c.assign(ngrid, 0);
  cbet.assign(ngrid, 0);
  cwet.assign(ngrid, 0);
  mupp[0] = rtmp;
  mmid[0] = -2 * rtmp;
  mlow[0] = 0;
  for (int i = 1; i < ngrid - 1; i++) {
    mupp[i] = rtmp;
    mmid[i] = -2 * rtmp;
    mlow[i] = rtmp;
  }
  mupp[ngrid - 1] = 0;
  mmid[ngrid - 1] = -2 * rtmp;
  mlow[ngrid - 1] = rtmp;
  for (int i = 0; i < ngrid; i++) {
    w1[i] = cd(0, -mupp[i]);
    w2[i] = cd(1, -mmid[i]);
    c[i] = cd(0, -mlow[i]);
  }
  cbet[0] = 1. / w2[0];
  cwet[0] = 0.;
  for (int i = 1; i < ngrid; i++) {
    cwet[i] = w1[i - 1] * cbet[i - 1];
    cbet[i] = 1. / (w2[i] - c[i] * cwet[i]);
  }
}

// Warm-up length of the segmented tridiagonal solve for one coefficient set. Both
// recurrences of the Thomas algorithm, d_k = (r_k - c_k d_{k-1}) cbet_k forward and
// x_k = d_k - cwet_{k+1} x_{k+1} backward, forget their starting value by the factor
// |c_k cbet_k| or |cwet_k| per element (about the step factor dz / (4 xks dgrid^2),
// a few percent on the grids of these runs). A line can then be split into segments
// solved in parallel, each started W elements early from zero: the error is below
// alpha^W <= 2^-bits of the solution (bits = 32 for the FP32 solves), under the
// form's rounding. Returns 0 when alpha is too large for a short warm-up (the solves
// then run one thread per line).
int segment_warmup(const std::vector<std::complex<double>> &c, const std::vector<std::complex<double>> &cbet,
                   const std::vector<std::complex<double>> &cwet, int bits) {
  double alpha = 0;
  for (size_t k = 0; k < c.size(); k++) alpha = std::max(alpha, std::max(std::abs(c[k] * cbet[k]), std::abs(cwet[k])));
  if (!(alpha < 0.5)) return 0;
  if (alpha <= 0) return 1;
  int w = (int)std::ceil(std::log(std::ldexp(1.0, -bits)) / std::log(alpha));
  if (w < 1) w = 1;
  return w <= 2 * bits / 3 ? w : 0;
}

// FieldSolverFFT::init (src/Core/FieldSolverFFT.cpp:117-155): the propagator
// exponent Im(K2) and the source filter on the shifted frequency map, per field,
// plus the n-th roots of unity and the prime factors of ngrid for the kernels.
int fft_tables(g4gpu_handle h) {
  const g4gpu_config &c = h->cfg;
  int n = c.ngrid;
  g4::FFTPlan &pl = h->fft_plan;
  pl.n = n;
  pl.nstage = 0;
  // radices of the register butterflies: the factors of two as 16s (then one 8, 4
  // or 2), threes paired with fives (15), the other threes as 9s (then one 3), the
  // other fives; any further prime factors in ascending order
  int m = n, twos = 0, threes = 0, fives = 0;
  for (; m % 2 == 0; m /= 2) twos++;
  for (; m % 3 == 0; m /= 3) threes++;
  for (; m % 5 == 0; m /= 5) fives++;
  for (; twos >= 4; twos -= 4) pl.radix[pl.nstage++] = 16;
  if (twos > 0) pl.radix[pl.nstage++] = twos == 3 ? 8 : (twos == 2 ? 4 : 2);
  for (; threes > 0 && fives > 0; threes--, fives--) pl.radix[pl.nstage++] = 15;
  for (; threes >= 2; threes -= 2) pl.radix[pl.nstage++] = 9;
  if (threes > 0) pl.radix[pl.nstage++] = 3;
  for (; fives > 0; fives--) pl.radix[pl.nstage++] = 5;
  for (int p = 7; p * p <= m; p += 2)
    while (m % p == 0 && pl.nstage < 31) {
      pl.radix[pl.nstage++] = p;
      m /= p;
    }
  if (m > 1) pl.radix[pl.nstage++] = m;
  // the n roots exp(-2 pi i m / n), then per stage the twiddles exp(-2 pi i q k / (ns R))
  const double two_pi = 2.0 * 3.14159265358979323846;
  std::vector<double> roots(2 * (2 * n - 1));
  for (int i = 0; i < n; i++) {
    double a = two_pi * (double)i / (double)n;
    roots[2 * i] = std::cos(a);
    roots[2 * i + 1] = -std::sin(a);
  }
  int off = 0, nsp = 1;
  auto magic = [](int d) { return d <= 1 ? 0u : (unsigned)((((unsigned long long)1 << 32) + d - 1) / d); };
  pl.mn = magic(n);
  for (int s = 0; s < pl.nstage; s++) {
    const int r = pl.radix[s];
    pl.tw_off[s] = off;
    pl.nb[s] = n / r;
    pl.mnb[s] = magic(n / r);
    pl.mns[s] = magic(nsp);
    if (nsp > 1)
      for (int q = 1; q < r; q++)
        for (int kk = 0; kk < nsp; kk++) {
          double a = two_pi * (double)(q * kk) / (double)(nsp * r);
          roots[2 * (n + off)] = std::cos(a);
          roots[2 * (n + off) + 1] = -std::sin(a);
          off++;
        }
    nsp *= r;
  }
  double xc = c.xcut, yc = c.ycut, sig = c.sigmoid;
  for (int k = 0; k < c.nfield; k++) {
    double xlambda = c.lambda0 / static_cast<double>(c.harm[k]);
    double xks = 4. * std::asin(1) / xlambda;
    double dgrid = 2 * c.gridmax[k] / static_cast<double>(n - 1);
    double dk = 4. * std::asin(1.) / (static_cast<double>(n) * dgrid);
    std::vector<double> sg((size_t)n * n);
    h->fft_k2c[k] = -dk * dk / 2. / xks;
    double shift = -0.5 * static_cast<double>(n - 1);
    for (int iy = 0; iy < n; iy++) {
      double dy = static_cast<double>(iy) + shift;
      double y = dy / static_cast<double>(n) / yc;
      for (int ix = 0; ix < n; ix++) {
        double dx = static_cast<double>(ix) + shift;
        double x = dx / static_cast<double>(n) / xc;
        int iiy = (iy + (n + 1) / 2) % n, iix = (ix + (n + 1) / 2) % n;
        // stored transposed (kx major) for the column pass
        size_t ii = (size_t)iix * n + iiy;
        double r = (std::sqrt(x * x + y * y) - 1) / sig;
        sg[ii] = 1. / (1 + std::exp(r));
      }
    }
    size_t es = h->mixed ? sizeof(float) : sizeof(double);
    int rc;
    if ((rc = alloc(h, &h->fft_roots[k], roots.size() * es))) return rc;
    if ((rc = alloc(h, &h->fft_sig[k], (size_t)n * n * es))) return rc;
    auto put = [&](void *dst, const std::vector<double> &v) -> int {
      if (h->mixed) {
        std::vector<float> f(v.begin(), v.end());
        return cudaMemcpy(dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
      }
      return cudaMemcpy(dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
    };
    if (put(h->fft_roots[k], roots) || put(h->fft_sig[k], sg))
      return fail(h, G4GPU_ERR_CUDA, "copy of the FFT tables failed");
  }
  return G4GPU_OK;
}

}  // namespace

int g4_fail(g4gpu_handle h, int code, const std::string &msg) { return fail(h, code, msg); }
int g4_cuda_fail(g4gpu_handle h, cudaError_t e, const char *what) { return cuda_fail(h, e, what); }
int g4_alloc(g4gpu_handle h, void **p, size_t n) { return alloc(h, p, n); }
int g4_check_device_flag(g4gpu_handle h) { return check_device_flag(h); }

extern "C" {

void g4gpu_config_defaults(g4gpu_config *cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->nslice = 1;
  cfg->npart = 8192;  // Setup.cpp: npart
  cfg->ngrid = 151;   // LoadField.cpp: ngrid
  cfg->nfield = 1;
  cfg->harm[0] = 1;
  cfg->gridmax[0] = 1e-3;  // LoadField.cpp: dgrid
  cfg->lambda0 = 1e-10;    // Setup.cpp: lambda0
  cfg->sample = 1;
  cfg->gammaref = 5800 / 0.511;  // Setup.cpp:19 gamma0
  cfg->precision = G4GPU_PLAIN;
  cfg->solver = G4GPU_SOLVER_ADI;
  cfg->xcut = cfg->ycut = cfg->sigmoid = 1;  // Track.cpp:73-75
  cfg->time_run = 0;
  cfg->periodic = 0;
  cfg->device = 0;
}

const char *g4gpu_last_error(g4gpu_handle h) {
  if (h) return h->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_create_err.c_str();
}

int g4gpu_create(const g4gpu_config *cfg, g4gpu_handle *out) {
  if (!cfg || !out) return fail(nullptr, G4GPU_ERR_ARG, "null argument");
  *out = nullptr;
  const g4gpu_config &c = *cfg;
  if (c.nslice < 1 || c.npart < 1 || c.ngrid < 3 || c.nfield < 1 || c.nfield > G4GPU_MAX_FIELDS)
    return fail(nullptr, G4GPU_ERR_ARG, "nslice, npart >= 1, ngrid >= 3, 1 <= nfield <= 8 required");
  if (c.precision != G4GPU_PLAIN && c.precision != G4GPU_MIXED)
    return fail(nullptr, G4GPU_ERR_ARG, "unknown precision");
  if (c.solver != G4GPU_SOLVER_ADI && c.solver != G4GPU_SOLVER_FFT)
    return fail(nullptr, G4GPU_ERR_ARG, "unknown solver");
  for (int k = 0; k < c.nfield; k++)
    if (c.harm[k] < 1 || !(c.gridmax[k] > 0))
      return fail(nullptr, G4GPU_ERR_ARG, "harm >= 1 and gridmax > 0 required for every field");
  if (!(c.lambda0 > 0) || !(c.sample > 0) || !(c.gammaref > 1))
    return fail(nullptr, G4GPU_ERR_ARG, "lambda0 > 0, sample > 0 and gammaref > 1 required");
  if ((long long)c.ngrid * c.ngrid > (1LL << 30))
    return fail(nullptr, G4GPU_ERR_ARG, "ngrid too large");

  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, G4GPU_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (c.device < 0 || c.device >= ndev) return fail(nullptr, G4GPU_ERR_ARG, "device ordinal out of range");

  g4gpu_handle h = new g4gpu_ctx;
  h->cfg = c;
  h->mixed = c.precision == G4GPU_MIXED;
  h->csize = h->mixed ? 8 : 16;
  h->rsize = h->mixed ? 4 : 8;
  int rc = G4GPU_OK;
  auto bail = [&](int code) {
    g_create_err = h->err;
    g4gpu_destroy(h);
    return code;
  };
  if ((e = cudaSetDevice(c.device)) != cudaSuccess) return bail(cuda_fail(h, e, "cudaSetDevice"));
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(h, e, "cudaStreamCreate"));

  size_t np = (size_t)c.nslice * c.npart;
  size_t ncell = (size_t)c.ngrid * c.ngrid;
  void **coords[5] = {&h->beam.gamma, &h->beam.x, &h->beam.y, &h->beam.px, &h->beam.py};
  for (auto p : coords)
    if ((rc = alloc(h, p, np * h->rsize))) return bail(rc);
  if ((rc = alloc(h, &h->beam.theta, np * sizeof(double)))) return bail(rc);
  if (!h->mixed) {
    if ((rc = alloc(h, &h->beam.phasor, (size_t)c.nfield * np * 16))) return bail(rc);
    if ((rc = alloc(h, (void **)&h->beam.phasor_ok, sizeof(int)))) return bail(rc);
    cudaMemsetAsync(h->beam.phasor_ok, 0, sizeof(int), h->stream);
  }
  if ((rc = alloc(h, (void **)&h->beam.current, c.nslice * sizeof(double)))) return bail(rc);
  // the fused mixed ADI kernel keeps the source and the intermediate on chip: no
  // source or intermediate arrays
  const bool fused = h->mixed && c.solver == G4GPU_SOLVER_ADI && c.ngrid <= g4::fused_max_ngrid();
  for (int k = 0; k < c.nfield; k++) {
    if ((rc = alloc(h, &h->field[k], (size_t)c.nslice * ncell * h->csize))) return bail(rc);
    cudaMemsetAsync(h->field[k], 0, (size_t)c.nslice * ncell * h->csize, h->stream);
    if (fused) continue;
    if ((rc = alloc(h, &h->src[k], (size_t)c.nslice * ncell * h->csize))) return bail(rc);
    cudaMemsetAsync(h->src[k], 0, (size_t)c.nslice * ncell * h->csize, h->stream);
  }
  if (!fused && (rc = alloc(h, &h->tmp, (size_t)c.nslice * ncell * h->csize))) return bail(rc);
  if (c.solver == G4GPU_SOLVER_FFT) {
    if (c.ngrid > g4::fft_max_ngrid(h->mixed))
      return bail(fail(h, G4GPU_ERR_ARG, "ngrid too large for the FFT solver"));
    if ((rc = fft_tables(h))) return bail(rc);
    if (!g4::fft_plan_fits(h->fft_plan))
      return bail(fail(h, G4GPU_ERR_ARG,
                       "ngrid " + std::to_string(c.ngrid) +
                           ": a stage of its FFT plan has more than 256 butterflies per line"));
  }
  if ((rc = alloc(h, (void **)&h->derr, sizeof(int)))) return bail(rc);
  cudaMemsetAsync(h->derr, 0, sizeof(int), h->stream);
  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return bail(cuda_fail(h, e, "init"));
  *out = h;
  return G4GPU_OK;
}

void g4gpu_destroy(g4gpu_handle h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void *ptrs[] = {h->beam.gamma, h->beam.theta, h->beam.x, h->beam.y, h->beam.px, h->beam.py,
                  h->beam.current, h->tmp, h->diag_work, h->coef, h->derr, h->ddiag, h->stage,
                  h->closure_basis, h->closure_feat, h->closure_corr, h->sc.st, h->sc.state, h->sc.ez,
                  h->wake_tab, h->wake_loss, h->wake_lossf, h->wake_scratch, h->count_buf, h->sort_iscratch,
                  h->sort_scratch[0], h->sort_scratch[1], h->sort_scratch[2], h->sort_scratch[3],
                  h->sort_scratch[4], h->sort_scratch[5], h->isr_ctr, h->sub_theta, h->sub_x, h->sub_y,
                  h->beam.phasor, h->beam.phasor_ok};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  for (int k = 0; k < G4GPU_MAX_FIELDS; k++) {
    void *fp[] = {h->field[k], h->src[k], h->fft_roots[k], h->fft_sig[k]};
    for (void *p : fp)
      if (p) cudaFree(p);
  }
  for (auto &p : h->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto ev : h->pool) cudaEventDestroy(ev);
  if (h->hdiag) cudaFreeHost(h->hdiag);
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int g4gpu_set_lattice(g4gpu_handle h, int nsteps, const double *tab) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (nsteps < 0 || (nsteps > 0 && !tab)) return fail(h, G4GPU_ERR_ARG, "bad lattice table");
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  int ng = c.ngrid;
  h->steps.assign(nsteps, StepConst{});
  h->slip.assign(nsteps, 0.0);
  h->substeps.clear();
  typedef std::complex<double> cd;
  std::map<std::pair<int, double>, int> sets;  // (field, delz) -> set
  std::vector<cd> coefs;                       // [nset][3][ng]
  std::vector<int> set_tw;                     // warm-up length per coefficient set
  for (int i = 0; i < nsteps; i++) {
    const double *r = tab + (size_t)i * G4GPU_LAT_NCOL;
    StepConst &s = h->steps[i];
    double aw = r[G4GPU_LAT_AW];
    bool inund = aw > 0;  // Undulator::inUndulator, Undulator.h:141-146
    double gamma0 = c.gammaref;
    // TrackBeam::track, TrackBeam.cpp:17-64
    double awt = inund ? aw : 0, dax = inund ? r[G4GPU_LAT_AX] : 0, day = inund ? r[G4GPU_LAT_AY] : 0;
    double kxt = inund ? r[G4GPU_LAT_KX] : 0, kyt = inund ? r[G4GPU_LAT_KY] : 0;
    double qf = r[G4GPU_LAT_QF];
    double dqx = qf == 0 ? 0 : r[G4GPU_LAT_QX], dqy = qf == 0 ? 0 : r[G4GPU_LAT_QY];
    double betpar0 = std::sqrt(1 - (1 + awt * awt) / gamma0 / gamma0);
    double qquad = qf * gamma0;
    double qnatx = kxt * awt * awt / gamma0 / betpar0;
    double qnaty = kyt * awt * awt / gamma0 / betpar0;
    double qx = qquad + qnatx, qy = -qquad + qnaty;
    double xoff = qquad * dqx + qnatx * dax, yoff = -qquad * dqy + qnaty * day;
    s.aw_t = awt;
    s.qx = qx;
    s.qy = qy;
    if (qx == 0) {
      s.kindx = 0;
      s.xoff = xoff;
    } else {
      s.xoff = xoff / qx;
      s.kindx = qx > 0 ? 1 : 2;
    }
    if (qy == 0) {
      s.kindy = 0;
      s.yoff = yoff;
    } else {
      s.yoff = yoff / qy;
      s.kindy = qy > 0 ? 1 : 2;
    }
    double cx = r[G4GPU_LAT_CX], cy = r[G4GPU_LAT_CY];
    s.cxk = cx * gamma0;
    s.cyk = cy * gamma0;
    s.corr = (cx != 0) || (cy != 0);
    // BeamSolver::advance, BeamSolver.cpp:19-41
    s.aw = aw;
    s.ax = r[G4GPU_LAT_AX];
    s.ay = r[G4GPU_LAT_AY];
    s.kx = r[G4GPU_LAT_KX];
    s.ky = r[G4GPU_LAT_KY];
    s.gradx = r[G4GPU_LAT_GRADX];
    s.grady = r[G4GPU_LAT_GRADY];
    s.autophase = r[G4GPU_LAT_PHASE];
    s.delz = r[G4GPU_LAT_DZ];
    s.ku_raw = r[G4GPU_LAT_KU];
    s.helical = r[G4GPU_LAT_HELICAL] != 0;
    s.gammaref = gamma0;
    s.nfld = c.nfield;
    int helical = r[G4GPU_LAT_HELICAL] != 0;
    double xks = 1;
    for (int k = 0; k < c.nfield; k++) {
      int harm = c.harm[k];
      double xlambda = c.lambda0 / static_cast<double>(harm);  // Field.cpp:42
      double fxks = 4. * std::asin(1) / xlambda;                // Field.cpp:65
      double fc = g4::host_fc(aw, helical, harm);
      xks = fxks / static_cast<double>(harm);
      g4::FieldStep &f = s.f[k];
      f.rtmp = fc / fxks;
      f.rharm = static_cast<double>(harm);
      f.fc = fc;
      f.xks = fxks;
      f.gridmax = c.gridmax[k];
      f.dgrid = 2 * c.gridmax[k] / static_cast<double>(ng - 1);  // Field.cpp:46
      f.dep_on = inund && (harm % 2 == 1);
      double dk = 4. * std::asin(1.) / (static_cast<double>(ng) * f.dgrid);
      f.k2scale = dk * dk / 2. / fxks;
      auto key = std::make_pair(k, s.delz);
      auto it = sets.find(key);
      if (it == sets.end()) {
        std::vector<cd> cc, cb, cw;
        double cs;
        adi_coefficients(s.delz, f.dgrid, fxks, ng, cc, cb, cw, &cs);
        int id = static_cast<int>(sets.size());
        sets[key] = id;
        coefs.insert(coefs.end(), cc.begin(), cc.end());
        coefs.insert(coefs.end(), cb.begin(), cb.end());
        coefs.insert(coefs.end(), cw.begin(), cw.end());
        set_tw.push_back(segment_warmup(cc, cb, cw, 32));
        it = sets.find(key);
      }
      f.coef = it->second;
      f.tw = set_tw[it->second];
      f.cstep = 0.25 * s.delz / (fxks * f.dgrid * f.dgrid);
    }
    s.xks = xks;
    s.xku = r[G4GPU_LAT_KU];
    if (s.xku == 0) s.xku = xks * 0.5 / gamma0 / gamma0;  // BeamSolver.cpp:34-38
    s.ztemp1 = -2. / s.xks;
    s.half_delz = s.delz * 0.5;
    s.aw_t2 = s.aw_t * s.aw_t;
    s.aw2 = s.aw * s.aw;
    {
      // dtheta/dz of the ODE (BeamSolver.cpp:144-163) at gammaref, on axis, no field
      const double bpar = std::sqrt(1. - (1. + aw * aw) / (gamma0 * gamma0));
      const double rate = s.xks * (1. - 1. / bpar) + s.xku;
      s.dnom_half = 0.5 * s.delz * rate;
      s.dnom_full = s.delz * rate;
      for (int k = 0; k < c.nfield; k++) {
        g4::FieldStep &f = s.f[k];
        f.idgrid = 1. / f.dgrid;
        f.gm_idg = f.gridmax * f.idgrid;
        f.rot_half[0] = std::cos(f.rharm * s.dnom_half);
        f.rot_half[1] = std::sin(f.rharm * s.dnom_half);
        f.rot_full[0] = std::cos(f.rharm * s.dnom_full);
        f.rot_full[1] = std::sin(f.rharm * s.dnom_full);
        f.rot_auto[0] = std::cos(f.rharm * s.autophase);
        f.rot_auto[1] = std::sin(f.rharm * s.autophase);
      }
    }
    h->slip[i] = r[G4GPU_LAT_SLIP];
  }
  h->nsteps = nsteps;
  // captured step sequences hold the previous lattice's constants
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  h->graphs.clear();
  h->graph_gen++;
  if (h->coef) {
    cudaFree(h->coef);
    h->bytes -= h->coef_bytes;
    h->coef = nullptr;
    h->coef_bytes = 0;
  }
  if (!coefs.empty()) {
    size_t n = coefs.size();
    int rc = alloc(h, &h->coef, n * h->csize);
    if (rc) return rc;
    h->coef_bytes = n * h->csize;
    if (h->mixed) {
      std::vector<float> fl(2 * n);
      for (size_t i = 0; i < n; i++) {
        fl[2 * i] = static_cast<float>(coefs[i].real());
        fl[2 * i + 1] = static_cast<float>(coefs[i].imag());
      }
      G4_CUDA(h, cudaMemcpy(h->coef, fl.data(), fl.size() * sizeof(float), cudaMemcpyHostToDevice));
    } else {
      G4_CUDA(h, cudaMemcpy(h->coef, coefs.data(), n * sizeof(cd), cudaMemcpyHostToDevice));
    }
  }
  return G4GPU_OK;
}

namespace {
// TrackBeam::matmul (TrackBeam.cpp:246-258): m = e m
void chicane_matmul(double m[4][4], const double e[4][4]) {
  double t[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      t[i][j] = 0;
      for (int k = 0; k < 4; k++) t[i][j] += e[i][k] * m[k][j];
    }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) m[i][j] = t[i][j];
}

// The transfer matrix of TrackBeam::applyChicane (TrackBeam.cpp:131-222): bend, edge,
// drift, edge, bend, middle drift, bend, edge, drift, edge, bend, then a drift back over
// the chicane's length, which the step's two half steps add again
void chicane_matrix(double angle, double lb, double ld, double lt, double m[4][4]) {
  double d1[4][4], d2[4][4], d3[4][4], bp[4][4], bn[4][4], ep[4][4], en[4][4];
  double *all[] = {&m[0][0], &d1[0][0], &d2[0][0], &d3[0][0], &bp[0][0], &bn[0][0], &ep[0][0], &en[0][0]};
  for (double *a : all)
    for (int i = 0; i < 16; i++) a[i] = (i % 5 == 0) ? 1 : 0;
  d1[0][1] = d1[2][3] = ld / std::cos(angle);
  d2[0][1] = d2[2][3] = lt - 4 * lb - 2 * ld;
  d3[0][1] = d3[2][3] = -lt;
  const double R = lb / std::sin(angle), L = R * angle;
  bp[2][3] = L;
  bp[0][0] = std::cos(angle);
  bp[0][1] = R * std::sin(angle);
  bp[1][0] = -std::sin(angle) / R;
  bp[1][1] = std::cos(angle);
  bn[2][3] = L;
  bn[0][0] = std::cos(-angle);
  bn[0][1] = R * std::sin(-angle) * -1;
  bn[1][0] = -std::sin(-angle) / R * -1;
  bn[1][1] = std::cos(-angle);
  const double efoc = std::tan(angle) / R;
  ep[1][0] = efoc;
  ep[3][2] = -efoc;
  en[1][0] = -efoc * -1;
  en[3][2] = efoc * -1;
  const double(*seq[])[4] = {bp, ep, d1, en, bn, d2, bn, en, d1, ep, bp, d3};
  for (auto e : seq) chicane_matmul(m, e);
}
}  // namespace

int g4gpu_set_incoherent(g4gpu_handle h, int seed, int do_loss, int do_spread, int nbins) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (nbins < 1) return fail(h, G4GPU_ERR_ARG, "nbins must be at least 1");
  cudaSetDevice(h->cfg.device);
  if (!h->isr_ctr) {
    int rc = alloc(h, (void **)&h->isr_ctr, sizeof(unsigned long long));
    if (rc) return rc;
  }
  // a new stream: the counter of drawing steps restarts
  G4_CUDA(h, cudaMemsetAsync(h->isr_ctr, 0, sizeof(unsigned long long), h->stream));
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  h->isr_loss = do_loss != 0;
  h->isr_spread = do_spread != 0;
  h->isr_seed = (unsigned)seed;
  h->isr_nbins = nbins;
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  h->graphs.clear();
  h->graph_gen++;
  return G4GPU_OK;
}

int g4gpu_set_field_substeps(g4gpu_handle h, int nsteps, const int *counts) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (nsteps != h->nsteps || (nsteps > 0 && !counts))
    return fail(h, G4GPU_ERR_ARG, "the sub-step counts need one entry per lattice step");
  const g4gpu_config &c = h->cfg;
  bool any = false;
  for (int i = 0; i < nsteps; i++) any = any || counts[i] > 1;
  if (any && !(h->mixed && c.nfield == 1 && c.solver == G4GPU_SOLVER_ADI && c.ngrid <= g4::fused_max_ngrid() &&
               c.npart % 4 == 0 && !h->beam.count && !h->sc_on))
    return fail(h, G4GPU_ERR_ARG,
                "coarse steps need the mixed form, one field, the ADI solver, ngrid <= 168, npart a multiple "
                "of 4, full slices and no space charge");
  cudaSetDevice(c.device);
  const size_t n = (size_t)c.nslice * c.npart;
  if (any && !h->sub_theta) {
    int rc = alloc(h, &h->sub_theta, n * 8);
    if (!rc) rc = alloc(h, &h->sub_x, n * 4);
    if (!rc) rc = alloc(h, &h->sub_y, n * 4);
    if (rc) return rc;
  }
  h->substeps.assign(counts, counts + nsteps);
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  h->graphs.clear();
  h->graph_gen++;
  return G4GPU_OK;
}

int g4gpu_set_chicanes(g4gpu_handle h, int nsteps, const double *table) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (nsteps != h->nsteps || (nsteps > 0 && !table))
    return fail(h, G4GPU_ERR_ARG, "the chicane table needs one row per lattice step");
  for (int i = 0; i < nsteps; i++) {
    const double *r = table + 4 * (size_t)i;
    g4::StepConst &s = h->steps[i];
    const double angle = r[0], lb = r[1], ld = r[2], lt = r[3];
    s.chic = angle != 0;
    if (!s.chic) continue;
    if (!(lb > 0) || !std::isfinite(angle) || std::fabs(angle) >= 2 * std::asin(1.0) / 2)
      return fail(h, G4GPU_ERR_ARG, "chicane rows need lb > 0 and |angle| below pi / 2");
    double m[4][4];
    chicane_matrix(angle, lb, ld, lt, m);
    const double cm[8] = {m[0][0], m[0][1], m[1][0], m[1][1], m[2][2], m[2][3], m[3][2], m[3][3]};
    std::copy(cm, cm + 8, s.cm);
    // TrackBeam::applyR56 (TrackBeam.cpp:265-268)
    double r56 = (4 * lb / std::sin(angle) * (1 - angle / std::tan(angle)) + 2 * ld * std::tan(angle) /
                  std::cos(angle)) * angle;
    s.r56 = r56 * 4 * std::asin(1) / h->cfg.lambda0 / h->cfg.gammaref;
  }
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  h->graphs.clear();
  h->graph_gen++;
  return G4GPU_OK;
}

// The FP64 push's cached phasors no longer match theta (a load, a sort, a restored state)
static void phasor_stale(g4gpu_handle h) {
  if (h->beam.phasor_ok) cudaMemsetAsync(h->beam.phasor_ok, 0, sizeof(int), h->stream);
}

static int ensure_stage(g4gpu_handle h, size_t n) {
  if (h->stage_bytes >= n) return G4GPU_OK;
  if (h->stage) {
    cudaFree(h->stage);
    h->bytes -= h->stage_bytes;
    h->stage = nullptr;
    h->stage_bytes = 0;
  }
  int rc = alloc(h, &h->stage, n);
  if (rc == G4GPU_OK) h->stage_bytes = n;
  return rc;
}

// Collective::update on the device: the slices' wake loss from the current
static int wake_update(g4gpu_handle h) {
  const int ns = h->cfg.nslice, nw = h->wake_ns;
  g4::Launch L{h->stream, h->derr};
  {
    Timed t(h, G4GPU_K_MISC, 2);
    g4::launch_wake_update(L, h->beam.current, ns, nw, h->wake_ds, h->wake_tab + 3 * (size_t)nw, h->wake_tab,
                           h->wake_tab + nw, h->wake_tab + 2 * (size_t)nw, h->wake_scratch, h->wake_loss,
                           h->wake_lossf);
  }
  G4_CUDA(h, cudaGetLastError());
  return G4GPU_OK;
}

static void drop_graphs(g4gpu_handle h) {
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  h->graphs.clear();
  h->graph_gen++;
}

int g4gpu_load_beam(g4gpu_handle h, const double *particles, const double *current) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!particles || !current) return fail(h, G4GPU_ERR_ARG, "null particles or current");
  cudaSetDevice(h->cfg.device);
  // every slice holds npart: the kernels take the fixed layout (captured graphs hold the
  // counts' pointer)
  if (h->beam.count) {
    h->beam.count = nullptr;
    h->hcount.clear();
    drop_graphs(h);
  }
  size_t n = (size_t)h->cfg.nslice * h->cfg.npart;
  int rc = ensure_stage(h, n * 6 * sizeof(double));
  if (rc) return rc;
  G4_CUDA(h, cudaMemcpyAsync(h->stage, particles, n * 6 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  G4_CUDA(h, cudaMemcpyAsync(h->beam.current, current, h->cfg.nslice * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream));
  void *soa[6] = {h->beam.gamma, h->beam.theta, h->beam.x, h->beam.y, h->beam.px, h->beam.py};
  {
    Timed t(h, G4GPU_K_MISC);
    g4::launch_aos_to_soa(h->stream, (const double *)h->stage, soa, h->mixed, h->cfg.gammaref, n);
  }
  phasor_stale(h);
  G4_CUDA(h, cudaGetLastError());
  h->beam_loaded = true;
  // the wake of every slice follows the window's current
  if (h->wake_on) return wake_update(h);
  return G4GPU_OK;
}

int g4gpu_load_beam_counts(g4gpu_handle h, const double *particles, const double *current, const int *counts) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!counts) return fail(h, G4GPU_ERR_ARG, "null counts");
  const g4gpu_config &c = h->cfg;
  for (int is = 0; is < c.nslice; is++)
    if (counts[is] < 0 || counts[is] > c.npart)
      return fail(h, G4GPU_ERR_ARG, "counts must lie in [0, npart] (npart is a slice's capacity)");
  if (h->mixed && std::fabs(c.sample - std::nearbyint(c.sample)) > 0)
    return fail(h, G4GPU_ERR_ARG, "one4one windows in the mixed form need an integer sample");
  int rc = g4gpu_load_beam(h, particles, current);
  if (rc) return rc;
  if (!h->count_buf && (rc = alloc(h, (void **)&h->count_buf, c.nslice * sizeof(int)))) return rc;
  G4_CUDA(h, cudaMemcpyAsync(h->count_buf, counts, c.nslice * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  h->hcount.assign(counts, counts + c.nslice);
  h->beam.count = h->count_buf;
  drop_graphs(h);
  // the wake follows the current (computed by g4gpu_load_beam already)
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  return G4GPU_OK;
}

int g4gpu_get_counts(g4gpu_handle h, int *counts) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!counts) return fail(h, G4GPU_ERR_ARG, "null counts");
  for (int is = 0; is < h->cfg.nslice; is++) counts[is] = h->beam.count ? h->hcount[is] : h->cfg.npart;
  return G4GPU_OK;
}

int g4gpu_sort(g4gpu_handle h, int *shift) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (shift) *shift = 0;  // Sorting::sort leaves the centre shift off (Sorting.cpp:66-67)
  if (!h->beam_loaded) return fail(h, G4GPU_ERR_STATE, "no beam loaded");
  // Sorting::sort: sorting is done for one4one windows only
  if (!h->beam.count) return G4GPU_OK;
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  const int ns = c.nslice, cap = c.npart;
  int rc;
  if (!h->sort_iscratch) {
    size_t np = (size_t)ns * cap;
    size_t es[6] = {h->rsize, 8, h->rsize, h->rsize, h->rsize, h->rsize};
    for (int k = 0; k < 6; k++)
      if ((rc = alloc(h, &h->sort_scratch[k], np * es[k]))) return rc;
    if ((rc = alloc(h, (void **)&h->sort_iscratch, (3 * (size_t)ns + 1) * sizeof(int)))) return rc;
  }
  {
    Timed t(h, G4GPU_K_MISC, 3);
    g4::launch_sort(h->stream, h->mixed, h->beam, h->sort_scratch, h->sort_iscratch, ns, cap, c.lambda0, c.sample);
  }
  G4_CUDA(h, cudaGetLastError());
  // the sorted window replaces the beam's arrays (their addresses stay: captured graphs
  // hold them)
  void *dst[6] = {h->beam.gamma, h->beam.theta, h->beam.x, h->beam.y, h->beam.px, h->beam.py};
  size_t es[6] = {h->rsize, 8, h->rsize, h->rsize, h->rsize, h->rsize};
  for (int k = 0; k < 6; k++)
    G4_CUDA(h, cudaMemcpyAsync(dst[k], h->sort_scratch[k], (size_t)ns * cap * es[k], cudaMemcpyDeviceToDevice,
                               h->stream));
  phasor_stale(h);
  int over = 0;
  G4_CUDA(h, cudaMemcpyAsync(&over, h->sort_iscratch + 3 * ns, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  G4_CUDA(h, cudaMemcpyAsync(h->hcount.data(), h->count_buf, ns * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  // Beam::sort: the wake follows the new current (Collective::forceUpdate)
  if (h->wake_on && (rc = wake_update(h))) return rc;
  if (over > 0)
    return fail(h, G4GPU_ERR_STATE,
                std::to_string(over) + " particles found no room in their slice: npart (the slices' capacity) is too small");
  return G4GPU_OK;
}

int g4gpu_get_beam(g4gpu_handle h, double *particles) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!particles) return fail(h, G4GPU_ERR_ARG, "null particles");
  if (!h->beam_loaded) return fail(h, G4GPU_ERR_STATE, "no beam loaded");
  cudaSetDevice(h->cfg.device);
  size_t n = (size_t)h->cfg.nslice * h->cfg.npart;
  int rc = ensure_stage(h, n * 6 * sizeof(double));
  if (rc) return rc;
  const void *soa[6] = {h->beam.gamma, h->beam.theta, h->beam.x, h->beam.y, h->beam.px, h->beam.py};
  {
    Timed t(h, G4GPU_K_MISC);
    g4::launch_soa_to_aos(h->stream, soa, (double *)h->stage, h->mixed, h->cfg.gammaref, n);
  }
  G4_CUDA(h, cudaGetLastError());
  G4_CUDA(h, cudaMemcpyAsync(particles, h->stage, n * 6 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_device_flag(h);
}

int g4gpu_load_field(g4gpu_handle h, int ifld, const double *field, int first, double accuslip) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (ifld < 0 || ifld >= h->cfg.nfield || !field) return fail(h, G4GPU_ERR_ARG, "bad field index or pointer");
  if (first < 0 || first >= h->cfg.nslice) return fail(h, G4GPU_ERR_ARG, "first out of range");
  cudaSetDevice(h->cfg.device);
  size_t n = (size_t)h->cfg.nslice * h->cfg.ngrid * h->cfg.ngrid;
  if (h->mixed) {
    int rc = ensure_stage(h, n * 16);
    if (rc) return rc;
    G4_CUDA(h, cudaMemcpyAsync(h->stage, field, n * 16, cudaMemcpyHostToDevice, h->stream));
    Timed t(h, G4GPU_K_MISC);
    g4::launch_convert_field(h->stream, h->stage, h->field[ifld], n, 1);
  } else {
    G4_CUDA(h, cudaMemcpyAsync(h->field[ifld], field, n * 16, cudaMemcpyHostToDevice, h->stream));
  }
  G4_CUDA(h, cudaGetLastError());
  h->first[ifld] = first;
  h->accuslip[ifld] = accuslip;
  h->field_loaded[ifld] = true;
  return G4GPU_OK;
}

int g4gpu_get_field(g4gpu_handle h, int ifld, double *field, int *first, double *accuslip) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (ifld < 0 || ifld >= h->cfg.nfield) return fail(h, G4GPU_ERR_ARG, "bad field index");
  cudaSetDevice(h->cfg.device);
  size_t n = (size_t)h->cfg.nslice * h->cfg.ngrid * h->cfg.ngrid;
  if (field) {
    if (h->mixed) {
      int rc = ensure_stage(h, n * 16);
      if (rc) return rc;
      {
        Timed t(h, G4GPU_K_MISC);
        g4::launch_convert_field(h->stream, h->field[ifld], h->stage, n, 0);
      }
      G4_CUDA(h, cudaMemcpyAsync(field, h->stage, n * 16, cudaMemcpyDeviceToHost, h->stream));
    } else {
      G4_CUDA(h, cudaMemcpyAsync(field, h->field[ifld], n * 16, cudaMemcpyDeviceToHost, h->stream));
    }
  }
  if (first) *first = h->first[ifld];
  if (accuslip) *accuslip = h->accuslip[ifld];
  return check_device_flag(h);
}

// Queues the kernels and copies of steps istep0 .. istep0+nsteps-1 on the handle's
// stream and advances the host-side ring state (first, accuslip) accordingly.
int g4gpu_set_efield(g4gpu_handle h, double rmax, int ngrid, int nz, int nphi, int longrange) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!(rmax >= 0) || ngrid < 0 || nz < 0 || nphi < 0)
    return fail(h, G4GPU_ERR_ARG, "rmax, ngrid, nz and nphi must be >= 0");
  const bool shortrange = nz > 0 && ngrid > 2;
  if (shortrange && g4::sc_bytes_per_mode(ngrid, h->mixed) > g4::sc_max_smem())
    return fail(h, G4GPU_ERR_ARG, "efield ngrid too large: one radial mode must fit in shared memory");
  if (shortrange && (long long)(2 * nphi + 1) * nz > (1 << 20))
    return fail(h, G4GPU_ERR_ARG, "too many space-charge modes");
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  int rc;
  if (!h->sc.st) {
    if ((rc = alloc(h, (void **)&h->sc.st, 7 * (size_t)c.nslice * sizeof(double)))) return rc;
    // the carried grid extent (a double) and the CTA counter of the moment kernel
    if ((rc = alloc(h, (void **)&h->sc.state, 2 * sizeof(double)))) return rc;
    h->sc.count = reinterpret_cast<unsigned *>(h->sc.state + 1);
  }
  if (shortrange && !h->sc.ez &&
      (rc = alloc(h, &h->sc.ez, (size_t)c.nslice * c.npart * h->rsize)))
    return rc;
  const double init[2] = {rmax, 0.0};  // the counter's bits are zero
  G4_CUDA(h, cudaMemcpyAsync(h->sc.state, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
  G4_CUDA(h, cudaMemsetAsync(h->sc.st, 0, 7 * (size_t)c.nslice * sizeof(double), h->stream));
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  h->sc_on = shortrange || longrange;
  h->sc_ngrid = ngrid;
  h->sc_nz = nz;
  h->sc_nphi = nphi;
  h->sc_longrange = longrange ? 1 : 0;
  // captured step sequences were recorded without (or with other) space charge
  for (auto &g : h->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  h->graphs.clear();
  h->graph_gen++;
  return G4GPU_OK;
}

int g4gpu_set_wake(g4gpu_handle h, int ns_hr, double ds, const double *ext, const double *res, const double *geo,
                   const double *rou, double ztrans, double radius, int transient) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  cudaSetDevice(h->cfg.device);
  // captured step sequences were recorded with other wakes
  if (!ext) {
    h->wake_on = false;
    drop_graphs(h);
    return G4GPU_OK;
  }
  const int ns = h->cfg.nslice;
  if (!res || !geo || !rou || !(ds > 0)) return fail(h, G4GPU_ERR_ARG, "null wake table or ds <= 0");
  // Collective::initWake / update: the fine grid covers the window, at least one fine
  // point per slice
  if (ns_hr < ns) return fail(h, G4GPU_ERR_ARG, "ns_hr must be at least nslice (nslice * sample)");
  if (h->wake_ns != ns_hr) {
    void *bufs[] = {h->wake_tab, h->wake_loss, h->wake_lossf, h->wake_scratch};
    for (void *p : bufs)
      if (p) cudaFree(p);
    h->wake_tab = h->wake_loss = h->wake_scratch = nullptr;
    h->wake_lossf = nullptr;
    h->wake_ns = 0;
    int rc;
    if ((rc = alloc(h, (void **)&h->wake_tab, (3 * (size_t)ns_hr + ns) * sizeof(double))) ||
        (rc = alloc(h, (void **)&h->wake_loss, ns * sizeof(double))) ||
        (rc = alloc(h, (void **)&h->wake_lossf, ns * sizeof(float))) ||
        (rc = alloc(h, (void **)&h->wake_scratch, 2 * (size_t)ns_hr * sizeof(double))))
      return rc;
    h->wake_ns = ns_hr;
  }
  std::vector<double> tab(3 * (size_t)ns_hr + ns);
  std::copy(res, res + ns_hr, tab.begin());
  std::copy(geo, geo + ns_hr, tab.begin() + ns_hr);
  std::copy(rou, rou + ns_hr, tab.begin() + 2 * (size_t)ns_hr);
  std::copy(ext, ext + ns, tab.begin() + 3 * (size_t)ns_hr);
  // self-loading theorem (Collective.cpp:103-105)
  tab[0] *= 0.5;
  tab[ns_hr] *= 0.5;
  tab[2 * (size_t)ns_hr] *= 0.5;
  G4_CUDA(h, cudaMemcpyAsync(h->wake_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice,
                             h->stream));
  h->wake_ds = ds;
  h->wake_ztrans = ztrans;
  h->wake_radius = radius;
  h->wake_transient = transient;
  h->wake_on = true;
  drop_graphs(h);
  int rc = h->beam_loaded ? wake_update(h) : G4GPU_OK;
  if (rc) return rc;
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  return G4GPU_OK;
}

// Control::applySlippage for a single rank (Control.cpp:158-276) on field k: the ring
// start moves by one slice per crossing of 0.8 sample and the slice that enters the
// window is cleared unless the window is periodic
static int apply_slippage(g4gpu_handle h, int k, double slippage) {
  const g4gpu_config &c = h->cfg;
  const int ns = c.nslice;
  const size_t ncell = (size_t)c.ngrid * c.ngrid;
  h->accuslip[k] += slippage;
  int direction = 1;
  // the slices that enter the window are cleared; a long slip (a chicane's delay spans
  // many windows) may enter every slice, which is then one clearing copy
  std::vector<char> cleared;
  int ncleared = 0;
  while (std::fabs(h->accuslip[k]) > (c.sample * 0.8)) {
    if (h->accuslip[k] < 0) direction = -1;
    h->accuslip[k] -= c.sample * direction;
    int last = (h->first[k] + ns - 1) % ns;
    if (direction < 0) last = (last + 1) % ns;
    if (!c.periodic) {
      if (cleared.empty()) cleared.assign(ns, 0);
      if (!cleared[last]) {
        cleared[last] = 1;
        ncleared++;
      }
    }
    h->first[k] = last;
    if (direction < 0) h->first[k] = (last + 1) % ns;
  }
  if (ncleared == ns) {
    G4_CUDA(h, cudaMemsetAsync(h->field[k], 0, (size_t)ns * ncell * h->csize, h->stream));
  } else if (ncleared > 0) {
    for (int is = 0; is < ns; is++)
      if (cleared[is])
        G4_CUDA(h, cudaMemsetAsync((char *)h->field[k] + (size_t)is * ncell * h->csize, 0, ncell * h->csize,
                                   h->stream));
  }
  // a record formed during the step holds the slices' sums before clearing
  if (ncleared > 0 && h->diag_fields_in_step) {
    const size_t fw = g4::kFieldSums + 2;
    double *d0 = h->diag_rec + (size_t)ns * g4::beam_diag_width(h->diag_nharm) + (size_t)k * ns * fw;
    for (int is = 0; is < ns; is++)
      if (cleared[is]) G4_CUDA(h, cudaMemsetAsync(d0 + (size_t)is * fw, 0, fw * sizeof(double), h->stream));
  }
  return G4GPU_OK;
}

// ---- sharded windows: the slippage exchange between ranks --------------------------

extern "C" int g4gpu_slip_shifts(double *accuslip, double slippage, double sample, int *direction) {
  if (!accuslip || !direction || !std::isfinite(slippage) || !(sample > 0)) return -1;
  // Control::applySlippage (Control.cpp:161-186): the shifts the accumulated slippage
  // yields, each moving it by one sample towards zero
  *accuslip += slippage;
  int n = 0, dir = 1;
  while (std::fabs(*accuslip) > (sample * 0.8)) {
    if (*accuslip < 0) dir = -1;
    *accuslip -= sample * dir;
    n++;
  }
  *direction = dir;
  return n;
}

int g4gpu_slip_count(g4gpu_handle h, int ifld, double slippage, int *nshift, int *direction) {
  if (!h || !nshift || !direction) return fail(h, G4GPU_ERR_ARG, "null argument");
  if (ifld < 0 || ifld >= h->cfg.nfield) return fail(h, G4GPU_ERR_ARG, "field index out of range");
  if (!std::isfinite(slippage)) return fail(h, G4GPU_ERR_ARG, "slippage must be finite");
  *nshift = 0;
  *direction = 1;
  if (!h->cfg.time_run) return G4GPU_OK;  // Control.cpp:159
  *nshift = g4gpu_slip_shifts(&h->accuslip[ifld], slippage, h->cfg.sample, direction);
  return G4GPU_OK;
}

size_t g4gpu_slice_bytes(g4gpu_handle h) {
  return h ? (size_t)h->cfg.ngrid * h->cfg.ngrid * h->csize : 0;
}

int g4gpu_shift_out(g4gpu_handle h, int ifld, int direction, void *send) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (ifld < 0 || ifld >= h->cfg.nfield) return fail(h, G4GPU_ERR_ARG, "field index out of range");
  if (direction != 1 && direction != -1) return fail(h, G4GPU_ERR_ARG, "direction must be +1 or -1");
  if (h->shift_slot[ifld] >= 0) return fail(h, G4GPU_ERR_STATE, "g4gpu_shift_in of the previous shift is missing");
  cudaSetDevice(h->cfg.device);
  const int ns = h->cfg.nslice;
  const size_t bytes = g4gpu_slice_bytes(h);
  // the slice leaving the block: the head (window slice ns - 1) forwards, the tail
  // (window slice 0) backwards (Control.cpp:199-204)
  int last = (h->first[ifld] + ns - 1) % ns;
  if (direction < 0) last = (last + 1) % ns;
  if (send)
    G4_CUDA(h, cudaMemcpyAsync(send, (char *)h->field[ifld] + (size_t)last * bytes, bytes, cudaMemcpyDefault,
                               h->stream));
  // its slot becomes the entering slice (Control.cpp:268-272)
  h->first[ifld] = direction > 0 ? last : (last + 1) % ns;
  h->shift_slot[ifld] = last;
  return G4GPU_OK;
}

int g4gpu_shift_in(g4gpu_handle h, int ifld, const void *recv) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (ifld < 0 || ifld >= h->cfg.nfield) return fail(h, G4GPU_ERR_ARG, "field index out of range");
  const int slot = h->shift_slot[ifld];
  if (slot < 0) return fail(h, G4GPU_ERR_STATE, "no g4gpu_shift_out before g4gpu_shift_in");
  cudaSetDevice(h->cfg.device);
  const size_t bytes = g4gpu_slice_bytes(h);
  char *dst = (char *)h->field[ifld] + (size_t)slot * bytes;
  if (recv)
    G4_CUDA(h, cudaMemcpyAsync(dst, recv, bytes, cudaMemcpyDefault, h->stream));
  else
    G4_CUDA(h, cudaMemsetAsync(dst, 0, bytes, h->stream));
  h->shift_slot[ifld] = -1;
  return G4GPU_OK;
}

int g4gpu_apply_slippage(g4gpu_handle h, int ifld, double slippage) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (ifld < 0 || ifld >= h->cfg.nfield) return fail(h, G4GPU_ERR_ARG, "field index out of range");
  if (!std::isfinite(slippage)) return fail(h, G4GPU_ERR_ARG, "slippage must be finite");
  if (!h->cfg.time_run) return G4GPU_OK;  // Control.cpp:159
  cudaSetDevice(h->cfg.device);
  return apply_slippage(h, ifld, slippage);
}

// A coarse step of g4gpu_set_field_substeps: the push over the whole step, c source
// sub-steps with their slippage, and the diffraction over the whole step.
static int enqueue_coarse_step(g4gpu_handle h, int istep, int cnt) {
  const g4gpu_config &c = h->cfg;
  const int ns = c.nslice, np = c.npart, ng = c.ngrid;
  g4::Launch L{h->stream, h->derr};
  StepConst sc = h->steps[istep];
  sc.f[0].first = h->first[0];
  g4::StepConstF scf = g4::to_float(sc, np);
  const size_t n = (size_t)ns * np;
  // the phases and positions at the start of the push
  G4_CUDA(h, cudaMemcpyAsync(h->sub_theta, h->beam.theta, n * 8, cudaMemcpyDeviceToDevice, h->stream));
  G4_CUDA(h, cudaMemcpyAsync(h->sub_x, h->beam.x, n * 4, cudaMemcpyDeviceToDevice, h->stream));
  G4_CUDA(h, cudaMemcpyAsync(h->sub_y, h->beam.y, n * 4, cudaMemcpyDeviceToDevice, h->stream));
  const void *wake = h->wake_on ? (const void *)h->wake_lossf : nullptr;
  {
    Timed t(h, G4GPU_K_PUSH);
    g4::launch_push_mixed_sc(L, scf, h->beam, h->field, nullptr, ns, np, ng, 0, h->push_block, 0, nullptr, nullptr,
                             wake, g4::IsrStream{});
  }
  // the sources of the c periods, each followed by its slippage
  for (int j = 0; j < cnt; j++) {
    scf.f[0].first = h->first[0];
    {
      Timed t(h, G4GPU_K_MISC);
      if (sc.f[0].dep_on)
        g4::launch_source_substep_mixed(L, scf, h->beam, h->sub_theta, h->sub_x, h->sub_y,
                                        (float)(j + 1) / (float)cnt, 2.f / (float)cnt, h->field[0], ns, np, ng);
    }
    if (c.time_run) {
      int rc = apply_slippage(h, 0, h->slip[istep] / cnt);
      if (rc) return rc;
    }
  }
  // the diffraction of the c periods: the ADI over the whole step without a source
  scf.f[0].first = h->first[0];
  const char *cb = (const char *)h->coef + (size_t)sc.f[0].coef * 3 * ng * h->csize;
  {
    Timed t(h, G4GPU_K_ADI_X);
    g4::launch_field_fused_mixed(L, scf, 0, h->beam, h->field[0], cb, ns, np, ng, 0, h->field_threads, nullptr,
                                 nullptr, 1, c.gammaref);
  }
  G4_CUDA(h, cudaGetLastError());
  return G4GPU_OK;
}

static int enqueue_steps(g4gpu_handle h, int istep0, int nsteps, int stages) {
  const g4gpu_config &c = h->cfg;
  int ns = c.nslice, np = c.npart, ng = c.ngrid;
  size_t ncell = (size_t)ng * ng;
  g4::Launch L{h->stream, h->derr};
  bool do_push = stages & G4GPU_STAGE_PUSH, do_field = stages & G4GPU_STAGE_FIELD;
  bool do_slip = (stages & G4GPU_STAGE_SLIP) && c.time_run;
  for (int istep = istep0; istep < istep0 + nsteps; istep++) {
    StepConst sc = h->steps[istep];
    // a coarse step (g4gpu_set_field_substeps) with every stage; with space charge,
    // one4one counts or incoherent radiation switched on since, the step runs whole
    if (istep < (int)h->substeps.size() && h->substeps[istep] > 1 && do_push && do_field &&
        (stages & G4GPU_STAGE_SLIP) && !sc.chic && !h->sc_on && !h->beam.count && !h->isr_loss &&
        !h->isr_spread) {
      int rc = enqueue_coarse_step(h, istep, h->substeps[istep]);
      if (rc) return rc;
      continue;
    }
    for (int k = 0; k < c.nfield; k++) sc.f[k].first = h->first[k];
    // Incoherent::apply (Incoherent.cpp:31-63): the step's loss and spread of gamma, in
    // undulators
    const bool isr_step = (h->isr_loss || h->isr_spread) && sc.aw > 0;
    if (isr_step) {
      const double gam0 = c.gammaref, awz = sc.aw, xkw0 = sc.ku_raw, delz = sc.delz;
      double dgamsig = 1.015e-27 * xkw0 * xkw0 * awz * awz;
      if (sc.helical)
        dgamsig *= 1.42 * awz + 1. / (1. + 1.5 * awz + 0.95 * awz * awz);
      else
        dgamsig *= 1.697 * awz + 1. / (1. + 1.88 * awz + 0.8 * awz * awz);
      if (!h->isr_spread) dgamsig = 0;
      dgamsig = std::sqrt(dgamsig * gam0 * gam0 * gam0 * gam0 * xkw0 * delz) * std::sqrt(3.);
      double dgamavg = xkw0 * gam0 * awz;
      if (!h->isr_loss) dgamavg = 0;
      dgamavg = dgamavg * dgamavg * 1.88e-15 * delz;
      sc.isr_avg = dgamavg;
      sc.isr_sig = dgamsig;
    }
    const g4::IsrStream isr{isr_step ? h->isr_ctr : nullptr, h->isr_seed, h->beam.count ? 1 : h->isr_nbins};
    g4::StepConstF scf_push{};
    if (h->mixed) scf_push = g4::to_float(sc, np);
    // Beam::track's push (Beam.cpp:97-112). With space charge, BeamSolver::advance
    // needs every slice after the first transverse half step (EFieldSolver::longRange
    // reads all slices' sizes): the first space-charge kernel runs the half step, and
    // the push the rest of the step.
    // Collective::apply after the integration (Beam.cpp:108)
    const void *wake = !h->wake_on ? nullptr : h->mixed ? (const void *)h->wake_lossf : (const void *)h->wake_loss;
    auto push = [&](void *const *src, int deposit) -> int {
      if (!h->sc_on) {
        Timed t(h, G4GPU_K_PUSH);
        if (h->mixed)
          g4::launch_push_mixed_sc(L, scf_push, h->beam, h->field, src, ns, np, ng, deposit, h->push_block, 0,
                                   nullptr, nullptr, wake, isr);
        else
          g4::launch_push_plain_sc(L, sc, h->beam, h->field, src, ns, np, ng, deposit, h->push_block, 0,
                                   nullptr, nullptr, wake, isr);
        if (isr.ctr) g4::launch_isr_advance(h->stream, h->isr_ctr);
        return G4GPU_OK;
      }
      const bool shortrange = h->sc_nz > 0 && h->sc_ngrid > 2;
      const void *ez = shortrange ? h->sc.ez : nullptr;
      const double *eloss = h->sc_longrange ? h->sc.st + 5 * (size_t)ns : nullptr;
      {
        g4::ScConst scc{};
        scc.ns = ns;
        scc.np = np;
        scc.ng = h->sc_ngrid;
        scc.nz = h->sc_nz;
        scc.nphi = h->sc_nphi;
        scc.longrange = h->sc_longrange;
        scc.shortrange = shortrange;
        if (shortrange) {
          const long long modes = (long long)(2 * h->sc_nphi + 1) * h->sc_nz;
          const size_t per = g4::sc_bytes_per_mode(h->sc_ngrid, h->mixed);
          scc.modes_per_pass = (int)std::max<long long>(1, std::min<long long>(modes, (96 << 10) / per));
        }
        // EFieldSolver.cpp:69, 103 and 216-218, with aw of the step (BeamSolver.cpp:40)
        const double aw = sc.aw;
        scc.slicelength = c.lambda0 * c.sample;
        scc.gamma_lr = c.gammaref / std::sqrt(1 + aw * aw);
        scc.lr_scl = scc.slicelength / 2. / std::asin(1) / 299792458.0 / 2 / 8.85e-12;
        scc.ks = 4 * std::asin(1) / c.lambda0;
        const double gz2 = c.gammaref * c.gammaref / (1 + aw * aw);
        scc.coef = -gz2 / scc.ks / scc.ks;
        for (int part = 0; part < 2; part++) {
          Timed t(h, part == 0 ? G4GPU_K_SC : G4GPU_K_SC_FIELD);
          if (h->mixed)
            g4::launch_sc_mixed(L, scc, scf_push, h->beam, h->sc, part);
          else
            g4::launch_sc_plain(L, scc, sc, h->beam, h->sc, part);
        }
      }
      Timed t(h, G4GPU_K_PUSH);
      if (h->mixed)
        g4::launch_push_mixed_sc(L, scf_push, h->beam, h->field, src, ns, np, ng, deposit, h->push_block, 2, ez,
                                 eloss, wake, isr);
      else
        g4::launch_push_plain_sc(L, sc, h->beam, h->field, src, ns, np, ng, deposit, h->push_block, 2, ez,
                                 eloss, wake, isr);
      if (isr.ctr) g4::launch_isr_advance(h->stream, h->isr_ctr);
      return G4GPU_OK;
    };
    bool any_dep = false;
    for (int k = 0; k < c.nfield; k++) any_dep = any_dep || sc.f[k].dep_on;
    // mixed form with the slice in shared memory: deposition and ADI in one kernel,
    // one CTA per slice or a cluster pair (chosen by the autotuner); grids too large
    // for one CTA take the smallest cluster whose bands fit (2 to 4 CTAs) when the
    // segmented solves apply
    bool fused = h->mixed && c.solver == G4GPU_SOLVER_ADI && ng <= g4::fused_max_ngrid();
    int band_w = 0;
    bool pair_ok = h->mixed && c.solver == G4GPU_SOLVER_ADI;
    for (int k = 0; k < c.nfield; k++) {
      pair_ok = pair_ok && sc.f[k].tw > 0;
      band_w = std::max(band_w, sc.f[k].tw);
    }
    const int band_cl = pair_ok ? g4::band_cluster(ng, band_w) : 0;
    bool pair = band_cl > 0 && (h->field_kernel == 1 || !fused);
    // the whole step in one kernel (push, deposition, ADI; one CTA per slice): chosen
    // by the autotuner (field_kernel 2) for one-field windows without space charge
    const bool rec_ok = h->diag_rec && g4::fused_diag_fits(ng, h->field_threads, h->diag_nharm);
    const bool step_fused = fused && h->field_kernel == 2 && do_push && do_field && !h->sc_on &&
                            g4::step_fused_ok(c.nfield, ng, h->field_threads, rec_ok, rec_ok, h->diag_nharm);
    if (step_fused) {
      const char *cb = (const char *)h->coef + (size_t)sc.f[0].coef * 3 * ng * h->csize;
      const int bw = g4::beam_diag_width(h->diag_nharm);
      {
        Timed t(h, G4GPU_K_STEP);
        g4::launch_step_fused_mixed(L, scf_push, h->beam, h->field[0], cb, ns, np, ng, sc.f[0].dep_on,
                                    h->field_threads, wake, isr, rec_ok ? h->diag_rec : nullptr,
                                    rec_ok ? h->diag_rec + (size_t)ns * bw : nullptr, h->diag_nharm, c.gammaref);
      }
      if (isr.ctr) g4::launch_isr_advance(h->stream, h->isr_ctr);
      if (rec_ok) h->diag_fields_in_step = h->diag_beam_in_step = true;
    } else if (fused || pair) {
      g4::StepConstF scf = scf_push;
      if (do_push) push(nullptr, 0);
      if (do_field) {
        // the diagnostic record of a step run by g4gpu_run_diag, formed by the fused
        // kernel itself when it holds the scratch for it
        const bool rec = h->diag_rec && !pair && g4::fused_diag_fits(ng, h->field_threads, h->diag_nharm);
        const int bw = g4::beam_diag_width(h->diag_nharm), fw = g4::kFieldSums + 2;
        for (int k = 0; k < c.nfield; k++) {
          const char *cb = (const char *)h->coef + (size_t)sc.f[k].coef * 3 * ng * h->csize;
          Timed t(h, G4GPU_K_ADI_X);
          if (pair)
            g4::launch_field_band_mixed(L, scf, k, h->beam, h->field[k], cb, ns, np, ng, sc.f[k].dep_on,
                                        band_cl);
          else
            g4::launch_field_fused_mixed(L, scf, k, h->beam, h->field[k], cb, ns, np, ng, sc.f[k].dep_on,
                                         h->field_threads, nullptr,
                                         rec ? h->diag_rec + (size_t)ns * bw + (size_t)k * ns * fw : nullptr,
                                         h->diag_nharm, c.gammaref);
        }
        if (rec) h->diag_fields_in_step = true;
      }
    } else {
    if (do_field && any_dep)
      for (int k = 0; k < c.nfield; k++)
        G4_CUDA(h, cudaMemsetAsync(h->src[k], 0, (size_t)ns * ncell * h->csize, h->stream));
    g4::StepConstF scf{};
    if (h->mixed) scf = g4::to_float(sc, np);
    if (do_push) {
      push(h->src, do_field && any_dep);
    } else if (do_field && any_dep) {
      Timed t(h, G4GPU_K_PUSH);
      if (h->mixed)
        g4::launch_deposit_mixed(L, scf, h->beam, h->src, ns, np, ng);
      else
        g4::launch_deposit_plain(L, sc, h->beam, h->src, ns, np, ng);
    }
    if (do_field && c.solver == G4GPU_SOLVER_FFT) {
      for (int k = 0; k < c.nfield; k++) {
        const void *srck = any_dep ? h->src[k] : nullptr;
        // a zero source makes the filtered term vanish (FieldSolverFFT.cpp:74-90)
        int filtered = c.source_filter && srck && c.sigmoid > 0 && c.xcut > 0 && c.ycut > 0;
        Timed t(h, G4GPU_K_FFT, 3);
        g4::launch_fft_solve(h->stream, h->mixed, h->field[k], srck, h->tmp, h->fft_roots[k], h->fft_k2c[k],
                             h->fft_sig[k], filtered, sc.delz, h->fft_plan, ns, sc.f[k].first);
      }
    } else if (do_field) {
      for (int k = 0; k < c.nfield; k++) {
        const char *cb = (const char *)h->coef + (size_t)sc.f[k].coef * 3 * ng * h->csize;
        // the source was cleared and deposited only when some field deposits
        const void *srck = any_dep ? h->src[k] : nullptr;
        for (int phase = 0; phase < 2; phase++) {
          Timed t(h, phase == 0 ? G4GPU_K_ADI_X : G4GPU_K_ADI_Y);
          if (h->mixed)
            g4::launch_adi_mixed(L, scf, k, phase, h->field[k], srck, h->tmp, cb, ns, ng);
          else
            g4::launch_adi_plain(L, sc, k, phase, h->field[k], srck, h->tmp, cb, ns, ng);
        }
      }
    }
    }
    G4_CUDA(h, cudaGetLastError());
    if (do_slip)
      for (int k = 0; k < c.nfield; k++) {
        int rc = apply_slippage(h, k, h->slip[istep]);
        if (rc) return rc;
      }
  }
  return G4GPU_OK;
}

int g4gpu_run(g4gpu_handle h, int istep0, int nsteps, int stages) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (istep0 < 0 || nsteps < 0 || istep0 + nsteps > h->nsteps)
    return fail(h, G4GPU_ERR_ARG, "step range outside the lattice");
  if (!h->beam_loaded) return fail(h, G4GPU_ERR_STATE, "no beam loaded");
  for (int k = 0; k < h->cfg.nfield; k++)
    if (!h->field_loaded[k]) return fail(h, G4GPU_ERR_STATE, "a field is not loaded");
  cudaSetDevice(h->cfg.device);
  if (!h->graph_mode || nsteps == 0) return enqueue_steps(h, istep0, nsteps, stages);

  // Graph mode: the whole step range is one CUDA graph, captured the first time a
  // range starts from a given ring state and replayed afterwards. The kernels take
  // the ring start by value, so a graph is valid for exactly that starting state.
  g4gpu_ctx::GraphKey key{istep0, nsteps, stages, h->push_block, h->field_threads, h->field_kernel, {}};
  for (int k = 0; k < h->cfg.nfield; k++) {
    long long bits;
    std::memcpy(&bits, &h->accuslip[k], sizeof(bits));
    key.state.push_back(h->first[k]);
    key.state.push_back(bits);
  }
  auto it = h->graphs.find(key);
  if (it == h->graphs.end()) {
    long long before[G4GPU_K_NCLASS];
    std::memcpy(before, h->launches, sizeof(before));
    cudaGraph_t graph = nullptr;
    G4_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->capturing = true;
    int rc = enqueue_steps(h, istep0, nsteps, stages);
    h->capturing = false;
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
    g4gpu_ctx::GraphEntry ent;
    e = cudaGraphInstantiate(&ent.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    for (int k = 0; k < h->cfg.nfield; k++) {
      ent.end_first.push_back(h->first[k]);
      ent.end_accuslip.push_back(h->accuslip[k]);
    }
    for (int c = 0; c < G4GPU_K_NCLASS; c++) ent.launches[c] = h->launches[c] - before[c];
    // the capture advanced the counters and the ring state without running anything
    std::memcpy(h->launches, before, sizeof(before));
    it = h->graphs.emplace(key, ent).first;
  }
  G4_CUDA(h, cudaGraphLaunch(it->second.exec, h->stream));
  for (int k = 0; k < h->cfg.nfield; k++) {
    h->first[k] = it->second.end_first[k];
    h->accuslip[k] = it->second.end_accuslip[k];
  }
  for (int c = 0; c < G4GPU_K_NCLASS; c++) h->launches[c] += it->second.launches[c];
  return G4GPU_OK;
}

int g4gpu_set_launch_shapes(g4gpu_handle h, int push_block, int field_threads, int field_kernel) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (push_block < 32 || push_block > 512 || push_block % 32)
    return fail(h, G4GPU_ERR_ARG, "push_block must be a multiple of 32 in [32, 512]");
  if (field_threads < 2 * h->cfg.ngrid || field_threads > 1024 || field_threads % 32)
    return fail(h, G4GPU_ERR_ARG, "field_threads must be a multiple of 32 in [2 ngrid, 1024]");
  if (field_kernel < 0 || field_kernel > 2) return fail(h, G4GPU_ERR_ARG, "field_kernel must be 0, 1 or 2");
  h->push_block = push_block;
  h->field_threads = field_threads;
  h->field_kernel = field_kernel;
  return G4GPU_OK;
}

int g4gpu_set_graph_mode(g4gpu_handle h, int on) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  h->graph_mode = on != 0;
  return G4GPU_OK;
}

int g4gpu_synchronize(g4gpu_handle h) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  cudaSetDevice(h->cfg.device);
  G4_CUDA(h, cudaStreamSynchronize(h->stream));
  G4_CUDA(h, cudaGetLastError());
  return check_device_flag(h);
}

}  // extern "C"

namespace {

// Device and pinned host buffers of the raw diagnostic sums, grown to `need` bytes.
int diag_buffers(g4gpu_handle h, size_t need) {
  if (need <= h->ddiag_bytes) return G4GPU_OK;
  if (h->ddiag) cudaFree(h->ddiag);
  if (h->hdiag) cudaFreeHost(h->hdiag);
  h->ddiag = nullptr;
  h->hdiag = nullptr;
  h->ddiag_bytes = 0;
  int rc = alloc(h, (void **)&h->ddiag, need);
  if (rc) return rc;
  cudaError_t e = cudaMallocHost((void **)&h->hdiag, need);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocHost (diagnostics)");
  h->ddiag_bytes = need;
  return G4GPU_OK;
}

// Raw sums of one diagnostic record: beam [nslice][beam_diag_width], then per field
// [nslice][kFieldSums + 2] in storage (ring) order.
size_t diag_record_doubles(const g4gpu_config &c, int nharm) {
  return (size_t)c.nslice * g4::beam_diag_width(nharm) + (size_t)c.nfield * c.nslice * (g4::kFieldSums + 2);
}

// Queues the kernels of one diagnostic record of the current state into `rec`.
void enqueue_diag(g4gpu_handle h, int nharm, double *rec, bool beam, bool field) {
  const g4gpu_config &c = h->cfg;
  int ns = c.nslice, np = c.npart, ng = c.ngrid;
  int bw = g4::beam_diag_width(nharm), fw = g4::kFieldSums + 2;
  g4::Launch L{h->stream, h->derr};
  double *db = rec, *dfd = rec + (size_t)ns * bw;
  if (beam) {
    Timed t(h, G4GPU_K_DIAG);
    if (h->mixed)
      g4::launch_diag_beam_mixed(L, h->beam, c.gammaref, ns, np, nharm, db);
    else
      g4::launch_diag_beam_plain(L, h->beam, ns, np, nharm, db);
  }
  if (field) {
    for (int k = 0; k < c.nfield; k++) {
      Timed t(h, G4GPU_K_DIAG);
      if (h->mixed)
        g4::launch_diag_field_mixed(L, h->field[k], ns, ng, dfd + (size_t)k * ns * fw);
      else
        g4::launch_diag_field_plain(L, h->field[k], ns, ng, dfd + (size_t)k * ns * fw);
    }
  }
}

// The diagnostics of one raw record, with the fields' ring starts `first` of that
// state: DiagBeam::getValues and DiagField::getValues finished on the host.
void finish_diag(g4gpu_handle h, const double *raw, int nharm, const int *first, double *beam_out,
                 double *field_out) {
  const g4gpu_config &c = h->cfg;
  int ns = c.nslice, np = c.npart, ng = c.ngrid;
  int bw = g4::beam_diag_width(nharm), fw = g4::kFieldSums + 2;
  (void)fw;

  if (beam_out) {
    // DiagBeam::getValues, Diagnostic.cpp:457-531
    int ow = G4GPU_DB_NCOL + 2 * nharm;
    for (int is = 0; is < ns; is++) {
      // Diagnostic.cpp:452-455: 1 / the slice's particles, 1 for an empty slice
      const int n = h->beam.count ? h->hcount[is] : np;
      double norm = n > 0 ? 1. / static_cast<double>(n) : 1.;
      const double *s = raw + (size_t)is * bw;
      double g1 = s[0] * norm, g2 = s[1] * norm, x1 = s[2] * norm, x2 = s[3] * norm;
      double y1 = s[4] * norm, y2 = s[5] * norm, px1 = s[6] * norm, px2 = s[7] * norm;
      double py1 = s[8] * norm, py2 = s[9] * norm, xpx = s[10] * norm, ypy = s[11] * norm;
      double *o = beam_out + (size_t)is * ow;
      o[G4GPU_DB_ENERGY] = g1;
      o[G4GPU_DB_ENERGYSPREAD] = std::sqrt(std::fabs(g2 - g1 * g1));
      o[G4GPU_DB_XPOS] = x1;
      o[G4GPU_DB_XSIZE] = std::sqrt(std::fabs(x2 - x1 * x1));
      o[G4GPU_DB_YPOS] = y1;
      o[G4GPU_DB_YSIZE] = std::sqrt(std::fabs(y2 - y1 * y1));
      o[G4GPU_DB_PXPOS] = px1;
      o[G4GPU_DB_PYPOS] = py1;
      double ex = std::sqrt(std::fabs((x2 - x1 * x1) * (px2 - px1 * px1) - (xpx - x1 * px1) * (xpx - x1 * px1)));
      double ey = std::sqrt(std::fabs((y2 - y1 * y1) * (py2 - py1 * py1) - (ypy - y1 * py1) * (ypy - y1 * py1)));
      o[G4GPU_DB_EMITX] = ex;
      o[G4GPU_DB_EMITY] = ey;
      o[G4GPU_DB_BETAX] = (x2 - x1 * x1) / ex * g1;
      o[G4GPU_DB_BETAY] = (y2 - y1 * y1) / ey * g1;
      o[G4GPU_DB_ALPHAX] = -(xpx - x1 * px1) / ex;
      o[G4GPU_DB_ALPHAY] = -(ypy - y1 * py1) / ey;
      for (int k = 0; k < 10; k++) o[G4GPU_DB_XMIN + k] = s[g4::kBeamSums + k];
      for (int hh = 0; hh < nharm; hh++) {
        double br = s[g4::kBeamSums + g4::kBeamMinMax + 2 * hh] * norm;
        double bi = s[g4::kBeamSums + g4::kBeamMinMax + 2 * hh + 1] * norm;
        o[G4GPU_DB_NCOL + 2 * hh] = std::abs(std::complex<double>(br, bi));
        o[G4GPU_DB_NCOL + 2 * hh + 1] = std::atan2(bi, br);
      }
    }
  }
  if (field_out) {
    // DiagField::getValues, Diagnostic.cpp:796-866
    for (int k = 0; k < c.nfield; k++) {
      double xlambda = c.lambda0 / static_cast<double>(c.harm[k]);
      double dgrid = 2 * c.gridmax[k] / static_cast<double>(ng - 1);
      double ks = 4. * std::asin(1) / xlambda;
      double scl = dgrid * g4::kEev / ks;
      for (int is0 = 0; is0 < ns; is0++) {
        const double *s = raw + (size_t)ns * bw + ((size_t)k * ns + is0) * fw;
        int is = (ns + is0 - first[k]) % ns;
        double power = s[0], x1 = s[1], x2 = s[2], y1 = s[3], y2 = s[4];
        if (power > 0) {
          x1 /= power;
          x2 /= power;
          y1 /= power;
          y2 /= power;
        }
        x2 = std::sqrt(std::fabs(x2 - x1 * x1));
        y2 = std::sqrt(std::fabs(y2 - y1 * y1));
        double inten = s[7] * s[7] + s[8] * s[8];
        double intenphi = std::atan2(s[8], s[7]);
        double farfield = (s[5] * s[5] + s[6] * s[6]) * dgrid * dgrid;
        double farphi = std::atan2(s[6], s[5]);
        double *o = field_out + ((size_t)k * ns + is) * G4GPU_DF_NCOL;
        o[G4GPU_DF_POWER] = power * scl * scl / g4::kVacimp;
        o[G4GPU_DF_XPOS] = x1 * dgrid;
        o[G4GPU_DF_XSIZE] = x2 * dgrid;
        o[G4GPU_DF_YPOS] = y1 * dgrid;
        o[G4GPU_DF_YSIZE] = y2 * dgrid;
        o[G4GPU_DF_NF_INT] = inten * g4::kEev * g4::kEev / ks / ks / g4::kVacimp;
        o[G4GPU_DF_NF_PHI] = intenphi;
        o[G4GPU_DF_FF_INT] = farfield;
        o[G4GPU_DF_FF_PHI] = farphi;
      }
    }
  }
}

}  // namespace

extern "C" {

int g4gpu_diag(g4gpu_handle h, int nharm, double *beam_out, double *field_out) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (nharm < 1 || nharm > G4GPU_MAX_HARM) return fail(h, G4GPU_ERR_ARG, "nharm must be 1..16");
  if (beam_out && !h->beam_loaded) return fail(h, G4GPU_ERR_STATE, "no beam loaded");
  cudaSetDevice(h->cfg.device);
  const size_t need = diag_record_doubles(h->cfg, nharm) * sizeof(double);
  int rc = diag_buffers(h, need);
  if (rc) return rc;
  enqueue_diag(h, nharm, h->ddiag, beam_out != nullptr, field_out != nullptr);
  G4_CUDA(h, cudaGetLastError());
  G4_CUDA(h, cudaMemcpyAsync(h->hdiag, h->ddiag, need, cudaMemcpyDeviceToHost, h->stream));
  rc = check_device_flag(h);
  if (rc) return rc;
  finish_diag(h, h->hdiag, nharm, h->first, beam_out, field_out);
  return G4GPU_OK;
}

int g4gpu_get_config(g4gpu_handle h, g4gpu_config *cfg) {
  if (!h || !cfg) return fail(h, G4GPU_ERR_ARG, "null argument");
  *cfg = h->cfg;
  return G4GPU_OK;
}

int g4gpu_diag_global(const g4gpu_config *cfg, int nharm, const double *current, const double *beam_diag,
                      const double *field_diag, const double *fft_diag, double *beam_global,
                      double *field_global) {
  if (!cfg || nharm < 1 || nharm > G4GPU_MAX_HARM) return G4GPU_ERR_ARG;
  if ((beam_global && (!beam_diag || !current)) || (field_global && !field_diag)) return G4GPU_ERR_ARG;
  const int ns = cfg->nslice;
  if (beam_global) {
    // DiagBeam, Diagnostic.cpp:551-606: per slice <g> = energy, <g^2> = spread^2 +
    // energy^2 (likewise x, y), weighted by the current
    const int bw = G4GPU_DB_NCOL + 2 * nharm;
    double wc = 0, g1 = 0, g2 = 0, x1 = 0, x2 = 0, y1 = 0, y2 = 0;
    for (int is = 0; is < ns; is++) {
      const double *b = beam_diag + (size_t)is * bw, c = current[is];
      wc += c;
      g1 += c * b[G4GPU_DB_ENERGY];
      g2 += c * (b[G4GPU_DB_ENERGYSPREAD] * b[G4GPU_DB_ENERGYSPREAD] + b[G4GPU_DB_ENERGY] * b[G4GPU_DB_ENERGY]);
      x1 += c * b[G4GPU_DB_XPOS];
      x2 += c * (b[G4GPU_DB_XSIZE] * b[G4GPU_DB_XSIZE] + b[G4GPU_DB_XPOS] * b[G4GPU_DB_XPOS]);
      y1 += c * b[G4GPU_DB_YPOS];
      y2 += c * (b[G4GPU_DB_YSIZE] * b[G4GPU_DB_YSIZE] + b[G4GPU_DB_YPOS] * b[G4GPU_DB_YPOS]);
    }
    const double w = wc > 0 ? 1. / wc : 1.;
    g1 *= w, g2 *= w, x1 *= w, x2 *= w, y1 *= w, y2 *= w;
    beam_global[G4GPU_DBG_ENERGY] = g1;
    beam_global[G4GPU_DBG_ENERGYSPREAD] = std::sqrt(std::fabs(g2 - g1 * g1));
    beam_global[G4GPU_DBG_XPOS] = x1;
    beam_global[G4GPU_DBG_XSIZE] = std::sqrt(std::fabs(x2 - x1 * x1));
    beam_global[G4GPU_DBG_YPOS] = y1;
    beam_global[G4GPU_DBG_YSIZE] = std::sqrt(std::fabs(y2 - y1 * y1));
  }
  if (field_global) {
    // DiagField, Diagnostic.cpp:902-975: centroids and sizes weighted by the slices'
    // power; the energy is the power summed over the window times slicelength / c
    const double slicelength = cfg->lambda0 * cfg->sample;
    for (int k = 0; k < cfg->nfield; k++) {
      double p = 0, x1 = 0, x2 = 0, y1 = 0, y2 = 0, ni = 0, fi = 0, fx1 = 0, fx2 = 0, fy1 = 0, fy2 = 0;
      for (int is = 0; is < ns; is++) {
        const double *f = field_diag + ((size_t)k * ns + is) * G4GPU_DF_NCOL, P = f[G4GPU_DF_POWER];
        p += P;
        x1 += P * f[G4GPU_DF_XPOS];
        x2 += P * (f[G4GPU_DF_XSIZE] * f[G4GPU_DF_XSIZE] + f[G4GPU_DF_XPOS] * f[G4GPU_DF_XPOS]);
        y1 += P * f[G4GPU_DF_YPOS];
        y2 += P * (f[G4GPU_DF_YSIZE] * f[G4GPU_DF_YSIZE] + f[G4GPU_DF_YPOS] * f[G4GPU_DF_YPOS]);
        ni += f[G4GPU_DF_NF_INT];
        fi += f[G4GPU_DF_FF_INT];
        if (fft_diag) {
          const double *q = fft_diag + ((size_t)k * ns + is) * G4GPU_DFFT_NCOL;
          fx1 += P * q[G4GPU_DFFT_XPOINT];
          fx2 += P * (q[G4GPU_DFFT_XDIV] * q[G4GPU_DFFT_XDIV] + q[G4GPU_DFFT_XPOINT] * q[G4GPU_DFFT_XPOINT]);
          fy1 += P * q[G4GPU_DFFT_YPOINT];
          fy2 += P * (q[G4GPU_DFFT_YDIV] * q[G4GPU_DFFT_YDIV] + q[G4GPU_DFFT_YPOINT] * q[G4GPU_DFFT_YPOINT]);
        }
      }
      const double w = p > 0 ? 1. / p : 1.;
      x1 *= w, x2 *= w, y1 *= w, y2 *= w, fx1 *= w, fx2 *= w, fy1 *= w, fy2 *= w;
      double *o = field_global + (size_t)k * G4GPU_DFG_NCOL;
      o[G4GPU_DFG_ENERGY] = p * slicelength / 299792458.0;
      o[G4GPU_DFG_XPOS] = x1;
      o[G4GPU_DFG_XSIZE] = std::sqrt(std::fabs(x2 - x1 * x1));
      o[G4GPU_DFG_YPOS] = y1;
      o[G4GPU_DFG_YSIZE] = std::sqrt(std::fabs(y2 - y1 * y1));
      o[G4GPU_DFG_NF_INT] = ns > 0 ? ni / ns : 0.;
      o[G4GPU_DFG_FF_INT] = ns > 0 ? fi / ns : 0.;
      o[G4GPU_DFG_XPOINT] = fft_diag ? fx1 : 0.;
      o[G4GPU_DFG_XDIV] = fft_diag ? std::sqrt(std::fabs(fx2 - fx1 * fx1)) : 0.;
      o[G4GPU_DFG_YPOINT] = fft_diag ? fy1 : 0.;
      o[G4GPU_DFG_YDIV] = fft_diag ? std::sqrt(std::fabs(fy2 - fy1 * fy1)) : 0.;
    }
  }
  return G4GPU_OK;
}

int g4gpu_diag_fft(g4gpu_handle h, double *out) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!out) return fail(h, G4GPU_ERR_ARG, "null output");
  const g4gpu_config &c = h->cfg;
  for (int k = 0; k < c.nfield; k++)
    if (!h->field_loaded[k]) return fail(h, G4GPU_ERR_STATE, "a field is not loaded");
  cudaSetDevice(c.device);
  int rc;
  // the transform's roots and plan: the FFT solver's, else built on the first call
  if (!h->fft_roots[0] && (rc = fft_tables(h))) return rc;
  if (!g4::fft_plan_fits(h->fft_plan))
    return fail(h, G4GPU_ERR_ARG, "ngrid " + std::to_string(c.ngrid) + ": no FFT plan for the far-field diagnostics");
  const int ns = c.nslice, n = c.ngrid;
  const size_t ncell = (size_t)n * n;
  void *work = h->tmp;
  if (!work) {
    if (!h->diag_work && (rc = alloc(h, &h->diag_work, (size_t)ns * ncell * h->csize))) return rc;
    work = h->diag_work;
  }
  const int L = g4::fft_diag_lines(h->fft_plan, h->mixed), nblk = (n + L - 1) / L;
  const size_t per_field = (size_t)ns * nblk * 5;
  if ((rc = diag_buffers(h, (size_t)c.nfield * per_field * sizeof(double)))) return rc;
  for (int k = 0; k < c.nfield; k++) {
    Timed t(h, G4GPU_K_DIAG, 2);
    g4::launch_fft_diag(h->stream, h->mixed, h->field[k], work, h->fft_roots[k], h->fft_plan, ns, h->first[k],
                        h->ddiag + k * per_field);
  }
  G4_CUDA(h, cudaGetLastError());
  G4_CUDA(h, cudaMemcpyAsync(h->hdiag, h->ddiag, (size_t)c.nfield * per_field * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
  if ((rc = check_device_flag(h))) return rc;
  // DiagField::getValues, Diagnostic.cpp:815-836 (moments) and 836-847 (scaling)
  for (int k = 0; k < c.nfield; k++) {
    const double xlambda = c.lambda0 / static_cast<double>(c.harm[k]);
    const double dgrid = 2 * c.gridmax[k] / static_cast<double>(n - 1);
    const double scltheta = xlambda / n / dgrid;
    for (int ii = 0; ii < ns; ii++) {
      double m[5] = {0, 0, 0, 0, 0};
      const double *p = h->hdiag + k * per_field + (size_t)ii * nblk * 5;
      for (int b = 0; b < nblk; b++)
        for (int q = 0; q < 5; q++) m[q] += p[(size_t)b * 5 + q];
      double fp = m[0], fx1 = m[1], fx2 = m[2], fy1 = m[3], fy2 = m[4];
      if (fp > 0) {
        fx1 /= fp;
        fx2 /= fp;
        fy1 /= fp;
        fy2 /= fp;
      }
      double *o = out + ((size_t)k * ns + ii) * G4GPU_DFFT_NCOL;
      o[G4GPU_DFFT_XPOINT] = fx1 * scltheta;
      o[G4GPU_DFFT_XDIV] = std::sqrt(std::fabs(fx2 - fx1 * fx1)) * scltheta;
      o[G4GPU_DFFT_YPOINT] = fy1 * scltheta;
      o[G4GPU_DFFT_YDIV] = std::sqrt(std::fabs(fy2 - fy1 * fy1)) * scltheta;
    }
  }
  return G4GPU_OK;
}

int g4gpu_run_diag(g4gpu_handle h, int istep0, int nsteps, int nharm, double *beam_out, double *field_out) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (nharm < 1 || nharm > G4GPU_MAX_HARM) return fail(h, G4GPU_ERR_ARG, "nharm must be 1..16");
  if (istep0 < 0 || nsteps < 0 || istep0 + nsteps > h->nsteps)
    return fail(h, G4GPU_ERR_ARG, "step range outside the lattice");
  if (!h->beam_loaded) return fail(h, G4GPU_ERR_STATE, "no beam loaded");
  for (int k = 0; k < h->cfg.nfield; k++)
    if (!h->field_loaded[k]) return fail(h, G4GPU_ERR_STATE, "a field is not loaded");
  if (nsteps == 0) return G4GPU_OK;
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  const size_t rec = diag_record_doubles(c, nharm);
  int rc = diag_buffers(h, (size_t)nsteps * rec * sizeof(double));
  if (rc) return rc;
  std::vector<int> firsts((size_t)nsteps * G4GPU_MAX_FIELDS);
  // each step's record is copied back as soon as it is formed and finished on the host
  // while the device runs the later steps
  // the records are copied on a stream of their own, so that a copy over the host link
  // runs beside the next step instead of in front of it (each step's record has its own
  // slot of ddiag)
  struct Events {
    std::vector<cudaEvent_t> ev;
    cudaEvent_t formed = nullptr;
    cudaStream_t copy = nullptr;
    ~Events() {
      for (cudaEvent_t e : ev) cudaEventDestroy(e);
      if (formed) cudaEventDestroy(formed);
      if (copy) {
        cudaStreamSynchronize(copy);
        cudaStreamDestroy(copy);
      }
    }
  } done;
  done.ev.reserve(nsteps);
  G4_CUDA(h, cudaStreamCreateWithFlags(&done.copy, cudaStreamNonBlocking));
  G4_CUDA(h, cudaEventCreateWithFlags(&done.formed, cudaEventDisableTiming));
  for (int s = 0; s < nsteps; s++) {
    // the fused field kernel forms the fields' record during the step where it can
    // (the slice is in its shared memory); the beam's, and the fields' elsewhere, come
    // from the diagnostic kernels after the step
    h->diag_rec = h->ddiag + (size_t)s * rec;
    h->diag_nharm = nharm;
    h->diag_fields_in_step = h->diag_beam_in_step = false;
    rc = enqueue_steps(h, istep0 + s, 1, G4GPU_STAGE_ALL);
    const bool fields_done = h->diag_fields_in_step, beam_done = h->diag_beam_in_step;
    h->diag_rec = nullptr;
    h->diag_fields_in_step = h->diag_beam_in_step = false;
    if (rc) return rc;
    for (int k = 0; k < c.nfield; k++) firsts[(size_t)s * G4GPU_MAX_FIELDS + k] = h->first[k];
    enqueue_diag(h, nharm, h->ddiag + (size_t)s * rec, beam_out != nullptr && !beam_done,
                 field_out != nullptr && !fields_done);
    G4_CUDA(h, cudaGetLastError());
    G4_CUDA(h, cudaEventRecord(done.formed, h->stream));
    G4_CUDA(h, cudaStreamWaitEvent(done.copy, done.formed, 0));
    G4_CUDA(h, cudaMemcpyAsync(h->hdiag + (size_t)s * rec, h->ddiag + (size_t)s * rec, rec * sizeof(double),
                               cudaMemcpyDeviceToHost, done.copy));
    cudaEvent_t e;
    G4_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    done.ev.push_back(e);
    G4_CUDA(h, cudaEventRecord(e, done.copy));
  }
  const size_t bstride = (size_t)c.nslice * (G4GPU_DB_NCOL + 2 * nharm);
  const size_t fstride = (size_t)c.nfield * c.nslice * G4GPU_DF_NCOL;
  for (int s = 0; s < nsteps; s++) {
    G4_CUDA(h, cudaEventSynchronize(done.ev[s]));
    finish_diag(h, h->hdiag + (size_t)s * rec, nharm, &firsts[(size_t)s * G4GPU_MAX_FIELDS],
                beam_out ? beam_out + s * bstride : nullptr, field_out ? field_out + s * fstride : nullptr);
  }
  // a device error raised by any step fails the call (its records are then not trusted)
  if ((rc = check_device_flag(h))) return rc;
  return G4GPU_OK;
}

int g4gpu_get_stream(g4gpu_handle h, void **stream) {
  if (!h || !stream) return fail(h, G4GPU_ERR_ARG, "null argument");
  *stream = h->stream;
  return G4GPU_OK;
}

int g4gpu_set_profiling(g4gpu_handle h, int on) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  collect_events(h);
  h->prof = on != 0;
  return G4GPU_OK;
}

int g4gpu_kernel_stats(g4gpu_handle h, long long *launches, double *ms) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  cudaSetDevice(h->cfg.device);
  collect_events(h);
  for (int k = 0; k < G4GPU_K_NCLASS; k++) {
    if (launches) launches[k] = h->launches[k];
    if (ms) ms[k] = h->ms[k];
  }
  return G4GPU_OK;
}

int g4gpu_reset_stats(g4gpu_handle h) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  collect_events(h);
  for (int k = 0; k < G4GPU_K_NCLASS; k++) {
    h->launches[k] = 0;
    h->ms[k] = 0;
  }
  return G4GPU_OK;
}

size_t g4gpu_device_bytes(g4gpu_handle h) { return h ? h->bytes : 0; }

// ---- launch-shape tuning -----------------------------------------------------

namespace {
struct TuneKey {
  int device, precision, npart, ngrid, nfield, solver;
  bool operator<(const TuneKey &o) const {
    return std::tie(device, precision, npart, ngrid, nfield, solver) <
           std::tie(o.device, o.precision, o.npart, o.ngrid, o.nfield, o.solver);
  }
};
std::mutex g_tune_mu;
struct TuneVal {
  int push_block, field_threads, field_kernel;
};
std::map<TuneKey, TuneVal> g_tune;

// device copies of everything a step modifies, to undo the tuning steps
struct StateBackup {
  std::vector<std::pair<void *, void *>> bufs;  // (live, copy)
  std::vector<size_t> sizes;
  int first[G4GPU_MAX_FIELDS];
  double accuslip[G4GPU_MAX_FIELDS];
};
}  // namespace

static int backup_state(g4gpu_handle h, StateBackup &b) {
  const g4gpu_config &c = h->cfg;
  size_t np = (size_t)c.nslice * c.npart, nf = (size_t)c.nslice * c.ngrid * c.ngrid * h->csize;
  std::vector<std::pair<void *, size_t>> live = {
      {h->beam.gamma, np * h->rsize}, {h->beam.theta, np * 8}, {h->beam.x, np * h->rsize},
      {h->beam.y, np * h->rsize},     {h->beam.px, np * h->rsize}, {h->beam.py, np * h->rsize}};
  for (int k = 0; k < c.nfield; k++) live.push_back({h->field[k], nf});
  // the radial grid extent of the space charge, carried from step to step, and the
  // incoherent radiation's counter of drawing steps: the trial steps leave neither moved
  if (h->sc.state) live.push_back({h->sc.state, 2 * sizeof(double)});
  if (h->isr_ctr) live.push_back({h->isr_ctr, sizeof(unsigned long long)});
  for (auto &l : live) {
    void *cp = nullptr;
    cudaError_t e = cudaMalloc(&cp, l.second);
    if (e != cudaSuccess) return cuda_fail(h, e, "autotune backup");
    G4_CUDA(h, cudaMemcpyAsync(cp, l.first, l.second, cudaMemcpyDeviceToDevice, h->stream));
    b.bufs.push_back({l.first, cp});
    b.sizes.push_back(l.second);
  }
  std::memcpy(b.first, h->first, sizeof(b.first));
  std::memcpy(b.accuslip, h->accuslip, sizeof(b.accuslip));
  return G4GPU_OK;
}

static void restore_state(g4gpu_handle h, StateBackup &b, bool release) {
  for (size_t i = 0; i < b.bufs.size(); i++) {
    cudaMemcpyAsync(b.bufs[i].first, b.bufs[i].second, b.sizes[i], cudaMemcpyDeviceToDevice, h->stream);
    if (release) {
      cudaStreamSynchronize(h->stream);
      cudaFree(b.bufs[i].second);
    }
  }
  std::memcpy(h->first, b.first, sizeof(b.first));
  std::memcpy(h->accuslip, b.accuslip, sizeof(b.accuslip));
  phasor_stale(h);
}

extern "C" int g4gpu_autotune(g4gpu_handle h, int *push_block, int *field_threads, int *field_kernel) {
  if (!h) return fail(nullptr, G4GPU_ERR_ARG, "null handle");
  if (!h->beam_loaded || h->nsteps < 1) return fail(h, G4GPU_ERR_STATE, "load a lattice and a beam first");
  for (int k = 0; k < h->cfg.nfield; k++)
    if (!h->field_loaded[k]) return fail(h, G4GPU_ERR_STATE, "a field is not loaded");
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  TuneKey key{c.device, c.precision, c.npart, c.ngrid, c.nfield, c.solver};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      h->push_block = it->second.push_block;
      h->field_threads = it->second.field_threads;
      h->field_kernel = it->second.field_kernel;
      if (push_block) *push_block = h->push_block;
      if (field_threads) *field_threads = h->field_threads;
      if (field_kernel) *field_kernel = h->field_kernel;
      return G4GPU_OK;
    }
  }
  // a representative step: the first one inside an undulator, if any
  int istep = 0;
  for (int i = 0; i < h->nsteps; i++)
    if (h->steps[i].aw > 0) {
      istep = i;
      break;
    }
  StateBackup b;
  int rc = backup_state(h, b);
  if (rc) return rc;
  bool fused = h->mixed && c.solver == G4GPU_SOLVER_ADI && c.ngrid <= g4::fused_max_ngrid();
  std::vector<int> pushes = {128, 256, 512};
  std::vector<int> fields = {512};
  if (fused) {
    fields.clear();
    int lo = (2 * c.ngrid + 31) / 32 * 32;
    for (int t : {lo, 512, 768, 1024})
      if (t >= lo && std::find(fields.begin(), fields.end(), t) == fields.end()) fields.push_back(t);
  }
  bool saved_graph = h->graph_mode, saved_prof = h->prof;
  h->graph_mode = false;
  h->prof = false;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_step = [&](int pb, int ft, float *ms, int fk = 0) -> int {
    h->push_block = pb;
    h->field_threads = ft;
    h->field_kernel = fk;
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {  // first repetition warms up
      restore_state(h, b, false);
      cudaEventRecord(e0, h->stream);
      int r = enqueue_steps(h, istep, 1, G4GPU_STAGE_ALL);
      if (r) return r;
      cudaEventRecord(e1, h->stream);
      cudaEventSynchronize(e1);
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0 && t < best) best = t;
    }
    *ms = best;
    return G4GPU_OK;
  };
  int best_pb = 256, best_ft = fields[0];
  float best_ms = 1e30f;
  for (int pb : pushes) {
    float ms;
    if ((rc = time_step(pb, best_ft, &ms))) break;
    if (ms < best_ms) {
      best_ms = ms;
      best_pb = pb;
    }
  }
  if (!rc && fields.size() > 1) {
    best_ms = 1e30f;
    for (int ft : fields) {
      float ms;
      if ((rc = time_step(best_pb, ft, &ms))) break;
      if (ms < best_ms) {
        best_ms = ms;
        best_ft = ft;
      }
    }
  }
  // the cluster-pair field kernel, where the step's segmented solves apply
  int best_fk = 0;
  bool pairable = fused;
  int band_w = 0;
  for (int k = 0; k < c.nfield; k++) {
    pairable = pairable && h->steps[istep].f[k].tw > 0;
    band_w = std::max(band_w, h->steps[istep].f[k].tw);
  }
  pairable = pairable && g4::band_cluster(c.ngrid, band_w) == 2;
  if (!rc && pairable) {
    float ms;
    if (!(rc = time_step(best_pb, best_ft, &ms))) {
      float single = ms;
      h->field_kernel = 1;
      float pms = 1e30f;
      for (int rep = 0; rep < 3 && !rc; rep++) {
        restore_state(h, b, false);
        cudaEventRecord(e0, h->stream);
        rc = enqueue_steps(h, istep, 1, G4GPU_STAGE_ALL);
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && t < pms) pms = t;
      }
      h->field_kernel = 0;
      if (!rc && pms < single) best_fk = 1;
    }
  }
  // the whole step in one kernel, over its CTA sizes (each with its own particles per
  // lane), against the best of the above
  if (!rc && fused && c.nfield == 1 && !h->sc_on) {
    float cur = 1e30f;
    if (!(rc = time_step(best_pb, best_ft, &cur, best_fk))) {
      int step_ft = 0;
      float step_ms = 1e30f;
      for (int ft : fields) {
        if (ft != (2 * c.ngrid + 31) / 32 * 32 && ft < 512) continue;
        float ms;
        if ((rc = time_step(best_pb, ft, &ms, 2))) break;
        if (ms < step_ms) {
          step_ms = ms;
          step_ft = ft;
        }
      }
      if (!rc && step_ms < cur) {
        best_fk = 2;
        best_ft = step_ft;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  restore_state(h, b, true);
  h->graph_mode = saved_graph;
  h->prof = saved_prof;
  std::memset(h->launches, 0, sizeof(h->launches));
  if (rc) return rc;
  h->push_block = best_pb;
  h->field_threads = best_ft;
  h->field_kernel = best_fk;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = {best_pb, best_ft, best_fk};
  }
  if (push_block) *push_block = best_pb;
  if (field_threads) *field_threads = best_ft;
  if (field_kernel) *field_kernel = best_fk;
  return check_device_flag(h);
}

// ---- batched ensembles ---------------------------------------------------------

// A batch: the members' handles, and the ensemble's step ranges as single CUDA graphs.
// One graph holds every member's steps of a range as parallel branches (forked from and
// joined into the batch's own stream), so the whole ensemble advances with one graph
// launch. Like a handle's own graphs it is valid for exactly the ring states (and launch
// shapes) it was captured from, which key it.
struct g4gpu_batch_ctx {
  std::vector<g4gpu_handle> members;
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr, post = nullptr;
  std::vector<cudaEvent_t> pre, join;
  struct Key {
    int istep0, nsteps, stages;
    std::vector<long long> state;  // per member: steps, launch shapes, first[], accuslip[] bits
    bool operator<(const Key &o) const {
      return std::tie(istep0, nsteps, stages, state) < std::tie(o.istep0, o.nsteps, o.stages, o.state);
    }
  };
  struct Entry {
    cudaGraphExec_t exec = nullptr;
    std::vector<std::vector<int>> end_first;
    std::vector<std::vector<double>> end_accuslip;
    std::vector<std::vector<long long>> launches;
  };
  std::map<Key, Entry> graphs;
  bool single_device = true;
};

extern "C" int g4gpu_batch_create(int nrun, const g4gpu_config *cfgs, g4gpu_batch *out) {
  if (!out || !cfgs || nrun < 1) return fail(nullptr, G4GPU_ERR_ARG, "bad batch arguments");
  *out = nullptr;
  g4gpu_batch b = new g4gpu_batch_ctx;
  for (int i = 0; i < nrun; i++) {
    g4gpu_handle h = nullptr;
    int rc = g4gpu_create(&cfgs[i], &h);
    if (rc) {
      for (auto m : b->members) g4gpu_destroy(m);
      delete b;
      return rc;
    }
    h->graph_mode = true;
    b->members.push_back(h);
    if (cfgs[i].device != cfgs[0].device) b->single_device = false;
  }
  if (b->single_device) {
    cudaSetDevice(cfgs[0].device);
    bool ok = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->post, cudaEventDisableTiming) == cudaSuccess;
    b->pre.assign(nrun, nullptr);
    b->join.assign(nrun, nullptr);
    for (int i = 0; i < nrun && ok; i++)
      ok = cudaEventCreateWithFlags(&b->pre[i], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      g4gpu_batch_destroy(b);
      return fail(nullptr, G4GPU_ERR_CUDA, "batch stream and events");
    }
  }
  *out = b;
  return G4GPU_OK;
}

extern "C" void g4gpu_batch_destroy(g4gpu_batch b) {
  if (!b) return;
  if (!b->members.empty()) cudaSetDevice(b->members[0]->cfg.device);
  for (auto &g : b->graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  for (cudaEvent_t e : b->pre)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->post) cudaEventDestroy(b->post);
  if (b->origin) cudaStreamDestroy(b->origin);
  for (auto m : b->members) g4gpu_destroy(m);
  delete b;
}

extern "C" g4gpu_handle g4gpu_batch_member(g4gpu_batch b, int i) {
  if (!b || i < 0 || i >= (int)b->members.size()) return nullptr;
  return b->members[i];
}

extern "C" int g4gpu_batch_run(g4gpu_batch b, int istep0, int nsteps, int stages) {
  if (!b || istep0 < 0 || nsteps < 0) return fail(nullptr, G4GPU_ERR_ARG, "bad batch arguments");
  const int nrun = (int)b->members.size();
  std::vector<int> nm(nrun);
  bool graph = b->single_device;
  for (int i = 0; i < nrun; i++) {
    g4gpu_handle m = b->members[i];
    nm[i] = std::max(0, std::min(nsteps, m->nsteps - istep0));
    graph = graph && m->graph_mode;
    if (nm[i] > 0) {
      if (!m->beam_loaded) return fail(nullptr, G4GPU_ERR_STATE, "batch member: no beam loaded");
      for (int k = 0; k < m->cfg.nfield; k++)
        if (!m->field_loaded[k]) return fail(nullptr, G4GPU_ERR_STATE, "batch member: a field is not loaded");
    }
  }
  if (!graph) {  // members on several devices, or graph mode off: one launch sequence per member
    for (int i = 0; i < nrun; i++) {
      if (nm[i] <= 0) continue;
      int rc = g4gpu_run(b->members[i], istep0, nm[i], stages);
      if (rc) {
        fail(nullptr, rc, std::string("batch member: ") + b->members[i]->err);
        return rc;
      }
    }
    return G4GPU_OK;
  }
  cudaSetDevice(b->members[0]->cfg.device);
  g4gpu_batch_ctx::Key key{istep0, nsteps, stages, {}};
  for (int i = 0; i < nrun; i++) {
    g4gpu_handle m = b->members[i];
    key.state.push_back(nm[i]);
    key.state.push_back(m->push_block);
    key.state.push_back(m->field_threads);
    key.state.push_back(m->field_kernel);
    key.state.push_back(m->graph_gen);  // the member's lattice and set-up the graph was captured with
    for (int k = 0; k < m->cfg.nfield; k++) {
      long long bits;
      std::memcpy(&bits, &m->accuslip[k], sizeof(bits));
      key.state.push_back(m->first[k]);
      key.state.push_back(bits);
    }
  }
  auto bfail = [&](cudaError_t e, const char *what) {
    return fail(nullptr, G4GPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    g4gpu_batch_ctx::Entry ent;
    std::vector<std::vector<long long>> before(nrun);
    for (int i = 0; i < nrun; i++) before[i].assign(b->members[i]->launches, b->members[i]->launches + G4GPU_K_NCLASS);
    cudaError_t e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bfail(e, "cudaStreamBeginCapture");
    cudaEventRecord(b->fork, b->origin);
    int rc = G4GPU_OK;
    for (int i = 0; i < nrun && !rc; i++) {
      g4gpu_handle m = b->members[i];
      if (nm[i] <= 0) continue;
      cudaStreamWaitEvent(m->stream, b->fork, 0);
      m->capturing = true;
      rc = enqueue_steps(m, istep0, nm[i], stages);
      m->capturing = false;
      cudaEventRecord(b->join[i], m->stream);
      cudaStreamWaitEvent(b->origin, b->join[i], 0);
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->origin, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return fail(nullptr, rc, "batch member: capture of its steps failed");
    }
    if (e != cudaSuccess) return bfail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&ent.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(e, "cudaGraphInstantiate");
    for (int i = 0; i < nrun; i++) {
      g4gpu_handle m = b->members[i];
      ent.end_first.emplace_back(m->first, m->first + m->cfg.nfield);
      ent.end_accuslip.emplace_back(m->accuslip, m->accuslip + m->cfg.nfield);
      std::vector<long long> d(G4GPU_K_NCLASS);
      for (int c = 0; c < G4GPU_K_NCLASS; c++) d[c] = m->launches[c] - before[i][c];
      ent.launches.push_back(d);
      // the capture advanced the counters without running anything
      std::memcpy(m->launches, before[i].data(), sizeof(long long) * G4GPU_K_NCLASS);
    }
    it = b->graphs.emplace(key, std::move(ent)).first;
  }
  // the graph follows the members' earlier work and their later work follows it
  for (int i = 0; i < nrun; i++) {
    cudaEventRecord(b->pre[i], b->members[i]->stream);
    cudaStreamWaitEvent(b->origin, b->pre[i], 0);
  }
  cudaError_t e = cudaGraphLaunch(it->second.exec, b->origin);
  if (e != cudaSuccess) return bfail(e, "cudaGraphLaunch");
  cudaEventRecord(b->post, b->origin);
  for (int i = 0; i < nrun; i++) {
    g4gpu_handle m = b->members[i];
    cudaStreamWaitEvent(m->stream, b->post, 0);
    for (int k = 0; k < m->cfg.nfield; k++) {
      m->first[k] = it->second.end_first[i][k];
      m->accuslip[k] = it->second.end_accuslip[i][k];
    }
    for (int c = 0; c < G4GPU_K_NCLASS; c++) m->launches[c] += it->second.launches[i][c];
  }
  return G4GPU_OK;
}

extern "C" int g4gpu_batch_synchronize(g4gpu_batch b) {
  if (!b) return fail(nullptr, G4GPU_ERR_ARG, "null batch");
  for (auto m : b->members) {
    int rc = g4gpu_synchronize(m);
    if (rc) {
      fail(nullptr, rc, std::string("batch member: ") + m->err);
      return rc;
    }
  }
  return G4GPU_OK;
}

// ---- ADI field step without device allocation ---------------------------------
// For callers that cannot call cudaMalloc (their device memory belongs to another
// allocator, or a cudaFree's device-wide synchronisation would stall their work in
// flight). Nothing here allocates device memory: the kernel's scratch, coefficients
// and error flag live in a static device array of the mixed-precision module, and
// the coefficients are computed on the host exactly as g4gpu_set_lattice computes
// them for a handle (adi_coefficients, FieldSolverADI::init).
extern "C" int g4gpu_adi_advance_noalloc(float *field, const float *source, int nslice, int ngrid,
                                         int first, double delz, double dgrid, double xks, int device,
                                         void *stream) {
  if (!field) return fail(nullptr, G4GPU_ERR_ARG, "null field");
  if (nslice < 1) return fail(nullptr, G4GPU_ERR_ARG, "nslice must be >= 1");
  if (ngrid < 3 || ngrid > G4GPU_NOALLOC_MAX_NGRID || ngrid > g4::fused_max_ngrid()) {
    char buf[160];
    snprintf(buf, sizeof(buf),
             "ngrid %d outside [3, %d]: a slice of ngrid^2 complex floats must fit in shared memory",
             ngrid, G4GPU_NOALLOC_MAX_NGRID);
    return fail(nullptr, G4GPU_ERR_ARG, buf);
  }
  if (first < 0 || first >= nslice) return fail(nullptr, G4GPU_ERR_ARG, "first must be in [0, nslice)");
  if (!std::isfinite(delz) || !(dgrid > 0) || !std::isfinite(dgrid) || !(xks > 0) || !std::isfinite(xks))
    return fail(nullptr, G4GPU_ERR_ARG, "delz must be finite, dgrid and xks finite and positive");
  if (reinterpret_cast<uintptr_t>(field) % 8 || (source && reinterpret_cast<uintptr_t>(source) % 8))
    return fail(nullptr, G4GPU_ERR_ARG, "field and source must be 8-byte aligned (complex float)");
  const size_t bytes = (size_t)nslice * ngrid * ngrid * 2 * sizeof(float);
  if (source) {
    uintptr_t f0 = reinterpret_cast<uintptr_t>(field), s0 = reinterpret_cast<uintptr_t>(source);
    if (f0 < s0 + bytes && s0 < f0 + bytes) return fail(nullptr, G4GPU_ERR_ARG, "source overlaps field");
  }
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  std::vector<std::complex<double>> cc, cb, cw;
  double cs = 0;
  adi_coefficients(delz, dgrid, xks, ngrid, cc, cb, cw, &cs);
  std::vector<float> coef(6 * (size_t)ngrid);
  const std::vector<std::complex<double>> *parts[3] = {&cc, &cb, &cw};
  for (int p = 0; p < 3; p++)
    for (int i = 0; i < ngrid; i++) {
      coef[2 * ((size_t)p * ngrid + i)] = static_cast<float>((*parts[p])[i].real());
      coef[2 * ((size_t)p * ngrid + i) + 1] = static_cast<float>((*parts[p])[i].imag());
    }
  std::string msg;
  int rc = g4::adi_noalloc_mixed(device, stream, field, source, coef.data(), static_cast<float>(cs), nslice,
                                 ngrid, first, &msg);
  if (prev >= 0 && prev != device) cudaSetDevice(prev);
  if (rc) return fail(nullptr, rc, msg);
  return G4GPU_OK;
}

}  // extern "C"
