// Single-particle longitudinal wakes for g4gpu_set_wake, computed on the host once per
// run: the resistive-wall, geometric (periodic gaps) and surface-roughness wakes of
// Wake::singleWakeResistive / singleWakeGeometric / singleWakeRoughness
// (src/Main/Wake.cpp:140-434).
//
// The numerical recipes are the reference's: the same k grid (1001 points up to
// 100 / s0), trapezoid weights, x grid of the flat-chamber integral (20000 points on
// [0, 15]), roughness quadrature (four segments of 128 / 1024 points) and the same
// order of every floating-point operation, so that the tables agree with the
// reference's to the last bit when both are built with the same compiler flags
// (-O2 -ffp-contract=off) against the same libm. The k points of the flat-chamber
// impedance, the cosine transform and the roughness integrals are independent per
// output point and run on several host threads; the threads do not change any sum.
#include <algorithm>
#include <cmath>
#include <complex>
#include <thread>
#include <vector>

#include "g4gpu.h"

namespace {

using cplx = std::complex<double>;

// constants of the reference (GenMain.cpp:63-68 and Wake.cpp)
constexpr double kZ0 = 376.73;            // vacimp
constexpr double kEC = 4.8032045e-11;     // ce
constexpr double kC = 299792458.0;        // speed of light
constexpr double kQe = 1.602176634e-19;   // elementary charge of the resistive wake's sign convention

// Runs f(i) for i in [0, n) on up to hardware_concurrency threads.
template <class F>
void parallel_for(int n, F f) {
  int nt = (int)std::max(1u, std::thread::hardware_concurrency());
  nt = std::min(nt, std::max(1, n / 8));
  if (nt <= 1) {
    for (int i = 0; i < n; i++) f(i);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++)
    th.emplace_back([=, &f] {
      for (int i = t; i < n; i += nt) f(i);
    });
  for (auto &x : th) x.join();
}

// sinh(x) / x, by its series 1 + x^2/6 + x^4/120 near 0
double sinhc(double x) {
  if (std::abs(x) < 1e-5) {
    const double x2 = x * x;
    return 1.0 + x2 * (1.0 / 6.0 + x2 * (1.0 / 120.0));
  }
  return std::sinh(x) / x;
}

// Leontovich surface impedance of a Drude conductor at wavenumber k:
// (1 - i) sqrt(k / (2 sigma(k) Z0)), sigma(k) = sigma0 / (1 - i k c tau)
cplx surface_impedance(double k, double sigma0, double ctau) {
  const cplx sigma = sigma0 / (cplx(1.0, 0.0) - cplx(0.0, 1.0) * k * ctau);
  const cplx ratio = cplx(k, 0.0) / (cplx(2.0, 0.0) * sigma * cplx(kZ0, 0.0));
  return cplx(1.0, -1.0) * std::sqrt(ratio);
}

// Resistive-wall wake (Bane & Stupakov, SLAC-PUB-10707): Re Z(k) of a round pipe of
// radius a, or of parallel plates of half gap a (integral over the transverse
// wavenumber x = q a), on k in [0, 100 / s0], then w(s) = (2c/pi) int Re Z cos(ks) dk,
// times the electron charge.
void wake_resistive(int ns, double ds, double a, double sigma0, double ctau, bool round, double *w) {
  for (int i = 0; i < ns; ++i) w[i] = 0.0;
  if (sigma0 <= 0.0) return;
  const double s0 = std::pow(2.0 * a * a / (kZ0 * sigma0), 1.0 / 3.0);
  const double pi = 2.0 * std::asin(1.0);
  const int nk = 1000;
  const double kmax = 100.0 / s0;
  const double dk = kmax / static_cast<double>(nk);
  const double pref = kZ0 / (2.0 * pi * a);

  std::vector<double> k(nk + 1), rez(nk + 1);
  for (int j = 0; j <= nk; ++j) k[j] = dk * static_cast<double>(j);

  if (round) {
    for (int j = 0; j <= nk; ++j) {
      if (k[j] == 0.0) {
        rez[j] = 0.0;
        continue;
      }
      const cplx zeta = surface_impedance(k[j], sigma0, ctau);
      const cplx den = cplx(1.0, 0.0) / zeta - cplx(0.0, 0.5 * k[j] * a);
      rez[j] = (std::isfinite(den.real()) && std::isfinite(den.imag())) ? (cplx(pref, 0.0) / den).real() : 0.0;
    }
  } else {
    const double xmax = 15.0;
    const int nq = 20000;
    const double dx = xmax / static_cast<double>(nq - 1);
    parallel_for(nk + 1, [&](int j) {
      const double kj = k[j];
      if (kj == 0.0) {
        rez[j] = 0.0;
        return;
      }
      const cplx zeta = surface_impedance(kj, sigma0, ctau);
      auto integrand = [&](double x) -> cplx {
        const double ch = std::cosh(x);
        const cplx den = cplx(ch, 0.0) * (cplx(ch, 0.0) / zeta + cplx(0.0, -kj * a * sinhc(x)));
        if (!std::isfinite(den.real()) || !std::isfinite(den.imag())) return cplx(0.0, 0.0);
        return cplx(pref, 0.0) / den;
      };
      cplx acc = integrand(0.0) * 0.5;
      for (int q = 1; q < nq - 1; ++q) acc += integrand(dx * static_cast<double>(q));
      acc += integrand(xmax) * 0.5;
      rez[j] = (acc * dx).real();
    });
  }

  rez.front() *= 0.5;
  rez.back() *= 0.5;
  const double cpref = (2.0 * kC / pi) * dk;
  parallel_for(ns, [&](int i) {
    const double s = i * ds;
    double acc = 0.0;
    for (int j = 0; j <= nk; ++j) acc += rez[j] * std::cos(k[j] * s);
    w[i] = acc * cpref;
  });
  for (int i = 0; i < ns; ++i) w[i] *= -kQe;
}

// Geometric wake of periodic gaps (length gap every lgap) in a round or flat chamber:
// coef sqrt(s), flat chambers scaled by 0.956
void wake_geometric(int ns, double ds, double a, double gap, double lgap, bool round, double *w) {
  for (int i = 0; i < ns; i++) w[i] = 0;
  if (gap <= 0) return;
  const double pi = 2. * std::asin(1.);
  double coef = -kZ0 * kEC / (pi * pi * a * lgap) * 2 * std::sqrt(0.5 * gap);
  if (!round) coef *= 0.956;
  for (int i = 0; i < ns; i++) w[i] = coef * std::sqrt(ds * i);
}

// Roughness kernel on `n` points from q1 to q2 with trapezoid end weights
void roughness_kernel(std::vector<cplx> &kern, int n, cplx q1, cplx q2, double r) {
  kern.resize(n);
  const cplx dq = (q2 - q1) / static_cast<double>(n - 1);
  const cplx I(0, 1);
  for (int j = 0; j < n; j++) {
    const cplx q = q1 + static_cast<double>(j) * dq;
    const cplx S = (std::sqrt(2. * q + 1.) - I * std::sqrt(2. * q - 1.)) * q / std::sqrt(4. * q * q - 1.);
    kern[j] = (S + 1.) / (1. - I * r * q * S) / (1. + I * r * q);
  }
  kern[0] *= 0.5;
  kern[n - 1] *= 0.5;
}

double roughness_integral(const std::vector<cplx> &kern, cplx q1, cplx q2, double tau) {
  const int n = (int)kern.size();
  const cplx dq = (q2 - q1) / static_cast<double>(n - 1);
  const cplx I(0, 1);
  cplx v(0., 0.);
  for (int j = 0; j < n; j++) {
    const cplx q = q1 + static_cast<double>(j) * dq;
    v += std::exp(-I * q * tau) * kern[j];
  }
  v *= dq;
  return v.real();
}

// Surface-roughness wake of a sinusoidal corrugation of height hrough and period
// lrough: a contour integral in the complex q plane in four straight segments
void wake_roughness(int ns, double ds, double a, double hrough, double lrough, double *w) {
  if (hrough <= 0) {
    for (int i = 0; i < ns; i++) w[i] = 0;
    return;
  }
  const double pi = 2. * std::asin(1);
  const double r = pi * pi * pi / lrough / lrough / lrough * hrough * hrough * a;
  const cplx q[5] = {cplx(0, 0), cplx(0, 2e-3), cplx(1, 2e-3), cplx(1, 0), cplx(100, 0)};
  const int n = 128, len[4] = {n, 8 * n, n, 8 * n};
  std::vector<cplx> kern[4];
  for (int s = 0; s < 4; s++) roughness_kernel(kern[s], len[s], q[s], q[s + 1], r);
  const double coef = r / pi * 4 / a / a * 1.6e-19 / 4 / pi / 8.854e-12;
  parallel_for(ns, [&](int i) {
    const double tau = 2 * pi * ds * i / lrough;
    double res = roughness_integral(kern[0], q[0], q[1], tau);
    for (int s = 1; s < 4; s++) res += roughness_integral(kern[s], q[s], q[s + 1], tau);
    w[i] = coef * res;
  });
}

}  // namespace

extern "C" int g4gpu_host_single_wakes(int ns, double ds, double radius, double conductivity, double relaxation,
                                       int roundpipe, double gap, double lgap, double hrough, double lrough,
                                       double *res, double *geo, double *rou) {
  if (ns < 1 || !(ds > 0) || !(radius > 0) || !res || !geo || !rou) return G4GPU_ERR_ARG;
  if (gap > 0 && !(lgap > 0)) return G4GPU_ERR_ARG;
  if (hrough > 0 && !(lrough > 0)) return G4GPU_ERR_ARG;
  wake_resistive(ns, ds, radius, conductivity, relaxation, roundpipe != 0, res);
  wake_geometric(ns, ds, radius, gap, lgap, roundpipe != 0, geo);
  wake_roughness(ns, ds, radius, hrough, lrough, rou);
  return G4GPU_OK;
}
