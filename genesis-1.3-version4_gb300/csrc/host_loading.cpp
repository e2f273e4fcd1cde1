// Host-side initialisation of the beam and the radiation field, bit-exact with the
// reference: the quiet (Hammersley) loading, shot noise and Gauss-Hermite seed
// of GENESIS 1.3 v4.6.14. Compiled with -ffp-contract=off so that every
// floating-point operation rounds as the reference's do, and linked to the same
// C math library.
//
// Loading is initialisation, not the per-step hot path: the shot-noise stream is
// one sequential ran2 generator over all slices (src/Loading/LoadBeam.cpp:166-200)
// whose Bays-Durham shuffle table prevents skip-ahead, so it runs on the CPU. The
// per-slice quiet loading is independent across slices and runs on all host
// threads; only the shot-noise pass is sequential.
#include <cmath>
#include <complex>
#include <cstring>
#include <thread>
#include <vector>

#include "g4gpu.h"
#include "g4gpu_internal.h"

namespace g4 {
namespace {

// Numerical Recipes ran2 with Bays-Durham shuffle (src/Util/RandomU.cpp:17-73).
class Ran2 {
 public:
  explicit Ran2(unsigned int start) {
    const int ia1 = 40014, im1 = 2147483563, iq1 = 53668, ir1 = 12211;
    seed1_ = (1u < start) ? static_cast<int>(start) : 1;
    seed2_ = seed1_;
    for (int i = kTab + 7; i >= 0; i--) {
      int k = seed1_ / iq1;
      seed1_ = ia1 * (seed1_ - k * iq1) - k * ir1;
      if (seed1_ < 0) seed1_ += im1;
      if (i < kTab) table_[i] = seed1_;
    }
    last_ = table_[0];
  }
  double next() {
    const int ia1 = 40014, ia2 = 40692, im1 = 2147483563, im2 = 2147483399;
    const int imm1 = 2147483562, iq1 = 53668, iq2 = 52774, ir1 = 12211, ir2 = 3791;
    const int ndiv = 67108862;
    const double am = 1. / 2147483563;
    const double rnmx = 1. - 1.2e-40;
    int k = seed1_ / iq1;
    seed1_ = ia1 * (seed1_ - k * iq1) - k * ir1;
    if (seed1_ < 0) seed1_ += im1;
    k = seed2_ / iq2;
    seed2_ = ia2 * (seed2_ - k * iq2) - k * ir2;
    if (seed2_ < 0) seed2_ += im2;
    int j = last_ / ndiv;
    last_ = table_[j] - seed2_;
    table_[j] = seed1_;
    if (last_ < 1) last_ += imm1;
    return (am * last_ < rnmx) ? am * last_ : rnmx;
  }

 private:
  static constexpr int kTab = 32;
  int table_[kTab];
  int last_, seed1_, seed2_;
};

// Radical inverse in a prime base (src/Util/Hammerslay.cpp:15-49).
class RadicalInverse {
 public:
  RadicalInverse(int base_index, unsigned int start) : base_(kBases[base_index]), idx_(start) {}
  double next() {
    double xs = 0, xsi = 1.0;
    unsigned int i1, i2 = ++idx_;
    do {
      xsi = xsi / base_;
      i1 = i2 / static_cast<unsigned int>(base_);
      xs += (i2 - base_ * i1) * xsi;
      i2 = i1;
    } while (i2 > 0);
    return xs;
  }

 private:
  static constexpr double kBases[6] = {2, 3, 5, 7, 11, 13};
  double base_;
  unsigned int idx_;
};

// Inverse complementary error function after T. Ooura (src/Util/Inverfc.cpp:16-65).
double inv_erfc(double y) {
  double z = y > 1 ? 2 - y : y;
  double w = 0.916461398268964 - std::log(z);
  double u = std::sqrt(w);
  double s = (std::log(u) + 0.488826640273108) / w;
  double t = 1 / (u + 0.231729200323405);
  double x = u * (1 - s * (s * 0.124610454613712 + 0.5)) -
             ((((-0.0728846765585675 * t + 0.269999308670029) * t + 0.150689047360223) * t +
               0.116065025341614) * t + 0.499999303439796) * t;
  t = 3.97886080735226 / (x + 3.97886080735226);
  u = t - 0.5;
  s = (((((((((0.00112648096188977922 * u + 1.05739299623423047e-4) * u -
              0.00351287146129100025) * u - 7.71708358954120939e-4) * u +
            0.00685649426074558612) * u + 0.00339721910367775861) * u -
          0.011274916933250487) * u - 0.0118598117047771104) * u +
        0.0142961988697898018) * u + 0.0346494207789099922) * u + 0.00220995927012179067;
  s = ((((((((((((s * u - 0.0743424357241784861) * u - 0.105872177941595488) * u +
                0.0147297938331485121) * u + 0.316847638520135944) * u +
              0.713657635868730364) * u + 1.05375024970847138) * u +
            1.21448730779995237) * u + 1.16374581931560831) * u +
          0.956464974744799006) * u + 0.686265948274097816) * u +
        0.434397492331430115) * u + 0.244044510593190935) * t -
      z * std::exp(x * x - 0.120782237635245222);
  x = x + s * (x * s + 1);
  return y > 1 ? -x : x;
}

struct P6 {
  double gamma, theta, x, y, px, py;
};

struct SliceParams {
  double gamma, delgam, ex, ey, betax, betay, alphax, alphay, xcen, ycen, pxcen, pycen, bunch,
      bunchphase, emod, emodphase, current;
  explicit SliceParams(const double *p)
      : gamma(p[0]), delgam(p[1]), ex(p[2]), ey(p[3]), betax(p[4]), betay(p[5]), alphax(p[6]),
        alphay(p[7]), xcen(p[8]), ycen(p[9]), pxcen(p[10]), pycen(p[11]), bunch(p[12]),
        bunchphase(p[13]), emod(p[14]), emodphase(p[15]), current(p[16]) {}
};

// Normalises the first and second moments of one plane and removes its
// position-momentum correlation (QuietLoading.cpp:110-156).
void decorrelate(P6 *b, int mpart, double norm, double P6::*q, double P6::*pq) {
  double z = 0, zz = 0, p = 0, zp = 0;
  for (int i = 0; i < mpart; i++) {
    z += b[i].*q;
    zz += b[i].*q * b[i].*q;
    p += b[i].*pq;
    zp += b[i].*q * b[i].*pq;
  }
  z *= norm;
  p *= norm;
  zz = std::sqrt(std::fabs(zz * norm - z * z));
  if (zz > 0) zz = 1. / zz;
  zp = (zp * norm - z * p) * zz * zz;
  for (int i = 0; i < mpart; i++) {
    b[i].*pq = b[i].*pq - p;
    b[i].*pq -= zp * b[i].*q;
    b[i].*q = (b[i].*q - z) * zz;
  }
}

// QuietLoading::loadQuiet (src/Loading/QuietLoading.cpp:50-260) for one slice
// with the six Hammersley streams of bases 2, 3, 5, 7, 11, 13.
void load_quiet_slice(P6 *b, const SliceParams &sl, int npart, int nbins, double theta0,
                      int islice) {
  Ran2 reseed(static_cast<unsigned int>(islice));
  int iseed = static_cast<int>(std::round(reseed.next() * 1e9));
  RadicalInverse st(0, iseed), sg(1, iseed), sx(2, iseed), sy(3, iseed), spx(4, iseed),
      spy(5, iseed);
  int mpart = npart / nbins;
  double dtheta = 1. / static_cast<double>(nbins);
  for (int i = 0; i < mpart; i++) {
    b[i].theta = st.next() * dtheta;
    b[i].gamma = inv_erfc(2 * sg.next());
    b[i].x = inv_erfc(2 * sx.next());
    b[i].y = inv_erfc(2 * sy.next());
    b[i].px = inv_erfc(2 * spx.next());
    b[i].py = inv_erfc(2 * spy.next());
  }
  double norm = mpart > 0 ? 1. / static_cast<double>(mpart) : 0;
  double z = 0, zz = 0;
  for (int i = 0; i < mpart; i++) {
    z += b[i].gamma;
    zz += b[i].gamma * b[i].gamma;
  }
  z *= norm;
  zz = std::sqrt(std::fabs(zz * norm - z * z));
  if (zz > 0) zz = 1 / zz;
  zz *= sl.delgam;
  for (int i = 0; i < mpart; i++) b[i].gamma = (b[i].gamma - z) * zz + sl.gamma;

  decorrelate(b, mpart, norm, &P6::x, &P6::px);
  decorrelate(b, mpart, norm, &P6::y, &P6::py);

  double p = 0, pp = 0;
  z = 0;
  zz = 0;
  for (int i = 0; i < mpart; i++) {
    z += b[i].px;
    zz += b[i].px * b[i].px;
    p += b[i].py;
    pp += b[i].py * b[i].py;
  }
  z *= norm;
  p *= norm;
  zz = std::sqrt(std::fabs(zz * norm - z * z));
  if (zz > 0) zz = 1. / zz;
  pp = std::sqrt(std::fabs(pp * norm - p * p));
  if (pp > 0) pp = 1. / pp;
  for (int i = 0; i < mpart; i++) {
    b[i].px = (b[i].px - z) * zz;
    b[i].py = (b[i].py - p) * pp;
  }

  double sigx = std::sqrt(sl.ex * sl.betax / sl.gamma);
  double sigy = std::sqrt(sl.ey * sl.betay / sl.gamma);
  double sigpx = std::sqrt(sl.ex / sl.betax / sl.gamma);
  double sigpy = std::sqrt(sl.ey / sl.betay / sl.gamma);
  double corx = -sl.alphax / sl.betax, cory = -sl.alphay / sl.betay;
  for (int i = 0; i < mpart; i++) {
    b[i].x *= sigx;
    b[i].y *= sigy;
    b[i].px = sigpx * b[i].px + corx * b[i].x;
    b[i].py = sigpy * b[i].py + cory * b[i].y;
    b[i].px *= b[i].gamma;
    b[i].py *= b[i].gamma;
    b[i].x += sl.xcen;
    b[i].y += sl.ycen;
    b[i].px += sl.pxcen;
    b[i].py += sl.pycen;
  }
  // nbins mirrored beamlets, filled from the back so no record is overwritten early
  for (int i = mpart; i > 0; i--) {
    int i1 = i - 1, i2 = nbins * i1;
    for (int j = 0; j < nbins; j++) {
      P6 q = b[i1];
      q.theta = b[i1].theta + j * dtheta;
      b[i2 + j] = q;
    }
  }
  for (int i = 0; i < npart; i++) b[i].theta *= theta0;

  const double pi = 2 * std::asin(1.);
  double blocal = sl.bunch;
  if (blocal != 0) {
    // bisection for the sinc(pi (1 - b)) = bunch target (QuietLoading.cpp:230-245)
    double blow = 0, bupp = 0.9999, bmid = 0;
    while ((bupp - blow) > 1e-6) {
      bmid = 0.5 * (blow + bupp);
      double bprobe = std::sin((1 - bmid) * pi) / ((1 - bmid) * pi);
      if (sl.bunch < bprobe)
        bupp = bmid;
      else
        blow = bmid;
    }
    blocal = bmid;
  }
  if ((blocal != 0) || (sl.emod != 0)) {
    for (int i = 0; i < npart; i++) {
      b[i].gamma -= sl.emod * std::sin(b[i].theta - sl.emodphase);
      if (sl.bunch > 0.1)
        b[i].theta += -blocal * b[i].theta + blocal * pi + sl.bunchphase + pi;
      else
        b[i].theta -= 2 * sl.bunch * std::sin(b[i].theta - sl.bunchphase);
    }
  }
}

// ShotNoise::applyShotNoise (src/Loading/ShotNoise.cpp:29-68).
void shot_noise_slice(P6 *b, int npart, int nbins, double ne, Ran2 &ran, std::vector<double> &w) {
  if (ne <= 0) return;
  int mpart = npart / nbins;
  double nbl = ne / static_cast<double>(mpart);
  if (nbl < 1) nbl = 1;
  w.assign(npart, 0.0);
  const double twopi = 4 * std::asin(1.);
  for (int ih = 0; ih < (nbins - 1) / 2; ih++) {
    for (int i1 = 0; i1 < mpart; i1++) {
      double phi = 4 * std::asin(1) * ran.next();
      double an = std::sqrt(-std::log(ran.next()) / nbl) * 2 / static_cast<double>(ih + 1);
      if (an > twopi) an = std::fmod(an, twopi);
      for (int i2 = 0; i2 < nbins; i2++) {
        int idx = i1 * nbins + i2;
        w[idx] -= an * std::sin(b[idx].theta * (ih + 1) + phi);
      }
    }
  }
  for (int i = 0; i < npart; i++) b[i].theta += w[i];
}

// Bessel J0, J1 and Jn (src/Util/BesselJ.cpp), Numerical Recipes approximations.
double bessel_j0(double x) {
  if (std::fabs(x) < 8) {
    double y = x * x;
    return (57568490574.e0 + y * (-13362590354.e0 + y * (651619640.7e0 + y * (-11214424.18e0 + y * (77392.33017e0 + y * -184.9052456e0))))) /
           (57568490411.e0 + y * (1029532985.e0 + y * (9494680.718e0 + y * (59272.64853e0 + y * (267.8532712e0 + y * 1.e0)))));
  }
  double ax = std::fabs(x), z = 8 / ax, y = z * z, xx = ax - 0.785398164;
  return std::sqrt(0.636619772 / ax) *
         (std::cos(xx) * (1.e0 + y * (-.1098628627e-2 + y * (.2734510407e-4 + y * (-.2073370639e-5 + y * .2093887211e-6)))) -
          z * std::sin(xx) * (-.1562499995e-1 + y * (.1430488765e-3 + y * (-.6911147651e-5 + y * (.7621095161e-6 + y * -.934945152e-7)))));
}
double bessel_j1(double x) {
  if (std::fabs(x) < 8) {
    double y = x * x;
    return x * (72362614232.e0 + y * (-7895059235.e0 + y * (242396853.1e0 + y * (-2972611.439e0 + y * (15704.48260e0 + y * -30.16036606e0))))) /
           (144725228442.e0 + y * (2300535178.e0 + y * (18583304.74e0 + y * (99447.43394e0 + y * (376.9991397e0 + y * 1.e0)))));
  }
  double ax = std::fabs(x), z = 8 / ax, y = z * z, xx = ax - 2.356194491;
  return std::sqrt(0.636619772 / ax) *
         (std::cos(xx) * (1.e0 + y * (.183105e-2 + y * (-.3516396496e-4 + y * (.2457520174e-5 + y * -.240337019e-6)))) -
          z * std::sin(xx) * (.04687499995e0 + y * (-.2002690873e-3 + y * (.8449199096e-5 + y * (-.88228987e-6 + y * .105787412e-6)))));
}
double bessel_jn(int n, double x) {
  if (n == 0) return bessel_j0(x);
  if (n == 1) return bessel_j1(x);
  if (x == 0) return 0;
  double ax = std::fabs(x), bessj = 0;
  if (ax > static_cast<double>(n)) {
    double tox = 2 / ax, bjm = bessel_j0(ax), bj = bessel_j1(ax);
    for (int j = 1; j < n; j++) {
      double bjp = j * tox * bj - bjm;
      bjm = bj;
      bj = bjp;
    }
    bessj = bj;
  } else {
    double tox = 2. / ax;
    int m = static_cast<int>(2 * (n + std::floor(std::sqrt(static_cast<double>(40 * n))) / 2));
    int jsum = 0;
    double sum = 0, bjp = 0, bj = 1;
    for (int j = m; j > 0; j--) {
      double bjm = j * tox * bj - bjp;
      bjp = bj;
      bj = bjm;
      if (std::fabs(bj) > 1e10) {
        bj *= 1e-10;
        bjp *= 1e-10;
        bessj *= 1e-10;
        sum *= 1e-10;
      }
      if (jsum != 0) sum += bj;
      jsum = 1 - jsum;
      if (j == n) bessj = bjp;
    }
    sum = 2 * sum - bj;
    bessj = bessj / sum;
  }
  if ((x < 0) && ((n % 2) == 1)) bessj = -bessj;
  return bessj;
}

double hermite(double x, int n) {
  if (n <= 0) return 1;
  if (n == 1) return 2 * x;
  return 2. * x * hermite(x, n - 1) - 2 * (n - 1) * hermite(x, n - 2);
}
int factorial(int n) { return n <= 1 ? 1 : n * factorial(n - 1); }

}  // namespace

// Undulator::fc (src/Core/Undulator.cpp:141-167)
double host_fc(double aw, int helical, int h) {
  if (helical) return h == 1 ? aw : 0;
  double xi = aw * aw;
  xi = 0.5 * xi / (1 + xi) * static_cast<double>(h);
  if ((h % 2) == 1) {
    int h0 = (h - 1) / 2, h1 = h0 + 1;
    return aw * (bessel_jn(h0, xi) - bessel_jn(h1, xi)) * std::pow(-1., h0);
  }
  return 0;
}

}  // namespace g4

extern "C" {

double g4gpu_host_fc(double aw, int helical, int h) { return g4::host_fc(aw, helical, h); }

int g4gpu_host_load_beam(int nslice, int islice0, int npart, int nbins, int seed, int shotnoise,
                         double lambda0, double sample, const double *slicepar, double *out) {
  using namespace g4;
  if (nslice < 0 || npart < 1 || nbins < 1 || (npart % nbins) != 0 || !slicepar || !out)
    return G4GPU_ERR_ARG;
  P6 *all = reinterpret_cast<P6 *>(out);
  const double theta0 = 4. * std::asin(1.);
  // quiet loading: independent per slice, spread over the host threads
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  if (static_cast<unsigned>(nslice) < nt) nt = nslice > 0 ? nslice : 1;
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; t++) {
    pool.emplace_back([=]() {
      for (int j = static_cast<int>(t); j < nslice; j += static_cast<int>(nt))
        load_quiet_slice(all + static_cast<size_t>(j) * npart, SliceParams(slicepar + 17 * static_cast<size_t>(j)),
                         npart, nbins, theta0, islice0 + j);
    });
  }
  for (auto &th : pool) th.join();
  if (shotnoise) {
    // one ran2 stream over the slices in order: ShotNoise::init for rank 0 draws
    // once from ran2(seed) and seeds the stream with round(u * 1e9)
    Ran2 rseed(static_cast<unsigned int>(seed));
    double val = rseed.next() * 1e9;
    Ran2 ran(static_cast<unsigned int>(static_cast<int>(std::round(val))));
    std::vector<double> w;
    for (int j = 0; j < nslice; j++) {
      double ne = slicepar[17 * static_cast<size_t>(j) + 16] * lambda0 * sample / kCe;
      shot_noise_slice(all + static_cast<size_t>(j) * npart, npart, nbins, ne, ran, w);
    }
  }
  return G4GPU_OK;
}

int g4gpu_host_gauss_hermite(const double *par, double gridmax, int ngrid, double *out) {
  using namespace g4;
  if (!par || !out || ngrid < 2) return G4GPU_ERR_ARG;
  typedef std::complex<double> cd;
  double lambda = par[0], power = par[1], phase = par[2];
  double k = 4. * std::asin(1) / lambda * static_cast<double>(static_cast<int>(par[11]));
  double z0 = -par[3], w0 = par[4];
  int nx = static_cast<int>(par[9]), ny = static_cast<int>(par[10]);
  double zr = w0 * w0 * k * 0.5;
  double f0 = std::sqrt(k * zr / (zr * zr + z0 * z0));
  cd qz(-z0, zr);
  cd coef = cd(0, 1) * 0.5 * k / qz;
  double unit = std::sqrt(power * kVacimp) * k / kEev;
  double norm = f0 / std::sqrt(2. * std::asin(1.) * factorial(nx) * factorial(ny) * (1 << (nx + ny)));
  cd zscale = unit * norm * cd(std::cos(phase), std::sin(phase));
  double xmid = gridmax + par[5], ymid = gridmax + par[6];
  double dxy = 2. * gridmax / (ngrid - 1.);
  double kx = k * par[7], ky = k * par[8];
  cd *f = reinterpret_cast<cd *>(out);
  for (int iy = 0; iy < ngrid; iy++) {
    double y = iy * dxy - ymid;
    double hy = hermite(f0 * y, ny);
    double y2 = y * y, phiy = ky * y;
    for (int ix = 0; ix < ngrid; ix++) {
      double x = ix * dxy - xmid;
      double hx = hermite(f0 * x, nx);
      double r2 = y2 + x * x;
      cd phi(0, phiy + kx * x);
      f[iy * ngrid + ix] = zscale * std::exp(-coef * r2 + phi) * hx * hy;
    }
  }
  return G4GPU_OK;
}

}  // extern "C"
