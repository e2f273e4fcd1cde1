/* g4oracle.c — plain-C FP64 restatement of the GENESIS 1.3 v4 undulator step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the product
 * never calls it. Compile with -ffp-contract=off so that every floating-point
 * operation rounds as the reference's (no fused multiply-add), and with C99
 * complex arithmetic, which GCC lowers exactly as it lowers std::complex<double>.
 * Citations are file:line in GENESIS 1.3 v4.6.14.
 */
#include "g4oracle.h"

#define _GNU_SOURCE
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

/* physical constants, GenMain.cpp:63-68 */
static const double kVacimp = 376.73;
static const double kEev = 510998.95069;
static const double kCe = 4.8032045e-11;
static const double kPi = 3.14159265358979323846;

/* ------------------------------------------------------------------------- */
/* host thread pool: a parallel-for over [0, n)                              */
/* ------------------------------------------------------------------------- */
typedef void (*range_fn)(void *ctx, int i0, int i1);
struct pf_arg {
  range_fn fn;
  void *ctx;
  int i0, i1;
};
static void *pf_thread(void *p) {
  struct pf_arg *a = (struct pf_arg *)p;
  a->fn(a->ctx, a->i0, a->i1);
  return NULL;
}
static void parallel_for(int n, int nthreads, range_fn fn, void *ctx) {
  if (nthreads <= 1 || n <= 1) {
    fn(ctx, 0, n);
    return;
  }
  if (nthreads > n) nthreads = n;
  pthread_t th[256];
  struct pf_arg args[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 0; t < nthreads; t++) {
    args[t].fn = fn;
    args[t].ctx = ctx;
    args[t].i0 = (int)((long long)n * t / nthreads);
    args[t].i1 = (int)((long long)n * (t + 1) / nthreads);
    pthread_create(&th[t], NULL, pf_thread, &args[t]);
  }
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------- */
/* random streams                                                            */
/* ------------------------------------------------------------------------- */
/* ran2 with Bays-Durham shuffle, RandomU.cpp:17-33 (seeding) and :46-73 (draw) */
typedef struct {
  int iv[32], iy, iseed, iseed2;
} ran2_t;

static void ran2_init(ran2_t *r, unsigned int istart) {
  const int ia1 = 40014, im1 = 2147483563, iq1 = 53668, ir1 = 12211, ntab = 32;
  /* RandomU.cpp:28: the comparison is unsigned, the stored seed an int */
  r->iseed = (1u < istart) ? (int)istart : 1;
  r->iseed2 = r->iseed;
  for (int i = ntab + 7; i >= 0; i--) {
    int k = r->iseed / iq1;
    r->iseed = ia1 * (r->iseed - k * iq1) - k * ir1;
    if (r->iseed < 0) r->iseed += im1;
    if (i < ntab) r->iv[i] = r->iseed;
  }
  r->iy = r->iv[0];
}

static double ran2_next(ran2_t *r) {
  const int ia1 = 40014, ia2 = 40692, im1 = 2147483563, im2 = 2147483399;
  const int imm1 = 2147483562, iq1 = 53668, iq2 = 52774, ir1 = 12211, ir2 = 3791;
  const int ndiv = 67108862;
  const double am = 1. / 2147483563;
  const double rnmx = 1. - 1.2e-40;
  int k = r->iseed / iq1;
  r->iseed = ia1 * (r->iseed - k * iq1) - k * ir1;
  if (r->iseed < 0) r->iseed = r->iseed + im1;
  k = r->iseed2 / iq2;
  r->iseed2 = ia2 * (r->iseed2 - k * iq2) - k * ir2;
  if (r->iseed2 < 0) r->iseed2 = r->iseed2 + im2;
  int j = r->iy / ndiv;
  r->iy = r->iv[j] - r->iseed2;
  r->iv[j] = r->iseed;
  if (r->iy < 1) r->iy = r->iy + imm1;
  return (am * r->iy < rnmx) ? am * r->iy : rnmx;
}

void orc_ran2(int seed, int n, double *out) {
  ran2_t r;
  ran2_init(&r, (unsigned int)seed);
  for (int i = 0; i < n; i++) out[i] = ran2_next(&r);
}

/* radical-inverse (Hammersley) sequence, Hammerslay.cpp:15-49 */
static const double kHamBases[26] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                     43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97, 101};
typedef struct {
  double base;
  unsigned int idx;
} ham_t;

static double ham_next(ham_t *h) {
  double xs = 0, xsi = 1.0;
  unsigned int i1, i2 = ++h->idx;
  do {
    xsi = xsi / h->base;
    i1 = i2 / (unsigned int)h->base;
    xs += (i2 - h->base * i1) * xsi;
    i2 = i1;
  } while (i2 > 0);
  return xs;
}

void orc_hammersley(int base_index, int start, int n, double *out) {
  ham_t h = {kHamBases[base_index], (unsigned int)start};
  for (int i = 0; i < n; i++) out[i] = ham_next(&h);
}

/* inverse erfc after T. Ooura, Inverfc.cpp:16-65 */
static double inverfc(double y) {
  double z = y;
  if (y > 1) z = 2 - y;
  double w = 0.916461398268964 - log(z);
  double u = sqrt(w);
  double s = (log(u) + 0.488826640273108) / w;
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
      z * exp(x * x - 0.120782237635245222);
  x = x + s * (x * s + 1);
  if (y > 1) x = -x;
  return x;
}

void orc_inverfc(int n, const double *in, double *out) {
  for (int i = 0; i < n; i++) out[i] = inverfc(in[i]);
}

/* ------------------------------------------------------------------------- */
/* Bessel functions and coupling, BesselJ.cpp and Undulator.cpp:141-167      */
/* ------------------------------------------------------------------------- */
static double bessj0(double x) {
  if (fabs(x) < 8) {
    double y = x * x;
    return (57568490574.e0 + y * (-13362590354.e0 + y * (651619640.7e0 + y * (-11214424.18e0 + y * (77392.33017e0 + y * -184.9052456e0))))) /
           (57568490411.e0 + y * (1029532985.e0 + y * (9494680.718e0 + y * (59272.64853e0 + y * (267.8532712e0 + y * 1.e0)))));
  }
  double ax = fabs(x), z = 8 / ax, y = z * z, xx = ax - 0.785398164;
  return sqrt(0.636619772 / ax) *
         (cos(xx) * (1.e0 + y * (-.1098628627e-2 + y * (.2734510407e-4 + y * (-.2073370639e-5 + y * .2093887211e-6)))) -
          z * sin(xx) * (-.1562499995e-1 + y * (.1430488765e-3 + y * (-.6911147651e-5 + y * (.7621095161e-6 + y * -.934945152e-7)))));
}

static double bessj1(double x) {
  if (fabs(x) < 8) {
    double y = x * x;
    return x * (72362614232.e0 + y * (-7895059235.e0 + y * (242396853.1e0 + y * (-2972611.439e0 + y * (15704.48260e0 + y * -30.16036606e0))))) /
           (144725228442.e0 + y * (2300535178.e0 + y * (18583304.74e0 + y * (99447.43394e0 + y * (376.9991397e0 + y * 1.e0)))));
  }
  double ax = fabs(x), z = 8 / ax, y = z * z, xx = ax - 2.356194491;
  return sqrt(0.636619772 / ax) *
         (cos(xx) * (1.e0 + y * (.183105e-2 + y * (-.3516396496e-4 + y * (.2457520174e-5 + y * -.240337019e-6)))) -
          z * sin(xx) * (.04687499995e0 + y * (-.2002690873e-3 + y * (.8449199096e-5 + y * (-.88228987e-6 + y * .105787412e-6)))));
}

double orc_besselj(int n, double x) {
  if (n == 0) return bessj0(x);
  if (n == 1) return bessj1(x);
  if (x == 0) return 0;
  double bessj = 0, ax = fabs(x);
  if (ax > (double)n) {
    /* upward recurrence */
    double tox = 2 / ax, bjm = bessj0(ax), bj = bessj1(ax);
    for (int j = 1; j < n; j++) {
      double bjp = j * tox * bj - bjm;
      bjm = bj;
      bj = bjp;
    }
    bessj = bj;
  } else {
    /* Miller's downward recurrence */
    double tox = 2. / ax;
    int m = (int)(2 * (n + floor(sqrt((double)(40 * n))) / 2));
    int jsum = 0;
    double sum = 0, bjp = 0, bj = 1;
    for (int j = m; j > 0; j--) {
      double bjm = j * tox * bj - bjp;
      bjp = bj;
      bj = bjm;
      if (fabs(bj) > 1e10) {
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

double orc_fc(double aw, int helical, int h) {
  double coup = aw;
  if (helical) return (h == 1) ? coup : 0;
  double xi = aw * aw;
  xi = 0.5 * xi / (1 + xi) * (double)h;
  if ((h % 2) == 1) {
    int h0 = (h - 1) / 2, h1 = h0 + 1;
    return coup * (orc_besselj(h0, xi) - orc_besselj(h1, xi)) * pow(-1., h0);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* beam loading, QuietLoading.cpp:50-260 and ShotNoise.cpp:16-68             */
/* ------------------------------------------------------------------------- */
typedef struct {
  double gamma, theta, x, y, px, py;
} part_t;

static void load_quiet(part_t *b, const double *sp, int npart, int nbins, double theta0,
                       int islice) {
  const double gamma0 = sp[0], delgam = sp[1], ex = sp[2], ey = sp[3], betax = sp[4],
               betay = sp[5], alphax = sp[6], alphay = sp[7], xcen = sp[8], ycen = sp[9],
               pxcen = sp[10], pycen = sp[11], bunch = sp[12], bunchphase = sp[13],
               emod = sp[14], emodphase = sp[15];
  ran2_t rs;
  ran2_init(&rs, (unsigned int)islice);
  int iseed = (int)round(ran2_next(&rs) * 1e9);
  ham_t st = {kHamBases[0], (unsigned)iseed}, sg = {kHamBases[1], (unsigned)iseed},
        sx = {kHamBases[2], (unsigned)iseed}, sy = {kHamBases[3], (unsigned)iseed},
        spx = {kHamBases[4], (unsigned)iseed}, spy = {kHamBases[5], (unsigned)iseed};
  int mpart = npart / nbins;
  double dtheta = 1. / (double)nbins;
  for (int i = 0; i < mpart; i++) {
    b[i].theta = ham_next(&st) * dtheta;
    b[i].gamma = inverfc(2 * ham_next(&sg));
    b[i].x = inverfc(2 * ham_next(&sx));
    b[i].y = inverfc(2 * ham_next(&sy));
    b[i].px = inverfc(2 * ham_next(&spx));
    b[i].py = inverfc(2 * ham_next(&spy));
  }
  double z = 0, zz = 0, norm = 0;
  if (mpart > 0) norm = 1. / (double)mpart;
  for (int i = 0; i < mpart; i++) {
    z += b[i].gamma;
    zz += b[i].gamma * b[i].gamma;
  }
  z *= norm;
  zz = sqrt(fabs(zz * norm - z * z));
  if (zz > 0) zz = 1 / zz;
  zz *= delgam;
  for (int i = 0; i < mpart; i++) b[i].gamma = (b[i].gamma - z) * zz + gamma0;

  /* x-px and y-py decorrelation, QuietLoading.cpp:110-156 */
  for (int plane = 0; plane < 2; plane++) {
    double p = 0, zp = 0;
    z = 0;
    zz = 0;
    for (int i = 0; i < mpart; i++) {
      double q = plane ? b[i].y : b[i].x, pq = plane ? b[i].py : b[i].px;
      z += q;
      zz += q * q;
      p += pq;
      zp += q * pq;
    }
    z *= norm;
    p *= norm;
    zz = sqrt(fabs(zz * norm - z * z));
    if (zz > 0) zz = 1. / zz;
    zp = (zp * norm - z * p) * zz * zz;
    for (int i = 0; i < mpart; i++) {
      double *q = plane ? &b[i].y : &b[i].x, *pq = plane ? &b[i].py : &b[i].px;
      *pq = *pq - p;
      *pq -= zp * *q;
      *q = (*q - z) * zz;
    }
  }
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
  zz = sqrt(fabs(zz * norm - z * z));
  if (zz > 0) zz = 1. / zz;
  pp = sqrt(fabs(pp * norm - p * p));
  if (pp > 0) pp = 1. / pp;
  for (int i = 0; i < mpart; i++) {
    b[i].px = (b[i].px - z) * zz;
    b[i].py = (b[i].py - p) * pp;
  }

  /* Twiss scaling, QuietLoading.cpp:185-203 */
  double sigx = sqrt(ex * betax / gamma0), sigy = sqrt(ey * betay / gamma0);
  double sigpx = sqrt(ex / betax / gamma0), sigpy = sqrt(ey / betay / gamma0);
  double corx = -alphax / betax, cory = -alphay / betay;
  for (int i = 0; i < mpart; i++) {
    b[i].x *= sigx;
    b[i].y *= sigy;
    b[i].px = sigpx * b[i].px + corx * b[i].x;
    b[i].py = sigpy * b[i].py + cory * b[i].y;
    b[i].px *= b[i].gamma;
    b[i].py *= b[i].gamma;
    b[i].x += xcen;
    b[i].y += ycen;
    b[i].px += pxcen;
    b[i].py += pycen;
  }
  /* beamlet mirroring, QuietLoading.cpp:207-218 */
  for (int i = mpart; i > 0; i--) {
    int i1 = i - 1, i2 = nbins * i1;
    for (int j = 0; j < nbins; j++) {
      b[i2 + j].gamma = b[i1].gamma;
      b[i2 + j].x = b[i1].x;
      b[i2 + j].y = b[i1].y;
      b[i2 + j].px = b[i1].px;
      b[i2 + j].py = b[i1].py;
      b[i2 + j].theta = b[i1].theta + j * dtheta;
    }
  }
  for (int i = 0; i < npart; i++) b[i].theta *= theta0;

  /* optional bunching / energy modulation, QuietLoading.cpp:227-259 */
  double pi = 2 * asin(1.);
  double blocal = bunch;
  if (blocal != 0) {
    double btar = blocal, blow = 0, bupp = 0.9999, bmid = 0;
    while ((bupp - blow) > 1e-6) {
      bmid = 0.5 * (blow + bupp);
      double bprobe = sin((1 - bmid) * pi) / ((1 - bmid) * pi);
      if (btar < bprobe)
        bupp = bmid;
      else
        blow = bmid;
    }
    blocal = bmid;
  }
  if ((blocal != 0) || (emod != 0)) {
    if (bunch > 0.1) {
      for (int i = 0; i < npart; i++) {
        b[i].gamma -= emod * sin(b[i].theta - emodphase);
        b[i].theta += -blocal * b[i].theta + blocal * pi + bunchphase + pi;
      }
    } else {
      for (int i = 0; i < npart; i++) {
        b[i].gamma -= emod * sin(b[i].theta - emodphase);
        b[i].theta -= 2 * bunch * sin(b[i].theta - bunchphase);
      }
    }
  }
}

static void shot_noise(part_t *b, int npart, int nbins, double ne, ran2_t *sran, double *work) {
  if (ne <= 0) return;
  int mpart = npart / nbins;
  double nbl = ne / (double)mpart;
  if (nbl < 1) nbl = 1;
  for (int i = 0; i < npart; i++) work[i] = 0;
  double twopi = 4 * asin(1.);
  for (int ih = 0; ih < (nbins - 1) / 2; ih++) {
    for (int i1 = 0; i1 < mpart; i1++) {
      double phi = 4 * asin(1) * ran2_next(sran);
      double an = sqrt(-log(ran2_next(sran)) / nbl) * 2 / (double)(ih + 1);
      if (an > twopi) an = fmod(an, twopi);
      for (int i2 = 0; i2 < nbins; i2++) {
        int idx = i1 * nbins + i2;
        work[idx] -= an * sin(b[idx].theta * (ih + 1) + phi);
      }
    }
  }
  for (int i = 0; i < npart; i++) b[i].theta += work[i];
}

void orc_load_beam(int nslice, int islice0, int npart, int nbins, int seed, int shotnoise,
                   double lambda, double sample, const double *slicepar, double *out) {
  /* ShotNoise::init for rank 0: one draw from ran2(seed), ShotNoise.cpp:16-27 */
  ran2_t rseed, sran;
  ran2_init(&rseed, (unsigned int)seed);
  double val = ran2_next(&rseed) * 1e9;
  ran2_init(&sran, (unsigned int)(int)round(val));
  part_t *b = (part_t *)malloc(sizeof(part_t) * (size_t)npart);
  double *work = (double *)malloc(sizeof(double) * (size_t)npart);
  for (int j = 0; j < nslice; j++) {
    const double *sp = slicepar + (size_t)j * 17;
    double ne = sp[16] * lambda * sample / kCe;
    load_quiet(b, sp, npart, nbins, 4. * asin(1.), islice0 + j);
    if (shotnoise) shot_noise(b, npart, nbins, ne, &sran, work);
    memcpy(out + (size_t)j * npart * 6, b, sizeof(part_t) * (size_t)npart);
  }
  free(work);
  free(b);
}

/* Gauss-Hermite mode, GaussHermite.cpp:20-85 */
static double hn(double x, int n) {
  if (n <= 0) return 1;
  if (n == 1) return 2 * x;
  return 2. * x * hn(x, n - 1) - 2 * (n - 1) * hn(x, n - 2);
}
static int fac(int n) { return n <= 1 ? 1 : n * fac(n - 1); }

void orc_gauss_hermite(const double *par, double gridmax, int ngrid, double *out) {
  double lambda = par[0], power = par[1], phase = par[2], z0in = par[3], w0 = par[4];
  double xcen = par[5], ycen = par[6], xangle = par[7], yangle = par[8];
  int nx = (int)par[9], ny = (int)par[10], harm = (int)par[11];
  double k = 4. * asin(1) / lambda * (double)harm;
  double z0 = -z0in;
  double zr = w0 * w0 * k * 0.5;
  double f0 = sqrt(k * zr / (zr * zr + z0 * z0));
  cplx qz = CMPLX(-z0, zr);
  cplx coef = CMPLX(0, 1) * 0.5 * k / qz;
  double unit = sqrt(power * kVacimp) * k / kEev;
  double norm = f0 / sqrt(2. * asin(1.) * fac(nx) * fac(ny) * (1 << (nx + ny)));
  cplx zscale = unit * norm * CMPLX(cos(phase), sin(phase));
  double xmid = gridmax + xcen, ymid = gridmax + ycen;
  double dxy = 2. * gridmax / (ngrid - 1.);
  double kx = k * xangle, ky = k * yangle;
  cplx *f = (cplx *)out;
  for (int iy = 0; iy < ngrid; iy++) {
    double y = iy * dxy - ymid;
    double hy = hn(f0 * y, ny);
    double y2 = y * y;
    double phiy = ky * y;
    for (int ix = 0; ix < ngrid; ix++) {
      double x = ix * dxy - xmid;
      double hx = hn(f0 * x, nx);
      double r2 = y2 + x * x;
      cplx phi = CMPLX(0, phiy + kx * x);
      f[iy * ngrid + ix] = zscale * cexp(-coef * r2 + phi) * hx * hy;
    }
  }
}

/* ------------------------------------------------------------------------- */
/* the integration step                                                      */
/* ------------------------------------------------------------------------- */
typedef struct {
  double aw, ax, ay, ku, kx, ky, gradx, grady, qf, qx, qy, cx, cy, dz, slip, phase, z;
  int helical;
  /* chicane: bend angle (0: none), dipole length, spacing, total length */
  double angle, lb, ld, lt;
} step_t;

/* chicanes of the following orc_run_steps calls: [n][4] angle, lb, ld, lt per row of
 * the lattice passed there */
static double *chic_tab = NULL;
static int chic_n = 0;

void orc_set_chicanes(int nsteps, const double *tab) {
  free(chic_tab);
  chic_tab = NULL;
  chic_n = 0;
  if (nsteps <= 0 || !tab) return;
  chic_tab = malloc(sizeof(double) * 4 * nsteps);
  memcpy(chic_tab, tab, sizeof(double) * 4 * nsteps);
  chic_n = nsteps;
}

static step_t get_step(const double *lat, int i) {
  const double *r = lat + (size_t)i * G4_LAT_NCOL;
  step_t s;
  s.angle = s.lb = s.ld = s.lt = 0;
  if (i < chic_n) {
    s.angle = chic_tab[4 * i];
    s.lb = chic_tab[4 * i + 1];
    s.ld = chic_tab[4 * i + 2];
    s.lt = chic_tab[4 * i + 3];
  }
  s.aw = r[G4_LAT_AW]; s.ax = r[G4_LAT_AX]; s.ay = r[G4_LAT_AY]; s.ku = r[G4_LAT_KU];
  s.kx = r[G4_LAT_KX]; s.ky = r[G4_LAT_KY]; s.gradx = r[G4_LAT_GRADX];
  s.grady = r[G4_LAT_GRADY]; s.qf = r[G4_LAT_QF]; s.qx = r[G4_LAT_QX]; s.qy = r[G4_LAT_QY];
  s.cx = r[G4_LAT_CX]; s.cy = r[G4_LAT_CY]; s.dz = r[G4_LAT_DZ]; s.slip = r[G4_LAT_SLIP];
  s.phase = r[G4_LAT_PHASE]; s.z = r[G4_LAT_Z];
  s.helical = r[G4_LAT_HELICAL] != 0;
  return s;
}

/* Undulator::faw / faw2, Undulator.cpp:170-182 */
static double faw(const step_t *u, double x, double y) {
  double dx = x - u->ax, dy = y - u->ay;
  return (1 + 0.5 * (u->kx * dx * dx + u->ky * dy * dy) + u->gradx * dx + u->grady * dy);
}
static double faw2(const step_t *u, double x, double y) {
  double dx = x - u->ax, dy = y - u->ay;
  return (1 + u->kx * dx * dx + u->ky * dy * dy + 2 * (u->gradx * dx + u->grady * dy));
}

/* Field::getLLGridpoint, Field.cpp:160-174 */
static int ll_gridpoint(double gridmax, double dgrid, int ngrid, double x, double y,
                        double *wx, double *wy, int *idx) {
  if ((x > -gridmax) && (x < gridmax) && (y > -gridmax) && (y < gridmax)) {
    *wx = (x + gridmax) / dgrid;
    *wy = (y + gridmax) / dgrid;
    int ix = (int)floor(*wx), iy = (int)floor(*wy);
    *wx = 1 + floor(*wx) - *wx;
    *wy = 1 + floor(*wy) - *wy;
    *idx = ix + iy * ngrid;
    return 1;
  }
  return 0;
}

typedef struct {
  int ns, npart, nfld, ngrid;
  part_t *beam;
  const double *current;
  cplx *fields;
  const int *harm;
  const int *first;
  const double *gridmax;
  double reflength;
  double gammaref;
  step_t st;
  double delz;
  /* push */
  double xks_fund, xku, rtmp[8], rharm[8];
  /* field solve */
  int ifld;
  int solver;
  double filt[3];
  cplx *cbet, *cwet, *cc, cstep;
  cplx *k2, *sigm;
  /* space charge: the slice's short-range field per particle and its long-range loss */
  const double *sc_ez;
  double sc_eloss;
  /* wakes: the loss of every slice (eV/m), NULL without &wake */
  const double *wake_loss;
  /* one4one windows: particles per slice (npart is then a slice's capacity), NULL when
   * every slice holds npart */
  const int *count;
} step_ctx;

/* the particles of slice is */
static int np_of(const step_ctx *c, int is) { return c->count ? c->count[is] : c->npart; }

/* TrackBeam::track, TrackBeam.cpp:8-116 (no chicane: the lattice has none) */
typedef struct {
  double q, off;
  int kind; /* 0 drift, 1 focusing, 2 defocusing */
} plane_t;

static void transverse_setup(const step_t *u, double gamma0, plane_t *px, plane_t *py,
                             double *aw_out) {
  int inund = u->aw > 0;
  double aw = inund ? u->aw : 0, dax = inund ? u->ax : 0, day = inund ? u->ay : 0;
  double kx = inund ? u->kx : 0, ky = inund ? u->ky : 0;
  double qf = u->qf, dqx = qf == 0 ? 0 : u->qx, dqy = qf == 0 ? 0 : u->qy;
  double betpar0 = sqrt(1 - (1 + aw * aw) / gamma0 / gamma0);
  double qquad = qf * gamma0;
  double qnatx = kx * aw * aw / gamma0 / betpar0;
  double qnaty = ky * aw * aw / gamma0 / betpar0;
  double qx = qquad + qnatx, qy = -qquad + qnaty;
  double xoff = qquad * dqx + qnatx * dax;
  double yoff = -qquad * dqy + qnaty * day;
  px->q = qx;
  py->q = qy;
  if (qx == 0) {
    px->kind = 0;
    px->off = xoff;
  } else {
    px->off = xoff / qx;
    px->kind = qx > 0 ? 1 : 2;
  }
  if (qy == 0) {
    py->kind = 0;
    py->off = yoff;
  } else {
    py->off = yoff / qy;
    py->kind = qy > 0 ? 1 : 2;
  }
  *aw_out = aw;
}

static void apply_plane(const plane_t *pl, double delz, double *x, double *p, double gammaz) {
  if (pl->kind == 0) {
    *x += (*p) * delz / gammaz;
  } else if (pl->kind == 1) {
    double foc = sqrt(pl->q / gammaz), omg = foc * delz;
    double a1 = cos(omg), a2 = sin(omg) / foc, a3 = -a2 * foc * foc;
    double xtmp = *x - pl->off;
    *x = a1 * xtmp + a2 * (*p) / gammaz + pl->off;
    *p = a3 * xtmp * gammaz + a1 * (*p);
  } else {
    double foc = sqrt(-pl->q / gammaz), omg = foc * delz;
    double a1 = cosh(omg), a2 = sinh(omg) / foc, a3 = a2 * foc * foc;
    double xtmp = *x - pl->off;
    *x = a1 * xtmp + a2 * (*p) / gammaz + pl->off;
    *p = a3 * xtmp * gammaz + a1 * (*p);
  }
}

/* TrackBeam::matmul, TrackBeam.cpp:246-258: m = e m */
static void mat4_mul(double m[4][4], double e[4][4]) {
  double t[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      t[i][j] = 0;
      for (int k = 0; k < 4; k++) t[i][j] += e[i][k] * m[k][j];
    }
  memcpy(m, t, sizeof(t));
}

/* The chicane's transfer matrix and the drift back over its length,
 * TrackBeam::applyChicane, TrackBeam.cpp:131-222 */
static void chicane_transfer(const step_t *u, double m[4][4]) {
  double d1[4][4], d2[4][4], d3[4][4], bp[4][4], bn[4][4], ep[4][4], en[4][4];
  double(*all[8])[4] = {m, d1, d2, d3, bp, bn, ep, en};
  for (int a = 0; a < 8; a++)
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) all[a][i][j] = i == j ? 1 : 0;
  double angle = u->angle, lb = u->lb, ld = u->ld, lt = u->lt;
  d1[0][1] = ld / cos(angle);
  d1[2][3] = ld / cos(angle);
  d2[0][1] = lt - 4 * lb - 2 * ld;
  d2[2][3] = lt - 4 * lb - 2 * ld;
  d3[0][1] = -lt;
  d3[2][3] = -lt;
  double R = lb / sin(angle), Lpath = R * angle;
  bp[2][3] = Lpath;
  bp[0][0] = cos(angle);
  bp[0][1] = R * sin(angle);
  bp[1][0] = -sin(angle) / R;
  bp[1][1] = cos(angle);
  bn[2][3] = Lpath;
  bn[0][0] = cos(-angle);
  bn[0][1] = R * sin(-angle) * -1;
  bn[1][0] = -sin(-angle) / R * -1;
  bn[1][1] = cos(-angle);
  double efoc = tan(angle) / R;
  ep[1][0] = efoc;
  ep[3][2] = -efoc;
  en[1][0] = -efoc * -1;
  en[3][2] = efoc * -1;
  double(*seq[12])[4] = {bp, ep, d1, en, bn, d2, bn, en, d1, ep, bp, d3};
  for (int a = 0; a < 12; a++) mat4_mul(m, seq[a]);
}

static void transverse_slices(step_ctx *c, int is0, int is1, int last) {
  plane_t pxp, pyp;
  double aw;
  transverse_setup(&c->st, c->gammaref, &pxp, &pyp, &aw);
  double delz = c->delz * 0.5;
  double cxk = c->st.cx * c->gammaref, cyk = c->st.cy * c->gammaref;
  int corr = last && ((c->st.cx != 0) || (c->st.cy != 0));
  int chic = !last && c->st.angle != 0;
  double m[4][4];
  if (chic) chicane_transfer(&c->st, m);
  for (int is = is0; is < is1; is++) {
    part_t *b = c->beam + (size_t)is * c->npart;
    for (int j = 0; j < np_of(c, is); j++) {
      part_t *p = b + j;
      if (corr) {
        p->px += cxk;
        p->py += cyk;
      }
      if (chic) {
        double gz = sqrt(p->gamma * p->gamma - 1 - p->px * p->px - p->py * p->py);
        double tmp = p->x;
        p->x = m[0][0] * tmp + m[0][1] * p->px / gz;
        p->px = m[1][0] * tmp * gz + m[1][1] * p->px;
        tmp = p->y;
        p->y = m[2][2] * tmp + m[2][3] * p->py / gz;
        p->py = m[3][2] * tmp * gz + m[3][3] * p->py;
      }
      double gammaz = sqrt(p->gamma * p->gamma - 1 - aw * aw - p->px * p->px - p->py * p->py);
      apply_plane(&pxp, delz, &p->x, &p->px, gammaz);
      apply_plane(&pyp, delz, &p->y, &p->py, gammaz);
    }
  }
}

/* BeamSolver::ODE, BeamSolver.cpp:144-163 */
static void ode(const step_ctx *c, int nf, const cplx *rpart, double btpar, double ez,
                double tgam, double tthet, double *k2gg, double *k2pp) {
  double ztemp1 = -2. / c->xks_fund;
  cplx ctmp = 0;
  for (int i = 0; i < nf; i++)
    ctmp += rpart[i] * CMPLX(cos(c->rharm[i] * tthet), -sin(c->rharm[i] * tthet));
  double btper0 = btpar + ztemp1 * creal(ctmp);
  double btpar0 = sqrt(1. - btper0 / (tgam * tgam));
  *k2pp += c->xks_fund * (1. - 1. / btpar0) + c->xku;
  *k2gg += cimag(ctmp) / btpar0 / tgam - ez;
}

/* BeamSolver::advance + RungeKutta, BeamSolver.cpp:13-141 */
static void push_slices(step_ctx *c, int is0, int is1) {
  const step_t *u = &c->st;
  double aw = u->aw, autophase = u->phase, delz = c->delz;
  size_t ncell = (size_t)c->ngrid * c->ngrid;
  for (int is = is0; is < is1; is++) {
    part_t *b = c->beam + (size_t)is * c->npart;
    for (int ip = 0; ip < np_of(c, is); ip++) {
      part_t *p = b + ip;
      double gamma = p->gamma, theta = p->theta + autophase;
      double x = p->x, y = p->y, px = p->px, py = p->py;
      double awloc = faw(u, x, y);
      double btpar = 1 + px * px + py * py + aw * aw * awloc * awloc;
      /* BeamSolver.cpp:61: the short-range field of the particle plus the slice's
       * long-range loss */
      double ez = c->sc_ez ? c->sc_ez[ip] + c->sc_eloss : 0;
      cplx rpart[8];
      for (int k = 0; k < c->nfld; k++) {
        int ns = c->ns;
        size_t islice = (size_t)((is + c->first[k]) % ns);
        const cplx *f = c->fields + ((size_t)k * ns + islice) * ncell;
        double gm = c->gridmax[k], dg = 2 * gm / (double)(c->ngrid - 1);
        double wx, wy;
        int idx;
        if (ll_gridpoint(gm, dg, c->ngrid, x, y, &wx, &wy, &idx)) {
          cplx cpart = f[idx] * wx * wy;
          idx++;
          cpart += f[idx] * (1 - wx) * wy;
          idx += c->ngrid - 1;
          cpart += f[idx] * wx * (1 - wy);
          idx++;
          cpart += f[idx] * (1 - wx) * (1 - wy);
          rpart[k] = c->rtmp[k] * awloc * conj(cpart);
        } else {
          rpart[k] = 0;
        }
      }
      /* RungeKutta, BeamSolver.cpp:89-141 */
      double k2gg = 0, k2pp = 0, k3gg, k3pp;
      ode(c, c->nfld, rpart, btpar, ez, gamma, theta, &k2gg, &k2pp);
      double stpz = 0.5 * delz;
      gamma += stpz * k2gg;
      theta += stpz * k2pp;
      k3gg = k2gg;
      k3pp = k2pp;
      k2gg = 0;
      k2pp = 0;
      ode(c, c->nfld, rpart, btpar, ez, gamma, theta, &k2gg, &k2pp);
      gamma += stpz * (k2gg - k3gg);
      theta += stpz * (k2pp - k3pp);
      k3gg /= 6;
      k3pp /= 6;
      k2gg *= -0.5;
      k2pp *= -0.5;
      ode(c, c->nfld, rpart, btpar, ez, gamma, theta, &k2gg, &k2pp);
      stpz = delz;
      gamma += stpz * k2gg;
      theta += stpz * k2pp;
      k3gg -= k2gg;
      k3pp -= k2pp;
      k2gg *= 2;
      k2pp *= 2;
      ode(c, c->nfld, rpart, btpar, ez, gamma, theta, &k2gg, &k2pp);
      gamma += stpz * (k3gg + k2gg / 6.0);
      theta += stpz * (k3pp + k2pp / 6.0);
      p->gamma = gamma;
      p->theta = theta;
    }
  }
}

/* source deposition, FieldSolverADI.cpp:13-52 (identical in FieldSolverFFT.cpp:13-52) */
static void deposit(const step_ctx *c, int ii, cplx *src) {
  int ng = c->ngrid;
  size_t ncell = (size_t)ng * ng;
  for (size_t i = 0; i < ncell; i++) src[i] = 0;
  int harm = c->harm[c->ifld];
  if (!(c->st.aw > 0) || (harm % 2 != 1)) return;
  double gm = c->gridmax[c->ifld], dgrid = 2 * gm / (double)(ng - 1);
  double xks = 4. * asin(1) / (c->reflength / (double)harm);
  double scl = orc_fc(c->st.aw, c->st.helical, harm) * kVacimp * c->current[ii] * xks * c->delz;
  /* the slice's own particle count (FieldSolverADI.cpp:27) */
  scl /= 4 * kEev * (double)np_of(c, ii) * dgrid * dgrid;
  const part_t *b = c->beam + (size_t)ii * c->npart;
  for (int ip = 0; ip < np_of(c, ii); ip++) {
    double x = b[ip].x, y = b[ip].y, theta = (double)harm * b[ip].theta, gamma = b[ip].gamma;
    double wx, wy;
    int idx;
    if (ll_gridpoint(gm, dgrid, ng, x, y, &wx, &wy, &idx)) {
      double part = sqrt(faw2(&c->st, x, y)) * scl / gamma;
      cplx cpart = CMPLX(sin(theta), cos(theta)) * part;
      double weight = wx * wy;
      src[idx] += weight * cpart;
      weight = (1 - wx) * wy;
      idx++;
      src[idx] += weight * cpart;
      weight = wx * (1 - wy);
      idx += ng - 1;
      src[idx] += weight * cpart;
      weight = (1 - wx) * (1 - wy);
      idx++;
      src[idx] += weight * cpart;
    }
  }
}

/* Crank-Nicolson ADI, FieldSolverADI.cpp:60-122 */
static void adi(const step_ctx *c, cplx *u, const cplx *src, cplx *r) {
  int ng = c->ngrid;
  cplx cstep = c->cstep;
  const cplx *cc = c->cc, *cbet = c->cbet, *cwet = c->cwet;
  int idx;
  for (idx = 0; idx < ng; idx++)
    r[idx] = src[idx] + u[idx] + cstep * (u[idx + ng] - 2.0 * u[idx]);
  for (idx = ng; idx < ng * (ng - 1); idx++)
    r[idx] = src[idx] + u[idx] + cstep * (u[idx + ng] - 2.0 * u[idx] + u[idx - ng]);
  for (idx = ng * (ng - 1); idx < ng * ng; idx++)
    r[idx] = src[idx] + u[idx] + cstep * (u[idx - ng] - 2.0 * u[idx]);
  /* tridagx */
  for (int i = 0; i < ng * ng; i += ng) {
    u[i] = r[i] * cbet[0];
    for (int k = 1; k < ng; k++) u[k + i] = (r[k + i] - cc[k] * u[k + i - 1]) * cbet[k];
    for (int k = ng - 2; k >= 0; k--) u[k + i] -= cwet[k + 1] * u[k + i + 1];
  }
  for (int ix = 0; ix < ng * ng; ix += ng) {
    idx = ix;
    r[idx] = src[idx] + u[idx] + cstep * (u[idx + 1] - 2.0 * u[idx]);
    for (idx = ix + 1; idx < ix + ng - 1; idx++)
      r[idx] = src[idx] + u[idx] + cstep * (u[idx + 1] - 2.0 * u[idx] + u[idx - 1]);
    idx = ix + ng - 1;
    r[idx] = src[idx] + u[idx] + cstep * (u[idx - 1] - 2.0 * u[idx]);
  }
  /* tridagy */
  for (int i = 0; i < ng; i++) u[i] = r[i] * cbet[0];
  for (int k = 1; k < ng; k++) {
    int n = k * ng;
    for (int i = 0; i < ng; i++) u[n + i] = (r[n + i] - cc[k] * u[n + i - ng]) * cbet[k];
  }
  for (int k = ng - 2; k >= 0; k--) {
    int n = k * ng;
    for (int i = 0; i < ng; i++) u[n + i] -= cwet[k + 1] * u[n + i + ng];
  }
}

/* FieldSolverADI::init coefficients, FieldSolverADI.cpp:125-182 */
static void adi_init(step_ctx *c, double delz, double dgrid, double xks) {
  int ng = c->ngrid;
  double rtmp = 0.25 * delz / (xks * dgrid * dgrid);
  c->cstep = CMPLX(0, rtmp);
  double *mupp = malloc(sizeof(double) * ng), *mmid = malloc(sizeof(double) * ng),
         *mlow = malloc(sizeof(double) * ng);
  cplx *w1 = malloc(sizeof(cplx) * ng), *w2 = malloc(sizeof(cplx) * ng);
  mupp[0] = rtmp;
  mmid[0] = -2 * rtmp;
  mlow[0] = 0;
  for (int i = 1; i < ng - 1; i++) {
    mupp[i] = rtmp;
    mmid[i] = -2 * rtmp;
    mlow[i] = rtmp;
  }
  mupp[ng - 1] = 0;
  mmid[ng - 1] = -2 * rtmp;
  mlow[ng - 1] = rtmp;
  for (int i = 0; i < ng; i++) {
    w1[i] = CMPLX(0, -mupp[i]);
    w2[i] = CMPLX(1, -mmid[i]);
    c->cc[i] = CMPLX(0, -mlow[i]);
  }
  c->cbet[0] = 1. / w2[0];
  c->cwet[0] = 0.;
  for (int i = 1; i < ng; i++) {
    c->cwet[i] = w1[i - 1] * c->cbet[i - 1];
    c->cbet[i] = 1. / (w2[i] - c->cc[i] * c->cwet[i]);
  }
  free(mupp);
  free(mmid);
  free(mlow);
  free(w1);
  free(w2);
}

/* ---- FFT (mixed radix, any length) used by the FFT field solver -------- */
/* out[k] = sum_j in[j*stride] exp(sign*2*pi*i*j*k/n); recursive decimation in time */
static void fft_rec(const cplx *in, cplx *out, int n, int stride, int sign, cplx *scratch) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  int p = 2;
  while (p * p <= n && n % p) p++;
  if (n % p) p = n; /* prime length: direct DFT */
  int m = n / p;
  if (p == n) {
    for (int k = 0; k < n; k++) {
      cplx s = 0;
      for (int j = 0; j < n; j++) {
        double ang = sign * 2.0 * kPi * (double)(((long long)j * k) % n) / (double)n;
        s += in[(size_t)j * stride] * CMPLX(cos(ang), sin(ang));
      }
      out[k] = s;
    }
    return;
  }
  /* p sub-transforms of length m on decimated inputs, stored contiguously in scratch */
  for (int r = 0; r < p; r++) fft_rec(in + (size_t)r * stride, scratch + (size_t)r * m, m, stride * p, sign, out);
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < p; q++) {
      cplx s = 0;
      int kk = k + q * m;
      for (int r = 0; r < p; r++) {
        double ang = sign * 2.0 * kPi * (double)(((long long)r * kk) % n) / (double)n;
        s += scratch[(size_t)r * m + k] * CMPLX(cos(ang), sin(ang));
      }
      out[kk] = s;
    }
  }
}

/* 2-D transform of an ngrid x ngrid row-major array (FFTW sign convention) */
static void fft2(cplx *a, int ng, int sign, cplx *tmp, cplx *tmp2) {
  cplx *line = tmp, *res = tmp + ng;
  for (int iy = 0; iy < ng; iy++) {
    fft_rec(a + (size_t)iy * ng, res, ng, 1, sign, tmp2);
    memcpy(a + (size_t)iy * ng, res, sizeof(cplx) * ng);
  }
  for (int ix = 0; ix < ng; ix++) {
    for (int iy = 0; iy < ng; iy++) line[iy] = a[(size_t)iy * ng + ix];
    fft_rec(line, res, ng, 1, sign, tmp2);
    for (int iy = 0; iy < ng; iy++) a[(size_t)iy * ng + ix] = res[iy];
  }
}

/* FieldSolverFFT::init tables, FieldSolverFFT.cpp:117-155 */
static void fft_init(step_ctx *c, double dgrid, double xks) {
  int ng = c->ngrid;
  double dk = 4. * asin(1.) / ((double)ng * dgrid);
  double xc = c->filt[0], yc = c->filt[1], sig = c->filt[2];
  double shift = -0.5 * (double)(ng - 1);
  for (int iy = 0; iy < ng; iy++) {
    double dy = (double)iy + shift;
    double y = dy / (double)ng / yc;
    for (int ix = 0; ix < ng; ix++) {
      double dx = (double)ix + shift;
      double x = dx / (double)ng / xc;
      int iiy = (iy + (ng + 1) / 2) % ng, iix = (ix + (ng + 1) / 2) % ng;
      int ii = iiy * ng + iix;
      c->k2[ii] = CMPLX(0, -(dx * dx + dy * dy) * dk * dk / 2. / xks);
      double r = (sqrt(x * x + y * y) - 1) / sig;
      c->sigm[ii] = 1. / (1 + exp(r));
    }
  }
}

/* FieldSolverFFT::FFT, FieldSolverFFT.cpp:64-114 */
static void fft_solve(const step_ctx *c, cplx *u, const cplx *src, cplx *work) {
  int ng = c->ngrid;
  size_t n2 = (size_t)ng * ng;
  cplx *uf = work, *sf = work + n2, *t1 = work + 2 * n2, *t2 = t1 + 2 * (size_t)ng;
  memcpy(uf, u, sizeof(cplx) * n2);
  fft2(uf, ng, -1, t1, t2);
  if (c->solver == 2) {
    memcpy(sf, src, sizeof(cplx) * n2);
    fft2(sf, ng, -1, t1, t2);
    for (size_t i = 0; i < n2; i++) sf[i] = sf[i] * c->sigm[i];
    for (size_t i = 0; i < n2; i++) uf[i] = uf[i] * cexp(c->k2[i] * c->delz) + 2. * sf[i];
  } else {
    for (size_t i = 0; i < n2; i++) uf[i] = uf[i] * cexp(c->k2[i] * c->delz);
  }
  fft2(uf, ng, +1, t1, t2);
  double norm = 1. / (double)(ng * ng);
  if (c->solver == 2) {
    for (size_t i = 0; i < n2; i++) u[i] = uf[i] * norm;
  } else {
    for (size_t i = 0; i < n2; i++) u[i] = uf[i] * norm + 2. * src[i];
  }
}

static void field_slices(step_ctx *c, int ii0, int ii1) {
  int ng = c->ngrid;
  size_t n2 = (size_t)ng * ng;
  cplx *src = malloc(sizeof(cplx) * n2);
  cplx *work = malloc(sizeof(cplx) * (3 * n2 + 4 * (size_t)ng));
  int k = c->ifld;
  for (int ii = ii0; ii < ii1; ii++) {
    deposit(c, ii, src);
    size_t i = (size_t)((ii + c->first[k]) % c->ns);
    cplx *u = c->fields + ((size_t)k * c->ns + i) * n2;
    if (c->solver == 0)
      adi(c, u, src, work);
    else
      fft_solve(c, u, src, work);
  }
  free(work);
  free(src);
}

/* ---- space charge (&efield), EFieldSolver.cpp ------------------------------ */
static struct {
  double rmax; /* the radial grid's extent, grown over the following runs */
  int ngrid, nz, nphi, longrange;
} sc_cfg = {0, 0, 0, 0, 0};

/* The &efield parameters of the following orc_run_steps calls (EField.cpp:19-39;
 * nz = 0 and longrange = 0 switch space charge off). The grid extent starts at rmax
 * and, as the reference's EFieldSolver member, carries over from call to call. */
void orc_set_efield(double rmax, int ngrid, int nz, int nphi, int longrange) {
  sc_cfg.rmax = rmax;
  sc_cfg.ngrid = ngrid;
  sc_cfg.nz = nz;
  sc_cfg.nphi = nphi;
  sc_cfg.longrange = longrange;
}

/* Beam::getSize, Beam.cpp:42-67 */
static double slice_size(const step_ctx *c, int is) {
  if (c->current[is] <= 0) return 1;
  const part_t *b = c->beam + (size_t)is * c->npart;
  double x1 = 0, x2 = 0, y1 = 0, y2 = 0;
  int count = 0;
  for (int ip = 0; ip < np_of(c, is); ip++) {
    x1 += b[ip].x;
    x2 += b[ip].x * b[ip].x;
    y1 += b[ip].y;
    y2 += b[ip].y * b[ip].y;
    count++;
  }
  if (count == 0) return 1.;
  x1 /= (double)count;
  x2 /= (double)count;
  y1 /= (double)count;
  y2 /= (double)count;
  return sqrt(fabs(x2 - x1 * x1)) * sqrt(fabs(y2 - y1 * y1));
}

/* EFieldSolver::longRange, EFieldSolver.cpp:56-118: eloss[is] = -longESC / eev */
static void sc_long_range(const step_ctx *c, double slicelength, double *eloss) {
  int ns = c->ns;
  if (!sc_cfg.longrange) {
    for (int i = 0; i < ns; i++) eloss[i] = 0;
    return;
  }
  double gamma = c->gammaref / sqrt(1 + c->st.aw * c->st.aw);
  double *fsize = malloc(sizeof(double) * ns);
  for (int i = 0; i < ns; i++) {
    fsize[i] = slice_size(c, i);
    if (fsize[i] <= 0) fsize[i] = 1;
  }
  double scl = slicelength / 2. / asin(1) / 299792458.0 / 2 / 8.85e-12;
  for (int i = 0; i < ns; i++) {
    double efld = 0;
    for (int j = 0; j < ns; j++) {
      double ds = (double)(j - i) * slicelength * gamma;
      double coef = 1 - sqrt(ds * ds / (ds * ds + fsize[j]));
      double sgn = (j > i) ? -1. : ((j < i) ? 1. : 0.);
      efld += sgn * coef * scl * c->current[j] / fsize[j];
    }
    eloss[i] = -efld / kEev;
  }
  free(fsize);
}

/* std::pow(complex<double>, int) as libstdc++ forms it: binary powering, and the
 * reciprocal of the power for a negative exponent (z^0 = 1 exactly) */
static cplx cpow_int(cplx z, int n) {
  unsigned u = n < 0 ? (unsigned)(-n) : (unsigned)n;
  cplx y = (u % 2) ? z : 1;
  while (u >>= 1) {
    z = z * z;
    if (u % 2) y = y * z;
  }
  return n < 0 ? 1 / y : y;
}

/* EFieldSolver::shortRange with analyseBeam, constructLaplaceOperator and tridiag,
 * EFieldSolver.cpp:120-272: ez[npart] of slice is; *rmax carries the radial grid's
 * extent from slice to slice (it grows to 1.5 times a slice's extreme radius) */
static void sc_short_range(const step_ctx *c, int is, double *rmax, double *ez) {
  int npart = np_of(c, is), ng = sc_cfg.ngrid;
  for (int i = 0; i < npart; i++) ez[i] = 0;
  if (!(sc_cfg.nz > 0 && ng > 2) || npart < 1) return;
  const part_t *b = c->beam + (size_t)is * c->npart;
  double xcen = 0, ycen = 0;
  for (int i = 0; i < npart; i++) {
    xcen += b[i].x;
    ycen += b[i].y;
  }
  xcen /= (double)npart;
  ycen /= (double)npart;
  double rbound = 0;
  for (int i = 0; i < npart; i++) {
    double tx = b[i].x - xcen, ty = b[i].y - ycen, rad2 = tx * tx + ty * ty;
    if (rad2 > rbound) rbound = rad2;
  }
  rbound = sqrt(rbound);
  if (rbound > *rmax) *rmax = rbound * 1.5;
  double dr = *rmax / (double)(ng - 1);
  cplx *cwork = malloc(sizeof(cplx) * npart);
  int *idxr = malloc(sizeof(int) * npart);
  for (int i = 0; i < npart; i++) {
    double tx = b[i].x - xcen, ty = b[i].y - ycen, radi = sqrt(tx * tx + ty * ty);
    cwork[i] = CMPLX(tx / radi, ty / radi);
    idxr[i] = (int)floor(radi / dr);
  }
  double pi = 2 * asin(1);
  double *vol = malloc(sizeof(double) * ng), *ldig = malloc(sizeof(double) * (ng + 1));
  double *rlog = malloc(sizeof(double) * ng), *lmid = malloc(sizeof(double) * ng);
  cplx *csrc = malloc(sizeof(cplx) * ng), *clow = malloc(sizeof(cplx) * ng), *cmid = malloc(sizeof(cplx) * ng);
  cplx *cupp = malloc(sizeof(cplx) * ng), *celm = malloc(sizeof(cplx) * ng), *gam = malloc(sizeof(cplx) * ng);
  vol[0] = pi * dr * dr;
  rlog[0] = 0.5;
  ldig[0] = 0;
  for (int j = 1; j < ng; j++) {
    vol[j] = pi * dr * dr * (2 * j + 1);
    ldig[j] = 2 * pi * j;
    rlog[j] = log((double)(j + 1) / (double)j);
  }
  ldig[ng] = 0;
  double ks = 4 * asin(1) / c->reflength;
  double gz2 = c->gammaref * c->gammaref / (1 + c->st.aw * c->st.aw);
  double coef = -gz2 / ks / ks;
  double econst = kVacimp / kEev * c->current[is] / ks / (double)npart;
  for (int m = -sc_cfg.nphi; m <= sc_cfg.nphi; m++) {
    for (int i = 0; i < ng; i++) lmid[i] = -ldig[i] - ldig[i + 1] - 2. * pi * m * m * rlog[i];
    lmid[ng - 1] -= 2 * pi * ng;
    for (int l = 1; l <= sc_cfg.nz; l++) {
      for (int i = 0; i < ng; i++) csrc[i] = 0;
      for (int i = 0; i < npart; i++)
        csrc[idxr[i]] += cpow_int(cwork[i], -m) * CMPLX(cos(l * b[i].theta), -sin(l * b[i].theta));
      for (int i = 0; i < ng; i++) {
        csrc[i] *= CMPLX(0, econst / l / vol[i]);
        clow[i] = coef * ldig[i] / l / l / vol[i];
        cmid[i] = 1 + coef * lmid[i] / l / l / vol[i];
        cupp[i] = coef * ldig[i + 1] / l / l / vol[i];
      }
      /* tridiag */
      cplx bet = cmid[0];
      celm[0] = csrc[0] / bet;
      for (int i = 1; i < ng; i++) {
        gam[i] = cupp[i - 1] / bet;
        bet = cmid[i] - clow[i] * gam[i];
        celm[i] = (csrc[i] - clow[i] * celm[i - 1]) / bet;
      }
      for (int i = ng - 2; i > -1; i--) celm[i] = celm[i] - gam[i + 1] * celm[i + 1];
      for (int i = 0; i < npart; i++) {
        cplx ctemp = cpow_int(cwork[i], m) * CMPLX(cos(l * b[i].theta), sin(l * b[i].theta));
        ez[i] += 2 * creal(ctemp * celm[idxr[i]]);
      }
    }
  }
  free(cwork), free(idxr), free(vol), free(ldig), free(rlog), free(lmid);
  free(csrc), free(clow), free(cmid), free(cupp), free(celm), free(gam);
}

/* ---- wakes (&wake), Collective.cpp ---------------------------------------- */
static struct {
  int on, ns, nslice, transient;
  double ds, ztrans, radius;
  double *ext, *res, *geo, *rou;
} wk = {0, 0, 0, 0, 0, 0, 0, NULL, NULL, NULL, NULL};

/* Collective::initWake (Collective.cpp:39-107) for the following orc_run_steps calls:
 * the external loss ext[nslice] (eV/m) and the single-particle wakes res, geo, rou on
 * ns_hr points spaced ds, whose first points are halved (self-loading theorem); on = 0
 * switches the wake off. */
void orc_set_wake(int on, int ns_hr, int nslice, double ds, const double *ext, const double *res,
                  const double *geo, const double *rou, double ztrans, double radius, int transient) {
  free(wk.ext), free(wk.res), free(wk.geo), free(wk.rou);
  wk.ext = wk.res = wk.geo = wk.rou = NULL;
  wk.on = on != 0;
  if (!wk.on) return;
  wk.ns = ns_hr;
  wk.nslice = nslice;
  wk.ds = ds;
  wk.ztrans = ztrans;
  wk.radius = radius;
  wk.transient = transient;
  wk.ext = malloc(sizeof(double) * nslice);
  wk.res = malloc(sizeof(double) * ns_hr);
  wk.geo = malloc(sizeof(double) * ns_hr);
  wk.rou = malloc(sizeof(double) * ns_hr);
  memcpy(wk.ext, ext, sizeof(double) * nslice);
  memcpy(wk.res, res, sizeof(double) * ns_hr);
  memcpy(wk.geo, geo, sizeof(double) * ns_hr);
  memcpy(wk.rou, rou, sizeof(double) * ns_hr);
  wk.geo[0] *= 0.5;
  wk.res[0] *= 0.5;
  wk.rou[0] *= 0.5;
}

/* Collective::update for a single rank (Collective.cpp:132-187): the slices' current
 * interpolated to the fine grid (electrons per fine slice) and its derivative, then
 * the wake of every slice from the fine points ahead of it, averaged over the slice's
 * `sample` fine points. The transient cut is computed there but not applied. */
static void wake_update(const double *current, int nslice, double *wakeint) {
  const unsigned ns = (unsigned)wk.ns;
  const int ncur = nslice;
  const double ds = wk.ds, dscur = ds * ns / ncur;
  double *cur = malloc(sizeof(double) * (ncur + 1));
  double *curh = malloc(sizeof(double) * ns), *dcur = malloc(sizeof(double) * ns);
  memcpy(cur, current, sizeof(double) * ncur);
  cur[ncur] = 0;
  for (int is = 0; is < (int)ns; is++) {
    double s = ds * (double)is;
    unsigned idx = (unsigned)(int)floor(s / dscur);
    double wei = 1 - (s - idx * dscur) / dscur;
    curh[is] = wei * cur[idx] + (1 - wei) * cur[idx + 1];
    curh[is] *= ds / kCe;
    dcur[is] = -(cur[idx + 1] - cur[idx]) * ds / kCe / dscur;
  }
  int sample = (int)(dscur / ds);
  if (sample < 1) sample = 1;
  for (int ic = 0; ic < nslice; ic++) {
    double w = 0;
    int is0 = ic * sample;
    for (int j = 0; j < sample; j++) {
      int is = is0 + j;
      for (unsigned long i = 0; i < ns - is; i++) {
        w += curh[is + i] * (wk.res[i] + wk.rou[i]);
        w += dcur[is + i] * wk.geo[i];
      }
    }
    wakeint[ic] = w / (double)sample;
  }
  free(cur), free(curh), free(dcur);
}

/* Collective::apply (Collective.cpp:109-129): every particle of a slice gains
 * loss * delz / eev */
static void apply_wake(step_ctx *c, int is0, int is1) {
  for (int is = is0; is < is1; is++) {
    double dg = c->wake_loss[is] * c->delz / kEev;
    part_t *b = c->beam + (size_t)is * c->npart;
    for (int ip = 0; ip < np_of(c, is); ip++) b[ip].gamma += dg;
  }
}

/* ---- incoherent synchrotron radiation (&sponrad), Incoherent.cpp ---------- */
static struct {
  int on, loss, spread, nbins;
  ran2_t sran;
} isr = {0, 0, 0, 1};

/* Incoherent::init (Incoherent.cpp:12-27) for rank 0: the stream is seeded with
 * round(1e9 u), u the first draw of a stream seeded with `seed`. The stream carries over
 * orc_run_steps calls as the reference's member does; nbins: the beamlet size, one draw
 * per beamlet (1 for one4one windows). */
void orc_set_incoherent(int seed, int do_loss, int do_spread, int nbins) {
  isr.on = do_loss || do_spread;
  isr.loss = do_loss;
  isr.spread = do_spread;
  isr.nbins = nbins > 0 ? nbins : 1;
  ran2_t rseed;
  ran2_init(&rseed, (unsigned int)seed);
  double val = ran2_next(&rseed);
  val *= 1e9;
  ran2_init(&isr.sran, (unsigned int)(int)round(val));
}

/* Incoherent::apply (Incoherent.cpp:31-80): the energy loss and the spread growth of
 * one step, slice after slice, one draw per beamlet */
static void apply_incoherent(step_ctx *c) {
  const step_t *u = &c->st;
  if (!(u->aw > 0)) return;
  if (!isr.on) return;
  double gam0 = c->gammaref, awz = u->aw, xkw0 = u->ku, delz = c->delz;
  double dgamsig = 1.015e-27 * xkw0 * xkw0 * awz * awz;
  if (u->helical)
    dgamsig *= 1.42 * awz + 1. / (1. + 1.5 * awz + 0.95 * awz * awz);
  else
    dgamsig *= 1.697 * awz + 1. / (1. + 1.88 * awz + 0.8 * awz * awz);
  if (!isr.spread) dgamsig = 0;
  dgamsig = sqrt(dgamsig * gam0 * gam0 * gam0 * gam0 * xkw0 * delz) * sqrt(3.);
  double dgamavg = xkw0 * gam0 * awz;
  if (!isr.loss) dgamavg = 0;
  dgamavg = dgamavg * dgamavg * 1.88e-15 * delz;
  int nbins = c->count ? 1 : isr.nbins;
  double dg = 0;
  for (int is = 0; is < c->ns; is++) {
    part_t *b = c->beam + (size_t)is * c->npart;
    for (int ip = 0; ip < np_of(c, is); ip++) {
      if ((ip % nbins) == 0) dg = -dgamavg + dgamsig * (2 * ran2_next(&isr.sran) - 1);
      b[ip].gamma += dg;
    }
  }
}

/* TrackBeam::applyR56, TrackBeam.cpp:260-277 */
static void apply_r56(step_ctx *c, int is0, int is1) {
  const step_t *u = &c->st;
  if (u->angle == 0) return;
  double angle = u->angle, lb = u->lb, ld = u->ld;
  double R56 = (4 * lb / sin(angle) * (1 - angle / tan(angle)) + 2 * ld * tan(angle) / cos(angle)) * angle;
  R56 = R56 * 4 * asin(1) / c->reflength / c->gammaref;
  for (int is = is0; is < is1; is++) {
    part_t *b = c->beam + (size_t)is * c->npart;
    for (int ip = 0; ip < np_of(c, is); ip++) b[ip].theta += R56 * (b[ip].gamma - c->gammaref);
  }
}

static void run_transverse_first(void *ctx, int i0, int i1) { transverse_slices((step_ctx *)ctx, i0, i1, 0); }
static void run_transverse_second(void *ctx, int i0, int i1) { transverse_slices((step_ctx *)ctx, i0, i1, 1); }

static void run_push(void *ctx, int i0, int i1) {
  step_ctx *c = (step_ctx *)ctx;
  transverse_slices(c, i0, i1, 0);
  push_slices(c, i0, i1);
  if (c->wake_loss) apply_wake(c, i0, i1);
  apply_r56(c, i0, i1);
  transverse_slices(c, i0, i1, 1);
}

/* the push in Beam::track's order when a step draws random numbers (the stream runs
 * slice after slice): first half, advance, incoherent radiation, wakes, R56, second half
 * (Beam.cpp:103-111) */
static void run_push_first(void *ctx, int i0, int i1) {
  step_ctx *c = (step_ctx *)ctx;
  transverse_slices(c, i0, i1, 0);
  push_slices(c, i0, i1);
}
static void run_push_second(void *ctx, int i0, int i1) {
  step_ctx *c = (step_ctx *)ctx;
  if (c->wake_loss) apply_wake(c, i0, i1);
  apply_r56(c, i0, i1);
  transverse_slices(c, i0, i1, 1);
}
static void run_field(void *ctx, int i0, int i1) { field_slices((step_ctx *)ctx, i0, i1); }

/* Control::applySlippage for one rank, Control.cpp:158-276 */
static void apply_slippage(double slippage, double sample, int periodic, int ns, size_t n2,
                           cplx *field, int *first, double *accuslip) {
  *accuslip += slippage;
  int direction = 1;
  while (fabs(*accuslip) > (sample * 0.8)) {
    if (*accuslip < 0) direction = -1;
    *accuslip -= sample * direction;
    int last = (*first + ns - 1) % ns;
    if (direction < 0) last = (last + 1) % ns;
    if (!periodic) {
      /* rank 0 zero-fills for forward slippage, the last rank for backward */
      cplx *f = field + (size_t)last * n2;
      for (size_t i = 0; i < n2; i++) f[i] = 0;
    }
    *first = last;
    if (direction < 0) *first = (last + 1) % ns;
  }
}

/* one4one windows: particles per slice of the following orc_run_steps calls, and the
 * steps after whose push the window is sorted (every sort_every-th, 0: never) */
static int *o4o_count = NULL;
static int o4o_ns = 0, o4o_sort_every = 0;

void orc_set_counts(int nslice, const int *counts, int sort_every) {
  free(o4o_count);
  o4o_count = NULL;
  o4o_ns = 0;
  o4o_sort_every = sort_every;
  if (nslice <= 0 || !counts) return;
  o4o_count = malloc(sizeof(int) * nslice);
  memcpy(o4o_count, counts, sizeof(int) * nslice);
  o4o_ns = nslice;
}

void orc_get_counts(int nslice, int *out) {
  for (int i = 0; i < nslice; i++) out[i] = (o4o_count && i < o4o_ns) ? o4o_count[i] : -1;
}

/* Beam::sort for one rank (Beam.cpp:81-94): Sorting::globalSort, whose single rank sends
 * nothing and so drops the particles outside the window (fillPushVectors,
 * Sorting.cpp:364-421), then Sorting::localSort (Sorting.cpp:74-145), which moves the
 * others to the slice their phase lies in, removing by a swap with the slice's last
 * particle and appending at the destination; the currents then follow the counts.
 * particles [ns][cap][6], counts updated in place (orc_set_counts' copy too). Returns
 * the number of particles that found no room (cap too small; 0 normally). */
int orc_sort(int ns, int cap, double *particles, int *counts, double *current, double reflength, double sample) {
  part_t *beam = (part_t *)particles;
  const double slicelength = reflength * sample;
  const double sl = 4 * asin(1.) * slicelength / reflength; /* Beam::initSorting */
  const double keepmax = sl * (unsigned long)ns;
  int lost = 0;
  /* fillPushVectors with s0 = 0, sendmin = keepmin = 0, sendmax = keepmax = sl ns */
  for (int i = 0; i < ns; i++) {
    part_t *b = beam + (size_t)i * cap;
    int j = 0;
    while (j < counts[i]) {
      double s = 0 + sl * i + b[j].theta;
      if ((s < 0) || (s > keepmax)) {
        b[j] = b[counts[i] - 1];
        counts[i]--;
      } else {
        j++;
      }
    }
  }
  /* localSort */
  double invslen = 1. / sl;
  for (int a = 0; a < ns; a++) {
    part_t *b = beam + (size_t)a * cap;
    int k = 0;
    while (k < counts[a]) {
      double theta = b[k].theta;
      int atar = (int)floor(theta * invslen);
      if (atar != 0) {
        part_t p = b[k];
        p.theta = b[k].theta - sl * (atar);
        int d = a + atar;
        if (d >= 0 && d < ns && counts[d] < cap) {
          beam[(size_t)d * cap + counts[d]] = p;
          counts[d]++;
        } else {
          lost++;
        }
        b[k] = b[counts[a] - 1];
        counts[a]--;
      } else {
        k++;
      }
    }
  }
  for (int i = 0; i < ns; i++) current[i] = (double)counts[i] * kCe / slicelength;
  if (o4o_count && o4o_ns == ns) memcpy(o4o_count, counts, sizeof(int) * ns);
  return lost;
}

int orc_run_steps(int nsteps, const double *lat, double gammaref, int ns, int npart,
                  double *particles, const double *current, double reflength,
                  double sample, int nfld, const int *harm, int ngrid,
                  const double *gridmax, double *fields, int *first, double *accuslip,
                  int time_run, int periodic, int stages, int solver, const double *filt,
                  int nthreads) {
  if (nfld > 8 || ngrid < 3) return 1;
  step_ctx c;
  memset(&c, 0, sizeof(c));
  c.ns = ns;
  c.npart = npart;
  c.nfld = nfld;
  c.ngrid = ngrid;
  c.beam = (part_t *)particles;
  c.count = (o4o_count && o4o_ns == ns) ? o4o_count : NULL;
  c.current = current;
  /* sorting changes the currents: a copy of them for this call */
  double *cur_local = NULL;
  if (c.count && o4o_sort_every > 0) {
    cur_local = malloc(sizeof(double) * ns);
    memcpy(cur_local, current, sizeof(double) * ns);
    c.current = cur_local;
  }
  c.fields = (cplx *)fields;
  c.harm = harm;
  c.first = first;
  c.gridmax = gridmax;
  c.reflength = reflength;
  c.gammaref = gammaref;
  c.solver = solver;
  if (filt) {
    c.filt[0] = filt[0];
    c.filt[1] = filt[1];
    c.filt[2] = filt[2];
  } else {
    c.filt[0] = c.filt[1] = c.filt[2] = 1;
  }
  /* FieldSolverFFT::initSourceFilter disables the filter for bad input */
  if (c.solver == 2 && (c.filt[2] <= 0 || c.filt[0] <= 0 || c.filt[1] <= 0)) c.solver = 1;
  size_t n2 = (size_t)ngrid * ngrid;
  cplx *coef = malloc(sizeof(cplx) * 3 * ngrid);
  c.cc = coef;
  c.cbet = coef + ngrid;
  c.cwet = coef + 2 * ngrid;
  int fft_ready[8] = {0};
  cplx *fft_tabs = NULL;
  if (solver) fft_tabs = malloc(sizeof(cplx) * 2 * n2 * nfld);

  /* the wake of every slice: Collective::update on its first use after initWake (and,
   * transient, on every step, with the same result); the loss adds the external one */
  double *wake_loss = NULL;
  if (wk.on && wk.nslice == ns) {
    wake_loss = malloc(sizeof(double) * ns);
    wake_update(c.current, ns, wake_loss);
    for (int i = 0; i < ns; i++) wake_loss[i] = wk.ext[i] + wake_loss[i];
  }
  c.wake_loss = wake_loss;

  for (int istep = 0; istep < nsteps; istep++) {
    c.st = get_step(lat, istep);
    c.delz = c.st.dz;
    if (stages & ORC_STAGE_PUSH) {
      /* BeamSolver::advance field-dependent constants, BeamSolver.cpp:19-38 */
      double xks = 1;
      for (int k = 0; k < nfld; k++) {
        double fxks = 4. * asin(1) / (reflength / (double)harm[k]);
        xks = fxks / (double)harm[k];
        c.rtmp[k] = orc_fc(c.st.aw, c.st.helical, harm[k]) / fxks;
        c.rharm[k] = (double)harm[k];
      }
      c.xks_fund = xks;
      c.xku = c.st.ku;
      if (c.xku == 0) c.xku = xks * 0.5 / gammaref / gammaref;
      if (sc_cfg.longrange || (sc_cfg.nz > 0 && sc_cfg.ngrid > 2)) {
        /* Beam::track with space charge (Beam.cpp:97-112, BeamSolver.cpp:43-61): the
         * first transverse half step of every slice, the long-range loss of every
         * slice, then slice by slice the short-range field and the push */
        parallel_for(ns, nthreads, run_transverse_first, &c);
        double *eloss = malloc(sizeof(double) * ns), *ez = malloc(sizeof(double) * npart);
        sc_long_range(&c, reflength * sample, eloss);
        for (int is = 0; is < ns; is++) {
          sc_short_range(&c, is, &sc_cfg.rmax, ez);
          c.sc_ez = ez;
          c.sc_eloss = eloss[is];
          push_slices(&c, is, is + 1);
        }
        apply_incoherent(&c);
        if (c.wake_loss) apply_wake(&c, 0, ns);
        apply_r56(&c, 0, ns);
        c.sc_ez = NULL;
        free(eloss);
        free(ez);
        parallel_for(ns, nthreads, run_transverse_second, &c);
      } else if (isr.on && c.st.aw > 0) {
        parallel_for(ns, nthreads, run_push_first, &c);
        apply_incoherent(&c);
        parallel_for(ns, nthreads, run_push_second, &c);
      } else {
        parallel_for(ns, nthreads, run_push, &c);
      }
    }
    /* Gencore.cpp:121-132: the sort after the push, before the field solve; the wake
     * follows the new currents (Collective::forceUpdate) */
    if (cur_local && (istep + 1) % o4o_sort_every == 0) {
      orc_sort(ns, npart, particles, o4o_count, cur_local, reflength, sample);
      if (wake_loss) {
        wake_update(c.current, ns, wake_loss);
        for (int i = 0; i < ns; i++) wake_loss[i] = wk.ext[i] + wake_loss[i];
      }
    }
    if (stages & ORC_STAGE_FIELD) {
      for (int k = 0; k < nfld; k++) {
        c.ifld = k;
        double gm = gridmax[k], dgrid = 2 * gm / (double)(ngrid - 1);
        double fxks = 4. * asin(1) / (reflength / (double)harm[k]);
        if (solver == 0) {
          /* FieldSolverADI.cpp:127 caches these per field and delz; they are a
           * pure function of (delz, dgrid, xks), so recomputing is identical */
          adi_init(&c, c.delz, dgrid, fxks);
        } else {
          c.k2 = fft_tabs + 2 * n2 * k;
          c.sigm = c.k2 + n2;
          if (!fft_ready[k]) fft_init(&c, dgrid, fxks);
          fft_ready[k] = 1;
        }
        parallel_for(ns, nthreads, run_field, &c);
      }
    }
    if ((stages & ORC_STAGE_SLIP) && time_run) {
      for (int k = 0; k < nfld; k++)
        apply_slippage(c.st.slip, sample, periodic, ns, n2, c.fields + (size_t)k * ns * n2,
                       &first[k], &accuslip[k]);
    }
  }
  free(coef);
  free(fft_tabs);
  free(wake_loss);
  free(cur_local);
  return 0;
}

/* The source term of one field for every beam slice at lattice step istep, as
 * FieldSolverADI::advance builds it (FieldSolverADI.cpp:13-52): out [ns][ngrid^2]
 * complex (re, im), zero outside undulators and for even harmonics. */
void orc_deposit_source(const double *lat, int istep, int ns, int npart, const double *particles,
                        const double *current, double reflength, int harm, int ngrid,
                        double gridmax, double *out) {
  step_ctx c;
  memset(&c, 0, sizeof(c));
  c.ns = ns;
  c.npart = npart;
  c.nfld = 1;
  c.ngrid = ngrid;
  c.beam = (part_t *)particles;
  c.current = current;
  c.harm = &harm;
  c.gridmax = &gridmax;
  c.reflength = reflength;
  c.ifld = 0;
  c.st = get_step(lat, istep);
  c.delz = c.st.dz;
  size_t n2 = (size_t)ngrid * ngrid;
  for (int ii = 0; ii < ns; ii++) deposit(&c, ii, (cplx *)out + (size_t)ii * n2);
}

/* One ADI step of every slice with a given source (the loop of
 * FieldSolverADI::advance, FieldSolverADI.cpp:9-58, with the source precomputed):
 * field storage slot (ii + first) % ns is advanced with source slice ii; source may
 * be NULL (no source). Coefficients from FieldSolverADI::init (:125-182). */
void orc_adi_advance(int ns, int ngrid, int first, double delz, double dgrid, double xks,
                     double *field, const double *source) {
  step_ctx c;
  memset(&c, 0, sizeof(c));
  c.ngrid = ngrid;
  size_t n2 = (size_t)ngrid * ngrid;
  cplx *coef = malloc(sizeof(cplx) * 3 * ngrid);
  cplx *work = malloc(sizeof(cplx) * n2);
  cplx *zero = calloc(n2, sizeof(cplx));
  c.cc = coef;
  c.cbet = coef + ngrid;
  c.cwet = coef + 2 * ngrid;
  adi_init(&c, delz, dgrid, xks);
  for (int ii = 0; ii < ns; ii++) {
    size_t i = (size_t)((ii + first) % ns);
    const cplx *src = source ? (const cplx *)source + (size_t)ii * n2 : zero;
    adi(&c, (cplx *)field + i * n2, src, work);
  }
  free(zero);
  free(work);
  free(coef);
}

/* ------------------------------------------------------------------------- */
/* diagnostics                                                               */
/* ------------------------------------------------------------------------- */
void orc_diag_beam(int ns, int npart, const double *particles, int nharm, double *out) {
  int ncol = ORC_DB_NCOL + 2 * nharm;
  cplx b[64];
  for (int is = 0; is < ns; is++) {
    const part_t *s = (const part_t *)particles + (size_t)is * npart;
    double g1 = 0, g2 = 0, x1 = 0, x2 = 0, y1 = 0, y2 = 0, px1 = 0, py1 = 0, px2 = 0, py2 = 0;
    double xpx = 0, ypy = 0, xmin = 1e5, xmax = -1e5, pxmin = 1e5, pxmax = -1e5, ymin = 1e5;
    double ymax = -1e5, pymin = 1e5, pymax = -1e5, gmin = 1e7, gmax = 1;
    for (int h = 0; h < nharm; h++) b[h] = 0;
    for (int i = 0; i < npart; i++) {
      const part_t *p = s + i;
      x1 += p->x;
      x2 += p->x * p->x;
      y1 += p->y;
      y2 += p->y * p->y;
      g1 += p->gamma;
      g2 += p->gamma * p->gamma;
      px1 += p->px;
      py1 += p->py;
      px2 += p->px * p->px;
      py2 += p->py * p->py;
      xpx += p->x * p->px;
      ypy += p->y * p->py;
      for (int h = 0; h < nharm; h++) b[h] += CMPLX(cos((h + 1) * p->theta), sin((h + 1) * p->theta));
    }
    for (int i = 0; i < npart; i++) {
      const part_t *p = s + i;
      if (p->x < xmin) xmin = p->x;
      if (p->x > xmax) xmax = p->x;
      if (p->px < pxmin) pxmin = p->px;
      if (p->px > pxmax) pxmax = p->px;
      if (p->y < ymin) ymin = p->y;
      if (p->y > ymax) ymax = p->y;
      if (p->py < pymin) pymin = p->py;
      if (p->py > pymax) pymax = p->py;
      if (p->gamma < gmin) gmin = p->gamma;
      if (p->gamma > gmax) gmax = p->gamma;
    }
    double norm = 1.;
    if (npart > 0) norm = 1. / (double)npart;
    x1 *= norm; x2 *= norm; y1 *= norm; y2 *= norm; px1 *= norm; px2 *= norm;
    py1 *= norm; py2 *= norm; g1 *= norm; g2 *= norm; xpx *= norm; ypy *= norm;
    for (int h = 0; h < nharm; h++) b[h] *= norm;
    double *o = out + (size_t)is * ncol;
    o[ORC_DB_ENERGY] = g1;
    o[ORC_DB_ENERGYSPREAD] = sqrt(fabs(g2 - g1 * g1));
    o[ORC_DB_XPOS] = x1;
    o[ORC_DB_XSIZE] = sqrt(fabs(x2 - x1 * x1));
    o[ORC_DB_YPOS] = y1;
    o[ORC_DB_YSIZE] = sqrt(fabs(y2 - y1 * y1));
    o[ORC_DB_PXPOS] = px1;
    o[ORC_DB_PYPOS] = py1;
    double ex = sqrt(fabs((x2 - x1 * x1) * (px2 - px1 * px1) - (xpx - x1 * px1) * (xpx - x1 * px1)));
    double ey = sqrt(fabs((y2 - y1 * y1) * (py2 - py1 * py1) - (ypy - y1 * py1) * (ypy - y1 * py1)));
    o[ORC_DB_EMITX] = ex;
    o[ORC_DB_EMITY] = ey;
    o[ORC_DB_BETAX] = (x2 - x1 * x1) / ex * g1;
    o[ORC_DB_BETAY] = (y2 - y1 * y1) / ey * g1;
    o[ORC_DB_ALPHAX] = -(xpx - x1 * px1) / ex;
    o[ORC_DB_ALPHAY] = -(ypy - y1 * py1) / ey;
    o[ORC_DB_XMIN] = xmin; o[ORC_DB_XMAX] = xmax; o[ORC_DB_PXMIN] = pxmin; o[ORC_DB_PXMAX] = pxmax;
    o[ORC_DB_YMIN] = ymin; o[ORC_DB_YMAX] = ymax; o[ORC_DB_PYMIN] = pymin; o[ORC_DB_PYMAX] = pymax;
    o[ORC_DB_EMIN] = gmin; o[ORC_DB_EMAX] = gmax;
    for (int h = 0; h < nharm; h++) {
      o[ORC_DB_NCOL + 2 * h] = cabs(b[h]);
      o[ORC_DB_NCOL + 2 * h + 1] = atan2(cimag(b[h]), creal(b[h]));
    }
  }
}

/* The window ("Global/") values of DiagBeam, Diagnostic.cpp:551-606: the slices'
 * moments <g>, <g^2>, <x>, <x^2>, <y>, <y^2> weighted by the current. out[6] = energy,
 * energyspread, xposition, xsize, yposition, ysize. */
void orc_diag_global_beam(int ns, int npart, const double *particles, const double *current, double *out) {
  double g_cur = 0, g_g1 = 0, g_g2 = 0, g_x1 = 0, g_x2 = 0, g_y1 = 0, g_y2 = 0;
  double norm = npart > 0 ? 1. / (double)npart : 1.;
  for (int is = 0; is < ns; is++) {
    double g1 = 0, g2 = 0, x1 = 0, x2 = 0, y1 = 0, y2 = 0;
    for (int ip = 0; ip < npart; ip++) {
      const double *p = particles + ((size_t)is * npart + ip) * 6;
      g1 += p[0];
      g2 += p[0] * p[0];
      x1 += p[2];
      x2 += p[2] * p[2];
      y1 += p[3];
      y2 += p[3] * p[3];
    }
    g1 *= norm, g2 *= norm, x1 *= norm, x2 *= norm, y1 *= norm, y2 *= norm;
    g_cur += current[is];
    g_g1 += current[is] * g1;
    g_g2 += current[is] * g2;
    g_x1 += current[is] * x1;
    g_x2 += current[is] * x2;
    g_y1 += current[is] * y1;
    g_y2 += current[is] * y2;
  }
  double w = g_cur > 0 ? 1. / g_cur : 1.;
  g_g1 *= w, g_g2 *= w, g_x1 *= w, g_x2 *= w, g_y1 *= w, g_y2 *= w;
  out[0] = g_g1;
  out[1] = sqrt(fabs(g_g2 - g_g1 * g_g1));
  out[2] = g_x1;
  out[3] = sqrt(fabs(g_x2 - g_x1 * g_x1));
  out[4] = g_y1;
  out[5] = sqrt(fabs(g_y2 - g_y1 * g_y1));
}

/* The window values of DiagField, Diagnostic.cpp:902-975, from the raw sums over all
 * slices: out[11] = energy [J], xposition, xsize, yposition, ysize,
 * intensity-nearfield, intensity-farfield (means over the slices), xpointing,
 * xdivergence, ypointing, ydivergence (from the far-field moments). */
static void fft2(cplx *a, int ng, int sign, cplx *tmp, cplx *tmp2);
void orc_diag_global_field(int ns, int ngrid, double gridmax, double lambda0, int harm, double sample,
                           const double *field, double *out) {
  const cplx *f = (const cplx *)field;
  const int n = ngrid;
  double xlambda = lambda0 / (double)harm;
  double dgrid = 2 * gridmax / (double)(n - 1);
  double ks = 4. * asin(1) / xlambda;
  double scl = dgrid * kEev / ks;
  double scltheta = xlambda / n / dgrid;
  double shift = -0.5 * (double)(n - 1);
  double g_pow = 0, g_x1 = 0, g_x2 = 0, g_y1 = 0, g_y2 = 0, g_ff = 0, g_inten = 0;
  double f_pow = 0, f_x1 = 0, f_x2 = 0, f_y1 = 0, f_y2 = 0;
  cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)n * n);
  cplx *t1 = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)n);
  cplx *t2 = (cplx *)malloc(sizeof(cplx) * (size_t)n);
  for (int is0 = 0; is0 < ns; is0++) {
    const cplx *sl = f + (size_t)is0 * n * n;
    cplx ff = 0;
    for (int iy = 0; iy < n; iy++) {
      double dy = (double)iy + shift;
      for (int ix = 0; ix < n; ix++) {
        double dx = (double)ix + shift;
        cplx loc = sl[iy * n + ix];
        double wei = creal(loc) * creal(loc) + cimag(loc) * cimag(loc);
        ff += loc;
        g_pow += wei;
        g_x1 += dx * wei;
        g_x2 += dx * dx * wei;
        g_y1 += dy * wei;
        g_y2 += dy * dy * wei;
      }
    }
    cplx c = sl[(n / 2) * n + n / 2];
    g_inten += creal(c) * creal(c) + cimag(c) * cimag(c);
    g_ff += (creal(ff) * creal(ff) + cimag(ff) * cimag(ff)) * dgrid * dgrid;
    memcpy(a, sl, sizeof(cplx) * (size_t)n * n);
    fft2(a, n, -1, t1, t2);
    for (int iy = 0; iy < n; iy++) {
      double dy = (double)iy + shift;
      for (int ix = 0; ix < n; ix++) {
        double dx = (double)ix + shift;
        int iiy = (iy + (n + 1) / 2) % n, iix = (ix + (n + 1) / 2) % n;
        cplx loc = a[(size_t)iiy * n + iix];
        double wei = creal(loc) * creal(loc) + cimag(loc) * cimag(loc);
        f_pow += wei;
        f_x1 += dx * wei;
        f_x2 += dx * dx * wei;
        f_y1 += dy * wei;
        f_y2 += dy * dy * wei;
      }
    }
  }
  free(a);
  free(t1);
  free(t2);
  double norm = g_pow > 0 ? 1. / g_pow : 1.;
  g_x1 *= norm, g_x2 *= norm, g_y1 *= norm, g_y2 *= norm;
  g_x2 = sqrt(fabs(g_x2 - g_x1 * g_x1)) * dgrid;
  g_y2 = sqrt(fabs(g_y2 - g_y1 * g_y1)) * dgrid;
  g_x1 *= dgrid;
  g_y1 *= dgrid;
  norm = f_pow > 0 ? 1. / f_pow : 1.;
  f_x1 *= norm, f_x2 *= norm, f_y1 *= norm, f_y2 *= norm;
  f_x2 = sqrt(fabs(f_x2 - f_x1 * f_x1)) * scltheta;
  f_y2 = sqrt(fabs(f_y2 - f_y1 * f_y1)) * scltheta;
  f_x1 *= scltheta;
  f_y1 *= scltheta;
  double slicelength = lambda0 * sample;
  g_pow *= scl * scl / kVacimp * slicelength / 299792458.0;
  norm = 1. / (double)ns;
  out[0] = g_pow;
  out[1] = g_x1;
  out[2] = g_x2;
  out[3] = g_y1;
  out[4] = g_y2;
  out[5] = g_inten * norm * kEev * kEev / ks / ks / kVacimp;
  out[6] = g_ff * norm;
  out[7] = f_x1;
  out[8] = f_x2;
  out[9] = f_y1;
  out[10] = f_y2;
}

/* DiagField's far-field moments, Diagnostic.cpp:786-847 (filter "fft"): the forward
 * 2-D transform of each slice (FFTW's convention: e^{-2 pi i jk/n}, unnormalised), its
 * power-weighted first and second moments on the shifted frequency map
 * ii = ((iy + (n+1)/2) % n) n + (ix + (n+1)/2) % n with dx = ix - (n-1)/2 (likewise y),
 * scaled by scltheta = xlambda / (ngrid dgrid): out[ns][4] = xpointing, xdivergence,
 * ypointing, ydivergence, indexed by window slice. */
void orc_diag_field_fft(int ns, int ngrid, double gridmax, double lambda0, int harm, const double *field,
                        int first, double *out) {
  const cplx *f = (const cplx *)field;
  const int n = ngrid;
  double xlambda = lambda0 / (double)harm;
  double dgrid = 2 * gridmax / (double)(n - 1);
  double scltheta = xlambda / n / dgrid;
  double shift = -0.5 * (double)(n - 1);
  cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)n * n);
  cplx *t1 = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)n);
  cplx *t2 = (cplx *)malloc(sizeof(cplx) * (size_t)n);
  for (int is0 = 0; is0 < ns; is0++) {
    int is = (ns + is0 - first) % ns;
    memcpy(a, f + (size_t)is0 * n * n, sizeof(cplx) * (size_t)n * n);
    fft2(a, n, -1, t1, t2);
    double fp = 0, fx1 = 0, fx2 = 0, fy1 = 0, fy2 = 0;
    for (int iy = 0; iy < n; iy++) {
      double dy = (double)iy + shift;
      for (int ix = 0; ix < n; ix++) {
        double dx = (double)ix + shift;
        int iiy = (iy + (n + 1) / 2) % n, iix = (ix + (n + 1) / 2) % n;
        cplx loc = a[(size_t)iiy * n + iix];
        double wei = creal(loc) * creal(loc) + cimag(loc) * cimag(loc);
        fp += wei;
        fx1 += dx * wei;
        fx2 += dx * dx * wei;
        fy1 += dy * wei;
        fy2 += dy * dy * wei;
      }
    }
    if (fp > 0) {
      fx1 /= fp;
      fx2 /= fp;
      fy1 /= fp;
      fy2 /= fp;
    }
    fx2 = sqrt(fabs(fx2 - fx1 * fx1)) * scltheta;
    fy2 = sqrt(fabs(fy2 - fy1 * fy1)) * scltheta;
    fx1 *= scltheta;
    fy1 *= scltheta;
    double *o = out + (size_t)is * 4;
    o[0] = fx1;
    o[1] = fx2;
    o[2] = fy1;
    o[3] = fy2;
  }
  free(a);
  free(t1);
  free(t2);
}

void orc_diag_field(int ns, int ngrid, double gridmax, double lambda0, int harm,
                    const double *field, int first, double *out) {
  const cplx *f = (const cplx *)field;
  double xlambda = lambda0 / (double)harm;
  double dgrid = 2 * gridmax / (double)(ngrid - 1);
  double ks = 4. * asin(1) / xlambda;
  double scl = dgrid * kEev / ks;
  double shift = -0.5 * (double)(ngrid - 1);
  for (int is0 = 0; is0 < ns; is0++) {
    int is = (ns + is0 - first) % ns;
    const cplx *sl = f + (size_t)is0 * ngrid * ngrid;
    double power = 0, x1 = 0, x2 = 0, y1 = 0, y2 = 0;
    cplx ff = 0;
    for (int iy = 0; iy < ngrid; iy++) {
      double dy = (double)iy + shift;
      for (int ix = 0; ix < ngrid; ix++) {
        double dx = (double)ix + shift;
        cplx loc = sl[iy * ngrid + ix];
        double wei = creal(loc) * creal(loc) + cimag(loc) * cimag(loc);
        ff += loc;
        power += wei;
        x1 += dx * wei;
        x2 += dx * dx * wei;
        y1 += dy * wei;
        y2 += dy * dy * wei;
      }
    }
    if (power > 0) {
      x1 /= power;
      x2 /= power;
      y1 /= power;
      y2 /= power;
    }
    x2 = sqrt(fabs(x2 - x1 * x1));
    y2 = sqrt(fabs(y2 - y1 * y1));
    int i = (ngrid / 2) * ngrid + (ngrid / 2);
    cplx loc = sl[i];
    double inten = creal(loc) * creal(loc) + cimag(loc) * cimag(loc);
    double intenphi = atan2(cimag(loc), creal(loc));
    double farfield = creal(ff) * creal(ff) + cimag(ff) * cimag(ff);
    double farfieldphi = atan2(cimag(ff), creal(ff));
    farfield *= dgrid * dgrid;
    power *= scl * scl / kVacimp;
    x1 *= dgrid;
    x2 *= dgrid;
    y1 *= dgrid;
    y2 *= dgrid;
    inten *= kEev * kEev / ks / ks / kVacimp;
    double *o = out + (size_t)is * ORC_DF_NCOL;
    o[ORC_DF_POWER] = power;
    o[ORC_DF_XPOS] = x1;
    o[ORC_DF_XSIZE] = x2;
    o[ORC_DF_YPOS] = y1;
    o[ORC_DF_YSIZE] = y2;
    o[ORC_DF_NF_INT] = inten;
    o[ORC_DF_NF_PHI] = intenphi;
    o[ORC_DF_FF_INT] = farfield;
    o[ORC_DF_FF_PHI] = farfieldphi;
  }
}
