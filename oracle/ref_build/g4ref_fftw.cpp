// The FFTW3 calls of the reference (declared in shim/fftw3.h), evaluated as the
// unnormalised 2-D DFT that FFTW documents, so that the reference's own FFT field
// solver and far-field diagnostics can be compiled and run as a checker.
//
// A plan keeps its arrays, sizes and sign, as an FFTW plan does; fftw_execute
// transforms the plan's input into its output (in place allowed). The transform is a
// row pass then a column pass, each a direct sum over the line with the roots of
// unity tabulated once per plan in long double and indexed by (j k) mod n. The sums
// are carried in long double and rounded to double once, at the end: the result is
// the exact DFT to about 1e-16 relative, which is what FFTW delivers to its own
// rounding (FFTW's error grows like log n in units of double rounding). Results
// therefore agree with an FFTW build of the reference to rounding, not to the bit.
//
// Test infrastructure only; the product never links or loads it.

#include <cmath>
#include <cstdlib>
#include <vector>

#include "fftw3.h"

struct fftw_plan_s {
  int n0, n1, sign;
  double *in, *out;
  std::vector<long double> w0, w1;  // [2 n] cos, sign * sin of 2 pi m / n
};

static void roots(std::vector<long double> &w, int n, int sign) {
  w.resize(2 * static_cast<size_t>(n));
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < n; m++) {
    // the angle reduced to [-pi, pi] keeps sinl / cosl at full precision
    const int mr = (2 * m <= n) ? m : m - n;
    const long double a = two_pi * static_cast<long double>(mr) / static_cast<long double>(n);
    w[2 * m] = cosl(a);
    w[2 * m + 1] = sign * sinl(a);
  }
}

extern "C" {

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
  (void)flags;
  if (n0 <= 0 || n1 <= 0) return nullptr;
  fftw_plan p = new fftw_plan_s;
  p->n0 = n0;
  p->n1 = n1;
  p->sign = sign < 0 ? -1 : 1;
  p->in = reinterpret_cast<double *>(in);
  p->out = reinterpret_cast<double *>(out);
  roots(p->w0, n0, p->sign);
  roots(p->w1, n1, p->sign);
  return p;
}

void fftw_execute(const fftw_plan p) {
  if (p == nullptr) return;
  const int n0 = p->n0, n1 = p->n1;
  const size_t n = static_cast<size_t>(n0) * n1;
  // row pass: along the contiguous index j1 -> k1, for every row j0
  std::vector<long double> t(2 * n);
  for (int j0 = 0; j0 < n0; j0++) {
    const double *row = p->in + 2 * static_cast<size_t>(j0) * n1;
    for (int k1 = 0; k1 < n1; k1++) {
      long double re = 0, im = 0;
      int m = 0;  // (j1 k1) mod n1
      for (int j1 = 0; j1 < n1; j1++) {
        const long double xr = row[2 * j1], xi = row[2 * j1 + 1];
        const long double c = p->w1[2 * m], s = p->w1[2 * m + 1];
        re += xr * c - xi * s;
        im += xr * s + xi * c;
        m += k1;
        if (m >= n1) m -= n1;
      }
      t[2 * (static_cast<size_t>(j0) * n1 + k1)] = re;
      t[2 * (static_cast<size_t>(j0) * n1 + k1) + 1] = im;
    }
  }
  // column pass: along j0 -> k0, for every column k1; the output is written only
  // after the row pass has read all of the input (in-place plans)
  std::vector<long double> col(2 * static_cast<size_t>(n0));
  for (int k1 = 0; k1 < n1; k1++) {
    for (int j0 = 0; j0 < n0; j0++) {
      col[2 * j0] = t[2 * (static_cast<size_t>(j0) * n1 + k1)];
      col[2 * j0 + 1] = t[2 * (static_cast<size_t>(j0) * n1 + k1) + 1];
    }
    for (int k0 = 0; k0 < n0; k0++) {
      long double re = 0, im = 0;
      int m = 0;  // (j0 k0) mod n0
      for (int j0 = 0; j0 < n0; j0++) {
        const long double xr = col[2 * j0], xi = col[2 * j0 + 1];
        const long double c = p->w0[2 * m], s = p->w0[2 * m + 1];
        re += xr * c - xi * s;
        im += xr * s + xi * c;
        m += k0;
        if (m >= n0) m -= n0;
      }
      p->out[2 * (static_cast<size_t>(k0) * n1 + k1)] = static_cast<double>(re);
      p->out[2 * (static_cast<size_t>(k0) * n1 + k1) + 1] = static_cast<double>(im);
    }
  }
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

}  // extern "C"
