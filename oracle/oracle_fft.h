// TEST INFRASTRUCTURE -- part of the CPU oracle, never linked into the product.
//
// Mixed-radix (2, 3, 4) complex FFT and 2-D in-place real FFT with the
// semantics of FFTW 2.1.5's rfftwnd_f77_one_real_to_complex /
// rfftwnd_f77_one_complex_to_real as the reference uses them (fft.f90:40-47):
// unnormalised, forward sign -1, x (the contiguous Fortran dimension) is the
// halved real dimension, complex output (lh,ny) in place over (ld,ny).  For a
// complex-to-real transform the imaginary parts of the kx=0 and kx=nx/2
// entries are ignored after the y pass, as FFTW's halfcomplex pass does.
//
// FFTW itself is a third-party C library absent from the reference tree
// (makefile:12-13 links fftw-2.1.5 from the author's home directory); this is
// a restatement of the published transform definition, pinned against
// numpy.fft in tests/test_oracle_fft.py.
#pragma once
#include <complex>
#include <vector>
#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <utility>

namespace les_oracle {

using cplx = std::complex<double>;

// Complex FFT of length n = 2^a 3^b, Stockham auto-sort, radix order 4..,2,3..
struct CFFT {
  int n = 0;
  std::vector<int> radix;
  std::vector<std::vector<cplx>> tw;  // per stage: tw[s][(r-1)*Ns + k] (forward)

  explicit CFFT(int n_ = 1) : n(n_) {
    int m = n;
    while (m % 4 == 0) { radix.push_back(4); m /= 4; }
    while (m % 2 == 0) { radix.push_back(2); m /= 2; }
    while (m % 3 == 0) { radix.push_back(3); m /= 3; }
    if (m != 1) throw std::runtime_error("CFFT: size must be 2^a 3^b");
    int Ns = 1;
    for (int R : radix) {
      std::vector<cplx> t((size_t)(R - 1) * Ns);
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < Ns; ++k) {
          long double ang = -2.0L * 3.14159265358979323846264338327950288L *
                            (long double)((long long)k * r) / (long double)((long long)Ns * R);
          t[(size_t)(r - 1) * Ns + k] = cplx((double)cosl(ang), (double)sinl(ang));
        }
      tw.push_back(std::move(t));
      Ns *= R;
    }
  }

  // In-place transform of x (length n) using scratch y (length n).
  void exec(cplx* x, cplx* y, int sign) const {
    int Ns = 1;
    cplx* src = x;
    cplx* dst = y;
    const double s3 = 0.86602540378443864676372317075294;  // sin(2 pi / 3)
    for (size_t st = 0; st < radix.size(); ++st) {
      const int R = radix[st];
      const int stride = n / R;
      const std::vector<cplx>& t = tw[st];
      for (int j = 0; j < stride; ++j) {
        const int k = j % Ns;
        cplx v[4];
        for (int r = 0; r < R; ++r) v[r] = src[j + r * stride];
        for (int r = 1; r < R; ++r) {
          cplx w = t[(size_t)(r - 1) * Ns + k];
          if (sign > 0) w = std::conj(w);
          v[r] = v[r] * w;
        }
        if (R == 2) {
          cplx a = v[0], b = v[1];
          v[0] = a + b;
          v[1] = a - b;
        } else if (R == 4) {
          cplx t0 = v[0] + v[2], t1 = v[0] - v[2];
          cplx t2 = v[1] + v[3], d = v[1] - v[3];
          // omega * d with omega = -i (forward) or +i (inverse)
          cplx t3 = (sign < 0) ? cplx(d.imag(), -d.real()) : cplx(-d.imag(), d.real());
          v[0] = t0 + t2;
          v[1] = t1 + t3;
          v[2] = t0 - t2;
          v[3] = t1 - t3;
        } else {  // R == 3
          cplx a0 = v[0], a1 = v[1], a2 = v[2];
          cplx sum = a1 + a2, dif = a1 - a2;
          cplx m = a0 - 0.5 * sum;
          double ss = (sign < 0) ? -s3 : s3;
          cplx rot(-ss * dif.imag(), ss * dif.real());  // i * ss * dif
          v[0] = a0 + sum;
          v[1] = m + rot;
          v[2] = m - rot;
        }
        const int base = (j / Ns) * Ns * R + k;
        for (int r = 0; r < R; ++r) dst[base + r * Ns] = v[r];
      }
      std::swap(src, dst);
      Ns *= R;
    }
    if (src != x)
      for (int i = 0; i < n; ++i) x[i] = src[i];
  }
};

// Real FFT of even length n through a length-n/2 complex FFT.
struct RFFT {
  int n = 0, m = 0;
  CFFT c;
  std::vector<cplx> w;  // exp(-2 pi i k / n), k = 0..m
  explicit RFFT(int n_ = 2) : n(n_), m(n_ / 2), c(n_ / 2) {
    w.resize(m + 1);
    for (int k = 0; k <= m; ++k) {
      long double ang = -2.0L * 3.14159265358979323846264338327950288L * k / (long double)n;
      w[k] = cplx((double)cosl(ang), (double)sinl(ang));
    }
  }
  // x: n reals in, X: m+1 complex out (may alias x's storage when sized 2m+2).
  void r2c(const double* x, cplx* X, cplx* s1, cplx* s2) const {
    for (int k = 0; k < m; ++k) s1[k] = cplx(x[2 * k], x[2 * k + 1]);
    c.exec(s1, s2, -1);
    const cplx z0 = s1[0];
    for (int k = 1; k < m; ++k) {
      cplx A = s1[k], B = std::conj(s1[m - k]);
      cplx E = 0.5 * (A + B);
      cplx D = 0.5 * (A - B);
      cplx O(D.imag(), -D.real());  // D / i
      s2[k] = E + w[k] * O;
    }
    s2[0] = cplx(z0.real() + z0.imag(), 0.0);
    s2[m] = cplx(z0.real() - z0.imag(), 0.0);
    for (int k = 0; k <= m; ++k) X[k] = s2[k];
  }
  // X: m+1 complex in (imag of X[0], X[m] ignored), x: n reals out.
  void c2r(const cplx* X, double* x, cplx* s1, cplx* s2) const {
    const cplx X0(X[0].real(), 0.0), Xm(X[m].real(), 0.0);
    for (int k = 0; k < m; ++k) {
      cplx a = (k == 0) ? X0 : X[k];
      cplx b = std::conj((k == 0) ? Xm : X[m - k]);
      cplx e = a + b;
      cplx d = (a - b) * std::conj(w[k]);  // times exp(+2 pi i k/n)
      s1[k] = e + cplx(-d.imag(), d.real());  // e + i d
    }
    c.exec(s1, s2, +1);
    for (int k = 0; k < m; ++k) {
      x[2 * k] = s1[k].real();
      x[2 * k + 1] = s1[k].imag();
    }
  }
};

// 2-D in-place real FFT over a (ld, ny) plane, ld = nx + 2.
struct FFT2 {
  int nx = 0, ny = 0, ld = 0, lh = 0;
  RFFT rx;
  CFFT cy;
  FFT2(int nx_, int ny_) : nx(nx_), ny(ny_), ld(nx_ + 2), lh(nx_ / 2 + 1), rx(nx_), cy(ny_) {}

  void r2c(double* pl) const {
    const int smax = (nx > 2 * ny ? nx : 2 * ny) + 8;
    std::vector<cplx> s1(smax), s2(smax), s3(smax);
    for (int jy = 0; jy < ny; ++jy) {
      double* row = pl + (size_t)jy * ld;
      rx.r2c(row, s3.data(), s1.data(), s2.data());
      for (int k = 0; k < lh; ++k) {
        row[2 * k] = s3[k].real();
        row[2 * k + 1] = s3[k].imag();
      }
    }
    for (int jx = 0; jx < lh; ++jx) {
      for (int jy = 0; jy < ny; ++jy) {
        const double* e = pl + (size_t)jy * ld + 2 * jx;
        s1[jy] = cplx(e[0], e[1]);
      }
      cy.exec(s1.data(), s2.data(), -1);
      for (int jy = 0; jy < ny; ++jy) {
        double* e = pl + (size_t)jy * ld + 2 * jx;
        e[0] = s1[jy].real();
        e[1] = s1[jy].imag();
      }
    }
  }

  void c2r(double* pl) const {
    const int smax = (nx > 2 * ny ? nx : 2 * ny) + 8;
    std::vector<cplx> s1(smax), s2(smax), s3(smax);
    for (int jx = 0; jx < lh; ++jx) {
      for (int jy = 0; jy < ny; ++jy) {
        const double* e = pl + (size_t)jy * ld + 2 * jx;
        s1[jy] = cplx(e[0], e[1]);
      }
      cy.exec(s1.data(), s2.data(), +1);
      for (int jy = 0; jy < ny; ++jy) {
        double* e = pl + (size_t)jy * ld + 2 * jx;
        e[0] = s1[jy].real();
        e[1] = s1[jy].imag();
      }
    }
    for (int jy = 0; jy < ny; ++jy) {
      double* row = pl + (size_t)jy * ld;
      for (int k = 0; k < lh; ++k) s3[k] = cplx(row[2 * k], row[2 * k + 1]);
      rx.c2r(s3.data(), row, s1.data(), s2.data());
      row[nx] = 0.0;  // padding columns: FFTW leaves unspecified values here
      row[nx + 1] = 0.0;
    }
  }
};

}  // namespace les_oracle
