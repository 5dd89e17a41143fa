// Host-side mode basis of the transformer (FP64): zeros of the Bessel
// functions and the disk-mode patterns of SeedModes
// (src/boost_fractor_transformer.jl:46-107).  Compiled with
// -ffp-contract=off so that both host architectures round alike.
#include <cmath>
#include <complex>
#include <vector>

namespace bfmodes {

using cd = std::complex<double>;

// J_nu(x) for integer nu of either sign: J_{-n}(x) = (-1)^n J_n(x).
double besselj(int nu, double x) {
  const int n = nu < 0 ? -nu : nu;
  double v = std::cyl_bessel_j((double)n, x);
  if (nu < 0 && (n & 1)) v = -v;
  return v;
}

// m-th positive zero (m >= 1) of J_nu, nu >= 0: sign changes are bracketed on
// a step of 0.05 (zeros are ~pi apart) and refined by bisection to the last
// representable double.
double besselj_zero(int nu, int m) {
  double x0 = 1e-3, f0 = besselj(nu, x0);
  int found = 0;
  const double step = 0.05;
  for (int i = 1; i < 10000000; ++i) {
    const double x1 = 1e-3 + step * i;
    const double f1 = besselj(nu, x1);
    if ((f0 < 0.0) != (f1 < 0.0) || f1 == 0.0) {
      if (++found == m) {
        double a = x0, b = x1, fa = f0;
        if (f1 == 0.0) return x1;
        for (int it = 0; it < 200; ++it) {
          const double c = 0.5 * (a + b);
          if (c == a || c == b) break;
          const double fc = besselj(nu, c);
          if (fc == 0.0) return c;
          if ((fa < 0.0) != (fc < 0.0)) {
            b = c;
          } else {
            a = c;
            fa = fc;
          }
        }
        return 0.5 * (a + b);
      }
    }
    x0 = x1;
    f0 = f1;
  }
  return NAN;
}

// Patterns in the reference's flat mode order k = (m-1)(2L+1) + l + L
// (m = 1..M, l = -L..L); out[k][y][x] (x fastest), kt[k].
void seed_modes(int M, int L, const std::vector<double>& X, const std::vector<double>& Y, double diskR,
                std::vector<cd>& out, std::vector<cd>& kt) {
  const size_t nx = X.size(), ny = Y.size(), npix = nx * ny;
  const int nl = 2 * L + 1;
  out.assign((size_t)M * nl * npix, cd(0.0, 0.0));
  kt.assign((size_t)M * nl, cd(0.0, 0.0));
  for (int m = 1; m <= M; ++m)
    for (int l = -L; l <= L; ++l) {
      const int k = (m - 1) * nl + l + L;
      const double kr = besselj_zero(l < 0 ? -l : l, m) / diskR;
      kt[k] = cd(kr, 0.0);
      cd* pat = out.data() + (size_t)k * npix;
      double norm2 = 0.0;
      for (size_t y = 0; y < ny; ++y)
        for (size_t x = 0; x < nx; ++x) {
          const double xx = X[x] * X[x];
          const double yy = Y[y] * Y[y];
          const double rr = std::sqrt(xx + yy);
          cd v(0.0, 0.0);
          if (!(rr > diskR)) {   // pattern[RR .> diskR] .*= 0
            const double phi = std::atan2(Y[y], X[x]);
            const double j = besselj(l, kr * rr);
            // exp(-1im*l*Phi)
            const double a = -(double)l * phi;
            v = cd(j * std::cos(a), j * std::sin(a));
          }
          pat[y * nx + x] = v;
          norm2 += std::norm(v);
        }
      const double s = std::sqrt(norm2);
      for (size_t i = 0; i < npix; ++i) pat[i] /= s;
    }
}

}  // namespace bfmodes
