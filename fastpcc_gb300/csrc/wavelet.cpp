// Complex wavelet families for wavelet PCC (host side); see wavelet.h.
#include "wavelet.h"

#include <cmath>
#include <cstdlib>

namespace fpcc {

static const double kPi = 3.14159265358979323846;

// erfi(z) = 2/sqrt(pi) * sum_{n>=0} z^(2n+1) / (n! (2n+1)), 500 terms as the
// reference evaluates it.
static double erfi_series(double z) {
  double term = z, sum = z;
  const double zz = z * z;
  for (unsigned n = 1; n < 500; n++) {
    term *= zz / n;
    sum += term / (2 * n + 1);
  }
  return sum * 2 / std::sqrt(kPi);
}

bool make_wavelet_family(int type, unsigned J, unsigned V, unsigned maxlen, double s0, double op1,
                         WaveletFamily* wf) {
  if (type != -1 && type != -2 && type != -3) return false;
  wf->type = type;
  wf->J = J;
  wf->V = V;
  wf->S = J * V;
  wf->s0 = s0;
  wf->op1 = op1;
  const unsigned S = wf->S;
  wf->scale.resize(S);
  wf->Ls.resize(S);
  wf->center.resize(S);
  wf->taps.assign(S, {});
  const double q = std::pow(2.0, 1.0 / (double)V);
  double s = s0;
  for (unsigned k = 0; k < S; k++) {
    wf->scale[k] = s;
    s *= q;
  }
  for (unsigned k = 0; k < S; k++) {
    const unsigned l = 2 * (unsigned)std::ceil(5 * wf->scale[k]) + 1;
    wf->Ls[k] = l > maxlen ? maxlen : l;
    const unsigned L = wf->Ls[k];
    const int u0 = (int)(L / 2);
    wf->center[k] = u0;
    const double sc = wf->scale[k];
    auto& t = wf->taps[k];
    t.resize(L);
    for (int u = -u0; u < (int)L - u0; u++) {
      const double d = (double)u / sc;
      std::complex<double> v;
      if (type == -1) {
        const double kk = 1 / std::sqrt(std::sqrt(kPi) * sc);
        v = kk * std::exp(std::complex<double>(0, op1 * d)) * std::exp(-0.5 * d * d);
      } else if (type == -2) {
        const double kk = 1 / std::sqrt(std::sqrt(kPi) * sc);
        const double ze = std::exp(-op1 * op1 / 2);
        v = kk * std::exp(-0.5 * d * d) * (std::exp(std::complex<double>(0, op1 * d)) - ze);
      } else {
        const double kk = 2 / std::sqrt(3 * std::sqrt(kPi) * sc);
        v = kk * ((d * d - 1) * std::exp(-d * d / 2) * std::complex<double>(1, erfi_series(d / std::sqrt(2.0))) -
                  std::complex<double>(0, std::sqrt(2 / kPi) * d));
      }
      t[u + u0] = v;
    }
  }
  return true;
}

int wpcc_setup(unsigned N, int Lag1, int Lag2, double pmin, double pmax, unsigned V, int type, double op1,
               WpccSetup* out) {
  const unsigned ua1 = (unsigned)std::abs(Lag1), ua2 = (unsigned)std::abs(Lag2);
  if (ua1 >= N || ua2 >= N || V == 0 || !(pmin > 0) || !(pmax > 0)) return -3;
  const unsigned M = ua1 > ua2 ? ua1 : ua2;
  unsigned Nz = 1u << (unsigned)std::ceil(std::log2((double)(N + M)));
  double s0;
  if (type == -3) {
    s0 = pmin / (std::sqrt(2.0) * kPi);
  } else if (type == -1 || type == -2) {
    if (op1 == 0) op1 = kPi * std::sqrt(2 / std::log(2.0));
    s0 = pmin * op1 / (2 * kPi);
  } else {
    return -3;
  }
  const unsigned J = (unsigned)std::lround(1. / (double)V + std::log(pmax / pmin) / std::log(2.0));
  if (J == 0) return -3;
  if (!make_wavelet_family(type, J, V, Nz, s0, op1, &out->wf)) return -3;
  out->Nz0 = Nz;
  out->Ls0 = out->wf.Ls[out->wf.S - 1];
  if (Nz - (N + M) < out->Ls0) Nz *= 2;
  out->Nz_ref = Nz;
  double K0 = 0;
  for (unsigned s = 0; s < out->wf.S; s++) K0 += 1 / out->wf.scale[s];
  out->K0 = K0;
  out->C = 1. / (K0 * (double)N);
  out->M = (int)M;
  return 0;
}

// Admissibility constants of the reconstruction: Morlet_Cpsi (the running sum
// of src/FWTa/wavelet_def_v7.c:133-144, kept step for step) and
// MexicanHat_Cpsi (:146-148).
double wavelet_cpsi(int type, double w0) {
  if (type == -3) return (4.0 / 3.0) * std::sqrt(kPi);
  double c = 0.0;
  for (double w = 0.01; w < 100; w += 0.01) {
    const double a = w - w0;
    c += std::exp(-a * a) / w;
  }
  return c * 0.01 * std::sqrt(kPi) / 2;
}

// Family of a ts-PWS stack over traces of L samples: s0 and the default w0
// from pmin as src/FFTapps.c:1097-1105, J = round(1/V + log2(pmax/pmin))
// (:1106), taps capped at L.  Returns 0 or -3.
int stack_family(unsigned L, double pmin, double pmax, unsigned V, int type, double op1, WaveletFamily* wf,
                 double* cpsi) {
  double s0;
  if (type == -3) {
    s0 = pmin / (std::sqrt(2.0) * kPi);
  } else if (type == -1 || type == -2) {
    if (op1 == 0) op1 = kPi * std::sqrt(2 / std::log(2.0));
    s0 = pmin * op1 / (2 * kPi);
  } else {
    return -3;
  }
  if (V == 0 || !(pmin > 0) || !(pmax > pmin) || L < 2) return -3;
  const unsigned J = (unsigned)std::lround(1. / (double)V + std::log(pmax / pmin) / std::log(2.0));
  if (J == 0 || !make_wavelet_family(type, J, V, L, s0, op1, wf)) return -3;
  *cpsi = wavelet_cpsi(type, op1);
  return 0;
}

}  // namespace fpcc
