// Complex wavelet families for wavelet PCC (host side).
//
// Restates the reference's frame construction (src/FWTa/wavelet_def_v7.c):
// scales s0 * 2^(k/V) (setscales0 :299-309), lengths 2*ceil(5*scale)+1 capped at
// the transform length (setwaveletlength0 :312-322), centre Ls/2, and the taps
// of the Morlet (:38-52), complete Morlet (:71-87) and complex Mexican-hat
// (:119-131, erfi by its Maclaurin series :104-117) wavelets.
#pragma once

#include <complex>
#include <vector>

namespace fpcc {

struct WaveletFamily {
  int type = -3;                 // -1 Morlet, -2 complete Morlet, -3 complex Mexican hat
  unsigned J = 0, V = 0, S = 0;  // octaves, voices, scales (S = J*V)
  double s0 = 0, op1 = 0;
  std::vector<double> scale;
  std::vector<unsigned> Ls;
  std::vector<int> center;
  std::vector<std::vector<std::complex<double>>> taps;   // S rows of Ls[s] taps
};

// Build the family with lengths capped at maxlen.  Returns false for an
// unknown type.
bool make_wavelet_family(int type, unsigned J, unsigned V, unsigned maxlen, double s0, double op1,
                         WaveletFamily* wf);

// WPCC set-up of the reference's tspcc2_set (src/FFTapps.c:1084-1115): w0
// default, s0 from pmin, J from pmax/pmin, the family with the power-of-two
// length cap, the padded length rule with its doubling.  Returns 0 or -3.
struct WpccSetup {
  WaveletFamily wf;
  unsigned Nz_ref = 0;   // the reference's transform length (after doubling)
  unsigned Nz0 = 0;      // the length cap used for the wavelet lengths
  unsigned Ls0 = 0;      // longest wavelet
  double K0 = 0;         // sum of 1/scale
  double C = 0;          // output scale 1/(K0 N)
  int M = 0;
};
int wpcc_setup(unsigned N, int Lag1, int Lag2, double pmin, double pmax, unsigned V, int type, double op1,
               WpccSetup* out);

// Reconstruction constant Cpsi of the wavelet type (w0 for the Morlets).
double wavelet_cpsi(int type, double w0);
// Family of a ts-PWS stack over traces of L samples (s0 and w0 from pmin, J from
// pmax/pmin, taps capped at L) and its Cpsi.  Returns 0 or -3.
int stack_family(unsigned L, double pmin, double pmax, unsigned V, int type, double op1, WaveletFamily* wf,
                 double* cpsi);

}  // namespace fpcc
