// butterworth.h - coefficients of the Butterworth low-cut and high-cut
// filters of the FWI data preprocessing (libs/libwave/bandpass.c, after
// Oppenheim and Schafer, Digital Signal Processing, 1975): cascades of
// second-order sections from the bilinear transform of the analogue
// Butterworth poles, the low-cut one obtained from a high-cut prototype at
// half Nyquist.  The float/double evaluation of each coefficient follows the
// reference's C source, so that the host library and the oracle compute the
// same floats.  Host only; compile with -ffp-contract=off.
#pragma once

#include <cmath>

namespace swave_bp {

// At most this many sections per filter (nplo, nphi <= 64).
constexpr int kMaxSections = 32;

struct Sections {
  int n = 0;               // sections
  float c[kMaxSections][5];
};

// highcut_ (bandpass.c): f = cutoff in cycles per sample; npoles is halved
// (rounded up) for a zero-phase (phase = 0) filter, which runs twice.
inline Sections highcut_sections(float f, int npoles, int phase) {
  const double pi = 3.1415926535897932384626433832795028841971693;
  int np = npoles;
  int nodd = np % 2;
  if (phase == 0) {
    np = nodd != 0 ? (np + 1) / 2 : np / 2;
    nodd = np % 2;
  }
  Sections s;
  s.n = (np + 1) / 2;
  const float a = (float)(2.0 * std::tan(pi * (double)f));
  const float aa = a * a;
  const float aap4 = (float)((double)aa + 4.0);
  const float dtheta = (float)(pi / (double)np);
  const float theta0 = nodd != 0 ? 0.0f : (float)((double)dtheta / 2.0);
  if (nodd != 0) {
    s.c[0][0] = (float)((double)a / ((double)a + 2.0));
    s.c[0][1] = s.c[0][0];
    s.c[0][2] = 0.0f;
    s.c[0][3] = (float)(((double)a - 2.0) / ((double)a + 2.0));
    s.c[0][4] = 0.0f;
  }
  for (int j = nodd; j < s.n; ++j) {
    const double c = 4.0 * (double)a * std::cos((double)(theta0 + (float)j * dtheta));
    s.c[j][0] = (float)((double)aa / ((double)aap4 + c));
    s.c[j][1] = (float)(2.0 * (double)s.c[j][0]);
    s.c[j][2] = s.c[j][0];
    s.c[j][3] = (float)((2.0 * (double)aa - 8.0) / ((double)aap4 + c));
    s.c[j][4] = (float)(((double)aap4 - c) / ((double)aap4 + c));
  }
  return s;
}

// lowcut_ (bandpass.c).
inline Sections lowcut_sections(float f, int npoles, int phase) {
  const double pi = 3.1415926535897932384626433832795028841971693;
  int np = npoles;
  int nodd = np % 2;
  if (phase == 0) {
    np = nodd != 0 ? (np + 1) / 2 : np / 2;
    nodd = np % 2;
  }
  Sections s;
  s.n = (np + 1) / 2;
  const float fno2 = 0.25f;
  const float a = (float)(2.0 * std::sin(pi * (double)fno2) / std::cos(pi * (double)fno2));
  const float aa = a * a;
  const float aap4 = aa + 4.0f;
  const float e = (float)(-std::cos(pi * (double)(f + fno2)) / std::cos(pi * (double)(f - fno2)));
  const float ee = e * e;
  const float dtheta = (float)(pi / (double)np);
  const float theta0 = nodd != 0 ? 0.0f : dtheta / 2.0f;
  if (nodd != 0) {
    const float b1 = a / (a + 2.0f);
    const float b2 = (a - 2.0f) / (a + 2.0f);
    const float den = (float)(1.0 - (double)(b2 * e));
    s.c[0][0] = (float)((double)b1 * (1.0 - (double)e) / (double)den);
    s.c[0][1] = -s.c[0][0];
    s.c[0][2] = 0.0f;
    s.c[0][3] = (e - b2) / den;
    s.c[0][4] = 0.0f;
  }
  for (int j = nodd; j < s.n; ++j) {
    const double c = 4.0 * (double)a * std::cos((double)(theta0 + (float)j * dtheta));
    const float b1 = (float)((double)aa / ((double)aap4 + c));
    const float b2 = (float)((2.0 * (double)aa - 8.0) / ((double)aap4 + c));
    const float b3 = (float)(((double)aap4 - c) / ((double)aap4 + c));
    const float den = (float)((1.0 - (double)(b2 * e)) + (double)(b3 * ee));
    s.c[j][0] = (float)((double)b1 * (1.0 - (double)e) * (1.0 - (double)e) / (double)den);
    s.c[j][1] = (float)(-2.0 * (double)s.c[j][0]);
    s.c[j][2] = s.c[j][0];
    s.c[j][3] = (float)((2.0 * (double)e * (1.0 + (double)b3) - (double)b2 * (1.0 + (double)ee)) /
                        (double)den);
    s.c[j][4] = ((ee - b2 * e) + b3) / den;
  }
  return s;
}

// The cosine-squared end tapers of the padded trace (Bandpass.f90:124-127):
// lead[j] = sin(j*pi/(2*(npad-1)))**2, trail[j] = sin((npad-1-j)*pi/(2*(npad-1)))**2
// for j = 0..npad-1, with the single-precision pi of the Fortran source.
inline void end_tapers(int npad, float *lead, float *trail) {
  const float pi = 3.1415926535f;
  for (int j = 1; j <= npad; ++j) {
    const float s1 = std::sin((float)(j - 1) * pi / (float)(2 * (npad - 1)));
    const float s2 = std::sin((float)(npad - j) * pi / (float)(2 * (npad - 1)));
    lead[j - 1] = s1 * s1;
    trail[j - 1] = s2 * s2;
  }
}

}  // namespace swave_bp
