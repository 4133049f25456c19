// Phase-function mixing of several scattering species into one table.
//
// Replaces phase_function_mixing (src/util.f90:240-348), called by
// mix_optical_properties (at3d/medium.py:900-1068).  For every grid point, in
// the caller's order (the reference visits x fastest):
//   * the scattering-weighted mean of the species' Wigner series,
//     w = sum_p sum_k scat_p wt_pk table[idx_pk] / sum_p scat_p;
//   * its asymmetry a1_1/3, and P11 and P12 at nangles scattering angles
//     0, 180/(nangles-1), ..., 180 degrees (PHASEFUNC_FROM_WIGNER,
//     src/shdomsub5.f:2785-2838: P11 = sum_l a1_l d^l_00 / 4pi,
//     P12 = -sum_l b1_l d^l_20 / 4pi); a P11 <= 0 at any angle is an error;
//   * the table entry kept so far with the smallest combined error
//     |da|/asym_tol + max|dP11/max(0.001, P11)|/phase_tol
//       + max|dDoLP/max(0.001, DoLP)|/dolp_tol
//     is used when each of the three terms is within its tolerance, otherwise
//     the point's series becomes a new entry.
// Points without scattering keep index 0.  Phase values, ratios and errors
// are single precision like the reference's REAL variables (the error terms
// are formed in double against the double tolerances, as there); the series
// sums over l are double.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/shdom_gb300.h"

namespace shdom {
int host_fail(const std::string &m);
}

namespace {

// d^l_00 and d^l_20 at x for l = 0..L (three-term recurrences in l).
void wigner_00_20(double x, int L, std::vector<double> &d00, std::vector<double> &d20) {
  d00.assign(L + 1, 0.0);
  d20.assign(L + 1, 0.0);
  d00[0] = 1.0;
  if (L >= 1) d00[1] = x;
  for (int l = 1; l < L; ++l) d00[l + 1] = ((2 * l + 1) * x * d00[l] - l * d00[l - 1]) / (l + 1);
  if (L >= 2) {
    d20[2] = 0.25 * std::sqrt(6.0) * (1.0 - x * x);
    double prev = 0.0;
    for (int l = 2; l < L; ++l) {
      const double q = std::sqrt((l + 1.0) * (l + 1.0) - 4.0);
      const double nx = ((2 * l + 1) * x * d20[l] - std::sqrt(l * l - 4.0) * prev) / q;
      prev = d20[l];
      d20[l + 1] = nx;
    }
  }
}

}  // namespace

extern "C" int shdom_phase_function_mixing(int npts, int npart, int nmicro, const float *scatter,
                                           const int *phase_index, const float *phase_weight, int numphase,
                                           int nleg, int nstleg, const float *phase_tables, double asym_tol,
                                           double phase_tol, double dolp_tol, int nangles, int maxnphase,
                                           float *mixed_table, int *mixed_index, int *nphase_out,
                                           int *fail_point) {
  if (!scatter || !phase_index || !phase_weight || !phase_tables || !mixed_table || !mixed_index || !nphase_out)
    return shdom::host_fail("shdom_phase_function_mixing: null argument");
  if (npts < 0 || npart < 1 || nmicro < 1 || numphase < 1 || nleg < 0 || (nstleg != 1 && nstleg != 6) ||
      nangles < 2 || maxnphase < 1)
    return shdom::host_fail("shdom_phase_function_mixing: bad sizes");
  if (!(asym_tol > 0) || !(phase_tol > 0) || !(dolp_tol > 0))
    return shdom::host_fail("shdom_phase_function_mixing: tolerances must be positive");
  const size_t row = (size_t)(nleg + 1) * nstleg;
  for (size_t i = 0; i < (size_t)npart * npts * nmicro; ++i)
    if (phase_index[i] < 1 || phase_index[i] > numphase)
      return shdom::host_fail("shdom_phase_function_mixing: phase index out of range");
  // Wigner functions at the test angles, once
  std::vector<std::vector<double>> D00(nangles), D20(nangles);
  for (int j = 0; j < nangles; ++j) {
    const double x = std::cos(M_PI * j / (nangles - 1));
    wigner_00_20(x, nleg, D00[j], D20[j]);
  }
  const double ofourpi = 1.0 / (4.0 * M_PI);
  std::vector<float> asym;                 // per kept entry
  std::vector<float> p11, dolp;            // [entry][nangles]
  std::vector<float> w(row), ph(nangles), dl(nangles);
  std::fill(mixed_table, mixed_table + (size_t)maxnphase * row, 0.0f);
  int nphase = 0;
  if (fail_point) *fail_point = -1;
  for (int i = 0; i < npts; ++i) {
    mixed_index[i] = 0;
    std::fill(w.begin(), w.end(), 0.0f);
    double scat = 0.0;
    for (int p = 0; p < npart; ++p) {
      const float sc = scatter[(size_t)i * npart + p];
      scat += sc;
      for (int k = 0; k < nmicro; ++k) {
        const size_t o = ((size_t)p * npts + i) * nmicro + k;
        const float f = sc * phase_weight[o];
        const float *t = phase_tables + (size_t)(phase_index[o] - 1) * row;
        for (size_t e = 0; e < row; ++e) w[e] += f * t[e];
      }
    }
    if (!(scat > 0.0)) continue;
    for (size_t e = 0; e < row; ++e) w[e] = (float)(w[e] / scat);
    const float a0 = nleg >= 1 ? w[(size_t)1 * nstleg] / 3.0f : 0.0f;
    for (int j = 0; j < nangles; ++j) {
      double a1 = 0.0, b1 = 0.0;
      for (int l = 0; l <= nleg; ++l) {
        a1 += (double)w[(size_t)l * nstleg] * D00[j][l];
        if (nstleg == 6) b1 -= (double)w[(size_t)l * nstleg + 4] * D20[j][l];
      }
      if (a1 <= 0.0)
        return shdom::host_fail("shdom_phase_function_mixing: negative phase function at grid point " +
                                std::to_string(i));
      ph[j] = (float)(a1 * ofourpi);
      dl[j] = (float)(b1 * ofourpi) / ph[j];
    }
    int use = -1;
    if (nphase > 0) {
      int best = 0;
      float besterr = 1000.0f;
      for (int q = 0; q < nphase; ++q) {
        float ep = 0.0f, ed = 0.0f;
        for (int j = 0; j < nangles; ++j) {
          const float r = p11[(size_t)q * nangles + j], d = dolp[(size_t)q * nangles + j];
          ep = std::max(ep, std::fabs((ph[j] - r) / std::max(0.001f, r)));
          ed = std::max(ed, std::fabs((dl[j] - d) / std::max(0.001f, d)));
        }
        const float err = (float)(std::fabs(a0 - asym[q]) / asym_tol + ep / phase_tol + ed / dolp_tol);
        if (err < besterr) { besterr = err; best = q; }
      }
      float ep = 0.0f, ed = 0.0f;
      for (int j = 0; j < nangles; ++j) {
        const float r = p11[(size_t)best * nangles + j], d = dolp[(size_t)best * nangles + j];
        ep = std::max(ep, std::fabs((ph[j] - r) / std::max(0.001f, r)));
        ed = std::max(ed, std::fabs((dl[j] - d) / std::max(0.001f, d)));
      }
      if (std::fabs(a0 - asym[best]) < asym_tol && phase_tol > ep && dolp_tol > ed) use = best;
    }
    if (use < 0) {
      if (nphase >= maxnphase) {
        *nphase_out = nphase + 1;
        if (fail_point) *fail_point = i + 1;
        return shdom::host_fail("Maximum number of phase functions exceeded when mixing optical properties of "
                                "different particle species. Either decrease accuracy tolerance or increase "
                                "maxnphase. nphase=" + std::to_string(nphase + 1) + " maxnphase=" +
                                std::to_string(maxnphase) + " gridpoint=" + std::to_string(i + 1));
      }
      std::copy(w.begin(), w.end(), mixed_table + (size_t)nphase * row);
      asym.push_back(a0);
      p11.insert(p11.end(), ph.begin(), ph.end());
      dolp.insert(dolp.end(), dl.begin(), dl.end());
      use = nphase++;
    }
    mixed_index[i] = use + 1;
  }
  *nphase_out = nphase;
  return 0;
}
