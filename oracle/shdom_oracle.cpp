// shdom_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference SHDOM solve / render path (AT3D 4.1.3,
// Fortran in src/polarized/*.f, src/shdom_nompi.f, src/surface.f).  It is
// the checker that the GPU path is compared against; nothing in the
// at3d_gb300 package may include, link or call it.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline leg use it.
//
// Parity pinning: the restatement is checked against the reference's own
// golden files tests/data/brdf_L1{f,r}.out (original SHDOM fluxes and
// radiances, tests/test_shdom.py:597-632) through tests/golden/.
//
// The numeric type of the reference's REAL arrays is the template parameter
// R (float reproduces the reference, double gives the FP64 oracle).  Local
// variables the reference declares DOUBLE PRECISION are double in both.
// Each routine cites the reference routine it restates.  Indices are 0-based
// here; "no neighbour" is -1 (the reference uses 0 with 1-based cells).
//
// Differences from the reference:
//  * the azimuthal transform always uses the DFT (the reference switches to
//    FFTPACK RFFTB/RFFTF when NPHI0>14, src/polarized/shdomsub2.f:1137); the
//    two are the same linear map (src/polarized/shdomsub1.f:3008-3030,
//    :3222-3237), only rounding differs;
//  * adaptive cell splitting is not implemented (splitacc must be <= 0);
//  * the 2D independent-pixel sweep (ipflag 1 or 2) is not implemented;
//  * NSTOKES is 1 or 3 (the V component, NSTOKES = 4, is not restated).

#include "../include/shdom_problem.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace orc {

static const int kGoodNFFT[256] = {
    1,   2,   3,   4,   5,   6,   7,   8,   9,   10,  11,  12,  13,  14,  16,  16,  18,  18,  20,
    20,  24,  24,  24,  24,  25,  27,  27,  30,  30,  30,  32,  32,  36,  36,  36,  36,  40,  40,
    40,  40,  45,  45,  45,  45,  45,  48,  48,  48,  50,  50,  54,  54,  54,  54,  60,  60,  60,
    60,  60,  60,  64,  64,  64,  64,  72,  72,  72,  72,  72,  72,  72,  72,  80,  80,  80,  80,
    80,  80,  80,  80,  81,  90,  90,  90,  90,  90,  90,  90,  90,  90,  96,  96,  96,  96,  96,
    96,  100, 100, 100, 100, 108, 108, 108, 108, 108, 108, 108, 108, 120, 120, 120, 120, 120, 120,
    120, 120, 120, 120, 120, 120, 128, 128, 128, 128, 128, 128, 128, 128, 144, 144, 144, 144, 144,
    144, 144, 144, 144, 144, 144, 144, 144, 144, 144, 144, 160, 160, 160, 160, 160, 160, 160, 160,
    160, 160, 160, 160, 160, 160, 160, 160, 180, 180, 180, 180, 180, 180, 180, 180, 180, 180, 180,
    180, 180, 180, 180, 180, 180, 180, 180, 180, 192, 192, 192, 192, 192, 192, 192, 192, 192, 192,
    192, 192, 200, 200, 200, 200, 200, 200, 200, 200, 216, 216, 216, 216, 216, 216, 216, 216, 216,
    216, 216, 216, 216, 216, 216, 216, 240, 240, 240, 240, 240, 240, 240, 240, 240, 240, 240, 240,
    240, 240, 240, 240, 240, 240, 240, 240, 240, 240, 240, 240, 256, 256, 256, 256, 256, 256, 256,
    256, 256, 256, 256, 256, 256, 256, 256, 256};

// Face corner table (GRIDFACE in src/polarized/shdomsub1.f:3726), 0-based.
static const int kGridFace[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5},
                                    {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
static const int kOppFace[6] = {1, 0, 3, 2, 5, 4};

// Normalized Wigner d^l_{m0}(x)*sqrt(l+1/2) for l = 0..lmax at fixed m >= 0
// (WIGNERFCT02P2M_NORMALIZED dm0 output, src/polarized/shdomsub2.f:4357-4395).
static void wigner_dm0(double x, int lmax, int m, std::vector<double> &d) {
  d.assign(lmax + 1, 0.0);
  if (m > lmax) return;
  if (m == 0) {
    d[0] = 1.0;
    if (lmax >= 1) d[1] = x;
    for (int n = 1; n < lmax; ++n) d[n + 1] = ((2 * n + 1) * x * d[n] - n * d[n - 1]) / (n + 1);
  } else {
    // d^m_{m0} = (-1)^m sqrt((2m)!)/(2^m m!) (1-x^2)^{m/2}  (DMM1_N0 with m1=0)
    double prod = 1.0;
    for (int p = 1; p <= m; ++p) prod *= std::sqrt((double)(m + p) / (double)p);
    double s = std::sqrt((1.0 - x) * (1.0 + x)) * 0.5;
    d[m] = ((m & 1) ? -1.0 : 1.0) * prod * std::pow(s, m);
    for (int n = m; n < lmax; ++n) {
      double a = std::sqrt((double)((n + 1) * (n + 1) - m * m));
      double b = (n > m) ? std::sqrt((double)(n * n - m * m)) : 0.0;
      d[n + 1] = ((2 * n + 1) * x * d[n] - b * (n > m ? d[n - 1] : 0.0)) / a;
    }
  }
  for (int n = 0; n <= lmax; ++n) d[n] *= std::sqrt(n + 0.5);
}

// Wigner d^n_{m m1}(x) at n = max(m, m1) for m, m1 >= 0 (DMM1_N0,
// src/polarized/shdomsub2.f:4431-4461): the closed form
// c sqrt(prod_{p=1}^{|m-m1|} (m+m1+p)/p) ((1-x)/2)^{|m-m1|/2} ((1+x)/2)^{(m+m1)/2}.
static double wigner_start(double x, int m, int m1) {
  if (m == m1) return std::pow((1.0 + x) / 2.0, m);
  const double c = (m1 > m) ? 1.0 : (((m - m1) & 1) ? -1.0 : 1.0);
  const int hi = std::max(m, m1), lo = std::min(m, m1);
  double prod = 1.0;
  for (int q = 1; q <= hi - lo; ++q) prod *= std::sqrt((double)(m + m1 + q) / (double)q);
  return c * prod * std::pow(std::sqrt((1.0 - x) / 2.0), hi - lo) * std::pow(std::sqrt((1.0 + x) / 2.0), hi + lo);
}

// Wigner d^n_{m m1}(x), n = 0..lmax, by the three-term upward recurrence in n
// (WIGNERFCT, src/polarized/shdomsub2.f:4604-4646), not normalised.
static void wigner_d(double x, int lmax, int m, int m1, std::vector<double> &d) {
  d.assign(lmax + 1, 0.0);
  const int n0 = std::max(m, m1);
  if (n0 == 0) {
    d[0] = 1.0;
    if (lmax >= 1) d[1] = x;
    for (int n = 1; n < lmax; ++n) d[n + 1] = (double)(2 * n + 1) * x / (n + 1) * d[n] - (double)n / (n + 1) * d[n - 1];
    return;
  }
  if (n0 > lmax) return;
  d[n0] = wigner_start(x, m, m1);
  for (int n = n0; n < lmax; ++n) {
    const double a = std::sqrt((double)((n + 1) * (n + 1) - m * m)), b = std::sqrt((double)((n + 1) * (n + 1) - m1 * m1));
    const double f1 = ((double)(n * (n + 1)) * x - (double)(m * m1)) / a / b * (double)(2 * n + 1) / n;
    const double f2 = std::sqrt((double)(n * n - m * m)) * std::sqrt((double)(n * n - m1 * m1)) / a / b * (double)(n + 1) / n;
    d[n + 1] = f1 * d[n] - f2 * (n > n0 ? d[n - 1] : 0.0);
  }
}

// The m1 = +2 and m1 = -2 functions of WIGNERFCT02P2M_NORMALIZED
// (src/polarized/shdomsub2.f:4363-4428): d^n_{m,2}(x) and
// d^n_{m,-2}(x) = (-1)^{n+m} d^n_{m,2}(-x), both times sqrt(n + 1/2).
static void wigner_d2pm(double x, int lmax, int m, std::vector<double> &dp, std::vector<double> &dm) {
  dp.assign(lmax + 1, 0.0); dm.assign(lmax + 1, 0.0);
  if (m > lmax || lmax < 2) return;
  const int n0 = std::max(m, 2);
  dp[n0] = wigner_start(x, m, 2);
  dm[n0] = wigner_start(-x, m, 2);
  for (int n = n0; n < lmax; ++n) {
    const double a = std::sqrt((double)((n + 1) * (n + 1) - m * m)), b = std::sqrt((double)((n + 1) * (n + 1) - 4));
    const double f1 = 1.0 / a / b * (double)(2 * n + 1) / n;
    const double f2 = std::sqrt((double)(n * n - m * m)) * std::sqrt((double)(n * n - 4)) / a / b * (double)(n + 1) / n;
    const double fp = (double)(n * (n + 1)) * x - 2.0 * m, fm = -(double)(n * (n + 1)) * x - 2.0 * m;
    dp[n + 1] = fp * f1 * dp[n] - f2 * (n > n0 ? dp[n - 1] : 0.0);
    dm[n + 1] = fm * f1 * dm[n] - f2 * (n > n0 ? dm[n - 1] : 0.0);
  }
  for (int n = 0; n <= lmax; ++n) {
    dm[n] *= ((n + m) & 1) ? -1.0 : 1.0;
    dp[n] *= std::sqrt(n + 0.5);
    dm[n] *= std::sqrt(n + 0.5);
  }
}

static inline int sh_index(int l, int m, int mm) {
  // J = L(L+1)+M (L<=MM) or (2MM+1)L-MM^2+M, 0-based (YLMALL header,
  // src/polarized/shdomsub2.f:4252-4253).
  return (l <= mm) ? l * (l + 1) + m : (2 * mm + 1) * l - mm * mm + m;
}

// The six elements of the real generalized spherical functions, in the
// reference's element order (1 I-I, 2 Q-Q, 3 U-U, 4 V-V, 5 I-Q, 6 Q-U):
// PLMALL (src/polarized/shdomsub2.f:4650-4755) for the mu part alone
// (phi < 0: out[j][6] is P), YLMALL (src/polarized/shdomsub2.f:4244-4354)
// with the azimuth factors.  transpose flips the sign of the 5/6 parts that
// the transposed matrices carry.
static void genylm6(bool transpose, double x, double phi, bool with_phi, int ml, int mm, std::vector<double> &out) {
  const int nlm = (2 * mm + 1) * (ml + 1) - mm * (mm + 1);
  out.assign((size_t)nlm * 6, 0.0);
  const double fct = 1.0 / std::sqrt(2.0 * std::acos(-1.0)), sg = transpose ? -1.0 : 1.0;
  std::vector<double> d0, dp, dm;
  for (int ma = 0; ma <= mm; ++ma) {
    wigner_dm0(x, ml, ma, d0);
    wigner_d2pm(x, ml, ma, dp, dm);
    const double c = (with_phi && ma > 0) ? std::cos(ma * phi) : 1.0, s = (with_phi && ma > 0) ? std::sin(ma * phi) : 0.0;
    for (int l = ma; l <= ml; ++l) {
      const double p1 = fct * d0[l], p2 = -0.5 * fct * (dp[l] + dm[l]), p3 = -0.5 * fct * (dp[l] - dm[l]);
      double *o = &out[(size_t)sh_index(l, ma, mm) * 6];
      if (ma == 0 || !with_phi) {
        o[0] = p1; o[1] = p2; o[2] = p2; o[3] = p1; o[4] = p3; o[5] = p3;
      } else {
        o[0] = p1 * c - p1 * s; o[1] = p2 * c - p2 * s; o[2] = p2 * c + p2 * s;
        o[3] = p1 * c + p1 * s; o[4] = p3 * c - sg * p3 * s; o[5] = p3 * c + sg * p3 * s;
      }
      if (ma == 0) continue;
      double *n = &out[(size_t)sh_index(l, -ma, mm) * 6];
      if (!with_phi) {
        n[0] = p1; n[1] = p2; n[2] = -p2; n[3] = -p1; n[4] = sg * p3; n[5] = -sg * p3;
      } else {
        n[0] = p1 * s + p1 * c; n[1] = p2 * s + p2 * c; n[2] = p2 * s - p2 * c;
        n[3] = p1 * s - p1 * c; n[4] = p3 * s + sg * p3 * c; n[5] = p3 * s - sg * p3 * c;
      }
    }
  }
}

template <typename R>
struct Solver {
  shdom_problem p{};
  std::vector<float> zlev, extp, albp, phwtp, legp, sfcalb;
  // input Legendre table: legenp [numphase][nlegp+1] or, polarized,
  // [numphase][nlegp+1][6] (LEGENP(NSTLEG,0:NLEGP,NUMPHASE))
  float leg_in(int i, int l, int k) const { return legp[((size_t)i * (p.nlegp + 1) + l) * nstleg + k]; }
  std::vector<int> iphp;
  std::string err;

  // grid
  int nx = 0, ny = 0, nz = 0, nx1 = 0, ny1 = 0, npts = 0, ncells = 0, bcflag = 0, ipflag = 0;
  std::vector<float> xgrid, ygrid, zgrid, gridpos;  // gridpos[npts][3]
  std::vector<int> gridptr, neighptr;              // [ncells][8], [ncells][6]
  std::vector<short> cellflags;
  // Adaptive grid (SPLIT_GRID and its helpers, src/polarized/shdomsub1.f:
  // 4703-5902): treeptr [ncells][2] holds the parent (-1 for a base cell)
  // and the first of the two children (0 for an end cell); bits 2-3 of
  // cellflags hold the direction a parent was split in (1 X, 2 Y, 3 Z).  A
  // neighbour that has children is stored as -(cell + 2); -1 is no
  // neighbour.  nbpts / nbcells: the base grid.
  std::vector<int> treeptr;
  int nbpts = 0, nbcells = 0;
  float adapt_grid_factor = 5.f, cell_to_point_ratio = 1.5f, num_sh_term_factor = 1.f;
  static int nb_cell(int v) { return v >= -1 ? v : -v - 2; }
  static int nb_parent(int c) { return -c - 2; }
  int split_dir(int c) const { return (cellflags[c] >> 2) & 3; }
  bool outofmem = false;
  int noct = 8;
  std::vector<int> sweep_cell, sweep_corner;  // [noct][npts]

  // angles
  int nmu = 0, nphi = 0, ml = 0, mm = 0, nlm = 0, nphi0max = 0, nang = 0, nleg = 0;
  std::vector<int> nphi0, lofj, mofj;
  std::vector<float> mu, wtmu, phi, wtdo;  // phi/wtdo [nmu][nphi0max]
  std::vector<R> cmu1, cmu2;               // [nmu][nlm]
  std::vector<R> cphi1, cphi2;             // [nmu][nphi0max][2mm+1] (m index offset +mm)
  std::vector<R> ylmsun;                   // [nlm]
  // polarized (nst = 3): Stokes components per SH term / ordinate value
  int nst = 1, nstleg = 1;
  std::vector<R> cmu1p, cmu2p;             // [nmu][nlm][6] generalized functions (CMU1 / CMU2)

  // medium on the grid
  int npart = 0, maxnmicro = 0, numphase = 0, nq = 0;
  std::vector<R> extinct, albedo, total_ext;  // [npart][npts], [npts]
  std::vector<int> iphase;                    // [npart][npts][8*maxnmicro]
  std::vector<R> phaseinterpwt;
  std::vector<R> legen;  // [numphase][nleg+1] (the I-I element)
  std::vector<R> legen6;  // [numphase][6][nleg+1] all six elements when nst = 3
  double extmin = 0, scatmin = 0;
  R albmax = 0;
  // RENDER's SINGLESCATTER / NOSURFACE switches (src/polarized/shdomsub2.f:3107-3142, :2721-2723)
  int rsingle = 0, rnosfc = 0;
  const float phasemax = 0.999f;

  // direct beam
  std::vector<R> dirflux;
  // solution
  std::vector<R> source, delsource, radiance, fluxes;  // fluxes [npts][2]
  std::vector<int> shptr, rshptr, oshptr;
  R deljdot = 0, deljold = 0, deljnew = 0, jnorm = 0;
  R solcrit = 1, accel_a = 0;
  int iter = 0;
  // boundaries
  std::vector<int> topp, botp;
  std::vector<R> sfcgridalb;  // per bottom point
  // bidirectional surface: type ('R', 'W'; 0 Lambertian), parameters on the
  // surface grid and at the bottom points, and the downwelling radiances at
  // the bottom points for every downward ordinate [nbot][nang/2][nst]
  int brdf = 0, nsfcpar = 0;
  std::vector<float> sfcpar;
  std::vector<R> botpar, bcdown;
  std::vector<R> bcrad_top, bcrad_bot;
  bool sweep_ready = false;
  // Thermal emission: srct is 'S', 'T' or 'B'; temp the temperature of each
  // grid point; planck_tot the extinction-weighted (1 - albedo) B(T) of each
  // point (TOTAL_PLANCK of COMPUTE_SOURCE); botplanck B at the bottom points
  // (SFCGRIDPARMS(1)); skyrad_bc the radiance of the top boundary.
  char srct = 'S', unitc = 'R';
  // INTLOW / INTHIGH: the integral of x^3/(e^x - 1) from 0 to x by its
  // Taylor series (the Bernoulli-number expansion of x/(e^x - 1), through
  // x^29) and from x to infinity by the exponential series (15 terms)
  static double int_low(double x) {
    double b[28], s = 0, fact = 1, pw;
    b[0] = 1;
    for (int m = 1; m < 28; ++m) {
      double acc = 0, binom = 1;  // C(m+1, k)
      for (int k = 0; k < m; ++k) { acc += binom * b[k]; binom = binom * (m + 1 - k) / (k + 1); }
      b[m] = -acc / (m + 1);
    }
    for (int n = 0; n + 3 <= 29; ++n) {
      if (n > 0) fact *= n;
      if (n != 1 && (n & 1)) continue;
      pw = std::pow(x, n + 3);
      s += b[n] / (fact * (n + 3)) * pw;
    }
    return s;
  }
  static double int_high(double x) {
    double s = 0;
    for (int n = 1; n <= 15; ++n)
      s += std::exp(-n * x) * (std::pow(x, 3) / n + 3 * x * x / std::pow(n, 2) + 6 * x / std::pow(n, 3) + 6.0 / std::pow(n, 4));
    return s;
  }
  static double band_integral(double x1, double x2) {
    if (x1 < 1.0 && x2 < 1.0) return int_low(x2) - int_low(x1);
    if (x1 < 1.0) return int_low(1.0) - int_low(x1) + int_high(1.0) - int_high(x2);
    return int_high(x1) - int_high(x2);
  }
  std::vector<float> tempp_in, sfctemp_in, temp;
  std::vector<R> planck_tot, botplanck;
  float skyrad_bc = 0.f;

  // PLANCK_FUNCTION (src/polarized/shdomsub2.f:4756-4791) for units 'R'
  // (W/(m^2 sr micron) at p.wavelen), 'T' (brightness temperature) and 'B'
  // (INTEGRATE_PLANCK over the band p.waveno, W/(m^2 sr)).
  float planck_fn(float t) const {
    if (unitc == 'T') return t;
    if (t <= 0.f) return 0.f;
    if (unitc == 'B') {
      const double x1 = 1.4388 * p.waveno[0] / t, x2 = 1.4388 * p.waveno[1] / t;
      return (float)(1.1911e-8 * std::pow(t / 1.4388, 4) * band_integral(x1, x2));
    }
    const float w = p.wavelen;
    return 1.1911e8f / (w * w * w * w * w) / (std::exp(1.4388e4f / (w * t)) - 1.0f);
  }

  // ------------------------------------------------------------ setup
  bool init(const shdom_problem *in) {
    p = *in;
    int ng = p.npx * p.npy * p.npz;
    zlev.assign(p.zlevels, p.zlevels + p.npz);
    extp.assign(p.extinctp, p.extinctp + (size_t)p.npart * ng);
    albp.assign(p.albedop, p.albedop + (size_t)p.npart * ng);
    iphp.assign(p.iphasep, p.iphasep + (size_t)p.npart * ng * p.maxnmicro);
    phwtp.assign(p.phasewtp, p.phasewtp + (size_t)p.npart * ng * p.maxnmicro);
    nst = p.nstokes;
    if (nst != 1 && nst != 3) { err = "nstokes must be 1 or 3"; return false; }
    nstleg = nst == 1 ? 1 : 6;
    legp.assign(p.legenp, p.legenp + (size_t)p.numphase * (p.nlegp + 1) * nstleg);
    if (p.sfc_variable) sfcalb.assign(p.sfc_albedo, p.sfc_albedo + (size_t)p.nxsfc * p.nysfc);
    brdf = p.sfc_brdf; nsfcpar = p.nsfcpar;
    if (brdf) {
      if ((brdf != 'R' && brdf != 'W' && brdf != 'D' && brdf != 'O' && brdf != 'M') ||
          p.nsfcpar < (brdf == 'D' ? 5 : brdf == 'O' ? 2 : 3) || !p.sfc_params || p.nxsfc < 1 || p.nysfc < 1) {
        err = "surface BRDF: types 'R' (RPV), 'W' (wave-Fresnel), 'M' (Ross-Li; 3 parameters each), 'D' (Diner; 5) and 'O' (ocean; 2) on a surface grid";
        return false;
      }
      if (brdf == 'R' && nst != 1) { err = "RPV BRDF is only for unpolarized case"; return false; }
      if (brdf == 'O' && nst != 1) { err = "Ocean BRDF from 6S is only for unpolarized case"; return false; }
      if (brdf == 'M' && nst != 1) { err = "RossLiThick-Sparse is only for unpolarized case"; return false; }
      if (brdf == 'O' && !(p.wavelen > 0.f)) { err = "the ocean BRDF needs the wavelength"; return false; }
      sfcpar.assign(p.sfc_params, p.sfc_params + (size_t)p.nxsfc * p.nysfc * p.nsfcpar);
    }
    srct = p.srctype ? (char)p.srctype : 'S';
    unitc = p.units ? (char)p.units : 'R';
    if (srct != 'S' && srct != 'T' && srct != 'B') { err = "srctype must be 'S', 'T' or 'B'"; return false; }
    if (unitc != 'R' && unitc != 'T' && unitc != 'B') { err = "units must be 'R', 'T' or 'B'"; return false; }
    if (srct != 'S') {
      if (!p.tempp) { err = "a thermal source needs the temperature field"; return false; }
      if (unitc == 'R' && !(p.wavelen > 0.f)) { err = "a thermal source in radiance units needs the wavelength"; return false; }
      tempp_in.assign(p.tempp, p.tempp + ng);
      if (p.sfc_temp && p.nxsfc > 0 && p.nysfc > 0 && (p.sfc_variable || brdf))
        sfctemp_in.assign(p.sfc_temp, p.sfc_temp + (size_t)p.nxsfc * p.nysfc);
    }
    p.tempp = nullptr; p.sfc_temp = nullptr;
    // COMPUTE_TOP_RADIANCES: the sky temperature becomes a radiance only for 'T'
    skyrad_bc = (srct == 'T') ? planck_fn(p.skyrad) : p.skyrad;
    p.sfc_params = nullptr;
    p.zlevels = nullptr; p.extinctp = p.albedop = p.phasewtp = p.legenp = p.sfc_albedo = nullptr;
    p.iphasep = nullptr;
    if (!setup_grid()) return false;
    if (p.splitacc > 0 && ipflag != 0) { err = "adaptive splitting is restated for 3D grids only"; return false; }
    setup_angles();
    if (!transfer_properties()) return false;
    return true;
  }

  // _setup_grid (at3d/solver.py:2036-2168), NEW_GRIDS and INIT_CELL_STRUCTURE
  // (src/polarized/shdomsub2.f:16-310).
  bool setup_grid() {
    nx = std::max(1, p.npx); ny = std::max(1, p.npy); nz = std::max(2, p.npz);
    ipflag = p.ipflag;
    if (nx == 1) ipflag |= 1;
    if (ny == 1) ipflag |= 2;
    bcflag = 0;
    if (p.bc_x_open && (ipflag == 0 || ipflag == 2 || ipflag == 4 || ipflag == 6)) bcflag += 1;
    if (p.bc_y_open && (ipflag == 0 || ipflag == 1 || ipflag == 4 || ipflag == 5)) bcflag += 2;
    if (bcflag == 1) { err = "open x with periodic y boundaries is not supported"; return false; }
    if ((ipflag & 3) == 1 || (ipflag & 3) == 2) { err = "2D independent pixel mode is not supported"; return false; }
    nx1 = nx + 1; ny1 = ny + 1;
    if ((bcflag & 5) || (ipflag & 1)) nx1 -= 1;
    if ((bcflag & 7) || (ipflag & 2)) ny1 -= 1;
    xgrid.resize(nx + 1); ygrid.resize(ny + 1);
    float dxp = p.delx > 0 ? p.delx : 1.0f, dyp = p.dely > 0 ? p.dely : 1.0f;
    for (int i = 0; i <= nx; ++i) xgrid[i] = ((float)i * (dxp * (float)p.npx)) / (float)nx;
    for (int i = 0; i <= ny; ++i) ygrid[i] = ((float)i * (dyp * (float)p.npy)) / (float)ny;
    zgrid = zlev;
    npts = nx1 * ny1 * nz;
    gridpos.resize((size_t)npts * 3);
    int ip = 0;
    for (int ix = 0; ix < nx1; ++ix)
      for (int iy = 0; iy < ny1; ++iy)
        for (int iz = 0; iz < nz; ++iz, ++ip) {
          gridpos[3 * ip] = xgrid[ix]; gridpos[3 * ip + 1] = ygrid[iy]; gridpos[3 * ip + 2] = zgrid[iz];
        }
    int nxc = nx, nyc = ny;
    if (bcflag & 1) nxc = nx + 1;
    if (bcflag & 2) nyc = ny + 1;
    ncells = nxc * nyc * (nz - 1);
    gridptr.assign((size_t)ncells * 8, 0); neighptr.assign((size_t)ncells * 6, -1);
    cellflags.assign(ncells, 0);
    int ic = 0;
    for (int ix = 1; ix <= nxc; ++ix) {
      int ix0, ix1;
      if (ipflag & 1) { ix0 = ix; ix1 = ix; }
      else if (bcflag & 1) { ix0 = std::max(1, ix - 1); ix1 = std::min(nx, ix); }
      else { ix0 = ix; ix1 = ix + 1; }
      for (int iy = 1; iy <= nyc; ++iy) {
        int iy0, iy1;
        if (ipflag & 2) { iy0 = iy; iy1 = iy; }
        else if (bcflag & 2) { iy0 = std::max(1, iy - 1); iy1 = std::min(ny, iy); }
        else { iy0 = iy; iy1 = iy + 1; }
        for (int iz = 1; iz <= nz - 1; ++iz, ++ic) {
          int *g = &gridptr[8 * ic];
          auto P = [&](int z, int y, int x) { return (z - 1) + nz * (y - 1) + nz * ny1 * (x - 1); };
          g[0] = P(iz, iy0, ix0); g[1] = P(iz, iy0, ix1); g[2] = P(iz, iy1, ix0); g[3] = P(iz, iy1, ix1);
          g[4] = P(iz + 1, iy0, ix0); g[5] = P(iz + 1, iy0, ix1); g[6] = P(iz + 1, iy1, ix0);
          g[7] = P(iz + 1, iy1, ix1);
          int *nb = &neighptr[6 * ic];
          int sx = (nz - 1) * nyc;
          if (ipflag & 1) { nb[0] = ic; nb[1] = ic; cellflags[ic] |= 1; }
          else if (bcflag & 1) {
            if (ix == 1) { nb[0] = ic; nb[1] = ic + sx; cellflags[ic] |= 1; }
            else if (ix == nxc) { nb[0] = ic - sx; nb[1] = ic; cellflags[ic] |= 1; }
            else { nb[0] = ic - sx; nb[1] = ic + sx; }
          } else {
            nb[0] = (ix == 1) ? ic + (nxc - 1) * sx : ic - sx;
            nb[1] = (ix == nx) ? ic - (nxc - 1) * sx : ic + sx;
          }
          int sy = nz - 1;
          if (ipflag & 2) { nb[2] = ic; nb[3] = ic; cellflags[ic] |= 2; }
          else if (bcflag & 2) {
            if (iy == 1) { nb[2] = ic; nb[3] = ic + sy; cellflags[ic] |= 2; }
            else if (iy == nyc) { nb[2] = ic - sy; nb[3] = ic; cellflags[ic] |= 2; }
            else { nb[2] = ic - sy; nb[3] = ic + sy; }
          } else {
            nb[2] = (iy == 1) ? ic + (nyc - 1) * sy : ic - sy;
            nb[3] = (iy == ny) ? ic - (nyc - 1) * sy : ic + sy;
          }
          nb[4] = (iz == 1) ? -1 : ic - 1;
          nb[5] = (iz == nz - 1) ? -1 : ic + 1;
        }
      }
    }
    treeptr.assign((size_t)2 * ncells, 0);
    for (int c = 0; c < ncells; ++c) treeptr[2 * c] = -1;
    nbpts = npts; nbcells = ncells;
    return true;
  }

  // NEXT_CELL (src/polarized/shdomsub1.f:4470-4527): the end cell across face
  // iface (0-5: -X,+X,-Y,+Y,-Z,+Z; jface its axis) of icell that contains
  // (xe, ye, ze).
  int next_cell(double xe, double ye, double ze, int iface, int jface, int icell) const {
    int v = neighptr[6 * icell + iface];
    if (v >= -1) return v;
    int ic = nb_cell(v);
    const double pos[3] = {xe, ye, ze};
    while (treeptr[2 * ic + 1] > 0) {
      int dir = split_dir(ic), c1 = treeptr[2 * ic + 1];
      if (dir == jface + 1) ic = c1 + 1 - (iface % 2);
      else ic = (pos[dir - 1] > gridpos[3 * gridptr[8 * c1 + 7] + dir - 1]) ? c1 + 1 : c1;
    }
    return ic;
  }

  // SWEEPING_ORDER / SWEEP_BASE_CELL (src/polarized/shdomsub1.f:3261-3351,
  // :4529-4622), base grid only.
  void sweeping_order() {
    static const int ioctorder[8] = {1, 5, 2, 6, 3, 7, 4, 8};
    if ((ipflag & 2) && (ipflag & 1)) noct = 2;
    else if (ipflag & 2) noct = 4;
    else noct = 8;
    int nxc = nx, nyc = ny;
    if (bcflag & 1) nxc = nx + 1;
    if (bcflag & 2) nyc = ny + 1;
    sweep_cell.assign((size_t)noct * npts, 0); sweep_corner.assign((size_t)noct * npts, 0);
    std::vector<char> done(npts);
    for (int joct = 0; joct < noct; ++joct) {
      int ioct = ioctorder[joct];
      int b = ioct - 1;
      int dix, six, eix, diy, siy, eiy, diz, siz, eiz;
      if (b & 1) { dix = 1; if (bcflag & 1) { six = nxc; eix = std::max(nxc - 1, 1); } else { six = 1; eix = nxc; } }
      else { dix = -1; if (bcflag & 1) { six = 1; eix = std::min(2, nxc); } else { six = nxc; eix = 1; } }
      if (b & 2) { diy = 1; if (bcflag & 2) { siy = nyc; eiy = std::max(nyc - 1, 1); } else { siy = 1; eiy = nyc; } }
      else { diy = -1; if (bcflag & 2) { siy = 1; eiy = std::min(2, nyc); } else { siy = nyc; eiy = 1; } }
      if (b & 4) { diz = 1; siz = 1; eiz = nz - 1; } else { diz = -1; siz = nz - 1; eiz = 1; }
      std::fill(done.begin(), done.end(), 0);
      int iorder = 0;
      int ix = six, iy = siy, iz = siz;
      std::vector<int> stack;
      while (true) {
        // SWEEP_NEXT_CELL: the end cells of this base cell's tree, the child
        // on the upwind side of each split first
        stack.assign(1, (iz - 1) + (nz - 1) * (iy - 1) + (nz - 1) * nyc * (ix - 1));
        while (!stack.empty()) {
          int icell = stack.back();
          stack.pop_back();
          if (treeptr[2 * icell + 1] > 0) {
            int c1 = treeptr[2 * icell + 1];
            bool first_neg = (b >> (split_dir(icell) - 1)) & 1;
            stack.push_back(first_neg ? c1 + 1 : c1);
            stack.push_back(first_neg ? c1 : c1 + 1);
            continue;
          }
          for (int k = 0; k < 8; ++k) {
            int corner = (k ^ b) ^ 7;
            int ipt = gridptr[8 * icell + corner];
            if (done[ipt]) continue;
            done[ipt] = 1;
            sweep_cell[(size_t)joct * npts + iorder] = icell;
            sweep_corner[(size_t)joct * npts + iorder] = corner;
            ++iorder;
          }
        }
        if (ix == eix) {
          if (iy == eiy) {
            if (iz == eiz) break;
            iz += diz;
            iy = siy;
          } else {
            iy = (iy + diy + nyc - 1) % nyc + 1;
          }
          ix = six;
        } else {
          ix = (ix + dix + nxc - 1) % nxc + 1;
        }
      }
    }
    sweep_ready = true;
  }

  // MAKE_ANGLE_SET / GAUSQUADS / MAKE_SH_DO_COEF / PLMALL / YLMALL_UNPOL
  // (src/polarized/shdomsub2.f:1061-1220, :4874-4912, :4650-4755, :4497-4535).
  void setup_angles() {
    nmu = std::max(2, 2 * ((p.nmu + 1) / 2));
    nphi = std::max(1, p.nphi);
    ml = nmu - 1;
    mm = std::max(0, nphi / 2 - 1);
    nlm = (2 * mm + 1) * (ml + 1) - mm * (mm + 1);
    nleg = p.deltam ? ml + 1 : ml;
    nphi0max = nphi;
    lofj.resize(nlm); mofj.resize(nlm);
    for (int l = 0, j = 0; l <= ml; ++l)
      for (int m = -std::min(l, mm); m <= std::min(l, mm); ++m, ++j) { lofj[j] = l; mofj[j] = m; }
    mu.resize(nmu); wtmu.resize(nmu);
    int k = nmu / 2;
    for (int j = 1; j <= k; ++j) {
      double x = std::cos(3.141592654 * (j - .25) / (nmu + .5)), xp, pl, pl1, pl2, dpl;
      int it = 0;
      do {
        pl1 = 1; pl = x;
        for (int l = 2; l <= nmu; ++l) { pl2 = pl1; pl1 = pl; pl = ((2 * l - 1) * x * pl1 - (l - 1) * pl2) / l; }
        dpl = nmu * (x * pl - pl1) / (x * x - 1);
        xp = x; x = xp - pl / dpl; ++it;
      } while (std::fabs(x - xp) > 3.0e-7 && it < 10);
      mu[j - 1] = (float)(-x); mu[j - 1 + k] = (float)x;
      wtmu[j - 1] = (float)(2.0 / ((1.0 - x * x) * dpl * dpl)); wtmu[j - 1 + k] = wtmu[j - 1];
    }
    nphi0.resize(nmu);
    phi.assign((size_t)nmu * nphi0max, 0.f); wtdo.assign((size_t)nmu * nphi0max, 0.f);
    nang = 0;
    const float pif = (float)std::acos(-1.0f);
    for (int j = 0; j < nmu; ++j) {
      if (p.angle_set == 1) nphi0[j] = nphi0max;
      else {
        int n = (int)(0.9f + (float)nphi0max * std::sqrt(1.0f - mu[j] * mu[j]));
        nphi0[j] = std::min(nphi0max, kGoodNFFT[std::max(1, n) - 1]);
      }
      float delphi = 2.0f * pif / (float)nphi0[j];
      for (int kk = 0; kk < nphi0[j]; ++kk) {
        phi[(size_t)j * nphi0max + kk] = (float)kk * delphi;
        wtdo[(size_t)j * nphi0max + kk] = delphi * wtmu[j];
      }
      nang += nphi0[j];
    }
    cmu1.assign((size_t)nmu * nlm, 0); cmu2.assign((size_t)nmu * nlm, 0);
    std::vector<double> d;
    const double fct = 1.0 / std::sqrt(2.0 * std::acos(-1.0));
    for (int i = 0; i < nmu; ++i) {
      for (int m = 0; m <= mm; ++m) {
        wigner_dm0((double)mu[i], ml, m, d);
        for (int l = m; l <= ml; ++l) {
          R v = (R)(fct * d[l]);
          int jp = sh_index(l, m, mm), jn = sh_index(l, -m, mm);
          cmu1[(size_t)i * nlm + jp] = v; cmu1[(size_t)i * nlm + jn] = v;
          cmu2[(size_t)i * nlm + jp] = v * (R)wtmu[i]; cmu2[(size_t)i * nlm + jn] = v * (R)wtmu[i];
        }
      }
    }
    if (nst == 3) {
      // MAKE_SH_DO_COEF: CMU1 = PLMALL(.FALSE.), CMU2 = PLMALL(.TRUE.) * WTMU
      cmu1p.assign((size_t)nmu * nlm * 6, 0); cmu2p.assign((size_t)nmu * nlm * 6, 0);
      std::vector<double> prc;
      for (int i = 0; i < nmu; ++i) {
        genylm6(false, (double)mu[i], 0.0, false, ml, mm, prc);
        for (int q = 0; q < nlm * 6; ++q) cmu1p[(size_t)i * nlm * 6 + q] = (R)prc[q];
        genylm6(true, (double)mu[i], 0.0, false, ml, mm, prc);
        for (int q = 0; q < nlm * 6; ++q) cmu2p[(size_t)i * nlm * 6 + q] = (R)prc[q] * (R)wtmu[i];
      }
    }
    int nm = 2 * mm + 1;
    cphi1.assign((size_t)nmu * nphi0max * nm, 0); cphi2.assign((size_t)nmu * nphi0max * nm, 0);
    for (int i = 0; i < nmu; ++i) {
      R w = (R)1 / (R)wtmu[i];
      for (int kk = 0; kk < nphi0[i]; ++kk) {
        R *c1 = &cphi1[((size_t)i * nphi0max + kk) * nm + mm];
        R *c2 = &cphi2[((size_t)i * nphi0max + kk) * nm + mm];
        R wd = (R)wtdo[(size_t)i * nphi0max + kk];
        c1[0] = 1; c2[0] = wd * w;
        for (int m = 1; m <= mm; ++m) {
          R ph = (R)phi[(size_t)i * nphi0max + kk];
          c1[m] = std::cos((R)m * ph); c1[-m] = std::sin((R)m * ph);
          c2[m] = c1[m] * wd * w; c2[-m] = c1[-m] * wd * w;
        }
      }
    }
    // YLMSUN (YLMALL_UNPOL at the solar direction)
    ylmsun = ylmall((double)p.solarmu, p.solaraz);
  }

  std::vector<R> ylmall(double muv, float phiv) const {
    std::vector<R> y(nlm, 0);
    std::vector<double> d;
    const double fct = 1.0 / std::sqrt(2.0 * std::acos(-1.0));
    double x = (double)(float)muv;
    for (int m = 0; m <= mm; ++m) {
      wigner_dm0(x, ml, m, d);
      double cosm = 1, sinm = 0;
      if (m > 0) { cosm = std::cos(m * (double)phiv); sinm = std::sin(m * (double)phiv); }
      for (int l = m; l <= ml; ++l) {
        double v = fct * d[l];
        int j = sh_index(l, m, mm);
        y[j] = (R)((cosm - sinm) * v);
        y[j - 2 * m] = (R)((cosm + sinm) * v);
      }
    }
    return y;
  }

  // TRANSFER_PA_TO_GRID -> INTERP_GRID -> TRILIN_INTERP_PROP -> PREPARE_PROP
  // (src/polarized/shdomsub1.f:19-110, src/polarized/shdomsub2.f:313-390,
  // src/polarized/shdom90.f90:17-350, src/polarized/shdomsub2.f:479-611).
  // TRILIN_INTERP_PROP (src/polarized/shdomsub2.f), 'N' method: species ipa
  // at grid point ipt from the property grid, before the delta-M scaling
  // (extinction, albedo, the phase indices and weights of the 8 corners
  // merged and sorted, and the temperature).
  bool trilin_point(int ipa, int ipt, R &extr) {
    const int npx = p.npx, npy = p.npy, npz = p.npz, ng = npx * npy * npz;
    float x = gridpos[3 * ipt], y = gridpos[3 * ipt + 1], z = gridpos[3 * ipt + 2];
    int il = 0, iu = npz;
    while (iu - il > 1) { int im = (iu + il) / 2; if (z >= zlev[im - 1]) il = im; else iu = im; }
    int iz = std::max(il, 1);
    double w = (double)(z - zlev[iz - 1]) / (zlev[iz] - zlev[iz - 1]);
    w = std::max(std::min(w, 1.0), 0.0);
    int ix = (int)(x / p.delx) + 1;
    if (std::fabs(x - npx * p.delx) < 0.01f * p.delx) ix = npx;
    if (ix < 1 || ix > npx) { err = "TRILIN: Beyond X domain"; return false; }
    int ixp = ix % npx + 1;
    double u = (double)(x - p.delx * (ix - 1)) / p.delx;
    u = std::max(std::min(u, 1.0), 0.0);
    if (u < 1e-5) u = 0; if (u > 1 - 1e-5) u = 1;
    int iy = (int)(y / p.dely) + 1;
    if (std::fabs(y - npy * p.dely) < 0.01f * p.dely) iy = npy;
    if (iy < 1 || iy > npy) { err = "TRILIN: Beyond Y domain"; return false; }
    int iyp = iy % npy + 1;
    double v = (double)(y - p.dely * (iy - 1)) / p.dely;
    v = std::max(std::min(v, 1.0), 0.0);
    if (v < 1e-5) v = 0; if (v > 1 - 1e-5) v = 1;
    double f[8] = {(1 - u) * (1 - v) * (1 - w), u * (1 - v) * (1 - w), (1 - u) * v * (1 - w),
                   u * v * (1 - w),             (1 - u) * (1 - v) * w, u * (1 - v) * w,
                   (1 - u) * v * w,             u * v * w};
    int i1 = (iz - 1) + npz * (iy - 1) + npz * npy * (ix - 1);
    int i2 = (iz - 1) + npz * (iy - 1) + npz * npy * (ixp - 1);
    int i3 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ix - 1);
    int i4 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ixp - 1);
    int ii[8] = {i1, i2, i3, i4, i1 + 1, i2 + 1, i3 + 1, i4 + 1};
    const float *E = &extp[(size_t)ipa * ng];
    const float *A = &albp[(size_t)ipa * ng];
    double ext = 0, scat[8], scatter = 0;
    for (int c = 0; c < 8; ++c) { ext += f[c] * E[ii[c]]; scat[c] = f[c] * E[ii[c]] * A[ii[c]]; scatter += scat[c]; }
    if (ipa == 0 && srct != 'S') {
      double t = 0;
      for (int c = 0; c < 8; ++c) t += f[c] * tempp_in[ii[c]];
      temp[ipt] = (float)t;
    }
    extr = (R)ext;
    R alb = (ext > extmin) ? (R)(scatter / ext) : (R)(scatter / extmin);
    extinct[(size_t)ipa * npts + ipt] = extr;
    albedo[(size_t)ipa * npts + ipt] = alb;
    int *IPH = &iphase[((size_t)ipa * npts + ipt) * nq];
    R *PW = &phaseinterpwt[((size_t)ipa * npts + ipt) * nq];
    for (int c = 0; c < 8; ++c)
      for (int q = 0; q < maxnmicro; ++q) {
        IPH[c * maxnmicro + q] = iphp[((size_t)ipa * ng + ii[c]) * maxnmicro + q];
        double pw = phwtp[((size_t)ipa * ng + ii[c]) * maxnmicro + q];
        PW[c * maxnmicro + q] = (R)(scatter >= scatmin ? pw * scat[c] / scatter : pw * scat[c] / scatmin);
      }
    for (int q = 0; q < nq; ++q)
      for (int q2 = q + 1; q2 < nq; ++q2)
        if (IPH[q] == IPH[q2]) { PW[q] += PW[q2]; PW[q2] = 0; }
    std::vector<std::pair<R, int>> srt(nq);
    for (int q = 0; q < nq; ++q) srt[q] = {PW[q], IPH[q]};
    std::stable_sort(srt.begin(), srt.end(), [](const std::pair<R, int> &a, const std::pair<R, int> &b) { return a.first > b.first; });
    for (int q = 0; q < nq; ++q) { PW[q] = srt[q].first; IPH[q] = srt[q].second; }
    return true;
  }

  // The delta-M scaling of one species' extinction and albedo at a grid point
  // (PREPARE_PROP / INTERPOLATE_POINT, 'N' method).
  void deltam_point(int ipa, int ipt) {
    const int *IPH = &iphase[((size_t)ipa * npts + ipt) * nq];
    const R *PW = &phaseinterpwt[((size_t)ipa * npts + ipt) * nq];
    R f;
    if (PW[0] >= phasemax) f = legen[(size_t)(IPH[0] - 1) * (nleg + 1) + ml + 1];
    else { f = 0; for (int q = 0; q < nq; ++q) f += legen[(size_t)(IPH[q] - 1) * (nleg + 1) + ml + 1] * PW[q]; }
    R &e = extinct[(size_t)ipa * npts + ipt];
    R &a = albedo[(size_t)ipa * npts + ipt];
    R anew = ((R)1 - f) * a / ((R)1 - a * f);
    e = ((R)1 - a * f) * e;
    a = anew;
  }

  void planck_point(int ipt) {
    const R bb = (R)planck_fn(temp[ipt]);
    R tp = 0;
    for (int ipa = 0; ipa < npart; ++ipa)
      tp = tp + extinct[(size_t)ipa * npts + ipt] * (((R)1 - albedo[(size_t)ipa * npts + ipt]) * bb);
    planck_tot[ipt] = total_ext[ipt] > (R)1e-10 ? tp / total_ext[ipt] : (R)0;
  }

  bool transfer_properties() {
    npart = p.npart; maxnmicro = p.maxnmicro; numphase = p.numphase;
    nq = 8 * maxnmicro;
    const int npz = p.npz;
    legen.assign((size_t)numphase * (nleg + 1), 0);
    for (int i = 0; i < numphase; ++i)
      for (int l = 0; l <= nleg; ++l)
        legen[(size_t)i * (nleg + 1) + l] =
            (l <= p.nlegp) ? (R)(leg_in(i, l, 0) / (float)(2 * l + 1)) : (R)0;
    if (nst == 3) {
      legen6.assign((size_t)numphase * 6 * (nleg + 1), 0);
      for (int i = 0; i < numphase; ++i)
        for (int k = 0; k < 6; ++k)
          for (int l = 0; l <= nleg && l <= p.nlegp; ++l)
            legen6[((size_t)i * 6 + k) * (nleg + 1) + l] = (R)(leg_in(i, l, k) / (float)(2 * l + 1));
    }
    extmin = (double)(1.0e-5f / ((zlev[npz - 1] - zlev[0]) / (float)npz));
    scatmin = 0.1 * extmin;
    extinct.assign((size_t)npart * npts, 0); albedo.assign((size_t)npart * npts, 0);
    total_ext.assign(npts, 0);
    iphase.assign((size_t)npart * npts * nq, 1); phaseinterpwt.assign((size_t)npart * npts * nq, 0);
    temp.assign(srct != 'S' ? npts : 0, 0.f);
    for (int ipa = 0; ipa < npart; ++ipa)
      for (int ipt = 0; ipt < npts; ++ipt) {
        R extr;
        if (!trilin_point(ipa, ipt, extr)) return false;
        total_ext[ipt] += extr;
      }
    // PREPARE_PROP, 'N' interpolation method
    if (p.deltam) {
      for (int i = 0; i < numphase; ++i) {
        R *L = &legen[(size_t)i * (nleg + 1)];
        R f = L[ml + 1];
        for (int l = 0; l <= ml; ++l) L[l] = L[l] - f;
        if (nst == 3) {
          // diagonal elements lose f, the off-diagonal ones are kept (PREPARE_PROP 'N')
          for (int k = 0; k < 4; ++k) {
            R *L6 = &legen6[((size_t)i * 6 + k) * (nleg + 1)];
            for (int l = 0; l <= ml; ++l) L6[l] = L6[l] - f;
          }
        }
      }
      for (int ipt = 0; ipt < npts; ++ipt) {
        R s = 0;
        for (int ipa = 0; ipa < npart; ++ipa) s += extinct[(size_t)ipa * npts + ipt];
        total_ext[ipt] = total_ext[ipt] - s;
        if (total_ext[ipt] < 0) total_ext[ipt] = 0;
      }
      for (int ipa = 0; ipa < npart; ++ipa)
        for (int ipt = 0; ipt < npts; ++ipt) {
          deltam_point(ipa, ipt);
          total_ext[ipt] += extinct[(size_t)ipa * npts + ipt];
        }
    }
    // PLANCK(I,IPA) = (1 - albedo) B(T) after the delta-M scaling
    // (src/polarized/shdomsub2.f:574-580), summed over the species with the
    // extinction weights of COMPUTE_SOURCE (src/polarized/shdomsub1.f:1092-1139)
    planck_tot.assign(npts, 0);
    if (srct != 'S')
      for (int ipt = 0; ipt < npts; ++ipt) planck_point(ipt);
    albmax = 0;
    for (auto a : albedo) albmax = std::max(albmax, a);
    return true;
  }

  // Per-point mixed, delta-M rescaled Legendre series (the LEGENT1 block of
  // COMPUTE_SOURCE, src/polarized/shdomsub1.f:1432-1450).
  void point_legen(int ipt, int ipa, std::vector<R> &lt, R &fout) const {
    const int *IPH = &iphase[((size_t)ipa * npts + ipt) * nq];
    const R *PW = &phaseinterpwt[((size_t)ipa * npts + ipt) * nq];
    lt.assign(nleg + 1, 0);
    if (PW[0] >= phasemax) {
      for (int l = 0; l <= nleg; ++l) lt[l] = legen[(size_t)(IPH[0] - 1) * (nleg + 1) + l];
    } else {
      for (int q = 0; q < nq; ++q) {
        if (PW[q] <= (R)1e-5) continue;
        for (int l = 0; l <= nleg; ++l) lt[l] += legen[(size_t)(IPH[q] - 1) * (nleg + 1) + l] * PW[q];
      }
    }
    fout = 0;
    if (p.deltam) {
      R f = lt[ml + 1];
      fout = f;
      for (int l = 0; l <= ml; ++l) lt[l] = lt[l] / ((R)1 - f);
    }
  }

  // point_legen for all six elements (lt [6][nleg+1]); the delta-M division
  // applies to every element's 0..ML terms (src/polarized/shdomsub1.f:1432-1450).
  void point_legen6(int ipt, int ipa, std::vector<R> &lt, R &fout) const {
    const int *IPH = &iphase[((size_t)ipa * npts + ipt) * nq];
    const R *PW = &phaseinterpwt[((size_t)ipa * npts + ipt) * nq];
    const int n1 = nleg + 1;
    lt.assign((size_t)6 * n1, 0);
    if (PW[0] >= phasemax) {
      for (int q = 0; q < 6 * n1; ++q) lt[q] = legen6[(size_t)(IPH[0] - 1) * 6 * n1 + q];
    } else {
      for (int q = 0; q < nq; ++q) {
        if (PW[q] <= (R)1e-5) continue;
        for (int t = 0; t < 6 * n1; ++t) lt[t] += legen6[(size_t)(IPH[q] - 1) * 6 * n1 + t] * PW[q];
      }
    }
    fout = 0;
    if (p.deltam) {
      R f = lt[ml + 1];
      fout = f;
      for (int k = 0; k < 6; ++k)
        for (int l = 0; l <= ml; ++l) lt[(size_t)k * n1 + l] = lt[(size_t)k * n1 + l] / ((R)1 - f);
    }
  }

  // DIRECT_BEAM_PROP (src/polarized/shdom90.f90:352-867) via MAKE_DIRECT
  // (src/polarized/shdomsub2.f:393-476); regular property grid, no gas.
  // Points from `from` to `to` (new points of a split get theirs one at a time).
  void make_direct(int from = 0, int to = -1) {
    if (from == 0) dirflux.assign(npts, 0); else dirflux.resize(npts, 0);
    if (srct == 'T') return;  // no solar beam for a thermal source
    int npx = p.npx, npy = p.npy, npz = p.npz, ng = npx * npy * npz;
    std::vector<double> extdirp(ng, 0.0);
    for (int ip = 0; ip < ng; ++ip) {
      float acc = 0.f;
      for (int ipa = 0; ipa < npart; ++ipa) {
        double e = extp[(size_t)ipa * ng + ip], a = albp[(size_t)ipa * ng + ip];
        if (p.deltam) {
          int L = ml + 1;
          double f = 0;
          for (int q = 0; q < maxnmicro; ++q) {
            int iph = iphp[((size_t)ipa * ng + ip) * maxnmicro + q];
            f += phwtp[((size_t)ipa * ng + ip) * maxnmicro + q] *
                 (double)(leg_in(iph - 1, L, 0) / (float)(2 * L + 1));
          }
          e = (1.0 - a * f) * e;
        }
        acc = (float)(acc + e);
      }
      extdirp[ip] = acc;
    }
    int ipdirect = ipflag;
    if (ipflag & 4) ipdirect = 0;
    double sunmu = -(double)p.solarmu;
    double sunaz = (double)(float)(p.solaraz + (float)std::acos(-1.0f));
    double cx = std::sqrt(1.0 - sunmu * sunmu) * std::cos(sunaz);
    double cy = std::sqrt(1.0 - sunmu * sunmu) * std::sin(sunaz);
    double cz = std::fabs(sunmu), cxinv, cyinv, czinv;
    if (std::fabs(cx) > 1e-6) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1e20; }
    if (std::fabs(cy) > 1e-6) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1e20; }
    if (std::fabs(cz) > 1e-6) czinv = 1.0 / cz; else { cz = 0; czinv = 1e20; }
    int di = cx >= 0 ? 1 : -1, dj = cy >= 0 ? 1 : -1, dk = cz >= 0 ? 1 : -1;
    double epsz = 1.0e-6 * (zlev[npz - 1] - zlev[0]);
    double epss = 1.0e-3 * (zlev[npz - 1] - zlev[0]) / npz;
    if (!(ipdirect & 1)) epss = std::max(epss, 1.0e-4 * p.delx);
    if (!(ipdirect & 2)) epss = std::max(epss, 1.0e-4 * p.dely);
    double delxd = p.delx, delyd = p.dely;
    epss = std::max(std::max(0.001 * delxd, 0.001 * delyd), epss);
    double xdomain = delxd * npx, ydomain = delyd * npy;
    for (int ipt = from; ipt < (to < 0 ? npts : to); ++ipt) {
      double z = gridpos[3 * ipt + 2], x = gridpos[3 * ipt], y = gridpos[3 * ipt + 1];
      int il = 0, iu = npz;
      while (iu - il > 1) { int im = (iu + il) / 2; if (z >= zlev[im - 1]) il = im; else iu = im; }
      int k = std::max(il, 1);
      int i = (int)(x / delxd) + 1;
      if (i > npx && std::fabs(x - xdomain) < 0.001 * delxd) i = npx;
      int j = (int)(y / delyd) + 1;
      if (j > npy && std::fabs(y - ydomain) < 0.001 * delyd) j = npy;
      double xe = x, ye = y, ze = z, xp = xe, yp = ye, zp = ze;
      bool constx = ipdirect & 1, consty = ipdirect & 2;
      if (cx == 0.0) constx = true;
      if (cy == 0.0) consty = true;
      if ((bcflag & 1) && (std::fabs(x) < 0.01 * delxd || std::fabs(x - (npx - 1) * delxd) < 0.01 * delxd)) constx = true;
      if ((bcflag & 2) && (std::fabs(y) < 0.01 * delyd || std::fabs(y - (npy - 1) * delyd) < 0.01 * delyd)) consty = true;
      double path = 0.0;
      int guard = 0;
      while (std::fabs(ze - zlev[npz - 1]) > epsz && guard++ < 10000000) {
        int ipn = i + 1;
        if (i == npx) ipn = (bcflag & 1) ? npx : 1;
        int jpn = j + 1;
        if (j == npy) jpn = (bcflag & 2) ? npy : 1;
        double x0 = delxd * (i - 1), x1 = x0 + delxd, y0 = delyd * (j - 1), y1 = y0 + delyd;
        double z0 = zlev[k - 1], z1 = zlev[k];
        int I1 = (k - 1) + npz * (j - 1) + npz * npy * (i - 1);
        int I2 = (k - 1) + npz * (j - 1) + npz * npy * (ipn - 1);
        int I3 = (k - 1) + npz * (jpn - 1) + npz * npy * (i - 1);
        int I4 = (k - 1) + npz * (jpn - 1) + npz * npy * (ipn - 1);
        double e1 = extdirp[I1], e2 = extdirp[I2], e3 = extdirp[I3], e4 = extdirp[I4];
        double e5 = extdirp[I1 + 1], e6 = extdirp[I2 + 1], e7 = extdirp[I3 + 1], e8 = extdirp[I4 + 1];
        double sox, soy, soz;
        if (constx) sox = 1e30; else if (cx > 0) { sox = (x1 - xe) * cxinv; xp = x1; } else { sox = (x0 - xe) * cxinv; xp = x0; }
        if (consty) soy = 1e30; else if (cy > 0) { soy = (y1 - ye) * cyinv; yp = y1; } else { soy = (y0 - ye) * cyinv; yp = y0; }
        if (cz > 0) { soz = (z1 - ze) * czinv; zp = z1; } else if (cz < 0) { soz = (z0 - ze) * czinv; zp = z0; } else soz = 1e30;
        double xoffs = 0, yoffs = 0, so;
        if (soz <= sox && soz <= soy) {
          so = soz;
          if (!constx) xp = xe + so * cx;
          if (!consty) yp = ye + so * cy;
          k += dk;
        } else if (sox <= soy) {
          so = sox;
          if (!consty) yp = ye + so * cy;
          zp = ze + so * cz;
          i += di;
          if (i == 0) { if (bcflag & 1) { i = 1; constx = true; } else { i = npx; xoffs = xdomain; } }
          else if (i == npx + 1) { if (bcflag & 1) { i = npx; constx = true; } else { i = 1; xoffs = -xdomain; } }
        } else {
          so = soy;
          if (!constx) xp = xe + so * cx;
          zp = ze + so * cz;
          j += dj;
          if (j == 0) { if (bcflag & 2) { j = 1; consty = true; } else { j = npy; yoffs = ydomain; } }
          else if (j == npy + 1) { if (bcflag & 2) { j = npy; consty = true; } else { j = 1; yoffs = -ydomain; } }
        }
        so = std::max(so, 0.0);
        double ax = 1.0 / (x1 - x0), ay = 1.0 / (y1 - y0), az = 1.0 / (z1 - z0);
        double u0 = (xe - x0) * ax, v0 = (ye - y0) * ay, w0 = (ze - z0) * az;
        double u1 = (xp - x0) * ax, v1 = (yp - y0) * ay, w1 = (zp - z0) * az;
        double u0m = 1 - u0, v0m = 1 - v0, w0m = 1 - w0;
        double du = u1 - u0, dv = v1 - v0, dw = w1 - w0;
        double uv = u0 * v0, umv = u0m * v0, uvm = u0 * v0m, umvm = u0m * v0m;
        double uw = u0 * w0, umw = u0m * w0, uwm = u0 * w0m, umwm = u0m * w0m;
        double vw = v0 * w0, vmw = v0m * w0, vwm = v0 * w0m, vmwm = v0m * w0m;
        double A = (e1 * u0m + e2 * u0) * vmwm + (e3 * u0m + e4 * u0) * vwm + (e5 * u0m + e6 * u0) * vmw +
                   (e7 * u0m + e8 * u0) * vw;
        double b1 = -du * vmwm - dv * umwm - dw * umvm, b2 = du * vmwm - dv * uwm - dw * uvm;
        double b3 = -du * vwm + dv * umwm - dw * umv, b4 = du * vwm + dv * uwm - dw * uv;
        double b5 = -du * vmw - dv * umw + dw * umvm, b6 = du * vmw - dv * uw + dw * uvm;
        double b7 = -du * vw + dv * umw + dw * umv, b8 = du * vw + dv * uw + dw * uv;
        double B = b1 * e1 + b2 * e2 + b3 * e3 + b4 * e4 + b5 * e5 + b6 * e6 + b7 * e7 + b8 * e8;
        double VW = dv * dw, vwu = VW * u0, vwum = VW * u0m, UW = du * dw, uwv = UW * v0, uwvm = UW * v0m;
        double UV = du * dv, uvw = UV * w0, uvwm = UV * w0m;
        double c1 = vwum + uwvm + uvwm, c2 = vwu - uwvm - uvwm, c3 = -vwum + uwv - uvwm, c4 = -vwu - uwv + uvwm;
        double c5 = -vwum - uwvm + uvw, c6 = -vwu + uwvm - uvw, c7 = vwum - uwv - uvw, c8 = vwu + uwv + uvw;
        double C = c1 * e1 + c2 * e2 + c3 * e3 + c4 * e4 + c5 * e5 + c6 * e6 + c7 * e7 + c8 * e8;
        double D = du * dv * dw * (e2 + e3 + e5 + e8 - e1 - e4 - e6 - e7);
        path += so * (A + 0.5 * B + 0.3333333333333333 * C + 0.25 * D);
        xe = xp + xoffs; ye = yp + yoffs; ze = zp;
      }
      dirflux[ipt] = (R)(p.solarflux * std::exp(-path));
    }
  }

  // INIT_RADIANCE / EDDRTF / TRIDIAG (src/polarized/shdomsub2.f:614-1058),
  // solar source, base grid columns.
  void init_radiance() {
    radiance.assign((size_t)npts * nlm * nst, 0);
    rshptr.assign(npts + 2, 0);
    const float pi = (float)std::acos(-1.0f);
    const float c0 = std::sqrt(1.0f / pi), c1 = std::sqrt(3.0f / (4 * pi));
    int nlayer = nz - 1, nxy = nx1 * ny1;
    std::vector<float> od(nlayer + 1), al(nlayer + 1), as(nlayer + 1);
    std::vector<double> fl(2 * (nlayer + 1));
    int ir = 0;
    std::vector<R> lt; R fdum;
    for (int col = 0; col < nxy; ++col) {
      for (int iz = 0; iz < nlayer; ++iz) {
        int L = nz - 1 - iz - 1;  // 0-based layer from the top
        int i0 = iz + nz * col, i1 = iz + 1 + nz * col;
        float ext0 = (float)total_ext[i0], ext1 = (float)total_ext[i1];
        float scat0 = 0, scat1 = 0, g0 = 0, g1 = 0;
        for (int ipa = 0; ipa < npart; ++ipa) {
          scat0 += (float)(albedo[(size_t)ipa * npts + i0] * extinct[(size_t)ipa * npts + i0]);
          scat1 += (float)(albedo[(size_t)ipa * npts + i1] * extinct[(size_t)ipa * npts + i1]);
        }
        od[L] = (zgrid[iz + 1] - zgrid[iz]) * (ext0 + ext1) / 2;
        al[L] = (ext0 + ext1 > 0) ? (scat0 + scat1) / (ext0 + ext1) : 0.f;
        for (int ipa = 0; ipa < npart; ++ipa) {
          point_legen(i0, ipa, lt, fdum);
          g0 += (float)(albedo[(size_t)ipa * npts + i0] * extinct[(size_t)ipa * npts + i0] * lt[1]);
          point_legen(i1, ipa, lt, fdum);
          g1 += (float)(albedo[(size_t)ipa * npts + i1] * extinct[(size_t)ipa * npts + i1] * lt[1]);
        }
        as[L] = (scat0 + scat1 > 0) ? (g0 + g1) / (scat0 + scat1) : 0.f;
      }
      // TEMPS from the top: TEMPS(k) = TEMP(NZ+1-k) of this column
      std::vector<float> temps(nz, 0.f);
      if (srct != 'S')
        for (int k = 0; k < nz; ++k) temps[k] = temp[(size_t)(nz - 1 - k) + (size_t)nz * col];
      eddrtf(nlayer, od, al, as, temps, fl);
      for (int iz = 0; iz < nz; ++iz) {
        int L = nz - 1 - iz;
        // Only the I Stokes parameter is initialised (Q, U stay zero)
        R *rad = &radiance[(size_t)ir * nst];
        for (int q = 0; q < 4 * nst; ++q) rad[q] = 0;
        rad[0] = (R)(c0 * (float)(fl[2 * L] + fl[2 * L + 1]));
        rad[2 * nst] = (R)(c1 * (float)(fl[2 * L] - fl[2 * L + 1]));
        ir += 4;
        rshptr[iz + nz * col + 1] = ir;
      }
    }
    rshptr[npts + 1] = ir;
  }

  void eddrtf(int nlayer, const std::vector<float> &od, const std::vector<float> &al,
              const std::vector<float> &as, const std::vector<float> &temps, std::vector<double> &fluxout) {
    int n = 2 * nlayer + 2;
    std::vector<double> lower(n + 1), upper(n + 1), diag(n + 1), rhs(n + 1);
    const double pi = 3.1415926535;
    double mu0 = std::fabs((double)p.solarmu), tau = 0.0, sf = p.solarflux;
    // thermal layers (SRCTYPE 'T' only): Planck function linear in optical depth
    const bool therm = srct == 'T';
    double planck1 = therm ? pi * (double)planck_fn(temps[0]) : 0.0;
    int i = 2;
    for (int l = 0; l < nlayer; ++l) {
      double deltau = od[l], trans, reflect, sourcep, sourcem;
      if (deltau == 0.0) { trans = 1; reflect = 0; sourcep = 0; sourcem = 0; }
      else {
        double omega = al[l], g = as[l];
        double r = (1.0 - omega * (4.0 - 3.0 * g)) / 4.0, t = (7.0 - omega * (4.0 + 3.0 * g)) / 4.0;
        double lambda = std::sqrt(3.0 * (1.0 - omega) * (1.0 - omega * g));
        double d, x1 = 0, x2 = 0, exlp = 0, exlm = 0;
        if (lambda == 0.0) { d = 1.0 / (1.0 + t * deltau); trans = d; reflect = -r * deltau * d; }
        else {
          x1 = -r; x2 = lambda + t;
          exlp = std::exp(std::min(lambda * deltau, 75.0)); exlm = 1.0 / exlp;
          trans = 2. * lambda / (x2 * exlp + (lambda - t) * exlm);
          reflect = x1 * (exlp - exlm) * trans / (2. * lambda);
          d = 1.0 / (x2 * x2 * exlp - x1 * x1 * exlm);
        }
        double radp1p, radp2m, radp2p, radp1m;
        if (therm) {
          const double planck2 = pi * (double)planck_fn(temps[l + 1]);
          const double v = 2.0 * (planck2 - planck1) / (3.0 * (1. - omega * g) * deltau);
          radp1p = -v + planck1; radp2m = v + planck2; radp2p = -v + planck2; radp1m = v + planck1;
          planck1 = planck2;
        } else {
          double ds = 1.0 / (lambda * lambda - 1.0 / (mu0 * mu0));
          double b1 = 0.5 * omega * (sf / mu0) * std::exp(-tau / mu0) * ds;
          double b2 = 0.5 * omega * (sf / mu0) * std::exp(-(tau + deltau) / mu0) * ds;
          double solpp = 1.0 + 1.5 * g * mu0, solpm = -1.0 + 1.5 * g * mu0;
          radp1p = ((t + 1.0 / mu0) * solpp + r * solpm) * b1;
          radp2m = ((-t + 1.0 / mu0) * solpm - r * solpp) * b2;
          radp2p = ((t + 1.0 / mu0) * solpp + r * solpm) * b2;
          radp1m = ((-t + 1.0 / mu0) * solpm - r * solpp) * b1;
        }
        if (lambda == 0.0) {
          double A = (r * deltau * radp1p - radp2m) * d, B = -(r * radp1p + t * radp2m) * d;
          sourcep = (B - t * (A + B * deltau)) / r + radp2p;
          sourcem = A + radp1m;
        } else {
          double cp = (x1 * exlm * radp1p - x2 * radp2m) * d, cm = (-x2 * exlp * radp1p + x1 * radp2m) * d;
          sourcep = x1 * cp * exlp + x2 * cm * exlm + radp2p;
          sourcem = x2 * cp + x1 * cm + radp1m;
        }
        if (!therm) tau += deltau;
      }
      diag[i] = -reflect; diag[i + 1] = -reflect;
      lower[i] = 1.0; lower[i + 1] = -trans;
      upper[i] = -trans; upper[i + 1] = 1.0;
      rhs[i] = sourcem; rhs[i + 1] = sourcep;
      i += 2;
    }
    double gndemis = 1.0 - (double)p.gndalbedo;
    double gndflux, skyflux;
    if (srct == 'S') {
      gndflux = (1.0 - gndemis) * sf * std::exp(-tau / mu0);
      skyflux = pi * p.skyrad;
    } else {  // 'T' and 'B': emitting ground and sky
      gndflux = pi * (double)planck_fn(p.gndtemp) * gndemis;
      skyflux = pi * (double)planck_fn(p.skyrad);
    }
    rhs[1] = skyflux; diag[1] = 0.0; upper[1] = 1.0;
    diag[n] = -(1.0 - gndemis); lower[n] = 1.0; rhs[n] = gndflux;
    // TRIDIAG (Linpack DGTSL style with pivoting), 1-based arrays
    lower[1] = diag[1]; diag[1] = upper[1]; upper[1] = 0.0; upper[n] = 0.0;
    for (int k = 1; k <= n - 1; ++k) {
      if (std::fabs(lower[k + 1]) >= std::fabs(lower[k])) {
        std::swap(lower[k + 1], lower[k]); std::swap(diag[k + 1], diag[k]);
        std::swap(upper[k + 1], upper[k]); std::swap(rhs[k + 1], rhs[k]);
      }
      double t = -lower[k + 1] / lower[k];
      lower[k + 1] = diag[k + 1] + t * diag[k];
      diag[k + 1] = upper[k + 1] + t * upper[k];
      upper[k + 1] = 0.0;
      rhs[k + 1] = rhs[k + 1] + t * rhs[k];
    }
    rhs[n] = rhs[n] / lower[n];
    rhs[n - 1] = (rhs[n - 1] - diag[n - 1] * rhs[n]) / lower[n - 1];
    for (int kb = 1; kb <= n - 2; ++kb) {
      int k = n - 2 - kb + 1;
      rhs[k] = (rhs[k] - diag[k] * rhs[k + 1] - upper[k] * rhs[k + 2]) / lower[k];
    }
    fluxout.assign(2 * (nlayer + 1), 0.0);
    const double cfl = unitc == 'T' ? 1.0 / pi : 1.0;
    for (int l = 0, ii = 1; l <= nlayer; ++l, ii += 2) {
      fluxout[2 * l] = (float)(cfl * rhs[ii]);
      fluxout[2 * l + 1] = (float)(cfl * rhs[ii + 1]);
    }
  }

  // Per-point source function SH vector (CALC_SOURCE_PNT_UNPOL with the
  // NEWMETHOD species mixing, src/polarized/shdomsub1.f:913-962, :1413-1485).
  void point_source(int i, std::vector<R> &sourcet, const std::vector<R> &rad, int ir, int nr,
                    std::vector<R> &lt, std::vector<R> &lt1) const {
    if (nst == 3) { point_source_pol(i, sourcet, rad, ir, nr, lt, lt1); return; }
    double alb = 0.0;
    lt.assign(nleg + 1, 0);
    R fdum;
    for (int ipa = 0; ipa < npart; ++ipa) {
      double scat = (double)(R)(extinct[(size_t)ipa * npts + i] * albedo[(size_t)ipa * npts + i]);
      alb += scat;
      point_legen(i, ipa, lt1, fdum);
      for (int l = 0; l <= nleg; ++l) lt[l] = (R)(lt[l] + scat * lt1[l]);
    }
    if (alb > 1e-10) { for (int l = 0; l <= nleg; ++l) lt[l] = (R)(lt[l] / alb); }
    else { for (int l = 0; l <= nleg; ++l) lt[l] = lt[l] / (R)npart; }
    R ext = total_ext[i];
    if (ext > (R)1e-10) alb = alb / ext; else alb = 0.0;
    lt[0] = 1;
    R albr = (R)alb;
    R flux0 = dirflux[i] * ((R)1 / std::fabs((R)p.solarmu));
    sourcet.assign(nlm, 0);
    for (int j = 0; j < nlm; ++j) sourcet[j] = flux0 * albr * lt[lofj[j]] * ylmsun[j];
    // isotropic thermal emission (CALC_SOURCE_PNT_UNPOL, C = sqrt(4 pi))
    if (srct != 'S') sourcet[0] = sourcet[0] + (R)3.544907703f * planck_tot[i];
    for (int j = 0; j < nr; ++j) sourcet[j] = sourcet[j] + albr * lt[lofj[j]] * rad[(size_t)ir + j];
  }

  // Polarized form: CALC_SOURCE_PNT (src/polarized/shdomsub1.f:823-909) with
  // the same species mixing applied to all six elements; sourcet [nlm][3]
  // (Stokes fastest), rad in the same layout from term ir.
  void point_source_pol(int i, std::vector<R> &sourcet, const std::vector<R> &rad, int ir, int nr,
                        std::vector<R> &lt, std::vector<R> &lt1) const {
    const int n1 = nleg + 1;
    double alb = 0.0;
    lt.assign((size_t)6 * n1, 0);
    R fdum;
    for (int ipa = 0; ipa < npart; ++ipa) {
      double scat = (double)(R)(extinct[(size_t)ipa * npts + i] * albedo[(size_t)ipa * npts + i]);
      alb += scat;
      point_legen6(i, ipa, lt1, fdum);
      for (int t = 0; t < 6 * n1; ++t) lt[t] = (R)(lt[t] + scat * lt1[t]);
    }
    if (alb > 1e-10) { for (int t = 0; t < 6 * n1; ++t) lt[t] = (R)(lt[t] / alb); }
    else { for (int t = 0; t < 6 * n1; ++t) lt[t] = lt[t] / (R)npart; }
    R ext = total_ext[i];
    if (ext > (R)1e-10) alb = alb / ext; else alb = 0.0;
    lt[0] = 1;
    const R albr = (R)alb;
    const R *a1 = &lt[0], *a2 = &lt[n1], *a3 = &lt[2 * n1], *b1 = &lt[4 * n1];
    const R *Rd = &rad[(size_t)ir * 3];
    sourcet.assign((size_t)nlm * 3, 0);
    for (int j = 0; j < nr; ++j) sourcet[3 * j] += a1[lofj[j]] * Rd[3 * j];
    for (int j = 0; j < nr; ++j) sourcet[3 * j] += b1[lofj[j]] * Rd[3 * j + 1];
    for (int j = 4; j < nr; ++j) {
      sourcet[3 * j + 1] += b1[lofj[j]] * Rd[3 * j] + a2[lofj[j]] * Rd[3 * j + 1];
      sourcet[3 * j + 2] += a3[lofj[j]] * Rd[3 * j + 2];
    }
    for (int t = 0; t < 3 * nlm; ++t) sourcet[t] = albr * sourcet[t];
    const R flux0 = dirflux[i] * ((R)1 / std::fabs((R)p.solarmu));
    for (int j = 0; j < nlm; ++j) sourcet[3 * j] += flux0 * albr * a1[lofj[j]] * ylmsun[j];
    for (int j = 4; j < nlm; ++j) sourcet[3 * j + 1] += flux0 * albr * b1[lofj[j]] * ylmsun[j];
    if (srct != 'S') sourcet[0] += (R)3.544907703f * planck_tot[i];  // unpolarized emission
  }

  // COMPUTE_SOURCE (src/polarized/shdomsub1.f:967-1611), NEWMETHOD, 'N'.
  void compute_source(bool fixsh, bool first) {
    std::vector<R> sourcet, lt, lt1;
    R srcmin = (R)p.shacc;
    if (!first) {
      R djdot = 0, djold = 0, djnew = 0, jn = 0;
      for (int i = 0; i < npts; ++i) {
        int ir = rshptr[i], nr = rshptr[i + 1] - ir;
        point_source(i, sourcet, radiance, ir, nr, lt, lt1);
        int is = shptr[i];
        if (p.accelflag) {
          int iso = oshptr[i];
          int ns = std::min(shptr[i + 1] - is, oshptr[i + 1] - iso);
          for (int t = 0; t < ns * nst; ++t) {
            const size_t js = (size_t)is * nst + t, jo = (size_t)iso * nst + t;
            R dn = sourcet[t] - source[js];
            djdot += dn * delsource[jo];
            djold += delsource[jo] * delsource[jo];
            djnew += dn * dn;
            jn += source[js] * source[js];
          }
        } else {
          int ns = shptr[i + 1] - is;
          for (int t = 0; t < ns * nst; ++t) {
            const size_t js = (size_t)is * nst + t;
            R dn = sourcet[t] - source[js];
            djnew += dn * dn;
            jn += source[js] * source[js];
          }
        }
      }
      deljdot = djdot; deljold = djold; deljnew = djnew; jnorm = jn;
      if (p.accelflag) {
        for (int i = 0; i < npts; ++i) {
          int ir = rshptr[i], nr = rshptr[i + 1] - ir;
          point_source(i, sourcet, radiance, ir, nr, lt, lt1);
          int is = shptr[i], ns = shptr[i + 1] - is;
          oshptr[i] = is;
          for (int t = 0; t < ns * nst; ++t)
            delsource[(size_t)is * nst + t] = sourcet[t] - source[(size_t)is * nst + t];
        }
        oshptr[npts] = shptr[npts];
      }
    }
    int is = 0;
    for (int i = 0; i < npts; ++i) {
      int ir = rshptr[i], nr = rshptr[i + 1] - ir;
      point_source(i, sourcet, radiance, ir, nr, lt, lt1);
      int ns;
      if (fixsh) ns = shptr[i + 1] - is;
      else {
        int js = 0;  // solar source
        for (int j = 1; j <= nlm; ++j)
          for (int k = 0; k < nst; ++k)
            if (std::fabs(sourcet[(size_t)(j - 1) * nst + k]) > srcmin) js = j;
        if (js == 0) ns = 0;
        else {
          int ls = lofj[js - 1];
          ns = (ls <= mm) ? ls * (ls + 1) + ls + 1 : (2 * mm + 1) * ls - mm * (mm - 1 + 1) + mm + 1;
        }
        shptr[i] = is;
      }
      for (int t = 0; t < ns * nst; ++t) source[(size_t)is * nst + t] = sourcet[t];
      is += ns;
    }
    shptr[npts] = is;
  }

  // RADIANCE_TRUNCATION (src/polarized/shdomsub1.f:1615-1803), 'N', no new points.
  void radiance_truncation(bool fixsh) {
    std::vector<int> newr(npts + 2, 0);
    if (!fixsh) {
      R radmin = (R)p.shacc;
      bool notend = true;
      int iro = 0, ir = 0;
      newr[0] = 0;
      for (int i = 0; i < npts; ++i) {
        int nro = rshptr[i + 1] - iro;
        if (nro == 0) notend = false;
        R ext = total_ext[i];
        int lr;
        if (notend) {
          std::vector<R> f(npart, 0);
          if (p.deltam) {
            for (int ipa = 0; ipa < npart; ++ipa) {
              std::vector<R> lt; R ff;
              const int *IPH = &iphase[((size_t)ipa * npts + i) * nq];
              const R *PW = &phaseinterpwt[((size_t)ipa * npts + i) * nq];
              if (PW[0] >= phasemax) f[ipa] = legen[(size_t)(IPH[0] - 1) * (nleg + 1) + ml + 1];
              else {
                // The reference indexes LEGEN(Q,ML+1,...) with the Stokes slot
                // (src/polarized/shdomsub1.f:1688); for scalar tables this
                // reads the series at L=ML+Q.  Restated as such.
                for (int q = 0; q < nq; ++q) {
                  if (PW[q] <= (R)1e-5) continue;
                  int L = ml + 1 + q;
                  R v = (L <= nleg) ? legen[(size_t)(IPH[q] - 1) * (nleg + 1) + L]
                                    : legen[(size_t)(IPH[q] - 1) * (nleg + 1) + std::min(L, nleg)];
                  f[ipa] += v * PW[q];
                }
              }
              (void)lt; (void)ff;
            }
            for (int ipa = 0; ipa < npart; ++ipa) f[ipa] = (R)1 / ((R)1 - f[ipa]);
          }
          lr = 1;
          for (int l = 1; l <= ml; ++l) {
            R rad = 0;
            for (int ipa = 0; ipa < npart; ++ipa) {
              R w = (ext == 0) ? (R)1 : extinct[(size_t)ipa * npts + i] / ext;
              if (w == 0) continue;
              const int *IPH = &iphase[((size_t)ipa * npts + i) * nq];
              const R *PW = &phaseinterpwt[((size_t)ipa * npts + i) * nq];
              R legt;
              if (PW[0] >= phasemax) legt = legen[(size_t)(IPH[0] - 1) * (nleg + 1) + l];
              else {
                legt = 0;
                for (int q = 0; q < nq; ++q) {
                  if (PW[q] <= (R)1e-5) continue;
                  legt += legen[(size_t)(IPH[q] - 1) * (nleg + 1) + l] * PW[q];
                }
              }
              if (p.deltam) legt = legt * f[ipa];
              rad += w * albedo[(size_t)ipa * npts + i] * legt * radiance[(size_t)iro * nst];
            }
            if (rad > radmin) lr = l;
          }
        } else {
          lr = ml;
        }
        iro += nro;
        int ns = std::max(1, shptr[i + 1] - shptr[i]);
        int ls = lofj[ns - 1];
        lr = std::min(lr, ls + ml / 8 + 2);
        if (p.highorderrad) lr = ml;
        int nr = (lr <= mm) ? lr * (lr + 1) + lr + 1 : (2 * mm + 1) * lr - mm * (mm - 1 + 1) + mm + 1;
        ir += nr;
        newr[i + 1] = ir;
      }
      newr[npts + 1] = ir;
    } else {
      int ir = 0;
      newr[0] = 0;
      for (int i = 0; i < npts; ++i) {
        int nr = std::max(4, shptr[i + 1] - shptr[i]);
        if (p.highorderrad) nr = nlm;
        ir += nr;
        newr[i + 1] = ir;
      }
      newr[npts + 1] = ir;
    }
    // RSHPTR only changes the view onto RADIANCE (which PATH_INTEGRATION zeroes
    // and rebuilds); COMPUTE_SOURCE reads the radiance with the old pointer
    // before this routine runs, so the array content is left in place.
    rshptr = newr;
  }

  void boundary_points() {
    topp.clear(); botp.clear();
    for (int i = 0; i < npts; ++i) {
      if (gridpos[3 * i + 2] >= zgrid[nz - 1]) topp.push_back(i);
      if (gridpos[3 * i + 2] <= zgrid[0]) botp.push_back(i);
    }
    sfcgridalb.assign(botp.size(), (R)p.gndalbedo);
    if (p.sfc_variable) {
      // PREP_SURFACE periodic surface grid + SURFACE_PARM_INTERP
      // (src/surface.f:2-270, src/polarized/shdomsub1.f:2218-2268).
      int nxs = p.nxsfc, nys = p.nysfc;
      std::vector<float> g((size_t)(nxs + 1) * (nys + 1));
      for (int iy = 0; iy <= nys; ++iy)
        for (int ix = 0; ix <= nxs; ++ix)
          g[(size_t)iy * (nxs + 1) + ix] = sfcalb[(size_t)(iy % nys) * nxs + (ix % nxs)];
      for (size_t b = 0; b < botp.size(); ++b) {
        int i = botp[b];
        float rx = gridpos[3 * i] / p.delxsfc, ry = gridpos[3 * i + 1] / p.delysfc;
        int ix = std::max(1, std::min(nxs, (int)rx + 1)), iy = std::max(1, std::min(nys, (int)ry + 1));
        float u = std::max(0.0f, std::min(1.0f, rx - (ix - 1))), v = std::max(0.0f, std::min(1.0f, ry - (iy - 1)));
        auto G = [&](int x, int y) { return g[(size_t)(y - 1) * (nxs + 1) + (x - 1)]; };
        sfcgridalb[b] = (R)((1 - u) * (1 - v) * G(ix, iy) + (1 - u) * v * G(ix, iy + 1) +
                            u * (1 - v) * G(ix + 1, iy) + u * v * G(ix + 1, iy + 1));
      }
    }
    if (brdf) brdf_parameters();
    // SURFACE_PARM_INTERP: B of the bilinearly interpolated ground temperature
    botplanck.assign(botp.size(), 0);
    if (srct != 'S') {
      const int nxs = p.nxsfc, nys = p.nysfc;
      for (size_t b = 0; b < botp.size(); ++b) {
        float t = p.gndtemp;
        if (!sfctemp_in.empty()) {
          const int i = botp[b];
          float rx = gridpos[3 * i] / p.delxsfc, ry = gridpos[3 * i + 1] / p.delysfc;
          int ix = std::max(1, std::min(nxs, (int)rx + 1)), iy = std::max(1, std::min(nys, (int)ry + 1));
          float u = std::max(0.0f, std::min(1.0f, rx - (ix - 1))), v = std::max(0.0f, std::min(1.0f, ry - (iy - 1)));
          auto G = [&](int x, int y) { return sfctemp_in[(size_t)((y - 1) % nys) * nxs + ((x - 1) % nxs)]; };
          t = (1 - u) * (1 - v) * G(ix, iy) + (1 - u) * v * G(ix, iy + 1) + u * (1 - v) * G(ix + 1, iy) +
              u * v * G(ix + 1, iy + 1);
        }
        botplanck[b] = (R)planck_fn(t);
      }
    }
  }

  // SURFACE_PARM_INTERP (src/polarized/shdomsub1.f:2218-2268) of the BRDF
  // parameters from the periodic surface grid to the bottom points.
  void brdf_parameters() {
    const int nxs = p.nxsfc, nys = p.nysfc, np_ = nsfcpar;
    botpar.assign(botp.size() * np_, 0);
    auto G = [&](int x, int y, int j) {
      return sfcpar[((size_t)((y - 1) % nys) * nxs + ((x - 1) % nxs)) * np_ + j];
    };
    for (size_t b = 0; b < botp.size(); ++b) {
      int i = botp[b];
      float rx = gridpos[3 * i] / p.delxsfc, ry = gridpos[3 * i + 1] / p.delysfc;
      int ix = std::max(1, std::min(nxs, (int)rx + 1)), iy = std::max(1, std::min(nys, (int)ry + 1));
      float u = std::max(0.0f, std::min(1.0f, rx - (ix - 1))), v = std::max(0.0f, std::min(1.0f, ry - (iy - 1)));
      for (int j = 0; j < np_; ++j)
        botpar[b * np_ + j] = (R)((1 - u) * (1 - v) * G(ix, iy, j) + (1 - u) * v * G(ix, iy + 1, j) +
                                  u * (1 - v) * G(ix + 1, iy, j) + u * v * G(ix + 1, iy + 1, j));
    }
  }

  // SURFACE_BRDF (src/polarized/shdomsub2.f:1222-1300): the reflection
  // matrix for incident direction (mu1 < 0, phi1) and outgoing (mu2 > 0,
  // phi2), normalised so that a Lambertian surface returns its albedo.

  // ---- 6S ocean BRDF (src/ocean_brdf.f, the 'O' type of SURFACE_BRDF),
  // single precision as the reference.  Tables: whitecap reflectance
  // (Koepke 1984) every 0.1 um, diffuse transmittances of the wavy surface
  // by zenith angle and wind speed, Morel's (1988) Case I water
  // coefficients every 5 nm over 400-700 nm, and the Hale & Querry (1973)
  // refractive index of water.
  static constexpr float kWhitecap[39] = {
      0.220f, 0.220f, 0.220f, 0.220f, 0.220f, 0.220f, 0.215f, 0.210f, 0.200f, 0.190f, 0.175f, 0.155f, 0.130f,
      0.080f, 0.100f, 0.105f, 0.100f, 0.080f, 0.045f, 0.055f, 0.065f, 0.060f, 0.055f, 0.040f, 0.f,    0.f,
      0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f};
  static constexpr float kAngBnd[5] = {0.0f, 45.0f, 60.0f, 75.0f, 85.0f};
  static constexpr float kWsBnd[6] = {1.0f, 3.0f, 5.0f, 7.0f, 9.0f, 20.0f};
  static constexpr float kTds[5][6] = {{0.9787803f, 0.9787738f, 0.9787626f, 0.9787467f, 0.9787264f, 0.9785573f},
                                       {0.9706900f, 0.9698871f, 0.9691746f, 0.9685547f, 0.9680276f, 0.9666586f},
                                       {0.9479931f, 0.9404608f, 0.9385692f, 0.9381815f, 0.9384519f, 0.9430056f},
                                       {0.9690591f, 0.9275920f, 0.9058769f, 0.8951812f, 0.8899654f, 0.8892645f},
                                       {0.9980542f, 0.9602273f, 0.9114283f, 0.8713799f, 0.8417820f, 0.7800314f}};
  static constexpr float kTdv[5][6] = {{0.9787764f, 0.9787535f, 0.9787106f, 0.9786453f, 0.9785548f, 0.9775019f},
                                       {0.9692680f, 0.9637051f, 0.9564344f, 0.9495727f, 0.9438773f, 0.9288712f},
                                       {0.9225163f, 0.9069787f, 0.9044844f, 0.9052351f, 0.9068328f, 0.9153687f},
                                       {0.8048478f, 0.8479503f, 0.8678726f, 0.8797889f, 0.8878716f, 0.9091171f},
                                       {0.7294627f, 0.8137348f, 0.8453338f, 0.8629867f, 0.8745421f, 0.9036854f}};
  static constexpr float kKw[61] = {
      0.0209f, 0.0200f, 0.0196f, 0.0189f, 0.0183f, 0.0182f, 0.0171f, 0.0170f, 0.0168f, 0.0166f, 0.0168f, 0.0170f, 0.0173f,
      0.0174f, 0.0175f, 0.0184f, 0.0194f, 0.0203f, 0.0217f, 0.0240f, 0.0271f, 0.0320f, 0.0384f, 0.0445f, 0.0490f, 0.0505f,
      0.0518f, 0.0543f, 0.0568f, 0.0615f, 0.0640f, 0.0640f, 0.0717f, 0.0762f, 0.0807f, 0.0940f, 0.1070f, 0.1280f, 0.1570f,
      0.2000f, 0.2530f, 0.2790f, 0.2960f, 0.3030f, 0.3100f, 0.3150f, 0.3200f, 0.3250f, 0.3300f, 0.3400f, 0.3500f, 0.3700f,
      0.4050f, 0.4180f, 0.4300f, 0.4400f, 0.4500f, 0.4700f, 0.5000f, 0.5500f, 0.6500f};
  static constexpr float kXc[61] = {
      0.1100f, 0.1110f, 0.1125f, 0.1135f, 0.1126f, 0.1104f, 0.1078f, 0.1065f, 0.1041f, 0.0996f, 0.0971f, 0.0939f, 0.0896f,
      0.0859f, 0.0823f, 0.0788f, 0.0746f, 0.0726f, 0.0690f, 0.0660f, 0.0636f, 0.0600f, 0.0578f, 0.0540f, 0.0498f, 0.0475f,
      0.0467f, 0.0450f, 0.0440f, 0.0426f, 0.0410f, 0.0400f, 0.0390f, 0.0375f, 0.0360f, 0.0340f, 0.0330f, 0.0328f, 0.0325f,
      0.0330f, 0.0340f, 0.0350f, 0.0360f, 0.0375f, 0.0385f, 0.0400f, 0.0420f, 0.0430f, 0.0440f, 0.0445f, 0.0450f, 0.0460f,
      0.0475f, 0.0490f, 0.0515f, 0.0520f, 0.0505f, 0.0440f, 0.0390f, 0.0340f, 0.0300f};
  static constexpr float kE[61] = {
      0.668f, 0.672f, 0.680f, 0.687f, 0.693f, 0.701f, 0.707f, 0.708f, 0.707f, 0.704f, 0.701f, 0.699f, 0.700f, 0.703f, 0.703f,
      0.703f, 0.703f, 0.704f, 0.702f, 0.700f, 0.700f, 0.695f, 0.690f, 0.685f, 0.680f, 0.675f, 0.670f, 0.665f, 0.660f, 0.655f,
      0.650f, 0.645f, 0.640f, 0.630f, 0.623f, 0.615f, 0.610f, 0.614f, 0.618f, 0.622f, 0.626f, 0.630f, 0.634f, 0.638f, 0.642f,
      0.647f, 0.653f, 0.658f, 0.663f, 0.667f, 0.672f, 0.677f, 0.682f, 0.687f, 0.695f, 0.697f, 0.693f, 0.665f, 0.640f, 0.620f,
      0.600f};
  static constexpr float kBw[61] = {
      0.0076f, 0.0072f, 0.0068f, 0.0064f, 0.0061f, 0.0058f, 0.0055f, 0.0052f, 0.0049f, 0.0047f, 0.0045f, 0.0043f, 0.0041f,
      0.0039f, 0.0037f, 0.0036f, 0.0034f, 0.0033f, 0.0031f, 0.0030f, 0.0029f, 0.0027f, 0.0026f, 0.0025f, 0.0024f, 0.0023f,
      0.0022f, 0.0022f, 0.0021f, 0.0020f, 0.0019f, 0.0018f, 0.0018f, 0.0017f, 0.0017f, 0.0016f, 0.0016f, 0.0015f, 0.0015f,
      0.0014f, 0.0014f, 0.0013f, 0.0013f, 0.0012f, 0.0012f, 0.0011f, 0.0011f, 0.0010f, 0.0010f, 0.0010f, 0.0010f, 0.0009f,
      0.0008f, 0.0008f, 0.0008f, 0.0007f, 0.0007f, 0.0007f, 0.0007f, 0.0007f, 0.0007f};
  static constexpr float kTwl[62] = {
      0.250f, 0.275f, 0.300f, 0.325f, 0.345f, 0.375f, 0.400f, 0.425f, 0.445f, 0.475f, 0.500f, 0.525f, 0.550f, 0.575f, 0.600f,
      0.625f, 0.650f, 0.675f, 0.700f, 0.725f, 0.750f, 0.775f, 0.800f, 0.825f, 0.850f, 0.875f, 0.900f, 0.925f, 0.950f, 0.975f,
      1.000f, 1.200f, 1.400f, 1.600f, 1.800f, 2.000f, 2.200f, 2.400f, 2.600f, 2.650f, 2.700f, 2.750f, 2.800f, 2.850f, 2.900f,
      2.950f, 3.000f, 3.050f, 3.100f, 3.150f, 3.200f, 3.250f, 3.300f, 3.350f, 3.400f, 3.450f, 3.500f, 3.600f, 3.700f, 3.800f,
      3.900f, 4.000f};
  static constexpr float kTnr[62] = {
      1.362f, 1.354f, 1.349f, 1.346f, 1.343f, 1.341f, 1.339f, 1.338f, 1.337f, 1.336f, 1.335f, 1.334f, 1.333f, 1.333f, 1.332f,
      1.332f, 1.331f, 1.331f, 1.331f, 1.330f, 1.330f, 1.330f, 1.329f, 1.329f, 1.329f, 1.328f, 1.328f, 1.328f, 1.327f, 1.327f,
      1.327f, 1.324f, 1.321f, 1.317f, 1.312f, 1.306f, 1.296f, 1.279f, 1.242f, 1.219f, 1.188f, 1.157f, 1.142f, 1.149f, 1.201f,
      1.292f, 1.371f, 1.426f, 1.467f, 1.483f, 1.478f, 1.467f, 1.450f, 1.432f, 1.420f, 1.410f, 1.400f, 1.385f, 1.374f, 1.364f,
      1.357f, 1.351f};
  static constexpr float kTni[62] = {
      3.35E-08f, 2.35E-08f, 1.60E-08f, 1.08E-08f, 6.50E-09f, 3.50E-09f, 1.86E-09f, 1.30E-09f, 1.02E-09f, 9.35E-10f, 1.00E-09f,
      1.32E-09f, 1.96E-09f, 3.60E-09f, 1.09E-08f, 1.39E-08f, 1.64E-08f, 2.23E-08f, 3.35E-08f, 9.15E-08f, 1.56E-07f, 1.48E-07f,
      1.25E-07f, 1.82E-07f, 2.93E-07f, 3.91E-07f, 4.86E-07f, 1.06E-06f, 2.93E-06f, 3.48E-06f, 2.89E-06f, 9.89E-06f, 1.38E-04f,
      8.55E-05f, 1.15E-04f, 1.10E-03f, 2.89E-04f, 9.56E-04f, 3.17E-03f, 6.70E-03f, 1.90E-02f, 5.90E-02f, 1.15E-01f, 1.85E-01f,
      2.68E-01f, 2.98E-01f, 2.72E-01f, 2.40E-01f, 1.92E-01f, 1.35E-01f, 9.24E-02f, 6.10E-02f, 3.68E-02f, 2.61E-02f, 1.95E-02f,
      1.32E-02f, 9.40E-03f, 5.15E-03f, 3.60E-03f, 3.40E-03f, 3.80E-03f, 4.60E-03f};

  // 1-based bracketing index of x in an increasing table of n entries
  // (getbound): the searched half depends on the midpoint, and x outside
  // the table takes the first or the last interval.
  static int bracket(const float *xv, int n, float x) {
    const int imid = n / 2 + 1;
    const int lo = x > xv[imid - 1] ? imid : 1, hi = x > xv[imid - 1] ? n - 1 : imid;
    for (int i = lo; i <= hi; ++i)
      if (xv[i - 1] <= x && xv[i] >= x) return i;
    return x < xv[0] ? 1 : n - 1;
  }

  // Sea-water reflectance below the surface for Case I waters (morcasiwat):
  // R = 0.33 bb / (u Kd), iterated on u; zero outside 400-700 nm.
  static float morel_water(float wl, float c) {
    if (wl < 0.400f || wl > 0.700f) return 0.f;
    const int iwl = 1 + (int)std::lround((wl - 0.400f) / 0.005f);  // NINT: half away from zero
    const float kw = kKw[iwl - 1], xc = kXc[iwl - 1], e = kE[iwl - 1], bw = kBw[iwl - 1];
    float bb, kd;
    if (std::fabs(c) < 0.0001f) { bb = 0.5f * bw; kd = kw; }
    else {
      const float b = 0.30f * std::pow(c, 0.62f);
      const float bbt = 0.002f + 0.02f * (0.5f - 0.25f * std::log10(c)) * 0.550f / wl;
      bb = 0.5f * bw + bbt * b;
      kd = kw + xc * std::pow(c, e);
    }
    float r1 = 0.33f * bb / 0.75f / kd, r2 = r1;
    for (int it = 0; it < 1000; ++it) {
      const float u2 = 0.90f * (1.f - r1) / (1.f + 2.25f * r1);
      r2 = 0.33f * bb / u2 / kd;
      if (std::fabs((r2 - r1) / r2) < 0.0001f) break;
      r1 = r2;
    }
    return r2;
  }

  // Unpolarized Fresnel reflectance of a facet (Fresnel), complex index (nr, ni).
  static float facet_fresnel(float nr, float ni, float coschi, float sinchi) {
    const float d = nr * nr - ni * ni - sinchi * sinchi;
    const float a1 = std::fabs(d), a2 = std::sqrt(d * d + 4 * nr * nr * ni * ni);
    const float u = std::sqrt(0.5f * (a1 + a2)), v = std::sqrt(std::max(0.0f, 0.5f * (-a1 + a2)));
    const float rr2 = ((coschi - u) * (coschi - u) + v * v) / ((coschi + u) * (coschi + u) + v * v);
    const float b1 = (nr * nr - ni * ni) * coschi, b2 = 2 * nr * ni * coschi;
    const float rl2 = ((b1 - u) * (b1 - u) + (b2 - v) * (b2 - v)) / ((b1 + u) * (b1 + u) + (b2 + v) * (b2 + v));
    return (rr2 + rl2) / 2.f;
  }

  // Sun glint of the Cox-Munk anisotropic (Gram-Charlier) slope
  // distribution (sunglint); angles in degrees.
  static float sun_glint(float wspd, float nr, float ni, float azw, float ts, float tv, float fi) {
    const float pi = std::atan(1.f) * 4.f, fac = pi / 180.f;
    const float phw = azw * fac, cs = std::cos(ts * fac), cv = std::cos(tv * fac), ss = std::sin(ts * fac),
                sv = std::sin(tv * fac), phi = fi * fac;
    const float zx = -sv * std::sin(phi) / (cs + cv), zy = (ss + sv * std::cos(phi)) / (cs + cv);
    const float tilt = std::atan(std::sqrt(zx * zx + zy * zy));
    const float sc = 0.003f + 0.00192f * wspd, su = 0.00316f * wspd;
    const float c21 = 0.01f - 0.0086f * wspd, c03 = 0.04f - 0.033f * wspd, c40 = 0.40f, c22 = 0.12f, c04 = 0.23f;
    const float xe = (std::cos(phw) * zx + std::sin(phw) * zy) / std::sqrt(sc);
    const float xn = (-std::sin(phw) * zx + std::cos(phw) * zy) / std::sqrt(su);
    const float xe2 = xe * xe, xn2 = xn * xn;
    float coef = 1 - c21 / 2.f * (xe2 - 1) * xn - c03 / 6.f * (xn2 - 3) * xn;
    coef = coef + c40 / 24.f * (xe2 * xe2 - 6 * xe2 + 3);
    coef = coef + c04 / 24.f * (xn2 * xn2 - 6 * xn2 + 3);
    coef = coef + c22 / 4.f * (xe2 - 1) * (xn2 - 1);
    const float proba = coef / 2.f / pi / std::sqrt(su) / std::sqrt(sc) * std::exp(-(xe2 + xn2) / 2.f);
    float cos2chi = cv * cs + sv * ss * std::cos(phi);
    cos2chi = std::min(1.0f, std::max(-1.0f, cos2chi));
    const float coschi = std::sqrt(0.5f * (1 + cos2chi)), sinchi = std::sqrt(0.5f * (1 - cos2chi));
    const float r1 = facet_fresnel(nr, ni, coschi, sinchi);
    const float ct = std::cos(tilt), ct2 = ct * ct;
    return pi * r1 * proba / 4.f / cs / cv / (ct2 * ct2);
  }

  // ocean_brdf_sw with the default salinity: whitecaps + glint + water body.
  static float ocean_reflection(float pws, float pcl, float pwl, float xmuo, float xmu, float xphi, float xpaw) {
    const float pi = std::atan(1.f) * 4.f, fac = pi / 180.f;
    const float paw = xpaw / fac;
    const float phi = xphi < 0.f ? -xphi : (xphi >= 2.0f * pi ? xphi - 2.0f * pi : xphi);
    const float tetas = std::acos(xmuo <= 0.028f ? 0.028f : xmuo) / fac;
    const float tetav = std::acos(xmu <= 0.028f ? 0.028f : xmu) / fac;
    const float wl = pwl < 0.4f ? 0.4f : (pwl > 4.0f ? 4.0f : pwl);
    const float fi = 180.0f - phi / fac;
    const float wspd = std::max(0.25f, pws);
    // refractive index of sea water (indwat): Hale & Querry pure water,
    // interpolated, plus 0.006 for the default salinity
    int i = 2;
    while (!(wl < kTwl[i - 1]) && i < 62) ++i;
    const float xwl = kTwl[i - 1] - kTwl[i - 2];
    float nr = kTnr[i - 2] + (wl - kTwl[i - 2]) * (kTnr[i - 1] - kTnr[i - 2]) / xwl;
    const float ni = kTni[i - 2] + (wl - kTwl[i - 2]) * (kTni[i - 1] - kTni[i - 2]) / xwl;
    nr = nr + 0.006f;
    const float n12 = std::sqrt(nr * nr + ni * ni);
    // whitecaps (Lambertian)
    const float w = 2.95E-06f * std::pow(wspd, 3.52f);
    const int iwl = 1 + (int)((wl - 0.2f) / 0.1f);
    const float wlp = 0.5f + (iwl - 1) * 0.1f;
    const float refi = kWhitecap[iwl] + (wl - wlp) / 0.1f * (kWhitecap[iwl - 1] - kWhitecap[iwl]);
    const float rwc = w * refi;
    const float rw = morel_water(wl, pcl);
    const int iws1 = bracket(kWsBnd, 6, wspd), isz1 = bracket(kAngBnd, 5, tetas), ivz1 = bracket(kAngBnd, 5, tetav);
    const float tds = kTds[isz1 - 1][iws1 - 1], tdv = kTdv[ivz1 - 1][iws1 - 1];
    const float rog = sun_glint(wspd, nr, ni, paw, tetas, tetav, fi);
    const float a = 0.485f;
    const float rwb = (1 / (n12 * n12)) * tds * tdv * rw / (1 - a * rw);
    return rwc + (1 - w) * rog + (1 - rwc) * rwb;
  }


  // ROSS_THICK_LI_SPARSE (src/polarized/shdomsub2.f:1303-1355): the MODIS
  // kernel BRDF fiso + fvol K_vol + fgeo K_geo (RossThick volume kernel,
  // LiSparse geometric kernel with crown shape h/b = 2, b/r = 1), kernels in
  // double precision from single-precision cosines, clipped at zero.
  static float ross_li_reflection(float fiso, float fgeo, float fvol, float hb, float br, float mud, float muu,
                                  float relaz) {
    const double pi = std::acos(-1.0);
    double coseta = (double)(mud * muu + std::sqrt(1.0f - mud * mud) * std::sqrt(1.0f - muu * muu) * std::cos(relaz));
    const float kvol = (float)((((pi / 2.0 - std::acos(coseta)) * coseta + std::sqrt(1.0 - coseta * coseta)) /
                                (double)(mud + muu)) - pi / 4.0);
    const double thd = std::fabs(std::atan(br * std::sqrt(1.0 - (double)(mud * mud)) / mud));
    const double thu = std::fabs(std::atan(br * std::sqrt(1.0 - (double)(muu * muu)) / muu));
    const double md = std::cos(thd), mu = std::cos(thu);
    coseta = md * mu + std::sqrt(1.0 - md * md) * std::sqrt(1.0 - mu * mu) * std::cos((double)relaz);
    const double secd = 1.0 / md, secu = 1.0 / mu;
    const double tand = std::sqrt(1.0 - md * md) / md, tanu = std::sqrt(1.0 - mu * mu) / mu;
    const double dsq = tand * tand + tanu * tanu - 2 * tanu * tand * std::cos((double)relaz);
    const double tts = tand * tanu * std::sin((double)relaz);
    double cost = hb * std::sqrt(dsq + tts * tts) / (secd + secu);
    cost = std::min(1.0, std::max(-1.0, cost));
    const double o = (std::acos(cost) - cost * std::sqrt(1.0 - cost * cost)) * (secd + secu) / pi;
    const float kgeo = (float)(o - secd - secu + 0.5 * (1.0 + coseta) * secu * secd);
    return std::max(fiso + fvol * kvol + fgeo * kgeo, 0.0f);
  }

  void surface_brdf(const R *par, float mu2, float phi2, float mu1, float phi1, double refl[3][3]) const {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) refl[i][j] = 0.0;
    if (brdf == 'M') {
      refl[0][0] = ross_li_reflection((float)par[0], (float)par[1], (float)par[2], 2.0f, 1.0f, -mu1, mu2, phi1 - phi2);
    } else if (brdf == 'O') {
      refl[0][0] = ocean_reflection((float)par[0], (float)par[1], p.wavelen, -mu1, mu2, phi1 - phi2, phi1);
    } else if (brdf == 'R') {
      refl[0][0] = rpv_reflection((float)par[0], (float)par[1], (float)par[2], -mu1, mu2,
                                  phi1 - phi2 - (float)std::acos(-1.0f));
    } else if (brdf == 'D') {
      diner_reflection((float)par[0], (float)par[1], (float)par[2], (float)par[3], (float)par[4], -mu1, mu2,
                       phi2 - phi1, refl);
    } else {
      wave_fresnel_reflection((float)par[0], (float)par[1], (float)par[2], mu1, mu2, phi1, phi2, refl);
    }
  }

  // DINER_REFLECTION (src/polarized/shdomsub2.f:1526-1657): depolarizing
  // modified-RPV volume term with the hotspot factor plus Fresnel
  // reflection (index 1.5) from microfacets with a uniform (sigma <= 0) or
  // Gaussian slope distribution, rotated into the meridional planes; single
  // precision (mu1, mu2 > 0, phi = phi2 - phi1).
  static void diner_reflection(float a, float k, float b, float zeta, float sigma, float mu1, float mu2, float phi,
                               double refl[3][3]) {
    float r[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const float sinth1 = std::sqrt(1.0f - mu1 * mu1), sinth2 = std::sqrt(1.0f - mu2 * mu2);
    const float cosphi = std::cos(phi);
    float cossc = -mu1 * mu2 + sinth1 * sinth2 * cosphi;
    cossc = std::min(1.0f, std::max(-1.0f, cossc));
    const float tan1 = sinth1 / mu1, tan2 = sinth2 / mu2;
    const float capg = std::sqrt(std::fabs(tan1 * tan1 + tan2 * tan2 + 2 * tan1 * tan2 * cosphi));
    const float hot = 1 + (1 - a) / (1 + capg);
    r[0][0] = a * std::pow((mu1 + mu2) * mu1 * mu2, k - 1) * std::exp(b * cossc);
    r[0][0] = r[0][0] * hot;
    if (zeta >= 0.0f) {
      const float gamma = 0.5f * std::acos(-cossc), cosg = std::cos(gamma);
      const float eps = 1.5f * 1.5f;
      const float d = std::sqrt(eps - 1.0f + cosg * cosg);
      const float rp = (eps * cosg - d) / (eps * cosg + d), rs = (cosg - d) / (cosg + d);
      const float f11 = 0.5f * (rp * rp + rs * rs), f12 = 0.5f * (rp * rp - rs * rs), f33 = rp * rs;
      const float cosbeta = 0.5f * (mu1 + mu2) / cosg;
      float h;
      if (sigma > 0.0f)
        h = zeta * std::exp(-0.5f * (1 / (cosbeta * cosbeta) - 1) / (sigma * sigma)) /
            (8 * sigma * sigma * mu2 * mu1 * cosbeta * cosbeta * cosbeta * cosbeta);
      else
        h = zeta / (8 * mu2 * mu1 * cosbeta);
      r[0][0] = r[0][0] + h * f11;
      const float sinphi = std::sin(phi);
      const float al1 = std::atan(sinth2 * sinphi / (mu2 * sinth1 + sinth2 * mu1 * cosphi));
      const float al2 = std::atan(sinth1 * sinphi / (sinth2 * mu1 + mu2 * sinth1 * cosphi));
      const float c1 = std::cos(2 * al1), s1 = std::sin(2 * al1), c2 = std::cos(2 * al2), s2 = std::sin(2 * al2);
      r[0][1] = h * f12 * c1;
      r[1][0] = h * f12 * c2;
      r[1][1] = h * (f11 * c1 * c2 + f33 * s1 * s2);
      r[0][2] = -h * f12 * s1;
      r[1][2] = h * (-f11 * s1 * c2 + f33 * c1 * s2);
      r[2][0] = -h * f12 * s2;
      r[2][1] = h * (-f11 * c1 * s2 + f33 * s1 * c2);
      r[2][2] = h * (f11 * s1 * s2 + f33 * c1 * c2);
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) refl[i][j] = r[i][j];
  }

  // RPV_REFLECTION (src/polarized/shdomsub2.f:1658-1696): Rahman, Pinty and
  // Verstraete (1993) with the small-mu floor of 0.03.
  static float rpv_reflection(float rho0, float k, float theta, float mu1, float mu2, float phi) {
    const float mu_min = 0.03f;
    float x1 = std::max(mu1, mu_min), x2 = std::max(mu2, mu_min);
    float m = std::pow(x1 * x2 * (x1 + x2), k - 1.0f);
    float cosphi = std::cos(phi);
    float sin1 = std::sqrt(1.0f - x1 * x1), sin2 = std::sqrt(1.0f - x2 * x2);
    float cosg = x1 * x2 + sin1 * sin2 * cosphi;
    float f = (1.0f - theta * theta) / std::pow(1.0f + 2.0f * theta * cosg + theta * theta, 1.5f);
    float tan1 = sin1 / x1, tan2 = sin2 / x2;
    float capg = std::sqrt(std::fabs(tan1 * tan1 + tan2 * tan2 - 2.0f * tan1 * tan2 * cosphi));
    float h = 1.0f + (1.0f - rho0) / (1.0f + capg);
    return rho0 * m * f * h;
  }

  // WAVE_FRESNEL_REFLECTION (src/polarized/shdomsub2.f:1358-1525): Fresnel
  // reflection of a dielectric interface (index mre + i mim) with a Gaussian
  // distribution of slopes of variance 0.0015 + 0.00256 wind speed (Cox and
  // Munk) and the shadowing factor; the I, Q, U block of the Mueller matrix.
  static void wave_fresnel_reflection(float mre, float mim, float wind, float mui, float mur, float phii, float phir,
                                      double refl[3][3]) {
    typedef std::complex<double> Cx;
    const Cx cn1(1.0, 0.0), cn2((double)mre, (double)mim);
    const double sigma2 = std::max(0.0005, 0.0015 + 0.00256 * (double)wind);
    double dmui = std::fabs((double)mui), dmur = (double)mur;
    if (std::fabs(dmui - 1.0) < 1e-10) dmui = 0.999999999999;
    if (std::fabs(dmur - 1.0) < 1e-10) dmur = 0.999999999999;
    const double dcosi = std::cos((double)phii), dsini = std::sin((double)phii);
    const double dcosr = std::cos((double)phir), dsinr = std::sin((double)phir);
    const double dsi = std::sqrt(1.0 - dmui * dmui), dsr = std::sqrt(1.0 - dmur * dmur);
    const double vi1 = dsi * dcosi, vi2 = dsi * dsini, vi3 = -dmui;
    const double vr1 = dsr * dcosr, vr2 = dsr * dsinr, vr3 = dmur;
    const double u1 = vi1 - vr1, u2 = vi2 - vr2, u3 = vi3 - vr3;
    const double fact1 = u1 * u1 + u2 * u2 + u3 * u3, factor = std::sqrt(1.0 / fact1);
    const double xi1 = factor * (u1 * vi1 + u2 * vi2 + u3 * vi3);
    const Cx cxi2 = std::sqrt(1.0 - (1.0 - xi1 * xi1) * cn1 * cn1 / (cn2 * cn2));
    Cx c1 = cn1 * xi1, c2 = cn2 * cxi2;
    const Cx crper = (c1 - c2) / (c1 + c2);
    c1 = cn2 * xi1; c2 = cn1 * cxi2;
    const Cx crpar = (c1 - c2) / (c1 + c2);
    const double ti1 = -dmui * dcosi, ti2 = -dmui * dsini, ti3 = -dsi;
    const double tr1 = dmur * dcosr, tr2 = dmur * dsinr, tr3 = -dsr;
    const double pi1 = -dsini, pi2 = dcosi, pr1 = -dsinr, pr2 = dcosr;
    const double pikr = pi1 * vr1 + pi2 * vr2, prki = pr1 * vi1 + pr2 * vi2;
    const double tikr = ti1 * vr1 + ti2 * vr2 + ti3 * vr3, trki = tr1 * vi1 + tr2 * vi2 + tr3 * vi3;
    const double e1 = pikr * prki, e2 = tikr * trki, e3 = tikr * prki, e4 = pikr * trki;
    const Cx cf11 = e1 * crper + e2 * crpar, cf12 = -e3 * crper + e4 * crpar;
    const Cx cf21 = -e4 * crper + e3 * crpar, cf22 = e2 * crper + e1 * crpar;
    const double vp1 = vi2 * vr3 - vi3 * vr2, vp2 = vi3 * vr1 - vi1 * vr3, vp3 = vi1 * vr2 - vi2 * vr1;
    const double dmod = std::pow(vp1 * vp1 + vp2 * vp2 + vp3 * vp3, 2);
    const double rdz2 = u3 * u3, rdz4 = rdz2 * rdz2;
    const double dex = std::exp(-(u1 * u1 + u2 * u2) / (2 * sigma2 * rdz2));
    const double dcoeff = fact1 * fact1 * dex / (4 * dmui * dmur * dmod * rdz4 * 2 * sigma2);
    const double af = 0.5 * dcoeff;
    const double af11 = std::norm(cf11), af12 = std::norm(cf12), af21 = std::norm(cf21), af22 = std::norm(cf22);
    refl[0][0] = (af11 + af12 + af21 + af22) * af;
    refl[0][1] = (af11 - af12 + af21 - af22) * af;
    refl[1][0] = (af11 - af22 + af12 - af21) * af;
    refl[1][1] = (af11 - af12 - af21 + af22) * af;
    const Cx c21 = std::conj(cf21), c22 = std::conj(cf22);
    const Cx ctttp = cf11 * std::conj(cf12), cttpt = cf11 * c21, cttpp = cf11 * c22;
    const Cx ctppt = cf12 * c21, ctppp = cf12 * c22, cptpp = cf21 * c22;
    refl[0][2] = ((-ctttp - cptpp) * dcoeff).real();
    refl[1][2] = ((-ctttp + cptpp) * dcoeff).real();
    refl[2][0] = ((-cttpt - ctppp) * dcoeff).real();
    refl[2][1] = ((-cttpt + ctppp) * dcoeff).real();
    refl[2][2] = ((cttpp + ctppt) * dcoeff).real();
    const double pp = std::acos(-1.0), s1 = std::sqrt(2 * sigma2 / pp), s3 = 1.0 / std::sqrt(2 * sigma2), s2 = s3 * s3;
    double dcot = dmui / std::sqrt(1.0 - dmui * dmui);
    const double shi = 0.5 * (s1 * std::exp(-s2 * dcot * dcot) / dcot - std::erfc(dcot * s3));
    dcot = dmur / std::sqrt(1.0 - dmur * dmur);
    const double shr = 0.5 * (s1 * std::exp(-s2 * dcot * dcot) / dcot - std::erfc(dcot * s3));
    const double shadow = 1.0 / (1.0 + shi + shr);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) refl[i][j] = (double)(float)(refl[i][j] * shadow);
  }

  // VARIABLE_BRDF_SURFACE (src/polarized/shdomsub1.f:2592-2664) at bottom
  // point b for the outgoing direction (mu2, phi2): the reflected direct
  // beam plus the reflection of the stored downwelling radiances (no
  // surface emission for a solar source).
  void variable_brdf(size_t b, float mu2, float phi2, R *out) const {
    const R *par = &botpar[b * nsfcpar];
    const float opi = 1.0f / (float)std::acos(-1.0f);
    double refl[3][3];
    surface_brdf(par, mu2, phi2, p.solarmu, p.solaraz, refl);
    for (int k = 0; k < nst; ++k) out[k] = (R)(opi * refl[k][0]) * dirflux[botp[b]];
    const int ndown = nang / 2;
    int jang = 0;
    for (int jmu = 0; jmu < nmu / 2; ++jmu)
      for (int jphi = 0; jphi < nphi0[jmu]; ++jphi, ++jang) {
        surface_brdf(par, mu2, phi2, mu[jmu], phi[(size_t)jmu * nphi0max + jphi], refl);
        const R w = (R)(opi * std::fabs(mu[jmu]) * wtdo[(size_t)jmu * nphi0max + jphi]);
        const R *rin = &bcdown[(b * ndown + jang) * nst];
        for (int k1 = 0; k1 < nst; ++k1)
          for (int k = 0; k < nst; ++k) out[k] = out[k] + w * (R)(float)refl[k][k1] * rin[k1];
        // polarized thermal emission, emissivity 1 - R11 (zero for a solar source)
        if (srct != 'S') {
          const R bp = botplanck[b];
          out[0] = out[0] + w * ((R)1 - (R)(float)refl[0][0]) * bp;
          for (int k = 1; k < nst; ++k) out[k] = out[k] - w * (R)(float)refl[k][0] * bp;
        }
      }
  }

  // FIXED/VARIABLE_LAMBERTIAN_BOUNDARY (src/polarized/shdomsub1.f:2438-2529).
  void lambertian_boundary() {
    bcrad_bot.assign(botp.size(), 0);
    const R opi = (R)1 / (R)std::acos(-1.0f);
    for (size_t b = 0; b < botp.size(); ++b) {
      int i = botp[b];
      bcrad_bot[b] = opi * sfcgridalb[b] * (dirflux[i] + fluxes[2 * (size_t)i]);
      if (srct != 'S') bcrad_bot[b] = bcrad_bot[b] + botplanck[b] * ((R)1 - sfcgridalb[b]);  // ground emission
    }
  }

  bool init_solution() {
    make_direct();
    init_radiance();
    source.assign((size_t)npts * nlm * nst, 0);
    delsource.assign(p.accelflag ? (size_t)npts * nlm * nst : 1, 0);
    shptr.assign(npts + 1, 0); oshptr.assign(npts + 1, 0);
    fluxes.assign((size_t)2 * npts, 0);
    compute_source(false, true);
    if (p.accelflag) {
      oshptr = shptr;
      std::fill(delsource.begin(), delsource.end(), (R)0);
    }
    boundary_points();
    iter = 0; solcrit = 1; accel_a = 0;
    return true;
  }

  // SH_TO_DO_UNPOL (src/polarized/shdomsub1.f:2928-3036) with the DFT branch.
  void sh_to_do(int imu, std::vector<R> &work) const {
    int n0 = nphi0[imu], nm = 2 * mm + 1;
    std::vector<R> sumuv(nm), sumcs(nm);
    for (int i = 0; i < npts; ++i) {
      int is = shptr[i], nsh = shptr[i + 1] - is;
      R *out = &work[(size_t)i * nphi0max];
      if (nsh == 0) { for (int k = 0; k < n0; ++k) out[k] = 0; continue; }
      int me = std::max(0, std::min(n0 / 2 - 1, mofj[nsh - 1]));
      std::fill(sumuv.begin(), sumuv.end(), (R)0);
      for (int j = 0; j < nsh; ++j) sumuv[mofj[j] + mm] += cmu1[(size_t)imu * nlm + j] * source[(size_t)is + j];
      sumcs[mm] = sumuv[mm];
      for (int m = 1; m <= me; ++m) {
        sumcs[mm + m] = sumuv[mm + m] + sumuv[mm - m];
        sumcs[mm - m] = sumuv[mm - m] - sumuv[mm + m];
      }
      for (int k = 0; k < n0; ++k) {
        const R *c = &cphi1[((size_t)imu * nphi0max + k) * nm + mm];
        R s = 0;
        for (int m = -me; m <= me; ++m) s += c[m] * sumcs[mm + m];
        out[k] = s;
      }
    }
  }

  // DO_TO_SH_UNPOL (src/polarized/shdomsub1.f:3164-3254) with the DFT branch.
  void do_to_sh(int imu, const std::vector<R> &work) {
    int n0 = nphi0[imu], nm = 2 * mm + 1;
    std::vector<R> sumuv(nm), sumcs(nm);
    int is = 0;
    for (int i = 0; i < npts; ++i) {
      int nsh = rshptr[i + 1] - rshptr[i];
      std::fill(sumcs.begin(), sumcs.end(), (R)0);
      int me = std::max(0, std::min(n0 / 2 - 1, mofj[std::max(nsh, 1) - 1]));
      const R *in = &work[(size_t)i * nphi0max];
      for (int m = -me; m <= me; ++m) {
        R s = 0;
        for (int k = 0; k < n0; ++k) s += cphi2[((size_t)imu * nphi0max + k) * nm + mm + m] * in[k];
        sumcs[mm + m] = s;
      }
      sumuv[mm] = sumcs[mm];
      for (int m = 1; m <= mm; ++m) {
        sumuv[mm + m] = sumcs[mm + m] - sumcs[mm - m];
        sumuv[mm - m] = sumcs[mm + m] + sumcs[mm - m];
      }
      for (int j = 0; j < nsh; ++j) radiance[(size_t)is + j] += cmu2[(size_t)imu * nlm + j] * sumuv[mofj[j] + mm];
      is += nsh;
    }
  }

  // SH_TO_DO (src/polarized/shdomsub1.f:2789-2926), DFT branch, NSTOKES = 3:
  // work [npts][nphi0max][3].
  void sh_to_do_pol(int imu, std::vector<R> &work) const {
    const int n0 = nphi0[imu], nm = 2 * mm + 1;
    std::vector<R> uv((size_t)3 * nm), cs((size_t)3 * nm);
    const R *C1 = &cmu1p[(size_t)imu * nlm * 6];
    for (int i = 0; i < npts; ++i) {
      const int is = shptr[i], nsh = shptr[i + 1] - is;
      R *out = &work[(size_t)i * nphi0max * 3];
      if (nsh == 0) { for (int k = 0; k < 3 * n0; ++k) out[k] = 0; continue; }
      const int me = std::max(0, std::min(n0 / 2 - 1, mofj[nsh - 1]));
      std::fill(uv.begin(), uv.end(), (R)0);
      const R *in = &source[(size_t)is * 3];
      for (int j = 0; j < nsh; ++j) {
        const int m = mofj[j] + mm;
        const R *c = &C1[(size_t)j * 6];
        uv[m] += c[0] * in[3 * j];
        uv[nm + m] += c[1] * in[3 * j + 1] + c[4] * in[3 * j + 2];
        uv[2 * nm + m] += c[5] * in[3 * j + 1] + c[2] * in[3 * j + 2];
      }
      std::fill(cs.begin(), cs.end(), (R)0);
      for (int n = 0; n < 3; ++n) cs[n * nm + mm] = uv[n * nm + mm];
      for (int m = 1; m <= me; ++m)
        for (int n = 0; n < 2; ++n) {
          cs[n * nm + mm + m] = uv[n * nm + mm + m] + uv[n * nm + mm - m];
          cs[n * nm + mm - m] = uv[n * nm + mm - m] - uv[n * nm + mm + m];
        }
      for (int m = 1; m <= me; ++m) {
        cs[2 * nm + mm - m] = uv[2 * nm + mm + m] - uv[2 * nm + mm - m];
        cs[2 * nm + mm + m] = uv[2 * nm + mm + m] + uv[2 * nm + mm - m];
      }
      for (int k = 0; k < n0; ++k) {
        const R *c = &cphi1[((size_t)imu * nphi0max + k) * nm + mm];
        for (int n = 0; n < 3; ++n) {
          R sum = 0;
          for (int m = -me; m <= me; ++m) sum += c[m] * cs[n * nm + mm + m];
          out[3 * k + n] = sum;
        }
      }
    }
  }

  // DO_TO_SH (src/polarized/shdomsub1.f:3041-3160), DFT branch, NSTOKES = 3.
  void do_to_sh_pol(int imu, const std::vector<R> &work) {
    const int n0 = nphi0[imu], nm = 2 * mm + 1;
    std::vector<R> uv((size_t)3 * nm), cs((size_t)3 * nm);
    const R *C2 = &cmu2p[(size_t)imu * nlm * 6];
    int is = 0;
    for (int i = 0; i < npts; ++i) {
      const int nsh = rshptr[i + 1] - rshptr[i];
      const int me = std::max(0, std::min(n0 / 2 - 1, mofj[std::max(nsh, 1) - 1]));
      const R *in = &work[(size_t)i * nphi0max * 3];
      std::fill(cs.begin(), cs.end(), (R)0);
      for (int m = -me; m <= me; ++m)
        for (int n = 0; n < 3; ++n) {
          R sum = 0;
          for (int k = 0; k < n0; ++k) sum += cphi2[((size_t)imu * nphi0max + k) * nm + mm + m] * in[3 * k + n];
          cs[n * nm + mm + m] = sum;
        }
      std::fill(uv.begin(), uv.end(), (R)0);
      for (int n = 0; n < 3; ++n) uv[n * nm + mm] = cs[n * nm + mm];
      for (int m = 1; m <= me; ++m) {
        for (int n = 0; n < 2; ++n) {
          uv[n * nm + mm + m] = cs[n * nm + mm + m] - cs[n * nm + mm - m];
          uv[n * nm + mm - m] = cs[n * nm + mm + m] + cs[n * nm + mm - m];
        }
        uv[2 * nm + mm + m] = cs[2 * nm + mm + m] + cs[2 * nm + mm - m];
        uv[2 * nm + mm - m] = cs[2 * nm + mm + m] - cs[2 * nm + mm - m];
      }
      R *out = &radiance[(size_t)is * 3];
      for (int j = 0; j < nsh; ++j) {
        const int m = mofj[j] + mm;
        const R *c = &C2[(size_t)j * 6];
        out[3 * j] += c[0] * uv[m];
        out[3 * j + 1] += c[1] * uv[nm + m] + c[4] * uv[2 * nm + m];
        out[3 * j + 2] += c[5] * uv[nm + m] + c[2] * uv[2 * nm + m];
      }
      is += nsh;
    }
  }

  // BACK_INT_GRID3D_UNPOL (src/polarized/shdomsub1.f:3695-4038).
  bool back_int_grid3d(float muv, float phiv, int kang, const std::vector<R> &work,
                       std::vector<R> &gridrad) {
    double eps = 1.0e-3 * (gridpos[3 * gridptr[7] + 2] - gridpos[3 * gridptr[0] + 2]);
    auto Wv = [&](int q, int k) { return (double)work[((size_t)q * nphi0max + kang) * nst + k]; };
    const double pi = (double)(float)std::acos(-1.0f);
    double smu = (double)std::sqrt(1.0f - muv * muv);
    double cx = smu * std::cos((double)phiv + pi);
    double cy = smu * std::sin((double)phiv + pi);
    double cz = -(double)muv, cxinv, cyinv, czinv;
    if (std::fabs(cx) > 1.0e-5) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1.0e6; }
    if (std::fabs(cy) > 1.0e-5) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1.0e6; }
    czinv = 1.0 / cz;
    int bitx = cx < 0 ? 1 : 0, bity = cy < 0 ? 1 : 0, bitz;
    if (cz < -1.0e-3) bitz = 1; else if (cz > 1.0e-3) bitz = 0; else { err = "BACK_INT_GRID: Bad MU"; return false; }
    int ioct = 1 + bitx + 2 * bity + 4 * bitz;
    static const int joctorder3[8] = {1, 3, 5, 7, 2, 4, 6, 8};
    int joct = joctorder3[ioct - 1] - 1;
    double transmin = p.transmin;
    for (int iorder = 0; iorder < npts; ++iorder) {
      int ipcell = sweep_cell[(size_t)joct * npts + iorder];
      int ipt = gridptr[8 * ipcell + sweep_corner[(size_t)joct * npts + iorder]];
      if (gridrad[(size_t)ipt * nst] >= 0) continue;
      int icell = ipcell;
      double rad[3] = {0.0, 0.0, 0.0}, transmit = 1.0, srcext1[3], srcext0[3];
      double ext1 = total_ext[ipt];
      for (int k = 0; k < nst; ++k) srcext1[k] = ext1 * Wv(ipt, k);
      double xe = gridpos[3 * ipt], ye = gridpos[3 * ipt + 1], ze = gridpos[3 * ipt + 2];
      bool validrad = false;
      int guard = 0;
      while (!validrad) {
        if (icell < 0 || ++guard > 100000) { err = "BACK_INT_GRID: ICELL=0"; return false; }
        bool ipinx = cellflags[icell] & 1, ipiny = cellflags[icell] & 2;
        int iopp = gridptr[8 * icell + (8 - ioct)];
        double sox = ipinx ? 1.0e20 : (gridpos[3 * iopp] - xe) * cxinv;
        double soy = ipiny ? 1.0e20 : (gridpos[3 * iopp + 1] - ye) * cyinv;
        double soz = (gridpos[3 * iopp + 2] - ze) * czinv;
        double so = std::min(sox, std::min(soy, soz));
        if (so < -eps) { err = "BACK_INT_GRID: SO<0"; return false; }
        xe += so * cx; ye += so * cy; ze += so * cz;
        int iface, jface;
        if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; }
        else if (soy <= soz) { iface = 3 - bity; jface = 1; }
        else { iface = 5 - bitz; jface = 2; }
        // across a face into smaller cells, the next cell's (smaller) face is
        // interpolated, otherwise this cell's
        const int nbv = neighptr[6 * icell + iface];
        const int inext = nbv >= -1 ? nbv : next_cell(xe, ye, ze, iface, jface, icell);
        const int kface = nbv >= -1 ? iface : kOppFace[iface];
        const int *g = &gridptr[8 * (nbv >= -1 ? icell : inext)];
        int i1 = g[kGridFace[kface][0]], i2 = g[kGridFace[kface][1]], i3 = g[kGridFace[kface][2]],
            i4 = g[kGridFace[kface][3]];
        double u, v;
        if (jface == 0) {
          u = (ze - gridpos[3 * i1 + 2]) / (gridpos[3 * i3 + 2] - gridpos[3 * i1 + 2]);
          v = ipiny ? 0.5 : (ye - gridpos[3 * i1 + 1]) / (gridpos[3 * i2 + 1] - gridpos[3 * i1 + 1]);
        } else if (jface == 1) {
          u = (ze - gridpos[3 * i1 + 2]) / (gridpos[3 * i3 + 2] - gridpos[3 * i1 + 2]);
          v = ipinx ? 0.5 : (xe - gridpos[3 * i1]) / (gridpos[3 * i2] - gridpos[3 * i1]);
        } else {
          u = ipiny ? 0.5 : (ye - gridpos[3 * i1 + 1]) / (gridpos[3 * i3 + 1] - gridpos[3 * i1 + 1]);
          v = ipinx ? 0.5 : (xe - gridpos[3 * i1]) / (gridpos[3 * i2] - gridpos[3 * i1]);
        }
        if (inext >= 0) {
          if (jface == 0) xe = gridpos[3 * gridptr[8 * inext + ioct - 1]];
          else if (jface == 1) ye = gridpos[3 * gridptr[8 * inext + ioct - 1] + 1];
          else ze = gridpos[3 * gridptr[8 * inext + ioct - 1] + 2];
        }
        double f1 = (1 - u) * (1 - v), f2 = (1 - u) * v, f3 = u * (1 - v), f4 = u * v;
        double ext0 = f1 * total_ext[i1] + f2 * total_ext[i2] + f3 * total_ext[i3] + f4 * total_ext[i4];
        for (int k = 0; k < nst; ++k)
          srcext0[k] = f1 * Wv(i1, k) * total_ext[i1] + f2 * Wv(i2, k) * total_ext[i2] + f3 * Wv(i3, k) * total_ext[i3] +
                       f4 * Wv(i4, k) * total_ext[i4];
        double ext = 0.5 * (ext0 + ext1), tau = ext * so, transcell, abscell;
        if (tau >= 0.5) { transcell = std::exp(-tau); abscell = 1.0 - transcell; }
        else { abscell = tau * (1.0 - 0.5 * tau * (1.0 - 0.33333333333 * tau * (1 - 0.25 * tau))); transcell = 1.0 - abscell; }
        for (int k = 0; k < nst; ++k) {
          double src;
          if (tau <= 2.0) {
            if (ext == 0.0) src = 0.0;
            else src = (0.5 * (srcext0[k] + srcext1[k]) + 0.08333333333 * (ext0 * srcext1[k] - ext1 * srcext0[k]) * so) / ext;
          } else {
            double ext0p = ext0, srcext0p = srcext0[k];
            if (tau > 4.0) { ext0p = ext1 + (ext0 - ext1) * 4.0 / tau; if (ext0 > 0.0) srcext0p = srcext0[k] * ext0p / ext0; }
            src = 1.0 / (ext0p + ext1) * (srcext0p + srcext1[k] + (ext0p * srcext1[k] - ext1 * srcext0p) * 2.0 / (ext0p + ext1) * (1 - 2 / tau + 2 * transcell / abscell));
          }
          if (k == 0) src = std::max(src, 0.0);  // only the I source is clipped
          rad[k] += transmit * src * abscell;
        }
        transmit *= transcell;
        auto G = [&](int q, int k) { return (double)gridrad[(size_t)q * nst + k]; };
        bool validface = G(i1, 0) >= -0.1 && G(i2, 0) >= -0.1 && G(i3, 0) >= -0.1 && G(i4, 0) >= -0.1;
        if (inext < 0 || (transmit <= transmin && validface)) {
          if (validface) {
            validrad = true;
            for (int k = 0; k < nst; ++k) rad[k] += transmit * (f1 * G(i1, k) + f2 * G(i2, k) + f3 * G(i3, k) + f4 * G(i4, k));
          } else { err = "BACK_INT_GRID3D: INEXTCELL=0"; return false; }
        } else {
          ext1 = ext0; for (int k = 0; k < nst; ++k) srcext1[k] = srcext0[k]; icell = inext;
        }
      }
      for (int k = 0; k < nst; ++k) gridrad[(size_t)ipt * nst + k] = (R)rad[k];
    }
    return true;
  }

  // BACK_INT_GRID1D (src/polarized/shdomsub1.f:4295-4465).
  bool back_int_grid1d(float muv, int kang, const std::vector<R> &work, std::vector<R> &gridrad) {
    double eps = 1.0e-3 * (gridpos[3 * gridptr[7] + 2] - gridpos[3 * gridptr[0] + 2]);
    (void)eps;
    auto Wv = [&](int q, int k) { return (double)work[((size_t)q * nphi0max + kang) * nst + k]; };
    double cz = -(double)muv, czinv = 1.0 / cz;
    int bitz;
    if (cz < -1.0e-3) bitz = 1; else if (cz > 1.0e-3) bitz = 0; else { err = "BACK_INT_GRID1D: Bad MU"; return false; }
    int ioct = 1 + 4 * bitz;
    int joct = bitz;  // JOCTORDER(1..4)=1, (5..8)=2
    for (int iorder = 0; iorder < npts; ++iorder) {
      int ipcell = sweep_cell[(size_t)joct * npts + iorder];
      int ipt = gridptr[8 * ipcell + sweep_corner[(size_t)joct * npts + iorder]];
      if (gridrad[(size_t)ipt * nst] >= 0) continue;
      int icell = ipcell;
      double transmit = 1.0, ext1 = total_ext[ipt], rad[3] = {0.0, 0.0, 0.0}, srcext1[3], srcext0[3], src[3];
      for (int k = 0; k < nst; ++k) srcext1[k] = ext1 * Wv(ipt, k);
      double ze = gridpos[3 * ipt + 2];
      bool validrad = false;
      int guard = 0;
      while (!validrad) {
        if (icell < 0 || ++guard > 100000) { err = "BACK_INT_GRID1D: ICELL=0"; return false; }
        int iopp = gridptr[8 * icell + (8 - ioct)];
        double so = (gridpos[3 * iopp + 2] - ze) * czinv;
        ze += so * cz;
        int iface = 5 - bitz;
        int inext = neighptr[6 * icell + iface];
        int i1 = gridptr[8 * icell + (iface == 4 ? 0 : 4)];
        if (inext >= 0) ze = gridpos[3 * gridptr[8 * inext + ioct - 1] + 2];
        double ext0 = total_ext[i1];
        for (int k = 0; k < nst; ++k) srcext0[k] = total_ext[i1] * Wv(i1, k);
        double ext = 0.5 * (ext0 + ext1), tau = ext * so, transcell, abscell;
        if (tau >= 0.5) { transcell = std::exp(-tau); abscell = 1.0 - transcell; }
        else { abscell = tau * (1.0 - 0.5 * tau * (1.0 - 0.33333333333 * tau * (1 - 0.25 * tau))); transcell = 1.0 - abscell; }
        for (int k = 0; k < nst; ++k) {
          if (tau <= 2.0) {
            if (ext == 0.0) src[k] = 0.0;
            else src[k] = (0.5 * (srcext0[k] + srcext1[k]) + 0.08333333333 * (ext0 * srcext1[k] - ext1 * srcext0[k]) * so) / ext;
          } else {
            double ext0p = ext0, srcext0p = srcext0[k];
            if (tau > 4.0) { ext0p = ext1 + (ext0 - ext1) * 4.0 / tau; if (ext0 > 0.0) srcext0p = srcext0[k] * ext0p / ext0; }
            src[k] = 1.0 / (ext0p + ext1) * (srcext0p + srcext1[k] + (ext0p * srcext1[k] - ext1 * srcext0p) * 2.0 / (ext0p + ext1) * (1 - 2 / tau + 2 * transcell / abscell));
          }
        }
        src[0] = std::max(src[0], 0.0);
        if (gridrad[(size_t)i1 * nst] >= -0.1) {
          validrad = true;
          for (int k = 0; k < nst; ++k) rad[k] += transmit * (gridrad[(size_t)i1 * nst + k] * transcell + src[k] * abscell);
        } else {
          for (int k = 0; k < nst; ++k) { rad[k] += transmit * src[k] * abscell; srcext1[k] = srcext0[k]; }
          transmit *= transcell; ext1 = ext0; icell = inext;
        }
      }
      for (int k = 0; k < nst; ++k) gridrad[(size_t)ipt * nst + k] = (R)rad[k];
    }
    return true;
  }

  // PATH_INTEGRATION (src/polarized/shdomsub1.f:1836-2167), Lambertian.
  bool path_integration() {
    if (!sweep_ready) sweeping_order();
    std::fill(fluxes.begin(), fluxes.end(), (R)0);
    std::vector<R> gridrad((size_t)npts * nst, (R)0);
    for (int i = 0; i < npts; ++i) gridrad[(size_t)i * nst] = -1;
    radiance.assign((size_t)npts * nlm * nst, 0);
    std::vector<R> work((size_t)npts * nphi0max * nst, 0);
    auto W = [&](int i, int k, int s) -> R & { return work[((size_t)i * nphi0max + k) * nst + s]; };
    const int ndown = nang / 2;
    if (brdf) bcdown.assign(botp.size() * ndown * nst, 0);
    int jang = 0;
    std::vector<R> rb(nst);
    for (int imu = 0; imu < nmu; ++imu) {
      if (imu == nmu / 2 && !brdf) lambertian_boundary();
      if (nst == 3) sh_to_do_pol(imu, work); else sh_to_do(imu, work);
      // the discrete-ordinate I source is made non-negative
      for (int i = 0; i < npts; ++i)
        for (int k = 0; k < nphi0[imu]; ++k) W(i, k, 0) = std::max((R)0, W(i, k, 0));
      for (int iphi = 0; iphi < nphi0[imu]; ++iphi) {
        int iupdown;
        // boundary radiances: unpolarized (Q = U = 0) sky and Lambertian surface
        if (mu[imu] < 0) {
          iupdown = 0;
          for (int t : topp) { gridrad[(size_t)t * nst] = (R)skyrad_bc; for (int s = 1; s < nst; ++s) gridrad[(size_t)t * nst + s] = 0; }
        } else {
          iupdown = 1;
          for (size_t b = 0; b < botp.size(); ++b) {
            if (brdf) {  // reflection of the stored downwelling radiances for this ordinate
              variable_brdf(b, mu[imu], phi[(size_t)imu * nphi0max + iphi], rb.data());
              for (int s = 0; s < nst; ++s) gridrad[(size_t)botp[b] * nst + s] = rb[s];
              continue;
            }
            gridrad[(size_t)botp[b] * nst] = bcrad_bot[b];
            for (int s = 1; s < nst; ++s) gridrad[(size_t)botp[b] * nst + s] = 0;
          }
        }
        bool ok;
        if ((ipflag & 2) && (ipflag & 1)) ok = back_int_grid1d(mu[imu], iphi, work, gridrad);
        else ok = back_int_grid3d(mu[imu], phi[(size_t)imu * nphi0max + iphi], iphi, work, gridrad);
        if (!ok) return false;
        for (int i = 0; i < npts; ++i) {
          if (gridrad[(size_t)i * nst] < (R)-0.0001) { err = "PATH_INTEGRATION: Grid point has no value"; return false; }
          for (int s = 0; s < nst; ++s) W(i, iphi, s) = gridrad[(size_t)i * nst + s];
          gridrad[(size_t)i * nst] = -1;
        }
        R a = std::fabs((R)mu[imu]) * (R)wtdo[(size_t)imu * nphi0max + iphi];
        for (int i = 0; i < npts; ++i) fluxes[2 * (size_t)i + iupdown] += a * W(i, iphi, 0);
        if (brdf && mu[imu] < 0) {  // keep the downwelling radiance at the surface
          for (size_t b = 0; b < botp.size(); ++b)
            for (int s = 0; s < nst; ++s) bcdown[(b * ndown + jang) * nst + s] = W(botp[b], iphi, s);
          ++jang;
        }
      }
      if (nst == 3) do_to_sh_pol(imu, work); else do_to_sh(imu, work);
    }
    return true;
  }

  // CALC_ACCEL_SOLCRIT (src/shdom_nompi.f:317-348) and ACCELERATE_SOLUTION
  // (src/polarized/shdomsub1.f:1807-1831).
  void accel_solcrit() {
    R accelpar;
    if (p.accelflag && accel_a == 0 && deljnew < deljold) {
      R r = std::sqrt(deljnew / deljold);
      R theta = std::acos(deljdot / std::sqrt(deljold * deljnew));
      R a = ((R)1 - r * std::cos(theta) + std::pow(r, (R)1 + (R)0.5 * (R)3.14159 / theta)) /
                ((R)1 + r * r - (R)2 * r * std::cos(theta)) - (R)1;
      accel_a = std::min((R)10, std::max((R)0, a));
    } else {
      accel_a = 0;
    }
    accelpar = accel_a;
    if (jnorm > 0) solcrit = std::sqrt(deljnew / jnorm);
    else if (deljnew == 0) solcrit = 0;
    if (accelpar > 0) {
      for (int i = 0; i < npts; ++i) {
        int is = shptr[i], ns = shptr[i + 1] - is, isd = oshptr[i], nsd = oshptr[i + 1] - isd;
        int nsc = std::min(ns, nsd);
        for (int t = 0; t < nsc * nst; ++t) source[(size_t)is * nst + t] += accelpar * delsource[(size_t)isd * nst + t];
      }
    }
  }

  // ------------------------------------------------------ adaptive grid
  // Every per-point array grown to n points (gridpos may already be); the
  // species-major arrays ([npart][npts]) are laid out again with the new
  // stride.  The SH pointers of the new points are set by interpolate_point.
  void grow_points(int n) {
    const int old = npts;
    auto relayout = [&](auto &v, size_t per) {
      typename std::decay<decltype(v)>::type nv((size_t)npart * n * per);
      for (int ipa = 0; ipa < npart; ++ipa)
        std::copy(v.begin() + (size_t)ipa * old * per, v.begin() + ((size_t)ipa * old + old) * per,
                  nv.begin() + (size_t)ipa * n * per);
      v.swap(nv);
    };
    relayout(extinct, 1); relayout(albedo, 1); relayout(iphase, nq); relayout(phaseinterpwt, nq);
    total_ext.resize(n, 0); dirflux.resize(n, 0); planck_tot.resize(n, 0);
    if (!temp.empty()) temp.resize(n, 0.f);
    gridpos.resize((size_t)3 * n);
    fluxes.resize((size_t)2 * n, 0);
    shptr.resize(n + 1, shptr[old]);
    oshptr.resize(n + 1, oshptr[old]);
    rshptr.resize(n + 2, rshptr[old]);
    // room for every point's full SH series (COMPUTE_SOURCE truncates in place)
    const size_t full = (size_t)n * nlm * nst;
    if (source.size() < full) source.resize(full, 0);
    if (p.accelflag && delsource.size() < full) delsource.resize(full, 0);
    npts = n;
  }

  // CELL_SPLIT_TEST (src/polarized/shdomsub1.f:5702-5791): for each axis the
  // mean over the four edges across it of |delta(ext J)| rms over angles
  // (from the SH terms of the I source) / ext x (1 - exp(-tau)); the largest
  // and its axis (1 X, 2 Y, 3 Z).
  void cell_split_test(int icell, float &maxadapt, int &idir) const {
    static const int gc[3][4][2] = {{{0, 1}, {2, 3}, {4, 5}, {6, 7}}, {{0, 2}, {1, 3}, {4, 6}, {5, 7}},
                                    {{0, 4}, {1, 5}, {2, 6}, {3, 7}}};
    const float c0 = 0.282095f;
    maxadapt = -1.0f; idir = 0;
    for (int id = 0; id < 3; ++id) {
      float sum1 = 0.0f;
      int num = 0;
      for (int ie = 0; ie < 4; ++ie) {
        const int ip1 = gridptr[8 * icell + gc[id][ie][0]], ip2 = gridptr[8 * icell + gc[id][ie][1]];
        if (ip1 == ip2) continue;
        ++num;
        const int is1 = shptr[ip1], is2 = shptr[ip2], ns1 = shptr[ip1 + 1] - is1, ns2 = shptr[ip2 + 1] - is2;
        const int ns = std::min(ns1, ns2);
        const float e1 = (float)total_ext[ip1], e2 = (float)total_ext[ip2];
        auto S = [&](int is, int j) { return (float)source[(size_t)(is + j) * nst]; };
        float jay = 0.0f;
        for (int j = 0; j < ns; ++j) { float d = e2 * S(is2, j) - e1 * S(is1, j); jay += d * d; }
        for (int j = ns; j < ns1; ++j) { float d = e1 * S(is1, j); jay += d * d; }
        for (int j = ns; j < ns2; ++j) { float d = e2 * S(is2, j); jay += d * d; }
        const float ext = 0.5f * (e1 + e2);
        jay = ext > 0.0f ? c0 * std::sqrt(jay) / ext : 0.0f;
        const float tau = std::fabs(ext * (gridpos[3 * ip2 + id] - gridpos[3 * ip1 + id]));
        sum1 += std::fabs(jay) * (1.0f - std::exp(-tau));
      }
      const float crit = num > 0 ? sum1 / (float)num : 0.0f;
      if (crit > maxadapt) { maxadapt = crit; idir = id + 1; }
    }
  }

  // MATCH_GRID_POINT (src/polarized/shdomsub1.f:5599-5700): an existing grid
  // point at (xp, yp, zp) on the cells across face iface of icell, or -1.
  int match_grid_point(float xp, float yp, float zp, int icell, int iface) const {
    const int idir = iface / 2 + 1, kface = kOppFace[iface];
    int ic = nb_cell(neighptr[6 * icell + iface]);
    if (ic < 0) return -1;
    const float pos[3] = {xp, yp, zp};
    std::vector<int> stack;
    while (true) {
      while (treeptr[2 * ic + 1] == 0) {
        for (int i = 0; i < 4; ++i) {
          const int ipt = gridptr[8 * ic + kGridFace[kface][i]];
          if (xp == gridpos[3 * ipt] && yp == gridpos[3 * ipt + 1] && zp == gridpos[3 * ipt + 2]) return ipt;
        }
        if (stack.empty()) return -1;
        ic = stack.back();
        stack.pop_back();
      }
      const int dir = split_dir(ic), ic1 = treeptr[2 * ic + 1];
      if (dir == idir) { ic = ic1 + 1 - (iface % 2); continue; }
      // a split across the face: follow the child holding the point, both when
      // the point is on the split line
      const float c = gridpos[3 * gridptr[8 * ic1 + 7] + dir - 1];
      ic = ic1;
      if (pos[dir - 1] == c) stack.push_back(ic1 + 1);
      else if (pos[dir - 1] > c) ic = ic1 + 1;
    }
  }

  // INHERIT_NEIGHBOR (src/polarized/shdomsub1.f:5454-5507): icell and every
  // descendant bordering face iface get neighbour `in`.
  void inherit_neighbor(int icell, int iface, int in) {
    const int jface = iface / 2 + 1;
    std::vector<int> stack;
    int ic = icell;
    while (true) {
      neighptr[6 * ic + iface] = in;
      if (treeptr[2 * ic + 1] == 0) {
        if (stack.empty()) return;
        ic = stack.back();
        stack.pop_back();
      } else if (split_dir(ic) == jface) {
        ic = treeptr[2 * ic + 1] + (iface % 2);
      } else {
        stack.push_back(treeptr[2 * ic + 1] + 1);
        ic = treeptr[2 * ic + 1];
      }
    }
  }

  // MATCH_NEIGHBOR_FACE (src/polarized/shdomsub1.f:5371-5451): the neighbour
  // pointer of new cell ic across face iface, and those of the cells on the
  // other side, from the sizes of the faces down the neighbour's tree.
  void match_neighbor_face(int iface, int ic) {
    int in = nb_cell(neighptr[6 * ic + iface]);
    if (in < 0) return;
    const int jface = iface / 2 + 1, dir1 = jface % 3 + 1, dir2 = (jface + 1) % 3 + 1;
    const int ic1 = gridptr[8 * ic], ic8 = gridptr[8 * ic + 7];
    auto G = [&](int ip, int d) { return gridpos[3 * ip + d - 1]; };
    float pos[3] = {0, 0, 0};
    pos[dir1 - 1] = (G(ic1, dir1) + G(ic8, dir1)) / 2;
    pos[dir2 - 1] = (G(ic1, dir2) + G(ic8, dir2)) / 2;
    bool done = false;
    while (!done && ic != in) {
      const int in1 = gridptr[8 * in], in8 = gridptr[8 * in + 7];
      if (G(ic1, dir1) >= G(in1, dir1) && G(ic8, dir1) <= G(in8, dir1) && G(ic1, dir2) >= G(in1, dir2) &&
          G(ic8, dir2) <= G(in8, dir2))
        neighptr[6 * ic + iface] = treeptr[2 * in + 1] == 0 ? in : nb_parent(in);
      if (G(in1, dir1) >= G(ic1, dir1) && G(in8, dir1) <= G(ic8, dir1) && G(in1, dir2) >= G(ic1, dir2) &&
          G(in8, dir2) <= G(ic8, dir2)) {
        inherit_neighbor(in, kOppFace[iface], ic);
      } else {
        int &w = neighptr[6 * in + kOppFace[iface]];
        if (w != -1) w = nb_parent(nb_cell(w));
      }
      if (treeptr[2 * in + 1] == 0) done = true;
      else {
        const int dir = split_dir(in), inn = treeptr[2 * in + 1];
        if (dir == jface) in = inn + 1 - (iface % 2);
        else in = pos[dir - 1] > G(gridptr[8 * inn + 7], dir) ? inn + 1 : inn;
      }
    }
  }

  // NEW_GRID_POINTS (src/polarized/shdomsub1.f:5509-5597): the corner
  // pointers of the two children, with a point at the middle of each of the
  // four edges along the split unless a neighbour already has one there.
  // newp[i] = {parent point 1, parent point 2, new point or -1}.
  void new_grid_points(int idir, int icell, int nc, int newp[4][3], int &nnew) {
    static const int gc[3][4][2] = {{{0, 1}, {2, 3}, {4, 5}, {6, 7}}, {{0, 2}, {1, 3}, {4, 6}, {5, 7}},
                                    {{0, 4}, {1, 5}, {2, 6}, {3, 7}}};
    static const int fg[3][4][2] = {{{2, 4}, {3, 4}, {2, 5}, {3, 5}}, {{0, 4}, {1, 4}, {0, 5}, {1, 5}},
                                    {{0, 2}, {1, 2}, {0, 3}, {1, 3}}};
    for (int k = 0; k < 8; ++k) gridptr[8 * nc + k] = gridptr[8 * (nc + 1) + k] = gridptr[8 * icell + k];
    for (int i = 0; i < 4; ++i) {
      const int i1 = gc[idir - 1][i][0], i2 = gc[idir - 1][i][1];
      const int ip1 = gridptr[8 * icell + i1], ip2 = gridptr[8 * icell + i2];
      const float xp = (gridpos[3 * ip1] + gridpos[3 * ip2]) / 2, yp = (gridpos[3 * ip1 + 1] + gridpos[3 * ip2 + 1]) / 2,
                  zp = (gridpos[3 * ip1 + 2] + gridpos[3 * ip2 + 2]) / 2;
      const int f1 = fg[idir - 1][i][0], f2 = fg[idir - 1][i][1];
      int ipm = match_grid_point(xp, yp, zp, icell, f1);
      if (ipm < 0) ipm = match_grid_point(xp, yp, zp, icell, f2);
      if (ipm < 0) {
        const int icell2 = nb_cell(neighptr[6 * icell + f1]);
        if (icell2 >= 0) ipm = match_grid_point(xp, yp, zp, icell2, f2);
      }
      if (ipm < 0) {
        const int ip = (int)(gridpos.size() / 3);
        gridpos.push_back(xp); gridpos.push_back(yp); gridpos.push_back(zp);
        gridptr[8 * nc + i2] = ip; gridptr[8 * (nc + 1) + i1] = ip;
        newp[i][0] = ip1; newp[i][1] = ip2; newp[i][2] = ip;
        ++nnew;
      } else {
        gridptr[8 * nc + i2] = ipm; gridptr[8 * (nc + 1) + i1] = ipm;
        newp[i][2] = -1;
      }
    }
  }

  // DIVIDE_CELL (src/polarized/shdomsub1.f:5286-5368): end cell icell split
  // in two along idir; the children are cells ncells and ncells + 1.
  void divide_cell(int icell, int idir, int newp[4][3], int &nnew) {
    const int nc = ncells;
    ncells += 2;
    treeptr.resize((size_t)2 * ncells, 0);
    gridptr.resize((size_t)8 * ncells, 0);
    neighptr.resize((size_t)6 * ncells, -1);
    cellflags.resize(ncells, 0);
    treeptr[2 * icell + 1] = nc;
    treeptr[2 * nc] = icell; treeptr[2 * nc + 1] = 0;
    treeptr[2 * (nc + 1)] = icell; treeptr[2 * (nc + 1) + 1] = 0;
    cellflags[icell] = (short)(cellflags[icell] | (idir << 2));
    cellflags[nc] = cellflags[nc + 1] = (short)(cellflags[icell] & 3);
    nnew = 0;
    new_grid_points(idir, icell, nc, newp, nnew);
    for (int iface = 0; iface < 6; ++iface) {
      const int v = neighptr[6 * icell + iface];
      if (v == icell) {
        neighptr[6 * nc + iface] = nc;
        neighptr[6 * (nc + 1) + iface] = nc + 1;
      } else if (iface == 2 * idir - 1) {
        neighptr[6 * nc + iface] = nc + 1;
        neighptr[6 * (nc + 1) + iface] = v;
      } else if (iface == 2 * idir - 2) {
        neighptr[6 * (nc + 1) + iface] = nc;
        neighptr[6 * nc + iface] = v;
      } else {
        neighptr[6 * nc + iface] = v;
        neighptr[6 * (nc + 1) + iface] = v;
      }
      match_neighbor_face(iface, nc);
      match_neighbor_face(iface, nc + 1);
    }
  }

  // GRID_SMOOTH_TEST (src/polarized/shdomsub1.f:5794-5902): the axis to split
  // icell along so that the grid stays smooth (finer cells on both sides, the
  // two opposite neighbours split alike, or a neighbour more than 2.5 times
  // finer where there is a source), 0 for none.
  int grid_smooth_test(int icell) const {
    static const int ec[3][2] = {{0, 1}, {0, 2}, {0, 4}};
    int idir = 0;
    float sizeratio = 1.0f;
    for (int id = 1; id <= 3; ++id) {
      const int ip1 = gridptr[8 * icell + ec[id - 1][0]], ip2 = gridptr[8 * icell + ec[id - 1][1]];
      if (ip1 == ip2) continue;
      const float cur = std::fabs(gridpos[3 * ip1 + id - 1] - gridpos[3 * ip2 + id - 1]);
      const float inv = 1.0f / cur;
      float gsize[2];
      int dirsplit[2];
      for (int j = 0; j < 2; ++j) {
        dirsplit[j] = 0;
        const int iface = 2 * (id - 1) + j;
        double xe = 0, ye = 0, ze = 0;
        for (int i = 0; i < 4; ++i) {
          const int ip = gridptr[8 * icell + kGridFace[iface][i]];
          xe += gridpos[3 * ip] * 0.25f; ye += gridpos[3 * ip + 1] * 0.25f; ze += gridpos[3 * ip + 2] * 0.25f;
        }
        const int inc = next_cell(xe, ye, ze, iface, id - 1, icell);
        if (inc < 0) gsize[j] = cur;
        else {
          gsize[j] = std::fabs(gridpos[3 * gridptr[8 * inc] + id - 1] - gridpos[3 * gridptr[8 * inc + 7] + id - 1]);
          if (treeptr[2 * inc] < 0) gsize[j] = cur;
          if (id <= 2 && ((cellflags[inc] >> (id - 1)) & 1)) gsize[j] = cur;
        }
        const int in = neighptr[6 * icell + iface];
        if (in <= -2) dirsplit[j] = split_dir(nb_cell(in));
      }
      if (gsize[0] * inv < 0.75f && gsize[1] * inv < 0.75f) idir = id;
      if (dirsplit[0] > 0 && dirsplit[0] != id && dirsplit[0] == dirsplit[1]) idir = dirsplit[0];
      const float ratio = std::min(gsize[0] * inv, gsize[1] * inv);
      if (ratio < 0.4f && ratio < sizeratio) {
        int isum = 0;
        for (int i = 0; i < 8; ++i) { const int ip = gridptr[8 * icell + i]; isum += shptr[ip + 1] - shptr[ip]; }
        if (isum > 0) { idir = id; sizeratio = ratio; }
      }
    }
    return idir;
  }

  // INTERPOLATE_POINT (src/polarized/shdomsub1.f:4934-5283): the medium of a
  // new point from the property grid, its direct beam, its radiance the mean
  // of its two parent points', and its source from that radiance.
  bool interpolate_point(int ip1, int ip2, int ip) {
    total_ext[ip] = 0;
    for (int ipa = 0; ipa < npart; ++ipa) {
      R e;
      if (!trilin_point(ipa, ip, e)) return false;
      if (p.deltam) deltam_point(ipa, ip);
      total_ext[ip] += extinct[(size_t)ipa * npts + ip];
    }
    if (srct != 'S') planck_point(ip);
    make_direct(ip, ip + 1);
    const int ir1 = rshptr[ip1], ir2 = rshptr[ip2], nr1 = rshptr[ip1 + 1] - ir1, nr2 = rshptr[ip2 + 1] - ir2;
    const int nr = std::max(nr1, nr2), ir = rshptr[ip];
    rshptr[ip + 1] = ir + nr;
    if (radiance.size() < (size_t)(ir + nr) * nst) radiance.resize((size_t)(ir + nr) * nst, 0);
    for (int j = 0; j < nr; ++j)
      for (int k = 0; k < nst; ++k) {
        const R r1 = j < nr1 ? radiance[(size_t)(ir1 + j) * nst + k] : (R)0;
        const R r2 = j < nr2 ? radiance[(size_t)(ir2 + j) * nst + k] : (R)0;
        radiance[(size_t)(ir + j) * nst + k] = (R)0.5 * (r1 + r2);
      }
    const int ns = std::max(shptr[ip1 + 1] - shptr[ip1], shptr[ip2 + 1] - shptr[ip2]), is = shptr[ip];
    shptr[ip + 1] = is + ns;
    if (p.accelflag) oshptr[ip + 1] = oshptr[ip];
    std::vector<R> sourcet, lt, lt1;
    point_source(ip, sourcet, radiance, ir, nr, lt, lt1);
    if (source.size() < (size_t)(is + ns) * nst) source.resize((size_t)(is + ns) * nst, 0);
    for (int t = 0; t < ns * nst; ++t) source[(size_t)is * nst + t] = sourcet[t];
    return true;
  }

  bool divide_and_interpolate(int icell, int idir) {
    int newp[4][3], nnew = 0;
    divide_cell(icell, idir, newp, nnew);
    if (nnew == 0) return true;
    grow_points(npts + nnew);
    for (int i = 0; i < 4; ++i)
      if (newp[i][2] >= 0 && !interpolate_point(newp[i][0], newp[i][1], newp[i][2])) return false;
    rshptr[npts + 1] = rshptr[npts];
    return true;
  }

  // SPLIT_GRID (src/polarized/shdomsub1.f:4703-4931): when dosplit, the end
  // cells are tested in batches (the cells split in one batch are tested in
  // the next), those above cursplitacc split in decreasing order of the
  // criterion while the memory limits allow, and the rest tested for grid
  // smoothness.  splitcrit: the largest criterion left after the divisions.
  bool split_grid(bool dosplit, float cursplit, float &splitcrit_out) {
    if (dosplit) {
      const long maxig = (long)(adapt_grid_factor * (float)nbpts);
      const long maxic = std::max((long)(cell_to_point_ratio * (float)maxig), (long)nbcells);
      const long maxiv = std::max((long)(num_sh_term_factor * (float)nlm * (float)maxig), (long)nbpts * 4);
      const long maxido = maxig * nphi0max;
      int icell1 = 0;
      bool outofmem0 = outofmem;
      while (icell1 < ncells) {
        std::vector<std::pair<float, int>> crit;
        for (int ic = icell1; ic < ncells; ++ic)
          if (treeptr[2 * ic + 1] == 0) {
            float c; int d;
            cell_split_test(ic, c, d);
            crit.push_back({c, 4 * ic + d});
          }
        icell1 = ncells;
        std::stable_sort(crit.begin(), crit.end(),
                         [](const std::pair<float, int> &a, const std::pair<float, int> &b) { return a.first > b.first; });
        const float frac = 0.03f;
        long maxcells = (long)(maxic - frac * (maxic - ncells) - 2);
        long maxpts = (long)(maxig - frac * (maxig - npts) - 4);
        long maxwork = (long)(maxido - frac * (maxido - (long)nphi0max * npts) - 4 * nphi0max);
        long maxsh = (long)(maxiv - frac * (maxiv - shptr[npts]) - 4 * nlm);
        long maxrad = (long)(maxiv + maxig - frac * (maxiv + maxig - rshptr[npts]) - 4 * nlm);
        auto full = [&]() {
          return ncells > maxcells || npts > maxpts || (long)npts * nphi0max > maxwork || shptr[npts] > maxsh ||
                 rshptr[npts] > maxrad;
        };
        outofmem0 = outofmem;
        size_t i = 0;
        while (i < crit.size() && crit[i].first > cursplit && !outofmem0) {
          if (full()) outofmem0 = true;
          else if (!divide_and_interpolate(crit[i].second / 4, crit[i].second & 3)) return false;
          ++i;
        }
        maxcells = maxic - 2; maxpts = maxig - 4; maxwork = maxido - 4 * nphi0max;
        maxsh = maxiv - 4 * nlm; maxrad = maxiv + maxig - 4 * nlm;
        while (!outofmem && i < crit.size()) {
          if (full()) outofmem = true;
          else {
            const int d = grid_smooth_test(crit[i].second / 4);
            if (d > 0 && !divide_and_interpolate(crit[i].second / 4, d)) return false;
          }
          ++i;
        }
      }
      if (outofmem0) outofmem = true;
      boundary_points();
      sweep_ready = false;
    }
    splitcrit_out = 0;
    for (int ic = 0; ic < ncells; ++ic)
      if (treeptr[2 * ic + 1] == 0) {
        float c; int d;
        cell_split_test(ic, c, d);
        splitcrit_out = std::max(splitcrit_out, c);
      }
    return true;
  }

  // SOLUTION_ITERATIONS (src/polarized/shdomsub1.f:445-818), with the
  // adaptive splitting schedule: splitting starts when the solution
  // criterion falls below 0.1, and the current splitting accuracy is lowered
  // from splitacc x 33.3 to splitacc as a geometric mean of the criterion
  // goes from 0.1 to 0.003 (all splitting stops below 0.001).
  bool solution_iterations(int maxiter, int verbose) {
    bool fixsh = false;
    const R endadaptsol = (R)0.001;
    const float splitacc = p.splitacc, startadapt = 0.1f, endadapt = 0.001f;
    const float adaptrange = startadapt / (3.0f * endadapt);
    float cursplit = splitacc * adaptrange, startsplit = cursplit, avgsolcrit = (float)solcrit, splitcrit = 0.0f;
    bool splittesting = true;
    while (iter < maxiter &&
           (solcrit > (R)p.solacc || (splitcrit > splitacc && cursplit > splitacc && !outofmem))) {
      ++iter;
      if (splitacc > 0.0f) {
        const float sc = (float)solcrit;
        avgsolcrit = std::sqrt(avgsolcrit * sc);
        const bool dosplit = sc <= startadapt && (sc > endadapt || cursplit > splitacc) && !outofmem;
        const float beta = std::log(startsplit / splitacc) / std::log(adaptrange);
        cursplit = std::min(cursplit, std::max(splitacc, splitacc * std::pow(avgsolcrit / (3.0f * endadapt), beta)));
        if (sc <= endadapt) cursplit = splitacc;
        if (splittesting) {
          if (!split_grid(dosplit, cursplit, splitcrit)) return false;
          if (sc > startadapt) startsplit = splitcrit;
        }
        if (sc <= endadapt) splittesting = false;
      }
      radiance_truncation(fixsh);
      if (!path_integration()) return false;
      if (solcrit < endadaptsol || iter > p.iterfixsh) fixsh = true;
      compute_source(fixsh, false);
      accel_solcrit();
      if (albmax < (R)p.solacc) solcrit = (R)p.solacc;
      if (verbose)
        std::printf("  %4d %8.3f %10.3e %8d %8.2f\n", iter, std::log10(std::max((double)solcrit, 1e-20)), (double)splitcrit,
                    npts, (double)shptr[npts] / npts);
    }
    return true;
  }

  // ---------------------------------------------------------- rendering
  // PRECOMPUTE_PHASE_CHECK (src/polarized/shdomsub4.f:2388-2491) on the
  // unscaled table (at3d/solver.py:2800-2825).
  int nscatangle = 0;
  std::vector<R> phasetab;   // [nscatangle][numphase]
  std::vector<R> phasetab2;  // [nscatangle][numphase] I-Q element (nst = 3)
  bool precompute_phase() {
    int nlegp = std::max(p.nlegp, nleg);
    nscatangle = std::max(36, std::min(721, 2 * nlegp));
    phasetab.assign((size_t)nscatangle * numphase, 0);
    if (nst == 3) phasetab2.assign((size_t)nscatangle * numphase, 0);
    std::vector<double> d2;
    const double pi = std::acos(-1.0), ofourpi = 1.0 / (4.0 * pi);
    std::vector<double> d;
    for (int j = 0; j < nscatangle; ++j) {
      double x = std::cos(pi * (double)j / (nscatangle - 1));
      // Legendre polynomials P_l(x) = d^l_{00}(x)
      d.assign(nlegp + 1, 0.0);
      d[0] = 1.0;
      if (nlegp >= 1) d[1] = x;
      for (int n = 1; n < nlegp; ++n) d[n + 1] = ((2 * n + 1) * x * d[n] - n * d[n - 1]) / (n + 1);
      for (int iph = 0; iph < numphase; ++iph) {
        double a1 = 0.0;
        for (int l = 0; l <= nlegp; ++l) {
          float lg = (l <= p.nlegp) ? leg_in(iph, l, 0) : 0.f;
          double unsc = (double)(float)(lg / (float)(2 * l + 1));
          a1 += (2.0 * l + 1.0) * unsc * d[l];
        }
        if (a1 <= 0.0) { err = "PRECOMPUTE_PHASE_CHECK: negative phase function"; return false; }
        phasetab[(size_t)j * numphase + iph] = (R)(a1 * ofourpi);
        if (nst == 3) {
          // B1 = -sum (2l+1) b1_l d^l_{20}(cos theta)
          if (iph == 0) wigner_d(x, nlegp, 2, 0, d2);
          double b1 = 0.0;
          for (int l = 0; l <= nlegp; ++l) {
            float lg = (l <= p.nlegp) ? leg_in(iph, l, 4) : 0.f;
            double unsc = (double)(float)(lg / (float)(2 * l + 1));
            b1 -= (2.0 * l + 1.0) * unsc * d2[l];
          }
          phasetab2[(size_t)j * numphase + iph] = (R)(b1 * ofourpi);
        }
      }
    }
    return true;
  }

  // LOCATE_GRID_CELL (src/polarized/shdomsub2.f:4043-4211), base grid.
  int locate_grid_cell(double &x0, double &y0, double z0) const {
    if (!(bcflag & 1)) {
      double xd = xgrid[nx] - xgrid[0];
      if (x0 < xgrid[0]) x0 = x0 - xd * ((int)((x0 - xgrid[0]) / xd) - 1);
      else if (x0 > xgrid[nx]) x0 = x0 - xd * (int)((x0 - xgrid[0]) / xd);
    }
    if (!(bcflag & 2)) {
      double yd = ygrid[ny] - ygrid[0];
      if (y0 < ygrid[0]) y0 = y0 - yd * ((int)((y0 - ygrid[0]) / yd) - 1);
      else if (y0 > ygrid[ny]) y0 = y0 - yd * (int)((y0 - ygrid[0]) / yd);
    }
    int il = 0, iu, ix, iy, iz;
    if (ipflag & 1) {
      iu = nx;
      while (iu - il > 1) { int im = (iu + il) / 2; if (x0 >= 0.5 * (xgrid[im - 1] + xgrid[im])) il = im; else iu = im; }
      il += 1;
    } else {
      iu = nx + 1;
      while (iu - il > 1) { int im = (iu + il) / 2; if (x0 >= xgrid[im - 1]) il = im; else iu = im; }
    }
    ix = std::max(il, 1);
    il = 0;
    if (ipflag & 2) {
      iu = ny;
      while (iu - il > 1) { int im = (iu + il) / 2; if (y0 >= 0.5 * (ygrid[im - 1] + ygrid[im])) il = im; else iu = im; }
      il += 1;
    } else {
      iu = ny + 1;
      while (iu - il > 1) { int im = (iu + il) / 2; if (y0 >= ygrid[im - 1]) il = im; else iu = im; }
    }
    iy = std::max(il, 1);
    il = 0; iu = nz;
    while (iu - il > 1) { int im = (iu + il) / 2; if (z0 >= zgrid[im - 1]) il = im; else iu = im; }
    iz = std::max(il, 1);
    int nxc = nx, nyc = ny;
    if (bcflag & 1) {
      nxc = nx + 1;
      if (x0 < xgrid[0]) ix = 1; else if (x0 > xgrid[nx - 1]) ix = nx + 1; else ix = ix + 1;
    }
    if (bcflag & 2) {
      nyc = ny + 1;
      if (y0 < ygrid[0]) iy = 1; else if (y0 > ygrid[ny - 1]) iy = ny + 1; else iy = iy + 1;
    }
    int icell = (iz - 1) + (nz - 1) * (iy - 1) + (nz - 1) * nyc * (ix - 1);
    // down the tree to the end cell that holds the point
    const double pos[3] = {x0, y0, z0};
    while (treeptr[2 * icell + 1] > 0) {
      int dir = split_dir(icell), c = treeptr[2 * icell + 1] + 1;
      if (pos[dir - 1] < gridpos[3 * gridptr[8 * c] + dir - 1]) c -= 1;
      icell = c;
    }
    return icell;
  }

  // INTEGRATE_1RAY + COMPUTE_SOURCE_1CELL_UNPOL + FIND_BOUNDARY_RADIANCE
  // (src/polarized/shdomsub2.f:2311-2863, :3046-3192); with nst = 3 the
  // polarized COMPUTE_SOURCE_1CELL (src/polarized/shdomsub2.f:2868-3042) and
  // ROTATE_POL_PLANE (src/polarized/shdomsub2.f:3277-3316).  radout[nst].
  bool integrate_1ray(double mu2, double phi2, double x0, double y0, double z0, double *radout,
                      std::string &err) const {
    const double pi = std::acos(-1.0);
    double eps = 1.0e-5 * (gridpos[3 * gridptr[7] + 2] - gridpos[3 * gridptr[0] + 2]);
    int maxcellscross = 500 * std::max(nx, std::max(ny, nz));
    std::vector<R> ylmdir, y6;  // y6 [nlm][6] generalized functions when nst = 3
    if (nst == 3) {
      std::vector<double> yd;
      genylm6(false, (double)(float)mu2, (double)(float)phi2, true, ml, mm, yd);
      y6.assign(yd.size(), 0);
      for (size_t q = 0; q < yd.size(); ++q) y6[q] = (R)yd[q];
      ylmdir.resize(nlm);
      for (int j = 0; j < nlm; ++j) ylmdir[j] = y6[(size_t)j * 6];
    } else {
      ylmdir = ylmall((double)(float)mu2, (float)phi2);
    }
    std::vector<R> singscat((size_t)numphase * nst, 0);  // [numphase][nst]
    bool tms = p.deltam;
    if (tms) {
      double cosscat = (double)p.solarmu * mu2 +
                       std::sqrt((1.0 - (double)p.solarmu * p.solarmu) * (1.0 - mu2 * mu2)) * std::cos((double)p.solaraz - phi2);
      cosscat = std::max(std::min(1.0, cosscat), -1.0);
      float F = (float)((nscatangle - 1) * (std::acos(cosscat) / pi) + 1);
      int J = std::min(nscatangle - 1, (int)F);
      F = F - J;
      for (int i = 0; i < numphase; ++i) {
        singscat[(size_t)i * nst] = (R)((1 - F) * phasetab[(size_t)(J - 1) * numphase + i] + F * phasetab[(size_t)J * numphase + i]);
        if (nst == 3) {
          // I-Q element, then the polarization plane turned from the
          // scattering plane to the outgoing meridional plane
          const float b1 = (float)((1 - F) * phasetab2[(size_t)(J - 1) * numphase + i] + F * phasetab2[(size_t)J * numphase + i]);
          const float smu = p.solarmu, mu2f = (float)mu2, dphi = p.solaraz - (float)phi2;
          const double sin_scat = std::sqrt(std::max(0.0, 1.0 - cosscat * cosscat));
          const double st1 = std::sqrt(1.0 - (double)(smu * smu)), st2 = std::sqrt(1.0 - (double)(mu2f * mu2f));
          const double sp = std::sin((double)dphi), cp = std::cos((double)dphi);
          double sin2, cos2;
          if (sin_scat == 0.0) { sin2 = 0.0; cos2 = -1.0; }
          else { sin2 = st1 * sp / sin_scat; cos2 = (st2 * smu - st1 * mu2f * cp) / sin_scat; }
          const double sin22 = 2.0 * sin2 * cos2, cos22 = 1.0 - 2.0 * sin2 * sin2;
          singscat[(size_t)i * 3 + 1] = (R)(float)(b1 * cos22);
          singscat[(size_t)i * 3 + 2] = (R)(float)(b1 * sin22);
        }
      }
    }
    double cx = std::sqrt(1.0 - mu2 * mu2) * std::cos(phi2 - pi), cy = std::sqrt(1.0 - mu2 * mu2) * std::sin(phi2 - pi);
    double cz = -mu2, cxinv, cyinv, czinv;
    if (std::fabs(cx) > 1e-6) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1e6; }
    if (std::fabs(cy) > 1e-6) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1e6; }
    if (std::fabs(cz) > 1e-6) czinv = 1.0 / cz; else { cz = 0; czinv = 1e6; }
    int bitx = cx < 0, bity = cy < 0, bitz = cz < 0;
    int ioct = 1 + bitx + 2 * bity + 4 * bitz;
    float xm = 0.5f * (xgrid[0] + xgrid[nx - 1]), ym = 0.5f * (ygrid[0] + ygrid[ny - 1]);
    double xe = x0, ye = y0, ze = z0;
    int icell = locate_grid_cell(xe, ye, ze);
    int iface = -1, ngrid = 0;
    double transmit = 1.0, radiance_acc[3] = {0.0, 0.0, 0.0};
    R extinct8[8] = {0, 0, 0, 0, 0, 0, 0, 0}, srcext8[3][8] = {{0}};
    int oldipts[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    bool validrad = false;
    double ext1 = 0, srcext1[3] = {0, 0, 0};
    const R secmu0 = (R)1 / std::fabs((R)p.solarmu);
    std::vector<R> lt; R fdum;
    // DONEFACE(8,7): which corner of the previous cell is reused (1-based, 0 none)
    static const int doneface[7][8] = {{0, 0, 0, 0, 0, 0, 0, 0}, {0, 1, 0, 3, 0, 5, 0, 7}, {2, 0, 4, 0, 6, 0, 8, 0},
                                       {0, 0, 1, 2, 0, 0, 5, 6}, {3, 4, 0, 0, 7, 8, 0, 0}, {0, 0, 0, 0, 1, 2, 3, 4},
                                       {5, 6, 7, 8, 0, 0, 0, 0}};
    while (!validrad && icell >= 0) {
      ++ngrid;
      R oext8[8], osrc8[3][8];
      for (int i = 0; i < 8; ++i) { oext8[i] = extinct8[i]; for (int k = 0; k < 3; ++k) osrc8[k][i] = srcext8[k][i]; }
      for (int n = 0; n < 8; ++n) {
        int ip = gridptr[8 * icell + n];
        int I = doneface[iface + 1][n];
        if (I > 0 && ip == oldipts[n]) {
          extinct8[n] = oext8[I - 1];
          for (int k = 0; k < nst; ++k) srcext8[k][n] = osrc8[k][I - 1];
          continue;
        }
        R ext = total_ext[ip];
        oldipts[n] = ip;
        // with SINGLESCATTER neither the harmonic source nor its truncated single scatter enters
        int is = shptr[ip], ns = rsingle ? 0 : shptr[ip + 1] - is;
        if (nst == 3) {
          R sv[3];
          source_1cell_pol(ip, ns, is, ext, y6, singscat, secmu0, sv);
          for (int k = 0; k < 3; ++k) srcext8[k][n] = sv[k] * ext;
          extinct8[n] = ext;
          continue;
        }
        R s = 0;
        for (int j = 0; j < ns; ++j) s += source[(size_t)is + j] * ylmdir[j];
        if (tms) {
          for (int ipa = 0; ipa < npart; ++ipa) {
            R w = (ext == 0) ? (R)1 : extinct[(size_t)ipa * npts + ip] / ext;
            if (w == 0) continue;
            point_legen(ip, ipa, lt, fdum);
            R f = fdum;
            R da = albedo[(size_t)ipa * npts + ip] * dirflux[ip] * secmu0 * w;
            int J = 0;
            for (int l = 0; l <= ml; ++l) {
              int me = std::min(l, mm);
              R a1 = da * lt[l];
              if (J < ns) {
                for (int m = -me; m <= me; ++m) { s = s - a1 * ylmdir[J] * ylmsun[J]; ++J; }
              }
            }
            const int *IPH = &iphase[((size_t)ipa * npts + ip) * nq];
            const R *PW = &phaseinterpwt[((size_t)ipa * npts + ip) * nq];
            if (PW[0] >= phasemax) s = s + da * singscat[IPH[0] - 1] / ((R)1 - f);
            else
              for (int q = 0; q < nq; ++q) {
                if (PW[q] <= (R)1e-5) continue;
                s = s + da * singscat[IPH[q] - 1] * PW[q] / ((R)1 - f);
              }
          }
        }
        srcext8[0][n] = s * ext;
        extinct8[n] = ext;
      }
      int ipt1 = gridptr[8 * icell], ipt2 = gridptr[8 * icell + 7];
      double delx = gridpos[3 * ipt2] - gridpos[3 * ipt1], dely = gridpos[3 * ipt2 + 1] - gridpos[3 * ipt1 + 1];
      double delz = gridpos[3 * ipt2 + 2] - gridpos[3 * ipt1 + 2];
      double invdelx = delx <= 0 ? 1.0 : 1.0 / delx, invdely = dely <= 0 ? 1.0 : 1.0 / dely, invdelz = 1.0 / delz;
      auto interp = [&](const R *a, double u, double v, double w) {
        return (R)((1 - w) * ((1 - v) * ((1 - u) * a[0] + u * a[1]) + v * ((1 - u) * a[2] + u * a[3])) +
                   w * ((1 - v) * ((1 - u) * a[4] + u * a[5]) + v * ((1 - u) * a[6] + u * a[7])));
      };
      double u = (xe - gridpos[3 * ipt1]) * invdelx, v = (ye - gridpos[3 * ipt1 + 1]) * invdely,
             w = (ze - gridpos[3 * ipt1 + 2]) * invdelz;
      for (int k = 0; k < nst; ++k) srcext1[k] = interp(srcext8[k], u, v, w);
      srcext1[0] = std::max(0.0, srcext1[0]);
      ext1 = interp(extinct8, u, v, w);
      bool ipinx = (cellflags[icell] & 1) && !((bcflag & 1) && ((cx > 0 && xe < xm) || (cx < 0 && xe > xm)));
      bool ipiny = (cellflags[icell] & 2) && !((bcflag & 2) && ((cy > 0 && ye < ym) || (cy < 0 && ye > ym)));
      int iopp = gridptr[8 * icell + (8 - ioct)];
      double sox = ipinx ? 1e20 : (gridpos[3 * iopp] - xe) * cxinv;
      double soy = ipiny ? 1e20 : (gridpos[3 * iopp + 1] - ye) * cyinv;
      double soz = (gridpos[3 * iopp + 2] - ze) * czinv;
      double so = std::min(sox, std::min(soy, soz));
      if (so < -eps) { err = "INTEGRATE_1RAY: SO<0"; return false; }
      double xn = xe + so * cx, yn = ye + so * cy, zn = ze + so * cz;
      u = (xn - gridpos[3 * ipt1]) * invdelx; v = (yn - gridpos[3 * ipt1 + 1]) * invdely; w = (zn - gridpos[3 * ipt1 + 2]) * invdelz;
      R extn = interp(extinct8, u, v, w);
      double taugrid = so * 0.5 * (ext1 + extn);
      int ntau = std::max(1, 1 + (int)(taugrid / p.tautol));
      double dels = so / ntau;
      for (int it = 1; it <= ntau; ++it) {
        double s = it * dels;
        double xi = xe + s * cx, yi = ye + s * cy, zi = ze + s * cz;
        u = (xi - gridpos[3 * ipt1]) * invdelx; v = (yi - gridpos[3 * ipt1 + 1]) * invdely; w = (zi - gridpos[3 * ipt1 + 2]) * invdelz;
        R ext0 = interp(extinct8, u, v, w);
        R srcext0[3];
        for (int k = 0; k < nst; ++k) srcext0[k] = interp(srcext8[k], u, v, w);
        srcext0[0] = std::max((R)0, srcext0[0]);
        double ext = 0.5 * (ext0 + ext1), tau, abscell, transcell;
        if (ext != 0.0) {
          tau = ext * dels;
          abscell = tau * (1.0 - 0.5 * tau * (1.0 - 0.33333333333 * tau));
          transcell = 1.0 - abscell;
        } else { abscell = 0; transcell = 1; }
        for (int k = 0; k < nst; ++k) {
          double src = 0.0;
          if (ext != 0.0)
            src = (0.5 * (srcext0[k] + srcext1[k]) + 0.08333333333 * (ext0 * srcext1[k] - ext1 * srcext0[k]) * dels * (1.0 - 0.05 * (ext1 - ext0) * dels)) / ext;
          radiance_acc[k] += transmit * src * abscell;
          srcext1[k] = srcext0[k];
        }
        transmit *= transcell;
        ext1 = ext0;
      }
      int jface; bool openbcface;
      if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; openbcface = (cellflags[icell] & 1) && (bcflag & 1); }
      else if (soy <= soz) { iface = 3 - bity; jface = 1; openbcface = (cellflags[icell] & 2) && (bcflag & 2); }
      else { iface = 5 - bitz; jface = 2; openbcface = false; }
      const int nbv = neighptr[6 * icell + iface];
      int inext = nbv >= -1 ? nbv : next_cell(xn, yn, zn, iface, jface, icell);
      int kface, ic;
      if (nbv >= -1 && !openbcface) { kface = iface; ic = icell; }
      else { kface = kOppFace[iface]; ic = inext; iface = -1; }
      if (inext >= 0) {
        if (jface == 0) xn = gridpos[3 * gridptr[8 * inext + ioct - 1]];
        else if (jface == 1) yn = gridpos[3 * gridptr[8 * inext + ioct - 1] + 1];
        else zn = gridpos[3 * gridptr[8 * inext + ioct - 1] + 2];
      }
      if (transmit < p.transcut || ngrid > maxcellscross) validrad = true;
      else if (inext < 0 && iface >= 4) {
        validrad = true;
        // FIND_BOUNDARY_RADIANCE, zero surface emission source
        double xs[4], ys[4], rb[4], rq[4] = {0, 0, 0, 0}, ru[4] = {0, 0, 0, 0};
        for (int jj = 0; jj < 4; ++jj) {
          int ipb = gridptr[8 * ic + kGridFace[kface][jj]];
          xs[jj] = gridpos[3 * ipb]; ys[jj] = gridpos[3 * ipb + 1];
          if ((float)mu2 < 0.0f) {
            rb[jj] = skyrad_bc;  // isotropic sky radiance at the top boundary
            if (std::find(topp.begin(), topp.end(), ipb) == topp.end()) { err = "FIND_BOUNDARY_RADIANCE: Not at boundary"; return false; }
          } else {
            auto itb = std::lower_bound(botp.begin(), botp.end(), ipb);
            if (itb == botp.end() || *itb != ipb) { err = "FIND_BOUNDARY_RADIANCE: Not at boundary"; return false; }
            if (brdf) {
              R o[3];
              variable_brdf(itb - botp.begin(), (float)mu2, (float)phi2, o);
              rb[jj] = o[0];
              if (nst == 3) { rq[jj] = o[1]; ru[jj] = o[2]; }
            } else {
              rb[jj] = bcrad_bot[itb - botp.begin()];
            }
          }
        }
        float uu = (xs[1] - xs[0] > 0) ? (float)((xn - xs[0]) / (xs[1] - xs[0])) : 0.f;
        float vv = (ys[2] - ys[0] > 0) ? (float)((yn - ys[0]) / (ys[2] - ys[0])) : 0.f;
        float radbnd = (1 - uu) * (1 - vv) * (float)rb[0] + uu * (1 - vv) * (float)rb[1] + (1 - uu) * vv * (float)rb[2] + uu * vv * (float)rb[3];
        if (!rnosfc) radiance_acc[0] += transmit * radbnd;
        if (!rnosfc && nst == 3 && brdf && (float)mu2 >= 0.0f) {  // a polarizing surface
          const double w1 = (1 - uu) * (1 - vv), w2 = uu * (1 - vv), w3 = (1 - uu) * vv, w4 = uu * vv;
          radiance_acc[1] += transmit * (float)(w1 * rq[0] + w2 * rq[1] + w3 * rq[2] + w4 * rq[3]);
          radiance_acc[2] += transmit * (float)(w1 * ru[0] + w2 * ru[1] + w3 * ru[2] + w4 * ru[3]);
        }
      } else {
        icell = inext;
      }
      xe = xn; ye = yn; ze = zn;
    }
    for (int k = 0; k < nst; ++k) radout[k] = radiance_acc[k];
    return true;
  }

  // Polarized COMPUTE_SOURCE_1CELL at one grid point (src/polarized/
  // shdomsub2.f:2868-3042): the Stokes source in the ray direction from the
  // generalized SH series, with the TMS single-scatter correction.
  void source_1cell_pol(int ip, int ns, int is, R ext, const std::vector<R> &y6, const std::vector<R> &singscat,
                        R secmu0, R *sv) const {
    sv[0] = sv[1] = sv[2] = 0;
    const R *S = &source[(size_t)is * 3];
    for (int j = 0; j < ns; ++j) sv[0] += S[3 * j] * y6[(size_t)j * 6];
    for (int j = 0; j < ns; ++j) {
      sv[1] += S[3 * j + 1] * y6[(size_t)j * 6 + 1] + S[3 * j + 2] * y6[(size_t)j * 6 + 4];
      sv[2] += S[3 * j + 1] * y6[(size_t)j * 6 + 5] + S[3 * j + 2] * y6[(size_t)j * 6 + 2];
    }
    if (!p.deltam) return;
    const int n1 = nleg + 1;
    std::vector<R> lt;
    for (int ipa = 0; ipa < npart; ++ipa) {
      R w = (ext == 0) ? (R)1 : extinct[(size_t)ipa * npts + ip] / ext;
      if (w == 0) continue;
      R f;
      point_legen6(ip, ipa, lt, f);
      const R da = albedo[(size_t)ipa * npts + ip] * dirflux[ip] * secmu0 * w;
      int J = 0;
      for (int l = 0; l <= ml; ++l) {
        const int me = std::min(l, mm);
        const R a1 = da * lt[l], b1 = da * lt[(size_t)4 * n1 + l];
        if (J < ns) {
          const int jt = J;
          for (int m = -me; m <= me; ++m, ++J) sv[0] = sv[0] - a1 * y6[(size_t)J * 6] * ylmsun[J];
          J = jt;
          for (int m = -me; m <= me; ++m, ++J) {
            sv[1] = sv[1] - b1 * y6[(size_t)J * 6 + 1] * ylmsun[J];
            sv[2] = sv[2] - b1 * y6[(size_t)J * 6 + 5] * ylmsun[J];
          }
        }
      }
      const int *IPH = &iphase[((size_t)ipa * npts + ip) * nq];
      const R *PW = &phaseinterpwt[((size_t)ipa * npts + ip) * nq];
      if (PW[0] >= phasemax) {
        for (int k = 0; k < 3; ++k) sv[k] = sv[k] + da * singscat[(size_t)(IPH[0] - 1) * 3 + k] / ((R)1 - f);
      } else {
        for (int q = 0; q < nq; ++q) {
          if (PW[q] <= (R)1e-5) continue;
          for (int k = 0; k < 3; ++k) sv[k] = sv[k] + da * singscat[(size_t)(IPH[q] - 1) * 3 + k] * PW[q] / ((R)1 - f);
        }
      }
    }
  }

  // RENDER (src/polarized/shdomsub4.f:93-286), scalar, solar.
  bool render(int n, const float *camx, const float *camy, const float *camz, const double *cammu,
              const double *camphi, float *out, int nthreads) {
    if (!precompute_phase()) return false;
    if (!brdf) lambertian_boundary();
    const double pi = std::acos(-1.0);
    std::vector<int> bad(std::max(1, nthreads), 0);
    std::vector<std::string> errs(std::max(1, nthreads));
    auto work = [&](int t, int b, int e) {
      Solver<R> &S = *this;
      for (int iv = b; iv < e; ++iv) {
        double x0 = camx[iv], y0 = camy[iv], z0 = camz[iv], mu2 = cammu[iv], phi2 = camphi[iv];
        double muray = -mu2, phiray = phi2 - pi;
        if (z0 > S.zgrid[nz - 1]) {
          if (muray >= 0.0) { for (int k = 0; k < S.nst; ++k) out[(size_t)iv * S.nst + k] = 0.f; continue; }
          double r = (S.zgrid[nz - 1] - z0) / muray;
          x0 = x0 + r * std::sqrt(1 - muray * muray) * std::cos(phiray);
          y0 = y0 + r * std::sqrt(1 - muray * muray) * std::sin(phiray);
          z0 = S.zgrid[nz - 1];
        } else if (z0 < S.zgrid[0]) { bad[t] = 1; errs[t] = "RENDER: Level below domain"; return; }
        double rad[3];
        if (!S.integrate_1ray(mu2, phi2, x0, y0, z0, rad, errs[t])) { bad[t] = 1; return; }
        for (int k = 0; k < S.nst; ++k) out[(size_t)iv * S.nst + k] = (float)rad[k];
      }
    };
    if (nthreads <= 1) work(0, 0, n);
    else {
      std::vector<std::thread> th;
      int chunk = (n + nthreads - 1) / nthreads;
      for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t, std::min(n, t * chunk), std::min(n, (t + 1) * chunk));
      for (auto &x : th) x.join();
    }
    for (int t = 0; t < (int)bad.size(); ++t) if (bad[t]) { err = errs[t]; return false; }
    return true;
  }

};

// ------------------------------------------------- Levis approximate gradient
// The adjoint branch of LEVISAPPROX_GRADIENT (src/polarized/shdomsub4.f:
// 288-809) for a scalar solar problem with a Lambertian surface: the
// unknowns are the extinction (IDR 0) and single-scattering albedo (IDR 1)
// of one species on the property grid, with the 'table' derivative method
// (DOEXACT = 0, no phase-function derivative), and the L2 cost with unit
// uncertainty, one ray per pixel, unit ray and Stokes weights.
template <typename R>
struct Levis {
  const Solver<R> &S;
  int ipa = 0, ng = 0;
  std::vector<int> interpptr;     // [npts][8] property point per trilinear corner (0-based)
  std::vector<R> optinterpwt;     // [npts][8]
  std::vector<R> fp, dextm;       // [ng], [ng][2]
  std::vector<R> dalbm, dfj;      // [npts][8][3]
  // Unknowns: 0 extinction, 1 albedo, 2 the phase function along a given
  // derivative series (DLEG with DIPHASEP of the reference; zero when none
  // is given): dleg [ndphase][nleg+1] in the LEGEN representation (divided
  // by 2l+1), diph [ng][maxnmicro] its 1-based rows at each property point
  // (weighted by the species' phase weights), dphasetab [nscatangle][ndphase]
  // its phase function for the exact single scatter, dfp [ng] the
  // derivative of the delta-M fraction f at each property point.
  static constexpr int NUMDER = 3;
  bool has_phase = false;
  int ndphase = 0;
  std::vector<R> dleg, dphasetab, dfp;
  std::vector<int> diph;
  explicit Levis(const Solver<R> &s) : S(s) {}

  R dext(int, int idr) const { return idr == 0 ? (R)1 : (R)0; }
  R dalb(int, int idr) const { return idr == 1 ? (R)1 : (R)0; }
  int diphp(int q, int ib) const { return diph[(size_t)ib * S.maxnmicro + q]; }

  // The phase-derivative table (given with the 2l+1 factor, like the
  // phase functions) and its phase function at the scattering angles of
  // PRECOMPUTE_PHASE_CHECK, without the positivity check.
  bool set_phase(int nd, int nlegd, const float *dleg_in, const int *diph_in, std::string &err) {
    const int ngp = S.p.npx * S.p.npy * S.p.npz, nl1 = S.nleg + 1;
    if (nd < 1 || nlegd < 0 || !dleg_in || !diph_in) { err = "phase derivative: bad table"; return false; }
    for (size_t k = 0; k < (size_t)ngp * S.maxnmicro; ++k)
      if (diph_in[k] < 1 || diph_in[k] > nd) { err = "phase derivative: index out of range"; return false; }
    has_phase = true;
    ndphase = nd;
    diph.assign(diph_in, diph_in + (size_t)ngp * S.maxnmicro);
    dleg.assign((size_t)nd * nl1, 0);
    for (int k = 0; k < nd; ++k)
      for (int l = 0; l <= std::min(nlegd, S.nleg); ++l)
        dleg[(size_t)k * nl1 + l] = (R)(dleg_in[(size_t)k * (nlegd + 1) + l] / (float)(2 * l + 1));
    const double pi = std::acos(-1.0), ofourpi = 1.0 / (4.0 * pi);
    dphasetab.assign((size_t)S.nscatangle * nd, 0);
    std::vector<double> d(nlegd + 1);
    for (int j = 0; j < S.nscatangle; ++j) {
      const double x = std::cos(pi * (double)j / (S.nscatangle - 1));
      d[0] = 1.0;
      if (nlegd >= 1) d[1] = x;
      for (int n = 1; n < nlegd; ++n) d[n + 1] = ((2 * n + 1) * x * d[n] - n * d[n - 1]) / (n + 1);
      for (int k = 0; k < nd; ++k) {
        double a1 = 0.0;
        for (int l = 0; l <= nlegd; ++l)
          a1 += (2.0 * l + 1.0) * (double)(float)(dleg_in[(size_t)k * (nlegd + 1) + l] / (float)(2 * l + 1)) * d[l];
        dphasetab[(size_t)j * nd + k] = (R)(a1 * ofourpi);
      }
    }
    return true;
  }
  R extp(int ib) const { return (R)S.extp[(size_t)ipa * ng + ib]; }
  R albp(int ib) const { return (R)S.albp[(size_t)ipa * ng + ib]; }
  int iphp(int q, int ib) const { return S.iphp[((size_t)ipa * ng + ib) * S.maxnmicro + q]; }
  R phwtp(int q, int ib) const { return (R)S.phwtp[((size_t)ipa * ng + ib) * S.maxnmicro + q]; }

  // COMPUTE_INTERP_WEIGHTS (src/polarized/shdomsub4.f:3083-3160) and
  // PREPARE_DERIV_INTERPS (src/polarized/shdomsub4.f:2917-3080).
  bool prepare(int ipa_der, std::string &err) {
    ipa = ipa_der;
    if (S.npts != S.nbpts) { err = "the Levis gradient is restated for the base grid (no split cells)"; return false; }
    const auto &p = S.p;
    const int npx = p.npx, npy = p.npy, npz = p.npz, npts = S.npts, ml = S.ml, nl1 = S.nleg + 1;
    ng = npx * npy * npz;
    interpptr.assign((size_t)npts * 8, 0); optinterpwt.assign((size_t)npts * 8, 0);
    for (int ip = 0; ip < npts; ++ip) {
      float x = S.gridpos[3 * ip], y = S.gridpos[3 * ip + 1], z = S.gridpos[3 * ip + 2];
      int il = 0, iu = npz;
      while (iu - il > 1) { int im = (iu + il) / 2; if (z >= S.zlev[im - 1]) il = im; else iu = im; }
      int iz = std::max(il, 1);
      double w = (double)(z - S.zlev[iz - 1]) / (S.zlev[iz] - S.zlev[iz - 1]);
      w = std::max(std::min(w, 1.0), 0.0);
      int ix = (int)(x / p.delx) + 1;
      if (std::fabs(x - npx * p.delx) < 0.01f * p.delx) ix = npx;
      if (ix < 1 || ix > npx) { err = "TRILIN: Beyond X domain"; return false; }
      int ixp = ix % npx + 1;
      double u = (double)(x - p.delx * (ix - 1)) / p.delx;
      u = std::max(std::min(u, 1.0), 0.0);
      if (u < 1e-5) u = 0; if (u > 1 - 1e-5) u = 1;
      int iy = (int)(y / p.dely) + 1;
      if (std::fabs(y - npy * p.dely) < 0.01f * p.dely) iy = npy;
      if (iy < 1 || iy > npy) { err = "TRILIN: Beyond Y domain"; return false; }
      int iyp = iy % npy + 1;
      double v = (double)(y - p.dely * (iy - 1)) / p.dely;
      v = std::max(std::min(v, 1.0), 0.0);
      if (v < 1e-5) v = 0; if (v > 1 - 1e-5) v = 1;
      const double f[8] = {(1 - u) * (1 - v) * (1 - w), u * (1 - v) * (1 - w), (1 - u) * v * (1 - w), u * v * (1 - w),
                           (1 - u) * (1 - v) * w,       u * (1 - v) * w,       (1 - u) * v * w,       u * v * w};
      int i1 = (iz - 1) + npz * (iy - 1) + npz * npy * (ix - 1), i2 = (iz - 1) + npz * (iy - 1) + npz * npy * (ixp - 1);
      int i3 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ix - 1), i4 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ixp - 1);
      const int ii[8] = {i1, i2, i3, i4, i1 + 1, i2 + 1, i3 + 1, i4 + 1};
      for (int k = 0; k < 8; ++k) { interpptr[(size_t)ip * 8 + k] = ii[k]; optinterpwt[(size_t)ip * 8 + k] = (R)f[k]; }
    }
    fp.assign(ng, 0); dfp.assign(ng, 0); dextm.assign((size_t)ng * NUMDER, 0);
    for (int ib = 0; ib < ng; ++ib) {
      R fv = 0, dfv = 0;
      if (p.deltam)
        for (int q = 0; q < S.maxnmicro; ++q) {
          fv += phwtp(q, ib) * S.legen[(size_t)(iphp(q, ib) - 1) * nl1 + ml + 1];
          if (has_phase) dfv += phwtp(q, ib) * dleg[(size_t)(diphp(q, ib) - 1) * nl1 + ml + 1];
        }
      fp[ib] = fv;
      dfp[ib] = dfv;
      for (int idr = 0; idr < NUMDER; ++idr)
        dextm[(size_t)ib * NUMDER + idr] = dext(ib, idr) * ((R)1 - fv * albp(ib)) - dalb(ib, idr) * fv * extp(ib) -
                                           (idr == 2 ? extp(ib) * albp(ib) * dfv : (R)0);
    }
    dalbm.assign((size_t)npts * 8 * NUMDER, 0); dfj.assign((size_t)npts * 8 * NUMDER, 0);
    for (int ip = 0; ip < npts; ++ip) {
      R F = 0, albj;
      const R alb = S.albedo[(size_t)ipa * npts + ip];
      if (p.deltam) {
        const int *IPH = &S.iphase[((size_t)ipa * npts + ip) * S.nq];
        const R *PW = &S.phaseinterpwt[((size_t)ipa * npts + ip) * S.nq];
        if (PW[0] >= S.phasemax) F = S.legen[(size_t)(IPH[0] - 1) * nl1 + ml + 1];
        else
          for (int q = 0; q < S.nq; ++q) {
            if (PW[q] < (R)1e-7) continue;
            F += PW[q] * S.legen[(size_t)(IPH[q] - 1) * nl1 + ml + 1];
          }
        albj = alb / (F * (alb - 1) + 1);
      } else {
        albj = alb;
      }
      const R divide = (R)1 / ((R)1 - albj * F);
      for (int nb = 0; nb < 8; ++nb) {
        const int ib = interpptr[(size_t)ip * 8 + nb];
        for (int idr = 0; idr < NUMDER; ++idr) {
          const R DE = dext(ib, idr), DA = dalb(ib, idr), FP = fp[ib], DFP = idr == 2 ? dfp[ib] : (R)0;
          dalbm[((size_t)ip * 8 + nb) * NUMDER + idr] =
              divide * (DE * (((R)1 - F) * (albp(ib) - albj) + (albj - 1) * albp(ib) * (FP - F)) +
                        DA * (((R)1 - F) * extp(ib) + (albj - 1) * extp(ib) * (FP - F)) +
                        DFP * (albj - 1) * extp(ib) * albp(ib));
          dfj[((size_t)ip * 8 + nb) * NUMDER + idr] =
              (DE * (FP - F) * albp(ib) + DA * (FP - F) * extp(ib) + DFP * extp(ib) * albp(ib)) / ((R)1 - F);
        }
      }
    }
    return true;
  }

  // COMPUTE_SOURCE_DIRECTION (src/polarized/shdomsub4.f:2836-2915), scalar.
  R source_direction(const R *L, int ip, const std::vector<R> &ylmdir, R secmu0) const {
    R s = 0;
    const int ris = S.rshptr[ip], rns = S.rshptr[ip + 1] - ris;
    for (int j = 0; j < rns; ++j) s += L[S.lofj[j]] * S.radiance[(size_t)ris + j] * ylmdir[j];
    if (!S.p.deltam)
      for (int j = 0; j < S.nlm; ++j) s += S.dirflux[ip] * secmu0 * L[S.lofj[j]] * S.ylmsun[j] * ylmdir[j];
    return s;
  }

  // COMPUTE_SOURCE_GRAD_1CELL (src/polarized/shdomsub4.f:1546-2042) for one
  // new grid point: extinction, source x extinction, single scatter x
  // extinction and GRAD8(NB, IDR).
  void point_grad(int ip, const std::vector<R> &ylmdir, const std::vector<R> &singscat,
                  const std::vector<R> &dsingscat, R &ext8, R &srcext8, R &singscat8, R grad8[8][NUMDER]) const {
    const auto &p = S.p;
    const int npts = S.npts, ml = S.ml, mm = S.mm, nl1 = S.nleg + 1;
    const R secmu0 = (R)1 / std::fabs((R)p.solarmu);
    const R ext = S.total_ext[ip];
    const int is = S.shptr[ip], ns = S.shptr[ip + 1] - is;
    for (int nb = 0; nb < 8; ++nb) for (int idr = 0; idr < NUMDER; ++idr) grad8[nb][idr] = 0;
    R src = 0, ss = 0;
    for (int j = 0; j < ns; ++j) src += S.source[(size_t)is + j] * ylmdir[j];
    std::vector<R> legent(nl1, 0);
    R F = 0;
    for (int ipa2 = 0; ipa2 < S.npart; ++ipa2) {
      const R w = (ext == 0) ? (R)1 : S.extinct[(size_t)ipa2 * npts + ip] / ext;
      if (w == 0) continue;
      S.point_legen(ip, ipa2, legent, F);  // delta-M divided when deltam
      const R da = S.albedo[(size_t)ipa2 * npts + ip] * S.dirflux[ip] * secmu0 * w;
      R trunc = 0;
      int J = 0;
      for (int l = 0; l <= ml; ++l) {
        const int me = std::min(l, mm);
        const R a1 = da * legent[l];
        if (J < ns)
          for (int m = -me; m <= me; ++m) { trunc += a1 * ylmdir[J] * S.ylmsun[J]; ++J; }
      }
      if (p.deltam) {
        const int *IPH = &S.iphase[((size_t)ipa2 * npts + ip) * S.nq];
        const R *PW = &S.phaseinterpwt[((size_t)ipa2 * npts + ip) * S.nq];
        if (PW[0] >= S.phasemax) ss += da * singscat[IPH[0] - 1] / ((R)1 - F);
        else
          for (int q = 0; q < S.nq; ++q) {
            if (PW[q] <= (R)1e-5) continue;
            ss += da * singscat[IPH[q] - 1] * PW[q] / ((R)1 - F);
          }
        src -= trunc;
      } else {
        ss += trunc;
      }
    }
    if (p.deltam) src += ss;
    // gradient: species ipa (the same for both derivatives)
    R scatterj = 0, singscatj = 0, sourcet;
    if (p.deltam) {
      for (int nb = 0; nb < 8; ++nb) {
        const int ib = interpptr[(size_t)ip * 8 + nb];
        const R xi = optinterpwt[(size_t)ip * 8 + nb];
        const R sw = xi * albp(ib) * extp(ib);
        scatterj += sw;
        if (sw <= (R)1e-6) continue;
        for (int q = 0; q < S.maxnmicro; ++q) {
          if (phwtp(q, ib) <= (R)1e-6) continue;
          singscatj += sw * phwtp(q, ib) * singscat[iphp(q, ib) - 1];
        }
      }
      singscatj = (scatterj > (R)S.scatmin) ? singscatj / scatterj : singscatj / (R)S.scatmin;
    }
    if (S.npart == 1) {
      const R a = S.albedo[(size_t)ipa * npts + ip];
      sourcet = (a > (R)1e-8) ? src / a : (R)0;
    } else {
      std::fill(legent.begin(), legent.end(), (R)0);
      F = 0;
      for (int nb = 0; nb < 8; ++nb) {
        const int ib = interpptr[(size_t)ip * 8 + nb];
        const R sw = optinterpwt[(size_t)ip * 8 + nb] * albp(ib) * extp(ib);
        if (sw <= (R)1e-6) continue;
        for (int q = 0; q < S.maxnmicro; ++q) {
          if (phwtp(q, ib) <= (R)1e-6) continue;
          const R *L = &S.legen[(size_t)(iphp(q, ib) - 1) * nl1];
          for (int l = 0; l < nl1; ++l) legent[l] += sw * phwtp(q, ib) * L[l];
        }
      }
      const R div = (scatterj > (R)S.scatmin) ? scatterj : (R)S.scatmin;
      for (int l = 0; l < nl1; ++l) legent[l] /= div;
      if (p.deltam) {
        F = legent[ml + 1];
        for (int l = 0; l <= ml; ++l) legent[l] /= ((R)1 - F);
      }
      sourcet = 0;
      if (scatterj > (R)S.scatmin) {
        sourcet = source_direction(legent.data(), ip, ylmdir, secmu0);
        if (p.deltam) sourcet += S.dirflux[ip] * singscatj * secmu0 / ((R)1 - F);
      }
    }
    sourcet = std::max((R)0, sourcet);
    if (p.deltam)
      for (int l = 0; l <= ml; ++l) legent[l] = legent[l] * ((R)1 - F) + F;
    std::vector<R> legenp(nl1), dlegt(nl1);
    const R albip = S.albedo[(size_t)ipa * npts + ip];
    // thermal source: B(T) of the point for the emission term of the source
    // derivative (src/polarized/shdomsub4.f:1792-1799, :2009-2016)
    const R bpl = S.srct != 'S' ? (R)S.planck_fn(S.temp[ip]) : (R)0;
    for (int nb = 0; nb < 8; ++nb) {
      const int ib = interpptr[(size_t)ip * 8 + nb];
      const R xi = optinterpwt[(size_t)ip * 8 + nb];
      if (xi < (R)1e-7) continue;
      std::fill(legenp.begin(), legenp.end(), (R)0);
      for (int q = 0; q < S.maxnmicro; ++q) {
        const R *L = &S.legen[(size_t)(iphp(q, ib) - 1) * nl1];
        const R ft = p.deltam ? L[ml + 1] : (R)0;
        for (int l = 0; l < nl1; ++l) legenp[l] += phwtp(q, ib) * ((p.deltam && l <= ml) ? L[l] + ft : L[l]);
      }
      R singscatp = 0;
      if (p.deltam)
        for (int q = 0; q < S.maxnmicro; ++q) singscatp += phwtp(q, ib) * singscat[iphp(q, ib) - 1];
      for (int idr = 0; idr < NUMDER; ++idr) {
        if (idr == 2 && !has_phase) continue;
        const R DE = dext(ib, idr), DA = dalb(ib, idr);
        const R DFJ = dfj[((size_t)ip * 8 + nb) * NUMDER + idr];
        for (int l = 0; l < nl1; ++l) {
          const R diff = legenp[l] - legent[l];
          dlegt[l] = DE * diff * albp(ib) + DA * diff * extp(ib) + (legent[l] - 1) * DFJ;
        }
        R dsingscatp = 0;
        if (idr == 2) {  // DLEGP (and DSINGSCATP): the derivative series at the property point
          for (int q = 0; q < S.maxnmicro; ++q) {
            const R w = phwtp(q, ib);
            const R *D = &dleg[(size_t)(diphp(q, ib) - 1) * nl1];
            for (int l = 0; l < nl1; ++l) dlegt[l] += w * D[l] * extp(ib) * albp(ib);
            if (p.deltam) dsingscatp += w * dsingscat[diphp(q, ib) - 1];
          }
        }
        const R dsource = source_direction(dlegt.data(), ip, ylmdir, secmu0);
        R g = xi * (sourcet * (albip * dextm[(size_t)ib * NUMDER + idr] + dalbm[((size_t)ip * 8 + nb) * NUMDER + idr]) + dsource);
        // emission e (1 - albedo) B: no temperature unknowns, so only the
        // extinction and albedo derivatives enter
        if (S.srct != 'S')
          g += xi * (bpl * ((R)1 - albip) * dextm[(size_t)ib * NUMDER + idr] - bpl * dalbm[((size_t)ip * 8 + nb) * NUMDER + idr]);
        if (p.deltam)
          g += S.dirflux[ip] * secmu0 * xi *
               (singscatj * DFJ + DA * (singscatp - singscatj) * extp(ib) + DE * (singscatp - singscatj) * albp(ib) +
                dsingscatp * extp(ib) * albp(ib));
        grad8[nb][idr] += g;
      }
    }
    singscat8 = ss * ext;
    srcext8 = src * ext;
    ext8 = ext;
  }

  // ADJOINT_INTEGRATE_1RAY (src/polarized/shdomsub4.f:3223-3967) with
  // COMPUTE_RADIANCE_DERIVATIVE_ADJOINT (:4037-4114); accumulates into
  // gradout [ng][2] and beam_weight [npts].
  bool adjoint_ray(double mu2, double phi2, double x0, double y0, double z0, double adj, std::vector<double> &gradout,
                   std::vector<double> &beam, std::string &err) const {
    const auto &p = S.p;
    const double pi = std::acos(-1.0);
    const int nx = S.nx, ny = S.ny;
    const double eps = 1.0e-5 * (S.gridpos[3 * S.gridptr[7] + 2] - S.gridpos[3 * S.gridptr[0] + 2]);
    std::vector<R> ylmdir = S.ylmall((double)(float)mu2, (float)phi2);
    std::vector<R> singscat(S.numphase, 0), dsingscat(std::max(1, ndphase), 0);
    if (p.deltam) {
      double cosscat = (double)p.solarmu * mu2 +
                       std::sqrt((1.0 - (double)p.solarmu * p.solarmu) * (1.0 - mu2 * mu2)) * std::cos((double)p.solaraz - phi2);
      cosscat = std::max(std::min(1.0, cosscat), -1.0);
      float F = (float)((S.nscatangle - 1) * (std::acos(cosscat) / pi) + 1);
      int J = std::min(S.nscatangle - 1, (int)F);
      F = F - J;
      for (int i = 0; i < S.numphase; ++i)
        singscat[i] = (R)((1 - F) * S.phasetab[(size_t)(J - 1) * S.numphase + i] + F * S.phasetab[(size_t)J * S.numphase + i]);
      for (int i = 0; i < ndphase; ++i)
        dsingscat[i] = (R)((1 - F) * dphasetab[(size_t)(J - 1) * ndphase + i] + F * dphasetab[(size_t)J * ndphase + i]);
    }
    double cx = std::sqrt(1.0 - mu2 * mu2) * std::cos(phi2 - pi), cy = std::sqrt(1.0 - mu2 * mu2) * std::sin(phi2 - pi);
    double cz = -mu2, cxinv, cyinv, czinv;
    if (std::fabs(cx) > 1e-6) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1e6; }
    if (std::fabs(cy) > 1e-6) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1e6; }
    if (std::fabs(cz) > 1e-6) czinv = 1.0 / cz; else { cz = 0; czinv = 1e6; }
    const int bitx = cx < 0, bity = cy < 0, bitz = cz < 0, ioct = 1 + bitx + 2 * bity + 4 * bitz;
    const float xm = 0.5f * (S.xgrid[0] + S.xgrid[nx - 1]), ym = 0.5f * (S.ygrid[0] + S.ygrid[ny - 1]);
    double xe = x0, ye = y0, ze = z0;
    int icell = S.locate_grid_cell(xe, ye, ze);
    int iface = -1;
    double transmit = 1.0;
    R extinct8[8] = {0}, srcext8[8] = {0}, singscat8[8] = {0}, grad8[8][8][NUMDER];
    for (auto &a : grad8) for (auto &b : a) for (auto &c : b) c = 0;
    int oldipts[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    static const int doneface[7][8] = {{0, 0, 0, 0, 0, 0, 0, 0}, {0, 1, 0, 3, 0, 5, 0, 7}, {2, 0, 4, 0, 6, 0, 8, 0},
                                       {0, 0, 1, 2, 0, 0, 5, 6}, {3, 4, 0, 0, 7, 8, 0, 0}, {0, 0, 0, 0, 1, 2, 3, 4},
                                       {5, 6, 7, 8, 0, 0, 0, 0}};
    // per subgrid interval (PASSED* arrays)
    std::vector<int> ppts;
    std::vector<double> pint0, pint1, pdels, prad, pabs, ptr;
    auto push = [&]() {
      ppts.resize(ppts.size() + 8, 0); pint0.resize(pint0.size() + 8, 0.0); pint1.resize(pint1.size() + 8, 0.0);
      pdels.push_back(0); prad.push_back(0); pabs.push_back(0); ptr.push_back(1);
    };
    push();
    int np = 0;  // current interval index (NPASSED - 1)
    bool validrad = false;
    const double c12 = (double)0.08333333333f;
    while (!validrad && icell >= 0) {
      R oext8[8], osrc8[8], oss8[8], ogr8[8][8][NUMDER];
      for (int i = 0; i < 8; ++i) {
        oext8[i] = extinct8[i]; osrc8[i] = srcext8[i]; oss8[i] = singscat8[i];
        for (int nb = 0; nb < 8; ++nb) for (int d = 0; d < NUMDER; ++d) ogr8[i][nb][d] = grad8[i][nb][d];
      }
      for (int n = 0; n < 8; ++n) {
        const int ip = S.gridptr[8 * icell + n];
        const int I = doneface[iface + 1][n];
        if (I > 0 && ip == oldipts[n]) {
          extinct8[n] = oext8[I - 1]; srcext8[n] = osrc8[I - 1]; singscat8[n] = oss8[I - 1];
          for (int nb = 0; nb < 8; ++nb) for (int d = 0; d < NUMDER; ++d) grad8[n][nb][d] = ogr8[I - 1][nb][d];
          continue;
        }
        oldipts[n] = ip;
        point_grad(ip, ylmdir, singscat, dsingscat, extinct8[n], srcext8[n], singscat8[n], grad8[n]);
      }
      const int ipt1 = S.gridptr[8 * icell], ipt2 = S.gridptr[8 * icell + 7];
      const double delx = S.gridpos[3 * ipt2] - S.gridpos[3 * ipt1], dely = S.gridpos[3 * ipt2 + 1] - S.gridpos[3 * ipt1 + 1];
      const double delz = S.gridpos[3 * ipt2 + 2] - S.gridpos[3 * ipt1 + 2];
      const double ivx = delx <= 0 ? 1.0 : 1.0 / delx, ivy = dely <= 0 ? 1.0 : 1.0 / dely, ivz = 1.0 / delz;
      auto kernel = [&](double x, double y, double z, double fc[8]) {
        const double u = (x - S.gridpos[3 * ipt1]) * ivx, v = (y - S.gridpos[3 * ipt1 + 1]) * ivy,
                     w = (z - S.gridpos[3 * ipt1 + 2]) * ivz;
        fc[0] = (1 - w) * (1 - v) * (1 - u); fc[1] = (1 - w) * (1 - v) * u; fc[2] = (1 - w) * v * (1 - u); fc[3] = (1 - w) * v * u;
        fc[4] = w * (1 - v) * (1 - u); fc[5] = w * (1 - v) * u; fc[6] = w * v * (1 - u); fc[7] = w * v * u;
      };
      double fc[8];
      kernel(xe, ye, ze, fc);
      R srcext1 = 0, ext1 = 0;
      for (int k = 0; k < 8; ++k) { srcext1 = (R)(srcext1 + fc[k] * srcext8[k]); }
      srcext1 = std::max((R)0, srcext1);
      for (int k = 0; k < 8; ++k) ext1 = (R)(ext1 + fc[k] * extinct8[k]);
      for (int k = 0; k < 8; ++k) pint1[8 * np + k] = fc[k];
      R ss1[8], gr1[8][8][NUMDER];
      for (int n = 0; n < 8; ++n) {
        ss1[n] = std::max((R)0, (R)(fc[n] * singscat8[n]));
        for (int nb = 0; nb < 8; ++nb) for (int d = 0; d < NUMDER; ++d) gr1[n][nb][d] = (R)(fc[n] * grad8[n][nb][d]);
      }
      const bool ipinx = (S.cellflags[icell] & 1) && !((S.bcflag & 1) && ((cx > 0 && xe < xm) || (cx < 0 && xe > xm)));
      const bool ipiny = (S.cellflags[icell] & 2) && !((S.bcflag & 2) && ((cy > 0 && ye < ym) || (cy < 0 && ye > ym)));
      const int iopp = S.gridptr[8 * icell + (8 - ioct)];
      const double sox = ipinx ? 1e20 : (S.gridpos[3 * iopp] - xe) * cxinv;
      const double soy = ipiny ? 1e20 : (S.gridpos[3 * iopp + 1] - ye) * cyinv;
      const double soz = (S.gridpos[3 * iopp + 2] - ze) * czinv;
      const double so = std::min(sox, std::min(soy, soz));
      if (so < -eps) { err = "ADJOINT_INTEGRATE_1RAY: SO<0"; return false; }
      double xn = xe + so * cx, yn = ye + so * cy, zn = ze + so * cz;
      double fcn[8];
      kernel(xn, yn, zn, fcn);
      R extn = 0;
      for (int k = 0; k < 8; ++k) extn = (R)(extn + fcn[k] * extinct8[k]);
      const double taugrid = so * 0.5 * (ext1 + extn);
      const int ntau = std::max(1, 1 + (int)(taugrid / p.tautol));
      const double dels = so / ntau;
      double srcss[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int it = 1; it <= ntau; ++it) {
        pdels[np] = dels;
        for (int k = 0; k < 8; ++k) { pint1[8 * np + k] = fc[k]; ppts[8 * np + k] = S.gridptr[8 * icell + k]; }
        const double s = it * dels;
        kernel(xe + s * cx, ye + s * cy, ze + s * cz, fc);
        R srcext0 = 0, ext0 = 0;
        for (int k = 0; k < 8; ++k) srcext0 = (R)(srcext0 + fc[k] * srcext8[k]);
        if (it != ntau) { for (int k = 0; k < 8; ++k) ext0 = (R)(ext0 + fc[k] * extinct8[k]); }
        else ext0 = extn;
        srcext0 = std::max((R)0, srcext0);
        for (int k = 0; k < 8; ++k) pint0[8 * np + k] = fc[k];
        R ss0[8], gr0[8][8][NUMDER];
        for (int n = 0; n < 8; ++n) {
          ss0[n] = std::max((R)0, (R)(fc[n] * singscat8[n]));
          for (int nb = 0; nb < 8; ++nb) for (int d = 0; d < NUMDER; ++d) gr0[n][nb][d] = (R)(fc[n] * grad8[n][nb][d]);
        }
        const double ext = 0.5 * (ext0 + ext1);
        double transcell;
        if (ext != 0.0) {
          const double tau = ext * dels;
          const double abscell = tau * (1.0 - 0.5 * tau * (1.0 - 0.33333333333 * tau));
          transcell = 1.0 - abscell;
          const double corr = dels * (1.0 - 0.05 * (ext1 - ext0) * dels);
          const double src = (0.5 * (srcext0 + srcext1) + c12 * (ext0 * srcext1 - ext1 * srcext0) * corr) / ext;
          for (int n = 0; n < 8; ++n) {
            srcss[n] += transmit * abscell * (0.5 * (ss0[n] + ss1[n]) + c12 * (ext0 * ss1[n] - ext1 * ss0[n]) * corr) / ext;
          }
          pabs[np] = abscell; ptr[np] = transmit; prad[np] = transmit * src * abscell;
          for (int kk = 0; kk < 8; ++kk) {
            const int ip = S.gridptr[8 * icell + kk];
            for (int k = 0; k < 8; ++k) {
              const int ib = interpptr[(size_t)ip * 8 + k];
              for (int d = 0; d < NUMDER; ++d) {
                const R sg = (R)((0.5 * (gr0[kk][k][d] + gr1[kk][k][d]) + c12 * (ext0 * gr1[kk][k][d] - ext1 * gr0[kk][k][d]) * corr) / ext);
                gradout[(size_t)ib * NUMDER + d] += transmit * (adj * sg) * abscell;
              }
            }
          }
          ++np;
          push();
        } else {
          transcell = 1.0;
          for (int n = 0; n < 8; ++n) srcss[n] = 0;
        }
        transmit *= transcell;
        ext1 = ext0; srcext1 = srcext0;
        for (int n = 0; n < 8; ++n) {
          ss1[n] = ss0[n];
          for (int nb = 0; nb < 8; ++nb) for (int d = 0; d < NUMDER; ++d) gr1[n][nb][d] = gr0[n][nb][d];
        }
      }
      for (int kk = 0; kk < 8; ++kk) beam[S.gridptr[8 * icell + kk]] += adj * srcss[kk];
      int jface;
      bool openbcface;
      if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; openbcface = (S.cellflags[icell] & 1) && (S.bcflag & 1); }
      else if (soy <= soz) { iface = 3 - bity; jface = 1; openbcface = (S.cellflags[icell] & 2) && (S.bcflag & 2); }
      else { iface = 5 - bitz; jface = 2; openbcface = false; }
      const int inext = S.neighptr[6 * icell + iface];
      int kface, ic;
      if (!openbcface) { kface = iface; ic = icell; }
      else { kface = kOppFace[iface]; ic = inext; iface = -1; }
      if (inext >= 0) {
        if (jface == 0) xn = S.gridpos[3 * S.gridptr[8 * inext + ioct - 1]];
        else if (jface == 1) yn = S.gridpos[3 * S.gridptr[8 * inext + ioct - 1] + 1];
        else zn = S.gridpos[3 * S.gridptr[8 * inext + ioct - 1] + 2];
      }
      if (transmit < p.transcut) {
        validrad = true;
        prad[np] = 0.0; ptr[np] = 1.0;
      } else if (inext < 0 && iface >= 4) {
        validrad = true;
        double xs[4], ys[4], rb[4], dr[4];
        int bp[4];
        for (int jj = 0; jj < 4; ++jj) {
          const int ipb = S.gridptr[8 * ic + kGridFace[kface][jj]];
          bp[jj] = ipb; xs[jj] = S.gridpos[3 * ipb]; ys[jj] = S.gridpos[3 * ipb + 1]; dr[jj] = 0;
          if ((float)mu2 < 0.0f) {
            rb[jj] = p.skyrad;
          } else {
            auto itb = std::lower_bound(S.botp.begin(), S.botp.end(), ipb);
            if (itb == S.botp.end() || *itb != ipb) { err = "FIND_BOUNDARY_RADIANCE: Not at boundary"; return false; }
            const size_t b = itb - S.botp.begin();
            rb[jj] = S.bcrad_bot[b];
            dr[jj] = (double)((float)(1.0 / std::acos(-1.0)) * S.sfcgridalb[b] * S.dirflux[ipb]);
          }
        }
        const double uu = (xs[1] - xs[0] > 0) ? (xn - xs[0]) / (xs[1] - xs[0]) : 0.0;
        const double vv = (ys[2] - ys[0] > 0) ? (yn - ys[0]) / (ys[2] - ys[0]) : 0.0;
        const double bi[4] = {(1 - uu) * (1 - vv), uu * (1 - vv), (1 - uu) * vv, uu * vv};
        const float radbnd = (float)(bi[0] * rb[0] + bi[1] * rb[1] + bi[2] * rb[2] + bi[3] * rb[3]);
        ptr[np] = transmit; pabs[np] = -1.0; prad[np] = transmit * radbnd;
        for (int kk = 0; kk < 4; ++kk) beam[bp[kk]] += adj * transmit * bi[kk] * dr[kk];
      } else {
        icell = inext;
      }
      xe = xn; ye = yn; ze = zn;
    }
    // future radiance: backward sum, divided by the transmission
    const int npassed = np + 1;
    for (int kk = npassed - 2; kk >= 0; --kk) prad[kk] += prad[kk + 1];
    for (int kk = 0; kk < npassed; ++kk) prad[kk] /= ptr[kk];
    for (int kk = 0; kk < npassed - 1; ++kk) {
      double ext0 = 0, ext1 = 0;
      for (int k = 0; k < 8; ++k) {
        ext0 += S.total_ext[ppts[8 * kk + k]] * pint0[8 * kk + k];
        ext1 += S.total_ext[ppts[8 * kk + k]] * pint1[8 * kk + k];
      }
      const double ext = 0.5 * (ext0 + ext1), dl = pdels[kk];
      if (ext == 0.0) continue;
      for (int k = 0; k < 8; ++k) {
        const int ip = ppts[8 * kk + k];
        const double g0 = -adj * prad[kk + 1] * pint0[8 * kk + k];
        const double g1 = -adj * prad[kk] * pint1[8 * kk + k];
        double ag = (0.5 * (g0 + g1) + c12 * (ext0 * g1 - ext1 * g0) * dl * (1.0 - 0.05 * (ext1 - ext0) * dl)) / ext;
        ag *= ptr[kk] * pabs[kk];
        for (int d = 0; d < NUMDER; ++d)
          for (int nb = 0; nb < 8; ++nb) {
            const int ib = interpptr[(size_t)ip * 8 + nb];
            const float eg = (float)(dextm[(size_t)ib * NUMDER + d] * optinterpwt[(size_t)ip * 8 + nb]);
            gradout[(size_t)ib * NUMDER + d] += eg * ag;
          }
      }
    }
    return true;
  }

  // COMPUTE_DIRECT_BEAM_DERIV_ADJOINT (src/polarized/shdomsub4.f:4117-4143)
  // with the sun-path derivatives of DIRECT_BEAM_AND_PATHS_PROP
  // (src/shdomsub5.f:1608-2345): d(optical path)/d(extinction at each
  // property corner) of the trilinear path integral, cell by cell.
  void direct_beam_deriv(int ipt, double weight, std::vector<double> &gradout) const {
    const auto &p = S.p;
    const int npx = p.npx, npy = p.npy, npz = p.npz, bcflag = S.bcflag;
    int ipdirect = S.ipflag;
    if (S.ipflag & 4) ipdirect = 0;
    const double sunmu = -(double)p.solarmu, sunaz = (double)(float)(p.solaraz + (float)std::acos(-1.0f));
    double cx = std::sqrt(1.0 - sunmu * sunmu) * std::cos(sunaz), cy = std::sqrt(1.0 - sunmu * sunmu) * std::sin(sunaz);
    double cz = std::fabs(sunmu), cxinv, cyinv, czinv;
    if (std::fabs(cx) > 1e-6) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1e20; }
    if (std::fabs(cy) > 1e-6) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1e20; }
    if (std::fabs(cz) > 1e-6) czinv = 1.0 / cz; else { cz = 0; czinv = 1e20; }
    const int di = cx >= 0 ? 1 : -1, dj = cy >= 0 ? 1 : -1, dk = cz >= 0 ? 1 : -1;
    const double epsz = 1.0e-6 * (S.zlev[npz - 1] - S.zlev[0]);
    const double delxd = p.delx, delyd = p.dely, xdomain = delxd * npx, ydomain = delyd * npy;
    const double z = S.gridpos[3 * ipt + 2], x = S.gridpos[3 * ipt], y = S.gridpos[3 * ipt + 1];
    int il = 0, iu = npz;
    while (iu - il > 1) { int im = (iu + il) / 2; if (z >= S.zlev[im - 1]) il = im; else iu = im; }
    int k = std::max(il, 1);
    int i = (int)(x / delxd) + 1;
    if (i > npx && std::fabs(x - xdomain) < 0.001 * delxd) i = npx;
    int j = (int)(y / delyd) + 1;
    if (j > npy && std::fabs(y - ydomain) < 0.001 * delyd) j = npy;
    double xe = x, ye = y, ze = z, xp = xe, yp = ye, zp = ze;
    bool constx = ipdirect & 1, consty = ipdirect & 2;
    if (cx == 0.0) constx = true;
    if (cy == 0.0) consty = true;
    if ((bcflag & 1) && (std::fabs(x) < 0.01 * delxd || std::fabs(x - (npx - 1) * delxd) < 0.01 * delxd)) constx = true;
    if ((bcflag & 2) && (std::fabs(y) < 0.01 * delyd || std::fabs(y - (npy - 1) * delyd) < 0.01 * delyd)) consty = true;
    int guard = 0;
    while (std::fabs(ze - S.zlev[npz - 1]) > epsz && guard++ < 10000000) {
      int ipn = i + 1;
      if (i == npx) ipn = (bcflag & 1) ? npx : 1;
      int jpn = j + 1;
      if (j == npy) jpn = (bcflag & 2) ? npy : 1;
      const double x0 = delxd * (i - 1), x1 = x0 + delxd, y0 = delyd * (j - 1), y1 = y0 + delyd;
      const double z0 = S.zlev[k - 1], z1 = S.zlev[k];
      const int I1 = (k - 1) + npz * (j - 1) + npz * npy * (i - 1), I2 = (k - 1) + npz * (j - 1) + npz * npy * (ipn - 1);
      const int I3 = (k - 1) + npz * (jpn - 1) + npz * npy * (i - 1), I4 = (k - 1) + npz * (jpn - 1) + npz * npy * (ipn - 1);
      double sox, soy, soz;
      if (constx) sox = 1e30; else if (cx > 0) { sox = (x1 - xe) * cxinv; xp = x1; } else { sox = (x0 - xe) * cxinv; xp = x0; }
      if (consty) soy = 1e30; else if (cy > 0) { soy = (y1 - ye) * cyinv; yp = y1; } else { soy = (y0 - ye) * cyinv; yp = y0; }
      if (cz > 0) { soz = (z1 - ze) * czinv; zp = z1; } else if (cz < 0) { soz = (z0 - ze) * czinv; zp = z0; } else soz = 1e30;
      double xoffs = 0, yoffs = 0, so;
      if (soz <= sox && soz <= soy) {
        so = soz;
        if (!constx) xp = xe + so * cx;
        if (!consty) yp = ye + so * cy;
        k += dk;
      } else if (sox <= soy) {
        so = sox;
        if (!consty) yp = ye + so * cy;
        zp = ze + so * cz;
        i += di;
        if (i == 0) { if (bcflag & 1) { i = 1; constx = true; } else { i = npx; xoffs = xdomain; } }
        else if (i == npx + 1) { if (bcflag & 1) { i = npx; constx = true; } else { i = 1; xoffs = -xdomain; } }
      } else {
        so = soy;
        if (!constx) xp = xe + so * cx;
        zp = ze + so * cz;
        j += dj;
        if (j == 0) { if (bcflag & 2) { j = 1; consty = true; } else { j = npy; yoffs = ydomain; } }
        else if (j == npy + 1) { if (bcflag & 2) { j = npy; consty = true; } else { j = 1; yoffs = -ydomain; } }
      }
      so = std::max(so, 0.0);
      const double ax = 1.0 / (x1 - x0), ay = 1.0 / (y1 - y0), az = 1.0 / (z1 - z0);
      const double u0 = (xe - x0) * ax, v0 = (ye - y0) * ay, w0 = (ze - z0) * az;
      const double du = (xp - x0) * ax - u0, dv = (yp - y0) * ay - v0, dw = (zp - z0) * az - w0;
      const double u0m = 1 - u0, v0m = 1 - v0, w0m = 1 - w0;
      const double uv = u0 * v0, umv = u0m * v0, uvm = u0 * v0m, umvm = u0m * v0m;
      const double uw = u0 * w0, umw = u0m * w0, uwm = u0 * w0m, umwm = u0m * w0m;
      const double vw = v0 * w0, vmw = v0m * w0, vwm = v0 * w0m, vmwm = v0m * w0m;
      const double A[8] = {u0m * vmwm, u0 * vmwm, u0m * vwm, u0 * vwm, u0m * vmw, u0 * vmw, u0m * vw, u0 * vw};
      const double B[8] = {-du * vmwm - dv * umwm - dw * umvm, du * vmwm - dv * uwm - dw * uvm,
                           -du * vwm + dv * umwm - dw * umv,   du * vwm + dv * uwm - dw * uv,
                           -du * vmw - dv * umw + dw * umvm,   du * vmw - dv * uw + dw * uvm,
                           -du * vw + dv * umw + dw * umv,     du * vw + dv * uw + dw * uv};
      const double VW = dv * dw, vwu = VW * u0, vwum = VW * u0m, UW = du * dw, uwv = UW * v0, uwvm = UW * v0m;
      const double UV = du * dv, uvw = UV * w0, uvwm = UV * w0m;
      const double C[8] = {vwum + uwvm + uvwm, vwu - uwvm - uvwm, -vwum + uwv - uvwm, -vwu - uwv + uvwm,
                           -vwum - uwvm + uvw, -vwu + uwvm - uvw, vwum - uwv - uvw,   vwu + uwv + uvw};
      const double sgn[8] = {-1, 1, 1, -1, 1, -1, -1, 1}, ddd = du * dv * dw;
      const int ptrs[8] = {I1, I2, I3, I4, I1 + 1, I2 + 1, I3 + 1, I4 + 1};
      for (int c = 0; c < 8; ++c) {
        const float dpath = (float)(so * (A[c] + 0.5 * B[c] + 0.3333333333333333 * C[c] + sgn[c] * 0.25 * ddd));
        for (int d = 0; d < NUMDER; ++d)
          gradout[(size_t)ptrs[c] * NUMDER + d] -= dextm[(size_t)ptrs[c] * NUMDER + d] * dpath * weight;
      }
      xe = xp + xoffs; ye = yp + yoffs; ze = zp;
    }
  }
};

// Render with the properties of one property-grid voxel of species ipa
// perturbed and the source function recomputed from the frozen RADIANCE
// (new delta-M medium and direct beam, same truncations): the forward model
// whose derivative the Levis approximation is.  The solver state is
// restored afterwards.
template <typename R>
bool frozen_render(Solver<R> &S, int ipa, int voxel, float dext, float dalb, int n, const float *camx,
                   const float *camy, const float *camz, const double *cammu, const double *camphi, float *out,
                   int nthreads) {
  const int ng = S.p.npx * S.p.npy * S.p.npz;
  if (ipa < 0 || ipa >= S.npart || voxel < 0 || voxel >= ng) { S.err = "frozen_render: bad index"; return false; }
  if (S.nst != 1) { S.err = "frozen_render: scalar problems only"; return false; }
  if (S.npts != S.nbpts) { S.err = "frozen_render: base grid only (no split cells)"; return false; }
  auto extp = S.extp, albp = S.albp;
  auto planck_tot = S.planck_tot;
  auto temp = S.temp;
  auto source = S.source;
  auto shptr = S.shptr;
  auto extinct = S.extinct, albedo = S.albedo, total_ext = S.total_ext, phaseinterpwt = S.phaseinterpwt;
  auto iphase = S.iphase;
  auto dirflux = S.dirflux;
  auto legen = S.legen;
  const R albmax = S.albmax;
  S.extp[(size_t)ipa * ng + voxel] += dext;
  S.albp[(size_t)ipa * ng + voxel] += dalb;
  bool ok = S.transfer_properties();
  if (ok) {
    S.make_direct();
    S.compute_source(true, true);
    ok = S.render(n, camx, camy, camz, cammu, camphi, out, nthreads);
  }
  S.extp = extp; S.albp = albp; S.source = source; S.shptr = shptr; S.extinct = extinct; S.albedo = albedo;
  S.total_ext = total_ext; S.phaseinterpwt = phaseinterpwt; S.iphase = iphase; S.dirflux = dirflux; S.legen = legen;
  S.albmax = albmax; S.planck_tot = planck_tot; S.temp = temp;
  return ok;
}

// A phase-derivative direction for the third unknown: a table of
// derivative series and its rows at each property point.
struct PhaseDeriv {
  int ndphase = 0, nlegd = 0;
  const float *dleg = nullptr;  // [ndphase][nlegd+1], with the 2l+1 factor
  const int *diph = nullptr;    // [npx*npy*npz][maxnmicro], 1-based
};

// frozen_render with the phase function of one voxel of species ipa moved
// along a derivative series (and its extinction and albedo by dext, dalb):
// the voxel gets a phase-table row of its own, its current mixture plus
// eps x dleg_row (nlegd+1 terms with the 2l+1 factor), with weight 1.
template <typename R>
bool frozen_render_phase(Solver<R> &S, int ipa, int voxel, float eps, int nlegd, const float *dleg_row, float dext,
                         float dalb, int n, const float *camx, const float *camy, const float *camz,
                         const double *cammu, const double *camphi, float *out, int nthreads) {
  const int ng = S.p.npx * S.p.npy * S.p.npz, nm = S.p.maxnmicro, nlp = S.p.nlegp;
  if (ipa < 0 || ipa >= S.npart || voxel < 0 || voxel >= ng) { S.err = "frozen_render_phase: bad index"; return false; }
  if (S.nst != 1) { S.err = "frozen_render_phase: scalar problems only"; return false; }
  const auto legp = S.legp;
  const auto iphp = S.iphp;
  const auto phwtp = S.phwtp;
  const shdom_problem p0 = S.p;
  std::vector<float> row(nlp + 1, 0.f);
  const size_t o = ((size_t)ipa * ng + voxel) * nm;
  for (int q = 0; q < nm; ++q)
    for (int l = 0; l <= nlp; ++l) row[l] += phwtp[o + q] * legp[(size_t)(iphp[o + q] - 1) * (nlp + 1) + l];
  for (int l = 0; l <= std::min(nlp, nlegd); ++l) row[l] += eps * dleg_row[l];
  S.legp.insert(S.legp.end(), row.begin(), row.end());
  S.p.numphase += 1;
  for (int q = 0; q < nm; ++q) { S.iphp[o + q] = S.p.numphase; S.phwtp[o + q] = q == 0 ? 1.f : 0.f; }
  bool ok = frozen_render(S, ipa, voxel, dext, dalb, n, camx, camy, camz, cammu, camphi, out, nthreads);
  S.legp = legp; S.iphp = iphp; S.phwtp = phwtp; S.p = p0;
  if (ok) ok = S.transfer_properties();   // back to the solver's own tables
  return ok;
}

template <typename R>
// With meas: the L2 cost of one-ray pixels and its adjoint weights; with
// weights (meas null): those ray weights (the gradient of sum_r w_r I_r).
// gradout [ng][nout]: extinction, albedo and (nout = 3, with pd) the phase.
bool levis_gradient(Solver<R> &S, int ipa, int n, const float *camx, const float *camy, const float *camz,
                    const double *cammu, const double *camphi, const float *meas, const double *weights,
                    double *gradout, double *cost, float *stokesout, int nthreads, const PhaseDeriv *pd = nullptr,
                    int nout = 2) {
  if (ipa < 0 || ipa >= S.npart) { S.err = "levis_gradient: bad species index"; return false; }
  if (S.nst != 1) { S.err = "levis_gradient: scalar problems only"; return false; }
  std::vector<float> own;
  if (!stokesout) { own.resize(n); stokesout = own.data(); }
  if (!S.render(n, camx, camy, camz, cammu, camphi, stokesout, nthreads)) return false;  // phase 1 (with phasetab, bcrad)
  Levis<R> L(S);
  if (pd && !L.set_phase(pd->ndphase, pd->nlegd, pd->dleg, pd->diph, S.err)) return false;
  if (!L.prepare(ipa, S.err)) return false;
  // phase 2: L2 adjoint weights and cost
  std::vector<double> adj(n);
  double c = 0.0;
  for (int i = 0; i < n; ++i) {
    if (meas) {
      const double e = (double)stokesout[i] - (double)meas[i];
      c += 0.5 * e * e;
      adj[i] = e;
    } else {
      adj[i] = weights[i];
    }
  }
  if (cost) *cost = c;
  // phase 3: adjoint rays (per-thread accumulators)
  const int nt = std::max(1, nthreads);
  const int ND = Levis<R>::NUMDER;
  std::vector<std::vector<double>> g(nt, std::vector<double>((size_t)L.ng * ND, 0.0)), bw(nt, std::vector<double>(S.npts, 0.0));
  std::vector<std::string> errs(nt);
  std::vector<int> bad(nt, 0);
  const double pi = std::acos(-1.0);
  auto work = [&](int t, int b, int e) {
    for (int iv = b; iv < e; ++iv) {
      double x0 = camx[iv], y0 = camy[iv], z0 = camz[iv], mu2 = cammu[iv], phi2 = camphi[iv];
      double muray = -mu2, phiray = phi2 - pi;
      if (z0 > S.zgrid[S.nz - 1]) {
        if (muray >= 0.0) continue;
        double r = (S.zgrid[S.nz - 1] - z0) / muray;
        x0 = x0 + r * std::sqrt(1 - muray * muray) * std::cos(phiray);
        y0 = y0 + r * std::sqrt(1 - muray * muray) * std::sin(phiray);
        z0 = S.zgrid[S.nz - 1];
      } else if (z0 < S.zgrid[0]) { bad[t] = 1; errs[t] = "LEVISAPPROX_GRADIENT: Level below domain"; return; }
      if (!L.adjoint_ray(mu2, phi2, x0, y0, z0, adj[iv], g[t], bw[t], errs[t])) { bad[t] = 1; return; }
    }
  };
  if (nt <= 1) work(0, 0, n);
  else {
    std::vector<std::thread> th;
    int chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t, std::min(n, t * chunk), std::min(n, (t + 1) * chunk));
    for (auto &x : th) x.join();
  }
  for (int t = 0; t < nt; ++t) if (bad[t]) { S.err = errs[t]; return false; }
  std::vector<double> G((size_t)L.ng * ND, 0.0), beam(S.npts, 0.0);
  for (int t = 0; t < nt; ++t) {
    for (size_t k = 0; k < G.size(); ++k) G[k] += g[t][k];
    for (int k = 0; k < S.npts; ++k) beam[k] += bw[t][k];
  }
  // phase 4: direct-beam derivative per grid point
  for (int ip = 0; ip < S.npts; ++ip)
    if (beam[ip] != 0.0) L.direct_beam_deriv(ip, beam[ip], G);
  for (int ib = 0; ib < L.ng; ++ib)
    for (int d = 0; d < nout; ++d) gradout[(size_t)ib * nout + d] = G[(size_t)ib * ND + d];
  return true;
}

struct Handle {
  int fp64 = 0;
  Solver<float> *s32 = nullptr;
  Solver<double> *s64 = nullptr;
  std::string err;
};

}  // namespace orc

using orc::Handle;

extern "C" {

void *oracle_create(const shdom_problem *p, int fp64) {
  Handle *h = new Handle();
  h->fp64 = fp64;
  bool ok;
  if (fp64) { h->s64 = new orc::Solver<double>(); ok = h->s64->init(p); if (!ok) h->err = h->s64->err; }
  else { h->s32 = new orc::Solver<float>(); ok = h->s32->init(p); if (!ok) h->err = h->s32->err; }
  return h;
}

const char *oracle_error(void *hv) {
  Handle *h = (Handle *)hv;
  if (!h->err.empty()) return h->err.c_str();
  if (h->fp64) return h->s64->err.c_str();
  return h->s32->err.c_str();
}

int oracle_sizes(void *hv, int *out) {
  Handle *h = (Handle *)hv;
  auto fill = [&](auto *s) {
    out[0] = s->npts; out[1] = s->nlm; out[2] = s->nmu; out[3] = s->nang; out[4] = s->ncells;
    out[5] = s->nx1; out[6] = s->ny1; out[7] = s->nz; out[8] = s->bcflag; out[9] = s->ipflag;
    out[10] = s->iter; out[11] = s->ml; out[12] = s->mm; out[13] = s->nst;
  };
  if (h->fp64) fill(h->s64); else fill(h->s32);
  return 0;
}

int oracle_solve(void *hv, int maxiter, int verbose, float *solcrit_out) {
  Handle *h = (Handle *)hv;
  auto run = [&](auto *s) -> int {
    if (s->source.empty()) { if (!s->init_solution()) return 1; }
    if (!s->solution_iterations(maxiter, verbose)) return 1;
    if (solcrit_out) *solcrit_out = (float)s->solcrit;
    return 0;
  };
  return h->fp64 ? run(h->s64) : run(h->s32);
}

int oracle_init_solution(void *hv) {
  Handle *h = (Handle *)hv;
  return h->fp64 ? !h->s64->init_solution() : !h->s32->init_solution();
}

// Exports the solution densely: source/radiance [npts][nstokes][nlm] (zero beyond
// the per-point truncation), ns/nr per point, fluxes [npts][2], dirflux.
int oracle_export(void *hv, float *source, int *ns, float *radiance, int *nr, float *fluxes, float *dirflux) {
  Handle *h = (Handle *)hv;
  auto ex = [&](auto *s) {
    int n = s->npts, L = s->nlm;
    for (int i = 0; i < n; ++i) {
      int is = s->shptr[i], k = s->shptr[i + 1] - is;
      if (ns) ns[i] = k;
      const int ns_ = s->nst;
      if (source)
        for (int q = 0; q < ns_; ++q)
          for (int j = 0; j < L; ++j)
            source[((size_t)i * ns_ + q) * L + j] = j < k ? (float)s->source[((size_t)is + j) * ns_ + q] : 0.f;
      int ir = s->rshptr[i], kr = s->rshptr[i + 1] - ir;
      if (nr) nr[i] = kr;
      if (radiance)
        for (int q = 0; q < ns_; ++q)
          for (int j = 0; j < L; ++j)
            radiance[((size_t)i * ns_ + q) * L + j] = j < kr ? (float)s->radiance[((size_t)ir + j) * ns_ + q] : 0.f;
      if (fluxes) { fluxes[2 * i] = (float)s->fluxes[2 * (size_t)i]; fluxes[2 * i + 1] = (float)s->fluxes[2 * (size_t)i + 1]; }
      if (dirflux) dirflux[i] = (float)s->dirflux[i];
    }
  };
  if (h->fp64) ex(h->s64); else ex(h->s32);
  return 0;
}

int oracle_set_render_options(void *hv, int single_scatter, int nosurface) {
  Handle *h = (Handle *)hv;
  if (h->fp64) { h->s64->rsingle = single_scatter != 0; h->s64->rnosfc = nosurface != 0; }
  else { h->s32->rsingle = single_scatter != 0; h->s32->rnosfc = nosurface != 0; }
  return 0;
}

int oracle_render(void *hv, int n, const float *camx, const float *camy, const float *camz, const double *cammu,
                  const double *camphi, float *out, int nthreads) {
  Handle *h = (Handle *)hv;
  bool ok = h->fp64 ? h->s64->render(n, camx, camy, camz, cammu, camphi, out, nthreads)
                    : h->s32->render(n, camx, camy, camz, cammu, camphi, out, nthreads);
  return ok ? 0 : 1;
}

// Levis approximate gradient (adjoint branch) of the L2 cost of n one-ray
// pixels with respect to the extinction and single-scattering albedo of
// species ipa (0-based) on the property grid: gradout [npx*npy*npz][2]
// (extinction, albedo), cost, and the rendered radiances.
int oracle_levis_gradient(void *hv, int ipa, int n, const float *camx, const float *camy, const float *camz,
                          const double *cammu, const double *camphi, const float *meas, double *gradout,
                          double *cost, float *stokesout, int nthreads) {
  Handle *h = (Handle *)hv;
  bool ok = h->fp64 ? orc::levis_gradient(*h->s64, ipa, n, camx, camy, camz, cammu, camphi, meas, nullptr, gradout, cost,
                                          stokesout, nthreads)
                    : orc::levis_gradient(*h->s32, ipa, n, camx, camy, camz, cammu, camphi, meas, nullptr, gradout, cost,
                                          stokesout, nthreads);
  return ok ? 0 : 1;
}

// The same adjoint pass with caller-supplied ray weights: the Levis
// gradient of sum_r w_r I_r, gradout [npx*npy*npz][2].
int oracle_levis_adjoint(void *hv, int ipa, int n, const float *camx, const float *camy, const float *camz,
                         const double *cammu, const double *camphi, const double *weights, double *gradout,
                         int nthreads) {
  Handle *h = (Handle *)hv;
  bool ok = h->fp64 ? orc::levis_gradient(*h->s64, ipa, n, camx, camy, camz, cammu, camphi, nullptr, weights, gradout,
                                          nullptr, nullptr, nthreads)
                    : orc::levis_gradient(*h->s32, ipa, n, camx, camy, camz, cammu, camphi, nullptr, weights, gradout,
                                          nullptr, nullptr, nthreads);
  return ok ? 0 : 1;
}

// The adjoint pass with the phase-derivative direction as a third unknown:
// gradout [npx*npy*npz][3] (extinction, albedo, phase).
int oracle_levis_adjoint_phase(void *hv, int ipa, int n, const float *camx, const float *camy, const float *camz,
                               const double *cammu, const double *camphi, const double *weights, int ndphase,
                               int nlegd, const float *dleg, const int *diph, double *gradout, int nthreads) {
  Handle *h = (Handle *)hv;
  orc::PhaseDeriv pd;
  pd.ndphase = ndphase; pd.nlegd = nlegd; pd.dleg = dleg; pd.diph = diph;
  bool ok = h->fp64 ? orc::levis_gradient(*h->s64, ipa, n, camx, camy, camz, cammu, camphi, nullptr, weights, gradout,
                                          nullptr, nullptr, nthreads, &pd, 3)
                    : orc::levis_gradient(*h->s32, ipa, n, camx, camy, camz, cammu, camphi, nullptr, weights, gradout,
                                          nullptr, nullptr, nthreads, &pd, 3);
  return ok ? 0 : 1;
}

int oracle_frozen_render_phase(void *hv, int ipa, int voxel, float eps, int nlegd, const float *dleg_row, float dext,
                               float dalb, int n, const float *camx, const float *camy, const float *camz,
                               const double *cammu, const double *camphi, float *out, int nthreads) {
  Handle *h = (Handle *)hv;
  bool ok = h->fp64 ? orc::frozen_render_phase(*h->s64, ipa, voxel, eps, nlegd, dleg_row, dext, dalb, n, camx, camy,
                                               camz, cammu, camphi, out, nthreads)
                    : orc::frozen_render_phase(*h->s32, ipa, voxel, eps, nlegd, dleg_row, dext, dalb, n, camx, camy,
                                               camz, cammu, camphi, out, nthreads);
  return ok ? 0 : 1;
}

int oracle_frozen_render(void *hv, int ipa, int voxel, float dext, float dalb, int n, const float *camx,
                         const float *camy, const float *camz, const double *cammu, const double *camphi, float *out,
                         int nthreads) {
  Handle *h = (Handle *)hv;
  bool ok = h->fp64 ? orc::frozen_render(*h->s64, ipa, voxel, dext, dalb, n, camx, camy, camz, cammu, camphi, out, nthreads)
                    : orc::frozen_render(*h->s32, ipa, voxel, dext, dalb, n, camx, camy, camz, cammu, camphi, out, nthreads);
  return ok ? 0 : 1;
}

int oracle_grid(void *hv, float *gridpos, int *gridptr, int *neighptr, short *cellflags) {
  Handle *h = (Handle *)hv;
  auto g = [&](auto *s) {
    if (gridpos) std::memcpy(gridpos, s->gridpos.data(), s->gridpos.size() * sizeof(float));
    if (gridptr) std::memcpy(gridptr, s->gridptr.data(), s->gridptr.size() * sizeof(int));
    if (neighptr) std::memcpy(neighptr, s->neighptr.data(), s->neighptr.size() * sizeof(int));
    if (cellflags) std::memcpy(cellflags, s->cellflags.data(), s->cellflags.size() * sizeof(short));
  };
  if (h->fp64) g(h->s64); else g(h->s32);
  return 0;
}

// The cell tree of an adaptive grid: treeptr [ncells][2] (parent or -1,
// first child or 0).
int oracle_tree(void *hv, int *treeptr) {
  Handle *h = (Handle *)hv;
  auto g = [&](auto *s) { std::memcpy(treeptr, s->treeptr.data(), s->treeptr.size() * sizeof(int)); };
  if (h->fp64) g(h->s64); else g(h->s32);
  return 0;
}

int oracle_angles(void *hv, float *mu, float *phi, float *wtdo, int *nphi0) {
  Handle *h = (Handle *)hv;
  auto g = [&](auto *s) {
    if (mu) std::memcpy(mu, s->mu.data(), s->mu.size() * sizeof(float));
    if (phi) std::memcpy(phi, s->phi.data(), s->phi.size() * sizeof(float));
    if (wtdo) std::memcpy(wtdo, s->wtdo.data(), s->wtdo.size() * sizeof(float));
    if (nphi0) std::memcpy(nphi0, s->nphi0.data(), s->nphi0.size() * sizeof(int));
  };
  if (h->fp64) g(h->s64); else g(h->s32);
  return 0;
}

void oracle_destroy(void *hv) {
  Handle *h = (Handle *)hv;
  delete h->s32; delete h->s64; delete h;
}

}  // extern "C"
