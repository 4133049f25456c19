// shdom_plan.cpp -- host-side planning for the GPU solve (see shdom_plan.h).
//
// Reference routines restated here (AT3D 4.1.3):
//   grid and cells        _setup_grid at3d/solver.py:2036-2168, NEW_GRIDS and
//                         INIT_CELL_STRUCTURE src/polarized/shdomsub2.f:16-310
//   sweep order           SWEEPING_ORDER / SWEEP_BASE_CELL
//                         src/polarized/shdomsub1.f:3261-3351, :4529-4622
//   ordinates, SH tables  MAKE_ANGLE_SET, GAUSQUADS, MAKE_SH_DO_COEF, PLMALL,
//                         YLMALL_UNPOL src/polarized/shdomsub2.f:1061-1220,
//                         :4874-4912, :4650-4755, :4497-4535
//   medium                TRILIN_INTERP_PROP src/polarized/shdom90.f90:17-350,
//                         PREPARE_PROP src/polarized/shdomsub2.f:479-611
//   direct beam           DIRECT_BEAM_PROP src/polarized/shdom90.f90:352-867
//   initial radiance      INIT_RADIANCE / EDDRTF / TRIDIAG
//                         src/polarized/shdomsub2.f:614-1058
//   single-scatter table  PRECOMPUTE_PHASE_CHECK src/polarized/shdomsub4.f:2388-2491
//
// The wavefront level schedule has no counterpart in the reference: the
// reference sweeps the points of one ordinate one at a time in SWEEPORD
// order, a point's trace stopping at the first face whose corners come
// earlier in that order.  Here level(P) = 1 + max level over every corner a
// trace from P can read for any ordinate of the octant, so all points of one
// level (and all ordinates) can run at once while every face a trace stops
// at is still "earlier" in the reference's sense.
#include "shdom_plan.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

namespace shdom {

namespace {
std::mutex g_pool_mu;
std::multimap<size_t, void *> g_pool;          // free blocks by size
size_t g_pool_bytes = 0;
constexpr size_t kPoolMin = size_t(1) << 20;   // smaller blocks use the ordinary heap
constexpr size_t kPoolKeep = size_t(4) << 30;  // bytes of free blocks kept at most
size_t pool_size(size_t bytes) { return (bytes + 65535) & ~size_t(65535); }
}  // namespace

void *host_block_alloc(size_t bytes) {
  if (bytes < kPoolMin) return ::operator new(bytes);
  const size_t sz = pool_size(bytes);
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pool.find(sz);
    if (it != g_pool.end()) {
      void *p = it->second;
      g_pool.erase(it);
      g_pool_bytes -= sz;
      return p;
    }
  }
  void *p = std::aligned_alloc(4096, sz);
  if (!p) throw std::bad_alloc();
  return p;
}

void host_block_free(void *p, size_t bytes) noexcept {
  if (!p) return;
  if (bytes < kPoolMin) { ::operator delete(p); return; }
  const size_t sz = pool_size(bytes);
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_pool.emplace(sz, p);
  g_pool_bytes += sz;
  while (g_pool_bytes > kPoolKeep) {  // drop the largest free blocks first
    auto it = std::prev(g_pool.end());
    g_pool_bytes -= it->first;
    std::free(it->second);
    g_pool.erase(it);
  }
}

namespace {

const int kGoodNFFT[256] = {
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

const int kFace[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};

template <class F>
void parallel_for(int n, F f) {
  int nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (n < 4096 || nt == 1) { f(0, n); return; }
  std::vector<std::thread> th;
  int chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    int b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) th.emplace_back(f, b, e);
  }
  for (auto &x : th) x.join();
}

// d^l_{m0}(x) * sqrt(l + 1/2), l = 0..lmax, by the standard upward recurrence
// in l started from the closed form at l = m.
void dm0(double x, int lmax, int m, std::vector<double> &d) {
  d.assign(lmax + 1, 0.0);
  if (m > lmax) return;
  if (m == 0) {
    d[0] = 1.0;
    if (lmax >= 1) d[1] = x;
    for (int n = 1; n < lmax; ++n) d[n + 1] = ((2 * n + 1) * x * d[n] - n * d[n - 1]) / (n + 1);
  } else {
    double c = 1.0;
    for (int k = 1; k <= m; ++k) c *= std::sqrt((double)(m + k) / (double)k);
    d[m] = ((m & 1) ? -c : c) * std::pow(0.5 * std::sqrt((1.0 - x) * (1.0 + x)), m);
    for (int n = m; n < lmax; ++n) {
      double prev = (n > m) ? std::sqrt((double)(n * n - m * m)) * d[n - 1] : 0.0;
      d[n + 1] = ((2 * n + 1) * x * d[n] - prev) / std::sqrt((double)((n + 1) * (n + 1) - m * m));
    }
  }
  for (int n = 0; n <= lmax; ++n) d[n] *= std::sqrt(n + 0.5);
}

inline int jidx(int l, int m, int mm) { return (l <= mm) ? l * (l + 1) + m : (2 * mm + 1) * l - mm * mm + m; }

// Wigner d^n_{m m1}(x) at its first degree n = max(m, m1) (m, m1 >= 0).
double wig_start(double x, int m, int m1) {
  if (m == m1) return std::pow(0.5 * (1.0 + x), m);
  const int hi = std::max(m, m1), lo = std::min(m, m1);
  double c = (m1 > m || ((m - m1) % 2 == 0)) ? 1.0 : -1.0;
  for (int q = 1; q <= hi - lo; ++q) c *= std::sqrt((double)(m + m1 + q) / q);
  return c * std::pow(std::sqrt(0.5 * (1.0 - x)), hi - lo) * std::pow(std::sqrt(0.5 * (1.0 + x)), hi + lo);
}

// d^n_{m m1}(x) for n = 0..lmax by the upward three-term recurrence in n.
void wig(double x, int lmax, int m, int m1, std::vector<double> &d) {
  d.assign(lmax + 1, 0.0);
  const int n0 = std::max(m, m1);
  if (n0 > lmax) return;
  if (n0 == 0) {
    d[0] = 1.0;
    if (lmax >= 1) d[1] = x;
    for (int n = 1; n < lmax; ++n) d[n + 1] = ((2 * n + 1) * x * d[n] - n * d[n - 1]) / (n + 1);
    return;
  }
  d[n0] = wig_start(x, m, m1);
  for (int n = n0; n < lmax; ++n) {
    const double a = std::sqrt((double)((n + 1) * (n + 1) - m * m)) * std::sqrt((double)((n + 1) * (n + 1) - m1 * m1));
    const double b = std::sqrt((double)(n * n - m * m)) * std::sqrt((double)(n * n - m1 * m1));
    d[n + 1] = ((n * (n + 1.0) * x - (double)m * m1) * (2 * n + 1) / n * d[n] - b * (n + 1.0) / n * (n > n0 ? d[n - 1] : 0.0)) / a;
  }
}

// The six generalized spherical functions of the mu part (PLMALL,
// src/polarized/shdomsub2.f:4650-4755) in the element order I-I, Q-Q, U-U,
// V-V, I-Q, Q-U: out [nlm][6].  With P1 = d^l_{m0}, P2 = -(d^l_{m2} +
// d^l_{m,-2})/2, P3 = -(d^l_{m2} - d^l_{m,-2})/2 (each times
// sqrt((2l+1)/(4 pi))), the m >= 0 terms hold (P1, P2, P2, P1, P3, P3) and
// the m < 0 terms (P1, P2, -P2, -P1, s P3, -s P3), s = -1 for the
// transposed (ordinate-to-harmonic) set.
void gen6_mu(bool transpose, double x, int ml, int mm, std::vector<double> &out) {
  const int nlm = (2 * mm + 1) * (ml + 1) - mm * (mm + 1);
  out.assign((size_t)nlm * 6, 0.0);
  const double fct = 1.0 / std::sqrt(2.0 * std::acos(-1.0)), sg = transpose ? -1.0 : 1.0;
  std::vector<double> d0, dp, dm;
  for (int m = 0; m <= mm; ++m) {
    dm0(x, ml, m, d0);
    wig(x, ml, m, 2, dp);
    wig(-x, ml, m, 2, dm);
    for (int l = m; l <= ml; ++l) {
      const double nrm = std::sqrt(l + 0.5), dpl = dp[l] * nrm, dml = (((l + m) & 1) ? -1.0 : 1.0) * dm[l] * nrm;
      const double p1 = fct * d0[l], p2 = -0.5 * fct * (dpl + dml), p3 = -0.5 * fct * (dpl - dml);
      double *o = &out[(size_t)jidx(l, m, mm) * 6];
      o[0] = p1; o[1] = p2; o[2] = p2; o[3] = p1; o[4] = p3; o[5] = p3;
      if (m == 0) continue;
      double *n = &out[(size_t)jidx(l, -m, mm) * 6];
      n[0] = p1; n[1] = p2; n[2] = -p2; n[3] = -p1; n[4] = sg * p3; n[5] = -sg * p3;
    }
  }
}

}  // namespace

void ylm_unpol(int ml, int mm, double mu, float phi, float *y) {
  std::vector<double> d;
  const double fct = 1.0 / std::sqrt(2.0 * std::acos(-1.0));
  double x = (double)(float)mu;
  for (int m = 0; m <= mm; ++m) {
    dm0(x, ml, m, d);
    double c = 1, s = 0;
    if (m > 0) { c = std::cos(m * (double)phi); s = std::sin(m * (double)phi); }
    for (int l = m; l <= ml; ++l) {
      double v = fct * d[l];
      int j = jidx(l, m, mm);
      y[j] = (float)((c - s) * v);
      y[j - 2 * m] = (float)((c + s) * v);
    }
  }
}


// Band integral of Planck's law (INTEGRATE_PLANCK, src/polarized/shdomsub2.f:
// 4795-4873): F = integral of x^3/(e^x - 1) between x1 < x2, from the series
// x^3/(e^x - 1) = x^2 sum_n B_n x^n / n! below x = 1 (Bernoulli numbers,
// terms through x^29) and sum_n e^(-n x) (x^3/n + 3x^2/n^2 + 6x/n^3 + 6/n^4)
// (15 terms) for the tail above it.
static double planck_int_low(double x) {
  // coefficient of x^k, built once (thread-safe static initialisation)
  static const std::array<double, 30> coef = [] {
    std::array<double, 30> c{};
    double b[28], bin[30][30];
    for (int n = 0; n < 30; ++n) { bin[n][0] = bin[n][n] = 1.0; for (int k = 1; k < n; ++k) bin[n][k] = bin[n - 1][k - 1] + bin[n - 1][k]; }
    b[0] = 1.0;
    for (int m = 1; m < 27; ++m) { double s = 0; for (int k = 0; k < m; ++k) s += bin[m + 1][k] * b[k]; b[m] = -s / (m + 1); }
    double fact = 1.0;
    for (int n = 0; n + 3 < 30; ++n) { if (n > 0) fact *= n; c[n + 3] = b[n] / (fact * (n + 3)); }
    return c;
  }();
  double s = coef[4] * x * x * x * x, f = x;
  for (int k = 3; k <= 29; k += 2) { f *= x * x; s += coef[k] * f; }
  return s;
}
static double planck_int_high(double x) {
  double s = 0.0;
  for (int n = 1; n <= 15; ++n)
    s += std::exp(-n * x) * (x * x * x / n + 3 * x * x / ((double)n * n) + 6 * x / ((double)n * n * n) + 6.0 / ((double)n * n * n * n));
  return s;
}
static double planck_band(double x1, double x2) {
  const double c = 1.0;
  if (x1 < c && x2 < c) return planck_int_low(x2) - planck_int_low(x1);
  if (x1 < c) return planck_int_low(c) - planck_int_low(x1) + planck_int_high(c) - planck_int_high(x2);
  return planck_int_high(x1) - planck_int_high(x2);
}

// PLANCK_FUNCTION (src/polarized/shdomsub2.f:4756-4791): Planck's law in
// SHDOM's units and single precision, c1 = 1.1911e8 W um^4/(m^2 sr),
// c2 = 1.4388e4 um K; units 'B' integrate it over the band waveno (cm^-1).
float planck_fn(float t, char units, float wavelen, const float *waveno) {
  if (units == 'T') return t;
  if (t <= 0.f) return 0.f;
  if (units == 'B') {
    const double x1 = 1.4388 * waveno[0] / t, x2 = 1.4388 * waveno[1] / t;
    return (float)(1.1911e-8 * std::pow(t / 1.4388, 4) * planck_band(x1, x2));
  }
  const float w = wavelen;
  return 1.1911e8f / (w * w * w * w * w) / (std::exp(1.4388e4f / (w * t)) - 1.0f);
}

namespace {

bool build_grid(const shdom_problem &p, Plan &P) {
  P.nx = std::max(1, p.npx); P.ny = std::max(1, p.npy); P.nz = std::max(2, p.npz);
  int ip = p.ipflag;
  if (P.nx == 1) ip |= 1;
  if (P.ny == 1) ip |= 2;
  P.ipflag = ip;
  int bc = 0;
  if (p.bc_x_open && (ip == 0 || ip == 2 || ip == 4 || ip == 6)) bc += 1;
  if (p.bc_y_open && (ip == 0 || ip == 1 || ip == 4 || ip == 5)) bc += 2;
  P.bcflag = bc;
  if (bc == 1) { P.err = "open x with periodic y boundary conditions is not supported"; return false; }
  if ((ip & 3) == 1 || (ip & 3) == 2) { P.err = "2D independent pixel mode (ip_flag 1 or 2) is not supported"; return false; }
  P.is1d = (ip & 3) == 3;
  P.noct = P.is1d ? 2 : 8;
  int nx = P.nx, ny = P.ny, nz = P.nz;
  P.nx1 = nx + 1; P.ny1 = ny + 1;
  if ((bc & 5) || (ip & 1)) P.nx1 -= 1;
  if ((bc & 7) || (ip & 2)) P.ny1 -= 1;
  float dxp = p.delx > 0 ? p.delx : 1.f, dyp = p.dely > 0 ? p.dely : 1.f;
  P.xgrid.resize(nx + 1); P.ygrid.resize(ny + 1);
  for (int i = 0; i <= nx; ++i) P.xgrid[i] = ((float)i * (dxp * (float)p.npx)) / (float)nx;
  for (int i = 0; i <= ny; ++i) P.ygrid[i] = ((float)i * (dyp * (float)p.npy)) / (float)ny;
  P.zgrid.assign(p.zlevels, p.zlevels + p.npz);
  P.npts = P.nx1 * P.ny1 * nz;
  P.gridpos.mut().resize((size_t)P.npts * 3);
  for (int ix = 0, i = 0; ix < P.nx1; ++ix)
    for (int iy = 0; iy < P.ny1; ++iy)
      for (int iz = 0; iz < nz; ++iz, ++i) {
        P.gridpos.mut()[3 * i] = P.xgrid[ix]; P.gridpos.mut()[3 * i + 1] = P.ygrid[iy]; P.gridpos.mut()[3 * i + 2] = P.zgrid[iz];
      }
  int nxc = (bc & 1) ? nx + 1 : nx, nyc = (bc & 2) ? ny + 1 : ny;
  P.ncells = nxc * nyc * (nz - 1);
  P.gridptr.assign((size_t)P.ncells * 8, 0);
  P.neighptr.assign((size_t)P.ncells * 6, -1);
  P.cellflags.assign(P.ncells, 0);
  int ic = 0;
  for (int ix = 1; ix <= nxc; ++ix) {
    int x0, x1;
    if (ip & 1) { x0 = x1 = ix; } else if (bc & 1) { x0 = std::max(1, ix - 1); x1 = std::min(nx, ix); } else { x0 = ix; x1 = ix + 1; }
    for (int iy = 1; iy <= nyc; ++iy) {
      int y0, y1;
      if (ip & 2) { y0 = y1 = iy; } else if (bc & 2) { y0 = std::max(1, iy - 1); y1 = std::min(ny, iy); } else { y0 = iy; y1 = iy + 1; }
      for (int iz = 1; iz < nz; ++iz, ++ic) {
        auto pt = [&](int z, int y, int x) { return (z - 1) + nz * (y - 1) + nz * P.ny1 * (x - 1); };
        int *g = &P.gridptr.mut()[8 * (size_t)ic];
        g[0] = pt(iz, y0, x0); g[1] = pt(iz, y0, x1); g[2] = pt(iz, y1, x0); g[3] = pt(iz, y1, x1);
        g[4] = pt(iz + 1, y0, x0); g[5] = pt(iz + 1, y0, x1); g[6] = pt(iz + 1, y1, x0); g[7] = pt(iz + 1, y1, x1);
        int *nb = &P.neighptr.mut()[6 * (size_t)ic];
        int sx = (nz - 1) * nyc, sy = nz - 1;
        if (ip & 1) { nb[0] = nb[1] = ic; P.cellflags.mut()[ic] |= 1; }
        else if (bc & 1) {
          nb[0] = (ix == 1) ? ic : ic - sx;
          nb[1] = (ix == nxc) ? ic : ic + sx;
          if (ix == 1 || ix == nxc) P.cellflags.mut()[ic] |= 1;
        } else {
          nb[0] = (ix == 1) ? ic + (nxc - 1) * sx : ic - sx;
          nb[1] = (ix == nx) ? ic - (nxc - 1) * sx : ic + sx;
        }
        if (ip & 2) { nb[2] = nb[3] = ic; P.cellflags.mut()[ic] |= 2; }
        else if (bc & 2) {
          nb[2] = (iy == 1) ? ic : ic - sy;
          nb[3] = (iy == nyc) ? ic : ic + sy;
          if (iy == 1 || iy == nyc) P.cellflags.mut()[ic] |= 2;
        } else {
          nb[2] = (iy == 1) ? ic + (nyc - 1) * sy : ic - sy;
          nb[3] = (iy == ny) ? ic - (nyc - 1) * sy : ic + sy;
        }
        nb[4] = (iz == 1) ? -1 : ic - 1;
        nb[5] = (iz == nz - 1) ? -1 : ic + 1;
      }
    }
  }
  P.bnd.assign(P.npts, 0);
  for (int i = 0; i < P.npts; ++i) {
    if (P.gridpos[3 * i + 2] >= P.zgrid[nz - 1]) { P.bnd[i] |= 1; P.topp.push_back(i); }
    if (P.gridpos[3 * i + 2] <= P.zgrid[0]) { P.bnd[i] |= 2; P.botp.push_back(i); }
  }
  return true;
}

// The reference's visiting order of grid points for one trace octant, as a
// rank per point and the cell through which the point was first reached.
void sweep_order(Plan &P, int ioct) {
  int nx = P.nx, ny = P.ny, nz = P.nz, bc = P.bcflag;
  int nxc = (bc & 1) ? nx + 1 : nx, nyc = (bc & 2) ? ny + 1 : ny;
  int b = ioct - 1;
  int six, eix, dix, siy, eiy, diy, siz, eiz, diz;
  if (b & 1) { dix = 1; if (bc & 1) { six = nxc; eix = std::max(nxc - 1, 1); } else { six = 1; eix = nxc; } }
  else { dix = -1; if (bc & 1) { six = 1; eix = std::min(2, nxc); } else { six = nxc; eix = 1; } }
  if (b & 2) { diy = 1; if (bc & 2) { siy = nyc; eiy = std::max(nyc - 1, 1); } else { siy = 1; eiy = nyc; } }
  else { diy = -1; if (bc & 2) { siy = 1; eiy = std::min(2, nyc); } else { siy = nyc; eiy = 1; } }
  if (b & 4) { diz = 1; siz = 1; eiz = nz - 1; } else { diz = -1; siz = nz - 1; eiz = 1; }
  int *rk = &P.rank.mut()[(size_t)b * P.npts];
  int *sc = &P.startcell.mut()[(size_t)b * P.npts];
  std::fill(rk, rk + P.npts, -1);
  int order = 0, ix = six, iy = siy, iz = siz;
  while (true) {
    int cell = (iz - 1) + (nz - 1) * (iy - 1) + (nz - 1) * nyc * (ix - 1);
    for (int k = 0; k < 8; ++k) {
      int corner = (k ^ b) ^ 7;  // furthest upstream corner first
      int pt = P.gridptr[8 * (size_t)cell + corner];
      if (rk[pt] >= 0) continue;
      rk[pt] = order++;
      sc[pt] = cell;
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

// Trace back from point pt along one ordinate with the reference's validity
// rule (a face is usable when all four corners precede pt in the sweep order
// or are preset boundary points); returns the corners of the stopping face.
bool trace_final_face(const Plan &P, int ioct, int pt, double cx, double cy, double cz, int hemi_bnd,
                      double transmin, int face_out[4]) {
  const int b = ioct - 1;
  const int *rk = &P.rank[(size_t)b * P.npts];
  double cxinv = cx != 0 ? 1.0 / cx : 1e6, cyinv = cy != 0 ? 1.0 / cy : 1e6, czinv = 1.0 / cz;
  int bitx = cx < 0, bity = cy < 0, bitz = cz < 0;
  int cell = P.startcell[(size_t)b * P.npts + pt];
  double xe = P.gridpos[3 * pt], ye = P.gridpos[3 * pt + 1], ze = P.gridpos[3 * pt + 2];
  double transmit = 1.0;
  const float *gp = P.gridpos.data();
  for (int guard = 0; guard < 1000000; ++guard) {
    if (cell < 0) return false;
    if (P.is1d) {
      int iface = 5 - bitz;
      int i1 = P.gridptr[8 * (size_t)cell + (iface == 4 ? 0 : 4)];
      int nxt = P.neighptr[6 * (size_t)cell + iface];
      if ((P.bnd[i1] & hemi_bnd) || rk[i1] < rk[pt]) { face_out[0] = face_out[1] = face_out[2] = face_out[3] = i1; return true; }
      cell = nxt;
      continue;
    }
    bool ipinx = P.cellflags[cell] & 1, ipiny = P.cellflags[cell] & 2;
    int iopp = P.gridptr[8 * (size_t)cell + (8 - ioct)];
    double sox = ipinx ? 1e20 : (gp[3 * iopp] - xe) * cxinv;
    double soy = ipiny ? 1e20 : (gp[3 * iopp + 1] - ye) * cyinv;
    double soz = (gp[3 * iopp + 2] - ze) * czinv;
    double so = std::min(sox, std::min(soy, soz));
    xe += so * cx; ye += so * cy; ze += so * cz;
    int iface, jface;
    if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; }
    else if (soy <= soz) { iface = 3 - bity; jface = 1; }
    else { iface = 5 - bitz; jface = 2; }
    int nxt = P.neighptr[6 * (size_t)cell + iface];
    int f[4];
    for (int k = 0; k < 4; ++k) f[k] = P.gridptr[8 * (size_t)cell + kFace[iface][k]];
    if (nxt >= 0) {
      int q = P.gridptr[8 * (size_t)nxt + ioct - 1];
      if (jface == 0) xe = gp[3 * q]; else if (jface == 1) ye = gp[3 * q + 1]; else ze = gp[3 * q + 2];
    }
    bool valid = true;
    for (int k = 0; k < 4; ++k) valid = valid && ((P.bnd[f[k]] & hemi_bnd) || rk[f[k]] < rk[pt]);
    if (nxt < 0 || (transmit <= transmin && valid)) {
      if (!valid) return false;
      for (int k = 0; k < 4; ++k) face_out[k] = f[k];
      return true;
    }
    cell = nxt;
  }
  return false;
}

void trace_dir(float mu, float phi, double &cx, double &cy, double &cz) {
  const double pi = (double)(float)std::acos(-1.0f);
  double s = (double)std::sqrt(1.0f - mu * mu);
  cx = s * std::cos((double)phi + pi);
  cy = s * std::sin((double)phi + pi);
  cz = -(double)mu;
  if (std::fabs(cx) <= 1.0e-5) cx = 0;
  if (std::fabs(cy) <= 1.0e-5) cy = 0;
}

int trace_octant(float mu, float phi, int is1d) {
  double cx, cy, cz;
  trace_dir(mu, phi, cx, cy, cz);
  int bz = cz < 0;
  if (is1d) return 1 + 4 * bz;
  return 1 + (cx < 0) + 2 * (cy < 0) + 4 * bz;
}

// Exit of a trace that starts at corner b of a full interior cell of size
// (dx, dy, dz) and leaves through the far side, with the same
// single-precision steps as the device trace: path length so, bilinear face
// coordinates (u, v) and the face index (0/1 x, 2/3 y, 4/5 z).
int regular_exit(float cx, float cy, float cz, int b, float dx, float dy, float dz, float &so, float &u, float &v) {
  const float cxinv = cx != 0.f ? 1.f / cx : 1.0e6f, cyinv = cy != 0.f ? 1.f / cy : 1.0e6f, czinv = 1.f / cz;
  const int bitx = cx < 0.f, bity = cy < 0.f, bitz = cz < 0.f;
  auto pos = [&](int k, float &x, float &y, float &z) { x = (k & 1) * dx; y = ((k >> 1) & 1) * dy; z = ((k >> 2) & 1) * dz; };
  float xe, ye, ze, xo, yo, zo;
  pos(b, xe, ye, ze);
  pos(7 - b, xo, yo, zo);
  float sox = (xo - xe) * cxinv, soy = (yo - ye) * cyinv, soz = (zo - ze) * czinv;
  so = std::min(sox, std::min(soy, soz));
  xe += so * cx; ye += so * cy; ze += so * cz;
  int iface, jface;
  if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; }
  else if (soy <= soz) { iface = 3 - bity; jface = 1; }
  else { iface = 5 - bitz; jface = 2; }
  float x1, y1, z1, x2, y2, z2, x3, y3, z3;
  pos(kFace[iface][0], x1, y1, z1); pos(kFace[iface][1], x2, y2, z2); pos(kFace[iface][2], x3, y3, z3);
  if (jface == 0) { u = (ze - z1) / (z3 - z1); v = (ye - y1) / (y2 - y1); }
  else if (jface == 1) { u = (ze - z1) / (z3 - z1); v = (xe - x1) / (x2 - x1); }
  else { u = (ye - y1) / (y3 - y1); v = (xe - x1) / (x2 - x1); }
  return iface;
}

// Padding ordinates per (octant, class) group (0: groups packed).  The
// device code handles padding ordinates (zero direction and weight) in
// every kernel, so the layout can be changed here alone.
constexpr int kColumnPad = 0;

void build_angles(const shdom_problem &p, Plan &P) {
  P.nmu = std::max(2, 2 * ((p.nmu + 1) / 2));
  P.nphi = std::max(1, p.nphi);
  P.ml = P.nmu - 1;
  P.mm = std::max(0, P.nphi / 2 - 1);
  P.nlm = (2 * P.mm + 1) * (P.ml + 1) - P.mm * (P.mm + 1);
  P.nleg = p.deltam ? P.ml + 1 : P.ml;
  P.nphi0max = P.nphi;
  P.lofj.resize(P.nlm); P.mofj.resize(P.nlm);
  for (int l = 0, j = 0; l <= P.ml; ++l)
    for (int m = -std::min(l, P.mm); m <= std::min(l, P.mm); ++m, ++j) { P.lofj[j] = l; P.mofj[j] = m; }
  int nmu = P.nmu, k = nmu / 2;
  P.mu.resize(nmu); P.wtmu.resize(nmu);
  for (int j = 1; j <= k; ++j) {  // Gauss-Legendre nodes by Newton iteration
    double x = std::cos(3.141592654 * (j - .25) / (nmu + .5)), xp, pl, pl1, pl2, dpl;
    int it = 0;
    do {
      pl1 = 1; pl = x;
      for (int l = 2; l <= nmu; ++l) { pl2 = pl1; pl1 = pl; pl = ((2 * l - 1) * x * pl1 - (l - 1) * pl2) / l; }
      dpl = nmu * (x * pl - pl1) / (x * x - 1);
      xp = x; x = xp - pl / dpl; ++it;
    } while (std::fabs(x - xp) > 3.0e-7 && it < 10);
    P.mu[j - 1] = (float)-x; P.mu[j - 1 + k] = (float)x;
    P.wtmu[j - 1] = P.wtmu[j - 1 + k] = (float)(2.0 / ((1.0 - x * x) * dpl * dpl));
  }
  P.nphi0.resize(nmu);
  P.phi.assign((size_t)nmu * P.nphi0max, 0.f); P.wtdo.assign((size_t)nmu * P.nphi0max, 0.f);
  const float pif = (float)std::acos(-1.0f);
  P.nang = 0;
  for (int j = 0; j < nmu; ++j) {
    if (p.angle_set == 1) P.nphi0[j] = P.nphi0max;
    else {
      int n = (int)(0.9f + (float)P.nphi0max * std::sqrt(1.0f - P.mu[j] * P.mu[j]));
      P.nphi0[j] = std::min(P.nphi0max, kGoodNFFT[std::max(1, std::min(256, n)) - 1]);
    }
    float dphi = 2.0f * pif / (float)P.nphi0[j];
    for (int q = 0; q < P.nphi0[j]; ++q) {
      P.phi[(size_t)j * P.nphi0max + q] = (float)q * dphi;
      P.wtdo[(size_t)j * P.nphi0max + q] = dphi * P.wtmu[j];
    }
    P.nang += P.nphi0[j];
  }
  // Face class of each ordinate: the face through which a trace from a
  // regular point leaves its cell, when it is the same kind (x, y or z) in
  // every layer; class 3 otherwise (and for 1D and single-column grids).
  auto face_class = [&](int j, int q) {
    if (P.is1d || P.nx1 < 2 || P.ny1 < 2 || P.nz < 2) return 3;
    double dcx, dcy, dcz;
    trace_dir(P.mu[j], P.phi[(size_t)j * P.nphi0max + q], dcx, dcy, dcz);
    const float cx = (float)dcx, cy = (float)dcy, cz = (float)dcz;
    const int b = (cx < 0.f) + 2 * (cy < 0.f) + 4 * (cz < 0.f);
    const float dx = P.xgrid[1] - P.xgrid[0], dy = P.ygrid[1] - P.ygrid[0];
    int mask = 0;
    for (int L = 0; L + 1 < P.nz; ++L) {
      float so, u, v;
      mask |= 1 << (regular_exit(cx, cy, cz, b, dx, dy, P.zgrid[L + 1] - P.zgrid[L], so, u, v) / 2);
    }
    return mask == 1 ? 0 : mask == 2 ? 1 : mask == 4 ? 2 : 3;
  };
  // column order: hemisphere, trace octant, face class, (imu, iphi)
  P.col_of.assign((size_t)nmu * P.nphi0max, -1);
  int col = 0;
  for (int hemi = 0; hemi < 2; ++hemi) {
    if (hemi == 1) P.ncol_down = col;
    for (int ioct = 1; ioct <= 8; ++ioct) {
      if (((ioct - 1) >> 2 & 1) != hemi) continue;  // bitz=1 traces down: upward ordinates
      P.oct_col0[ioct - 1] = col;
      for (int cls = 0; cls < 4; ++cls) {
        P.cls_col0[ioct - 1][cls] = col;
        for (int j = (hemi ? k : 0); j < (hemi ? nmu : k); ++j)
          for (int q = 0; q < P.nphi0[j]; ++q) {
            if (trace_octant(P.mu[j], P.phi[(size_t)j * P.nphi0max + q], P.is1d) != ioct) continue;
            if (face_class(j, q) != cls) continue;
            P.col_of[(size_t)j * P.nphi0max + q] = col++;
            P.col_imu.push_back(j); P.col_iphi.push_back(q); P.col_oct.push_back(ioct); P.col_cls.push_back(cls);
          }
        P.cls_ncol[ioct - 1][cls] = col - P.cls_col0[ioct - 1][cls];
        // (Padding each group to whole 32-byte sectors was measured: fewer
        // partly written sectors in the sweep, but 24% wider transforms; a
        // net loss at NMU=16, so the groups are packed.)
        for (int pad = 0; pad < kColumnPad && P.cls_ncol[ioct - 1][cls] > 0 && (col - P.cls_col0[ioct - 1][cls]) % 8 != 0; ++pad) {
          ++col;
          P.col_imu.push_back(-1); P.col_iphi.push_back(-1); P.col_oct.push_back(ioct); P.col_cls.push_back(cls);
        }
      }
      P.oct_ncol[ioct - 1] = col - P.oct_col0[ioct - 1];
    }
  }
  P.nang_real = P.nang;
  P.nang = col;  // columns including the padding ordinates
  P.col_cx.assign(P.nang, 0.f); P.col_cy.assign(P.nang, 0.f); P.col_cz.assign(P.nang, 0.f);
  P.col_fluxw.assign(P.nang, 0.f);
  for (int c = 0; c < P.nang; ++c) {
    int j = P.col_imu[c], q = P.col_iphi[c];
    if (j < 0) continue;  // padding: zero direction and weight
    double cx, cy, cz;
    trace_dir(P.mu[j], P.phi[(size_t)j * P.nphi0max + q], cx, cy, cz);
    P.col_cx[c] = (float)cx; P.col_cy[c] = (float)cy; P.col_cz[c] = (float)cz;
    P.col_fluxw[c] = std::fabs(P.mu[j]) * P.wtdo[(size_t)j * P.nphi0max + q];
  }
  // transform coefficients
  int nlm = P.nlm, mm = P.mm, nm = 2 * mm + 1;
  P.cmu1.assign((size_t)nmu * nlm, 0.f); P.cmu2.assign((size_t)nmu * nlm, 0.f);
  std::vector<double> d;
  const double fct = 1.0 / std::sqrt(2.0 * std::acos(-1.0));
  for (int i = 0; i < nmu; ++i)
    for (int m = 0; m <= mm; ++m) {
      dm0((double)P.mu[i], P.ml, m, d);
      for (int l = m; l <= P.ml; ++l) {
        float v = (float)(fct * d[l]);
        for (int s : {m, -m}) {
          int j = jidx(l, s, mm);
          P.cmu1[(size_t)i * nlm + j] = v;
          P.cmu2[(size_t)i * nlm + j] = v * P.wtmu[i];
        }
      }
    }
  if (p.nstokes == 3) {  // MAKE_SH_DO_COEF: CMU1 = PLMALL(.FALSE.), CMU2 = PLMALL(.TRUE.) * WTMU
    P.cmu1p.assign((size_t)nmu * nlm * 6, 0.f); P.cmu2p.assign((size_t)nmu * nlm * 6, 0.f);
    std::vector<double> g;
    for (int i = 0; i < nmu; ++i) {
      gen6_mu(false, (double)P.mu[i], P.ml, mm, g);
      for (int q = 0; q < nlm * 6; ++q) P.cmu1p[(size_t)i * nlm * 6 + q] = (float)g[q];
      gen6_mu(true, (double)P.mu[i], P.ml, mm, g);
      for (int q = 0; q < nlm * 6; ++q) P.cmu2p[(size_t)i * nlm * 6 + q] = (float)g[q] * P.wtmu[i];
    }
  }
  P.cphi1.assign((size_t)nmu * P.nphi0max * nm, 0.f); P.cphi2.assign((size_t)nmu * P.nphi0max * nm, 0.f);
  for (int i = 0; i < nmu; ++i) {
    float w = 1.0f / P.wtmu[i];
    for (int q = 0; q < P.nphi0[i]; ++q) {
      float *c1 = &P.cphi1[((size_t)i * P.nphi0max + q) * nm + mm];
      float *c2 = &P.cphi2[((size_t)i * P.nphi0max + q) * nm + mm];
      float wd = P.wtdo[(size_t)i * P.nphi0max + q], ph = P.phi[(size_t)i * P.nphi0max + q];
      c1[0] = 1.f; c2[0] = wd * w;
      for (int m = 1; m <= mm; ++m) {
        c1[m] = std::cos((float)m * ph); c1[-m] = std::sin((float)m * ph);
        c2[m] = c1[m] * wd * w; c2[-m] = c1[-m] * wd * w;
      }
    }
  }
}

bool build_medium(const shdom_problem &p, Plan &P) {
  P.ylmsun.resize(P.nlm);
  ylm_unpol(P.ml, P.mm, (double)p.solarmu, p.solaraz, P.ylmsun.data());
  const int npx = p.npx, npy = p.npy, npz = p.npz, ng = npx * npy * npz;
  const int npart = p.npart, nmic = p.maxnmicro, nq = 8 * nmic, npts = P.npts, nleg = P.nleg, ml = P.ml;
  P.npart = npart; P.numphase = p.numphase;
  // input table: [numphase][nlegp+1], or [numphase][nlegp+1][6] (a1 a2 a3 a4 b1 b2) when polarized
  const int nstleg = p.nstokes == 3 ? 6 : 1;
  auto legin = [&](int i, int l, int k) { return p.legenp[((size_t)i * (p.nlegp + 1) + l) * nstleg + k]; };
  // Legendre table divided by 2l+1; with delta-M the 0..ML terms hold
  // chi_l - f (the 'N' interpolation method keeps f in term ML+1).
  std::vector<float> leg((size_t)p.numphase * (nleg + 1), 0.f);
  for (int i = 0; i < p.numphase; ++i) {
    for (int l = 0; l <= nleg && l <= p.nlegp; ++l)
      leg[(size_t)i * (nleg + 1) + l] = legin(i, l, 0) / (float)(2 * l + 1);
    if (p.deltam) {
      float f = leg[(size_t)i * (nleg + 1) + ml + 1];
      for (int l = 0; l <= ml; ++l) leg[(size_t)i * (nleg + 1) + l] -= f;
    }
  }
  // polarized elements a2, a3, b1 (PREPARE_PROP 'N': the diagonal elements
  // lose f, the off-diagonal b1 is kept), [numphase][3][nleg+1]
  std::vector<float> legp3;
  if (nstleg == 6) {
    legp3.assign((size_t)p.numphase * 3 * (nleg + 1), 0.f);
    const int kel[3] = {1, 2, 4};
    for (int i = 0; i < p.numphase; ++i)
      for (int e = 0; e < 3; ++e) {
        float *L = &legp3[((size_t)i * 3 + e) * (nleg + 1)];
        for (int l = 0; l <= nleg && l <= p.nlegp; ++l) L[l] = legin(i, l, kel[e]) / (float)(2 * l + 1);
        if (p.deltam && e < 2) {
          const float f = leg[(size_t)i * (nleg + 1) + ml + 1];
          for (int l = 0; l <= ml; ++l) L[l] -= f;
        }
      }
  }
  for (int k = 0; k < ng * npart * nmic; ++k)
    if (p.iphasep[k] < 1 || p.iphasep[k] > p.numphase) { P.err = "Phase function indices are out of bounds."; return false; }
  const float zspan = p.zlevels[npz - 1] - p.zlevels[0];
  const double extmin = (double)(1.0e-5f / (zspan / (float)npz)), scatmin = 0.1 * extmin;
  // every element of these is written by the interpolation pass
  HostVec<float> &ext = P.sp_ext, &alb = P.sp_alb;  // the delta-M scaled species properties, kept for the gradient
  ext.clear(); ext.resize((size_t)npart * npts);
  alb.clear(); alb.resize((size_t)npart * npts);
  HostVec<int> iph((size_t)npart * npts * nq);
  HostVec<float> pw((size_t)npart * npts * nq);
  P.total_ext.assign(npts, 0.f);
  const bool therm = P.srct != 'S';
  HostVec<float> temp(therm ? npts : 0);  // TEMP of the grid points (TRILIN_INTERP_PROP)
  bool bad = false;
  for (int ipa = 0; ipa < npart; ++ipa) {
    parallel_for(npts, [&](int b, int e) {
      std::vector<std::pair<float, int>> srt(nq);
      for (int ipt = b; ipt < e; ++ipt) {
        float x = P.gridpos[3 * ipt], y = P.gridpos[3 * ipt + 1], z = P.gridpos[3 * ipt + 2];
        int il = 0, iu = npz;
        while (iu - il > 1) { int im = (iu + il) / 2; if (z >= p.zlevels[im - 1]) il = im; else iu = im; }
        int iz = std::max(il, 1);
        double w = std::max(0.0, std::min(1.0, (double)(z - p.zlevels[iz - 1]) / (p.zlevels[iz] - p.zlevels[iz - 1])));
        int ix = (int)(x / p.delx) + 1;
        if (std::fabs(x - npx * p.delx) < 0.01f * p.delx) ix = npx;
        int iy = (int)(y / p.dely) + 1;
        if (std::fabs(y - npy * p.dely) < 0.01f * p.dely) iy = npy;
        if (ix < 1 || ix > npx || iy < 1 || iy > npy) { bad = true; continue; }
        int ixp = ix % npx + 1, iyp = iy % npy + 1;
        double u = std::max(0.0, std::min(1.0, (double)(x - p.delx * (ix - 1)) / p.delx));
        if (u < 1e-5) u = 0;
        if (u > 1 - 1e-5) u = 1;
        double v = std::max(0.0, std::min(1.0, (double)(y - p.dely * (iy - 1)) / p.dely));
        if (v < 1e-5) v = 0;
        if (v > 1 - 1e-5) v = 1;
        double f[8] = {(1 - u) * (1 - v) * (1 - w), u * (1 - v) * (1 - w), (1 - u) * v * (1 - w), u * v * (1 - w),
                       (1 - u) * (1 - v) * w,       u * (1 - v) * w,       (1 - u) * v * w,       u * v * w};
        int i1 = (iz - 1) + npz * (iy - 1) + npz * npy * (ix - 1), i2 = (iz - 1) + npz * (iy - 1) + npz * npy * (ixp - 1);
        int i3 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ix - 1), i4 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ixp - 1);
        int ii[8] = {i1, i2, i3, i4, i1 + 1, i2 + 1, i3 + 1, i4 + 1};
        const float *E = p.extinctp + (size_t)ipa * ng, *A = p.albedop + (size_t)ipa * ng;
        double e = 0, sc[8], scat = 0;
        for (int c = 0; c < 8; ++c) { e += f[c] * E[ii[c]]; sc[c] = f[c] * E[ii[c]] * A[ii[c]]; scat += sc[c]; }
        if (therm && ipa == 0) {
          double t = 0;
          for (int c = 0; c < 8; ++c) t += f[c] * p.tempp[ii[c]];
          temp[ipt] = (float)t;
        }
        size_t o = (size_t)ipa * npts + ipt;
        ext[o] = (float)e;
        alb[o] = (float)(e > extmin ? scat / e : scat / extmin);
        int *IP = &iph[o * nq];
        float *PW = &pw[o * nq];
        for (int c = 0; c < 8; ++c)
          for (int q = 0; q < nmic; ++q) {
            size_t src = ((size_t)ipa * ng + ii[c]) * nmic + q;
            IP[c * nmic + q] = p.iphasep[src];
            PW[c * nmic + q] = (float)(scat >= scatmin ? p.phasewtp[src] * sc[c] / scat : p.phasewtp[src] * sc[c] / scatmin);
          }
        for (int q = 0; q < nq; ++q)
          for (int q2 = q + 1; q2 < nq; ++q2)
            if (IP[q] == IP[q2]) { PW[q] += PW[q2]; PW[q2] = 0.f; }
        bool sorted = true;  // weights already non-increasing: the stable sort would keep them as they are
        for (int q = 1; q < nq && sorted; ++q) sorted = !(PW[q] > PW[q - 1]);
        if (!sorted) {
          for (int q = 0; q < nq; ++q) srt[q] = {PW[q], IP[q]};
          std::stable_sort(srt.begin(), srt.end(), [](const std::pair<float, int> &a, const std::pair<float, int> &b2) { return a.first > b2.first; });
          for (int q = 0; q < nq; ++q) { PW[q] = srt[q].first; IP[q] = srt[q].second; }
        }
      }
    });
    for (int ipt = 0; ipt < npts; ++ipt) P.total_ext[ipt] += ext[(size_t)ipa * npts + ipt];
  }
  if (bad) { P.err = "TRILIN: grid point beyond the property grid"; return false; }
  const float phasemax = kPhaseMax;
  auto fterm = [&](size_t o) {  // f = mixed Legendre term ML+1 of one species at one point
    const int *IP = &iph[o * nq];
    const float *PW = &pw[o * nq];
    if (PW[0] >= phasemax) return leg[(size_t)(IP[0] - 1) * (nleg + 1) + ml + 1];
    float f = 0.f;
    for (int q = 0; q < nq; ++q) f += leg[(size_t)(IP[q] - 1) * (nleg + 1) + ml + 1] * PW[q];
    return f;
  };
  if (p.deltam) {  // per point, the species in order (the additions of the serial loops)
    parallel_for(npts, [&](int b, int e) {
      for (int ipt = b; ipt < e; ++ipt) {
        float s = 0.f;
        for (int ipa = 0; ipa < npart; ++ipa) s += ext[(size_t)ipa * npts + ipt];
        P.total_ext[ipt] = std::max(0.f, P.total_ext[ipt] - s);
        for (int ipa = 0; ipa < npart; ++ipa) {
          size_t o = (size_t)ipa * npts + ipt;
          float f = fterm(o);
          float a = alb[o];
          alb[o] = (1.f - f) * a / (1.f - a * f);
          ext[o] = (1.f - a * f) * ext[o];
          P.total_ext[ipt] += ext[o];
        }
      }
    });
  }
  P.albmax = 0.f;
  for (float a : alb) P.albmax = std::max(P.albmax, a);
  // thermal source: PLANCK = (1 - albedo) B(T) per species after the delta-M
  // scaling (src/polarized/shdomsub2.f:574-580), mixed with the extinction
  // weights of COMPUTE_SOURCE (TOTAL_PLANCK, src/polarized/shdomsub1.f:1092-1139)
  P.thermal.clear(); P.planckpt.clear();
  if (therm) {
    P.thermal.clear(); P.thermal.resize(npts);      // written for every point below
    P.planckpt.clear(); P.planckpt.resize(npts);
    parallel_for(npts, [&](int b, int e) {
      for (int ipt = b; ipt < e; ++ipt) {
        const float bb = planck_fn(temp[ipt], P.unitc, p.wavelen, p.waveno);
        P.planckpt[ipt] = bb;
        float tp = 0.f;
        for (int ipa = 0; ipa < npart; ++ipa) {
          const size_t o = (size_t)ipa * npts + ipt;
          tp += ext[o] * ((1.0f - alb[o]) * bb);
        }
        P.thermal[ipt] = P.total_ext[ipt] > 1e-10f ? tp / P.total_ext[ipt] : 0.f;
      }
    });
  }
  // kept for the gradient: the property grid of every species, the stored
  // Legendre table and the scaled species properties on the grid points
  P.npx = npx; P.npy = npy; P.npz = npz; P.maxnmicro = nmic; P.delx = p.delx; P.dely = p.dely;
  P.scatmin = scatmin;
  P.prop_ext.assign(p.extinctp, p.extinctp + (size_t)npart * ng);
  P.prop_alb.assign(p.albedop, p.albedop + (size_t)npart * ng);
  P.prop_iph.assign(p.iphasep, p.iphasep + (size_t)npart * ng * nmic);
  P.prop_phw.assign(p.phasewtp, p.phasewtp + (size_t)npart * ng * nmic);
  P.leg = leg;
  P.sp_f.clear(); P.sp_f.resize((size_t)npart * npts);  // written for every (species, point) below
  // Per-point source coefficients c_l = albedo_mix * chi_mix(l) (the
  // NEWMETHOD mixing of COMPUTE_SOURCE, src/polarized/shdomsub1.f:1413-1485)
  // and the exact single-scatter mixture of COMPUTE_SOURCE_1CELL_UNPOL
  // (src/polarized/shdomsub2.f:3113-3170).
  const int nl = ml + 1;
  // coefficient rows: every entry is written by the pass below
  P.coef.clear(); P.coef.resize((size_t)npts * nl);
  P.coefp.clear();
  if (nstleg == 6) P.coefp.resize((size_t)npts * 3 * nl);
  P.tms_ptr.clear(); P.tms_ptr.resize(npts + 1);
  P.tms_ptr[0] = 0;
  P.tms_iph.clear(); P.tms_w.clear();
  // two passes over the points on host threads: the coefficients and the
  // number of single-scatter entries of each point, then (after the prefix
  // sum) the entries themselves
  HostVec<int> tcnt(npts);  // written for every point
  parallel_for(npts, [&](int pb, int pe) {
    std::vector<double> ltp(nstleg == 6 ? 3 * nl : 0);
    std::vector<float> ltp1(nstleg == 6 ? 3 * nl : 0);
    std::vector<float> lt1(nleg + 1);
    std::vector<double> lt(nleg + 1);
    for (int ipt = pb; ipt < pe; ++ipt) {
      double sumscat = 0.0;
      std::fill(lt.begin(), lt.end(), 0.0);
      std::fill(ltp.begin(), ltp.end(), 0.0);
      float etot = P.total_ext[ipt];
      int nt = 0;
      for (int ipa = 0; ipa < npart; ++ipa) {
        size_t o = (size_t)ipa * npts + ipt;
        const int *IP = &iph[o * nq];
        const float *PW = &pw[o * nq];
        std::fill(lt1.begin(), lt1.end(), 0.f);
        bool single = PW[0] >= phasemax;
        if (single) for (int l = 0; l <= nleg; ++l) lt1[l] = leg[(size_t)(IP[0] - 1) * (nleg + 1) + l];
        else
          for (int q = 0; q < nq; ++q) {
            if (PW[q] <= 1e-5f) continue;
            for (int l = 0; l <= nleg; ++l) lt1[l] += leg[(size_t)(IP[q] - 1) * (nleg + 1) + l] * PW[q];
          }
        float f = 0.f;
        if (p.deltam) { f = lt1[ml + 1]; for (int l = 0; l <= ml; ++l) lt1[l] /= (1.f - f); }
        P.sp_f[o] = f;
        double scat = (double)(ext[o] * alb[o]);
        sumscat += scat;
        for (int l = 0; l <= nleg; ++l) lt[l] += scat * lt1[l];
        if (nstleg == 6) {  // a2, a3, b1 mixed the same way (all six elements are divided by 1 - f)
          std::fill(ltp1.begin(), ltp1.end(), 0.f);
          for (int e = 0; e < 3; ++e) {
            float *L1 = &ltp1[(size_t)e * nl];
            if (single) for (int l = 0; l < nl; ++l) L1[l] = legp3[((size_t)(IP[0] - 1) * 3 + e) * (nleg + 1) + l];
            else
              for (int q = 0; q < nq; ++q) {
                if (PW[q] <= 1e-5f) continue;
                for (int l = 0; l < nl; ++l) L1[l] += legp3[((size_t)(IP[q] - 1) * 3 + e) * (nleg + 1) + l] * PW[q];
              }
            if (p.deltam) for (int l = 0; l < nl; ++l) L1[l] /= (1.f - f);
            for (int l = 0; l < nl; ++l) ltp[(size_t)e * nl + l] += scat * L1[l];
          }
        }
        // exact single scatter entries of this species
        float wgt = (etot == 0.f) ? 1.f : ext[o] / etot;
        if (wgt != 0.f && p.deltam) {
          if (single) ++nt;
          else
            for (int q = 0; q < nq; ++q) nt += PW[q] > 1e-5f;
        }
      }
      tcnt[ipt] = nt;
      double albp = (etot > 1e-10f) ? sumscat / etot : 0.0;
      // chi = lt / sumscat (lt / npart without scattering), by one reciprocal per point
      const double inv = (sumscat > 1e-10) ? 1.0 / sumscat : 1.0 / npart;
      for (int l = 0; l <= ml; ++l) {
        const double chi = (l == 0) ? 1.0 : lt[l] * inv;
        P.coef[(size_t)ipt * nl + l] = (float)(albp * chi);
      }
      if (nstleg == 6)
        for (int e = 0; e < 3; ++e)
          for (int l = 0; l < nl; ++l) P.coefp[((size_t)ipt * 3 + e) * nl + l] = (float)(albp * (ltp[(size_t)e * nl + l] * inv));
    }
  });
  // scattering points: the coefficient row is non-zero exactly when its l = 0 term (the albedo) is
  P.scat.assign(npts, 0);
  // a point has a source when it scatters or (thermal source) emits
  parallel_for(npts, [&](int b, int e) {
    for (int ipt = b; ipt < e; ++ipt)
      P.scat[ipt] = P.coef[(size_t)ipt * nl] != 0.f || (!P.thermal.empty() && P.thermal[ipt] != 0.f);
  });
  for (int ipt = 0; ipt < npts; ++ipt) P.tms_ptr[ipt + 1] = P.tms_ptr[ipt] + tcnt[ipt];
  P.tms_iph.clear(); P.tms_iph.resize(P.tms_ptr[npts]);  // every entry is written below
  P.tms_w.clear(); P.tms_w.resize(P.tms_ptr[npts]);
  // exact single scatter: weight (albedo * ext_ipa / ext) / (1 - f) per phase function
  parallel_for(npts, [&](int pb, int pe) {
    for (int ipt = pb; ipt < pe; ++ipt) {
      int w0 = P.tms_ptr[ipt];
      const float etot = P.total_ext[ipt];
      for (int ipa = 0; ipa < npart; ++ipa) {
        const size_t o = (size_t)ipa * npts + ipt;
        const int *IP = &iph[o * nq];
        const float *PW = &pw[o * nq];
        const float wgt = (etot == 0.f) ? 1.f : ext[o] / etot;
        if (!(wgt != 0.f && p.deltam)) continue;
        const float base = alb[o] * wgt / (1.f - P.sp_f[o]);
        if (PW[0] >= phasemax) { P.tms_iph[w0] = IP[0] - 1; P.tms_w[w0] = base; ++w0; }
        else
          for (int q = 0; q < nq; ++q) {
            if (PW[q] <= 1e-5f) continue;
            P.tms_iph[w0] = IP[q] - 1; P.tms_w[w0] = base * PW[q]; ++w0;
          }
      }
    }
  });
  // Eddington initial radiance per column (INIT_RADIANCE).
  P.rad0.clear(); P.rad0.resize((size_t)npts * 4);  // all four terms of every point are written below
  const int nz = P.nz, nlay = nz - 1;
  const float pif = (float)std::acos(-1.0f);
  const float c0 = std::sqrt(1.0f / pif), c1 = std::sqrt(3.0f / (4 * pif));
  const int ncol = P.nx1 * P.ny1;
  parallel_for(ncol, [&](int cb, int ce) {
    std::vector<double> lo(2 * nlay + 3), up(2 * nlay + 3), dg(2 * nlay + 3), rhs(2 * nlay + 3);
    std::vector<float> od(nlay), al(nlay), as(nlay);
    for (int col = cb; col < ce; ++col) {
      for (int iz = 0; iz < nlay; ++iz) {
        int L = nz - iz - 2, i0 = iz + nz * col, i1 = i0 + 1;
        float e0 = P.total_ext[i0], e1 = P.total_ext[i1], s0 = 0, s1 = 0, g0 = 0, g1 = 0;
        for (int ipa = 0; ipa < npart; ++ipa) {
          size_t o0 = (size_t)ipa * npts + i0, o1 = (size_t)ipa * npts + i1;
          s0 += alb[o0] * ext[o0]; s1 += alb[o1] * ext[o1];
          for (int side = 0; side < 2; ++side) {
            size_t o = side ? o1 : o0;
            const int *IP = &iph[o * nq];
            const float *PW = &pw[o * nq];
            float l1 = 0.f, fm = 0.f;
            if (PW[0] >= phasemax) { l1 = leg[(size_t)(IP[0] - 1) * (nleg + 1) + 1]; fm = p.deltam ? leg[(size_t)(IP[0] - 1) * (nleg + 1) + ml + 1] : 0.f; }
            else
              for (int q = 0; q < nq; ++q) {
                l1 += leg[(size_t)(IP[q] - 1) * (nleg + 1) + 1] * PW[q];
                if (p.deltam) fm += leg[(size_t)(IP[q] - 1) * (nleg + 1) + ml + 1] * PW[q];
              }
            if (p.deltam) l1 /= (1.f - fm);
            (side ? g1 : g0) += alb[o] * ext[o] * l1;
          }
        }
        od[L] = (P.zgrid[iz + 1] - P.zgrid[iz]) * (e0 + e1) / 2;
        al[L] = (e0 + e1 > 0) ? (s0 + s1) / (e0 + e1) : 0.f;
        as[L] = (s0 + s1 > 0) ? (g0 + g1) / (s0 + s1) : 0.f;
      }
      // Eddington two-stream layer coefficients and the pentadiagonal system
      // reduced to tridiagonal form; solved with partial pivoting.
      const int n = 2 * nlay + 2;
      const double mu0 = std::fabs((double)p.solarmu), sf = p.solarflux;
      const double pid = 3.1415926535;
      double tau = 0.0;
      // thermal layers ('T' only): the Planck function is linear in optical
      // depth between the column's levels, taken from the top down
      const bool eth = P.srct == 'T';
      auto tlev = [&](int k) { return temp[(size_t)(nz - 1 - k) + (size_t)nz * col]; };
      double planck1 = eth ? pid * (double)planck_fn(tlev(0), P.unitc, p.wavelen, p.waveno) : 0.0;
      for (int l = 0, i = 2; l < nlay; ++l, i += 2) {
        double dt = od[l], tr, rf, sp, sm;
        if (dt == 0.0) { tr = 1; rf = 0; sp = 0; sm = 0; }
        else {
          double om = al[l], g = as[l];
          double r = (1.0 - om * (4.0 - 3.0 * g)) / 4.0, t = (7.0 - om * (4.0 + 3.0 * g)) / 4.0;
          double lam = std::sqrt(3.0 * (1.0 - om) * (1.0 - om * g)), dd, x1 = 0, x2 = 0, ep = 0, em = 0;
          if (lam == 0.0) { dd = 1.0 / (1.0 + t * dt); tr = dd; rf = -r * dt * dd; }
          else {
            x1 = -r; x2 = lam + t;
            ep = std::exp(std::min(lam * dt, 75.0)); em = 1.0 / ep;
            tr = 2. * lam / (x2 * ep + (lam - t) * em);
            rf = x1 * (ep - em) * tr / (2. * lam);
            dd = 1.0 / (x2 * x2 * ep - x1 * x1 * em);
          }
          double r1p, r2m, r2p, r1m;
          if (eth) {
            const double planck2 = pid * (double)planck_fn(tlev(l + 1), P.unitc, p.wavelen, p.waveno);
            const double vv = 2.0 * (planck2 - planck1) / (3.0 * (1. - om * g) * dt);
            r1p = -vv + planck1; r2m = vv + planck2; r2p = -vv + planck2; r1m = vv + planck1;
            planck1 = planck2;
          } else {
            double ds = 1.0 / (lam * lam - 1.0 / (mu0 * mu0));
            double b1 = 0.5 * om * (sf / mu0) * std::exp(-tau / mu0) * ds;
            double b2 = 0.5 * om * (sf / mu0) * std::exp(-(tau + dt) / mu0) * ds;
            double spp = 1.0 + 1.5 * g * mu0, spm = -1.0 + 1.5 * g * mu0;
            r1p = ((t + 1.0 / mu0) * spp + r * spm) * b1; r2m = ((-t + 1.0 / mu0) * spm - r * spp) * b2;
            r2p = ((t + 1.0 / mu0) * spp + r * spm) * b2; r1m = ((-t + 1.0 / mu0) * spm - r * spp) * b1;
          }
          if (lam == 0.0) {
            double A = (r * dt * r1p - r2m) * dd, B = -(r * r1p + t * r2m) * dd;
            sp = (B - t * (A + B * dt)) / r + r2p; sm = A + r1m;
          } else {
            double cp = (x1 * em * r1p - x2 * r2m) * dd, cm = (-x2 * ep * r1p + x1 * r2m) * dd;
            sp = x1 * cp * ep + x2 * cm * em + r2p; sm = x2 * cp + x1 * cm + r1m;
          }
          if (!eth) tau += dt;
        }
        dg[i] = -rf; dg[i + 1] = -rf; lo[i] = 1.0; lo[i + 1] = -tr; up[i] = -tr; up[i + 1] = 1.0;
        rhs[i] = sm; rhs[i + 1] = sp;
      }
      double gem = 1.0 - (double)p.gndalbedo;
      if (P.srct == 'S') {
        rhs[1] = pid * p.skyrad; rhs[n] = (1.0 - gem) * sf * std::exp(-tau / mu0);
      } else {  // emitting ground and sky ('T' and 'B')
        rhs[1] = pid * (double)planck_fn(p.skyrad, P.unitc, p.wavelen, p.waveno);
        rhs[n] = pid * (double)planck_fn(p.gndtemp, P.unitc, p.wavelen, p.waveno) * gem;
      }
      dg[1] = 0.0; up[1] = 1.0;
      dg[n] = -(1.0 - gem); lo[n] = 1.0;
      lo[1] = dg[1]; dg[1] = up[1]; up[1] = 0.0; up[n] = 0.0;
      for (int k = 1; k <= n - 1; ++k) {
        if (std::fabs(lo[k + 1]) >= std::fabs(lo[k])) {
          std::swap(lo[k + 1], lo[k]); std::swap(dg[k + 1], dg[k]); std::swap(up[k + 1], up[k]); std::swap(rhs[k + 1], rhs[k]);
        }
        double t = -lo[k + 1] / lo[k];
        lo[k + 1] = dg[k + 1] + t * dg[k];
        dg[k + 1] = up[k + 1] + t * up[k];
        up[k + 1] = 0.0;
        rhs[k + 1] += t * rhs[k];
      }
      rhs[n] /= lo[n];
      rhs[n - 1] = (rhs[n - 1] - dg[n - 1] * rhs[n]) / lo[n - 1];
      for (int k = n - 2; k >= 1; --k) rhs[k] = (rhs[k] - dg[k] * rhs[k + 1] - up[k] * rhs[k + 2]) / lo[k];
      const double cfl = P.unitc == 'T' ? 1.0 / pid : 1.0;  // brightness temperature fluxes
      for (int iz = 0; iz < nz; ++iz) {
        int L = nz - 1 - iz;
        float fu = (float)(cfl * rhs[2 * L + 1]), fd = (float)(cfl * rhs[2 * L + 2]);
        float *r = &P.rad0[(size_t)(iz + nz * col) * 4];
        r[0] = c0 * (fu + fd); r[1] = 0.f; r[2] = c1 * (fu - fd); r[3] = 0.f;
      }
    }
  });
  // Unscaled single-scatter phase table (PRECOMPUTE_PHASE_CHECK).
  int nlegp = std::max(p.nlegp, nleg);
  P.nscatangle = std::max(36, std::min(721, 2 * nlegp));
  P.phasetab.assign((size_t)P.nscatangle * p.numphase, 0.f);
  const double pi = std::acos(-1.0);
  std::vector<double> pl(nlegp + 1);
  for (int j = 0; j < P.nscatangle; ++j) {
    double x = std::cos(pi * (double)j / (P.nscatangle - 1));
    pl[0] = 1.0;
    if (nlegp >= 1) pl[1] = x;
    for (int n2 = 1; n2 < nlegp; ++n2) pl[n2 + 1] = ((2 * n2 + 1) * x * pl[n2] - n2 * pl[n2 - 1]) / (n2 + 1);
    for (int i = 0; i < p.numphase; ++i) {
      double a1 = 0.0;
      for (int l = 0; l <= nlegp; ++l) {
        float lg = (l <= p.nlegp) ? legin(i, l, 0) : 0.f;
        a1 += (2.0 * l + 1.0) * (double)(lg / (float)(2 * l + 1)) * pl[l];
      }
      if (a1 <= 0.0) { P.err = "PRECOMPUTE_PHASE_CHECK: negative phase function"; return false; }
      P.phasetab[(size_t)j * p.numphase + i] = (float)(a1 / (4.0 * pi));
    }
  }
  // polarized: the I-Q element -sum_l b1_l d^l_{20}(cos theta) / (4 pi)
  P.phasetab2.clear();
  if (nstleg == 6) {
    P.phasetab2.assign((size_t)P.nscatangle * p.numphase, 0.f);
    std::vector<double> d2;
    for (int j = 0; j < P.nscatangle; ++j) {
      const double x = std::cos(pi * (double)j / (P.nscatangle - 1));
      wig(x, nlegp, 2, 0, d2);
      for (int i = 0; i < p.numphase; ++i) {
        double b1 = 0.0;
        for (int l = 0; l <= nlegp; ++l) {
          float lg = (l <= p.nlegp) ? legin(i, l, 4) : 0.f;
          b1 -= (2.0 * l + 1.0) * (double)(lg / (float)(2 * l + 1)) * d2[l];
        }
        P.phasetab2[(size_t)j * p.numphase + i] = (float)(b1 / (4.0 * pi));
      }
    }
  }
  // the per-point phase indices and weights, kept for species_series
  P.sp_iph = std::move(iph);
  P.sp_pw = std::move(pw);
  P.sp_nq = nq;
  return true;
}

// DIRECT_BEAM_PROP: per grid point, integrate the delta-M scaled extinction
// of the property grid along the ray to the sun (trilinear extinction
// integrated exactly within each property cell).
void build_direct(const shdom_problem &p, Plan &P) {
  // The delta-M scaled extinction of the property grid (the EXTDIRP field of
  // DIRECT_BEAM_PROP); the per-point path integrals to the sun run on the
  // device (k_direct_beam) when the plan is put on a GPU.
  const int npx = p.npx, npy = p.npy, npz = p.npz, ng = npx * npy * npz, ml = P.ml, nmic = p.maxnmicro;
  P.extdirp.clear(); P.extdirp.resize(ng);  // written for every property point
  for (int ip = 0; ip < ng; ++ip) {
    float acc = 0.f;
    for (int ipa = 0; ipa < p.npart; ++ipa) {
      double e = p.extinctp[(size_t)ipa * ng + ip], a = p.albedop[(size_t)ipa * ng + ip];
      if (p.deltam) {
        int L = ml + 1;
        double f = 0;
        for (int q = 0; q < nmic; ++q) {
          int iph = p.iphasep[((size_t)ipa * ng + ip) * nmic + q];
          float a_l = (L <= p.nlegp) ? p.legenp[((size_t)(iph - 1) * (p.nlegp + 1) + L) * (p.nstokes == 3 ? 6 : 1)] : 0.f;
          f += (double)(p.phasewtp[((size_t)ipa * ng + ip) * nmic + q] * a_l) / (2 * L + 1);
        }
        e = (1.0 - a * f) * e;
      }
      acc = (float)(acc + e);
    }
    P.extdirp[ip] = acc;
  }
}

bool build_schedule(const shdom_problem &p, Plan &P) {
  const int n = P.npts;
  P.rank.assign((size_t)8 * n, -1);
  P.startcell.assign((size_t)8 * n, -1);
  P.level.assign((size_t)32 * n, 0);
  P.kind.assign((size_t)32 * n, 0);
  P.regular.assign((size_t)8 * n, 0);
  std::vector<int> octs = P.is1d ? std::vector<int>{1, 5} : std::vector<int>{1, 2, 3, 4, 5, 6, 7, 8};
  const double transmin = p.transmin;
  bool ok = true;
  std::vector<std::thread> th;
  std::vector<std::string> errs(8);
  std::vector<int> deep(8, 0);  // octants whose wavefront is too deep for level scheduling
  for (int ioct : octs) {
    th.emplace_back([&, ioct]() {
      sweep_order(P, ioct);
      const int b = ioct - 1;
      const int hemi_bnd = (b & 4) ? 2 : 1;  // trace down: bottom points preset
      const int *rk = &P.rank[(size_t)b * n];
      const int *sc = &P.startcell[(size_t)b * n];
      std::vector<int> order(n), corners;
      for (int i = 0; i < n; ++i) order[rk[i]] = i;
      for (int r = 0; r < n; ++r) {
        int pt = order[r];
        if (P.bnd[pt] & hemi_bnd) continue;
        int cell = sc[pt];
        const int *g = &P.gridptr[8 * (size_t)cell];
        bool fast = transmin >= 1.0 && !P.is1d && g[b] == pt && P.cellflags[cell] == 0;
        for (int k = 0; k < 8 && fast; ++k) {
          if (k == b) continue;
          int q = g[k];
          if (q == pt || !((P.bnd[q] & hemi_bnd) || rk[q] < r)) fast = false;
        }
        if (fast) P.regular.mut()[(size_t)b * n + pt] = 1;
        for (int cls = 0; cls < 4; ++cls) {
          const int nc = P.cls_ncol[b][cls], c0 = P.cls_col0[b][cls];
          if (nc == 0) continue;
          int *lv = &P.level.mut()[((size_t)b * 4 + cls) * n];
          uint8_t *kd = &P.kind.mut()[((size_t)b * 4 + cls) * n];
          // the corners the point's traces for this class end on
          corners.clear();
          if (fast) {
            if (cls < 3) {
              const int bit = (b >> cls) & 1;
              const int iface = 2 * cls + 1 - bit;
              for (int k = 0; k < 4; ++k) corners.push_back(g[kFace[iface][k]]);
            } else {
              for (int k = 0; k < 8; ++k) if (k != b) corners.push_back(g[k]);
            }
          } else {
            for (int c = c0; c < c0 + nc; ++c) {
              int f[4];
              double tcx, tcy, tcz;
              trace_dir(P.mu[P.col_imu[c]], P.phi[(size_t)P.col_imu[c] * P.nphi0max + P.col_iphi[c]], tcx, tcy, tcz);
              if (!trace_final_face(P, ioct, pt, tcx, tcy, tcz, hemi_bnd, transmin, f)) {
                errs[b] = "sweep planning: trace found no valid face (BACK_INT_GRID: INEXTCELL=0)";
                return;
              }
              for (int k = 0; k < 4; ++k) corners.push_back(f[k]);
            }
          }
          // A general-trace point whose corners are all preset or phase-1
          // points is a phase-1 point (boundary-plane chains); any other
          // point is phase 2, where phase-1 corners count as level 0.
          bool one = !fast;
          int m1 = 0, m2 = 0;
          for (int q : corners) {
            if (P.bnd[q] & hemi_bnd) continue;
            if (kd[q] == 3) m1 = std::max(m1, lv[q]);
            else { one = false; m2 = std::max(m2, lv[q] - Plan::kPhase2); }
          }
          if (one) { kd[pt] = 3; lv[pt] = m1 + 1; }
          else { kd[pt] = fast ? 1 : 2; lv[pt] = Plan::kPhase2 + m2 + 1; }
          if (lv[pt] >= 2 * Plan::kPhase2 - 1 || (one && lv[pt] >= Plan::kPhase2)) {
            // (periodic grids chain whole rows through the wrap-around) the
            // hemisphere is swept in the reference order instead
            deep[b] = 1;
            return;
          }
        }
      }
    });
  }
  for (auto &t : th) t.join();
  for (auto &e : errs) if (!e.empty()) { P.err = e; ok = false; }
  if (!ok) return false;
  for (int hemi = 0; hemi < 2; ++hemi) {
    P.deep[hemi] = 0;
    for (int ioct : octs)
      if (((((ioct - 1) >> 2) & 1) == hemi) && deep[ioct - 1]) P.deep[hemi] = 1;
    if (P.deep[hemi]) {
      P.tasks[hemi].mut().clear(); P.p1segs[hemi].clear(); P.p1off[hemi].assign(1, 0); P.p1depth[hemi] = 0;
      P.segs[hemi].clear(); P.seg_off[hemi].assign(1, 0); P.level_items[hemi].clear();
      P.nirr[hemi] = 0; P.nitems[hemi] = 0;
      continue;
    }
    std::vector<std::pair<int, int>> groups;  // (octant, class) pairs of this hemisphere
    for (int ioct : octs) {
      int b = ioct - 1;
      if (((b >> 2) & 1) != hemi) continue;
      for (int cls = 0; cls < 4; ++cls)
        if (P.cls_ncol[b][cls] > 0) groups.push_back({b, cls});
    }
    const int ng = (int)groups.size();
    std::vector<uint32_t> &tasks = P.tasks[hemi].mut();
    tasks.clear();
    long long irr = 0;
    // Phase 1: per (octant, class) group, one segment per level.
    P.p1segs[hemi].clear();
    P.p1off[hemi].assign(1, 0);
    P.p1depth[hemi] = 0;
    for (int gi = 0; gi < ng; ++gi) {
      const int b = groups[gi].first, cls = groups[gi].second;
      const int *lv = &P.level[((size_t)b * 4 + cls) * n];
      const uint8_t *kd = &P.kind[((size_t)b * 4 + cls) * n];
      int depth = 0;
      for (int i = 0; i < n; ++i) if (kd[i] == 3) depth = std::max(depth, lv[i]);
      if (depth == 0) continue;
      std::vector<std::vector<int>> by(depth + 1);
      for (int i = 0; i < n; ++i) if (kd[i] == 3) by[lv[i]].push_back(i);
      for (int l = 1; l <= depth; ++l) {
        Seg sg;
        sg.t0 = (int)tasks.size(); sg.ntask = (int)by[l].size(); sg.start = 0; sg.b = b; sg.cls = cls;
        sg.col0 = P.cls_col0[b][cls]; sg.ncol = P.cls_ncol[b][cls]; sg.regular = 0; sg.irr0 = (int)irr;
        irr += (long long)sg.ntask * sg.ncol;
        for (int i : by[l]) tasks.push_back((uint32_t)i);
        P.p1segs[hemi].push_back(sg);
      }
      P.p1off[hemi].push_back((int)P.p1segs[hemi].size());
      P.p1depth[hemi] = std::max(P.p1depth[hemi], depth);
    }
    // Phase 2: per level, the (group, regular or not) segments.
    int maxl = 0;
    for (int gi = 0; gi < ng; ++gi) {
      const int b = groups[gi].first, cls = groups[gi].second;
      const int *lv = &P.level[((size_t)b * 4 + cls) * n];
      const uint8_t *kd = &P.kind[((size_t)b * 4 + cls) * n];
      for (int i = 0; i < n; ++i) if (kd[i] == 1 || kd[i] == 2) maxl = std::max(maxl, lv[i] - Plan::kPhase2);
    }
    std::vector<int> cnt((size_t)(maxl + 1) * ng * 2, 0);
    for (int gi = 0; gi < ng; ++gi) {
      const int b = groups[gi].first, cls = groups[gi].second;
      const int *lv = &P.level[((size_t)b * 4 + cls) * n];
      const uint8_t *kd = &P.kind[((size_t)b * 4 + cls) * n];
      for (int i = 0; i < n; ++i)
        if (kd[i] == 1 || kd[i] == 2) cnt[((size_t)(lv[i] - Plan::kPhase2) * ng + gi) * 2 + (kd[i] == 1 ? 0 : 1)]++;
    }
    P.segs[hemi].clear();
    P.seg_off[hemi].assign(1, 0);
    P.level_items[hemi].clear();
    std::vector<int> fill((size_t)(maxl + 1) * ng * 2, 0);
    long long gitems = 0;
    int t = (int)tasks.size();
    for (int l = 1; l <= maxl; ++l) {
      long long items = 0;
      for (int gi = 0; gi < ng; ++gi)
        for (int isirr = 0; isirr < 2; ++isirr) {
          const int c = cnt[((size_t)l * ng + gi) * 2 + isirr];
          if (c == 0) continue;
          const int b = groups[gi].first, cls = groups[gi].second;
          Seg sg;
          sg.t0 = t; sg.ntask = c; sg.start = (int)items; sg.b = b; sg.cls = cls;
          sg.col0 = P.cls_col0[b][cls]; sg.ncol = P.cls_ncol[b][cls]; sg.regular = isirr ? 0 : 1;
          sg.irr0 = (int)irr;
          if (isirr) irr += (long long)c * sg.ncol;
          fill[((size_t)l * ng + gi) * 2 + isirr] = t;
          P.segs[hemi].push_back(sg);
          t += c;
          items += (long long)c * sg.ncol;
        }
      if (items >= (1LL << 31) || irr >= (1LL << 31)) { P.err = "sweep level too large"; return false; }
      P.seg_off[hemi].push_back((int)P.segs[hemi].size());
      P.level_items[hemi].push_back((int)items);
      gitems += items;
    }
    P.nirr[hemi] = irr;
    P.nitems[hemi] = gitems;
    tasks.resize(t);
    for (int gi = 0; gi < ng; ++gi) {
      const int b = groups[gi].first, cls = groups[gi].second;
      const int *lv = &P.level[((size_t)b * 4 + cls) * n];
      const uint8_t *kd = &P.kind[((size_t)b * 4 + cls) * n];
      for (int i = 0; i < n; ++i)
        if (kd[i] == 1 || kd[i] == 2)
          tasks[fill[((size_t)(lv[i] - Plan::kPhase2) * ng + gi) * 2 + (kd[i] == 1 ? 0 : 1)]++] = (uint32_t)i;
    }
  }
  return true;
}

// Polarized column layout: every (octant, face class) group [c0, c0+n) of
// the scalar layout becomes [3 c0, 3 c0 + 3n) holding the group's ordinates
// for I, then Q, then U.  A sweep segment always spans a whole group, so its
// columns, item offsets and general-trace table offsets scale by three.
void expand_stokes(Plan &P) {
  const int n = P.nang;
  std::vector<int> g0(n, -1), gn(n, 0);
  for (int b = 0; b < 8; ++b)
    for (int cls = 0; cls < 4; ++cls)
      for (int c = P.cls_col0[b][cls]; c < P.cls_col0[b][cls] + P.cls_ncol[b][cls]; ++c) { g0[c] = P.cls_col0[b][cls]; gn[c] = P.cls_ncol[b][cls]; }
  auto nc = [&](int c, int st) { return 3 * g0[c] + st * gn[c] + (c - g0[c]); };
  std::vector<int> imu(3 * n), iphi(3 * n), oct(3 * n), cls(3 * n);
  std::vector<float> cx(3 * n), cy(3 * n), cz(3 * n), fw(3 * n, 0.f);
  P.col_stk.assign(3 * n, 0);
  for (int c = 0; c < n; ++c)
    for (int st = 0; st < 3; ++st) {
      const int d = nc(c, st);
      imu[d] = P.col_imu[c]; iphi[d] = P.col_iphi[c]; oct[d] = P.col_oct[c]; cls[d] = P.col_cls[c];
      cx[d] = P.col_cx[c]; cy[d] = P.col_cy[c]; cz[d] = P.col_cz[c];
      if (st == 0) fw[d] = P.col_fluxw[c];  // the hemispheric fluxes are fluxes of I
      P.col_stk[d] = (uint8_t)st;
    }
  for (int &c : P.col_of)
    if (c >= 0) c = nc(c, 0);
  P.col_imu.swap(imu); P.col_iphi.swap(iphi); P.col_oct.swap(oct); P.col_cls.swap(cls);
  P.col_cx.swap(cx); P.col_cy.swap(cy); P.col_cz.swap(cz); P.col_fluxw.swap(fw);
  for (int b = 0; b < 8; ++b) {
    P.oct_col0[b] *= 3; P.oct_ncol[b] *= 3;
    for (int k = 0; k < 4; ++k) { P.cls_col0[b][k] *= 3; P.cls_ncol[b][k] *= 3; }
  }
  P.ncol_down *= 3;
  P.nang = 3 * n;
  for (int h = 0; h < 2; ++h) {
    for (auto *v : {&P.segs[h], &P.p1segs[h]})
      for (Seg &g : *v) { g.col0 *= 3; g.ncol *= 3; g.start *= 3; g.irr0 *= 3; }
    for (int &x : P.level_items[h]) x *= 3;
    P.nirr[h] *= 3; P.nitems[h] *= 3;
  }
}

// Plane-march groups of each hemisphere (see MarchGrp).  A hemisphere
// marches when every one of its (octant, class) groups has a face class
// x, y or z, no general-trace phase-2 point, and exactly the points the
// kernel treats as fixed (the hemisphere's preset boundary layer and, on
// open boundaries, the edge planes) are not phase-2 points.  Runs on the
// scalar column layout's kind table, so it does not depend on the Stokes
// expansion; the groups' columns are set after it.
void build_march(Plan &P) {
  const int n = P.npts;
  const int stride[3] = {P.ny1 * P.nz, P.nz, 1}, cnt[3] = {P.nx1, P.ny1, P.nz};
  const bool xopen = (P.bcflag & 1) != 0, yopen = (P.bcflag & 2) != 0;
  for (int h = 0; h < 2; ++h) {
    P.march[h].clear();
    if (P.is1d || P.deep[h] || P.segs[h].empty()) continue;
    std::vector<MarchGrp> out;
    bool ok = true;
    for (int b = 0; b < 8 && ok; ++b) {
      if (((b >> 2) & 1) != h) continue;
      for (int cls = 0; cls < 4 && ok; ++cls) {
        if (P.cls_ncol[b][cls] == 0) continue;
        if (cls == 3) { ok = false; break; }
        MarchGrp g{};
        g.b = b; g.cls = cls; g.col0 = P.cls_col0[b][cls]; g.ncol = P.cls_ncol[b][cls];
        const int ia = cls, iu = cls == 0 ? 1 : 0, iv = cls == 2 ? 1 : 2;
        g.nA = cnt[ia]; g.nU = cnt[iu]; g.nV = cnt[iv];
        g.sa = stride[ia]; g.su = stride[iu]; g.sv = stride[iv];
        const int sA = ((b >> ia) & 1) ? -1 : 1;  // the stopping face lies at a + sA
        g.da = -sA;
        g.a0 = sA > 0 ? g.nA - 1 : 0;
        const int iface = 2 * cls + 1 - ((b >> cls) & 1);
        for (int k = 0; k < 4; ++k) {
          const int d = kFace[iface][k] ^ b;
          g.du[k] = ((d >> iu) & 1) ? ((((b >> iu) & 1) ? -1 : 1)) : 0;
          g.dv[k] = ((d >> iv) & 1) ? ((((b >> iv) & 1) ? -1 : 1)) : 0;
        }
        g.upu = ((b >> iu) & 1) ? -1 : 1;
        g.zfix = h == 0 ? P.nz - 1 : 0;
        g.xedge = xopen ? 1 : 0; g.yedge = yopen ? 1 : 0;
        const uint8_t *kd = &P.kind[((size_t)b * 4 + cls) * n];
        for (int p = 0; p < n && ok; ++p) {
          const int ix = p / (P.ny1 * P.nz), iy = (p / P.nz) % P.ny1, iz = p % P.nz;
          const bool fixed = iz == g.zfix || (xopen && (ix == 0 || ix == P.nx1 - 1)) ||
                             (yopen && (iy == 0 || iy == P.ny1 - 1));
          const int ic[3] = {ix, iy, iz};
          // fixed points are exactly the non-phase-2 ones; phase-2 points are
          // regular and never lie in the first plane of the march
          if (fixed ? (kd[p] == 1 || kd[p] == 2) : (kd[p] != 1)) ok = false;
          if (!fixed && ic[ia] == g.a0) ok = false;
        }
        out.push_back(g);
      }
    }
    if (ok) P.march[h] = out;
  }
}

// Exit geometry of regular-point traces per (layer, ordinate): so, u, v, face.
void build_geo(Plan &P) {
  const int nl = P.nz - 1, nang = P.nang;
  P.geo.assign((size_t)std::max(nl, 1) * nang * 4, 0.f);
  if (P.is1d || P.nx1 < 2 || P.ny1 < 2) return;
  const float dx = P.xgrid[1] - P.xgrid[0], dy = P.ygrid[1] - P.ygrid[0];
  for (int L = 0; L < nl; ++L)
    for (int c = 0; c < nang; ++c) {
      if (P.col_imu[c] < 0) continue;
      float *g = &P.geo[((size_t)L * nang + c) * 4];
      const int b = P.col_oct[c] - 1;
      g[3] = (float)regular_exit(P.col_cx[c], P.col_cy[c], P.col_cz[c], b, dx, dy, P.zgrid[L + 1] - P.zgrid[L], g[0], g[1], g[2]);
    }
}

}  // namespace

// The geometric part of a plan (grid, cells, ordinates, transform
// coefficients, sweep order and schedule) depends only on the grid, the
// boundary flags, the angular resolution and TRANSMIN.  Several solves on
// one grid (wavelengths, inversion iterates) share it: the last few are kept.
namespace {
std::string geometry_key(const shdom_problem &p) {
  std::string k;
  auto put = [&](const void *d, size_t n) { k.append(static_cast<const char *>(d), n); };
  put(&p.npx, sizeof(int)); put(&p.npy, sizeof(int)); put(&p.npz, sizeof(int));
  put(&p.delx, sizeof(float)); put(&p.dely, sizeof(float)); put(p.zlevels, sizeof(float) * (size_t)p.npz);
  put(&p.bc_x_open, sizeof(int)); put(&p.bc_y_open, sizeof(int)); put(&p.ipflag, sizeof(int));
  put(&p.nmu, sizeof(int)); put(&p.nphi, sizeof(int)); put(&p.angle_set, sizeof(int));
  put(&p.deltam, sizeof(int)); put(&p.transmin, sizeof(float)); put(&p.nstokes, sizeof(int));
  return k;
}

std::mutex g_geom_mu;
std::list<std::pair<std::string, std::shared_ptr<const Plan>>> g_geom;  // most recent first
constexpr size_t kGeomCache = 2;
}  // namespace

bool build_plan(const shdom_problem &p, Plan &P) {
  if (p.nstokes != 1 && p.nstokes != 3) { P.err = "nstokes must be 1 or 3"; return false; }
  if (p.splitacc > 0) { P.err = "adaptive cell splitting is not supported (split_accuracy must be <= 0)"; return false; }
  if (p.npart < 1 || p.numphase < 1 || p.maxnmicro < 1) { P.err = "empty medium"; return false; }
  const std::string key = geometry_key(p);
  std::shared_ptr<const Plan> hit;
  {
    std::lock_guard<std::mutex> lk(g_geom_mu);
    for (auto it = g_geom.begin(); it != g_geom.end(); ++it)
      if (it->first == key) { hit = it->second; g_geom.splice(g_geom.begin(), g_geom, it); break; }
  }
  if (hit) {
    P = *hit;
  } else {
    P.prob = p;
    if (!build_grid(p, P)) return false;
    build_angles(p, P);
    if (P.npts >= (1 << 28)) { P.err = "grid too large for the sweep task encoding"; return false; }
    if (!build_schedule(p, P)) return false;
    P.nst = p.nstokes;
    P.col_stk.assign(P.nang, 0);
    build_march(P);
    if (P.nst == 3) expand_stokes(P);
    for (int h = 0; h < 2; ++h)  // the groups' columns in the final (Stokes-expanded) layout
      for (MarchGrp &g : P.march[h]) { g.col0 = P.cls_col0[g.b][g.cls]; g.ncol = P.cls_ncol[g.b][g.cls]; }
    build_geo(P);
    auto keep = std::make_shared<const Plan>(P);
    std::lock_guard<std::mutex> lk(g_geom_mu);
    g_geom.emplace_front(key, std::move(keep));
    while (g_geom.size() > kGeomCache) g_geom.pop_back();
  }
  P.prob = p;
  P.err.clear();
  P.srct = p.srctype ? (char)p.srctype : 'S';
  P.unitc = p.units ? (char)p.units : 'R';
  if (P.srct != 'S' && P.srct != 'T' && P.srct != 'B') { P.err = "srctype must be 'S', 'T' or 'B'"; return false; }
  if (P.unitc != 'R' && P.unitc != 'T' && P.unitc != 'B') { P.err = "units must be 'R', 'T' or 'B'"; return false; }
  if (P.srct != 'S' && P.unitc == 'B' && !(p.waveno[0] > 0.f && p.waveno[1] > p.waveno[0])) {
    P.err = "band units need 0 < waveno[0] < waveno[1]"; return false;
  }
  if (P.srct != 'S') {
    if (!p.tempp) { P.err = "a thermal source needs the temperature field"; return false; }
    if (P.unitc == 'R' && !(p.wavelen > 0.f)) { P.err = "a thermal source in radiance units needs the wavelength"; return false; }
  }
  // COMPUTE_TOP_RADIANCES: the sky brightness temperature becomes a radiance for 'T'
  P.skyrad_bc = P.srct == 'T' ? planck_fn(p.skyrad, P.unitc, p.wavelen, p.waveno) : p.skyrad;
  if (!build_medium(p, P)) return false;
  build_direct(p, P);
  // bottom surface albedo (PREP_SURFACE periodic grid + SURFACE_PARM_INTERP)
  P.botalb.assign(P.botp.size(), p.gndalbedo);
  if (p.sfc_variable) {
    int nxs = p.nxsfc, nys = p.nysfc;
    auto G = [&](int x, int y) { return p.sfc_albedo[(size_t)((y - 1) % nys) * nxs + ((x - 1) % nxs)]; };
    for (size_t k = 0; k < P.botp.size(); ++k) {
      int i = P.botp[k];
      float rx = P.gridpos[3 * i] / p.delxsfc, ry = P.gridpos[3 * i + 1] / p.delysfc;
      int ix = std::max(1, std::min(nxs, (int)rx + 1)), iy = std::max(1, std::min(nys, (int)ry + 1));
      float u = std::max(0.f, std::min(1.f, rx - (ix - 1))), v = std::max(0.f, std::min(1.f, ry - (iy - 1)));
      P.botalb[k] = (1 - u) * (1 - v) * G(ix, iy) + (1 - u) * v * G(ix, iy + 1) + u * (1 - v) * G(ix + 1, iy) + u * v * G(ix + 1, iy + 1);
    }
  }
  // ground emission: B of the bilinearly interpolated surface temperature
  // (SURFACE_PARM_INTERP) or of the one ground temperature
  P.botplanck.clear();
  if (P.srct != 'S') {
    P.botplanck.assign(P.botp.size(), planck_fn(p.gndtemp, P.unitc, p.wavelen, p.waveno));
    if (p.sfc_temp && p.nxsfc > 0 && p.nysfc > 0 && (p.sfc_variable || p.sfc_brdf)) {
      const int nxs = p.nxsfc, nys = p.nysfc;
      auto G = [&](int x, int y) { return p.sfc_temp[(size_t)((y - 1) % nys) * nxs + ((x - 1) % nxs)]; };
      for (size_t k = 0; k < P.botp.size(); ++k) {
        int i = P.botp[k];
        float rx = P.gridpos[3 * i] / p.delxsfc, ry = P.gridpos[3 * i + 1] / p.delysfc;
        int ix = std::max(1, std::min(nxs, (int)rx + 1)), iy = std::max(1, std::min(nys, (int)ry + 1));
        float u = std::max(0.f, std::min(1.f, rx - (ix - 1))), v = std::max(0.f, std::min(1.f, ry - (iy - 1)));
        const float t = (1 - u) * (1 - v) * G(ix, iy) + (1 - u) * v * G(ix, iy + 1) + u * (1 - v) * G(ix + 1, iy) + u * v * G(ix + 1, iy + 1);
        P.botplanck[k] = planck_fn(t, P.unitc, p.wavelen, p.waveno);
      }
    }
  }
  // bidirectional surface: parameters at the bottom points (SURFACE_PARM_INTERP,
  // src/polarized/shdomsub1.f:2218-2268) and the ordinate tables of the
  // reflection sums (VARIABLE_BRDF_SURFACE, src/polarized/shdomsub1.f:2592-2664)
  P.brdf = p.sfc_brdf;
  P.nsfcpar = 0;
  P.botpar.clear(); P.brdf_dn.clear(); P.brdf_up.clear();
  if (p.sfc_brdf) {
    const char bt = (char)p.sfc_brdf;
    if ((bt != 'R' && bt != 'W' && bt != 'D' && bt != 'O' && bt != 'M') || p.nsfcpar < (bt == 'D' ? 5 : bt == 'O' ? 2 : 3) ||
        !p.sfc_params || p.nxsfc < 1 || p.nysfc < 1) {
      P.err = "surface BRDF: types 'R' (RPV), 'W' (wave-Fresnel), 'M' (Ross-Li; 3 parameters each), 'D' (Diner; 5) and 'O' (ocean; 2) on a surface grid";
      return false;
    }
    if (bt == 'R' && p.nstokes != 1) { P.err = "RPV BRDF is only for unpolarized case"; return false; }
    if (bt == 'O' && p.nstokes != 1) { P.err = "Ocean BRDF from 6S is only for unpolarized case"; return false; }
    if (bt == 'M' && p.nstokes != 1) { P.err = "RossLiThick-Sparse is only for unpolarized case"; return false; }
    if (bt == 'O' && !(p.wavelen > 0.f)) { P.err = "the ocean BRDF needs the wavelength"; return false; }
    const int nxs = p.nxsfc, nys = p.nysfc, np_ = p.nsfcpar;
    // the ocean model also takes the wavelength: appended to every bottom
    // point's parameters (wind speed, pigment, wavelength)
    const int npb = bt == 'O' ? 3 : np_;
    P.nsfcpar = npb;
    P.botpar.assign(P.botp.size() * npb, 0.f);
    auto G = [&](int x, int y, int j) { return p.sfc_params[((size_t)((y - 1) % nys) * nxs + ((x - 1) % nxs)) * np_ + j]; };
    for (size_t k = 0; k < P.botp.size(); ++k) {
      int i = P.botp[k];
      float rx = P.gridpos[3 * i] / p.delxsfc, ry = P.gridpos[3 * i + 1] / p.delysfc;
      int ix = std::max(1, std::min(nxs, (int)rx + 1)), iy = std::max(1, std::min(nys, (int)ry + 1));
      float u = std::max(0.f, std::min(1.f, rx - (ix - 1))), v = std::max(0.f, std::min(1.f, ry - (iy - 1)));
      for (int j = 0; j < std::min(np_, npb); ++j)
        P.botpar[k * npb + j] = (1 - u) * (1 - v) * G(ix, iy, j) + (1 - u) * v * G(ix, iy + 1, j) +
                                u * (1 - v) * G(ix + 1, iy, j) + u * v * G(ix + 1, iy + 1, j);
      if (bt == 'O') P.botpar[k * npb + 2] = p.wavelen;
    }
    const float opi = 1.0f / (float)std::acos(-1.0f);
    for (int j = 0; j < P.nmu; ++j)
      for (int q = 0; q < P.nphi0[j]; ++q) {
        const int c = P.col_of[(size_t)j * P.nphi0max + q];
        const int off = P.nst == 3 ? P.cls_ncol[P.col_oct[c] - 1][P.col_cls[c]] / 3 : 0;
        const float mu = P.mu[j], ph = P.phi[(size_t)j * P.nphi0max + q];
        if (j < P.nmu / 2) {
          const float w = opi * std::fabs(mu) * P.wtdo[(size_t)j * P.nphi0max + q];
          P.brdf_dn.push_back({mu, ph, w, (float)c, (float)off});
        } else {
          P.brdf_up.push_back({mu, ph, 0.f, (float)c, (float)off});
        }
      }
  }
  return true;
}

// The species' own series at a grid point, delta-M scaling undone (the
// series COMPUTE_SOURCE_GRAD_1CELL uses): the same mixture and scaling as
// the coefficient loop of build_medium.
void species_series(const Plan &P, int ipa, int ipt, float *u) {
  const int nq = P.sp_nq, nl1 = P.nleg + 1, ml = P.ml;
  const size_t o = (size_t)ipa * P.npts + ipt;
  const int *IP = &P.sp_iph[o * nq];
  const float *PW = &P.sp_pw[o * nq];
  std::vector<float> lt1(nl1, 0.f);
  if (PW[0] >= kPhaseMax) {
    for (int l = 0; l < nl1; ++l) lt1[l] = P.leg[(size_t)(IP[0] - 1) * nl1 + l];
  } else {
    for (int q = 0; q < nq; ++q) {
      if (PW[q] <= 1e-5f) continue;
      for (int l = 0; l < nl1; ++l) lt1[l] += P.leg[(size_t)(IP[q] - 1) * nl1 + l] * PW[q];
    }
  }
  const bool deltam = P.prob.deltam != 0;
  float f = 0.f;
  if (deltam) { f = lt1[ml + 1]; for (int l = 0; l <= ml; ++l) lt1[l] /= (1.f - f); }
  for (int l = 0; l <= ml; ++l) u[l] = deltam ? lt1[l] * (1.f - f) + f : lt1[l];
}

}  // namespace shdom
