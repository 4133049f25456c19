// Lorenz-Mie single scattering of homogeneous spheres: the monodisperse table
// that feeds the polydisperse optical properties of a species.
//
// Replaces MIE_ONE (src/polarized/miewig.f:5-108) as called for every radius
// by COMPUTE_MIE_ALL_SIZES (src/polarized/make_mie_table.f90:381-482) with
// avgflag 'C'.  The result has the reference's meaning and layout:
//   extinct, scatter  cross sections pi r^2 Qext, pi r^2 Qsca [um^2];
//   nleg              min(maxleg, 2 nterms), nterms the series length;
//   legcoef[r][l][k]  the six Wigner-function expansion coefficients of the
//                     phase matrix (k = a1, a2, a3, a4, b1, b2) times the
//                     scattering cross section, so legcoef[r][0][0] = scatter.
//
// Method (own code, from the published algorithm):
// * the coefficients a_n, b_n of Bohren and Huffman (Absorption and Scattering
//   of Light by Small Particles, 1983, appendix A): the logarithmic derivative
//   D_n(mx) by downward recurrence from max(nterms, |mx|) + 15, the
//   Riccati-Bessel functions psi_n, chi_n by upward recurrence;
// * the series length nterms = x + 6.5 x^0.3334 + 2, the rule of MIECALC
//   (miewig.f:110-175), which fixes nleg;
// * the amplitudes S1, S2 at Gauss-Legendre nodes from the angular functions
//   pi_n, tau_n; for a node pair (mu, -mu) one pass serves both, since
//   pi_n(-mu) = (-1)^(n+1) pi_n(mu) and tau_n(-mu) = (-1)^n tau_n(mu);
// * P1 = (|S1|^2 + |S2|^2)/2, P2 = (|S2|^2 - |S1|^2)/2, P3 = Re(S1* S2),
//   P4 = -Im(S1* S2), projected on the Wigner d-functions d00, d22, d2-2,
//   d20 by the quadrature; the d-functions follow their three-term
//   recurrence in l, with d^l_{mn}(-mu) = (-1)^(l+m) d^l_{m,-n}(mu) giving the
//   negative node from the positive one.  a2, a3 come from the d22 and d2-2
//   projections of P1 + P3 and P1 - P3; b1, b2 carry a minus sign, as in the
//   reference's table (Rayleigh scattering has b1 > 0);
// * the quadrature has (nleg + 2 nterms + 2)/2 * 1.25 nodes (rounded up to a
//   multiple of 32 so that radii share node sets): it integrates the degree
//   nleg + 2 nterms products exactly.
//
// All host work; radii are shared out to threads largest first.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/shdom_gb300.h"

namespace shdom {
int host_fail(const std::string &m);
}

namespace {

using cd = std::complex<double>;

int series_terms(double x) { return (int)(x + 6.5 * std::pow(x, 0.3334) + 2.0); }

// Gauss-Legendre nodes in (0, 1) (descending) and weights on [-1, 1]: Newton
// iteration on P_n from the asymptotic first guess cos(pi (j - 1/4)/(n + 1/2)).
struct Quad {
  int n = 0;
  std::vector<double> mu, w;   // the n/2 (or (n+1)/2) non-negative nodes
};

Quad gauss_legendre(int n) {
  Quad q;
  q.n = n;
  const int k = (n + 1) / 2;
  q.mu.resize(k);
  q.w.resize(k);
  for (int j = 1; j <= k; ++j) {
    double x = std::cos(M_PI * (j - 0.25) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int l = 2; l <= n; ++l) {
        double p2 = ((2 * l - 1) * x * p1 - (l - 1) * p0) / l;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) p0 = 1.0;
      dp = n * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-15) break;
    }
    // recompute the derivative at the converged node
    {
      double p0 = 1.0, p1 = x;
      for (int l = 2; l <= n; ++l) {
        double p2 = ((2 * l - 1) * x * p1 - (l - 1) * p0) / l;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) p0 = 1.0;
      dp = n * (x * p1 - p0) / (x * x - 1.0);
    }
    q.mu[j - 1] = x;
    q.w[j - 1] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  return q;
}

// Recurrence factors of the Wigner d-functions: d_{l+1} = (A1 mu + A0) d_l - B d_{l-1}.
struct Wigner {
  std::vector<double> a1_00, b_00, a1_22, a0_22, b_22, a1_20, b_20;
  void build(int L) {
    a1_00.assign(L + 1, 0); b_00.assign(L + 1, 0);
    a1_22.assign(L + 1, 0); a0_22.assign(L + 1, 0); b_22.assign(L + 1, 0);
    a1_20.assign(L + 1, 0); b_20.assign(L + 1, 0);
    for (int l = 0; l <= L; ++l) {
      const double dl = l;
      a1_00[l] = (2 * dl + 1) / (dl + 1);
      b_00[l] = dl / (dl + 1);
      if (l >= 2) {
        const double q = (dl + 1) * (dl + 1) - 4.0;
        a1_22[l] = (2 * dl + 1) * (dl + 1) / q;
        a0_22[l] = -4.0 * (2 * dl + 1) / (dl * q);
        b_22[l] = (dl + 1) * (dl * dl - 4.0) / (dl * q);
        a1_20[l] = (2 * dl + 1) / std::sqrt(q);
        b_20[l] = std::sqrt(dl * dl - 4.0) / std::sqrt(q);
      }
    }
  }
};

struct MieJob {
  double wavelength;
  cd m;                 // Bohren-Huffman convention, Im(m) >= 0 absorbs
  int maxleg;
};

// One radius: cross sections and the scaled expansion coefficients.
void mie_radius(const MieJob &job, double radius, const Quad &q, const Wigner &W, float &ext_out,
                float &sca_out, int &nleg_out, float *leg_out) {
  const double x = 2.0 * M_PI * radius / job.wavelength;
  const int nt = std::max(1, series_terms(x));
  const cd y = job.m * x;
  const int nstart = std::max(nt, (int)std::ceil(std::abs(y))) + 15;
  std::vector<cd> D(nstart + 1);
  D[nstart] = 0.0;
  for (int n = nstart; n >= 1; --n) D[n - 1] = double(n) / y - 1.0 / (D[n] + double(n) / y);
  std::vector<cd> a(nt + 1), b(nt + 1);
  double psi0 = std::cos(x), psi1 = std::sin(x), chi0 = -std::sin(x), chi1 = std::cos(x);
  double sum_e = 0.0, sum_s = 0.0;
  for (int n = 1; n <= nt; ++n) {
    const double psi = (2 * n - 1) / x * psi1 - psi0;
    const double chi = (2 * n - 1) / x * chi1 - chi0;
    const cd xi(psi, -chi), xi1(psi1, -chi1);
    const cd ta = D[n] / job.m + double(n) / x;
    const cd tb = job.m * D[n] + double(n) / x;
    a[n] = (ta * psi - psi1) / (ta * xi - xi1);
    b[n] = (tb * psi - psi1) / (tb * xi - xi1);
    sum_e += (2 * n + 1) * (a[n].real() + b[n].real());
    sum_s += (2 * n + 1) * (std::norm(a[n]) + std::norm(b[n]));
    psi0 = psi1; psi1 = psi;
    chi0 = chi1; chi1 = chi;
  }
  const double area = M_PI * radius * radius;
  const double qext = 2.0 / (x * x) * sum_e, qsca = 2.0 / (x * x) * sum_s;
  const int L = std::min(job.maxleg, 2 * nt);
  // c_n a_n, c_n b_n with c_n = (2n+1)/(n(n+1))
  for (int n = 1; n <= nt; ++n) {
    const double c = (2.0 * n + 1.0) / (double(n) * (n + 1.0));
    a[n] *= c;
    b[n] *= c;
  }
  std::vector<double> coef(6 * (size_t)(L + 1), 0.0);   // a1, a2+a3, a2-a3, a4, b1, b2
  const int npair = (int)q.mu.size();
  for (int i = 0; i < npair; ++i) {
    const double mu = q.mu[i];
    const bool centre = (q.n % 2 == 1) && (i == npair - 1);   // mu = 0 counted once
    const double w = q.w[i];
    // amplitudes at +mu and -mu from even/odd partial sums
    cd se_api = 0, so_api = 0, se_btau = 0, so_btau = 0;   // S1 pieces
    cd se_atau = 0, so_atau = 0, se_bpi = 0, so_bpi = 0;   // S2 pieces
    double pim = 0.0, pin = 1.0;
    for (int n = 1; n <= nt; ++n) {
      const double tau = n * mu * pin - (n + 1) * pim;
      if (n & 1) {
        so_api += a[n] * pin; so_btau += b[n] * tau;
        so_atau += a[n] * tau; so_bpi += b[n] * pin;
      } else {
        se_api += a[n] * pin; se_btau += b[n] * tau;
        se_atau += a[n] * tau; se_bpi += b[n] * pin;
      }
      const double nx = ((2 * n + 1) * mu * pin - (n + 1) * pim) / n;
      pim = pin;
      pin = nx;
    }
    // pi_n(-mu) = (-1)^(n+1) pi_n(mu): odd n keep the sign; tau_n(-mu) = (-1)^n tau_n(mu)
    const cd s1p = se_api + so_api + se_btau + so_btau;
    const cd s2p = se_atau + so_atau + se_bpi + so_bpi;
    const cd s1m = -se_api + so_api + se_btau - so_btau;
    const cd s2m = se_atau - so_atau - se_bpi + so_bpi;
    auto elems = [](const cd &s1, const cd &s2, double *p) {
      const double n1 = std::norm(s1), n2 = std::norm(s2);
      const cd c = std::conj(s1) * s2;
      p[0] = 0.5 * (n1 + n2);
      p[1] = 0.5 * (n2 - n1);
      p[2] = c.real();
      p[3] = -c.imag();
    };
    double pp[4], pm[4];
    elems(s1p, s2p, pp);
    elems(s1m, s2m, pm);
    if (centre) {   // a single node at mu = 0: the pair sum would count it twice
      for (int k = 0; k < 4; ++k) pm[k] = 0.0;
    }
    // Wigner functions at +mu; the -mu values follow from parity:
    // d00(-mu) = (-1)^l d00(mu), d20(-mu) = (-1)^l d20(mu),
    // d2-2(+mu) = (-1)^l d22(-mu), d2-2(-mu) = (-1)^l d22(+mu).
    double d00m1 = 0.0, d00 = 1.0;
    double d22p_m1 = 0.0, d22p = 0.0, d22n_m1 = 0.0, d22n = 0.0, d20m1 = 0.0, d20 = 0.0;
    const double one_p = 1.0 + mu, one_m = 1.0 - mu;
    for (int l = 0; l <= L; ++l) {
      if (l == 2) {
        d22p = 0.25 * one_p * one_p;
        d22n = 0.25 * one_m * one_m;
        d20 = 0.25 * std::sqrt(6.0) * (1.0 - mu * mu);
      }
      const double sg = (l & 1) ? -1.0 : 1.0;
      const double f = (l + 0.5) * w;
      double *c = &coef[6 * (size_t)l];
      // a1, a4: P1, P3 against d00 at both nodes
      c[0] += f * d00 * (pp[0] + sg * pm[0]);
      c[3] += f * d00 * (pp[2] + sg * pm[2]);
      if (l >= 2) {
        // d22 at +mu is d22p, at -mu is d22n; d2-2 at +mu is sg d22n, at -mu sg d22p
        c[1] += f * ((pp[0] + pp[2]) * d22p + (pm[0] + pm[2]) * d22n);
        c[2] += f * sg * ((pp[0] - pp[2]) * d22n + (pm[0] - pm[2]) * d22p);
        c[4] -= f * d20 * (pp[1] + sg * pm[1]);
        c[5] -= f * d20 * (pp[3] + sg * pm[3]);
      }
      // advance to l + 1
      const double n00 = W.a1_00[l] * mu * d00 - W.b_00[l] * d00m1;
      d00m1 = d00; d00 = n00;
      if (l >= 2) {
        const double n22p = (W.a1_22[l] * mu + W.a0_22[l]) * d22p - W.b_22[l] * d22p_m1;
        const double n22n = (-W.a1_22[l] * mu + W.a0_22[l]) * d22n - W.b_22[l] * d22n_m1;
        const double n20 = W.a1_20[l] * mu * d20 - W.b_20[l] * d20m1;
        d22p_m1 = d22p; d22p = n22p;
        d22n_m1 = d22n; d22n = n22n;
        d20m1 = d20; d20 = n20;
      }
    }
  }
  const double scale = job.wavelength * job.wavelength / M_PI;
  for (int l = 0; l <= L; ++l) {
    const double *c = &coef[6 * (size_t)l];
    float *o = leg_out + 6 * (size_t)l;
    o[0] = (float)(scale * c[0]);
    o[1] = (float)(scale * 0.5 * (c[1] + c[2]));
    o[2] = (float)(scale * 0.5 * (c[1] - c[2]));
    o[3] = (float)(scale * c[3]);
    o[4] = (float)(scale * c[4]);
    o[5] = (float)(scale * c[5]);
  }
  ext_out = (float)(area * qext);
  sca_out = (float)(area * qsca);
  nleg_out = L;
}

int quad_nodes(int L, int nt) {
  const int base = (L + 2 * nt + 2) / 2;
  const int n = (int)std::ceil(1.25 * base);
  return (n + 31) / 32 * 32;
}

}  // namespace

extern "C" int shdom_mie_mono(double wavelength, double m_re, double m_im, int nsize, const float *radii,
                              int maxleg, int nthreads, float *extinct, float *scatter, int *nleg,
                              float *legcoef) {
  if (nsize < 0 || maxleg < 0) return shdom::host_fail("shdom_mie_mono: negative size");
  if (nsize == 0) return 0;
  if (!radii || !extinct || !scatter || !nleg || !legcoef)
    return shdom::host_fail("shdom_mie_mono: null argument");
  if (!(wavelength > 0.0)) return shdom::host_fail("shdom_mie_mono: wavelength must be positive");
  if (!(m_re > 0.0) || m_im > 0.0)
    return shdom::host_fail("shdom_mie_mono: refractive index must be n - ik with n > 0, k >= 0 (m_im <= 0)");
  for (int i = 0; i < nsize; ++i)
    if (!(radii[i] > 0.0f)) return shdom::host_fail("shdom_mie_mono: radii must be positive");
  MieJob job{wavelength, cd(m_re, -m_im), maxleg};
  // node sets by size: computed once each, shared by the radii that use them
  std::vector<int> nodes(nsize);
  std::map<int, std::unique_ptr<Quad>> quads;
  int Lmax = 0;
  for (int i = 0; i < nsize; ++i) {
    const double x = 2.0 * M_PI * radii[i] / wavelength;
    const int nt = std::max(1, series_terms(x));
    const int L = std::min(maxleg, 2 * nt);
    Lmax = std::max(Lmax, L);
    nodes[i] = quad_nodes(L, nt);
    quads.emplace(nodes[i], nullptr);
  }
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  {
    std::vector<int> keys;
    for (auto &kv : quads) keys.push_back(kv.first);
    std::atomic<int> next(0);
    auto work = [&]() {
      for (int k; (k = next.fetch_add(1)) < (int)keys.size();)
        quads[keys[k]].reset(new Quad(gauss_legendre(keys[k])));
    };
    std::vector<std::thread> th;
    for (int t = 1; t < std::min(nthreads, (int)keys.size()); ++t) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
  }
  Wigner W;
  W.build(Lmax + 1);
  std::fill(legcoef, legcoef + (size_t)nsize * (maxleg + 1) * 6, 0.0f);
  // largest radius first: the cost grows with the square of the size parameter
  std::vector<int> order(nsize);
  for (int i = 0; i < nsize; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int p, int r) { return radii[p] > radii[r]; });
  std::atomic<int> next(0);
  auto work = [&]() {
    for (int k; (k = next.fetch_add(1)) < nsize;) {
      const int i = order[k];
      mie_radius(job, radii[i], *quads.at(nodes[i]), W, extinct[i], scatter[i], nleg[i],
                 legcoef + (size_t)i * (maxleg + 1) * 6);
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < std::min(nthreads, nsize); ++t) th.emplace_back(work);
  work();
  for (auto &t : th) t.join();
  return 0;
}
