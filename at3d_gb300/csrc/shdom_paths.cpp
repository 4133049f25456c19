// shdom_paths.cpp -- ray integrals of the extinction field on the host plan
// (RTE.optical_path, at3d/solver.py:793-867; OPTICAL_DEPTH and
// OPTICAL_DEPTH_1RAY, src/shdomsub5.f:387-739).  A diagnostic the reference
// also runs on the CPU, before or after a solve; it reads the delta-M scaled
// species properties the plan keeps for the gradient.
#include <algorithm>
#include <cmath>
#include <thread>

#include "shdom_plan.h"

namespace shdom {
namespace {

// LOCATE_GRID_CELL (src/polarized/shdomsub2.f:4043-4215) on the base grid;
// wraps x and y into a periodic domain.
int locate_cell(const Plan &P, double &x0, double &y0, double z0) {
  const int nx = P.nx, ny = P.ny, nz = P.nz, bc = P.bcflag, ip = P.ipflag;
  const std::vector<float> &xg = P.xgrid, &yg = P.ygrid, &zg = P.zgrid;
  if (!(bc & 1)) {
    const double xd = xg[nx] - xg[0];
    if (x0 < xg[0]) x0 -= xd * ((int)((x0 - xg[0]) / xd) - 1);
    else if (x0 > xg[nx]) x0 -= xd * (int)((x0 - xg[0]) / xd);
  }
  if (!(bc & 2)) {
    const double yd = yg[ny] - yg[0];
    if (y0 < yg[0]) y0 -= yd * ((int)((y0 - yg[0]) / yd) - 1);
    else if (y0 > yg[ny]) y0 -= yd * (int)((y0 - yg[0]) / yd);
  }
  auto bisect = [](const std::vector<float> &g, int n, double v, bool mid) {
    int il = 0, iu = mid ? n : n + 1;
    while (iu - il > 1) {
      const int im = (iu + il) / 2;
      const double edge = mid ? 0.5 * (g[im - 1] + g[im]) : (double)g[im - 1];
      if (v >= edge) il = im; else iu = im;
    }
    return mid ? il + 1 : std::max(il, 1);
  };
  int ix = bisect(xg, nx, x0, ip & 1), iy = bisect(yg, ny, y0, ip & 2);
  int il = 0, iu = nz;
  while (iu - il > 1) { const int im = (iu + il) / 2; if (z0 >= zg[im - 1]) il = im; else iu = im; }
  const int iz = std::max(il, 1);
  int nyc = ny;
  if (bc & 1) ix = x0 < xg[0] ? 1 : x0 > xg[nx - 1] ? nx + 1 : ix + 1;
  if (bc & 2) {
    nyc = ny + 1;
    iy = y0 < yg[0] ? 1 : y0 > yg[ny - 1] ? ny + 1 : iy + 1;
  }
  return (iz - 1) + (nz - 1) * (iy - 1) + (nz - 1) * nyc * (ix - 1);
}

}  // namespace

bool ray_paths(const Plan &P, int n, const float *camx, const float *camy, const float *camz,
               const double *cammu, const double *camphi, int deltam_path, float *out, float *minpath, int do_all,
               std::string &err);

bool optical_path(const Plan &P, int n, const float *camx, const float *camy, const float *camz,
                  const double *cammu, const double *camphi, int deltam_path, float *out, std::string &err) {
  return ray_paths(P, n, camx, camy, camz, cammu, camphi, deltam_path, out, nullptr, 0, err);
}

bool min_optical_path(const Plan &P, int n, const float *camx, const float *camy, const float *camz,
                      const double *cammu, const double *camphi, int deltam_path, int do_all, float *minpath,
                      std::string &err) {
  if (!minpath) { err = "min_optical_path: null output"; return false; }
  std::vector<float> tau(std::max(n, 0));
  return ray_paths(P, n, camx, camy, camz, cammu, camphi, deltam_path, tau.data(), minpath, do_all, err);
}

// The ray walk shared by OPTICAL_DEPTH and MIN_OPTICAL_DEPTH
// (src/shdomsub5.f:17-385): out[r] the path of ray r; with minpath, after
// each cell crossing every corner of the cell keeps the smallest path so far
// ([npts], or [n][npts] per ray with do_all; 999 where no ray passed).
bool ray_paths(const Plan &P, int n, const float *camx, const float *camy, const float *camz,
               const double *cammu, const double *camphi, int deltam_path, float *out, float *minpath, int do_all,
               std::string &err) {
  if (n < 0 || (n > 0 && (!camx || !camy || !camz || !cammu || !camphi || !out))) {
    err = "optical_path: bad arguments";
    return false;
  }
  if (P.is1d || P.ipflag) { err = "optical_path: 3D grids only"; return false; }
  const int npts = P.npts, npart = P.prob.npart, nq = P.sp_nq, nl1 = P.nleg + 1, ml = P.ml;
  if (P.sp_ext.size() < (size_t)npart * npts || (size_t)nq * npart * npts > P.sp_pw.size()) {
    err = "optical_path: the plan holds no species properties";
    return false;
  }
  // Per point and species the extinction the path integrates: the delta-M
  // scaled value, or the unscaled one ext / (1 - w0 f) with the unscaled
  // albedo w0 = w / (f (w - 1) + 1) and f mixed as the reference does (every
  // phase weight, the single table row at PHASEMAX).
  std::vector<float> e((size_t)npart * npts);
  const bool unscale = P.prob.deltam && !deltam_path;
  for (int ipa = 0; ipa < npart; ++ipa)
    for (int ip = 0; ip < npts; ++ip) {
      const size_t o = (size_t)ipa * npts + ip;
      float ext = P.sp_ext[o];
      if (unscale) {
        const int *IP = &P.sp_iph[o * nq];
        const float *PW = &P.sp_pw[o * nq];
        float fm;
        if (PW[0] >= kPhaseMax) fm = P.leg[(size_t)(IP[0] - 1) * nl1 + ml + 1];
        else {
          fm = 0.f;
          for (int q = 0; q < nq; ++q) fm += PW[q] * P.leg[(size_t)(IP[q] - 1) * nl1 + ml + 1];
        }
        const float w = P.sp_alb[o];
        const float w0 = w / (fm * (w - 1.0f) + 1.0f);
        ext = ext / (1.0f - w0 * fm);
      }
      e[o] = ext;
    }
  const float *gp = P.gridpos.vec().data();
  const int *gptr = P.gridptr.vec().data(), *nbp = P.neighptr.vec().data(), *cf = P.cellflags.vec().data();
  const int nx = P.nx, ny = P.ny, nz = P.nz, bc = P.bcflag;
  const double zt = P.zgrid[nz - 1], zb = P.zgrid[0];
  const double eps = 1.0e-5 * (gp[3 * gptr[7] + 2] - gp[3 * gptr[0] + 2]);
  const int maxcross = 50 * std::max(nx, std::max(ny, nz));
  const float xm = 0.5f * (P.xgrid[0] + P.xgrid[nx - 1]), ym = 0.5f * (P.ygrid[0] + P.ygrid[ny - 1]);
  std::vector<std::string> errs;

  auto one_ray = [&](int r, float *mp, std::string &rerr) -> bool {
    double x0 = camx[r], y0 = camy[r], z0 = camz[r];
    const double mu2 = cammu[r], phi2 = camphi[r];
    const double muray = -mu2, phiray = phi2 - std::acos(-1.0);
    out[r] = 0.f;
    if (z0 > zt) {  // extrapolate to the domain top; a ray leaving upward sees nothing
      if (muray >= 0.0) return true;
      const double rr = (zt - z0) / muray;
      x0 += rr * std::sqrt(1 - muray * muray) * std::cos(phiray);
      y0 += rr * std::sqrt(1 - muray * muray) * std::sin(phiray);
      z0 = zt;
    } else if (z0 < zb) {
      rerr = "OPTICAL_DEPTH: level below the domain";
      return false;
    }
    double cx = std::sqrt(1.0 - muray * muray) * std::cos(phiray), cy = std::sqrt(1.0 - muray * muray) * std::sin(phiray);
    double cz = muray, cxi, cyi, czi;
    if (std::fabs(cx) > 1.0e-6) cxi = 1.0 / cx; else { cx = 0; cxi = 1.0e6; }
    if (std::fabs(cy) > 1.0e-6) cyi = 1.0 / cy; else { cy = 0; cyi = 1.0e6; }
    if (std::fabs(cz) > 1.0e-6) czi = 1.0 / cz; else { cz = 0; czi = 1.0e6; }
    const int bitx = cx < 0, bity = cy < 0, bitz = cz < 0, ioct = 1 + bitx + 2 * bity + 4 * bitz;
    double xe = x0, ye = y0, ze = z0;
    int icell = locate_cell(P, xe, ye, ze);
    auto ext_at = [&](int ic, double x, double y, double z) {
      const int *g = &gptr[8 * ic];
      const float *a = &gp[3 * g[0]], *b = &gp[3 * g[7]];
      const double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
      const double u = (x - a[0]) * (dx <= 0 ? 1.0 : 1.0 / dx), v = (y - a[1]) * (dy <= 0 ? 1.0 : 1.0 / dy),
                   w = (z - a[2]) * (1.0 / dz);
      const double f[8] = {(1 - w) * (1 - v) * (1 - u), (1 - w) * (1 - v) * u, (1 - w) * v * (1 - u), (1 - w) * v * u,
                           w * (1 - v) * (1 - u),       w * (1 - v) * u,       w * v * (1 - u),       w * v * u};
      float s = 0.f;
      for (int ipa = 0; ipa < npart; ++ipa)
        for (int j = 0; j < 8; ++j) s = (float)(s + f[j] * e[(size_t)ipa * npts + g[j]]);
      return s;
    };
    float tau = 0.f;
    for (int ngrid = 1; ngrid <= maxcross; ++ngrid) {
      const float ext1 = ext_at(icell, xe, ye, ze);
      const bool ipinx = (cf[icell] & 1) && !((bc & 1) && ((cx > 0 && xe < xm) || (cx < 0 && xe > xm)));
      const bool ipiny = (cf[icell] & 2) && !((bc & 2) && ((cy > 0 && ye < ym) || (cy < 0 && ye > ym)));
      const int iopp = gptr[8 * icell + (8 - ioct)];
      const double sox = ipinx ? 1e20 : (gp[3 * iopp] - xe) * cxi;
      const double soy = ipiny ? 1e20 : (gp[3 * iopp + 1] - ye) * cyi;
      const double soz = (gp[3 * iopp + 2] - ze) * czi;
      const double so = std::min(sox, std::min(soy, soz));
      if (so < -eps) { rerr = "OPTICAL_DEPTH: SO<0"; return false; }
      double xn = xe + so * cx, yn = ye + so * cy, zn = ze + so * cz;
      const float extn = ext_at(icell, xn, yn, zn);
      tau = (float)(tau + so * 0.5 * (ext1 + extn));
      if (mp) {
        float *col = do_all ? mp + (size_t)r * npts : mp;
        for (int k = 0; k < 8; ++k) { float &m = col[gptr[8 * icell + k]]; m = std::min(m, tau); }
      }
      int iface, jface;
      if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; }
      else if (soy <= soz) { iface = 3 - bity; jface = 1; }
      else { iface = 5 - bitz; jface = 2; }
      const int inext = nbp[6 * icell + iface];
      if (inext >= 0) {
        const int c = gptr[8 * inext + ioct - 1];
        if (jface == 0) xn = gp[3 * c]; else if (jface == 1) yn = gp[3 * c + 1]; else zn = gp[3 * c + 2];
      }
      if (inext < 0) break;
      xe = xn; ye = yn; ze = zn;
      icell = inext;
    }
    out[r] = tau;
    return true;
  };

  const int nt = std::max(1, std::min<int>(16, std::min<int>((int)std::thread::hardware_concurrency(), n / 64 + 1)));
  errs.assign(nt, std::string());
  // one minimum buffer per thread when the rays share it, folded afterwards
  std::vector<std::vector<float>> part(minpath && !do_all ? nt : 0);
  if (minpath) std::fill(minpath, minpath + (size_t)npts * (do_all ? n : 1), 999.0f);
  for (auto &v : part) v.assign(npts, 999.0f);
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&, t]() {
      float *mp = !minpath ? nullptr : do_all ? minpath : part[t].data();
      for (int r = t; r < n; r += nt)
        if (!one_ray(r, mp, errs[t])) return;
    });
  for (auto &th : pool) th.join();
  for (auto &v : part)
    for (int i = 0; i < npts; ++i) minpath[i] = std::min(minpath[i], v[i]);
  for (auto &m : errs)
    if (!m.empty()) { err = m; return false; }
  return true;
}

bool point_absorption(const Plan &P, float *absorb, float *emit, std::string &err) {
  const int npts = P.npts, npart = P.prob.npart;
  if (!absorb || !emit) { err = "point_absorption: null output"; return false; }
  if (P.sp_ext.size() < (size_t)npart * npts) { err = "point_absorption: the plan holds no species properties"; return false; }
  const bool thermal = P.prob.srctype == 'T' || P.prob.srctype == 'B';
  if (thermal && P.planckpt.size() < (size_t)npts) { err = "point_absorption: no Planck values"; return false; }
  for (int i = 0; i < npts; ++i) {
    float a = 0.f, e = 0.f;
    for (int ipa = 0; ipa < npart; ++ipa) {
      const size_t o = (size_t)ipa * npts + i;
      const float k = P.sp_ext[o], w = P.sp_alb[o];
      a += k * (1.0f - w);
      if (thermal) e += k * ((1.0f - w) * P.planckpt[i]);
    }
    absorb[i] = a;
    emit[i] = e;
  }
  return true;
}

}  // namespace shdom
