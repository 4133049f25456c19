// shdom_grad.cuh -- Levis approximate gradient on the GPU (included by
// shdom_gpu.cu after the render kernel, whose traversal it shares).
//
// LEVISAPPROX_GRADIENT, adjoint branch (src/polarized/shdomsub4.f:288-809):
// with the radiance field frozen, the derivative of a weighted sum of
// rendered radiances, sum_r w_r I_r, with respect to the extinction and
// single-scattering albedo of one species on the property grid is
//  (i)  the derivative of the local source x extinction at the grid points
//       a ray visits (GRAD8 of COMPUTE_SOURCE_GRAD_1CELL, :1546-2042),
//       integrated along the ray with the ray's transmission;
//  (ii) the change of the ray's own attenuation, weighted by the radiance
//       still to come from beyond each path interval
//       (COMPUTE_RADIANCE_DERIVATIVE_ADJOINT, :4037-4114);
//  (iii) the change of the direct solar beam at the points whose exact
//       single scattering (and surface reflection) the ray sees
//       (COMPUTE_DIRECT_BEAM_DERIV_ADJOINT, :4117-4143, with the sun-path
//       derivatives of DIRECT_BEAM_AND_PATHS_PROP, src/shdomsub5.f:1608-2345).
//
// One warp per ray, the eight corners of a cell on eight groups of four
// lanes as in k_render.  Instead of storing the path (the reference's
// PASSED* arrays) the ray is traversed twice: pass A sums the radiance
// contributions F_n, pass B recomputes them in the same order and gets the
// radiance still to come at interval n as (R - sum_{k<n} F_k) / T_n with an
// FP64 running sum.  Within a cell every interval's contribution to a
// corner is a scalar weight times that corner's GRAD8, so the FP64 atomics
// into the gradient are issued once per cell.
#pragma once

namespace shdom {

struct GradArgs {
  RenderArgs r;
  const float *radiance;                   // [npts][nlm]
  const int *nr;                           // radiance truncation per point
  const int *interpptr;                    // [npts][8] property point of each trilinear corner
  const float *optinterpwt;                // [npts][8]
  const float *planck;                     // thermal source: [npts] B(T) of each point, else null
  const float *dextm;                      // [ng][2] delta-M scaled d(extinction)/d(unknown)
  const float *dalbm, *dfj;                // [npts][8][2]
  const float *alb_sp;                     // [npts] scaled albedo of the species
  const int *sj_ptr, *sj_iph;              // CSR per point: mixed exact single scatter of the species
  const float *sj_w;
  const float *legent_u;                   // [npts][nl] species phase series, unscaled
  const float *legent_s;                   // [npts][nl] property-mixed, delta-M scaled (several species)
  const float *fmix;                       // [npts] (several species)
  const float *scatterj;                   // [npts]
  const float *legenp_u;                   // [ng][nl] unscaled phase series per property point
  const float *extp, *albp;                // [ng] species extinction and albedo
  const int *piph;                         // [ng][maxnmicro]
  const float *pphw;
  const double *adj;                       // [nrays] adjoint weight of each ray
  double *gradout;                         // [ng][2]
  double *beam;                            // [npts]
  const float *botalb;                     // surface albedo of the bottom points
  int npart, maxnmicro, ng;
  float scatmin;
};

constexpr int GWARPS = 4;

// Exact single scatter of phase function iph at this ray's scattering angle.
__device__ __forceinline__ float ss_phase(const RenderArgs &a, int sj, float sf, int iph) {
  return (1.f - sf) * a.phasetab[(size_t)sj * a.numphase + iph] + sf * a.phasetab[(size_t)(sj + 1) * a.numphase + iph];
}

// Sum over the four lanes of a corner group.  Only the group's lanes take
// part, so it may be called where the groups of a warp have diverged (a
// branch on the corner's point is uniform within its group).
__device__ __forceinline__ float group_sum(float v) {
  const unsigned gm = 0xfu << ((threadIdx.x & 31) & ~3u);
  v += __shfl_xor_sync(gm, v, 1);
  v += __shfl_xor_sync(gm, v, 2);
  return v;
}

template <bool GRAD>
__device__ void levis_traverse(const GradArgs &G, int ray, const float *ydir, const float *tl, double rtot,
                               double *rtot_out) {
  const RenderArgs &a = G.r;
  const int lane = threadIdx.x & 31, grp = lane >> 2, gl = lane & 3;
  const double pi = 3.141592653589793;
  double x0 = a.camx[ray], y0 = a.camy[ray], z0 = a.camz[ray], mu2 = a.cammu[ray], phi2 = a.camphi[ray];
  const double muray = -mu2, phiray = phi2 - pi;
  const float ztop = a.zgrid[a.nz - 1];
  if (z0 > ztop) {
    if (muray >= 0.0) { if (rtot_out) *rtot_out = 0.0; return; }
    double r = (ztop - z0) / muray;
    x0 += r * sqrt(1 - muray * muray) * cos(phiray);
    y0 += r * sqrt(1 - muray * muray) * sin(phiray);
    z0 = ztop;
  } else if (z0 < a.zgrid[0]) {
    if (lane == 0) atomicCAS(a.err, ERR_NONE, ERR_RAY_BELOW);
    if (rtot_out) *rtot_out = 0.0;
    return;
  }
  const double adj = GRAD ? G.adj[ray] : 0.0;
  int sj = 0;
  float sf = 0.f;
  if (a.deltam) {
    double cosscat = (double)a.solarmu * mu2 + sqrt((1.0 - (double)a.solarmu * a.solarmu) * (1.0 - mu2 * mu2)) * cos((double)a.solaraz - phi2);
    cosscat = fmax(fmin(1.0, cosscat), -1.0);
    float F = (float)((a.nscatangle - 1) * (acos(cosscat) / pi) + 1);
    int J = min(a.nscatangle - 1, (int)F);
    sf = F - J; sj = J - 1;
  }
  double cx = sqrt(1.0 - mu2 * mu2) * cos(phi2 - pi), cy = sqrt(1.0 - mu2 * mu2) * sin(phi2 - pi), cz = -mu2;
  double cxinv, cyinv, czinv;
  if (fabs(cx) > 1e-6) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1e6; }
  if (fabs(cy) > 1e-6) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1e6; }
  if (fabs(cz) > 1e-6) czinv = 1.0 / cz; else { cz = 0; czinv = 1e6; }
  const int bitx = cx < 0, bity = cy < 0, bitz = cz < 0, ioct0 = bitx + 2 * bity + 4 * bitz;
  const float xm = 0.5f * (a.xgrid[0] + a.xgrid[a.nx - 1]), ym = 0.5f * (a.ygrid[0] + a.ygrid[a.ny - 1]);
  double xe = x0, ye = y0, ze = z0;
  int cell = locate_cell(a, xe, ye, ze);
  const double eps = 1.0e-5 * (a.gridpos[3 * a.gridptr[7] + 2] - a.gridpos[3 * a.gridptr[0] + 2]);
  const double c12 = (double)0.08333333333f;
  const int nl = a.ml + 1;
  int oldp[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  float myJ = 0.f, myss = 0.f, myext = 0.f, g4[4] = {0.f, 0.f, 0.f, 0.f};
  double transmit = 1.0, cumf = 0.0, racc = 0.0;
  bool validrad = false;
  int guard = 0;
  while (!validrad && cell >= 0 && guard++ < (1 << 22)) {
    const int *g = a.gridptr + 8 * (size_t)cell;
    const int mypt = g[grp];
    int reuse = -1;
#pragma unroll
    for (int k = 0; k < 8; ++k) if (oldp[k] == mypt) reuse = k;
    // values of the reused corner from the group that held it
    const int srcl = reuse >= 0 ? 4 * reuse + gl : lane;
    const float oJ = __shfl_sync(0xffffffffu, myJ, srcl), oss = __shfl_sync(0xffffffffu, myss, srcl);
    const float oext = __shfl_sync(0xffffffffu, myext, srcl);
    float og[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) og[i] = __shfl_sync(0xffffffffu, g4[i], srcl);
    const bool need = reuse < 0;
    const int ns = need ? a.ns[mypt] : 0;
    float s = 0.f;
    {
      const float *S = a.source + (size_t)mypt * a.nlm;
      for (int j = gl; j < ns; j += 4) s += S[j] * ydir[j];
    }
    s = group_sum(s);
    // single scattering of the direct beam: with delta-M the exact term of
    // the unscaled phase function replaces the truncated one in the source;
    // without, the truncated term (from the series) is the single scatter
    float ss = 0.f;
    if (need) {
      const float da = a.dirflux[mypt] * a.secmu0;
      const float *cf = a.coef + (size_t)mypt * a.nl;
      float sub = 0.f;
      if (ns > 0) {
        int ls = a.lofj[ns - 1];
        for (int l = 0; l <= ls; ++l) sub += cf[l] * tl[l];
      }
      if (a.deltam) {
        s -= da * sub;
        float add = 0.f;
        for (int q = a.tms_ptr[mypt]; q < a.tms_ptr[mypt + 1]; ++q) add += a.tms_w[q] * ss_phase(a, sj, sf, a.tms_iph[q]);
        ss = da * add;
        s += ss;
      } else if (GRAD) {
        ss = da * sub;
      }
    }
    if (need) {
      myJ = s; myss = ss; myext = a.text[mypt];
      if (GRAD) {
        // COMPUTE_SOURCE_GRAD_1CELL for the species at this point
        const int ip = mypt;
        const float secmu0 = a.secmu0, dirf = a.dirflux[ip];
        float singscatj = 0.f;
        if (a.deltam) {
          float t = 0.f;
          for (int q = G.sj_ptr[ip] + gl; q < G.sj_ptr[ip + 1]; q += 4) t += G.sj_w[q] * ss_phase(a, sj, sf, G.sj_iph[q]);
          singscatj = group_sum(t);
        }
        // RY_l = sum_m R(l,m) Ydir(l,m) over the point's radiance terms; lane gl keeps l = gl, gl+4, ...
        float ry[8];
        const int rns = G.nr[ip];
        const float *Rp = G.radiance + (size_t)ip * a.nlm;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int l = gl + 4 * i;
          float v = 0.f;
          if (l < nl) {
            const int me = min(l, a.mm), j0 = (l <= a.mm) ? l * l : (2 * a.mm + 1) * l - a.mm * a.mm - a.mm;
            for (int k = 0; k < 2 * me + 1; ++k) {
              const int j = j0 + k;
              if (j < rns) v += Rp[j] * ydir[j];
            }
          }
          ry[i] = v;
        }
        auto dot_ry = [&](const float *f) {
          float t = 0.f;
#pragma unroll
          for (int i = 0; i < 8; ++i) { const int l = gl + 4 * i; if (l < nl) t += f[l] * ry[i]; }
          return group_sum(t);
        };
        auto dot_tl = [&](const float *f) {
          float t = 0.f;
          for (int l = gl; l < nl; l += 4) t += f[l] * tl[l];
          return group_sum(t);
        };
        float sourcet;
        const float albip = G.alb_sp[ip];
        if (G.npart == 1) {
          sourcet = (albip > 1e-8f) ? s / albip : 0.f;
        } else {
          sourcet = 0.f;
          if (G.scatterj[ip] > G.scatmin) {
            const float *ls = G.legent_s + (size_t)ip * nl;
            sourcet = dot_ry(ls);
            if (!a.deltam) sourcet += dirf * secmu0 * dot_tl(ls);
            else sourcet += dirf * singscatj * secmu0 / (1.f - G.fmix[ip]);
          }
        }
        sourcet = fmaxf(0.f, sourcet);
        const float *lt = G.legent_u + (size_t)ip * nl;
        // D2 = sum_l (lt_l - 1) RY_l, the DFJ part of DSOURCE
        float tmp[32];
        for (int l = 0; l < nl; ++l) tmp[l] = lt[l] - 1.f;
        const float d2 = dot_ry(tmp) + (a.deltam ? 0.f : dirf * secmu0 * dot_tl(tmp));
#pragma unroll
        for (int i = 0; i < 4; ++i) g4[i] = 0.f;
        for (int nb = 0; nb < 8; ++nb) {
          const float xi = G.optinterpwt[(size_t)ip * 8 + nb];
          if (xi < 1e-7f) continue;
          const int ib = G.interpptr[(size_t)ip * 8 + nb];
          const float *lp = G.legenp_u + (size_t)ib * nl;
          for (int l = 0; l < nl; ++l) tmp[l] = lp[l] - lt[l];
          const float d1 = dot_ry(tmp) + (a.deltam ? 0.f : dirf * secmu0 * dot_tl(tmp));
          float ssp = 0.f;
          if (a.deltam)
            for (int q = 0; q < G.maxnmicro; ++q) ssp += G.pphw[(size_t)ib * G.maxnmicro + q] * ss_phase(a, sj, sf, G.piph[(size_t)ib * G.maxnmicro + q] - 1);
          const float ep = G.extp[ib], ap = G.albp[ib];
#pragma unroll
          for (int d = 0; d < 2; ++d) {
            const float DE = d == 0 ? 1.f : 0.f, DA = d == 1 ? 1.f : 0.f;
            const float DFJ = G.dfj[((size_t)ip * 8 + nb) * 2 + d];
            const float dsource = (DE * ap + DA * ep) * d1 + DFJ * d2;
            float v = xi * (sourcet * (albip * G.dextm[(size_t)ib * 2 + d] + G.dalbm[((size_t)ip * 8 + nb) * 2 + d]) + dsource);
            // emission e (1 - albedo) B (src/polarized/shdomsub4.f:2009-2016), no temperature unknowns
            if (G.planck)
              v += xi * (G.planck[ip] * (1.f - albip) * G.dextm[(size_t)ib * 2 + d] -
                         G.planck[ip] * G.dalbm[((size_t)ip * 8 + nb) * 2 + d]);
            if (a.deltam) v += dirf * secmu0 * xi * (singscatj * DFJ + DA * (ssp - singscatj) * ep + DE * (ssp - singscatj) * ap);
            if ((nb >> 1) == gl) g4[(nb & 1) * 2 + d] = v;
          }
        }
      }
    } else {
      myJ = oJ; myss = oss; myext = oext;
#pragma unroll
      for (int i = 0; i < 4; ++i) g4[i] = og[i];
    }
    float ext8[8], src8[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float e = __shfl_sync(0xffffffffu, myext, 4 * k);
      ext8[k] = e;
      src8[k] = __shfl_sync(0xffffffffu, myJ, 4 * k) * e;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) oldp[k] = g[k];
    const int ip1 = g[0], ip2 = g[7];
    const float *P1 = a.gridpos + 3 * ip1, *P2 = a.gridpos + 3 * ip2;
    const float delx = P2[0] - P1[0], dely = P2[1] - P1[1], delz = P2[2] - P1[2];
    const double idx = delx <= 0.f ? 1.0 : 1.0 / delx, idy = dely <= 0.f ? 1.0 : 1.0 / dely, idz = 1.0 / delz;
    // Positions, path lengths and the trilinear weights are FP64, as in
    // ADJOINT_INTEGRATE_1RAY; the interpolated extinction and source are
    // single precision sums of FP64 products.  The weight terms of the
    // gradient divide by the interpolated extinction, which cancels to
    // nearly zero beside clouds and in the extrapolating open-boundary edge
    // cells, so FP32 weights (relative error 1e-7 of terms of size 50/km)
    // would not do there.
    auto kernel8 = [&](double s, double fc[8]) {
      const double u = (xe + s * cx - P1[0]) * idx, v = (ye + s * cy - P1[1]) * idy, w = (ze + s * cz - P1[2]) * idz;
      fc[0] = (1 - w) * (1 - v) * (1 - u); fc[1] = (1 - w) * (1 - v) * u; fc[2] = (1 - w) * v * (1 - u); fc[3] = (1 - w) * v * u;
      fc[4] = w * (1 - v) * (1 - u); fc[5] = w * (1 - v) * u; fc[6] = w * v * (1 - u); fc[7] = w * v * u;
    };
    // sum_k fc[k] val[k], each step rounded to single precision
    auto interp = [](const double fc[8], const float val[8]) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < 8; ++k) acc = (float)((double)acc + fc[k] * (double)val[k]);
      return acc;
    };
    double fc1[8], fc0[8];
    kernel8(0.0, fc1);
    float srcext1 = fmaxf(0.f, interp(fc1, src8));
    float ext1 = interp(fc1, ext8);
    const int cf = a.cellflags[cell];
    const bool ipinx = (cf & 1) && !((a.bcflag & 1) && ((cx > 0 && xe < xm) || (cx < 0 && xe > xm)));
    const bool ipiny = (cf & 2) && !((a.bcflag & 2) && ((cy > 0 && ye < ym) || (cy < 0 && ye > ym)));
    const int iopp = g[7 - ioct0];
    const double sox = ipinx ? 1e20 : (a.gridpos[3 * iopp] - xe) * cxinv;
    const double soy = ipiny ? 1e20 : (a.gridpos[3 * iopp + 1] - ye) * cyinv;
    const double soz = (a.gridpos[3 * iopp + 2] - ze) * czinv;
    const double so = fmin(sox, fmin(soy, soz));
    if (so < -eps) { if (lane == 0) atomicCAS(a.err, ERR_NONE, ERR_RAY_SO); break; }
    double xn = xe + so * cx, yn = ye + so * cy, zn = ze + so * cz;
    double fcn[8];
    kernel8(so, fcn);
    const float extn = interp(fcn, ext8);
    const double taugrid = so * 0.5 * (ext1 + extn);
    const int ntau = max(1, 1 + (int)(taugrid / a.tautol));
    const double dels = so / ntau;
    double accG = 0.0, accS = 0.0, accR = 0.0;  // per-cell weights of this lane's corner
    const float ss8 = myss * myext;                // this corner's single scatter x extinction
    for (int it = 1; it <= ntau; ++it) {
      kernel8(it * dels, fc0);
      float srcext0 = interp(fc0, src8);
      const float ext0 = it != ntau ? interp(fc0, ext8) : extn;
      srcext0 = fmaxf(0.f, srcext0);
      const double ext = 0.5 * ((double)ext0 + (double)ext1);
      double transcell;
      if (ext != 0.0) {
        const double tau = ext * dels;
        const double abscell = tau * (1.0 - 0.5 * tau * (1.0 - 0.33333333333 * tau));
        transcell = 1.0 - abscell;
        const double corr = dels * (1.0 - 0.05 * ((double)ext1 - (double)ext0) * dels);
        const double src = (0.5 * ((double)srcext0 + srcext1) + c12 * ((double)ext0 * srcext1 - (double)ext1 * srcext0) * corr) / ext;
        const double fn = transmit * src * abscell;
        if (GRAD) {
          const double w0 = fc0[grp], w1 = fc1[grp];
          const double wk = (0.5 * (w0 + w1) + c12 * ((double)ext0 * w1 - (double)ext1 * w0) * corr) / ext;
          accG += transmit * abscell * wk;
          // the single scatter is interpolated with each corner's term
          // clamped at zero (SINGSCAT0/1 of ADJOINT_INTEGRATE_1RAY); the
          // trilinear weights go negative where open-boundary edge cells
          // extrapolate beyond the cell
          const double s0 = fmaxf(0.f, (float)(w0 * ss8)), s1 = fmaxf(0.f, (float)(w1 * ss8));
          accS += transmit * abscell * (0.5 * (s0 + s1) + c12 * ((double)ext0 * s1 - (double)ext1 * s0) * corr) / ext;
          // radiance still to come from the start and from the end of this interval
          const double pr1 = (rtot - cumf) / transmit;
          const double tnext = transmit * transcell;
          const double pr0 = (rtot - cumf - fn) / tnext;
          double e0 = 0.0, e1 = 0.0;  // (COMPUTE_RADIANCE_DERIVATIVE_ADJOINT sums these in double)
#pragma unroll
          for (int k = 0; k < 8; ++k) { e0 += (double)ext8[k] * fc0[k]; e1 += (double)ext8[k] * fc1[k]; }
          const double eavg = 0.5 * (e0 + e1);
          if (eavg != 0.0) {
            const double gb0 = -adj * pr0 * w0, gb1 = -adj * pr1 * w1;
            double ag = (0.5 * (gb0 + gb1) + c12 * (e0 * gb1 - e1 * gb0) * dels * (1.0 - 0.05 * (e1 - e0) * dels)) / eavg;
            accR += ag * transmit * abscell;
          }
        }
        cumf += fn;
        racc += fn;
      } else {
        transcell = 1.0;
        accS = 0.0;
      }
      transmit *= transcell;
      ext1 = ext0; srcext1 = srcext0;
#pragma unroll
      for (int k = 0; k < 8; ++k) fc1[k] = fc0[k];
    }
    if (GRAD) {
      // source-gradient and attenuation terms for this lane's corner, property neighbours 2gl and 2gl+1
      const int ip = mypt;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int nb = 2 * gl + h;
        const float xi = G.optinterpwt[(size_t)ip * 8 + nb];
        const int ib = G.interpptr[(size_t)ip * 8 + nb];
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          const double v = adj * accG * (double)g4[h * 2 + d];
          const float eg = G.dextm[(size_t)ib * 2 + d] * xi;
          const double r = (double)eg * accR;
          const double tot = v + r;
          if (tot != 0.0) atomicAdd(&G.gradout[(size_t)ib * 2 + d], tot);
        }
      }
      if (gl == 0 && accS != 0.0) {
        const double bw = adj * accS;
        if (bw != 0.0) atomicAdd(&G.beam[ip], bw);
      }
    }
    int iface, jface;
    bool openbc;
    if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; openbc = (cf & 1) && (a.bcflag & 1); }
    else if (soy <= soz) { iface = 3 - bity; jface = 1; openbc = (cf & 2) && (a.bcflag & 2); }
    else { iface = 5 - bitz; jface = 2; openbc = false; }
    const int nxt = a.neighptr[6 * (size_t)cell + iface];
    int kface = iface, kc = cell;
    if (openbc) { kface = iface ^ 1; kc = nxt; iface = -1; }
    if (nxt >= 0) {
      const float *q = a.gridpos + 3 * a.gridptr[8 * (size_t)nxt + ioct0];
      if (jface == 0) xn = q[0]; else if (jface == 1) yn = q[1]; else zn = q[2];
    }
    if (transmit < a.transcut) {
      validrad = true;
    } else if (nxt < 0 && iface >= 4) {
      validrad = true;
      const int *gk = a.gridptr + 8 * (size_t)kc;
      float xs[4], ys[4], rb[4], dr[4];
      int bp[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int q = gk[c_face[kface][k]];
        bp[k] = q; xs[k] = a.gridpos[3 * q]; ys[k] = a.gridpos[3 * q + 1]; dr[k] = 0.f;
        if ((float)mu2 < 0.f) rb[k] = a.skyrad;
        else {
          const int bi = a.bot_index[q];
          rb[k] = bi >= 0 ? a.bcrad_bot[bi] : 0.f;
          if (bi >= 0) dr[k] = 0.318309886f * G.botalb[bi] * a.dirflux[q];
        }
      }
      const double uu = (xs[1] - xs[0] > 0) ? (xn - xs[0]) / (xs[1] - xs[0]) : 0.0;
      const double vv = (ys[2] - ys[0] > 0) ? (yn - ys[0]) / (ys[2] - ys[0]) : 0.0;
      const double bi4[4] = {(1 - uu) * (1 - vv), uu * (1 - vv), (1 - uu) * vv, uu * vv};
      const float radbnd = (float)(bi4[0] * rb[0] + bi4[1] * rb[1] + bi4[2] * rb[2] + bi4[3] * rb[3]);
      racc += transmit * radbnd;
      if (GRAD && lane < 4) {
        const double bw = adj * transmit * bi4[lane] * (double)dr[lane];
        if (bw != 0.0) atomicAdd(&G.beam[bp[lane]], bw);
      }
    } else {
      cell = nxt;
    }
    xe = xn; ye = yn; ze = zn;
  }
  if (rtot_out) *rtot_out = racc;
}

// Pass A then pass B for each ray (one warp per ray).
__global__ void __launch_bounds__(GWARPS * 32) k_levis_adjoint(GradArgs G) {
  __shared__ float ydir_s[GWARPS][RNLM];
  __shared__ float tl_s[GWARPS][64];
  const RenderArgs &a = G.r;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ray = blockIdx.x * GWARPS + w;
  if (ray >= a.nrays) return;
  if (G.adj[ray] == 0.0) return;
  float *ydir = ydir_s[w], *tl = tl_s[w];
  ylm_dir_warp(ydir, (float)a.cammu[ray], (float)a.camphi[ray], a.ml, a.mm, lane);
  __syncwarp();
  for (int l = lane; l <= a.ml; l += 32) {
    int me = min(l, a.mm), j0 = (l <= a.mm) ? l * l : (2 * a.mm + 1) * l - a.mm * a.mm - a.mm;
    float s = 0.f;
    for (int k = 0; k < 2 * me + 1; ++k) s += ydir[j0 + k] * a.ylmsun[j0 + k];
    tl[l] = s;
  }
  __syncwarp();
  double rtot = 0.0;
  levis_traverse<false>(G, ray, ydir, tl, 0.0, &rtot);
  levis_traverse<true>(G, ray, ydir, tl, rtot, nullptr);
}

// Direct-beam term: for each point with a non-zero beam weight, the sun
// path's d(optical path)/d(extinction) per property corner, cell by cell
// (the path of DIRECT_BEAM_PROP).
struct BeamArgs {
  const float *gridpos, *zlev;
  const double *beam;
  const float *dextm;
  double *gradout;
  int npts, npx, npy, npz, bcflag, ipflag;
  float delx, dely, solarmu, solaraz;
};

__global__ void k_levis_beam(BeamArgs b) {
  const int ipt = blockIdx.x * blockDim.x + threadIdx.x;
  if (ipt >= b.npts) return;
  const double weight = b.beam[ipt];
  if (weight == 0.0) return;
  const int npx = b.npx, npy = b.npy, npz = b.npz, bcflag = b.bcflag;
  int ipdirect = b.ipflag;
  if (b.ipflag & 4) ipdirect = 0;
  const double sunmu = -(double)b.solarmu, sunaz = (double)(float)(b.solaraz + 3.14159265f);
  double cx = sqrt(1.0 - sunmu * sunmu) * cos(sunaz), cy = sqrt(1.0 - sunmu * sunmu) * sin(sunaz);
  double cz = fabs(sunmu), cxinv, cyinv, czinv;
  if (fabs(cx) > 1e-6) cxinv = 1.0 / cx; else { cx = 0; cxinv = 1e20; }
  if (fabs(cy) > 1e-6) cyinv = 1.0 / cy; else { cy = 0; cyinv = 1e20; }
  if (fabs(cz) > 1e-6) czinv = 1.0 / cz; else { cz = 0; czinv = 1e20; }
  const int di = cx >= 0 ? 1 : -1, dj = cy >= 0 ? 1 : -1, dk = cz >= 0 ? 1 : -1;
  const double epsz = 1.0e-6 * (b.zlev[npz - 1] - b.zlev[0]);
  const double delxd = b.delx, delyd = b.dely, xdomain = delxd * npx, ydomain = delyd * npy;
  const double z = b.gridpos[3 * ipt + 2], x = b.gridpos[3 * ipt], y = b.gridpos[3 * ipt + 1];
  int il = 0, iu = npz;
  while (iu - il > 1) { int im = (iu + il) / 2; if (z >= b.zlev[im - 1]) il = im; else iu = im; }
  int k = max(il, 1);
  int i = (int)(x / delxd) + 1;
  if (i > npx && fabs(x - xdomain) < 0.001 * delxd) i = npx;
  int j = (int)(y / delyd) + 1;
  if (j > npy && fabs(y - ydomain) < 0.001 * delyd) j = npy;
  double xe = x, ye = y, ze = z, xp = xe, yp = ye, zp = ze;
  bool constx = ipdirect & 1, consty = ipdirect & 2;
  if (cx == 0.0) constx = true;
  if (cy == 0.0) consty = true;
  if ((bcflag & 1) && (fabs(x) < 0.01 * delxd || fabs(x - (npx - 1) * delxd) < 0.01 * delxd)) constx = true;
  if ((bcflag & 2) && (fabs(y) < 0.01 * delyd || fabs(y - (npy - 1) * delyd) < 0.01 * delyd)) consty = true;
  const int guard_max = 4 * (npx + npy + npz) * 64;
  for (int guard = 0; fabs(ze - b.zlev[npz - 1]) > epsz && guard < guard_max; ++guard) {
    int ipn = i + 1;
    if (i == npx) ipn = (bcflag & 1) ? npx : 1;
    int jpn = j + 1;
    if (j == npy) jpn = (bcflag & 2) ? npy : 1;
    const double x0 = delxd * (i - 1), x1 = x0 + delxd, y0 = delyd * (j - 1), y1 = y0 + delyd;
    const double z0 = b.zlev[k - 1], z1 = b.zlev[k];
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
    so = fmax(so, 0.0);
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
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float dpath = (float)(so * (A[c] + 0.5 * B[c] + 0.3333333333333333 * C[c] + sgn[c] * 0.25 * ddd));
      if (dpath == 0.f) continue;
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        const double v = -(double)b.dextm[(size_t)ptrs[c] * 2 + d] * dpath * weight;
        if (v != 0.0) atomicAdd(&b.gradout[(size_t)ptrs[c] * 2 + d], v);
      }
    }
    xe = xp + xoffs; ye = yp + yoffs; ze = zp;
  }
}

}  // namespace shdom
