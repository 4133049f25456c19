// shdom_gpu.cu -- device kernels and the C-ABI (include/shdom_gb300.h) of
// the GB300 SHDOM solve / render path.
//
// One iteration (SOLUTION_ITERATIONS, src/polarized/shdomsub1.f:674-797):
//   1. SH -> DO   : SRCDO[p][c] = max(0, source in ordinate c)  (tensor-core
//                   k_tc_gemm, or the factorized k_sh_to_do)
//   2. sweeps     : downward ordinates, Lambertian bottom, upward ordinates;
//                   boundary-plane chains (k_sweep_p1) beside the source
//                   pass (k_sweep_prep), then the wavefront levels
//                   (k_sweep_levels, or one k_sweep per level); grids whose
//                   wavefront is too deep are walked in the reference order
//                   (k_sweep_seq)
//   3. DO -> SH   : RADIANCE[p][j] from the ordinate radiances (masked to
//                   the point's radiance truncation) + hemispheric fluxes
//                   (k_tc_gemm, or k_do_to_sh)
//   4. source     : k_source (COMPUTE_SOURCE fused: dot products in FP64,
//                   delta-source, new truncation, next radiance truncation)
//   5. k_accel_param, k_accelerate (CALC_ACCEL_SOLCRIT, ACCELERATE_SOLUTION)
// Layouts are dense: [point][term] for the spherical-harmonic fields (terms
// beyond a point's truncation are zero) and [point][column] for the
// ordinate fields, columns grouped by hemisphere and trace octant.

#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <list>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/shdom_gb300.h"
#include "shdom_plan.h"
#include "shdom_tc.cuh"

namespace shdom {

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                               " at " #x);                                           \
    }                                                                                \
  } while (0)

// Device error codes written to Dev::err (first error wins).
enum {
  ERR_NONE = 0, ERR_SWEEP_NOFACE = 1, ERR_SWEEP_STEPS = 2, ERR_RAY_STEPS = 3, ERR_RAY_SO = 4, ERR_RAY_BELOW = 5,
  ERR_TC_WAIT = 6  // a tensor-core transform gave up waiting on its pipeline
};

__constant__ int c_face[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};

// ------------------------------------------------------------ transforms
// Spherical harmonics <-> discrete ordinates, factorized as in SH_TO_DO_UNPOL
// and DO_TO_SH_UNPOL (src/polarized/shdomsub1.f:2928-3036, :3164-3254): a
// Legendre contraction over l for each azimuthal mode m (CMU1/CMU2) and an
// azimuthal Fourier synthesis/analysis per zenith angle (CPHI1/CPHI2; the
// reference's FFT branch is the same linear map).  One warp per point; for
// the Legendre step lane t handles mode m = t - mm, for the Fourier step the
// lanes run over azimuths (synthesis) or modes (analysis).
struct XfArgs {
  const float *cmu;      // [nlm][nmu] (CMU1 for sh_to_do, CMU2 for do_to_sh)
  const float *cphi;     // sh_to_do: [nmu][nm][nphi0max] (CPHI1 transposed); do_to_sh: [nmu][nphi0max][nm]
  const int *nphi0, *col_of;
  const float *fluxw;
  const int *nr;
  float *fluxes;
  int npts, nlm, ml, mm, nmu, nang, nphi0max, ncol_down;
  int ldo;               // row stride of the ordinate arrays (nang rounded up to 4)
};

__device__ __forceinline__ int jindex(int l, int m, int mm) {
  return (l <= mm) ? l * (l + 1) + m : (2 * mm + 1) * l - mm * mm + m;
}

template <int NMU>
__global__ void __launch_bounds__(256) k_sh_to_do(XfArgs x, const float *__restrict__ S, float *__restrict__ srcdo) {
  extern __shared__ float sm[];
  const int nm = 2 * x.mm + 1;
  float *scmu = sm;                                   // [nlm][NMU+1]
  float *sw = sm + x.nlm * (NMU + 1) + (threadIdx.x >> 5) * NMU * nm;
  for (int t = threadIdx.x; t < x.nlm * NMU; t += blockDim.x) {
    int j = t / NMU, i = t - j * NMU;
    scmu[j * (NMU + 1) + i] = (i < x.nmu) ? x.cmu[(size_t)j * x.nmu + i] : 0.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool active = lane < nm;
  const int m = lane - x.mm, ma = m < 0 ? -m : m;
  const int partner = active ? 2 * x.mm - lane : lane;
  for (int p = warp; p < x.npts; p += nwarps) {
    const float *Sp = S + (size_t)p * x.nlm;
    float U[NMU];
#pragma unroll
    for (int i = 0; i < NMU; ++i) U[i] = 0.f;
    if (active)
      for (int l = ma; l <= x.ml; ++l) {
        const int j = jindex(l, m, x.mm);
        const float sv = Sp[j];
        const float *c = scmu + j * (NMU + 1);
#pragma unroll
        for (int i = 0; i < NMU; ++i) U[i] = fmaf(c[i], sv, U[i]);
      }
#pragma unroll
    for (int i = 0; i < NMU; ++i) {
      const float up = __shfl_sync(0xffffffffu, U[i], partner);
      if (active && i < x.nmu) {
        const int me = max(0, x.nphi0[i] / 2 - 1);
        float cs = (m == 0) ? U[i] : (m > 0 ? U[i] + up : U[i] - up);
        sw[i * nm + lane] = (ma <= me) ? cs : 0.f;
      }
    }
    __syncwarp();
    for (int i = 0; i < x.nmu; ++i) {
      const int n0 = x.nphi0[i], me = max(0, n0 / 2 - 1);
      const float *cs = sw + i * nm + x.mm;
      for (int k = lane; k < n0; k += 32) {
        const float *c = x.cphi + ((size_t)i * nm + x.mm) * x.nphi0max + k;
        float o = 0.f;
        for (int mm2 = -me; mm2 <= me; ++mm2) o = fmaf(c[mm2 * x.nphi0max], cs[mm2], o);
        srcdo[(size_t)p * x.ldo + x.col_of[i * x.nphi0max + k]] = fmaxf(o, 0.f);
      }
    }
    __syncwarp();
  }
}

template <int NMU>
__global__ void __launch_bounds__(256) k_do_to_sh(XfArgs x, const float *__restrict__ raddo, float *__restrict__ R) {
  extern __shared__ float sm[];
  const int nm = 2 * x.mm + 1;
  float *scmu = sm;                                               // [nlm][NMU+1]
  float *sr = sm + x.nlm * (NMU + 1) + (threadIdx.x >> 5) * x.nang;  // this warp's ordinate radiances
  for (int t = threadIdx.x; t < x.nlm * NMU; t += blockDim.x) {
    int j = t / NMU, i = t - j * NMU;
    scmu[j * (NMU + 1) + i] = (i < x.nmu) ? x.cmu[(size_t)j * x.nmu + i] : 0.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool active = lane < nm;
  const int m = lane - x.mm, ma = m < 0 ? -m : m;
  const int partner = active ? 2 * x.mm - lane : lane;
  for (int p = warp; p < x.npts; p += nwarps) {
    float fd = 0.f, fu = 0.f;
    for (int c = lane; c < x.nang; c += 32) {
      const float r = raddo[(size_t)p * x.ldo + c];
      sr[c] = r;
      const float w = x.fluxw[c] * r;
      if (c < x.ncol_down) fd += w; else fu += w;
    }
    for (int o = 16; o > 0; o >>= 1) {
      fd += __shfl_xor_sync(0xffffffffu, fd, o);
      fu += __shfl_xor_sync(0xffffffffu, fu, o);
    }
    if (lane == 0) { x.fluxes[2 * (size_t)p] = fd; x.fluxes[2 * (size_t)p + 1] = fu; }
    __syncwarp();
    float CS[NMU];
#pragma unroll
    for (int i = 0; i < NMU; ++i) {
      CS[i] = 0.f;
      if (active && i < x.nmu) {
        const int n0 = x.nphi0[i], me = max(0, n0 / 2 - 1);
        if (ma <= me) {
          const float *c = x.cphi + (size_t)i * x.nphi0max * nm + lane;
          const int *co = x.col_of + i * x.nphi0max;
          float s = 0.f;
          for (int k = 0; k < n0; ++k) s = fmaf(c[k * nm], sr[co[k]], s);
          CS[i] = s;
        }
      }
    }
    const int nrp = x.nr[p];
    float *Rp = R + (size_t)p * x.nlm;
#pragma unroll
    for (int i = 0; i < NMU; ++i) {
      const float cp = __shfl_sync(0xffffffffu, CS[i], partner);
      CS[i] = (m == 0) ? CS[i] : (m > 0 ? CS[i] - cp : cp + CS[i]);  // SUMUV(m)
    }
    if (active)
      for (int l = ma; l <= x.ml; ++l) {
        const int j = jindex(l, m, x.mm);
        const float *c = scmu + j * (NMU + 1);
        float v = 0.f;
#pragma unroll
        for (int i = 0; i < NMU; ++i) v = fmaf(c[i], CS[i], v);
        Rp[j] = (j < nrp) ? v : 0.f;
      }
    __syncwarp();
  }
}

// ----------------------------------------------------------------- sweep
// Final face of a general (not regular) trace: corner indices q and the
// bilinear face coordinates.  g = (so, u, v, 1) for a trace that stops on
// the first face it meets (the open-boundary edge cells, points off their
// start cell's corner), built once per handle; g.w = 0 for a trace that
// needs the run-time cell walk, whose face the source pass writes each
// iteration (q, and g = (0, u, v, 0)).
struct IrrRec {
  int4 q;
  float4 g;
};

// A trace reduced to what the radiance combination needs: rad = radsrc +
// tr * sum_k f_k(u, v) rad(q_k), f the bilinear weights of the stopping face.
struct TraceRec {
  float radsrc, tr, u, v;
  int4 q;
};

struct SweepArgs {
  const float *gridpos;
  const int *gridptr, *neighptr, *cellflags;
  const uint8_t *bnd;
  const int *rank, *start, *level;  // level: [8 octants][4 face classes][npts]
  const float *text, *srcdo;
  float *raddo;
  const float *col_cx, *col_cy, *col_cz;
  const uint32_t *tasks;          // point indices of the level schedule
  const uint8_t *regular;
  const float *geo;
  const IrrRec *irr;               // stored single-cell general traces of this hemisphere
  const uint8_t *stk;              // polarized: Stokes component per column (null: all I)
  int *err;
  int npts, nang, ldo, is1d, nz, ny1, nx1;
  float transmin;
  int oct_col0[8], oct_ncol[8];
};

// One backward short-characteristic trace (BACK_INT_GRID3D_UNPOL,
// src/polarized/shdomsub1.f:3695-4038, and BACK_INT_GRID1D :4295-4465 for the
// 1D independent-pixel case) up to the face it stops at.  The result does
// not depend on radiance values: rad(P) = radsrc + tr * sum_k f[k] rad(q[k]).
// A face is usable when each corner is a preset boundary point or precedes P
// in the reference sweep order (and, with use_level, sits at a lower
// wavefront level, so level-synchronous execution never reads a value that
// is not yet computed).
struct Trace {
  float radsrc, tr, f[4], u, v;  // u, v: bilinear coordinates of the final face
  int q[4];
  int status;  // 0 ok, ERR_* otherwise
};

// Regular-point traces: one interior cell, exit geometry (so, u, v, face)
// from the per-(layer, ordinate) table, corner indices by arithmetic on the
// (x, y, z) point numbering of the base grid.  Split in a load step (all
// memory reads, no use of their values) and a combine step so that a thread
// can keep the reads of several traces in flight.
struct RegLoad {
  float4 g;
  float e1, s1, e[4], s[4], r[4];
  int pt, col;
  bool clamp;  // the column holds I (its cell source is kept non-negative)
};

__device__ __forceinline__ void reg_load(const SweepArgs &a, int b, int pt, int col, RegLoad &x, bool upstream) {
  const int ldo = a.ldo;
  const int iz = pt % a.nz;
  const int layer = (b & 4) ? iz - 1 : iz;
  x.pt = pt; x.col = col;
  x.clamp = !a.stk || !a.stk[col];
  x.g = __ldg(reinterpret_cast<const float4 *>(a.geo) + (size_t)layer * a.nang + col);
  const int iface = (int)x.g.w;
  const int ox = (b & 1) ? -a.nz * a.ny1 : a.nz * a.ny1, oy = (b & 2) ? -a.nz : a.nz, oz = (b & 4) ? -1 : 1;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int d = c_face[iface][k] ^ b;
    const int q = pt + ((d & 1) ? ox : 0) + ((d & 2) ? oy : 0) + ((d & 4) ? oz : 0);
    x.e[k] = __ldg(a.text + q);
    x.s[k] = __ldg(a.srcdo + (size_t)q * ldo + col);
    x.r[k] = upstream ? a.raddo[(size_t)q * ldo + col] : 0.f;
  }
  x.e1 = __ldg(a.text + pt);
  x.s1 = __ldg(a.srcdo + (size_t)pt * ldo + col);
}

// Same inputs for a stored single-cell general trace.
__device__ __forceinline__ void rec_load(const SweepArgs &a, const IrrRec &rec, int pt, int col, RegLoad &x,
                                         bool upstream) {
  const int ldo = a.ldo;
  x.pt = pt; x.col = col;
  x.clamp = !a.stk || !a.stk[col];
  x.g = rec.g;
  const int q[4] = {rec.q.x, rec.q.y, rec.q.z, rec.q.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    x.e[k] = __ldg(a.text + q[k]);
    x.s[k] = __ldg(a.srcdo + (size_t)q[k] * ldo + col);
    x.r[k] = upstream ? a.raddo[(size_t)q[k] * ldo + col] : 0.f;
  }
  x.e1 = __ldg(a.text + pt);
  x.s1 = __ldg(a.srcdo + (size_t)pt * ldo + col);
}

// Source integral over one cell (the reference's linear-in-tau source
// approximation, with the large-tau limiting form).  Quotients use the
// fast reciprocal-based division (2 ulp), which keeps the integral free of
// the IEEE division's slow-path branches.
__device__ __forceinline__ void cell_source(float ext0, float srcext0, float ext1, float srcext1, float so,
                                            float &radsrc, float &transcell, bool clamp = true) {
  const float ext = 0.5f * (ext0 + ext1), tau = ext * so;
  float abscell, src;
  if (tau >= 0.5f) { transcell = __expf(-tau); abscell = 1.f - transcell; }
  else {
    abscell = tau * (1.f - 0.5f * tau * (1.f - 0.33333333333f * tau * (1.f - 0.25f * tau)));
    transcell = 1.f - abscell;
  }
  if (tau <= 2.f) {
    src = (ext == 0.f) ? 0.f
                       : __fdividef(0.5f * (srcext0 + srcext1) + 0.08333333333f * (ext0 * srcext1 - ext1 * srcext0) * so, ext);
  } else {
    float ext0p = ext0, srcext0p = srcext0;
    if (tau > 4.f) {
      ext0p = ext1 + __fdividef((ext0 - ext1) * 4.f, tau);
      if (ext0 > 0.f) srcext0p = __fdividef(srcext0 * ext0p, ext0);
    }
    const float rs = __fdividef(1.f, ext0p + ext1);
    src = rs * (srcext0p + srcext1 + (ext0p * srcext1 - ext1 * srcext0p) * 2.f * rs *
                                         (1.f - __fdividef(2.f, tau) + __fdividef(2.f * transcell, abscell)));
  }
  if (clamp) src = fmaxf(src, 0.f);  // the I source only; Q and U keep their sign
  radsrc = src * abscell;
}

__device__ __forceinline__ Trace reg_trace(const RegLoad &x, int b, int pt_unused) {
  Trace t;
  const float u = x.g.y, v = x.g.z;
  t.u = u; t.v = v;
  t.f[0] = (1.f - u) * (1.f - v); t.f[1] = (1.f - u) * v; t.f[2] = u * (1.f - v); t.f[3] = u * v;
  float ext0 = 0.f, srcext0 = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    ext0 += t.f[k] * x.e[k];
    srcext0 += t.f[k] * x.s[k] * x.e[k];
  }
  cell_source(ext0, srcext0, x.e1, x.e1 * x.s1, x.g.x, t.radsrc, t.tr, x.clamp);
  t.status = ERR_NONE;
  return t;
}

__device__ __forceinline__ Trace trace_regular(const SweepArgs &a, int b, int pt, int col) {
  RegLoad x;
  reg_load(a, b, pt, col, x, false);
  Trace t = reg_trace(x, b, pt);
  const int iface = (int)x.g.w;
  const int ox = (b & 1) ? -a.nz * a.ny1 : a.nz * a.ny1, oy = (b & 2) ? -a.nz : a.nz, oz = (b & 4) ? -1 : 1;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int d = c_face[iface][k] ^ b;
    t.q[k] = pt + ((d & 1) ? ox : 0) + ((d & 2) ? oy : 0) + ((d & 4) ? oz : 0);
  }
  return t;
}

// Exit of a backward trace from (xe, ye, ze) through one cell of a 3D grid
// (the geometry step of BACK_INT_GRID3D): the face's four corners, the next
// cell, the path length and the bilinear face coordinates; the position is
// advanced to the exit point.
struct CellExit {
  int i[4];
  int nxt;
  float so, u, v;
};

__device__ __forceinline__ CellExit cell_exit3d(const SweepArgs &a, int b, int cell, float &xe, float &ye, float &ze,
                                                float cx, float cy, float cz, float cxinv, float cyinv, float czinv) {
  CellExit c;
  const int bitx = cx < 0.f, bity = cy < 0.f, bitz = cz < 0.f;
  const int *g = a.gridptr + 8 * (size_t)cell;
  const int cf = a.cellflags[cell];
  const bool ipx = cf & 1, ipy = cf & 2;
  const int iopp = g[7 - b];
  float sox = ipx ? 1.0e20f : (a.gridpos[3 * iopp] - xe) * cxinv;
  float soy = ipy ? 1.0e20f : (a.gridpos[3 * iopp + 1] - ye) * cyinv;
  float soz = (a.gridpos[3 * iopp + 2] - ze) * czinv;
  c.so = fminf(sox, fminf(soy, soz));
  xe += c.so * cx; ye += c.so * cy; ze += c.so * cz;
  int iface, jface;
  if (sox <= soz && sox <= soy) { iface = 1 - bitx; jface = 0; }
  else if (soy <= soz) { iface = 3 - bity; jface = 1; }
  else { iface = 5 - bitz; jface = 2; }
  c.nxt = a.neighptr[6 * (size_t)cell + iface];
#pragma unroll
  for (int k = 0; k < 4; ++k) c.i[k] = g[c_face[iface][k]];
  const float *p1 = a.gridpos + 3 * c.i[0], *p2 = a.gridpos + 3 * c.i[1], *p3 = a.gridpos + 3 * c.i[2];
  if (jface == 0) {
    c.u = (ze - p1[2]) / (p3[2] - p1[2]);
    c.v = ipy ? 0.5f : (ye - p1[1]) / (p2[1] - p1[1]);
  } else if (jface == 1) {
    c.u = (ze - p1[2]) / (p3[2] - p1[2]);
    c.v = ipx ? 0.5f : (xe - p1[0]) / (p2[0] - p1[0]);
  } else {
    c.u = ipy ? 0.5f : (ye - p1[1]) / (p3[1] - p1[1]);
    c.v = ipx ? 0.5f : (xe - p1[0]) / (p2[0] - p1[0]);
  }
  if (c.nxt >= 0) {
    const float *q = a.gridpos + 3 * a.gridptr[8 * (size_t)c.nxt + b];
    if (jface == 0) xe = q[0]; else if (jface == 1) ye = q[1]; else ze = q[2];
  }
  return c;
}

__device__ __forceinline__ IrrRec trace_geom1(const SweepArgs &a, int b, int cls, int pt, int col) {
  IrrRec r;
  r.q = make_int4(pt, pt, pt, pt);
  r.g = make_float4(0.f, 0.f, 0.f, 0.f);
  const int n = a.npts;
  const int cell = a.start[(size_t)b * n + pt];
  if (a.is1d || cell < 0 || a.transmin < 1.f) return r;
  const float cx = a.col_cx[col], cy = a.col_cy[col], cz = a.col_cz[col];
  const float cxinv = cx != 0.f ? 1.f / cx : 1.0e6f, cyinv = cy != 0.f ? 1.f / cy : 1.0e6f, czinv = 1.f / cz;
  const int hb = (cz < 0.f) ? 2 : 1;
  const int *rk = a.rank + (size_t)b * n, *lv = a.level + ((size_t)b * 4 + cls) * n;
  const int rP = rk[pt], lP = lv[pt];
  float xe = a.gridpos[3 * pt], ye = a.gridpos[3 * pt + 1], ze = a.gridpos[3 * pt + 2];
  const CellExit c = cell_exit3d(a, b, cell, xe, ye, ze, cx, cy, cz, cxinv, cyinv, czinv);
  bool valid = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int q = c.i[k];
    valid = valid && ((a.bnd[q] & hb) || (rk[q] < rP && lv[q] < lP));
  }
  if (valid) {
    r.q = make_int4(c.i[0], c.i[1], c.i[2], c.i[3]);
    r.g = make_float4(c.so, c.u, c.v, 1.f);
  }
  return r;
}

// General trace (any point); with use_level the level of the ordinate's
// face class must also precede the point's (level-synchronous execution).
__device__ __forceinline__ Trace trace_general(const SweepArgs &a, int b, int cls, int pt, int col, bool use_level) {
  Trace t;
  t.radsrc = 0.f; t.tr = 1.f; t.status = ERR_SWEEP_STEPS; t.u = 0.f; t.v = 0.f;
  t.q[0] = t.q[1] = t.q[2] = t.q[3] = pt; t.f[0] = t.f[1] = t.f[2] = t.f[3] = 0.f;
  const int ldo = a.ldo, n = a.npts;
  const float cx = a.col_cx[col], cy = a.col_cy[col], cz = a.col_cz[col];
  const float cxinv = cx != 0.f ? 1.f / cx : 1.0e6f, cyinv = cy != 0.f ? 1.f / cy : 1.0e6f, czinv = 1.f / cz;
  const int bitz = cz < 0.f;
  const int hb = bitz ? 2 : 1;
  const int *rk = a.rank + (size_t)b * n, *lv = a.level + ((size_t)b * 4 + cls) * n;
  const int rP = rk[pt], lP = use_level ? lv[pt] : 0;
  int cell = a.start[(size_t)b * n + pt];
  float xe = a.gridpos[3 * pt], ye = a.gridpos[3 * pt + 1], ze = a.gridpos[3 * pt + 2];
  float ext1 = a.text[pt];
  float srcext1 = ext1 * a.srcdo[(size_t)pt * ldo + col];
  float rad = 0.f, tr = 1.f;
  const bool clamp = !a.stk || !a.stk[col];
  for (int guard = 0; guard < 65536; ++guard) {
    if (cell < 0) break;
    const int *g = a.gridptr + 8 * (size_t)cell;
    int i1, i2, i3, i4, nxt;
    float so, f1, f2, f3, f4, fu = 0.f, fv = 0.f;
    if (a.is1d) {
      int iopp = g[7 - b];
      so = (a.gridpos[3 * iopp + 2] - ze) * czinv;
      ze += so * cz;
      int iface = 5 - bitz;
      nxt = a.neighptr[6 * (size_t)cell + iface];
      i1 = i2 = i3 = i4 = g[iface == 4 ? 0 : 4];
      if (nxt >= 0) ze = a.gridpos[3 * a.gridptr[8 * (size_t)nxt + b] + 2];
      f1 = 1.f; f2 = f3 = f4 = 0.f;
    } else {
      const CellExit c = cell_exit3d(a, b, cell, xe, ye, ze, cx, cy, cz, cxinv, cyinv, czinv);
      i1 = c.i[0]; i2 = c.i[1]; i3 = c.i[2]; i4 = c.i[3]; nxt = c.nxt; so = c.so;
      const float u = c.u, v = c.v;
      fu = u; fv = v;
      f1 = (1.f - u) * (1.f - v); f2 = (1.f - u) * v; f3 = u * (1.f - v); f4 = u * v;
    }
    const float e1 = a.text[i1], e2 = a.text[i2], e3 = a.text[i3], e4 = a.text[i4];
    const float ext0 = f1 * e1 + f2 * e2 + f3 * e3 + f4 * e4;
    const float srcext0 = f1 * a.srcdo[(size_t)i1 * ldo + col] * e1 + f2 * a.srcdo[(size_t)i2 * ldo + col] * e2 +
                          f3 * a.srcdo[(size_t)i3 * ldo + col] * e3 + f4 * a.srcdo[(size_t)i4 * ldo + col] * e4;
    float radsrc, transcell;
    cell_source(ext0, srcext0, ext1, srcext1, so, radsrc, transcell, clamp);
    rad += tr * radsrc;
    tr *= transcell;
    auto ok = [&](int q) { return (a.bnd[q] & hb) || (rk[q] < rP && (!use_level || lv[q] < lP)); };
    const bool valid = ok(i1) && ok(i2) && ok(i3) && ok(i4);
    if (nxt < 0 || (tr <= a.transmin && valid)) {
      t.radsrc = rad; t.tr = tr;
      t.q[0] = i1; t.q[1] = i2; t.q[2] = i3; t.q[3] = i4;
      t.f[0] = f1; t.f[1] = f2; t.f[2] = f3; t.f[3] = f4;
      t.u = fu; t.v = fv;
      t.status = valid ? ERR_NONE : ERR_SWEEP_NOFACE;
      if (!valid) t.tr = 0.f;
      return t;
    }
    ext1 = ext0; srcext1 = srcext0; cell = nxt;
  }
  t.radsrc = 0.f; t.tr = 0.f;
  return t;
}

__device__ __forceinline__ Trace trace_point(const SweepArgs &a, int b, int pt, int col) {
  if (a.regular[(size_t)b * a.npts + pt]) return trace_regular(a, b, pt, col);
  return trace_general(a, b, 3, pt, col, false);
}

// Level-synchronous sweep of one hemisphere in three parts.
//
// Every trace gives rad(P) = radsrc + tr * sum_k f_k rad(q_k), and radsrc, tr
// depend on the source function only.
//  * Phase 1 (k_sweep_p1, one block per (octant, face class) group, on a
//    second stream): the general-trace points whose dependencies are all
//    preset or phase-1 points -- on open boundaries the edge-cell planes,
//    whose traces stay in the plane.  Levels are separated by block
//    barriers.
//  * Source pass (k_sweep_prep, point-major, concurrent with phase 1):
//    (radsrc, tr) of every phase-2 item into w[point][column].
//  * Phase 2 (k_sweep_levels, cooperative): the remaining levels; per item
//    one read of the point index, then (radsrc, tr) and the four upstream
//    radiances, then the combine.  Phase-1 values count as level 0 here.
// A level's items (task x column of a face class) are numbered
// consecutively (Seg::start); consecutive threads take consecutive columns
// of one point.
constexpr int MAXSEG = 32;

// Locates item j of a table of general-trace items: segs sorted by irr0,
// the segment with the largest irr0 <= j.
__device__ __forceinline__ int irr_seg_find(const Seg *__restrict__ segs, int nseg, int j) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].irr0 <= j) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Source pass, regular phase-2 items, one thread per (point, column).  A
// regular trace stays in the point's start cell; where no point of the
// cells around the point scatters (nbscat = 0) the source function is zero
// in every iteration, so radsrc = 0 and tr depends on the extinction only:
// once w holds those items (*ready != 0) they are skipped.
__global__ void __launch_bounds__(256) k_sweep_prep(SweepArgs a, const uint8_t *__restrict__ kind,
                                                    const int *__restrict__ col_oct, const int *__restrict__ col_cls,
                                                    int c0, int nc, float2 *__restrict__ w,
                                                    const uint8_t *__restrict__ nbscat, const int *__restrict__ ready) {
  const int total = a.npts * nc;
  const bool skip_static = *ready != 0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int pt = idx / nc, col = c0 + (idx - pt * nc);
    if (skip_static && !__ldg(nbscat + pt)) continue;
    if (__ldg(a.col_cz + col) == 0.f) continue;  // padding ordinate
    const int b = __ldg(col_oct + col) - 1, cls = __ldg(col_cls + col);
    if (__ldg(kind + ((size_t)b * 4 + cls) * a.npts + pt) != 1) continue;
    RegLoad x;
    reg_load(a, b, pt, col, x, false);
    const Trace t = reg_trace(x, b, pt);
    w[(size_t)pt * a.ldo + col] = make_float2(t.radsrc, t.tr);
  }
}

// Source pass, general phase-2 items (irr table entries [j0, j0 + n)); a
// trace that needs the cell walk also stores its final face.
__global__ void __launch_bounds__(256) k_sweep_prep_irr(SweepArgs a, const Seg *__restrict__ segs, int nseg, int j0,
                                                        int n, float2 *__restrict__ w, IrrRec *__restrict__ irr) {
  for (int jj = blockIdx.x * blockDim.x + threadIdx.x; jj < n; jj += gridDim.x * blockDim.x) {
    const int j = j0 + jj;
    const Seg g = segs[irr_seg_find(segs, nseg, j)];
    const int li = j - g.irr0, task = li / g.ncol, slot = li - task * g.ncol;
    const int pt = (int)__ldg(a.tasks + g.t0 + task), col = g.col0 + slot;
    const IrrRec rec = irr[j];
    float2 out;
    if (rec.g.w > 0.5f) {
      RegLoad x;
      rec_load(a, rec, pt, col, x, false);
      const Trace t = reg_trace(x, g.b, pt);
      out = make_float2(t.radsrc, t.tr);
    } else {
      const Trace t = trace_general(a, g.b, g.cls, pt, col, true);
      if (t.status != ERR_NONE) atomicCAS(a.err, ERR_NONE, t.status);
      out = make_float2(t.radsrc, t.tr);
      IrrRec r;
      r.q = make_int4(t.q[0], t.q[1], t.q[2], t.q[3]);
      r.g = make_float4(0.f, t.u, t.v, 0.f);
      irr[j] = r;
    }
    w[(size_t)pt * a.ldo + col] = out;
  }
}

// Stored first-face records of all general-trace items of a hemisphere.
__global__ void __launch_bounds__(256) k_irr_build(SweepArgs a, const Seg *__restrict__ segs, int nseg, int nirr,
                                                   IrrRec *__restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nirr; j += gridDim.x * blockDim.x) {
    const Seg g = segs[irr_seg_find(segs, nseg, j)];
    const int li = j - g.irr0, task = li / g.ncol, slot = li - task * g.ncol;
    const int pt = (int)a.tasks[g.t0 + task];
    out[j] = trace_geom1(a, g.b, g.cls, pt, g.col0 + slot);
  }
}

// Phase 1: the levels of each group with block barriers.  The ordinates
// of a group are independent of one another, so a group's columns are
// split into P1_SPLIT contiguous ranges, one block each (block b: group
// b / P1_SPLIT, range b % P1_SPLIT): shorter levels per block, more SMs.
// The levels are software-pipelined: a thread's first P1_STAGE items of the
// next level that have a stored face record get their record, point and
// the face corners' extinctions and ordinate sources loaded before the
// barrier; after it only the corners' radiances, which the level just
// finished may have written, are read.  Further items and traces that
// walk several cells are done in place.
constexpr int P1_THREADS = 512;
constexpr int P1_SPLIT = 4;
constexpr int P1_STAGE = 2;
constexpr int P1_SEGCAP = 512;  // level segments of a phase-1 group kept in shared memory
constexpr int P1S_THREADS = 512;  // threads of a block-local phase-1 block (256: 0.47 -> 0.50 ms per hemisphere)

__global__ void __launch_bounds__(P1_THREADS) k_sweep_p1(SweepArgs a, const Seg *__restrict__ p1segs,
                                                         const int *__restrict__ p1off) {
  const int grp = blockIdx.x / P1_SPLIT, sid = blockIdx.x % P1_SPLIT;
  const int s0 = p1off[grp], s1 = p1off[grp + 1];
  const int ldo = a.ldo;
  // staged items: the inputs of a single-face trace but the corner radiances
  RegLoad st[P1_STAGE];
  int sq[P1_STAGE][4];
  bool staged[P1_STAGE];
  auto items_of = [&](const Seg &g, int &cbeg, int &ncs) {
    const int cw = (g.ncol + P1_SPLIT - 1) / P1_SPLIT;
    cbeg = sid * cw; ncs = max(0, min(g.ncol, cbeg + cw) - cbeg);
    return g.ntask * ncs;
  };
  auto stage = [&](int si) {
#pragma unroll
    for (int k = 0; k < P1_STAGE; ++k) staged[k] = false;
    if (si >= s1) return;
    const Seg g = p1segs[si];
    int cbeg, ncs;
    const int items = items_of(g, cbeg, ncs);
#pragma unroll
    for (int k = 0; k < P1_STAGE; ++k) {
      const int ii = threadIdx.x + k * blockDim.x;
      if (ii >= items) break;
      const int task = ii / ncs, slot = cbeg + (ii - task * ncs);
      const IrrRec rec = a.irr[g.irr0 + task * g.ncol + slot];
      if (rec.g.w <= 0.5f) continue;  // a cell walk: done in place
      const int pt = (int)__ldg(a.tasks + g.t0 + task), col = g.col0 + slot;
      rec_load(a, rec, pt, col, st[k], false);
      sq[k][0] = rec.q.x; sq[k][1] = rec.q.y; sq[k][2] = rec.q.z; sq[k][3] = rec.q.w;
      staged[k] = true;
    }
  };
  stage(s0);
  for (int si = s0; si < s1; ++si) {
    const Seg g = p1segs[si];
    int cbeg, ncs;
    const int items = items_of(g, cbeg, ncs);
    auto coords = [&](int ii, int &task, int &i, int &col) {
      task = ii / ncs;
      const int slot = cbeg + (ii - task * ncs);
      i = task * g.ncol + slot;  // item of the segment
      col = g.col0 + slot;
    };
    auto item_staged = [&](int ii, RegLoad &x, const int (&q)[4]) {
      int task, i, col;
      coords(ii, task, i, col);
#pragma unroll
      for (int c = 0; c < 4; ++c) x.r[c] = a.raddo[(size_t)q[c] * ldo + col];
      const Trace t = reg_trace(x, g.b, x.pt);
      float rad = t.radsrc;
      if (t.tr != 0.f) rad += t.tr * (t.f[0] * x.r[0] + t.f[1] * x.r[1] + t.f[2] * x.r[2] + t.f[3] * x.r[3]);
      a.raddo[(size_t)x.pt * ldo + col] = rad;
    };
    auto item_plain = [&](int ii) {
      int task, i, col;
      coords(ii, task, i, col);
      const int pt = (int)__ldg(a.tasks + g.t0 + task);
      const IrrRec rec = a.irr[g.irr0 + i];
      float rad;
      if (rec.g.w > 0.5f) {
        RegLoad y;
        rec_load(a, rec, pt, col, y, true);
        const Trace t = reg_trace(y, g.b, pt);
        rad = t.radsrc;
        if (t.tr != 0.f) rad += t.tr * (t.f[0] * y.r[0] + t.f[1] * y.r[1] + t.f[2] * y.r[2] + t.f[3] * y.r[3]);
      } else {
        const Trace t = trace_general(a, g.b, g.cls, pt, col, true);
        if (t.status != ERR_NONE) atomicCAS(a.err, ERR_NONE, t.status);
        rad = t.radsrc;
        if (t.tr != 0.f)
          rad += t.tr * (t.f[0] * a.raddo[(size_t)t.q[0] * ldo + col] + t.f[1] * a.raddo[(size_t)t.q[1] * ldo + col] +
                         t.f[2] * a.raddo[(size_t)t.q[2] * ldo + col] + t.f[3] * a.raddo[(size_t)t.q[3] * ldo + col]);
      }
      a.raddo[(size_t)pt * ldo + col] = rad;
    };
    static_assert(P1_STAGE == 2, "the staged items are handled one by one below");
    if (threadIdx.x < items) {
      if (staged[0]) item_staged(threadIdx.x, st[0], sq[0]); else item_plain(threadIdx.x);
    }
    if (threadIdx.x + blockDim.x < items) {
      if (staged[1]) item_staged(threadIdx.x + blockDim.x, st[1], sq[1]); else item_plain(threadIdx.x + blockDim.x);
    }
    for (int ii = threadIdx.x + P1_STAGE * blockDim.x; ii < items; ii += blockDim.x) item_plain(ii);
    stage(si + 1);  // the next level's inputs that do not depend on this level
    __syncthreads();
  }
}

// Phase 2, one item: point, (radsrc, tr), face corners and weights, then the
// four upstream radiances.
// Phase 1 ahead of the plane march: every phase-1 item's trace (its
// stored first face, or the cell walk) in one parallel pass, as records
// indexed like the general-trace table (irr entries [0, n)); traces depend
// on the source function only.
__global__ void __launch_bounds__(256) k_p1_prep(SweepArgs a, const Seg *__restrict__ segs, int nseg, int n,
                                                 TraceRec *__restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const Seg g = segs[irr_seg_find(segs, nseg, j)];
    const int li = j - g.irr0, task = li / g.ncol, slot = li - task * g.ncol;
    const int pt = (int)__ldg(a.tasks + g.t0 + task), col = g.col0 + slot;
    const IrrRec rec = a.irr[j];
    Trace t;
    if (rec.g.w > 0.5f) {
      RegLoad x;
      rec_load(a, rec, pt, col, x, false);
      t = reg_trace(x, g.b, pt);
      t.q[0] = rec.q.x; t.q[1] = rec.q.y; t.q[2] = rec.q.z; t.q[3] = rec.q.w;
    } else {
      t = trace_general(a, g.b, g.cls, pt, col, true);
      if (t.status != ERR_NONE) atomicCAS(a.err, ERR_NONE, t.status);
    }
    TraceRec r;
    r.radsrc = t.radsrc; r.tr = t.tr; r.u = t.u; r.v = t.v;
    r.q = make_int4(t.q[0], t.q[1], t.q[2], t.q[3]);
    out[j] = r;
  }
}

// Phase 1 from the records of k_p1_prep: per level and item, the four
// corner radiances (written by earlier levels) and the combination.  Block
// layout as k_sweep_p1; a thread's first P1_STAGE items of the next level
// have their record and point loaded before the barrier.
__global__ void __launch_bounds__(P1_THREADS) k_sweep_p1r(SweepArgs a, const Seg *__restrict__ p1segs,
                                                          const int *__restrict__ p1off,
                                                          const TraceRec *__restrict__ recs) {
  const int grp = blockIdx.x / P1_SPLIT, sid = blockIdx.x % P1_SPLIT;
  const int s0 = p1off[grp], s1 = p1off[grp + 1];
  const int ldo = a.ldo;
  // the group's level segments, in shared memory when they fit
  __shared__ Seg ssg[P1_SEGCAP];
  const bool local = s1 - s0 <= P1_SEGCAP;
  if (local)
    for (int t = threadIdx.x; t < s1 - s0; t += blockDim.x) ssg[t] = p1segs[s0 + t];
  __syncthreads();
  auto seg = [&](int si) { return local ? ssg[si - s0] : p1segs[si]; };
  TraceRec sr[P1_STAGE];
  int spt[P1_STAGE], scol[P1_STAGE];
  auto items_of = [&](const Seg &g, int &cbeg, int &ncs) {
    const int cw = (g.ncol + P1_SPLIT - 1) / P1_SPLIT;
    cbeg = sid * cw; ncs = max(0, min(g.ncol, cbeg + cw) - cbeg);
    return g.ntask * ncs;
  };
  auto locate = [&](const Seg &g, int cbeg, int ncs, int ii, int &pt, int &col, int &j) {
    const int task = ii / ncs, slot = cbeg + (ii - task * ncs);
    pt = (int)__ldg(a.tasks + g.t0 + task);
    col = g.col0 + slot;
    j = g.irr0 + task * g.ncol + slot;
  };
  auto combine = [&](const TraceRec &R, int pt, int col) {
    float rad = R.radsrc;
    if (R.tr != 0.f) {
      const float r0 = a.raddo[(size_t)R.q.x * ldo + col], r1 = a.raddo[(size_t)R.q.y * ldo + col];
      const float r2 = a.raddo[(size_t)R.q.z * ldo + col], r3 = a.raddo[(size_t)R.q.w * ldo + col];
      const float u = R.u, v = R.v;
      rad += R.tr * ((1.f - u) * (1.f - v) * r0 + (1.f - u) * v * r1 + u * (1.f - v) * r2 + u * v * r3);
    }
    a.raddo[(size_t)pt * ldo + col] = rad;
  };
  auto stage = [&](int si) {
    if (si >= s1) return;
    const Seg g = seg(si);
    int cbeg, ncs;
    const int items = items_of(g, cbeg, ncs);
#pragma unroll
    for (int k = 0; k < P1_STAGE; ++k) {
      const int ii = threadIdx.x + k * blockDim.x;
      if (ii < items) {
        int j;
        locate(g, cbeg, ncs, ii, spt[k], scol[k], j);
        sr[k] = recs[j];
      }
    }
  };
  stage(s0);
  for (int si = s0; si < s1; ++si) {
    const Seg g = seg(si);
    int cbeg, ncs;
    const int items = items_of(g, cbeg, ncs);
#pragma unroll
    for (int k = 0; k < P1_STAGE; ++k)
      if (threadIdx.x + k * blockDim.x < items) combine(sr[k], spt[k], scol[k]);
    for (int ii = threadIdx.x + P1_STAGE * blockDim.x; ii < items; ii += blockDim.x) {
      int pt, col, j;
      locate(g, cbeg, ncs, ii, pt, col, j);
      combine(recs[j], pt, col);
    }
    stage(si + 1);  // the next level's records, which do not depend on this level
    __syncthreads();
  }
}

// Phase 1 with block-local radiances.  A phase-1 point's corners are
// preset boundary points (final before phase 1) or phase-1 points of the
// same ordinates, i.e. of the same (octant, class) group.  Each group's
// phase-1 points are numbered in level order (slots); a block owns a slice
// of the group's columns and keeps the slice's radiances of all the
// group's phase-1 points in shared memory, so a level reads its corners
// from there.  k_p1_prep_s folds the boundary corners into radsrc and
// turns the other corners into slots (q[k] = slot, or -1).
struct P1Blk {
  int grp, cbeg, ncs, nslots;  // group, its column slice [cbeg, cbeg + ncs), the group's phase-1 points
};

__global__ void __launch_bounds__(256) k_p1_prep_s(SweepArgs a, const Seg *__restrict__ segs, int nseg, int n,
                                                   const int *__restrict__ seggrp, const int *__restrict__ p1slot,
                                                   TraceRec *__restrict__ out) {
  const int ldo = a.ldo;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int si = irr_seg_find(segs, nseg, j);
    const Seg g = segs[si];
    const int li = j - g.irr0, task = li / g.ncol, slot = li - task * g.ncol;
    const int pt = (int)__ldg(a.tasks + g.t0 + task), col = g.col0 + slot;
    const IrrRec rec = a.irr[j];
    Trace t;
    if (rec.g.w > 0.5f) {
      RegLoad x;
      rec_load(a, rec, pt, col, x, false);
      t = reg_trace(x, g.b, pt);
      t.q[0] = rec.q.x; t.q[1] = rec.q.y; t.q[2] = rec.q.z; t.q[3] = rec.q.w;
    } else {
      t = trace_general(a, g.b, g.cls, pt, col, true);
      if (t.status != ERR_NONE) atomicCAS(a.err, ERR_NONE, t.status);
    }
    const int hb = (g.b & 4) ? 2 : 1;
    const int *slots = p1slot + (size_t)seggrp[si] * a.npts;
    const float f[4] = {(1.f - t.u) * (1.f - t.v), (1.f - t.u) * t.v, t.u * (1.f - t.v), t.u * t.v};
    TraceRec r;
    r.radsrc = t.radsrc; r.tr = t.tr; r.u = t.u; r.v = t.v;
    int sl[4] = {-1, -1, -1, -1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float w = t.tr * f[k];
      if (w == 0.f) continue;
      if (a.bnd[t.q[k]] & hb) {
        r.radsrc += w * a.raddo[(size_t)t.q[k] * ldo + col];  // preset: final
      } else {
        sl[k] = slots[t.q[k]];
        if (sl[k] < 0) atomicCAS(a.err, ERR_NONE, ERR_SWEEP_NOFACE);  // not a phase-1 point of the group
      }
    }
    r.q = make_int4(sl[0], sl[1], sl[2], sl[3]);
    out[j] = r;
  }
}

__global__ void __launch_bounds__(P1S_THREADS) k_sweep_p1s(SweepArgs a, const Seg *__restrict__ p1segs,
                                                          const int *__restrict__ p1off, const P1Blk *__restrict__ blks,
                                                          const int *__restrict__ segbase,
                                                          const TraceRec *__restrict__ recs) {
  extern __shared__ float sv[];  // [slot][column of the slice]
  __shared__ Seg ssg[P1_SEGCAP];
  __shared__ int sbase[P1_SEGCAP];
  const P1Blk B = blks[blockIdx.x];
  const int s0 = p1off[B.grp], s1 = p1off[B.grp + 1], ncs = B.ncs;
  const int ldo = a.ldo;
  for (int t = threadIdx.x; t < s1 - s0; t += blockDim.x) { ssg[t] = p1segs[s0 + t]; sbase[t] = segbase[s0 + t]; }
  __syncthreads();
  TraceRec sr[P1_STAGE];
  int spt[P1_STAGE];
  auto rec_of = [&](const Seg &g, int ii, int &pt, int &col, int &slot, int &c) {
    const int task = ii / ncs;
    c = ii - task * ncs;
    pt = (int)__ldg(a.tasks + g.t0 + task);
    col = g.col0 + B.cbeg + c;
    slot = task;
    return g.irr0 + task * g.ncol + B.cbeg + c;
  };
  auto combine = [&](const TraceRec &R, int pt, int col, int slot, int c) {
    float rad = R.radsrc;
    if (R.tr != 0.f) {
      const float u = R.u, v = R.v;
      const float f0 = (1.f - u) * (1.f - v), f1 = (1.f - u) * v, f2 = u * (1.f - v), f3 = u * v;
      float acc = 0.f;
      if (R.q.x >= 0) acc += f0 * sv[R.q.x * ncs + c];
      if (R.q.y >= 0) acc += f1 * sv[R.q.y * ncs + c];
      if (R.q.z >= 0) acc += f2 * sv[R.q.z * ncs + c];
      if (R.q.w >= 0) acc += f3 * sv[R.q.w * ncs + c];
      rad += R.tr * acc;
    }
    sv[slot * ncs + c] = rad;
    a.raddo[(size_t)pt * ldo + col] = rad;
  };
  auto stage = [&](int si) {
    if (si >= s1) return;
    const Seg &g = ssg[si - s0];
    const int items = g.ntask * ncs;
#pragma unroll
    for (int k = 0; k < P1_STAGE; ++k) {
      const int ii = threadIdx.x + k * blockDim.x;
      if (ii < items) {
        int col, slot, c;
        sr[k] = recs[rec_of(g, ii, spt[k], col, slot, c)];
      }
    }
  };
  stage(s0);
  for (int si = s0; si < s1; ++si) {
    const Seg &g = ssg[si - s0];
    const int items = g.ntask * ncs, base = sbase[si - s0];
#pragma unroll
    for (int k = 0; k < P1_STAGE; ++k) {
      const int ii = threadIdx.x + k * blockDim.x;
      if (ii < items) {
        const int task = ii / ncs, c = ii - task * ncs;
        combine(sr[k], spt[k], g.col0 + B.cbeg + c, base + task, c);
      }
    }
    for (int ii = threadIdx.x + P1_STAGE * blockDim.x; ii < items; ii += blockDim.x) {
      int pt, col, slot, c;
      const int j = rec_of(g, ii, pt, col, slot, c);
      combine(recs[j], pt, col, base + slot, c);
    }
    stage(si + 1);  // the next level's records, which do not depend on this level
    __syncthreads();
  }
}

struct LevelItem {
  float2 w;
  float u, v;
  int pt, col, q[4];
};

__device__ __forceinline__ void level_load(const SweepArgs &a, const Seg &g, int li, const float2 *__restrict__ w,
                                           LevelItem &x, float r[4]) {
  const int task = li / g.ncol, slot = li - task * g.ncol;
  x.col = g.col0 + slot;
  x.pt = (int)__ldg(a.tasks + g.t0 + task);
  x.w = w[(size_t)x.pt * a.ldo + x.col];
  if (g.regular) {
    const int b = g.b, iz = x.pt % a.nz, layer = (b & 4) ? iz - 1 : iz;
    const float4 geo = __ldg(reinterpret_cast<const float4 *>(a.geo) + (size_t)layer * a.nang + x.col);
    x.u = geo.y; x.v = geo.z;
    const int iface = (g.cls < 3) ? 2 * g.cls + 1 - ((b >> g.cls) & 1) : (int)geo.w;
    const int ox = (b & 1) ? -a.nz * a.ny1 : a.nz * a.ny1, oy = (b & 2) ? -a.nz : a.nz, oz = (b & 4) ? -1 : 1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int d = c_face[iface][k] ^ b;
      x.q[k] = x.pt + ((d & 1) ? ox : 0) + ((d & 2) ? oy : 0) + ((d & 4) ? oz : 0);
    }
  } else {
    const IrrRec rec = a.irr[g.irr0 + li];
    x.q[0] = rec.q.x; x.q[1] = rec.q.y; x.q[2] = rec.q.z; x.q[3] = rec.q.w;
    x.u = rec.g.y; x.v = rec.g.z;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) r[k] = a.raddo[(size_t)x.q[k] * a.ldo + x.col];
}

__device__ __forceinline__ void level_finish(const SweepArgs &a, const LevelItem &x, const float r[4]) {
  const float u = x.u, v = x.v;
  const float f0 = (1.f - u) * (1.f - v), f1 = (1.f - u) * v, f2 = u * (1.f - v), f3 = u * v;
  float rad = x.w.x;
  if (x.w.y != 0.f) rad += x.w.y * (f0 * r[0] + f1 * r[1] + f2 * r[2] + f3 * r[3]);
  a.raddo[(size_t)x.pt * a.ldo + x.col] = rad;
}

__device__ __forceinline__ int seg_find(const Seg *sg, int nseg, int i, int si) {
  while (si + 1 < nseg && i >= sg[si + 1].start) ++si;
  return si;
}

__device__ __forceinline__ void sweep_level(const SweepArgs &a, const Seg *sg, int nseg, int items,
                                            const float2 *__restrict__ w, int gtid, int gstride) {
  int si = 0;
  for (int i = gtid; i < items; i += 2 * gstride) {
    const int i2 = i + gstride;
    si = seg_find(sg, nseg, i, si);
    const int sj = i2 < items ? seg_find(sg, nseg, i2, si) : si;
    LevelItem x1, x2;
    float r1[4], r2[4];
    level_load(a, sg[si], i - sg[si].start, w, x1, r1);
    if (i2 < items) level_load(a, sg[sj], i2 - sg[sj].start, w, x2, r2);
    level_finish(a, x1, r1);
    if (i2 < items) level_finish(a, x2, r2);
    si = sj;
  }
}

// One launch per phase-2 level (used when a cooperative launch is not available).
__global__ void __launch_bounds__(256) k_sweep(SweepArgs a, const Seg *__restrict__ segs, int nseg, int items,
                                               const float2 *__restrict__ w) {
  __shared__ Seg sg[MAXSEG];
  for (int t = threadIdx.x; t < nseg; t += blockDim.x) sg[t] = segs[t];
  __syncthreads();
  sweep_level(a, sg, nseg, items, w, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// All phase-2 levels of one hemisphere in one cooperative launch: the blocks
// share out the items of a level, then meet at a grid barrier.
__global__ void __launch_bounds__(256) k_sweep_levels(SweepArgs a, const Seg *__restrict__ segs,
                                                      const int *__restrict__ seg_off,
                                                      const int *__restrict__ level_items,
                                                      const float2 *__restrict__ w, int nlev) {
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  __shared__ Seg sg[MAXSEG];
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
  for (int l = 0; l < nlev; ++l) {
    const int s0 = seg_off[l], ns = seg_off[l + 1] - s0;
    for (int t = threadIdx.x; t < ns; t += blockDim.x) sg[t] = segs[s0 + t];
    __syncthreads();
    sweep_level(a, sg, ns, level_items[l], w, gtid, gstride);
    grid.sync();
  }
}

// ------------------------------------------------------------ plane march
// Phase 2 of a hemisphere whose (octant, face class) groups all march
// (MarchGrp, planned on the host): each phase-2 point's regular trace stops
// on a face in the previous plane along the group's class axis, so the
// group's columns are swept plane by plane, every point of a plane
// independent of the others.  One thread-block cluster per (group, column
// slice): the cluster's CTAs split each plane into strips of rows along U.
// A CTA keeps, for the previous and the current plane (two buffers swapped
// every plane), its strip's radiances, ordinate sources times extinction
// and extinctions in shared memory, plus one halo row on the upwind side
// that the upwind CTA stores into it (distributed shared memory) when it
// computes that row; the cluster meets at one cluster barrier per plane.
// The source pass is fused: (radsrc, tr) of BACK_INT_GRID3D's cell
// integral come from the ordinate source and extinction of the point
// (loaded from global memory one plane ahead) and of the face corners (the
// previous plane, in shared memory), with the arithmetic of reg_trace.
// DRAM sees one read of the point's ordinate source and one write of its
// radiance per item.
struct MarchUnit {
  int grp, c0, nc, tw;  // group, absolute columns [c0, c0+nc), rows per CTA
};
constexpr int MT = 256;  // threads per CTA
constexpr int MK = 16;   // (row, v) pairs per thread at most

// Shared memory of one CTA: the face geometry of the strip's columns
// [nv][nc] (float4), then two plane buffers, each rad[tw+2][nv][nc],
// se[tw+2][nv][nc] and ext[tw+2][nv] (rows -1 and tw are halo rows).
__host__ __device__ inline size_t march_buf_floats(int tw, int nv, int nc) {
  return (size_t)(tw + 2) * nv * (2 * nc + 1);
}
__host__ __device__ inline size_t march_smem_bytes(int tw, int nv, int nc) {
  return sizeof(float) * (4 * (size_t)nv * nc + 2 * march_buf_floats(tw, nv, nc));
}

__global__ void __launch_bounds__(MT, 2) k_sweep_march(SweepArgs a, const MarchGrp *__restrict__ grps,
                                                       const MarchUnit *__restrict__ units) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int cs = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const MarchUnit U = units[blockIdx.x / cs];
  const MarchGrp G = grps[U.grp];
  const int nc = U.nc, nV = G.nV, tw = U.tw, ldo = a.ldo;
  const int u0 = rank * tw, nrow = max(0, min(tw, G.nU - u0));
  extern __shared__ float4 msm4[];
  float4 *sgeo = msm4;                                   // [nV][nc]
  float *buf0 = reinterpret_cast<float *>(msm4 + (size_t)nV * nc);
  const int bsz = (int)march_buf_floats(tw, nV, nc);
  const int rsz = (tw + 2) * nV * nc;                    // one rad (or se) array
  // this CTA's row that the downwind CTA (rank - upu) reads as its halo row,
  // and the halo row's index in that CTA's buffers
  const int cons = rank - G.upu;
  const bool push = nrow > 0 && cons >= 0 && cons < cs && cons * tw < G.nU;
  const int push_row = G.upu > 0 ? 0 : tw - 1;
  const int halo_lr = G.upu > 0 ? tw : -1;
  float *cons_buf0 = push ? cl.map_shared_rank(buf0, cons) : nullptr;
  // thread -> column c and the strip's (row, v) pairs k0, k0 + tpc, ... (at most MK)
  const int tpc = MT / nc, c = threadIdx.x % nc, k0 = threadIdx.x / nc;
  const int col = U.c0 + c;
  const bool clamp = !a.stk || !a.stk[col];
  const bool pad = __ldg(a.col_cz + col) == 0.f;
  const int kn = k0 < tpc ? max(0, (nrow * nV - k0 + tpc - 1) / tpc) : 0;
  const int r0 = k0 / nV, v0 = k0 - r0 * nV;
  const int ndn = G.cls == 0 ? a.nx1 : (G.cls == 1 ? a.ny1 : a.nz);  // extent of the class axis
  auto plane_fixed = [&](int A) {
    return pad || (G.cls == 2 && A == G.zfix) || (G.cls == 0 && G.xedge && (A == 0 || A == ndn - 1)) ||
           (G.cls == 1 && G.yedge && (A == 0 || A == ndn - 1));
  };
  // per pair: fixed in every plane (from u, v alone), and whether the face
  // corners lie inside the grid
  unsigned uvfix = 0, valid = 0;
  {
    int r = r0, v = v0;
#pragma unroll 1
    for (int j = 0; j < kn; ++j) {
      const int u = u0 + r;
      const bool f = (G.cls != 2 && v == G.zfix) || (G.xedge && G.cls != 0 && (u == 0 || u == a.nx1 - 1)) ||
                     (G.yedge && ((G.cls == 0 && (u == 0 || u == a.ny1 - 1)) ||
                                  (G.cls == 2 && (v == 0 || v == a.ny1 - 1))));
      bool ok = true;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int uu = u + G.du[k], vv = v + G.dv[k];
        ok = ok && uu >= 0 && uu < G.nU && vv >= 0 && vv < nV;
      }
      uvfix |= (unsigned)f << j;
      valid |= (unsigned)ok << j;
      v += tpc;
      while (v >= nV) { v -= nV; ++r; }
    }
  }
  // face geometry of the x and y classes: one entry per (v, column)
  if (G.cls != 2) {
    for (int i = threadIdx.x; i < nV * nc; i += MT) {
      const int v = i / nc, cc = i - v * nc;
      const int layer = (G.b & 4) ? v - 1 : v;
      sgeo[i] = (layer >= 0 && layer < a.nz - 1)
                    ? __ldg(reinterpret_cast<const float4 *>(a.geo) + (size_t)layer * a.nang + U.c0 + cc)
                    : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  // plane 0 (the upwind boundary plane) is fixed: radiance, source x extinction
  // and extinction into buffer 0 (and its halo row into the downwind CTA's)
  {
    int r = r0, v = v0;
#pragma unroll 1
    for (int j = 0; j < kn; ++j) {
      const int p = G.a0 * G.sa + (u0 + r) * G.su + v * G.sv;
      const float rad = __ldg(a.raddo + (size_t)p * ldo + col), s = __ldg(a.srcdo + (size_t)p * ldo + col),
                  e = __ldg(a.text + p);
      const int sp = (r + 1) * nV + v, si = sp * nc + c;
      buf0[si] = rad; buf0[rsz + si] = s * e; buf0[2 * rsz + sp] = e;
      if (push && r == push_row) {
        const int hp = (halo_lr + 1) * nV + v, hi = hp * nc + c;
        cons_buf0[hi] = rad; cons_buf0[rsz + hi] = s * e; cons_buf0[2 * rsz + hp] = e;
      }
      v += tpc;
      while (v >= nV) { v -= nV; ++r; }
    }
  }
  // the point's own ordinate source and extinction (and, at fixed points,
  // its final radiance), loaded one plane ahead
  float ps[MK], pe[MK], pr[MK];
  {
    const int A = G.a0 + G.da;
    const bool pf = G.nA > 1 && plane_fixed(A);
    int r = r0, v = v0;
#pragma unroll
    for (int j = 0; j < MK; ++j) {
      ps[j] = 0.f; pe[j] = 0.f; pr[j] = 0.f;
      if (j < kn && G.nA > 1) {
        const int p = A * G.sa + (u0 + r) * G.su + v * G.sv;
        ps[j] = __ldg(a.srcdo + (size_t)p * ldo + col);
        pe[j] = __ldg(a.text + p);
        if (pf || ((uvfix >> j) & 1)) pr[j] = __ldg(a.raddo + (size_t)p * ldo + col);
      }
      v += tpc;
      while (v >= nV) { v -= nV; ++r; }
    }
  }
  float4 gz = make_float4(0.f, 0.f, 0.f, 0.f);
  auto load_gz = [&](int A) {
    const int layer = (G.b & 4) ? A - 1 : A;
    return (G.cls == 2 && kn > 0 && layer >= 0 && layer < a.nz - 1)
               ? __ldg(reinterpret_cast<const float4 *>(a.geo) + (size_t)layer * a.nang + col)
               : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  if (G.nA > 1) gz = load_gz(G.a0 + G.da);
  // corner offsets relative to the point itself, in the previous plane's buffers
  int qs[4], qe[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) { qe[k] = G.du[k] * nV + G.dv[k]; qs[k] = qe[k] * nc; }
  // pair j sits at strip point k0 + j tpc: buffer point sp0 + j tpc, item si0 + j tpc nc
  const int sp0 = k0 + nV, si0 = sp0 * nc + c, sstep = tpc * nc;
  const int pb0 = (u0 + r0) * G.su + v0 * G.sv;  // pair 0's point index less the plane's
  cl.sync();
  for (int t = 1; t < G.nA; ++t) {
    const int A = G.a0 + t * G.da, An = A + G.da;
    const bool more = t + 1 < G.nA;
    const bool pf = plane_fixed(A), pfn = more && plane_fixed(An);
    const float *prev = buf0 + ((t - 1) & 1) * bsz;
    float *cur = buf0 + (t & 1) * bsz;
    float *ccur = push ? cons_buf0 + (t & 1) * bsz : nullptr;
    const float4 g2 = gz;
    if (more) gz = load_gz(An);
    // the plane's radiances from the previous plane, into shared memory,
    // and each pair's inputs in the next plane into registers
    const int Aoff = A * G.sa, step_n = G.da * G.sa;
    {
      int r = r0, v = v0, pb = pb0;
#pragma unroll
      for (int j = 0; j < MK; ++j) {
        if (j < kn) {
          const int sp = sp0 + j * tpc, si = si0 + j * sstep;
          const float s1 = ps[j], e1 = pe[j];
          float rad;
          if (pf || ((uvfix >> j) & 1)) {
            rad = pr[j];
          } else if (!((valid >> j) & 1)) {
            atomicCAS(a.err, ERR_NONE, ERR_SWEEP_NOFACE);
            rad = 0.f;
          } else {
            const float4 g = G.cls == 2 ? g2 : sgeo[v * nc + c];
            const float fu = g.y, fv = g.z;
            const float f0 = (1.f - fu) * (1.f - fv), f1 = (1.f - fu) * fv, f2 = fu * (1.f - fv), f3 = fu * fv;
            const float *pe_ = prev + 2 * rsz + sp, *ps_ = prev + rsz + si, *pr_ = prev + si;
            const float ext0 = f0 * pe_[qe[0]] + f1 * pe_[qe[1]] + f2 * pe_[qe[2]] + f3 * pe_[qe[3]];
            const float srcext0 = f0 * ps_[qs[0]] + f1 * ps_[qs[1]] + f2 * ps_[qs[2]] + f3 * ps_[qs[3]];
            float radsrc, tr;
            cell_source(ext0, srcext0, e1, e1 * s1, g.x, radsrc, tr, clamp);
            rad = radsrc;
            if (tr != 0.f) rad += tr * (f0 * pr_[qs[0]] + f1 * pr_[qs[1]] + f2 * pr_[qs[2]] + f3 * pr_[qs[3]]);
          }
          if (!(pf || ((uvfix >> j) & 1))) a.raddo[(size_t)(Aoff + pb) * ldo + col] = rad;
          cur[si] = rad; cur[rsz + si] = s1 * e1; cur[2 * rsz + sp] = e1;
          if (push && r == push_row) {
            const int hp = (halo_lr + 1) * nV + v, hi = hp * nc + c;
            ccur[hi] = rad; ccur[rsz + hi] = s1 * e1; ccur[2 * rsz + hp] = e1;
          }
          if (more) {
            const int pn = Aoff + pb + step_n;
            ps[j] = __ldg(a.srcdo + (size_t)pn * ldo + col);
            pe[j] = __ldg(a.text + pn);
            if (pfn || ((uvfix >> j) & 1)) pr[j] = __ldg(a.raddo + (size_t)pn * ldo + col);
          }
        }
        v += tpc; pb += tpc * G.sv;
        while (v >= nV) { v -= nV; ++r; pb += G.su - nV * G.sv; }
      }
    }
    cl.sync();  // plane t is in every strip's current buffer and halo row; the previous buffers are free
  }
}

// Sequential-order sweep for grids whose wavefront is too deep (periodic
// wrap-around long characteristics chain points of one ordinate through the
// whole grid), in two kernels.
//  * k_seq_prep: every (ordinate, point) trace of the hemisphere at once,
//    since a trace depends on the source function only: its (radsrc, tr),
//    the four corners of the face it stops on and the face coordinates, as
//    a 32-byte record in [ordinate][rank] order.  The long characteristics
//    (a row's first point crossing the wrap-around to the previous row, a
//    chain of cells) run here in parallel instead of inside the walk.
//  * k_sweep_seq: one block per ordinate walks the reference sweep order in
//    windows of SEQN ranks.  One thread runs a window's chain in rank
//    order, the item just before in a register (the usual dependency: the
//    neighbour along the row) and the others in shared memory; a chain
//    step is a few dependent instructions instead of a round of warp
//    votes.  Meanwhile the other seven warps prepare the next window (read
//    its records, coalesced; add its final dependencies; list the others
//    with their weights) and write the window before back to the field.
constexpr int SEQW = 256;  // threads of a walking block
constexpr int SEQN = 512;  // ranks of a window

__device__ __forceinline__ int col_octant(const SweepArgs &a, int col) {
  int b = 0;
  for (int k = 0; k < 8; ++k)
    if (a.oct_ncol[k] > 0 && col >= a.oct_col0[k] && col < a.oct_col0[k] + a.oct_ncol[k]) b = k;
  return b;
}

__global__ void __launch_bounds__(256) k_seq_prep(SweepArgs a, const int *__restrict__ order, int col_begin, int nc,
                                                   TraceRec *__restrict__ rec) {
  const int n = a.npts;
  const long long total = (long long)nc * n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int cl = (int)(i / n), r = (int)(i - (long long)cl * n);
    const int col = col_begin + cl;
    if (a.col_cz[col] == 0.f) continue;  // padding ordinate
    const int b = col_octant(a, col);
    const int hb = (b & 4) ? 2 : 1;
    const int pt = order[(size_t)b * n + r];
    if (a.bnd[pt] & hb) continue;  // preset boundary point
    const Trace t = trace_point(a, b, pt, col);
    if (t.status != ERR_NONE) atomicCAS(a.err, ERR_NONE, t.status);
    TraceRec x;
    x.radsrc = t.radsrc; x.tr = t.tr; x.u = t.u; x.v = t.v;
    x.q = make_int4(t.q[0], t.q[1], t.q[2], t.q[3]);
    rec[i] = x;
  }
}

__global__ void __launch_bounds__(SEQW) k_sweep_seq(SweepArgs a, const int *order, int col_begin,
                                                    const TraceRec *__restrict__ rec) {
  // sval: the values of the last two windows walked, by window parity (a
  // ring of 2 SEQN).  Per item of a window being walked or prepared (by
  // parity): the part from final dependencies, the weight of the item just
  // before it, and up to four other dependencies (ring indices, weight 0 for
  // none).  spt: the items' points, kept three windows for the write-back.
  __shared__ float sval[2 * SEQN];
  __shared__ float swv[2][SEQN], scp[2][SEQN];
  __shared__ float4 sc[2][SEQN];
  __shared__ short4 sd[2][SEQN];
  __shared__ int spt[3][SEQN];
  const int col = col_begin + blockIdx.x, ldo = a.ldo, n = a.npts;
  if (a.col_cz[col] == 0.f) return;  // padding ordinate
  const int b = col_octant(a, col);
  const int hb = (b & 4) ? 2 : 1;
  const int *ord = order + (size_t)b * n, *rk = a.rank + (size_t)b * n;
  const TraceRec *crec = rec + (size_t)blockIdx.x * n;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nwin = (n + SEQN - 1) / SEQN;
  for (int j = tid; j < 2 * SEQN; j += SEQW) sval[j] = 0.f;

  // window w's item list, by threads [t0, t0 + nt).  Dependencies: on a
  // preset point or a window before w - 2, final in the field; on window
  // w - 2, final in the ring; on window w - 1 or w, ring indices for the
  // walk (window w - 1 may still be walking while w is prepared).
  auto prep = [&](int w, int t0, int nt) {
    const int r0 = w * SEQN, m = min(SEQN, n - r0), pw = w & 1;
    for (int j = tid - t0; j < SEQN; j += nt) {
      const int r = r0 + j;
      float wv = 0.f, cp = 0.f;
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      short d[4] = {0, 0, 0, 0};
      int pt = -1;
      if (j < m) {
        const int p = ord[r];
        if (!(a.bnd[p] & hb)) {
          pt = p;
          const TraceRec R = crec[r];
          const int q[4] = {R.q.x, R.q.y, R.q.z, R.q.w};
          const float f[4] = {(1.f - R.u) * (1.f - R.v), (1.f - R.u) * R.v, R.u * (1.f - R.v), R.u * R.v};
          wv = R.radsrc;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float wt = R.tr * f[k];
            if (wt == 0.f) continue;
            if (a.bnd[q[k]] & hb) {  // a preset boundary point: final
              wv += wt * a.raddo[(size_t)q[k] * ldo + col];
              continue;
            }
            const int rq = rk[q[k]];
            if (rq >= r0) {  // this window
              const int off = rq - r0;
              if (off >= j) { atomicCAS(a.err, ERR_NONE, ERR_SWEEP_NOFACE); continue; }  // not rank-earlier
              if (off == j - 1) cp += wt;
              else { d[k] = (short)(pw * SEQN + off); c[k] = wt; }
            } else if (rq >= r0 - SEQN) {  // window w - 1: walked just before this one
              d[k] = (short)((pw ^ 1) * SEQN + (rq - (r0 - SEQN))); c[k] = wt;
            } else if (rq >= r0 - 2 * SEQN) {  // window w - 2: final, in the ring
              wv += wt * sval[pw * SEQN + (rq - (r0 - 2 * SEQN))];
            } else {
              wv += wt * a.raddo[(size_t)q[k] * ldo + col];
            }
          }
        }
      }
      spt[w % 3][j] = pt;
      swv[pw][j] = wv; scp[pw][j] = cp;
      sc[pw][j] = make_float4(c[0], c[1], c[2], c[3]);
      sd[pw][j] = make_short4(d[0], d[1], d[2], d[3]);
    }
  };
  // window w's radiances to the field, by threads [t0, t0 + nt)
  auto writeback = [&](int w, int t0, int nt) {
    const int pw = w & 1;
    for (int j = tid - t0; j < SEQN; j += nt) {
      const int pt = spt[w % 3][j];
      if (pt >= 0) a.raddo[(size_t)pt * ldo + col] = sval[pw * SEQN + j];
    }
  };
  if (nwin > 0) prep(0, 0, SEQW);
  __syncthreads();
  for (int w = 0; w < nwin; ++w) {
    if (warp == 0) {
      if (tid == 0) {  // the chain of window w in rank order, the item just before in a register
        const int pw = w & 1, m = min(SEQN, n - w * SEQN);
        float *out = sval + pw * SEQN;
        float prev = 0.f;
#pragma unroll 4
        for (int i = 0; i < m; ++i) {
          const float4 cc = sc[pw][i];
          const short4 dd = sd[pw][i];
          float v = swv[pw][i] + cc.x * sval[dd.x] + cc.y * sval[dd.y] + cc.z * sval[dd.z] + cc.w * sval[dd.w];
          v = fmaf(scp[pw][i], prev, v);
          out[i] = v;
          prev = v;
        }
      }
    } else {  // meanwhile: prepare window w + 1, write back window w - 1
      if (w + 1 < nwin) prep(w + 1, 32, SEQW - 32);
      if (w >= 1) writeback(w - 1, 32, SEQW - 32);
    }
    __syncthreads();
  }
  if (nwin > 0) writeback(nwin - 1, 0, SEQW);
}

// Preset boundary radiances for one hemisphere: top points get the sky
// radiance for downward columns; bottom points get the Lambertian surface
// radiance computed from the downwelling flux (FIXED/VARIABLE_LAMBERTIAN_
// BOUNDARY, src/polarized/shdomsub1.f:2438-2529).
// Rows of the scattering points gathered into a dense block (the A operand
// of the compacted tensor-core transforms); rowlen a multiple of 4.
__global__ void k_gather_rows(const float *__restrict__ src, const int *__restrict__ rows, int nrows, int rowlen,
                              float *__restrict__ dst) {
  const int q = rowlen >> 2;
  const long long total = (long long)nrows * q;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / q), k = (int)(t - (long long)i * q);
    reinterpret_cast<float4 *>(dst + (size_t)i * rowlen)[k] =
        __ldg(reinterpret_cast<const float4 *>(src + (size_t)__ldg(rows + i) * rowlen) + k);
  }
}

// Ordinate-to-harmonic transform of the points that do not scatter (a zero
// coefficient row): their source is zero in every iteration and their
// radiance is truncated to its first 4 terms, so only those 4 and the two
// hemispheric fluxes are formed (FP32 sums over the ordinates, one warp
// per point).  t4: the first 4 rows of the transform matrix [4][nang].
__global__ void __launch_bounds__(256) k_do_to_sh_light(const float *__restrict__ raddo, int ldo, int nang, int ncol_down,
                                                         const int *__restrict__ pts, int npts_light,
                                                         const float *__restrict__ t4, const float *__restrict__ fluxw,
                                                         float *__restrict__ radiance, int nlm, float *__restrict__ fluxes) {
  // weights per column, padded with zeros to ldo: the four l <= 1 terms,
  // then the downward and the upward flux weights
  extern __shared__ float4 wsm4[];
  float *wsm = reinterpret_cast<float *>(wsm4);
  for (int i = threadIdx.x; i < 6 * ldo; i += blockDim.x) {
    const int r = i / ldo, c = i - r * ldo;
    float v = 0.f;
    if (c < nang) {
      if (r < 4) v = __ldg(t4 + r * nang + c);
      else if (r == 4) v = c < ncol_down ? __ldg(fluxw + c) : 0.f;
      else v = c >= ncol_down ? __ldg(fluxw + c) : 0.f;
    }
    wsm[i] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, n4 = ldo >> 2;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < npts_light; w += nw) {
    const int p = __ldg(pts + w);
    const float4 *row = reinterpret_cast<const float4 *>(raddo + (size_t)p * ldo);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int q = lane; q < n4; q += 32) {
      const float4 v = __ldcs(row + q);  // read once: streamed past L1
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        const float4 wr = wsm4[r * n4 + q];
        acc[r] = fmaf(wr.x, v.x, fmaf(wr.y, v.y, fmaf(wr.z, v.z, fmaf(wr.w, v.w, acc[r]))));
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int r = 0; r < 6; ++r) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
    if (lane == 0) {
      float *rr = radiance + (size_t)p * nlm;
      rr[0] = acc[0]; rr[1] = acc[1]; rr[2] = acc[2]; rr[3] = acc[3];
      fluxes[2 * (size_t)p] = acc[4];
      fluxes[2 * (size_t)p + 1] = acc[5];
    }
  }
}

// stk (polarized): Stokes component per column; the sky and the surface
// emit unpolarized radiance, so the Q and U columns are preset to zero.
__global__ void k_preset_top(const int *topp, int ntop, float *raddo, int ldo, int ncol_down, float skyrad,
                             const uint8_t *stk) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntop * ncol_down) return;
  int k = t / ncol_down, c = t - k * ncol_down;
  raddo[(size_t)topp[k] * ldo + c] = (stk && stk[c]) ? 0.f : skyrad;
}

// FIXED/VARIABLE_LAMBERTIAN_BOUNDARY (src/polarized/shdomsub1.f:2438-2529):
// the reflected direct beam and downwelling flux plus, with a thermal
// source, the ground emission (1 - albedo) B (botplanck null otherwise).
__global__ void k_lambertian(const int *botp, int nbot, const float *botalb, const float *dirflux, const float *fluxw,
                             float *raddo, int nang, int ldo, int ncol_down, float *bcrad, const uint8_t *stk,
                             const float *botplanck) {
  int k = blockIdx.x;
  if (k >= nbot) return;
  int p = botp[k];
  __shared__ float red[256];
  float s = 0.f;
  for (int c = threadIdx.x; c < ncol_down; c += blockDim.x) s += fluxw[c] * raddo[(size_t)p * ldo + c];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const float opi = 0.318309886f;
  float b = opi * botalb[k] * (dirflux[p] + red[0]);
  if (botplanck) b += botplanck[k] * (1.f - botalb[k]);
  if (threadIdx.x == 0) bcrad[k] = b;
  for (int c = ncol_down + threadIdx.x; c < nang; c += blockDim.x) raddo[(size_t)p * ldo + c] = (stk && stk[c]) ? 0.f : b;
}

// Polarized transforms on the CUDA cores (the FP32 path): C[M][N] = A[M][K]
// (row stride lda) x B[K][N], 64 x 64 tiles, 4 x 4 outputs per thread, K in
// steps of 16 through shared memory.  mode 0 writes the ordinate sources
// (I clamped at zero, Q and U kept); mode 1 writes the harmonic radiance
// rows masked to the radiance truncation ((col mod nlm) < nr).
__global__ void __launch_bounds__(256) k_dense_xf(const float *__restrict__ A, int lda, const float *__restrict__ B,
                                                  int K, int N, int M, int mode, float *__restrict__ C, int ldc,
                                                  const uint8_t *__restrict__ stk, const int *__restrict__ nr, int nlm) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][64];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row0 = blockIdx.y * 64, col0 = blockIdx.x * 64;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int t = threadIdx.x; t < 64 * 16; t += 256) {
      const int r = t >> 4, kk = t & 15, gr = row0 + r, gk = k0 + kk;
      As[kk][r] = (gr < M && gk < K) ? A[(size_t)gr * lda + gk] : 0.f;
    }
    for (int t = threadIdx.x; t < 16 * 64; t += 256) {
      const int kk = t >> 6, c = t & 63, gk = k0 + kk, gc = col0 + c;
      Bs[kk][c] = (gk < K && gc < N) ? B[(size_t)gk * N + gc] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = row0 + ty * 4 + i;
    if (row >= M) continue;
    const int nrp = mode == 1 ? nr[row] : 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = col0 + tx * 4 + j;
      if (col >= N) continue;
      float v = acc[i][j];
      if (mode == 0) { if (!stk[col]) v = fmaxf(v, 0.f); }
      else if (col % nlm >= nrp) v = 0.f;
      C[(size_t)row * ldc + col] = v;
    }
  }
}

// Hemispheric fluxes of every point from its ordinate radiances (one warp per point).
__global__ void __launch_bounds__(256) k_do_fluxes(const float *__restrict__ raddo, int ldo, int nang, int ncol_down,
                                                   const float *__restrict__ fluxw, int npts, float *__restrict__ fluxes) {
  const int lane = threadIdx.x & 31;
  for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < npts; p += (gridDim.x * blockDim.x) >> 5) {
    float fd = 0.f, fu = 0.f;
    for (int c = lane; c < nang; c += 32) {
      const float v = fluxw[c] * raddo[(size_t)p * ldo + c];
      if (c < ncol_down) fd += v; else fu += v;
    }
    for (int o = 16; o > 0; o >>= 1) { fd += __shfl_xor_sync(0xffffffffu, fd, o); fu += __shfl_xor_sync(0xffffffffu, fu, o); }
    if (lane == 0) { fluxes[2 * (size_t)p] = fd; fluxes[2 * (size_t)p + 1] = fu; }
  }
}

// Marks every corner of each cell that has a scattering corner (nb zeroed
// beforehand; concurrent writes all store 1).
__global__ void k_spread_scat(const int *__restrict__ gridptr, int ncells, const uint8_t *__restrict__ sc,
                              uint8_t *__restrict__ nb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int *g = gridptr + 8 * (size_t)c;
  bool any = false;
#pragma unroll
  for (int k = 0; k < 8; ++k) any = any || sc[g[k]];
  if (any)
#pragma unroll
    for (int k = 0; k < 8; ++k) nb[g[k]] = 1;
}

// ------------------------------------------------------------ direct beam
// DIRECT_BEAM_PROP (src/polarized/shdom90.f90:352-867) via MAKE_DIRECT
// (src/polarized/shdomsub2.f:393-476): per grid point, the delta-M scaled
// extinction of the property grid integrated exactly (trilinear in each
// property cell: a + b/2 + c/3 + d/4 of the segment) along the ray to the
// sun, in double precision; one thread per point.
struct BeamGeom {
  const double *edp;      // [npx*npy*npz] delta-M scaled property-grid extinction
  const float *zlev, *gridpos;
  float *dirflux;
  int npts, npx, npy, npz, bcflag, ipflag;
  float delx, dely, solarmu, solaraz, solarflux;
};

// DIRECT_BEAM_PROP per grid point: the ray toward the sun through the
// property grid, the exact integral of the trilinear extinction over each
// cell it crosses.  The reference runs the walk in double precision; here
// the per-cell geometry and the cell integral are FP32 on offsets from the
// cell's own corner (cell-relative coordinates in [0, 1], as the render
// does), and the path sum and the set-up stay FP64.
__global__ void __launch_bounds__(128) k_direct_beam(BeamGeom b) {
  const int ipt = blockIdx.x * blockDim.x + threadIdx.x;
  if (ipt >= b.npts) return;
  const int npx = b.npx, npy = b.npy, npz = b.npz, bc = b.bcflag;
  const int ipd = (b.ipflag & 4) ? 0 : b.ipflag;
  const double sunmu = -(double)b.solarmu, sunaz = (double)(float)(b.solaraz + 3.14159274f);
  double cxd = sqrt(1.0 - sunmu * sunmu) * cos(sunaz), cyd = sqrt(1.0 - sunmu * sunmu) * sin(sunaz);
  double czd = fabs(sunmu), cxid, cyid, czid;
  if (fabs(cxd) > 1e-6) cxid = 1.0 / cxd; else { cxd = 0; cxid = 1e20; }
  if (fabs(cyd) > 1e-6) cyid = 1.0 / cyd; else { cyd = 0; cyid = 1e20; }
  if (fabs(czd) > 1e-6) czid = 1.0 / czd; else { czd = 0; czid = 1e20; }
  const float cx = (float)cxd, cy = (float)cyd, cz = (float)czd;
  const float cxi = (float)cxid, cyi = (float)cyid, czi = (float)czid;
  const int di = cxd >= 0 ? 1 : -1, dj = cyd >= 0 ? 1 : -1, dk = czd >= 0 ? 1 : -1;
  const double dxd = b.delx, dyd = b.dely, xdom = dxd * npx, ydom = dyd * npy;
  const float dx = b.delx, dy = b.dely;
  const double z = b.gridpos[3 * ipt + 2], x = b.gridpos[3 * ipt], y = b.gridpos[3 * ipt + 1];
  int il = 0, iu = npz;
  while (iu - il > 1) { int im = (iu + il) / 2; if (z >= b.zlev[im - 1]) il = im; else iu = im; }
  int k = max(il, 1), i = (int)(x / dxd) + 1, j = (int)(y / dyd) + 1;
  if (i > npx && fabs(x - xdom) < 0.001 * dxd) i = npx;
  if (j > npy && fabs(y - ydom) < 0.001 * dyd) j = npy;
  bool cxf = (ipd & 1) || cxd == 0.0, cyf = (ipd & 2) || cyd == 0.0;
  if ((bc & 1) && (fabs(x) < 0.01 * dxd || fabs(x - (npx - 1) * dxd) < 0.01 * dxd)) cxf = true;
  if ((bc & 2) && (fabs(y) < 0.01 * dyd || fabs(y - (npy - 1) * dyd) < 0.01 * dyd)) cyf = true;
  // the position as offsets from the current cell's low corner
  float lx = (float)(x - dxd * (i - 1)), ly = (float)(y - dyd * (j - 1)), lz = (float)(z - (double)b.zlev[k - 1]);
  const float epsz = 1.0e-6f * (b.zlev[npz - 1] - b.zlev[0]);
  double path = 0.0;
  const int guard_max = 4 * (npx + npy + npz) * 64;
  for (int guard = 0; guard < guard_max; ++guard) {
    if (k >= npz || fabsf((b.zlev[k - 1] + lz) - b.zlev[npz - 1]) <= epsz) break;  // at the top level
    const int ipn = (i == npx) ? ((bc & 1) ? npx : 1) : i + 1, jpn = (j == npy) ? ((bc & 2) ? npy : 1) : j + 1;
    const float dz = b.zlev[k] - b.zlev[k - 1];
    const int I1 = (k - 1) + npz * (j - 1) + npz * npy * (i - 1), I2 = (k - 1) + npz * (j - 1) + npz * npy * (ipn - 1);
    const int I3 = (k - 1) + npz * (jpn - 1) + npz * npy * (i - 1), I4 = (k - 1) + npz * (jpn - 1) + npz * npy * (ipn - 1);
    const float e1 = (float)b.edp[I1], e2 = (float)b.edp[I2], e3 = (float)b.edp[I3], e4 = (float)b.edp[I4];
    const float e5 = (float)b.edp[I1 + 1], e6 = (float)b.edp[I2 + 1], e7 = (float)b.edp[I3 + 1], e8 = (float)b.edp[I4 + 1];
    float sox, soy, soz, lxp = lx, lyp = ly, lzp = lz;
    if (cxf) sox = 1e30f; else if (cx > 0) { sox = (dx - lx) * cxi; lxp = dx; } else { sox = (0.f - lx) * cxi; lxp = 0.f; }
    if (cyf) soy = 1e30f; else if (cy > 0) { soy = (dy - ly) * cyi; lyp = dy; } else { soy = (0.f - ly) * cyi; lyp = 0.f; }
    if (cz > 0) { soz = (dz - lz) * czi; lzp = dz; } else if (cz < 0) { soz = (0.f - lz) * czi; lzp = 0.f; } else soz = 1e30f;
    float so;
    int face;  // 0 x, 1 y, 2 z
    if (soz <= sox && soz <= soy) {
      so = soz; if (!cxf) lxp = lx + so * cx; if (!cyf) lyp = ly + so * cy; face = 2;
    } else if (sox <= soy) {
      so = sox; if (!cyf) lyp = ly + so * cy; lzp = lz + so * cz; face = 0;
    } else {
      so = soy; if (!cxf) lxp = lx + so * cx; lzp = lz + so * cz; face = 1;
    }
    so = fmaxf(so, 0.f);
    const float ax = 1.f / dx, ay = 1.f / dy, az = 1.f / dz;
    const float u0 = lx * ax, v0 = ly * ay, w0 = lz * az;
    const float du = lxp * ax - u0, dv = lyp * ay - v0, dw = lzp * az - w0;
    const float u0m = 1 - u0, v0m = 1 - v0, w0m = 1 - w0;
    const float A = (e1 * u0m + e2 * u0) * v0m * w0m + (e3 * u0m + e4 * u0) * v0 * w0m +
                    (e5 * u0m + e6 * u0) * v0m * w0 + (e7 * u0m + e8 * u0) * v0 * w0;
    const float B = (-du * v0m * w0m - dv * u0m * w0m - dw * u0m * v0m) * e1 + (du * v0m * w0m - dv * u0 * w0m - dw * u0 * v0m) * e2 +
                    (-du * v0 * w0m + dv * u0m * w0m - dw * u0m * v0) * e3 + (du * v0 * w0m + dv * u0 * w0m - dw * u0 * v0) * e4 +
                    (-du * v0m * w0 - dv * u0m * w0 + dw * u0m * v0m) * e5 + (du * v0m * w0 - dv * u0 * w0 + dw * u0 * v0m) * e6 +
                    (-du * v0 * w0 + dv * u0m * w0 + dw * u0m * v0) * e7 + (du * v0 * w0 + dv * u0 * w0 + dw * u0 * v0) * e8;
    const float vw = dv * dw, uw = du * dw, uv = du * dv;
    const float Cc = (vw * u0m + uw * v0m + uv * w0m) * e1 + (vw * u0 - uw * v0m - uv * w0m) * e2 +
                     (-vw * u0m + uw * v0 - uv * w0m) * e3 + (-vw * u0 - uw * v0 + uv * w0m) * e4 +
                     (-vw * u0m - uw * v0m + uv * w0) * e5 + (-vw * u0 + uw * v0m - uv * w0) * e6 +
                     (vw * u0m - uw * v0 - uv * w0) * e7 + (vw * u0 + uw * v0 + uv * w0) * e8;
    const float D = du * dv * dw * (e2 + e3 + e5 + e8 - e1 - e4 - e6 - e7);
    path += (double)(so * (A + 0.5f * B + 0.3333333333f * Cc + 0.25f * D));
    // into the next cell: the crossed face's offset is 0 or the new cell's extent
    if (face == 2) {
      k += dk;
      lx = lxp; ly = lyp;
      lz = (dk > 0) ? 0.f : ((k >= 1 && k < npz) ? b.zlev[k] - b.zlev[k - 1] : 0.f);
      if (k < 1) break;
    } else if (face == 0) {
      i += di;
      if (i == 0) { if (bc & 1) { i = 1; cxf = true; } else { i = npx; } }
      else if (i == npx + 1) { if (bc & 1) { i = npx; cxf = true; } else { i = 1; } }
      lx = cxf ? lxp : ((di > 0) ? 0.f : dx);
      ly = lyp; lz = lzp;
    } else {
      j += dj;
      if (j == 0) { if (bc & 2) { j = 1; cyf = true; } else { j = npy; } }
      else if (j == npy + 1) { if (bc & 2) { j = npy; cyf = true; } else { j = 1; } }
      ly = cyf ? lyp : ((dj > 0) ? 0.f : dy);
      lx = lxp; lz = lzp;
    }
  }
  b.dirflux[ipt] = (float)(b.solarflux * exp(-path));
}

// ------------------------------------------------ bidirectional surfaces
// SURFACE_BRDF (src/polarized/shdomsub2.f:1222-1300) for the built types:
// 'R' RPV_REFLECTION (:1658-1696, single precision), 'W'
// WAVE_FRESNEL_REFLECTION (:1358-1525, double precision with complex
// Fresnel coefficients) and 'D' DINER_REFLECTION (:1526-1657, single
// precision; its Fresnel index 1.5 is real, so the coefficients are real).  Incident direction (mu1 < 0, phi1), outgoing
// (mu2 > 0, phi2); R[3][3] is the I, Q, U block of the reflection matrix,
// normalised so that a Lambertian surface gives its albedo.
struct BrdfOrd {
  float mu, phi, w, col, off;  // ordinate, weight |mu| wtdo / pi (downward), I column, Stokes column stride
};

struct Cd {
  double r, i;
};
__device__ __forceinline__ Cd cadd(Cd a, Cd b) { return {a.r + b.r, a.i + b.i}; }
__device__ __forceinline__ Cd csub(Cd a, Cd b) { return {a.r - b.r, a.i - b.i}; }
__device__ __forceinline__ Cd cmul(Cd a, Cd b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ Cd cscale(Cd a, double s) { return {a.r * s, a.i * s}; }
__device__ __forceinline__ Cd cconj(Cd a) { return {a.r, -a.i}; }
__device__ __forceinline__ double cnorm(Cd a) { return a.r * a.r + a.i * a.i; }
__device__ __forceinline__ Cd cdiv(Cd a, Cd b) {
  const double d = b.r * b.r + b.i * b.i;
  return {(a.r * b.r + a.i * b.i) / d, (a.i * b.r - a.r * b.i) / d};
}
__device__ __forceinline__ Cd csqrt_(Cd a) {  // principal branch
  const double m = hypot(a.r, a.i);
  if (m == 0.0) return {0.0, 0.0};
  const double re = sqrt(0.5 * (m + a.r)), im = sqrt(0.5 * (m - a.r));
  return {re, signbit(a.i) ? -im : im};
}

__device__ float rpv_reflection_d(float rho0, float k, float theta, float mu1, float mu2, float phi) {
  const float mu_min = 0.03f;
  const float x1 = fmaxf(mu1, mu_min), x2 = fmaxf(mu2, mu_min);
  const float m = powf(x1 * x2 * (x1 + x2), k - 1.0f);
  const float cosphi = cosf(phi);
  const float sin1 = sqrtf(1.0f - x1 * x1), sin2 = sqrtf(1.0f - x2 * x2);
  const float cosg = x1 * x2 + sin1 * sin2 * cosphi;
  const float f = (1.0f - theta * theta) / powf(1.0f + 2.0f * theta * cosg + theta * theta, 1.5f);
  const float tan1 = sin1 / x1, tan2 = sin2 / x2;
  const float capg = sqrtf(fabsf(tan1 * tan1 + tan2 * tan2 - 2.0f * tan1 * tan2 * cosphi));
  const float h = 1.0f + (1.0f - rho0) / (1.0f + capg);
  return rho0 * m * f * h;
}

__device__ void wave_fresnel_d(float mre, float mim, float wind, float mui, float mur, float phii, float phir,
                               float R[3][3]) {
  const Cd cn1 = {1.0, 0.0}, cn2 = {(double)mre, (double)mim};
  const double sigma2 = fmax(0.0005, 0.0015 + 0.00256 * (double)wind);
  double dmui = fabs((double)mui), dmur = (double)mur;
  if (fabs(dmui - 1.0) < 1e-10) dmui = 0.999999999999;
  if (fabs(dmur - 1.0) < 1e-10) dmur = 0.999999999999;
  double dsini, dcosi, dsinr, dcosr;
  sincos((double)phii, &dsini, &dcosi);
  sincos((double)phir, &dsinr, &dcosr);
  const double dsi = sqrt(1.0 - dmui * dmui), dsr = sqrt(1.0 - dmur * dmur);
  const double vi1 = dsi * dcosi, vi2 = dsi * dsini, vi3 = -dmui;
  const double vr1 = dsr * dcosr, vr2 = dsr * dsinr, vr3 = dmur;
  const double u1 = vi1 - vr1, u2 = vi2 - vr2, u3 = vi3 - vr3;
  const double fact1 = u1 * u1 + u2 * u2 + u3 * u3, factor = sqrt(1.0 / fact1);
  const double xi1 = factor * (u1 * vi1 + u2 * vi2 + u3 * vi3);
  const Cd cxi2 = csqrt_(csub({1.0, 0.0}, cscale(cdiv(cmul(cn1, cn1), cmul(cn2, cn2)), 1.0 - xi1 * xi1)));
  Cd c1 = cscale(cn1, xi1), c2 = cmul(cn2, cxi2);
  const Cd crper = cdiv(csub(c1, c2), cadd(c1, c2));
  c1 = cscale(cn2, xi1); c2 = cmul(cn1, cxi2);
  const Cd crpar = cdiv(csub(c1, c2), cadd(c1, c2));
  const double ti1 = -dmui * dcosi, ti2 = -dmui * dsini, ti3 = -dsi;
  const double tr1 = dmur * dcosr, tr2 = dmur * dsinr, tr3 = -dsr;
  const double pikr = -dsini * vr1 + dcosi * vr2, prki = -dsinr * vi1 + dcosr * vi2;
  const double tikr = ti1 * vr1 + ti2 * vr2 + ti3 * vr3, trki = tr1 * vi1 + tr2 * vi2 + tr3 * vi3;
  const double e1 = pikr * prki, e2 = tikr * trki, e3 = tikr * prki, e4 = pikr * trki;
  const Cd cf11 = cadd(cscale(crper, e1), cscale(crpar, e2)), cf12 = cadd(cscale(crper, -e3), cscale(crpar, e4));
  const Cd cf21 = cadd(cscale(crper, -e4), cscale(crpar, e3)), cf22 = cadd(cscale(crper, e2), cscale(crpar, e1));
  const double vp1 = vi2 * vr3 - vi3 * vr2, vp2 = vi3 * vr1 - vi1 * vr3, vp3 = vi1 * vr2 - vi2 * vr1;
  const double vpm = vp1 * vp1 + vp2 * vp2 + vp3 * vp3, dmod = vpm * vpm;
  const double rdz2 = u3 * u3, rdz4 = rdz2 * rdz2;
  const double dex = exp(-(u1 * u1 + u2 * u2) / (2 * sigma2 * rdz2));
  const double dcoeff = fact1 * fact1 * dex / (4 * dmui * dmur * dmod * rdz4 * 2 * sigma2);
  const double af = 0.5 * dcoeff;
  const double af11 = cnorm(cf11), af12 = cnorm(cf12), af21 = cnorm(cf21), af22 = cnorm(cf22);
  double r[3][3];
  r[0][0] = (af11 + af12 + af21 + af22) * af;
  r[0][1] = (af11 - af12 + af21 - af22) * af;
  r[1][0] = (af11 - af22 + af12 - af21) * af;
  r[1][1] = (af11 - af12 - af21 + af22) * af;
  const Cd c21 = cconj(cf21), c22 = cconj(cf22);
  const Cd ctttp = cmul(cf11, cconj(cf12)), cttpt = cmul(cf11, c21), cttpp = cmul(cf11, c22);
  const Cd ctppt = cmul(cf12, c21), ctppp = cmul(cf12, c22), cptpp = cmul(cf21, c22);
  r[0][2] = (-ctttp.r - cptpp.r) * dcoeff;
  r[1][2] = (-ctttp.r + cptpp.r) * dcoeff;
  r[2][0] = (-cttpt.r - ctppp.r) * dcoeff;
  r[2][1] = (-cttpt.r + ctppp.r) * dcoeff;
  r[2][2] = (cttpp.r + ctppt.r) * dcoeff;
  const double pp = 3.141592653589793, s1 = sqrt(2 * sigma2 / pp), s3 = 1.0 / sqrt(2 * sigma2), s2 = s3 * s3;
  double dcot = dmui / sqrt(1.0 - dmui * dmui);
  const double shi = 0.5 * (s1 * exp(-s2 * dcot * dcot) / dcot - erfc(dcot * s3));
  dcot = dmur / sqrt(1.0 - dmur * dmur);
  const double shr = 0.5 * (s1 * exp(-s2 * dcot * dcot) / dcot - erfc(dcot * s3));
  const double shadow = 1.0 / (1.0 + shi + shr);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i][j] = (float)(r[i][j] * shadow);
}

__device__ void diner_d(float a, float k, float b, float zeta, float sigma, float mu1, float mu2, float phi, float R[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i][j] = 0.f;
  const float sinth1 = sqrtf(1.0f - mu1 * mu1), sinth2 = sqrtf(1.0f - mu2 * mu2);
  const float cosphi = cosf(phi);
  const float cossc = fminf(1.0f, fmaxf(-1.0f, -mu1 * mu2 + sinth1 * sinth2 * cosphi));
  const float tan1 = sinth1 / mu1, tan2 = sinth2 / mu2;
  const float capg = sqrtf(fabsf(tan1 * tan1 + tan2 * tan2 + 2 * tan1 * tan2 * cosphi));
  const float hot = 1 + (1 - a) / (1 + capg);
  R[0][0] = a * powf((mu1 + mu2) * mu1 * mu2, k - 1) * expf(b * cossc) * hot;
  if (zeta < 0.0f) return;
  const float gamma = 0.5f * acosf(-cossc), cosg = cosf(gamma);
  const float eps = 2.25f;
  const float d = sqrtf(eps - 1.0f + cosg * cosg);
  const float rp = (eps * cosg - d) / (eps * cosg + d), rs = (cosg - d) / (cosg + d);
  const float f11 = 0.5f * (rp * rp + rs * rs), f12 = 0.5f * (rp * rp - rs * rs), f33 = rp * rs;
  const float cosbeta = 0.5f * (mu1 + mu2) / cosg;
  const float h = sigma > 0.0f ? zeta * expf(-0.5f * (1 / (cosbeta * cosbeta) - 1) / (sigma * sigma)) /
                                     (8 * sigma * sigma * mu2 * mu1 * cosbeta * cosbeta * cosbeta * cosbeta)
                               : zeta / (8 * mu2 * mu1 * cosbeta);
  R[0][0] += h * f11;
  const float sinphi = sinf(phi);
  const float al1 = atanf(sinth2 * sinphi / (mu2 * sinth1 + sinth2 * mu1 * cosphi));
  const float al2 = atanf(sinth1 * sinphi / (sinth2 * mu1 + mu2 * sinth1 * cosphi));
  const float c1 = cosf(2 * al1), s1 = sinf(2 * al1), c2 = cosf(2 * al2), s2 = sinf(2 * al2);
  R[0][1] = h * f12 * c1;
  R[1][0] = h * f12 * c2;
  R[1][1] = h * (f11 * c1 * c2 + f33 * s1 * s2);
  R[0][2] = -h * f12 * s1;
  R[1][2] = h * (-f11 * s1 * c2 + f33 * c1 * s2);
  R[2][0] = -h * f12 * s2;
  R[2][1] = h * (-f11 * c1 * s2 + f33 * s1 * c2);
  R[2][2] = h * (f11 * s1 * s2 + f33 * c1 * c2);
}

__constant__ float kOcWhitecap[39] = {
    0.220f, 0.220f, 0.220f, 0.220f, 0.220f, 0.220f, 0.215f, 0.210f, 0.200f, 0.190f, 0.175f, 0.155f, 0.130f,
    0.080f, 0.100f, 0.105f, 0.100f, 0.080f, 0.045f, 0.055f, 0.065f, 0.060f, 0.055f, 0.040f, 0.f,    0.f,
    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f,    0.f};
__constant__ float kOcAngBnd[5] = {0.0f, 45.0f, 60.0f, 75.0f, 85.0f};
__constant__ float kOcWsBnd[6] = {1.0f, 3.0f, 5.0f, 7.0f, 9.0f, 20.0f};
__constant__ float kOcTds[5][6] = {{0.9787803f, 0.9787738f, 0.9787626f, 0.9787467f, 0.9787264f, 0.9785573f},
                                     {0.9706900f, 0.9698871f, 0.9691746f, 0.9685547f, 0.9680276f, 0.9666586f},
                                     {0.9479931f, 0.9404608f, 0.9385692f, 0.9381815f, 0.9384519f, 0.9430056f},
                                     {0.9690591f, 0.9275920f, 0.9058769f, 0.8951812f, 0.8899654f, 0.8892645f},
                                     {0.9980542f, 0.9602273f, 0.9114283f, 0.8713799f, 0.8417820f, 0.7800314f}};
__constant__ float kOcTdv[5][6] = {{0.9787764f, 0.9787535f, 0.9787106f, 0.9786453f, 0.9785548f, 0.9775019f},
                                     {0.9692680f, 0.9637051f, 0.9564344f, 0.9495727f, 0.9438773f, 0.9288712f},
                                     {0.9225163f, 0.9069787f, 0.9044844f, 0.9052351f, 0.9068328f, 0.9153687f},
                                     {0.8048478f, 0.8479503f, 0.8678726f, 0.8797889f, 0.8878716f, 0.9091171f},
                                     {0.7294627f, 0.8137348f, 0.8453338f, 0.8629867f, 0.8745421f, 0.9036854f}};
__constant__ float kOcKw[61] = {
    0.0209f, 0.0200f, 0.0196f, 0.0189f, 0.0183f, 0.0182f, 0.0171f, 0.0170f, 0.0168f, 0.0166f, 0.0168f, 0.0170f, 0.0173f,
    0.0174f, 0.0175f, 0.0184f, 0.0194f, 0.0203f, 0.0217f, 0.0240f, 0.0271f, 0.0320f, 0.0384f, 0.0445f, 0.0490f, 0.0505f,
    0.0518f, 0.0543f, 0.0568f, 0.0615f, 0.0640f, 0.0640f, 0.0717f, 0.0762f, 0.0807f, 0.0940f, 0.1070f, 0.1280f, 0.1570f,
    0.2000f, 0.2530f, 0.2790f, 0.2960f, 0.3030f, 0.3100f, 0.3150f, 0.3200f, 0.3250f, 0.3300f, 0.3400f, 0.3500f, 0.3700f,
    0.4050f, 0.4180f, 0.4300f, 0.4400f, 0.4500f, 0.4700f, 0.5000f, 0.5500f, 0.6500f};
__constant__ float kOcXc[61] = {
    0.1100f, 0.1110f, 0.1125f, 0.1135f, 0.1126f, 0.1104f, 0.1078f, 0.1065f, 0.1041f, 0.0996f, 0.0971f, 0.0939f, 0.0896f,
    0.0859f, 0.0823f, 0.0788f, 0.0746f, 0.0726f, 0.0690f, 0.0660f, 0.0636f, 0.0600f, 0.0578f, 0.0540f, 0.0498f, 0.0475f,
    0.0467f, 0.0450f, 0.0440f, 0.0426f, 0.0410f, 0.0400f, 0.0390f, 0.0375f, 0.0360f, 0.0340f, 0.0330f, 0.0328f, 0.0325f,
    0.0330f, 0.0340f, 0.0350f, 0.0360f, 0.0375f, 0.0385f, 0.0400f, 0.0420f, 0.0430f, 0.0440f, 0.0445f, 0.0450f, 0.0460f,
    0.0475f, 0.0490f, 0.0515f, 0.0520f, 0.0505f, 0.0440f, 0.0390f, 0.0340f, 0.0300f};
__constant__ float kOcE[61] = {
    0.668f, 0.672f, 0.680f, 0.687f, 0.693f, 0.701f, 0.707f, 0.708f, 0.707f, 0.704f, 0.701f, 0.699f, 0.700f, 0.703f, 0.703f,
    0.703f, 0.703f, 0.704f, 0.702f, 0.700f, 0.700f, 0.695f, 0.690f, 0.685f, 0.680f, 0.675f, 0.670f, 0.665f, 0.660f, 0.655f,
    0.650f, 0.645f, 0.640f, 0.630f, 0.623f, 0.615f, 0.610f, 0.614f, 0.618f, 0.622f, 0.626f, 0.630f, 0.634f, 0.638f, 0.642f,
    0.647f, 0.653f, 0.658f, 0.663f, 0.667f, 0.672f, 0.677f, 0.682f, 0.687f, 0.695f, 0.697f, 0.693f, 0.665f, 0.640f, 0.620f,
    0.600f};
__constant__ float kOcBw[61] = {
    0.0076f, 0.0072f, 0.0068f, 0.0064f, 0.0061f, 0.0058f, 0.0055f, 0.0052f, 0.0049f, 0.0047f, 0.0045f, 0.0043f, 0.0041f,
    0.0039f, 0.0037f, 0.0036f, 0.0034f, 0.0033f, 0.0031f, 0.0030f, 0.0029f, 0.0027f, 0.0026f, 0.0025f, 0.0024f, 0.0023f,
    0.0022f, 0.0022f, 0.0021f, 0.0020f, 0.0019f, 0.0018f, 0.0018f, 0.0017f, 0.0017f, 0.0016f, 0.0016f, 0.0015f, 0.0015f,
    0.0014f, 0.0014f, 0.0013f, 0.0013f, 0.0012f, 0.0012f, 0.0011f, 0.0011f, 0.0010f, 0.0010f, 0.0010f, 0.0010f, 0.0009f,
    0.0008f, 0.0008f, 0.0008f, 0.0007f, 0.0007f, 0.0007f, 0.0007f, 0.0007f, 0.0007f};
__constant__ float kOcTwl[62] = {
    0.250f, 0.275f, 0.300f, 0.325f, 0.345f, 0.375f, 0.400f, 0.425f, 0.445f, 0.475f, 0.500f, 0.525f, 0.550f, 0.575f, 0.600f,
    0.625f, 0.650f, 0.675f, 0.700f, 0.725f, 0.750f, 0.775f, 0.800f, 0.825f, 0.850f, 0.875f, 0.900f, 0.925f, 0.950f, 0.975f,
    1.000f, 1.200f, 1.400f, 1.600f, 1.800f, 2.000f, 2.200f, 2.400f, 2.600f, 2.650f, 2.700f, 2.750f, 2.800f, 2.850f, 2.900f,
    2.950f, 3.000f, 3.050f, 3.100f, 3.150f, 3.200f, 3.250f, 3.300f, 3.350f, 3.400f, 3.450f, 3.500f, 3.600f, 3.700f, 3.800f,
    3.900f, 4.000f};
__constant__ float kOcTnr[62] = {
    1.362f, 1.354f, 1.349f, 1.346f, 1.343f, 1.341f, 1.339f, 1.338f, 1.337f, 1.336f, 1.335f, 1.334f, 1.333f, 1.333f, 1.332f,
    1.332f, 1.331f, 1.331f, 1.331f, 1.330f, 1.330f, 1.330f, 1.329f, 1.329f, 1.329f, 1.328f, 1.328f, 1.328f, 1.327f, 1.327f,
    1.327f, 1.324f, 1.321f, 1.317f, 1.312f, 1.306f, 1.296f, 1.279f, 1.242f, 1.219f, 1.188f, 1.157f, 1.142f, 1.149f, 1.201f,
    1.292f, 1.371f, 1.426f, 1.467f, 1.483f, 1.478f, 1.467f, 1.450f, 1.432f, 1.420f, 1.410f, 1.400f, 1.385f, 1.374f, 1.364f,
    1.357f, 1.351f};
__constant__ float kOcTni[62] = {
    3.35E-08f, 2.35E-08f, 1.60E-08f, 1.08E-08f, 6.50E-09f, 3.50E-09f, 1.86E-09f, 1.30E-09f, 1.02E-09f, 9.35E-10f, 1.00E-09f,
    1.32E-09f, 1.96E-09f, 3.60E-09f, 1.09E-08f, 1.39E-08f, 1.64E-08f, 2.23E-08f, 3.35E-08f, 9.15E-08f, 1.56E-07f, 1.48E-07f,
    1.25E-07f, 1.82E-07f, 2.93E-07f, 3.91E-07f, 4.86E-07f, 1.06E-06f, 2.93E-06f, 3.48E-06f, 2.89E-06f, 9.89E-06f, 1.38E-04f,
    8.55E-05f, 1.15E-04f, 1.10E-03f, 2.89E-04f, 9.56E-04f, 3.17E-03f, 6.70E-03f, 1.90E-02f, 5.90E-02f, 1.15E-01f, 1.85E-01f,
    2.68E-01f, 2.98E-01f, 2.72E-01f, 2.40E-01f, 1.92E-01f, 1.35E-01f, 9.24E-02f, 6.10E-02f, 3.68E-02f, 2.61E-02f, 1.95E-02f,
    1.32E-02f, 9.40E-03f, 5.15E-03f, 3.60E-03f, 3.40E-03f, 3.80E-03f, 4.60E-03f};

// 1-based bracketing index of x in an increasing table of n entries
// (getbound): the searched half depends on the midpoint, and x outside
// the table takes the first or the last interval.
__device__ int oc_bracket(const float *xv, int n, float x) {
  const int imid = n / 2 + 1;
  const int lo = x > xv[imid - 1] ? imid : 1, hi = x > xv[imid - 1] ? n - 1 : imid;
  for (int i = lo; i <= hi; ++i)
    if (xv[i - 1] <= x && xv[i] >= x) return i;
  return x < xv[0] ? 1 : n - 1;
}

// Sea-water reflectance below the surface for Case I waters (morcasiwat):
// R = 0.33 bb / (u Kd), iterated on u; zero outside 400-700 nm.
__device__ float oc_morel_water(float wl, float c) {
  if (wl < 0.400f || wl > 0.700f) return 0.f;
  const int iwl = 1 + (int)lroundf((wl - 0.400f) / 0.005f);  // NINT: half away from zero
  const float kw = kOcKw[iwl - 1], xc = kOcXc[iwl - 1], e = kOcE[iwl - 1], bw = kOcBw[iwl - 1];
  float bb, kd;
  if (fabsf(c) < 0.0001f) { bb = 0.5f * bw; kd = kw; }
  else {
    const float b = 0.30f * powf(c, 0.62f);
    const float bbt = 0.002f + 0.02f * (0.5f - 0.25f * log10f(c)) * 0.550f / wl;
    bb = 0.5f * bw + bbt * b;
    kd = kw + xc * powf(c, e);
  }
  float r1 = 0.33f * bb / 0.75f / kd, r2 = r1;
  for (int it = 0; it < 1000; ++it) {
    const float u2 = 0.90f * (1.f - r1) / (1.f + 2.25f * r1);
    r2 = 0.33f * bb / u2 / kd;
    if (fabsf((r2 - r1) / r2) < 0.0001f) break;
    r1 = r2;
  }
  return r2;
}

// Unpolarized Fresnel reflectance of a facet (Fresnel), complex index (nr, ni).
__device__ float oc_facet_fresnel(float nr, float ni, float coschi, float sinchi) {
  const float d = nr * nr - ni * ni - sinchi * sinchi;
  const float a1 = fabsf(d), a2 = sqrtf(d * d + 4 * nr * nr * ni * ni);
  const float u = sqrtf(0.5f * (a1 + a2)), v = sqrtf(fmaxf(0.0f, 0.5f * (-a1 + a2)));
  const float rr2 = ((coschi - u) * (coschi - u) + v * v) / ((coschi + u) * (coschi + u) + v * v);
  const float b1 = (nr * nr - ni * ni) * coschi, b2 = 2 * nr * ni * coschi;
  const float rl2 = ((b1 - u) * (b1 - u) + (b2 - v) * (b2 - v)) / ((b1 + u) * (b1 + u) + (b2 + v) * (b2 + v));
  return (rr2 + rl2) / 2.f;
}

// Sun glint of the Cox-Munk anisotropic (Gram-Charlier) slope
// distribution (sunglint); angles in degrees.
__device__ float oc_sun_glint(float wspd, float nr, float ni, float azw, float ts, float tv, float fi) {
  const float pi = atanf(1.f) * 4.f, fac = pi / 180.f;
  const float phw = azw * fac, cs = cosf(ts * fac), cv = cosf(tv * fac), ss = sinf(ts * fac),
              sv = sinf(tv * fac), phi = fi * fac;
  const float zx = -sv * sinf(phi) / (cs + cv), zy = (ss + sv * cosf(phi)) / (cs + cv);
  const float tilt = atanf(sqrtf(zx * zx + zy * zy));
  const float sc = 0.003f + 0.00192f * wspd, su = 0.00316f * wspd;
  const float c21 = 0.01f - 0.0086f * wspd, c03 = 0.04f - 0.033f * wspd, c40 = 0.40f, c22 = 0.12f, c04 = 0.23f;
  const float xe = (cosf(phw) * zx + sinf(phw) * zy) / sqrtf(sc);
  const float xn = (-sinf(phw) * zx + cosf(phw) * zy) / sqrtf(su);
  const float xe2 = xe * xe, xn2 = xn * xn;
  float coef = 1 - c21 / 2.f * (xe2 - 1) * xn - c03 / 6.f * (xn2 - 3) * xn;
  coef = coef + c40 / 24.f * (xe2 * xe2 - 6 * xe2 + 3);
  coef = coef + c04 / 24.f * (xn2 * xn2 - 6 * xn2 + 3);
  coef = coef + c22 / 4.f * (xe2 - 1) * (xn2 - 1);
  const float proba = coef / 2.f / pi / sqrtf(su) / sqrtf(sc) * expf(-(xe2 + xn2) / 2.f);
  float cos2chi = cv * cs + sv * ss * cosf(phi);
  cos2chi = fminf(1.0f, fmaxf(-1.0f, cos2chi));
  const float coschi = sqrtf(0.5f * (1 + cos2chi)), sinchi = sqrtf(0.5f * (1 - cos2chi));
  const float r1 = oc_facet_fresnel(nr, ni, coschi, sinchi);
  const float ct = cosf(tilt), ct2 = ct * ct;
  return pi * r1 * proba / 4.f / cs / cv / (ct2 * ct2);
}

// ocean_brdf_sw with the default salinity: whitecaps + glint + water body.
__device__ __noinline__ float ocean_reflection_d(float pws, float pcl, float pwl, float xmuo, float xmu, float xphi, float xpaw) {
  const float pi = atanf(1.f) * 4.f, fac = pi / 180.f;
  const float paw = xpaw / fac;
  const float phi = xphi < 0.f ? -xphi : (xphi >= 2.0f * pi ? xphi - 2.0f * pi : xphi);
  const float tetas = acosf(xmuo <= 0.028f ? 0.028f : xmuo) / fac;
  const float tetav = acosf(xmu <= 0.028f ? 0.028f : xmu) / fac;
  const float wl = pwl < 0.4f ? 0.4f : (pwl > 4.0f ? 4.0f : pwl);
  const float fi = 180.0f - phi / fac;
  const float wspd = fmaxf(0.25f, pws);
  // refractive index of sea water (indwat): Hale & Querry pure water,
  // interpolated, plus 0.006 for the default salinity
  int i = 2;
  while (!(wl < kOcTwl[i - 1]) && i < 62) ++i;
  const float xwl = kOcTwl[i - 1] - kOcTwl[i - 2];
  float nr = kOcTnr[i - 2] + (wl - kOcTwl[i - 2]) * (kOcTnr[i - 1] - kOcTnr[i - 2]) / xwl;
  const float ni = kOcTni[i - 2] + (wl - kOcTwl[i - 2]) * (kOcTni[i - 1] - kOcTni[i - 2]) / xwl;
  nr = nr + 0.006f;
  const float n12 = sqrtf(nr * nr + ni * ni);
  // whitecaps (Lambertian)
  const float w = 2.95E-06f * powf(wspd, 3.52f);
  const int iwl = 1 + (int)((wl - 0.2f) / 0.1f);
  const float wlp = 0.5f + (iwl - 1) * 0.1f;
  const float refi = kOcWhitecap[iwl] + (wl - wlp) / 0.1f * (kOcWhitecap[iwl - 1] - kOcWhitecap[iwl]);
  const float rwc = w * refi;
  const float rw = oc_morel_water(wl, pcl);
  const int iws1 = oc_bracket(kOcWsBnd, 6, wspd), isz1 = oc_bracket(kOcAngBnd, 5, tetas), ivz1 = oc_bracket(kOcAngBnd, 5, tetav);
  const float tds = kOcTds[isz1 - 1][iws1 - 1], tdv = kOcTdv[ivz1 - 1][iws1 - 1];
  const float rog = oc_sun_glint(wspd, nr, ni, paw, tetas, tetav, fi);
  const float a = 0.485f;
  const float rwb = (1 / (n12 * n12)) * tds * tdv * rw / (1 - a * rw);
  return rwc + (1 - w) * rog + (1 - rwc) * rwb;
}

// ROSS_THICK_LI_SPARSE (src/polarized/shdomsub2.f:1303-1355): the MODIS
// kernel BRDF fiso + fvol K_vol + fgeo K_geo (RossThick volume kernel,
// LiSparse geometric kernel with crown shape h/b = 2, b/r = 1), kernels in
// double precision from single-precision cosines, clipped at zero.
__device__ __noinline__ float ross_li_reflection_d(float fiso, float fgeo, float fvol, float hb, float br, float mud, float muu,
                                float relaz) {
  const double pi = acos(-1.0);
  double coseta = (double)(mud * muu + sqrtf(1.0f - mud * mud) * sqrtf(1.0f - muu * muu) * cosf(relaz));
  const float kvol = (float)((((pi / 2.0 - acos(coseta)) * coseta + sqrt(1.0 - coseta * coseta)) /
                              (double)(mud + muu)) - pi / 4.0);
  const double thd = fabs(atan(br * sqrt(1.0 - (double)(mud * mud)) / mud));
  const double thu = fabs(atan(br * sqrt(1.0 - (double)(muu * muu)) / muu));
  const double md = cos(thd), mu = cos(thu);
  coseta = md * mu + sqrt(1.0 - md * md) * sqrt(1.0 - mu * mu) * cos((double)relaz);
  const double secd = 1.0 / md, secu = 1.0 / mu;
  const double tand = sqrt(1.0 - md * md) / md, tanu = sqrt(1.0 - mu * mu) / mu;
  const double dsq = tand * tand + tanu * tanu - 2 * tanu * tand * cos((double)relaz);
  const double tts = tand * tanu * sin((double)relaz);
  double cost = hb * sqrt(dsq + tts * tts) / (secd + secu);
  cost = fmin(1.0, fmax(-1.0, cost));
  const double o = (acos(cost) - cost * sqrt(1.0 - cost * cost)) * (secd + secu) / pi;
  const float kgeo = (float)(o - secd - secu + 0.5 * (1.0 + coseta) * secu * secd);
  return fmaxf(fiso + fvol * kvol + fgeo * kgeo, 0.0f);
}

__device__ __forceinline__ void surface_brdf_d(int type, const float *par, float mu2, float phi2, float mu1, float phi1,
                                               float R[3][3]) {
  if (type == 'D') {
    diner_d(par[0], par[1], par[2], par[3], par[4], -mu1, mu2, phi2 - phi1, R);
  } else if (type == 'M') {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[i][j] = 0.f;
    R[0][0] = ross_li_reflection_d(par[0], par[1], par[2], 2.0f, 1.0f, -mu1, mu2, phi1 - phi2);
  } else if (type == 'O') {  // par: wind speed, pigment, wavelength (appended by the plan)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[i][j] = 0.f;
    R[0][0] = ocean_reflection_d(par[0], par[1], par[2], -mu1, mu2, phi1 - phi2, phi1);
  } else if (type == 'R') {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[i][j] = 0.f;
    R[0][0] = rpv_reflection_d(par[0], par[1], par[2], -mu1, mu2, phi1 - phi2 - 3.14159274f);
  } else {
    wave_fresnel_d(par[0], par[1], par[2], mu1, mu2, phi1, phi2, R);
  }
}

// VARIABLE_BRDF_SURFACE (src/polarized/shdomsub1.f:2592-2664) for every
// bottom point (block) and upward ordinate (thread): the reflected direct
// beam plus the reflection of the downwelling radiances that the downward
// sweep left at the point, written as the upward sweep's boundary values.
__global__ void __launch_bounds__(128) k_brdf_bottom(const int *__restrict__ botp, int nbot, const float *__restrict__ botpar,
                                                     int npar, int type, const BrdfOrd *__restrict__ dn, int ndn,
                                                     const BrdfOrd *__restrict__ up, int nup, const float *__restrict__ dirflux,
                                                     float solarmu, float solaraz, float *raddo, int ldo, int nst,
                                                     const float *__restrict__ botplanck) {
  const int b = blockIdx.x;
  if (b >= nbot) return;
  const int p = botp[b];
  const float *par = botpar + (size_t)b * npar;
  const float opi = 0.318309886f;
  const float *row = raddo + (size_t)p * ldo;
  for (int u = threadIdx.x; u < nup; u += blockDim.x) {
    const BrdfOrd o = up[u];
    float R[3][3], out[3];
    surface_brdf_d(type, par, o.mu, o.phi, solarmu, solaraz, R);
    for (int k = 0; k < nst; ++k) out[k] = opi * R[k][0] * dirflux[p];
    for (int d = 0; d < ndn; ++d) {
      const BrdfOrd i = dn[d];
      surface_brdf_d(type, par, o.mu, o.phi, i.mu, i.phi, R);
      const int ci = (int)i.col, oi = (int)i.off;
      for (int k1 = 0; k1 < nst; ++k1) {
        const float rin = row[ci + k1 * oi];
        for (int k = 0; k < nst; ++k) out[k] += i.w * R[k][k1] * rin;
      }
      if (botplanck) {  // polarized thermal emission, emissivity 1 - R11
        const float bp = botplanck[b];
        out[0] += i.w * (1.f - R[0][0]) * bp;
        for (int k = 1; k < nst; ++k) out[k] -= i.w * R[k][0] * bp;
      }
    }
    const int co = (int)o.col, oo = (int)o.off;
    for (int k = 0; k < nst; ++k) raddo[(size_t)p * ldo + co + k * oo] = out[k];
  }
}

// ---------------------------------------------------------------- source
struct SourceArgs {
  const float *coef;      // [npts][nl]
  const float *coefp;     // polarized: [npts][3][nl] a2, a3, b1 times the albedo
  const float *dirflux, *radiance, *ylmsun;
  const float *thermal;   // thermal source: [npts] extinction-weighted (1 - albedo) B(T), else null
  const int *lofj;
  float *source, *delsource;
  int *ns, *nso, *nr;     // nr is read (current) and rewritten (next)
  double *red;            // [4] deljdot, deljold, deljnew, jnorm
  int npts, nlm, nl, ml, mm;
  float secmu0, shacc;
  int first, fixsh, accel, highorder;
};

// COMPUTE_SOURCE (src/polarized/shdomsub1.f:967-1611) for all three passes
// at once, one warp per point, plus the next RADIANCE_TRUNCATION
// (src/polarized/shdomsub1.f:1615-1803) for the same point.
__global__ void __launch_bounds__(256) k_source(SourceArgs a) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double djdot = 0, djold = 0, djnew = 0, jn = 0;
  for (int p = warp; p < a.npts; p += nwarps) {
    const float *cf = a.coef + (size_t)p * a.nl;
    const float f0 = a.dirflux[p] * a.secmu0;
    const int nrp = a.nr[p];
    const int nsold = a.ns[p], nsoold = a.nso[p];
    const int nsmin = min(nsold, nsoold);
    float *S = a.source + (size_t)p * a.nlm;
    float *D = a.delsource + (size_t)p * a.nlm;
    const float *R = a.radiance + (size_t)p * a.nlm;
    int jlast = 0;  // 1-based index of the last term above shacc
    float pdot = 0.f, pold = 0.f, pnew = 0.f, pn = 0.f;  // this point's partial sums
    int jstart = 0;
    if ((a.nlm & 3) == 0) {
      // four consecutive terms per lane: 16-byte loads and stores, 128 terms per warp pass
      for (int j0 = 0; j0 < a.nlm; j0 += 128) {
        const int j = j0 + 4 * lane;
        float jt[4] = {0.f, 0.f, 0.f, 0.f};
        if (j < a.nlm) {
          // rows are read only as far as the truncations use them (clear points keep few terms)
          const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
          const float4 y4 = *reinterpret_cast<const float4 *>(a.ylmsun + j);
          const float4 r4 = j < nrp ? *reinterpret_cast<const float4 *>(R + j) : z4;
          const float yv[4] = {y4.x, y4.y, y4.z, y4.w}, rv[4] = {r4.x, r4.y, r4.z, r4.w};
          float4 s4 = z4, d4 = z4;
          if (!a.first) {
            if (j < nsold) s4 = *reinterpret_cast<const float4 *>(S + j);
            if (a.accel && j < nsmin) d4 = *reinterpret_cast<const float4 *>(D + j);
          }
          const float sv[4] = {s4.x, s4.y, s4.z, s4.w}, dv[4] = {d4.x, d4.y, d4.z, d4.w};
          float dnew[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float c = cf[a.lofj[j + q]];
            jt[q] = f0 * c * yv[q];
            if (j + q == 0 && a.thermal) jt[q] += 3.544907703f * a.thermal[p];  // isotropic emission, sqrt(4 pi) B
            if (j + q < nrp) jt[q] += c * rv[q];
            dnew[q] = 0.f;
            if (!a.first) {
              const float dn = jt[q] - sv[q];
              if (a.accel) {
                if (j + q < nsmin) { pdot += dn * dv[q]; pold += dv[q] * dv[q]; pnew += dn * dn; pn += sv[q] * sv[q]; }
                if (j + q < nsold) dnew[q] = dn;
              } else if (j + q < nsold) {
                pnew += dn * dn; pn += sv[q] * sv[q];
              }
            }
          }
          if (!a.first && a.accel) *reinterpret_cast<float4 *>(D + j) = make_float4(dnew[0], dnew[1], dnew[2], dnew[3]);
          // stash the new terms in the output row; truncated below once jlast is known
          *reinterpret_cast<float4 *>(S + j) = make_float4(jt[0], jt[1], jt[2], jt[3]);
        }
        int lastq = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (j + q < a.nlm && fabsf(jt[q]) > a.shacc) lastq = j + q + 1;
        jlast = max(jlast, __reduce_max_sync(0xffffffffu, lastq));
      }
      jstart = a.nlm;
    }
    for (int j0 = jstart; j0 < a.nlm; j0 += 32) {
      int j = j0 + lane;
      float jt = 0.f;
      if (j < a.nlm) {
        float c = cf[a.lofj[j]];
        jt = f0 * c * a.ylmsun[j];
        if (j == 0 && a.thermal) jt += 3.544907703f * a.thermal[p];
        if (j < nrp) jt += c * R[j];
        if (!a.first) {
          float sold = S[j];
          if (a.accel) {
            if (j < nsmin) {
              float dn = jt - sold, dd = D[j];
              pdot += dn * dd; pold += dd * dd; pnew += dn * dn; pn += sold * sold;
            }
            if (j < nsold) D[j] = jt - sold; else D[j] = 0.f;
          } else if (j < nsold) {
            float dn = jt - sold;
            pnew += dn * dn; pn += sold * sold;
          }
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, j < a.nlm && fabsf(jt) > a.shacc);
      if (m) jlast = j0 + 32 - __clz(m);
      // stash the new term in the output row; truncated below once jlast is known
      if (j < a.nlm) S[j] = jt;
    }
    djdot += (double)pdot; djold += (double)pold; djnew += (double)pnew; jn += (double)pn;
    int nsnew;
    if (a.fixsh && !a.first) nsnew = nsold;
    else if (jlast == 0) nsnew = 0;
    else {
      int ls = a.lofj[jlast - 1];
      nsnew = (ls <= a.mm) ? ls * (ls + 1) + ls + 1 : (2 * a.mm + 1) * ls - a.mm * a.mm + a.mm + 1;
    }
    for (int j = nsnew + lane; j < a.nlm; j += 32) S[j] = 0.f;
    // next radiance truncation
    int nrnext;
    if (a.fixsh && !a.first) nrnext = max(4, nsnew);
    else {
      float r0 = a.radiance[(size_t)p * a.nlm];
      int lr = 1;
      for (int l = 1; l <= a.ml; ++l)
        if (cf[l] * r0 > a.shacc) lr = l;
      int ls = a.lofj[max(1, nsnew) - 1];
      lr = min(lr, ls + a.ml / 8 + 2);
      if (a.highorder) lr = a.ml;
      nrnext = (lr <= a.mm) ? lr * (lr + 1) + lr + 1 : (2 * a.mm + 1) * lr - a.mm * a.mm + a.mm + 1;
    }
    if (a.highorder && a.fixsh && !a.first) nrnext = a.nlm;
    __syncwarp();
    if (lane == 0) {
      a.ns[p] = nsnew;
      if (!a.first && a.accel) a.nso[p] = nsold;
      if (a.first) a.nso[p] = nsnew;
      a.nr[p] = nrnext;
    }
  }
  if (!a.first) {
    for (int o = 16; o > 0; o >>= 1) {
      djdot += __shfl_xor_sync(0xffffffffu, djdot, o);
      djold += __shfl_xor_sync(0xffffffffu, djold, o);
      djnew += __shfl_xor_sync(0xffffffffu, djnew, o);
      jn += __shfl_xor_sync(0xffffffffu, jn, o);
    }
    __shared__ double sred[4][8];
    int w = threadIdx.x >> 5;
    if (lane == 0) { sred[0][w] = djdot; sred[1][w] = djold; sred[2][w] = djnew; sred[3][w] = jn; }
    __syncthreads();
    if (threadIdx.x < 4) {
      double s = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sred[threadIdx.x][k];
      atomicAdd(&a.red[threadIdx.x], s);
    }
  }
}

// Polarized COMPUTE_SOURCE: CALC_SOURCE_PNT (src/polarized/shdomsub1.f:
// 823-909) per point, one warp per point, rows [I][Q][U] of nlm terms:
//   S_I = c1 (f0 Ysun + R_I) + cb1 R_Q,  S_Q = cb1 (R_I + f0 Ysun) + ca2 R_Q,
//   S_U = ca3 R_U  (Q and U from the term j = 4 on, that is l >= 2),
// the series-acceleration sums over all three Stokes rows, the truncation
// at the last term where any Stokes component exceeds SHACC, and the next
// radiance truncation from the I row as in the scalar kernel.
__global__ void __launch_bounds__(256) k_source_pol(SourceArgs a) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nlm = a.nlm, nl = a.nl;
  double djdot = 0, djold = 0, djnew = 0, jn = 0;
  for (int p = warp; p < a.npts; p += nwarps) {
    const float *c1 = a.coef + (size_t)p * nl, *cp = a.coefp + (size_t)p * 3 * nl;
    const float f0 = a.dirflux[p] * a.secmu0;
    const int nrp = a.nr[p], nsold = a.ns[p], nsoold = a.nso[p], nsmin = min(nsold, nsoold);
    float *S = a.source + (size_t)p * 3 * nlm;
    float *D = a.delsource + (size_t)p * 3 * nlm;
    const float *R = a.radiance + (size_t)p * 3 * nlm;
    int jlast = 0;
    float pdot = 0.f, pold = 0.f, pnew = 0.f, pn = 0.f;
    for (int j0 = 0; j0 < nlm; j0 += 32) {
      const int j = j0 + lane;
      float jt[3] = {0.f, 0.f, 0.f};
      if (j < nlm) {
        const int l = a.lofj[j];
        const float ri = j < nrp ? R[j] : 0.f, rq = j < nrp ? R[nlm + j] : 0.f, ru = j < nrp ? R[2 * nlm + j] : 0.f;
        const float ys = f0 * a.ylmsun[j], ca = c1[l], ca2 = cp[l], ca3 = cp[nl + l], cb1 = cp[2 * nl + l];
        jt[0] = ca * ys + ca * ri + cb1 * rq;
        if (j == 0 && a.thermal) jt[0] += 3.544907703f * a.thermal[p];  // unpolarized emission
        if (j >= 4) { jt[1] = cb1 * ri + ca2 * rq + cb1 * ys; jt[2] = ca3 * ru; }
        if (!a.first) {
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float sold = S[k * nlm + j];
            if (a.accel) {
              if (j < nsmin) {
                const float dn = jt[k] - sold, dd = D[k * nlm + j];
                pdot += dn * dd; pold += dd * dd; pnew += dn * dn; pn += sold * sold;
              }
              D[k * nlm + j] = j < nsold ? jt[k] - sold : 0.f;
            } else if (j < nsold) {
              const float dn = jt[k] - sold;
              pnew += dn * dn; pn += sold * sold;
            }
          }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) S[k * nlm + j] = jt[k];  // truncated below once jlast is known
      }
      const bool big = j < nlm && (fabsf(jt[0]) > a.shacc || fabsf(jt[1]) > a.shacc || fabsf(jt[2]) > a.shacc);
      const unsigned m = __ballot_sync(0xffffffffu, big);
      if (m) jlast = j0 + 32 - __clz(m);
    }
    djdot += (double)pdot; djold += (double)pold; djnew += (double)pnew; jn += (double)pn;
    int nsnew;
    if (a.fixsh && !a.first) nsnew = nsold;
    else if (jlast == 0) nsnew = 0;
    else {
      const int ls = a.lofj[jlast - 1];
      nsnew = (ls <= a.mm) ? ls * (ls + 1) + ls + 1 : (2 * a.mm + 1) * ls - a.mm * a.mm + a.mm + 1;
    }
    for (int j = nsnew + lane; j < nlm; j += 32) { S[j] = 0.f; S[nlm + j] = 0.f; S[2 * nlm + j] = 0.f; }
    int nrnext;
    if (a.fixsh && !a.first) nrnext = max(4, nsnew);
    else {
      const float r0 = R[0];
      int lr = 1;
      for (int l = 1; l <= a.ml; ++l)
        if (c1[l] * r0 > a.shacc) lr = l;
      const int ls = a.lofj[max(1, nsnew) - 1];
      lr = min(lr, ls + a.ml / 8 + 2);
      if (a.highorder) lr = a.ml;
      nrnext = (lr <= a.mm) ? lr * (lr + 1) + lr + 1 : (2 * a.mm + 1) * lr - a.mm * a.mm + a.mm + 1;
    }
    if (a.highorder && a.fixsh && !a.first) nrnext = nlm;
    __syncwarp();
    if (lane == 0) {
      a.ns[p] = nsnew;
      if (!a.first && a.accel) a.nso[p] = nsold;
      if (a.first) a.nso[p] = nsnew;
      a.nr[p] = nrnext;
    }
  }
  if (!a.first) {
    for (int o = 16; o > 0; o >>= 1) {
      djdot += __shfl_xor_sync(0xffffffffu, djdot, o);
      djold += __shfl_xor_sync(0xffffffffu, djold, o);
      djnew += __shfl_xor_sync(0xffffffffu, djnew, o);
      jn += __shfl_xor_sync(0xffffffffu, jn, o);
    }
    __shared__ double sred[4][8];
    const int w = threadIdx.x >> 5;
    if (lane == 0) { sred[0][w] = djdot; sred[1][w] = djold; sred[2][w] = djnew; sred[3][w] = jn; }
    __syncthreads();
    if (threadIdx.x < 4) {
      double t = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sred[threadIdx.x][k];
      atomicAdd(&a.red[threadIdx.x], t);
    }
  }
}

struct AccelState {
  double a;        // acceleration parameter of the last iteration
  float solcrit;
  float accelpar;
};

// CALC_ACCEL_SOLCRIT (src/shdom_nompi.f:317-348).
__global__ void k_accel_param(const double *red, AccelState *st, int doaccel) {
  double djdot = red[0], djold = red[1], djnew = red[2], jn = red[3];
  double a;
  if (doaccel && st->a == 0.0 && djnew < djold) {
    double r = sqrt(djnew / djold);
    double theta = acos(djdot / sqrt(djold * djnew));
    a = (1 - r * cos(theta) + pow(r, 1 + 0.5 * 3.14159 / theta)) / (1 + r * r - 2 * r * cos(theta)) - 1.0;
    a = fmin(10.0, fmax(0.0, a));
    if (!(a == a)) a = 0.0;
  } else {
    a = 0.0;
  }
  st->a = a;
  st->accelpar = (float)a;
  if (jn > 0) st->solcrit = (float)sqrt(djnew / jn);
  else if (djnew == 0) st->solcrit = 0.f;
}

// ACCELERATE_SOLUTION (src/polarized/shdomsub1.f:1807-1831).
// rows of nst * nlm values per point (Stokes rows of nlm terms)
__global__ void k_accelerate(float *source, const float *delsource, const int *ns, const int *nso, int npts, int nlm,
                             const AccelState *st, int nst) {
  float a = st->accelpar;
  if (!(a > 0.f)) return;
  const int row = nst * nlm;
  size_t total = (size_t)npts * row;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    int p = (int)(t / row), j = (int)(t - (size_t)p * row) % nlm;
    if (j < min(ns[p], nso[p])) source[t] += a * delsource[t];
  }
}

// Eddington initial radiance: 4 I terms per point, Q and U zero (INIT_RADIANCE).
__global__ void k_init_radiance(const float *rad0, float *radiance, int *nr, int npts, int nlm, int nst) {
  const int row = nst * nlm;
  size_t total = (size_t)npts * row;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    int p = (int)(t / row), j = (int)(t - (size_t)p * row);
    radiance[t] = j < 4 ? rad0[(size_t)p * 4 + j] : 0.f;
    if (j == 0) nr[p] = 4;
  }
}

// ---------------------------------------------------------------- render
struct RenderArgs {
  const float *gridpos, *xgrid, *ygrid, *zgrid;
  const int *gridptr, *neighptr, *cellflags;
  const float *text, *source, *coef, *dirflux;
  const int *ns, *lofj;
  const int *tms_ptr, *tms_iph;
  const float *tms_w, *phasetab, *ylmsun;
  const int *botp;
  const float *bcrad_bot;
  const int *bot_index;  // point -> bottom list index or -1
  const float *coefp, *phasetab2;  // polarized: a2/a3/b1 coefficients, I-Q single-scatter table
  // bidirectional surface (brdf != 0): parameters at the bottom points, the
  // downward ordinates of the reflection sum and the ordinate radiances of
  // the last sweep (the downwelling radiances at the surface)
  int brdf, nsfcpar, nbrdf_dn, ldo;
  const float *botpar, *raddo;
  const float *botplanck;  // thermal source: B at the bottom points, else null
  const BrdfOrd *brdf_dn;
  const float *camx, *camy, *camz;
  const double *cammu, *camphi;
  float *out;
  int *err;
  int nrays, nx, ny, nz, nlm, nl, ml, mm, bcflag, ipflag, numphase, nscatangle, deltam;
  // RENDER's SINGLESCATTER (the source is the exact single scatter of the
  // direct beam only) and NOSURFACE (no boundary radiance is added)
  int single_scatter = 0, nosurface = 0;
  float solarmu, solaraz, secmu0, skyrad;
  double tautol, transcut;
};

// Reflected radiance of bottom point bi toward (mu2, phi2) (the BRDF branch
// of FIND_BOUNDARY_RADIANCE, src/polarized/shdomsub2.f:2748-2863): the
// warp sums the downward ordinates; every lane gets the Stokes vector.
__device__ __noinline__ void brdf_radiance_warp(const RenderArgs &a, int bi, float mu2, float phi2, int lane, int nst, float out[3]) {
  const float *par = a.botpar + (size_t)bi * a.nsfcpar;
  const int p = a.botp[bi];
  const float *row = a.raddo + (size_t)p * a.ldo;
  float acc[3] = {0.f, 0.f, 0.f}, R[3][3];
  if (lane == 0) {
    surface_brdf_d(a.brdf, par, mu2, phi2, a.solarmu, a.solaraz, R);
    for (int k = 0; k < nst; ++k) acc[k] = 0.318309886f * R[k][0] * a.dirflux[p];
  }
  for (int d = lane; d < a.nbrdf_dn; d += 32) {
    const BrdfOrd i = a.brdf_dn[d];
    surface_brdf_d(a.brdf, par, mu2, phi2, i.mu, i.phi, R);
    const int ci = (int)i.col, oi = (int)i.off;
    for (int k1 = 0; k1 < nst; ++k1) {
      const float rin = row[ci + k1 * oi];
      for (int k = 0; k < nst; ++k) acc[k] += i.w * R[k][k1] * rin;
    }
    if (a.botplanck) {
      const float bp = a.botplanck[bi];
      acc[0] += i.w * (1.f - R[0][0]) * bp;
      for (int k = 1; k < nst; ++k) acc[k] -= i.w * R[k][0] * bp;
    }
  }
  for (int k = 0; k < 3; ++k) {
    float v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    out[k] = v;
  }
}

__device__ int locate_cell(const RenderArgs &a, double &x0, double &y0, double z0) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  if (!(a.bcflag & 1)) {
    double xd = a.xgrid[nx] - a.xgrid[0];
    if (x0 < a.xgrid[0]) x0 = x0 - xd * ((int)((x0 - a.xgrid[0]) / xd) - 1);
    else if (x0 > a.xgrid[nx]) x0 = x0 - xd * (int)((x0 - a.xgrid[0]) / xd);
  }
  if (!(a.bcflag & 2)) {
    double yd = a.ygrid[ny] - a.ygrid[0];
    if (y0 < a.ygrid[0]) y0 = y0 - yd * ((int)((y0 - a.ygrid[0]) / yd) - 1);
    else if (y0 > a.ygrid[ny]) y0 = y0 - yd * (int)((y0 - a.ygrid[0]) / yd);
  }
  int il = 0, iu, ix, iy, iz;
  if (a.ipflag & 1) {
    iu = nx;
    while (iu - il > 1) { int im = (iu + il) / 2; if (x0 >= 0.5 * (a.xgrid[im - 1] + a.xgrid[im])) il = im; else iu = im; }
    il += 1;
  } else {
    iu = nx + 1;
    while (iu - il > 1) { int im = (iu + il) / 2; if (x0 >= a.xgrid[im - 1]) il = im; else iu = im; }
  }
  ix = max(il, 1);
  il = 0;
  if (a.ipflag & 2) {
    iu = ny;
    while (iu - il > 1) { int im = (iu + il) / 2; if (y0 >= 0.5 * (a.ygrid[im - 1] + a.ygrid[im])) il = im; else iu = im; }
    il += 1;
  } else {
    iu = ny + 1;
    while (iu - il > 1) { int im = (iu + il) / 2; if (y0 >= a.ygrid[im - 1]) il = im; else iu = im; }
  }
  iy = max(il, 1);
  il = 0; iu = nz;
  while (iu - il > 1) { int im = (iu + il) / 2; if (z0 >= a.zgrid[im - 1]) il = im; else iu = im; }
  iz = max(il, 1);
  int nyc = ny;
  if (a.bcflag & 1) { if (x0 < a.xgrid[0]) ix = 1; else if (x0 > a.xgrid[nx - 1]) ix = nx + 1; else ix = ix + 1; }
  if (a.bcflag & 2) { nyc = ny + 1; if (y0 < a.ygrid[0]) iy = 1; else if (y0 > a.ygrid[ny - 1]) iy = ny + 1; else iy = iy + 1; }
  return (iz - 1) + (nz - 1) * (iy - 1) + (nz - 1) * nyc * (ix - 1);
}

constexpr int RWARPS = 4;     // rays (warps) per block
constexpr int RNLM = 1024;    // max spherical-harmonic terms for the per-ray tables

// One warp per ray (RENDER / INTEGRATE_1RAY / COMPUTE_SOURCE_1CELL_UNPOL /
// FIND_BOUNDARY_RADIANCE, src/polarized/shdomsub4.f:93-286,
// src/polarized/shdomsub2.f:2311-2863, :3046-3192).  The spherical-harmonic
// dot products of the new cell corners are split over groups of four lanes;
// the path integration is evaluated uniformly by all lanes.
// Real spherical harmonics Y_lm of one direction (mu, phi) into y[NLM] (the
// j(l, m) term order of the solver), lane m of the warp running the upward
// l recurrence of the normalised Wigner d^l_{m0}(mu) for its m.  FP32: the
// values are stored as FP32 and dotted with FP32 coefficients.
__device__ __forceinline__ void ylm_dir_warp(float *y, float x, float phf, int ml, int mm, int lane) {
  const float fct = 0.3989422804014327f;  // 1/sqrt(2 pi)
  for (int m = lane; m <= mm; m += 32) {
    float c = 1.f, s = 0.f;
    if (m > 0) sincosf(m * phf, &s, &c);
    float dprev = 0.f, dcur;
    if (m == 0) dcur = 1.f;
    else {
      float cc = 1.f;
      for (int k = 1; k <= m; ++k) cc *= sqrtf((float)(m + k) / (float)k);
      dcur = ((m & 1) ? -cc : cc) * powf(0.5f * sqrtf((1.f - x) * (1.f + x)), (float)m);
    }
    for (int l = m; l <= ml; ++l) {
      const float v = fct * dcur * sqrtf(l + 0.5f);
      const int j = (l <= mm) ? l * (l + 1) + m : (2 * mm + 1) * l - mm * mm + m;
      y[j] = (c - s) * v;
      y[j - 2 * m] = (c + s) * v;
      float dn;
      if (m == 0) dn = ((2 * l + 1) * x * dcur - l * dprev) / (l + 1);
      else dn = ((2 * l + 1) * x * dcur - (l > m ? sqrtf((float)(l * l - m * m)) * dprev : 0.f)) /
                sqrtf((float)((l + 1) * (l + 1) - m * m));
      dprev = dcur;
      dcur = dn;
    }
  }
}

// The ray's direction for the cell walk, in FP32: direction cosines,
// their inverses (1e6 where a cosine is below 1e-6 and set to zero, as the
// reference's INTEGRATE_1RAY) and the octant bits.
struct RayDir {
  float c[3], ci[3];
  int bit[3], ioct;
};
__device__ __forceinline__ RayDir ray_dir(double mu2, double phi2) {
  const double pi = 3.141592653589793;
  const double st = sqrt(1.0 - mu2 * mu2);
  double c[3] = {st * cos(phi2 - pi), st * sin(phi2 - pi), -mu2};
  RayDir r;
  for (int k = 0; k < 3; ++k) {
    double ci;
    if (fabs(c[k]) > 1e-6) ci = 1.0 / c[k]; else { c[k] = 0.0; ci = 1e6; }
    r.c[k] = (float)c[k]; r.ci[k] = (float)ci; r.bit[k] = c[k] < 0;
  }
  r.ioct = r.bit[0] + 2 * r.bit[1] + 4 * r.bit[2];
  return r;
}

template <bool BRDF>
__global__ void __launch_bounds__(RWARPS * 32) k_render(RenderArgs a) {
  __shared__ float ydir[RWARPS][RNLM];
  __shared__ float tl[RWARPS][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ray = blockIdx.x * RWARPS + w;
  if (ray >= a.nrays) return;
  const double pi = 3.141592653589793;
  double x0 = a.camx[ray], y0 = a.camy[ray], z0 = a.camz[ray], mu2 = a.cammu[ray], phi2 = a.camphi[ray];
  const double muray = -mu2, phiray = phi2 - pi;
  const float ztop = a.zgrid[a.nz - 1];
  if (z0 > ztop) {
    if (muray >= 0.0) { if (lane == 0) a.out[ray] = 0.f; return; }
    double r = (ztop - z0) / muray;
    x0 += r * sqrt(1 - muray * muray) * cos(phiray);
    y0 += r * sqrt(1 - muray * muray) * sin(phiray);
    z0 = ztop;
  } else if (z0 < a.zgrid[0]) {
    if (lane == 0) { atomicCAS(a.err, ERR_NONE, ERR_RAY_BELOW); a.out[ray] = 0.f; }
    return;
  }
  // Y_lm in the ray direction: lane m runs the l recurrence of its m
  ylm_dir_warp(ydir[w], (float)mu2, (float)phi2, a.ml, a.mm, lane);
  __syncwarp();
  // t_l = sum_m Ydir(l,m) Ysun(l,m)
  for (int l = lane; l <= a.ml; l += 32) {
    int me = min(l, a.mm), j0 = (l <= a.mm) ? l * l : (2 * a.mm + 1) * l - a.mm * a.mm - a.mm;
    float s = 0.f;
    for (int k = 0; k < 2 * me + 1; ++k) s += ydir[w][j0 + k] * a.ylmsun[j0 + k];
    tl[w][l] = s;
  }
  __syncwarp();
  // single-scatter phase table interpolation parameters
  int sj = 0;
  float sf = 0.f;
  if (a.deltam) {
    double cosscat = (double)a.solarmu * mu2 + sqrt((1.0 - (double)a.solarmu * a.solarmu) * (1.0 - mu2 * mu2)) * cos((double)a.solaraz - phi2);
    cosscat = fmax(fmin(1.0, cosscat), -1.0);
    float F = (float)((a.nscatangle - 1) * (acos(cosscat) / pi) + 1);
    int J = min(a.nscatangle - 1, (int)F);
    sf = F - J; sj = J - 1;
  }
  RayDir rd = ray_dir(mu2, phi2);
  const int ioct0 = rd.ioct;
  const float xm = 0.5f * (a.xgrid[0] + a.xgrid[a.nx - 1]), ym = 0.5f * (a.ygrid[0] + a.ygrid[a.ny - 1]);
  double xe = x0, ye = y0, ze = z0;
  int cell = locate_cell(a, xe, ye, ze);
  // the position as the cell's low corner (grid coordinates) plus an FP32 offset
  float lx, ly, lz;
  if (cell >= 0) {
    const float *P = a.gridpos + 3 * a.gridptr[8 * (size_t)cell];
    lx = (float)(xe - P[0]); ly = (float)(ye - P[1]); lz = (float)(ze - P[2]);
  }
  const float eps = 1.0e-5f * (a.gridpos[3 * a.gridptr[7] + 2] - a.gridpos[3 * a.gridptr[0] + 2]);
  const int maxcross = 500 * max(a.nx, max(a.ny, a.nz));
  int oldp[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  float osrc[8] = {0};
  float ext8[8], src8[8];
  double radacc = 0.0, transmit = 1.0;
  const float inv_tautol = 1.0f / a.tautol;
  int ngrid = 0;
  bool validrad = false;
  const int grp = lane >> 2, gl = lane & 3;  // 8 groups of 4 lanes, one corner per group
  while (!validrad && cell >= 0) {
    ++ngrid;
    const int *g = a.gridptr + 8 * (size_t)cell;
    int mypt = g[grp];
    // reuse corners already evaluated for the previous cell
    int reuse = -1;
#pragma unroll
    for (int k = 0; k < 8; ++k) if (oldp[k] == mypt) reuse = k;
    float cval = 0.f, cext = a.text[mypt];
    const bool need = reuse < 0;
    const int ns = (need && !a.single_scatter) ? a.ns[mypt] : 0;
    float s = 0.f;
    {
      const float *S = a.source + (size_t)mypt * a.nlm;
      for (int j = gl; j < ns; j += 4) s += S[j] * ydir[w][j];
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (!need) {
      cval = osrc[reuse];
    } else {
      if (a.deltam) {
        const float da = a.dirflux[mypt] * a.secmu0;
        const float *cf = a.coef + (size_t)mypt * a.nl;
        if (ns > 0) {
          int ls = a.lofj[ns - 1];
          float sub = 0.f;
          for (int l = 0; l <= ls; ++l) sub += cf[l] * tl[w][l];
          s -= da * sub;
        }
        float add = 0.f;
        for (int q = a.tms_ptr[mypt]; q < a.tms_ptr[mypt + 1]; ++q) {
          int iph = a.tms_iph[q];
          float ss = (1.f - sf) * a.phasetab[(size_t)sj * a.numphase + iph] + sf * a.phasetab[(size_t)(sj + 1) * a.numphase + iph];
          add += a.tms_w[q] * ss;
        }
        s += da * add;
      }
      cval = s * cext;
    }
    // gather the 8 corners from the groups
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      src8[k] = __shfl_sync(0xffffffffu, cval, 4 * k);
      ext8[k] = __shfl_sync(0xffffffffu, cext, 4 * k);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) { oldp[k] = g[k]; osrc[k] = src8[k]; }
    const int ip1 = g[0], ip2 = g[7];
    const float *P1 = a.gridpos + 3 * ip1, *P2 = a.gridpos + 3 * ip2;
    const float delx = P2[0] - P1[0], dely = P2[1] - P1[1], delz = P2[2] - P1[2];
    const float idx = delx <= 0.f ? 1.f : 1.f / delx, idy = dely <= 0.f ? 1.f : 1.f / dely, idz = 1.f / delz;
    // The geometry of the step runs in FP32 on cell-relative offsets (an
    // offset from the cell's own corner keeps FP32's relative precision on
    // the cell size); only the two ray accumulators stay FP64.  The
    // trilinear weights are cell-relative coordinates in [0, 1].
    auto tri = [&](const float *v, float u, float vv, float ww) {
      const float a0 = fmaf(u, v[1] - v[0], v[0]), a1 = fmaf(u, v[3] - v[2], v[2]);
      const float a2 = fmaf(u, v[5] - v[4], v[4]), a3 = fmaf(u, v[7] - v[6], v[6]);
      const float b0 = fmaf(vv, a1 - a0, a0), b1 = fmaf(vv, a3 - a2, a2);
      return fmaf(ww, b1 - b0, b0);
    };
    const float u0 = lx * idx, v0 = ly * idy, w0 = lz * idz;
    float srcext1 = fmaxf(0.f, tri(src8, u0, v0, w0));
    float ext1 = tri(ext8, u0, v0, w0);
    const int cf = a.cellflags[cell];
    const float cx = rd.c[0], cy = rd.c[1], cz = rd.c[2];
    bool ipinx = (cf & 1) && !((a.bcflag & 1) && ((cx > 0 && P1[0] + lx < xm) || (cx < 0 && P1[0] + lx > xm)));
    bool ipiny = (cf & 2) && !((a.bcflag & 2) && ((cy > 0 && P1[1] + ly < ym) || (cy < 0 && P1[1] + ly > ym)));
    const float *Po = a.gridpos + 3 * g[7 - ioct0];
    const float sox = ipinx ? 1e20f : ((Po[0] - P1[0]) - lx) * rd.ci[0];
    const float soy = ipiny ? 1e20f : ((Po[1] - P1[1]) - ly) * rd.ci[1];
    const float soz = ((Po[2] - P1[2]) - lz) * rd.ci[2];
    const float so = fminf(sox, fminf(soy, soz));
    if (so < -eps) { if (lane == 0) atomicCAS(a.err, ERR_NONE, ERR_RAY_SO); break; }
    const float lxn = fmaf(so, cx, lx), lyn = fmaf(so, cy, ly), lzn = fmaf(so, cz, lz);
    // per unit path length, the cell-relative coordinates move by (du, dv, dw)
    const float du = cx * idx, dv = cy * idy, dw = cz * idz;
    const float sof = so;
    float extn = tri(ext8, fmaf(sof, du, u0), fmaf(sof, dv, v0), fmaf(sof, dw, w0));
    const float taugrid = so * 0.5f * (ext1 + extn);
    int ntau = max(1, 1 + (int)(taugrid * inv_tautol));
    const float delsf = sof / (float)ntau;
    // the cell's source integral and transmission from its entry, in FP32;
    // folded into the FP64 ray accumulators once per cell
    float cacc = 0.f, ctr = 1.f;
    for (int it = 1; it <= ntau; ++it) {
      const float sf_ = it * delsf;
      const float uu_ = fmaf(sf_, du, u0), vv_ = fmaf(sf_, dv, v0), ww_ = fmaf(sf_, dw, w0);
      float ext0 = tri(ext8, uu_, vv_, ww_);
      float srcext0 = fmaxf(0.f, tri(src8, uu_, vv_, ww_));
      float ext = 0.5f * (ext0 + ext1);
      float absc, trc, src;
      if (ext != 0.f) {
        float tau = ext * delsf;
        absc = tau * (1.f - 0.5f * tau * (1.f - 0.33333333333f * tau));
        trc = 1.f - absc;
        src = (0.5f * (srcext0 + srcext1) + 0.08333333333f * (ext0 * srcext1 - ext1 * srcext0) * delsf *
                                                (1.f - 0.05f * (ext1 - ext0) * delsf)) / ext;
      } else { absc = 0.f; trc = 1.f; src = 0.f; }
      cacc = fmaf(ctr * src, absc, cacc);
      ctr *= trc;
      ext1 = ext0; srcext1 = srcext0;
    }
    radacc += transmit * (double)cacc;
    transmit *= (double)ctr;
    int iface, jface;
    bool openbc;
    if (sox <= soz && sox <= soy) { iface = 1 - rd.bit[0]; jface = 0; openbc = (cf & 1) && (a.bcflag & 1); }
    else if (soy <= soz) { iface = 3 - rd.bit[1]; jface = 1; openbc = (cf & 2) && (a.bcflag & 2); }
    else { iface = 5 - rd.bit[2]; jface = 2; openbc = false; }
    int nxt = a.neighptr[6 * (size_t)cell + iface];
    int kface = iface, kc = cell;
    if (openbc) { kface = iface ^ 1; kc = nxt; iface = -1; }
    if (transmit < a.transcut || ngrid > maxcross) {
      validrad = true;
    } else if (nxt < 0 && iface >= 4) {
      validrad = true;
      const int *gk = a.gridptr + 8 * (size_t)kc;
      float xs[4], ys[4], rb[4];
      for (int k = 0; k < 4; ++k) {
        int q = gk[c_face[kface][k]];
        xs[k] = a.gridpos[3 * q]; ys[k] = a.gridpos[3 * q + 1];
        if ((float)mu2 < 0.f) rb[k] = a.skyrad;
        else {
          int bi = a.bot_index[q];
          rb[k] = bi >= 0 ? a.bcrad_bot[bi] : 0.f;
          if constexpr (BRDF) {
            if (bi >= 0) {
              float o[3];
              brdf_radiance_warp(a, bi, (float)mu2, (float)phi2, lane, 1, o);
              rb[k] = o[0];
            }
          }
        }
      }
      float uu = (xs[1] - xs[0] > 0) ? ((P1[0] - xs[0]) + lxn) / (xs[1] - xs[0]) : 0.f;
      float vv = (ys[2] - ys[0] > 0) ? ((P1[1] - ys[0]) + lyn) / (ys[2] - ys[0]) : 0.f;
      if (!a.nosurface)
        radacc += transmit * ((1 - uu) * (1 - vv) * rb[0] + uu * (1 - vv) * rb[1] + (1 - uu) * vv * rb[2] + uu * vv * rb[3]);
    } else {
      // into the next cell: offsets from its corner, the crossed face's
      // coordinate taken from the grid
      const float *Pn = a.gridpos + 3 * a.gridptr[8 * (size_t)nxt];
      const float *q = a.gridpos + 3 * a.gridptr[8 * (size_t)nxt + ioct0];
      lx = jface == 0 ? q[0] - Pn[0] : (P1[0] - Pn[0]) + lxn;
      ly = jface == 1 ? q[1] - Pn[1] : (P1[1] - Pn[1]) + lyn;
      lz = jface == 2 ? q[2] - Pn[2] : (P1[2] - Pn[2]) + lzn;
      cell = nxt;
    }
  }
  if (lane == 0) a.out[ray] = (float)radacc;
}

// Wigner d^n_{m m1}(x) at n = max(m, m1), m, m1 >= 0 (double precision).
__device__ __forceinline__ double wig_start_d(double x, int m, int m1) {
  if (m == m1) return pow(0.5 * (1.0 + x), (double)m);
  const int hi = max(m, m1), lo = min(m, m1);
  double c = (m1 > m || ((m - m1) % 2 == 0)) ? 1.0 : -1.0;
  for (int q = 1; q <= hi - lo; ++q) c *= sqrt((double)(m + m1 + q) / q);
  return c * pow(sqrt(0.5 * (1.0 - x)), (double)(hi - lo)) * pow(sqrt(0.5 * (1.0 + x)), (double)(hi + lo));
}

// The five generalized spherical functions a polarized ray needs (YLMALL,
// src/polarized/shdomsub2.f:4244-4354, elements 1 I-I, 2 Q-Q, 3 U-U, 5 I-Q,
// 6 Q-U) at one direction: y[e * nlm + j], e = 0..4.  Lane m runs the upward
// recurrences in l of d^l_{m0}(x), d^l_{m2}(x) and d^l_{m2}(-x) in double
// precision.
__device__ void ylm6_dir_warp(float *y, int nlm, double x, double phi, int ml, int mm, int lane) {
  const double fct = 0.3989422804014327;  // 1/sqrt(2 pi)
  for (int m = lane; m <= mm; m += 32) {
    double c = 1.0, sn = 0.0;
    if (m > 0) sincos(m * phi, &sn, &c);
    // d^l_{m0}
    double a0p = 0.0, a0 = (m == 0) ? 1.0 : 0.0;
    if (m > 0) {
      double cc = 1.0;
      for (int k = 1; k <= m; ++k) cc *= sqrt((double)(m + k) / (double)k);
      a0 = ((m & 1) ? -cc : cc) * pow(0.5 * sqrt((1.0 - x) * (1.0 + x)), (double)m);
    }
    // d^l_{m2}(x) and d^l_{m2}(-x), from l = max(m, 2)
    const int n2 = max(m, 2);
    double bp = 0.0, bpp = 0.0, bm = 0.0, bmp = 0.0;
    for (int l = m; l <= ml; ++l) {
      if (l == n2) { bp = wig_start_d(x, m, 2); bm = wig_start_d(-x, m, 2); bpp = 0.0; bmp = 0.0; }
      const double nrm = sqrt(l + 0.5);
      const double dp = (l >= n2) ? bp * nrm : 0.0, dm = (l >= n2) ? (((l + m) & 1) ? -bm : bm) * nrm : 0.0;
      const double p1 = fct * a0 * nrm, p2 = -0.5 * fct * (dp + dm), p3 = -0.5 * fct * (dp - dm);
      const int j = (l <= mm) ? l * (l + 1) + m : (2 * mm + 1) * l - mm * mm + m;
      y[j] = (float)(p1 * (c - sn));
      y[nlm + j] = (float)(p2 * (c - sn));
      y[2 * nlm + j] = (float)(p2 * (c + sn));
      y[3 * nlm + j] = (float)(p3 * (c - sn));
      y[4 * nlm + j] = (float)(p3 * (c + sn));
      if (m > 0) {
        const int jn = j - 2 * m;
        y[jn] = (float)(p1 * (sn + c));
        y[nlm + jn] = (float)(p2 * (sn + c));
        y[2 * nlm + jn] = (float)(p2 * (sn - c));
        y[3 * nlm + jn] = (float)(p3 * (sn + c));
        y[4 * nlm + jn] = (float)(p3 * (sn - c));
      }
      // next degree
      double an;
      if (m == 0) an = ((2 * l + 1) * x * a0 - l * a0p) / (l + 1);
      else an = ((2 * l + 1) * x * a0 - (l > m ? sqrt((double)(l * l - m * m)) * a0p : 0.0)) / sqrt((double)((l + 1) * (l + 1) - m * m));
      a0p = a0; a0 = an;
      if (l >= n2) {
        const double q = sqrt((double)((l + 1) * (l + 1) - m * m)) * sqrt((double)((l + 1) * (l + 1) - 4));
        const double r = sqrt((double)(l * l - m * m)) * sqrt((double)(l * l - 4));
        const double f1 = (2.0 * l + 1.0) / l / q, f2 = r * (l + 1.0) / l / q;
        const double np_ = (l * (l + 1.0) * x - 2.0 * m) * f1 * bp - f2 * (l > n2 ? bpp : 0.0);
        const double nm_ = (-l * (l + 1.0) * x - 2.0 * m) * f1 * bm - f2 * (l > n2 ? bmp : 0.0);
        bpp = bp; bp = np_; bmp = bm; bm = nm_;
      }
    }
  }
}

// Polarized ray integration (INTEGRATE_1RAY with the polarized
// COMPUTE_SOURCE_1CELL, src/polarized/shdomsub2.f:2311-2863, :2868-3042,
// and ROTATE_POL_PLANE :3277-3316): as k_render, with the I, Q, U sources
// of each corner and a Stokes vector along the ray.  Dynamic shared memory:
// the five generalized functions (5 nlm floats) per warp.  out[ray][3].
template <bool BRDF>
__global__ void __launch_bounds__(RWARPS * 32) k_render_pol(RenderArgs a) {
  extern __shared__ float rsm[];
  __shared__ float tl[RWARPS][3][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ray = blockIdx.x * RWARPS + w;
  if (ray >= a.nrays) return;
  const int nlm = a.nlm;
  float *Y = rsm + (size_t)w * 5 * nlm;
  const double pi = 3.141592653589793;
  double x0 = a.camx[ray], y0 = a.camy[ray], z0 = a.camz[ray], mu2 = a.cammu[ray], phi2 = a.camphi[ray];
  const double muray = -mu2, phiray = phi2 - pi;
  const float ztop = a.zgrid[a.nz - 1];
  if (z0 > ztop) {
    if (muray >= 0.0) { if (lane < 3) a.out[(size_t)ray * 3 + lane] = 0.f; return; }
    double r = (ztop - z0) / muray;
    x0 += r * sqrt(1 - muray * muray) * cos(phiray);
    y0 += r * sqrt(1 - muray * muray) * sin(phiray);
    z0 = ztop;
  } else if (z0 < a.zgrid[0]) {
    if (lane == 0) atomicCAS(a.err, ERR_NONE, ERR_RAY_BELOW);
    if (lane < 3) a.out[(size_t)ray * 3 + lane] = 0.f;
    return;
  }
  ylm6_dir_warp(Y, nlm, (double)(float)mu2, (double)(float)phi2, a.ml, a.mm, lane);
  __syncwarp();
  // TMS subtraction series: t_k(l) = sum_m Y_k(l, m) Ysun(l, m) for k = I-I, Q-Q, Q-U
  for (int l = lane; l <= a.ml; l += 32) {
    const int me = min(l, a.mm), j0 = (l <= a.mm) ? l * l : (2 * a.mm + 1) * l - a.mm * a.mm - a.mm;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    for (int k = 0; k < 2 * me + 1; ++k) {
      const float ys = a.ylmsun[j0 + k];
      s0 += Y[j0 + k] * ys; s1 += Y[nlm + j0 + k] * ys; s2 += Y[4 * nlm + j0 + k] * ys;
    }
    tl[w][0][l] = s0; tl[w][1][l] = s1; tl[w][2][l] = s2;
  }
  __syncwarp();
  int sj = 0;
  float sf = 0.f, cos22 = 1.f, sin22 = 0.f;
  if (a.deltam) {
    double cosscat = (double)a.solarmu * mu2 + sqrt((1.0 - (double)a.solarmu * a.solarmu) * (1.0 - mu2 * mu2)) * cos((double)a.solaraz - phi2);
    cosscat = fmax(fmin(1.0, cosscat), -1.0);
    float F = (float)((a.nscatangle - 1) * (acos(cosscat) / pi) + 1);
    int J = min(a.nscatangle - 1, (int)F);
    sf = F - J; sj = J - 1;
    // rotation of the single-scatter polarization to the outgoing meridional plane
    const float smu = a.solarmu, mu2f = (float)mu2, dphi = a.solaraz - (float)phi2;
    const double sin_scat = sqrt(fmax(0.0, 1.0 - cosscat * cosscat));
    const double st1 = sqrt(1.0 - (double)(smu * smu)), st2 = sqrt(1.0 - (double)(mu2f * mu2f));
    double sp, cp;
    sincos((double)dphi, &sp, &cp);
    double sin2, cos2;
    if (sin_scat == 0.0) { sin2 = 0.0; cos2 = -1.0; }
    else { sin2 = st1 * sp / sin_scat; cos2 = (st2 * smu - st1 * mu2f * cp) / sin_scat; }
    cos22 = (float)(1.0 - 2.0 * sin2 * sin2);
    sin22 = (float)(2.0 * sin2 * cos2);
  }
  RayDir rd = ray_dir(mu2, phi2);
  const int ioct0 = rd.ioct;
  const float xm = 0.5f * (a.xgrid[0] + a.xgrid[a.nx - 1]), ym = 0.5f * (a.ygrid[0] + a.ygrid[a.ny - 1]);
  double xe = x0, ye = y0, ze = z0;
  int cell = locate_cell(a, xe, ye, ze);
  // the position as the cell's low corner (grid coordinates) plus an FP32 offset (as k_render)
  float lx, ly, lz;
  if (cell >= 0) {
    const float *P = a.gridpos + 3 * a.gridptr[8 * (size_t)cell];
    lx = (float)(xe - P[0]); ly = (float)(ye - P[1]); lz = (float)(ze - P[2]);
  }
  const float eps = 1.0e-5f * (a.gridpos[3 * a.gridptr[7] + 2] - a.gridpos[3 * a.gridptr[0] + 2]);
  const int maxcross = 500 * max(a.nx, max(a.ny, a.nz));
  int oldp[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  float osrc[3][8] = {{0}};
  float ext8[8], src8[3][8];
  double radacc[3] = {0.0, 0.0, 0.0}, transmit = 1.0;
  const float inv_tautol = 1.0f / a.tautol;
  const int nl = a.nl;
  int ngrid = 0;
  bool validrad = false;
  const int grp = lane >> 2, gl = lane & 3;
  while (!validrad && cell >= 0) {
    ++ngrid;
    const int *g = a.gridptr + 8 * (size_t)cell;
    const int mypt = g[grp];
    int reuse = -1;
#pragma unroll
    for (int k = 0; k < 8; ++k) if (oldp[k] == mypt) reuse = k;
    const float cext = a.text[mypt];
    const bool need = reuse < 0;
    const int ns = (need && !a.single_scatter) ? a.ns[mypt] : 0;
    float sI = 0.f, sQ = 0.f, sU = 0.f;
    {
      const float *S = a.source + (size_t)mypt * 3 * nlm;
      for (int j = gl; j < ns; j += 4) {
        const float si = S[j], sq = S[nlm + j], su = S[2 * nlm + j];
        sI += si * Y[j];
        sQ += sq * Y[nlm + j] + su * Y[3 * nlm + j];
        sU += sq * Y[4 * nlm + j] + su * Y[2 * nlm + j];
      }
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      sI += __shfl_xor_sync(0xffffffffu, sI, o);
      sQ += __shfl_xor_sync(0xffffffffu, sQ, o);
      sU += __shfl_xor_sync(0xffffffffu, sU, o);
    }
    float cv[3];
    if (!need) {
      cv[0] = osrc[0][reuse]; cv[1] = osrc[1][reuse]; cv[2] = osrc[2][reuse];
    } else {
      if (a.deltam) {
        const float da = a.dirflux[mypt] * a.secmu0;
        const float *c1 = a.coef + (size_t)mypt * nl, *cb1 = a.coefp + ((size_t)mypt * 3 + 2) * nl;
        if (ns > 0) {
          const int ls = a.lofj[ns - 1];
          float s0 = 0.f, s1 = 0.f, s2 = 0.f;
          for (int l = 0; l <= ls; ++l) { s0 += c1[l] * tl[w][0][l]; s1 += cb1[l] * tl[w][1][l]; s2 += cb1[l] * tl[w][2][l]; }
          sI -= da * s0; sQ -= da * s1; sU -= da * s2;
        }
        float add0 = 0.f, add1 = 0.f;
        for (int q = a.tms_ptr[mypt]; q < a.tms_ptr[mypt + 1]; ++q) {
          const int iph = a.tms_iph[q];
          const size_t o0 = (size_t)sj * a.numphase + iph, o1 = (size_t)(sj + 1) * a.numphase + iph;
          add0 += a.tms_w[q] * ((1.f - sf) * a.phasetab[o0] + sf * a.phasetab[o1]);
          add1 += a.tms_w[q] * ((1.f - sf) * a.phasetab2[o0] + sf * a.phasetab2[o1]);
        }
        sI += da * add0; sQ += da * add1 * cos22; sU += da * add1 * sin22;
      }
      cv[0] = sI * cext; cv[1] = sQ * cext; cv[2] = sU * cext;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      ext8[k] = __shfl_sync(0xffffffffu, cext, 4 * k);
#pragma unroll
      for (int c = 0; c < 3; ++c) src8[c][k] = __shfl_sync(0xffffffffu, cv[c], 4 * k);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) { oldp[k] = g[k]; osrc[0][k] = src8[0][k]; osrc[1][k] = src8[1][k]; osrc[2][k] = src8[2][k]; }
    const int ip1 = g[0], ip2 = g[7];
    const float *P1 = a.gridpos + 3 * ip1, *P2 = a.gridpos + 3 * ip2;
    const float delx = P2[0] - P1[0], dely = P2[1] - P1[1], delz = P2[2] - P1[2];
    const float idx = delx <= 0.f ? 1.f : 1.f / delx, idy = dely <= 0.f ? 1.f : 1.f / dely, idz = 1.f / delz;
    auto tri = [&](const float *v, float u, float vv, float ww) {
      const float a0 = fmaf(u, v[1] - v[0], v[0]), a1 = fmaf(u, v[3] - v[2], v[2]);
      const float a2 = fmaf(u, v[5] - v[4], v[4]), a3 = fmaf(u, v[7] - v[6], v[6]);
      const float b0 = fmaf(vv, a1 - a0, a0), b1 = fmaf(vv, a3 - a2, a2);
      return fmaf(ww, b1 - b0, b0);
    };
    const float u0 = lx * idx, v0 = ly * idy, w0 = lz * idz;
    float srcext1[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) srcext1[c] = tri(src8[c], u0, v0, w0);
    srcext1[0] = fmaxf(0.f, srcext1[0]);
    float ext1 = tri(ext8, u0, v0, w0);
    const int cf = a.cellflags[cell];
    const float cx = rd.c[0], cy = rd.c[1], cz = rd.c[2];
    bool ipinx = (cf & 1) && !((a.bcflag & 1) && ((cx > 0 && P1[0] + lx < xm) || (cx < 0 && P1[0] + lx > xm)));
    bool ipiny = (cf & 2) && !((a.bcflag & 2) && ((cy > 0 && P1[1] + ly < ym) || (cy < 0 && P1[1] + ly > ym)));
    const float *Po = a.gridpos + 3 * g[7 - ioct0];
    const float sox = ipinx ? 1e20f : ((Po[0] - P1[0]) - lx) * rd.ci[0];
    const float soy = ipiny ? 1e20f : ((Po[1] - P1[1]) - ly) * rd.ci[1];
    const float soz = ((Po[2] - P1[2]) - lz) * rd.ci[2];
    const float so = fminf(sox, fminf(soy, soz));
    if (so < -eps) { if (lane == 0) atomicCAS(a.err, ERR_NONE, ERR_RAY_SO); break; }
    const float lxn = fmaf(so, cx, lx), lyn = fmaf(so, cy, ly), lzn = fmaf(so, cz, lz);
    const float du = cx * idx, dv = cy * idy, dw = cz * idz;
    const float sof = so;
    float extn = tri(ext8, fmaf(sof, du, u0), fmaf(sof, dv, v0), fmaf(sof, dw, w0));
    const float taugrid = so * 0.5f * (ext1 + extn);
    int ntau = max(1, 1 + (int)(taugrid * inv_tautol));
    const float delsf = sof / (float)ntau;
    float cacc[3] = {0.f, 0.f, 0.f}, ctr = 1.f;  // as in k_render: per cell in FP32, folded once per cell
    for (int it = 1; it <= ntau; ++it) {
      const float sf_ = it * delsf;
      const float uu_ = fmaf(sf_, du, u0), vv_ = fmaf(sf_, dv, v0), ww_ = fmaf(sf_, dw, w0);
      const float ext0 = tri(ext8, uu_, vv_, ww_);
      float srcext0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) srcext0[c] = tri(src8[c], uu_, vv_, ww_);
      srcext0[0] = fmaxf(0.f, srcext0[0]);
      const float ext = 0.5f * (ext0 + ext1);
      float absc, trc;
      if (ext != 0.f) {
        const float tau = ext * delsf;
        absc = tau * (1.f - 0.5f * tau * (1.f - 0.33333333333f * tau));
        trc = 1.f - absc;
        const float iext = 1.f / ext, corr = delsf * (1.f - 0.05f * (ext1 - ext0) * delsf);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float src = (0.5f * (srcext0[c] + srcext1[c]) + 0.08333333333f * (ext0 * srcext1[c] - ext1 * srcext0[c]) * corr) * iext;
          cacc[c] = fmaf(ctr * src, absc, cacc[c]);
        }
      } else { trc = 1.f; }
      ctr *= trc;
      ext1 = ext0;
#pragma unroll
      for (int c = 0; c < 3; ++c) srcext1[c] = srcext0[c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) radacc[c] += transmit * (double)cacc[c];
    transmit *= (double)ctr;
    int iface, jface;
    bool openbc;
    if (sox <= soz && sox <= soy) { iface = 1 - rd.bit[0]; jface = 0; openbc = (cf & 1) && (a.bcflag & 1); }
    else if (soy <= soz) { iface = 3 - rd.bit[1]; jface = 1; openbc = (cf & 2) && (a.bcflag & 2); }
    else { iface = 5 - rd.bit[2]; jface = 2; openbc = false; }
    int nxt = a.neighptr[6 * (size_t)cell + iface];
    int kface = iface, kc = cell;
    if (openbc) { kface = iface ^ 1; kc = nxt; iface = -1; }
    if (transmit < a.transcut || ngrid > maxcross) {
      validrad = true;
    } else if (nxt < 0 && iface >= 4) {
      validrad = true;  // unpolarized sky and Lambertian surface (I only); a BRDF surface polarizes
      const int *gk = a.gridptr + 8 * (size_t)kc;
      float xs[4], ys[4], rb[3][4];
      for (int k = 0; k < 4; ++k) {
        int q = gk[c_face[kface][k]];
        xs[k] = a.gridpos[3 * q]; ys[k] = a.gridpos[3 * q + 1];
        rb[1][k] = rb[2][k] = 0.f;
        if ((float)mu2 < 0.f) rb[0][k] = a.skyrad;
        else {
          int bi = a.bot_index[q];
          rb[0][k] = bi >= 0 ? a.bcrad_bot[bi] : 0.f;
          if constexpr (BRDF) {
            if (bi >= 0) {
              float o[3];
              brdf_radiance_warp(a, bi, (float)mu2, (float)phi2, lane, 3, o);
              rb[0][k] = o[0]; rb[1][k] = o[1]; rb[2][k] = o[2];
            }
          }
        }
      }
      float uu = (xs[1] - xs[0] > 0) ? ((P1[0] - xs[0]) + lxn) / (xs[1] - xs[0]) : 0.f;
      float vv = (ys[2] - ys[0] > 0) ? ((P1[1] - ys[0]) + lyn) / (ys[2] - ys[0]) : 0.f;
      if (!a.nosurface)
        for (int c = 0; c < 3; ++c)
          radacc[c] += transmit * ((1 - uu) * (1 - vv) * rb[c][0] + uu * (1 - vv) * rb[c][1] + (1 - uu) * vv * rb[c][2] +
                                   uu * vv * rb[c][3]);
    } else {
      const float *Pn = a.gridpos + 3 * a.gridptr[8 * (size_t)nxt];
      const float *q = a.gridpos + 3 * a.gridptr[8 * (size_t)nxt + ioct0];
      lx = jface == 0 ? q[0] - Pn[0] : (P1[0] - Pn[0]) + lxn;
      ly = jface == 1 ? q[1] - Pn[1] : (P1[1] - Pn[1]) + lyn;
      lz = jface == 2 ? q[2] - Pn[2] : (P1[2] - Pn[2]) + lzn;
      cell = nxt;
    }
  }
  if (lane < 3) a.out[(size_t)ray * 3 + lane] = (float)radacc[lane];
}

__global__ void k_bcrad_bottom(const int *botp, int nbot, const float *botalb, const float *dirflux,
                               const float *fluxes, float *bcrad, const float *botplanck) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nbot) return;
  int p = botp[k];
  bcrad[k] = 0.318309886f * botalb[k] * (dirflux[p] + fluxes[2 * (size_t)p]);
  if (botplanck) bcrad[k] += botplanck[k] * (1.f - botalb[k]);
}

}  // namespace shdom

#include "shdom_grad.cuh"

namespace shdom {

// ----------------------------------------------------------------- memory
// Device memory comes from the device's stream-ordered pool, which keeps
// freed memory for reuse (release threshold: never): a handle's state is
// put back without cudaFree, whose device-wide synchronization would stall
// every other handle's work (the serving loop frees units while others
// solve), and a new handle of the same sizes takes it again in
// microseconds.  Allocations and frees go through one non-blocking stream
// per device and are synchronized there, so a buffer is ready for any
// stream when alloc returns; a buffer is freed only after every stream that
// used it has been synchronized (the handle's destructor).
constexpr int kMaxDevices = 64;
static std::mutex g_alloc_mu;
static cudaStream_t g_alloc_stream[kMaxDevices] = {};

static cudaStream_t alloc_stream(int dev) {
  if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("device index out of range");
  std::lock_guard<std::mutex> lk(g_alloc_mu);
  if (!g_alloc_stream[dev]) {
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t keep = UINT64_MAX;
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    CK(cudaStreamCreateWithFlags(&g_alloc_stream[dev], cudaStreamNonBlocking));
  }
  return g_alloc_stream[dev];
}

// bytes on the current device; dev receives that device
static void *dev_alloc(size_t bytes, int &dev) {
  CK(cudaGetDevice(&dev));
  cudaStream_t s = alloc_stream(dev);
  void *p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, s);
  if (e == cudaErrorMemoryAllocation) {  // give the pool's unused memory back and try once more
    cudaGetLastError();
    CK(cudaStreamSynchronize(s));
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    CK(cudaMemPoolTrimTo(pool, 0));
    e = cudaMallocAsync(&p, bytes, s);
  }
  CK(e);
  CK(cudaStreamSynchronize(s));
  return p;
}

static void dev_free(void *p, int dev) {
  if (!p || dev < 0 || dev >= kMaxDevices) return;
  int cur = -1;
  cudaGetDevice(&cur);
  if (cur != dev) cudaSetDevice(dev);
  try {
    cudaFreeAsync(p, alloc_stream(dev));
  } catch (const std::exception &) {
  }
  if (cur != dev && cur >= 0) cudaSetDevice(cur);
}

// ----------------------------------------------------------------- handle
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  bool own = true;  // false: a view of a buffer that a shared geometry owns
  int dev = -1;
  void alloc(size_t k) {
    free();
    n = k;
    own = true;
    if (k) p = static_cast<T *>(dev_alloc(k * sizeof(T), dev));
  }
  void view(const DBuf &o) {
    free();
    p = o.p; n = o.n; own = false;
  }
  void upload(const std::vector<T> &v) { upload(v.data(), v.size()); }
  void upload(const HostVec<T> &v) { upload(v.data(), v.size()); }
  void upload(const T *src, size_t count) {
    alloc(count);
    if (n) CK(cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice));
  }
  // on the handle's (non-blocking) stream, so that later kernels on it are ordered after the fill
  void zero(cudaStream_t st) { if (n) CK(cudaMemsetAsync(p, 0, n * sizeof(T), st)); }
  void free() {
    if (p && own) dev_free(p, dev);
    p = nullptr; n = 0; own = true;
  }
  ~DBuf() { free(); }
};

// Device copies of a plan's grid geometry and sweep schedule: shared by all
// handles whose plans share the host geometry (the wavelengths of one
// medium, inversion iterates), so a new handle uploads only its medium and
// allocates only its state.  The last few stay cached after their handles
// are gone.
struct DevGeom {
  int device = -1;
  std::shared_ptr<const void> key;  // the host geometry (the plan's level table)
  DBuf<float> gridpos, xgrid, ygrid, zgrid, geo;
  DBuf<int> gridptr, neighptr, cellflags, rank, start, level, order, topp, botp, bot_index;
  DBuf<uint8_t> bnd, regular, kind;
  DBuf<uint32_t> tasks[2];
  DBuf<Seg> segs[2], p1segs[2], irrsegs[2];
  DBuf<int> seg_off[2], level_items[2], p1off[2];
  DBuf<IrrRec> irr[2];
  bool irr_built = false;
  // block-local phase 1 (setup_p1s): per hemisphere, built once per grid and device
  bool p1s_built = false, p1s_ok[2] = {false, false};
  DBuf<P1Blk> p1blk[2];
  DBuf<int> p1base[2], p1grp[2], p1slot[2];
  int np1blk[2] = {0, 0};
  size_t p1smem[2] = {0, 0};
  std::mutex mu;  // guards the one-time builds of irr and of the phase-1 tables
};
static std::mutex g_devgeom_mu;
static std::list<std::shared_ptr<DevGeom>> g_devgeom;  // most recent first
constexpr size_t kDevGeomCache = 2;

struct Handle {
  Plan P;
  std::shared_ptr<DevGeom> geom;  // device geometry shared with other handles on the same grid
  std::string err;
  int device = 0;
  cudaStream_t stream = nullptr;
  // geometry
  DBuf<float> gridpos, xgrid, ygrid, zgrid;
  DBuf<int> gridptr, neighptr, cellflags, rank, start, level, order, topp, botp, bot_index, lofj;
  DBuf<uint8_t> bnd, regular;
  DBuf<float> geo;
  DBuf<uint32_t> tasks[2];
  DBuf<Seg> segs[2], p1segs[2], irrsegs[2];
  DBuf<int> seg_off[2], level_items[2], p1off[2], col_oct, col_cls;
  DBuf<uint8_t> kind;
  DBuf<IrrRec> irr[2];
  DBuf<float2> sweepw;  // (radsrc, tr) of the phase-2 items, [npts][ldo]
  int n_irrseg[2] = {0, 0}, p2_irrseg0[2] = {0, 0}, p2_irr_j0[2] = {0, 0};
  cudaStream_t stream2 = nullptr;  // phase-1 sweeps, concurrent with the source pass
  // Levis gradient tables for one species (built on the first gradient call)
  int grad_ipa = -1;
  DBuf<int> g_interpptr, g_sjptr, g_sjiph, g_piph;
  DBuf<float> g_optwt, g_dextm, g_dalbm, g_dfj, g_albsp, g_sjw, g_legu, g_legs, g_fmix, g_scatj, g_legp, g_extp,
      g_albp, g_pphw;
  DBuf<double> g_grad, g_beam, g_adj;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_caller[2] = {nullptr, nullptr};  // ordering against a caller's stream (device-buffer calls)
  cudaEvent_t ev_ext = nullptr;  // after the last render launched on a caller's stream
  int coop_blocks = 0;
  int nsm = 152;  // streaming multiprocessors of the handle's device
  // 0: cooperative persistent kernel when available; 1: one launch per level;
  // 2: as 1, with each iteration's launches replayed from a CUDA graph
  int sweep_mode = 0;
  cudaGraphExec_t iter_graph[2] = {nullptr, nullptr};  // one iteration, without / with the fixed truncation
  long long iter_graph_launches[2] = {0, 0};
  DBuf<float> col_cx, col_cy, col_cz, col_fluxw, cmu1t, cmu2t, cphi1t, cphi2, ylmsun;
  // polarized (nst = 3): Stokes component per ordinate column, the a2/a3/b1
  // source coefficients and the I-Q single-scatter table
  int nst = 1;
  DBuf<uint8_t> col_stk;
  DBuf<float> coefp, phasetab2;
  DBuf<float> pol_t[2];  // FP32 dense transform matrices for the CUDA-core path, [K][N]
  // bidirectional surface
  DBuf<float> botpar;
  DBuf<BrdfOrd> brdf_dn, brdf_up;
  DBuf<int> nphi0, col_of;
  // medium
  DBuf<float> text, dirflux, coef, tms_w, phasetab, botalb, rad0;
  DBuf<float> thermal, botplanck, planckpt;  // thermal source only (empty for a solar source)
  DBuf<double> edp;      // delta-M scaled property-grid extinction (input of the direct beam)
  DBuf<uint8_t> nbscat;  // 1 where a cell containing the point has a scattering corner
  DBuf<int> wready;      // per hemisphere: the source pass has filled every item once
  DBuf<int> tms_ptr, tms_iph;
  // state
  DBuf<float> source, delsource, radiance, srcdo, raddo, fluxes, bcrad;
  DBuf<int> ns, nso, nr, errflag;
  DBuf<double> red;
  DBuf<AccelState> accel;
  int ldo = 0;  // row stride of srcdo/raddo: nang rounded up to 4 (16-byte rows for TMA)
  // tensor-core transforms, per direction (0: SH -> DO, 1: DO -> SH)
  int xf_mode = 0;  // 0: 3xTF32 tensor cores, 1: single TF32 product, 2: CUDA-core factorized
  bool tc_ok[2] = {false, false};
  int tc_bn[2] = {0, 0}, tc_ntiles[2] = {0, 0}, tc_kpad[2] = {0, 0};
  // compacted transforms: the scattering points' rows only (non-scattering
  // points have a zero source and a 4-term radiance)
  bool compact = false;
  int nheavy = 0, nlight = 0;
  DBuf<int> heavy, light;
  DBuf<float> src_c, rad_c, t4;
  CUtensorMap tm_ac[2];
  DBuf<float> tc_bh[2], tc_bl[2];
  CUtensorMap tm_a[2], tm_bh[2], tm_bl[2];
  bool seq[2] = {false, false};  // reference-order sweep engine per hemisphere
  DBuf<TraceRec> seqrec;            // its trace records, [ordinate][rank] of one hemisphere
  DBuf<TraceRec> p1rec;             // phase-1 trace records ahead of the plane march, [irr entry]
  bool p1s[2] = {false, false};     // phase 1 with block-local radiances (k_sweep_p1s)
  DBuf<P1Blk> p1blk[2];
  int np1blk[2] = {0, 0};
  size_t p1smem[2] = {0, 0};
  DBuf<int> p1base[2], p1grp[2], p1slot[2];  // per segment: first slot, group; [group][point]: slot or -1
  // plane-march phase 2 per hemisphere (k_sweep_march): units of (group,
  // column slice), one cluster of mcs[h] CTAs each
  bool march[2] = {false, false};
  bool march_off = false;  // sweep mode 3: the level schedule even where the march applies
  int render_single_scatter = 0, render_nosurface = 0;  // RENDER options of the following renders
  int tc_wait_limit = tc::kWaitLimit;  // polls of a tensor-core pipeline wait (0 only to test the abort path)
  DBuf<MarchGrp> mgrp[2];
  DBuf<MarchUnit> munit[2];
  int mnunits[2] = {0, 0}, mcs[2] = {0, 0};
  size_t msmem[2] = {0, 0};

  bool initialized = false;
  int iters = 0;
  float solcrit = 1.f;
  float timings[5] = {0, 0, 0, 0, 0};
  // sweep kernels of the last solve: [0] phase 1 beside the source pass (or
  // the whole reference-order sweep), [1] the level pass; launches counted
  float ktimes[2] = {0, 0};
  int klaunches[2] = {0, 0};
  bool ktime_on = false;             // record the sweep events in this iteration
  bool ktime_rec[2] = {false, false};
  cudaEvent_t ev_k[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  long long launches = 0;
};

// ---------------------------------------------- dense transform matrices
// The factorized transforms above are linear maps; their matrices are formed
// here once per plan from the same coefficients (CMU1/CPHI1, CMU2/CPHI2 with
// the per-zenith azimuthal cut ME = NPHI0/2 - 1), in double precision.
// T1[c][j]: ordinate column c from harmonic term j (SH_TO_DO_UNPOL,
// src/polarized/shdomsub1.f:2928-3036).
static void dense_sh_to_do(const Plan &P, std::vector<double> &T) {
  const int nlm = P.nlm, nm = 2 * P.mm + 1, np0 = P.nphi0max;
  T.assign((size_t)P.nang * nlm, 0.0);
  for (int j = 0; j < nlm; ++j) {
    const int m = P.mofj[j], ma = std::abs(m);
    for (int i = 0; i < P.nmu; ++i) {
      const int n0 = P.nphi0[i], me = std::max(0, n0 / 2 - 1);
      if (ma > me) continue;
      const double u = P.cmu1[(size_t)i * nlm + j];
      for (int k = 0; k < n0; ++k) {
        const float *cp = &P.cphi1[((size_t)i * np0 + k) * nm + P.mm];
        double w = (m == 0) ? cp[0] : (m > 0 ? (double)cp[m] - cp[-m] : (double)cp[m] + cp[-m]);
        T[(size_t)P.col_of[i * np0 + k] * nlm + j] += u * w;
      }
    }
  }
}

// T2[j][c]: harmonic term j from ordinate column c (DO_TO_SH_UNPOL,
// src/polarized/shdomsub1.f:3164-3254); rows nlm and nlm+1 are the downward
// and upward hemispheric flux weights.
static void dense_do_to_sh(const Plan &P, std::vector<double> &T) {
  const int nlm = P.nlm, nm = 2 * P.mm + 1, np0 = P.nphi0max, nang = P.nang;
  T.assign((size_t)(nlm + 2) * nang, 0.0);
  for (int j = 0; j < nlm; ++j) {
    const int m = P.mofj[j], ma = std::abs(m);
    for (int i = 0; i < P.nmu; ++i) {
      const int n0 = P.nphi0[i], me = std::max(0, n0 / 2 - 1);
      if (ma > me) continue;
      const double u = P.cmu2[(size_t)i * nlm + j];
      for (int k = 0; k < n0; ++k) {
        const float *cp = &P.cphi2[((size_t)i * np0 + k) * nm + P.mm];
        double w = (m == 0) ? cp[0] : (m > 0 ? (double)cp[m] - cp[-m] : (double)cp[-m] + cp[m]);
        T[(size_t)j * nang + P.col_of[i * np0 + k]] += u * w;
      }
    }
  }
  for (int c = 0; c < nang; ++c) T[(size_t)(c < P.ncol_down ? nlm : nlm + 1) * nang + c] = P.col_fluxw[c];
}

// Polarized matrices (SH_TO_DO / DO_TO_SH, src/polarized/shdomsub1.f:
// 2789-2926, :3041-3160).  Harmonic rows are [Stokes][nlm] (I, Q, U), ordinate
// columns are the plan's Stokes columns.  The mu part mixes Q and U with the
// generalized functions (elements 2, 3, 5, 6); in azimuth the I and Q
// harmonics use cos/sin like the scalar transform and U the swapped pair
// (the reference's SUMCS(3, +-m) rules).
// T1[c][s * nlm + j]: column c from Stokes harmonic (s, j).
static void dense_sh_to_do_pol(const Plan &P, std::vector<double> &T) {
  const int nlm = P.nlm, nm = 2 * P.mm + 1, np0 = P.nphi0max, K = 3 * nlm;
  T.assign((size_t)P.nang * K, 0.0);
  // mu coefficient of input Stokes si in output Stokes so, element index into the 6 generalized functions
  const int el[3][3] = {{0, -1, -1}, {-1, 1, 4}, {-1, 5, 2}};
  for (int j = 0; j < nlm; ++j) {
    const int m = P.mofj[j], ma = std::abs(m);
    for (int i = 0; i < P.nmu; ++i) {
      const int n0 = P.nphi0[i], me = std::max(0, n0 / 2 - 1);
      if (ma > me) continue;
      const float *c6 = &P.cmu1p[((size_t)i * nlm + j) * 6];
      for (int k = 0; k < n0; ++k) {
        const float *cp = &P.cphi1[((size_t)i * np0 + k) * nm + P.mm];
        const int c0 = P.col_of[i * np0 + k];  // the I column; Q and U follow at the group's stride
        for (int so = 0; so < 3; ++so) {
          double w;
          if (m == 0) w = cp[0];
          else if (so < 2) w = m > 0 ? (double)cp[ma] - cp[-ma] : (double)cp[ma] + cp[-ma];
          else w = m > 0 ? (double)cp[ma] + cp[-ma] : (double)cp[ma] - cp[-ma];
          const int col = c0 + so * (P.cls_ncol[P.col_oct[c0] - 1][P.col_cls[c0]] / 3);
          for (int si = 0; si < 3; ++si) {
            const int e = el[so][si];
            if (e < 0) continue;
            T[(size_t)col * K + si * nlm + j] += (double)c6[e] * w;
          }
        }
      }
    }
  }
}

// T2[s * nlm + j][c]: Stokes harmonic (s, j) from column c.
static void dense_do_to_sh_pol(const Plan &P, std::vector<double> &T) {
  const int nlm = P.nlm, nm = 2 * P.mm + 1, np0 = P.nphi0max, nang = P.nang;
  T.assign((size_t)(3 * nlm) * nang, 0.0);
  // mu coefficient of ordinate Stokes si in harmonic Stokes so
  const int el[3][3] = {{0, -1, -1}, {-1, 1, 4}, {-1, 5, 2}};
  for (int j = 0; j < nlm; ++j) {
    const int m = P.mofj[j], ma = std::abs(m);
    for (int i = 0; i < P.nmu; ++i) {
      const int n0 = P.nphi0[i], me = std::max(0, n0 / 2 - 1);
      if (ma > me) continue;
      const float *c6 = &P.cmu2p[((size_t)i * nlm + j) * 6];
      for (int k = 0; k < n0; ++k) {
        const float *cp = &P.cphi2[((size_t)i * np0 + k) * nm + P.mm];
        const int c0 = P.col_of[i * np0 + k];
        for (int si = 0; si < 3; ++si) {
          double w;
          if (m == 0) w = cp[0];
          else if (si < 2) w = m > 0 ? (double)cp[ma] - cp[-ma] : (double)cp[ma] + cp[-ma];
          else w = m > 0 ? (double)cp[ma] + cp[-ma] : (double)cp[ma] - cp[-ma];
          const int col = c0 + si * (P.cls_ncol[P.col_oct[c0] - 1][P.col_cls[c0]] / 3);
          for (int so = 0; so < 3; ++so) {
            const int e = el[so][si];
            if (e < 0) continue;
            T[(size_t)(so * nlm + j) * nang + col] += (double)c6[e] * w;
          }
        }
      }
    }
  }
}

// Round to TF32 (10 explicit mantissa bits), nearest with ties away from
// zero, as cvt.rna.tf32.f32 does on the device.
static float tf32_rna(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  if ((b & 0x7f800000u) != 0x7f800000u) b = (b + 0x1000u) & 0xffffe000u;
  float y;
  std::memcpy(&y, &b, 4);
  return y;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw std::runtime_error("cuTensorMapEncodeTiled not available");
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 2-D fp32 tensor map: rows x inner elements, row stride ld elements, box of
// box_rows x 32 elements (one 128-byte swizzle row), zero fill outside.
static void make_map(CUtensorMap *m, const float *base, uint64_t inner, uint64_t rows, uint64_t ld, uint32_t box_rows) {
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {ld * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)tc::BK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_tiled()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)base, dims, strides, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

// The tensor-core GEMM is instantiated for N tiles of 32..128 columns.
template <int BN>
static void tc_attr1() {
  CK(cudaFuncSetAttribute(tc::k_tc_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::smem_bytes<BN>()));
}
static void tc_attr(int bn) {
  switch (bn) {
    case 32: tc_attr1<32>(); break;   case 64: tc_attr1<64>(); break;
    case 96: tc_attr1<96>(); break;   case 128: tc_attr1<128>(); break;
    default: throw std::runtime_error("tensor-core transform: unsupported tile width");
  }
}
template <int BN>
static void tc_launch1(int nblocks, cudaStream_t st, const CUtensorMap &a, const CUtensorMap &bh,
                       const CUtensorMap &bl, int K, int ntn, int ntiles, const tc::Epilogue &g) {
  tc::k_tc_gemm<BN><<<nblocks, tc::kThreads, tc::smem_bytes<BN>(), st>>>(a, bh, bl, K, ntn, ntiles, g);
}
// Persistent launch: one CTA per SM (the pipeline fills the shared memory),
// each walking its share of the ntiles = ntn x row-tile tiles.
static void tc_launch(int bn, int nsm, cudaStream_t st, const CUtensorMap &a, const CUtensorMap &bh,
                      const CUtensorMap &bl, int K, int ntn, int ntiles, const tc::Epilogue &g) {
  const int nb = std::max(1, std::min(ntiles, nsm));
  switch (bn) {
    case 32: tc_launch1<32>(nb, st, a, bh, bl, K, ntn, ntiles, g); break;
    case 64: tc_launch1<64>(nb, st, a, bh, bl, K, ntn, ntiles, g); break;
    case 96: tc_launch1<96>(nb, st, a, bh, bl, K, ntn, ntiles, g); break;
    case 128: tc_launch1<128>(nb, st, a, bh, bl, K, ntn, ntiles, g); break;
    default: throw std::runtime_error("tensor-core transform: unsupported tile width");
  }
}

// Forms the dense matrices, splits them into TF32 high and low parts
// ([Npad][Kpad], zero padded) and encodes the tensor maps.  A direction whose
// operand rows are not 16-byte multiples, or too small for one tile, keeps
// the factorized CUDA-core transform.
static void setup_tc(Handle &H) {
  Plan &P = H.P;
  int dev = 0, major = 0, minor = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  CK(cudaDeviceGetAttribute(&H.nsm, cudaDevAttrMultiProcessorCount, dev));
  if (H.nst == 3) {  // [K][N] FP32 matrices of the CUDA-core transforms
    std::vector<double> T;
    const int nsh3 = 3 * P.nlm;
    dense_sh_to_do_pol(P, T);  // [nang][3 nlm]
    std::vector<float> t((size_t)nsh3 * P.nang);
    for (int c = 0; c < P.nang; ++c)
      for (int k = 0; k < nsh3; ++k) t[(size_t)k * P.nang + c] = (float)T[(size_t)c * nsh3 + k];
    H.pol_t[0].upload(t);
    dense_do_to_sh_pol(P, T);  // [3 nlm][nang]
    t.assign((size_t)P.nang * nsh3, 0.f);
    for (int j = 0; j < nsh3; ++j)
      for (int c = 0; c < P.nang; ++c) t[(size_t)c * nsh3 + j] = (float)T[(size_t)j * P.nang + c];
    H.pol_t[1].upload(t);
  }
  if (major != 10) return;
  const int nsh = H.nst * P.nlm;  // harmonic row length (I, Q, U rows when polarized)
  for (int dir = 0; dir < 2; ++dir) {
    // the ordinate-to-harmonic direction forms the fluxes from A on the CUDA cores
    const int K = dir == 0 ? nsh : P.nang, N = dir == 0 ? P.nang : nsh;
    const int lda = dir == 0 ? nsh : H.ldo;
    if (lda % 4 != 0 || K < tc::BK || P.npts < tc::BM) continue;
    if (dir == 1 && (K + tc::BK - 1) / tc::BK * tc::BK * 8 > 16 * 1024) continue;  // flux weight table
    const int ntiles = (N + 127) / 128;  // tiles of at most 128 columns keep the FP32 sums in registers
    const int bn = ((N + ntiles - 1) / ntiles + 31) / 32 * 32;
    const int npad = ntiles * bn, kpad = (K + tc::BK - 1) / tc::BK * tc::BK;
    std::vector<double> T;
    if (H.nst == 3) { if (dir == 0) dense_sh_to_do_pol(P, T); else dense_do_to_sh_pol(P, T); }
    else if (dir == 0) dense_sh_to_do(P, T);
    else dense_do_to_sh(P, T);  // rows [0, N) are used
    std::vector<float> bh((size_t)npad * kpad, 0.f), bl((size_t)npad * kpad, 0.f);
    for (int n = 0; n < N; ++n)
      for (int k = 0; k < K; ++k) {
        const double t = T[(size_t)n * K + k];
        const float h = tf32_rna((float)t);
        bh[(size_t)n * kpad + k] = h;
        bl[(size_t)n * kpad + k] = tf32_rna((float)(t - (double)h));
      }
    H.tc_bh[dir].upload(bh);
    H.tc_bl[dir].upload(bl);
    const float *a = dir == 0 ? H.source.p : H.raddo.p;
    make_map(&H.tm_a[dir], a, (uint64_t)K, (uint64_t)P.npts, (uint64_t)lda, tc::BM);
    make_map(&H.tm_bh[dir], H.tc_bh[dir].p, (uint64_t)kpad, (uint64_t)npad, (uint64_t)kpad, (uint32_t)bn);
    make_map(&H.tm_bl[dir], H.tc_bl[dir].p, (uint64_t)kpad, (uint64_t)npad, (uint64_t)kpad, (uint32_t)bn);
    H.tc_bn[dir] = bn; H.tc_ntiles[dir] = ntiles; H.tc_kpad[dir] = kpad;
    tc_attr(bn);
    H.tc_ok[dir] = true;
    if (dir == 1) {  // first 4 rows of the ordinate-to-harmonic matrix, for the non-scattering points
      std::vector<float> t4((size_t)4 * P.nang, 0.f);
      for (int n = 0; n < std::min(4, N); ++n)
        for (int k = 0; k < K; ++k) t4[(size_t)n * P.nang + k] = (float)T[(size_t)n * K + k];
      H.t4.upload(t4);
    }
  }
  // Non-scattering points (zero coefficient row) have a zero source in every
  // iteration and a 4-term radiance (the radiance truncation of a point
  // without scattering stays at 4), so the transforms need only the
  // scattering points' rows: gathered into dense blocks for the tensor
  // cores; the others get their 4 radiance terms and fluxes on the CUDA
  // cores.  (Not with HIGHORDERRAD, which keeps every radiance term.)
  if (H.tc_ok[0] && H.tc_ok[1] && !P.prob.highorderrad && P.nlm >= 4 && H.nst == 1) {
    std::vector<int> hv, lt;
    for (int p = 0; p < P.npts; ++p) (P.scat[p] ? hv : lt).push_back(p);
    if (!lt.empty() && (long long)hv.size() * 10 < (long long)P.npts * 9) {
      H.compact = true;
      H.nheavy = (int)hv.size(); H.nlight = (int)lt.size();
      H.heavy.upload(hv); H.light.upload(lt);
      if (H.nheavy > 0) {
        H.src_c.alloc((size_t)H.nheavy * P.nlm);
        H.rad_c.alloc((size_t)H.nheavy * H.ldo);
        make_map(&H.tm_ac[0], H.src_c.p, (uint64_t)P.nlm, (uint64_t)H.nheavy, (uint64_t)P.nlm, tc::BM);
        make_map(&H.tm_ac[1], H.rad_c.p, (uint64_t)P.nang, (uint64_t)H.nheavy, (uint64_t)H.ldo, tc::BM);
      }
    }
  }
}

// Device memory a handle for this plan holds: the uploaded tables, the
// solution state and the tensor-core transform matrices.
template <typename T, typename A>
static long long vbytes(const std::vector<T, A> &v) { return (long long)v.size() * (long long)sizeof(T); }
template <typename T>
static long long vbytes(const SharedVec<T> &v) { return (long long)v.size() * (long long)sizeof(T); }

// A hemisphere is swept in the reference order when its wavefront is too
// deep for level scheduling.
static bool reference_order(const Plan &P, int h) {
  const int nlev = (int)P.seg_off[h].size() - 1;
  return P.deep[h] || std::max(nlev, P.p1depth[h]) > 4 * (P.nx1 + P.ny1 + P.nz) + 64;
}

static long long plan_device_bytes(const Plan &P) {
  long long b = 0;
  b += vbytes(P.gridpos) + vbytes(P.xgrid) + vbytes(P.ygrid) + vbytes(P.zgrid) + vbytes(P.gridptr) + vbytes(P.neighptr);
  b += vbytes(P.cellflags) + vbytes(P.rank) + vbytes(P.startcell) + vbytes(P.level) + vbytes(P.rank);  // + order
  b += vbytes(P.topp) + vbytes(P.botp) + 4LL * P.npts + vbytes(P.lofj) + vbytes(P.bnd) + vbytes(P.regular) + vbytes(P.geo);
  for (int h = 0; h < 2; ++h)
    b += vbytes(P.tasks[h]) + vbytes(P.segs[h]) + vbytes(P.seg_off[h]) + vbytes(P.level_items[h]) + 32LL * P.nirr[h];
  b += 8LL * P.npts * ((P.nang + 3) & ~3) + vbytes(P.kind);  // (radsrc, tr) per point and ordinate
  b += 4LL * 5 * P.nang + vbytes(P.cmu1) + vbytes(P.cmu2) + vbytes(P.cphi1) + vbytes(P.cphi2) + vbytes(P.ylmsun);
  b += vbytes(P.nphi0) + vbytes(P.col_of) + vbytes(P.total_ext) + 4LL * P.npts + vbytes(P.coef) + vbytes(P.tms_ptr);
  b += vbytes(P.tms_iph) + vbytes(P.tms_w) + vbytes(P.phasetab) + vbytes(P.botalb) + vbytes(P.rad0);
  b += vbytes(P.thermal) + vbytes(P.botplanck) + vbytes(P.planckpt);
  const long long ldo = (P.nang + 3) & ~3;
  b += 4LL * P.npts * (3LL * P.nst * P.nlm + 2 * ldo + 2 + 3) + 4LL * (long long)P.botp.size() + 64;
  if (P.nst == 3) b += vbytes(P.col_stk) + vbytes(P.coefp) + vbytes(P.phasetab2) + 8LL * P.nlm * 3 * P.nang;
  {  // gathered rows of the scattering points for the compacted transforms
    long long nh = 0;
    for (int p = 0; p < P.npts; ++p) nh += P.scat[p];
    if (nh * 10 < (long long)P.npts * 9) b += 4LL * nh * (P.nlm + ldo) + 4LL * P.npts + 16LL * P.nang;
  }
  {  // phase-1 trace records ahead of a plane march (at most one per general-trace item), and the
     // block-local phase 1's slot tables ([group][point])
    long long n1 = 0;
    for (int h = 0; h < 2; ++h)
      if (!P.march[h].empty()) {
        n1 = std::max<long long>(n1, (long long)P.nirr[h]);
        b += 4LL * P.npts * std::max(0, (int)P.p1off[h].size() - 1) + 8LL * (long long)P.p1segs[h].size();
      }
    b += 32LL * n1;
  }
  {  // trace records of a reference-order sweep (32 bytes per point and ordinate of a hemisphere)
    long long nrec = 0;
    for (int h = 0; h < 2; ++h)
      if (reference_order(P, h)) nrec = std::max<long long>(nrec, (long long)P.npts * (h ? P.nang - P.ncol_down : P.ncol_down));
    b += 32LL * nrec;
  }
  const long long nsh = (long long)P.nst * P.nlm;
  const long long kp0 = (nsh + 31) / 32 * 32, kp1 = (P.nang + 31) / 32 * 32;
  const long long np0 = ((P.nang + 255) / 256) * 256 + 256, np1 = ((nsh + 2 + 255) / 256) * 256 + 256;
  b += 8LL * (np0 * kp0 + np1 * kp1);  // upper bound of the padded hi/lo matrices
  return b;
}

static void fill_sizes(const Plan &P, shdom_sizes *o) {
  o->npts = P.npts; o->ncells = P.ncells; o->nx1 = P.nx1; o->ny1 = P.ny1; o->nz = P.nz; o->nlm = P.nlm;
  o->nmu = P.nmu; o->nang = P.nang_real; o->ml = P.ml; o->mm = P.mm; o->bcflag = P.bcflag; o->ipflag = P.ipflag;
  o->albmax = P.albmax;
  o->nlevels_down = (int)P.seg_off[0].size() - 1;
  o->nlevels_up = (int)P.seg_off[1].size() - 1;
  o->device_bytes = plan_device_bytes(P);
  o->nstokes = P.nst;
  o->march = (P.march[0].empty() ? 0 : 1) | (P.march[1].empty() ? 0 : 2);
  o->march_units_down = o->march_units_up = o->march_cluster_down = o->march_cluster_up = 0;
}

// Units and cluster shape of the plane march of each hemisphere that has
// one.  Of 16-CTA and 8-CTA clusters the shape with more CTAs resident at
// once is taken; the groups are split into column slices in proportion to
// their work, about as many units as clusters fit on the device at once.
// (Measured against two other plans: filling whole waves with twice as many
// narrower units, and the fewest, widest units that fit; both were slower,
// since a plane's time is mostly the latency of its dependent chain.)  A
// hemisphere whose units cannot be launched on this device keeps the level
// schedule.
constexpr size_t kMarchSmemCap = 110 * 1024;  // two CTAs per SM

static int march_max_clusters(int cs, size_t smem) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)cs); cfg.blockDim = dim3(MT); cfg.dynamicSmemBytes = smem;
  cfg.attrs = at; cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_sweep_march, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

static void setup_march(Handle &H) {
  Plan &P = H.P;
  int dev = 0, clus = 0, maxsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&clus, cudaDevAttrClusterLaunch, dev));
  CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  H.march[0] = H.march[1] = false;
  if (!clus || (size_t)maxsm < kMarchSmemCap) return;
  CK(cudaFuncSetAttribute(k_sweep_march, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm));
  const bool big = cudaFuncSetAttribute(k_sweep_march, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  if (!big) cudaGetLastError();
  // resident clusters of each shape at the shared-memory cap; the shape with
  // more CTAs resident at once is taken
  int best_cs = 0, best_n = 0;
  for (int cs : {16, 8}) {
    if (cs > 8 && !big) continue;
    const int n = march_max_clusters(cs, kMarchSmemCap);
    if (n * cs > best_n * best_cs) { best_cs = cs; best_n = n; }
  }
  if (best_n < 1) return;
  for (int h = 0; h < 2; ++h) {
    if (P.march[h].empty() || H.seq[h]) continue;
    for (int cs : {best_cs, best_cs == 16 ? 8 : 0}) {
      if (cs == 0) break;
      const int nclusters = march_max_clusters(cs, kMarchSmemCap);
      if (nclusters < 1) continue;
      // Column slices per group in proportion to its work (planes x plane
      // points x columns), about one unit per resident cluster, and at
      // least as many as fit: every thread of a CTA takes one column and at
      // most MK (row, v) pairs of its strip.
      double tot = 0;
      for (const MarchGrp &g : P.march[h]) tot += (double)g.nA * g.nU * g.nV * g.ncol;
      std::vector<MarchUnit> units;
      size_t smem = 0;
      for (size_t gi = 0; gi < P.march[h].size(); ++gi) {
        const MarchGrp &g = P.march[h][gi];
        const double w = (double)g.nA * g.nU * g.nV * g.ncol;
        int nsl = std::max(1, (int)std::floor(nclusters * w / tot));
        nsl = std::min(nsl, g.ncol);
        const int tw = (g.nU + cs - 1) / cs;
        auto fits = [&](int nc) {
          const int tpc = MT / nc;
          return tpc >= 1 && (tw * g.nV + tpc - 1) / tpc <= MK && march_smem_bytes(tw, g.nV, nc) <= kMarchSmemCap;
        };
        while (nsl < g.ncol && !fits((g.ncol + nsl - 1) / nsl)) ++nsl;
        if (!fits((g.ncol + nsl - 1) / nsl)) { units.clear(); break; }
        const int base = g.ncol / nsl, extra = g.ncol % nsl;
        int c0 = g.col0;
        for (int k = 0; k < nsl; ++k) {
          const int nc = base + (k < extra ? 1 : 0);
          units.push_back(MarchUnit{(int)gi, c0, nc, tw});
          smem = std::max(smem, march_smem_bytes(tw, g.nV, nc));
          c0 += nc;
        }
      }
      if (units.empty()) continue;
      // longest units first (planes x pairs per thread), so that the units
      // left for the second wave of clusters are the short ones
      auto unit_time = [&](const MarchUnit &u) {
        const MarchGrp &g = P.march[h][u.grp];
        const int tpc = MT / u.nc;
        return (long long)g.nA * ((u.tw * g.nV + tpc - 1) / tpc);
      };
      std::stable_sort(units.begin(), units.end(),
                       [&](const MarchUnit &x, const MarchUnit &y) { return unit_time(x) > unit_time(y); });
      std::vector<MarchGrp> grps(P.march[h].begin(), P.march[h].end());
      H.mgrp[h].upload(grps);
      H.munit[h].upload(units);
      H.mnunits[h] = (int)units.size(); H.mcs[h] = cs; H.msmem[h] = smem;
      H.march[h] = true;
      break;
    }
  }
}

// Block-local phase 1 (k_sweep_p1s) for each marching hemisphere whose
// phase-1 groups fit: a group's phase-1 points are numbered in level order,
// and a block takes as many of its columns as keep the slice's radiances
// of all those points in kP1SmemCap bytes (and a level's items within four
// per thread).  Otherwise the hemisphere keeps k_sweep_p1r.
constexpr size_t kP1SmemCap = 192 * 1024;

static void setup_p1s(Handle &H) {
  Plan &P = H.P;
  int dev = 0, maxsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t static_smem = sizeof(Seg) * P1_SEGCAP + sizeof(int) * P1_SEGCAP;
  if ((size_t)maxsm >= kP1SmemCap + static_smem)
    CK(cudaFuncSetAttribute(k_sweep_p1s, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(maxsm - static_smem)));
  DevGeom &G = *H.geom;
  std::lock_guard<std::mutex> lk(G.mu);
  if (!G.p1s_built) {
    for (int h = 0; h < 2; ++h) {
      G.p1s_ok[h] = false;
      const std::vector<int> &off = P.p1off[h];
      const int ng1 = (int)off.size() - 1;
      if (!H.march[h] || ng1 <= 0 || (size_t)maxsm < kP1SmemCap + static_smem) continue;
      const std::vector<Seg> &sg = P.p1segs[h];
      std::vector<int> base(sg.size(), 0), grp(sg.size(), 0), nslots(ng1, 0);
      bool ok = true;
      for (int g = 0; g < ng1 && ok; ++g) {
        if (off[g + 1] - off[g] > P1_SEGCAP) ok = false;
        for (int si = off[g]; si < off[g + 1]; ++si) {
          base[si] = nslots[g];
          grp[si] = g;
          nslots[g] += sg[si].ntask;
          if (sg[si].col0 != sg[off[g]].col0 || sg[si].ncol != sg[off[g]].ncol) ok = false;
        }
        if ((size_t)nslots[g] * sizeof(float) > kP1SmemCap) ok = false;
      }
      if (!ok) continue;
      std::vector<P1Blk> blks;
      size_t smem = 0;
      for (int g = 0; g < ng1; ++g) {
        if (off[g + 1] == off[g]) continue;
        const Seg &s0 = sg[off[g]];
        int maxtask = 0;
        for (int si = off[g]; si < off[g + 1]; ++si) maxtask = std::max(maxtask, sg[si].ntask);
        int ncs = (int)std::min<size_t>(kP1SmemCap / ((size_t)nslots[g] * sizeof(float)), (size_t)s0.ncol);
        ncs = std::max(1, std::min(ncs, 4 * P1S_THREADS / std::max(1, maxtask)));
        for (int c0 = 0; c0 < s0.ncol; c0 += ncs) {
          const int nc = std::min(ncs, s0.ncol - c0);
          blks.push_back(P1Blk{g, c0, nc, nslots[g]});
          smem = std::max(smem, (size_t)nslots[g] * nc * sizeof(float));
        }
      }
      std::vector<int> slot((size_t)ng1 * P.npts, -1);
      for (int g = 0; g < ng1; ++g)
        for (int si = off[g]; si < off[g + 1]; ++si)
          for (int t = 0; t < sg[si].ntask; ++t) slot[(size_t)g * P.npts + P.tasks[h][sg[si].t0 + t]] = base[si] + t;
      G.p1blk[h].upload(blks);
      G.p1base[h].upload(base);
      G.p1grp[h].upload(grp);
      G.p1slot[h].upload(slot);
      G.np1blk[h] = (int)blks.size();
      G.p1smem[h] = smem;
      G.p1s_ok[h] = true;
    }
    G.p1s_built = true;
  }
  for (int h = 0; h < 2; ++h) {
    H.p1s[h] = G.p1s_ok[h] && H.march[h];
    if (!H.p1s[h]) continue;
    H.p1blk[h].view(G.p1blk[h]); H.p1base[h].view(G.p1base[h]);
    H.p1grp[h].view(G.p1grp[h]); H.p1slot[h].view(G.p1slot[h]);
    H.np1blk[h] = G.np1blk[h]; H.p1smem[h] = G.p1smem[h];
  }
}

static void upload_plan(Handle &H) {
  Plan &P = H.P;
  H.nst = P.nst;
  {  // the grid geometry and sweep schedule: shared with handles on the same grid and device
    int dev = 0;
    CK(cudaGetDevice(&dev));
    std::shared_ptr<const void> key = P.level.owner();
    std::lock_guard<std::mutex> lk(g_devgeom_mu);
    for (auto it = g_devgeom.begin(); it != g_devgeom.end(); ++it)
      if ((*it)->device == dev && (*it)->key == key) { H.geom = *it; g_devgeom.splice(g_devgeom.begin(), g_devgeom, it); break; }
    if (!H.geom) {
      auto G = std::make_shared<DevGeom>();
      G->device = dev; G->key = key;
      G->gridpos.upload(P.gridpos); G->xgrid.upload(P.xgrid); G->ygrid.upload(P.ygrid); G->zgrid.upload(P.zgrid);
      G->gridptr.upload(P.gridptr); G->neighptr.upload(P.neighptr); G->cellflags.upload(P.cellflags);
      G->rank.upload(P.rank); G->start.upload(P.startcell); G->level.upload(P.level);
      std::vector<int> ord((size_t)8 * P.npts, 0);
      for (int b = 0; b < 8; ++b)
        for (int i = 0; i < P.npts; ++i) {
          int r = P.rank[(size_t)b * P.npts + i];
          if (r >= 0) ord[(size_t)b * P.npts + r] = i;
        }
      G->order.upload(ord);
      G->regular.upload(P.regular); G->geo.upload(P.geo);
      G->bnd.upload(P.bnd); G->topp.upload(P.topp); G->botp.upload(P.botp);
      std::vector<int> bi(P.npts, -1);
      for (size_t k = 0; k < P.botp.size(); ++k) bi[P.botp[k]] = (int)k;
      G->bot_index.upload(bi);
      for (int h = 0; h < 2; ++h) {
        G->tasks[h].upload(P.tasks[h]); G->segs[h].upload(P.segs[h]);
        G->seg_off[h].upload(P.seg_off[h]); G->level_items[h].upload(P.level_items[h]);
        G->p1segs[h].upload(P.p1segs[h]); G->p1off[h].upload(P.p1off[h]);
        // general-trace segments of both phases in irr0 order
        std::vector<Seg> is(P.p1segs[h]);
        for (const Seg &g : P.segs[h]) if (!g.regular) is.push_back(g);
        G->irrsegs[h].upload(is);
      }
      G->kind.upload(P.kind);
      g_devgeom.emplace_front(G);
      while (g_devgeom.size() > kDevGeomCache) g_devgeom.pop_back();
      H.geom = G;
    }
    DevGeom &G = *H.geom;
    H.gridpos.view(G.gridpos); H.xgrid.view(G.xgrid); H.ygrid.view(G.ygrid); H.zgrid.view(G.zgrid);
    H.gridptr.view(G.gridptr); H.neighptr.view(G.neighptr); H.cellflags.view(G.cellflags);
    H.rank.view(G.rank); H.start.view(G.start); H.level.view(G.level); H.order.view(G.order);
    H.regular.view(G.regular); H.geo.view(G.geo); H.bnd.view(G.bnd); H.topp.view(G.topp); H.botp.view(G.botp);
    H.bot_index.view(G.bot_index); H.kind.view(G.kind);
    for (int h = 0; h < 2; ++h) {
      H.tasks[h].view(G.tasks[h]); H.segs[h].view(G.segs[h]); H.seg_off[h].view(G.seg_off[h]);
      H.level_items[h].view(G.level_items[h]); H.p1segs[h].view(G.p1segs[h]); H.p1off[h].view(G.p1off[h]);
      H.irrsegs[h].view(G.irrsegs[h]);
    }
  }
  for (int h = 0; h < 2; ++h) {
    int nlev = (int)P.seg_off[h].size() - 1;
    H.seq[h] = reference_order(P, h);
    for (int l = 0; l < nlev; ++l)
      if (P.seg_off[h][l + 1] - P.seg_off[h][l] > MAXSEG) throw std::runtime_error("sweep schedule: too many segments in a level");
  }

  H.lofj.upload(P.lofj);
  for (int h = 0; h < 2; ++h) {
    H.p2_irrseg0[h] = (int)P.p1segs[h].size();
    H.p2_irr_j0[h] = 0;
    for (const Seg &g : P.p1segs[h]) H.p2_irr_j0[h] = std::max(H.p2_irr_j0[h], g.irr0 + g.ntask * g.ncol);
    int nis = (int)P.p1segs[h].size();
    for (const Seg &g : P.segs[h]) if (!g.regular) ++nis;
    H.n_irrseg[h] = nis;
  }
  {
    std::vector<int> cls(P.col_cls.begin(), P.col_cls.end());
    H.col_oct.upload(P.col_oct); H.col_cls.upload(cls);
  }
  {
    int dev = 0, nsm = 0, per = 0, coop = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sweep_levels, 256, 0));
    H.coop_blocks = coop ? nsm * per : 0;
  }
  H.col_cx.upload(P.col_cx); H.col_cy.upload(P.col_cy); H.col_cz.upload(P.col_cz); H.col_fluxw.upload(P.col_fluxw);
  H.ylmsun.upload(P.ylmsun);
  // transform tables: CMU1/CMU2 as [j][mu], CPHI1 as [mu][m][phi], CPHI2 as [mu][phi][m]
  {
    const int nlm = P.nlm, nmu = P.nmu, nm = 2 * P.mm + 1, np0 = P.nphi0max;
    std::vector<float> c1t((size_t)nlm * nmu), c2t((size_t)nlm * nmu), p1t((size_t)nmu * nm * np0, 0.f);
    for (int i = 0; i < nmu; ++i)
      for (int j = 0; j < nlm; ++j) { c1t[(size_t)j * nmu + i] = P.cmu1[(size_t)i * nlm + j]; c2t[(size_t)j * nmu + i] = P.cmu2[(size_t)i * nlm + j]; }
    for (int i = 0; i < nmu; ++i)
      for (int k = 0; k < np0; ++k)
        for (int m = 0; m < nm; ++m) p1t[((size_t)i * nm + m) * np0 + k] = P.cphi1[((size_t)i * np0 + k) * nm + m];
    H.cmu1t.upload(c1t); H.cmu2t.upload(c2t); H.cphi1t.upload(p1t); H.cphi2.upload(P.cphi2);
    H.nphi0.upload(P.nphi0); H.col_of.upload(P.col_of);
  }
  H.text.upload(P.total_ext); H.coef.upload(P.coef);
  {  // direct beam of every grid point (DIRECT_BEAM_PROP) on the device, on the handle's stream
    H.edp.upload(P.extdirp);
    CK(cudaStreamSynchronize(cudaStreamLegacy));
    H.dirflux.alloc(P.npts);
    BeamGeom g;
    g.edp = H.edp.p; g.zlev = H.zgrid.p; g.gridpos = H.gridpos.p; g.dirflux = H.dirflux.p;
    g.npts = P.npts; g.npx = P.prob.npx; g.npy = P.prob.npy; g.npz = P.prob.npz; g.bcflag = P.bcflag;
    g.ipflag = P.ipflag; g.delx = P.prob.delx; g.dely = P.prob.dely; g.solarmu = P.prob.solarmu;
    g.solaraz = P.prob.solaraz; g.solarflux = P.srct == 'T' ? 0.f : P.prob.solarflux;  // no beam for 'T'
    if (P.srct == 'T') {
      H.dirflux.zero(H.stream);  // a thermal source has no solar beam: skip the path integrals
    } else {
      k_direct_beam<<<(P.npts + 127) / 128, 128, 0, H.stream>>>(g);
      CK(cudaGetLastError());
      H.launches += 1;
    }
  }
  {
    // scattering points (a non-zero coefficient row makes a non-zero source), spread to their cells' corners
    DBuf<uint8_t> sc;
    sc.upload(P.scat);
    CK(cudaStreamSynchronize(cudaStreamLegacy));
    H.nbscat.alloc(P.npts);
    H.nbscat.zero(H.stream);
    if (P.ncells > 0) k_spread_scat<<<(P.ncells + 255) / 256, 256, 0, H.stream>>>(H.gridptr.p, P.ncells, sc.p, H.nbscat.p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(H.stream));
    H.launches += 1;
    H.wready.alloc(2);
    H.wready.zero(H.stream);
  }
  H.tms_ptr.upload(P.tms_ptr); H.tms_iph.upload(P.tms_iph); H.tms_w.upload(P.tms_w);
  H.phasetab.upload(P.phasetab); H.botalb.upload(P.botalb); H.rad0.upload(P.rad0);
  H.thermal.upload(P.thermal); H.botplanck.upload(P.botplanck); H.planckpt.upload(P.planckpt);
  if (H.nst == 3) { H.col_stk.upload(P.col_stk); H.coefp.upload(P.coefp); H.phasetab2.upload(P.phasetab2); }
  if (P.brdf) {
    static_assert(sizeof(BrdfOrd) == sizeof(Plan::BrdfOrd), "BRDF ordinate records");
    H.botpar.upload(P.botpar);
    std::vector<BrdfOrd> dn(P.brdf_dn.size()), up(P.brdf_up.size());
    std::memcpy(dn.data(), P.brdf_dn.data(), dn.size() * sizeof(BrdfOrd));
    std::memcpy(up.data(), P.brdf_up.data(), up.size() * sizeof(BrdfOrd));
    H.brdf_dn.upload(dn); H.brdf_up.upload(up);
  }
  H.ldo = (P.nang + 3) & ~3;
  const size_t nf = (size_t)P.npts * H.nst * P.nlm, nd = (size_t)P.npts * H.ldo;
  H.source.alloc(nf); H.delsource.alloc(nf); H.radiance.alloc(nf);
  H.srcdo.alloc(nd); H.raddo.alloc(nd);
  H.srcdo.zero(H.stream); H.raddo.zero(H.stream);
  H.fluxes.alloc((size_t)P.npts * 2); H.bcrad.alloc(std::max<size_t>(1, P.botp.size()));
  H.ns.alloc(P.npts); H.nso.alloc(P.npts); H.nr.alloc(P.npts); H.errflag.alloc(1);
  H.red.alloc(4); H.accel.alloc(1);
  setup_tc(H);
  // the uploads are legacy-stream copies from pageable memory, which may
  // return before their DMA lands; the handle's non-blocking stream is not
  // ordered after them
  CK(cudaStreamSynchronize(cudaStreamLegacy));
}

static void launch_source(Handle &H, int first, int fixsh) {
  Plan &P = H.P;
  SourceArgs a;
  a.coef = H.coef.p; a.dirflux = H.dirflux.p; a.radiance = H.radiance.p; a.ylmsun = H.ylmsun.p; a.lofj = H.lofj.p;
  a.thermal = H.thermal.n ? H.thermal.p : nullptr;
  a.source = H.source.p; a.delsource = H.delsource.p; a.ns = H.ns.p; a.nso = H.nso.p; a.nr = H.nr.p; a.red = H.red.p;
  a.npts = P.npts; a.nlm = P.nlm; a.nl = P.ml + 1; a.ml = P.ml; a.mm = P.mm;
  a.secmu0 = 1.0f / std::fabs(P.prob.solarmu); a.shacc = P.prob.shacc;
  a.first = first; a.fixsh = fixsh; a.accel = P.prob.accelflag; a.highorder = P.prob.highorderrad;
  a.coefp = H.nst == 3 ? H.coefp.p : nullptr;
  CK(cudaMemsetAsync(H.red.p, 0, 4 * sizeof(double), H.stream));
  int blocks = std::min((P.npts + 7) / 8, 152 * 16);
  if (H.nst == 3) k_source_pol<<<blocks, 256, 0, H.stream>>>(a);
  else k_source<<<blocks, 256, 0, H.stream>>>(a);
  H.launches += 1;
  CK(cudaGetLastError());
}

template <int NMU>
static void transforms_launch(Handle &H, int dir) {
  Plan &P = H.P;
  XfArgs x;
  x.cmu = dir == 0 ? H.cmu1t.p : H.cmu2t.p;
  x.cphi = dir == 0 ? H.cphi1t.p : H.cphi2.p;
  x.nphi0 = H.nphi0.p; x.col_of = H.col_of.p; x.fluxw = H.col_fluxw.p; x.nr = H.nr.p; x.fluxes = H.fluxes.p;
  x.npts = P.npts; x.nlm = P.nlm; x.ml = P.ml; x.mm = P.mm; x.nmu = P.nmu; x.nang = P.nang; x.nphi0max = P.nphi0max;
  x.ncol_down = P.ncol_down; x.ldo = H.ldo;
  const int nm = 2 * P.mm + 1;
  size_t smem = (size_t)P.nlm * (NMU + 1) * sizeof(float) + 8 * sizeof(float) * (dir == 0 ? (size_t)NMU * nm : (size_t)P.nang);
  int blocks = std::min((P.npts + 7) / 8, 152 * 8);
  if (dir == 0) {
    CK(cudaFuncSetAttribute(k_sh_to_do<NMU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_sh_to_do<NMU><<<blocks, 256, smem, H.stream>>>(x, H.source.p, H.srcdo.p);
  } else {
    CK(cudaFuncSetAttribute(k_do_to_sh<NMU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_do_to_sh<NMU><<<blocks, 256, smem, H.stream>>>(x, H.raddo.p, H.radiance.p);
  }
  CK(cudaGetLastError());
  H.launches += 1;
}

// dir 0: SOURCE -> SRCDO (with the non-negativity clamp); dir 1: RADDO ->
// RADIANCE (masked to the radiance truncation) and the hemispheric fluxes.
static void transform(Handle &H, int dir) {
  const int nsh = H.nst * H.P.nlm;
  if (H.xf_mode != 2 && H.tc_ok[dir]) {
    Plan &P = H.P;
    tc::Epilogue g{};
    g.M = P.npts; g.err = H.errflag.p; g.split = H.xf_mode == 0 ? 1 : 0;
    g.wait_limit = H.tc_wait_limit;
    if (dir == 0) {
      g.N = P.nang; g.mode = 0; g.C = H.srcdo.p; g.ldc = H.ldo;
      g.stk = H.nst == 3 ? H.col_stk.p : nullptr;
    } else {
      g.N = nsh; g.mode = 1; g.R = H.radiance.p; g.nlm = P.nlm; g.ldr = nsh; g.nr = H.nr.p; g.fluxes = H.fluxes.p;
      g.fluxw = H.col_fluxw.p; g.ncol_down = P.ncol_down;
    }
    const int ntn = H.tc_ntiles[dir];
    if (H.compact) {
      // the scattering points' rows, gathered; the rest on the CUDA cores (ordinate-to-harmonic) or zero (source)
      g.rowmap = H.heavy.p;
      g.M = H.nheavy;
      const int rowlen = dir == 0 ? P.nlm : H.ldo;
      if (H.nheavy > 0) {
        const long long q = (long long)H.nheavy * (rowlen / 4);
        const int gb = (int)std::min<long long>((q + 255) / 256, 152 * 16);
        k_gather_rows<<<gb, 256, 0, H.stream>>>(dir == 0 ? H.source.p : H.raddo.p, H.heavy.p, H.nheavy, rowlen,
                                                 dir == 0 ? H.src_c.p : H.rad_c.p);
        CK(cudaGetLastError());
        const int ntiles = ntn * ((H.nheavy + tc::BM - 1) / tc::BM);
        tc_launch(H.tc_bn[dir], H.nsm, H.stream, H.tm_ac[dir], H.tm_bh[dir], H.tm_bl[dir], dir == 0 ? P.nlm : P.nang,
                  ntn, ntiles, g);
        CK(cudaGetLastError());
        H.launches += 1;
      }
      if (dir == 1 && H.nlight > 0) {
        const int lb = std::min((H.nlight + 7) / 8, 152 * 16);
        k_do_to_sh_light<<<lb, 256, 6 * H.ldo * sizeof(float), H.stream>>>(H.raddo.p, H.ldo, P.nang, P.ncol_down, H.light.p, H.nlight, H.t4.p,
                                                    H.col_fluxw.p, H.radiance.p, P.nlm, H.fluxes.p);
        CK(cudaGetLastError());
        H.launches += 1;
      }
      H.launches += 1;
      return;
    }
    const int ntiles = ntn * ((P.npts + tc::BM - 1) / tc::BM);
    tc_launch(H.tc_bn[dir], H.nsm, H.stream, H.tm_a[dir], H.tm_bh[dir], H.tm_bl[dir], dir == 0 ? nsh : P.nang, ntn,
              ntiles, g);
    CK(cudaGetLastError());
    H.launches += 1;
    return;
  }
  if (H.nst == 3) {  // FP32 dense transforms on the CUDA cores
    Plan &P = H.P;
    const int K = dir == 0 ? nsh : P.nang, N = dir == 0 ? P.nang : nsh;
    const dim3 grid((N + 63) / 64, (P.npts + 63) / 64);
    if (dir == 0)
      k_dense_xf<<<grid, 256, 0, H.stream>>>(H.source.p, nsh, H.pol_t[0].p, K, N, P.npts, 0, H.srcdo.p, H.ldo,
                                              H.col_stk.p, nullptr, P.nlm);
    else
      k_dense_xf<<<grid, 256, 0, H.stream>>>(H.raddo.p, H.ldo, H.pol_t[1].p, K, N, P.npts, 1, H.radiance.p, nsh,
                                              nullptr, H.nr.p, P.nlm);
    CK(cudaGetLastError());
    H.launches += 1;
    if (dir == 1) {
      const int fb = std::min((P.npts + 7) / 8, 152 * 16);
      k_do_fluxes<<<fb, 256, 0, H.stream>>>(H.raddo.p, H.ldo, P.nang, P.ncol_down, H.col_fluxw.p, P.npts, H.fluxes.p);
      CK(cudaGetLastError());
      H.launches += 1;
    }
    return;
  }
  const int nmu = H.P.nmu;
  if (nmu <= 8) transforms_launch<8>(H, dir);
  else if (nmu <= 16) transforms_launch<16>(H, dir);
  else transforms_launch<32>(H, dir);
}

static SweepArgs sweep_args(Handle &H, int hemi) {
  Plan &P = H.P;
  SweepArgs a;
  a.gridpos = H.gridpos.p; a.gridptr = H.gridptr.p; a.neighptr = H.neighptr.p; a.cellflags = H.cellflags.p;
  a.bnd = H.bnd.p; a.rank = H.rank.p; a.start = H.start.p; a.level = H.level.p; a.text = H.text.p;
  a.srcdo = H.srcdo.p; a.raddo = H.raddo.p; a.col_cx = H.col_cx.p; a.col_cy = H.col_cy.p; a.col_cz = H.col_cz.p;
  a.tasks = H.tasks[hemi].p; a.err = H.errflag.p; a.npts = P.npts; a.nang = P.nang; a.ldo = H.ldo; a.is1d = P.is1d;
  a.regular = H.regular.p; a.geo = H.geo.p; a.nz = P.nz; a.ny1 = P.ny1; a.nx1 = P.nx1;
  a.transmin = P.prob.transmin;
  a.irr = H.irr[hemi].p;
  a.stk = H.nst == 3 ? H.col_stk.p : nullptr;
  for (int b = 0; b < 8; ++b) { a.oct_col0[b] = P.oct_col0[b]; a.oct_ncol[b] = P.oct_ncol[b]; }
  return a;
}

// Stored single-cell general traces of both hemispheres (once per handle;
// they depend on the geometry and the sweep schedule only).
static void build_irr(Handle &H) {
  Plan &P = H.P;
  {  // once per shared geometry (the records depend on the grid and schedule only)
    DevGeom &G = *H.geom;
    std::lock_guard<std::mutex> lk(G.mu);
    if (!G.irr_built) {
      for (int h = 0; h < 2; ++h) {
        G.irr[h].alloc((size_t)std::max<long long>(P.nirr[h], 1));
        H.irr[h].view(G.irr[h]);
        if (P.nirr[h] == 0 || H.n_irrseg[h] == 0 || H.seq[h]) continue;
        SweepArgs a = sweep_args(H, h);
        const int nirr = (int)P.nirr[h];
        const int blocks = std::min((nirr + 255) / 256, 152 * 16);
        k_irr_build<<<blocks, 256, 0, H.stream>>>(a, H.irrsegs[h].p, H.n_irrseg[h], nirr, G.irr[h].p);
        CK(cudaGetLastError());
        H.launches += 1;
      }
      CK(cudaStreamSynchronize(H.stream));
      G.irr_built = true;
    }
    for (int h = 0; h < 2; ++h) H.irr[h].view(G.irr[h]);
  }
  setup_march(H);
  setup_p1s(H);
  if ((!H.march[0] && !H.seq[0] && P.seg_off[0].size() > 1) || (!H.march[1] && !H.seq[1] && P.seg_off[1].size() > 1))
    H.sweepw.alloc((size_t)P.npts * H.ldo);
  {  // phase-1 trace records ahead of the plane march
    int n1 = 0;
    for (int h = 0; h < 2; ++h)
      if (H.march[h]) n1 = std::max(n1, H.p2_irr_j0[h]);
    if (n1) H.p1rec.alloc((size_t)n1);
  }
  {  // trace records of the reference-order sweep, sized for its larger hemisphere
    size_t nrec = 0;
    for (int h = 0; h < 2; ++h)
      if (H.seq[h]) nrec = std::max(nrec, (size_t)P.npts * (h ? P.nang - P.ncol_down : P.ncol_down));
    if (nrec) H.seqrec.alloc(nrec);
  }
  {  // phase 1 runs on a high-priority stream so its blocks start before the source pass fills the SMs
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CK(cudaStreamCreateWithPriority(&H.stream2, cudaStreamNonBlocking, hi));
  }
  CK(cudaEventCreateWithFlags(&H.ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&H.ev_join, cudaEventDisableTiming));
  for (auto &hs : H.ev_k)
    for (auto &e : hs) CK(cudaEventCreate(&e));
}

static void sweep_hemisphere(Handle &H, int hemi) {
  Plan &P = H.P;
  SweepArgs a = sweep_args(H, hemi);
  H.ktime_rec[hemi] = H.ktime_on;
  if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][0], H.stream));
  if (H.seq[hemi]) {
    const int c0 = hemi ? P.ncol_down : 0, nc = hemi ? P.nang - P.ncol_down : P.ncol_down;
    if (nc > 0) {
      const long long total = (long long)nc * P.npts;
      const int blocks = (int)std::min<long long>((total + 255) / 256, (long long)H.nsm * 8);
      k_seq_prep<<<blocks, 256, 0, H.stream>>>(a, H.order.p, c0, nc, H.seqrec.p);
      CK(cudaGetLastError());
      k_sweep_seq<<<nc, SEQW, 0, H.stream>>>(a, H.order.p, c0, H.seqrec.p);
      CK(cudaGetLastError());
      H.launches += 2;
    }
    if (H.ktime_on) {
      CK(cudaEventRecord(H.ev_k[hemi][1], H.stream));
      CK(cudaEventRecord(H.ev_k[hemi][2], H.stream));
    }
    return;
  }
  const std::vector<int> &off = P.seg_off[hemi];
  const int nlev = (int)off.size() - 1;
  const int ng1 = (int)P.p1off[hemi].size() - 1;
  if (H.march[hemi] && !H.march_off) {
    // phase 1 (the boundary-plane chains: their traces in one parallel pass,
    // then the levels), then the plane march of phase 2
    if (ng1 > 0) {
      const int n1 = H.p2_irr_j0[hemi];
      const int blocks = std::min((n1 + 255) / 256, H.nsm * 8);
      if (H.p1s[hemi]) {
        if (n1 > 0) {
          k_p1_prep_s<<<blocks, 256, 0, H.stream>>>(a, H.irrsegs[hemi].p, H.p2_irrseg0[hemi], n1, H.p1grp[hemi].p,
                                                    H.p1slot[hemi].p, H.p1rec.p);
          CK(cudaGetLastError());
          H.launches += 1;
        }
        k_sweep_p1s<<<H.np1blk[hemi], P1S_THREADS, H.p1smem[hemi], H.stream>>>(
            a, H.p1segs[hemi].p, H.p1off[hemi].p, H.p1blk[hemi].p, H.p1base[hemi].p, H.p1rec.p);
      } else {
        if (n1 > 0) {
          k_p1_prep<<<blocks, 256, 0, H.stream>>>(a, H.irrsegs[hemi].p, H.p2_irrseg0[hemi], n1, H.p1rec.p);
          CK(cudaGetLastError());
          H.launches += 1;
        }
        k_sweep_p1r<<<ng1 * P1_SPLIT, P1_THREADS, 0, H.stream>>>(a, H.p1segs[hemi].p, H.p1off[hemi].p, H.p1rec.p);
      }
      CK(cudaGetLastError());
      H.launches += 1;
    }
    if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][1], H.stream));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = H.mcs[hemi]; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(H.mnunits[hemi] * H.mcs[hemi])); cfg.blockDim = dim3(MT);
    cfg.dynamicSmemBytes = H.msmem[hemi]; cfg.stream = H.stream; cfg.attrs = at; cfg.numAttrs = 1;
    const MarchGrp *gp = H.mgrp[hemi].p;
    const MarchUnit *up = H.munit[hemi].p;
    CK(cudaLaunchKernelEx(&cfg, k_sweep_march, a, gp, up));
    H.launches += 1;
    if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][2], H.stream));
    return;
  }
  // phase 1 on the second stream, after everything queued so far
  if (ng1 > 0) {
    CK(cudaEventRecord(H.ev_fork, H.stream));
    CK(cudaStreamWaitEvent(H.stream2, H.ev_fork, 0));
    k_sweep_p1<<<ng1 * P1_SPLIT, P1_THREADS, 0, H.stream2>>>(a, H.p1segs[hemi].p, H.p1off[hemi].p);
    CK(cudaGetLastError());
    CK(cudaEventRecord(H.ev_join, H.stream2));
    H.launches += 1;
  }
  // source pass of the phase-2 items
  if (nlev > 0) {
    const int c0 = hemi ? P.ncol_down : 0, nc = hemi ? P.nang - P.ncol_down : P.ncol_down;
    const long long total = (long long)P.npts * nc;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 152 * 16);
    k_sweep_prep<<<blocks, 256, 0, H.stream>>>(a, H.kind.p, H.col_oct.p, H.col_cls.p, c0, nc, H.sweepw.p, H.nbscat.p,
                                                H.wready.p + hemi);
    CK(cudaMemsetAsync(H.wready.p + hemi, 0xff, sizeof(int), H.stream));
    CK(cudaGetLastError());
    H.launches += 1;
    const int n2 = (int)P.nirr[hemi] - H.p2_irr_j0[hemi];
    if (n2 > 0) {
      const int b2 = std::min((n2 + 255) / 256, 152 * 16);
      k_sweep_prep_irr<<<b2, 256, 0, H.stream>>>(a, H.irrsegs[hemi].p, H.n_irrseg[hemi], H.p2_irr_j0[hemi], n2,
                                                   H.sweepw.p, H.irr[hemi].p);
      CK(cudaGetLastError());
      H.launches += 1;
    }
  }
  if (ng1 > 0) CK(cudaStreamWaitEvent(H.stream, H.ev_join, 0));
  if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][1], H.stream));
  if (nlev <= 0) {
    if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][2], H.stream));
    return;
  }
  if (H.coop_blocks > 0 && H.sweep_mode == 0) {  // (graph mode never takes the cooperative path)
    const Seg *sp = H.segs[hemi].p;
    const int *so = H.seg_off[hemi].p, *li = H.level_items[hemi].p;
    const float2 *wp = H.sweepw.p;
    int nl = nlev;
    void *args[] = {&a, (void *)&sp, (void *)&so, (void *)&li, (void *)&wp, &nl};
    CK(cudaLaunchCooperativeKernel((const void *)k_sweep_levels, dim3(H.coop_blocks), dim3(256), args, 0, H.stream));
    H.launches += 1;
    if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][2], H.stream));
    return;
  }
  for (int l = 0; l < nlev; ++l) {
    const int items = P.level_items[hemi][l];
    if (items <= 0) continue;
    int blocks = std::min((items + 511) / 512, 152 * 8);
    k_sweep<<<blocks, 256, 0, H.stream>>>(a, H.segs[hemi].p + off[l], off[l + 1] - off[l], items, H.sweepw.p);
    H.launches += 1;
  }
  CK(cudaGetLastError());
  if (H.ktime_on) CK(cudaEventRecord(H.ev_k[hemi][2], H.stream));
}

static int check_device_error(Handle &H) {
  int e = 0;
  CK(cudaMemcpy(&e, H.errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e == ERR_NONE) return 0;
  const char *m = "device error";
  if (e == ERR_SWEEP_NOFACE) m = "BACK_INT_GRID3D: INEXTCELL=0 (no valid face for a boundary trace)";
  if (e == ERR_SWEEP_STEPS) m = "BACK_INT_GRID: trace exceeded the step limit";
  if (e == ERR_RAY_SO) m = "INTEGRATE_1RAY: SO<0";
  if (e == ERR_RAY_BELOW) m = "RENDER: Level below domain";
  if (e == ERR_TC_WAIT) m = "tensor-core transform: pipeline wait expired";
  H.err = m;
  CK(cudaMemsetAsync(H.errflag.p, 0, sizeof(int), H.stream));
  CK(cudaStreamSynchronize(H.stream));
  return 1;
}

}  // namespace shdom

using shdom::Handle;

struct shdom_handle {
  Handle h;
  ~shdom_handle() {
    // the state's buffers go back to the pool after this body: first let every
    // stream that used them finish (the handle's two, and a caller's stream
    // that a device-buffer render ran on)
    if (h.stream) cudaStreamSynchronize(h.stream);
    if (h.stream2) cudaStreamSynchronize(h.stream2);
    if (h.ev_ext) cudaEventSynchronize(h.ev_ext);
    for (auto &g : h.iter_graph)
      if (g) cudaGraphExecDestroy(g);
    if (h.ev_ext) cudaEventDestroy(h.ev_ext);
    if (h.stream) cudaStreamDestroy(h.stream);
    if (h.stream2) cudaStreamDestroy(h.stream2);
    if (h.ev_fork) cudaEventDestroy(h.ev_fork);
    if (h.ev_join) cudaEventDestroy(h.ev_join);
    for (auto &e : h.ev_caller)
      if (e) cudaEventDestroy(e);
    for (auto &hs : h.ev_k)
      for (auto &e : hs)
        if (e) cudaEventDestroy(e);
  }
};

struct shdom_plan {
  shdom::Plan P;
};

static thread_local std::string g_static_err;

static int fail(shdom_handle *h, const std::string &m) {
  if (h) h->h.err = m; else g_static_err = m;
  return 1;
}

namespace shdom {
// Error return of the host-only entry points (no handle): the message is read
// back with shdom_last_error(NULL) on the same thread.
int host_fail(const std::string &m) { return fail(nullptr, m); }
}  // namespace shdom

// Makes a handle's device current for the length of an entry point and puts
// the caller's current device back afterwards, so that a handle created on
// one device can be used from a thread whose current device is another.
struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
  }
  ~DevGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Device staging memory of one host-buffer call, freed on every return path.
// A call's temporary device buffer; the call synchronizes the streams that
// used it before returning.
struct CallMem {
  void *p = nullptr;
  int dev = -1;
  void alloc(size_t bytes) { p = shdom::dev_alloc(bytes, dev); }
  ~CallMem() { shdom::dev_free(p, dev); }
};

extern "C" {

// Device part of shdom_create: H->h.P holds a finished host plan.
static int create_on_device(std::unique_ptr<shdom_handle> &H, int device, shdom_handle **out) {
  try {
    if (device >= 0) CK(cudaSetDevice(device));
    CK(cudaGetDevice(&H->h.device));
    CK(cudaStreamCreateWithFlags(&H->h.stream, cudaStreamNonBlocking));
    shdom::upload_plan(H->h);
    CK(cudaMemsetAsync(H->h.errflag.p, 0, sizeof(int), H->h.stream));
    shdom::build_irr(H->h);
  } catch (const std::exception &e) {
    return fail(nullptr, e.what());
  }
  *out = H.release();
  return 0;
}

int shdom_create(const shdom_problem *problem, int device, shdom_handle **out) {
  if (!problem || !out) return fail(nullptr, "shdom_create: null argument");
  *out = nullptr;
  std::unique_ptr<shdom_handle> H(new shdom_handle());
  try {
    if (!shdom::build_plan(*problem, H->h.P)) return fail(nullptr, H->h.P.err);
  } catch (const std::exception &e) {
    return fail(nullptr, e.what());
  }
  return create_on_device(H, device, out);
}

int shdom_plan_create(const shdom_problem *problem, shdom_plan **out, shdom_sizes *sizes) {
  if (!problem || !out) return fail(nullptr, "shdom_plan_create: null argument");
  *out = nullptr;
  if (sizes) std::memset(sizes, 0, sizeof(*sizes));
  std::unique_ptr<shdom_plan> p(new shdom_plan());
  try {
    if (!shdom::build_plan(*problem, p->P)) return fail(nullptr, p->P.err);
    // the plan keeps copies of everything it uses; drop the caller's array pointers
    shdom_problem &pr = p->P.prob;
    pr.zlevels = nullptr; pr.extinctp = nullptr; pr.albedop = nullptr; pr.iphasep = nullptr;
    pr.phasewtp = nullptr; pr.legenp = nullptr; pr.sfc_albedo = nullptr; pr.sfc_params = nullptr;
    pr.tempp = nullptr; pr.sfc_temp = nullptr;
    if (sizes) {
      shdom::fill_sizes(p->P, sizes);
      sizes->solcrit = 1.f;
    }
  } catch (const std::exception &e) {
    return fail(nullptr, e.what());
  }
  *out = p.release();
  return 0;
}

int shdom_create_planned(shdom_plan *plan, int device, shdom_handle **out) {
  std::unique_ptr<shdom_plan> p(plan);  // released by this call in every case
  if (!plan || !out) return fail(nullptr, "shdom_create_planned: null argument");
  *out = nullptr;
  std::unique_ptr<shdom_handle> H(new shdom_handle());
  H->h.P = std::move(p->P);
  p.reset();
  return create_on_device(H, device, out);
}

void shdom_plan_destroy(shdom_plan *plan) { delete plan; }

int shdom_plan_optical_path(const shdom_plan *plan, int nrays, const float *camx, const float *camy,
                            const float *camz, const double *cammu, const double *camphi, int deltam_path,
                            float *path_out) {
  if (!plan) return fail(nullptr, "shdom_plan_optical_path: null plan");
  std::string err;
  if (!shdom::optical_path(plan->P, nrays, camx, camy, camz, cammu, camphi, deltam_path, path_out, err))
    return fail(nullptr, err);
  return 0;
}

int shdom_plan_min_optical_path(const shdom_plan *plan, int nrays, const float *camx, const float *camy,
                                const float *camz, const double *cammu, const double *camphi, int deltam_path,
                                int do_all, float *minpath_out) {
  if (!plan) return fail(nullptr, "shdom_plan_min_optical_path: null plan");
  std::string err;
  if (!shdom::min_optical_path(plan->P, nrays, camx, camy, camz, cammu, camphi, deltam_path, do_all, minpath_out, err))
    return fail(nullptr, err);
  return 0;
}

int shdom_plan_point_absorption(const shdom_plan *plan, float *absorb, float *emit) {
  if (!plan) return fail(nullptr, "shdom_plan_point_absorption: null plan");
  std::string err;
  if (!shdom::point_absorption(plan->P, absorb, emit, err)) return fail(nullptr, err);
  return 0;
}

int shdom_point_absorption(shdom_handle *h, float *absorb, float *emit) {
  if (!h) return fail(nullptr, "shdom_point_absorption: null handle");
  std::string err;
  if (!shdom::point_absorption(h->h.P, absorb, emit, err)) return fail(h, err);
  return 0;
}

int shdom_optical_path(shdom_handle *h, int nrays, const float *camx, const float *camy, const float *camz,
                       const double *cammu, const double *camphi, int deltam_path, float *path_out) {
  if (!h) return fail(nullptr, "shdom_optical_path: null handle");
  std::string err;
  if (!shdom::optical_path(h->h.P, nrays, camx, camy, camz, cammu, camphi, deltam_path, path_out, err))
    return fail(h, err);
  return 0;
}

int shdom_init_solution(shdom_handle *hh) {
  if (!hh) return fail(nullptr, "null handle");
  Handle &H = hh->h;
  DevGuard dg(H.device);
  try {
    shdom::Plan &P = H.P;
    size_t tot = (size_t)P.npts * H.nst * P.nlm;
    int blocks = (int)std::min<size_t>((tot + 255) / 256, 152 * 64);
    shdom::k_init_radiance<<<blocks, 256, 0, H.stream>>>(H.rad0.p, H.radiance.p, H.nr.p, P.npts, P.nlm, H.nst);
    H.launches += 1;
    CK(cudaMemsetAsync(H.source.p, 0, tot * sizeof(float), H.stream));
    CK(cudaMemsetAsync(H.delsource.p, 0, tot * sizeof(float), H.stream));
    CK(cudaMemsetAsync(H.ns.p, 0, P.npts * sizeof(int), H.stream));
    CK(cudaMemsetAsync(H.nso.p, 0, P.npts * sizeof(int), H.stream));
    CK(cudaMemsetAsync(H.fluxes.p, 0, (size_t)P.npts * 2 * sizeof(float), H.stream));
    shdom::AccelState st{0.0, 1.0f, 0.0f};
    CK(cudaMemcpyAsync(H.accel.p, &st, sizeof(st), cudaMemcpyHostToDevice, H.stream));
    shdom::launch_source(H, 1, 0);
    CK(cudaStreamSynchronize(H.stream));
    H.initialized = true;
    H.iters = 0;
    H.solcrit = 1.f;
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

int shdom_solution_iterations(shdom_handle *hh, int maxiter, int *iters, float *solcrit) {
  if (!hh) return fail(nullptr, "null handle");
  Handle &H = hh->h;
  DevGuard dg(H.device);
  if (!H.initialized) {
    int rc = shdom_init_solution(hh);
    if (rc) return rc;
  }
  try {
    shdom::Plan &P = H.P;
    cudaEvent_t ev[6];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (float &t : H.timings) t = 0.f;
    H.ktimes[0] = H.ktimes[1] = 0.f;
    H.klaunches[0] = H.klaunches[1] = 0;
    bool fixsh = false;
    const int nlm = P.nlm, nang = P.nang;
    {  // SOLUTION_ITERATIONS starts every call with no acceleration pending
      double zero = 0.0;
      CK(cudaMemcpyAsync(&H.accel.p->a, &zero, sizeof(double), cudaMemcpyHostToDevice, H.stream));
    }
    // one iteration's launches; with timing, events between the phases
    auto body = [&](bool fix, bool timed) {
      if (timed) CK(cudaEventRecord(ev[0], H.stream));
      shdom::transform(H, 0);
      if (timed) CK(cudaEventRecord(ev[1], H.stream));
      int ntop = (int)P.topp.size(), nbot = (int)P.botp.size();
      if (ntop && P.ncol_down) {
        int t = ntop * P.ncol_down;
        shdom::k_preset_top<<<(t + 255) / 256, 256, 0, H.stream>>>(H.topp.p, ntop, H.raddo.p, H.ldo, P.ncol_down, P.skyrad_bc,
                                                                   H.nst == 3 ? H.col_stk.p : nullptr);
        H.launches += 1;
      }
      shdom::sweep_hemisphere(H, 0);
      if (nbot && P.brdf) {
        shdom::k_brdf_bottom<<<nbot, 128, 0, H.stream>>>(H.botp.p, nbot, H.botpar.p, P.nsfcpar, P.brdf, H.brdf_dn.p,
                                                          (int)P.brdf_dn.size(), H.brdf_up.p, (int)P.brdf_up.size(),
                                                          H.dirflux.p, P.prob.solarmu, P.prob.solaraz, H.raddo.p, H.ldo,
                                                          H.nst, H.botplanck.n ? H.botplanck.p : nullptr);
        H.launches += 1;
      } else if (nbot) {
        shdom::k_lambertian<<<nbot, 256, 0, H.stream>>>(H.botp.p, nbot, H.botalb.p, H.dirflux.p, H.col_fluxw.p, H.raddo.p,
                                                         nang, H.ldo, P.ncol_down, H.bcrad.p, H.nst == 3 ? H.col_stk.p : nullptr,
                                                         H.botplanck.n ? H.botplanck.p : nullptr);
        H.launches += 1;
      }
      shdom::sweep_hemisphere(H, 1);
      if (timed) CK(cudaEventRecord(ev[2], H.stream));
      shdom::transform(H, 1);
      if (timed) CK(cudaEventRecord(ev[3], H.stream));
      shdom::launch_source(H, 0, fix ? 1 : 0);
      shdom::k_accel_param<<<1, 1, 0, H.stream>>>(H.red.p, H.accel.p, P.prob.accelflag);
      H.launches += 2;
      int blocks = (int)std::min<size_t>(((size_t)P.npts * H.nst * nlm + 255) / 256, 152 * 64);
      shdom::k_accelerate<<<blocks, 256, 0, H.stream>>>(H.source.p, H.delsource.p, H.ns.p, H.nso.p, P.npts, nlm, H.accel.p,
                                                        H.nst);
    };
    const bool graphed = H.sweep_mode == 2;
    while (H.iters < maxiter && H.solcrit > P.prob.solacc) {
      ++H.iters;
      if (H.solcrit < 0.001f || H.iters > P.prob.iterfixsh) fixsh = true;
      if (graphed) {
        const int gi = fixsh ? 1 : 0;
        if (!H.iter_graph[gi]) {
          // capture only this thread's launches, so that other threads' handles keep working
          const long long l0 = H.launches;
          cudaGraph_t g = nullptr;
          CK(cudaStreamBeginCapture(H.stream, cudaStreamCaptureModeThreadLocal));
          body(fixsh, false);
          CK(cudaStreamEndCapture(H.stream, &g));
          const cudaError_t ie = cudaGraphInstantiate(&H.iter_graph[gi], g, 0);
          cudaGraphDestroy(g);
          CK(ie);
          H.iter_graph_launches[gi] = H.launches - l0;
          H.launches = l0;
        }
        CK(cudaEventRecord(ev[0], H.stream));
        CK(cudaGraphLaunch(H.iter_graph[gi], H.stream));
        H.launches += H.iter_graph_launches[gi];
        // graph mode: the whole iteration counts as the first phase
        CK(cudaEventRecord(ev[1], H.stream));
        CK(cudaEventRecord(ev[2], H.stream));
        CK(cudaEventRecord(ev[3], H.stream));
      } else {
        H.ktime_on = true;
        body(fixsh, true);
        H.ktime_on = false;
      }
      CK(cudaEventRecord(ev[4], H.stream));
      shdom::AccelState st;
      CK(cudaMemcpyAsync(&st, H.accel.p, sizeof(st), cudaMemcpyDeviceToHost, H.stream));
      CK(cudaStreamSynchronize(H.stream));
      if (shdom::check_device_error(H)) { for (auto &e : ev) cudaEventDestroy(e); return 1; }
      H.solcrit = st.solcrit;
      if (P.albmax < P.prob.solacc) H.solcrit = P.prob.solacc;
      float t01, t12, t23, t34;
      CK(cudaEventElapsedTime(&t01, ev[0], ev[1])); CK(cudaEventElapsedTime(&t12, ev[1], ev[2]));
      CK(cudaEventElapsedTime(&t23, ev[2], ev[3])); CK(cudaEventElapsedTime(&t34, ev[3], ev[4]));
      H.timings[0] += t01; H.timings[1] += t12; H.timings[2] += t23; H.timings[3] += t34;
      H.timings[4] += t01 + t12 + t23 + t34;  // (graph mode: the whole iteration is in the first entry)
      for (int h = 0; h < 2; ++h) {
        if (!H.ktime_rec[h]) continue;
        float a0, a1;
        CK(cudaEventElapsedTime(&a0, H.ev_k[h][0], H.ev_k[h][1]));
        CK(cudaEventElapsedTime(&a1, H.ev_k[h][1], H.ev_k[h][2]));
        H.ktimes[0] += a0; H.ktimes[1] += a1;
        H.klaunches[0] += 1; H.klaunches[1] += 1;
        H.ktime_rec[h] = false;
      }
    }
    for (auto &e : ev) cudaEventDestroy(e);
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  if (iters) *iters = H.iters;
  if (solcrit) *solcrit = H.solcrit;
  return 0;
}

static shdom::RenderArgs render_args(Handle &H, int nrays, const float *camx, const float *camy, const float *camz,
                                     const double *cammu, const double *camphi, float *out) {
  shdom::Plan &P = H.P;
  shdom::RenderArgs a;
  a.gridpos = H.gridpos.p; a.xgrid = H.xgrid.p; a.ygrid = H.ygrid.p; a.zgrid = H.zgrid.p;
  a.gridptr = H.gridptr.p; a.neighptr = H.neighptr.p; a.cellflags = H.cellflags.p;
  a.text = H.text.p; a.source = H.source.p; a.coef = H.coef.p; a.dirflux = H.dirflux.p;
  a.ns = H.ns.p; a.lofj = H.lofj.p; a.tms_ptr = H.tms_ptr.p; a.tms_iph = H.tms_iph.p; a.tms_w = H.tms_w.p;
  a.phasetab = H.phasetab.p; a.ylmsun = H.ylmsun.p; a.botp = H.botp.p; a.bcrad_bot = H.bcrad.p;
  a.bot_index = H.bot_index.p; a.camx = camx; a.camy = camy; a.camz = camz; a.cammu = cammu; a.camphi = camphi;
  a.out = out; a.err = H.errflag.p; a.nrays = nrays; a.nx = P.nx; a.ny = P.ny; a.nz = P.nz; a.nlm = P.nlm;
  a.nl = P.ml + 1; a.ml = P.ml; a.mm = P.mm; a.bcflag = P.bcflag; a.ipflag = P.ipflag; a.numphase = P.numphase;
  a.nscatangle = P.nscatangle; a.deltam = P.prob.deltam; a.solarmu = P.prob.solarmu; a.solaraz = P.prob.solaraz;
  a.secmu0 = 1.0f / std::fabs(P.prob.solarmu); a.skyrad = P.skyrad_bc; a.tautol = P.prob.tautol;
  a.botplanck = H.botplanck.n ? H.botplanck.p : nullptr;
  a.transcut = P.prob.transcut;
  a.coefp = H.nst == 3 ? H.coefp.p : nullptr;
  a.phasetab2 = H.nst == 3 ? H.phasetab2.p : nullptr;
  a.brdf = P.brdf; a.nsfcpar = P.nsfcpar; a.nbrdf_dn = (int)P.brdf_dn.size(); a.ldo = H.ldo;
  a.botpar = H.botpar.p; a.raddo = H.raddo.p; a.brdf_dn = H.brdf_dn.p;
  return a;
}

// Bottom-boundary radiance of the Lambertian surface from the solved fluxes
// (what the render and the adjoint read at the ground).
static void bcrad_update(Handle &H, cudaStream_t stream) {
  const int nbot = (int)H.P.botp.size();
  if (!nbot) return;
  shdom::k_bcrad_bottom<<<(nbot + 127) / 128, 128, 0, stream>>>(H.botp.p, nbot, H.botalb.p, H.dirflux.p, H.fluxes.p,
                                                                H.bcrad.p, H.botplanck.n ? H.botplanck.p : nullptr);
  H.launches += 1;
}

static int render_impl(shdom_handle *hh, int nrays, const float *camx, const float *camy, const float *camz,
                       const double *cammu, const double *camphi, float *out, cudaStream_t stream) {
  Handle &H = hh->h;
  shdom::Plan &P = H.P;
  bcrad_update(H, stream);
  shdom::RenderArgs a = render_args(H, nrays, camx, camy, camz, cammu, camphi, out);
  a.single_scatter = H.render_single_scatter; a.nosurface = H.render_nosurface;
  if (P.nlm > shdom::RNLM || P.ml + 1 > 64) return fail(hh, "render: too many spherical-harmonic terms");
  int blocks = (nrays + shdom::RWARPS - 1) / shdom::RWARPS;
  if (blocks > 0) {
    if (H.nst == 3) {
      const size_t smem = (size_t)shdom::RWARPS * 5 * P.nlm * sizeof(float);
      if (P.brdf) {
        CK(cudaFuncSetAttribute(shdom::k_render_pol<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        shdom::k_render_pol<true><<<blocks, shdom::RWARPS * 32, smem, stream>>>(a);
      } else {
        CK(cudaFuncSetAttribute(shdom::k_render_pol<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        shdom::k_render_pol<false><<<blocks, shdom::RWARPS * 32, smem, stream>>>(a);
      }
    } else if (P.brdf) {
      shdom::k_render<true><<<blocks, shdom::RWARPS * 32, 0, stream>>>(a);
    } else {
      shdom::k_render<false><<<blocks, shdom::RWARPS * 32, 0, stream>>>(a);
    }
    H.launches += 1;
  }
  CK(cudaGetLastError());
  if (stream != H.stream) {  // the handle's buffers are in use on the caller's stream until this event
    if (!H.ev_ext) CK(cudaEventCreateWithFlags(&H.ev_ext, cudaEventDisableTiming));
    CK(cudaEventRecord(H.ev_ext, stream));
  }
  return 0;
}

// Derivative tables of PREPARE_DERIV_INTERPS (src/polarized/shdomsub4.f:
// 2917-3080) and the direction-independent parts of
// COMPUTE_SOURCE_GRAD_1CELL (:1546-2042) for the extinction and albedo of
// species ipa, with the 'table' derivative method (no phase derivative).
static void prepare_grad(Handle &H, int ipa) {
  shdom::Plan &P = H.P;
  const int npx = P.npx, npy = P.npy, npz = P.npz, ng = npx * npy * npz, npts = P.npts;
  const int ml = P.ml, nl = ml + 1, nl1 = P.nleg + 1, nmic = P.maxnmicro;
  const bool deltam = P.prob.deltam != 0;
  const float *E = &P.prop_ext[(size_t)ipa * ng], *A = &P.prop_alb[(size_t)ipa * ng];
  const int *IPH = &P.prop_iph[(size_t)ipa * ng * nmic];
  const float *PHW = &P.prop_phw[(size_t)ipa * ng * nmic];
  auto L = [&](int iph1, int l) { return P.leg[(size_t)(iph1 - 1) * nl1 + l]; };
  std::vector<int> iptr((size_t)npts * 8);
  std::vector<float> owt((size_t)npts * 8);
  for (int ip = 0; ip < npts; ++ip) {  // COMPUTE_INTERP_WEIGHTS
    float x = P.gridpos[3 * ip], y = P.gridpos[3 * ip + 1], z = P.gridpos[3 * ip + 2];
    int il = 0, iu = npz;
    while (iu - il > 1) { int im = (iu + il) / 2; if (z >= P.zgrid[im - 1]) il = im; else iu = im; }
    int iz = std::max(il, 1);
    double w = std::max(0.0, std::min(1.0, (double)(z - P.zgrid[iz - 1]) / (P.zgrid[iz] - P.zgrid[iz - 1])));
    int ix = (int)(x / P.delx) + 1;
    if (std::fabs(x - npx * P.delx) < 0.01f * P.delx) ix = npx;
    int iy = (int)(y / P.dely) + 1;
    if (std::fabs(y - npy * P.dely) < 0.01f * P.dely) iy = npy;
    ix = std::max(1, std::min(npx, ix)); iy = std::max(1, std::min(npy, iy));
    int ixp = ix % npx + 1, iyp = iy % npy + 1;
    double u = std::max(0.0, std::min(1.0, (double)(x - P.delx * (ix - 1)) / P.delx));
    if (u < 1e-5) u = 0;
    if (u > 1 - 1e-5) u = 1;
    double v = std::max(0.0, std::min(1.0, (double)(y - P.dely * (iy - 1)) / P.dely));
    if (v < 1e-5) v = 0;
    if (v > 1 - 1e-5) v = 1;
    const double f[8] = {(1 - u) * (1 - v) * (1 - w), u * (1 - v) * (1 - w), (1 - u) * v * (1 - w), u * v * (1 - w),
                         (1 - u) * (1 - v) * w,       u * (1 - v) * w,       (1 - u) * v * w,       u * v * w};
    int i1 = (iz - 1) + npz * (iy - 1) + npz * npy * (ix - 1), i2 = (iz - 1) + npz * (iy - 1) + npz * npy * (ixp - 1);
    int i3 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ix - 1), i4 = (iz - 1) + npz * (iyp - 1) + npz * npy * (ixp - 1);
    const int ii[8] = {i1, i2, i3, i4, i1 + 1, i2 + 1, i3 + 1, i4 + 1};
    for (int k = 0; k < 8; ++k) { iptr[(size_t)ip * 8 + k] = ii[k]; owt[(size_t)ip * 8 + k] = (float)f[k]; }
  }
  std::vector<float> fp(ng, 0.f), dextm((size_t)ng * 2), legp((size_t)ng * nl, 0.f);
  for (int ib = 0; ib < ng; ++ib) {
    float fv = 0.f;
    if (deltam) for (int q = 0; q < nmic; ++q) fv += PHW[(size_t)ib * nmic + q] * L(IPH[(size_t)ib * nmic + q], ml + 1);
    fp[ib] = fv;
    dextm[(size_t)ib * 2 + 0] = 1.f - fv * A[ib];  // d/d(extinction)
    dextm[(size_t)ib * 2 + 1] = -fv * E[ib];       // d/d(albedo)
    for (int q = 0; q < nmic; ++q) {
      const int i1 = IPH[(size_t)ib * nmic + q];
      const float w = PHW[(size_t)ib * nmic + q], ft = deltam ? L(i1, ml + 1) : 0.f;
      for (int l = 0; l < nl; ++l) legp[(size_t)ib * nl + l] += w * (L(i1, l) + ft);
    }
  }
  std::vector<float> dalbm((size_t)npts * 16), dfj((size_t)npts * 16), scatj(npts, 0.f), legu((size_t)npts * nl),
      legs((size_t)npts * nl, 0.f), fmix(npts, 0.f), sjw;
  std::vector<int> sjptr(npts + 1, 0), sjiph;
  const float scatmin = (float)P.scatmin;
  std::vector<float> lt(nl + 1);
  for (int ip = 0; ip < npts; ++ip) {
    const size_t o = (size_t)ipa * npts + ip;
    const float F = P.sp_f[o], alb = P.sp_alb[o];
    const float albj = deltam ? alb / (F * (alb - 1.f) + 1.f) : alb;
    const float divide = 1.f / (1.f - albj * F);
    float sc = 0.f;
    for (int nb = 0; nb < 8; ++nb) {
      const int ib = iptr[(size_t)ip * 8 + nb];
      const float FP = fp[ib];
      // d = 0: extinction (DEXT 1, DALB 0); d = 1: albedo (DEXT 0, DALB 1)
      dalbm[((size_t)ip * 8 + nb) * 2 + 0] = divide * (((1.f - F) * (A[ib] - albj) + (albj - 1.f) * A[ib] * (FP - F)));
      dalbm[((size_t)ip * 8 + nb) * 2 + 1] = divide * (((1.f - F) * E[ib] + (albj - 1.f) * E[ib] * (FP - F)));
      dfj[((size_t)ip * 8 + nb) * 2 + 0] = ((FP - F) * A[ib]) / (1.f - F);
      dfj[((size_t)ip * 8 + nb) * 2 + 1] = ((FP - F) * E[ib]) / (1.f - F);
      if (deltam) sc += owt[(size_t)ip * 8 + nb] * A[ib] * E[ib];
    }
    scatj[ip] = sc;
    const float div = sc > scatmin ? sc : scatmin;
    if (deltam) {
      for (int nb = 0; nb < 8; ++nb) {
        const int ib = iptr[(size_t)ip * 8 + nb];
        const float sw = owt[(size_t)ip * 8 + nb] * A[ib] * E[ib];
        if (sw <= 1e-6f) continue;
        for (int q = 0; q < nmic; ++q) {
          const float w = PHW[(size_t)ib * nmic + q];
          if (w <= 1e-6f) continue;
          sjiph.push_back(IPH[(size_t)ib * nmic + q] - 1);
          sjw.push_back(sw * w / div);
        }
      }
    }
    sjptr[ip + 1] = (int)sjiph.size();
    if (P.npart == 1) {
      shdom::species_series(P, ipa, ip, &legu[(size_t)ip * nl]);
    } else {
      std::fill(lt.begin(), lt.end(), 0.f);
      for (int nb = 0; nb < 8; ++nb) {
        const int ib = iptr[(size_t)ip * 8 + nb];
        const float sw = owt[(size_t)ip * 8 + nb] * A[ib] * E[ib];
        if (sw <= 1e-6f) continue;
        for (int q = 0; q < nmic; ++q) {
          const float w = PHW[(size_t)ib * nmic + q];
          if (w <= 1e-6f) continue;
          for (int l = 0; l <= nl; ++l) lt[l] += sw * w * L(IPH[(size_t)ib * nmic + q], l);
        }
      }
      for (int l = 0; l <= nl; ++l) lt[l] /= div;
      float Fm = 0.f;
      if (deltam) { Fm = lt[ml + 1]; for (int l = 0; l < nl; ++l) lt[l] /= (1.f - Fm); }
      fmix[ip] = Fm;
      for (int l = 0; l < nl; ++l) {
        legs[(size_t)ip * nl + l] = lt[l];
        legu[(size_t)ip * nl + l] = deltam ? lt[l] * (1.f - Fm) + Fm : lt[l];
      }
    }
  }
  if (sjiph.empty()) { sjiph.push_back(0); sjw.push_back(0.f); }
  std::vector<float> albsp(P.sp_alb.begin() + (size_t)ipa * npts, P.sp_alb.begin() + (size_t)(ipa + 1) * npts);
  std::vector<float> ep(E, E + ng), ap(A, A + ng), phw(PHW, PHW + (size_t)ng * nmic);
  std::vector<int> piph(IPH, IPH + (size_t)ng * nmic);
  H.g_interpptr.upload(iptr); H.g_optwt.upload(owt); H.g_dextm.upload(dextm); H.g_dalbm.upload(dalbm);
  H.g_dfj.upload(dfj); H.g_albsp.upload(albsp); H.g_sjptr.upload(sjptr); H.g_sjiph.upload(sjiph); H.g_sjw.upload(sjw);
  H.g_legu.upload(legu); H.g_legs.upload(legs); H.g_fmix.upload(fmix); H.g_scatj.upload(scatj); H.g_legp.upload(legp);
  H.g_extp.upload(ep); H.g_albp.upload(ap); H.g_piph.upload(piph); H.g_pphw.upload(phw);
  H.g_grad.alloc((size_t)ng * 2); H.g_beam.alloc(npts);
  CK(cudaStreamSynchronize(cudaStreamLegacy));  // uploads land before the stream's kernels read them
  H.grad_ipa = ipa;
}

// Phases 3 and 4 of the adjoint branch on device-resident rays and weights;
// the gradient is left in H.g_grad.
static void levis_adjoint_device(Handle &H, int nrays, const float *dx, const float *dy, const float *dz,
                                 const double *dmu, const double *dphi, const double *dadj) {
  shdom::Plan &P = H.P;
  shdom::GradArgs G;
  G.r = render_args(H, nrays, dx, dy, dz, dmu, dphi, nullptr);
  G.radiance = H.radiance.p; G.nr = H.nr.p; G.interpptr = H.g_interpptr.p; G.optinterpwt = H.g_optwt.p;
  G.dextm = H.g_dextm.p; G.dalbm = H.g_dalbm.p; G.dfj = H.g_dfj.p; G.alb_sp = H.g_albsp.p;
  G.planck = H.planckpt.n ? H.planckpt.p : nullptr;
  G.sj_ptr = H.g_sjptr.p; G.sj_iph = H.g_sjiph.p; G.sj_w = H.g_sjw.p; G.legent_u = H.g_legu.p; G.legent_s = H.g_legs.p;
  G.fmix = H.g_fmix.p; G.scatterj = H.g_scatj.p; G.legenp_u = H.g_legp.p; G.extp = H.g_extp.p; G.albp = H.g_albp.p;
  G.piph = H.g_piph.p; G.pphw = H.g_pphw.p; G.adj = dadj; G.gradout = H.g_grad.p; G.beam = H.g_beam.p;
  G.botalb = H.botalb.p; G.npart = P.npart; G.maxnmicro = P.maxnmicro; G.ng = P.npx * P.npy * P.npz;
  G.scatmin = (float)P.scatmin;
  CK(cudaMemsetAsync(H.g_grad.p, 0, H.g_grad.n * sizeof(double), H.stream));
  CK(cudaMemsetAsync(H.g_beam.p, 0, H.g_beam.n * sizeof(double), H.stream));
  const int blocks = (nrays + shdom::GWARPS - 1) / shdom::GWARPS;
  shdom::k_levis_adjoint<<<blocks, shdom::GWARPS * 32, 0, H.stream>>>(G);
  CK(cudaGetLastError());
  shdom::BeamArgs b;
  b.gridpos = H.gridpos.p; b.zlev = H.zgrid.p; b.beam = H.g_beam.p; b.dextm = H.g_dextm.p; b.gradout = H.g_grad.p;
  b.npts = P.npts; b.npx = P.npx; b.npy = P.npy; b.npz = P.npz; b.bcflag = P.bcflag; b.ipflag = P.ipflag;
  b.delx = P.delx; b.dely = P.dely; b.solarmu = P.prob.solarmu; b.solaraz = P.prob.solaraz;
  shdom::k_levis_beam<<<(P.npts + 255) / 256, 256, 0, H.stream>>>(b);
  CK(cudaGetLastError());
  H.launches += 2;
}

// Checks shared by the gradient entry points; builds the derivative tables
// of the species on its first use.
static int levis_ready(shdom_handle *hh, int species) {
  Handle &H = hh->h;
  shdom::Plan &P = H.P;
  if (species < 0 || species >= P.npart) return fail(hh, "levis gradient: species index out of range");
  if (H.nst != 1) return fail(hh, "levis gradient: scalar (nstokes = 1) problems only");
  if (P.brdf) return fail(hh, "levis gradient: Lambertian surfaces only");
  if (P.ml + 1 > 32 || P.nlm > shdom::RNLM) return fail(hh, "levis gradient: at most 32 Legendre terms are supported");
  if (!H.initialized) return fail(hh, "levis gradient: the solution has not been initialized");
  if (H.grad_ipa != species) prepare_grad(H, species);
  return 0;
}

// Host-buffer form of the gradient: measurements given -> L2 cost and its
// adjoint weights (COMPUTE_ADJOINT_WEIGHTS, unit uncertainty); otherwise
// the caller's weights.
static int levis_host(shdom_handle *hh, int species, int nrays, const float *camx, const float *camy,
                      const float *camz, const double *cammu, const double *camphi, const float *meas,
                      const double *weights, double *gradient, double *cost, float *stokes_out) {
  Handle &H = hh->h;
  shdom::Plan &P = H.P;
  if (int rc = levis_ready(hh, species)) return rc;
  const int ng = P.npx * P.npy * P.npz;
  CallMem mem;
  const size_t fb = (size_t)nrays * sizeof(float), db = (size_t)nrays * sizeof(double);
  mem.alloc(4 * fb + 3 * db);
  float *d = (float *)mem.p;
  float *dx = d, *dy = d + nrays, *dz = d + 2 * (size_t)nrays, *dout = d + 3 * (size_t)nrays;
  double *dmu = (double *)(d + 4 * (size_t)nrays), *dphi = dmu + nrays, *dadj = dphi + nrays;
  int rc = 0;
  CK(cudaMemcpyAsync(dx, camx, fb, cudaMemcpyHostToDevice, H.stream));
  CK(cudaMemcpyAsync(dy, camy, fb, cudaMemcpyHostToDevice, H.stream));
  CK(cudaMemcpyAsync(dz, camz, fb, cudaMemcpyHostToDevice, H.stream));
  CK(cudaMemcpyAsync(dmu, cammu, db, cudaMemcpyHostToDevice, H.stream));
  CK(cudaMemcpyAsync(dphi, camphi, db, cudaMemcpyHostToDevice, H.stream));
  rc = render_impl(hh, nrays, dx, dy, dz, dmu, dphi, dout, H.stream);  // forward radiances, surface radiance
  std::vector<double> adj(nrays, 0.0);
  std::vector<float> st(nrays, 0.f);
  if (!rc) {
    CK(cudaMemcpyAsync(st.data(), dout, fb, cudaMemcpyDeviceToHost, H.stream));
    CK(cudaStreamSynchronize(H.stream));
    if (meas) {
      double c = 0.0;
      for (int i = 0; i < nrays; ++i) {
        const double e = (double)st[i] - (double)meas[i];
        c += 0.5 * e * e;
        adj[i] = e;
      }
      if (cost) *cost = c;
    } else {
      for (int i = 0; i < nrays; ++i) adj[i] = weights[i];
    }
    if (stokes_out) std::memcpy(stokes_out, st.data(), fb);
    CK(cudaMemcpyAsync(dadj, adj.data(), db, cudaMemcpyHostToDevice, H.stream));
    levis_adjoint_device(H, nrays, dx, dy, dz, dmu, dphi, dadj);
    CK(cudaMemcpyAsync(gradient, H.g_grad.p, (size_t)ng * 2 * sizeof(double), cudaMemcpyDeviceToHost, H.stream));
  }
  CK(cudaStreamSynchronize(H.stream));
  if (rc) return rc;
  if (shdom::check_device_error(H)) return 1;
  return 0;
}

int shdom_render_device(shdom_handle *hh, int nrays, const float *camx, const float *camy, const float *camz,
                        const double *cammu, const double *camphi, float *stokes_out, void *stream) {
  if (!hh) return fail(nullptr, "null handle");
  DevGuard dg(hh->h.device);
  try {
    return render_impl(hh, nrays, camx, camy, camz, cammu, camphi, stokes_out, (cudaStream_t)stream);
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
}

int shdom_render(shdom_handle *hh, int nrays, const float *camx, const float *camy, const float *camz,
                 const double *cammu, const double *camphi, float *stokes_out) {
  if (!hh) return fail(nullptr, "null handle");
  Handle &H = hh->h;
  if (nrays <= 0) return 0;
  DevGuard dg(H.device);
  try {
    CallMem mem;
    size_t fb = (size_t)nrays * sizeof(float), db = (size_t)nrays * sizeof(double);
    mem.alloc(3 * fb + 2 * db + fb * H.nst);
    float *d = (float *)mem.p;
    // the double arrays first: every array starts on its own element size for any nrays
    double *dmu = (double *)d, *dphi = dmu + nrays;
    float *dx = (float *)(dphi + nrays), *dy = dx + nrays, *dz = dy + nrays, *dout = dz + nrays;
    CK(cudaMemcpyAsync(dx, camx, fb, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dy, camy, fb, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dz, camz, fb, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dmu, cammu, db, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dphi, camphi, db, cudaMemcpyHostToDevice, H.stream));
    int rc = render_impl(hh, nrays, dx, dy, dz, dmu, dphi, dout, H.stream);
    if (!rc) CK(cudaMemcpyAsync(stokes_out, dout, fb * H.nst, cudaMemcpyDeviceToHost, H.stream));
    CK(cudaStreamSynchronize(H.stream));
    if (rc) return rc;
    if (shdom::check_device_error(H)) return 1;
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

int shdom_levis_gradient(shdom_handle *hh, int species, int nrays, const float *camx, const float *camy,
                         const float *camz, const double *cammu, const double *camphi, const float *measurements,
                         double *gradient, double *cost, float *stokes_out) {
  if (!hh) return fail(nullptr, "null handle");
  if (nrays <= 0 || !measurements || !gradient) return fail(hh, "shdom_levis_gradient: bad arguments");
  DevGuard dg(hh->h.device);
  try {
    return levis_host(hh, species, nrays, camx, camy, camz, cammu, camphi, measurements, nullptr, gradient, cost,
                      stokes_out);
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
}

int shdom_levis_adjoint(shdom_handle *hh, int species, int nrays, const float *camx, const float *camy,
                        const float *camz, const double *cammu, const double *camphi, const double *weights,
                        double *gradient) {
  if (!hh) return fail(nullptr, "null handle");
  if (nrays <= 0 || !weights || !gradient) return fail(hh, "shdom_levis_adjoint: bad arguments");
  DevGuard dg(hh->h.device);
  try {
    return levis_host(hh, species, nrays, camx, camy, camz, cammu, camphi, nullptr, weights, gradient, nullptr,
                      nullptr);
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
}

int shdom_levis_adjoint_device(shdom_handle *hh, int species, int nrays, const float *camx, const float *camy,
                               const float *camz, const double *cammu, const double *camphi, const double *weights,
                               double *gradient, void *stream) {
  if (!hh) return fail(nullptr, "null handle");
  if (nrays <= 0 || !camx || !camy || !camz || !cammu || !camphi || !weights || !gradient)
    return fail(hh, "shdom_levis_adjoint_device: bad arguments");
  Handle &H = hh->h;
  DevGuard dg(H.device);
  try {
    if (int rc = levis_ready(hh, species)) return rc;
    const cudaStream_t cs = (cudaStream_t)stream;
    for (auto &e : H.ev_caller)
      if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // the caller's stream has produced the rays and weights: the handle's stream waits for it
    CK(cudaEventRecord(H.ev_caller[0], cs));
    CK(cudaStreamWaitEvent(H.stream, H.ev_caller[0], 0));
    bcrad_update(H, H.stream);
    levis_adjoint_device(H, nrays, camx, camy, camz, cammu, camphi, weights);
    const shdom::Plan &P = H.P;
    CK(cudaMemcpyAsync(gradient, H.g_grad.p, (size_t)P.npx * P.npy * P.npz * 2 * sizeof(double),
                       cudaMemcpyDeviceToDevice, H.stream));
    // and the caller's stream waits for the gradient
    CK(cudaEventRecord(H.ev_caller[1], H.stream));
    CK(cudaStreamWaitEvent(cs, H.ev_caller[1], 0));
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

}  // extern "C"

// ------------------------------------------------ render without allocation
// Staging for shdom_render_noalloc: the rays and the radiances of one call
// in a fixed device array (x, y, z, out as float, mu, phi as double), so
// the call needs no device allocation.  Its address is looked up once per
// device.
namespace shdom {
constexpr int kNoAllocMaxRays = 1 << 16;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocMaxRays * (4 * sizeof(float) + 2 * sizeof(double));
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];
}  // namespace shdom

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64] = {nullptr};

// Address of the scratch array on device `dev`, which must be the current
// device (set up on first use on that device).
static void *noalloc_scratch(int dev, std::string &err) {
  if (dev < 0 || dev >= 64) { err = "shdom_render_noalloc: device index out of range"; return nullptr; }
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return nullptr; }
  if (cur != dev) { err = "shdom_render_noalloc: the handle's device is not the current device"; return nullptr; }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, shdom::g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return nullptr;
    }
    g_noalloc_ptr[dev] = p;
  }
  return g_noalloc_ptr[dev];
}

extern "C" {

int shdom_render_noalloc(shdom_handle *hh, int nrays, const float *camx, const float *camy, const float *camz,
                         const double *cammu, const double *camphi, float *stokes_out) {
  if (!hh) return fail(nullptr, "null handle");
  Handle &H = hh->h;
  if (nrays <= 0) return 0;
  if (nrays > shdom::kNoAllocMaxRays)
    return fail(hh, "shdom_render_noalloc: at most " + std::to_string(shdom::kNoAllocMaxRays) +
                        " rays per call (got " + std::to_string(nrays) + ")");
  if (!camx || !camy || !camz || !cammu || !camphi || !stokes_out) return fail(hh, "shdom_render_noalloc: null argument");
  if (H.nst != 1) return fail(hh, "shdom_render_noalloc: scalar (nstokes = 1) problems only");
  // the handle's device is made current, so the staging array is the one on that device
  DevGuard dg(H.device);
  try {
    std::string err;
    void *base = noalloc_scratch(H.device, err);
    if (!base) return fail(hh, err);
    const size_t n = (size_t)nrays, cap = (size_t)shdom::kNoAllocMaxRays;
    double *dmu = (double *)base, *dphi = dmu + cap;
    float *dx = (float *)(dphi + cap), *dy = dx + cap, *dz = dy + cap, *dout = dz + cap;
    const size_t fb = n * sizeof(float), db = n * sizeof(double);
    CK(cudaMemcpyAsync(dx, camx, fb, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dy, camy, fb, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dz, camz, fb, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dmu, cammu, db, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemcpyAsync(dphi, camphi, db, cudaMemcpyHostToDevice, H.stream));
    CK(cudaMemsetAsync(dout, 0, fb, H.stream));
    int rc = render_impl(hh, nrays, dx, dy, dz, dmu, dphi, dout, H.stream);
    if (!rc) CK(cudaMemcpyAsync(stokes_out, dout, fb, cudaMemcpyDeviceToHost, H.stream));
    CK(cudaStreamSynchronize(H.stream));
    if (rc) return rc;
    if (shdom::check_device_error(H)) return 1;
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

int shdom_export_state(shdom_handle *hh, float *source, int *ns, float *radiance, int *nr, float *fluxes,
                       float *dirflux) {
  if (!hh) return fail(nullptr, "null handle");
  Handle &H = hh->h;
  DevGuard dg(H.device);
  shdom::Plan &P = H.P;
  try {
    CK(cudaStreamSynchronize(H.stream));
    size_t nf = (size_t)P.npts * H.nst * P.nlm;
    if (source) CK(cudaMemcpy(source, H.source.p, nf * sizeof(float), cudaMemcpyDeviceToHost));
    if (radiance) CK(cudaMemcpy(radiance, H.radiance.p, nf * sizeof(float), cudaMemcpyDeviceToHost));
    if (ns) CK(cudaMemcpy(ns, H.ns.p, P.npts * sizeof(int), cudaMemcpyDeviceToHost));
    if (nr) CK(cudaMemcpy(nr, H.nr.p, P.npts * sizeof(int), cudaMemcpyDeviceToHost));
    if (fluxes) CK(cudaMemcpy(fluxes, H.fluxes.p, (size_t)P.npts * 2 * sizeof(float), cudaMemcpyDeviceToHost));
    if (dirflux) CK(cudaMemcpy(dirflux, H.dirflux.p, (size_t)P.npts * sizeof(float), cudaMemcpyDeviceToHost));
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

int shdom_set_sweep_mode(shdom_handle *hh, int mode) {
  if (!hh) return fail(nullptr, "null handle");
  if (mode < 0 || mode > 3) return fail(hh, "shdom_set_sweep_mode: mode must be 0, 1, 2 or 3");
  Handle &H = hh->h;
  DevGuard dg(H.device);
  try {
    const bool levels_only = mode == 3;
    if (levels_only != H.march_off) {
      H.march_off = levels_only;
      // the level schedule's source pass needs its (radsrc, tr) table
      if (levels_only && !H.sweepw.p && (H.march[0] || H.march[1])) {
        CK(cudaStreamSynchronize(H.stream));
        H.sweepw.alloc((size_t)H.P.npts * H.ldo);
      }
      for (auto &g : H.iter_graph)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    }
    H.sweep_mode = levels_only ? 0 : mode;
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

int shdom_set_transform_wait_limit(shdom_handle *hh, int limit) {
  if (!hh) return fail(nullptr, "null handle");
  if (limit > shdom::tc::kWaitLimit) return fail(hh, "shdom_set_transform_wait_limit: limit above the default");
  Handle &H = hh->h;
  DevGuard dg(H.device);
  try {
    H.tc_wait_limit = limit < 0 ? shdom::tc::kWaitLimit : limit;
    for (auto &g : H.iter_graph)  // captured launches hold the old limit
      if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  } catch (const std::exception &e) {
    return fail(hh, e.what());
  }
  return 0;
}

int shdom_set_render_options(shdom_handle *hh, int single_scatter, int nosurface) {
  if (!hh) return fail(nullptr, "null handle");
  hh->h.render_single_scatter = single_scatter ? 1 : 0;
  hh->h.render_nosurface = nosurface ? 1 : 0;
  return 0;
}

int shdom_set_transform_mode(shdom_handle *hh, int mode) {
  if (!hh) return fail(nullptr, "null handle");
  if (mode < 0 || mode > 2) return fail(hh, "shdom_set_transform_mode: mode must be 0, 1 or 2");
  hh->h.xf_mode = mode;
  return 0;
}

int shdom_get_sizes(shdom_handle *hh, shdom_sizes *o) {
  if (!hh || !o) return fail(hh, "null argument");
  shdom::fill_sizes(hh->h.P, o);
  o->iters = hh->h.iters; o->solcrit = hh->h.solcrit;
  o->launches = hh->h.launches;
  const shdom::Handle &H = hh->h;
  o->march = H.march_off ? 0 : ((H.march[0] ? 1 : 0) | (H.march[1] ? 2 : 0));
  o->march_units_down = H.march[0] ? H.mnunits[0] : 0; o->march_units_up = H.march[1] ? H.mnunits[1] : 0;
  o->march_cluster_down = H.march[0] ? H.mcs[0] : 0; o->march_cluster_up = H.march[1] ? H.mcs[1] : 0;
  return 0;
}

int shdom_plan_summary(const shdom_problem *problem, shdom_sizes *o) {
  if (!problem || !o) return fail(nullptr, "shdom_plan_summary: null argument");
  std::memset(o, 0, sizeof(*o));
  try {
    std::unique_ptr<shdom::Plan> P(new shdom::Plan());
    if (!shdom::build_plan(*problem, *P)) return fail(nullptr, P->err);
    shdom::fill_sizes(*P, o);
    o->solcrit = 1.f;
  } catch (const std::exception &e) {
    return fail(nullptr, e.what());
  }
  return 0;
}

int shdom_last_timings(shdom_handle *hh, float *ms5) {
  if (!hh || !ms5) return fail(hh, "null argument");
  for (int i = 0; i < 5; ++i) ms5[i] = hh->h.timings[i];
  return 0;
}

int shdom_sweep_timings(shdom_handle *hh, float *ms2, int *launches2) {
  if (!hh || !ms2) return fail(hh, "null argument");
  for (int i = 0; i < 2; ++i) {
    ms2[i] = hh->h.ktimes[i];
    if (launches2) launches2[i] = hh->h.klaunches[i];
  }
  return 0;
}

const char *shdom_last_error(shdom_handle *hh) { return hh ? hh->h.err.c_str() : g_static_err.c_str(); }

void shdom_destroy(shdom_handle *hh) {
  if (!hh) return;
  DevGuard dg(hh->h.device);
  delete hh;
}

}  // extern "C"
