// shdom_plan.h -- host-side planning for one SHDOM solve on the GPU.
//
// The planner turns a shdom_problem into the flat tables the device kernels
// read: the base grid and its cells, the reference's sweep order expressed
// as per-octant ranks and start cells, the wavefront level schedule that
// lets all ordinates of a hemisphere sweep concurrently, the discrete
// ordinates with their transform coefficients, and the delta-M scaled
// medium, direct beam and Eddington initial radiance.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/shdom_problem.h"

namespace shdom {

// A vector shared between plans of the same grid geometry (the host keeps a
// cache of geometry plans; a new plan takes references to the large tables
// instead of copies).  Reads go through the const interface; writes go
// through mut(), which copies the table first when another plan shares it.
template <class T>
class SharedVec {
 public:
  SharedVec() : p_(std::make_shared<std::vector<T>>()) {}
  size_t size() const { return p_->size(); }
  bool empty() const { return p_->empty(); }
  const T *data() const { return p_->data(); }
  const T &operator[](size_t i) const { return (*p_)[i]; }
  typename std::vector<T>::const_iterator begin() const { return p_->begin(); }
  typename std::vector<T>::const_iterator end() const { return p_->end(); }
  operator const std::vector<T> &() const { return *p_; }
  const std::vector<T> &vec() const { return *p_; }
  // identity of the shared table (plans that share it share its device copy too)
  std::shared_ptr<const void> owner() const { return p_; }
  std::vector<T> &mut() {
    if (p_.use_count() > 1) p_ = std::make_shared<std::vector<T>>(*p_);
    return *p_;
  }
  void assign(size_t n, const T &v) { mut().assign(n, v); }
  template <class It>
  void assign(It a, It b) { mut().assign(a, b); }

 private:
  std::shared_ptr<std::vector<T>> p_;
};

// The large per-medium host tables (a few bytes per grid point each) live
// in blocks taken from a process-wide pool of warm blocks and are not
// zero-filled when allocated: re-planning a medium of the same size (the
// next wavelength, the next iterate of a retrieval) reuses memory that is
// already mapped instead of faulting in and clearing fresh pages.  Blocks
// under 1 MiB use the ordinary heap; at most 4 GiB of free blocks are kept.
// Every element must be written before it is read (resize() and the size
// constructor leave the elements uninitialised; assign(n, v) sets them).
void *host_block_alloc(size_t bytes);
void host_block_free(void *p, size_t bytes) noexcept;
template <class T>
struct HostAlloc {
  using value_type = T;
  HostAlloc() = default;
  template <class U>
  HostAlloc(const HostAlloc<U> &) {}
  T *allocate(size_t n) { return static_cast<T *>(host_block_alloc(n * sizeof(T))); }
  void deallocate(T *p, size_t n) noexcept { host_block_free(p, n * sizeof(T)); }
  template <class U, class... A>
  void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
  template <class U>
  void construct(U *p) { ::new ((void *)p) U; }
  template <class U>
  bool operator==(const HostAlloc<U> &) const { return true; }
  template <class U>
  bool operator!=(const HostAlloc<U> &) const { return false; }
};
template <class T>
using HostVec = std::vector<T, HostAlloc<T>>;

// One group of sweep tasks at one wavefront level: the points (tasks[t0,
// t0+ntask)) of trace octant b whose traces for the ordinates of face class
// cls (columns [col0, col0+ncol)) are all regular or all not.  start is the
// group's first item (task x column) within its level; for a group that is
// not regular, irr0 is its first item in the hemisphere's table of general
// traces.
struct Seg {
  int t0, ntask, start, b, cls, col0, ncol, regular, irr0;
};

// Plane march of one (octant, face class) group of columns: every phase-2
// point of the group has a regular trace whose stopping face lies in the
// neighbouring plane along the class axis (x, y or z), so the group's
// phase-2 points can be swept plane by plane, each plane depending only on
// the one before.  Axes: A the march (class) axis, U and V the two others
// (U the strip axis, V the row axis); points are p = a*sa + u*su + v*sv.
struct MarchGrp {
  int b, cls, col0, ncol;
  int nA, nU, nV, sa, su, sv;
  int a0, da;          // first plane in march order (the upwind boundary plane) and the step
  int du[4], dv[4];    // transverse offsets (0 or +-1) of the stopping face's corners, face-weight order
  int upu;             // the sign of the U offsets: +1 when the upwind rows are at higher U
  // fixed points (preset boundary or phase 1): the layer iz == zfix, and
  // with open x (y) boundaries the planes ix == 0 or nx1 - 1 (iy == 0 or ny1 - 1)
  int zfix, xedge, yedge;
};

struct Plan {
  // Level numbers of phase-2 points start at kPhase2 (phase 1 < kPhase2).
  static constexpr int kPhase2 = 1 << 16;
  // ---- base grid (INIT_CELL_STRUCTURE layout, 0-based, -1 = no neighbour)
  int nx = 0, ny = 0, nz = 0, nx1 = 0, ny1 = 0, npts = 0, ncells = 0;
  int bcflag = 0, ipflag = 0, is1d = 0, noct = 8;
  std::vector<float> xgrid, ygrid, zgrid;
  SharedVec<float> gridpos;        // [npts][3]
  SharedVec<int> gridptr;          // [ncells][8]
  SharedVec<int> neighptr;         // [ncells][6]
  SharedVec<int> cellflags;        // [ncells]
  std::vector<uint8_t> bnd;        // [npts] bit0 top boundary point, bit1 bottom
  std::vector<int> topp, botp;     // boundary point lists in point order
  // ---- sweep order per trace octant (index ioct-1): rank and start cell
  SharedVec<int> rank;             // [8][npts], -1 when the octant is unused
  SharedVec<int> startcell;        // [8][npts]
  SharedVec<int> level;            // [8][4][npts] wavefront level per octant and face class (0: preset)
  // kind[8][4][npts]: 0 preset or unused, 1 phase-2 regular trace, 2 phase-2
  // general trace, 3 phase 1 (a general-trace point whose dependencies are
  // all preset or phase-1 points: the open-boundary planes' own chains).
  SharedVec<uint8_t> kind;
  // regular[b][p] = 1 when point p's trace for trace octant b crosses one
  // full interior cell whose seven other corners all precede p; such traces
  // depend only on the ordinate and the z layer, tabulated in geo.
  SharedVec<uint8_t> regular;      // [8][npts]
  std::vector<float> geo;          // [nz-1][nang][4]: so, u, v, face
  // ---- discrete ordinates
  // nang counts the ordinate columns including the padding ordinates that
  // align each (octant, face class) group to 8 columns; nang_real = NANG.
  int nmu = 0, nphi = 0, ml = 0, mm = 0, nlm = 0, nleg = 0, nang = 0, nang_real = 0, nphi0max = 0;
  std::vector<int> nphi0, lofj, mofj;
  std::vector<float> mu, wtmu, phi, wtdo;        // phi/wtdo [nmu][nphi0max]
  // Column order of the ordinate-space arrays: hemisphere (down, up), then
  // trace octant, then (mu, phi) in the reference order.
  std::vector<int> col_imu, col_iphi, col_oct;   // [nang]; col_imu < 0 for a padding ordinate
  std::vector<int> col_cls;                      // [nang] face class: 0 x, 1 y, 2 z, 3 mixed
  int cls_col0[8][4] = {{0}}, cls_ncol[8][4] = {{0}};  // first column and real ordinates per octant and class
  std::vector<int> col_of;                       // [nmu][nphi0max] -> column
  int ncol_down = 0;                             // columns [0, ncol_down) are mu < 0
  int oct_col0[8] = {0}, oct_ncol[8] = {0};      // column range of each trace octant
  std::vector<float> col_cx, col_cy, col_cz;     // trace (back) direction per column
  std::vector<float> col_fluxw;                  // |mu| * wtdo per column (I columns only)
  // Polarized problems (nst = 3) hold I, Q and U of every ordinate in
  // separate columns: within each (octant, face class) group the group's
  // ordinates appear three times, I then Q then U, so a sweep segment's
  // columns keep one shared trace geometry per ordinate.
  int nst = 1;
  std::vector<uint8_t> col_stk;                  // [nang] Stokes component of each column (0 I, 1 Q, 2 U)
  std::vector<float> cmu1, cmu2;                 // [nmu][nlm]
  std::vector<float> cmu1p, cmu2p;               // nst = 3: [nmu][nlm][6] generalized functions (PLMALL)
  std::vector<float> cphi1, cphi2;               // [nmu][nphi0max][2mm+1]
  std::vector<float> ylmsun;                     // [nlm]
  // ---- medium on the grid
  int npart = 0, numphase = 0;
  HostVec<float> total_ext;
  HostVec<double> extdirp;                   // [npx*npy*npz] delta-M scaled extinction for the direct beam
  HostVec<float> coef;                       // [npts][ml+1]: albedo * delta-M scaled Legendre term
  HostVec<float> coefp;                      // nst = 3: [npts][3][ml+1] the same for a2, a3 and b1
  std::vector<uint8_t> scat;                     // [npts] 1 where the point has a source: it scatters (a non-zero
                                                 // coefficient row) or emits (a non-zero thermal term)
  HostVec<int> tms_ptr, tms_iph;             // CSR per point: exact single-scatter mixture
  HostVec<float> tms_w;
  std::vector<float> phasetab;                   // [nscatangle][numphase]
  std::vector<float> phasetab2;                  // nst = 3: [nscatangle][numphase] the I-Q element
  int nscatangle = 0;
  float albmax = 0.f;
  HostVec<float> rad0;                       // [npts][4] Eddington initial radiance
  std::vector<float> botalb;                     // surface albedo at the bottom points
  // thermal emission (srct 'T' thermal, 'B' thermal and solar; empty for
  // 'S'): thermal[i] the extinction-weighted (1 - albedo) B(T) of point i,
  // botplanck B at the bottom points, skyrad_bc the top boundary radiance
  char srct = 'S', unitc = 'R';
  HostVec<float> thermal;                    // [npts]
  HostVec<float> planckpt;                   // [npts] B(T) of each point (the gradient's emission term)
  std::vector<float> botplanck;                  // [nbot]
  float skyrad_bc = 0.f;
  // bidirectional surface ('R' RPV, 'W' wave-Fresnel; 0 Lambertian): its
  // parameters at the bottom points and the downward / upward ordinates of
  // the reflection sums, in the reference order: mu, phi, weight
  // (|mu| wtdo / pi, downward only), I column, Stokes column stride
  int brdf = 0, nsfcpar = 0;
  std::vector<float> botpar;                     // [nbot][nsfcpar]
  struct BrdfOrd { float mu, phi, w, col, off; };
  std::vector<BrdfOrd> brdf_dn, brdf_up;
  // ---- species data kept for the gradient (property grid and grid points)
  int npx = 0, npy = 0, npz = 0, maxnmicro = 0;
  float delx = 0.f, dely = 0.f;
  double scatmin = 0.0;
  HostVec<float> prop_ext, prop_alb, prop_phw;  // [npart][ng], [npart][ng][maxnmicro]
  HostVec<int> prop_iph;                        // [npart][ng][maxnmicro], 1-based table rows
  std::vector<float> leg;                           // [numphase][nleg+1] l/(2l+1) scaled, minus f for l <= ML with delta-M
  HostVec<float> sp_ext, sp_alb, sp_f;          // [npart][npts] delta-M scaled extinction, albedo, f
  // [npart][npts][sp_nq] the phase-table indices (1-based) and weights each
  // grid point interpolates from the property grid (for the gradient's
  // species phase series, formed on demand by species_series)
  HostVec<int> sp_iph;
  HostVec<float> sp_pw;
  int sp_nq = 0;
  // ---- numerical parameters
  shdom_problem prob{};
  // ---- wavefront schedule, per hemisphere (0 down, 1 up)
  SharedVec<uint32_t> tasks[2];                  // point indices: phase-1 segments, then phase-2 levels
  std::vector<Seg> p1segs[2];                    // phase 1: one segment per level per (octant, class) group
  std::vector<int> p1off[2];                     // group -> first segment (ngroups + 1 entries)
  int p1depth[2] = {0, 0};
  int deep[2] = {0, 0};  // hemisphere swept in the reference order (no level schedule)
  std::vector<Seg> segs[2];
  std::vector<int> seg_off[2];                   // level -> first segment (nlevels + 1 entries)
  std::vector<int> level_items[2];               // level -> task x column items
  long long nirr[2] = {0, 0};                    // general-trace items per hemisphere
  long long nitems[2] = {0, 0};                  // phase-2 task x column items per hemisphere
  // plane-march groups per hemisphere; empty when some group of the
  // hemisphere does not march (general phase-2 traces, the mixed face
  // class, points other than the boundary and edge planes that are fixed)
  std::vector<MarchGrp> march[2];
  std::string err;
};

// Fills every table of the plan; returns false with plan.err set on error.
bool build_plan(const shdom_problem &p, Plan &plan);

// A phase-table weight at or above this makes a point use that one entry.
constexpr float kPhaseMax = 0.999f;

// The Legendre series of species ipa at grid point ipt with the delta-M
// scaling undone (u[0..ml]), formed with the medium build's arithmetic.
void species_series(const Plan &P, int ipa, int ipt, float *u);

// PLANCK_FUNCTION for units 'R' (W/(m^2 sr micron) at wavelen microns),
// 'T' (the temperature itself) and 'B' (W/(m^2 sr) over the band waveno[2], cm^-1).
float planck_fn(float t, char units, float wavelen, const float *waveno);

// OPTICAL_DEPTH (src/shdomsub5.f:387-739 of the reference): the extinction
// integrated along each ray (x, y, z, mu, phi as for the render) through
// the base grid, trapezoid per cell crossing, with the delta-M scaling
// undone unless deltam_path.  Host code on the plan's medium; out [n].
bool optical_path(const Plan &P, int n, const float *camx, const float *camy, const float *camz,
                  const double *cammu, const double *camphi, int deltam_path, float *out, std::string &err);

// MIN_OPTICAL_DEPTH (src/shdomsub5.f:17-385): per grid point the smallest
// optical path, over the rays, at which a ray leaves a cell the point is a
// corner of; minpath [npts] (or [n][npts] per ray with do_all), 999 where no
// ray passes.
bool min_optical_path(const Plan &P, int n, const float *camx, const float *camy, const float *camz,
                      const double *cammu, const double *camphi, int deltam_path, int do_all, float *minpath,
                      std::string &err);

// Per grid point the absorption sum_species ext (1 - albedo) and the
// emission sum_species ext (1 - albedo) B(T) of the delta-M scaled medium
// (ABSORB and EMIT of COMPUTE_NETFLUXDIV, src/polarized/shdomsub2.f:1725-1764).
bool point_absorption(const Plan &P, float *absorb, float *emit, std::string &err);

// Real generalized spherical harmonics (unpolarized element) at one
// direction, NLM values in the SHDOM term order.
void ylm_unpol(int ml, int mm, double mu, float phi, float *y);

}  // namespace shdom
