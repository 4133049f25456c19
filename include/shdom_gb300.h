/*
 * shdom_gb300.h -- C-ABI of the GB300-native SHDOM solve / render path.
 *
 * The reference reaches its Fortran core through f2py (module at3d.core,
 * exported list tools/generate_pyf.py:51-139).  A drop-in replacement binds
 * these entry points instead; each one names the at3d.core routine (and the
 * Python call site) it replaces.  All buffers are plain host pointers unless
 * the name says _device; sizes are explicit; no library types cross the
 * boundary.  Every call returns an SHDOM error code with the meaning of
 * at3d/checks.py:300-311: 0 ok, 1 error (message from shdom_last_error),
 * 2 out of memory for spherical-harmonic terms.  No call aborts the process.
 *
 * A handle owns one solve's state in HBM (medium, source function, radiance,
 * fluxes, sweep schedule) between calls, the way RTE keeps its numpy arrays
 * between solve() and integrate_to_sensor() (at3d/solver.py:2635-2652).
 * Calls on one handle must not overlap; different handles are independent.
 */
#ifndef SHDOM_GB300_H
#define SHDOM_GB300_H

#include <stdint.h>

#include "shdom_problem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shdom_handle shdom_handle;

typedef struct shdom_sizes {
    int npts;      /* grid points (NPTS) */
    int ncells;    /* grid cells (NCELLS) */
    int nx1, ny1, nz;
    int nlm;       /* spherical-harmonic terms (NLM) */
    int nmu, nang; /* zenith angles, discrete ordinates (NANG) */
    int ml, mm;
    int bcflag, ipflag;
    int iters;     /* iterations done so far (RTE._iters) */
    int nlevels_down, nlevels_up; /* sweep wavefront levels per hemisphere (0: swept in the reference order) */
    float solcrit; /* current solution criterion (RTE._solcrit) */
    float albmax;
    long long launches; /* kernels launched on this handle since creation */
    long long device_bytes; /* device memory the handle holds (estimate before creation) */
    int nstokes;   /* Stokes components (1, or 3 for I, Q, U) */
    int march;     /* hemispheres swept by the plane march (bit 0 down, bit 1 up; plan: eligible, handle: in use) */
    int march_units_down, march_units_up;     /* handle: thread-block clusters of each hemisphere's march launch */
    int march_cluster_down, march_cluster_up; /* handle: CTAs per cluster (16 or 8) */
} shdom_sizes;

/* Builds the grid, the cell structure, the sweep schedule and the medium on
 * the device for one problem.  Replaces RTE.__init__'s _setup_grid
 * (core.new_grids, core.init_cell_structure; at3d/solver.py:2036-2168) and
 * _prepare_optical_properties (core.transfer_pa_to_grid;
 * at3d/solver.py:2324-2519).  device < 0 keeps the current CUDA device. */
int shdom_create(const shdom_problem *problem, int device, shdom_handle **out);

/* Plans a problem on the host only (grid, sweep schedule, ordinates, medium)
 * and reports its sizes, wavefront depths and the device memory a handle for
 * it would hold; touches no GPU.  For admission by memory budget before
 * shdom_create.  No direct reference counterpart (the reference sizes its
 * arrays in RTE._setup_grid, at3d/solver.py:2122-2191). */
int shdom_plan_summary(const shdom_problem *problem, shdom_sizes *out);

/* Two-stage form of shdom_create for callers that admit work by device
 * memory: shdom_plan_create does the host part (grid, cell structure, sweep
 * schedule, ordinates, medium, direct beam) without touching a GPU and
 * reports the sizes (device_bytes: the memory the handle will hold; sizes
 * may be NULL); the plan keeps copies of the problem's arrays.
 * shdom_create_planned puts a plan on the device and takes ownership of it:
 * the plan is released by that call whether it succeeds or not.
 * shdom_plan_destroy releases a plan that is not used.  The pair does what
 * shdom_create does. */
typedef struct shdom_plan shdom_plan;
int shdom_plan_create(const shdom_problem *problem, shdom_plan **out, shdom_sizes *sizes);
int shdom_create_planned(shdom_plan *plan, int device, shdom_handle **out);
void shdom_plan_destroy(shdom_plan *plan);

/* The extinction integrated along each ray (RTE.optical_path,
 * at3d/solver.py:793-867; OPTICAL_DEPTH, src/shdomsub5.f:387-739): rays as
 * for shdom_render (position, mu and phi toward the sensor), traced back
 * through the base grid with the trapezoid rule per cell crossing; the
 * delta-M scaled extinction when deltam_path, else the unscaled one.  Host
 * computation on the plan's medium (no GPU work); a ray starting above the
 * domain is extended to its top, one leaving upward gets 0.  3D grids. */
int shdom_plan_optical_path(const shdom_plan *plan, int nrays, const float *camx, const float *camy,
                            const float *camz, const double *cammu, const double *camphi, int deltam_path,
                            float *path_out);
/* RTE.min_optical_path (at3d/solver.py:921-990; MIN_OPTICAL_DEPTH,
 * src/shdomsub5.f:17-385): per grid point the smallest optical path, over
 * the rays, at which a ray leaves a cell the point is a corner of;
 * minpath_out [npts], or [nrays][npts] per ray with do_all; 999 where no
 * ray passes.  Host computation on the plan's medium. */
int shdom_plan_min_optical_path(const shdom_plan *plan, int nrays, const float *camx, const float *camy,
                                const float *camz, const double *cammu, const double *camphi, int deltam_path,
                                int do_all, float *minpath_out);
/* Per grid point [npts] the absorption sum_species ext (1 - albedo) and the
 * emission sum_species ext (1 - albedo) B(T) of the delta-M scaled medium
 * (ABSORB and EMIT of COMPUTE_NETFLUXDIV, src/polarized/shdomsub2.f:
 * 1725-1764, for RTE.net_flux_divergence, at3d/solver.py:1207-1260); emit
 * is 0 for a solar source.  Host computation. */
int shdom_plan_point_absorption(const shdom_plan *plan, float *absorb, float *emit);
int shdom_point_absorption(shdom_handle *h, float *absorb, float *emit);
/* The same on a handle's medium. */
int shdom_optical_path(shdom_handle *h, int nrays, const float *camx, const float *camy, const float *camz,
                       const double *cammu, const double *camphi, int deltam_path, float *path_out);

/* Direct beam, Eddington initial radiance and the first source function.
 * Replaces core.make_angle_set, core.make_sh_do_coef and core.init_solution
 * (at3d/solver.py:2539-2798). */
int shdom_init_solution(shdom_handle *h);

/* Runs iterations until the solution criterion reaches solacc or the
 * iteration count reaches maxiter (the count persists across calls, as
 * RTE._iters does).  Replaces core.solution_iterations
 * (at3d/solver.py:447-618, SOLUTION_ITERATIONS
 * src/polarized/shdomsub1.f:445-818).  iters/solcrit may be NULL. */
int shdom_solution_iterations(shdom_handle *h, int maxiter, int *iters, float *solcrit);

/* Radiance along nrays rays through the solved field.  Host buffers; ray
 * positions are single precision and directions double precision as in the
 * reference's RENDER interface (src/polarized/shdomsub4.f:164-165); mu/phi
 * point towards the sensor.  Replaces core.render (at3d/solver.py:681-759).
 * stokes_out: [nrays][nstokes] (Stokes I, or I, Q, U in the meridional
 * plane of the outgoing direction, the reference's STOKES(NSTOKES,NPIX)). */
int shdom_render(shdom_handle *h, int nrays, const float *camx, const float *camy, const float *camz,
                 const double *cammu, const double *camphi, float *stokes_out);

/* Same as shdom_render with device-resident ray and output buffers, launched
 * on the given CUDA stream (cudaStream_t passed as void*, NULL = legacy
 * default stream).  Asynchronous: returns after the launch. */
int shdom_render_device(shdom_handle *h, int nrays, const float *camx, const float *camy,
                        const float *camz, const double *cammu, const double *camphi,
                        float *stokes_out, void *stream);

/* Levis approximate gradient of the L2 cost 0.5 * sum_r (I_r - m_r)^2 of
 * nrays one-ray pixels (unit uncertainty, ray and Stokes weights) with
 * respect to the extinction and single-scattering albedo of species
 * `species` (0-based, the order of the problem's species) on the property
 * grid.  Replaces core.levisapprox_gradient in its adjoint branch
 * (at3d/gradient.py:262-398, LEVISAPPROX_GRADIENT src/polarized/shdomsub4.f:
 * 288-809) for a scalar solar problem with a Lambertian surface and the
 * 'table' derivative method.  gradient: [npx*npy*npz][2] (d/d extinction,
 * d/d albedo) in the property-grid order (z fastest); cost and stokes_out
 * (the rendered radiances, [nrays]) may be NULL.  The solution is frozen:
 * call after shdom_solution_iterations.  Scalar (nstokes = 1) problems. */
int shdom_levis_gradient(shdom_handle *h, int species, int nrays, const float *camx, const float *camy,
                         const float *camz, const double *cammu, const double *camphi,
                         const float *measurements, double *gradient, double *cost, float *stokes_out);

/* The same adjoint for caller-supplied ray weights w_r: the Levis gradient
 * of sum_r w_r I_r (the vector-Jacobian product of the rendered radiances).
 * No reference counterpart as a separate call: it is the adjoint pass of
 * LEVISAPPROX_GRADIENT with ADJ_WEIGHTS given, used for automatic
 * differentiation. */
int shdom_levis_adjoint(shdom_handle *h, int species, int nrays, const float *camx, const float *camy,
                        const float *camz, const double *cammu, const double *camphi, const double *weights,
                        double *gradient);

/* Device-resident form of shdom_levis_adjoint, for automatic
 * differentiation with the data on the GPU: rays (float x/y/z, double
 * mu/phi), the ray weights w_r (double) and the output gradient
 * ([npx*npy*npz][2] double, d/d extinction and d/d albedo of `species`) are
 * device buffers.  The work is ordered after what the caller queued on
 * `stream` (cudaStream_t as void*, NULL = legacy default stream), and work
 * queued on `stream` after the call sees the gradient; the call returns after
 * the launch.  Same reference routine as shdom_levis_adjoint (the adjoint
 * pass of LEVISAPPROX_GRADIENT, src/polarized/shdomsub4.f:288-809, with
 * ADJ_WEIGHTS given). */
int shdom_levis_adjoint_device(shdom_handle *h, int species, int nrays, const float *camx, const float *camy,
                               const float *camz, const double *cammu, const double *camphi,
                               const double *weights, double *gradient, void *stream);

/* shdom_render for callers that cannot allocate device memory during the
 * call (scalar problems).  It has no counterpart in the reference.  The rays and radiances of
 * the call are staged in one fixed device array inside the library (2 MiB)
 * instead of memory allocated per call, so at most 65536 rays per call are
 * accepted; more is refused with an error.  The array is shared by every
 * handle on a device: calls that overlap in time (any thread or stream)
 * overwrite each other's rays and must be serialized by the caller.  The
 * first call on a device looks the array's address up; make that first
 * call before any stream capture.  Same arguments and results as
 * shdom_render. */
int shdom_render_noalloc(shdom_handle *h, int nrays, const float *camx, const float *camy,
                         const float *camz, const double *cammu, const double *camphi, float *stokes_out);

/* Solution state export (RTE.save_solution fields, at3d/solver.py:1621-1686)
 * in a dense layout: source/radiance [npts][nstokes][nlm] with the terms beyond each
 * point's truncation set to zero, ns/nr the truncations (SHPTR/RSHPTR
 * differences), fluxes [npts][2] (down, up) and dirflux [npts].  Any output
 * pointer may be NULL. */
int shdom_export_state(shdom_handle *h, float *source, int *ns, float *radiance, int *nr,
                       float *fluxes, float *dirflux);

int shdom_get_sizes(shdom_handle *h, shdom_sizes *out);

/* Device time (ms, CUDA events) of the last shdom_solution_iterations call
 * split by phase: [0] source->ordinate transform, [1] sweeps, [2]
 * ordinate->harmonic transform, [3] source + acceleration, [4] total. */
int shdom_last_timings(shdom_handle *h, float *ms5);

/* Device time (ms, CUDA events on the handle's stream) of the sweep's two
 * parts over the last shdom_solution_iterations call, summed over both
 * hemispheres and all iterations: ms2[0] from the start of a hemisphere's
 * sweep to the start of its level pass (phase 1 beside the source pass, or
 * the whole reference-order sweep), ms2[1] the level pass.  launches2
 * (may be NULL) counts the hemisphere sweeps timed; sweep mode 2 records
 * none.  No reference counterpart (diagnostics). */
int shdom_sweep_timings(shdom_handle *h, float *ms2, int *launches2);

/* RENDER's SINGLESCATTER and NOSURFACE switches for the renders that follow
 * on this handle (shdom_render, shdom_render_device, shdom_render_noalloc;
 * the Levis gradient always renders the full radiance):
 *   single_scatter != 0: the source along the ray is only the exact single
 *     scattering of the direct solar beam (with delta-M; zero without), not
 *     the spherical-harmonic source (src/polarized/shdomsub2.f:3107-3142);
 *   nosurface != 0: the radiance leaving the domain boundary (surface or
 *     sky) is not added where the ray ends (:2721-2723).
 * Replaces the single_scatter / nosurface arguments of
 * RTE.integrate_to_sensor (at3d/solver.py:633, :684-686).  Both 0 by default. */
int shdom_set_render_options(shdom_handle *h, int single_scatter, int nosurface);

/* Polls of each pipeline wait in the tensor-core transforms before the
 * kernel gives up, drains the loads and products it has issued, releases
 * its tensor memory and reports "pipeline wait expired" (the next
 * shdom_solution_iterations returns 1 with that message; the handle stays
 * usable).  limit < 0 restores the default; 0 makes every transform give up
 * at its first wait (for testing that path).  No reference counterpart. */
int shdom_set_transform_wait_limit(shdom_handle *h, int limit);

/* Arithmetic of the two spherical-harmonic <-> discrete-ordinate transforms
 * of each iteration (SH_TO_DO / DO_TO_SH, src/polarized/shdomsub1.f:2928-3254,
 * which the reference runs in FP32 on the CPU):
 *   0 (default) tensor cores, TF32 operands split into high and low parts,
 *     three products accumulated in FP32 (FP32-level accuracy);
 *   1 tensor cores, one TF32 product (about 1e-3 relative; reduced precision);
 *   2 CUDA-core FP32 factorized transforms.
 * Problems whose operand rows are not multiples of 16 bytes use 2 in every
 * mode.  No reference counterpart: the reference has a single FP32 path. */
int shdom_set_transform_mode(shdom_handle *h, int mode);

/* How the sweep's interior points are scheduled.  A hemisphere whose
 * interior points all trace through one full cell to the previous plane
 * along their ordinate group's face axis (open boundaries) is swept by the
 * plane march: one kernel per hemisphere, thread-block clusters that keep
 * the previous plane in shared memory, no waits between clusters.  Other
 * hemispheres use the wavefront level schedule: 0 (default) one persistent
 * cooperative kernel per hemisphere with a grid barrier between levels
 * (when the device supports cooperative launch), 1 one kernel launch per
 * level, 2 as 1 with each solution iteration's launches captured once in
 * a CUDA graph (one per source-truncation state) and replayed; mode 2
 * replays the plane march from the graph as well.  3 is 0 with the plane
 * march turned off (the level schedule everywhere; for comparisons).  Use 1
 * or 2 when several handles solve concurrently on one device: they have no
 * waits between thread blocks.  In mode 2 shdom_last_timings reports the
 * whole iteration in its first entry.  No reference counterpart. */
int shdom_set_sweep_mode(shdom_handle *h, int mode);

/* Lorenz-Mie single scattering of homogeneous spheres at one wavelength, a
 * table over radii (host computation in FP64, threaded over radii; no device
 * work and no handle).  Replaces core.compute_mie_all_sizes with avgflag 'C'
 * (at3d/mie.py:223-236; MIE_ONE, src/polarized/miewig.f:5-108, from
 * COMPUTE_MIE_ALL_SIZES, src/polarized/make_mie_table.f90:381-482).
 * wavelength and radii in microns; the refractive index is m_re + i m_im
 * with m_im <= 0 for absorbing particles (n - ik, the reference's sign).  nthreads
 * <= 0 uses every core.  Outputs: extinct, scatter [nsize] cross sections in
 * um^2; nleg [nsize] = min(maxleg, 2 x series length); legcoef
 * [nsize][maxleg+1][6] the Wigner expansion coefficients a1, a2, a3, a4, b1,
 * b2 of the phase matrix times the scattering cross section (zero beyond
 * nleg).  Errors: 1, message from shdom_last_error(NULL). */
int shdom_mie_mono(double wavelength, double m_re, double m_im, int nsize, const float *radii, int maxleg,
                   int nthreads, float *extinct, float *scatter, int *nleg, float *legcoef);

/* Phase-function mixing of several species into one table (host only, no
 * handle).  Replaces core.phase_function_mixing (at3d/medium.py:1007-1017;
 * phase_function_mixing, src/util.f90:240-348).  For each of npts grid
 * points in the given order, the scattering-weighted mean of the species'
 * series (scatter [npts][npart]; 1-based phase_index and phase_weight
 * [npart][npts][nmicro] into phase_tables [numphase][nleg+1][nstleg],
 * nstleg 1 or 6) is matched against the entries kept so far by asymmetry,
 * P11 and P12/P11 at nangles angles within asym_tol, phase_tol, dolp_tol,
 * or kept as a new entry.  Outputs: mixed_table [maxnphase][nleg+1][nstleg],
 * mixed_index [npts] (1-based; 0 where nothing scatters), *nphase.  When
 * more than maxnphase entries are needed: 1, with *nphase the count reached
 * and *fail_point the 1-based point (may be NULL).  A non-positive P11 is
 * an error.  Errors: message from shdom_last_error(NULL). */
int shdom_phase_function_mixing(int npts, int npart, int nmicro, const float *scatter, const int *phase_index,
                                const float *phase_weight, int numphase, int nleg, int nstleg,
                                const float *phase_tables, double asym_tol, double phase_tol, double dolp_tol,
                                int nangles, int maxnphase, float *mixed_table, int *mixed_index, int *nphase,
                                int *fail_point);

/* Message of the last non-zero return on this handle (CHARACTER*600 errmsg
 * of the reference); a static message when h is NULL. */
const char *shdom_last_error(shdom_handle *h);

void shdom_destroy(shdom_handle *h);

#ifdef __cplusplus
}
#endif
#endif
