/*
 * shdom_problem.h -- plain-C description of one SHDOM radiative-transfer
 * problem (medium on a property grid, boundary conditions, solar source,
 * Lambertian surface, numerical parameters).
 *
 * This is the input format of the drop-in C-ABI (shdom_gb300.h).  Every
 * field mirrors an argument that at3d.solver.RTE passes to the Fortran
 * core through f2py:
 *   property grid / species  : at3d/solver.py:2336-2411 (extinctp, albedop,
 *                              iphasep, phasewtp, legenp) and
 *                              at3d/solver.py:2057-2064 (npx, npy, npz,
 *                              delx, dely, zlevels)
 *   boundary conditions      : at3d/solver.py:2110-2127 (bcflag, ipflag)
 *   source                   : at3d/source.py:14-80 (solar)
 *   surface                  : at3d/surface.py:28-105 (lambertian)
 *   temperature              : at3d/solver.py:1765-1800 (tempp)
 *   numerical parameters     : at3d/solver.py:1960-2034, default_config.json
 *
 * Array layouts are the Fortran (column-major) layouts of the reference,
 * written here as C row-major with the slowest index first:
 *   extinctp[npart][npx][npy][npz]
 *   iphasep [npart][npx][npy][npz][maxnmicro]   (1-based table index)
 *   legenp  [numphase][nlegp+1]                 (scalar legcoef a_l, which
 *                                                carry the 2l+1 factor)
 *   sfc_albedo[nysfc][nxsfc]                    (x fastest)
 */
#ifndef SHDOM_PROBLEM_H
#define SHDOM_PROBLEM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shdom_problem {
    /* ---- property grid ---- */
    int npx, npy, npz;
    float delx, dely;
    const float *zlevels;          /* [npz] km, increasing, zlevels[0] is the ground */
    /* ---- scattering species ---- */
    int npart, maxnmicro;
    const float *extinctp;         /* [npart][npx*npy*npz] 1/km */
    const float *albedop;          /* [npart][npx*npy*npz] */
    const int   *iphasep;          /* [npart][npx*npy*npz][maxnmicro], 1..numphase */
    const float *phasewtp;         /* [npart][npx*npy*npz][maxnmicro] */
    int numphase, nlegp;
    const float *legenp;           /* [numphase][nlegp+1] */
    /* ---- boundary conditions ---- */
    int bc_x_open, bc_y_open;      /* 0 periodic, 1 open */
    int ipflag;                    /* independent-pixel bit flags, 0..7 */
    /* ---- solar source (SHDOM convention: solarmu < 0, radians) ---- */
    float solarflux, solarmu, solaraz, skyrad;
    /* ---- Lambertian surface ---- */
    int sfc_variable;              /* 0: fixed 'FL', 1: variable 'VL' */
    float gndalbedo, gndtemp;
    int nxsfc, nysfc;
    float delxsfc, delysfc;
    const float *sfc_albedo;       /* [nysfc][nxsfc] when sfc_variable */
    /* ---- numerical parameters ---- */
    int nmu, nphi, angle_set;
    int deltam, accelflag, highorderrad, iterfixsh;
    float solacc, shacc, splitacc; /* splitacc must be <= 0 (no adaptive splitting) */
    double tautol, transcut;
    float transmin;
    int nstokes;                   /* 1 (scalar) or 3 (I, Q, U); with 3, legenp is
                                      [numphase][nlegp+1][6] (a1 a2 a3 a4 b1 b2 fastest) */
    /* ---- bidirectional surface reflection (at3d/surface.py RPV_unpolarized,
     *      wave_fresnel, diner; VARIABLE_BRDF_SURFACE
     *      src/polarized/shdomsub1.f:2592-2664).  When sfc_brdf != 0 it
     *      replaces the Lambertian surface; the parameters live on the
     *      nxsfc x nysfc surface grid (delxsfc, delysfc, periodic) ---- */
    int sfc_brdf;                  /* 0, 'R' (RPV: rho0, k, theta), 'W' (wave-Fresnel:
                                      real and imaginary index, wind speed m/s), 'D'
                                      (Diner: a, k, b, zeta, sigma) */
    int nsfcpar;                   /* parameters per surface grid point */
    const float *sfc_params;       /* [nysfc][nxsfc][nsfcpar] */
    /* ---- thermal emission (at3d/source.py thermal, combined; PLANCK_FUNCTION
     *      src/polarized/shdomsub2.f:4756-4791).  srctype 'T' replaces the solar
     *      beam by emission of (1 - albedo) B(T) from every grid point, the
     *      ground ((1 - albedo) B(ground temperature), or the BRDF emissivity)
     *      and the sky (skyrad is then a brightness temperature); 'B' adds
     *      both sources.  0 means 'S' (solar only) ---- */
    int srctype;                   /* 0 or 'S', 'T', 'B' */
    int units;                     /* 'R' radiance W/(m^2 sr um) (0 means 'R'), 'T' brightness
                                      temperature, 'B' band-integrated over waveno */
    float wavelen;                 /* micron, for the Planck function */
    const float *tempp;            /* [npx][npy][npz] K on the property grid ('T', 'B') */
    const float *sfc_temp;         /* [nysfc][nxsfc] K on the surface grid, or NULL: gndtemp everywhere */
    float waveno[2];               /* cm^-1, band limits for units 'B' (band-integrated W/(m^2 sr)) */
} shdom_problem;

#ifdef __cplusplus
}
#endif
#endif
