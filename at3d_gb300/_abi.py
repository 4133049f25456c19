"""ctypes mirror of ``include/shdom_problem.h`` and the numpy-side problem builder.

The problem struct carries plain pointers into numpy arrays; :class:`Problem`
keeps those arrays alive for as long as the struct is in use.  Field meanings
and layouts follow the arguments ``at3d.solver.RTE`` hands to the Fortran core
(at3d/solver.py:2324-2478 for the property arrays, at3d/solver.py:1960-2034
for the numerical parameters).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int)


class ShdomProblem(C.Structure):
    _fields_ = [
        ("npx", C.c_int), ("npy", C.c_int), ("npz", C.c_int),
        ("delx", C.c_float), ("dely", C.c_float),
        ("zlevels", _f),
        ("npart", C.c_int), ("maxnmicro", C.c_int),
        ("extinctp", _f), ("albedop", _f), ("iphasep", _i), ("phasewtp", _f),
        ("numphase", C.c_int), ("nlegp", C.c_int), ("legenp", _f),
        ("bc_x_open", C.c_int), ("bc_y_open", C.c_int), ("ipflag", C.c_int),
        ("solarflux", C.c_float), ("solarmu", C.c_float), ("solaraz", C.c_float), ("skyrad", C.c_float),
        ("sfc_variable", C.c_int), ("gndalbedo", C.c_float), ("gndtemp", C.c_float),
        ("nxsfc", C.c_int), ("nysfc", C.c_int), ("delxsfc", C.c_float), ("delysfc", C.c_float),
        ("sfc_albedo", _f),
        ("nmu", C.c_int), ("nphi", C.c_int), ("angle_set", C.c_int),
        ("deltam", C.c_int), ("accelflag", C.c_int), ("highorderrad", C.c_int), ("iterfixsh", C.c_int),
        ("solacc", C.c_float), ("shacc", C.c_float), ("splitacc", C.c_float),
        ("tautol", C.c_double), ("transcut", C.c_double),
        ("transmin", C.c_float),
        ("nstokes", C.c_int),
        ("sfc_brdf", C.c_int), ("nsfcpar", C.c_int), ("sfc_params", _f),
        ("srctype", C.c_int), ("units", C.c_int), ("wavelen", C.c_float),
        ("tempp", _f), ("sfc_temp", _f), ("waveno", C.c_float * 2),
    ]


def _fp(a):
    return a.ctypes.data_as(_f)


def _ip(a):
    return a.ctypes.data_as(_i)


@dataclass
class NumericalParams:
    """Numerical parameters with the reference defaults (default_config.json)."""
    num_mu_bins: int = 16
    num_phi_bins: int = 32
    deltam: bool = True
    acceleration_flag: bool = True
    solution_accuracy: float = 1e-4
    spherical_harmonics_accuracy: float = 0.0
    split_accuracy: float = 0.0
    high_order_radiance: bool = False
    iterfixsh: int = 30
    tautol: float = 0.1
    transcut: float = 1e-5
    transmin: float = 1.0
    angle_set: int = 2
    ip_flag: int = 0
    x_boundary_condition: str = "open"
    y_boundary_condition: str = "open"


@dataclass
class Species:
    """One scattering species on the property grid (a member of RTE.medium)."""
    extinction: np.ndarray            # [npx, npy, npz] 1/km
    ssalb: np.ndarray                 # [npx, npy, npz]
    legcoef: np.ndarray               # [nleg+1] or [ntable, nleg+1]; a_l with the 2l+1 factor.
                                      # Polarized problems: [6, nleg+1] or [ntable, 6, nleg+1], the
                                      # elements a1, a2, a3, a4, b1, b2 (at3d legcoef 'stokes_index')
    table_index: np.ndarray | None = None   # [nmicro, npx, npy, npz], 1-based into legcoef rows
    phase_weights: np.ndarray | None = None  # [nmicro, npx, npy, npz]


@dataclass
class Problem:
    """All inputs of one RTE solve, held as numpy arrays."""
    delx: float
    dely: float
    zlevels: np.ndarray
    species: list
    solarmu: float                    # SHDOM convention: negative, radiance propagation direction
    solaraz: float                    # radians
    solarflux: float = 1.0
    skyrad: float = 0.0
    surface_albedo: float | np.ndarray = 0.0
    surface_delx: float = 0.0
    surface_dely: float = 0.0
    params: NumericalParams = field(default_factory=NumericalParams)
    num_stokes: int = 1               # 1 (scalar) or 3 (I, Q, U)
    surface_brdf: str = ""            # '' Lambertian (surface_albedo), or 'R' / 'W' with surface_params
    surface_params: np.ndarray | None = None  # [nxsfc, nysfc, nparams] on (surface_delx, surface_dely)
    srctype: str = "S"                # 'S' solar, 'T' thermal, 'B' both (at3d.source solar/thermal/combined)
    units: str = "R"                  # thermal units: 'R' radiance, 'T' brightness temperature, 'B' band
    waveno: tuple = (10000.0, 10001.0)  # cm^-1 band limits for units 'B' (at3d.source's placeholder)
    wavelength: float = 0.0           # micron (Planck function)
    temperature: np.ndarray | None = None       # [npx, npy, npz] K, required for 'T' and 'B'
    ground_temperature: float | np.ndarray = 288.0  # K; an array lives on the surface grid [nxsfc, nysfc]
    _keep: list = field(default_factory=list, repr=False)

    @property
    def shape(self):
        return self.species[0].extinction.shape

    def to_struct(self) -> ShdomProblem:
        npx, npy, npz = self.shape
        ng = npx * npy * npz
        nspec = len(self.species)
        maxnmicro = max((s.table_index.shape[0] if s.table_index is not None else 1) for s in self.species)
        # Concatenate every species' Legendre table into one table
        # (at3d/solver.py:2376-2411): each species' indices are offset by the
        # number of rows already in the table.
        if self.num_stokes not in (1, 3):
            raise ValueError("num_stokes must be 1 or 3")
        pol = self.num_stokes == 3
        rows, offsets = [], []
        for s in self.species:
            lc = np.asarray(s.legcoef, dtype=np.float64)
            if pol:
                if lc.ndim == 2 and lc.shape[0] != 6:
                    raise ValueError("a polarized legcoef has the 6 elements a1 a2 a3 a4 b1 b2 as rows")
                lc = lc.reshape(-1, 6, lc.shape[-1])
            else:
                lc = np.atleast_2d(lc)
                if lc.ndim != 2:
                    raise ValueError("a scalar problem takes [nleg+1] or [ntable, nleg+1] legcoef")
            offsets.append(len(rows))
            rows.extend(list(lc))
        nl = self.params.num_mu_bins
        nmu = max(2, 2 * int((nl + 1) / 2))
        ml = nmu - 1
        nleg = ml + 1 if self.params.deltam else ml
        nlegp = max(max(r.shape[-1] for r in rows) - 1, nleg)
        if pol:
            # LEGENP(NSTLEG, 0:NLEGP, NUMPHASE): [numphase][nlegp+1][6]
            legenp = np.zeros((len(rows), nlegp + 1, 6), np.float32)
            for k, r in enumerate(rows):
                legenp[k, :r.shape[-1], :] = r.T
        else:
            legenp = np.zeros((len(rows), nlegp + 1), np.float32)
            for k, r in enumerate(rows):
                legenp[k, :len(r)] = r
        ext = np.zeros((nspec, ng), np.float32)
        alb = np.zeros((nspec, ng), np.float32)
        iph = np.ones((nspec, ng, maxnmicro), np.int32)
        pwt = np.zeros((nspec, ng, maxnmicro), np.float32)
        for k, s in enumerate(self.species):
            ext[k] = np.asarray(s.extinction, np.float32).reshape(-1)
            alb[k] = np.asarray(s.ssalb, np.float32).reshape(-1)
            if s.table_index is None:
                iph[k, :, 0] = 1 + offsets[k]
                pwt[k, :, 0] = 1.0
            else:
                nm = s.table_index.shape[0]
                iph[k, :, :nm] = (np.asarray(s.table_index).reshape(nm, -1).T + offsets[k]).astype(np.int32)
                pwt[k, :, :nm] = np.asarray(s.phase_weights, np.float32).reshape(nm, -1).T
        zl = np.ascontiguousarray(self.zlevels, np.float32)
        p = self.params
        st = ShdomProblem()
        st.npx, st.npy, st.npz = npx, npy, npz
        st.delx, st.dely = self.delx, self.dely
        st.zlevels = _fp(zl)
        st.npart, st.maxnmicro = nspec, maxnmicro
        st.extinctp, st.albedop, st.iphasep, st.phasewtp = _fp(ext), _fp(alb), _ip(iph), _fp(pwt)
        st.numphase, st.nlegp, st.legenp = legenp.shape[0], nlegp, _fp(legenp)
        st.bc_x_open = int(p.x_boundary_condition == "open")
        st.bc_y_open = int(p.y_boundary_condition == "open")
        st.ipflag = p.ip_flag
        st.solarflux, st.solarmu, st.solaraz, st.skyrad = self.solarflux, self.solarmu, self.solaraz, self.skyrad
        sa = np.asarray(self.surface_albedo, np.float32)
        keep = [zl, ext, alb, iph, pwt, legenp]
        if sa.size == 1:
            st.sfc_variable, st.gndalbedo = 0, float(sa.reshape(-1)[0])
            st.nxsfc = st.nysfc = 0
        else:
            sa2 = np.atleast_2d(sa)                   # [nxsfc, nysfc]
            buf = np.ascontiguousarray(sa2.T, np.float32)  # [nysfc][nxsfc]
            keep.append(buf)
            st.sfc_variable = 1
            st.nxsfc, st.nysfc = sa2.shape
            st.delxsfc, st.delysfc = self.surface_delx, self.surface_dely
            st.sfc_albedo = _fp(buf)
            st.gndalbedo = float(sa2.mean())
        gt = np.asarray(self.ground_temperature, np.float32)
        st.gndtemp = float(gt.reshape(-1)[0]) if gt.size == 1 else float(gt.mean())
        if self.surface_brdf:
            par = np.asarray(self.surface_params, np.float32)
            if par.ndim != 3:
                raise ValueError("surface_params is [nxsfc, nysfc, nparams]")
            buf = np.ascontiguousarray(par.transpose(1, 0, 2), np.float32)  # [nysfc][nxsfc][nparams]
            keep.append(buf)
            st.sfc_brdf = ord(self.surface_brdf)
            st.nsfcpar = par.shape[2]
            st.sfc_params = _fp(buf)
            st.sfc_variable = 0
            st.nxsfc, st.nysfc = par.shape[0], par.shape[1]
            st.delxsfc, st.delysfc = self.surface_delx, self.surface_dely
        st.nmu, st.nphi, st.angle_set = p.num_mu_bins, p.num_phi_bins, p.angle_set
        st.deltam, st.accelflag = int(p.deltam), int(p.acceleration_flag)
        st.highorderrad, st.iterfixsh = int(p.high_order_radiance), p.iterfixsh
        st.solacc, st.shacc, st.splitacc = p.solution_accuracy, p.spherical_harmonics_accuracy, p.split_accuracy
        st.tautol, st.transcut, st.transmin = p.tautol, p.transcut, p.transmin
        st.nstokes = self.num_stokes
        if self.srctype not in ("S", "T", "B"):
            raise ValueError("srctype must be 'S', 'T' or 'B'")
        if self.units not in ("R", "T", "B"):
            raise ValueError("units must be 'R' (radiance), 'T' (brightness temperature) or 'B' (band)")
        st.srctype, st.units, st.wavelen = ord(self.srctype), ord(self.units), float(self.wavelength)
        st.waveno[0], st.waveno[1] = float(self.waveno[0]), float(self.waveno[1])
        if self.srctype != "S":
            if self.temperature is None:
                raise KeyError("a thermal source needs the temperature of the medium")
            tp = np.ascontiguousarray(np.broadcast_to(np.asarray(self.temperature, np.float32), (npx, npy, npz)))
            keep.append(tp)
            st.tempp = _fp(tp)
            if gt.size > 1:
                if gt.shape != (st.nxsfc, st.nysfc):
                    raise ValueError("a ground temperature array lives on the surface grid [nxsfc, nysfc]")
                gbuf = np.ascontiguousarray(gt.T, np.float32)  # [nysfc][nxsfc]
                keep.append(gbuf)
                st.sfc_temp = _fp(gbuf)
        self._keep = keep
        return st
