"""Benchmark of the SHDOM solve + render path on GB300.

Workload (one step): the four-wavelength scalar scene -- a 128x128x64 grid
(dx=dy=0.02 km, dz=0.025 km), NMU=16 / NPHI=32 (NLM=256, 354 ordinates), a
seeded k^-5/3 power-law cloud field at 30% cloud fraction with lognormal
in-cloud extinction (mean 30/km), per-wavelength ssa 0.99999/0.9999/0.999/0.99
and Henyey-Greenstein g 0.85/0.84/0.82/0.80 (128 Legendre terms), open
boundaries (the workload does not state them), solar zenith 30 deg,
Lambertian albedo 0.05 -- solved to solution accuracy 1e-4 and rendered on
64x64 pixels x 9 view zeniths per wavelength.  All data synthetic (seeded).

value: solves/s with the medium resident in HBM (init + iterations + render
from device-resident rays; the four wavelengths solve at once,
SolversDict.solve(n_jobs=4) as in the reference's containers); e2e: the same
through the public host-buffer API (problem arrays and rays from host memory,
radiances back to host).

--impl reference times the CPU restatement of the reference Fortran
(oracle/, the reference's Fortran core cannot be compiled: no Fortran
compiler) on the same scenes.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NWAVE = 4
# DRAM bytes (read + write) per point-ordinate of one k_sweep_levels launch,
# from an ncu capture of that kernel on the 96x96x48 field (2.195 GB for
# 73.5M point-ordinates).
LEVELS_DRAM_BYTES_PER_ITEM = 29.9
# The same for one k_sweep_march launch, from an ncu capture of that kernel
# on the 96x96x48 field (1.846 GB for 78.3M point-ordinates).
MARCH_DRAM_BYTES_PER_ITEM = 23.6


def scenes(args):
    from at3d_gb300.scenes import cloud_field, orthographic_views
    pbs = [cloud_field(seed=2, wavelength_index=w, nx=args.nx, ny=args.nx, nz=args.nz,
                       boundary=args.boundary, solacc=args.solacc) for w in range(args.nwave)]
    rays = orthographic_views(pbs[0], args.npix, args.npix)
    return pbs, rays


def dist_init():
    """One process per GPU under torchrun; replicas only (at3d_gb300.replicas)."""
    from at3d_gb300 import replicas
    return replicas.init()


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    def __init__(self, gpu: int):
        self.gpu, self.samples, self.proc = gpu, [], None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons}


def gb300_arm(args, rank, ws):
    import torch
    from at3d_gb300.containers import SolversDict
    from at3d_gb300.solver import RTE

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    pbs, rays = scenes(args)
    nr = len(rays[0])
    rtes = [RTE.from_problem(pb, device=dev, name=f"wavelength {w}") for w, pb in enumerate(pbs)]
    for r in rtes:
        r.set_sweep_mode(args.sweep_mode)
    solvers = SolversDict()
    for w, r in enumerate(rtes):
        solvers.add_solver(w, r)
    d = [torch.tensor(np.asarray(r), dtype=torch.float32 if i < 3 else torch.float64, device="cuda")
         for i, r in enumerate(rays)]
    outs = [torch.empty(nr, dtype=torch.float32, device="cuda") for _ in range(args.nwave)]
    iters = [0] * args.nwave

    def step():
        # the wavelengths' solves (SolversDict.solve; n_jobs of them at once), then their renders
        solvers.solve(n_jobs=args.jobs, overwrite_solver=True, maxiter=args.maxiter, verbose=False)
        for w, r in enumerate(rtes):
            iters[w] = r.sizes["iters"]
            r.render_device(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), d[4].data_ptr(),
                            outs[w].data_ptr(), nr, 0)

    def barrier():
        from at3d_gb300 import replicas
        torch.cuda.synchronize()
        replicas.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    launches0 = sum(r.sizes["launches"] for r in rtes)
    phase = np.zeros(5)
    sweep_parts = np.zeros(3)  # prep-side ms, level-pass ms, hemisphere sweeps timed
    t_ev0, t_ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        barrier()
        t_ev0.record()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        t_ev1.record()
        barrier()
        wall = time.perf_counter() - t0
    launches = sum(r.sizes["launches"] for r in rtes) - launches0
    # per-kernel times (CUDA events on each handle's stream) from one more
    # step solved one wavelength at a time with the persistent sweep, for the roofline
    for w, r in enumerate(rtes):
        r.set_sweep_mode("persistent")  # per-phase event times need the launches one by one
        r.solve(args.maxiter, verbose=False)
        phase += np.asarray(r.timings(), np.float64)
        st = r.sweep_timings()
        sweep_parts += (st["prep"], st["levels"], st["sweeps"])
    ms_dev = t_ev0.elapsed_time(t_ev1)
    ms_step = max(ms_dev, wall * 1e3) / args.steps
    from at3d_gb300 import replicas
    ms_step = replicas.max_over_ranks(ms_step)  # the slowest rank's step
    solves_per_s = ws * args.nwave / (ms_step / 1e3)
    rays_per_s = ws * args.nwave * nr / (ms_step / 1e3)

    # ---- end to end through the host-buffer API (create + solve + render)
    def e2e_step():
        sd = SolversDict()
        for w, pb in enumerate(pbs):
            # host planning on background threads, overlapping the solves already running
            sd.add_solver(w, RTE.from_problem(pb, device=dev, defer=True))
        if args.sweep_mode != "persistent":
            for r in sd.values():
                r.set_sweep_mode(args.sweep_mode)
        sd.solve(n_jobs=args.jobs, maxiter=args.maxiter, verbose=False)
        res = [r.render(*rays) for r in sd.values()]
        for r in sd.values():
            r.close()
        return res

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    ne = max(1, args.steps // 2)
    for _ in range(ne):
        res = e2e_step()
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / ne
    h2d = 0
    for pb in pbs:
        for s in pb.species:
            h2d += s.extinction.nbytes + s.ssalb.nbytes + np.asarray(s.legcoef).nbytes
        h2d += pb.zlevels.nbytes
    h2d += args.nwave * sum(np.asarray(r, np.float32 if i < 3 else np.float64).nbytes for i, r in enumerate(rays))
    d2h = args.nwave * nr * 4
    e2e = {"value": ws * args.nwave / (e2e_ms / 1e3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms}

    # ---- roofline of the dominant kernel: the sweep's phase-2 pass, the plane
    # march (k_sweep_march) where both hemispheres march, else the level pass
    # (k_sweep_levels)
    s0 = rtes[0].sizes
    npts, nlm, nang = s0["npts"], s0["nlm"], s0["nang"]
    total_iters = sum(iters)
    names = ["transform_sh_to_do", "sweep", "transform_do_to_sh", "source"]
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    nsweeps = max(1.0, sweep_parts[2])
    items = npts * (nang / 2.0)                # point-ordinates of one hemisphere
    march = s0.get("march", 0) == 3 and rtes[0].sweep_mode != "levels_only"
    if march:
        # ordinate source read + radiance write per point-ordinate (the
        # source pass is fused; extinction and face geometry are per point)
        alg = 8.0 * items
        per_item = MARCH_DRAM_BYTES_PER_ITEM
        kernel, p1_name, p2_name = "k_sweep_march", "phase1", "plane_march"
    else:
        alg = 12.0 * items                     # (radsrc, tr) read + radiance write per point-ordinate
        per_item = LEVELS_DRAM_BYTES_PER_ITEM
        kernel, p1_name, p2_name = "k_sweep_levels", "phase1_and_source_pass", "level_pass"
    p2_ms = sweep_parts[1] / nsweeps           # mean CUDA-event time of one phase-2 launch
    achieved = alg / (p2_ms / 1e3) / 1e9
    # DRAM bytes per launch from ncu (96x96x48 capture, bytes per point-ordinate), scaled
    traffic = per_item * items if per_item else None
    roofline = {"kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic, "alg_bytes_per_launch": alg,
                "ms_per_launch": p2_ms, "peak_source": "measured" if peaks else "fallback",
                "phase_ms_per_iter": {n: float(phase[i] / max(1, total_iters)) for i, n in enumerate(names)},
                "sweep_ms_per_hemisphere": {p1_name: float(sweep_parts[0] / nsweeps), p2_name: float(p2_ms)}}
    if march:
        sz = rtes[0].sizes
        roofline["march_launch"] = {"clusters": [sz["march_units_down"], sz["march_units_up"]],
                                    "ctas_per_cluster": [sz["march_cluster_down"], sz["march_cluster_up"]]}
    # the whole iteration against the per-iteration algorithmic bytes of the scope table:
    # 4 NPTS (NLM (4 + 2 accel) + 8)
    it_ms = phase[4] / max(1, total_iters)
    b_it = 4.0 * npts * (nlm * 6 + 8)
    roofline["iteration"] = {"alg_bytes": b_it, "ms": float(it_ms), "achieved": b_it / (it_ms / 1e3) / 1e9,
                             "frac": b_it / (it_ms / 1e3) / 1e9 / hbm_peak}
    return dict(solves_per_s=solves_per_s, rays_per_s=rays_per_s, ms_step=ms_step, launches=launches,
                iters=list(iters), e2e=e2e, roofline=roofline, clocks=clk.summary(), npts=npts)


def relrms(a, b) -> float:
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


PRECISION_FIXTURE = os.path.join(ROOT, "tests", "golden", "fp64_cloud_field_128x128x64.npz")


def precision_block(args, dev):
    """The transform arithmetics on the benchmark scenes at a fixed iteration
    count: solves/s and rays/s of each mode (one step of all wavelengths,
    timed with CUDA events, inputs resident), and the relative RMS of its
    radiances against the plain FP32 GPU mode and against an FP64 run of the
    plain algorithm (committed fixture, made by
    tests/golden/make_fp64_fixture.py with the same scenes, rays and
    iteration count)."""
    import torch
    from at3d_gb300.scenes import cloud_field, orthographic_views
    fx = np.load(PRECISION_FIXTURE) if os.path.exists(PRECISION_FIXTURE) else None
    if fx is not None and (args.nx, args.nz, args.npix, args.boundary) != (128, 64, 64, "open"):
        fx = None  # the fixture holds the 128x128x64 open-boundary field at 64x64 pixels
    niter = int(fx["iterations"]) if fx is not None else 30
    pbs = [cloud_field(seed=2, wavelength_index=w, nx=args.nx, ny=args.nx, nz=args.nz, boundary=args.boundary,
                       solacc=0.0) for w in range(args.nwave)]
    rays = orthographic_views(pbs[0], args.npix, args.npix)
    nr = len(rays[0])
    from at3d_gb300.solver import RTE
    rtes = [RTE.from_problem(pb, device=dev) for pb in pbs]
    d = [torch.tensor(np.asarray(r), dtype=torch.float32 if i < 3 else torch.float64, device="cuda")
         for i, r in enumerate(rays)]
    outs = [torch.empty(nr, dtype=torch.float32, device="cuda") for _ in pbs]
    res = {}
    for mode in ("fp32", "tf32x3", "tf32"):
        for r in rtes:
            r.set_transform_mode(mode)
        ms = []
        for rep in range(2):  # the second pass is timed (the first warms the mode's code path)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for w, r in enumerate(rtes):
                r.solve(niter, verbose=False)
                r.render_device(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(),
                                d[4].data_ptr(), outs[w].data_ptr(), nr, 0)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        rad = [o.cpu().numpy() for o in outs]
        res[mode] = {"solves_per_s": len(rtes) / (ms[-1] / 1e3), "rays_per_s": len(rtes) * nr / (ms[-1] / 1e3),
                     "ms_per_step": ms[-1], "rad": rad}
    for r in rtes:
        r.close()
    out = {"iterations": niter, "modes": {}}
    for mode, v in res.items():
        e = {"solves_per_s": v["solves_per_s"], "rays_per_s": v["rays_per_s"], "ms_per_step": v["ms_per_step"],
             "relrms_vs_fp32": max(relrms(a, b) for a, b in zip(v["rad"], res["fp32"]["rad"]))}
        if fx is not None:
            e["relrms_vs_fp64"] = [relrms(a, fx[f"radiance_{w}"]) for w, a in enumerate(v["rad"])]
            e["max_relrms_vs_fp64"] = max(e["relrms_vs_fp64"])
        out["modes"][mode] = e
    out["fp64_reference"] = ("oracle FP64 (CPU restatement of the reference algorithm), same scenes, rays and "
                             f"{niter} iterations" if fx is not None else "fixture absent")
    return out


def gradient_block(args, dev):
    """Levis approximate gradient on the differentiation workload: 64x64x32
    cloud field at 20% cloud fraction, NMU=8/NPHI=16; L2 cost of 64x64-pixel
    radiances at 9 views against a target rendered from a second seeded
    field.  Times the gradient call (forward render with the adjoint
    weights + adjoint ray pass + direct-beam term, FP64 reductions) with
    the solved field resident."""
    import torch
    from at3d_gb300.scenes import cloud_field, orthographic_views
    from at3d_gb300.solver import RTE
    mk = lambda seed: cloud_field(seed=seed, nx=64, ny=64, nz=32, fraction=0.2, nmu=8, nphi=16, nleg=64,
                                  solacc=1e-4)
    pb, pt = mk(4), mk(5)
    rays = orthographic_views(pb, 64, 64)
    tgt = RTE.from_problem(pt, device=dev)
    tgt.solve(args.maxiter, verbose=False)
    meas = tgt.render(*rays)
    tgt.close()
    r = RTE.from_problem(pb, device=dev)
    t0 = time.perf_counter()
    it, _ = r.solve(args.maxiter, verbose=False)
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t0
    ms = []
    for rep in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g, cost, _ = r.levis_gradient(rays, meas, species=0)
        ms.append((time.perf_counter() - t0) * 1e3)
    r.close()
    nr = len(rays[0])
    return {"workload": "64x64x32 cloud field, 20% cloud fraction, NMU=8 NPHI=16, 64x64 px x 9 views",
            "ms_per_gradient": float(np.median(ms[1:])), "rays_per_s": nr / (np.median(ms[1:]) / 1e3),
            "solve_s": t_solve, "iterations": it, "cost": float(cost),
            "note": "host buffers in and out (rays, measurements, gradient), wall clock"}


def polarized_block(args, dev):
    """The polarized workload (NSTOKES=3): 64x64x40 grid with the cloud-blob
    geometry, NMU=8/NPHI=16, one six-element phase matrix (Rayleigh +
    HG-derived mix), Lambertian albedo 0.1, sun zenith 45 deg; Stokes I, Q, U
    on 64x64 pixels x 9 views.  Periodic boundaries (the stated
    configuration) and open boundaries.  For each transform arithmetic: a
    full solve (initialisation to convergence) plus the render, timed with
    CUDA events after a warm-up solve, inputs resident; the render alone;
    and the relative RMS of the I, Q, U images against the FP32 mode
    (normalised by the RMS of I).  With the CPU baseline: the polarized
    oracle, initialisation plus one iteration scaled to the solve's
    iterations, single thread."""
    import torch
    from at3d_gb300.scenes import orthographic_views, polarized_blob
    from at3d_gb300.solver import RTE
    out = {"workload": "NSTOKES=3 64x64x40 blob (dx=dy=0.02 km, dz=0.04 km), NMU=8 NPHI=16, "
                       "64x64 px x 9 views (I, Q, U)", "boundaries": {}}
    for bc in args.pol_boundaries:
        pb = polarized_blob(boundary=bc)
        rays = orthographic_views(pb, 64, 64)
        nr = len(rays[0])
        d = [torch.tensor(np.asarray(r), dtype=torch.float32 if i < 3 else torch.float64, device="cuda")
             for i, r in enumerate(rays)]
        img = torch.empty(nr * 3, dtype=torch.float32, device="cuda")
        res = {}
        for mode in ("fp32", "tf32x3"):
            r = RTE.from_problem(pb, device=dev)
            r.set_transform_mode(mode)
            ptrs = (d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), d[4].data_ptr(), img.data_ptr())
            r.solve(3, verbose=False)
            r.render_device(*ptrs, nr, 0)
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e[0].record()
            it, sc = r.solve(args.maxiter, verbose=False)
            e[1].record()
            r.render_device(*ptrs, nr, 0)
            e[2].record()
            torch.cuda.synchronize()
            t_solve, t_render = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
            res[mode] = {"iterations": it, "solcrit": sc, "ms_solve": t_solve, "ms_render": t_render,
                         "solves_per_s": 1e3 / (t_solve + t_render), "render_rays_per_s": nr / (t_render / 1e3),
                         "img": img.view(nr, 3).cpu().numpy().copy()}
            r.close()
        ref = res["fp32"]["img"]
        den = float(np.sqrt(np.mean(ref[:, 0].astype(np.float64) ** 2)))
        entry = {}
        for mode, v in res.items():
            dif = v.pop("img") - ref
            v["relrms_vs_fp32_iqu"] = [float(np.sqrt(np.mean(dif[:, k].astype(np.float64) ** 2)) / den) for k in range(3)]
            entry[mode] = v
        entry["rays"] = nr
        entry["mean_iqu"] = [float(np.mean(ref[:, k])) for k in range(3)]
        out["boundaries"][bc] = entry
    if not args.no_cpu_baseline and "periodic" in out["boundaries"]:
        from oracle.oracle import Oracle
        pb = polarized_blob(boundary="periodic")
        t0 = time.perf_counter()
        o = Oracle(pb)
        o.init_solution()
        t1 = time.perf_counter()
        o.solve(1)
        t2 = time.perf_counter()
        its = out["boundaries"]["periodic"]["fp32"]["iterations"]
        t = (t1 - t0) + its * (t2 - t1)
        out["cpu_baseline"] = {"value": 1.0 / t, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"polarized oracle on the periodic grid: initialisation ({t1 - t0:.1f} s) "
                                         f"plus one iteration ({t2 - t1:.1f} s), scaled to {its} iterations"}
    return out


def render_block(args, dev):
    """The render alone on the differentiation field (64x64x32 at 20% cloud,
    NMU 8 / NPHI 16, 64x64 px x 9 views = 36,864 rays), solved first: mean
    CUDA-event time of a device-resident render (rays and radiances in HBM)
    and of the host-buffer call."""
    import torch
    from at3d_gb300.scenes import cloud_field, orthographic_views
    from at3d_gb300.solver import RTE
    pb = cloud_field(seed=4, nx=64, ny=64, nz=32, fraction=0.2, nmu=8, nphi=16, nleg=64)
    rays = orthographic_views(pb, 64, 64)
    n = len(rays[0])
    r = RTE.from_problem(pb, device=dev)
    it, _ = r.solve(args.maxiter, verbose=False)
    d = [torch.tensor(np.asarray(x), dtype=torch.float32 if i < 3 else torch.float64, device=f"cuda:{dev}")
         for i, x in enumerate(rays)]
    out = torch.zeros(n, dtype=torch.float32, device=f"cuda:{dev}")
    st = torch.cuda.current_stream()
    args_dev = [t.data_ptr() for t in d] + [out.data_ptr(), n, st.cuda_stream]
    for _ in range(3):
        r.render_device(*args_dev)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        r.render_device(*args_dev)
    e1.record()
    torch.cuda.synchronize()
    ms_dev = e0.elapsed_time(e1) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        host = r.render(*rays)
    ms_host = (time.perf_counter() - t0) * 1e3 / reps
    r.close()
    return {"workload": "64x64x32 cloud field, 20% cloud fraction, NMU=8 NPHI=16, 64x64 px x 9 views",
            "rays": n, "iterations": it, "ms_device": ms_dev, "ms_host_buffers": ms_host,
            "rays_per_s": n / (ms_dev / 1e3), "mean_radiance": float(np.mean(host))}


def thermal_block(args, dev):
    """Thermal emission (srctype 'T') on the headline grid: the 128x128x64
    cloud field of wavelength 0 made an 11 um scene (cloud single-scattering
    albedo scaled by 0.55, temperature 290 K at the ground falling 6.5 K/km
    with a 4 K wave across x, 295 K ground of albedo 0.05, cold sky), one
    full solve (initialisation to convergence) plus the 64x64x9 render,
    timed with CUDA events after a warm-up solve, inputs resident."""
    import torch
    from at3d_gb300.scenes import cloud_field, orthographic_views
    from at3d_gb300.solver import RTE
    pb = cloud_field(seed=2, wavelength_index=0, nx=args.nx, ny=args.nx, nz=args.nz, boundary=args.boundary,
                     solacc=args.solacc)
    npx, npy, npz = pb.shape
    pb.species[0].ssalb = (np.asarray(pb.species[0].ssalb, np.float32) * 0.55).astype(np.float32)
    X, _, Z = np.meshgrid(np.arange(npx) * pb.delx, np.arange(npy) * pb.dely, pb.zlevels, indexing="ij")
    pb.temperature = (290.0 - 6.5 * Z + 4.0 * np.sin(2 * np.pi * X / (npx * pb.delx))).astype(np.float32)
    pb.srctype, pb.wavelength, pb.solarflux, pb.skyrad = "T", 11.0, 0.0, 0.0
    pb.ground_temperature, pb.surface_albedo = 295.0, 0.05
    rays = orthographic_views(pb, args.npix, args.npix)
    nr = len(rays[0])
    d = [torch.tensor(np.asarray(r), dtype=torch.float32 if i < 3 else torch.float64, device="cuda")
         for i, r in enumerate(rays)]
    img = torch.empty(nr, dtype=torch.float32, device="cuda")
    r = RTE.from_problem(pb, device=dev)
    ptrs = (d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), d[4].data_ptr(), img.data_ptr())
    r.solve(3, verbose=False)
    r.render_device(*ptrs, nr, 0)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    it, sc = r.solve(args.maxiter, verbose=False)
    e[1].record()
    r.render_device(*ptrs, nr, 0)
    e[2].record()
    torch.cuda.synchronize()
    t_solve, t_render = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    im = img.cpu().numpy()
    r.close()
    return {"workload": f"thermal 11 um, {npx}x{npy}x{npz} cloud field, NMU=16 NPHI=32, "
                        f"{args.npix}x{args.npix} px x 9 views", "iterations": it, "solcrit": sc,
            "ms_solve": t_solve, "ms_render": t_render, "solves_per_s": 1e3 / (t_solve + t_render),
            "render_rays_per_s": nr / (t_render / 1e3), "mean_radiance": float(im.mean()),
            "note": "no separate CPU baseline: the oracle's per-iteration cost is the headline cpu_baseline's"}


def config1_block(args, dev):
    """The plain scalar workload as stated: the 32x32x24 periodic cloud blob
    (two species: cloud with HG g 0.85 as 64 Legendre terms and a Rayleigh
    layer), NMU 8 / NPHI 16, solution accuracy 1e-5, 32x32 pixels x 9 view
    zeniths.  A full solve from initialisation plus the render, timed with
    CUDA events after a warm-up solve, inputs resident; beside it the oracle
    solving the same problem on one host thread (a full solve, measured)."""
    import torch
    from at3d_gb300.scenes import cloud_blob, orthographic_views
    from at3d_gb300.solver import RTE
    pb = cloud_blob()
    rays = orthographic_views(pb, 32, 32)
    nr = len(rays[0])
    d = [torch.tensor(np.asarray(r), dtype=torch.float32 if i < 3 else torch.float64, device="cuda")
         for i, r in enumerate(rays)]
    img = torch.empty(nr, dtype=torch.float32, device="cuda")
    r = RTE.from_problem(pb, device=dev)
    ptrs = (d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), d[4].data_ptr(), img.data_ptr())
    r.solve(args.maxiter, verbose=False)
    r.render_device(*ptrs, nr, 0)
    torch.cuda.synchronize()
    reps, ms = 3, []
    for _ in range(reps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        it, sc = r.solve(args.maxiter, verbose=False)
        e[1].record()
        r.render_device(*ptrs, nr, 0)
        e[2].record()
        torch.cuda.synchronize()
        ms.append((e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])))
    t_solve, t_render = (float(np.median([m[0] for m in ms])), float(np.median([m[1] for m in ms])))
    s = r.sizes
    out = {"workload": "32x32x24 periodic cloud blob + Rayleigh, NMU=8 NPHI=16, solacc 1e-5, 32x32 px x 9 views",
           "iterations": it, "solcrit": sc, "ms_solve": t_solve, "ms_render": t_render,
           "solves_per_s": 1e3 / (t_solve + t_render), "render_rays_per_s": nr / (t_render / 1e3),
           "sweep": "reference-order walk" if s["nlevels_down"] == 0 else f"{s['nlevels_down']} wavefront levels"}
    r.close()
    if not args.no_cpu_baseline:
        from oracle.oracle import Oracle
        t0 = time.perf_counter()
        o = Oracle(pb, fp64=False)
        ito, _ = o.solve(args.maxiter)
        t1 = time.perf_counter()
        o.render(*rays, nthreads=1)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"value": 1.0 / (t2 - t0), "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"the full solve ({ito} iterations, {t1 - t0:.2f} s) and render "
                                         f"({t2 - t1:.2f} s) of the same problem, measured, one host thread"}
    return out


def producers_block(args):
    """Host cost of the optical-property producers that feed a solve: a full
    water Mie table at 0.672 um (radii 0.08-65 um), the poly table of 25 x 2
    gamma distributions over it, and table_to_grid of a microphysics field
    on the benchmark grid (density from the benchmark cloud field, effective
    radius rising with height).  Wall clock, host threads."""
    from at3d_gb300 import medium, mie
    from at3d_gb300 import size_distribution as sd
    from at3d_gb300.scenes import cloud_field
    out = {"workload": "water Mie table 0.672 um (4-65 um), 25x2 gamma poly table, table_to_grid on "
                       f"{args.nx}x{args.nx}x{args.nz}", "host_threads": os.cpu_count()}
    t0 = time.perf_counter()
    mono = mie.get_mono_table("Water", (0.672, 0.672), refractive_index=1.331 - 1.6e-8j, verbose=False)
    out["mono_s"] = time.perf_counter() - t0
    out["mono_radii"], out["mono_legendre"] = int(mono.radius.size), int(mono.legendre.shape[1] - 1)
    t0 = time.perf_counter()
    grid = sd.get_size_distribution_grid(mono.radius, sd.gamma, reff={"coord_min": 4.0, "coord_max": 25.0,
                                                                       "npoints": 25, "spacing": "logarithmic"},
                                         veff=np.array([0.09, 0.11]))
    poly = mie.get_poly_table(grid, mono)
    out["poly_s"] = time.perf_counter() - t0
    pb = cloud_field(seed=2, wavelength_index=0, nx=args.nx, ny=args.nx, nz=args.nz)
    ext = np.asarray(pb.species[0].extinction, np.float64)
    z = np.linspace(0.0, 1.0, args.nz)[None, None, :]
    micro = {"density": ext / 150.0, "reff": np.broadcast_to(6.0 + 10.0 * z, ext.shape),
             "veff": np.full(ext.shape, 0.1)}
    t0 = time.perf_counter()
    sp = medium.table_to_grid(micro, poly)
    out["table_to_grid_s"] = time.perf_counter() - t0
    out["phase_functions"] = int(sp.legcoef.shape[0])
    return out


def serving_block(args, dev):
    """A Poisson stream of mixed requests through the continuous-admission
    loop (at3d_gb300.serving): grids 32x32x24 to 128x128x64, NMU/NPHI 8/16
    or 16/32, 1-8 wavelengths each, 32-64 px renders at 5 views."""
    from at3d_gb300.scenes import request_mix
    from at3d_gb300.serving import SolveServer, poisson_arrivals, run_stream
    out = []
    reqs = request_mix(100, args.serve_requests)  # the same requests at every rate and slot count
    runs = [(rate, slots) for rate in args.serve_rates for slots in args.serve_slots]
    for k, (rate, slots) in enumerate(runs):
        arr = poisson_arrivals(rate, len(reqs), seed=7 + args.serve_rates.index(rate))
        with SolveServer(device=dev, slots=slots) as srv:
            run_stream(srv, reqs, arr, maxiter=args.maxiter)
            st = srv.stats()
        st.update({"rate_per_s": rate, "requests": len(reqs), "slots": slots,
                   "wavelength_solves": int(sum(len(p) for p, _ in reqs))})
        out.append(st)
    return out


class CpuSolves:
    """The oracle (the C++ restatement of the reference Fortran) solving the
    benchmark wavelengths concurrently, one host thread per wavelength, as
    the reference's SolversDict.solve(n_jobs) does (at3d/containers.py:
    699-744; each solve is single-threaded Fortran).  The solves advance in
    slices: init() creates the solvers and runs INIT_SOLUTION; step(k)
    runs the next k iterations of every unconverged wavelength (each slice
    is one call of the solver's iteration loop, which restarts its
    acceleration state as SOLUTION_ITERATIONS does per call).  Every slice
    is timed with the wall clock; the iteration counts and the solution
    criteria come from the CPU solves themselves."""

    def __init__(self, pbs):
        from oracle.oracle import Oracle
        self.pbs = pbs
        self.Oracle = Oracle
        self.solacc = [pb.params.solution_accuracy for pb in pbs]

    def _parallel(self, fn):
        res = [None] * len(self.pbs)

        def run(w):
            res[w] = fn(w)

        th = [threading.Thread(target=run, args=(w,)) for w in range(len(self.pbs))]
        t0 = time.perf_counter()
        for t in th:
            t.start()
        for t in th:
            t.join()
        return time.perf_counter() - t0, res

    def init(self):
        self.orc = [None] * len(self.pbs)
        self.iters = [0] * len(self.pbs)
        self.crit = [[] for _ in self.pbs]  # solution criterion after each iteration

        def mk(w):
            self.orc[w] = self.Oracle(self.pbs[w], fp64=False)
            self.orc[w].init_solution()

        self.t_init, _ = self._parallel(mk)
        return self.t_init

    def converged(self, w):
        return bool(self.crit[w]) and self.crit[w][-1] <= self.solacc[w]

    def step(self, k: int = 1):
        def adv(w):
            for _ in range(k):
                if self.converged(w) or self.iters[w] >= 100:
                    break
                it, sc = self.orc[w].solve(self.iters[w] + 1)
                self.iters[w] = it
                self.crit[w].append(sc)

        wall, _ = self._parallel(adv)
        return wall

    def remaining_iterations(self, w):
        """Iterations still needed by wavelength w: 0 when converged, else
        the solution criterion's geometric trend over the last iterations
        extrapolated to the solution accuracy."""
        c = self.crit[w]
        if self.converged(w):
            return 0
        if len(c) < 3:
            return None
        y = np.log(np.asarray(c[-4:], np.float64))
        slope = np.polyfit(np.arange(len(y)), y, 1)[0]
        if slope >= 0:
            return None
        return int(np.ceil((np.log(self.solacc[w]) - y[-1]) / slope))


def cpu_solve_rate(pbs, iters_hint, slices: int = 1):
    """A bounded sample of the CPU solves (initialisation plus `slices`
    iterations of every wavelength at once), projected to a full solve with
    the measured mean iteration wall time: (solves/s, description)."""
    cs = CpuSolves(pbs)
    t_init = cs.init()
    walls = [cs.step(1) for _ in range(slices)]
    rem = [cs.remaining_iterations(w) for w in range(len(pbs))]
    need = max(cs.iters[w] + (rem[w] if rem[w] is not None else iters_hint[w] - cs.iters[w])
               for w in range(len(pbs)))
    t_it = float(np.mean(walls))
    t_solve = t_init + need * t_it
    cpu_solve_rate.last = cs
    return len(pbs) / t_solve, (f"{len(pbs)} wavelengths solved at once on {len(pbs)} host threads (oracle, the "
                                f"C++ restatement of the reference Fortran): initialisation {t_init:.1f} s plus "
                                f"{slices} iterations measured ({t_it:.1f} s each, wall), projected to {need} "
                                f"iterations per solve")


def cpu_render_sample(args, nrays: int = 4096):
    """The oracle's render of the first nrays rays of the benchmark views on
    every host core (one ray slice per thread, as the reference's joblib
    ray slicing), from the state of the last CPU sample: rays/s and cores."""
    _, rays = scenes(args)
    sub = tuple(np.ascontiguousarray(np.asarray(a)[:nrays]) for a in rays)
    cores = os.cpu_count() or 1
    o = cpu_solve_rate.last.orc[0]
    t0 = time.perf_counter()
    o.render(*sub, nthreads=cores)
    dt = time.perf_counter() - t0
    return nrays / dt, cores


def host_cpu():
    """Model name and logical core count of the host."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"model": model or "unknown", "logical_cores": os.cpu_count()}


def reference_arm(args, rank, ws):
    """The reference's CPU path timed on the host: the oracle solving the
    benchmark wavelengths concurrently, one thread per wavelength.  Each
    step is a measured slice of those solves (args.ref_slice iterations of
    every wavelength; the first step also holds the initialisation), and
    ms_per_step is the measured wall time of a timed step.  When the solves
    converge within the steps, the time per solve is measured in full;
    otherwise the remaining iterations come from the CPU solves' own
    convergence trend and the rate is marked projected."""
    if rank != 0:
        return None
    pbs, _ = scenes(args)
    cs = CpuSolves(pbs)
    t_init = cs.init()
    slices = [cs.step(args.ref_slice) for _ in range(args.warmup + args.steps)]
    walls = [w + (t_init if i == 0 else 0.0) for i, w in enumerate(slices)]  # per step, as run
    timed = walls[args.warmup:] if args.steps > 0 else walls
    ms_step = float(np.mean(timed)) * 1e3
    # the remaining iterations come from each CPU solve's own convergence trend, which
    # needs three solution criteria: a run shorter than that measures up to three more
    # slices (counted in the solves' time, not in the steps)
    extra_measured = 0
    while extra_measured < 3 and any(cs.remaining_iterations(w) is None and not cs.converged(w)
                                     for w in range(len(pbs))):
        slices.append(cs.step(args.ref_slice))
        extra_measured += 1
    # wall time of the concurrent solves: the initialisation and every measured slice, plus,
    # when they have not converged yet, the remaining slices at the mean wall of the last three
    rem = [cs.remaining_iterations(w) for w in range(len(pbs))]
    done = all(r == 0 for r in rem)
    extra, known = 0, True
    if not done:
        est = [r for r in rem if r is not None]
        known = len(est) == len(rem)
        extra = int(np.ceil(max(est, default=0) / max(1, args.ref_slice)))
    t_solves = t_init + float(np.sum(slices)) + extra * float(np.mean(slices[-3:]))
    v = len(pbs) / t_solves
    iters = [cs.iters[w] + (rem[w] or 0) for w in range(len(pbs))]
    sample = (f"one step = {args.ref_slice} iteration(s) of each of the {len(pbs)} wavelength solves at once "
              f"({len(pbs)} host threads, one per solve as SolversDict.solve(n_jobs)); initialisation "
              f"{t_init:.1f} s in the first step; {sum(cs.iters)} iterations measured in total")
    cpu = host_cpu()
    return {"metric": "SHDOM solves/s", "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": config_dict(args),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": len(pbs), "kind": "port", "sample": sample,
                             "host": cpu},
            "projection": {"projected": not done, "measured_iterations": list(cs.iters),
                           "iterations_per_solve": iters, "solution_criteria": [c[-1] if c else None
                                                                                for c in cs.crit],
                           "init_s": t_init, "step_walls_s": walls,
                           "remaining_slices_estimated": extra,
                           "slices_measured_beyond_the_steps": extra_measured,
                           "estimate_complete": known},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def config_dict(args):
    return {"workload": f"{args.nwave}-wavelength scalar SHDOM {args.nx}x{args.nx}x{args.nz}, NMU=16 NPHI=32, "
                        f"{args.npix}x{args.npix}x9 renders per wavelength",
            "grid": [args.nx, args.nx, args.nz], "wavelengths": args.nwave, "nmu": 16, "nphi": 32,
            "boundary": args.boundary, "solution_accuracy": args.solacc,
            "rays_per_wavelength": args.npix * args.npix * 9,
            "transform_mode": "tf32x3 (SH<->DO transforms on tcgen05 tensor cores, 3-product TF32 split, "
                              "FP32-level accuracy)",
            "sweep": "plane march (open boundaries) / level schedule / reference order (periodic), per hemisphere",
            "l2": "inputs larger than L2 (about 6 GB of state per wavelength)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=128)
    ap.add_argument("--nz", type=int, default=64)
    ap.add_argument("--npix", type=int, default=64)
    ap.add_argument("--boundary", default="open")
    ap.add_argument("--solacc", type=float, default=1e-4)
    ap.add_argument("--maxiter", type=int, default=100)
    ap.add_argument("--nwave", type=int, default=NWAVE, help="wavelengths per step (profiling runs use 1)")
    ap.add_argument("--ref-slice", type=int, default=1, help="CPU solve iterations per reference-arm step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep-mode", default="persistent", choices=["persistent", "per_level", "graph", "levels_only"],
                    help="RTE.set_sweep_mode of the headline solves")
    ap.add_argument("--jobs", type=int, default=1,
                    help="wavelengths solved at once (0: all; default 1, the fastest on one GPU: each solve's "
                         "plane march already fills it)")
    ap.add_argument("--no-extras", action="store_true", help="skip the precision, gradient and serving blocks")
    ap.add_argument("--serve-rates", type=str, default="1,4,16", help="Poisson arrival rates (requests/s) to run")
    ap.add_argument("--serve-requests", type=int, default=16)
    ap.add_argument("--serve-slots", type=str, default="4,8,16", help="slot counts to run at each rate")
    ap.add_argument("--only", default="", choices=["", "precision", "gradient", "polarized", "serving", "thermal",
                                                    "config1", "render"],
                    help="run one extra block alone and print its JSON (for profiling)")
    ap.add_argument("--pol-boundaries", type=str, default="periodic,open")
    args = ap.parse_args()
    args.serve_rates = [float(x) for x in args.serve_rates.split(",") if x]
    args.serve_slots = [int(x) for x in args.serve_slots.split(",") if x]
    args.pol_boundaries = [x for x in args.pol_boundaries.split(",") if x]
    args.jobs = args.jobs or args.nwave
    rank, ws = dist_init()
    if args.only:
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        blk = {"precision": precision_block, "gradient": gradient_block, "polarized": polarized_block,
               "serving": serving_block, "thermal": thermal_block, "config1": config1_block,
               "render": render_block}[args.only]
        print(json.dumps({args.only: blk(args, dev)}))
        return
    if args.impl == "reference":
        out = reference_arm(args, rank, ws)
        if out:
            print(json.dumps(out))
        return
    r = gb300_arm(args, rank, ws)
    if rank != 0:
        return
    extras = {}
    if ws == 1 and not args.no_extras:
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        extras["precision"] = precision_block(args, dev)
        extras["gradient"] = gradient_block(args, dev)
        extras["polarized"] = polarized_block(args, dev)
        extras["thermal"] = thermal_block(args, dev)
        extras["config1"] = config1_block(args, dev)
        extras["render"] = render_block(args, dev)
        extras["serving"] = serving_block(args, dev)
        extras["producers"] = producers_block(args)
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        pbs, _ = scenes(args)
        v, desc = cpu_solve_rate(pbs, r["iters"])
        rr, cores = cpu_render_sample(args)
        cpu = {"value": v, "unit": "solves/s", "cores": len(pbs), "kind": "port", "sample": desc,
               "projected": True, "host": host_cpu(),
               "render_rays_per_s": rr, "render_cores": cores,
               "render_sample": "4096 rays of the benchmark views, one ray slice per host core"}
    out = {"metric": "SHDOM solves/s", "value": r["solves_per_s"], "unit": "solves/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_step"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": config_dict(args), "rays_per_s": r["rays_per_s"], "iterations_per_solve": r["iters"],
           "e2e": r["e2e"], "gpu_launches": r["launches"], "roofline": r["roofline"], "cpu_baseline": cpu,
           "clocks": r["clocks"]}
    out.update(extras)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
