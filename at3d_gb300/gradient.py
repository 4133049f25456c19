"""Levis approximate gradient and its automatic-differentiation wrapper.

``levis_approximation_grad`` mirrors
``at3d.gradient.LevisApproxGradient.levis_approximation_grad``
(at3d/gradient.py:164-415) for one solver and one sensor: sub-pixel rays
with ray weights, the 'L2' and 'LL' cost functions with per-pixel
uncertainties, and the Jacobian at chosen property-grid indices.  It
returns the gradient of the cost with respect to the extinction and
single-scattering albedo of one species on the property grid, the cost,
the pixel values and the Jacobian.  The derivative is the reference's
Levis approximation (the radiance field is frozen; LEVISAPPROX_GRADIENT,
src/polarized/shdomsub4.f:288-809) computed by the GPU adjoint behind
``shdom_levis_adjoint``.

``LevisRender`` is a ``torch.autograd.Function`` of the species'
extinction and single-scattering albedo: its forward compares them with the
medium the solver holds, and when they differ it rebuilds the medium and
re-solves (``RTE.update_species`` then ``RTE.solve``) before rendering, so
the radiances are those of the given properties.  Its backward runs the
Levis adjoint with the incoming gradient as ray weights and returns
d/d(extinction) and d/d(albedo); for CUDA tensors the rays, weights and
gradient stay on the device (``shdom_levis_adjoint_device``).
"""
from __future__ import annotations

import numpy as np

from .solver import RTE


COST_FUNCTIONS = ("L2", "LL")


def cost_and_adjoint_weights(stokes, measurement, uncertainties, cost_function="L2"):
    """Cost and adjoint weights of each pixel (COMPUTE_ADJOINT_WEIGHTS,
    src/polarized/shdomsub4.f:3969-4034, the same sums as UPDATE_COSTFUNCTION
    :13-91).  stokes, measurement: [npix, nstokes] pixel values;
    uncertainties: [npix, nu, nu] inverse error covariances.  Returns the
    total cost and adj [npix, nstokes] with dCost/dStokes = adj:

    * 'L2': cost += 0.5 U[i, j] (R_i - M_i)^2 and adj_i += U[i, j] (R_i - M_i)
      for every i, j (the reference's weighted least squares, which weights
      each component's squared error by its row of U);
    * 'LL': the log radiance, 0.5 U[0, 0] (log R_0 - log M_0)^2, and with
      Q and U the log degree of linear polarization weighted by U[1, 1]."""
    st = np.asarray(stokes, np.float64)
    me = np.asarray(measurement, np.float64)
    if st.ndim == 1:
        st, me = st[:, None], me[:, None]
    un = np.asarray(uncertainties, np.float64)
    npix, nst = st.shape
    if un.ndim == 0:
        un = np.broadcast_to(un, (npix, 1, 1))
    adj = np.zeros((npix, nst))
    if cost_function == "L2":
        nu = un.shape[-1]
        if nu < nst:
            raise ValueError(f"L2 cost needs a {nst}x{nst} uncertainty matrix per pixel")
        err = st - me
        rowsum = un[:, :nst, :nst].sum(axis=2)
        cost = float(np.sum(0.5 * rowsum * err ** 2))
        adj = rowsum * err
    elif cost_function == "LL":
        if np.any(st[:, 0] <= 0) or np.any(me[:, 0] <= 0):
            raise ValueError("LL cost needs positive radiances and measurements")
        raderr = np.log(st[:, 0]) - np.log(me[:, 0])
        cost = float(np.sum(0.5 * raderr ** 2 * un[:, 0, 0]))
        adj[:, 0] = raderr * un[:, 0, 0] / st[:, 0]
        if nst > 1:
            p1 = st[:, 1] ** 2 + st[:, 2] ** 2
            dolp1 = np.sqrt(p1) / st[:, 0]
            dolp2 = np.sqrt(me[:, 1] ** 2 + me[:, 2] ** 2) / me[:, 0]
            dolperr = np.log(dolp1) - np.log(dolp2)
            cost += float(np.sum(0.5 * dolperr ** 2 * un[:, 1, 1]))
            adj[:, 1] = dolperr * un[:, 1, 1] * st[:, 1] / p1
            adj[:, 2] = dolperr * un[:, 1, 1] * st[:, 2] / p1
    else:
        raise ValueError(f"cost_function must be one of {COST_FUNCTIONS}, not '{cost_function}'")
    return cost, adj


def levis_approximation_grad(rte_solver: RTE, sensor: dict, measurements=None, species: int = 0,
                             cost_function: str = "L2", uncertainties=None, indices_for_jacobian=None,
                             stokes_weights=None):
    """Levis approximate gradient of the cost of one sensor's pixels with
    respect to the extinction and single-scattering albedo of one species
    on the property grid (LevisApproxGradient.levis_approximation_grad,
    at3d/gradient.py:164-415, adjoint branch of LEVISAPPROX_GRADIENT,
    src/polarized/shdomsub4.f:630-809), for a scalar solve:

    * the sensor's rays are rendered on the GPU and each pixel is the sum of
      its rays' radiances times their ``ray_weight`` (``pixel_index``; one
      ray per pixel when the sensor has no sub-pixel rays) times the pixel's
      Stokes weight;
    * the cost ('L2' or 'LL') and the pixels' adjoint weights come from
      ``cost_and_adjoint_weights`` with the pixels' inverse error
      covariances ``uncertainties`` ([npix, 1, 1], a scalar, or None for the
      identity);
    * the adjoint pass runs on the GPU with each ray weighted by its pixel's
      adjoint weight times its ray and Stokes weights.

    measurements: the measured pixel values [npix] (default ``sensor['I']``).
    indices_for_jacobian: flat property-grid indices (z fastest); when given,
    also d(pixel)/d(extinction, albedo) at those indices, [npix, nidx, 2],
    one adjoint pass per pixel (the Jacobian branch's per-pixel derivative).
    Returns (gradient [npx, npy, npz, 2], loss, pixel values, jacobian or None)."""
    if rte_solver.num_stokes != 1:
        raise NotImplementedError("the Levis gradient is built for scalar (num_stokes = 1) solves")
    rays = (sensor["ray_x"], sensor["ray_y"], sensor["ray_z"], sensor["ray_mu"], sensor["ray_phi"])
    nr = len(rays[0])
    pix = np.asarray(sensor.get("pixel_index", np.arange(nr)))
    rw = np.asarray(sensor.get("ray_weight", np.ones(nr)), np.float64)
    npix = int(pix.max()) + 1 if nr else 0
    sw = np.ones(npix) if stokes_weights is None else np.broadcast_to(np.asarray(stokes_weights, np.float64), (npix,))
    meas = np.asarray(sensor["I"] if measurements is None else measurements, np.float64).ravel()
    if meas.size != npix:
        raise ValueError(f"{meas.size} measurements for {npix} pixels")
    un = np.ones((npix, 1, 1)) if uncertainties is None else np.asarray(uncertainties, np.float64)
    if un.ndim == 0:
        un = np.broadcast_to(un, (npix, 1, 1))
    elif un.ndim == 1:
        un = un.reshape(npix, 1, 1)
    radiances = rte_solver.render(*rays).astype(np.float64)
    pixels = np.zeros(npix)
    np.add.at(pixels, pix, radiances * rw)
    pixels *= sw
    loss, adj = cost_and_adjoint_weights(pixels, meas, un, cost_function)
    weights = adj[pix, 0] * rw * sw[pix]
    gradient = rte_solver.levis_adjoint(rays, weights, species)
    jacobian = None
    if indices_for_jacobian is not None:
        idx = np.asarray(indices_for_jacobian, np.int64).ravel()
        jacobian = np.zeros((npix, idx.size, 2))
        for p in range(npix):
            w = np.where(pix == p, rw * sw[p], 0.0)
            jacobian[p] = rte_solver.levis_adjoint(rays, w, species).reshape(-1, 2)[idx]
    return gradient, loss, pixels, jacobian


def _torch():
    import torch
    return torch


def _device_rays(rays, device):
    torch = _torch()
    t = [torch.as_tensor(np.ascontiguousarray(r), dtype=torch.float32 if i < 3 else torch.float64).to(device)
         for i, r in enumerate(rays)]
    return t


class _LevisRenderFn:
    """Built lazily so that importing this module does not import torch."""
    cls = None

    @classmethod
    def get(cls):
        if cls.cls is None:
            torch = _torch()

            class LevisRender(torch.autograd.Function):
                @staticmethod
                def forward(ctx, extinction, ssalb, rte, rays, species, maxiter):
                    ext = extinction.detach().to("cpu", torch.float32).numpy()
                    alb = ssalb.detach().to("cpu", torch.float32).numpy()
                    cur_ext, cur_alb = rte.species_properties(species)
                    if ext.shape != cur_ext.shape or alb.shape != cur_alb.shape:
                        raise ValueError("extinction / ssalb must have the property-grid shape "
                                         f"{cur_ext.shape}")
                    if not (np.array_equal(ext, cur_ext) and np.array_equal(alb, cur_alb)):
                        rte.update_species(species, ext, alb)
                        rte.solve(maxiter, verbose=False)
                    elif not rte._initialized:
                        rte.solve(maxiter, verbose=False)
                    ctx.rte, ctx.species = rte, species
                    ctx.shape = tuple(extinction.shape)
                    ctx.device, ctx.dtype = extinction.device, extinction.dtype
                    nrays = len(rays[0])
                    if extinction.is_cuda:
                        # rays, radiances and (in backward) weights and gradient stay on the device
                        dev = torch.device("cuda", rte._device)
                        dr = _device_rays(rays, dev)
                        out = torch.empty(nrays, dtype=torch.float32, device=dev)
                        st = torch.cuda.current_stream(dev).cuda_stream
                        rte.render_device(*[t.data_ptr() for t in dr], out.data_ptr(), nrays, st)
                        ctx.dev_rays = (tuple(t.data_ptr() for t in dr), nrays)
                        ctx.keep = dr
                        ctx.rays = None
                        return out.to(device=extinction.device, dtype=extinction.dtype)
                    ctx.rays = rays
                    out = rte.render(*rays)
                    return torch.as_tensor(out, device=extinction.device, dtype=extinction.dtype)

                @staticmethod
                def backward(ctx, grad_out):
                    rte = ctx.rte
                    if ctx.rays is None:
                        dev = torch.device("cuda", rte._device)
                        w = grad_out.detach().to(device=dev, dtype=torch.float64).contiguous()
                        g = torch.empty(int(np.prod(ctx.shape)) * 2, dtype=torch.float64, device=dev)
                        st = torch.cuda.current_stream(dev).cuda_stream
                        rte.levis_adjoint_device(ctx.dev_rays, w.data_ptr(), g.data_ptr(), ctx.species, st)
                        g = g.view(ctx.shape + (2,)).to(device=ctx.device, dtype=ctx.dtype)
                    else:
                        w = grad_out.detach().to("cpu", torch.float64).numpy()
                        g = rte.levis_adjoint(ctx.rays, w, ctx.species)
                        g = torch.as_tensor(g, device=ctx.device, dtype=ctx.dtype)
                    return g[..., 0].reshape(ctx.shape), g[..., 1].reshape(ctx.shape), None, None, None, None

            cls.cls = LevisRender
        return cls.cls


def render_differentiable(rte: RTE, extinction, ssalb, rays, species: int = 0, maxiter: int = 100):
    """Radiances along `rays` for the medium whose species `species` has the
    given `extinction` and `ssalb` (torch tensors shaped like its property
    grid), differentiable with respect to both through the Levis adjoint.
    When the tensors differ from the medium `rte` holds, `rte` is updated to
    them and re-solved (up to `maxiter` iterations) first."""
    return _LevisRenderFn.get().apply(extinction, ssalb, rte, tuple(rays), species, maxiter)


class LevisApproxGradientUncorrelated:
    """Cost and Levis gradient of every sensor of a SensorsDict, wavelengths
    uncorrelated (LevisApproxGradient / LevisApproxGradientUncorrelated,
    at3d/gradient.py:21-449).

    On construction every instrument gets its uncertainty model (the
    ``NullUncertainty`` of ``gradient_kwargs['cost_function']`` when it has
    none, with a warning; a model assuming another cost function is an
    error), its uncertainties are evaluated, and with
    ``uncertainty_kwargs['add_noise']`` its measurements are perturbed by the
    model.  A call solves the solvers (``parallel_solve_kwargs``), runs
    ``levis_approximation_grad`` for every sensor with its solver (the key
    is the sensor's 'wavelength'), stores the forward pixel values in the
    matching sensor of ``forward_sensors`` (when given) and returns (loss,
    {solver key: gradient [npx, npy, npz, 2]}, Jacobian rows or None), the
    loss and gradients divided by the number of measurements.
    ``unknown_scatterers``: the species index whose extinction and albedo
    are differentiated."""

    def __init__(self, measurements, solvers, forward_sensors, unknown_scatterers, parallel_solve_kwargs=None,
                 gradient_kwargs=None, uncertainty_kwargs=None):
        import warnings

        from .containers import SensorsDict, SolversDict
        from .uncertainties import NullUncertainty
        if not isinstance(measurements, SensorsDict):
            raise TypeError(f"`measurements` should be of type '{SensorsDict}' not '{type(measurements)}'")
        if not isinstance(solvers, SolversDict):
            raise TypeError(f"`solvers` should be of type '{SolversDict}' not '{type(solvers)}'")
        if forward_sensors is not None and not isinstance(forward_sensors, SensorsDict):
            raise TypeError(f"`forward_sensors` should be of type '{SensorsDict}' not '{type(forward_sensors)}'")
        uncertainty_kwargs = dict(uncertainty_kwargs or {})
        if "add_noise" not in uncertainty_kwargs:
            uncertainty_kwargs["add_noise"] = False
        elif not isinstance(uncertainty_kwargs["add_noise"], bool):
            raise TypeError("uncertainty_kwargs['add_noise'] should be of boolean type.")
        gradient_kwargs = dict(gradient_kwargs if gradient_kwargs is not None else {"cost_function": "L2"})
        if "cost_function" not in gradient_kwargs:
            raise ValueError("'cost_function' must be specified in `gradient_kwargs`. Supported values are 'L2' "
                             "or 'LL'.")
        if not isinstance(gradient_kwargs["cost_function"], str):
            raise TypeError("gradient_kwargs['cost_function'] should be of string type.")
        self.measurements = measurements
        self.solvers = solvers
        self.forward_sensors = forward_sensors
        self.unknown_scatterers = unknown_scatterers
        self.parallel_solve_kwargs = dict({"maxiter": 100, "verbose": False, "init_solution": True},
                                          **(parallel_solve_kwargs or {}))
        self.gradient_kwargs = gradient_kwargs
        self.uncertainty_kwargs = uncertainty_kwargs
        cost = gradient_kwargs["cost_function"]
        for name, instrument in measurements.items():
            if instrument.get("uncertainty_model") is None:
                warnings.warn(f"No uncertainty model supplied for instrument '{name}'. Using "
                              "at3d_gb300.uncertainties.NullUncertainty, which is unweighted least squares.")
                measurements.add_uncertainty_model(name, NullUncertainty(cost))
            if measurements[name]["uncertainty_model"].cost_function != cost:
                raise ValueError(f"Uncertainty model's assumed cost_function "
                                 f"'{measurements[name]['uncertainty_model'].cost_function}' is inconsistent with "
                                 f"the one being used '{cost}'")
            measurements.calculate_uncertainties(name)
            if uncertainty_kwargs["add_noise"]:
                measurements.add_noise(name)

    def __call__(self):
        kw = dict(self.parallel_solve_kwargs)
        kw.setdefault("overwrite_solver", True)
        self.solvers.solve(**kw)
        idx = self.gradient_kwargs.get("indices_for_jacobian")
        loss, grads, jac = 0.0, {}, []
        for name, instrument in self.measurements.items():
            for i, sensor in enumerate(instrument["sensor_list"]):
                key = sensor["wavelength"]
                if key not in self.solvers:
                    raise KeyError(f"no solver for the sensor's wavelength {key}")
                g, l, pixels, j = levis_approximation_grad(
                    self.solvers[key], sensor, species=self.unknown_scatterers,
                    cost_function=self.gradient_kwargs["cost_function"],
                    uncertainties=np.asarray(sensor["uncertainties"]).transpose(2, 0, 1),
                    indices_for_jacobian=idx)
                loss += l
                grads[key] = grads[key] + g if key in grads else g
                if j is not None:
                    jac.append(j)
                if self.forward_sensors is not None:
                    self.forward_sensors[name]["sensor_list"][i]["I"] = pixels
        n = max(1, self.measurements.nmeasurements)
        return loss / n, {k: v / n for k, v in grads.items()}, (jac if jac else None)
