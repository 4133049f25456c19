"""The request loop: results of requests solved concurrently (admitted by
slots and memory budget, overlapping on the device) equal the results of
the same requests solved alone; the loop reports p50 / p99 latency."""
import numpy as np
import pytest

from at3d_gb300.scenes import cloud_blob, cloud_field, orthographic_views

pytestmark = pytest.mark.gpu


def relrms(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


@pytest.fixture(scope="module")
def requests():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    out = []
    for i, (kind, n) in enumerate([("blob", 12), ("field", 16), ("blob", 16), ("field", 20), ("blob", 10), ("field", 12)]):
        if kind == "blob":
            pb = cloud_blob(seed=20 + i, nx=n, ny=n, nz=10, dx=0.04, dz=0.08)
        else:
            pb = cloud_field(seed=20 + i, wavelength_index=i % 4, nx=n, ny=n, nz=10, nmu=8, nphi=16, nleg=64)
        out.append((pb, orthographic_views(pb, 8, 8, zeniths=[0.0, 45.6])))
    return out


def test_mix_equals_alone(requests):
    from at3d_gb300.serving import SolveServer, poisson_arrivals, run_stream
    from at3d_gb300.solver import RTE
    alone = []
    for k, (pb, rays) in enumerate(requests):
        r = RTE.from_problem(pb)
        r.set_sweep_mode("graph")
        r.solve(100, verbose=False)
        alone.append(r.render(*rays))
        it_graph = r.sizes["iters"]
        r.close()
        if k < 2:  # the three sweep launch modes give the same field
            for mode in ("persistent", "per_level"):
                r = RTE.from_problem(pb)
                r.set_sweep_mode(mode)
                r.solve(100, verbose=False)
                assert r.sizes["iters"] == it_graph
                assert relrms(r.render(*rays), alone[-1]) < 1e-6
                r.close()
    with SolveServer(slots=3) as srv:
        res = run_stream(srv, requests, poisson_arrivals(200.0, len(requests), seed=3))
        st = srv.stats()
    assert st["completed"] == len(requests) and st["failed"] == 0
    assert st["peak_in_flight"] >= 2
    assert st["p50_ms"] is not None and st["p99_ms"] >= st["p50_ms"]
    for a, r in zip(alone, res):
        assert relrms(r.radiance, a) < 1e-6


def test_budget_admission(requests):
    from at3d_gb300.serving import SolveServer
    from at3d_gb300.solver import plan_summary
    need = [plan_summary(pb)["device_bytes"] for pb, _ in requests]
    # a budget that holds the largest request but not two of them
    budget = int(max(need) * 1.5)
    with SolveServer(slots=4, hbm_budget=budget) as srv:
        futs = [srv.submit(pb, rays) for pb, rays in requests]
        res = [f.result() for f in futs]
        st = srv.stats()
    assert st["completed"] == len(requests)
    assert st["peak_device_bytes"] <= budget
    too_big = SolveServer(slots=1, hbm_budget=min(need) // 2)
    with pytest.raises(MemoryError):
        too_big.submit(*requests[0]).result()
    too_big.close()


def test_solvers_dict_concurrent_equals_sequential(requests):
    """SolversDict.solve(n_jobs) (at3d/containers.py:699-742) solving several
    wavelengths at once gives each solver the result it has alone."""
    from at3d_gb300.containers import SolversDict
    from at3d_gb300.solver import RTE
    sub = requests[:4]
    alone = []
    for pb, rays in sub:
        r = RTE.from_problem(pb)
        r.solve(100, verbose=False)
        alone.append((r.sizes["iters"], r.render(*rays)))
        r.close()
    sd = SolversDict()
    for k, (pb, _) in enumerate(sub):
        sd.add_solver(k, RTE.from_problem(pb, defer=True))  # planned in the background
    sd.solve(n_jobs=4, maxiter=100, verbose=False)
    for k, (pb, rays) in enumerate(sub):
        r = sd[k]
        assert r.sweep_mode == "persistent"          # restored after the threaded solve
        assert r.sizes["iters"] == alone[k][0]
        assert relrms(r.render(*rays), alone[k][1]) < 1e-6
        assert r.check_solved(verbose=False)
        r.close()
