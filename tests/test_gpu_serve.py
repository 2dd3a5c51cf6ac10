"""A job's result is the same alone and in the mix: four jobs of different
boards run one at a time, then together through the server (own CUDA stream
and state each, admitted concurrently); every path and tally must match."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from orthoroute_gb300.serve import RouteJob, RouteServer


def _bounds(nx, ny, pitch=0.4):
    sx = (nx - 1) * pitch - 6.0 + 1e-6
    sy = (ny - 1) * pitch - 6.0 + 1e-6
    return (7.0, 7.0, 10.0 + sx + 3.0, 10.0 + sy + 3.0)


def _nets(nx, ny, n, seed, dmax=60):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        x0, x1 = rng.integers(0, nx, size=2)
        y0, y1 = rng.integers(0, ny, size=2)
        if 4 <= abs(int(x1) - int(x0)) + abs(int(y1) - int(y0)) <= dmax:
            out.append((f"N{len(out)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
    return out


def _jobs():
    spec = [(40, 36, 6, 50, 1), (48, 40, 8, 60, 2), (140, 40, 6, 30, 3), (36, 30, 4, 40, 4)]
    return [RouteJob(f"J{i}", nx, ny, nz, _nets(nx, ny, n, seed, dmax=160), max_iterations=5,
                     bounds=_bounds(nx, ny)) for i, (nx, ny, nz, n, seed) in enumerate(spec)]


def test_jobs_alone_and_in_the_mix_agree():
    alone_srv = RouteServer(slots=1)
    alone = [f.result() for f in [alone_srv.submit(j) for j in _jobs()]]
    alone_srv.close()
    mix_srv = RouteServer(slots=4)
    mixed = [f.result() for f in [mix_srv.submit(j) for j in _jobs()]]
    mix_srv.close()
    assert mix_srv.peak_running >= 2
    for a, m in zip(alone, mixed):
        assert a.error is None and m.error is None, (a.error, m.error)
        assert a.result == m.result, a.name


def test_job_writes_its_solution_as_ors(tmp_path):
    from orthoroute_gb300 import ors
    job = _jobs()[0]
    job.ors_path = str(tmp_path / "J0.ORS")
    srv = RouteServer(slots=1)
    res = srv.submit(job).result()
    srv.close()
    assert res.error is None, res.error
    geom, md = ors.import_solution_from_ors(job.ors_path)
    assert md["metadata"]["board_name"] == "J0"
    assert md["metadata"]["total_iterations"] == res.result["iterations"]
    assert len(md["iteration_metrics"]) == res.result["iterations"]
    routed = {n for n, p in res.result["paths"].items() if len(p) >= 2}
    assert set(geom["by_net"]) <= routed and geom["all_tracks"]


def test_concurrent_whole_lattice_searches_agree():
    """Two jobs whose nets all need whole-lattice searches (Manhattan length
    >= 125), each on its share of the resident CTAs, run together: the same
    paths and tallies as each job alone on the whole GPU."""
    def long_nets(n, seed, nx=170, ny=40):
        rng = np.random.default_rng(seed)
        out = []
        for k in range(n):
            x0, x1 = int(rng.integers(0, 15)), int(rng.integers(nx - 15, nx))
            y0, y1 = int(rng.integers(0, ny)), int(rng.integers(0, ny))
            out.append((f"N{k}", y0 * nx + x0, y1 * nx + x1))
        return out

    def jobs():
        return [RouteJob(f"W{i}", 170, 40, 6, long_nets(6, 30 + i), max_iterations=3, bounds=_bounds(170, 40))
                for i in range(2)]
    js = jobs()
    assert all(abs(s % 170 - d % 170) + abs(s // 170 - d // 170) >= 125 for j in js for _, s, d in j.requests)
    alone_srv = RouteServer(slots=1, sm_share=False)
    alone = [f.result() for f in [alone_srv.submit(j) for j in jobs()]]
    alone_srv.close()
    mix_srv = RouteServer(slots=2)
    mixed = [f.result() for f in [mix_srv.submit(j) for j in jobs()]]
    mix_srv.close()
    assert mix_srv.peak_running == 2
    for a, m in zip(alone, mixed):
        assert a.error is None and m.error is None, (a.error, m.error)
        assert a.result == m.result, a.name
