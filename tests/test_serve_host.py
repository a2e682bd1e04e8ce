"""Host-side parts of the serving loop (no GPU): the seeded request stream
and the per-request mesh descriptors on the PREM meshes."""
import numpy as np

from axisem_gb300.serve import PERIODS, request_mesh, request_stream


def test_request_stream_is_seeded():
    a, b = request_stream(16, 5.0, seed=3), request_stream(16, 5.0, seed=3)
    assert [(r.period, r.pole, r.n_rec, r.depth_km) for r in a] == [(r.period, r.pole, r.n_rec, r.depth_km) for r in b]
    assert all(x.t_arrive < y.t_arrive for x, y in zip(a, a[1:]))
    assert {r.period for r in request_stream(64, 5.0)} == set(PERIODS)


def test_request_meshes_of_one_key_are_one_mesh():
    """Requests on the same (period, pole) differ only in source, receivers
    and run length: everything axg_create_sharing takes from the mesh is
    equal."""
    reqs = [r for r in request_stream(64, 5.0, seed=5) if r.period == 50 and r.pole == 1][:2]
    a, b = request_mesh(reqs[0]), request_mesh(reqs[1])
    assert np.array_equal(a.igloc_solid, b.igloc_solid) and np.array_equal(a.igloc_fluid, b.igloc_fluid)
    for name in a.m_solid:
        assert np.array_equal(a.m_solid[name], b.m_solid[name])
    for name in a.m_fluid:
        assert np.array_equal(a.m_fluid[name], b.m_fluid[name])
    assert np.array_equal(a.inv_mass_rho, b.inv_mass_rho) and np.array_equal(a.bdry_matr, b.bdry_matr)
    assert a.niter == reqs[0].niter and b.niter == reqs[1].niter
    # the request's own source depth and receivers
    assert a.recfile_el.shape[0] == reqs[0].n_rec and b.recfile_el.shape[0] == reqs[1].n_rec
    assert abs(a.meta["source"]["depth_km"] - reqs[0].depth_km) < 60.0


# ---- the batched serving loop's logic, on fakes of the solve and batch objects

class _FakeSolver:
    def __init__(self, mesh, lib=None, share_with=None, **kw):
        self.mesh, self.shared, self.iters, self.closed, self.comp = mesh, share_with is not None, [], False, None

    def set_compensated(self, on):
        self.comp = on

    def info(self):
        return {"device_bytes": 1000, "mesh_bytes": 400 if self.shared else 0}

    def receivers(self):
        return np.array(self.iters, dtype=np.float32)

    def close(self):
        self.closed = True


class _FakeBatch:
    log = []

    def __init__(self, solvers):
        assert not any(s.closed for s in solvers)
        self.solvers, self.closed = solvers, False
        _FakeBatch.log.append(("create", tuple(id(s) for s in solvers)))

    def run_async(self, firsts, n):
        assert not self.closed
        for s, f in zip(self.solvers, firsts):
            assert f + n - 1 <= s.mesh.niter
            s.iters.extend(range(f, f + n))
        _FakeBatch.log.append(("run", tuple(id(s) for s in self.solvers), n))

    def poll(self):
        return True

    def close(self):
        self.closed = True


def _serve(monkeypatch, reqs, **kw):
    from axisem_gb300 import serve
    monkeypatch.setattr(serve, "Solver", _FakeSolver)
    monkeypatch.setattr(serve, "Batch", _FakeBatch)
    monkeypatch.setattr(serve, "plan_shape", lambda mesh, ctas, lib: (64, 1))
    _FakeBatch.log = []
    srv = serve.Server(lib=object(), **kw)
    stats = srv.run(reqs, batched=True)
    return srv, stats


def test_batched_loop_steps_every_solve_once(monkeypatch):
    from axisem_gb300.serve import Request
    reqs = [Request(k, 0.0005 * k, 50, k % 3, 100.0 * k, 20, 1800.0 + 200 * k, 0.05) for k in range(7)]
    srv, stats = _serve(monkeypatch, reqs, chunk=40)
    assert set(stats.results) == {r.rid for r in reqs}
    for r in reqs:  # each solve ran iterations 1..niter exactly once, in order
        assert np.array_equal(stats.results[r.rid].seismograms, np.arange(1, r.niter + 1, dtype=np.float32))
    runs = [e for e in _FakeBatch.log if e[0] == "run"]
    assert all(n <= 40 for _, _, n in runs)
    # a batch is created again only when its members change
    creates = [e[1] for e in _FakeBatch.log if e[0] == "create"]
    assert all(a != b for a, b in zip(creates, creates[1:]))
    assert stats.max_concurrent > 1 and srv.used == sum(srv.mesh_bytes.values())


def test_batched_loop_keeps_to_the_budget(monkeypatch):
    from axisem_gb300.serve import Request
    reqs = [Request(k, 0.0, 50, k % 3, 200.0, 20, 1800.0, 0.05) for k in range(4)]
    _, stats = _serve(monkeypatch, reqs, budget_bytes=1, chunk=32)
    assert len(stats.results) == 4 and stats.max_concurrent == 1


def test_served_solves_are_compensated_by_default(monkeypatch):
    from axisem_gb300 import serve
    from axisem_gb300.serve import Request
    made = []
    monkeypatch.setattr(serve, "Solver", lambda *a, **k: made.append(_FakeSolver(*a, **k)) or made[-1])
    monkeypatch.setattr(serve, "Batch", _FakeBatch)
    monkeypatch.setattr(serve, "plan_shape", lambda mesh, ctas, lib: (64, 1))
    serve.Server(lib=object()).run([Request(0, 0.0, 50, 1, 10.0, 20, 1800.0, 0.05)], batched=True)
    assert made and all(s.comp for s in made if s.shared)


def test_concurrent_loop_steps_every_solve_once(monkeypatch):
    from axisem_gb300 import serve
    from axisem_gb300.serve import Request

    class S(_FakeSolver):
        def run_async(self, first, n):
            assert first + n - 1 <= self.mesh.niter
            self.iters.extend(range(first, first + n))

        def poll(self):
            return True

    monkeypatch.setattr(serve, "Solver", S)
    monkeypatch.setattr(serve, "plan_shape", lambda mesh, ctas, lib: (64, 1))
    reqs = [Request(k, 0.0003 * k, 25 if k % 2 else 50, k % 3, 50.0 * k, 30, 2000.0, 0.05) for k in range(6)]
    for seq in (False, True):
        srv = serve.Server(lib=object(), chunk=48)
        stats = srv.run(reqs, sequential=seq)
        for r in reqs:
            assert np.array_equal(stats.results[r.rid].seismograms, np.arange(1, r.niter + 1, dtype=np.float32))
        assert (stats.max_concurrent == 1) == seq


def test_resident_meshes_take_the_shared_patch_shape(monkeypatch):
    """The server plans its resident meshes for launches the mesh fills
    (concurrent solves fill the GPU together); with tuning="alone" they take
    axg_create's own tuning."""
    from axisem_gb300 import serve
    from axisem_gb300.serve import Request
    made, asked = [], []
    monkeypatch.setattr(serve, "Solver", lambda *a, **k: made.append((k.get("patch_elems"), k.get("growth"))) or
                        _FakeSolver(*a, **k))
    monkeypatch.setattr(serve, "plan_shape", lambda mesh, ctas, lib: asked.append(ctas) or (56, 0))
    req = Request(0, 0.0, 50, 1, 10.0, 20, 1800.0, 0.05)
    serve.Server(lib=object())._holder(req)
    assert made == [(56, 0)] and asked == [0]
    made.clear()
    serve.Server(lib=object(), tuning="alone")._holder(req)
    assert made == [(0, -1)] and asked == [0]
