"""Host-side parts of the serving loop (no GPU): the seeded request stream
and the per-request mesh descriptors."""
import numpy as np

from axisem_gb300.serve import MESH_OF_PERIOD, request_mesh, request_stream


def test_request_stream_is_seeded():
    a, b = request_stream(16, 5.0, seed=3), request_stream(16, 5.0, seed=3)
    assert [(r.period, r.pole, r.n_rec, r.depth_km) for r in a] == [(r.period, r.pole, r.n_rec, r.depth_km) for r in b]
    assert all(x.t_arrive < y.t_arrive for x, y in zip(a, a[1:]))
    assert {r.period for r in request_stream(64, 5.0)} == set(MESH_OF_PERIOD)


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
