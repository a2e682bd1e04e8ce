"""GPU tests of batches (axg_batch_*): several solves advanced together, one
launch per colour and kernel class covering all of them, replayed from one
CUDA graph per step.

A solve's patches are processed in the same order, with the same summation,
in a batch as alone, so every result must be bit-for-bit the solve's own.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh, gauss_at
from axisem_gb300.solver import AxgError, Batch, Solver, symplectic_coefficients

pytestmark = pytest.mark.gpu

FIELDS = (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_ACC0, _abi.FIELD_CHI, _abi.FIELD_DCHI, _abi.FIELD_DDCHI0)


def _alone(m, comp=False):
    with Solver(m) as s:
        s.set_compensated(comp)
        s.run()
        return s.receivers(), {f: s.get_state(f) for f in FIELDS}


def _same(s, ref):
    rec, st = ref
    assert np.array_equal(s.receivers(), rec)
    for f, a in st.items():
        assert np.array_equal(s.get_state(f), a), f


def test_batch_uneven_meshes_equal_alone(gpu_lib):
    """Poles, mesh sizes, precision modes and run lengths all differ."""
    cases = [(coupled_mesh(16, 12, 4, 0, niter=40, num_rec=5), False),
             (coupled_mesh(24, 10, 6, 1, niter=40, num_rec=7, src_row=4), False),
             (coupled_mesh(10, 5, 4, 2, niter=40, num_rec=3), False),
             (coupled_mesh(32, 16, 8, 2, niter=40, num_rec=9, src_row=9), True),
             (coupled_mesh(8, 4, 0, 1, niter=40, num_rec=4), True)]          # no fluid
    refs = [_alone(m, c) for m, c in cases]
    solvers = [Solver(m) for m, _ in cases]
    try:
        for s, (_, c) in zip(solvers, cases):
            s.set_compensated(c)
        with Batch(solvers) as b:
            assert b.launches_per_step() > 0
            b.run([1] * len(solvers), 40)
        for s, ref in zip(solvers, refs):
            _same(s, ref)
    finally:
        for s in solvers:
            s.close()


def test_batch_staggered_starts_and_pieces(gpu_lib):
    """Solves join at different iterations; runs in pieces, alone and batched."""
    ma = coupled_mesh(12, 8, 4, 2, niter=60, num_rec=4)
    mb = coupled_mesh(12, 8, 4, 0, niter=45, num_rec=6, src_row=3)
    ra, rb = _alone(ma), _alone(mb)
    with Solver(ma) as a, Solver(mb) as b:
        a.run(1, 15)                      # a alone first
        with Batch([a, b]) as bt:
            bt.run([16, 1], 30)           # a 16..45, b 1..30
        b.run(31, 15)                     # b alone to its end (45)
        with Batch([a]) as bt:
            bt.run([46], 15)              # a 46..60
        _same(a, ra)
        _same(b, rb)


def test_batch_of_shared_meshes(gpu_lib):
    """Solves sharing one resident mesh (axg_create_sharing) in one batch."""
    base = coupled_mesh(16, 12, 4, 1, niter=50, num_rec=5)
    others = [coupled_mesh(16, 12, 4, 1, niter=50, num_rec=3 + k, src_row=2 + 2 * k) for k in range(4)]
    refs = [_alone(m) for m in others]
    with Solver(base) as holder:
        solvers = [Solver(m, share_with=holder) for m in others]
        try:
            with Batch(solvers) as b:
                b.run_async([1] * 4, 50)
                while not b.poll():
                    pass
            for s, ref in zip(solvers, refs):
                _same(s, ref)
        finally:
            for s in solvers:
                s.close()


def test_batch_larger_than_one_launch(gpu_lib):
    """More solves than one launch's descriptors hold (split into launches)."""
    meshes = [coupled_mesh(6, 3, 2, k % 3, niter=20, num_rec=2, src_row=1 + k % 2, seed=100 + k) for k in range(37)]
    refs = [_alone(m) for m in meshes]
    solvers = [Solver(m) for m in meshes]
    try:
        with Batch(solvers) as b:
            b.run([1] * len(solvers), 20)
        for s, ref in zip(solvers, refs):
            _same(s, ref)
    finally:
        for s in solvers:
            s.close()


def test_batch_blowup_is_reported_and_others_continue(gpu_lib):
    good = coupled_mesh(8, 4, 2, 0, niter=40, num_rec=3)
    bad = coupled_mesh(8, 4, 0, 0, niter=40)
    bad.magnitude = 1e-20
    ref = _alone(good)
    with Solver(good) as g, Solver(bad) as x:
        with Batch([g, x]) as b:
            with pytest.raises(AxgError) as ei:
                b.run([1, 1], 40)
            assert ei.value.code == _abi.AXG_ERR_BLOWUP
            assert "solve 1" in str(ei.value)
        _same(g, ref)


def test_batch_with_attenuated_members_equal_alone(gpu_lib):
    """cg4-attenuated solves (different SLS counts and poles, one compensated)
    batched with an elastic one: seismograms, fields and memory variables
    bit-for-bit their own."""
    cases = [(add_attenuation(coupled_mesh(16, 12, 4, 0, niter=40, num_rec=5, src_row=9), n_sls=5, seed=3), False),
             (add_attenuation(coupled_mesh(12, 10, 6, 1, niter=40, num_rec=4, src_row=7), n_sls=3, seed=4), False),
             (add_attenuation(coupled_mesh(20, 8, 4, 2, niter=40, num_rec=6, src_row=5), n_sls=5, seed=5), True),
             (coupled_mesh(10, 6, 3, 2, niter=40, num_rec=3), False)]
    refs = []
    for m, c in cases:
        with Solver(m) as s:
            s.set_compensated(c)
            s.run()
            mv = s.get_state(_abi.FIELD_MEMVAR) if m.anel else None
            refs.append((s.receivers(), {f: s.get_state(f) for f in FIELDS}, mv))
    assert np.abs(refs[0][2]).max() > 0
    solvers = [Solver(m) for m, _ in cases]
    try:
        for s, (_, c) in zip(solvers, cases):
            s.set_compensated(c)
        with Batch(solvers) as b:
            b.run([1] * len(solvers), 20)
            b.run([21] * len(solvers), 20)
        for s, (m, _), (rec, st, mv) in zip(solvers, cases, refs):
            _same(s, (rec, st))
            if m.anel:
                assert np.array_equal(s.get_state(_abi.FIELD_MEMVAR), mv)
    finally:
        for s in solvers:
            s.close()


def _stf_stages(m, scheme):
    _, _, coeff = symplectic_coefficients(scheme, m.deltat)
    return gauss_at(np.arange(m.niter)[:, None] * m.deltat + coeff[None, :], 20 * m.deltat)


def test_batch_with_symplectic_members_equal_alone(gpu_lib):
    """Symplectic solves of different stage counts (4, 5, 7, 17), one
    attenuated and one compensated, batched with Newmark ones: every solve
    bit-for-bit its own, run in two pieces."""
    cases = [(coupled_mesh(12, 8, 4, 0, niter=30, num_rec=4), _abi.SCHEME_SYMPLEC4, False),
             (add_attenuation(coupled_mesh(10, 6, 4, 1, niter=30, num_rec=3, src_row=4), n_sls=3, seed=8),
              _abi.SCHEME_ML_SO4M5, False),
             (coupled_mesh(14, 6, 5, 2, niter=30, num_rec=5), _abi.SCHEME_ML_SO6M7, True),
             (coupled_mesh(8, 5, 0, 2, niter=30, num_rec=2), _abi.SCHEME_KL_O8M17, False),
             (coupled_mesh(16, 10, 4, 1, niter=30, num_rec=6), _abi.SCHEME_NEWMARK2, False),
             (add_attenuation(coupled_mesh(12, 8, 3, 2, niter=30, num_rec=3, src_row=6), n_sls=5, seed=9),
              _abi.SCHEME_NEWMARK2, True)]

    def setup(s, m, scheme, comp):
        if scheme != _abi.SCHEME_NEWMARK2:
            s.set_time_scheme(scheme, _stf_stages(m, scheme))
        s.set_compensated(comp)

    refs = []
    for m, scheme, comp in cases:
        with Solver(m) as s:
            setup(s, m, scheme, comp)
            s.run()
            mv = s.get_state(_abi.FIELD_MEMVAR) if m.anel else None
            refs.append((s.receivers(), {f: s.get_state(f) for f in FIELDS if f != _abi.FIELD_ACC0}, mv))
    solvers = [Solver(m) for m, _, _ in cases]
    try:
        for s, (m, scheme, comp) in zip(solvers, cases):
            setup(s, m, scheme, comp)
        with Batch(solvers) as b:
            b.run([1] * len(solvers), 13)
            b.run([14] * len(solvers), 17)
        for s, (m, _, _), (rec, st, mv) in zip(solvers, cases, refs):
            _same(s, (rec, st))
            if m.anel:
                assert np.array_equal(s.get_state(_abi.FIELD_MEMVAR), mv)
    finally:
        for s in solvers:
            s.close()


def test_batch_rejects(gpu_lib):
    m = coupled_mesh(6, 3, 2, 0, niter=10)
    with Solver(m) as a, Solver(m) as ck:
        out = np.zeros((m.niter // m.seis_it + 1, 3, m.num_rec), np.float32, order="F")
        ck.set_seismogram_checkpoint(5, out)
        with pytest.raises(AxgError) as ei:
            Batch([a, ck])
        assert ei.value.code == _abi.AXG_ERR_UNSUPPORTED
        with pytest.raises(AxgError) as ei:
            Batch([a, a])
        assert ei.value.code == _abi.AXG_ERR_BAD_ARG
        with Batch([a]) as b:
            with pytest.raises(AxgError) as ei:
                b.run([5], 10)            # 5..14 > niter
            assert ei.value.code == _abi.AXG_ERR_BAD_ARG
