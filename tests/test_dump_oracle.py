"""CPU checks of the oracle's restatement of the kernel wavefield dumps
(compute_strain, dump_*_global, SOLVER/time_evol_wave.F90:1264-1410,
SOLVER/wavefields_io.f90:840-1115).  The reference has no known answers for
the dumps; these pin the restatement's structure: the displacement fields are
the state itself (dipole: +/- to s/phi), the strain is linear in the state,
float and double agree, and a sub-range of points is the slice of the full
range."""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_pointwise, coupled_mesh, dump_desc
from oracle import oracle as orc


def _state(m, seed=5):
    rng = np.random.default_rng(seed)
    d = rng.normal(0, 1, (5, 5, m.nel_solid, 3))
    v = rng.normal(0, 1, (5, 5, m.nel_solid, 3))
    c = rng.normal(0, 1, (5, 5, m.nel_fluid))
    dc = rng.normal(0, 1, (5, 5, m.nel_fluid))
    return d, v, c, dc


def _nfields(pole, t, fluid):
    nm = pole != 0
    strain = 6 if nm else 4
    vec = 3 if nm else 2
    return {1: vec, 2: strain, 3: (2 if fluid else 2 * vec), 4: strain + vec}[t]


@pytest.mark.parametrize("pole", [0, 1, 2])
def test_displ_fields_are_the_state(pole):
    m = add_pointwise(coupled_mesh(6, 3, 2, pole, niter=4))
    d, v, c, dc = _state(m)
    dd = dump_desc(m, _abi.DUMP_DISPL_ONLY, 1, None, 1)
    out, nfld = orc.wavefield_dump(m, dd, d, v, c, dc)
    nes = m.nel_solid
    f = out[: _nfields(pole, 1, False) * nes * 25].reshape(-1, nes, 25)
    u = d.reshape(25, nes, 3, order="F").transpose(1, 0, 2)  # (nel, 25, 3)
    if pole == 1:
        assert np.array_equal(f[0], u[..., 0] + u[..., 1]) and np.array_equal(f[1], u[..., 0] - u[..., 1])
    elif pole == 2:
        assert np.array_equal(f[0], u[..., 0]) and np.array_equal(f[1], u[..., 1])
    else:
        assert np.array_equal(f[0], u[..., 0])
    assert np.array_equal(f[-1], u[..., 2])
    assert nfld == _nfields(pole, 1, False) + _nfields(pole, 1, True)


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("dtype_", [2, 4])
def test_strain_linear_and_precisions_agree(pole, dtype_):
    m = add_pointwise(coupled_mesh(6, 3, 2, pole, niter=4))
    a, b = _state(m, 1), _state(m, 2)
    dd = dump_desc(m, dtype_, 1, None, 1)
    fa = orc.wavefield_dump(m, dd, *a)[0]
    fb = orc.wavefield_dump(m, dd, *b)[0]
    fab = orc.wavefield_dump(m, dd, *[2.0 * x - 0.5 * y for x, y in zip(a, b)])[0]
    assert np.abs(fa).max() > 0
    lin = 2.0 * fa - 0.5 * fb
    assert np.linalg.norm(fab - lin) <= 1e-12 * np.linalg.norm(lin)
    f32 = orc.wavefield_dump(m, dd, *a, dtype=np.float32)[0]
    assert np.linalg.norm(f32 - fa) <= 1e-5 * np.linalg.norm(fa)


def test_sub_range_is_a_slice():
    m = add_pointwise(coupled_mesh(6, 3, 2, 2, niter=4))
    st = _state(m)
    full, n = orc.wavefield_dump(m, dump_desc(m, _abi.DUMP_FULLFIELDS, 1, None, 1), *st)
    part, n2 = orc.wavefield_dump(m, dump_desc(m, _abi.DUMP_FULLFIELDS, 1, None, 1, 1, 3, 0, 2), *st)
    assert n == n2
    nes, nef = m.nel_solid, m.nel_fluid
    ns = _nfields(2, 4, False)
    fs = full[: ns * nes * 25].reshape(ns, nes, 5, 5, order="C")       # (field, e, j, i)
    ps = part[: ns * nes * 9].reshape(ns, nes, 3, 3, order="C")
    assert np.array_equal(ps, fs[:, :, 0:3, 1:4])
    ff = full[ns * nes * 25: ns * nes * 25 + n2 * 0 + _nfields(2, 4, True) * nef * 25].reshape(-1, nef, 5, 5)
    pf = part[ns * nes * 9: ns * nes * 9 + _nfields(2, 4, True) * nef * 9].reshape(-1, nef, 3, 3)
    assert np.array_equal(pf, ff[:, :, 0:3, 1:4])
