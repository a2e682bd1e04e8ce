"""GPU tests of the kernel wavefield dumps (axg_set_wavefield_dump; dump_stuff,
SOLVER/time_evol_wave.F90:1201-1249).

Each snapshot is checked against the FP64 oracle (compute_strain and the
dump_* routines restated) evaluated on the very state the GPU dumped: a second
solve without dumps, stepped to each dump iteration (bit-identical, the solve
being deterministic), provides it through axg_get_state.  Tolerance: relative
L2 <= 2e-5 per field (FP32 derivatives with fused multiply-adds against FP64).
The dumps must leave the solve itself unchanged bit for bit.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_pointwise, coupled_mesh, dump_desc
from axisem_gb300.solver import AxgError, Batch, Solver

pytestmark = pytest.mark.gpu

TOL = 2e-5
TYPES = [_abi.DUMP_DISPL_ONLY, _abi.DUMP_STRAIN_ONLY, _abi.DUMP_DISPL_VELO, _abi.DUMP_FULLFIELDS]


def _mesh(pole, niter=24, **kw):
    return add_pointwise(coupled_mesh(10, 5, 4, pole, niter=niter, **kw))


def _check_snapshots(m, dump_type, snaps, ns, nf, names, strain_it, rng_ij=(0, 4, 0, 4), comp=False,
                     src_mask=False):
    np_el = (rng_ij[1] - rng_ij[0] + 1) * (rng_ij[3] - rng_ij[2] + 1)
    nes, nef = m.nel_solid, m.nel_fluid
    dd = dump_desc(m, dump_type, strain_it, None, 1, *rng_ij, src_mask=src_mask)
    with Solver(m) as s:
        s.set_compensated(comp)
        for k in range(snaps.shape[0]):
            s.run(k * strain_it + 1, strain_it)
            st = [s.get_state(f) for f in (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_CHI, _abi.FIELD_DCHI)]
            ref, nfld = orc_dump(m, dd, st)
            assert nfld == ns + nf
            for q in range(ns + nf):
                n_el = nes if q < ns else nef
                off = (q * nes if q < ns else ns * nes + (q - ns) * nef) * np_el
                g = snaps[k, off: off + n_el * np_el].astype(np.float64)
                r = ref[off: off + n_el * np_el]
                if not r.any():                    # the fluid's p components are zero
                    assert not g.any(), (k, names[q])
                    continue
                assert np.linalg.norm(g - r) <= TOL * np.linalg.norm(r), (k, names[q])


def orc_dump(m, dd, st):
    from oracle import oracle as orc
    return orc.wavefield_dump(m, dd, *st, dtype=np.float64)


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("dtype_", TYPES)
def test_dump_parity(gpu_lib, pole, dtype_):
    m = _mesh(pole)
    strain_it = 4
    with Solver(m) as s:
        snaps = s.set_wavefield_dump(dtype_, strain_it, capacity=m.niter // strain_it)
        ns, nf, floats, names = s.dump_layout()
        assert snaps.shape == (6, floats) and len(names) == ns + nf
        s.run()
        rec = s.receivers()
    assert np.abs(snaps).max() > 0
    _check_snapshots(m, dtype_, snaps, ns, nf, names, strain_it)
    with Solver(m) as plain:                      # the dumps leave the solve unchanged
        plain.run()
        assert np.array_equal(plain.receivers(), rec)


def test_dump_sub_range_and_pieces(gpu_lib):
    """Points (1:3, 0:2) of each element; a run in pieces whose boundaries
    do not fall on dump steps; steps per graph unlike strain_it."""
    m = _mesh(2, niter=30)
    with Solver(m) as s:
        s.set_tuning(steps_per_graph=8)
        snaps = s.set_wavefield_dump(_abi.DUMP_FULLFIELDS, 3, capacity=10, ibeg=1, iend=3, jbeg=0, jend=2)
        ns, nf, floats, names = s.dump_layout()
        assert floats == 9 * (ns * m.nel_solid + nf * m.nel_fluid)
        s.run(1, 7)
        s.run(8, 11)
        s.run(19, 12)
    _check_snapshots(m, _abi.DUMP_FULLFIELDS, snaps, ns, nf, names, 3, rng_ij=(1, 3, 0, 2))


def test_dump_compensated_and_names(gpu_lib):
    m = _mesh(1, niter=16)
    with Solver(m) as s:
        s.set_compensated(True)
        snaps = s.set_wavefield_dump(_abi.DUMP_STRAIN_ONLY, 8, capacity=2)
        ns, nf, _, names = s.dump_layout()
        s.run()
    assert names[:6] == ["strain_dsus_sol", "strain_dsuz_sol", "strain_dpup_sol", "straintrace_sol",
                         "strain_dsup_sol", "strain_dzup_sol"]
    assert names[6:] == [n.replace("_sol", "_flu") for n in names[:6]]
    _check_snapshots(m, _abi.DUMP_STRAIN_ONLY, snaps, ns, nf, names, 8, comp=True)


@pytest.mark.parametrize("dtype_", [_abi.DUMP_DISPL_ONLY, _abi.DUMP_FULLFIELDS])
def test_dump_source_mask(gpu_lib, dtype_):
    """src_dump_type = 'mask' (the reference's default): the solid fields
    are zero on the source elements and as without the mask elsewhere; the
    whole snapshot against the oracle's masked dump."""
    m = _mesh(1, niter=16)
    with Solver(m) as s:
        snaps = s.set_wavefield_dump(dtype_, 8, capacity=2, src_mask=True)
        ns, nf, _, names = s.dump_layout()
        s.run()
    with Solver(m) as s:
        plain = s.set_wavefield_dump(dtype_, 8, capacity=2)
        s.run()
    nes = m.nel_solid
    src = np.asarray(m.ielsrc[:m.nelsrc], dtype=np.int64) - 1
    for q in range(ns):
        a = snaps[:, q * nes * 25:(q + 1) * nes * 25].reshape(2, nes, 25)
        b = plain[:, q * nes * 25:(q + 1) * nes * 25].reshape(2, nes, 25)
        assert not a[:, src].any()
        keep = np.setdiff1d(np.arange(nes), src)
        assert np.array_equal(a[:, keep], b[:, keep])
        assert np.abs(b[:, src]).max() > 0 or q == 1
    assert np.array_equal(snaps[:, ns * nes * 25:], plain[:, ns * nes * 25:])   # the fluid is not masked
    _check_snapshots(m, dtype_, snaps, ns, nf, names, 8, src_mask=True)


def test_dump_errors(gpu_lib):
    m = _mesh(0, niter=12)
    with Solver(m) as s:
        s.set_wavefield_dump(_abi.DUMP_DISPL_ONLY, 2, capacity=3)
        with pytest.raises(AxgError) as ei:
            s.run()                               # 6 snapshots, room for 3
        assert ei.value.code == _abi.AXG_ERR_BAD_ARG
        with pytest.raises(AxgError) as ei:
            Batch([s])                            # a dumping solve runs alone
        assert ei.value.code == _abi.AXG_ERR_UNSUPPORTED
        with pytest.raises(AxgError):
            s.set_wavefield_dump(_abi.DUMP_DISPL_ONLY, 0, capacity=3)
        s.set_wavefield_dump(_abi.DUMP_NONE)
        s.run()                                   # dumps off again
    bare = coupled_mesh(6, 3, 2, 0, niter=4)      # no data_pointwise arrays
    with Solver(bare) as s:
        with pytest.raises(AxgError):
            s.set_wavefield_dump(_abi.DUMP_STRAIN_ONLY, 1, capacity=4)


@pytest.mark.parametrize("pole", [0, 2])
@pytest.mark.parametrize("dtype_", [_abi.DUMP_DISPL_ONLY, _abi.DUMP_STRAIN_ONLY])
def test_dump_kernel_wavefield_layout(gpu_lib, pole, dtype_):
    """With kwf_mask / mapping_ijel_ikwf the snapshots come in the point
    layout of the reference's NetCDF kernel wavefields (kwf_mapping_sol /
    _flu, SOLVER/wavefields_io.f90:743-780): every kwf point holds the value
    its marking element point has in the packed dump (bit for bit: the same
    kernel computes both), here for the inner points 1..3 plus the axis."""
    from axisem_gb300.mesh import kwf_mapping
    m = _mesh(pole)
    strain_it = 4
    cap = m.niter // strain_it
    kmask, kmap, nps, npf = kwf = kwf_mapping(m, 1, 3, 1, 3)
    with Solver(m) as s:
        packed = s.set_wavefield_dump(dtype_, strain_it, capacity=cap).copy() * 0
        packed = s.set_wavefield_dump(dtype_, strain_it, capacity=cap, out=packed)
        s.run()
        ns, nf, _, names = s.dump_layout()
    with Solver(m) as s:
        kw = s.set_wavefield_dump(dtype_, strain_it, capacity=cap, kwf=kwf)
        assert s.dump_layout()[2] == ns * nps + nf * npf
        s.run()
    nes, nef = m.nel_solid, m.nel_fluid
    for k in range(cap):
        for q in range(ns + nf):
            fluid = q >= ns
            nel = nef if fluid else nes
            off = (ns * nes + (q - ns) * nef) * 25 if fluid else q * nes * 25
            field = packed[k, off: off + nel * 25].reshape(nel, 25)      # [e, i + 5 j]
            koff = ns * nps + (q - ns) * npf if fluid else q * nps
            npt = npf if fluid else nps
            got = kw[k, koff: koff + npt]
            want = np.zeros(npt, np.float32)
            e0 = nes if fluid else 0
            for e in range(nel):
                for j in range(5):
                    for i in range(5):
                        if kmask[i, j, e0 + e]:
                            want[kmap[i, j, e0 + e] - 1 - (nps if fluid else 0)] = field[e, i + 5 * j]
            assert np.array_equal(got, want), (k, names[q])
