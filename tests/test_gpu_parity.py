"""GPU parity: the CUDA path through the C-ABI against the CPU oracle.

Tolerances (seismograms are required within relative L2 1e-4 of the FP32
reference): the GPU sums element contributions in patch/colour order and uses
fused multiply-adds, so it differs from the oracle at the FP32 rounding level.
  * stiffness + assembly: relative L2 <= 1e-5 against the FP64 oracle
    (and against the FP32 oracle);
  * seismograms and wavefields of short Newmark runs: relative L2 <= 1e-4
    against the FP32 oracle, and the FP64-oracle error is reported;
  * integer work (numbering, colouring, receiver/source indices): exact.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import coupled_mesh, random_gvec, structured_mesh
from axisem_gb300.solver import AxgError, Solver

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("axial", ["random1pct", "column", "none"])
def test_stiffness_assembled_parity(gpu_lib, orc, pole, axial):
    m = structured_mesh(23, 17, pole, seed=100 + pole, axial=axial)
    u = random_gvec(m, seed=7)
    with Solver(m) as s:
        f = s.stiffness_assembled(u)
        f2 = s.stiffness_assembled(u)
    ref64 = orc.stiffness_assembled(m, u, np.float64)
    ref32 = orc.stiffness_assembled(m, u, np.float32)
    assert rel(f, ref64) < 1e-5
    assert rel(f, ref32) < 1e-5
    assert np.array_equal(f, f2), "assembly must be bit-reproducible"
    if pole == 0:
        assert not f[:, 1].any()


@pytest.mark.parametrize("pole", [0, 2])
def test_gvec_io_pinned_and_pageable(gpu_lib, orc, pole):
    """The gvec I/O is in the reference's numbering (the device arrays are
    in the plan's): pinned and pageable host buffers, and uploads and
    downloads mixed with device-side stiffness calls, give one result."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    m = structured_mesh(37, 29, pole, seed=300 + pole)
    u = random_gvec(m, seed=9)
    ng = m.nglob_solid
    hu = torch.empty((3, ng), dtype=torch.float32, pin_memory=True).numpy()
    hf = torch.full((3, ng), np.nan, dtype=torch.float32, pin_memory=True).numpy()
    hu[:] = u.T
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    with Solver(m) as s:
        f_pageable = s.stiffness_assembled(u)
        assert s.lib.axg_stiffness_assembled(s.h, fp(hu), fp(hf)) == 0
        f_pinned = hf.T.copy()
        s.upload_disp(u)                        # staged upload, pinned download
        s.stiffness_device()
        assert s.lib.axg_download_gvec_force(s.h, fp(hf)) == 0
        f_mixed = hf.T.copy()
        assert s.lib.axg_upload_gvec_disp(s.h, fp(hu)) == 0   # pinned upload, staged download
        s.stiffness_device()
        f_mixed2 = s.download_force()
    assert np.array_equal(f_pinned, f_pageable)
    assert np.array_equal(f_mixed, f_pageable) and np.array_equal(f_mixed2, f_pageable)
    assert rel(f_pageable, orc.stiffness_assembled(m, u, np.float64)) < 1e-5


def test_stiffness_golden_fixture(gpu_lib, orc):
    from pathlib import Path
    gold = np.load(Path(__file__).resolve().parent / "golden" / "oracle_golden.npz")
    for pole in (0, 1, 2):
        m = structured_mesh(5, 4, pole, seed=11 + pole)
        m.ax_el_solid = np.array([1, 6, 13], dtype=np.int32)
        u = random_gvec(m, seed=21 + pole)
        with Solver(m) as s:
            f = s.stiffness_assembled(u)
        assert rel(f, gold[f"force_p{pole}"]) < 1e-5


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("variant", ["plain", "fluid_src", "free_surface", "absorbing", "no_axis"])
def test_time_loop_parity(gpu_lib, orc, pole, variant):
    kw = dict(niter=50)
    if variant == "fluid_src":
        kw["fluid_src"] = True
    if variant == "free_surface":
        kw["free_surface"] = True
    if variant == "absorbing":
        kw["absorbing"] = True
    if variant == "no_axis":
        kw["axial_column"] = False
    m = coupled_mesh(10, 5, 4, pole, **kw)
    with Solver(m) as s:
        s.run(1, m.niter)
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        chi = s.get_state(_abi.FIELD_CHI)
    t32 = orc.TimeLoop(m, np.float32)
    t64 = orc.TimeLoop(m, np.float64)
    assert t32.run(1, m.niter) == 0 and t64.run(1, m.niter) == 0
    assert np.abs(t64.receivers()).max() > 0
    assert rel(rec, t32.receivers()) < 1e-4
    assert rel(rec, t64.receivers()) < 1e-4
    comps = [0, 2] if pole == 0 else [0, 1, 2]
    assert rel(disp[..., comps], t64.disp[..., comps]) < 1e-4
    assert rel(chi, t64.chi) < 1e-4


def test_run_in_pieces_equals_one_run(gpu_lib):
    """Pieces of odd and even lengths: the plain Newmark step's displacement
    and prediction buffers trade roles every step, so the pieces start at
    either parity and replay the step graphs of both; seismograms and every
    state field (axis points included) as one run."""
    fields = (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_ACC0, _abi.FIELD_CHI, _abi.FIELD_DCHI,
              _abi.FIELD_DDCHI0)
    m = coupled_mesh(10, 5, 4, 1, niter=60)
    with Solver(m) as s:
        s.set_tuning(steps_per_graph=8)
        s.run(1, 60)
        a = s.receivers()
        sa = [s.get_state(f) for f in fields]
        s.reset()
        s.run(1, 13)
        s.run(14, 30)
        s.run(44, 1)
        s.run(45, 16)
        b = s.receivers()
        sb = [s.get_state(f) for f in fields]
    assert np.array_equal(a, b)
    for x, y in zip(sa, sb):
        assert np.array_equal(x, y)


def test_state_round_trip_and_restart(gpu_lib, orc):
    """Continue a run from a state set through the ABI: the same as the oracle
    continuing from the same element-local state."""
    m = coupled_mesh(9, 4, 3, 2, niter=40)
    t = orc.TimeLoop(m, np.float32)
    assert t.run(1, 20) == 0
    with Solver(m) as s:
        for fld, arr in ((_abi.FIELD_DISP, t.disp), (_abi.FIELD_VELO, t.velo), (_abi.FIELD_ACC0, t.acc0),
                         (_abi.FIELD_CHI, t.chi), (_abi.FIELD_DCHI, t.dchi), (_abi.FIELD_DDCHI0, t.ddchi0)):
            s.set_state(fld, arr)
            back = s.get_state(fld)
            assert np.array_equal(back, arr.astype(np.float32))
        s.run(21, 20)
        d = s.get_state(_abi.FIELD_DISP)
    assert t.run(21, 20) == 0
    assert rel(d, t.disp) < 1e-4


def test_blowup_detected(gpu_lib):
    m = coupled_mesh(8, 4, 0, 0, niter=40)
    m.magnitude = 1e-20
    with Solver(m) as s:
        with pytest.raises(AxgError) as ei:
            s.run()
        assert ei.value.code == _abi.AXG_ERR_BLOWUP


def test_colouring_is_conflict_free(gpu_lib):
    m = structured_mesh(40, 30, 2)
    with Solver(m) as s:
        pe, cp = s.solid_colouring()
        info = s.info()
    assert info["n_colours_solid"] == cp.max() + 1
    colour_of_elem = cp[pe]
    # no global point is touched by two different patches of one colour
    ig = (m.igloc_solid - 1).reshape(m.nel_solid, 25)
    owner = {}
    for e in range(m.nel_solid):
        for g in set(ig[e].tolist()):
            key = (g, int(colour_of_elem[e]))
            assert owner.setdefault(key, int(pe[e])) == int(pe[e])


def test_full_size_properties(gpu_lib):
    """1024 x 1024 quadrupole mesh: linearity of K and bit-reproducibility."""
    m = structured_mesh(1024, 1024, 2, terms="pole")
    u = random_gvec(m, seed=1)
    v = random_gvec(m, seed=2)
    with Solver(m) as s:
        fu = s.stiffness_assembled(u)
        fv = s.stiffness_assembled(v)
        fw = s.stiffness_assembled((2.0 * u - 0.5 * v).astype(np.float32))
        fu2 = s.stiffness_assembled(u)
    assert np.array_equal(fu, fu2)
    lin = 2.0 * fu.astype(np.float64) - 0.5 * fv
    assert rel(fw, lin) < 1e-5
