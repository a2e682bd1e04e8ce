"""Benchmark of the stiffness + assembly step on one GB300.

Workload (the synthetic stiffness/assembly micro-benchmark): a structured
1024 x 1024 grid of npol = 4 solid elements (2^20 elements, 16 785 409 global
points), 1 % axial elements, seeded bilinear geometry and materials,
3-component FP32 displacement ~ N(0, 1e-6).  One step = one evaluation of the
assembled quadrupole stiffness force
    f = pdistsum_solid(axis_mask(glob_stiffness_quad_4(axis_mask(u))))
over all elements (SOLVER/stiffness_quad.f90:238, SOLVER/commun.F90:69).
The metric is GLL-point-steps/s: 25 * 2^20 element-local GLL points per step.

  value : device-resident inputs, CUDA events on the library's stream;
  e2e   : through the C-ABI call with host (pinned) buffers, the host->device
          copy of u and the device->host copy of f inside every step;
  poles : the same for each pole type, each with its roofline.
  cpu_baseline / --impl reference : the same stiffness + assembly of the same
          mesh on the host cores, the oracle's FP32 timing build on all threads
          (the reference's Fortran cannot be compiled here: no compiler).
The inputs (2.8 GB of metric terms) are far larger than the 129 MB L2, so no
L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun each rank runs an independent replica on its own GPU (the
stiffness/assembly step has no exchange step on one mesh); rank 0 prints the
JSON line with the whole-job throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
# The serving stream keeps tens of solves' streams busy at once: let the
# CUDA runtime map them onto 32 hardware work queues instead of its default
# 8 (read once, when CUDA initialises).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

POLES = {"mono": 0, "di": 1, "quad": 2}
N_TERMS = {0: 15, 1: 24, 2: 26}
N_AXIAL = {0: 3, 1: 9, 2: 6}
N_COMP = {0: 2, 1: 3, 2: 3}
METRIC = "GLL-point-steps/s (stiffness+assembly, 1 GB300)"


def algorithmic_bytes(nel: int, nglob: int, nax: int, pole: int) -> int:
    """Bytes one stiffness+assembly must move at least: every metric array and
    the numbering read once (E (100 n_m + 100)), u read and f written once per
    global point (G 8 n_c), axial vectors (A 20 n_a)."""
    return nel * (100 * N_TERMS[pole] + 100) + nglob * 8 * N_COMP[pole] + nax * 20 * N_AXIAL[pole]


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("AXG_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"   # gloo reduces host tensors
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_build() -> str:
    """The oracle timing build's flags (oracle/Makefile)."""
    import platform
    native = " -mcpu=native" if platform.machine() == "aarch64" else ""
    return f"oracle FP32 restatement, gcc -O3{native} -ffp-contract=fast, OpenMP over coloured elements"


def bench_mesh(pole: int, n: int, rank: int = 0):
    """The micro-benchmark's mesh and displacement (seeded per replica)."""
    from axisem_gb300.mesh import random_gvec, structured_mesh
    m = structured_mesh(n, n, pole, terms="pole", seed=20261203 + rank)
    return m, random_gvec(m, seed=20261204 + rank)


def time_cpu(mesh, u, seconds: float, threads: int, min_steps: int = 1):
    """Stiffness + assembly of the whole mesh on the host cores with the
    oracle's timing build (the FP32 restatement at -O3 for the host CPU,
    coloured elements on `threads` threads); steps for about `seconds`.
    Returns (GLL-point-steps/s, steps)."""
    from oracle import oracle as orc
    cs = orc.CpuStiffness(mesh)
    f = np.zeros_like(u, order="F")
    cs(u, f, threads)   # warm-up
    n, t0 = 0, time.perf_counter()
    while n < min_steps or time.perf_counter() - t0 < seconds:
        cs(u, f, threads)
        n += 1
    dt = time.perf_counter() - t0
    assert np.isfinite(f).all()
    return n * mesh.nel_solid * 25 / dt, n


def run_reference(args):
    """The reference's algorithm on the host cores: the oracle's FP32 timing
    build (the reference cannot be compiled here or on the GPU hosts: no
    Fortran compiler) on the same 1024 x 1024 mesh and pole as the GPU arm,
    all host threads, elements coloured so that threads scatter without
    races.  One step = one stiffness + assembly of the whole mesh."""
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.build()
    pole = POLES[args.pole]
    n = args.size
    threads = os.cpu_count() or 1
    mesh, u = bench_mesh(pole, n)
    cs = orc.CpuStiffness(mesh)
    f = np.zeros_like(u, order="F")
    for _ in range(args.warmup):
        cs(u, f, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cs(u, f, threads)
    dt = time.perf_counter() - t0
    assert np.isfinite(f).all()
    pts = mesh.nel_solid * 25
    value = args.steps * pts / dt
    sample = (f"{args.steps} full steps of the {n}x{n} mesh ({mesh.nel_solid} elements), "
              f"{threads} threads, {cs.ncol} element colours")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GLL-point-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"stiffness+assembly, {args.pole}pole, {n}x{n} structured quads "
                                   f"({mesh.nel_solid} elements, {mesh.nglob_solid} global points, 1% axial)",
                       "pole": args.pole, "elements": mesh.nel_solid, "global_points": mesh.nglob_solid},
            "cpu_baseline": {"value": value, "unit": "GLL-point-steps/s", "cores": threads, "kind": "port",
                             "sample": sample,
                             "build": cpu_build()},
            "e2e": {"value": value, "unit": "GLL-point-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_stiffness(args, pole, ws, rank, local, e2e=True):
    """Stiffness + assembly of one pole type on the benchmark mesh: device
    timing (CUDA events on the library's stream), optionally end to end
    through the C-ABI with pinned host buffers, and the roofline."""
    import torch
    from axisem_gb300.solver import Solver
    n = args.size
    t0 = time.perf_counter()
    mesh, u = bench_mesh(pole, n, rank)
    t_mesh = time.perf_counter() - t0
    t0 = time.perf_counter()
    s = Solver(mesh)
    t_create = time.perf_counter() - t0
    info = s.info()
    s.upload_disp(u)
    for _ in range(max(args.warmup, 3)):
        s.stiffness_device()
    torch.cuda.synchronize()

    with ClockSampler(local) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        ms = s.time_stiffness(args.steps)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        barrier(ws)
    clocks = clk.summary()
    ms = max_over_ranks(ms, ws)
    pts_step = mesh.nel_solid * 25
    ng = mesh.nglob_solid
    out = {"value": ws * pts_step / (ms * 1e-3), "ms_per_step": ms, "clocks": clocks, "wall_s": wall,
           "info": info, "setup_s": {"mesh": round(t_mesh, 2), "create": round(t_create, 2)},
           "mesh": mesh, "u": u}
    if e2e:
        hu = torch.empty((3, ng), dtype=torch.float32, pin_memory=True).numpy()
        hu[:] = u.T
        hf = torch.empty((3, ng), dtype=torch.float32, pin_memory=True).numpy()
        import ctypes as C
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
        for _ in range(2):
            s.lib.axg_stiffness_assembled(s.h, fp(hu), fp(hf))
        barrier(ws)
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        for _ in range(args.steps):
            rc = s.lib.axg_stiffness_assembled(s.h, fp(hu), fp(hf))
            assert rc == 0, s.lib.axg_last_error(s.h)
        torch.cuda.synchronize()
        e_s = max_over_ranks((time.perf_counter() - e0) / args.steps, ws)
        assert np.isfinite(hf).all()
        out["e2e"] = {"value": ws * pts_step / e_s, "unit": "GLL-point-steps/s",
                      "h2d_bytes_per_step": int(ng * 12), "d2h_bytes_per_step": int(ng * 12)}
    s.close()
    nbytes = algorithmic_bytes(mesh.nel_solid, ng, len(mesh.ax_el_solid), pole)
    peak, peak_kind = measured_peaks()
    achieved = nbytes / (ms * 1e-3) / 1e9
    name = {v: k for k, v in POLES.items()}[pole]
    prof = ROOT / "profiles" / f"stiffness_assembly_{name}_{n}x{n}.traffic.json"
    traffic = json.loads(prof.read_text()).get("dram_bytes_per_step") if prof.exists() else None
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                       "algorithmic_bytes_per_step": nbytes,
                       "kernel": f"solid_patch_kernel<{name},force> (all colour launches of one step)"}
    return out


def run_gpu(args):
    ws, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    import axisem_gb300.build as b
    b.build()

    pole = POLES[args.pole]
    n = args.size
    head = measure_stiffness(args, pole, ws, rank, local)
    mesh, u, info = head.pop("mesh"), head.pop("u"), head["info"]
    ng = mesh.nglob_solid

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v_all, k_all = time_cpu(mesh, u, args.cpu_seconds, threads)
        v_one, k_one = time_cpu(mesh, u, args.cpu_seconds / 2, 1)
        cpu = {"value": v_all, "unit": "GLL-point-steps/s", "cores": threads, "kind": "port",
               "sample": f"the benchmark's {n}x{n} mesh: {k_all} stiffness+assembly steps on {threads} threads; "
                         f"{k_one} on one thread",
               "single_core": v_one,
               "build": cpu_build()}
    del mesh, u

    poles = {args.pole: {"value": head["value"], "ms_per_step": head["ms_per_step"], "roofline": head["roofline"],
                         "e2e": head["e2e"]}}
    if not args.no_other_poles:
        for other in (k for k in POLES if k != args.pole):
            r = measure_stiffness(args, POLES[other], ws, rank, local)
            r.pop("mesh"), r.pop("u")
            poles[other] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "roofline": r["roofline"],
                            "e2e": r["e2e"], "clocks": r["clocks"]}

    timeloop = timeloop_anel = timeloop_comp = timeloop_dumps = None
    if args.timeloop_steps > 0:
        timeloop = run_timeloop(args, pole, ws, rank)
        timeloop_anel = run_timeloop(args, pole, ws, rank, anel=True)
        timeloop_comp = run_timeloop(args, pole, ws, rank, compensated=True)
        timeloop_dumps = run_timeloop_dumps(args, pole, ws, rank)

    physical = run_physical(args, ws, rank) if args.physical_steps > 0 else None
    precision = run_precision(ws, rank) if not args.no_precision else None
    serving = run_serving(args) if args.serve_requests > 0 else None

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": head["value"], "unit": "GLL-point-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"stiffness+assembly, {args.pole}pole, {n}x{n} structured quads "
                               f"({n * n} elements, {ng} global points, 1% axial)",
                   "pole": args.pole, "elements": n * n, "global_points": ng,
                   "parallelism": f"replicas x{ws}",
                   "l2": "inputs (metric terms) 20x larger than L2; no flush needed"},
        "e2e": head["e2e"],
        "roofline": head["roofline"],
        "cpu_baseline": cpu,
        "poles": poles,
        "timeloop": timeloop,
        "timeloop_anel": timeloop_anel,
        "timeloop_compensated": timeloop_comp,
        "timeloop_dumps": timeloop_dumps,
        "physical": physical,
        "precision": precision,
        "serving": serving,
        "clocks": head["clocks"],
        "gpu_launches": int(args.steps * info["kernels_per_force"]),
        "plan": {"patches": info["n_patches_solid"], "colours": info["n_colours_solid"],
                 "patch_elems": info["patch_elems_solid"], "growth": ["compact", "layered"][info["growth_solid"]],
                 "ctas_per_sm": info["ctas_per_sm_force"],
                 "patch_points_over_global": info["patch_points_solid"] / ng,
                 "device_gb": info["device_bytes"] / 1e9},
        "setup_s": head["setup_s"],
        "wall_s": head["wall_s"],
    }
    print(json.dumps(line), flush=True)


def timeloop_bytes(m, pole: int) -> int:
    """Algorithmic bytes of one Newmark step: metric terms and numbering read
    once, the solid state disp/velo/acc0 read and written and the inverse mass
    read once per global point and component, the fluid likewise, the
    solid-fluid boundary terms once."""
    nc = N_COMP[pole]
    nfm = 3 if pole == 0 else 4
    b = m.nel_solid * (100 * N_TERMS[pole] + 100) + m.nglob_solid * (24 * nc + 4)
    b += len(m.ax_el_solid) * 20 * N_AXIAL[pole]
    if m.nel_fluid:
        b += m.nel_fluid * (100 * nfm + 100) + m.nglob_fluid * 28
        b += len(m.bdry_solid_el) * 5 * 56 // 5
    return b


def anel_bytes(m, pole: int) -> int:
    """Algorithmic bytes the cg4 attenuation adds to a Newmark step: per solid
    element the memory variables (4 cg points x n_e components x n_sls, n_e = 4
    monopole, 6 otherwise) and the previous step's sources (4 x (1 + n_e))
    read and written, and the 48 constant floats plus 2 Q indices read."""
    ne = 4 if pole == 0 else 6
    nsls = len(m.anel["y_j"])
    return m.nel_solid * (4 * ne * nsls * 8 + 4 * (1 + ne) * 8 + 48 * 4 + 8)


def run_timeloop(args, pole, ws, rank, anel=False, compensated=False):
    """Newmark steps (SOLVER/time_evol_wave.F90:353-500) on a coupled mesh of
    1024 x 768 solid over 1024 x 256 fluid elements, through axg_run; with
    `anel`, cg4 attenuation with 5 standard linear solids in the solid; with
    `compensated`, the Kahan-compensated predictor/corrector."""
    import torch
    from axisem_gb300.mesh import add_attenuation, coupled_mesh
    from axisem_gb300.solver import Solver
    n = args.size
    nsteps = args.timeloop_steps
    m = coupled_mesh(n, 3 * n // 4, n // 4, pole, niter=64 + nsteps, seed=5 + rank, num_rec=200,
                     seis_it=4, deltat=2e-6, terms="pole")
    if anel:
        m = add_attenuation(m, n_sls=5, seed=77 + rank)
    s = Solver(m)
    if compensated:
        s.set_compensated(True)
    spg = s.autotune()   # measured steps per CUDA graph
    warm = max(16, spg)  # the warm-up instantiates the step graph
    s.run(1, warm)
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    s.run(warm + 1, nsteps)
    torch.cuda.synchronize()
    dt = max_over_ranks((time.perf_counter() - t0) / nsteps, ws)
    info = s.info()
    rec = s.receivers()
    s.close()
    pts = 25 * (m.nel_solid + m.nel_fluid)
    nb = timeloop_bytes(m, pole) + (anel_bytes(m, pole) if anel else 0)
    if compensated:  # the compensation of disp/velo (chi/dchi) read and written once per point
        nb += m.nglob_solid * 16 * N_COMP[pole] + m.nglob_fluid * 16
    peak, _ = measured_peaks()
    return {"value": ws * pts / dt, "unit": "GLL-point-steps/s", "ms_per_step": dt * 1e3,
            "mesh": f"{n}x{3 * n // 4} solid + {n}x{n // 4} fluid elements, {args.pole}pole, "
                    f"source + 200 receivers" + (", cg4 attenuation with 5 SLS" if anel else "")
                    + (", compensated (Kahan) time integration" if compensated else ""),
            "algorithmic_bytes_per_step": nb, "achieved_gbs": nb / dt / 1e9,
            "frac_of_hbm": nb / dt / 1e9 / peak, "kernels_per_step": info["kernels_per_step"],
            "solid_ctas_per_sm": info["ctas_per_sm_step"], "steps_per_graph": spg,
            "finite": bool(np.isfinite(rec).all())}


def run_physical(args, ws, rank):
    """Time loops on the whole-Earth prem_iso meshes (axisem_gb300.sphere):
    config 1 -- 50 s, monopole explosion at 100 km, 1800 s, 20 receivers --
    as a whole solve, and config 3 -- 10 s, 5-SLS cg4 attenuation, explosion,
    mrt and mtp at 50 km, 200 receivers -- over `physical_steps` steps of each
    source type, with the whole 3600 s solve's time projected from them."""
    import torch
    from axisem_gb300 import sphere
    from axisem_gb300.solver import Solver
    out = {}
    sk50 = sphere.build_skeleton(50.0)
    m = sphere.build_mesh(50.0, sphere.SphereSolve(pole=0, seconds=1800.0), skeleton=sk50)
    with Solver(m) as s:
        s.autotune()
        s.reset()
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        s.run()
        torch.cuda.synchronize()
        dt = max_over_ranks(time.perf_counter() - t0, ws)
        rec = s.receivers()
    pts = 25 * (m.nel_solid + m.nel_fluid)
    out["config1_prem50s_explosion_1800s"] = {
        "elements": m.nel_solid + m.nel_fluid, "steps": m.niter, "deltat_s": m.deltat, "solve_s": dt,
        "value": ws * pts * m.niter / dt, "unit": "GLL-point-steps/s", "ms_per_step": dt / m.niter * 1e3,
        "finite": bool(np.isfinite(rec).all())}
    sk10 = sphere.build_skeleton(10.0)
    for pole, src in ((0, "explosion"), (1, "mtr"), (2, "mtp")):
        m = sphere.build_mesh(10.0, sphere.SphereSolve(pole=pole, source=src, depth_km=50.0, seconds=3600.0,
                                                       receivers_deg=np.linspace(0.0, 180.0, 200)),
                              skeleton=sk10, attenuation=sphere.Attenuation(), pointwise=False)
        n = min(args.physical_steps, m.niter)
        with Solver(m) as s:
            spg = s.autotune()
            s.reset()
            s.run(1, min(64, m.niter))
            torch.cuda.synchronize()
            barrier(ws)
            t0 = time.perf_counter()
            s.run(65, n)
            torch.cuda.synchronize()
            dt = max_over_ranks((time.perf_counter() - t0) / n, ws)
            rec = s.receivers()
        pts = 25 * (m.nel_solid + m.nel_fluid)
        out[f"config3_prem10s_anelastic_{src}"] = {
            "elements": m.nel_solid + m.nel_fluid, "steps_timed": n, "steps_solve": m.niter,
            "deltat_s": m.deltat, "ms_per_step": dt * 1e3, "value": ws * pts / dt, "unit": "GLL-point-steps/s",
            "solve_s_projected": dt * m.niter, "steps_per_graph": spg, "finite": bool(np.isfinite(rec).all())}
    return out


def run_precision(ws, rank):
    """The precision study: 1e5 steps of the anelastic dipole run of
    axisem_gb300.sphere.long_run_mesh (prem_ani 50 s, cg4 attenuation with 5
    SLS, Mrt at 100 km, 10 surface receivers), plain FP32 and compensated,
    each against the FP64 oracle's seismograms of the same mesh
    (tests/golden/precision_long_run.npz): relative L2 per component (s, phi,
    z), with the oracle's own FP32 run beside them."""
    import torch
    from axisem_gb300 import sphere
    from axisem_gb300.solver import Solver
    fx_path = ROOT / "tests" / "golden" / "precision_long_run.npz"
    if not fx_path.exists():
        return {"unavailable": "no FP64 oracle fixture (tests/golden/make_precision_reference.py makes it)"}
    fx = np.load(fx_path)
    ref = np.asarray(fx["rec_float64"], np.float64)

    def per_component(rec):
        rec = np.asarray(rec, np.float64)
        return [float(np.linalg.norm(rec[:, c] - ref[:, c]) / np.linalg.norm(ref[:, c])) for c in range(3)]

    def per_receiver(rec):
        """max and median over receivers of each component's relative L2,
        receivers whose trace of that component is below 1e-3 of the largest
        left out (their misfit is that of a near-zero trace)"""
        rec = np.asarray(rec, np.float64)
        num = np.linalg.norm(rec - ref, axis=0)   # (3, num_rec)
        den = np.linalg.norm(ref, axis=0)
        out = {"max": [], "median": [], "receivers": []}
        for c in range(3):
            keep = den[c] >= 1e-3 * den[c].max()
            r = num[c, keep] / den[c, keep]
            out["max"].append(float(r.max()))
            out["median"].append(float(np.median(r)))
            out["receivers"].append(int(keep.sum()))
        return out

    m = sphere.long_run_mesh(int(fx["niter"]))
    out = {"mesh": f"prem_ani 50 s, {m.nel_solid} solid + {m.nel_fluid} fluid elements, cg4 attenuation (5 SLS), "
                   f"dipole Mrt at 100 km, {m.num_rec} receivers",
           "steps": m.niter, "deltat_s": m.deltat, "components": ["s", "phi", "z"],
           "oracle_fp32": per_component(fx["rec_float32"]),
           "oracle_fp32_per_receiver": per_receiver(fx["rec_float32"])}
    for mode in ("plain", "compensated"):
        with Solver(m) as s:
            s.set_compensated(mode == "compensated")
            torch.cuda.synchronize()
            barrier(ws)
            t0 = time.perf_counter()
            s.run()
            torch.cuda.synchronize()
            dt = max_over_ranks(time.perf_counter() - t0, ws)
            rec = s.receivers()
            out[mode] = per_component(rec)
            out[f"{mode}_per_receiver"] = per_receiver(rec)
            out[f"{mode}_solve_s"] = dt
    return out


def run_timeloop_dumps(args, pole, ws, rank, strain_it=8):
    """The elastic time loop of run_timeloop without and with kernel wavefield
    dumps (axg_set_wavefield_dump: displ_only and strain_only every strain_it
    steps into page-locked host memory): the cost of a snapshot, whose
    device-to-host copy overlaps the following steps."""
    import torch
    from axisem_gb300 import _abi
    from axisem_gb300.mesh import add_pointwise, coupled_mesh
    from axisem_gb300.solver import Solver
    n, nsteps, warm = args.size, args.timeloop_steps, 16
    m = add_pointwise(coupled_mesh(n, 3 * n // 4, n // 4, pole, niter=warm + nsteps, seed=5 + rank, num_rec=200,
                                   seis_it=4, deltat=2e-6, terms="pole"))
    out = {"strain_it": strain_it, "steps": nsteps}
    s = Solver(m)
    s.set_tuning(steps_per_graph=16)

    def timed():
        s.reset()
        s.run(1, warm)
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        s.run(warm + 1, nsteps)
        torch.cuda.synchronize()
        return max_over_ranks((time.perf_counter() - t0) / nsteps, ws)

    base = timed()
    out["plain_ms_per_step"] = base * 1e3
    cap = (warm + nsteps) // strain_it
    for name, t in (("displ_only", _abi.DUMP_DISPL_ONLY), ("strain_only", _abi.DUMP_STRAIN_ONLY)):
        s.set_wavefield_dump(t, strain_it, capacity=1)
        floats = s.dump_layout()[2]
        buf = torch.empty((cap, floats), dtype=torch.float32, pin_memory=True).numpy()
        s.set_wavefield_dump(t, strain_it, capacity=cap, out=buf)
        dt = timed()
        snaps = nsteps // strain_it
        out[name] = {"ms_per_step": dt * 1e3, "snapshot_bytes": floats * 4,
                     "ms_per_snapshot": (dt - base) * nsteps / snaps * 1e3,
                     "snapshot_gbs": floats * 4 * snaps / (dt * nsteps) / 1e9,
                     "finite": bool(np.isfinite(buf).all())}
        s.set_wavefield_dump(_abi.DUMP_NONE)
        del buf
    s.close()
    return out


def run_serving(args):
    """The serving stream of the workload's config 4 (axisem_gb300.serve) on
    the prem_iso meshes of 50, 25 and 10 s, compensated FP32, the meshes
    resident before the streams start.  Requests draw period, pole, depth
    (0-700 km), receivers (20-500) and duration (1800-3600 s, times
    duration_scale; physical time steps).  Capacity: every request at once,
    served concurrently, batched, and one at a time on the resident meshes
    (the baseline); seismograms must be identical in all three.  The server
    plans its meshes for a shared GPU; the baseline is also timed on meshes
    tuned for a lone solve (axg_create's tuning), its fastest form.  Then a
    sweep of Poisson arrival rates with p50/p99 latency per rate."""
    from axisem_gb300.serve import PERIODS, POLES, Server, request_stream, template
    scale = args.serve_duration_scale
    srv = Server(budget_bytes=64e9, chunk=1024)
    try:
        t0 = time.perf_counter()
        srv.preload({(p, q) for p in PERIODS for q in POLES})
        t_preload = time.perf_counter() - t0
        sat = request_stream(args.serve_requests, 0.0, seed=2026, duration_scale=scale)
        served = srv.run(sat)
        batched = srv.run(sat, batched=True)
        seq = srv.run(sat, sequential=True, resident=True)
        same = all(np.array_equal(served.results[r.rid].seismograms, seq.results[r.rid].seismograms) and
                   np.array_equal(batched.results[r.rid].seismograms, seq.results[r.rid].seismograms)
                   for r in sat)
        # the baseline at its best: one solve at a time on meshes tuned for
        # a lone solve (smaller patches on the 50 and 25 s meshes)
        alone = Server(budget_bytes=64e9, chunk=1024, tuning="alone")
        try:
            alone.preload({(p, q) for p in PERIODS for q in POLES})
            seq_alone = alone.run(sat, sequential=True, resident=True)
        finally:
            alone.close()
        sweep = []
        for lam in [float(x) for x in args.serve_rates.split(",") if x]:
            n = int(np.clip(round(12 * lam), 6, args.serve_requests))
            reqs = request_stream(n, lam, seed=2027, duration_scale=scale)
            sweep.append({"rate_per_s": lam, "requests": n, "served": srv.run(reqs).summary(),
                          "served_batched": srv.run(reqs, batched=True).summary()})
    finally:
        srv.close()
    a, b, c, c1 = served.summary(), batched.summary(), seq.summary(), seq_alone.summary()
    steps = [r.niter for r in sat]
    # the mix's work in the headline unit: GLL-point-steps of every solve
    work = sum(25 * (template(r.period, r.pole).nel_solid + template(r.period, r.pole).nel_fluid) * r.niter
               for r in sat)
    for x in (a, b, c, c1):
        x["gll_point_steps_per_s"] = work / x["wall_s"]
    return {"requests": len(sat), "arrival": "all at once (capacity)",
            "mix": "prem_iso meshes of 50/25/10 s (6.6k/22k/117k elements, CFL time steps), pole "
                   "{mono,di,quad}, depth 0-700 km, 20-500 receivers sampled every period/8, "
                   f"1800-3600 s of seismogram times {scale} ({min(steps)}-{max(steps)} steps); "
                   "compensated (Kahan) FP32",
            "duration_scale": scale, "mesh_preload_s": round(t_preload, 1), "gll_point_steps": work,
            "chunk_steps": srv.chunk,
            "mesh_tuning": "resident meshes planned for launches the mesh fills (shared GPU)",
            "served": a, "served_batched": b, "sequential_resident_meshes": c,
            "sequential_meshes_tuned_alone": c1,
            "solves_per_hour_ratio": a["solves_per_hour"] / c["solves_per_hour"],
            "solves_per_hour_ratio_vs_tuned_alone": a["solves_per_hour"] / c1["solves_per_hour"],
            "batched_solves_per_hour_ratio": b["solves_per_hour"] / c["solves_per_hour"],
            "results_identical_to_sequential": bool(same), "sweep": sweep}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--pole", default="quad", choices=list(POLES))
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-other-poles", action="store_true")
    ap.add_argument("--timeloop-steps", type=int, default=64)
    ap.add_argument("--physical-steps", type=int, default=2000)
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-rates", default="0.5,1,2,5,10,20")
    ap.add_argument("--serve-duration-scale", type=float, default=0.1)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
