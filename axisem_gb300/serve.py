"""Continuous-batching serving of time-loop solves on one GB300.

No counterpart in the reference, which runs one solve per MPI job.  A request
is one solve: a dominant period (which, with the source type, selects the
mesh), a source type (monopole / dipole / quadrupole), a source depth, a
receiver count and a seismogram duration.  The server

  * keeps one resident mesh per (period, source type) in HBM: a small holder
    solve creates it (axg_create) the first time it is needed, every request
    on it shares it (axg_create_sharing) and owns only its wavefields,
    source, receivers and stream;
  * admits waiting requests in arrival order while their device bytes fit
    the budget (a mesh not yet resident counts with its own bytes);
  * advances every admitted solve in chunks of steps queued on its own
    stream (axg_run_async), so that the solves' kernels overlap on the GPU,
    and polls them (axg_poll); a finished solve returns its seismograms and
    frees its memory, which admits the next request;
  * or, batched, advances all admitted solves together (axg_batch_*): one
    launch per colour and kernel class covers every solve's patches, and a
    step is one CUDA graph replay.  Between chunks finished solves retire and
    waiting ones join (continuous batching at chunk granularity); new solves
    are created while the current chunk runs.

Solves run in the compensated (Kahan) FP32 mode by default, the precision of
the serving workload.  With tens of solves' streams in flight, a process that
serves should let the CUDA runtime use more hardware work queues than its
default 8 (CUDA_DEVICE_MAX_CONNECTIONS=32 in the environment before CUDA
initialises; the benchmark does so).

The meshes are the whole-Earth prem_iso meshes of axisem_gb300.sphere at the
request's period (50 s: 6.6k elements, 25 s: 22k, 10 s: 117k), each with its
CFL time step; a request puts its own source depth, receivers and run length
on the cached mesh (sphere.with_solve).  Seismograms are sampled every
period / 8 seconds.  `duration_scale` shortens every run by the same factor
(the default benchmark serves 1/10 of the requested seismogram lengths so
that a rate sweep fits in minutes); the steps keep the physical time step.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi, sphere
from .mesh import Mesh
from .solver import Batch, Solver, plan_shape

PERIODS = (50, 25, 10)
POLES = (_abi.MONOPOLE, _abi.DIPOLE, _abi.QUADPOLE)
SOURCE_OF_POLE = {_abi.MONOPOLE: "explosion", _abi.DIPOLE: "mtr", _abi.QUADPOLE: "mtp"}


@dataclass
class Request:
    rid: int
    t_arrive: float      # s after the start of the stream
    period: int          # 50, 25 or 10 s
    pole: int            # 0 mono, 1 di, 2 quad
    depth_km: float      # source depth, 0..700 km
    n_rec: int           # receivers on the surface
    duration_s: float    # seismogram length requested
    duration_scale: float = 1.0

    @property
    def key(self):
        return (self.period, self.pole)

    @property
    def seconds(self) -> float:
        return self.duration_s * self.duration_scale

    @property
    def niter(self) -> int:
        return int(np.ceil((self.seconds + 1e-11) / template(self.period, self.pole).deltat))


def request_stream(n: int, rate_per_s: float, seed: int = 2026, duration_scale: float = 1.0) -> list[Request]:
    """Seeded Poisson arrivals; period uniform in {50, 25, 10} s, source type
    uniform, depth uniform in [0, 700] km, receivers uniform in [20, 500],
    duration uniform in [1800, 3600] s (times duration_scale).  A rate of
    0 or less makes every request arrive at once (a saturating stream)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s if rate_per_s > 0 else 1.0, size=n)
    t = np.cumsum(gaps) if rate_per_s > 0 else np.zeros(n)
    return [Request(k, float(t[k]), int(rng.choice([50, 25, 10])), int(rng.integers(0, 3)),
                    float(rng.uniform(0, 700)), int(rng.integers(20, 501)), float(rng.uniform(1800, 3600)),
                    duration_scale)
            for k in range(n)]


_SKELETONS: dict = {}   # period -> skeleton
_TEMPLATES: dict = {}   # (period, pole) -> Mesh: the mesh database a server keeps loaded


def template(period: int, pole: int) -> Mesh:
    """The period's prem_iso mesh for a pole type (built once per process)."""
    if (period, pole) not in _TEMPLATES:
        if period not in _SKELETONS:
            _SKELETONS[period] = sphere.build_skeleton(float(period))
        _TEMPLATES[(period, pole)] = sphere.build_mesh(
            float(period), sphere.SphereSolve(pole=pole, source=SOURCE_OF_POLE[pole], seconds=float(period),
                                              receivers_deg=np.array([90.0])),
            skeleton=_SKELETONS[period], pointwise=False)
    return _TEMPLATES[(period, pole)]


def request_mesh(req: Request, niter: int | None = None) -> Mesh:
    """The solve's mesh descriptor: the period's cached mesh with this
    request's source depth, receivers (uniform in colatitude), run length
    and sampling (period / 8)."""
    t = template(req.period, req.pole)
    seis_it = max(1, int(round(req.period / 8.0 / t.deltat)))
    seconds = req.seconds if niter is None else niter * t.deltat
    solve = sphere.SphereSolve(pole=req.pole, source=SOURCE_OF_POLE[req.pole], depth_km=req.depth_km,
                               seconds=seconds, receivers_deg=np.linspace(0.0, 180.0, req.n_rec),
                               seis_it=seis_it)
    return sphere.with_solve(t, solve, _SKELETONS[req.period])


@dataclass
class Job:
    req: Request
    solver: Solver
    bytes: int
    next_iter: int = 1
    t_admit: float = 0.0


@dataclass
class Result:
    rid: int
    latency_s: float
    seismograms: np.ndarray


@dataclass
class ServeStats:
    wall_s: float
    results: dict = field(default_factory=dict)
    peak_bytes: int = 0
    max_concurrent: int = 0

    def summary(self) -> dict:
        lat = np.array([r.latency_s for r in self.results.values()])
        return {"solves": len(lat), "wall_s": self.wall_s,
                "solves_per_hour": len(lat) / self.wall_s * 3600.0,
                "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "peak_device_gb": self.peak_bytes / 1e9, "max_concurrent": self.max_concurrent}


def _solve_bytes(s: Solver) -> tuple[int, int]:
    inf = s.info()
    return inf["device_bytes"] - inf["mesh_bytes"], inf["mesh_bytes"]


class Server:
    """The serving loop; `budget_bytes` bounds the HBM the solves and
    resident meshes may hold."""

    def __init__(self, budget_bytes: float = 64e9, chunk: int = 1024, lib=None, compensated: bool = True,
                 tuning: str = "shared"):
        """chunk: steps queued per call for a solve (0: all of them at once).
        A whole long solve is tens of thousands of kernel launches: queueing
        it fills the launch queue, and the call blocks the host loop until
        most of it has run, so the solves behind it start late.  In chunks
        every admitted solve is queued at once and refilled as it drains;
        in the batched loop, the most steps a batch runs before solves may
        join it (0: until its first solve finishes).  tuning: the patch
        shape of the resident meshes, "shared" (planned for launches the mesh
        fills, as concurrent solves fill the GPU together) or "alone" (as
        axg_create tunes for one solve on the device: smaller patches on the
        small meshes, faster alone, slower shared)."""
        if tuning not in ("shared", "alone"):
            raise ValueError("tuning is 'shared' or 'alone'")
        self.tuning = tuning
        self.lib = lib or _abi.load_library()
        self.budget = budget_bytes
        self.chunk = chunk
        self.compensated = compensated
        self.meshes: dict = {}      # key -> holder Solver (keeps the mesh resident)
        self.mesh_bytes: dict = {}
        self.used = 0

    def close(self):
        for s in self.meshes.values():
            s.close()
        self.meshes.clear()

    def _solver(self, req: Request, share: bool) -> Solver:
        s = Solver(request_mesh(req), lib=self.lib, share_with=self._holder(req) if share else None)
        s.set_compensated(self.compensated)
        return s

    def _holder(self, req: Request) -> Solver:
        if req.key not in self.meshes:
            m = request_mesh(req, niter=1)
            pe, gr = plan_shape(m, 0, self.lib) if self.tuning == "shared" else (0, -1)
            s = Solver(m, lib=self.lib, patch_elems=pe, growth=gr)
            own, mesh = _solve_bytes(s)
            self.meshes[req.key] = s
            self.mesh_bytes[req.key] = own + mesh
            self.used += own + mesh
        return self.meshes[req.key]

    def _estimate(self, req: Request) -> int:
        t = template(req.period, req.pole)
        nglob = t.nglob_solid + t.nglob_fluid
        need = nglob * 4 * 4 * 3 + 4 * req.niter * 3 * req.n_rec + (1 << 20)   # wavefields, seismograms
        if req.key not in self.meshes:
            need += 4 * need   # a mesh is a few times its wavefields
        return need

    def preload(self, keys):
        """Make the meshes of `keys` ((period, pole) pairs) resident."""
        for period, pole in keys:
            self._holder(Request(-1, 0.0, period, pole, 0.0, 1, 1800.0))

    def _launch(self, job: Job):
        left = job.req.niter - job.next_iter + 1
        n = left if self.chunk <= 0 else min(self.chunk, left)
        job.solver.run_async(job.next_iter, n)
        job.next_iter += n

    def run(self, requests: list[Request], sequential: bool = False, resident: bool = False,
            batched: bool = False) -> ServeStats:
        """Serves `requests` (arrival times relative to the call).  sequential:
        one solve at a time, each on its own freshly built mesh -- the plain
        path run request after request, the baseline -- or, with `resident`,
        on the server's resident meshes (the gain of overlapping alone).
        batched: the admitted solves advance together in batches."""
        if batched:
            return self._run_batched(requests)
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrive))
        waiting: collections.deque = collections.deque()
        active: list[Job] = []
        stats = ServeStats(wall_s=0.0)
        t0 = time.perf_counter()
        while pending or waiting or active:
            now = time.perf_counter() - t0
            while pending and pending[0].t_arrive <= now:
                waiting.append(pending.popleft())
            # admission
            while waiting and (not sequential or not active):
                req = waiting[0]
                if active and self.used + self._estimate(req) > self.budget:
                    break
                waiting.popleft()
                fresh = sequential and not resident
                s = self._solver(req, share=not fresh)
                own, mesh = _solve_bytes(s)
                nbytes = own + (mesh if fresh else 0)
                self.used += nbytes
                job = Job(req, s, nbytes, t_admit=time.perf_counter() - t0)
                self._launch(job)
                active.append(job)
            stats.peak_bytes = max(stats.peak_bytes, self.used)
            stats.max_concurrent = max(stats.max_concurrent, len(active))
            # progress
            progressed = False
            for job in list(active):
                if not job.solver.poll():
                    continue
                progressed = True
                if job.next_iter <= job.req.niter:
                    self._launch(job)
                    continue
                rec = job.solver.receivers().copy()
                done = time.perf_counter() - t0
                stats.results[job.req.rid] = Result(job.req.rid, done - job.req.t_arrive, rec)
                job.solver.close()
                self.used -= job.bytes
                active.remove(job)
            if not progressed:
                if not active and pending and not waiting:
                    time.sleep(max(0.0, min(0.01, pending[0].t_arrive - (time.perf_counter() - t0))))
                else:
                    time.sleep(20e-6)
        stats.wall_s = time.perf_counter() - t0
        return stats

    def _run_batched(self, requests: list[Request]) -> ServeStats:
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrive))
        waiting: collections.deque = collections.deque()
        active: list[Job] = []
        stats = ServeStats(wall_s=0.0)
        batch, members, n_steps = None, [], 0
        t0 = time.perf_counter()
        while pending or waiting or active:
            now = time.perf_counter() - t0
            while pending and pending[0].t_arrive <= now:
                waiting.append(pending.popleft())
            # admission, also while a batch runs: the new solves join the next one
            while waiting:
                req = waiting[0]
                if active and self.used + self._estimate(req) > self.budget:
                    break
                waiting.popleft()
                s = self._solver(req, share=True)
                own, _ = _solve_bytes(s)
                self.used += own
                active.append(Job(req, s, own, t_admit=time.perf_counter() - t0))
            stats.peak_bytes = max(stats.peak_bytes, self.used)
            if batch is not None:
                if not batch.poll():
                    time.sleep(20e-6)
                    continue
                done = time.perf_counter() - t0
                for job in members:
                    job.next_iter += n_steps
                finished = [j for j in members if j.next_iter > j.req.niter]
                if finished:
                    batch.close()
                    batch = None
                for job in finished:
                    stats.results[job.req.rid] = Result(job.req.rid, done - job.req.t_arrive,
                                                        job.solver.receivers().copy())
                    job.solver.close()
                    self.used -= job.bytes
                    active.remove(job)
            if not active:
                if pending and not waiting:
                    time.sleep(max(0.0, min(0.01, pending[0].t_arrive - (time.perf_counter() - t0))))
                continue
            # the next chunk: the same batch while no solve joined or left
            if batch is None or [j.req.rid for j in members] != [j.req.rid for j in active]:
                if batch is not None:
                    batch.close()
                members = list(active)
                batch = Batch([j.solver for j in members])
            stats.max_concurrent = max(stats.max_concurrent, len(members))
            n_steps = min(j.req.niter - j.next_iter + 1 for j in members)
            if self.chunk > 0:
                n_steps = min(n_steps, self.chunk)
            batch.run_async([j.next_iter for j in members], n_steps)
        if batch is not None:
            batch.close()
        stats.wall_s = time.perf_counter() - t0
        return stats


def solve_alone(req: Request, lib=None, compensated: bool = True, tuning: str = "shared") -> np.ndarray:
    """The request's seismograms from a solve on its own, built from scratch
    with the patch shape a Server of that `tuning` gives its mesh (the same
    shape sums every point's contributions in the same order)."""
    m = request_mesh(req)
    pe, gr = plan_shape(m, 0, lib) if tuning == "shared" else (0, -1)
    with Solver(m, lib=lib, patch_elems=pe, growth=gr) as s:
        s.set_compensated(compensated)
        s.run()
        return s.receivers().copy()
