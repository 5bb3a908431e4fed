"""Continuous-batching request server for particle simulations.

Requests (a Chimera or vortex system with its own N, box, parameters, initial
state and step count) arrive over time.  The server keeps every admitted
system's state resident in device memory inside one batch (spc_batch_*),
admits waiting requests whenever the batch has room for them (pool particles,
cells and system slots, i.e. device-memory footprint), advances all admitted
systems together in chunks of steps, and hands back each result as soon as
its own step budget is spent.  Requests that arrive while others are running
join the next chunk: their work overlaps with the running ones on the device.

A system's result does not depend on what else is in the batch (its noise is
keyed by seed, system id, step and particle; its neighbour sums see only its
own particles), so a served result equals the same request run alone.

Host work overlaps the device: a chunk is enqueued on the batch's stream and,
while it runs, the server draws the initial states of the requests that have
arrived (the costly host step for large N), so that their admission after the
chunk is only the upload.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable, Optional

import numpy as np

from . import abi


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float           # seconds after the trace start
    model: int               # abi.MODEL_*
    n: int
    L: float
    v0: float
    sigma: float
    rho: float
    alpha: float
    D_phi: float
    steps: int
    seed: int
    # filled by the server
    admitted_at: Optional[float] = None
    finished_at: Optional[float] = None
    result: Optional[np.ndarray] = None
    prepared: Optional[tuple] = None  # inputs() drawn ahead of admission

    def params(self, stepper: int, precision: int) -> abi.Params:
        return abi.make_params(L=self.L, v0=self.v0, sigma=self.sigma, rho=self.rho,
                               alpha=self.alpha, D_phi=self.D_phi, model=self.model,
                               stepper=stepper, precision=precision, seed=self.seed,
                               system_id=self.rid)

    def inputs(self):
        """Initial state (x, y ~ U[0, L), phi ~ U[-pi, pi)) and, for vortex
        requests, omega ~ N(0, 0.5^2): a pure function of (seed, rid)."""
        rng = np.random.default_rng([self.seed, self.rid])
        st = np.empty(3 * self.n)
        st[0::3] = rng.uniform(0.0, self.L, self.n)
        st[1::3] = rng.uniform(0.0, self.L, self.n)
        st[2::3] = rng.uniform(-math.pi, math.pi, self.n)
        om = rng.normal(0.0, 0.5, self.n) if self.model == abi.MODEL_VORTEX else None
        return st, om

    @property
    def cells(self) -> int:
        return abi.cells_of(self.L, self.rho)

    @property
    def work(self) -> int:
        return self.n * self.steps


def make_trace(rate: float = 200.0, duration: float = 60.0, seed: int = 3,
               n_range=(512, 262144), steps_range=(500, 5000), density: float = 1000.0,
               vortex_fraction: float = 0.5) -> list[Request]:
    """Poisson arrivals at `rate` per second over `duration` seconds.  Each
    request: Chimera or vortex (vortex with probability vortex_fraction), N
    log-uniform in n_range, L = sqrt(N / density), alpha ~ U[1.2, 1.6],
    sigma ~ U[0.5, 2], D ~ U[0, 0.02], rho ~ U[0.05, 0.15], v0 = 0.01, steps
    uniform in steps_range; vortex requests have alpha = 0."""
    rng = np.random.default_rng(seed)
    t, out, rid = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        vortex = rng.random() < vortex_fraction
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        L = math.sqrt(n / density)
        alpha = float(rng.uniform(1.2, 1.6))
        out.append(Request(
            rid=rid, arrival=t, model=abi.MODEL_VORTEX if vortex else abi.MODEL_CHIMERA, n=n,
            L=L, v0=0.01, sigma=float(rng.uniform(0.5, 2.0)), rho=float(rng.uniform(0.05, 0.15)),
            alpha=0.0 if vortex else alpha, D_phi=float(rng.uniform(0.0, 0.02)),
            steps=int(rng.integers(steps_range[0], steps_range[1] + 1)), seed=seed))
        rid += 1
    return out


@dataclasses.dataclass
class ServeStats:
    completed: int
    wall_s: float
    particle_steps: int
    throughput: float            # particle-steps/s over the whole run
    p50_s: Optional[float]
    p99_s: Optional[float]
    mean_s: Optional[float]
    max_active: int
    offered: float               # particle-steps/s the trace asks for
    saturated: bool

    def as_dict(self):
        return dataclasses.asdict(self)


class Server:
    """Continuous batching over one spc_batch.

    backend: an object with the Batch interface (abi.Batch on a GPU; tests
    pass a stand-in to check the scheduling on the CPU).  keep_results: True
    keeps every result on its request, a set of request ids keeps those."""

    def __init__(self, backend, stepper: int, precision: int, dt: float = 0.01,
                 chunk: int = 50, backfill: int = 64,
                 clock: Callable[[], float] = time.perf_counter, keep_results: bool = False,
                 limits: Optional[tuple[int, int]] = None, prefetch_particles: int = 1 << 21):
        self.b = backend
        # initial states drawn ahead, while a chunk runs: at most this many
        # particles' worth (host memory bound), in arrival order
        self.prefetch_particles = int(prefetch_particles)
        self.limits = limits  # (max_particles, max_cells): larger requests are refused
        self.stepper, self.precision = stepper, precision
        self.dt, self.chunk, self.backfill = dt, int(chunk), int(backfill)
        self.clock = clock
        self.keep_results = keep_results

    @staticmethod
    def capacities(hbm_bytes: int, stepper: int, precision: int, max_systems: int = 1024,
                   cell_share: float = 0.02):
        """(max_particles, max_cells) of a batch that fits hbm_bytes."""
        bp, bc = abi.footprint(stepper, precision)
        cells_bytes = int(hbm_bytes * cell_share)
        return int((hbm_bytes - cells_bytes) // bp), int(cells_bytes // bc), max_systems

    def _may_fit(self, req: Request) -> bool:
        """A necessary condition for admitting `req` now, from the batch's
        totals: a free system slot and room for its particles (the pool also
        needs a contiguous range, and the cells are checked by the batch).
        Checked before the request's initial state is generated, so that a
        blocked queue does not draw the states of requests that cannot fit."""
        cap = getattr(self.b, "capacity", None)
        if cap is None:
            return True
        u = self.b.usage()
        return u["systems"] < cap["systems"] and u["particles"] + req.n <= cap["particles"]

    def _prefetch(self, waiting) -> int:
        """Draw the initial states of waiting requests (arrival order) up to
        the prefetch budget; returns how many were drawn."""
        held = sum(r.n for r in waiting if r.prepared is not None)
        drawn = 0
        for req in waiting:
            if req.prepared is not None:
                continue
            if held + req.n > self.prefetch_particles:
                break
            req.prepared = req.inputs()
            held += req.n
            drawn += 1
        return drawn

    def run(self, trace: list[Request], time_scale: float = 1.0) -> ServeStats:
        pending = collections.deque(sorted(trace, key=lambda r: r.arrival))
        waiting: collections.deque[Request] = collections.deque()
        active: dict[int, Request] = {}
        done: list[Request] = []
        t0 = self.clock()
        now = lambda: (self.clock() - t0) / time_scale  # noqa: E731
        max_active = 0
        self.refused: list[Request] = []
        self.prefetched = 0
        while pending or waiting or active:
            t = now()
            while pending and pending[0].arrival <= t:
                req = pending.popleft()
                if self.limits and (req.n > self.limits[0] or req.cells > self.limits[1]):
                    self.refused.append(req)  # could never fit, even in an empty batch
                else:
                    waiting.append(req)
            # admission: FIFO with a bounded backfill window behind a blocked head
            skipped = 0
            for req in list(waiting):
                if skipped > self.backfill:
                    break
                if active and not self._may_fit(req):
                    skipped += 1  # its initial state is not generated until it may fit
                    continue
                st, om = req.prepared if req.prepared is not None else req.inputs()
                req.prepared = None
                try:
                    slot = self.b.admit(req.n, req.params(self.stepper, self.precision), st, om,
                                        steps=req.steps)
                except abi.SpcError as e:
                    if e.code != -7:  # capacity: try later; anything else is a real error
                        raise
                    skipped += 1
                    continue
                req.admitted_at = now()
                active[slot] = req
                waiting.remove(req)
            max_active = max(max_active, len(active))
            if not active:
                if pending:
                    wait = pending[0].arrival - now()
                    if wait > 0:
                        time.sleep(min(wait * time_scale, 0.05))
                continue
            self.b.step(self.dt, self.chunk)  # enqueued; runs while the host works
            t = now()
            while pending and pending[0].arrival <= t:
                req = pending.popleft()
                if self.limits and (req.n > self.limits[0] or req.cells > self.limits[1]):
                    self.refused.append(req)
                else:
                    waiting.append(req)
            self.prefetched += self._prefetch(waiting)
            self.b.synchronize()
            for slot in list(active):
                _, remaining = self.b.status(slot)
                if remaining <= 0:
                    req = active.pop(slot)
                    res = self.b.download(slot)
                    if self.keep_results is True or (self.keep_results and req.rid in self.keep_results):
                        req.result = res
                    self.b.release(slot)
                    req.finished_at = now()
                    done.append(req)
        wall = now()
        lat = np.array([r.finished_at - r.arrival for r in done]) if done else np.array([])
        work = sum(r.work for r in done)
        span = max((r.arrival for r in trace), default=0.0)
        offered = sum(r.work for r in trace) / span if span > 0 else 0.0
        return ServeStats(
            completed=len(done), wall_s=wall, particle_steps=work,
            throughput=work / wall if wall > 0 else 0.0,
            p50_s=float(np.percentile(lat, 50)) if lat.size else None,
            p99_s=float(np.percentile(lat, 99)) if lat.size else None,
            mean_s=float(lat.mean()) if lat.size else None, max_active=max_active,
            offered=offered, saturated=bool(wall > 1.5 * max(span, 1e-9)))
