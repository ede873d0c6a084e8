"""A continuously batched Gauss-Newton mapping server.

Requests (one slice of measured MRF signals each, of any voxel count) arrive
over time. The server admits a request when its measured samples and its
per-voxel state fit in the device-memory budget, appends its voxels to ONE
device-resident pool (:class:`torchsim_gb300.recon.VoxelPool`) shared by every
request in flight, and runs the pool's Levenberg-Marquardt iterations: one
fused normal-equation sweep per iteration over the live voxels of ALL
requests, so a request that arrives while others are on the GPU joins the very
next launch. Finished voxels are retired every iteration; a request completes
the moment its last voxel does, independently of the others. Each voxel's
arithmetic does not depend on which voxels share its launch, so a request's
maps are the same alone and in the mix.

The reference has no server: ``NonlinearLeastSquares.map`` solves one volume
per call (``estimators/_nlls.py:203-301``).
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import torch

from .recon import UNKNOWN, GaussNewton, TrustRegion, VoxelPool, fixed_shape, natural_of, to_free
from .sequence import Program


@dataclass
class MapRequest:
    """One mapping job: measured (V, P) complex64 on the device, B1 (V,)."""

    measured: torch.Tensor
    b1: torch.Tensor | None = None
    arrival: float = 0.0
    id: int = -1
    # Filled in by the server.
    admitted: float | None = None
    completed: float | None = None
    maps: dict[str, torch.Tensor] | None = None
    slot: int = -1
    start_row: int = -1
    remaining: int = 0

    @property
    def voxels(self) -> int:
        return int(self.measured.shape[0])

    @property
    def latency(self) -> float | None:
        return None if self.completed is None else self.completed - self.arrival


class Arena:
    """First-fit ranges of rows of a fixed device buffer."""

    def __init__(self, rows: int) -> None:
        self.rows = rows
        self.free: list[tuple[int, int]] = [(0, rows)]

    def allocate(self, n: int) -> int | None:
        for i, (start, length) in enumerate(self.free):
            if length >= n:
                if length == n:
                    self.free.pop(i)
                else:
                    self.free[i] = (start + n, length - n)
                return start
        return None

    def release(self, start: int, n: int) -> None:
        self.free.append((start, n))
        self.free.sort()
        merged: list[tuple[int, int]] = []
        for s, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == s:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((s, ln))
        self.free = merged


@dataclass
class ServerStats:
    iterations: int = 0
    launches: int = 0
    voxel_iterations: int = 0
    admitted: int = 0
    completed: int = 0
    peak_live_voxels: int = 0
    waits_for_memory: int = 0
    samples_live: list = field(default_factory=list)


class GNServer:
    """Admission by memory budget + one fused GN iteration per step over every
    live voxel of every admitted request."""

    def __init__(self, program: Program, states: int, bounds: dict, start: torch.Tensor,
                 loop: GaussNewton | None = None, *, budget_bytes: int = 120 * 2**30,
                 device: torch.device | None = None, launch=None) -> None:
        self.program = program
        self.states = int(states)
        self.bounds = dict(bounds)
        self.loop = loop if loop is not None else GaussNewton(TrustRegion(), max_iterations=10)
        self.config = self.loop.config(self.bounds)
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        # One launch shape for every iteration, whatever the live voxel count:
        # a voxel's arithmetic then never depends on the batch it is in.
        self.launch = launch if launch is not None else fixed_shape(self.states)
        self.outputs = int(program.outputs)
        bytes_per_voxel = self.outputs * 8 + VoxelPool.BYTES_PER_VOXEL + 8 * 3 + 4
        self.capacity = max(1, int(budget_bytes // bytes_per_voxel))
        self.budget_bytes = int(budget_bytes)
        self.measured = torch.empty((self.capacity, self.outputs), dtype=torch.complex64,
                                    device=self.device)
        self.answer_u = torch.zeros((self.capacity, 3), dtype=torch.float64, device=self.device)
        self.slot_of_row = torch.zeros(self.capacity, dtype=torch.int64, device=self.device)
        self.arena = Arena(self.capacity)
        self.u0 = to_free(torch.as_tensor(start, dtype=torch.float64).reshape(1, 3),
                          self.bounds).to(self.device)
        self.pool = VoxelPool(self.device)
        self.queue: deque[MapRequest] = deque()
        self.active: dict[int, MapRequest] = {}
        self.finished: list[MapRequest] = []
        self.stats = ServerStats()
        self._next_slot = 0
        self._free_slots: list[int] = []

    # -- admission --------------------------------------------------------
    def submit(self, request: MapRequest) -> None:
        if request.voxels > self.capacity:
            raise ValueError(f"a request of {request.voxels} voxels exceeds the budget of "
                             f"{self.capacity} voxels")
        if request.measured.shape[-1] != self.outputs:
            raise ValueError("request samples do not match the sequence")
        self.queue.append(request)

    def _slot(self) -> int:
        if self._free_slots:
            return self._free_slots.pop()
        self._next_slot += 1
        return self._next_slot - 1

    def admit(self, now: float) -> int:
        """Admit queued requests, in order, while they fit; returns how many."""
        n = 0
        while self.queue:
            req = self.queue[0]
            start = self.arena.allocate(req.voxels)
            if start is None:
                self.stats.waits_for_memory += 1
                break
            self.queue.popleft()
            rows = torch.arange(start, start + req.voxels, device=self.device)
            self.measured[start:start + req.voxels].copy_(req.measured, non_blocking=True)
            req.slot = self._slot()
            self.slot_of_row[start:start + req.voxels] = req.slot
            req.start_row, req.remaining, req.admitted = start, req.voxels, now
            self.answer_u[start:start + req.voxels] = self.u0
            self.pool.add(self.u0.expand(req.voxels, 3), req.b1, rows, rows)
            self.active[req.slot] = req
            self.stats.admitted += 1
            n += 1
        return n

    # -- serving ----------------------------------------------------------
    def step(self, clock) -> list[MapRequest]:
        """One iteration over every live voxel; returns requests completed."""
        if self.pool.n == 0:
            return []
        live = self.pool.n
        self.stats.peak_live_voxels = max(self.stats.peak_live_voxels, live)
        self.stats.samples_live.append(live)
        self.pool.iterate(self.program, self.measured, self.states, self.config, self.launch)
        self.stats.iterations += 1
        self.stats.launches += 3
        self.stats.voxel_iterations += live
        # The one host read of the iteration: finished voxels per request slot.
        out = self.pool.retire(self.slot_of_row.index_select(0, self.pool.t["owner"]),
                               self._next_slot)
        counts = out["counts"]
        done: list[MapRequest] = []
        if sum(counts):
            self.answer_u[out["owner"]] = out["u"]
            now = clock()
            for slot, c in enumerate(counts):
                if c == 0:
                    continue
                req = self.active[slot]
                req.remaining -= c
                if req.remaining == 0:
                    self._complete(req, now)
                    done.append(req)
        return done

    def _complete(self, req: MapRequest, now: float) -> None:
        rows = slice(req.start_row, req.start_row + req.voxels)
        x = natural_of(self.answer_u[rows], self.config)
        req.maps = {name: x[:, k].clone() for k, name in enumerate(UNKNOWN)}
        req.completed = now
        self.arena.release(req.start_row, req.voxels)
        del self.active[req.slot]
        self._free_slots.append(req.slot)
        self.finished.append(req)
        self.stats.completed += 1

    def serve(self, requests: list[MapRequest], *, realtime: bool = True) -> list[MapRequest]:
        """Serve requests whose ``arrival`` times (s, from now) come in order.

        With ``realtime`` the wall clock decides what has arrived; without it
        every request is submitted at once (for tests of the mix).
        """
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        t0 = time.perf_counter()

        def clock():
            return time.perf_counter() - t0

        if not realtime:
            for r in pending:
                r.arrival = 0.0
        while pending or self.queue or self.active:
            now = clock()
            while pending and (not realtime or pending[0].arrival <= now):
                self.submit(pending.popleft())
            self.admit(now)
            if self.pool.n == 0:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.01)))
                    continue
                if self.queue:
                    raise RuntimeError("a queued request can never be admitted")
                break
            self.step(clock)
        return self.finished


def latency_summary(requests: list[MapRequest]) -> dict[str, float]:
    lat = sorted(r.latency for r in requests if r.latency is not None)
    if not lat:
        return {"p50_s": float("nan"), "p99_s": float("nan")}

    def q(p):
        k = min(len(lat) - 1, max(0, int(round(p * (len(lat) - 1)))))
        return lat[k]

    return {"p50_s": q(0.50), "p99_s": q(0.99), "max_s": lat[-1], "mean_s": sum(lat) / len(lat)}


def serve_plain(program: Program, states: int, bounds: dict, start: torch.Tensor,
                requests: list[MapRequest], loop: GaussNewton) -> list[MapRequest]:
    """The plain form: one request at a time, first come first served, each
    solved to completion before the next starts (what repeated calls of a
    per-volume solver give)."""
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    t0 = time.perf_counter()
    done = []
    while pending:
        now = time.perf_counter() - t0
        if pending[0].arrival > now:
            time.sleep(min(pending[0].arrival - now, 0.01))
            continue
        req = pending.popleft()
        req.admitted = time.perf_counter() - t0
        sol = loop.minimize_program(program, req.measured, start, bounds, states, b1=req.b1)
        torch.cuda.synchronize()
        req.maps = {name: sol.x[:, k] for k, name in enumerate(UNKNOWN)}
        req.completed = time.perf_counter() - t0
        done.append(req)
    return done
