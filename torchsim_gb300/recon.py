"""Gauss-Newton parameter mapping on the device.

The reference maps (T1, T2, M0) per voxel with ``NonlinearLeastSquares``
(``estimators/_nlls.py:18-327``): a ``GaussNewton`` loop under a per-voxel
``TrustRegion`` (Levenberg-Marquardt with Nielsen's damping update,
``recon/_gauss_newton.py:366-631``) over a ``ModelOperator`` whose bounds map
each property to an unconstrained variable (``_bounds.py``). Each of its
iterations evaluates the model and its Jacobian blocks with 1 + 3 x (forward +
JVP) passes, stores the (V, 3, 2P) real blocks and solves an augmented least
squares problem per voxel in FP32.

Here the state of every voxel stays on the device (:class:`VoxelPool`), each
iteration is three launches -- the FP64 step (``tsg_gn_step``), ONE fused sweep
that reduces the model and both tangents straight to the normal equations
against the measured samples (``tsg_gn_evaluate``), and the FP64 accept /
damping update (``tsg_gn_judge``) -- and finished voxels are compacted away,
as the reference's ``_retire`` does (``_gauss_newton.py:759-793``).
"""

from __future__ import annotations

import ctypes
import math
from collections.abc import Mapping
from dataclasses import dataclass, field
from typing import Any

import torch

from . import _native, engine
from .sequence import Program

EDGE = 1e-6  # _bounds.py:48
UNKNOWN = ("T1", "T2", "M0")


# ---- bounds (the reference's _bounds.py:77-199, FP64) ------------------------


def bound_of(bounds: Mapping[str, Any], name: str) -> tuple[float | None, float | None]:
    low, high = bounds.get(name, (None, None))
    if low is not None and high is not None and not high > low:
        raise ValueError(f"{name}: the bound ({low}, {high}) is not increasing")
    return low, high


def to_free(natural: torch.Tensor, bounds: Mapping[str, Any], names=UNKNOWN) -> torch.Tensor:
    """Unconstrained variables standing for ``natural`` (..., 3)."""
    cols = []
    for k, name in enumerate(names):
        low, high = bound_of(bounds, name)
        v = natural[..., k].to(torch.float64)
        if low is not None and high is not None:
            t = ((v - low) / (high - low)).clamp(EDGE, 1.0 - EDGE)
            cols.append(torch.log(t) - torch.log1p(-t))
        elif low is not None:
            x = (v - low).clamp_min(EDGE)
            cols.append(x + torch.log(-torch.expm1(-x)))
        elif high is not None:
            x = (high - v).clamp_min(EDGE)
            cols.append(-(x + torch.log(-torch.expm1(-x))))
        else:
            cols.append(v)
    return torch.stack(cols, dim=-1)


def config_of(bounds: Mapping[str, Any], tau: float, gradient_tolerance: float,
              step_tolerance: float, max_iterations: int) -> _native.GNConfig:
    low, high = [], []
    for name in UNKNOWN:
        lo, hi = bound_of(bounds, name)
        low.append(-math.inf if lo is None else float(lo))
        high.append(math.inf if hi is None else float(hi))
    return _native.GNConfig((ctypes.c_double * 3)(*low), (ctypes.c_double * 3)(*high), float(tau),
                            float(gradient_tolerance), float(step_tolerance), int(max_iterations))


def fixed_shape(states: int) -> tuple[int, int, int]:
    """A (lanes per voxel, orders per lane, warps per CTA) of the GN sweep
    table that covers ``states``, chosen from the state count alone."""
    for lanes, orders in ((1, 10), (5, 4), (8, 4), (8, 8), (16, 4), (32, 4)):
        if lanes * orders >= states:
            return (lanes, orders, 4)
    raise ValueError("more than 128 states")


# ---- the loop ---------------------------------------------------------------


@dataclass
class TrustRegion:
    """Per-voxel Levenberg-Marquardt damping (``_gauss_newton.py:366-415``):
    the first damping is ``tau`` times the largest curvature at the start."""

    tau: float = 1e-2

    def __post_init__(self) -> None:
        if self.tau <= 0.0:
            raise ValueError(f"tau must be positive, got {self.tau}")


@dataclass
class Solution:
    """The reference's ``Solution`` fields that a per-voxel fit fills
    (``_gauss_newton.py:88-114``): maps, final cost per voxel, steps taken."""

    x: torch.Tensor
    cost: torch.Tensor
    iterations: int
    unconverged: int
    steps: torch.Tensor = field(default=None)


class VoxelPool:
    """Device-resident LM state of a set of voxels, possibly from several
    requests; rows are compacted away as voxels finish."""

    FIELDS_F64 = {"u": 3, "cand": 3, "cost": 0, "normal": 10, "trial": 10, "damping": 0,
                  "rising": 0, "predicted": 0}
    FIELDS_I32 = ("status", "flags", "iterations")
    FIELDS_F32 = ("t1", "t2", "m0", "b1")
    # Bytes of state per voxel (for admission budgets).
    BYTES_PER_VOXEL = 8 * (3 + 3 + 1 + 10 + 10 + 1 + 1 + 1) + 4 * 3 + 4 * 4 + 8 * 2

    def __init__(self, device: torch.device) -> None:
        self.device = device
        self.n = 0
        self.t: dict[str, torch.Tensor] = {}
        for name, width in self.FIELDS_F64.items():
            shape = (0, width) if width else (0,)
            self.t[name] = torch.zeros(shape, dtype=torch.float64, device=device)
        for name in self.FIELDS_I32:
            self.t[name] = torch.zeros(0, dtype=torch.int32, device=device)
        for name in self.FIELDS_F32:
            self.t[name] = torch.zeros(0, dtype=torch.float32, device=device)
        self.t["rows"] = torch.zeros(0, dtype=torch.int64, device=device)   # measured row
        self.t["owner"] = torch.zeros(0, dtype=torch.int64, device=device)  # answer row

    def add(self, u0: torch.Tensor, b1: torch.Tensor | None, rows: torch.Tensor,
            owner: torch.Tensor) -> None:
        """Append voxels starting at free variables ``u0`` (k, 3)."""
        k = int(rows.numel())
        if k == 0:
            return
        new = {name: torch.zeros((k, w) if w else (k,), dtype=torch.float64, device=self.device)
               for name, w in self.FIELDS_F64.items()}
        new["u"] = u0.to(self.device, torch.float64).expand(k, 3).contiguous()
        for name in self.FIELDS_I32:
            new[name] = torch.zeros(k, dtype=torch.int32, device=self.device)
        for name in ("t1", "t2", "m0"):
            new[name] = torch.zeros(k, dtype=torch.float32, device=self.device)
        new["b1"] = (torch.ones(k, dtype=torch.float32, device=self.device) if b1 is None
                     else b1.to(self.device, torch.float32).reshape(k))
        new["rows"] = rows.to(self.device, torch.int64)
        new["owner"] = owner.to(self.device, torch.int64)
        for name in self.t:
            self.t[name] = torch.cat([self.t[name], new[name]]).contiguous()
        self.n += k

    def state(self) -> _native.GNState:
        t = self.t
        return _native.GNState(*[t[n].data_ptr() for n in (
            "u", "cand", "cost", "normal", "trial", "damping", "rising", "predicted", "status",
            "flags", "iterations", "t1", "t2", "m0")])

    def iterate(self, program: Program, measured: torch.Tensor, states: int,
                config: _native.GNConfig, launch=None) -> None:
        """step -> fused evaluation at the candidates -> judge, all on the stream."""
        if self.n == 0:
            return
        lib = _native.library()
        stream = torch.cuda.current_stream().cuda_stream
        st = self.state()
        _native.check(lib.tsg_gn_step(ctypes.byref(st), self.n, ctypes.byref(config), stream))
        t = self.t
        tissue = _native.Tissue(t["t1"].data_ptr(), t["t2"].data_ptr(), t["m0"].data_ptr(),
                                t["b1"].data_ptr(), None)
        _native.check(lib.tsg_gn_evaluate(program.handle, ctypes.byref(tissue), self.n, states,
                                          measured.data_ptr(), t["rows"].data_ptr(),
                                          t["trial"].data_ptr(), _native.launch_shape(launch),
                                          stream))
        _native.check(lib.tsg_gn_judge(ctypes.byref(st), self.n, ctypes.byref(config), stream))

    def retire(self) -> dict[str, torch.Tensor]:
        """Remove finished voxels; returns their owner rows, free variables,
        costs and step counts (one host sync)."""
        done = self.t["status"] == _native_done()
        out = {"owner": self.t["owner"][done], "u": self.t["u"][done],
               "cost": self.t["cost"][done], "iterations": self.t["iterations"][done],
               "limited": (self.t["flags"][done] & 4)}
        keep = ~done
        for name in self.t:
            self.t[name] = self.t[name][keep].contiguous()
        self.n = int(self.t["rows"].numel())
        return out


def _native_done() -> int:
    return 2  # TSG_GN_DONE


def natural_of(u: torch.Tensor, config: _native.GNConfig) -> torch.Tensor:
    """Natural (T1, T2, M0) of free variables, float32 (k, 3)."""
    out = torch.empty((u.shape[0], 3), dtype=torch.float32, device=u.device)
    if u.shape[0]:
        _native.check(_native.library().tsg_gn_natural(
            u.contiguous().data_ptr(), u.shape[0], ctypes.byref(config), out.data_ptr(),
            torch.cuda.current_stream().cuda_stream))
    return out


class GaussNewton:
    """Levenberg-Marquardt over independent voxels (``GaussNewton`` +
    ``TrustRegion`` + ``direct`` of ``recon/_gauss_newton.py``), device-resident.

    ``max_iterations`` bounds the steps per voxel; a voxel stops early when
    its gradient is flat or its step is short, with the reference's
    tolerances (``gradient_tolerance``, ``step_tolerance``, :445-473).
    """

    def __init__(self, damping: TrustRegion | None = None, *, max_iterations: int = 8,
                 gradient_tolerance: float = 1e-8, step_tolerance: float = 1e-8,
                 launch=None) -> None:
        if max_iterations < 1:
            raise ValueError(f"max_iterations must be positive, got {max_iterations}")
        self.damping = damping if damping is not None else TrustRegion()
        self.max_iterations = int(max_iterations)
        self.gradient_tolerance = gradient_tolerance
        self.step_tolerance = step_tolerance
        self.launch = launch

    def config(self, bounds: Mapping[str, Any]) -> _native.GNConfig:
        return config_of(bounds, self.damping.tau, self.gradient_tolerance, self.step_tolerance,
                         self.max_iterations)

    @torch.no_grad()
    def minimize(self, program: Program, measured: torch.Tensor, start: torch.Tensor,
                 bounds: Mapping[str, Any], states: int, b1: torch.Tensor | None = None
                 ) -> Solution:
        """Fit (T1, T2, M0) to ``measured`` (V, P) complex64 from ``start``
        (natural, (3,) or (V, 3))."""
        device = measured.device
        V = measured.shape[0]
        config = self.config(bounds)
        pool = VoxelPool(device)
        u0 = to_free(torch.as_tensor(start, dtype=torch.float64, device=device).reshape(-1, 3),
                     bounds)
        idx = torch.arange(V, device=device)
        pool.add(u0.expand(V, 3), b1, idx, idx)
        measured = measured.contiguous()
        answer_u = u0.expand(V, 3).clone()
        cost = torch.zeros(V, dtype=torch.float64, device=device)
        steps = torch.zeros(V, dtype=torch.int32, device=device)
        unconverged = torch.zeros(V, dtype=torch.int32, device=device)
        for _ in range(self.max_iterations + 1):
            pool.iterate(program, measured, states, config, self.launch)
            out = pool.retire()
            answer_u[out["owner"]] = out["u"]
            cost[out["owner"]] = out["cost"]
            steps[out["owner"]] = out["iterations"]
            unconverged[out["owner"]] = out["limited"]
            if pool.n == 0:
                break
        iterations = int(steps.max().item()) if V else 0
        return Solution(x=natural_of(answer_u, config), cost=cost, iterations=iterations,
                        unconverged=int((unconverged != 0).sum().item()), steps=steps)


class NonlinearLeastSquares:
    """The estimator face (``estimators/_nlls.py:18-327``) for MRF maps of
    (T1, T2, M0) with B1 known: :meth:`fit` takes the starting point from the
    median of a training draw, :meth:`map` runs :class:`GaussNewton`."""

    def __init__(self, acquisition, *, bounds: Mapping[str, Any] | None = None,
                 initial: Mapping[str, float] | None = None,
                 loop: GaussNewton | None = None) -> None:
        self.acquisition = acquisition
        self.bounds = dict(bounds or {})
        self.initial = dict(initial or {})
        self.loop = loop if loop is not None else GaussNewton(TrustRegion(), max_iterations=20)
        self._start: torch.Tensor | None = None
        self.iterations = 0
        self.unconverged = 0

    def fit(self, *, seed: int | None = None, samples: int = 4096,
            parameters: torch.Tensor | None = None, **ranges) -> NonlinearLeastSquares:
        """Start at the median of the parameters drawn uniformly over ``ranges``
        (``{"T1": (lo, hi), ...}``), or of ``parameters`` (samples, 3)."""
        if parameters is None:
            gen = torch.Generator().manual_seed(0 if seed is None else seed)
            cols = []
            for name in UNKNOWN:
                lo, hi = ranges[name]
                cols.append(lo + (hi - lo) * torch.rand(samples, generator=gen))
            parameters = torch.stack(cols, dim=-1)
        median = torch.as_tensor(parameters).to(torch.float32).reshape(-1, 3).median(dim=0).values
        start = []
        for k, name in enumerate(UNKNOWN):
            value = float(self.initial.get(name, median[k]))
            low, high = bound_of(self.bounds, name)
            if (low is not None and value <= low) or (high is not None and value >= high):
                raise ValueError(f"{name}: the starting value {value:g} is not strictly inside "
                                 f"its bound ({low}, {high})")
            start.append(value)
        self._start = torch.tensor(start, dtype=torch.float32)
        return self

    def map(self, volume: torch.Tensor, known: Mapping[str, Any] | None = None
            ) -> dict[str, torch.Tensor]:
        if self._start is None:
            raise RuntimeError("the estimator has no starting point; call fit() first")
        sim = self.acquisition
        device = engine.require_cuda(volume.device if isinstance(volume, torch.Tensor) else None)
        volume = torch.as_tensor(volume).to(device, torch.complex64)
        shape = volume.shape[:-1]
        measured = volume.reshape(-1, volume.shape[-1])
        protocol = dict(sim.protocol)
        states = int(protocol.pop("states", sim.states))
        events = sim.events(**{k: v for k, v in protocol.items()})
        from .sequence import program_for

        program = program_for(events, device)
        b1 = None
        if known and "B1" in known:
            b1 = torch.as_tensor(known["B1"], dtype=torch.float32, device=device).reshape(-1)
            b1 = b1.expand(measured.shape[0]) if b1.numel() == 1 else b1
        sol = self.loop.minimize(program, measured, self._start.to(device), self.bounds, states,
                                 b1=b1)
        self.iterations, self.unconverged = sol.iterations, sol.unconverged
        return {name: sol.x[:, k].reshape(shape) for k, name in enumerate(UNKNOWN)}



def _solve3(M: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Batched 3x3 SPD solve by Cholesky in torch ops (NaN where not SPD)."""
    l00 = torch.sqrt(M[:, 0, 0])
    l10 = M[:, 1, 0] / l00
    l20 = M[:, 2, 0] / l00
    l11 = torch.sqrt(M[:, 1, 1] - l10 * l10)
    l21 = (M[:, 2, 1] - l20 * l10) / l11
    l22 = torch.sqrt(M[:, 2, 2] - l20 * l20 - l21 * l21)
    y0 = b[:, 0] / l00
    y1 = (b[:, 1] - l10 * y0) / l11
    y2 = (b[:, 2] - l20 * y0 - l21 * y1) / l22
    x2 = y2 / l22
    x1 = (y1 - l21 * x2) / l11
    x0 = (y0 - l10 * x1 - l20 * x2) / l00
    return torch.stack([x0, x1, x2], dim=-1)


class PlainGaussNewton(GaussNewton):
    """The plain GPU form of the same Levenberg-Marquardt loop, laid out as
    the reference lays it out (``_at`` -> ``ModelOperator.jacobian`` ->
    ``direct``, ``recon/_gauss_newton.py:633-651``): per iteration one forward
    pass and one pass per Jacobian column, the (V, 3, P) Jacobian and the
    residual written to HBM, then torch reductions and a batched FP64 solve.
    It serves as the baseline the fused evaluation is measured against."""

    @torch.no_grad()
    def minimize(self, program: Program, measured: torch.Tensor, start: torch.Tensor,
                 bounds: Mapping[str, Any], states: int, b1: torch.Tensor | None = None
                 ) -> Solution:
        device = measured.device
        V = measured.shape[0]
        config = self.config(bounds)
        u = to_free(torch.as_tensor(start, dtype=torch.float64, device=device).reshape(-1, 3),
                    bounds).expand(V, 3).clone()
        b1v = None if b1 is None else b1.to(device, torch.float32).reshape(V)
        live = torch.arange(V, device=device)
        answer = u.clone()
        steps = torch.zeros(V, dtype=torch.int32, device=device)
        limited = torch.zeros(V, dtype=torch.bool, device=device)
        lows = torch.tensor([config.low[k] for k in range(3)], dtype=torch.float64, device=device)
        highs = torch.tensor([config.high[k] for k in range(3)], dtype=torch.float64, device=device)

        def natural(x):
            return lows + (highs - lows) * torch.sigmoid(x)

        def widen(x):
            s = torch.sigmoid(x)
            return (highs - lows) * s * (1 - s)

        def at(x, rows):
            nat = natural(x).to(torch.float32)
            tissue = engine.TissueMaps(nat[:, 0].contiguous(), nat[:, 1].contiguous(),
                                       nat[:, 2].contiguous(),
                                       None if b1v is None else b1v[rows].contiguous(), None)
            sig = engine.forward(program, tissue, states)
            cols = [engine.forward_tangents(program, tissue, states, (name,), with_signal=False)[1]
                    for name in UNKNOWN]
            jac = torch.cat(cols, dim=1).real.to(torch.float64) * widen(x)[:, :, None]
            r = sig - measured[rows]
            cost = (r.real.double() ** 2 + r.imag.double() ** 2).sum(-1)
            A = torch.einsum("vkp,vlp->vkl", jac, jac)
            g = torch.einsum("vkp,vp->vk", jac, r.real.double())
            return cost, A, g

        if any(not (math.isfinite(config.low[k]) and math.isfinite(config.high[k]))
               for k in range(3)):
            raise NotImplementedError("the plain form takes two-sided bounds")
        cost, A, g = at(u, live)
        damping = self.damping.tau * A.diagonal(dim1=-2, dim2=-1).amax(-1)
        rising = torch.full_like(damping, 2.0)
        eye = torch.eye(3, dtype=torch.float64, device=device)
        for _ in range(self.max_iterations):
            flat = g.abs().amax(-1) < self.gradient_tolerance
            if bool(flat.any()):
                answer[live[flat]] = u[flat]
                keep = ~flat
                live, u, cost, A, g = live[keep], u[keep], cost[keep], A[keep], g[keep]
                damping, rising = damping[keep], rising[keep]
            if live.numel() == 0:
                break
            step = _solve3(A + damping[:, None, None] * eye, -g)
            singular = ~torch.isfinite(step).all(-1)
            short = step.norm(dim=-1) < self.step_tolerance * (u.norm(dim=-1) + self.step_tolerance)
            cand = u + step
            tcost, tA, tg = at(cand, live)
            predicted = (step * (damping[:, None] * step - g)).sum(-1)
            gain = torch.where(predicted > 0, (cost - tcost) / predicted.clamp_min(1.1754943508222875e-38),
                               torch.zeros_like(predicted))
            better = (gain > 0) & ~singular
            lowered = damping * (1.0 - (2.0 * gain - 1.0) ** 3).clamp_min(1.0 / 3.0)
            damping = torch.where(better, lowered, damping * rising)
            rising = torch.where(better, torch.full_like(rising, 2.0), rising * 2.0)
            u = torch.where(better[:, None], cand, u)
            cost = torch.where(better, tcost, cost)
            A = torch.where(better[:, None, None], tA, A)
            g = torch.where(better[:, None], tg, g)
            steps[live] += 1
            staying = ~(short & ~singular)
            if not bool(staying.all()):
                done = ~staying
                answer[live[done]] = u[done]
                live, u, cost, A, g = live[staying], u[staying], cost[staying], A[staying], g[staying]
                damping, rising = damping[staying], rising[staying]
            if live.numel() == 0:
                break
        if live.numel():
            answer[live] = u
            limited[live] = True
        x = natural(answer).to(torch.float32)
        return Solution(x=x, cost=torch.zeros(V, dtype=torch.float64, device=device),
                        iterations=int(steps.max().item()) if V else 0,
                        unconverged=int(limited.sum().item()), steps=steps)
