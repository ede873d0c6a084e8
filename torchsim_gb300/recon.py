"""Gauss-Newton parameter mapping on the device.

The reference maps (T1, T2, M0) per voxel with ``NonlinearLeastSquares``
(``estimators/_nlls.py:18-327``): a ``GaussNewton`` loop under a per-voxel
``TrustRegion`` (Levenberg-Marquardt with Nielsen's damping update,
``recon/_gauss_newton.py:366-631``) over a ``ModelOperator``
(``recon/_operator.py:49-484``) whose bounds map each property to an
unconstrained variable (``_bounds.py``). Each of its iterations evaluates the
model and its Jacobian blocks with 1 + 3 x (forward + JVP) passes, stores the
(V, 3, 2P) real blocks and solves an augmented least squares problem per voxel
in FP32.

The same faces are kept here -- :class:`ModelOperator` (``A``, ``A_jvp``,
``A_vjp``, ``jacobian``, ``initial``, ``split``, ``select``),
``GaussNewton(damping).minimize(operator, measured, initial)`` returning a
:class:`Solution`, and ``NonlinearLeastSquares(acquisition, bounds=...)
.fit(unknown, *, known, noise_std, ...) .map(volume, known, *, uncertainty)``
-- with two routes under ``minimize``:

* the fused route, for the MRF model of (T1, T2, M0) with B1 known (the
  mapping workload): the state of every voxel stays on the device
  (:class:`VoxelPool`), each iteration is three launches -- the FP64 step
  (``tsg_gn_step``), ONE fused sweep that reduces the model and both tangents
  straight to the normal equations against the measured samples
  (``tsg_gn_evaluate``), and the FP64 accept / damping update
  (``tsg_gn_judge``) -- and finished voxels are compacted away, as the
  reference's ``_retire`` does (``_gauss_newton.py:759-793``);
* the block route, for any other operator: the reference's loop over the
  operator's Jacobian blocks, which come from one fused forward + tangents
  sweep per evaluation, with the damped step solved from the normal equations
  in FP64.
"""

from __future__ import annotations

import ctypes
import math
from collections.abc import Callable, Mapping, Sequence
from copy import copy as shallow_copy
from dataclasses import dataclass, field
from typing import Any

import torch

from . import _native, engine
from .sequence import Program, program_for

EDGE = 1e-6  # _bounds.py:48
UNKNOWN = ("T1", "T2", "M0")
_TINY = 1.1754943508222875e-38  # smallest normal float (_gauss_newton.py's clamp)
_SAMPLES = 10_000  # training draws where nothing states a count (estimators/_mapping.py:43)


# ---- bounds (the reference's _bounds.py:77-199) ------------------------------


def bound_of(bounds: Mapping[str, Any], name: str) -> tuple[float | None, float | None]:
    low, high = bounds.get(name, (None, None))
    if low is not None and high is not None and not high > low:
        raise ValueError(f"{name}: the bound ({low}, {high}) is not increasing")
    return low, high


def to_free(natural: torch.Tensor, bounds: Mapping[str, Any], names=UNKNOWN) -> torch.Tensor:
    """Unconstrained variables standing for ``natural`` (..., k), in FP64:
    the logit of the position inside a two-sided bound, the inverse softplus
    of the distance from a one-sided one (``_bounds.py:108-160``)."""
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


def to_natural(free: torch.Tensor, bounds: Mapping[str, Any], names: Sequence[str]
               ) -> torch.Tensor:
    """The properties the unconstrained variables stand for, in ``free``'s
    dtype (``_bounds.py:77-105``): ``low + (high - low) * sigmoid(u)``,
    ``low + softplus(u)``, ``high - softplus(-u)`` or ``u``."""
    if not bounds:
        return free
    cols = []
    for k, name in enumerate(names):
        low, high = bound_of(bounds, name)
        u = free[..., k]
        if low is not None and high is not None:
            cols.append(low + (high - low) * torch.sigmoid(u))
        elif low is not None:
            cols.append(low + torch.nn.functional.softplus(u))
        elif high is not None:
            cols.append(high - torch.nn.functional.softplus(-u))
        else:
            cols.append(u)
    return torch.stack(cols, dim=-1)


def widen(bounds: Mapping[str, Any], names: Sequence[str], free: torch.Tensor) -> torch.Tensor:
    """d(property)/d(free variable), the chain factor that multiplies the
    Jacobian (``_bounds.py:163-199``)."""
    if not bounds:
        return torch.ones_like(free)
    cols = []
    for k, name in enumerate(names):
        low, high = bound_of(bounds, name)
        u = free[..., k]
        if low is not None and high is not None:
            s = torch.sigmoid(u)
            cols.append((high - low) * s * (1.0 - s))
        elif low is not None:
            cols.append(torch.sigmoid(u))
        elif high is not None:
            cols.append(torch.sigmoid(-u))
        else:
            cols.append(torch.ones_like(u))
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


# ---- damping policies and the pieces of a solve ------------------------------


@dataclass
class TrustRegion:
    """Per-voxel Levenberg-Marquardt damping (``_gauss_newton.py:366-415``):
    the first damping is ``tau`` times the largest curvature at the start; a
    step that lowered the cost is taken and the damping falls by Nielsen's
    factor ``max(1/3, 1 - (2 gain - 1)^3)``, a rejected one multiplies it by a
    factor that doubles with every rejection in a row."""

    tau: float = 1e-2
    anchored = False   # the damping shortens a step; it pulls it nowhere
    per_voxel = True   # each voxel carries its own weight and retires alone

    def __post_init__(self) -> None:
        if self.tau <= 0.0:
            raise ValueError(f"tau must be positive, got {self.tau}")

    def begin(self, curvature: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """(damping, rising factor) at the start."""
        damping = self.tau * curvature.diagonal(dim1=-2, dim2=-1).amax(-1)
        return damping, torch.full_like(damping, 2.0)

    def judge(self, damping, rising, gain, singular):
        """(accepted, next damping, next rising factor)."""
        better = (gain > 0) & ~singular
        lowered = damping * (1.0 - (2.0 * gain - 1.0).pow(3)).clamp_min(1.0 / 3.0)
        return (better, torch.where(better, lowered, damping * rising),
                torch.where(better, torch.full_like(rising, 2.0), rising * 2.0))


@dataclass
class Schedule:
    """One damping for the whole volume, lowered geometrically, every step
    taken and pulled towards the start: the iteratively regularised
    Gauss-Newton (``_gauss_newton.py:310-363``)."""

    initial: float = 1.0
    factor: float = 1.0 / 3.0
    minimum: float = 1e-3
    anchored = True
    per_voxel = False

    def __post_init__(self) -> None:
        if self.initial <= 0.0:
            raise ValueError(f"initial must be positive, got {self.initial}")
        if not 0.0 < self.factor < 1.0:
            raise ValueError(f"factor must lower the damping, got {self.factor}")
        if self.minimum <= 0.0:
            raise ValueError(f"minimum must be positive, got {self.minimum}")

    def begin(self, curvature: torch.Tensor) -> tuple[torch.Tensor, None]:
        return torch.as_tensor(self.initial, dtype=torch.float32, device=curvature.device), None

    def judge(self, damping, rising, gain, singular):
        return (torch.ones_like(gain, dtype=torch.bool),
                (damping * self.factor).clamp_min(self.minimum), None)


@dataclass(frozen=True)
class Linearization:
    """The model's derivative at one point as products with it
    (``_gauss_newton.py:60-83``): ``matvec`` d -> J d, ``rmatvec``
    v -> Re(J^H v), and the per-voxel ``blocks`` (voxels, channels, contrasts)."""

    matvec: Callable[[torch.Tensor], torch.Tensor]
    rmatvec: Callable[[torch.Tensor], torch.Tensor]
    blocks: torch.Tensor | None = None


def _diagonal(blocks: torch.Tensor) -> Linearization:
    return Linearization(
        matvec=lambda d: torch.einsum("vpt,vp->vt", blocks, d.to(blocks.dtype)),
        rmatvec=lambda v: torch.einsum("vpt,vt->vp", blocks.conj(), v.to(blocks.dtype)).real,
        blocks=blocks)


def _as_real(blocks: torch.Tensor, rhs: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """A complex contrast counts as two real measurements."""
    if not torch.is_complex(blocks):
        return blocks, rhs.real if torch.is_complex(rhs) else rhs
    return (torch.cat((blocks.real, blocks.imag), dim=-1),
            torch.cat((rhs.real, rhs.imag), dim=-1))


def direct(linearization: Linearization, rhs: torch.Tensor, damping: torch.Tensor,
           reference: torch.Tensor) -> torch.Tensor:
    """Every voxel's damped step at once (``_gauss_newton.py:247-307``): the
    minimiser of ``||J^T d - rhs||^2 + a ||d - z||^2``. The reference solves
    it as the augmented least-squares system in FP32; here its normal
    equations ``(J J^T + a I) d = J rhs + a z`` are factorised by Cholesky in
    FP64 (a voxel whose matrix is not positive definite gets a NaN step,
    which the loop treats as singular)."""
    blocks = linearization.blocks
    if blocks is None:
        raise ValueError("direct() needs the per-voxel Jacobian blocks")
    rows, columns = _as_real(blocks, rhs)
    rows = rows.to(torch.float64)
    a = torch.broadcast_to(torch.as_tensor(damping, device=rows.device).to(torch.float64),
                           reference.shape)
    eye = torch.eye(rows.shape[-2], dtype=torch.float64, device=rows.device)
    system = rows @ rows.mT + a[..., None] * eye
    target = (rows @ columns.to(torch.float64)[..., None]).squeeze(-1) + a * reference.double()
    factor, info = torch.linalg.cholesky_ex(system)
    step = torch.cholesky_solve(target[..., None], factor).squeeze(-1)
    step = torch.where((info == 0)[..., None], step, torch.full_like(step, float("nan")))
    return step.to(reference.dtype)


@dataclass
class Solution:
    """What a solve returned (``_gauss_newton.py:86-114``): ``x`` the maps as
    the variables solved for (``ModelOperator.split`` gives the properties),
    ``cost`` the summed squared residual after each step, ``damping`` the mean
    damping each step ran at, the steps taken and how many voxels were still
    moving when the loop stopped. ``steps`` adds the steps each voxel took."""

    x: torch.Tensor
    cost: torch.Tensor
    damping: torch.Tensor
    iterations: int
    unconverged: int
    steps: torch.Tensor | None = field(default=None)


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

    def retire(self, group: torch.Tensor | None = None, groups: int = 1
               ) -> dict[str, torch.Tensor | list[int]]:
        """Remove finished voxels; returns their owner rows, free variables,
        costs, step counts and limit flags, and ``counts``: how many finished,
        per group when ``group`` gives each live voxel's group (in
        ``range(groups)``), else one total.

        One device-to-host read per call, of those counts. The rows are then
        partitioned stably (kept rows first, each side in pool order) by two
        prefix sums and a scatter, and every copy is sized from the counts
        already on the host."""
        done = self.t["status"] == _native_done()
        if group is not None:
            tally = torch.zeros(groups, dtype=torch.int64, device=self.device)
            tally.index_add_(0, group, done.to(torch.int64))
        else:
            tally = done.sum(dtype=torch.int64).reshape(1)
        counts = tally.cpu().tolist()
        finished = int(sum(counts))
        kept = self.n - finished
        if finished:
            flag = done.to(torch.int64)
            dest = torch.where(done, torch.cumsum(flag, 0) + (kept - 1),
                               torch.cumsum(1 - flag, 0) - 1)
            order = torch.empty_like(dest).scatter_(
                0, dest, torch.arange(self.n, device=self.device))
            keep_rows, done_rows = order[:kept], order[kept:]
        else:
            done_rows = torch.zeros(0, dtype=torch.int64, device=self.device)
        t = self.t
        out = {"owner": t["owner"].index_select(0, done_rows),
               "u": t["u"].index_select(0, done_rows),
               "cost": t["cost"].index_select(0, done_rows),
               "iterations": t["iterations"].index_select(0, done_rows),
               "limited": t["flags"].index_select(0, done_rows) & 4,
               "counts": counts}
        if finished:
            for name in t:
                t[name] = t[name].index_select(0, keep_rows)
            self.n = kept
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


# ---- the model as an operator (recon/_operator.py:49-484) ---------------------

_AMPLITUDE = ("amplitude.real", "amplitude.imag")


class ModelOperator(torch.nn.Module):
    """A simulator over parameter maps, with its derivatives
    (``recon/_operator.py:49-484``). Maps are stacked on the last axis:
    ``(..., channels)`` in, ``(..., contrasts)`` complex out, every leading
    axis a voxel axis. The channels are the ``unknown`` properties, each as
    its unconstrained variable divided by its ``scale``, then (with
    ``amplitude``) the real and imaginary parts of a complex amplitude that
    multiplies the model.

    ``jacobian`` builds every voxel's block, ``(..., channels, contrasts)``,
    from ONE fused forward + tangents sweep (the reference pays one
    forward-mode pass per column); ``A_jvp`` and ``A_vjp`` are products with
    those blocks. ``subspace`` is any object with ``project(tensor)``, applied
    to the prediction and its blocks.
    """

    def __init__(self, acquisition: Any, *unknown: str,
                 bounds: Mapping[str, tuple[float | None, float | None]] | None = None,
                 scale: Mapping[str, float] | None = None, amplitude: bool = True,
                 subspace: Any = None) -> None:
        super().__init__()
        if not unknown:
            raise ValueError("name at least one property to solve for")
        self.acquisition = acquisition
        self.unknown = tuple(unknown)
        self.bounds = dict(bounds or {})
        self.amplitude = bool(amplitude)
        self.subspace = subspace
        for label, given in (("bounds", self.bounds), ("scale", scale or {})):
            stray = set(given) - set(self.unknown)
            if stray:
                raise ValueError(f"{label} names {sorted(stray)}, which "
                                 f"{'is' if len(stray) == 1 else 'are'} not being solved for")
        for name in self.unknown:
            bound_of(self.bounds, name)
        self.scale = tuple(float((scale or {}).get(name, 1.0)) for name in self.unknown)
        if any(value <= 0.0 for value in self.scale):
            raise ValueError("every scale must be positive")

    @property
    def channels(self) -> int:
        return len(self.unknown) + 2 * self.amplitude

    @property
    def names(self) -> tuple[str, ...]:
        return self.unknown + (_AMPLITUDE if self.amplitude else ())

    def _parts(self, x: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        if x.shape[-1] != self.channels:
            raise ValueError(f"this operator has {self.channels} channels, got {x.shape[-1]}")
        free = x[..., :len(self.unknown)]
        return free, torch.tensor(self.scale, dtype=free.dtype, device=free.device)

    def _named(self, x: torch.Tensor) -> tuple[dict[str, torch.Tensor], torch.Tensor | None]:
        free, scale = self._parts(x)
        natural = to_natural(free * scale, self.bounds, self.unknown)
        given = {name: natural[..., k] for k, name in enumerate(self.unknown)}
        rho = torch.complex(x[..., -2], x[..., -1]) if self.amplitude else None
        return given, rho

    def split(self, x: torch.Tensor) -> dict[str, torch.Tensor]:
        """The maps ``x`` stands for, in their own units (plus ``amplitude``)."""
        given, rho = self._named(x)
        return given if rho is None else {**given, "amplitude": rho}

    def initial(self, shape: Sequence[int] = (), **values: Any) -> torch.Tensor:
        """Maps to start from as the variables solved for, ``(*shape,
        channels)``: a value (or map) per unknown in its own units, the middle
        of a two-sided bound where left out; amplitude 1 unless given."""
        stray = set(values) - set(self.unknown) - {"amplitude"}
        if stray:
            raise ValueError(f"{sorted(stray)} is not a channel of this operator")
        columns = []
        for name in self.unknown:
            low, high = bound_of(self.bounds, name)
            if name in values:
                start = torch.as_tensor(values[name], dtype=torch.float32)
            elif low is not None and high is not None:
                start = torch.tensor(0.5 * (low + high))
            else:
                raise ValueError(f"{name} has no two-sided bound, so give it a starting value")
            start = torch.broadcast_to(start, tuple(shape)).to(torch.float32)
            if ((low is not None and bool((start <= low).any()))
                    or (high is not None and bool((start >= high).any()))):
                raise ValueError(f"{name}: {start.min() if low is not None else start.max()} "
                                 f"is not strictly inside its bound ({low}, {high})")
            columns.append(start)
        natural = torch.stack(columns, dim=-1)
        free = (to_free(natural, self.bounds, self.unknown).to(torch.float32)
                / torch.tensor(self.scale))
        if not self.amplitude:
            return free
        rho = torch.broadcast_to(torch.as_tensor(values.get("amplitude", 1.0 + 0.0j)),
                                 tuple(shape)).to(torch.complex64)
        return torch.cat((free, rho.real[..., None], rho.imag[..., None]), dim=-1)

    def select(self, keep: torch.Tensor) -> ModelOperator:
        """This operator over a subset of the voxels: every property map bound
        on the acquisition (one value per voxel) is narrowed with it."""
        narrowed = {name: value[keep] for name, value in self.acquisition.bound.items()
                    if torch.is_tensor(value) and value.ndim}
        if not narrowed:
            return self
        chosen = shallow_copy(self)
        chosen.acquisition = self.acquisition.bind(**narrowed)
        return chosen

    def _flat(self, x: torch.Tensor) -> tuple[torch.Tensor, tuple[int, ...]]:
        return x.reshape(-1, x.shape[-1]), tuple(x.shape[:-1])

    def _predict(self, x: torch.Tensor) -> torch.Tensor:
        given, rho = self._named(x)
        signal = torch.as_tensor(self.acquisition.simulate(**given))
        if self.subspace is not None:
            signal = self.subspace.project(signal)
        return signal if rho is None else signal * rho[..., None]

    def _blocks(self, x: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """(prediction, blocks) from one fused forward + tangents sweep."""
        given, rho = self._named(x)
        free, scale = self._parts(x)
        signal, derivative = self.acquisition.jacobian(self.unknown, **given)
        if self.subspace is not None:
            signal = self.subspace.project(signal)
            derivative = self.subspace.project(derivative)
        chain = widen(self.bounds, self.unknown, free * scale) * scale
        columns = derivative * chain[..., None]
        if rho is None:
            return signal, columns
        columns = columns * rho[..., None, None]
        return (signal * rho[..., None],
                torch.cat((columns, signal[..., None, :], (1j * signal)[..., None, :]), dim=-2))

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        """The contrasts these maps record, ``(..., contrasts)``."""
        flat, shape = self._flat(x)
        out = self._predict(flat)
        return out.reshape(*shape, out.shape[-1])

    A = forward

    def jacobian(self, x: torch.Tensor) -> torch.Tensor:
        """Every voxel's derivative block, ``(..., channels, contrasts)``."""
        flat, shape = self._flat(x)
        out = self._blocks(flat)[1]
        return out.reshape(*shape, *out.shape[-2:])

    def A_jvp(self, x: torch.Tensor, d: torch.Tensor) -> torch.Tensor:
        """``J d``, ``(..., contrasts)``."""
        flat, shape = self._flat(x)
        blocks = self._blocks(flat)[1]
        out = torch.einsum("vct,vc->vt", blocks, d.reshape(flat.shape).to(blocks.dtype))
        return out.reshape(*shape, out.shape[-1])

    def A_vjp(self, x: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
        """``Re(J^H v)``, ``(..., channels)`` real: the adjoint of ``A_jvp``
        under the real inner product."""
        flat, shape = self._flat(x)
        blocks = self._blocks(flat)[1]
        out = torch.einsum("vct,vt->vc", blocks.conj(),
                           v.reshape(flat.shape[0], v.shape[-1]).to(blocks.dtype)).real
        return out.reshape(*shape, out.shape[-1])


# ---- the loop -----------------------------------------------------------------


class GaussNewton:
    """Solve for the maps that explain a measurement by repeated
    linearisation (``recon/_gauss_newton.py:420-651``): ``damping`` a
    :class:`TrustRegion` (Levenberg-Marquardt, per voxel, the default of the
    mapping estimator) or a :class:`Schedule`; ``solve`` the inner solve
    (:func:`direct` when left out); ``max_iterations`` the most steps; a voxel
    stops when its gradient is flat or its step is short
    (``gradient_tolerance``, ``step_tolerance``).

    :meth:`minimize` takes the reference's ``(operator, measured, initial)``.
    Where the operator is the MRF model of (T1, T2, M0) with B1 known on a
    TrustRegion loop, it runs the fused device route (:meth:`minimize_program`);
    any other operator runs the block route.
    """

    def __init__(self, damping: Any = None, *, solve: Callable[..., torch.Tensor] | None = None,
                 max_iterations: int = 8, gradient_tolerance: float = 1e-8,
                 step_tolerance: float = 1e-8, launch=None) -> None:
        if max_iterations < 1:
            raise ValueError(f"max_iterations must be positive, got {max_iterations}")
        self.damping = damping if damping is not None else Schedule()
        self.solve = solve
        self.max_iterations = int(max_iterations)
        self.gradient_tolerance = gradient_tolerance
        self.step_tolerance = step_tolerance
        self.launch = launch

    def config(self, bounds: Mapping[str, Any]) -> _native.GNConfig:
        tau = getattr(self.damping, "tau", None)
        if tau is None:
            raise ValueError("the fused route runs a TrustRegion loop")
        return config_of(bounds, tau, self.gradient_tolerance, self.step_tolerance,
                         self.max_iterations)

    # -- the reference's face ---------------------------------------------------

    @torch.no_grad()
    def minimize(self, operator: ModelOperator, measured: torch.Tensor, initial: torch.Tensor,
                 *, encoding: Any = None) -> Solution:
        """Solve for the maps that explain ``measured`` ``(..., contrasts)``
        from ``initial`` ``(..., channels)`` (build it with
        :meth:`ModelOperator.initial`). ``encoding`` (an operator in front of
        the model, e.g. Fourier encoding) is not on this path."""
        if encoding is not None:
            raise NotImplementedError(
                "an encoding operator in front of the model (a k-space reconstruction) is not "
                "on this path; the voxel-wise fit is")
        plan = self._fused_plan(operator)
        if plan is not None:
            return self._minimize_fused(operator, measured, initial, *plan)
        return self._minimize_blocks(operator, measured, initial)

    def _fused_plan(self, operator: Any):
        """(program, states, B1 map or None) where the fused route computes
        exactly this operator's model, else None."""
        from .simulators import MRFSimulator, _leaves_real_subspace

        if not isinstance(operator, ModelOperator):
            raise TypeError("minimize takes a ModelOperator (build one over a simulator)")
        acquisition = operator.acquisition
        if (not isinstance(acquisition, MRFSimulator) or operator.amplitude
                or operator.subspace is not None or sorted(operator.unknown) != sorted(UNKNOWN)
                or any(s != 1.0 for s in operator.scale)
                or not isinstance(self.damping, TrustRegion)
                or self.solve not in (None, direct)):
            return None
        held, protocol, states, device, repetitions = acquisition._split({})
        for name, value in held.items():
            if name == "B1":
                continue
            if name in ("B0", "B1phase") and not torch.is_tensor(value) and float(value) == 0.0:
                continue
            if name == "inv_efficiency" and not torch.is_tensor(value) and float(value) == 1.0:
                continue
            return None
        plain = {k: (v.detach() if torch.is_tensor(v) else v) for k, v in protocol.items()}
        events = acquisition.events(repetitions=repetitions, **plain)
        if _leaves_real_subspace(events, {}):
            return None
        return events, states, held.get("B1")

    def _minimize_fused(self, operator: ModelOperator, measured: torch.Tensor,
                        initial: torch.Tensor, events, states: int, b1: Any) -> Solution:
        device = engine.require_cuda(measured.device if measured.device.type == "cuda" else None)
        shape = initial.shape[:-1]
        start = initial.reshape(-1, initial.shape[-1]).to(device)
        V = start.shape[0]
        data = measured.reshape(V, measured.shape[-1]).to(device, torch.complex64).contiguous()
        order = [operator.unknown.index(name) for name in UNKNOWN]
        u0 = start.to(torch.float64)[:, order]
        if b1 is not None:
            b1 = torch.as_tensor(b1, dtype=torch.float32).to(device).reshape(-1)
            b1 = b1.expand(V) if b1.numel() == 1 else b1
        with torch.cuda.device(device):
            program = program_for(events, device)
            u, cost, steps, limited, history, weights = self._pool_solve(
                program, data, u0, b1, self.config(operator.bounds), states)
        x = torch.empty_like(start)
        x[:, order] = u.to(start.dtype)
        return Solution(x=x.reshape(*shape, x.shape[-1]), cost=history, damping=weights,
                        iterations=int(steps.max().item()) if V else 0,
                        unconverged=int((limited != 0).sum().item()), steps=steps)

    def _pool_solve(self, program: Program, measured: torch.Tensor, u0: torch.Tensor,
                    b1: torch.Tensor | None, config: _native.GNConfig, states: int):
        """The fused device loop over a voxel pool: (free variables in
        T1, T2, M0 order, final cost, steps and limit flags per voxel, the
        summed cost and mean damping after every iteration)."""
        device = measured.device
        V = measured.shape[0]
        pool = VoxelPool(device)
        idx = torch.arange(V, device=device)
        pool.add(u0, b1, idx, idx)
        answer_u = u0.clone()
        cost = torch.zeros(V, dtype=torch.float64, device=device)
        steps = torch.zeros(V, dtype=torch.int32, device=device)
        limited = torch.zeros(V, dtype=torch.int32, device=device)
        history, weights = [], []
        for it in range(self.max_iterations + 1):
            if it and pool.n:
                weights.append(pool.t["damping"].mean())
            pool.iterate(program, measured, states, config, self.launch)
            out = pool.retire()
            answer_u[out["owner"]] = out["u"]
            cost[out["owner"]] = out["cost"]
            steps[out["owner"]] = out["iterations"]
            limited[out["owner"]] = out["limited"]
            history.append(cost.sum() + pool.t["cost"].sum())
            if pool.n == 0:
                break
        empty = torch.zeros(0, dtype=torch.float64, device=device)
        return (answer_u, cost, steps, limited,
                torch.stack(history) if history else empty,
                torch.stack(weights) if weights else empty)

    @torch.no_grad()
    def minimize_program(self, program: Program, measured: torch.Tensor, start: torch.Tensor,
                         bounds: Mapping[str, Any], states: int, b1: torch.Tensor | None = None
                         ) -> Solution:
        """The fused route on a compiled program: fit (T1, T2, M0) to
        ``measured`` (V, P) complex64 from ``start`` (natural, (3,) or (V, 3));
        ``x`` of the answer is natural (T1, T2, M0) float32 and ``cost`` the
        final cost per voxel. What the mapping server and the bench call."""
        device = measured.device
        V = measured.shape[0]
        config = self.config(bounds)
        u0 = to_free(torch.as_tensor(start, dtype=torch.float64, device=device).reshape(-1, 3),
                     bounds).expand(V, 3).contiguous()
        u, cost, steps, limited, history, weights = self._pool_solve(
            program, measured.contiguous(), u0, b1, config, states)
        return Solution(x=natural_of(u, config), cost=cost, damping=weights,
                        iterations=int(steps.max().item()) if V else 0,
                        unconverged=int((limited != 0).sum().item()), steps=steps)

    def _minimize_blocks(self, operator: ModelOperator, measured: torch.Tensor,
                         initial: torch.Tensor) -> Solution:
        """The reference's loop (``_gauss_newton.py:475-631``, no encoding)
        over the operator's Jacobian blocks."""
        solve = self.solve or direct
        policy = self.damping
        shape = initial.shape[:-1]
        start = initial.reshape(-1, initial.shape[-1])
        data = measured.reshape(start.shape[0], measured.shape[-1]).to(start.device)
        retiring = bool(getattr(policy, "per_voxel", False))
        answer = start.clone()
        live = torch.arange(start.shape[0], device=start.device)
        x = start.clone()

        def at(point):
            predicted, blocks = operator._blocks(point)
            dtype = torch.promote_types(predicted.dtype, data.dtype)
            return predicted.to(dtype) - data.to(dtype), _diagonal(blocks.to(dtype))

        def cost_of(r):
            return r.real.square().sum(-1) + (r.imag.square().sum(-1) if torch.is_complex(r)
                                              else 0.0)

        def curvature(lin):
            rows = (torch.cat((lin.blocks.real, lin.blocks.imag), dim=-1)
                    if torch.is_complex(lin.blocks) else lin.blocks)
            return rows @ rows.mT

        def shaped(d):
            return d[..., None] if d.ndim == 1 else d

        residual, lin = at(x)
        cost = cost_of(residual)
        damping, rising = policy.begin(curvature(lin))
        history = [cost.sum()]
        weights = []

        def retire(keep):
            nonlocal x, live, data, residual, lin, cost, damping, rising, operator
            done = ~keep
            if bool(done.any()):
                answer[live[done]] = x[done]
            if bool(keep.all()):
                return
            x, live, data, residual = x[keep], live[keep], data[keep], residual[keep]
            lin = _diagonal(lin.blocks[keep])
            cost, damping = cost[keep], damping[keep]
            rising = None if rising is None else rising[keep]
            operator = operator.select(keep)

        iterations = 0
        for _ in range(self.max_iterations):
            gradient = lin.rmatvec(residual)
            flat = gradient.abs().amax(-1) < self.gradient_tolerance
            if retiring:
                retire(~flat)
                if x.shape[0] == 0:
                    break
                gradient = lin.rmatvec(residual)
            elif bool(flat.all()):
                break
            iterations += 1
            weights.append(damping.detach().reshape(-1).mean())
            reference = (start[live] - x if getattr(policy, "anchored", False)
                         else torch.zeros_like(x))
            step = solve(lin, -residual, shaped(damping), reference)
            walked = torch.linalg.vector_norm(step, dim=-1)
            short = walked < self.step_tolerance * (torch.linalg.vector_norm(x, dim=-1)
                                                    + self.step_tolerance)
            singular = ~torch.isfinite(step).all(-1)
            candidate = x + torch.nan_to_num(step)
            trial, trial_lin = at(candidate)
            trial_cost = cost_of(trial)
            predicted = (step * (shaped(damping) * step - gradient)).sum(-1)
            gain = torch.where(predicted > 0, (cost - trial_cost) / predicted.clamp_min(_TINY),
                               torch.zeros_like(predicted))
            better, damping, rising = policy.judge(damping, rising, gain, singular)
            x = torch.where(better[..., None] if better.ndim else better, candidate, x)
            residual = torch.where(better[:, None] if better.ndim else better, trial, residual)
            lin = _diagonal(torch.where(better[:, None, None] if better.ndim else better,
                                        trial_lin.blocks, lin.blocks))
            cost = torch.where(better, trial_cost, cost)
            history.append(cost.sum())
            if retiring:
                retire(~(short & ~singular))
                if x.shape[0] == 0:
                    break
            elif bool((short & ~singular).all()):
                break
        unconverged = int(x.shape[0]) if retiring else 0
        if retiring:
            if unconverged:
                answer[live] = x
        else:
            answer = x
        return Solution(x=answer.reshape(*shape, answer.shape[-1]), cost=torch.stack(history),
                        damping=(torch.stack(weights) if weights
                                 else torch.zeros(0, device=start.device)),
                        iterations=iterations, unconverged=unconverged)


# ---- the estimator face (estimators/_mapping.py, estimators/_nlls.py) ----------


def _draw(name: str, spec: Any, samples: int, generator: torch.Generator) -> torch.Tensor:
    """One property's training values: a range drawn uniformly, or values
    given (``estimators/_mapping.py:575-593``)."""
    if isinstance(spec, (tuple, list)) and len(spec) == 2:
        low, high = (float(v) for v in spec)
        if not high > low:
            raise ValueError(f"{name}: the range {spec} is not increasing")
        return low + (high - low) * torch.rand(samples, generator=generator)
    values = torch.as_tensor(spec, dtype=torch.float32).reshape(-1)
    if values.numel() == 1:
        return values.expand(samples).clone()
    if values.numel() != samples:
        raise ValueError(f"{name}: {values.numel()} values for {samples} training samples")
    return values


class NonlinearLeastSquares(torch.nn.Module):
    """Levenberg-Marquardt over every voxel at once (``estimators/_nlls.py:18-327``
    on the ``Estimator`` face of ``estimators/_mapping.py``): an estimator
    made from the acquisition it inverts, with every property that is neither
    unknown nor measured fixed on it (``MRFSimulator(...).bind(B1=...)``).
    :meth:`fit` names the unknowns and their ranges and starts the fit at the
    median of the training draw (or at ``initial``); :meth:`map` runs
    ``loop`` (default ``GaussNewton(TrustRegion(), solve=direct,
    max_iterations=20)``) over a :class:`ModelOperator` and returns one map
    per unknown.

    The reference's fit also simulates the training signals, which this
    method then ignores (``_nlls.py:174-176``); only the draw is made here.
    The draw uses the same generator and order, so the start is the
    reference's.
    """

    def __init__(self, acquisition: Any = None, *,
                 bounds: Mapping[str, tuple[float | None, float | None]] | None = None,
                 initial: Mapping[str, float] | None = None,
                 loop: GaussNewton | None = None) -> None:
        super().__init__()
        self.acquisition = acquisition
        self.bounds = dict(bounds or {})
        self.initial = dict(initial or {})
        self.loop = loop if loop is not None else GaussNewton(TrustRegion(), solve=direct,
                                                              max_iterations=20)
        self.noise_std: float | torch.Tensor = 0.0
        self.seed: int | None = None
        self._unknown: dict[str, Any] = {}
        self._known: dict[str, Any] = {}
        self._start: torch.Tensor | None = None
        self.iterations = 0
        self.unconverged = 0

    @property
    def unknown(self) -> tuple[str, ...]:
        return tuple(self._unknown)

    @property
    def known(self) -> tuple[str, ...]:
        return tuple(self._known)

    @property
    def fitted(self) -> bool:
        return self.acquisition is not None and self._start is not None

    def fit(self, unknown: Mapping[str, Any] | None = None, *,
            known: Mapping[str, Any] | None = None, noise_std: float | torch.Tensor = 0.0,
            rank: int | None = None, subspace: Any = None, seed: int | None = None,
            samples: int | None = None, chunk: int = 4096, signals: torch.Tensor | None = None,
            parameters: torch.Tensor | None = None, **ranges: Any) -> NonlinearLeastSquares:
        """Name the unknowns (``{name: (low, high)}`` or values, as a mapping
        or keywords) and the separately measured ``known`` properties, and take
        the start from the training draw (``estimators/_mapping.py:118-262``).
        ``signals`` + ``parameters`` give the training set outright."""
        del chunk
        properties = {**(unknown or {}), **ranges}
        measured = known if isinstance(known, Mapping) else None
        overlap = set(properties) & set(measured or ())
        if overlap:
            raise ValueError(f"{sorted(overlap)} cannot be both unknown and known")
        if rank is not None or subspace is not None:
            raise NotImplementedError("a temporal subspace is not on this path")
        if properties:
            self._unknown = dict(properties)
        if measured is not None:
            self._known = dict(measured)
        self.noise_std = noise_std
        self.seed = seed
        if signals is None:
            if self.acquisition is None:
                raise RuntimeError("nothing to fit from: give this estimator the acquisition "
                                   "it is inverting, or hand fit() the signals directly")
            if not self._unknown:
                raise ValueError("name at least one property to estimate")
            if samples is None:
                samples = self._stated_samples() or _SAMPLES
            if samples < 1:
                raise ValueError(f"samples must be positive, got {samples}")
            generator = torch.Generator()
            if seed is not None:
                generator.manual_seed(int(seed))
            drawn = {name: _draw(name, spec, samples, generator)
                     for name, spec in (*self._unknown.items(), *self._known.items())}
            parameters = torch.stack([drawn[name] for name in self._unknown], dim=-1)
        elif parameters is None:
            raise ValueError("signals given without their parameters")
        self._fit_arrays(parameters)
        return self

    def _stated_samples(self) -> int | None:
        lengths = {torch.as_tensor(spec).reshape(-1).numel()
                   for spec in (*self._unknown.values(), *self._known.values())
                   if not (isinstance(spec, (tuple, list)) and len(spec) == 2)}
        lengths.discard(1)
        if len(lengths) > 1:
            raise ValueError(f"properties given as values disagree on length: {sorted(lengths)}")
        return int(lengths.pop()) if lengths else None

    def _fit_arrays(self, parameters: torch.Tensor) -> None:
        """The start: the median of the drawn parameters, or ``initial``,
        strictly inside each bound (``_nlls.py:133-209``)."""
        names = self.unknown or UNKNOWN
        stray = {n for given in (self.bounds, self.initial) for n in given} - set(names)
        if stray:
            raise ValueError(f"bounds or initial name {sorted(stray)}, which "
                             f"{'is' if len(stray) == 1 else 'are'} not being estimated")
        if self.acquisition is None:
            raise RuntimeError("no model to fit; give this estimator the acquisition it is "
                               "inverting when it is made")
        drawn = torch.as_tensor(parameters).reshape(-1, len(names))
        median = drawn.to(torch.float32).median(dim=0).values
        start = []
        for k, name in enumerate(names):
            stated = name in self.initial
            value = float(self.initial[name]) if stated else float(median[k])
            low, high = bound_of(self.bounds, name)
            if (low is not None and value <= low) or (high is not None and value >= high):
                whose = "the starting value" if stated else "the median of the training range"
                raise ValueError(f"{name}: {whose}, {value:g}, is not strictly inside its "
                                 f"bound ({low}, {high})")
            start.append(value)
        self._start = torch.tensor(start, dtype=torch.float32)

    def _operator(self, known: torch.Tensor | None) -> ModelOperator:
        acquisition = self.acquisition
        if known is not None:
            acquisition = acquisition.bind(
                **{name: known[:, k] for k, name in enumerate(self.known)})
        return ModelOperator(acquisition, *(self.unknown or UNKNOWN), bounds=self.bounds,
                             amplitude=False)

    def _known_matrix(self, given: Any, voxels: int, device) -> torch.Tensor | None:
        if not self._known:
            return None
        if given is None:
            raise ValueError(f"this estimator needs {sorted(self._known)} measured")
        if isinstance(given, torch.Tensor):
            return given.reshape(voxels, len(self._known)).to(device, torch.float32)
        columns = []
        for name in self._known:
            if name not in given:
                raise ValueError(f"{name} is measured separately and must be given")
            value = torch.as_tensor(given[name], dtype=torch.float32).to(device).reshape(-1)
            if value.numel() == 1:
                value = value.expand(voxels)
            if value.numel() != voxels:
                raise ValueError(f"{name}: {value.numel()} values for {voxels} voxels")
            columns.append(value)
        return torch.stack(columns, dim=-1)

    def map(self, volume: Any, known: Any = None, *, uncertainty: bool = False) -> Any:
        """One map per unknown, shaped like ``volume`` ``(..., contrasts)``
        without its contrast axis, on the volume's device; with
        ``uncertainty=True`` also the standard deviation the noise told to
        :meth:`fit` leaves on each (the inverse Fisher information at the
        answer, ``_nlls.py:238-283``). Fitted from bare arrays (no names),
        the parameter columns come back as one tensor."""
        if not self.fitted:
            raise RuntimeError("the estimator has no starting point; call fit() first")
        signals = torch.as_tensor(volume)
        home = signals.device
        device = engine.require_cuda(home if home.type == "cuda" else None)
        shape = signals.shape[:-1]
        voxels = math.prod(shape) if shape else 1
        measured = signals.reshape(voxels, signals.shape[-1]).to(device, torch.complex64)
        columns = self._known_matrix(known, voxels, device)
        operator = self._operator(columns)
        names = operator.unknown
        start = operator.initial((voxels,), **{n: float(self._start[k])
                                               for k, n in enumerate(names)}).to(device)
        found = self.loop.minimize(operator, measured, start)
        self.iterations, self.unconverged = found.iterations, found.unconverged
        maps = operator.split(found.x)
        values = torch.stack([maps[n] for n in names], dim=-1)

        def laid_out(matrix):
            if not self._unknown:
                return matrix.reshape(*shape, len(names)).to(home)
            return {n: matrix[..., k].reshape(shape).to(home) for k, n in enumerate(names)}

        if not uncertainty:
            return laid_out(values)
        return laid_out(values), laid_out(self._spread(operator, values))

    forward = map

    def uncertainty_of(self, volume: Any, known: Any = None) -> Any:
        return self.map(volume, known, uncertainty=True)[1]

    def _spread(self, operator: ModelOperator, values: torch.Tensor) -> torch.Tensor:
        """sqrt of the Cramer-Rao diagonal of the fit's own sensitivity at the
        answer, the Jacobian divided by the noise standard deviation (per
        voxel or one number); zeros without noise."""
        from .design import crlb

        scale = torch.as_tensor(self.noise_std, dtype=torch.float32, device=values.device)
        if not bool(torch.any(scale != 0)):
            return torch.zeros_like(values)
        names = operator.unknown
        _, sensitivity = operator.acquisition.jacobian(
            list(names), **{n: values[..., k] for k, n in enumerate(names)})
        sensitivity = sensitivity / scale.reshape(*scale.shape,
                                                  *((1,) * (sensitivity.ndim - scale.ndim)))
        return crlb(sensitivity, noise_variance=1.0, singular="infinite").clamp_min(0.0).sqrt()


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
    def minimize_program(self, program: Program, measured: torch.Tensor, start: torch.Tensor,
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
                        damping=torch.zeros(0, dtype=torch.float64, device=device),
                        iterations=int(steps.max().item()) if V else 0,
                        unconverged=int(limited.sum().item()), steps=steps)
