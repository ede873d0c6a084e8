"""Sequence design: gradient descent on a user cost through the EPG adjoint.

The interface follows the reference's ``optim/_design.py``: a cost function of
named sequence parameters, each optionally held between limits
(:class:`Bounded`, ``optim/_design.py:50-67``), minimised by Adam
(``SequenceDesign.minimize``, ``optim/_design.py:142-194``) and reported as a
:class:`SequenceOptimization` (``optim/_design.py:70-82``). Limits are exact:
the optimiser moves an unconstrained variable ``u`` and the cost sees
``lower + (upper - lower) * sigmoid(u)`` (``optim/_design.py:263-278``).

The gradient of a cost that simulates through :func:`torchsim_gb300.mrf_sim`
or a simulator's ``simulate`` comes from the adjoint kernel
(``engine.EpgFunction``): one forward sweep that stores the trajectory (or a
checkpoint every few pulses), one reverse sweep. A cost that differentiates a
Jacobian (a Cramer-Rao bound from :func:`crlb`) backs through the
second-order sweep (``engine.JacobianFunction``): one forward of the signal
and its tangents that stores their trajectory, one reverse sweep over all the
Jacobian's columns, where the reference pays one forward-over-reverse pass per
column (``sequence/_accelerators.py:1780-1800``).
"""

from __future__ import annotations

from collections.abc import Callable
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

__all__ = ["Bounded", "SequenceDesign", "SequenceOptimization", "crlb"]

# Fractions are kept this far from 0 and 1 before the logit, so a start on a
# limit maps to a finite variable (optim/_design.py:271).
_EDGE = 1e-6


@dataclass(frozen=True)
class Bounded:
    """A starting value and the closed range ``[lower, upper]`` it may take
    (scalars or per-element arrays)."""

    initial: Any
    lower: Any
    upper: Any


@dataclass(frozen=True)
class SequenceOptimization:
    """``parameters``: the designed values after the last step (inside their
    limits); ``loss``: the cost evaluated at every step, in order."""

    parameters: dict[str, torch.Tensor]
    loss: torch.Tensor


def _tensor(value: Any) -> torch.Tensor:
    if isinstance(value, torch.Tensor):
        return value.detach()
    array = np.asarray(value)
    if array.dtype.kind in "iub":
        array = array.astype(np.float32)
    return torch.from_numpy(np.array(array, copy=True))


class _Limits:
    """The map between a bounded value and its unconstrained variable."""

    def __init__(self, lower: Any, upper: Any, like: torch.Tensor) -> None:
        self.lower = torch.as_tensor(lower, dtype=like.dtype, device=like.device)
        self.upper = torch.as_tensor(upper, dtype=like.dtype, device=like.device)
        if bool(torch.any(self.lower >= self.upper)):
            raise ValueError("each lower limit must be below its upper limit")

    def free(self, value: torch.Tensor) -> torch.Tensor:
        fraction = (value - self.lower) / (self.upper - self.lower)
        return torch.logit(fraction.clamp(_EDGE, 1.0 - _EDGE))

    def bounded(self, free: torch.Tensor) -> torch.Tensor:
        return torch.addcmul(self.lower, self.upper - self.lower, torch.sigmoid(free))


class SequenceDesign(torch.nn.Module):
    """A cost and the parameters it is minimised over.

    ``cost(**values)`` returns one number; each keyword parameter is a
    :class:`Bounded` (moved inside its limits) or an array (moved freely).
    """

    def __init__(self, cost: Callable[..., torch.Tensor], **parameters: Any) -> None:
        super().__init__()
        if not parameters:
            raise ValueError("a design needs at least one parameter")
        self.cost = cost
        self._limits: dict[str, _Limits | None] = {}
        free: dict[str, torch.nn.Parameter] = {}
        for name, entry in parameters.items():
            start = _tensor(entry.initial if isinstance(entry, Bounded) else entry)
            limits = _Limits(entry.lower, entry.upper, start) if isinstance(entry, Bounded) else None
            self._limits[name] = limits
            variable = limits.free(start) if limits is not None else start.clone()
            free[name] = torch.nn.Parameter(variable.clone())
        self.raw = torch.nn.ParameterDict(free)

    def values(self) -> dict[str, torch.Tensor]:
        """The parameters as the cost sees them (inside their limits)."""
        out = {}
        for name, variable in self.raw.items():
            limits = self._limits[name]
            out[name] = variable if limits is None else limits.bounded(variable)
        return out

    def forward(self) -> torch.Tensor:
        """The cost at the current parameters."""
        loss = self.cost(**self.values())
        if not isinstance(loss, torch.Tensor) or loss.numel() != 1:
            raise ValueError("a design cost must return one number")
        return loss

    def minimize(self, *, iterations: int = 200, learning_rate: float = 0.05,
                 optimizer_factory: Callable[[list[torch.nn.Parameter]], torch.optim.Optimizer]
                 | None = None,
                 callback: Callable[[int, dict[str, torch.Tensor], torch.Tensor], bool | None]
                 | None = None) -> SequenceOptimization:
        """Take ``iterations`` optimiser steps (Adam at ``learning_rate`` unless a
        factory is given). ``callback(step, values, loss)`` runs after each
        step with detached tensors; returning ``True`` stops early."""
        if iterations < 1 or learning_rate <= 0:
            raise ValueError("iterations and learning_rate must be positive")
        variables = list(self.raw.values())
        optimizer = (optimizer_factory(variables) if optimizer_factory is not None
                     else torch.optim.Adam(variables, lr=learning_rate))
        losses = []
        for step in range(iterations):
            optimizer.zero_grad(set_to_none=True)
            loss = self()
            loss.backward()
            optimizer.step()
            losses.append(loss.detach().reshape(()))
            if callback is not None:
                current = {k: v.detach() for k, v in self.values().items()}
                if callback(step, current, losses[-1]):
                    break
        final = {k: v.detach() for k, v in self.values().items()}
        return SequenceOptimization(parameters=final, loss=torch.stack(losses))


def crlb(jacobian: torch.Tensor, *, noise_variance: float = 1.0,
         singular: str = "raise") -> torch.Tensor:
    """Diagonal of the inverse Fisher information, ``(..., parameters)``.

    ``jacobian`` is ``(..., parameters, samples)``; for complex input the real
    and imaginary channels count as independent measurements
    (``optim/_design.py:196-256``). ``singular="raise"`` raises
    ``torch.linalg.LinAlgError`` for an unidentifiable set of parameters;
    ``"infinite"`` returns ``inf`` for those entries instead.
    """
    if jacobian.ndim < 2:
        raise ValueError("a Jacobian is (..., parameters, samples)")
    if singular not in ("raise", "infinite"):
        raise ValueError(f"singular is 'raise' or 'infinite', got {singular!r}")
    if torch.is_complex(jacobian):
        rows = torch.cat((jacobian.real, jacobian.imag), dim=-1)
    else:
        rows = jacobian
    fisher = rows @ rows.transpose(-1, -2)
    if singular == "raise":
        return noise_variance * torch.diagonal(torch.linalg.inv(fisher), dim1=-2, dim2=-1)
    inverse, info = torch.linalg.inv_ex(fisher)
    bound = noise_variance * torch.diagonal(inverse, dim1=-2, dim2=-1)
    return bound.masked_fill((info != 0).unsqueeze(-1).expand_as(bound), float("inf"))

