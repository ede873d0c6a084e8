"""CPU restatement of the voxel-wise Gauss-Newton mapping loop.

TEST INFRASTRUCTURE and the CPU baseline of the mapping workload: only the
tests and bench.py's CPU legs use this file; nothing in the package imports
it.

The loop is the reference's Levenberg-Marquardt under a TrustRegion
(``recon/_gauss_newton.py:475-631``; the damping policy ``:366-415``: the
first damping ``tau`` times the largest curvature at the start, Nielsen's
``max(1/3, 1 - (2 gain - 1)^3)`` after an accepted step, a factor that doubles
with every rejection in a row otherwise) over bounded variables
(``_bounds.py:77-199``: sigmoid for a two-sided bound, softplus for a one-sided
one). The model is the oracle's FP32 port of the reference's EPG kernels,
called as the reference's Jacobian calls them (``model/_signal.py:233-268``):
per iteration one forward pass and one tangent pass per EPG-dependent
unknown (T1, T2); the M0 column is the forward's own record. The damped step
``(J^T J + lambda I) d = -J^T r`` is solved in FP64 per voxel.

Unknowns are (T1, T2, M0); B1 is known per voxel. The signal model is the
public MRF signal, ``s = -m0 F+[0]`` on the real axis; ``measured`` is
complex.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import oracle as O

FIRST, LIVE, DONE = 0, 1, 2


def _sigmoid(u):
    return 1.0 / (1.0 + np.exp(-u))


def _softplus(u):
    return np.where(u > 30.0, u, np.log1p(np.exp(np.minimum(u, 30.0))))


def to_natural(u: np.ndarray, low: np.ndarray, high: np.ndarray) -> np.ndarray:
    """Natural values of free variables ``u`` (V, 3), FP64."""
    x = np.empty_like(u)
    for k in range(3):
        lo, hi = low[k], high[k]
        if np.isfinite(lo) and np.isfinite(hi):
            x[:, k] = lo + (hi - lo) * _sigmoid(u[:, k])
        elif np.isfinite(lo):
            x[:, k] = lo + _softplus(u[:, k])
        elif np.isfinite(hi):
            x[:, k] = hi - _softplus(-u[:, k])
        else:
            x[:, k] = u[:, k]
    return x


def to_free(x: np.ndarray, low: np.ndarray, high: np.ndarray) -> np.ndarray:
    """Free variables of natural values strictly inside their bounds."""
    u = np.empty_like(x, dtype=np.float64)
    for k in range(3):
        lo, hi = low[k], high[k]
        v = x[:, k].astype(np.float64)
        if np.isfinite(lo) and np.isfinite(hi):
            t = (v - lo) / (hi - lo)
            u[:, k] = np.log(t) - np.log1p(-t)
        elif np.isfinite(lo):
            u[:, k] = np.log(np.expm1(v - lo))
        elif np.isfinite(hi):
            u[:, k] = -np.log(np.expm1(hi - v))
        else:
            u[:, k] = v
    return u


def widen(u: np.ndarray, low: np.ndarray, high: np.ndarray) -> np.ndarray:
    """d natural / d free per variable (V, 3)."""
    w = np.empty_like(u)
    for k in range(3):
        lo, hi = low[k], high[k]
        if np.isfinite(lo) and np.isfinite(hi):
            s = _sigmoid(u[:, k])
            w[:, k] = (hi - lo) * s * (1.0 - s)
        elif np.isfinite(lo):
            w[:, k] = _sigmoid(u[:, k])
        elif np.isfinite(hi):
            w[:, k] = _sigmoid(-u[:, k])
        else:
            w[:, k] = 1.0
    return w


def normal_equations(events, measured: np.ndarray, x: np.ndarray, b1: np.ndarray | None,
                     states: int, threads: int = 1) -> np.ndarray:
    """Per voxel (V, 10): the cost sum |s - y|^2, then J^T J (upper triangle
    of the natural T1, T2, M0 columns of dv, v = m0 F+[0] = -s) and the sums
    dv (v + y), which equal J_s^T r for the public signal s = -v."""
    V = x.shape[0]
    t1 = x[:, 0].astype(np.float32)
    t2 = x[:, 1].astype(np.float32)
    m0 = x[:, 2].astype(np.float32)
    b1 = None if b1 is None else np.asarray(b1, np.float32)
    packed = O.Packed(t1_ms=t1, t2_ms=t2, duration_s=events.duration, kind=events.kind,
                      flip_rad=events.flip, action=events.action,
                      output_index=events.output_index, state_count=states, b1=b1)
    p0 = O.forward(packed, "f32", threads)                      # F+[0], m0 = 1
    ones = np.ones(V, np.float32)
    d1 = O.tangent(packed, "f32", threads, t1_ms=ones)          # dF+[0]/dT1
    d2 = O.tangent(packed, "f32", threads, t2_ms=ones)          # dF+[0]/dT2
    m = m0[:, None]
    v = (m * p0).astype(np.float64)
    j1 = (m * d1).astype(np.float64)
    j2 = (m * d2).astype(np.float64)
    j3 = p0.astype(np.float64)
    res = v + measured.real.astype(np.float64)
    out = np.empty((V, 10))
    out[:, 0] = (res * res).sum(1) + (measured.imag.astype(np.float64) ** 2).sum(1)
    out[:, 1] = (j1 * j1).sum(1)
    out[:, 2] = (j1 * j2).sum(1)
    out[:, 3] = (j1 * j3).sum(1)
    out[:, 4] = (j2 * j2).sum(1)
    out[:, 5] = (j2 * j3).sum(1)
    out[:, 6] = (j3 * j3).sum(1)
    out[:, 7] = (j1 * res).sum(1)
    out[:, 8] = (j2 * res).sum(1)
    out[:, 9] = (j3 * res).sum(1)
    return out


def _free_system(ne: np.ndarray, w: np.ndarray):
    A = np.empty((ne.shape[0], 3, 3))
    idx = {(0, 0): 1, (0, 1): 2, (0, 2): 3, (1, 1): 4, (1, 2): 5, (2, 2): 6}
    for (i, j), c in idx.items():
        A[:, i, j] = A[:, j, i] = w[:, i] * w[:, j] * ne[:, c]
    g = w * ne[:, 7:10]
    return A, g


def _damped_solve(M: np.ndarray, g: np.ndarray):
    """d with M d = -g for each symmetric 3x3 M by Cholesky; ok is False
    (and d NaN) where M is not positive definite."""
    with np.errstate(invalid="ignore", divide="ignore"):
        s0 = M[:, 0, 0]
        l00 = np.sqrt(s0)
        l10 = M[:, 1, 0] / l00
        l20 = M[:, 2, 0] / l00
        s1 = M[:, 1, 1] - l10 * l10
        l11 = np.sqrt(s1)
        l21 = (M[:, 2, 1] - l20 * l10) / l11
        s2 = M[:, 2, 2] - l20 * l20 - l21 * l21
        l22 = np.sqrt(s2)
        y0 = -g[:, 0] / l00
        y1 = (-g[:, 1] - l10 * y0) / l11
        y2 = (-g[:, 2] - l20 * y0 - l21 * y1) / l22
        d2 = y2 / l22
        d1 = (y1 - l21 * d2) / l11
        d0 = (y0 - l10 * d1 - l20 * d2) / l00
    d = np.stack([d0, d1, d2], axis=1)
    ok = ((s0 > 0) & (s1 > 0) & (s2 > 0) & np.isfinite(s0) & np.isfinite(s1) & np.isfinite(s2)
          & np.isfinite(d).all(1))
    d[~ok] = np.nan
    return d, ok


@dataclass
class Fit:
    x: np.ndarray          # natural (T1, T2, M0) per voxel, FP64
    cost: np.ndarray       # final cost per voxel
    steps: np.ndarray      # LM steps taken per voxel
    limited: np.ndarray    # True where the step limit stopped the voxel
    passes: int            # EPG passes (forward + tangents) run, over all voxels' chunks


def fit(events, measured: np.ndarray, start: np.ndarray, low, high, states: int,
        b1: np.ndarray | None = None, tau: float = 1e-2, gradient_tolerance: float = 1e-8,
        step_tolerance: float = 1e-8, max_iterations: int = 10, threads: int = 1) -> Fit:
    """Levenberg-Marquardt on every voxel of ``measured`` (V, P) complex from
    the natural ``start`` ((3,) or (V, 3)); evaluations run only on the voxels
    still moving."""
    low = np.asarray(low, np.float64)
    high = np.asarray(high, np.float64)
    V = measured.shape[0]
    u = to_free(np.broadcast_to(np.asarray(start, np.float64).reshape(-1, 3), (V, 3)).copy(),
                low, high)
    status = np.full(V, FIRST, np.int32)
    normal = np.zeros((V, 10))
    cost = np.zeros(V)
    damping = np.zeros(V)
    rising = np.full(V, 2.0)
    steps = np.zeros(V, np.int32)
    flags = np.zeros(V, np.int32)
    predicted = np.zeros(V)
    cand = u.copy()
    passes = 0
    for _ in range(max_iterations + 1):
        live = np.flatnonzero(status != DONE)
        if live.size == 0:
            break
        # Step (gn_step): flat gradient -> done; else the damped step.
        moving = live[status[live] == LIVE]
        cand[live] = u[live]
        if moving.size:
            A, g = _free_system(normal[moving], widen(u[moving], low, high))
            flat = np.abs(g).max(1) < gradient_tolerance
            status[moving[flat]] = DONE
            keep = ~flat
            moving, A, g = moving[keep], A[keep], g[keep]
            lam = damping[moving]
            d, ok = _damped_solve(A + lam[:, None, None] * np.eye(3), g)
            pred = (d * (lam[:, None] * d - g)).sum(1)
            walked = np.sqrt((d * d).sum(1))
            norm_u = np.sqrt((u[moving] ** 2).sum(1))
            f = np.where(ok, 0, 2)
            f = f | np.where(ok & (walked < step_tolerance * (norm_u + step_tolerance)), 1, 0)
            predicted[moving] = pred
            flags[moving] = f
            cand[moving] = u[moving] + d
        live = np.flatnonzero(status != DONE)
        if live.size == 0:
            break
        # Evaluate at the candidates (the fused sweep's normal equations).
        x = to_natural(cand[live], low, high)
        trial = normal_equations(events, measured[live], x,
                                 None if b1 is None else b1[live], states, threads)
        passes += 3
        # Judge (gn_judge).
        first = status[live] == FIRST
        fl = live[first]
        if fl.size:
            normal[fl] = trial[first]
            cost[fl] = trial[first, 0]
            A, _ = _free_system(normal[fl], widen(u[fl], low, high))
            damping[fl] = tau * np.max(np.diagonal(A, axis1=1, axis2=2), axis=1)
            rising[fl] = 2.0
            steps[fl] = 0
            status[fl] = LIVE
        jl = live[~first]
        if jl.size:
            tr = trial[~first]
            singular = (flags[jl] & 2) != 0
            short = (flags[jl] & 1) != 0
            pred = predicted[jl]
            with np.errstate(invalid="ignore", divide="ignore"):
                gain = np.where(pred > 0.0,
                                (cost[jl] - tr[:, 0]) / np.maximum(pred, 1.1754943508222875e-38),
                                0.0)
            better = (gain > 0.0) & ~singular
            lam = damping[jl]
            q = 2.0 * gain - 1.0
            lowered = lam * np.maximum(1.0 - q * q * q, 1.0 / 3.0)
            damping[jl] = np.where(better, lowered, lam * rising[jl])
            rising[jl] = np.where(better, 2.0, rising[jl] * 2.0)
            acc = jl[better]
            u[acc] = cand[acc]
            normal[acc] = tr[better]
            cost[acc] = tr[better, 0]
            it = steps[jl] + 1
            steps[jl] = it
            stop_short = short & ~singular
            status[jl[stop_short]] = DONE
            at_limit = ~stop_short & (it >= max_iterations)
            status[jl[at_limit]] = DONE
            flags[jl[at_limit]] |= 4
    return Fit(x=to_natural(u, low, high), cost=cost, steps=steps, limited=(flags & 4) != 0,
               passes=passes)
