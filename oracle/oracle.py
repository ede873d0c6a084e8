"""ORACLE — test infrastructure only.

Python face of ``oracle/epg_oracle.c``: the CPU restatement of the
reference's real-subspace EPG recursion (src/torchsim/_epg_cpu.cpp:3010-3285,
5950-6232). Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg import this module; the product never does.

Every function takes the reference's packed buffers (the tissue properties
and the event stream, as ``sequence/_accelerators.py:_pack_events`` lays them
out) as NumPy arrays and returns NumPy arrays. ``precision`` picks the FP64
oracle (``"f64"``) or the FP32 port that keeps the reference's statement
order (``"f32"``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "_lib" / "libepg_oracle.so"


class _Case(ctypes.Structure):
    _fields_ = [
        ("t1_ms", ctypes.c_void_p),
        ("t2_ms", ctypes.c_void_p),
        ("m0", ctypes.c_void_p),
        ("b1", ctypes.c_void_p),
        ("inversion", ctypes.c_void_p),
        ("duration_s", ctypes.c_void_p),
        ("kind", ctypes.c_void_p),
        ("flip_rad", ctypes.c_void_p),
        ("action", ctypes.c_void_p),
        ("output_index", ctypes.c_void_p),
        ("atom_count", ctypes.c_int64),
        ("train_count", ctypes.c_int64),
        ("event_count", ctypes.c_int64),
        ("state_count", ctypes.c_int64),
        ("output_count", ctypes.c_int64),
    ]


class _Offaxis(ctypes.Structure):
    _fields_ = [
        ("phase_rad", ctypes.c_void_p),
        ("b1_phase_rad", ctypes.c_void_p),
        ("b0_hz", ctypes.c_void_p),
    ]


class _Direction(ctypes.Structure):
    _fields_ = [
        ("t1_ms", ctypes.c_void_p),
        ("t2_ms", ctypes.c_void_p),
        ("m0", ctypes.c_void_p),
        ("b1", ctypes.c_void_p),
        ("inversion", ctypes.c_void_p),
        ("duration_s", ctypes.c_void_p),
        ("flip_rad", ctypes.c_void_p),
    ]


_lib = None


def build() -> Path:
    """Compile the oracle library with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIBRARY


def _library() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIBRARY.exists():
            build()
        _lib = ctypes.CDLL(str(LIBRARY))
    return _lib


@dataclass
class Packed:
    """One run's packed inputs (the reference's buffer ABI, real subset)."""

    t1_ms: np.ndarray
    t2_ms: np.ndarray
    duration_s: np.ndarray  # (events,) or (trains, events)
    kind: np.ndarray
    flip_rad: np.ndarray  # (events,) or (trains, events)
    action: np.ndarray
    output_index: np.ndarray
    state_count: int
    m0: np.ndarray | None = None
    b1: np.ndarray | None = None
    inversion: np.ndarray | None = None
    # The complex path only: per-event RF / receiver phase ((events,) or
    # (trains, events)) and per-voxel transmit phase and off-resonance.
    phase_rad: np.ndarray | None = None
    b1_phase_rad: np.ndarray | None = None
    b0_hz: np.ndarray | None = None

    @property
    def atom_count(self) -> int:
        return int(np.asarray(self.t1_ms).size)

    @property
    def event_count(self) -> int:
        return int(np.asarray(self.kind).size)

    @property
    def train_count(self) -> int:
        d = np.asarray(self.duration_s)
        return 1 if d.ndim == 1 else int(d.shape[0])

    @property
    def output_count(self) -> int:
        oi = np.asarray(self.output_index)
        return int(oi.max()) + 1 if oi.size and oi.max() >= 0 else 0


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return None if a is None else a.ctypes.data


def _case(p: Packed, keep: list) -> _Case:
    arrays = {
        "t1_ms": _f32(p.t1_ms),
        "t2_ms": _f32(p.t2_ms),
        "m0": _f32(p.m0),
        "b1": _f32(p.b1),
        "inversion": _f32(p.inversion),
        "duration_s": _f32(np.broadcast_to(p.duration_s, (p.train_count, p.event_count))),
        "kind": np.ascontiguousarray(p.kind, dtype=np.int32),
        "flip_rad": _f32(np.broadcast_to(p.flip_rad, (p.train_count, p.event_count))),
        "action": np.ascontiguousarray(p.action, dtype=np.uint8),
        "output_index": np.ascontiguousarray(p.output_index, dtype=np.int32),
    }
    keep.append(arrays)
    c = _Case()
    for name, value in arrays.items():
        setattr(c, name, _ptr(value))
    c.atom_count = p.atom_count
    c.train_count = p.train_count
    c.event_count = p.event_count
    c.state_count = int(p.state_count)
    c.output_count = p.output_count
    return c


def _dtype(precision: str):
    if precision not in ("f64", "f32"):
        raise ValueError(f"precision must be 'f64' or 'f32', got {precision!r}")
    return (np.float64, ctypes.c_double) if precision == "f64" else (np.float32, ctypes.c_float)


def _shape(p: Packed):
    return (p.atom_count, p.output_count) if p.train_count == 1 else (
        p.train_count, p.atom_count, p.output_count)


def forward(p: Packed, precision: str = "f64", threads: int = 1) -> np.ndarray:
    """Recorded samples' imaginary plane, ``m0 * F+[0]`` (the real plane is 0).

    Follows ``simulate_real_range`` (src/torchsim/_epg_cpu.cpp:3041-3128).
    """
    dtype, _ = _dtype(precision)
    keep: list = []
    c = _case(p, keep)
    real = np.zeros(_shape(p), dtype=dtype)
    imag = np.zeros(_shape(p), dtype=dtype)
    fn = getattr(_library(), f"oracle_forward_{precision}")
    fn(ctypes.byref(c), ctypes.c_void_p(real.ctypes.data), ctypes.c_void_p(imag.ctypes.data),
       ctypes.c_int(threads))
    return imag


def forward_complex(p: Packed, precision: str = "f64", threads: int = 1) -> np.ndarray:
    """Recorded samples, complex: ``m0 * F+[0]`` demodulated by the receiver
    phase, on the complex path (``simulate_range<INSTANT, ONE>``,
    src/torchsim/_epg_cpu.cpp:4216-4566)."""
    dtype, _ = _dtype(precision)
    keep: list = []
    c = _case(p, keep)
    arrays = {
        "phase_rad": None if p.phase_rad is None else _f32(
            np.broadcast_to(p.phase_rad, (p.train_count, p.event_count))),
        "b1_phase_rad": _f32(p.b1_phase_rad),
        "b0_hz": _f32(p.b0_hz),
    }
    keep.append(arrays)
    o = _Offaxis()
    for name, value in arrays.items():
        setattr(o, name, _ptr(value))
    real = np.zeros(_shape(p), dtype=dtype)
    imag = np.zeros(_shape(p), dtype=dtype)
    fn = getattr(_library(), f"oracle_forward_complex_{precision}")
    fn(ctypes.byref(c), ctypes.byref(o), ctypes.c_void_p(real.ctypes.data),
       ctypes.c_void_p(imag.ctypes.data), ctypes.c_int(threads))
    return real + 1j * imag


def tangent(p: Packed, precision: str = "f64", threads: int = 1, lanes: bool | None = None,
            **direction) -> np.ndarray:
    """One forward-mode tangent of the recorded samples' imaginary plane.

    ``direction`` names any of ``t1_ms, t2_ms, m0, b1, inversion`` (per atom)
    and ``duration_s, flip_rad`` (per event or per train and event). Follows
    ``simulate_real_jvp_range`` (src/torchsim/_epg_cpu.cpp:3136-3285), or with
    ``lanes=True`` the eight-atom lane kernel (``simulate_real_jvp_atom_lane_range``,
    :3503-3695); the two round differently in FP32. ``lanes=None`` picks as the
    reference's dispatch does for the real subspace (:10957-10965): the lane
    kernel whenever the run has eight atoms or more. (The reference's train-lane
    kernel, for fewer than eight atoms but eight trains or more, is not restated;
    such runs take the per-atom kernel here.)
    """
    if lanes is None:
        lanes = p.atom_count >= 8
    dtype, _ = _dtype(precision)
    keep: list = []
    c = _case(p, keep)
    d = _Direction()
    shape = (p.train_count, p.event_count)
    for name in ("t1_ms", "t2_ms", "m0", "b1", "inversion", "duration_s", "flip_rad"):
        value = direction.pop(name, None)
        if value is None:
            continue
        if name in ("duration_s", "flip_rad"):
            value = np.broadcast_to(np.asarray(value, np.float32), shape)
        else:
            value = np.broadcast_to(np.asarray(value, np.float32), (p.atom_count,))
        value = _f32(value)
        keep.append(value)
        setattr(d, name, _ptr(value))
    if direction:
        raise ValueError(f"unknown tangent directions {sorted(direction)}")
    real = np.zeros(_shape(p), dtype=dtype)
    imag = np.zeros(_shape(p), dtype=dtype)
    fn = getattr(_library(), f"oracle_tangent{'_lanes' if lanes else ''}_{precision}")
    fn(ctypes.byref(c), ctypes.byref(d), ctypes.c_void_p(real.ctypes.data),
       ctypes.c_void_p(imag.ctypes.data), ctypes.c_int(threads))
    return imag


def adjoint(p: Packed, seed_imag: np.ndarray, precision: str = "f64") -> dict[str, np.ndarray]:
    """First-order adjoint for a seed on the imaginary output plane.

    Returns per-atom gradients ``t1_ms, t2_ms, m0, b1, inversion`` and per
    (train, event) gradients ``flip_rad, duration_s``. Follows
    ``simulate_real_vjp_range`` (src/torchsim/_epg_cpu.cpp:5985-6232).
    """
    dtype, _ = _dtype(precision)
    keep: list = []
    c = _case(p, keep)
    seed = _f32(np.broadcast_to(seed_imag, _shape(p)))
    grads = {n: np.zeros(p.atom_count, dtype=dtype) for n in ("t1_ms", "t2_ms", "m0", "b1", "inversion")}
    grads["flip_rad"] = np.zeros((p.train_count, p.event_count), dtype=dtype)
    grads["duration_s"] = np.zeros((p.train_count, p.event_count), dtype=dtype)
    fn = getattr(_library(), f"oracle_adjoint_{precision}")
    order = ("t1_ms", "t2_ms", "m0", "b1", "inversion", "flip_rad", "duration_s")
    fn(ctypes.byref(c), ctypes.c_void_p(seed.ctypes.data),
       *[ctypes.c_void_p(grads[n].ctypes.data) for n in order])
    if p.train_count == 1:
        grads["flip_rad"] = grads["flip_rad"][0]
        grads["duration_s"] = grads["duration_s"][0]
    return grads


COMPLEX_GRADIENTS = ("t1_ms", "t2_ms", "m0", "b1", "inversion", "b1_phase_rad", "b0_hz",
                     "flip_rad", "duration_s", "phase_rad")


def adjoint_complex(p: Packed, seed: np.ndarray, precision: str = "f64") -> dict[str, np.ndarray]:
    """First-order adjoint of the complex path for a complex seed (the
    cotangent of both output planes): gradients keyed as
    :data:`COMPLEX_GRADIENTS`, per atom or per (train, event). Follows the
    single-pool instant-RF case of ``simulate_vjp_range``
    (src/torchsim/_epg_cpu.cpp:4840-5985)."""
    dtype, _ = _dtype(precision)
    keep: list = []
    c = _case(p, keep)
    arrays = {
        "phase_rad": None if p.phase_rad is None else _f32(
            np.broadcast_to(p.phase_rad, (p.train_count, p.event_count))),
        "b1_phase_rad": _f32(p.b1_phase_rad),
        "b0_hz": _f32(p.b0_hz),
    }
    keep.append(arrays)
    o = _Offaxis()
    for name, value in arrays.items():
        setattr(o, name, _ptr(value))
    sd = np.broadcast_to(np.asarray(seed, np.complex64), _shape(p))
    sr, si = _f32(sd.real), _f32(sd.imag)
    g = {n: np.zeros(p.atom_count, dtype=dtype) for n in COMPLEX_GRADIENTS[:7]}
    for n in COMPLEX_GRADIENTS[7:]:
        g[n] = np.zeros((p.train_count, p.event_count), dtype=dtype)
    ptrs = (ctypes.c_void_p * 10)(*[g[n].ctypes.data for n in COMPLEX_GRADIENTS])
    fn = getattr(_library(), f"oracle_adjoint_complex_{precision}")
    fn(ctypes.byref(c), ctypes.byref(o), ctypes.c_void_p(sr.ctypes.data),
       ctypes.c_void_p(si.ctypes.data), ptrs)
    if p.train_count == 1:
        for n in COMPLEX_GRADIENTS[7:]:
            g[n] = g[n][0]
    return g


def _direction(p: Packed, direction: dict, keep: list) -> _Direction:
    d = _Direction()
    shape = (p.train_count, p.event_count)
    direction = dict(direction)
    for name in ("t1_ms", "t2_ms", "m0", "b1", "inversion", "duration_s", "flip_rad"):
        value = direction.pop(name, None)
        if value is None:
            continue
        if name in ("duration_s", "flip_rad"):
            value = np.broadcast_to(np.asarray(value, np.float32), shape)
        else:
            value = np.broadcast_to(np.asarray(value, np.float32), (p.atom_count,))
        value = _f32(value)
        keep.append(value)
        setattr(d, name, _ptr(value))
    if direction:
        raise ValueError(f"unknown tangent directions {sorted(direction)}")
    return d


SECOND_ORDER = ("t1_ms", "t2_ms", "m0", "b1", "inversion", "flip_rad", "duration_s")


def second(p: Packed, seed_imag: np.ndarray, precision: str = "f64",
           **direction) -> tuple[dict[str, np.ndarray], dict[str, np.ndarray]]:
    """Forward over reverse: the first-order adjoint for a seed on the
    imaginary output plane, differentiated along ``direction`` (names as
    :func:`tangent`). Returns ``(values, curvature)``: the gradient of
    ``<seed, J d>`` with respect to the direction (``J^T seed``) and with
    respect to the inputs, each keyed ``t1_ms, t2_ms, m0, b1, inversion``
    (per atom) and ``flip_rad, duration_s`` (per event, or per train and
    event). Follows ``simulate_real_vjp_jvp_range``
    (src/torchsim/_epg_cpu.cpp:7028-7330)."""
    dtype, _ = _dtype(precision)
    keep: list = []
    c = _case(p, keep)
    d = _direction(p, direction, keep)
    seed = _f32(np.broadcast_to(seed_imag, _shape(p)))
    sides = []
    for _ in range(2):
        g = {n: np.zeros(p.atom_count, dtype=dtype) for n in SECOND_ORDER[:5]}
        for n in SECOND_ORDER[5:]:
            g[n] = np.zeros((p.train_count, p.event_count), dtype=dtype)
        sides.append(g)
    ptrs = [(ctypes.c_void_p * 7)(*[side[n].ctypes.data for n in SECOND_ORDER])
            for side in sides]
    fn = getattr(_library(), f"oracle_second_{precision}")
    fn(ctypes.byref(c), ctypes.byref(d), ctypes.c_void_p(seed.ctypes.data), ptrs[0], ptrs[1])
    if p.train_count == 1:
        for side in sides:
            for n in SECOND_ORDER[5:]:
                side[n] = side[n][0]
    return sides[0], sides[1]


REFERENCE_DIR = HERE / "_ref"


def reference_module():
    """The reference's own compiled CPU kernel (``_epg_cpu``, built by
    ``oracle/build_ref.sh`` from the reference's sources into ``oracle/_ref``),
    or None where no build for this machine exists."""
    import importlib.util
    import sysconfig

    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    path = REFERENCE_DIR / f"_epg_cpu{suffix}"
    if not path.exists():
        return None
    try:
        spec = importlib.util.spec_from_file_location("_epg_cpu", path)
        module = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(module)
    except (ImportError, OSError):
        return None
    return module


# The reference's feature mask (_epg_cpu.cpp:95-100): which optional tissue
# maps a call declares; an undeclared map reads as its identity.
_TRANSMIT, _DENSITY, _INVERTING = 1 << 3, 1 << 4, 1 << 5


def _reference_call(p: Packed, keep: list, threads: int):
    """The 17 tissue and 9 event pointers of ``_parameters.py``'s packed order,
    two output planes, and the scalar arguments of ``_epg_cpu.simulate``
    (``_epg_cpu.cpp:10740-10788``) for a single-pool instant-RF real-axis run."""
    A = p.atom_count
    E = p.event_count
    zeros = np.zeros(A, np.float32)
    ones = np.ones(A, np.float32)
    features = 0
    tissue = [_f32(p.t1_ms), _f32(p.t2_ms)]
    for value, bit in ((p.m0, _DENSITY), (p.b1, _TRANSMIT)):
        tissue.append(ones if value is None else _f32(value))
        features |= 0 if value is None else bit
    tissue += [zeros, zeros]  # B1 phase, B0: the real axis
    tissue.append(ones if p.inversion is None else _f32(p.inversion))
    features |= 0 if p.inversion is None else _INVERTING
    tissue += [zeros] * 10  # diffusion, flow and pools: absent
    shape = (p.train_count, E)
    events = [_f32(np.broadcast_to(p.duration_s, shape)), np.ascontiguousarray(p.kind, np.int32),
              _f32(np.broadcast_to(p.flip_rad, shape)), np.zeros(shape, np.float32),
              np.ascontiguousarray(p.action, np.uint8),
              np.ascontiguousarray(p.output_index, np.int32), np.zeros(E, np.int32),
              np.zeros(E, np.float32), np.zeros(E, np.float32)]
    keep += tissue + events
    scalars = (A, p.train_count, E, int(p.state_count), p.output_count, threads, 1, 0.0, 0.0,
               1, 1, 0, 1.0, 0, 1.0, 0, features, 0, 0, 0)
    return tissue, events, scalars


def reference_forward(ref, p: Packed, threads: int = 1) -> np.ndarray:
    """The imaginary output plane of the reference's ``simulate``."""
    keep: list = []
    tissue, events, scalars = _reference_call(p, keep, threads)
    real = np.zeros(_shape(p), np.float32)
    imag = np.zeros(_shape(p), np.float32)
    ref.simulate([a.ctypes.data for a in (*tissue, *events, real, imag)] + [0] * 13, *scalars)
    return imag


def reference_jvp(ref, p: Packed, column: int, threads: int = 1) -> np.ndarray:
    """The imaginary tangent plane of the reference's ``simulate_jvp``
    (``_epg_cpu.cpp:11017-11148``) along one tissue property, a one-hot
    direction on tissue slot ``column`` (0 T1, 1 T2, 2 M0, 3 B1, 6 inversion)."""
    keep: list = []
    tissue, events, scalars = _reference_call(p, keep, threads)
    tangents = [np.zeros(p.atom_count, np.float32) for _ in range(17)]
    tangents[column] = np.ones(p.atom_count, np.float32)
    tangents += [np.zeros((p.train_count, p.event_count), np.float32) for _ in range(3)]
    keep += tangents
    real = np.zeros(_shape(p), np.float32)
    imag = np.zeros(_shape(p), np.float32)
    ref.simulate_jvp([a.ctypes.data for a in (*tissue, *events, *tangents, real, imag)]
                     + [0] * 13, *scalars)
    return imag


def cpu_threads() -> int:
    """Host cores this process may use."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
