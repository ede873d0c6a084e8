"""Event streams for the sequences on the accelerated path, packed as the
reference packs them, and compiled into device pulse programs.

The packed layout is the reference's kernel ABI
(``src/torchsim/sequence/_accelerators.py:_pack_events``, 913-1170): per event
a ``duration`` (seconds since the previous event, read off a clock by one
difference), a ``kind`` (0 wait, 1 RF, 2 ADC), a ``flip`` and ``phase`` in
radians, an ``action`` bit word and an ``output_index`` (-1 if not recorded).

The builders below lay out the same events, in the same order and with the
same clock arithmetic, as the reference's simulators:

* :func:`mrf_events` — ``MRFSimulator.layout`` (``simulators/mrf.py:46-77``):
  an inversion, then per repetition an excitation and an SSFP-FID readout
  (sample, unbalanced gradient, delay of TR), the last playing recorded.
* :func:`fse_events` — ``FSESimulator._train`` (``simulators/fse.py:75-104``):
  an excitation, then per echo a crushed refocusing pulse at (j - 1/2) ESP
  and a sample at j ESP.
"""

from __future__ import annotations

import hashlib
import math
import threading
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import torch

from . import _native

# The packed action word (sequence/_accelerators.py:77-84).
PRE_SHIFT = 1
POST_SHIFT = 2
INVERSION = 4
SPOIL_AFTER = 8
SHIFT_AFTER = 16
RECORD = 32
EXCITATION = 64
REFOCUSING = 128

WAIT, RF, ADC = 0, 1, 2

# The time integral of the reference's default hard-pulse envelope on its
# 1 us raster (``RfDefinition.integral``, sequence/_description.py:463-510).
# A pulse's flip is stored as an amplitude and read back as
# 2*pi*|amplitude*area| in float32 (``flip_angle``, :542-568), which is what
# puts its last bit where the reference has it.
_HARD_PULSE_AREA = 0.15915493667125702


def _played_flip(angles: torch.Tensor) -> np.ndarray:
    amplitude = angles.to(torch.float32)
    return (2.0 * torch.pi * torch.abs(amplitude * _HARD_PULSE_AREA)).numpy()


@dataclass
class PackedEvents:
    """One event stream in the reference's packed layout (NumPy, host)."""

    duration: np.ndarray  # float32 (trains, events)
    kind: np.ndarray  # int32 (events,)
    flip: np.ndarray  # float32 (trains, events)
    phase: np.ndarray  # float32 (trains, events)
    action: np.ndarray  # uint8 (events,)
    output_index: np.ndarray  # int32 (events,)
    time_us: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    # Labels of the recorded samples: the playing each belongs to (builders
    # record only the last of `repetitions`), and whether it is a spin echo.
    repetitions: int = 1
    echo: np.ndarray | None = None  # bool (outputs,)

    def sample_events(self) -> np.ndarray:
        """Index of the event that records each sample, (outputs,) int64."""
        where = np.flatnonzero(self.output_index >= 0)
        order = np.argsort(self.output_index[where], kind="stable")
        return where[order].astype(np.int64)

    @property
    def trains(self) -> int:
        return int(self.duration.shape[0])

    @property
    def events(self) -> int:
        return int(self.kind.shape[0])

    @property
    def outputs(self) -> int:
        recorded = self.output_index[self.output_index >= 0]
        return int(recorded.max()) + 1 if recorded.size else 0

    def key(self, with_phase: bool = False) -> str:
        h = hashlib.sha1()
        arrays = (self.duration, self.kind, self.flip, self.action, self.output_index)
        for a in (*arrays, self.phase) if with_phase else arrays:
            h.update(np.ascontiguousarray(a).tobytes())
            h.update(str(a.shape).encode())
        return h.hexdigest()

    def real_axis(self, tol: float = 0.0) -> int:
        """1 when the stream stays in the real subspace, else -1.

        The real subspace holds when every non-inversion RF pulse and every
        recorded sample share one phase (the kernel records i*m0*F+[0] in
        that frame), which is the condition the reference's real kernels
        assume (src/torchsim/_epg_cpu.cpp:3031-3039).
        """
        turning = (self.kind == RF) & ((self.action & INVERSION) == 0)
        sampled = (self.kind == ADC) & ((self.action & RECORD) != 0)
        phases = np.concatenate([self.phase[:, turning].ravel(), self.phase[:, sampled].ravel()])
        if phases.size == 0:
            return 1
        return 1 if np.all(np.abs(phases - phases[0]) <= tol) else -1


def _clock_to_durations(clock: torch.Tensor) -> np.ndarray:
    """Intervals as the reference reads them off its clock: one difference,
    scaled to seconds, narrowed to float32 (_accelerators.py:1125-1128)."""
    intervals = (torch.diff(clock, prepend=clock.new_zeros(1)) * 1e-6).to(torch.float32)
    return intervals.numpy()


def _as_tensor(value: Any) -> torch.Tensor:
    if isinstance(value, torch.Tensor):
        return value.detach().cpu()
    return torch.as_tensor(np.asarray(value) if not isinstance(value, (int, float)) else value)


def _matched(value: Any, reference: torch.Tensor) -> torch.Tensor:
    held = _as_tensor(value).to(reference.dtype)
    if held.numel() == 1:
        return held.reshape(()).expand(reference.shape)
    if held.shape != reference.shape:
        raise ValueError(
            f"expected one value per event or a single one, got {tuple(held.shape)} "
            f"against {tuple(reference.shape)}"
        )
    return held


def mrf_events(flip_deg: Any, TR_ms: Any, TI_ms: Any = 0.0, phases_deg: Any = 0.0,
               repetitions: int = 1) -> PackedEvents:
    """The MRF train of ``MRFSimulator.layout`` (simulators/mrf.py:46-77).

    Per repetition: an ideal inversion (held TI), then for each flip an
    excitation followed by a sample, one unbalanced gradient and the rest of
    the TR. Only the last playing is recorded (``_pack_events``'s
    ``repetitions``).
    """
    angles = torch.deg2rad(torch.atleast_1d(_as_tensor(flip_deg)))
    if angles.ndim != 1:
        raise ValueError("flip must be one angle per repetition")
    turns = torch.deg2rad(_matched(phases_deg, angles))
    spacing_s = _matched(TR_ms, angles) * 1e-3
    n = int(angles.numel())
    if n == 0:
        raise ValueError("an MRF train needs at least one pulse")
    per_rep = 1 + 4 * n
    clock_t = _mrf_clock(spacing_s, TI_ms, n, repetitions)
    kind = np.zeros(per_rep, np.int32)
    action = np.zeros(per_rep, np.uint8)
    flip = np.zeros(per_rep, np.float32)
    phase = np.zeros(per_rep, np.float32)
    kind[0] = RF
    action[0] = INVERSION
    a32 = _played_flip(angles)
    p32 = turns.to(torch.float32).numpy()
    exc = 1 + 4 * np.arange(n)
    kind[exc] = RF
    action[exc] = EXCITATION
    flip[exc] = a32
    phase[exc] = p32
    kind[exc + 1] = ADC
    phase[exc + 1] = p32
    action[exc + 2] = POST_SHIFT
    kind_all = np.tile(kind, repetitions)
    action_all = np.tile(action, repetitions)
    flip_all = np.tile(flip, repetitions)
    phase_all = np.tile(phase, repetitions)
    output_index = np.full(per_rep * repetitions, -1, np.int32)
    last = (repetitions - 1) * per_rep
    output_index[last + exc + 1] = np.arange(n, dtype=np.int32)
    action_all[last + exc + 1] |= RECORD
    duration = _clock_to_durations(clock_t)
    recorded = output_index >= 0
    return PackedEvents(
        duration=duration[None, :].copy(),
        kind=kind_all,
        flip=flip_all[None, :].copy(),
        phase=phase_all[None, :].copy(),
        action=action_all,
        output_index=output_index,
        time_us=clock_t.to(torch.float32).numpy()[recorded],
        repetitions=repetitions,
        echo=np.zeros(n, bool),
    )


def _mrf_clock(spacing_s: torch.Tensor, TI_ms: Any, n: int, repetitions: int) -> torch.Tensor:
    """Event times (us) of the MRF train, as compose() walks them.

    The inversion sits at 0; repetition k's pulses start at the cursor, which
    begins at TI and advances by each TR in turn; a later playing is offset
    by the whole train's length. The arithmetic is the reference's, in the
    precision it has there: the TRs are float32 seconds, so every cursor step
    after the first is a float32 addition (a sequential float32 prefix sum
    here), the first start keeps TI's own precision, and times are float32
    products by 1e6 (``simulators/mrf.py:46-77``, ``_accelerators.py:1125``).
    """
    s32 = spacing_s.detach().to(torch.float32).cpu().numpy()
    if isinstance(TI_ms, (int, float)):
        ti = float(TI_ms) * 1e-3
        first_stamp = np.float32(1e6 * ti)  # a Python float, rounded once
        c0 = np.float32(ti)
    else:
        ti_t = _as_tensor(TI_ms) * 1e-3
        c0 = np.float32(ti_t.to(torch.float32).item())
        first_stamp = np.float32(np.float32(1e6) * c0)
    # cursor[k] = start of pulse k; cursor[n] = the train's length.
    cursor = np.cumsum(np.concatenate([np.float32([c0]), s32]), dtype=np.float32)
    starts = np.float32(1e6) * cursor[:n]
    starts[0] = first_stamp
    stamps = np.concatenate([np.float32([0.0]), np.repeat(starts, 4)])
    if n == 1 and repetitions == 1 and isinstance(TI_ms, (int, float)):
        # No float32 value reaches the clock: it stays in double.
        return torch.tensor([0.0] + [1e6 * ti] * 4, dtype=torch.float64)
    tr_us = np.float32(1e6) * cursor[n]
    clock = [stamps] + [np.float32(tr_us * np.float32(rep)) + stamps for rep in range(1, repetitions)]
    return torch.from_numpy(np.concatenate(clock).astype(np.float32))


def mrf_gradient_map(pulses: int, repetitions: int = 1) -> dict[str, np.ndarray]:
    """Where the MRF protocol's values land in the packed stream.

    ``flip``: (repetitions, pulses) event indices whose flip is pulse k's;
    ``tr``: (m, 2) pairs (event, k) whose duration is TR_k; ``ti``: events whose
    duration is TI. Read off the layout of :func:`mrf_events`: repetition
    ``r`` starts at ``r*(1+4n)`` with the inversion, pulse k's excitation is
    at ``1+4k`` and its duration is the previous TR (TI for the first); the
    inversion of a later repetition follows the last TR.
    """
    per_rep = 1 + 4 * pulses
    exc = 1 + 4 * np.arange(pulses)
    flip = np.stack([r * per_rep + exc for r in range(repetitions)])
    tr = [(r * per_rep + exc[k + 1], k) for r in range(repetitions) for k in range(pulses - 1)]
    tr += [(r * per_rep, pulses - 1) for r in range(1, repetitions)]
    ti = np.array([r * per_rep + exc[0] for r in range(repetitions)], np.int64)
    return {"flip": flip.astype(np.int64), "tr": np.array(tr, np.int64).reshape(-1, 2), "ti": ti}


def played_flip_torch(flip_deg: torch.Tensor) -> torch.Tensor:
    """The flip a pulse plays, differentiable: 2*pi*|deg2rad(flip)*area|."""
    return 2.0 * torch.pi * torch.abs(torch.deg2rad(flip_deg.to(torch.float32)) * _HARD_PULSE_AREA)


def fse_events(flip_deg: Any, ESP_ms: float, phases_deg: Any = 0.0, exc_flip: float = 90.0,
               exc_phase: float = 90.0) -> PackedEvents:
    """The refocused train of ``FSESimulator._train`` (simulators/fse.py:75-104)."""
    angles = torch.deg2rad(torch.atleast_1d(_as_tensor(flip_deg)))
    turns = torch.deg2rad(_matched(phases_deg, angles))
    if angles.ndim != 1:
        raise ValueError("flip must be one angle per echo")
    n = int(angles.numel())
    spacing_s = float(ESP_ms) * 1e-3
    events = 1 + 3 * n
    kind = np.zeros(events, np.int32)
    action = np.zeros(events, np.uint8)
    flip = np.zeros(events, np.float32)
    phase = np.zeros(events, np.float32)
    output_index = np.full(events, -1, np.int32)
    clock = [0.0]
    kind[0] = RF
    action[0] = EXCITATION
    flip[0] = _played_flip(torch.tensor([math.pi / 180.0 * exc_flip]))[0]
    phase[0] = np.float32(math.pi / 180.0 * exc_phase)
    a32 = _played_flip(angles)
    p32 = turns.to(torch.float32).numpy()
    for index in range(n):
        echo_s = (index + 1) * spacing_s
        base = 1 + 3 * index
        kind[base] = RF
        action[base] = REFOCUSING | PRE_SHIFT | POST_SHIFT
        flip[base] = a32[index]
        phase[base] = p32[index]
        kind[base + 1] = ADC
        action[base + 1] = RECORD
        phase[base + 1] = p32[index]
        output_index[base + 1] = index
        clock.extend([1e6 * (echo_s - 0.5 * spacing_s), 1e6 * echo_s, 1e6 * echo_s])
    clock_t = torch.tensor(clock, dtype=torch.float64)
    recorded = output_index >= 0
    return PackedEvents(
        duration=_clock_to_durations(clock_t)[None, :].copy(),
        kind=kind,
        flip=flip[None, :].copy(),
        phase=phase[None, :].copy(),
        action=action,
        output_index=output_index,
        time_us=clock_t.to(torch.float32).numpy()[recorded],
        echo=np.ones(n, bool),
    )


class Program:
    """A compiled pulse program resident on the current CUDA device.

    ``phased`` keeps each event's phase in the program (per op: the phase of
    its pulse and of its receiver), which the complex kernel needs."""

    def __init__(self, events: PackedEvents, unmerged: bool = False,
                 duration_tangent: np.ndarray | None = None, phased: bool = False) -> None:
        lib = _native.library()
        self.events = events
        self.phased = phased
        dur = np.ascontiguousarray(events.duration, np.float32)
        kind = np.ascontiguousarray(events.kind, np.int32)
        flip = np.ascontiguousarray(events.flip, np.float32)
        action = np.ascontiguousarray(events.action, np.uint8)
        oi = np.ascontiguousarray(events.output_index, np.int32)
        tangent = None if duration_tangent is None else np.ascontiguousarray(
            np.broadcast_to(duration_tangent, dur.shape), np.float32)
        handle = _native.ctypes.c_void_p()
        if phased:
            if unmerged or tangent is not None:
                raise ValueError("a phased program is compiled merged, without a duration tangent")
            phase = np.ascontiguousarray(np.broadcast_to(events.phase, dur.shape), np.float32)
            _native.check(lib.tsg_program_create_phased(
                dur.ctypes.data, kind.ctypes.data, flip.ctypes.data, phase.ctypes.data,
                action.ctypes.data, oi.ctypes.data, events.trains, events.events,
                _native.ctypes.byref(handle)))
        else:
            _native.check(lib.tsg_program_create(
                dur.ctypes.data, kind.ctypes.data, flip.ctypes.data, action.ctypes.data,
                oi.ctypes.data, events.trains, events.events, int(unmerged),
                None if tangent is None else tangent.ctypes.data, _native.ctypes.byref(handle)))
        self.handle = handle
        i64 = _native.ctypes.c_int64
        trains, ops, outputs, nev = i64(), i64(), i64(), i64()
        _native.check(lib.tsg_program_info(handle, _native.ctypes.byref(trains),
                                           _native.ctypes.byref(ops), _native.ctypes.byref(outputs),
                                           _native.ctypes.byref(nev)))
        self.trains = trains.value
        self.ops = ops.value
        self.outputs = outputs.value

    def __del__(self) -> None:
        handle = getattr(self, "handle", None)
        if handle is not None and handle.value:
            try:
                _native.library().tsg_program_destroy(handle)
            except Exception:  # pragma: no cover - interpreter shutdown
                pass
            self.handle = None


_cache: dict[tuple, Program] = {}
_cache_lock = threading.Lock()


def program_for(events: PackedEvents, device: torch.device | None = None,
                phased: bool = False) -> Program:
    """The compiled program of a stream, cached by content and device
    (``phased``: with the event phases, for the complex kernel)."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    key = (events.key(phased), device.index, phased)
    with _cache_lock:
        hit = _cache.get(key)
        if hit is None:
            with torch.cuda.device(device):
                hit = Program(events, phased=phased)
            if len(_cache) > 64:
                _cache.pop(next(iter(_cache)))
            _cache[key] = hit
    return hit


# ---- programs rebound on the device ------------------------------------------


class ProgramView:
    """A pulse program whose op values live in a device tensor rebound from
    device-resident event values (``tsg_program_rebind``), sharing its
    template's structure and event source map (``tsg_program_view``). It
    stands wherever a :class:`Program` does and keeps the template and the
    op array alive."""

    def __init__(self, template: Program, ops: torch.Tensor) -> None:
        handle = _native.ctypes.c_void_p()
        _native.check(_native.library().tsg_program_view(template.handle, ops.data_ptr(),
                                                          _native.ctypes.byref(handle)))
        self.handle = handle
        self.template = template
        self.ops_buffer = ops
        self.events = template.events
        self.phased = False
        self.trains = template.trains
        self.ops = template.ops
        self.outputs = template.outputs

    def __del__(self) -> None:
        handle = getattr(self, "handle", None)
        if handle is not None and handle.value:
            try:
                _native.library().tsg_program_destroy(handle)
            except Exception:  # pragma: no cover - interpreter shutdown
                pass
            self.handle = None


def rebind(template: Program, duration: torch.Tensor, flip: torch.Tensor) -> ProgramView:
    """``template`` with every op's dt and flip taken from the device event
    buffers ``duration`` (s) and ``flip`` (rad), ``(trains, events)`` float32,
    by one kernel on the current stream. ``duration`` must be zero wherever
    the template's events were (they are folded into the op before them)."""
    duration = duration.to(torch.float32).contiguous()
    flip = flip.to(torch.float32).contiguous()
    ops = torch.empty((max(template.trains * template.ops, 1), 4), dtype=torch.float32,
                      device=duration.device)
    _native.check(_native.library().tsg_program_rebind(
        template.handle, duration.data_ptr(), flip.data_ptr(), ops.data_ptr(),
        torch.cuda.current_stream(duration.device).cuda_stream))
    return ProgramView(template, ops)


def sequential_sum(x: torch.Tensor) -> torch.Tensor:
    """Running sums of a float32 device vector added left to right, one
    rounding per addition (``np.cumsum(..., dtype=float32)``), on the device."""
    x = x.to(torch.float32).contiguous()
    out = torch.empty_like(x)
    _native.check(_native.library().tsg_sequential_sum(
        x.data_ptr(), x.numel(), out.data_ptr(), torch.cuda.current_stream(x.device).cuda_stream))
    return out


_templates: dict[tuple, Program] = {}


def mrf_stream_on_device(flip_deg: torch.Tensor, TR_ms: Any, TI_ms: float,
                         device: torch.device) -> tuple[ProgramView, torch.Tensor, torch.Tensor]:
    """The MRF train of :func:`mrf_events` (one playing, TI a number, zero
    phases) built from device-resident flips and TRs without leaving the
    device: the played flips and the clock's intervals by the same float32
    arithmetic as the host builder (the cursor by :func:`sequential_sum`), and
    the program by rebinding a template compiled once per (pulses, TI) with
    :func:`rebind`. Returns ``(program, flip (1, events), duration (1,
    events))``, the last two the packed event buffers on the device."""
    angles = torch.deg2rad(torch.atleast_1d(flip_deg.detach()).to(device))
    if angles.ndim != 1:
        raise ValueError("flip must be one angle per repetition")
    n = int(angles.numel())
    if n < 2:
        raise ValueError("the device builder takes two pulses or more")
    if isinstance(TR_ms, torch.Tensor):
        tr = TR_ms.detach().to(device)
    elif isinstance(TR_ms, (int, float)):
        tr = torch.full((), float(TR_ms), dtype=torch.float32, device=device)
    else:
        tr = torch.as_tensor(np.asarray(TR_ms, np.float32)).to(device)
    tr = tr.to(angles.dtype)
    tr = tr.reshape(()).expand(n) if tr.numel() == 1 else tr
    if tr.shape != angles.shape:
        raise ValueError(f"expected one value per event or a single one, got {tuple(tr.shape)} "
                         f"against {tuple(angles.shape)}")
    s32 = (tr * 1e-3).to(torch.float32)
    ti = float(TI_ms) * 1e-3
    key = (n, ti, device.index)
    template = _templates.get(key)
    if template is None:
        template = program_for(mrf_events(np.full(n, 10.0, np.float32),
                                          np.full(n, 10.0, np.float32), TI_ms=float(TI_ms)),
                               device)
        _templates[key] = template
    start = torch.full((1,), float(np.float32(ti)), dtype=torch.float32, device=device)
    cursor = sequential_sum(torch.cat((start, s32)))
    starts = cursor[:n] * np.float32(1e6)
    starts[:1].fill_(float(np.float32(1e6 * ti)))  # a fill, not a host-to-device copy
    stamps = torch.cat((starts.new_zeros(1), starts.repeat_interleave(4)))
    duration = (torch.diff(stamps, prepend=stamps.new_zeros(1)) * 1e-6).to(torch.float32)
    played = (2.0 * torch.pi * torch.abs(angles.to(torch.float32) * _HARD_PULSE_AREA))
    flip = torch.zeros(1 + 4 * n, dtype=torch.float32, device=device)
    flip[1::4] = played
    program = rebind(template, duration[None], flip[None])
    return program, flip[None], duration[None]
