"""Many sequences of uneven length and voxel count in ONE persistent launch.

The reference simulates one sequence description per call, one kernel launch
each (``sequence/_epg_triton.py:17120-17300``); a batch of CPMG protocols with
different echo-train lengths and voxel counts is as many launches, each sized
to its own problem, with a tail of idle SMs after every small one.
:class:`SequenceBatch` packs all of them into one table: the sequences'
compiled programs back to back, their tissue back to back, and a list of
(sequence, voxel tile) units sorted largest first. A single launch of the
persistent kernel (``tsg_epg_batched_forward``) works through the list; the
launch and the counter reset are captured once in a CUDA graph and replayed.
The launch shape (orders per lane, warps per CTA, CTAs per SM) is picked by
:mod:`torchsim_gb300.autotune`.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native, autotune, engine
from .sequence import PackedEvents, program_for

OP_DTYPE = np.dtype([("dt", "<f4"), ("flip", "<f4"), ("record", "<i4"), ("code", "<u4")])


def compile_ops(events: PackedEvents) -> np.ndarray:
    """The event stream's pulse program as a host array of 16-byte ops."""
    lib = _native.library()
    if events.trains != 1:
        raise ValueError("a batched sequence is a single train")
    dur = np.ascontiguousarray(events.duration, np.float32)
    kind = np.ascontiguousarray(events.kind, np.int32)
    flip = np.ascontiguousarray(events.flip, np.float32)
    action = np.ascontiguousarray(events.action, np.uint8)
    oi = np.ascontiguousarray(events.output_index, np.int32)
    n_ops, n_out = ctypes.c_int64(), ctypes.c_int64()
    args = (dur.ctypes.data, kind.ctypes.data, flip.ctypes.data, action.ctypes.data, oi.ctypes.data,
            1, events.events, 0, None, ctypes.byref(n_ops), ctypes.byref(n_out))
    _native.check(lib.tsg_program_plan(*args, None, None, None, None, 0))
    ops = np.zeros(n_ops.value, OP_DTYPE)
    dt = np.zeros(n_ops.value, np.float32)
    fl = np.zeros(n_ops.value, np.float32)
    rec = np.zeros(n_ops.value, np.int32)
    code = np.zeros(n_ops.value, np.uint32)
    _native.check(lib.tsg_program_plan(*args, dt.ctypes.data, fl.ctypes.data, rec.ctypes.data,
                                       code.ctypes.data, n_ops.value))
    ops["dt"], ops["flip"], ops["record"], ops["code"] = dt, fl, rec, code
    return ops


@dataclass
class BatchEntry:
    events: PackedEvents
    states: int
    t1: np.ndarray
    t2: np.ndarray
    b1: np.ndarray | None = None
    m0: np.ndarray | None = None

    @property
    def voxels(self) -> int:
        return int(np.asarray(self.t1).size)


class SequenceBatch:
    """A device-resident batch of sequences, run by one persistent launch."""

    def __init__(self, entries: list[BatchEntry], device: torch.device) -> None:
        if not entries:
            raise ValueError("empty batch")
        for e in entries:
            if e.events.real_axis() != 1:
                raise NotImplementedError("batched sequences must stay in the real subspace")
            if e.states < 1 or e.states > 256:
                raise ValueError("states must be 1..256")
        self.entries = entries
        self.device = device
        programs = [compile_ops(e.events) for e in entries]
        self.op_offset = np.cumsum([0] + [len(p) for p in programs])[:-1]
        self.op_count = np.array([len(p) for p in programs], np.int64)
        self.outputs = np.array([e.events.outputs for e in entries], np.int64)
        self.voxels = np.array([e.voxels for e in entries], np.int64)
        self.states = np.array([e.states for e in entries], np.int64)
        self.voxel_offset = np.cumsum([0] + list(self.voxels))[:-1]
        self.output_offset = np.cumsum([0] + list(self.voxels * self.outputs))[:-1]
        if int(self.op_offset[-1] + self.op_count[-1]) >= 2**31:
            raise ValueError("batch programs exceed 2^31 ops")
        ops = np.concatenate(programs)
        self.d_ops = torch.from_numpy(ops.view(np.uint8)).to(device)
        cat = lambda xs: torch.from_numpy(np.concatenate(xs).astype(np.float32)).to(device)  # noqa: E731
        self.t1 = cat([np.asarray(e.t1, np.float32) for e in entries]).clamp_min(
            engine.MINIMUM_RELAXATION_TIME_MS)
        self.t2 = cat([np.asarray(e.t2, np.float32) for e in entries]).clamp_min(
            engine.MINIMUM_RELAXATION_TIME_MS)
        has_b1 = any(e.b1 is not None for e in entries)
        has_m0 = any(e.m0 is not None for e in entries)
        self.b1 = cat([np.asarray(e.b1 if e.b1 is not None else np.ones(e.voxels), np.float32)
                       for e in entries]) if has_b1 else None
        self.m0 = cat([np.asarray(e.m0 if e.m0 is not None else np.ones(e.voxels), np.float32)
                       for e in entries]) if has_m0 else None
        total = int((self.voxels * self.outputs).sum())
        self.out = torch.empty(total, dtype=torch.complex64, device=device)
        self.counter = torch.zeros(1, dtype=torch.int32, device=device)
        self.shape: tuple[int, int, int] | None = None
        self.graph: torch.cuda.CUDAGraph | None = None
        self._tables: dict[tuple, tuple] = {}

    # -- planning ---------------------------------------------------------
    def updates(self) -> int:
        """voxel x pulse x state updates of one pass (pulses = recorded echoes)."""
        return int((self.voxels * self.outputs * self.states).sum())

    def _plan(self, orders: int, warps: int) -> tuple:
        key = (orders, warps)
        if key in self._tables:
            return self._tables[key]
        lanes = -(-self.states // orders)
        if (lanes > 32).any():
            raise ValueError(f"orders_per_lane {orders} cannot hold {int(self.states.max())} states")
        seq = np.zeros(len(self.entries), np.dtype([
            ("op_offset", "<i4"), ("op_count", "<i4"), ("states", "<i4"), ("lanes", "<i4"),
            ("outputs", "<i4"), ("voxel_count", "<i4"), ("voxel_offset", "<i8"),
            ("output_offset", "<i8")]))
        seq["op_offset"], seq["op_count"], seq["states"] = self.op_offset, self.op_count, self.states
        seq["lanes"], seq["outputs"], seq["voxel_count"] = lanes, self.outputs, self.voxels
        seq["voxel_offset"], seq["output_offset"] = self.voxel_offset, self.output_offset
        per_unit = warps * (32 // lanes)
        counts = -(-self.voxels // per_unit)
        seq_of = np.repeat(np.arange(len(self.entries)), counts)
        first = np.cumsum(np.concatenate([[0], counts]))[:-1]
        begin = (np.arange(int(counts.sum())) - np.repeat(first, counts)) * per_unit[seq_of]
        count = np.minimum(per_unit[seq_of], self.voxels[seq_of] - begin)
        # Every unit holds a CTA for (ops x padded orders) steps: largest first.
        cost = self.op_count[seq_of] * lanes[seq_of] * orders
        order = np.argsort(-cost, kind="stable")
        unit_arr = np.stack([seq_of, begin, count, np.zeros_like(count)], axis=1).astype(np.int32)
        unit_arr = unit_arr[order]
        units = unit_arr
        d_seq = torch.from_numpy(seq.view(np.uint8)).to(self.device)
        d_units = torch.from_numpy(np.ascontiguousarray(unit_arr).view(np.uint8)).to(self.device)
        self._tables[key] = (d_seq, d_units, int(units.shape[0]))
        return self._tables[key]

    def launch(self, shape: tuple[int, int, int]) -> None:
        """One persistent launch with (orders per lane, warps per CTA, CTAs per SM)."""
        orders, warps, per_sm = shape
        d_seq, d_units, n_units = self._plan(orders, warps)
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        tissue = _native.Tissue(self.t1.data_ptr(), self.t2.data_ptr(),
                                None if self.m0 is None else self.m0.data_ptr(),
                                None if self.b1 is None else self.b1.data_ptr(), None)
        _native.check(_native.library().tsg_epg_batched_forward(
            self.d_ops.data_ptr(), d_seq.data_ptr(), d_units.data_ptr(), n_units,
            self.counter.data_ptr(), ctypes.byref(tissue), self.out.data_ptr(), orders, warps,
            sms * per_sm, torch.cuda.current_stream().cuda_stream))

    def candidates(self) -> list[tuple[int, int, int]]:
        cands = []
        for orders in (2, 4, 8, 16):
            if (-(-self.states // orders) > 32).any():
                continue
            for warps in (2, 4, 8):
                for per_sm in (2, 4, 5, 6, 8, 10, 12, 16):
                    if warps * per_sm <= 64:
                        cands.append((orders, warps, per_sm))
        return cands

    def tune(self, use_cache: bool = True) -> tuple[tuple[int, int, int], dict]:
        sig = f"n={len(self.entries)},u={self.updates() // 10**6}M,smax={int(self.states.max())}"
        key = autotune.workload_key("batched", workload=sig)
        best, timings = autotune.tune(key, self.candidates(), self.launch, use_cache=use_cache,
                                      warmup=1, repeats=2)
        self.shape = tuple(best)
        return self.shape, timings

    def capture(self) -> torch.cuda.CUDAGraph:
        """Capture the counter reset and the persistent launch in a CUDA graph."""
        if self.shape is None:
            self.tune()
        self.launch(self.shape)  # tables built and kernel loaded outside capture
        torch.cuda.synchronize()
        stream = torch.cuda.Stream(self.device)
        stream.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream), torch.cuda.graph(graph, stream=stream):
            self.launch(self.shape)
        torch.cuda.current_stream().wait_stream(stream)
        self.graph = graph
        return graph

    def run(self) -> None:
        """Replay the captured launch (capturing it first if needed)."""
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def signal(self, index: int) -> torch.Tensor:
        """Sequence ``index``'s samples, ``(voxels, outputs)`` complex64,
        complex(real plane, imaginary plane) as the reference's runs return."""
        start = int(self.output_offset[index])
        n = int(self.voxels[index] * self.outputs[index])
        return self.out[start:start + n].view(int(self.voxels[index]), int(self.outputs[index]))

    # -- the plain form, for comparison -----------------------------------
    def run_plain(self, launch=None) -> None:
        """One fixed-shape sweep launch per sequence into the same outputs."""
        lib = _native.library()
        stream = torch.cuda.current_stream().cuda_stream
        for s, e in enumerate(self.entries):
            prog = program_for(e.events, self.device)
            v0, n = int(self.voxel_offset[s]), int(self.voxels[s])
            sl = slice(v0, v0 + n)
            tissue = engine.TissueMaps(self.t1[sl], self.t2[sl],
                                       None if self.m0 is None else self.m0[sl],
                                       None if self.b1 is None else self.b1[sl], None)
            t = tissue.struct()
            _native.check(lib.tsg_epg_forward(prog.handle, ctypes.byref(t), n, int(self.states[s]),
                                              _native.LAYOUT_COMPLEX, self.signal(s).data_ptr(),
                                              None, _native.launch_shape(launch), stream))
