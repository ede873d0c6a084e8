"""The C ABI library (no GPU needed): exports, and the pulse-program compiler.

The compiler folds zero-duration events into the op before them. An op-level
FP64 emulator written here runs the compiled programs; it must reproduce the
event-level oracle, which shows the folding keeps the reference's semantics.
"""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import packed_from_golden

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols() -> set[str]:
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(tsg_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(built_library):
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in sorted(names) if not hasattr(built_library, n)]
    assert not missing, missing


def test_version_and_error_without_gpu(built_library):
    from torchsim_gb300 import _native

    assert built_library.tsg_version() >= 1
    rc = built_library.tsg_program_plan(None, None, None, None, None, 0, 5, 0, None, None, None,
                                        None, None, None, None, 0)
    assert rc == _native.TSG_ERR_ARGUMENT
    assert b"dimensions" in built_library.tsg_last_error()


def plan(events, unmerged=False, duration_tangent=None):
    from torchsim_gb300 import _native

    lib = _native.library()
    dur = np.ascontiguousarray(events.duration, np.float32)
    kind = np.ascontiguousarray(events.kind, np.int32)
    flip = np.ascontiguousarray(events.flip, np.float32)
    action = np.ascontiguousarray(events.action, np.uint8)
    oi = np.ascontiguousarray(events.output_index, np.int32)
    tan = None if duration_tangent is None else np.ascontiguousarray(duration_tangent, np.float32)
    n_ops, n_out = ctypes.c_int64(), ctypes.c_int64()
    _native.check(lib.tsg_program_plan(dur.ctypes.data, kind.ctypes.data, flip.ctypes.data,
                                       action.ctypes.data, oi.ctypes.data, events.trains,
                                       events.events, int(unmerged),
                                       None if tan is None else tan.ctypes.data,
                                       ctypes.byref(n_ops), ctypes.byref(n_out), None, None,
                                       None, None, 0))
    cap = n_ops.value * events.trains
    dt = np.zeros(cap, np.float32)
    fl = np.zeros(cap, np.float32)
    rec = np.zeros(cap, np.int32)
    code = np.zeros(cap, np.uint32)
    _native.check(lib.tsg_program_plan(dur.ctypes.data, kind.ctypes.data, flip.ctypes.data,
                                       action.ctypes.data, oi.ctypes.data, events.trains,
                                       events.events, int(unmerged),
                                       None if tan is None else tan.ctypes.data,
                                       ctypes.byref(n_ops), ctypes.byref(n_out), dt.ctypes.data,
                                       fl.ctypes.data, rec.ctypes.data, code.ctypes.data, cap))
    return n_ops.value, n_out.value, dt, fl, rec, code


def emulate(n_ops, n_out, dt, fl, rec, code, trains, t1, t2, b1, m0, inv, states):
    """FP64 run of a compiled program (the op template's micro-steps in order)."""
    V = t1.size
    out = np.zeros((trains, V, n_out))
    S = states
    for t in range(trains):
        p = np.zeros((V, S)); m = np.zeros((V, S)); z = np.zeros((V, S)); z[:, 0] = 1
        r1 = 1000.0 / t1.astype(np.float64); r2 = 1000.0 / t2.astype(np.float64)

        def shift():
            m[:, :-1] = m[:, 1:].copy(); m[:, -1] = 0
            p[:, 1:] = p[:, :-1].copy(); p[:, 0] = -m[:, 0]

        for i in range(t * n_ops, (t + 1) * n_ops):
            c = int(code[i])
            if c & 1:
                e1 = np.exp(-r1 * dt[i])[:, None]; e2 = np.exp(-r2 * dt[i])[:, None]
                p *= e2; m *= e2; z *= e1; z[:, 0] += 1 - e1[:, 0]
            for _ in range((c >> 1) & 3):
                shift()
            rf = (c >> 3) & 3
            if rf == 1:
                a = (fl[i] * b1.astype(np.float64))[:, None]
                co, si = np.cos(a), np.sin(a)
                P = 0.5 * (1 + co) * p + 0.5 * (1 - co) * m - si * z
                M = 0.5 * (1 - co) * p + 0.5 * (1 + co) * m + si * z
                Z = 0.5 * si * (p - m) + co * z
                p[:], m[:], z[:] = P, M, Z
            elif rf == 2:
                z *= -inv.astype(np.float64)[:, None]
            for _ in range((c >> 5) & 3):
                shift()
            if c & (1 << 7):
                p[:] = 0; m[:] = 0
            if c & (1 << 8):
                out[t, :, rec[i]] = m0 * p[:, 0]
            for _ in range((c >> 9) & 3):
                shift()
            if c & (1 << 11):
                p[:] = 0; m[:] = 0
    return out[0] if trains == 1 else out


@pytest.mark.parametrize("name", ["mrf880", "mrf_prep", "fse_cpmg"])
@pytest.mark.parametrize("unmerged", [False, True])
def test_compiled_program_keeps_event_semantics(built_library, golden, name, unmerged):
    from torchsim_gb300.sequence import PackedEvents

    d = golden(name)
    ev = PackedEvents(d["event_duration"][None], d["event_kind"], d["event_flip"][None],
                      d["event_phase"][None], d["event_action"], d["event_output_index"])
    n_ops, n_out, dt, fl, rec, code = plan(ev, unmerged)
    if unmerged:
        assert n_ops == ev.events
    p = packed_from_golden(d)
    got = emulate(n_ops, n_out, dt, fl, rec, code, 1, p.t1_ms, p.t2_ms, p.b1, p.m0, p.inversion,
                  p.state_count)
    ref = O.forward(p, "f64")
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12)


def test_merge_counts(built_library):
    from torchsim_gb300.sequence import fse_events, mrf_events

    ev = mrf_events(np.linspace(5, 60, 880).astype(np.float32), 10.0)
    n_ops, n_out, *_ = plan(ev)
    assert (n_ops, n_out) == (881, 880)  # the inversion, then one op per repetition
    ev = fse_events(np.full(12, 150.0, np.float32), 8.0, phases_deg=90.0)
    n_ops, n_out, *_ = plan(ev)
    assert (n_ops, n_out) == (1 + 2 * 12, 12)


def test_duration_direction_keeps_zero_duration_steps(built_library):
    from torchsim_gb300.sequence import mrf_events

    ev = mrf_events(np.float32([10, 20, 30]), 10.0)
    tangent = np.zeros_like(ev.duration)
    tangent[0, 2] = 1.0  # the first sample has zero duration
    merged, *_ = plan(ev)
    split, *_ = plan(ev, duration_tangent=tangent)
    assert split == merged + 1
