"""Forward-mode tangents on the complex path (RF and receiver phases, B0,
B1phase): the general tangent kernel against the reference's own complex
simulate_jvp_range, recorded call by call in tests/golden/complex_jvp.npz
(made by tests/golden/make_golden.py from the reference's _run_packed_jvp),
and every direction against central differences of the FP64 restatement of
the reference's complex forward. Tolerance: 1e-4 of max |reference|, the
Jacobian tolerance of the reference's CUDA parity tests
(tests/sequence/test_cuda_parity.py:137-138)."""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import max_rel, packed_complex_from_golden
from tests.test_gpu_parity import EVENT_ORDER, TISSUE_ORDER, _pointer_array

pytestmark = pytest.mark.gpu

JACOBIAN_TOL = 1e-4
FEATURES = 1 | 8 | 16 | 32  # off-axis, transmit, density, inversion (_epg_cpu.cpp:95-100)


def _call_arrays(d, k):
    tissue = [np.ascontiguousarray(d[f"c{k}_tissue_{n}"]) for n in TISSUE_ORDER]
    events = [np.ascontiguousarray(d[f"c{k}_event_{n}"]) for n in EVENT_ORDER]
    tangents = [np.ascontiguousarray(d[f"c{k}_tissue_tangent_{j}"], np.float32) for j in range(17)]
    tangents += [np.ascontiguousarray(d[f"c{k}_event_tangent_{j}"], np.float32) for j in range(3)]
    return tissue, events, tangents


def test_dropin_complex_jvp_matches_the_reference(built_library, cuda, golden):
    """tsg_epg_simulate_jvp with real_axis = -1 on each of the reference's
    recorded calls: one-hot T1, T2, B1, M0, inversion, B0 and B1phase, and
    one direction in duration, flip and phase at once."""
    from torchsim_gb300 import _native

    d = golden("complex_jvp")
    assert int(d["calls"]) == 8
    for k in range(int(d["calls"])):
        assert int(d[f"c{k}_real_axis"]) != 1
        tissue, events, tangents = _call_arrays(d, k)
        ref = d[f"c{k}_result"]
        V, P = ref.shape
        out_r = np.full((V, P), 7.0, np.float32)
        out_i = np.full((V, P), 7.0, np.float32)
        arrays = [*tissue, *events, *tangents, out_r, out_i, *([None] * 13)]
        _native.check(built_library.tsg_epg_simulate_jvp(
            _pointer_array(arrays), len(arrays), V, 1, events[1].size, int(d["states"]), P, -1,
            FEATURES))
        assert max_rel(out_r + 1j * out_i, ref) <= JACOBIAN_TOL, k


def _tangent(cuda, p: O.Packed, direction=None, offaxis=None) -> np.ndarray:
    """The general complex tangent on the GPU, as the complex value of the
    reference's two planes (the public value is 1j times it)."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import PackedEvents, Program

    ev = PackedEvents(duration=np.atleast_2d(p.duration_s), kind=p.kind,
                      flip=np.atleast_2d(p.flip_rad), phase=np.atleast_2d(p.phase_rad),
                      action=p.action, output_index=p.output_index)
    prog = Program(ev, phased=True)

    def dev(a):
        return None if a is None else torch.from_numpy(np.asarray(a, np.float32)).to(cuda)

    tissue = engine.tissue_maps(cuda, p.atom_count, dev(p.t1_ms), dev(p.t2_ms), dev(p.m0),
                                dev(p.b1), dev(p.inversion))
    off, keep = engine.offaxis_maps(cuda, p.atom_count, dev(p.b1_phase_rad), dev(p.b0_hz))
    out = engine.tangent_complex(
        prog, tissue, int(p.state_count), off,
        direction={k: dev(v) for k, v in (direction or {}).items()},
        offaxis_direction={k: dev(v) for k, v in (offaxis or {}).items()})
    del keep
    return (out * -1j).cpu().numpy()


def _central(p: O.Packed, name: str, dv: np.ndarray, h: float):
    """Central difference of the FP64 complex oracle along ``dv`` on buffer
    ``name``, and the direction actually taken: the oracle reads float32
    buffers, so the effective direction is (f32(x + h dv) - f32(x - h dv)) / 2h."""
    base = np.asarray(getattr(p, name), np.float64)
    plus = (base + h * dv).astype(np.float32)
    minus = (base - h * dv).astype(np.float32)
    taken = (plus.astype(np.float64) - minus.astype(np.float64)) / (2 * h)
    f = [O.forward_complex(dataclasses.replace(p, **{name: x}), "f64") for x in (plus, minus)]
    return (f[0] - f[1]) / (2 * h), taken


# Steps small enough that the central difference's truncation stays far
# below the tolerance; the float32 rounding of the step is taken out exactly
# (the direction actually applied is what the tangent is asked for).
TISSUE_DIRECTIONS = [("t1_ms", "direction", 1e-3), ("t2_ms", "direction", 1e-3),
                     ("m0", "direction", 1e-3), ("b1", "direction", 1e-3),
                     ("inversion", "direction", 1e-3), ("b1_phase_rad", "offaxis", 1e-3),
                     ("b0_hz", "offaxis", 0.05)]


@pytest.mark.parametrize("name,group,h", TISSUE_DIRECTIONS)
def test_complex_tangent_tissue_directions_against_central_differences(cuda, golden, name,
                                                                      group, h):
    d = golden("complex_jvp")
    p = packed_complex_from_golden(d, "c0_")
    rng = np.random.default_rng(len(name))
    base = np.asarray(getattr(p, name), np.float64)
    # A relative step for the positive maps, an absolute one for the phases.
    scale = np.abs(base) if name in ("t1_ms", "t2_ms", "m0", "b1", "inversion") else 1.0
    dv = rng.standard_normal(base.shape) * scale
    fd, taken = _central(p, name, dv, h)
    got = _tangent(cuda, p, **{group: {name: taken}})
    assert max_rel(got, fd) <= JACOBIAN_TOL, name


# Durations are ~10 ms and the relaxation and off-resonance rates reach
# ~250 per second, so the duration step is kept to 2 us for the truncation.
@pytest.mark.parametrize("name,group,h", [("duration_s", "direction", 2e-6),
                                          ("flip_rad", "direction", 1e-3),
                                          ("phase_rad", "offaxis", 1e-3)])
def test_complex_tangent_event_directions_against_central_differences(cuda, golden, name,
                                                                     group, h):
    d = golden("complex_jvp")
    p = packed_complex_from_golden(d, "c0_")
    base = np.atleast_2d(np.asarray(getattr(p, name), np.float64))
    p = dataclasses.replace(p, **{name: base.astype(np.float32)})
    rng = np.random.default_rng(len(name))
    dv = rng.standard_normal(base.shape)
    if name == "duration_s":
        # Zero-length events are folded into the op before them; a direction
        # on one is a direction the program has no op boundary for.
        dv = np.where(base > 0, dv, 0.0)
    fd, taken = _central(p, name, dv, h)
    got = _tangent(cuda, p, **{group: {name: taken}})
    assert max_rel(got, fd) <= JACOBIAN_TOL, name


def test_public_jacobian_complex_columns_match_the_reference(cuda, golden):
    """MRFSimulator.jacobian on the complex path with every column the
    reference's public Jacobian gives there -- T1, T2, B1, M0, inversion
    efficiency, B0 and B1phase -- against the reference's."""
    from torchsim_gb300 import MRFSimulator

    d = golden("complex_jvp")
    names = tuple(str(n) for n in d["jacobian_names"])
    g = lambda a: torch.from_numpy(np.asarray(a)).to(cuda)
    sim = MRFSimulator(TI=float(d["ti_ms"]), states=int(d["states"]))
    _, jac = sim.jacobian(names, flip=d["flip_deg"], TR=d["tr_ms"], phases=d["phases_deg"],
                          T1=g(d["t1"]), T2=g(d["t2"]), B1=g(d["b1"]), B0=g(d["b0"]),
                          B1phase=g(d["b1_phase"]), M0=g(d["m0"]), inv_efficiency=g(d["inv"]))
    for c, name in enumerate(names):
        assert max_rel(jac[:, c].cpu().numpy(), d["jacobian"][:, c]) <= JACOBIAN_TOL, name
