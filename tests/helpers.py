"""Shared helpers for the tests: seeded workloads and oracle adapters."""

from __future__ import annotations

import numpy as np

from oracle import oracle as O


def mrf_schedule() -> np.ndarray:
    """The 880-pulse MRF flip schedule: 5->60 deg (300), 60->2 deg (300), 280 x 2 deg."""
    return np.concatenate(
        [np.linspace(5, 60, 300), np.linspace(60, 2, 300), np.full(280, 2.0)]
    ).astype(np.float32)


def draw_tissue(seed: int, n: int, b1=(0.8, 1.2)):
    """T1 log-uniform 100-3000 ms, T2 log-uniform 10-300 ms clipped below T1, B1 uniform."""
    rng = np.random.default_rng(seed)
    t1 = np.exp(rng.uniform(np.log(100), np.log(3000), n)).astype(np.float32)
    t2 = np.exp(rng.uniform(np.log(10), np.log(300), n)).astype(np.float32)
    t2 = np.minimum(t2, np.float32(0.999) * t1).astype(np.float32)
    b1v = rng.uniform(b1[0], b1[1], n).astype(np.float32)
    return t1, t2, b1v


def packed_from_events(events, t1, t2, states, m0=None, b1=None, inv=None) -> O.Packed:
    return O.Packed(t1_ms=t1, t2_ms=t2, duration_s=events.duration, kind=events.kind,
                    flip_rad=events.flip, action=events.action,
                    output_index=events.output_index, state_count=states, m0=m0, b1=b1,
                    inversion=inv)


def packed_from_golden(d, prefix: str = "") -> O.Packed:
    return O.Packed(
        t1_ms=d[prefix + "tissue_t1_ms"], t2_ms=d[prefix + "tissue_t2_ms"],
        duration_s=d[prefix + "event_duration"], kind=d[prefix + "event_kind"],
        flip_rad=d[prefix + "event_flip"], action=d[prefix + "event_action"],
        output_index=d[prefix + "event_output_index"], state_count=int(d["states"]),
        m0=d[prefix + "tissue_m0"], b1=d[prefix + "tissue_b1"],
        inversion=d[prefix + "tissue_inversion_efficiency"])


def packed_complex_from_golden(d, prefix: str = "") -> O.Packed:
    """The packed inputs of a complex-path fixture: the real-path buffers plus
    the event phases and the per-voxel transmit phase and off-resonance."""
    p = packed_from_golden(d, prefix)
    p.phase_rad = d[prefix + "event_phase"]
    p.b1_phase_rad = d[prefix + "tissue_b1_phase_rad"]
    p.b0_hz = d[prefix + "tissue_b0_hz"]
    return p


reference_module = O.reference_module
reference_jvp = O.reference_jvp


def max_rel(actual, expected) -> float:
    """max |a - e| / max |e|, the normalisation of the reference's CUDA parity
    tests (tests/sequence/test_cuda_parity.py:137-138)."""
    actual = np.asarray(actual)
    expected = np.asarray(expected)
    scale = float(np.abs(expected).max()) if expected.size else 0.0
    if scale == 0.0:
        return float(np.abs(actual).max()) if actual.size else 0.0
    return float(np.abs(actual - expected).max() / scale)


def gn_slice_measured(d) -> np.ndarray:
    """The noisy signals of the `gn_slice` fixture, (voxels, pulses)
    complex64: the reference's noise-free MRF signal (1j times the recorded
    sample 1j m0 F+[0], i.e. -m0 F+[0] on the real axis, which the oracle's
    FP32 port reproduces bit for bit) plus the
    fixture's seeded complex Gaussian noise, added in float64 and rounded to
    complex64 as the fixture's generator did."""
    from torchsim_gb300.sequence import mrf_events

    events = mrf_events(d["flip_deg"], float(d["tr_ms"]))
    imag = O.forward(packed_from_events(events, d["t1"], d["t2"], int(d["states"]),
                                        m0=d["m0"], b1=d["b1"]), "f32", threads=8)
    sig = (-imag.astype(np.float32)).astype(np.complex64)
    rng = np.random.default_rng(int(d["noise_seed"]))
    sigma = float(d["sigma"])
    noise = (rng.standard_normal(sig.shape) + 1j * rng.standard_normal(sig.shape)) * sigma
    return (sig + noise).astype(np.complex64)
