"""The oracle pinned to the reference: its FP32 port reproduces the
reference's own compiled CPU kernel on the committed fixtures, and the FP64
oracle agrees with it to FP32 rounding."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import (max_rel, packed_complex_from_golden, packed_from_golden,
                           reference_jvp, reference_module)

FORWARD_CASES = ["mrf880", "mrf_prep", "fse_cpmg"]
KEYS = {"T1": "t1_ms", "T2": "t2_ms", "B1": "b1", "M0": "m0", "inv_efficiency": "inversion"}


@pytest.mark.parametrize("name", FORWARD_CASES)
def test_fp32_port_is_bitwise_the_reference_kernel(golden, name):
    d = golden(name)
    assert int(d["real_axis"]) == 1
    raw = d["raw_forward"]
    out = O.forward(packed_from_golden(d), "f32")
    assert np.array_equal(out, raw.imag)
    assert not raw.real.any()


@pytest.mark.parametrize("name", FORWARD_CASES)
def test_fp64_oracle_matches_reference(golden, name):
    d = golden(name)
    out = O.forward(packed_from_golden(d), "f64")
    assert max_rel(out, d["raw_forward"].imag) < 5e-6


@pytest.mark.parametrize("name", ["mrf880", "mrf_prep"])
def test_oracle_tangents_match_reference_jacobian(golden, name):
    """The FP32 port picks the reference's kernel by atom count (eight atoms or
    more: the eight-atom lane kernel) and reproduces its Jacobian bit for bit:
    mrf880 has 8 atoms (lane kernel), mrf_prep 5 (per-atom kernel)."""
    d = golden(name)
    p = packed_from_golden(d)
    for col, prop in enumerate(d["jacobian_names"]):
        ref = -d["jacobian"][:, col].real  # the API returns 1j * (i * tangent)
        t = O.tangent(p, "f32", **{KEYS[str(prop)]: 1.0})
        assert np.array_equal(t, ref), prop
        assert max_rel(O.tangent(p, "f64", **{KEYS[str(prop)]: 1.0}), ref) < 5e-6, prop


def test_lane_and_per_atom_tangents_agree():
    """The two FP32 layouts differ only in rounding, on a ragged atom count
    (a partial block of eight) and two trains."""
    rng = np.random.default_rng(3)
    atoms, events = 21, 120
    flip = np.deg2rad(rng.uniform(5, 70, (2, events))).astype(np.float32)
    kind = np.ones(events, np.int32)
    kind[1::2] = 2
    action = np.where(kind == 2, 32 | 16, 0).astype(np.uint8)
    out_index = np.where(kind == 2, np.cumsum(kind == 2) - 1, -1).astype(np.int32)
    duration = np.full((2, events), 5e-3, np.float32)
    t1 = rng.uniform(300, 2000, atoms).astype(np.float32)
    p = O.Packed(t1, (0.1 * t1).astype(np.float32), duration, kind, flip, action, out_index, 12,
                 b1=rng.uniform(0.8, 1.2, atoms).astype(np.float32))
    for key in ("t1_ms", "t2_ms", "b1", "flip_rad", "duration_s"):
        a = O.tangent(p, "f32", lanes=True, threads=3, **{key: 1.0})
        b = O.tangent(p, "f32", lanes=False, **{key: 1.0})
        c = O.tangent(p, "f64", **{key: 1.0})
        assert max_rel(a, c) < 2e-5 and max_rel(b, c) < 2e-5, key
        assert max_rel(a, b) < 2e-5, key


def test_lane_tangent_is_bitwise_the_reference_kernel():
    """Against the reference's own compiled CPU kernel (built from its sources
    where they lie into oracle/_ref), on the dictionary sequence at 45 atoms (a
    partial block), through its ``simulate_jvp`` entry point."""
    ref = reference_module()
    if ref is None:
        pytest.skip("the reference's CPU kernel is not built here")
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(5)
    atoms = 45
    flip = np.concatenate([np.linspace(5, 60, 100), np.linspace(60, 2, 100)]).astype(np.float32)
    ev = mrf_events(flip, 10.0)
    t1 = np.exp(rng.uniform(np.log(100), np.log(3000), atoms)).astype(np.float32)
    t2 = np.minimum(np.exp(rng.uniform(np.log(10), np.log(300), atoms)), 0.999 * t1).astype(np.float32)
    b1 = rng.uniform(0.8, 1.2, atoms).astype(np.float32)
    p = O.Packed(t1, t2, ev.duration, ev.kind, ev.flip, ev.action, ev.output_index, 16, b1=b1)
    for col, key in ((0, "t1_ms"), (1, "t2_ms"), (3, "b1")):
        expected = reference_jvp(ref, p, col)
        assert np.array_equal(O.tangent(p, "f32", threads=4, **{key: 1.0}), expected), key


def test_public_signal_is_minus_raw_plane(golden):
    d = golden("mrf880")
    # MRFSimulator.evaluate returns 1j * signal (simulators/mrf.py:84).
    np.testing.assert_array_equal(d["signal"].real, -d["raw_forward"].imag)


@pytest.mark.parametrize("precision,tol", [("f32", 0.0), ("f64", 1e-6)])
def test_oracle_adjoint_matches_reference_vjp(golden, precision, tol):
    d = golden("mrf_adjoint")
    p = packed_from_golden(d, "vjp_")
    g = O.adjoint(p, d["vjp_seed"].imag, precision)
    pairs = {"t1_ms": "vjp_grad_t1_ms", "t2_ms": "vjp_grad_t2_ms", "b1": "vjp_grad_b1",
             "m0": "vjp_grad_m0", "flip_rad": "vjp_grad_flip",
             "duration_s": "vjp_grad_duration"}
    for mine, ref in pairs.items():
        assert max_rel(g[mine], d[ref]) <= tol, mine


def test_oracle_adjoint_is_transpose_of_tangent():
    """<seed, J v> == <J^T seed, v> on a small seeded case (FP64)."""
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(7)
    flips = rng.uniform(5, 70, 12).astype(np.float32)
    trs = rng.uniform(8, 15, 12).astype(np.float32)
    ev = mrf_events(flips, trs, TI_ms=5.0)
    t1 = np.array([800.0, 300.0], np.float32)
    t2 = np.array([60.0, 40.0], np.float32)
    b1 = np.array([0.9, 1.1], np.float32)
    p = O.Packed(t1, t2, ev.duration, ev.kind, ev.flip, ev.action, ev.output_index, 6, b1=b1)
    seed = rng.standard_normal((2, ev.outputs)).astype(np.float32)
    g = O.adjoint(p, seed, "f64")
    v_flip = rng.standard_normal(ev.duration.shape).astype(np.float32)
    v_dur = rng.standard_normal(ev.duration.shape).astype(np.float32) * 1e-3
    v_t1 = rng.standard_normal(2).astype(np.float32)
    jv = O.tangent(p, "f64", flip_rad=v_flip, duration_s=v_dur, t1_ms=v_t1)
    lhs = float((seed.astype(np.float64) * jv).sum())
    rhs = float((g["flip_rad"] * v_flip[0]).sum() + (g["duration_s"] * v_dur[0]).sum()
                + (g["t1_ms"] * v_t1).sum())
    assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(lhs))


def test_oracle_planted_mistake_is_caught(golden):
    """A wrong shift rule in the checker must show up against the fixture."""
    d = golden("mrf880")
    p = packed_from_golden(d)
    p.state_count = 9  # truncating one order early changes the answer
    out = O.forward(p, "f64")
    assert max_rel(out, d["raw_forward"].imag) > 1e-5


# ---- the complex path (RF phases, B0, B1phase) -------------------------------


@pytest.mark.parametrize("name", ["fse_phase0", "mrf_offaxis"])
def test_complex_fp32_port_is_bitwise_the_reference_kernel(golden, name):
    d = golden(name)
    assert int(d["real_axis"]) == -1  # the reference ran its complex kernel
    got = O.forward_complex(packed_complex_from_golden(d), "f32").astype(np.complex64)
    assert np.array_equal(got, d["raw_forward"])


@pytest.mark.parametrize("name", ["fse_phase0", "mrf_offaxis"])
def test_complex_fp64_oracle_matches_reference(golden, name):
    d = golden(name)
    got = O.forward_complex(packed_complex_from_golden(d), "f64")
    assert max_rel(got, d["raw_forward"]) <= 2e-6


def test_complex_public_mrf_signal_is_1j_raw(golden):
    d = golden("mrf_offaxis")
    raw = d["raw_forward"]
    assert np.array_equal(d["signal"], (1j * raw).astype(np.complex64))


def test_complex_oracle_reduces_to_the_real_one(golden):
    """With every phase at 90 degrees and no B0 or B1phase the complex
    recursion is the real one: the recorded sample is i * (real plane)."""
    d = golden("fse_cpmg")
    p = packed_complex_from_golden(d)
    p.b1_phase_rad = None
    p.b0_hz = None
    full = O.forward_complex(p, "f64")
    real = O.forward(packed_from_golden(d), "f64")
    assert max_rel(full.imag, real) <= 1e-12
    assert np.abs(full.real).max() <= 1e-12 * np.abs(real).max()


# ---- second order (forward over reverse) -------------------------------------

SECOND_NAMES = {"t1_ms": "t1_ms", "t2_ms": "t2_ms", "m0": "m0", "b1": "b1",
                "inversion": "inversion_efficiency", "flip_rad": "flip",
                "duration_s": "duration"}


def second_case(d, prefix: str):
    """The packed inputs, direction and seed of one recorded forward-over-
    reverse call of the mrf_second fixture."""
    p = packed_from_golden(d, prefix)
    direction = {k: d[f"{prefix}tangent_{v}"] for k, v in SECOND_NAMES.items()}
    return p, direction, d[f"{prefix}seed"].imag


@pytest.mark.parametrize("prefix", ["design0_", "design1_", "direct_"])
@pytest.mark.parametrize("precision,tol", [("f32", 0.0), ("f64", 5e-6)])
def test_oracle_second_order_matches_reference(golden, prefix, precision, tol):
    """Both the value side (J^T seed) and the curvature side of
    ``_run_packed_vjp_jvp``: the CRLB design's two column calls (one-hot T2,
    T1 directions) and a direct call along every tissue property, duration
    and flip at once. The FP32 port is bitwise the reference's kernel."""
    d = golden("mrf_second")
    p, direction, seed = second_case(d, prefix)
    values, curvature = O.second(p, seed, precision, **direction)
    for mine, ref in SECOND_NAMES.items():
        assert max_rel(values[mine], d[f"{prefix}value_{ref}"]) <= tol, ("value", mine)
        assert max_rel(curvature[mine], d[f"{prefix}curvature_{ref}"]) <= tol, ("curve", mine)


def test_oracle_second_order_is_the_derivative_of_the_adjoint(golden):
    """The curvature side against central differences of the first-order
    adjoint stepped along the direction (FP64), and the value side against the
    adjoint itself."""
    d = golden("mrf_second")
    p, direction, seed = second_case(d, "direct_")
    values, curvature = O.second(p, seed, "f64", **direction)
    first = O.adjoint(p, seed, "f64")
    for name in ("t1_ms", "t2_ms", "m0", "b1", "flip_rad", "duration_s"):
        assert max_rel(values[name], first[name]) <= 1e-12, name
    h = 1e-3

    def stepped(sign):
        q = packed_from_golden(d, "direct_")
        for name, attr in (("t1_ms", "t1_ms"), ("t2_ms", "t2_ms"), ("m0", "m0"), ("b1", "b1"),
                           ("inversion", "inversion"), ("duration_s", "duration_s"),
                           ("flip_rad", "flip_rad")):
            base = np.asarray(getattr(q, attr), np.float64)
            setattr(q, attr, base + sign * h * np.asarray(direction[name], np.float64))
        return O.adjoint(q, seed, "f64")

    # The packed inputs are FP32, so the step is applied in FP64 and rounded;
    # h keeps that rounding well below the difference.
    up, down = stepped(1.0), stepped(-1.0)
    for name in ("t1_ms", "t2_ms", "m0", "b1", "flip_rad", "duration_s"):
        fd = (up[name] - down[name]) / (2 * h)
        assert max_rel(curvature[name], fd) <= 1e-3, name


def test_oracle_second_order_planted_mistake_is_caught(golden):
    """A direction the checker drops must show up against the fixture."""
    d = golden("mrf_second")
    p, direction, seed = second_case(d, "direct_")
    direction.pop("duration_s")
    _, curvature = O.second(p, seed, "f64", **direction)
    assert max_rel(curvature["flip_rad"], d["direct_curvature_flip"]) > 1e-3


# ---- gradients on the complex path ------------------------------------------

COMPLEX_GRADS = {"t1_ms": "t1_ms", "t2_ms": "t2_ms", "m0": "m0", "b1": "b1",
                 "inversion": "inversion_efficiency", "b1_phase_rad": "b1_phase_rad",
                 "b0_hz": "b0_hz", "flip_rad": "flip", "duration_s": "duration",
                 "phase_rad": "phase"}


def complex_adjoint_case(d, prefix: str):
    fields = {k: d[k] for k in d.files}
    fields["states"] = d[prefix.split("_")[0] + "_states"]
    return packed_complex_from_golden(fields, prefix + "vjp_")


@pytest.mark.parametrize("prefix", ["mrf", "fse"])
def test_oracle_complex_adjoint_matches_reference(golden, prefix):
    """Every gradient slot of the reference's complex first-order adjoint (an
    off-axis MRF with B0, B1phase and M0 maps; a default-phase CPMG) against
    the FP64 restatement. Gradients the reference forms as rounding noise
    (B0 and B1phase of the on-resonance CPMG) are compared absolutely."""
    d = golden("complex_adjoint")
    p = complex_adjoint_case(d, prefix + "_")
    g = O.adjoint_complex(p, d[f"{prefix}_vjp_seed"], "f64")
    scale = max(float(np.abs(d[f"{prefix}_vjp_grad_{v}"]).max()) for v in COMPLEX_GRADS.values())
    for mine, ref in COMPLEX_GRADS.items():
        want = d[f"{prefix}_vjp_grad_{ref}"]
        if np.abs(want).max() < 1e-6 * scale:
            assert np.abs(g[mine]).max() <= 1e-6 * scale, mine
        else:
            assert max_rel(g[mine], want) <= 5e-6, mine


def test_oracle_complex_adjoint_is_the_gradient_of_the_forward(golden):
    """Central differences of the FP64 complex forward along random
    directions of the tissue, flip, duration and phase buffers."""
    d = golden("complex_adjoint")
    p = complex_adjoint_case(d, "mrf_")
    seed = d["mrf_vjp_seed"]
    g = O.adjoint_complex(p, seed, "f64")
    rng = np.random.default_rng(11)
    # The packed inputs are FP32: the step must stay well above their
    # rounding, which bounds the agreement at about 1e-3.
    h = 1e-3
    for name, attr in (("t1_ms", "t1_ms"), ("t2_ms", "t2_ms"), ("b1", "b1"), ("b0_hz", "b0_hz"),
                       ("b1_phase_rad", "b1_phase_rad"), ("flip_rad", "flip_rad"),
                       ("duration_s", "duration_s"), ("phase_rad", "phase_rad")):
        base = np.asarray(getattr(p, attr), np.float64)
        v = rng.standard_normal(base.shape) * np.maximum(np.abs(base), 1e-3)

        def loss(sign):
            q = complex_adjoint_case(d, "mrf_")
            setattr(q, attr, base + sign * h * v)
            out = O.forward_complex(q, "f64")
            return float((seed.real * out.real + seed.imag * out.imag).sum())

        fd = (loss(1.0) - loss(-1.0)) / (2 * h)
        got = float((g[name].reshape(v.shape) * v).sum())
        assert abs(got - fd) <= 2e-3 * max(abs(fd), 1e-9), (name, got, fd)


def test_gn_slice_signals_regenerate_bitwise(golden):
    """The 4,096-voxel mapping fixture keeps the tissue, the noise seed and
    sigma instead of its 4 MB of signals: the oracle's FP32 port gives the
    reference's noise-free signal bit for bit, so the regenerated noisy
    signals equal the stored sample of rows exactly."""
    from tests.helpers import gn_slice_measured

    d = golden("gn_slice")
    y = gn_slice_measured(d)
    assert y.shape == (4096, 120)
    assert np.array_equal(y[::64], d["measured_every_64th"])


def test_gn_port_matches_the_reference_estimator(golden):
    """The CPU restatement of the mapping loop (oracle/gn_port.py: the
    reference's Levenberg-Marquardt and TrustRegion damping over the oracle's
    FP32 port of its kernels) against the reference's NonlinearLeastSquares
    on 512 voxels of the 4,096-voxel fixture, from the same start, 20 steps."""
    from oracle import gn_port
    from tests.helpers import gn_slice_measured
    from torchsim_gb300.sequence import mrf_events

    d = golden("gn_slice")
    n = 512
    y = gn_slice_measured(d)[:n]
    events = mrf_events(d["flip_deg"], float(d["tr_ms"]))
    got = gn_port.fit(events, y, d["start"], d["bounds"][:, 0], d["bounds"][:, 1],
                      int(d["states"]), b1=d["b1"][:n], max_iterations=20, threads=8)
    for k, key in enumerate(("map_t1", "map_t2", "map_m0")):
        ref = d[key][:n].astype(np.float64)
        err = np.abs(got.x[:, k] - ref) / np.abs(ref)
        assert np.median(err) <= 1e-5, key
        assert np.quantile(err, 0.99) <= 1e-3, key
        assert err.max() <= 1e-2, key


def test_gn_port_matches_the_reference_on_the_small_fixture(golden):
    """The same restatement on the 16-voxel `gn_mrf` fixture, whose measured
    signals are stored: the reference estimator's maps from its start."""
    from oracle import gn_port
    from torchsim_gb300.sequence import mrf_events

    d = golden("gn_mrf")
    events = mrf_events(d["flip_deg"], float(d["tr_ms"]))
    got = gn_port.fit(events, d["measured"], d["start"], d["bounds"][:, 0], d["bounds"][:, 1],
                      int(d["states"]), b1=d["b1"], max_iterations=20, threads=4)
    for k, key in enumerate(("map_t1", "map_t2", "map_m0")):
        ref = d[key].astype(np.float64)
        assert np.max(np.abs(got.x[:, k] - ref) / np.abs(ref)) <= 2e-3, key
