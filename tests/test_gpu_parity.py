"""GPU parity: the sm_103a sweep kernels against the FP64 oracle and the
reference's own fixtures.

Tolerances are those stated for this path: signal max-relative error <= 1e-5
and Jacobian <= 1e-4 against the FP64 oracle, normalised by max |reference| as
the reference's CUDA parity tests do (tests/sequence/test_cuda_parity.py:
137-138).
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import draw_tissue, max_rel, mrf_schedule, packed_from_events, packed_from_golden

pytestmark = pytest.mark.gpu

SIGNAL_TOL = 1e-5
JACOBIAN_TOL = 1e-4
KEYS = {"T1": "t1_ms", "T2": "t2_ms", "B1": "b1", "M0": "m0", "inv_efficiency": "inversion"}


def oracle_jacobian(p, names):
    cols = []
    for name in names:
        cols.append(-O.tangent(p, "f64", **{KEYS[name]: 1.0}))
    return np.stack(cols, axis=-2)


def test_mrf880_signal_matches_reference_and_oracle(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("mrf880")
    sig = ts.mrf_sim(torch.from_numpy(d["flip_deg"]), 10.0, torch.from_numpy(d["t1"]),
                     torch.from_numpy(d["t2"]), B1=torch.from_numpy(d["b1"]), states=10)
    assert sig.dtype == torch.complex64 and sig.shape == (8, 880)
    sig = sig.numpy()
    assert not sig.imag.any()
    assert max_rel(sig.real, d["signal"].real) <= SIGNAL_TOL
    oracle = -O.forward(packed_from_golden(d), "f64")
    assert max_rel(sig.real, oracle) <= SIGNAL_TOL


def test_mrf880_jacobian_one_fused_pass(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("mrf880")
    names = ("T1", "T2", "B1", "M0")
    sig, jac = ts.mrf_sim(torch.from_numpy(d["flip_deg"]), 10.0, torch.from_numpy(d["t1"]),
                          torch.from_numpy(d["t2"]), B1=torch.from_numpy(d["b1"]), states=10,
                          diff=names)
    assert jac.shape == (8, 4, 880)
    jac = jac.numpy()
    p = packed_from_golden(d)
    ref = oracle_jacobian(p, names)
    for k in range(4):
        assert max_rel(jac[:, k].real, d["jacobian"][:, k].real) <= JACOBIAN_TOL, names[k]
        assert max_rel(jac[:, k].real, ref[:, k]) <= JACOBIAN_TOL, names[k]
    assert max_rel(sig.numpy().real, d["signal"].real) <= SIGNAL_TOL


def test_config0_workload(cuda):
    """1,024 voxels, the 880-pulse schedule, nstates 10, Jacobian (T1, T2)."""
    import torchsim_gb300 as ts
    from torchsim_gb300.sequence import mrf_events

    t1, t2, b1 = draw_tissue(0, 1024)
    flip = mrf_schedule()
    sig, jac = ts.mrf_sim(torch.from_numpy(flip), 10.0, torch.from_numpy(t1),
                          torch.from_numpy(t2), B1=torch.from_numpy(b1), states=10,
                          diff=("T1", "T2"))
    ev = mrf_events(flip, 10.0)
    p = packed_from_events(ev, t1, t2, 10, b1=b1)
    assert max_rel(sig.numpy().real, -O.forward(p, "f64", threads=O.cpu_threads())) <= SIGNAL_TOL
    ref = oracle_jacobian(p, ("T1", "T2"))
    for k in range(2):
        assert max_rel(jac.numpy()[:, k].real, ref[:, k]) <= JACOBIAN_TOL


def test_dictionary_workload_at_full_size(cuda):
    """The dictionary workload at its full size -- 262,144 grid atoms (T1
    geomspace(100, 4000, 128) x T2 geomspace(5, 500, 64) x B1 linspace(0.6,
    1.4, 32)), the 880-pulse schedule, nstates 20, Jacobian (T1, T2, B1) in
    one fused launch -- through properties that do not depend on its size:
    1,024 atoms spread over the grid against the FP64 oracle; the same atoms
    swept alone, bitwise equal to their rows of the full launch at the same
    launch shape; the signal against the forward-only kernel's."""
    import torchsim_gb300 as ts
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    axes = (np.geomspace(100, 4000, 128), np.geomspace(5, 500, 64), np.linspace(0.6, 1.4, 32))
    g1, g2, g3 = (x.ravel().astype(np.float32) for x in np.meshgrid(*axes, indexing="ij"))
    A = g1.size
    flip = mrf_schedule()
    T1, T2, B1 = (torch.from_numpy(x).to(cuda) for x in (g1, g2, g3))
    names = ("T1", "T2", "B1")
    rng = np.random.default_rng(11)
    pick = np.unique(np.concatenate([np.linspace(0, A - 1, 768).astype(np.int64),
                                     rng.integers(0, A, 256)]))
    idx = torch.from_numpy(pick).to(cuda)

    sig, jac = ts.mrf_sim(torch.from_numpy(flip), 10.0, T1, T2, B1=B1, states=20, diff=names)
    assert sig.shape == (A, 880) and jac.shape == (A, 3, 880)
    s, j = sig[idx].cpu().numpy(), jac[idx].cpu().numpy()
    del sig, jac
    ev = mrf_events(flip, 10.0)
    p = packed_from_events(ev, g1[pick], g2[pick], 20, b1=g3[pick])
    assert max_rel(s.real, -O.forward(p, "f64", threads=O.cpu_threads())) <= SIGNAL_TOL
    ref = oracle_jacobian(p, names)
    for k in range(3):
        assert max_rel(j[:, k].real, ref[:, k]) <= JACOBIAN_TOL, names[k]

    program = program_for(ev, cuda)
    shape = (5, 4, 4, 5)  # the register-budget shape the full launch picks
    full = engine.tissue_maps(cuda, A, T1, T2, None, B1, None)
    fs, fj = engine.forward_tangents(program, full, 20, names, launch=shape)
    alone = engine.tissue_maps(cuda, len(pick), T1[idx], T2[idx], None, B1[idx], None)
    a_s, a_j = engine.forward_tangents(program, alone, 20, names, launch=shape)
    assert torch.equal(fs[idx], a_s) and torch.equal(fj[idx], a_j)
    plain = engine.forward(program, full, 20)
    got, want = fs.cpu().numpy(), plain.cpu().numpy()
    assert np.abs(want).max() > 0 and max_rel(got, want) <= SIGNAL_TOL


def test_prepared_repeated_mrf_all_columns(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("mrf_prep")
    names = tuple(str(n) for n in d["jacobian_names"])
    sig, jac = ts.mrf_sim(torch.from_numpy(d["flip_deg"]), torch.from_numpy(d["tr_ms"]),
                          torch.from_numpy(d["t1"]), torch.from_numpy(d["t2"]),
                          B1=torch.from_numpy(d["b1"]), M0=torch.from_numpy(d["m0"]),
                          inv_efficiency=torch.from_numpy(d["inv"]), TI=float(d["ti_ms"]),
                          states=int(d["states"]), nreps=int(d["nreps"]), diff=names)
    assert max_rel(sig.numpy().real, d["signal"].real) <= SIGNAL_TOL
    for k in range(len(names)):
        assert max_rel(jac.numpy()[:, k].real, d["jacobian"][:, k].real) <= JACOBIAN_TOL, names[k]


def test_fse_cpmg_signal_and_jacobian(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("fse_cpmg")
    names = tuple(str(n) for n in d["jacobian_names"])
    sig, jac = ts.fse_sim(torch.from_numpy(d["flip_deg"]), float(d["esp_ms"]),
                          torch.from_numpy(d["t1"]), torch.from_numpy(d["t2"]), phases=90.0,
                          B1=torch.from_numpy(d["b1"]), states=int(d["states"]), diff=names)
    assert max_rel(sig.numpy(), d["signal"]) <= SIGNAL_TOL
    for k in range(len(names)):
        assert max_rel(jac.numpy()[:, k], d["jacobian"][:, k]) <= JACOBIAN_TOL, names[k]


def _entries(mode_table):
    from torchsim_gb300 import _native  # noqa: F401

    return mode_table


# Launch shapes instantiated per family (lanes_per_voxel, orders_per_lane).
SHAPES = {
    "forward": [(1, 10), (1, 20), (5, 2), (2, 6), (5, 4), (10, 2), (4, 4), (4, 6), (4, 8), (8, 4),
                (8, 8), (16, 4), (16, 8), (32, 4), (32, 8)],
    ("T1", "T2"): [(1, 10), (5, 2), (2, 6), (5, 4), (10, 2), (4, 4), (4, 6), (4, 8), (8, 4),
                   (8, 8), (16, 4), (32, 4)],
    ("T1", "T2", "B1"): [(5, 2), (2, 6), (5, 4), (10, 2), (4, 4), (4, 6), (8, 4), (16, 4),
                         (32, 4)],
    ("T1", "T2", "B1", "inv_efficiency"): [(5, 2), (5, 4), (10, 2), (4, 4), (8, 4), (16, 4),
                                           (32, 4)],
}


@pytest.mark.parametrize("family", list(SHAPES))
def test_every_launch_shape_agrees(cuda, family):
    """Each (lanes per voxel, orders per lane) kernel, with padded orders
    beyond the state count, on a ragged voxel count."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(11)
    flips = rng.uniform(5, 70, 150).astype(np.float32)
    ev = mrf_events(flips, 10.0, TI_ms=15.0)
    V = 77
    t1, t2, b1 = draw_tissue(5, V)
    inv = rng.uniform(0.8, 1.0, V).astype(np.float32)
    prog = program_for(ev, cuda)
    tissue = engine.tissue_maps(cuda, V, t1, t2, None, b1, inv)
    for lanes, orders in SHAPES[family]:
        for states in sorted({lanes * orders, max(1, lanes * orders - 3)}):
            p = packed_from_events(ev, t1, t2, states, b1=b1, inv=inv)
            ref = -O.forward(p, "f64")
            shape = (lanes, orders, 4)
            if family == "forward":
                sig = engine.forward(prog, tissue, states, launch=shape).cpu().numpy()
                assert max_rel(sig.real, ref) <= SIGNAL_TOL, (lanes, orders, states)
                continue
            sig, jac = engine.forward_tangents(prog, tissue, states, family, launch=shape)
            assert max_rel(sig.cpu().numpy().real, ref) <= SIGNAL_TOL, (lanes, orders, states)
            jref = oracle_jacobian(p, family)
            for k, name in enumerate(family):
                assert max_rel(jac.cpu().numpy()[:, k].real, jref[:, k]) <= JACOBIAN_TOL, (
                    lanes, orders, states, name)


@pytest.mark.parametrize("states", [1, 2, 3, 64, 200])
def test_state_count_edges(cuda, states):
    import torchsim_gb300 as ts
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(states)
    flips = rng.uniform(5, 90, 40).astype(np.float32)
    t1, t2, b1 = draw_tissue(3, 33)
    sig = ts.mrf_sim(torch.from_numpy(flips), 7.0, torch.from_numpy(t1), torch.from_numpy(t2),
                     B1=torch.from_numpy(b1), states=states)
    p = packed_from_events(mrf_events(flips, 7.0), t1, t2, states, b1=b1)
    assert max_rel(sig.numpy().real, -O.forward(p, "f64")) <= SIGNAL_TOL


@pytest.mark.parametrize("voxels", [0, 1, 31, 129])
def test_ragged_and_empty_voxel_counts(cuda, voxels):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    flips = np.linspace(5, 60, 50).astype(np.float32)
    ev = mrf_events(flips, 10.0)
    t1, t2, b1 = draw_tissue(9, voxels)
    tissue = engine.tissue_maps(cuda, voxels, t1, t2, None, b1, None)
    sig = engine.forward(program_for(ev, cuda), tissue, 10).cpu().numpy()
    assert sig.shape == (voxels, 50)
    if voxels:
        p = packed_from_events(ev, t1, t2, 10, b1=b1)
        assert max_rel(sig.real, -O.forward(p, "f64")) <= SIGNAL_TOL


def test_program_longer_than_one_staging_chunk(cuda):
    """3,000 repetitions: the op stream is staged through shared memory in chunks."""
    import torchsim_gb300 as ts
    from torchsim_gb300.sequence import mrf_events

    flips = (5 + 50 * np.abs(np.sin(np.arange(3000) / 70.0))).astype(np.float32)
    t1, t2, b1 = draw_tissue(4, 40)
    sig = ts.mrf_sim(torch.from_numpy(flips), 6.0, torch.from_numpy(t1), torch.from_numpy(t2),
                     B1=torch.from_numpy(b1), states=12)
    p = packed_from_events(mrf_events(flips, 6.0), t1, t2, 12, b1=b1)
    assert max_rel(sig.numpy().real, -O.forward(p, "f64")) <= SIGNAL_TOL


def test_bitwise_deterministic(cuda):
    import torchsim_gb300 as ts

    t1, t2, b1 = draw_tissue(8, 500)
    args = (torch.from_numpy(mrf_schedule()), 10.0, torch.from_numpy(t1), torch.from_numpy(t2))
    a = ts.mrf_sim(*args, B1=torch.from_numpy(b1), diff=("T1", "T2"))
    b = ts.mrf_sim(*args, B1=torch.from_numpy(b1), diff=("T1", "T2"))
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_voxel_result_independent_of_batch(cuda):
    """A voxel's samples do not depend on which voxels share its launch."""
    import torchsim_gb300 as ts

    t1, t2, b1 = draw_tissue(12, 300)
    flip = torch.from_numpy(mrf_schedule())
    full = ts.mrf_sim(flip, 10.0, torch.from_numpy(t1), torch.from_numpy(t2),
                      B1=torch.from_numpy(b1))
    part = ts.mrf_sim(flip, 10.0, torch.from_numpy(t1[100:137]), torch.from_numpy(t2[100:137]),
                      B1=torch.from_numpy(b1[100:137]))
    assert torch.equal(full[100:137], part)


# ---- the C ABI drop-ins with host buffers ---------------------------------


def _pointer_array(arrays):
    ptrs = (ctypes.c_void_p * len(arrays))()
    for i, a in enumerate(arrays):
        ptrs[i] = None if a is None else a.ctypes.data
    return ptrs


TISSUE_ORDER = ("t1_ms", "t2_ms", "m0", "b1", "b1_phase_rad", "b0_hz", "inversion_efficiency",
                "diffusion_um2_per_ms", "velocity_m_per_s", "bound_fraction", "bound_exchange_hz",
                "t1_bound_ms", "pool_b_fraction", "pool_b_exchange_hz", "t1_pool_b_ms",
                "t2_pool_b_ms", "pool_b_shift_hz")
EVENT_ORDER = ("duration", "kind", "flip", "phase", "action", "output_index", "shim_index",
               "saturation", "rf_frequency_hz")
# Transmit, density and inversion terms on (_epg_cpu.cpp:91-98).
FEATURES = 8 | 16 | 32


def _packed_arrays(d):
    tissue = [np.ascontiguousarray(d["tissue_" + n]) for n in TISSUE_ORDER]
    events = [np.ascontiguousarray(d["event_" + n]) for n in EVENT_ORDER]
    return tissue, events


def test_dropin_simulate_host_buffers(built_library, cuda, golden):
    from torchsim_gb300 import _native

    d = golden("mrf880")
    tissue, events = _packed_arrays(d)
    V, P = 8, 880
    out_r = np.full((V, P), 7.0, np.float32)
    out_i = np.zeros((V, P), np.float32)
    arrays = [*tissue, *events, out_r, out_i, *([None] * 13)]
    ptrs = _pointer_array(arrays)
    _native.check(built_library.tsg_epg_simulate(ptrs, len(arrays), V, 1, d["event_kind"].size, 10,
                                                 P, 1, FEATURES))
    assert not out_r.any()
    assert max_rel(out_i, d["raw_forward"].imag) <= SIGNAL_TOL


def test_dropin_rejects_outside_subset(built_library, cuda, golden):
    from torchsim_gb300 import _native

    d = golden("mrf880")
    tissue, events = _packed_arrays(d)
    out = np.zeros((8, 880), np.float32)
    arrays = [*tissue, *events, out, out.copy(), *([None] * 13)]
    ptrs = _pointer_array(arrays)
    n = d["event_kind"].size
    assert built_library.tsg_epg_simulate_jvp(ptrs, len(arrays), 8, 1, n, 10, 880, -1,
                                              FEATURES) != 0
    assert built_library.tsg_epg_simulate(ptrs, len(arrays) - 1, 8, 1, n, 10, 880, 1,
                                          FEATURES) == _native.TSG_ERR_ARGUMENT
    assert built_library.tsg_epg_simulate(ptrs, len(arrays), 8, 1, n, 0, 880, 1,
                                          FEATURES) == _native.TSG_ERR_ARGUMENT


@pytest.mark.parametrize("name", ["fse_phase0", "mrf_offaxis"])
def test_dropin_simulate_complex_path(built_library, cuda, golden, name):
    """real_axis = -1: the drop-in runs the complex kernel, as the reference's
    simulate switches to simulate_range."""
    from torchsim_gb300 import _native

    d = golden(name)
    tissue, events = _packed_arrays(d)
    V, P = d["raw_forward"].shape
    out_r = np.full((V, P), 7.0, np.float32)
    out_i = np.full((V, P), 7.0, np.float32)
    arrays = [*tissue, *events, out_r, out_i, *([None] * 13)]
    ptrs = _pointer_array(arrays)
    features = FEATURES | 1  # off-axis buffers present
    _native.check(built_library.tsg_epg_simulate(ptrs, len(arrays), V, 1, d["event_kind"].size,
                                                 int(d["states"]), P, -1, features))
    assert max_rel(out_r + 1j * out_i, d["raw_forward"]) <= SIGNAL_TOL


def test_dropin_jvp_general_direction(built_library, cuda, golden):
    """Tissue, duration and flip directions at once, against the oracle."""
    from torchsim_gb300 import _native

    d = golden("mrf_prep")
    tissue, events = _packed_arrays(d)
    V, P, E = 5, 60, d["event_kind"].size
    rng = np.random.default_rng(5)
    tangents = [np.zeros(V, np.float32) for _ in range(17)] + [
        np.zeros(E, np.float32), np.zeros(E, np.float32), np.zeros(E, np.float32)]
    tangents[0] = rng.standard_normal(V).astype(np.float32) * 50
    tangents[1] = rng.standard_normal(V).astype(np.float32) * 5
    tangents[2] = rng.standard_normal(V).astype(np.float32)
    tangents[3] = rng.standard_normal(V).astype(np.float32) * 0.1
    tangents[6] = rng.standard_normal(V).astype(np.float32) * 0.1
    tangents[17] = rng.standard_normal(E).astype(np.float32) * 1e-3  # every event's duration
    tangents[18] = rng.standard_normal(E).astype(np.float32) * 0.1
    out_r = np.zeros((V, P), np.float32)
    out_i = np.zeros((V, P), np.float32)
    arrays = [*tissue, *events, *tangents, out_r, out_i, *([None] * 13)]
    ptrs = _pointer_array(arrays)
    _native.check(built_library.tsg_epg_simulate_jvp(ptrs, len(arrays), V, 1, E, 7, P, 1,
                                                     FEATURES))
    p = packed_from_golden(d)
    ref = O.tangent(p, "f64", t1_ms=tangents[0], t2_ms=tangents[1], m0=tangents[2],
                    b1=tangents[3], inversion=tangents[6], duration_s=tangents[17],
                    flip_rad=tangents[18])
    assert max_rel(out_i, ref) <= JACOBIAN_TOL
    assert not out_r.any()


def test_dropin_several_trains(built_library, cuda):
    """train_count > 1: per-train flips and durations over shared structure."""
    from torchsim_gb300 import _native
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(21)
    trains, V, S = 3, 19, 9
    base = mrf_events(rng.uniform(5, 60, 30).astype(np.float32), 10.0)
    E = base.events
    dur = np.stack([base.duration[0] * (1 + 0.1 * k) for k in range(trains)]).astype(np.float32)
    flip = np.stack([base.flip[0] * (1 + 0.2 * k) for k in range(trains)]).astype(np.float32)
    t1, t2, b1 = draw_tissue(2, V)
    zeros = np.zeros(V, np.float32)
    tissue = [t1, t2, np.ones(V, np.float32), b1, zeros, zeros, np.ones(V, np.float32),
              *([zeros] * 10)]
    events = [dur, base.kind, flip, np.zeros_like(flip), base.action, base.output_index,
              np.zeros(E, np.int32), np.zeros(E, np.float32), np.zeros(E, np.float32)]
    out_r = np.zeros((trains, V, 30), np.float32)
    out_i = np.zeros((trains, V, 30), np.float32)
    arrays = [*tissue, *events, out_r, out_i, *([None] * 13)]
    _native.check(built_library.tsg_epg_simulate(_pointer_array(arrays), len(arrays), V, trains,
                                                 E, S, 30, 1, FEATURES))
    p = O.Packed(t1, t2, dur, base.kind, flip, base.action, base.output_index, S, b1=b1)
    assert max_rel(out_i, O.forward(p, "f64")) <= SIGNAL_TOL


def test_dropin_simulate_in_chunks(built_library, cuda, golden):
    """A single-train drop-in call large enough to run in chunks (65,536
    atoms x 880 samples, rows three samples wider than the program's
    outputs): every chunk's rows equal the fixture's reference forward, the
    real plane and the extra columns are zero."""
    from torchsim_gb300 import _native

    d = golden("mrf880")
    tissue, events = _packed_arrays(d)
    reps = 8192
    V, P, W = 8 * reps, 880, 883
    tissue = [np.ascontiguousarray(np.tile(a, reps)) if a.size == 8 else a for a in tissue]
    out_r = np.full((V, W), 7.0, np.float32)
    out_i = np.full((V, W), 7.0, np.float32)
    arrays = [*tissue, *events, out_r, out_i, *([None] * 13)]
    ptrs = _pointer_array(arrays)
    _native.check(built_library.tsg_epg_simulate(ptrs, len(arrays), V, 1, d["event_kind"].size, 10,
                                                 W, 1, FEATURES))
    assert not out_r.any()
    assert not out_i[:, P:].any()
    want = np.tile(d["raw_forward"].imag, (reps, 1))
    assert max_rel(out_i[:, :P], want) <= SIGNAL_TOL
