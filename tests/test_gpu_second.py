"""GPU parity of the second-order sweeps (the adjoint of the tangent sweep).

Against the reference's own forward-over-reverse results (the committed
fixture: the two column calls of a Cramer-Rao design and a direct call along
every tissue property, duration and flip) through the host-buffer drop-in of
``_epg_cpu.simulate_vjp_jvp``; the fused K-direction sweep against the sum of
the FP64 oracle's single-direction calls; the public route (a Cramer-Rao cost
of ``MRFSimulator.jacobian`` backpropagated to the flip angles and TRs)
against the reference's gradients; and a directional derivative of that cost
against central differences of the FP64 oracle's Jacobian.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import draw_tissue, max_rel, packed_from_events, packed_from_golden

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
SECOND_NAMES = {"t1_ms": "t1_ms", "t2_ms": "t2_ms", "m0": "m0", "b1": "b1",
                "inversion": "inversion_efficiency", "flip_rad": "flip",
                "duration_s": "duration"}


@pytest.mark.parametrize("prefix", ["design0_", "design1_", "direct_"])
def test_dropin_vjp_jvp_matches_reference(built_library, cuda, golden, prefix):
    """All 40 gradient slots of the drop-in against the reference's kernel."""
    from tests.test_gpu_parity import EVENT_ORDER, FEATURES, TISSUE_ORDER, _pointer_array
    from torchsim_gb300 import _native

    d = golden("mrf_second")
    seed = d[prefix + "seed"]
    V, P = seed.shape
    E = d[prefix + "event_kind"].size
    tissue = [np.ascontiguousarray(d[prefix + "tissue_" + n]) for n in TISSUE_ORDER]
    events = [np.ascontiguousarray(d[prefix + "event_" + n]) for n in EVENT_ORDER]
    slots = (*TISSUE_ORDER, "duration", "flip", "phase")
    tangents = [np.ascontiguousarray(d[f"{prefix}tangent_{n}"], dtype=np.float32) for n in slots]
    seeds = [np.ascontiguousarray(seed.real), np.ascontiguousarray(seed.imag)]
    values = [np.full(V if i < 17 else E, 9.0, np.float32) for i in range(20)]
    curves = [np.full(V if i < 17 else E, 9.0, np.float32) for i in range(20)]
    arrays = [*tissue, *events, *tangents, *seeds, *values, *curves, *([None] * 13)]
    _native.check(built_library.tsg_epg_simulate_vjp_jvp(
        _pointer_array(arrays), len(arrays), V, 1, E, int(d["states"]), P, 1, FEATURES))
    for name, got_v, got_c in zip(slots, values, curves, strict=True):
        # Directions outside the real subspace, and diffusion (whose damping
        # is not built; the reference forms its derivative even at zero
        # diffusion), are written as zero.
        if name in ("b1_phase_rad", "b0_hz", "phase", "diffusion_um2_per_ms") or \
                f"{prefix}value_{name}" not in d.files:
            assert not got_v.any() and not got_c.any(), name
            continue
        assert max_rel(got_v, d[f"{prefix}value_{name}"]) <= GRAD_TOL, ("value", name)
        assert max_rel(got_c, d[f"{prefix}curvature_{name}"]) <= GRAD_TOL, ("curvature", name)


def test_dropin_vjp_jvp_rejects_bad_calls(built_library):
    from torchsim_gb300 import _native

    ptrs = (__import__("ctypes").c_void_p * 101)()
    assert built_library.tsg_epg_simulate_vjp_jvp(ptrs, 100, 1, 1, 1, 4, 1, 1, 0) == \
        _native.TSG_ERR_ARGUMENT
    assert built_library.tsg_epg_simulate_vjp_jvp(ptrs, 101, 1, 1, 1, 4, 1, -1, 0) == \
        _native.TSG_ERR_UNSUPPORTED


def _case(seed, voxels, pulses, states, ti=12.0):
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(seed)
    flips = rng.uniform(5, 70, pulses).astype(np.float32)
    trs = rng.uniform(8, 15, pulses).astype(np.float32)
    ev = mrf_events(flips, trs, TI_ms=ti)
    t1, t2, b1 = draw_tissue(seed + 1, voxels)
    m0 = rng.uniform(0.5, 1.5, voxels).astype(np.float32)
    return rng, flips, trs, ev, t1, t2, b1, m0


@pytest.mark.parametrize("names,states,shape", [
    (("T1",), 8, None), (("T1", "T2"), 12, None), (("T1", "T2", "B1"), 20, None),
    (("T2", "B1"), 33, None), (("T1", "T2", "B1"), 20, (10, 2, 0)), (("T1", "T2"), 12, (10, 2, 0)),
    (("B1",), 7, (4, 2, 0)), (("T1", "T2", "B1"), 20, (8, 4, 0))])
def test_fused_directions_match_the_oracle(cuda, names, states, shape):
    """One reverse sweep over K one-hot directions (and the signal's own
    cotangent) against the FP64 oracle: the first-order adjoint of the signal
    seed plus, per direction, the forward-over-reverse call with its seed."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import program_for

    rng, flips, trs, ev, t1, t2, b1, m0 = _case(41, 37, 60, states)
    V = t1.size
    prog = program_for(ev, cuda)
    tissue = engine.tissue_maps(cuda, V, t1, t2, m0, b1, None)
    ones = torch.ones(V, device=cuda)
    directions = [{engine.DIRECTION_OF[n]: ones} for n in names]
    sig, jac, traj, ws = engine.second_forward(prog, tissue, states, directions, launch=shape)
    p = packed_from_events(ev, t1, t2, states, m0=m0, b1=b1)
    key = {"T1": "t1_ms", "T2": "t2_ms", "B1": "b1"}
    # Forward: signal and derivatives (1j * values).
    assert max_rel(sig.real.cpu().numpy(), -O.forward(p, "f64")) <= 1e-5
    for k, n in enumerate(names):
        ref = -O.tangent(p, "f64", **{key[n]: 1.0})
        assert max_rel(jac[:, k].real.cpu().numpy(), ref) <= GRAD_TOL, n
    s0 = rng.standard_normal((V, ev.outputs)).astype(np.float32)
    sk = rng.standard_normal((V, len(names), ev.outputs)).astype(np.float32)
    # Cotangents of 1j * (value): the imaginary-plane seed is minus the real part.
    seed_sig = torch.from_numpy((-s0).astype(np.complex64)).to(cuda)
    seed_jac = torch.from_numpy((-sk).astype(np.complex64)).to(cuda)
    curvature = {n: torch.zeros(V, device=cuda) for n in ("t1_ms", "t2_ms", "m0", "b1")}
    curvature["flip_rad"] = torch.zeros((1, ev.events), device=cuda)
    curvature["duration_s"] = torch.zeros((1, ev.events), device=cuda)
    values = [{n: torch.zeros(V, device=cuda) for n in ("t1_ms", "t2_ms", "m0", "b1")}
              for _ in names]
    engine.second_reverse(prog, tissue, states, directions, seed_jac, traj, ws,
                          seed_signal=seed_sig, curvature=curvature, values=values, launch=shape)
    want = O.adjoint(p, s0, "f64")
    want_values = []
    for k, n in enumerate(names):
        v, c = O.second(p, sk[:, k], "f64", **{key[n]: 1.0})
        want_values.append(v)
        for g in want:
            want[g] = want[g] + c[g]
    for g in ("t1_ms", "t2_ms", "m0", "b1", "flip_rad"):
        got = curvature[g].cpu().numpy().reshape(want[g].shape)
        assert max_rel(got, want[g]) <= GRAD_TOL, g
    # Durations: events of zero duration fold into the op before them on the
    # merged program, so only the others are formed.
    dur = curvature["duration_s"].cpu().numpy()[0]
    formed = ev.duration.reshape(-1) != 0
    assert max_rel(dur[formed], want["duration_s"][formed]) <= GRAD_TOL
    for k, n in enumerate(names):
        for g in ("t1_ms", "t2_ms", "m0", "b1"):
            assert max_rel(values[k][g].cpu().numpy(), want_values[k][g]) <= GRAD_TOL, (n, g)


@pytest.mark.parametrize("names,states,shape", [
    (("T1",), 8, None), (("T2", "B1"), 12, None), (("T1", "T2", "B1"), 20, None),
    (("T1", "T2", "B1"), 20, (5, 4, 0)), (("T1", "B1"), 33, (32, 2, 0)), (("T1", "T2"), 6, (2, 4, 0))])
def test_design_sweep_matches_the_oracle(cuda, names, states, shape):
    """The one-hot design sweeps (no per-voxel or per-event directions): the
    curvature of the signal seed plus the derivatives' seeds, and an M0
    column, against the FP64 oracle."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import program_for

    rng, flips, trs, ev, t1, t2, b1, m0 = _case(43, 29, 50, states)
    V = t1.size
    prog = program_for(ev, cuda)
    tissue = engine.tissue_maps(cuda, V, t1, t2, m0, b1, None)
    mask = sum(engine.DESIGN_BITS[n] for n in names)
    sig, jac, traj = engine.design_forward(prog, tissue, states, mask, with_m0=True, launch=shape)
    p = packed_from_events(ev, t1, t2, states, m0=m0, b1=b1)
    key = {"T1": "t1_ms", "T2": "t2_ms", "B1": "b1"}
    assert max_rel(sig.real.cpu().numpy(), -O.forward(p, "f64")) <= 1e-5
    for k, n in enumerate(names):
        assert max_rel(jac[:, k].real.cpu().numpy(), -O.tangent(p, "f64", **{key[n]: 1.0})) <= \
            GRAD_TOL, n
    p0 = O.forward(p, "f64") / m0[:, None]
    assert max_rel(jac[:, -1].real.cpu().numpy(), -p0) <= 1e-5
    s0 = rng.standard_normal((V, ev.outputs)).astype(np.float32)
    sk = rng.standard_normal((V, len(names) + 1, ev.outputs)).astype(np.float32)
    curvature = {n: torch.zeros(V, device=cuda) for n in ("t1_ms", "t2_ms", "m0", "b1")}
    curvature["flip_rad"] = torch.zeros((1, ev.events), device=cuda)
    engine.design_reverse(prog, tissue, states, mask,
                          torch.from_numpy((-sk).astype(np.complex64)).to(cuda), traj,
                          seed_signal=torch.from_numpy((-s0).astype(np.complex64)).to(cuda),
                          with_m0=True, curvature=curvature, launch=shape)
    # The M0 column's seed acts on F+[0] = signal / m0.
    want = O.adjoint(p, s0 + sk[:, -1] / m0[:, None], "f64")
    want["m0"] = want["m0"] - (sk[:, -1] * p0).sum(1) / m0
    for k, n in enumerate(names):
        _, c = O.second(p, sk[:, k], "f64", **{key[n]: 1.0})
        for g in want:
            want[g] = want[g] + c[g]
    for g in ("t1_ms", "t2_ms", "m0", "b1", "flip_rad"):
        got = curvature[g].cpu().numpy().reshape(want[g].shape)
        assert max_rel(got, want[g]) <= GRAD_TOL, g


def test_m0_column_and_order(cuda):
    """An M0 column (F+[0] itself, no tangent state) and columns in the
    caller's order: the backward of the public Jacobian against the oracle."""
    from torchsim_gb300 import MRFSimulator

    rng, flips, trs, ev, t1, t2, b1, m0 = _case(5, 9, 40, 10, ti=0.0)
    names = ("M0", "T2", "T1")
    theta = torch.tensor(flips, device=cuda, requires_grad=True)
    m0t = torch.tensor(m0, device=cuda, requires_grad=True)
    sim = MRFSimulator(flip=theta, TR=torch.tensor(trs), states=10)
    sig, jac = sim.jacobian(names, T1=torch.tensor(t1, device=cuda),
                            T2=torch.tensor(t2, device=cuda), B1=torch.tensor(b1, device=cuda),
                            M0=m0t)
    w = torch.from_numpy(rng.standard_normal(jac.shape).astype(np.float32)).to(cuda)
    loss = (w * jac.real).sum()
    loss.backward()
    p = packed_from_events(ev, t1, t2, 10, m0=m0, b1=b1)
    # jac.real = -(derivative of m0*F+[0]): the oracle's seeds are -w.
    wn = -w.cpu().numpy()
    want_m0 = np.zeros(t1.size)
    want_flip = np.zeros(ev.events)
    for k, n in enumerate(names):
        if n == "M0":
            # <w, F+[0]>: F+[0] = signal / m0, so its flip gradient is the
            # first-order adjoint of the seed w / m0; it does not depend on m0.
            want_flip += O.adjoint(p, wn[:, k] / m0[:, None], "f64")["flip_rad"]
            continue
        _, c = O.second(p, wn[:, k], "f64", **{{"T1": "t1_ms", "T2": "t2_ms"}[n]: 1.0})
        want_flip += c["flip_rad"]
        want_m0 += c["m0"]
    from torchsim_gb300.sequence import mrf_gradient_map, played_flip_torch

    where = mrf_gradient_map(flips.size, 1)["flip"].reshape(-1)
    deg = torch.tensor(flips, requires_grad=True)
    played_flip_torch(deg).sum().backward()
    want_deg = want_flip[where] * deg.grad.numpy()
    assert max_rel(theta.grad.cpu().numpy(), want_deg) <= GRAD_TOL
    assert max_rel(m0t.grad.cpu().numpy(), want_m0) <= GRAD_TOL


def test_crlb_design_matches_reference(cuda, golden):
    """The reference's design cost (the Cramer-Rao bound of a (T1, T2)
    Jacobian, relative to T^2) differentiated with respect to flip angle and
    TR through the public simulator."""
    from torchsim_gb300 import MRFSimulator, crlb

    d = golden("mrf_second")
    theta = torch.tensor(d["flip_deg"], device=cuda, requires_grad=True)
    tau = torch.tensor(d["tr_ms"], device=cuda, requires_grad=True)
    tissue = {k: torch.tensor(d[v], device=cuda) for k, v in
              (("T1", "t1"), ("T2", "t2"), ("B1", "b1"), ("M0", "m0"))}
    sig, jac = MRFSimulator(flip=theta, TR=tau, states=int(d["states"])).jacobian(
        ("T1", "T2"), **tissue)
    assert max_rel(jac.detach().cpu().numpy(), d["jacobian"]) <= GRAD_TOL
    scale = torch.stack((tissue["T1"], tissue["T2"]), dim=-1)
    loss = (crlb(jac) / scale.square()).sum()
    loss.backward()
    assert abs(loss.item() - float(d["loss"])) <= 1e-3 * abs(float(d["loss"]))
    assert max_rel(theta.grad.cpu().numpy(), d["grad_flip_deg"]) <= 1e-3
    assert max_rel(tau.grad.cpu().numpy(), d["grad_tr_ms"]) <= 1e-3


def test_design_gradient_matches_finite_differences(cuda):
    """A directional derivative of a Cramer-Rao cost at 20 states against
    central differences of the same cost built from the FP64 oracle's
    Jacobian."""
    from torchsim_gb300 import MRFSimulator, crlb
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(12)
    pulses, V, S = 80, 16, 20
    flips = rng.uniform(5, 70, pulses)
    trs = rng.uniform(8, 15, pulses)
    t1, t2, b1 = draw_tissue(13, V)

    def cost_oracle(fl, tr):
        ev = mrf_events(fl.astype(np.float32), tr.astype(np.float32))
        p = packed_from_events(ev, t1, t2, S, b1=b1)
        j = np.stack([O.tangent(p, "f64", t1_ms=1.0), O.tangent(p, "f64", t2_ms=1.0)], axis=1)
        fisher = np.einsum("vps,vqs->vpq", j, j)
        bound = np.diagonal(np.linalg.inv(fisher), axis1=1, axis2=2)
        return float((bound / np.stack([t1, t2], 1).astype(np.float64) ** 2).sum())

    theta = torch.tensor(flips.astype(np.float32), device=cuda, requires_grad=True)
    tau = torch.tensor(trs.astype(np.float32), device=cuda, requires_grad=True)
    _, jac = MRFSimulator(flip=theta, TR=tau, states=S).jacobian(
        ("T1", "T2"), T1=torch.tensor(t1, device=cuda), T2=torch.tensor(t2, device=cuda),
        B1=torch.tensor(b1, device=cuda))
    scale = torch.stack((torch.tensor(t1), torch.tensor(t2)), -1).to(cuda)
    loss = (crlb(jac) / scale.square()).sum()
    loss.backward()
    vf = rng.standard_normal(pulses)
    vt = rng.standard_normal(pulses)
    # Steps of 0.1 deg and 0.1 ms keep the FP32 rounding of the stepped
    # stream well below the difference.
    h = 0.1
    fd = (cost_oracle(flips + h * vf, trs + h * vt) - cost_oracle(flips - h * vf, trs - h * vt)) / (2 * h)
    got = float((theta.grad.cpu().numpy() * vf).sum() + (tau.grad.cpu().numpy() * vt).sum())
    assert abs(got - fd) <= 1e-3 * max(abs(fd), 1e-12), (got, fd)


def test_second_order_is_deterministic(cuda):
    from torchsim_gb300 import MRFSimulator, crlb

    rng = np.random.default_rng(3)
    flips = rng.uniform(5, 70, 50).astype(np.float32)
    t1, t2, b1 = draw_tissue(4, 300)

    def grad():
        theta = torch.tensor(flips, device=cuda, requires_grad=True)
        _, jac = MRFSimulator(flip=theta, TR=10.0, states=16).jacobian(
            ("T1", "T2", "B1"), T1=torch.tensor(t1, device=cuda),
            T2=torch.tensor(t2, device=cuda), B1=torch.tensor(b1, device=cuda))
        crlb(jac).sum().backward()
        return theta.grad.clone()

    first = grad()
    for _ in range(2):
        assert torch.equal(first, grad())
