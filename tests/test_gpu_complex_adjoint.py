"""GPU parity of the complex path's first-order adjoint.

Against the reference's own gradients (the committed fixture: an off-axis
MRF with B0, B1phase and M0 maps and every tissue map, flip and TR a leaf; a
default-phase CPMG with its refocusing flips and tissue as leaves), through
the host-buffer drop-in and through the public simulators, and against the
FP64 oracle's complex adjoint on larger cases at every launch shape family.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import draw_tissue, max_rel

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
SLOTS = ("t1_ms", "t2_ms", "m0", "b1", "b1_phase_rad", "b0_hz", "inversion_efficiency")


def _scale(d, prefix):
    names = [*SLOTS, "duration", "flip", "phase"]
    return max(float(np.abs(d[f"{prefix}grad_{n}"]).max()) for n in names)


def _close(got, want, scale):
    """max-rel, or absolute against the other slots' scale where the
    reference's gradient is rounding noise (B0 and B1phase on resonance)."""
    if np.abs(want).max() < 1e-6 * scale:
        return np.abs(got).max() <= 1e-5 * scale
    return max_rel(got, want) <= GRAD_TOL


@pytest.mark.parametrize("case", ["mrf", "fse"])
def test_dropin_complex_vjp_matches_reference(built_library, cuda, golden, case):
    from tests.test_gpu_parity import EVENT_ORDER, TISSUE_ORDER, _pointer_array
    from torchsim_gb300 import _native

    d = golden("complex_adjoint")
    prefix = f"{case}_vjp_"
    seed = d[prefix + "seed"]
    V, P = seed.shape
    E = d[prefix + "event_kind"].size
    tissue = [np.ascontiguousarray(d[prefix + "tissue_" + n]) for n in TISSUE_ORDER]
    events = [np.ascontiguousarray(d[prefix + "event_" + n]) for n in EVENT_ORDER]
    seeds = [np.ascontiguousarray(seed.real), np.ascontiguousarray(seed.imag)]
    grads = [np.full(V, 9.0, np.float32) for _ in range(17)] + [np.full(E, 9.0, np.float32)
                                                                  for _ in range(3)]
    arrays = [*tissue, *events, *seeds, *grads, *([None] * 13)]
    features = 1 | 8 | 16 | 32  # off-axis, transmit, density, inversion
    _native.check(built_library.tsg_epg_simulate_vjp(_pointer_array(arrays), len(arrays), V, 1, E,
                                                     int(d[f"{case}_states"]), P, -1, features))
    names = [*TISSUE_ORDER, "flip", "phase", "duration"]
    scale = _scale(d, prefix)
    for name, got in zip(names, grads, strict=True):
        if name in (*SLOTS, "flip", "phase", "duration"):
            assert _close(got, d[f"{prefix}grad_{name}"], scale), name
        else:
            assert not got.any(), name


def test_public_mrf_offaxis_gradients_match_reference(cuda, golden):
    from torchsim_gb300 import MRFSimulator

    d = golden("complex_adjoint")
    leaves = {k: torch.tensor(d[f"mrf_{v}"], device=cuda, requires_grad=True) for k, v in
              (("T1", "t1"), ("T2", "t2"), ("B1", "b1"), ("B0", "b0"), ("B1phase", "b1_phase"),
               ("M0", "m0"))}
    theta = torch.tensor(d["mrf_flip_deg"], device=cuda, requires_grad=True)
    tau = torch.tensor(d["mrf_tr_ms"], device=cuda, requires_grad=True)
    sig = MRFSimulator(flip=theta, TR=tau, TI=15.0, states=int(d["mrf_states"])).simulate(**leaves)
    assert max_rel(sig.detach().cpu().numpy(), d["mrf_signal"]) <= 1e-5
    loss = (sig - torch.as_tensor(d["mrf_target"], device=cuda)).abs().square().sum()
    loss.backward()
    assert abs(loss.item() - float(d["mrf_loss"])) <= 1e-4 * abs(float(d["mrf_loss"]))
    assert max_rel(theta.grad.cpu().numpy(), d["mrf_grad_flip_deg"]) <= GRAD_TOL
    assert max_rel(tau.grad.cpu().numpy(), d["mrf_grad_tr_ms"]) <= GRAD_TOL
    for k, v in leaves.items():
        assert max_rel(v.grad.cpu().numpy(), d[f"mrf_grad_{k}"]) <= GRAD_TOL, k


def test_public_default_phase_fse_gradients_match_reference(cuda, golden):
    from torchsim_gb300 import FSESimulator

    d = golden("complex_adjoint")
    leaves = {k: torch.tensor(d[f"fse_{v}"], device=cuda, requires_grad=True) for k, v in
              (("T1", "t1"), ("T2", "t2"), ("B1", "b1"))}
    phi = torch.tensor(d["fse_flip_deg"], device=cuda, requires_grad=True)
    sig = FSESimulator(flip=phi, ESP=float(d["fse_esp_ms"]),
                       states=int(d["fse_states"])).simulate(**leaves)
    assert max_rel(sig.detach().cpu().numpy(), d["fse_signal"]) <= 1e-5
    loss = (sig - torch.as_tensor(d["fse_target"], device=cuda)).abs().square().sum()
    loss.backward()
    assert max_rel(phi.grad.cpu().numpy(), d["fse_grad_flip_deg"]) <= GRAD_TOL
    for k, v in leaves.items():
        assert max_rel(v.grad.cpu().numpy(), d[f"fse_grad_{k}"]) <= GRAD_TOL, k


@pytest.mark.parametrize("states,shape", [(8, None), (20, None), (20, (5, 4, 0)), (33, None),
                                          (12, (4, 4, 0)), (6, (2, 4, 0))])
def test_complex_adjoint_matches_the_oracle(cuda, states, shape):
    """Off-axis MRF with RF phases and an inversion, 41 voxels: every gradient
    of the kernel against the FP64 oracle."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(17)
    pulses = 48
    flips = rng.uniform(5, 70, pulses).astype(np.float32)
    trs = rng.uniform(8, 15, pulses).astype(np.float32)
    ev = mrf_events(flips, trs, TI_ms=10.0, phases_deg=rng.uniform(-40, 40, pulses))
    V = 41
    t1, t2, b1 = draw_tissue(18, V)
    m0 = rng.uniform(0.5, 1.5, V).astype(np.float32)
    b0 = rng.uniform(-40, 40, V).astype(np.float32)
    b1p = rng.uniform(-0.5, 0.5, V).astype(np.float32)
    inv = rng.uniform(0.8, 1.0, V).astype(np.float32)
    prog = program_for(ev, cuda, phased=True)
    tissue = engine.tissue_maps(cuda, V, t1, t2, m0, b1, inv)
    off, keep = engine.offaxis_maps(cuda, V, b1p, b0)
    sig, traj = engine.forward_complex_trajectory(prog, tissue, states, off, launch=shape)
    p = O.Packed(t1, t2, ev.duration, ev.kind, ev.flip, ev.action, ev.output_index, states, m0=m0,
                 b1=b1, inversion=inv)
    p.phase_rad, p.b1_phase_rad, p.b0_hz = ev.phase, b1p, b0
    ref = O.forward_complex(p, "f64")
    assert max_rel(sig.cpu().numpy(), 1j * ref) <= 1e-5
    seed = (rng.standard_normal((V, ev.outputs)) + 1j * rng.standard_normal((V, ev.outputs)))
    seed = seed.astype(np.complex64)
    grads = {n: torch.zeros(V, device=cuda) for n in engine.COMPLEX_GRAD_NAMES[:7]}
    for n in engine.COMPLEX_GRAD_NAMES[7:]:
        grads[n] = torch.zeros((1, ev.events), device=cuda)
    engine.adjoint_complex(prog, tissue, states, torch.from_numpy(seed).to(cuda), traj, grads, off,
                           launch=shape)
    want = O.adjoint_complex(p, seed, "f64")
    for name in ("t1_ms", "t2_ms", "m0", "b1", "inversion", "b1_phase_rad", "b0_hz", "flip_rad",
                 "phase_rad"):
        got = grads[name].cpu().numpy().reshape(want[name].shape)
        assert max_rel(got, want[name]) <= GRAD_TOL, name
    # Zero-duration events fold into the op before them on the merged
    # program; the others' duration gradients are formed.
    formed = ev.duration.reshape(-1) != 0
    dur = grads["duration_s"].cpu().numpy()[0]
    assert max_rel(dur[formed], want["duration_s"][formed]) <= GRAD_TOL


def test_complex_adjoint_is_deterministic(cuda):
    from torchsim_gb300 import MRFSimulator

    rng = np.random.default_rng(2)
    flips = rng.uniform(5, 70, 40).astype(np.float32)
    t1, t2, b1 = draw_tissue(3, 500)
    b0 = torch.tensor(rng.uniform(-30, 30, 500).astype(np.float32), device=cuda)

    def grad():
        theta = torch.tensor(flips, device=cuda, requires_grad=True)
        sig = MRFSimulator(flip=theta, TR=10.0, states=12).simulate(
            T1=torch.tensor(t1, device=cuda), T2=torch.tensor(t2, device=cuda),
            B1=torch.tensor(b1, device=cuda), B0=b0)
        sig.abs().square().sum().backward()
        return theta.grad.clone()

    first = grad()
    for _ in range(2):
        assert torch.equal(first, grad())
