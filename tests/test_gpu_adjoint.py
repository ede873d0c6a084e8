"""GPU parity of the checkpointed adjoint kernel.

Against the reference's own gradients (the committed fixture of a loss
backpropagated through its MRF simulator), against the FP64 oracle's adjoint
(including every event's duration gradient through the host-buffer drop-in),
and against central finite differences of the FP64 oracle's loss.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import draw_tissue, max_rel, packed_from_events, packed_from_golden

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4


def _loss_grads(flip, tr, t1, t2, b1, target, states, device, ops_per_checkpoint=None):
    from torchsim_gb300 import MRFSimulator

    theta = torch.tensor(flip, device=device, requires_grad=True)
    tau = torch.tensor(tr, device=device, requires_grad=True)
    t1t = torch.tensor(t1, device=device, requires_grad=True)
    t2t = torch.tensor(t2, device=device, requires_grad=True)
    b1t = torch.tensor(b1, device=device, requires_grad=True)
    sig = MRFSimulator(flip=theta, TR=tau, states=states).simulate(T1=t1t, T2=t2t, B1=b1t)
    loss = (sig - torch.as_tensor(target, device=device)).abs().square().sum()
    loss.backward()
    return {"loss": loss.item(), "flip": theta.grad.cpu().numpy(), "tr": tau.grad.cpu().numpy(),
            "t1": t1t.grad.cpu().numpy(), "t2": t2t.grad.cpu().numpy(),
            "b1": b1t.grad.cpu().numpy(), "signal": sig.detach().cpu().numpy()}


def test_adjoint_matches_reference_gradients(cuda, golden):
    d = golden("mrf_adjoint")
    g = _loss_grads(d["flip_deg"], d["tr_ms"], d["t1"], d["t2"], d["b1"], d["target"],
                    int(d["states"]), cuda)
    assert max_rel(g["signal"], d["signal"]) <= 1e-5
    assert abs(g["loss"] - float(d["loss"])) <= 1e-4 * abs(float(d["loss"]))
    for mine, ref in (("flip", "grad_flip_deg"), ("tr", "grad_tr_ms"), ("t1", "grad_t1"),
                      ("t2", "grad_t2"), ("b1", "grad_b1")):
        assert max_rel(g[mine], d[ref]) <= GRAD_TOL, mine


def test_dropin_vjp_every_event(built_library, cuda, golden):
    """The host-buffer drop-in of _epg_cpu.simulate_vjp: all 20 gradient slots."""
    from tests.test_gpu_parity import EVENT_ORDER, FEATURES, TISSUE_ORDER, _pointer_array
    from torchsim_gb300 import _native

    d = golden("mrf_adjoint")
    V, P = d["vjp_seed"].shape
    E = d["vjp_event_kind"].size
    tissue = [np.ascontiguousarray(d["vjp_tissue_" + n]) for n in TISSUE_ORDER]
    events = [np.ascontiguousarray(d["vjp_event_" + n]) for n in EVENT_ORDER]
    seeds = [np.ascontiguousarray(d["vjp_seed"].real), np.ascontiguousarray(d["vjp_seed"].imag)]
    grads = [np.full(V, 9.0, np.float32) for _ in range(17)] + [np.full(E, 9.0, np.float32)
                                                                  for _ in range(3)]
    arrays = [*tissue, *events, *seeds, *grads, *([None] * 13)]
    _native.check(built_library.tsg_epg_simulate_vjp(_pointer_array(arrays), len(arrays), V, 1, E,
                                                     int(d["states"]), P, 1, FEATURES))
    names = [*TISSUE_ORDER, "flip", "phase", "duration"]
    for name, got in zip(names, grads, strict=True):
        key = "vjp_grad_" + name
        if key in d.files and name not in ("b1_phase_rad", "b0_hz", "phase",
                                           "diffusion_um2_per_ms"):
            assert max_rel(got, d[key]) <= GRAD_TOL, name
    # Oracle (FP64): every event's duration gradient, zero-duration events too.
    ref = O.adjoint(packed_from_golden(d, "vjp_"), d["vjp_seed"].imag, "f64")
    assert max_rel(grads[19], ref["duration_s"]) <= GRAD_TOL
    assert max_rel(grads[17], ref["flip_rad"]) <= GRAD_TOL
    assert not grads[18].any()


@pytest.mark.parametrize("ops_per_checkpoint", [1, 3, 7, 16])
def test_segment_length_does_not_change_gradients(cuda, ops_per_checkpoint):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(31)
    flips = rng.uniform(5, 70, 90).astype(np.float32)
    trs = rng.uniform(8, 15, 90).astype(np.float32)
    ev = mrf_events(flips, trs, TI_ms=12.0)
    V, S = 45, 12
    t1, t2, b1 = draw_tissue(7, V)
    prog = program_for(ev, cuda)
    tissue = engine.tissue_maps(cuda, V, t1, t2, None, b1, None)
    seed = torch.from_numpy(rng.standard_normal((V, ev.outputs)).astype(np.complex64)).to(cuda)
    c, ck, _ = engine.adjoint_plan(prog, V, S, None, ops_per_checkpoint)
    assert c == ops_per_checkpoint
    ckpt = torch.empty(ck // 4, dtype=torch.float32, device=cuda)
    engine.forward_checkpointed(prog, tissue, S, c, ckpt)
    grads = {n: torch.zeros(V, device=cuda) for n in ("t1_ms", "t2_ms", "m0", "b1", "inversion")}
    grads["flip_rad"] = torch.zeros((1, ev.events), device=cuda)
    grads["duration_s"] = torch.zeros((1, ev.events), device=cuda)
    engine.adjoint(prog, tissue, S, seed, ckpt, c, grads)
    p = packed_from_events(ev, t1, t2, S, b1=b1)
    ref = O.adjoint(p, -seed.real.cpu().numpy(), "f64")
    for name in ("t1_ms", "t2_ms", "m0", "b1", "flip_rad"):
        got = grads[name].cpu().numpy().reshape(ref[name].shape)
        assert max_rel(got, ref[name]) <= GRAD_TOL, name
    # Zero-duration events fold into the op before them: their duration
    # gradient is not formed on the merged program; the others agree.
    dur = grads["duration_s"].cpu().numpy()[0]
    nz = ev.duration[0] != 0
    assert max_rel(dur[nz], ref["duration_s"][nz]) <= GRAD_TOL


@pytest.mark.parametrize("shape", [(1, 20, 4), (1, 10, 2), (5, 2, 4), (2, 6, 4), (5, 4, 2),
                                   (10, 2, 4), (4, 4, 2), (4, 6, 4), (8, 4, 4), (8, 8, 2),
                                   (16, 4, 4), (32, 4, 4)])
@pytest.mark.parametrize("mode", ["checkpointed", "trajectory"])
def test_adjoint_launch_shapes(cuda, shape, mode):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    lanes, orders, warps = shape
    rng = np.random.default_rng(lanes * 7 + orders)
    flips = rng.uniform(5, 70, 60).astype(np.float32)
    ev = mrf_events(flips, 9.0)
    V = 50
    S = max(2, lanes * orders - 2)
    t1, t2, b1 = draw_tissue(lanes, V)
    inv = rng.uniform(0.8, 1.0, V).astype(np.float32)
    prog = program_for(ev, cuda)
    tissue = engine.tissue_maps(cuda, V, t1, t2, None, b1, inv)
    seed = torch.from_numpy(rng.standard_normal((V, ev.outputs)).astype(np.complex64)).to(cuda)
    c, ck, _ = engine.adjoint_plan(prog, V, S, shape, 1 if mode == "trajectory" else 0)
    assert (c == 1) == (mode == "trajectory")
    ckpt = torch.empty(ck // 4, dtype=torch.float32, device=cuda)
    # The checkpoint layout does not depend on the forward's launch shape.
    engine.forward_checkpointed(prog, tissue, S, c, ckpt)
    grads = {n: torch.zeros(V, device=cuda) for n in ("t1_ms", "t2_ms", "b1", "inversion")}
    grads["flip_rad"] = torch.zeros((1, ev.events), device=cuda)
    engine.adjoint(prog, tissue, S, seed, ckpt, c, grads, launch=shape)
    ref = O.adjoint(packed_from_events(ev, t1, t2, S, b1=b1, inv=inv), -seed.real.cpu().numpy(),
                    "f64")
    for name in ("t1_ms", "t2_ms", "b1", "inversion", "flip_rad"):
        got = grads[name].cpu().numpy().reshape(ref[name].shape)
        assert max_rel(got, ref[name]) <= GRAD_TOL, (shape, mode, name)


def test_adjoint_workload_at_full_size(cuda):
    """The sequence-optimisation workload at its full size -- 16,384 voxels,
    600 pulses (flip U(5, 70) deg, TR U(8, 15) ms), 20 states, trajectory
    mode -- through properties that do not depend on its size: the tissue
    gradients of 512 voxels spread over the batch against the FP64 oracle run
    on those voxels alone, and each event's gradient equal to the sum of the
    two half batches' (the loss is a sum over voxels)."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(5)
    V, S = 16384, 20
    flips = rng.uniform(5, 70, 600).astype(np.float32)
    trs = rng.uniform(8, 15, 600).astype(np.float32)
    ev = mrf_events(flips, trs)
    prog = program_for(ev, cuda)
    t1, t2, b1 = draw_tissue(3, V)
    seed = rng.standard_normal((V, ev.outputs)).astype(np.complex64)

    def run(rows):
        n = len(rows)
        tissue = engine.tissue_maps(cuda, n, t1[rows], t2[rows], None, b1[rows], None)
        c, ck, _ = engine.adjoint_plan(prog, n, S, None, 1)
        assert c == 1
        ckpt = torch.empty(ck // 4, dtype=torch.float32, device=cuda)
        engine.forward_checkpointed(prog, tissue, S, c, ckpt)
        grads = {k: torch.zeros(n, device=cuda) for k in ("t1_ms", "t2_ms", "b1")}
        for k in ("flip_rad", "duration_s"):
            grads[k] = torch.zeros((1, ev.events), device=cuda)
        engine.adjoint(prog, tissue, S, torch.from_numpy(seed[rows]).to(cuda), ckpt, c, grads)
        return {k: v.cpu().numpy() for k, v in grads.items()}

    rows = np.arange(V)
    full = run(rows)
    sample = np.unique(np.concatenate([np.linspace(0, V - 1, 384).astype(np.int64),
                                       rng.integers(0, V, 128)]))
    ref = O.adjoint(packed_from_events(ev, t1[sample], t2[sample], S, b1=b1[sample]),
                    -seed[sample].real, "f64")
    for name in ("t1_ms", "t2_ms", "b1"):
        assert max_rel(full[name][sample], ref[name]) <= GRAD_TOL, name
    low, high = run(rows[: V // 2]), run(rows[V // 2:])
    for name in ("flip_rad", "duration_s"):
        assert np.abs(full[name]).max() > 0, name
        assert max_rel(full[name], low[name] + high[name]) <= 1e-5, name


def test_adjoint_against_central_differences(cuda):
    """Config-3 shapes in small: 600 pulses, nstates 20; central differences
    (h = 1e-3 deg / ms) of the FP64 oracle's loss on sampled coordinates."""
    from torchsim_gb300.sequence import mrf_events, mrf_gradient_map

    rng = np.random.default_rng(3)
    n, V, S = 600, 24, 20
    t1, t2, b1 = draw_tissue(0, V)
    flips = rng.uniform(5, 70, n).astype(np.float32)
    trs = rng.uniform(8, 15, n).astype(np.float32)
    tgt_flip = rng.uniform(5, 70, n).astype(np.float32)
    tgt_tr = rng.uniform(8, 15, n).astype(np.float32)
    ev_t = mrf_events(tgt_flip, tgt_tr)
    target = -O.forward(packed_from_events(ev_t, t1, t2, S, b1=b1), "f64")
    g = _loss_grads(flips, trs, t1, t2, b1, target.astype(np.complex64), S, cuda)

    base = mrf_events(flips, trs)
    where = mrf_gradient_map(n)

    def loss(fl, tr):
        # Durations set from the TRs directly: the reference's float32 clock
        # (which the event builder reproduces) resolves 0.5 us at the end of
        # this train, too coarse for a 1e-3 ms difference.
        ev = mrf_events(fl.astype(np.float32), trs)
        dur = ev.duration.astype(np.float64).copy()
        dur[0, where["tr"][:, 0]] = tr[where["tr"][:, 1]] * 1e-3
        p = packed_from_events(ev, t1, t2, S, b1=b1)
        p.duration_s = dur.astype(np.float32)
        s = -O.forward(p, "f64")
        return float(((s - target) ** 2).sum())

    picks = [0, 7, 150, 301, 598]
    for k in picks:
        h = 1e-3
        up, dn = flips.astype(np.float64).copy(), flips.astype(np.float64).copy()
        up[k] += h
        dn[k] -= h
        fd = (loss(up, trs) - loss(dn, trs)) / (2 * h)
        assert abs(g["flip"][k] - fd) <= 1e-3 * max(abs(fd), np.abs(g["flip"]).max() * 1e-2), k
    for k in [0, 10, 299, 597]:
        h = 1e-3
        up, dn = trs.astype(np.float64).copy(), trs.astype(np.float64).copy()
        up[k] += h
        dn[k] -= h
        fd = (loss(flips, up) - loss(flips, dn)) / (2 * h)
        # A 1e-3 ms step rounds to float32 durations: the difference itself is
        # good to about 3e-4 relative here.
        assert abs(g["tr"][k] - fd) <= 2e-3 * max(abs(fd), np.abs(g["tr"]).max() * 1e-2), k
    assert g["tr"][-1] == 0.0  # the last TR moves nothing recorded


def test_adjoint_deterministic(cuda, golden):
    d = golden("mrf_adjoint")
    a = _loss_grads(d["flip_deg"], d["tr_ms"], d["t1"], d["t2"], d["b1"], d["target"], 8, cuda)
    b = _loss_grads(d["flip_deg"], d["tr_ms"], d["t1"], d["t2"], d["b1"], d["target"], 8, cuda)
    for k in ("flip", "tr", "t1", "t2", "b1"):
        assert np.array_equal(a[k], b[k]), k


def test_adjoint_block_size_is_checked(cuda):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    prog = program_for(mrf_events(np.full(8, 20.0, np.float32), 9.0), cuda)
    with pytest.raises(ValueError):
        engine.adjoint_plan(prog, 16, 10, (5, 2, 8), 0)


def test_second_backward_matches_reference(cuda, golden):
    """Reverse over reverse through the public simulator: the gradient of
    <directions, d<seed, s>/d(inputs)> with respect to the inputs and the
    seed against the reference's (its _NativeEpg backward differentiated once
    more; here the second-order sweep)."""
    from torchsim_gb300 import MRFSimulator

    d = golden("double_backward")
    leaves = {k: torch.tensor(d[v], device=cuda, requires_grad=True) for k, v in
              (("T1", "t1"), ("T2", "t2"), ("B1", "b1"), ("M0", "m0"))}
    theta = torch.tensor(d["flip_deg"], device=cuda, requires_grad=True)
    tau = torch.tensor(d["tr_ms"], device=cuda, requires_grad=True)
    sig = MRFSimulator(flip=theta, TR=tau, states=int(d["states"])).simulate(**leaves)
    seed = torch.tensor(d["seed"], device=cuda, requires_grad=True)
    inputs = (theta, tau, *leaves.values())
    grads = torch.autograd.grad(sig, inputs, seed, create_graph=True)
    names = ("flip_deg", "tr_ms", "T1", "T2", "B1", "M0")
    for name, g in zip(names, grads, strict=True):
        assert max_rel(g.detach().cpu().numpy(), d[f"grad_{name}"]) <= GRAD_TOL, name
    directions = [torch.tensor(d[f"direction_{n}"], device=cuda) for n in names]
    contraction = sum((g * v).sum() for g, v in zip(grads, directions, strict=True))
    assert abs(contraction.item() - float(d["contraction"])) <= 1e-4 * abs(float(d["contraction"]))
    second = torch.autograd.grad(contraction, (*inputs, seed))
    for name, h in zip(names, second[:-1], strict=True):
        assert max_rel(h.cpu().numpy(), d[f"second_{name}"]) <= GRAD_TOL, name
    assert max_rel(second[-1].cpu().numpy(), d["second_seed"]) <= GRAD_TOL


def test_hessian_vector_product_matches_finite_differences(cuda):
    """d/dT2 of the T2 gradient of a loss along a direction, against central
    differences of the first-order gradient (the check of the reference's
    tests/sequence/test_vjp.py:344-385, with steps of 0.1% of each T2)."""
    from torchsim_gb300 import MRFSimulator

    rng = np.random.default_rng(21)
    flips = rng.uniform(5, 70, 40).astype(np.float32)
    t1, t2, b1 = draw_tissue(22, 6)
    w = torch.from_numpy((rng.standard_normal((6, 40)) + 1j * rng.standard_normal((6, 40)))
                         .astype(np.complex64)).to(cuda)
    # A direction scaled by each voxel's T2, so a step is the same fraction
    # of every voxel's T2.
    v = torch.from_numpy((rng.standard_normal(6) * t2).astype(np.float32)).to(cuda)

    def grad_t2(t2v, create):
        x = t2v.clone().requires_grad_(True)
        sig = MRFSimulator(flip=torch.tensor(flips), TR=10.0, states=10).simulate(
            T1=torch.tensor(t1, device=cuda), T2=x, B1=torch.tensor(b1, device=cuda))
        (g,) = torch.autograd.grad(sig, (x,), w, create_graph=create)
        return x, g

    base = torch.tensor(t2, device=cuda)
    x, g = grad_t2(base, True)
    (hv,) = torch.autograd.grad((g * v).sum(), (x,))
    h = 1e-3
    _, gp = grad_t2(base + h * v, False)
    _, gm = grad_t2(base - h * v, False)
    fd = (gp - gm) / (2 * h)
    assert max_rel(hv.cpu().numpy(), fd.cpu().numpy()) <= 1e-2
