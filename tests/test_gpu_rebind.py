"""Programs rebound on the device from device-resident flips and TRs: the
event buffers and the op table are bitwise the host builder's and compiler's,
simulation and gradients through them are bitwise the host path's, and the
program path of a design step makes no host synchronisation."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import draw_tissue
from tests.test_program import plan

pytestmark = pytest.mark.gpu


def _protocol(seed, n, cuda):
    rng = np.random.default_rng(seed)
    flip = rng.uniform(5, 70, n).astype(np.float32)
    tr = rng.uniform(8, 15, n).astype(np.float32)
    return flip, tr, torch.from_numpy(flip).to(cuda), torch.from_numpy(tr).to(cuda)


@pytest.mark.parametrize("ti", [0.0, 20.0])
def test_rebound_stream_and_ops_are_the_host_compilers(cuda, ti):
    from torchsim_gb300.sequence import mrf_events, mrf_stream_on_device

    flip, tr, flip_d, tr_d = _protocol(3, 600, cuda)
    program, flip_ev, dur_ev = mrf_stream_on_device(flip_d, tr_d, ti, cuda)
    host = mrf_events(flip, tr, TI_ms=ti)
    assert torch.equal(flip_ev.cpu(), torch.from_numpy(host.flip))
    assert torch.equal(dur_ev.cpu(), torch.from_numpy(host.duration))
    n_ops, n_out, dt, fl, rec, code = plan(host)
    assert (program.ops, program.outputs) == (n_ops, n_out)
    ops = program.ops_buffer[:n_ops].cpu()
    assert torch.equal(ops[:, 0], torch.from_numpy(dt))
    assert torch.equal(ops[:, 1], torch.from_numpy(fl))
    bits = ops.view(torch.int32)
    assert torch.equal(bits[:, 2], torch.from_numpy(rec))
    assert torch.equal(bits[:, 3], torch.from_numpy(code.view(np.int32)))
    # A scalar TR and a new train of flips rebind the same template.
    program2, _, dur2 = mrf_stream_on_device(flip_d * 0.5, 9.5, ti, cuda)
    assert program2.template is program.template
    assert torch.equal(dur2.cpu(), torch.from_numpy(mrf_events(flip * 0.5, 9.5, TI_ms=ti).duration))


def test_rebound_simulation_and_gradients_equal_the_host_path(cuda):
    from torchsim_gb300 import MRFSimulator

    flip, tr, flip_d, tr_d = _protocol(5, 300, cuda)
    t1, t2, b1 = (torch.from_numpy(a).to(cuda) for a in draw_tissue(5, 512))
    target = torch.randn((512, 300), dtype=torch.complex64, device=cuda)
    results = []
    for on_device in (True, False):
        f = (flip_d if on_device else torch.from_numpy(flip)).clone().requires_grad_(True)
        r = (tr_d if on_device else torch.from_numpy(tr)).clone().requires_grad_(True)
        sim = MRFSimulator(flip=f, TR=r, states=20)
        sig = sim.simulate(T1=t1, T2=t2, B1=b1)
        loss = (sig - target).abs().square().sum()
        loss.backward()
        plain = MRFSimulator(flip=f.detach(), TR=r.detach(), states=20).simulate(T1=t1, T2=t2, B1=b1)
        results.append((sig.detach(), plain, f.grad.cpu(), r.grad.cpu()))
    for a, b in zip(*results, strict=True):
        assert torch.equal(a.cpu(), b.cpu())


def test_design_step_program_path_makes_no_host_sync(cuda):
    """Once its template is compiled, rebinding a 600-pulse protocol makes no
    synchronising call (torch's sync debug mode raises on any), and neither
    does a whole differentiable simulate and backward through it."""
    from torchsim_gb300 import MRFSimulator
    from torchsim_gb300.sequence import mrf_stream_on_device

    flip, tr, flip_d, tr_d = _protocol(7, 600, cuda)
    t1, t2, b1 = (torch.from_numpy(a).to(cuda) for a in draw_tissue(7, 1024))
    target = torch.zeros((1024, 600), dtype=torch.complex64, device=cuda)

    def step():
        f = flip_d.clone().requires_grad_(True)
        r = tr_d.clone().requires_grad_(True)
        sig = MRFSimulator(flip=f, TR=r, states=20).simulate(T1=t1, T2=t2, B1=b1)
        (sig - target).abs().square().sum().backward()
        return f.grad, r.grad

    step()  # compiles the template, uploads the index maps, warms the caches
    torch.cuda.synchronize()
    torch.cuda.set_sync_debug_mode("error")
    try:
        mrf_stream_on_device(flip_d, tr_d, 0.0, cuda)
        g = step()
    finally:
        torch.cuda.set_sync_debug_mode("default")
    torch.cuda.synchronize()
    assert all(bool(torch.isfinite(x).all()) for x in g)
