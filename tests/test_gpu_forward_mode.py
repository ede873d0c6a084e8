"""Forward-mode derivatives through the simulators (the reference's
``_NativeEpg.jvp``: ``torch.func.jvp`` and ``torch.autograd.forward_ad`` dual
tensors through ``simulate``), on the real and the complex path: one general
tangent sweep along every input's tangent at once, against the fused
Jacobian columns and against reverse mode (``<w, J v> = <J^T w, v>``)."""

from __future__ import annotations

import numpy as np
import pytest
import torch
import torch.autograd.forward_ad as fwAD

from tests.helpers import draw_tissue, max_rel, mrf_schedule

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _maps(cuda, V, seed):
    t1, t2, b1 = draw_tissue(seed, V)
    return tuple(torch.from_numpy(a).to(cuda) for a in (t1, t2, b1))


def test_jvp_along_tissue_maps_equals_the_jacobian_columns(cuda):
    from torchsim_gb300 import MRFSimulator

    V = 300
    t1, t2, b1 = _maps(cuda, V, 5)
    sim = MRFSimulator(flip=torch.from_numpy(mrf_schedule()[:200]), TR=10.0, states=12)
    rng = np.random.default_rng(5)
    v1, v2, vb = (torch.from_numpy(rng.standard_normal(V).astype(np.float32)).to(cuda)
                  for _ in range(3))
    sig, tan = torch.func.jvp(lambda a, b, c: sim.simulate(T1=a, T2=b, B1=c),
                              (t1, t2, b1), (v1, v2, vb))
    ref_sig, jac = sim.jacobian(("T1", "T2", "B1"), T1=t1, T2=t2, B1=b1)
    assert max_rel(sig.cpu().numpy(), ref_sig.cpu().numpy()) <= 1e-6
    want = (jac * torch.stack((v1, v2, vb), dim=1)[:, :, None]).sum(1)
    assert max_rel(tan.cpu().numpy(), want.cpu().numpy()) <= TOL


def test_dual_tensors_give_the_same_tangent(cuda):
    from torchsim_gb300 import MRFSimulator

    V = 64
    t1, t2, b1 = _maps(cuda, V, 6)
    sim = MRFSimulator(flip=torch.from_numpy(mrf_schedule()[:120]), TR=10.0, states=10)
    v = torch.from_numpy(np.random.default_rng(6).standard_normal(V).astype(np.float32)).to(cuda)
    with fwAD.dual_level():
        out = sim.simulate(T1=t1, T2=fwAD.make_dual(t2, v), B1=b1)
        tan = fwAD.unpack_dual(out).tangent
    _, jac = sim.jacobian("T2", T1=t1, T2=t2, B1=b1)
    assert max_rel(tan.cpu().numpy(), (jac * v[:, None]).cpu().numpy()) <= TOL


def test_jvp_along_flips_and_trs_agrees_with_reverse_mode(cuda):
    """A direction in the protocol (flip angles and TRs of a 150-pulse MRF
    train): the tangent's inner product with a random cotangent equals the
    reverse-mode gradient's inner product with the direction."""
    from torchsim_gb300 import MRFSimulator

    V = 96
    t1, t2, b1 = _maps(cuda, V, 7)
    rng = np.random.default_rng(7)
    flip = torch.from_numpy(rng.uniform(5, 70, 150).astype(np.float32)).to(cuda)
    tr = torch.from_numpy(rng.uniform(8, 15, 150).astype(np.float32)).to(cuda)
    dflip = torch.from_numpy(rng.standard_normal(150).astype(np.float32)).to(cuda)
    dtr = torch.from_numpy(rng.standard_normal(150).astype(np.float32)).to(cuda)
    w = torch.from_numpy((rng.standard_normal((V, 150))
                          + 1j * rng.standard_normal((V, 150))).astype(np.complex64)).to(cuda)

    def signal(f, r):
        return MRFSimulator(flip=f, TR=r, states=20).simulate(T1=t1, T2=t2, B1=b1)

    _, tan = torch.func.jvp(signal, (flip, tr), (dflip, dtr))
    forward = float((w.conj() * tan).real.sum())
    f = flip.clone().requires_grad_()
    r = tr.clone().requires_grad_()
    (w.conj() * signal(f, r)).real.sum().backward()
    reverse = float((f.grad * dflip).sum() + (r.grad * dtr).sum())
    assert abs(forward - reverse) <= TOL * max(abs(reverse), 1e-3), (forward, reverse)


def test_jvp_on_the_complex_path(cuda):
    """With off-resonance and a transmit phase (the complex kernel): the
    tangent along B0 and B1phase against the public Jacobian's columns."""
    from torchsim_gb300 import MRFSimulator

    V = 80
    t1, t2, b1 = _maps(cuda, V, 8)
    rng = np.random.default_rng(8)
    b0 = torch.from_numpy(rng.uniform(-40, 40, V).astype(np.float32)).to(cuda)
    ph = torch.from_numpy(rng.uniform(-0.5, 0.5, V).astype(np.float32)).to(cuda)
    vb0 = torch.from_numpy(rng.standard_normal(V).astype(np.float32)).to(cuda)
    vph = torch.from_numpy(rng.standard_normal(V).astype(np.float32)).to(cuda)
    sim = MRFSimulator(flip=torch.from_numpy(mrf_schedule()[:100]), TR=10.0, states=12)
    _, tan = torch.func.jvp(lambda a, c: sim.simulate(T1=t1, T2=t2, B1=b1, B0=a, B1phase=c),
                            (b0, ph), (vb0, vph))
    _, jac = sim.jacobian(("B0", "B1phase"), T1=t1, T2=t2, B1=b1, B0=b0, B1phase=ph)
    want = jac[:, 0] * vb0[:, None] + jac[:, 1] * vph[:, None]
    assert max_rel(tan.cpu().numpy(), want.cpu().numpy()) <= TOL
