"""Sequence design on the GPU: Adam over bounded flips and TRs of an MRF train,
with the gradient from the adjoint kernel (the reference's
optim/_design.py:142-194 loop; tests/optim/test_design.py)."""

import numpy as np
import pytest
import torch

from helpers import draw_tissue

pytestmark = pytest.mark.gpu


def test_mrf_design_fits_a_target_inside_its_limits(cuda):
    from torchsim_gb300 import Bounded, SequenceDesign, mrf_sim

    rng = np.random.default_rng(5)
    n, V = 40, 64
    t1, t2, b1 = draw_tissue(11, V)
    T1 = torch.from_numpy(t1).to(cuda)
    T2 = torch.from_numpy(t2).to(cuda)
    B1 = torch.from_numpy(b1).to(cuda)
    true_flip = torch.from_numpy(rng.uniform(10, 60, n).astype(np.float32)).to(cuda)
    true_tr = torch.from_numpy(rng.uniform(9, 14, n).astype(np.float32)).to(cuda)
    target = mrf_sim(true_flip, true_tr, T1, T2, B1=B1, states=12)

    def cost(flip, TR):
        return (mrf_sim(flip, TR, T1, T2, B1=B1, states=12) - target).abs().pow(2).sum()

    start_flip = torch.full((n,), 35.0, device=cuda)
    start_tr = torch.full((n,), 11.0, device=cuda)
    design = SequenceDesign(cost, flip=Bounded(start_flip, 5.0, 70.0),
                            TR=Bounded(start_tr, 8.0, 15.0))
    result = design.minimize(iterations=40, learning_rate=0.05)
    loss = result.loss.cpu().numpy()
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.25 * loss[0]
    flip, tr = result.parameters["flip"], result.parameters["TR"]
    assert float(flip.min()) >= 5.0 and float(flip.max()) <= 70.0
    assert float(tr.min()) >= 8.0 and float(tr.max()) <= 15.0


def test_a_cramer_rao_design_lowers_its_bound(cuda):
    """A design cost that differentiates a Jacobian (the Cramer-Rao bound of
    T1 and T2, relative to their squares) backs through the second-order
    sweep; minimising it over the flip angles lowers the bound and keeps the
    limits (the reference's optim/_design.py with crlb)."""
    from torchsim_gb300 import Bounded, SequenceDesign, crlb, mrf_sim

    T1 = torch.tensor([800.0, 1300.0, 400.0, 2000.0], device=cuda)
    T2 = torch.tensor([60.0, 110.0, 40.0, 150.0], device=cuda)
    scale = torch.stack((T1, T2), dim=-1)

    def cost(flip):
        _, jac = mrf_sim(flip, 12.0, T1, T2, diff=("T1", "T2"), states=12)
        return (crlb(jac) / scale.square()).sum()

    design = SequenceDesign(cost, flip=Bounded(torch.full((24,), 30.0, device=cuda), 5.0, 70.0))
    result = design.minimize(iterations=30, learning_rate=0.1)
    loss = result.loss.cpu().numpy()
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.8 * loss[0]
    flip = result.parameters["flip"]
    assert float(flip.min()) >= 5.0 and float(flip.max()) <= 70.0
