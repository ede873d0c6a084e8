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


def test_jacobian_of_a_design_variable_is_refused(cuda):
    from torchsim_gb300 import mrf_sim

    flip = torch.full((8,), 20.0, device=cuda, requires_grad=True)
    T1 = torch.full((4,), 800.0, device=cuda)
    T2 = torch.full((4,), 60.0, device=cuda)
    with pytest.raises(NotImplementedError):
        mrf_sim(flip, 10.0, T1, T2, diff=("T1", "T2"))
