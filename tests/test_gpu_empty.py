"""Empty inputs through every public entry point on the path: zero voxels
give empty results of the right shapes (and zero gradients), not errors."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import mrf_schedule

pytestmark = pytest.mark.gpu


def _empty(device=None):
    return torch.zeros(0, dtype=torch.float32, device=device)


def test_mrf_sim_with_no_voxels(cuda):
    import torchsim_gb300 as ts

    flip = torch.from_numpy(mrf_schedule()[:50])
    for device in ("cpu", cuda):
        sig = ts.mrf_sim(flip, 10.0, _empty(device), _empty(device), B1=_empty(device), states=10)
        assert sig.shape == (0, 50) and sig.dtype == torch.complex64
        sig, jac = ts.mrf_sim(flip, 10.0, _empty(device), _empty(device), B1=_empty(device),
                              diff=("T1", "T2", "B1"), states=10)
        assert sig.shape == (0, 50) and jac.shape == (0, 3, 50)


def test_gradients_with_no_voxels(cuda):
    from torchsim_gb300 import MRFSimulator

    theta = torch.tensor(mrf_schedule()[:40], device=cuda, requires_grad=True)
    t1 = _empty(cuda).requires_grad_()
    sig = MRFSimulator(flip=theta, TR=10.0, states=10).simulate(T1=t1, T2=_empty(cuda))
    assert sig.shape == (0, 40)
    sig.abs().square().sum().backward()
    assert theta.grad is not None and not bool(theta.grad.any())
    assert t1.grad is not None and t1.grad.shape == (0,)


def test_matching_with_no_signals(cuda):
    from torchsim_gb300 import DictionaryMatcher

    rng = np.random.default_rng(0)
    atoms = torch.from_numpy(rng.standard_normal((300, 64)).astype(np.float32) + 0j).to(
        torch.complex64).to(cuda)
    res = DictionaryMatcher(dictionary=atoms).match(torch.zeros((0, 64), dtype=torch.complex64,
                                                                device=cuda))
    assert res.indices.shape[0] == 0


def test_mapping_with_no_voxels(cuda):
    from torchsim_gb300 import MRFSimulator, NonlinearLeastSquares

    flip = torch.from_numpy(mrf_schedule()[:60])
    est = NonlinearLeastSquares(MRFSimulator(flip=flip, TR=10.0, states=10),
                                bounds={"T1": (50.0, 5000.0), "T2": (2.0, 1000.0),
                                        "M0": (0.0, 5.0)})
    est.fit(T1=(100.0, 3000.0), T2=(10.0, 300.0), M0=(0.5, 1.5), known={"B1": (0.8, 1.2)},
            seed=0)
    maps = est.map(torch.zeros((0, 60), dtype=torch.complex64, device=cuda),
                   known={"B1": _empty(cuda)})
    for name in ("T1", "T2", "M0"):
        assert maps[name].shape == (0,)


def test_batch_with_an_empty_sequence(cuda):
    from torchsim_gb300.batching import BatchEntry, SequenceBatch
    from torchsim_gb300.sequence import fse_events

    ev = fse_events(np.full(8, 150.0, np.float32), 10.0, phases_deg=90.0)
    entries = [BatchEntry(ev, 16, np.zeros(0, np.float32), np.zeros(0, np.float32)),
               BatchEntry(ev, 16, np.full(5, 1000.0, np.float32), np.full(5, 80.0, np.float32))]
    batch = SequenceBatch(entries, cuda)
    batch.launch((16, 2, 2))
    torch.cuda.synchronize()
    assert batch.signal(0).shape[0] == 0
    assert batch.signal(1).shape == (5, 8)
    assert bool(torch.isfinite(batch.signal(1)).all())
