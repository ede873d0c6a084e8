"""GPU parity of the persistent batched launch over uneven CPMG sequences."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import max_rel, packed_from_events

pytestmark = pytest.mark.gpu


def make_batch(device, seed=0, etls=(8, 13, 21, 32, 47, 64), voxels=(1, 7, 100, 333)):
    from torchsim_gb300.batching import BatchEntry, SequenceBatch
    from torchsim_gb300.sequence import fse_events

    rng = np.random.default_rng(seed)
    entries = []
    for i, etl in enumerate(etls):
        for j, v in enumerate(voxels[(i % 2)::2] if len(etls) > 3 else voxels):
            flips = rng.uniform(100, 180, etl).astype(np.float32)
            ev = fse_events(flips, float(rng.uniform(5, 15)), phases_deg=90.0)
            entries.append(BatchEntry(ev, 2 * etl, rng.uniform(300, 3000, v).astype(np.float32),
                                      rng.uniform(10, 300, v).astype(np.float32),
                                      rng.uniform(0.7, 1.3, v).astype(np.float32)))
    return SequenceBatch(entries, device)


def _check_against_oracle(batch):
    for s, e in enumerate(batch.entries):
        ref = O.forward(packed_from_events(e.events, e.t1, e.t2, e.states, b1=e.b1), "f64")
        got = batch.signal(s).cpu().numpy()
        assert not got.real.any()
        assert max_rel(got.imag, ref) <= 1e-5, s


@pytest.mark.parametrize("shape", [(2, 2, 2), (4, 4, 4), (8, 8, 2), (4, 1, 16), (16, 2, 8)])
def test_batched_matches_oracle(cuda, shape):
    batch = make_batch(cuda, etls=(8, 13, 21, 32) if shape[0] == 2 else (8, 13, 21, 32, 47, 64))
    batch.out.fill_(float("nan"))
    batch.launch(shape)
    torch.cuda.synchronize()
    _check_against_oracle(batch)


def test_graph_replay_and_plain_form_agree(cuda):
    batch = make_batch(cuda, seed=1)
    batch.shape = (4, 4, 4)
    batch.capture()
    batch.out.zero_()
    batch.run()
    torch.cuda.synchronize()
    _check_against_oracle(batch)
    graph_out = batch.out.clone()
    batch.out.zero_()
    batch.run_plain()
    torch.cuda.synchronize()
    _check_against_oracle(batch)
    assert torch.allclose(graph_out, batch.out, rtol=0, atol=1e-6)


def test_sequence_alone_equals_in_the_mix(cuda):
    from torchsim_gb300.batching import SequenceBatch

    batch = make_batch(cuda, seed=2)
    batch.launch((4, 4, 4))
    alone = SequenceBatch([batch.entries[5]], cuda)
    alone.launch((4, 4, 4))
    torch.cuda.synchronize()
    assert torch.equal(alone.signal(0), batch.signal(5))


def test_autotuner_picks_a_working_shape(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("TORCHSIM_GB300_CACHE", str(tmp_path / "tuning.json"))
    batch = make_batch(cuda, seed=3, etls=(8, 16), voxels=(50, 200))
    shape, timings = batch.tune(use_cache=False)
    assert shape in batch.candidates() and timings
    batch.out.zero_()
    batch.launch(shape)
    torch.cuda.synchronize()
    _check_against_oracle(batch)
    again, cached = batch.tune()
    assert again == shape and cached == {}
