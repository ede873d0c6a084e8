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


def test_batched_workload_at_full_size(cuda):
    """The uneven-CPMG workload at its full size -- 512 sequences (ETL
    U{8..64}, refocusing U(100, 180) deg, ESP U(5, 15) ms, phases 90 deg,
    round(exp(U(ln 1e3, ln 6.4e4))) voxels each, nstates 2 x ETL), one
    persistent launch at 16 orders per lane, 2 warps, 8 blocks per SM --
    through properties that do not depend on its size: up to 64 voxels of
    every 16th sequence against the FP64 oracle, and three sequences launched
    alone bitwise equal to their rows of the full launch."""
    from torchsim_gb300.batching import BatchEntry, SequenceBatch
    from torchsim_gb300.sequence import fse_events

    rng = np.random.default_rng(2)
    entries = []
    for _ in range(512):
        etl = int(rng.integers(8, 65))
        flips = rng.uniform(100, 180, etl).astype(np.float32)
        ev = fse_events(flips, float(rng.uniform(5, 15)), phases_deg=90.0)
        v = int(round(np.exp(rng.uniform(np.log(1e3), np.log(6.4e4)))))
        entries.append(BatchEntry(ev, 2 * etl, rng.uniform(300, 3000, v).astype(np.float32),
                                  rng.uniform(10, 300, v).astype(np.float32),
                                  rng.uniform(0.7, 1.3, v).astype(np.float32)))
    batch = SequenceBatch(entries, cuda)
    assert sum(e.t1.size for e in entries) > 7_000_000
    shape = (16, 2, 8)
    batch.out.fill_(float("nan"))
    batch.launch(shape)
    torch.cuda.synchronize()
    for s in range(0, 512, 16):
        e = entries[s]
        rows = np.unique(np.linspace(0, e.t1.size - 1, 64).astype(np.int64))
        ref = O.forward(packed_from_events(e.events, e.t1[rows], e.t2[rows], e.states,
                                           b1=e.b1[rows]), "f64")
        got = batch.signal(s)[torch.from_numpy(rows).to(cuda)].cpu().numpy()
        assert not got.real.any()
        assert max_rel(got.imag, ref) <= 1e-5, s
    for s in (0, 255, 511):
        alone = SequenceBatch([entries[s]], cuda)
        alone.launch(shape)
        torch.cuda.synchronize()
        assert torch.equal(alone.signal(0), batch.signal(s)), s


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


def test_cpmg_echo_loop_and_op_loop_in_one_launch(cuda):
    """CPMG trains run the kernel's echo loop; any other program (MRF trains
    after an inversion, at a fixed or a varying TR) runs the general op loop.
    Both kinds in one launch, each against the FP64 oracle, and a CPMG train
    alone equal to its row in the mix."""
    from torchsim_gb300.batching import BatchEntry, SequenceBatch
    from torchsim_gb300.sequence import fse_events, mrf_events
    from tests.helpers import mrf_schedule

    rng = np.random.default_rng(7)

    def tissue(v):
        return (rng.uniform(300, 3000, v).astype(np.float32),
                rng.uniform(10, 300, v).astype(np.float32),
                rng.uniform(0.7, 1.3, v).astype(np.float32))

    entries = [
        BatchEntry(fse_events(rng.uniform(100, 180, 24).astype(np.float32), 8.0,
                              phases_deg=90.0), 48, *tissue(200)),
        BatchEntry(mrf_events(mrf_schedule()[:120], 10.0), 20, *tissue(150)),
        BatchEntry(mrf_events(rng.uniform(5, 70, 90).astype(np.float32),
                              rng.uniform(8, 15, 90).astype(np.float32), TI_ms=20.0), 33,
                   *tissue(64)),
        BatchEntry(fse_events(rng.uniform(100, 180, 9).astype(np.float32), 12.0,
                              phases_deg=90.0), 18, *tissue(77)),
    ]
    for shape in ((16, 2, 8), (4, 4, 4)):
        batch = SequenceBatch(entries, cuda)
        batch.out.fill_(float("nan"))
        batch.launch(shape)
        torch.cuda.synchronize()
        _check_against_oracle(batch)
        alone = SequenceBatch([entries[0]], cuda)
        alone.launch(shape)
        torch.cuda.synchronize()
        assert torch.equal(alone.signal(0), batch.signal(0))
