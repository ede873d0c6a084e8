"""The direct route: EpgEngine.simulate on a packed stream, against the
functional API and the FP64 oracle, with the sample labels
(sequence/_simulation.py:239-484)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import draw_tissue, max_rel, packed_from_events

pytestmark = pytest.mark.gpu

SIGNAL_TOL = 1e-5


def test_engine_matches_mrf_sim_and_oracle(cuda, golden):
    import torchsim_gb300 as ts
    from torchsim_gb300.sequence import mrf_events

    d = golden("mrf880")
    flip = torch.from_numpy(d["flip_deg"])
    t1, t2, b1 = (torch.from_numpy(d[k]) for k in ("t1", "t2", "b1"))
    ev = mrf_events(flip, 10.0)
    res = ts.EpgEngine().simulate(ev, {"T1": t1.to(cuda), "T2": t2.to(cuda), "B1": b1.to(cuda)},
                                  nstates=10)
    direct = ts.mrf_sim(flip, 10.0, t1.to(cuda), t2.to(cuda), B1=b1.to(cuda), states=10)
    assert torch.equal(res.signal, direct)
    assert res.signal.shape == (t1.numel(), 880)
    assert torch.equal(res.time_us.cpu(), torch.from_numpy(ev.time_us))
    assert res.event_index.cpu().tolist() == (2 + 4 * np.arange(880)).tolist()
    assert int(res.repetition.max()) == 0 and not bool(res.echo.any())
    ref = O.forward(packed_from_events(ev, d["t1"], d["t2"], 10, b1=d["b1"]), "f64")
    assert max_rel(-res.signal.real.cpu().numpy(), ref) <= SIGNAL_TOL


def test_engine_default_states_and_echo_record(cuda):
    import torchsim_gb300 as ts
    from torchsim_gb300.sequence import fse_events

    rng = np.random.default_rng(4)
    ev = fse_events(rng.uniform(120, 180, 12).astype(np.float32), 8.0, phases_deg=90.0)
    T1 = torch.from_numpy(rng.uniform(500, 2000, 64).astype(np.float32)).to(cuda)
    T2 = torch.from_numpy(rng.uniform(30, 200, 64).astype(np.float32)).to(cuda)
    eng = ts.EpgEngine()
    res = eng.simulate(ev, {"T1": T1, "T2": T2}, record="echo")
    # 12 echoes wind the states by 2 each: 1 + 24 states.
    states = max(8, min(64, 1 + eng.shifts_per_repetition(ev)))
    assert states == 25
    same = eng.simulate(ev, {"T1": T1, "T2": T2}, nstates=states)
    assert torch.equal(res.signal, same.signal)
    assert res.signal.shape == (64, 12) and bool(res.echo.all())
    ref = O.forward(packed_from_events(ev, T1.cpu().numpy(), T2.cpu().numpy(), states), "f64")
    assert max_rel(-res.signal.real.cpu().numpy(), ref) <= SIGNAL_TOL


def test_host_pipeline_matches_the_device_pass(cuda):
    """forward_tangents_host (pinned host maps in, pinned host samples out,
    chunked with overlapping copies) gives the device pass's bits."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(9)
    ev = mrf_events(rng.uniform(5, 60, 70).astype(np.float32), 9.0)
    prog = program_for(ev, cuda)
    V = 1000
    t1, t2, b1 = draw_tissue(10, V)
    names = ("T1", "T2", "B1")
    dev_maps = engine.tissue_maps(cuda, V, t1, t2, None, b1, None)
    sig, jac = engine.forward_tangents(prog, dev_maps, 12, names)
    host = engine.TissueMaps(*[torch.from_numpy(a).pin_memory() for a in (t1, t2)], None,
                             torch.from_numpy(b1).pin_memory(), None)
    sig_h = torch.empty((V, ev.outputs), dtype=torch.complex64).pin_memory()
    jac_h = torch.empty((V, 3, ev.outputs), dtype=torch.complex64).pin_memory()
    for chunks in (1, 7, 16):
        sig_h.zero_()
        jac_h.zero_()
        engine.forward_tangents_host(prog, host, 12, names, sig_h, jac_h, chunks=chunks,
                                     device=cuda)
        torch.cuda.synchronize()
        assert torch.equal(sig_h, sig.cpu()) and torch.equal(jac_h, jac.cpu()), chunks
    with pytest.raises(ValueError):
        engine.forward_tangents_host(prog, host, 12, names, torch.empty_like(sig_h, device="cpu"),
                                     jac_h, device=cuda)


def test_host_tensor_calls_match_device_calls(cuda):
    """mrf_sim with CPU tensors sweeps in chunks whose copies back overlap
    the next chunk (here 3 chunks of the Jacobian call) and returns CPU
    tensors bitwise equal to the device call's results."""
    import torchsim_gb300 as ts
    from tests.helpers import draw_tissue, mrf_schedule

    t1, t2, b1 = (torch.from_numpy(a) for a in draw_tissue(21, 8192))
    flip = torch.from_numpy(mrf_schedule())
    for diff in (None, ("T1", "T2", "B1")):
        host = ts.mrf_sim(flip, 10.0, t1, t2, B1=b1, diff=diff, states=12)
        dev = ts.mrf_sim(flip.to(cuda), 10.0, t1.to(cuda), t2.to(cuda), B1=b1.to(cuda),
                         diff=diff, states=12)
        host = host if isinstance(host, tuple) else (host,)
        dev = dev if isinstance(dev, tuple) else (dev,)
        for h, d in zip(host, dev, strict=True):
            assert h.device.type == "cpu"
            assert torch.equal(h, d.cpu())
