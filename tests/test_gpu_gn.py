"""GPU tests of the Gauss-Newton mapping and the continuously batched server."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from tests.helpers import draw_tissue

pytestmark = pytest.mark.gpu

BOUNDS = {"T1": (50.0, 5000.0), "T2": (2.0, 1000.0), "M0": (0.0, 5.0)}


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_gn_matches_reference_nlls(cuda, golden):
    """The reference's NonlinearLeastSquares (LM, 20 steps) on noisy MRF."""
    from torchsim_gb300 import MRFSimulator
    from torchsim_gb300.recon import GaussNewton, NonlinearLeastSquares, TrustRegion

    d = golden("gn_mrf")
    bounds = {k: tuple(d["bounds"][i]) for i, k in enumerate(("T1", "T2", "M0"))}
    est = NonlinearLeastSquares(MRFSimulator(flip=d["flip_deg"], TR=10.0, states=10), bounds=bounds,
                                loop=GaussNewton(TrustRegion(), max_iterations=20))
    est.fit(parameters=torch.from_numpy(d["start"][None, :]))
    maps = est.map(torch.from_numpy(d["measured"]).to(cuda), known={"B1": torch.from_numpy(d["b1"])})
    for name, key in (("T1", "map_t1"), ("T2", "map_t2"), ("M0", "map_m0")):
        assert rel(maps[name].cpu().numpy(), d[key]) <= 2e-3, name
    # The reference converged all 16 within its 20 steps, the last on its
    # 20th; with FP64 normal equations a slow voxel may need one more.
    assert est.unconverged <= 1


def _signals(cuda, V, seed, noise=True, pulses=None):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for
    from tests.helpers import mrf_schedule

    rng = np.random.default_rng(seed)
    t1, t2, b1 = draw_tissue(seed, V)
    m0 = rng.uniform(0.5, 1.5, V).astype(np.float32)
    flip = mrf_schedule() if pulses is None else mrf_schedule()[:pulses]
    prog = program_for(mrf_events(flip, 10.0), cuda)
    tissue = engine.tissue_maps(cuda, V, t1, t2, m0, b1, None)
    sig = engine.forward(prog, tissue, 10)
    if noise:
        g = torch.Generator(device=cuda).manual_seed(seed)
        sigma = sig.abs().mean() / 50
        sig = sig + sigma * torch.complex(torch.randn(sig.shape, device=cuda, generator=g),
                                          torch.randn(sig.shape, device=cuda, generator=g))
    return prog, sig, (t1, t2, m0, b1)


def test_gn_noiseless_recovery(cuda):
    from torchsim_gb300.recon import GaussNewton, TrustRegion

    prog, sig, (t1, t2, m0, b1) = _signals(cuda, 500, 1, noise=False)
    start = torch.tensor([1000.0, 80.0, 1.0])
    sol = GaussNewton(TrustRegion(), max_iterations=40).minimize(
        prog, sig, start, BOUNDS, 10, b1=torch.from_numpy(b1))
    x = sol.x.cpu().numpy()
    for k, truth in enumerate((t1, t2, m0)):
        assert np.median(np.abs(x[:, k] - truth) / truth) <= 1e-4, k
        assert np.quantile(np.abs(x[:, k] - truth) / truth, 0.95) <= 1e-2, k


def test_fused_and_plain_forms_agree(cuda):
    from torchsim_gb300.recon import GaussNewton, PlainGaussNewton, TrustRegion

    prog, sig, (t1, t2, m0, b1) = _signals(cuda, 300, 2)
    start = torch.tensor([1000.0, 80.0, 1.0])
    b1t = torch.from_numpy(b1)
    fused = GaussNewton(TrustRegion(), max_iterations=10).minimize(prog, sig, start, BOUNDS, 10, b1=b1t)
    plain = PlainGaussNewton(TrustRegion(), max_iterations=10).minimize(prog, sig, start, BOUNDS, 10,
                                                                       b1=b1t)
    for k in range(3):
        a, b = fused.x[:, k].cpu().numpy(), plain.x[:, k].cpu().numpy()
        assert np.median(np.abs(a - b) / np.abs(b)) <= 1e-3, k


def test_server_alone_equals_mix_and_respects_budget(cuda):
    from torchsim_gb300.serving import GNServer, MapRequest

    prog, _, _ = _signals(cuda, 4, 0, pulses=200)
    reqs = []
    for i, V in enumerate((300, 37, 1024, 5, 640)):
        _, sig, (_, _, _, b1) = _signals(cuda, V, 10 + i, pulses=200)
        reqs.append(MapRequest(sig, torch.from_numpy(b1).to(cuda), arrival=0.0, id=i))
    start = torch.tensor([1000.0, 80.0, 1.0])
    alone = {}
    for r in reqs:
        server = GNServer(prog, 10, BOUNDS, start, budget_bytes=64 << 20, device=cuda)
        out = server.serve([MapRequest(r.measured, r.b1, id=r.id)], realtime=False)
        alone[r.id] = out[0].maps
    # A budget that holds about two of the larger requests at once forces
    # requests to wait for memory and to join batches already running.
    per_voxel = 200 * 8 + 400
    server = GNServer(prog, 10, BOUNDS, start, budget_bytes=1500 * per_voxel, device=cuda)
    done = server.serve([MapRequest(r.measured, r.b1, id=r.id) for r in reqs], realtime=False)
    assert len(done) == len(reqs) and server.stats.waits_for_memory > 0
    for r in done:
        for name in ("T1", "T2", "M0"):
            assert torch.equal(r.maps[name], alone[r.id][name]), (r.id, name)
    assert all(r.latency is not None and r.latency >= 0 for r in done)
    with pytest.raises(ValueError):
        server.submit(MapRequest(torch.zeros((1, 200), dtype=torch.complex64,
                                             device=cuda).expand(10**6, 200)))
