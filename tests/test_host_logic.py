"""Host-side logic that needs no GPU: the server's memory arena, latency
statistics, bound transforms, program caching keys and the autotuner cache."""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch


def test_arena_first_fit_and_merge():
    from torchsim_gb300.serving import Arena

    a = Arena(100)
    x = a.allocate(40)
    y = a.allocate(40)
    assert (x, y) == (0, 40)
    assert a.allocate(30) is None
    a.release(x, 40)
    assert a.allocate(30) == 0
    a.release(0, 30)
    a.release(y, 40)
    assert a.free == [(0, 100)]


def test_latency_summary():
    from torchsim_gb300.serving import MapRequest, latency_summary

    reqs = []
    for i in range(101):
        r = MapRequest(torch.zeros((1, 1), dtype=torch.complex64), arrival=0.0)
        r.completed = float(i)
        reqs.append(r)
    s = latency_summary(reqs)
    assert s["p50_s"] == 50.0 and s["p99_s"] == 99.0


def test_bounds_round_trip():
    from torchsim_gb300.recon import to_free

    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, 1000.0), "M0": (0.0, 5.0)}
    nat = torch.tensor([[1000.0, 80.0, 1.0], [60.0, 900.0, 4.5]], dtype=torch.float64)
    u = to_free(nat, bounds)
    lows = torch.tensor([50.0, 2.0, 0.0], dtype=torch.float64)
    highs = torch.tensor([5000.0, 1000.0, 5.0], dtype=torch.float64)
    back = lows + (highs - lows) * torch.sigmoid(u)
    assert torch.allclose(back, nat, rtol=1e-12)
    one_sided = to_free(torch.tensor([[3.0, 3.0, 3.0]], dtype=torch.float64),
                        {"T1": (1.0, None), "T2": (None, 5.0)})
    assert math.isclose(float(1.0 + torch.nn.functional.softplus(one_sided[0, 0])), 3.0)
    assert math.isclose(float(5.0 - torch.nn.functional.softplus(-one_sided[0, 1])), 3.0)
    with pytest.raises(ValueError):
        to_free(nat, {"T1": (10.0, 5.0)})


def test_nlls_start_is_median_and_checked():
    from torchsim_gb300 import MRFSimulator
    from torchsim_gb300.recon import NonlinearLeastSquares

    sim = MRFSimulator(flip=[10.0, 20.0], TR=10.0)
    est = NonlinearLeastSquares(sim, bounds={"T1": (50.0, 5000.0), "T2": (2.0, 1000.0),
                                             "M0": (0.0, 5.0)})
    est.fit(T1=[100.0, 300.0, 200.0], T2=[10.0, 30.0, 20.0], M0=[1.0, 2.0, 3.0])
    assert est._start.tolist() == [200.0, 20.0, 2.0]
    assert est.unknown == ("T1", "T2", "M0") and est.known == ()
    with pytest.raises(ValueError):
        NonlinearLeastSquares(sim, bounds={"T1": (50.0, 150.0)}).fit(
            T1=[100.0, 300.0, 200.0], T2=[10.0, 30.0, 20.0], M0=[1.0, 2.0, 3.0])
    with pytest.raises(ValueError):
        NonlinearLeastSquares(sim, bounds={"B1": (0.5, 1.5)}).fit(T1=(100.0, 3000.0))
    with pytest.raises(ValueError):
        est.fit(T1=(100.0, 3000.0), known={"T1": (100.0, 200.0)})
    with pytest.raises(RuntimeError):
        NonlinearLeastSquares(None).fit(T1=(100.0, 3000.0))
    with pytest.raises(RuntimeError):
        NonlinearLeastSquares(sim).map(torch.zeros(3, 2, dtype=torch.complex64))


def test_nlls_start_is_the_references(golden):
    """fit() draws the training parameters with the reference's generator and
    order (unknowns, then the measured properties; estimators/_mapping.py:
    339-361) and starts at their median: the reference's own start on the
    gn_mrf fixture, bit for bit."""
    from torchsim_gb300 import MRFSimulator
    from torchsim_gb300.recon import NonlinearLeastSquares

    d = golden("gn_mrf")
    sim = MRFSimulator(flip=torch.from_numpy(d["flip_deg"]), TR=10.0, states=10)
    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, 1000.0), "M0": (0.0, 5.0)}
    est = NonlinearLeastSquares(sim, bounds=bounds).fit(
        T1=(100.0, 3000.0), T2=(10.0, 300.0), M0=(0.5, 1.5), known={"B1": (0.8, 1.2)}, seed=0)
    assert torch.equal(est._start, torch.from_numpy(d["start"]))
    bound = NonlinearLeastSquares(sim.bind(B1=torch.from_numpy(d["b1"])), bounds=bounds).fit(
        T1=(100.0, 3000.0), T2=(10.0, 300.0), M0=(0.5, 1.5), seed=0)
    assert torch.equal(bound._start, torch.from_numpy(d["start"]))


def test_bind_holds_values_on_a_copy():
    from torchsim_gb300 import MRFSimulator

    sim = MRFSimulator(flip=[10.0, 20.0], TR=10.0, states=8)
    held = sim.bind(B1=torch.tensor([0.9, 1.1]), T1=1000.0, states=12)
    assert "B1" not in sim.protocol and sim.protocol["states"] == 8
    assert set(held.bound) == {"B1", "T1"} and held.protocol["states"] == 12
    assert held.protocol["flip"] == [10.0, 20.0]
    assert "T2" in held.exposes and held.accepts == held.exposes


def test_model_operator_host_logic():
    """ModelOperator's channels, its start (a value per unknown, the middle of
    a two-sided bound, the amplitude) and split() back, on the host."""
    from torchsim_gb300 import MRFSimulator
    from torchsim_gb300.recon import ModelOperator

    sim = MRFSimulator(flip=[10.0, 20.0], TR=10.0)
    op = ModelOperator(sim, "T1", "T2", bounds={"T1": (50.0, 5000.0), "T2": (2.0, None)},
                       scale={"T2": 4.0})
    assert op.channels == 4 and op.names == ("T1", "T2", "amplitude.real", "amplitude.imag")
    x = op.initial((5,), T2=torch.linspace(10.0, 90.0, 5), amplitude=2.0 - 1.0j)
    assert x.shape == (5, 4)
    back = op.split(x)
    torch.testing.assert_close(back["T1"], torch.full((5,), 2525.0), rtol=1e-5, atol=0)
    torch.testing.assert_close(back["T2"], torch.linspace(10.0, 90.0, 5), rtol=1e-5, atol=0)
    assert torch.equal(back["amplitude"], torch.full((5,), 2.0 - 1.0j))
    with pytest.raises(ValueError):
        ModelOperator(sim)
    with pytest.raises(ValueError):
        ModelOperator(sim, "T1", bounds={"T2": (1.0, 2.0)})
    with pytest.raises(ValueError):
        op.initial((2,))  # T2 has no two-sided bound
    with pytest.raises(ValueError):
        op.initial((2,), T1=50.0, T2=10.0)  # on the bound
    with pytest.raises(ValueError):
        op.split(torch.zeros(2, 3))


def test_natural_and_chain_factor_match_the_reference(golden):
    """to_natural on the reference's free variables gives the reference's own
    to_natural output (_bounds.py:77-105), and widen is its derivative."""
    import numpy as np

    from torchsim_gb300.recon import to_natural, widen

    d = golden("bounds")
    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, None), "M0": (None, 5.0)}
    names = ("T1", "T2", "M0", "B1")
    free = torch.from_numpy(d["free"])
    np.testing.assert_allclose(to_natural(free, bounds, names).numpy(), d["back"], rtol=1e-12,
                               atol=1e-12)
    u = free.clone().requires_grad_(True)
    to_natural(u, bounds, names).sum().backward()
    # torch's softplus takes its linear branch above 20, where its derivative
    # is 1 rather than sigmoid(u) = 1 - O(1e-9).
    np.testing.assert_allclose(widen(bounds, names, free).numpy(), u.grad.numpy(), rtol=1e-9,
                               atol=1e-300)


def test_autotune_cache(tmp_path, monkeypatch):
    from torchsim_gb300 import autotune

    monkeypatch.setenv("TORCHSIM_GB300_CACHE", str(tmp_path / "t.json"))
    autotune._memory.clear()
    autotune._store("k", [1, 2, 3])
    assert autotune._load()["k"] == [1, 2, 3]
    assert autotune.sweep_shapes(20, [(4, 5), (2, 5), (8, 4)], warps=(4,)) == [(4, 5, 4), (8, 4, 4)]


def test_program_key_changes_with_content():
    from torchsim_gb300.sequence import mrf_events

    a = mrf_events(np.float32([10, 20]), 10.0)
    b = mrf_events(np.float32([10, 21]), 10.0)
    assert a.key() != b.key() and a.key() == mrf_events(np.float32([10, 20]), 10.0).key()


def test_engine_facade_defaults_and_labels():
    from torchsim_gb300 import EpgEngine
    from torchsim_gb300.sequence import fse_events, mrf_events

    mrf = mrf_events(np.float32([10, 20, 30]), 10.0, repetitions=2)
    eng = EpgEngine()
    assert eng.shifts_per_repetition(mrf) == 3
    fse = fse_events(np.float32([180, 150]), 10.0, phases_deg=90.0)
    assert eng.shifts_per_repetition(fse) == 4
    # Samples are recorded by the ADC events of the last playing, in order.
    assert mrf.sample_events().tolist() == [13 + 2, 13 + 6, 13 + 10]
    assert fse.sample_events().tolist() == [2, 5]
    assert mrf.echo.tolist() == [False] * 3 and fse.echo.tolist() == [True, True]
    with pytest.raises(ValueError):
        eng.simulate(mrf, {"T1": 1000.0, "T2": 80.0}, repetitions=3)
    with pytest.raises(ValueError):
        eng.simulate(mrf, {"T1": 1000.0, "T2": 80.0}, record="odd")
    with pytest.raises(ValueError):
        eng.simulate(mrf, {"T1": 1000.0})


def test_free_variables_match_the_reference(golden):
    """The reference's own to_free (_bounds.py:113-160) on values inside
    two-sided, lower-only, upper-only and absent bounds, edges included
    (tests/golden/bounds.npz, made by tests/golden/make_golden.py)."""
    import numpy as np

    from torchsim_gb300.recon import to_free

    d = golden("bounds")
    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, None), "M0": (None, 5.0)}
    got = to_free(torch.from_numpy(d["natural"]), bounds, ("T1", "T2", "M0", "B1")).numpy()
    np.testing.assert_allclose(got, d["free"], rtol=1e-12, atol=1e-12)
    # And the reference's inverse takes them back (inside the edge clamps).
    inside = np.abs(d["back"] - d["natural"]) <= 1e-6 * np.maximum(1.0, np.abs(d["natural"]))
    assert inside.mean() > 0.95


def test_autodiff_routing_sees_every_kind_of_tracked_tensor():
    """The simulators take the differentiable route for a tensor that
    requires grad, one inside torch.func.jvp and a forward-AD dual tensor, and
    read the values of each on the host outside the transform."""
    import torch
    import torch.autograd.forward_ad as fwAD

    from torchsim_gb300.simulators import _primal, _tracked

    x = torch.arange(4, dtype=torch.float32)
    assert not _tracked(x) and not _tracked(1.0) and not _tracked(None)
    assert _tracked(x.clone().requires_grad_())
    with torch.no_grad():
        assert not _tracked(x.clone().requires_grad_())
    seen = {}

    def inside(a):
        seen["tracked"] = _tracked(a)
        with torch._C._DisableFuncTorch():
            seen["values"] = _primal(a).numpy().copy()
        return a * 2

    torch.func.jvp(inside, (x,), (torch.ones(4),))
    assert seen["tracked"] and np.array_equal(seen["values"], x.numpy())
    with fwAD.dual_level():
        d = fwAD.make_dual(x, torch.ones(4))
        assert _tracked(d)
        assert np.array_equal(_primal(d).numpy(), x.numpy())
