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
    from torchsim_gb300.recon import NonlinearLeastSquares

    est = NonlinearLeastSquares(None, bounds={"T1": (50.0, 5000.0), "T2": (2.0, 1000.0),
                                              "M0": (0.0, 5.0)})
    params = torch.tensor([[100.0, 10.0, 1.0], [300.0, 30.0, 2.0], [200.0, 20.0, 3.0]])
    est.fit(parameters=params)
    assert est._start.tolist() == [200.0, 20.0, 2.0]
    bad = NonlinearLeastSquares(None, bounds={"T1": (50.0, 150.0)})
    with pytest.raises(ValueError):
        bad.fit(parameters=params)


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
